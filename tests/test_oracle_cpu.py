"""Known-answer tests of the CPU oracle (no GPU).

The reference has no tests for this path, so the oracle is pinned here by
analytic cases (two-body force, Newton's third law, symmetric lattice,
hand-derived octrees, theta -> 0 equals direct sum), by an independent
pure-Python restatement of the octree key descent on small inputs, and by the
committed golden fixtures.
"""
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLD = os.path.join(os.path.dirname(__file__), "golden", "nbody_small.npz")


def recs(pos, mass, vel=None):
    pos = np.asarray(pos, np.float32)
    p = np.zeros(pos.shape[0], O.PARTICLE_DTYPE)
    p["position"] = pos
    p["mass"] = mass
    if vel is not None:
        p["velocity"] = vel
    return p


# --- pure-Python octree descent (src/Sim/Octree.cpp:16-51, Octree.hpp:18-22) ---
def py_key(p, half=4000.0, levels=21):
    """Octant path of a point, float32 Split arithmetic, one level at a time."""
    f = np.float32
    x = [f(c) for c in p]
    lo = [f(-half)] * 3
    hi = [f(half)] * 3
    if not all(lo[a] <= x[a] < hi[a] for a in range(3)):
        return (1 << 64) - 1, 0
    size = f(hi[0] - lo[0])
    key = 0
    for level in range(levels):
        s = f(size / f(2))
        mid = [f(lo[a] + s) for a in range(3)]
        top = [f(mid[a] + s) for a in range(3)]
        oct_ = 0
        nlo, nhi = list(lo), list(hi)
        for a in range(3):
            if mid[a] <= x[a] < top[a]:
                oct_ |= 1 << a
                nlo[a], nhi[a] = mid[a], top[a]
            elif lo[a] <= x[a] < mid[a]:
                nlo[a], nhi[a] = lo[a], mid[a]
            else:
                return key, level
        lo, hi = nlo, nhi
        size = f(hi[0] - lo[0])
        key = (key << 3) | oct_
    return key, levels


def test_particle_record_layout():
    d = O.PARTICLE_DTYPE
    assert d.itemsize == 104
    assert d.fields["position"][1] == 0
    assert d.fields["colour"][1] == 12
    assert d.fields["original_colour"][1] == 28
    assert d.fields["velocity"][1] == 48
    assert d.fields["forces"][1] == 72
    assert d.fields["mass"][1] == 96


@pytest.mark.parametrize("S", [0.0, 1e-4, 0.5])
def test_two_body_reference_law(S):
    p = recs([[0, 0, 0], [1, 0, 0]], [2.0, 3.0])
    F = O.direct_forces(p, G=1.0, S=S)
    expect = 6.0 / (1.0 + S)
    np.testing.assert_allclose(F[0], [expect, 0, 0], rtol=1e-15)
    np.testing.assert_allclose(F[1], [-expect, 0, 0], rtol=1e-15)


def test_two_body_plummer_law():
    p = recs([[0, 0, 0], [0, 2, 0]], [1.0, 4.0])
    S = 0.25
    F = O.direct_forces(p, G=2.0, S=S, law=1)
    expect = 2.0 * 1.0 * 4.0 * 2.0 / (4.0 + S) ** 1.5
    np.testing.assert_allclose(F[0], [0, expect, 0], rtol=1e-7)
    np.testing.assert_allclose(F[1], [0, -expect, 0], rtol=1e-7)


def test_newton_third_law():
    rng = np.random.default_rng(3)
    pos = rng.normal(size=(200, 3)).astype(np.float32)
    m = rng.uniform(0.5, 2.0, 200).astype(np.float32).astype(np.float64)
    F = O.direct_forces(recs(pos, m), G=1.0, S=1e-3)
    tot = np.abs(F).sum()
    assert np.abs(F.sum(axis=0)).max() < 1e-13 * tot


def test_symmetric_lattice_zero_force_at_centre():
    g = np.array([[x, y, z] for x in (-1, 0, 1) for y in (-1, 0, 1) for z in (-1, 0, 1)], np.float32)
    F = O.direct_forces(recs(g, np.ones(27)), G=1.0, S=0.0)
    centre = 13
    assert np.allclose(g[centre], 0)
    assert np.abs(F[centre]).max() < 1e-14
    assert np.abs(F[0]).max() > 0.1


def test_fp64_oracle_matches_float_oracle():
    rng = np.random.default_rng(5)
    pos = rng.normal(size=(300, 3)).astype(np.float32)
    m = np.full(300, 1.0 / 300)
    F = O.direct_forces(recs(pos, m), G=1.0, S=1e-4)
    F64 = O.fp64_forces(pos.astype(np.float64), m, np.arange(300), G=1.0, S=1e-4)
    assert O.rel_l2(F, F64) < 1e-6


def test_tree_two_bodies_octants():
    t = O.OracleTree(recs([[1, 1, 1], [-1, -1, -1]], [1.0, 1.0]))
    nd = t.nodes()
    assert len(nd["level"]) == 9
    assert nd["count"][0] == 2 and nd["first_child"][0] == 1
    # octant i = x + 2y + 4z: (+,+,+) -> 7, (-,-,-) -> 0
    assert nd["body"][1 + 7] == 0 and nd["body"][1 + 0] == 1
    assert all(nd["count"][1 + k] == 0 for k in range(1, 7))
    np.testing.assert_array_equal(nd["side"][1:], np.float32(4000.0))
    keys, depth = t.keys()
    assert keys[0] >> 60 == 7 and keys[1] >> 60 == 0
    assert list(depth) == [21, 21]


def test_tree_three_bodies_chain_and_com():
    pts = [[1, 1, 1], [2, 2, 2], [-1, -1, -1]]
    m = [1.0, 3.0, 2.0]
    t = O.OracleTree(recs(pts, m))
    nd = t.nodes()
    keys, _ = t.keys()
    k0, k1 = int(keys[0]), int(keys[1])
    common = 0
    for lv in range(21):
        if (k0 >> (60 - 3 * lv)) & 7 == (k1 >> (60 - 3 * lv)) & 7:
            common += 1
        else:
            break
    # internal nodes: root + one per shared level of bodies 0 and 1
    internal = int((nd["first_child"] >= 0).sum())
    assert internal == 1 + common
    assert len(nd["level"]) == 1 + 8 * internal
    # root: mass 6, com = (1*1 + 3*2 - 2*1)/6 in float arithmetic order
    assert nd["mass"][0] == 6.0
    np.testing.assert_allclose(nd["com"][0], [5.0 / 6] * 3, rtol=1e-6)


def test_tree_boundaries_and_dropped_body():
    pts = [[0, 0, 0], [-2000, -2000, -2000], [4000, 0, 0], [-4000, -4000, -4000], [3999.0, 1, 1]]
    t = O.OracleTree(recs(pts, [1, 1, 1, 1, 1]))
    keys, depth = t.keys()
    nd = t.nodes()
    assert nd["count"][0] == 5            # the dropped body is still counted
    assert depth[2] == 0 and keys[2] == np.uint64(2**64 - 1)   # x = +4000 is outside [lo, hi)
    assert keys[0] >> 60 == 7             # 0 belongs to the upper half
    assert depth[3] == 21                 # -4000 is inside (closed lower bound)
    for i, p in enumerate(pts):
        k, d = py_key(p)
        assert (int(keys[i]), int(depth[i])) == (k, d), i


def test_keys_match_python_descent_random():
    rng = np.random.default_rng(9)
    pos = np.concatenate([rng.normal(scale=2.0, size=(60, 3)), rng.uniform(-3999, 3999, size=(20, 3)),
                          rng.normal(scale=1e-3, size=(20, 3))]).astype(np.float32)
    t = O.OracleTree(recs(pos, np.ones(len(pos))))
    keys, depth = t.keys()
    for i in range(len(pos)):
        k, d = py_key(pos[i])
        assert (int(keys[i]), int(depth[i])) == (k, d)


def test_tree_topology_is_prefix_closure():
    """Internal nodes are exactly the key prefixes shared by >= 2 bodies."""
    rng = np.random.default_rng(1)
    pos = rng.normal(size=(400, 3)).astype(np.float32)
    t = O.OracleTree(recs(pos, np.ones(400)))
    keys, depth = t.keys()
    nd = t.nodes()
    internal = set()
    for lv in range(0, 21):
        sh = 63 - 3 * lv
        pref = keys >> np.uint64(sh) if lv else np.zeros_like(keys)
        u, c = np.unique(pref, return_counts=True)
        internal |= {(lv, int(x)) for x in u[c >= 2]}
    got = {(int(l), int(p)) for l, p, fc in zip(nd["level"], nd["prefix"], nd["first_child"]) if fc >= 0}
    assert got == internal


def test_theta_zero_equals_direct_sum():
    rng = np.random.default_rng(2)
    pos = rng.normal(size=(150, 3)).astype(np.float32)
    m = rng.uniform(0.5, 1.5, 150)
    p = recs(pos, m)
    Fd = O.direct_forces(p, G=1.0, S=1e-3)
    t = O.OracleTree(p)
    Fb, inter = t.forces(G=1.0, S=1e-3, theta=0.0)
    assert inter == 150 * 149
    assert O.rel_l2(Fb, Fd) < 1e-13


def test_bh_error_against_direct_at_half():
    rng = np.random.default_rng(4)
    pos = rng.normal(size=(2000, 3)).astype(np.float32)
    p = recs(pos, np.full(2000, 1.0 / 2000))
    Fd = O.direct_forces(p, G=1.0, S=1e-4)
    Fb, _ = O.OracleTree(p).forces(G=1.0, S=1e-4, theta=0.5)
    assert O.rel_l2(Fb, Fd) < 1e-2


def test_kick_drift_order():
    """v += F/m dt, then x += float(v dt / scale), Forces zeroed (direct sum)."""
    p = recs([[0, 0, 0], [1, 0, 0]], [1.0, 1.0], vel=[[0, 0.5, 0], [0, 0, 0]])
    out = O.direct_step(p, 0.1, 1, G=1.0, S=0.0)
    dt = float(np.float32(0.1))          # Update(float dt) promotes dt to double
    v0 = np.array([1.0 * dt, 0.5, 0.0])
    np.testing.assert_array_equal(out["velocity"][0], v0)
    np.testing.assert_array_equal(out["position"][0], (v0 * dt).astype(np.float32))
    assert np.all(out["forces"] == 0)
    bh = O.bh_step(p, 0.1, 1, G=1.0, S=0.0, theta=0.5)
    np.testing.assert_allclose(bh["forces"][0], [1.0, 0, 0], rtol=1e-12)   # assigned, not reset


def test_depth_cap_bucket():
    p = recs([[1, 1, 1], [1, 1, 1], [1, 1, 1.0000001]], [1.0, 2.0, 3.0])
    t = O.OracleTree(p, max_depth=21)
    nd = t.nodes()
    leaf_buckets = np.nonzero(nd["bucket_size"] >= 2)[0]
    assert len(leaf_buckets) == 1
    b = leaf_buckets[0]
    assert nd["level"][b] == 21
    assert sorted(t.bucket(b)) == [0, 1, 2]
    assert t.deeper_buckets() == 1       # bodies 0,1 vs 2 differ: the reference would split further
    F, _ = t.forces(G=1.0, S=1e-4, theta=0.5)
    Fd = O.direct_forces(p, G=1.0, S=1e-4)
    assert O.rel_l2(F, Fd) < 1e-12


def test_golden_fixtures_reproduce():
    g = np.load(GOLD)
    rec = O.particles_from_soa(g["plummer256_pos_mass"], g["plummer256_vel"])
    np.testing.assert_array_equal(O.direct_forces(rec, G=1.0, S=1e-4), g["plummer256_direct_forces"])
    after = O.direct_step(rec, 1e-3, 10, G=1.0, S=1e-4)
    np.testing.assert_array_equal(after["position"], g["plummer256_direct_10_pos"])
    rec = O.particles_from_soa(g["disk512_pos_mass"], g["disk512_vel"])
    t = O.OracleTree(rec)
    keys, depth = t.keys()
    np.testing.assert_array_equal(keys, g["disk512_keys"])
    nd = t.nodes()
    for k in ("level", "count", "first_child", "body", "prefix", "mass", "com", "side", "lo"):
        np.testing.assert_array_equal(nd[k], g["disk512_node_" + k])
    f, inter = t.forces(G=1.0, S=0.005 ** 2, theta=0.5)
    np.testing.assert_array_equal(f, g["disk512_bh_forces"])
    assert inter == int(g["disk512_bh_interactions"][0])
