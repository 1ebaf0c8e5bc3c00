"""GPU parity of the Barnes-Hut path (K2 keys, K3 sort, K4 topology, K5 mass,
K6 traversal) against the CPU oracle (restated BarnesHut + Octree).

Bit-exact: Morton keys and depths, the set of non-empty nodes with their
NumParticles, TotalMass, CentreOfMass, side and TopLeft, one-body leaves and
depth-cap bucket membership, and the number of interactions (the per-body
opening decisions are exact).  Forces: within 1e-3 relative L2 error of the
oracle (the path reproduces the reference's decisions, so the measured error
is ~1e-6).  Against the FP64 direct sum the reference algorithm itself
(monopoles, opening test side/|p - COM| < theta) errs by a few 1e-3 at
theta = 0.5; REF_ALGO_FP64_TOL bounds that.
"""
import os

import numpy as np
import pytest

import nbody_gb300 as nb
from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden", "nbody_small.npz")
BH_TOL = 1e-3
REF_ALGO_FP64_TOL = 1e-2


def bh_sim(**kw):
    kw.setdefault("softening2", 0.005 ** 2)
    return nb.NBodySim(kind=nb.SIM_BARNES_HUT, **kw)


def codes(level, prefix):
    level = np.asarray(level, np.uint64)
    return (np.uint64(1) << (np.uint64(3) * level)) | np.asarray(prefix, np.uint64)


def assert_same_tree(s: nb.NBodySim, t: O.OracleTree):
    """Keys, depths and every non-empty node agree bit for bit."""
    k, d = s.tree_keys()
    ko, do = t.keys()
    np.testing.assert_array_equal(k, ko)
    np.testing.assert_array_equal(d, do)
    g = s.tree_nodes()
    order = s.tree_order()
    o = t.nodes()
    ne = np.nonzero(o["count"] > 0)[0]
    oc = codes(o["level"][ne], o["prefix"][ne])
    gc = codes(g["level"], g["prefix"])
    oi = ne[np.argsort(oc)]
    gi = np.argsort(gc)
    np.testing.assert_array_equal(np.sort(gc), np.sort(oc))
    for f in ("level", "count", "mass", "side"):
        np.testing.assert_array_equal(g[f][gi], o[f][oi], err_msg=f)
    np.testing.assert_array_equal(g["com"][gi], o["com"][oi])
    np.testing.assert_array_equal(g["lo"][gi], o["lo"][oi])
    np.testing.assert_array_equal(g["first_child"][gi] >= 0, o["first_child"][oi] >= 0)
    single = o["body"][oi] >= 0
    np.testing.assert_array_equal(g["body"][gi][single], o["body"][oi][single])
    for gj, oj in zip(gi, oi):
        if o["bucket_size"][oj] >= 2:
            mem = np.sort(order[g["bucket_begin"][gj]:g["bucket_end"][gj]])
            np.testing.assert_array_equal(mem, t.bucket(int(oj)))
    st = s.tree_stats()
    assert st["lookup_failures"] == 0
    assert st["deeper_buckets"] == t.deeper_buckets()
    return st


def test_golden_disk512_tree_and_forces():
    g = np.load(GOLD)
    with bh_sim(theta=0.5) as s:
        s.init_soa(g["disk512_pos_mass"], g["disk512_vel"])
        k, d = s.tree_keys()
        np.testing.assert_array_equal(k, g["disk512_keys"])
        np.testing.assert_array_equal(d, g["disk512_depth"])
        F = s.compute_forces()
        assert s.last_interactions() == int(g["disk512_bh_interactions"][0])
    assert O.rel_l2(F, g["disk512_bh_forces"]) < 1e-5


@pytest.mark.parametrize("model,n,seed", [("disk", 20000, 1), ("plummer", 30000, 2), ("collision", 16384, 3)])
def test_tree_bit_exact_and_forces(model, n, seed):
    pm, v = getattr(nb, "seed_" + model)(seed, n)
    rec = nb.records_from_soa(pm, v)
    t = O.OracleTree(rec)
    S = 0.005 ** 2
    with bh_sim(theta=0.5) as s:
        s.init(rec)
        F = s.compute_forces()
        inter = s.last_interactions()
        st = assert_same_tree(s, t)
        F64 = s.fp64_forces(np.arange(0, n, 5))
    assert st["gaps"] == 0
    Fo, inter_o = t.forces(G=1.0, S=S, theta=0.5)
    assert inter == inter_o
    assert O.rel_l2(F, Fo) < 1e-5          # same decisions: only FP32 vs FP64 summation differs
    assert O.rel_l2(F[::5], F64) < REF_ALGO_FP64_TOL


@pytest.mark.parametrize("spread_second", [1.0, 1500.0])
def test_tree_when_root_octants_fix_the_upper_digits(spread_second):
    """The radix sort skips a pass whose digit is fixed within each root
    octant (the top pass orders the octants).  Two clusters in opposite root
    octants: both tight (levels 2-7 fixed in each octant, passes skipped), or
    the second spread over its octant (those passes must run); bodies outside
    the root form their own group.  The tree stays the oracle's either way."""
    rng = np.random.default_rng(7)
    a = rng.normal(20.0, 1.0, (3000, 3))
    b = rng.normal(-20.0, 1.0, (3000, 3)) if spread_second < 10 else -rng.uniform(1.0, spread_second, (3000, 3))
    out = np.array([[5000.0, 1.0, 1.0], [-4500.0, 0.0, 3.0]])
    x = np.concatenate([a, b, out]).astype(np.float32)
    pm = np.concatenate([x, np.full((len(x), 1), 1.0 / len(x), np.float32)], axis=1).astype(np.float32)
    v = np.zeros_like(pm)
    rec = nb.records_from_soa(pm, v)
    t = O.OracleTree(rec)
    with bh_sim(theta=0.5) as s:
        s.init(rec)
        F = s.compute_forces()
        inter = s.last_interactions()
        assert_same_tree(s, t)
    Fo, inter_o = t.forces(G=1.0, S=0.005 ** 2, theta=0.5)
    assert inter == inter_o
    assert O.rel_l2(F, Fo) < 1e-5


@pytest.mark.parametrize("theta", [0.0, 0.3, 0.6, 1.0, 2.0])
def test_theta_semantics(theta):
    """theta=0 is direct summation; theta=0.6 lets a body accept its own cell."""
    pm, v = nb.seed_plummer(4, 5000)
    rec = nb.records_from_soa(pm, v)
    t = O.OracleTree(rec)
    with bh_sim(theta=theta, softening2=1e-4) as s:
        s.init(rec)
        F = s.compute_forces()
        inter = s.last_interactions()
    Fo, inter_o = t.forces(G=1.0, S=1e-4, theta=theta)
    assert inter == inter_o
    assert O.rel_l2(F, Fo) < 1e-5
    if theta == 0.0:
        assert inter == 5000 * 4999


def test_edge_inputs_boundaries_dropped_and_coincident():
    rng = np.random.default_rng(11)
    pts = [rng.normal(size=(300, 3)),
           np.array([[0, 0, 0], [-2000, -2000, -2000], [4000, 0, 0], [-4000, -4000, -4000],
                     [3999.0, 1, 1], [1e5, 0, 0], [-3999.9, 3999.9, 0]]),
           np.tile([[0.5, 0.25, 0.125]], (5, 1)),                       # coincident: a bucket
           np.array([[0.5, 0.25, 0.1250001], [1e-30, -1e-30, 0.0]])]
    pos = np.concatenate(pts).astype(np.float32)
    n = len(pos)
    pm = np.zeros((n, 4), np.float32)
    pm[:, :3] = pos
    pm[:, 3] = rng.uniform(0.5, 2.0, n).astype(np.float32)
    v = np.zeros((n, 4), np.float32)
    rec = nb.records_from_soa(pm, v)
    t = O.OracleTree(rec)
    with bh_sim(theta=0.5, softening2=1e-4) as s:
        s.init(rec)
        F = s.compute_forces()
        inter = s.last_interactions()
        st = assert_same_tree(s, t)
    assert st["outside"] == 2
    assert st["deeper_buckets"] >= 1
    Fo, inter_o = t.forces(G=1.0, S=1e-4, theta=0.5)
    assert inter == inter_o
    assert O.rel_l2(F, Fo) < 1e-5


@pytest.mark.parametrize("n", [1, 2, 3, 17])
def test_tiny_counts(n):
    pm, v = nb.seed_plummer(6, max(n, 2))
    pm, v = pm[:n].copy(), v[:n].copy()
    rec = nb.records_from_soa(pm, v)
    with bh_sim(theta=0.5, softening2=1e-4) as s:
        s.init(rec)
        F = s.compute_forces()
    if n == 1:
        assert np.all(F == 0)
    else:
        Fo, _ = O.OracleTree(rec).forces(G=1.0, S=1e-4, theta=0.5)
        assert O.rel_l2(F, Fo) < 1e-5


def test_steps_match_oracle_and_forces_persist():
    pm, v = nb.seed_disk(7, 8192)
    rec = nb.records_from_soa(pm, v)
    S = 0.005 ** 2
    ref = O.bh_step(rec, 5e-4, 5, G=1.0, S=S, theta=0.5)
    with bh_sim(theta=0.5) as s:
        s.init(rec)
        s.step(5e-4, 5)
        out = rec.copy()
        s.write_back(out)
    assert O.rel_l2(out["position"], ref["position"]) < 1e-5
    assert O.rel_l2(out["velocity"], ref["velocity"]) < 1e-4
    # BarnesHut assigns Forces and never resets them
    assert O.rel_l2(out["forces"], ref["forces"]) < 1e-3
    assert np.abs(out["forces"]).sum() > 0


def test_plummer_law_tree():
    pm, v = nb.seed_plummer(8, 10000)
    rec = nb.records_from_soa(pm, v)
    with bh_sim(theta=0.5, law=nb.LAW_PLUMMER, softening2=1e-4) as s:
        s.init(rec)
        F = s.compute_forces()
    Fo, _ = O.OracleTree(rec).forces(G=1.0, S=1e-4, law=1, theta=0.5)
    assert O.rel_l2(F, Fo) < 1e-5


def test_full_size_config2_keys_topology_and_force_error():
    """N=1,048,576 disk + bulge: keys and topology bit-exact, force error vs FP64."""
    n = 1 << 20
    pm, v = nb.seed_disk(1234, n)
    rec = nb.records_from_soa(pm, v)
    t = O.OracleTree(rec)
    rng = np.random.default_rng(0)
    targets = np.sort(rng.choice(n, 4096, replace=False)).astype(np.int32)
    with bh_sim(theta=0.5) as s:
        s.init(rec)
        F = s.compute_forces()
        st = assert_same_tree(s, t)
        F64 = s.fp64_forces(targets)
    assert st["gaps"] == 0
    Fo = t.forces_subset(targets, G=1.0, S=0.005 ** 2, theta=0.5)
    assert O.rel_l2(F[targets], Fo) < 1e-5
    assert O.rel_l2(F[targets], F64) < REF_ALGO_FP64_TOL


def test_reinit_same_count_new_tree_shape():
    """Re-initialising a simulator with the same body count but a tree of a
    different shape (many more internal nodes than the node arrays were sized
    for; then no body inside the root cube; then the first set again) steps to
    exactly what a fresh simulator computes: node arrays grow, and no node of
    an earlier tree leaks into the next."""
    rng = np.random.default_rng(21)
    n = 16384
    S = 1e-4

    def state(pos):
        pm = np.zeros((n, 4), np.float32)
        pm[:, :3] = pos
        pm[:, 3] = 1.0 / n
        v = np.zeros((n, 4), np.float32)
        v[:, :3] = rng.normal(scale=1e-3, size=(n, 3))
        return nb.records_from_soa(pm, v)

    uniform = state(rng.uniform(-1, 1, (n, 3)))
    centres = rng.uniform(-1, 1, (n // 2, 3))
    pairs = state(np.concatenate([centres, centres + 1e-4]))   # deep chains: many more internal nodes
    outside = state(rng.uniform(1e5, 2e5, (n, 3)))              # no body in the root cube
    dt = 1e-3

    def fresh(rec, k):
        with bh_sim(theta=0.5, softening2=S) as f:
            f.init(rec)
            f.step(dt, k)
            out = rec.copy()
            f.write_back(out)
        return out

    with bh_sim(theta=0.5, softening2=S) as s:
        s.init(uniform)
        s.step(dt, 2)
        small = s.tree_stats()
        for rec, k in ((pairs, 2), (outside, 1), (uniform, 2)):
            s.init(rec)
            s.step(dt, k)
            out = rec.copy()
            s.write_back(out)
            ref = fresh(rec, k)
            for f in ("position", "velocity", "forces"):
                assert np.array_equal(out[f], ref[f]), f
            if rec is pairs:
                assert s.tree_stats()["internal"] > 2 * small["internal"]


def test_launches_per_step():
    """One launch per phase: a plain Barnes-Hut step is at most 20 kernel
    launches (keys with histograms, sort plan, one per radix pass, gather,
    positions scan, emit, link, child-count scan, place, mass, traversal,
    kick-drift)."""
    import ctypes
    pm, v = nb.seed_disk(8, 50000)
    with bh_sim(theta=0.5) as s:
        s.init_soa(pm, v)
        s.step(5e-4, 1)
        s.synchronize()
        a, b = ctypes.c_uint64(0), ctypes.c_uint64(0)
        nb.lib().nb_launch_count(s.handle, ctypes.byref(a))
        s.step(5e-4, 3)
        s.synchronize()
        nb.lib().nb_launch_count(s.handle, ctypes.byref(b))
    assert (b.value - a.value) / 3 <= 20
