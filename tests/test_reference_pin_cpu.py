"""The oracle pinned to the reference's own code.

oracle/ref/Makefile compiles the reference's src/Sim/Octree.cpp,
BarnesHut.cpp and BruteForceCPU.cpp unmodified (type-only stand-ins for the
DirectXTK / Direct3D headers they include), and oracle/reference_build.py
drives them.  Where the reference sources are present, these tests run the
reference's recursion (Octree::Add / Split / CalculateMass / CalculateForce)
and its two CPU simulators' Update on the same inputs as the oracle and ask
for bit-identical results: every octree node, every force, every updated
record.  Everywhere, the oracle must reproduce the committed vectors that the
reference build generated (tests/golden/reference_small.npz).

The oracle's documented deviations are shown here too: the reference's
thread-pool remainder slice leaves tail bodies with stale forces (the oracle
computes them), and the reference splits without a depth limit (the oracle
stops at 21 levels and keeps a bucket).
"""
import os

import numpy as np
import pytest

import nbody_gb300 as nb
from oracle import oracle as O
from oracle import reference_build as R

REF_GOLD = os.path.join(os.path.dirname(__file__), "golden", "reference_small.npz")
SMALL_GOLD = os.path.join(os.path.dirname(__file__), "golden", "nbody_small.npz")

needs_ref = pytest.mark.skipif(not R.available(), reason="reference sources not present on this machine")


def codes(level, prefix):
    return (np.uint64(1) << (np.uint64(3) * np.asarray(level, np.uint64))) | np.asarray(prefix, np.uint64)


def assert_oracle_tree_equals(ref_nodes: dict, ot: O.OracleTree):
    """Every node of the reference tree (all eight children of each split)
    against the oracle's arena, matched by (level, octant path)."""
    on = ot.nodes()
    rc = codes(ref_nodes["level"], ref_nodes["prefix"])
    oc = codes(on["level"], on["prefix"])
    ri, oi = np.argsort(rc), np.argsort(oc)
    np.testing.assert_array_equal(rc[ri], oc[oi])
    for f in ("count", "mass", "side", "body"):
        np.testing.assert_array_equal(ref_nodes[f][ri], on[f][oi], err_msg=f)
    np.testing.assert_array_equal(ref_nodes["is_leaf"][ri], on["is_leaf"][oi])
    np.testing.assert_array_equal(ref_nodes["com"][ri].view(np.uint32), on["com"][oi].view(np.uint32))
    np.testing.assert_array_equal(ref_nodes["lo"][ri], on["lo"][oi])
    assert ot.deeper_buckets() == 0


def ref_records(seeder, seed, n):
    r = nb.seed_reference(seeder, seed, n)
    r["mass"] = r["mass"].astype(np.float32).astype(np.float64)
    return r


# ---- the committed vectors (every machine) --------------------------------------

def test_oracle_reproduces_reference_vectors():
    g = np.load(REF_GOLD)
    G, S, scale, dt = (float(x) for x in g["meta"][:4])
    gal = g["galaxy_records"]
    t = O.OracleTree(gal)
    assert_oracle_tree_equals({k[len("galaxy_node_"):]: g[k] for k in g.files if k.startswith("galaxy_node_")}, t)
    for th, key in ((0.5, "galaxy_forces_t05"), (1.0, "galaxy_forces_t10")):
        F, _ = t.forces(G=G, S=S, theta=th)
        np.testing.assert_array_equal(F, g[key])
    t.close()
    up = O.bh_step(gal, dt, 1, G=G, S=S, theta=0.5, scale=scale)
    for f in ("position", "velocity", "forces"):
        np.testing.assert_array_equal(up[f], g["galaxy_bh_update"][f], err_msg=f)
    up = O.direct_step(g["random_records"], dt, 2, G=G, S=S, scale=scale)
    for f in ("position", "velocity", "forces"):
        np.testing.assert_array_equal(up[f], g["random_bf_update2"][f], err_msg=f)


def test_oracle_fixture_tree_is_the_reference_tree():
    """nbody_small.npz (made by the oracle at N-body units) holds the same
    octree as the reference builds for its 512-body disk."""
    s = np.load(SMALL_GOLD)
    g = np.load(REF_GOLD)
    t = O.OracleTree(O.particles_from_soa(s["disk512_pos_mass"], s["disk512_vel"]))
    assert_oracle_tree_equals({k[len("disk512_node_"):]: g[k] for k in g.files if k.startswith("disk512_node_")}, t)


# ---- live comparisons with the reference build ----------------------------------

@needs_ref
def test_fixture_is_current():
    """The committed vectors are what the reference build gives now."""
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "make_golden", os.path.join(os.path.dirname(__file__), "golden", "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    s = np.load(SMALL_GOLD)
    fresh = mg.reference_fixture(s["disk512_pos_mass"], s["disk512_vel"])
    g = np.load(REF_GOLD)
    assert sorted(fresh) == sorted(g.files)
    for k in g.files:
        if k == "meta":
            np.testing.assert_array_equal(fresh[k][:4], g[k][:4])
        else:
            np.testing.assert_array_equal(fresh[k], g[k], err_msg=k)


@needs_ref
@pytest.mark.parametrize("seeder,seed,n", [(nb.SEEDER_GALAXY, 7, 20000), (nb.SEEDER_RANDOM, 8, 7000),
                                           (nb.SEEDER_GALAXY, 9, 5000)])
def test_tree_and_forces_bit_exact(seeder, seed, n):
    rec = ref_records(seeder, seed, n)
    rt = R.RefOctree(rec)
    assert rt.max_depth() <= 21
    ot = O.OracleTree(rec)
    assert_oracle_tree_equals(rt.nodes(), ot)
    targets = np.arange(0, n, 3, dtype=np.int32)
    for th in (0.0, 0.5, 1.0, 2.0):
        Fr = rt.forces(targets, theta=th)
        Fo = ot.forces_subset(targets, G=R.G, S=R.S, theta=th)
        np.testing.assert_array_equal(Fo, Fr)


@needs_ref
def test_tree_bit_exact_at_nbody_units():
    """The workloads' galaxies (G = 1 units, positions of order 1) where the
    reference tree stays within 21 levels: same nodes; forces at the
    reference's constants."""
    compared = 0
    for pm, v in (nb.seed_plummer(4, 4096), nb.seed_disk(5, 2000), nb.seed_collision(6, 3000)):
        rec = O.particles_from_soa(pm, v)
        rt = R.RefOctree(rec)
        if rt.max_depth() > 21:
            continue
        ot = O.OracleTree(rec)
        assert_oracle_tree_equals(rt.nodes(), ot)
        np.testing.assert_array_equal(ot.forces(G=R.G, S=R.S, theta=0.5)[0], rt.forces(theta=0.5))
        compared += 1
    assert compared >= 2


@needs_ref
def test_edge_inputs_boundaries_dropped_bodies():
    """Bodies on cell boundaries, at the closed lower bound -4000, on the open
    upper bound +4000 (dropped but counted), far outside, and a first body
    outside the root cube (kept by the root until the second body arrives)."""
    pts = np.array([[1e5, 0, 0], [0, 0, 0], [-2000, -2000, -2000], [4000, 0, 0], [-4000, -4000, -4000],
                    [3999.0, 1, 1], [-3999.9, 3999.9, 0], [1000, 1000, 1000], [1000, -1000, 0.5],
                    [0.25, 0.5, 0.75], [-0.25, 0.5, -0.75]], np.float32)
    rng = np.random.default_rng(3)
    pts = np.concatenate([pts, rng.uniform(-3000, 3000, (40, 3)).astype(np.float32)])
    pm = np.zeros((len(pts), 4), np.float32)
    pm[:, :3] = pts
    pm[:, 3] = rng.uniform(1.0, 3.0, len(pts)).astype(np.float32)
    rec = O.particles_from_soa(pm, np.zeros_like(pm))
    rt, ot = R.RefOctree(rec), O.OracleTree(rec)
    assert_oracle_tree_equals(rt.nodes(), ot)
    np.testing.assert_array_equal(ot.forces(G=R.G, S=R.S, theta=0.5)[0], rt.forces(theta=0.5))
    # a lone body outside the cube: the root keeps it as its one body
    one = rec[:1].copy()
    rt1, ot1 = R.RefOctree(one), O.OracleTree(one)
    assert_oracle_tree_equals(rt1.nodes(), ot1)


@needs_ref
@pytest.mark.parametrize("steps", [1, 3])
def test_barnes_hut_update_bit_exact(steps):
    T = R.workers()
    rec = ref_records(nb.SEEDER_GALAXY, 12, T * 1000)
    a = R.bh_update(rec, 1.0, 0.5, steps)
    b = O.bh_step(rec, 1.0, steps, G=R.G, S=R.S, theta=0.5, scale=R.STAR_SYSTEM_SCALE)
    for f in ("position", "velocity", "forces"):
        np.testing.assert_array_equal(a[f], b[f], err_msg=f)


@needs_ref
def test_brute_force_update_bit_exact():
    T = R.workers()
    rec = ref_records(nb.SEEDER_RANDOM, 13, T * 200)
    a = R.bf_update(rec, 1.0, 2)
    b = O.direct_step(rec, 1.0, 2, G=R.G, S=R.S, scale=R.STAR_SYSTEM_SCALE)
    for f in ("position", "velocity", "forces"):
        np.testing.assert_array_equal(a[f], b[f], err_msg=f)


@needs_ref
def test_deviation_remainder_slice_leaves_tail_forces_stale():
    """BarnesHut::Update's caller thread recomputes [T, T + rem) instead of the
    tail (src/Sim/BarnesHut.cpp:70-77): the last rem bodies keep whatever
    force they had.  The oracle computes every body once."""
    T = R.workers()
    n = T * 300 + 5
    rec = ref_records(nb.SEEDER_GALAXY, 14, n)
    rec["forces"] = 12345.0
    a = R.bh_update(rec, 1.0, 0.5, 1)
    tail = slice(T * (n // T), n)
    assert np.all(a["forces"][tail] == 12345.0)
    assert not np.any(a["forces"][:T * (n // T)] == 12345.0)
    b = O.bh_step(rec, 1.0, 1, G=R.G, S=R.S, theta=0.5, scale=R.STAR_SYSTEM_SCALE)
    np.testing.assert_array_equal(a["forces"][:T * (n // T)], b["forces"][:T * (n // T)])
    assert not np.any(b["forces"][tail] == 12345.0)


def assert_same_above_cap(rt, ot):
    """Nodes down to the depth cap: same set, same counts."""
    rn, on = rt.nodes(), ot.nodes()
    keep = rn["level"] <= 21
    rc = codes(rn["level"][keep], rn["prefix"][keep])
    oc = codes(on["level"], on["prefix"])
    np.testing.assert_array_equal(np.sort(rc), np.sort(oc))
    np.testing.assert_array_equal(rn["count"][keep][np.argsort(rc)], on["count"][np.argsort(oc)])


@needs_ref
def test_deviation_depth_cap_star_system():
    """The StarSystem distribution puts bodies closer than a depth-21 cell:
    above the cap the trees agree node for node; forces agree to rounding."""
    rec = ref_records(nb.SEEDER_STAR_SYSTEM, 9, 2000)
    rt, ot = R.RefOctree(rec), O.OracleTree(rec)
    assert rt.max_depth() > 21
    assert_same_above_cap(rt, ot)
    t = np.arange(0, 2000, 2, dtype=np.int32)
    assert O.rel_l2(ot.forces_subset(t, G=R.G, S=R.S, theta=0.5), rt.forces(t, theta=0.5)) < 1e-6


@needs_ref
def test_deviation_depth_cap_bucket():
    """Two bodies closer than a depth-21 cell (8000 / 2^21 = 0.0038): the
    reference splits on below 21 levels, the oracle keeps one bucket.  Every
    node above the cap is the same; the force on a distant body agrees to
    rounding."""
    rng = np.random.default_rng(15)
    pts = rng.uniform(-100, 100, (200, 3)).astype(np.float32)
    pts[1] = pts[0] + np.float32(1e-4)
    pm = np.zeros((200, 4), np.float32)
    pm[:, :3] = pts
    pm[:, 3] = 1.0
    rec = O.particles_from_soa(pm, np.zeros_like(pm))
    rt, ot = R.RefOctree(rec), O.OracleTree(rec)
    assert rt.max_depth() > 21
    assert_same_above_cap(rt, ot)
    assert ot.deeper_buckets() == 1
    Fr = rt.forces(np.arange(2, 200, dtype=np.int32), theta=0.5)
    Fo = ot.forces_subset(np.arange(2, 200, dtype=np.int32), G=R.G, S=R.S, theta=0.5)
    assert O.rel_l2(Fo, Fr) < 1e-6
