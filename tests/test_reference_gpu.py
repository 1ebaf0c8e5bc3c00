"""GPU path against vectors generated by the reference's own CPU code.

tests/golden/reference_small.npz was made by the reference's src/Sim/Octree.cpp,
BarnesHut.cpp and BruteForceCPU.cpp, compiled unmodified (make_golden.py), at
the reference's constants (G = 6.674e-11, S = 10, drift divisor 2.3e13, root
cube +-4000).  The octree the GPU builds must be the reference's node for node
(every non-empty node: level, octant path, NumParticles, TotalMass,
CentreOfMass, side, TopLeft, the body of each one-body leaf); its forces and
one Update step must agree within 1e-5 relative L2 error for Barnes-Hut (the
decisions are the reference's, only FP32 against FP64 summation differs) and
1e-5 for direct sum.
"""
import os

import numpy as np
import pytest

import nbody_gb300 as nb

pytestmark = pytest.mark.gpu
REF_GOLD = os.path.join(os.path.dirname(__file__), "golden", "reference_small.npz")
SMALL_GOLD = os.path.join(os.path.dirname(__file__), "golden", "nbody_small.npz")
TOL = 1e-5


def rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))


def ref_params(g, **kw):
    G, S, scale = (float(x) for x in g["meta"][:3])
    return dict(G=G, softening2=S, pos_scale=scale, law=nb.LAW_REFERENCE, **kw)


def assert_gpu_tree_is_reference(sim, g, prefix):
    """Non-empty reference nodes against the GPU's node export."""
    r = {k[len(prefix):]: g[k] for k in g.files if k.startswith(prefix)}
    ne = r["count"] > 0
    rc = (np.uint64(1) << (np.uint64(3) * r["level"][ne].astype(np.uint64))) | r["prefix"][ne]
    nodes = sim.tree_nodes()
    gc = (np.uint64(1) << (np.uint64(3) * nodes["level"].astype(np.uint64))) | nodes["prefix"]
    ri, gi = np.argsort(rc), np.argsort(gc)
    np.testing.assert_array_equal(rc[ri], gc[gi])
    for f in ("level", "count", "mass", "side"):
        np.testing.assert_array_equal(r[f][ne][ri], nodes[f][gi], err_msg=f)
    np.testing.assert_array_equal(r["com"][ne][ri].view(np.uint32), nodes["com"][gi].view(np.uint32))
    np.testing.assert_array_equal(r["lo"][ne][ri], nodes["lo"][gi])
    single = r["body"][ne][ri] >= 0
    np.testing.assert_array_equal(r["body"][ne][ri][single], nodes["body"][gi][single])
    internal_ref = r["is_leaf"][ne][ri] == 0
    np.testing.assert_array_equal(internal_ref, nodes["first_child"][gi] >= 0)


def test_octree_is_the_reference_octree_galaxy():
    g = np.load(REF_GOLD)
    with nb.NBodySim(kind=nb.SIM_BARNES_HUT, **ref_params(g, theta=0.5)) as s:
        s.init(g["galaxy_records"])
        s.compute_forces()
        assert_gpu_tree_is_reference(s, g, "galaxy_node_")


def test_octree_is_the_reference_octree_disk512():
    """The 512-body disk at the workloads' N-body units (the tree does not
    depend on G or S)."""
    g = np.load(REF_GOLD)
    s0 = np.load(SMALL_GOLD)
    with nb.NBodySim(kind=nb.SIM_BARNES_HUT, theta=0.5, softening2=0.005 ** 2) as s:
        s.init_soa(s0["disk512_pos_mass"], s0["disk512_vel"])
        s.compute_forces()
        assert_gpu_tree_is_reference(s, g, "disk512_node_")


@pytest.mark.parametrize("theta,key", [(0.5, "galaxy_forces_t05"), (1.0, "galaxy_forces_t10")])
def test_barnes_hut_forces_vs_reference(theta, key):
    g = np.load(REF_GOLD)
    with nb.NBodySim(kind=nb.SIM_BARNES_HUT, **ref_params(g, theta=theta)) as s:
        s.init(g["galaxy_records"])
        F = s.compute_forces()
    assert rel_l2(F, g[key]) < TOL


def test_barnes_hut_update_vs_reference():
    """One BarnesHut::Update: forces assigned, v += F/m dt, x += v dt / 2.3e13."""
    g = np.load(REF_GOLD)
    dt = float(g["meta"][3])
    rec = g["galaxy_records"].copy()
    with nb.NBodySim(kind=nb.SIM_BARNES_HUT, **ref_params(g, theta=0.5)) as s:
        s.init(rec)
        s.update(dt, rec)
    ref = g["galaxy_bh_update"]
    assert rel_l2(rec["forces"], ref["forces"]) < TOL
    assert rel_l2(rec["velocity"] - g["galaxy_records"]["velocity"],
                  ref["velocity"] - g["galaxy_records"]["velocity"]) < TOL
    assert rel_l2(rec["position"], ref["position"]) < TOL


def test_brute_force_two_updates_vs_reference():
    """Two BruteForceCPU::Update: forces accumulated, kick-drift, forces zeroed."""
    g = np.load(REF_GOLD)
    dt = float(g["meta"][3])
    rec = g["random_records"].copy()
    with nb.NBodySim(kind=nb.SIM_BRUTE_FORCE, **ref_params(g)) as s:
        s.init(rec)
        s.step(dt, 2)
        s.write_back(rec)
    ref = g["random_bf_update2"]
    assert np.all(rec["forces"] == 0) and np.all(ref["forces"] == 0)
    dv, dv_ref = rec["velocity"] - g["random_records"]["velocity"], ref["velocity"] - g["random_records"]["velocity"]
    assert rel_l2(dv, dv_ref) < TOL
    assert rel_l2(rec["position"], ref["position"]) < TOL


def test_heavy_masses_self_pair_stays_zero():
    """Masses of the reference's seeders (1e20..1e30) with its constants: the
    direct sum's self pair must add exactly zero, not inf * 0 = NaN, in the
    plain path and in the batched form's direct-sum members; the batched
    form's Barnes-Hut members (float quadrupoles) refuse such a state."""
    g = np.load(REF_GOLD)
    rec = g["random_records"]
    assert rec["mass"].max() > 1e29
    with nb.NBodySim(kind=nb.SIM_BRUTE_FORCE, **ref_params(g)) as s:
        s.init(rec)
        F = s.compute_forces()
    assert np.all(np.isfinite(F))
    from oracle import oracle as O
    G, S = (float(x) for x in g["meta"][:2])
    assert rel_l2(F, O.direct_forces(rec, G=G, S=S)) < TOL
    pm = np.zeros((len(rec), 4), np.float32)
    pm[:, :3] = rec["position"]
    pm[:, 3] = rec["mass"]
    v = np.zeros_like(pm)
    batch = dict(bh_threshold=1000, bh_theta=0.3, G=G, softening2=S, pos_scale=float(g["meta"][2]))
    with nb.NBodyBatch(**batch) as b:
        b.add(pm[:900], v[:900])          # a direct-sum member
        b.commit()
        F = b.forces(0)
    assert np.all(np.isfinite(F))
    assert rel_l2(F, O.direct_forces(rec[:900], G=G, S=S)) < TOL
    # a Barnes-Hut member's float quadrupoles cannot hold such masses: refused, not NaN
    with nb.NBodyBatch(**batch) as b:
        b.add(pm, v)
        with pytest.raises(nb.NBodyError) as ei:
            b.commit()
        assert ei.value.code == nb.NB_ENOTSUP
