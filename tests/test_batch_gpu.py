"""GPU tests of the batched form (many galaxies per launch, CUDA-graph replay,
autotuner).  Barnes-Hut members are checked against the FP64 direct sum
(<= 1e-3 relative L2 force error, the batched form's parity), direct-sum
members against the plain direct path (<= 1e-5)."""
import numpy as np
import pytest

import nbody_gb300 as nb
from oracle import oracle as O

pytestmark = pytest.mark.gpu
BH_FP64_TOL = 1e-3
DIRECT_TOL = 1e-5
EPS2 = 1e-4


def galaxies():
    specs = [("plummer", 300, 1), ("disk", 1000, 2), ("plummer", 5000, 3), ("disk", 9000, 4),
             ("plummer", 20000, 5), ("disk", 30000, 6), ("plummer", 8191, 7), ("disk", 8192, 8)]
    out = []
    for model, n, seed in specs:
        pm, v = nb.seed_disk(seed, n, bulge_frac=0.0) if model == "disk" else nb.seed_plummer(seed, n)
        out.append((pm, v))
    return out


def fp64_forces(pm, v, targets):
    with nb.NBodySim(kind=nb.SIM_BRUTE_FORCE, softening2=EPS2) as s:
        s.init_soa(pm, v)
        return s.fp64_forces(targets)


def plain_direct_forces(pm, v):
    with nb.NBodySim(kind=nb.SIM_BRUTE_FORCE, softening2=EPS2) as s:
        s.init_soa(pm, v)
        return s.compute_forces()


def make_batch(gals, **tune):
    b = nb.NBodyBatch(bh_threshold=8192, bh_theta=0.6, softening2=EPS2)
    for pm, v in gals:
        b.add(pm, v)
    if tune:
        b.set_tuning(**tune)
    b.commit()
    return b


def test_batched_forces_error_bounds():
    gals = galaxies()
    with make_batch(gals) as b:
        info = b.info()
        assert info["galaxies"] == len(gals) and info["bodies"] == sum(pm.shape[0] for pm, _ in gals)
        for g, (pm, v) in enumerate(gals):
            F = b.forces(g)
            n = pm.shape[0]
            if n >= 8192:
                t = np.arange(0, n, max(1, n // 2048))
                err = O.rel_l2(F[t], fp64_forces(pm, v, t))
                assert err < BH_FP64_TOL, (g, n, err)
            else:
                err = O.rel_l2(F, plain_direct_forces(pm, v))
                assert err < DIRECT_TOL, (g, n, err)


@pytest.mark.parametrize("leaf", [8, 16, 32, 64])
def test_leaf_sizes_keep_error_bound(leaf):
    pm, v = nb.seed_plummer(11, 25000)
    with make_batch([(pm, v)], leaf_size=leaf) as b:
        F = b.forces(0)
    t = np.arange(0, 25000, 13)
    assert O.rel_l2(F[t], fp64_forces(pm, v, t)) < BH_FP64_TOL


def test_graph_replay_is_deterministic_and_matches_eager_forces():
    gals = galaxies()[:6]
    with make_batch(gals) as a, make_batch(gals) as b:
        a.step(1e-3, 4)
        b.step(1e-3, 2)
        b.step(1e-3, 2)
        for g in range(len(gals)):
            pa, va = a.read(g)
            pb, vb = b.read(g)
            np.testing.assert_array_equal(pa, pb)
            np.testing.assert_array_equal(va, vb)


def test_alone_equals_in_the_mix():
    gals = galaxies()
    with make_batch(gals) as mix:
        mix.step(1e-3, 3)
        for g in (1, 4):
            with make_batch([gals[g]]) as alone:
                alone.step(1e-3, 3)
                pa, va = alone.read(0)
            pm, vm = mix.read(g)
            np.testing.assert_array_equal(pa, pm)
            np.testing.assert_array_equal(va, vm)


def test_direct_members_track_plain_path_over_steps():
    pm, v = nb.seed_plummer(21, 3000)
    with make_batch([(pm, v)]) as b:
        b.step(1e-3, 10)
        pb, vb = b.read(0)
    with nb.NBodySim(kind=nb.SIM_BRUTE_FORCE, softening2=EPS2) as s:
        s.init_soa(pm, v)
        s.step(1e-3, 10)
        ps, vs, _ = s.read_state()
    assert O.rel_l2(pb[:, :3], ps) < DIRECT_TOL
    assert O.rel_l2(vb[:, :3], vs) < DIRECT_TOL


def test_bh_members_track_fp64_integration():
    """10 steps of a 12k-body disk: batched Barnes-Hut vs the direct sum."""
    pm, v = nb.seed_disk(22, 12000)
    with make_batch([(pm, v)]) as b:
        b.step(5e-4, 10)
        pb, vb = b.read(0)
    with nb.NBodySim(kind=nb.SIM_BRUTE_FORCE, softening2=EPS2) as s:
        s.init_soa(pm, v)
        s.step(5e-4, 10)
        ps, vs, _ = s.read_state()
    dv_b = vb[:, :3] - v[:, :3]
    dv_s = vs - v[:, :3]
    assert O.rel_l2(dv_b, dv_s) < BH_FP64_TOL


def test_autotune_picks_a_valid_tuning():
    gals = galaxies()
    with make_batch(gals) as b:
        b.autotune(1e-3, 2)
        t = b.tuning()
        assert t["leaf_size"] in (8, 16, 32, 64)
        assert t["direct_block"] * t["direct_ipt"] <= 256
        F = b.forces(5)
        pm, v = gals[5]
        idx = np.arange(0, pm.shape[0], 17)
        assert O.rel_l2(F[idx], fp64_forces(pm, v, idx)) < BH_FP64_TOL
