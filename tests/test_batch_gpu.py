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


def test_coincident_bodies_and_far_field():
    """A Plummer sphere with 150 bodies on one point: the coincident bodies end
    in a depth-cap bucket larger than a traversal group (cut into chunks, and
    summed body by body where it is opened); the far field's local expansion
    is on by default and off with eta = 0 and alpha = 0, both within the
    error bound."""
    pm, v = nb.seed_plummer(21, 20000)
    clump = np.tile(np.array([[0.3, -0.2, 0.1, pm[0, 3]]], np.float32), (150, 1))
    pm = np.concatenate([pm, clump]).astype(np.float32)
    v = np.concatenate([v, np.zeros((150, 4), np.float32)]).astype(np.float32)
    n = pm.shape[0]
    t = np.concatenate([np.arange(0, 20000, 37), np.arange(20000, n, 7)]).astype(np.int32)
    ref = fp64_forces(pm, v, t)
    with make_batch([(pm, v)]) as b:
        F_far = b.forces(0)
        b.set_far_field(0.0)
        b.set_far_accuracy(0.0)
        F_near = b.forces(0)
        assert b.info()["interactions"] > 0
    assert np.all(np.isfinite(F_far)) and np.all(np.isfinite(F_near))
    assert O.rel_l2(F_far[t], ref) < BH_FP64_TOL
    assert O.rel_l2(F_near[t], ref) < BH_FP64_TOL
    assert not np.array_equal(F_far, F_near)   # the expansion was used


def test_far_field_relative_rule():
    """A state's first evaluation takes the geometric far-field rule; later
    ones (accelerations known) the relative rule, which must differ from it
    and stay within the error bound at the workload's theta for galaxies of
    4,096 to 200,000 bodies.  alpha 0 keeps the geometric rule (the second
    evaluation then repeats the first bit for bit); bad values are refused."""
    for pm, v in (nb.seed_disk(91, 4096), nb.seed_plummer(77, 65536), nb.seed_disk(5, 200_000)):
        n = pm.shape[0]
        t = np.arange(0, n, max(1, n // 1024)).astype(np.int32)
        ref = fp64_forces(pm, v, t)
        with nb.NBodyBatch(bh_threshold=1024, bh_theta=0.5, softening2=EPS2) as b:
            b.add(pm, v)
            b.commit()
            F_geo = b.forces(0)
            F_rel = b.forces(0)
            assert not np.array_equal(F_geo, F_rel)
            assert O.rel_l2(F_geo[t], ref) < BH_FP64_TOL, n
            assert O.rel_l2(F_rel[t], ref) < BH_FP64_TOL, n
            b.set_far_accuracy(0.0)
            np.testing.assert_array_equal(b.forces(0), F_geo)
            for bad in ((-1.0, 0.5), (1e-4, 0.0), (1e-4, 1.0)):
                with pytest.raises(nb.NBodyError):
                    b.set_far_accuracy(*bad)


def test_ragged_galaxy_sizes():
    """Direct-sum members of 2, 3, 255, 256 and 257 bodies (padded to multiples
    of 256 in the layout) beside one Barnes-Hut member: each matches its own
    reference, so padding bodies add nothing and galaxies do not mix."""
    sizes = [2, 3, 255, 256, 257]
    gals = [nb.seed_plummer(40 + k, n) for k, n in enumerate(sizes)] + [nb.seed_plummer(49, 9000)]
    with make_batch(gals) as b:
        for g, (pm, v) in enumerate(gals):
            F = b.forces(g)
            n = pm.shape[0]
            if n >= 8192:
                t = np.arange(0, n, 7)
                assert O.rel_l2(F[t], fp64_forces(pm, v, t)) < BH_FP64_TOL
            else:
                assert O.rel_l2(F, plain_direct_forces(pm, v)) < DIRECT_TOL, (g, n)


def test_batch_without_galaxies_is_refused():
    b = nb.NBodyBatch(bh_threshold=8192, bh_theta=0.6, softening2=EPS2)
    with pytest.raises(nb.NBodyError):
        b.commit()
    b.close()


def test_full_size_config4_error_bounds():
    """The 512-galaxy batch of the batched workload (n log-uniform in
    [256, 65,536], Plummer or disk): every Barnes-Hut member within 1e-3 of
    the FP64 direct sum on sampled bodies, sampled direct members within 1e-5
    of the plain direct path."""
    import bench_forms
    gals = bench_forms.batch_galaxies(nb)
    with nb.NBodyBatch(bh_threshold=8192, bh_theta=0.6, softening2=EPS2) as b:
        for pm, v in gals:
            b.add(pm, v)
        b.commit()
        worst = 0.0
        direct_checked = 0
        for g, (pm, v) in enumerate(gals):
            n = pm.shape[0]
            if n >= 8192:
                t = np.arange(0, n, max(1, n // 128)).astype(np.int32)
                err = O.rel_l2(b.forces(g)[t], fp64_forces(pm, v, t))
                worst = max(worst, err)
                assert err < BH_FP64_TOL, (g, n, err)
            elif g % 16 == 0:
                assert O.rel_l2(b.forces(g), plain_direct_forces(pm, v)) < DIRECT_TOL, (g, n)
                direct_checked += 1
        assert direct_checked >= 10


def test_octree_outgrowing_its_arrays_is_resized_and_steps_rerun():
    """The batched octree's arrays are sized at commit (twice the counts then).
    A state written into the committed batch whose octree needs far more nodes
    (every body with a partner 1e-4 away: long chains of internal nodes) makes
    the steps on that tree hold -- state unchanged -- until the wait resizes
    the tree and runs them again: the result equals a batch committed with
    that state."""
    gals = [galaxies()[k] for k in (4, 5, 0)]   # two Barnes-Hut members, one direct-sum member
    pairs = []
    for pm, v in gals:
        n = len(pm)
        q = pm.copy()
        half = (n + 1) // 2
        q[half:, :3] = pm[: n - half, :3] + np.float32(1e-4)
        pairs.append((q, v.copy()))
    with make_batch(gals) as a:
        a.step(1e-3, 2)
        before = a.tree_stats()["internal"]
        a.write_state(np.concatenate([p for p, _ in pairs]), np.concatenate([w for _, w in pairs]))
        a.step(1e-3, 3)
        assert a.tree_stats()["internal"] > 2 * before
        with make_batch(pairs) as b:
            b.step(1e-3, 3)
            for g in range(len(gals)):
                pa, va = a.read(g)
                pb, vb = b.read(g)
                np.testing.assert_array_equal(pa, pb)
                np.testing.assert_array_equal(va, vb)
