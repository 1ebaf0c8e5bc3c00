"""GPU parity of the direct-sum path (K1 force + K7 kick-drift) against the
CPU oracle (restated BruteForceCPU) and the FP64 oracle.

Tolerances: forces within 1e-5 relative L2 error of the oracle; positions and
velocities after 100 steps within 1e-5 relative L2 error.
"""
import os

import numpy as np
import pytest

import nbody_gb300 as nb
from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden", "nbody_small.npz")
FORCE_TOL = 1e-5


def direct_sim(**kw):
    return nb.NBodySim(kind=nb.SIM_BRUTE_FORCE, **kw)


def test_golden_plummer256_forces():
    g = np.load(GOLD)
    with direct_sim() as s:
        s.init_soa(g["plummer256_pos_mass"], g["plummer256_vel"])
        F = s.compute_forces()
    assert O.rel_l2(F, g["plummer256_direct_forces"]) < FORCE_TOL


def test_golden_plummer256_ten_steps():
    g = np.load(GOLD)
    with direct_sim() as s:
        s.init_soa(g["plummer256_pos_mass"], g["plummer256_vel"])
        s.step(1e-3, 10)
        pos, vel, _ = s.read_state()
    assert O.rel_l2(pos, g["plummer256_direct_10_pos"]) < FORCE_TOL
    assert O.rel_l2(vel, g["plummer256_direct_10_vel"]) < FORCE_TOL


@pytest.mark.parametrize("n", [4096, 5000])
def test_forces_match_oracle_plummer(n):
    pm, v = nb.seed_plummer(1, n)
    rec = nb.records_from_soa(pm, v)
    F_ref = O.direct_forces(rec, G=1.0, S=1e-4)
    with direct_sim() as s:
        s.init(rec)
        F = s.compute_forces()
        F64 = s.fp64_forces(np.arange(n))
        assert s.last_interactions() == n * (n - 1)
    assert O.rel_l2(F, F_ref) < FORCE_TOL
    assert O.rel_l2(F, F64) < FORCE_TOL


def test_plummer_law_matches_oracle():
    pm, v = nb.seed_plummer(2, 3000)
    rec = nb.records_from_soa(pm, v)
    F_ref = O.direct_forces(rec, G=1.0, S=1e-4, law=1)
    with direct_sim(law=nb.LAW_PLUMMER) as s:
        s.init(rec)
        F = s.compute_forces()
    assert O.rel_l2(F, F_ref) < FORCE_TOL


def test_g_and_softening_parameters():
    pm, v = nb.seed_plummer(3, 2048)
    rec = nb.records_from_soa(pm, v)
    F_ref = O.direct_forces(rec, G=6.5, S=0.01)
    with direct_sim(G=6.5, softening2=0.01) as s:
        s.init(rec)
        F = s.compute_forces()
    assert O.rel_l2(F, F_ref) < FORCE_TOL


def test_hundred_steps_config1_parity():
    """Plummer N=4096, eps=0.01, dt=1e-3, 100 steps: forces, final state, drift."""
    n, dt, steps = 4096, 1e-3, 100
    pm, v = nb.seed_plummer(2024, n)
    rec = nb.records_from_soa(pm, v)
    ref = O.direct_step(rec, dt, steps, G=1.0, S=1e-4)
    with direct_sim() as s:
        s.init(rec)
        e0 = s.diagnostics(half_kick_dt=0.0)
        s.step(dt, steps)
        out = rec.copy()
        s.write_back(out)
        e1 = s.diagnostics(half_kick_dt=0.5 * dt)
    assert O.rel_l2(out["position"], ref["position"]) < FORCE_TOL
    assert O.rel_l2(out["velocity"], ref["velocity"]) < FORCE_TOL
    assert np.all(out["forces"] == 0.0)                 # BruteForceCPU zeroes Forces after Update
    np.testing.assert_array_equal(out["colour"], rec["colour"])
    drift = abs(e1["total"] - e0["total"]) / abs(e0["total"])
    assert drift < 1e-3, drift


def test_initial_forces_are_added_like_reference():
    pm, v = nb.seed_plummer(5, 1024)
    rec = nb.records_from_soa(pm, v)
    rec["forces"][:, 0] = 1e-3 * rec["mass"]
    ref = O.direct_step(rec, 1e-3, 1, G=1.0, S=1e-4)
    with direct_sim() as s:
        s.init(rec)
        s.step(1e-3, 1)
        out = rec.copy()
        s.write_back(out)
    assert O.rel_l2(out["velocity"], ref["velocity"]) < FORCE_TOL


def test_small_counts():
    with direct_sim(softening2=0.0) as s:
        rec = np.zeros(1, nb.PARTICLE_DTYPE)
        rec["mass"] = 1.0
        rec["velocity"] = [[1.0, 0, 0]]
        s.init(rec)
        s.step(0.5, 2)
        out = rec.copy()
        s.write_back(out)
        np.testing.assert_allclose(out["position"][0], [1.0, 0, 0], rtol=1e-7)
        rec = np.zeros(2, nb.PARTICLE_DTYPE)
        rec["position"] = [[0, 0, 0], [1, 0, 0]]
        rec["mass"] = [2.0, 3.0]
        s.init(rec)
        F = s.compute_forces()
        np.testing.assert_allclose(F, [[6, 0, 0], [-6, 0, 0]], rtol=1e-6)


def test_bounded_wait_runs_out_and_handle_recovers():
    """The force kernel's waits for its source tiles are bounded.  With the
    budget lowered to zero polls every block gives up at its first tile: the
    in-flight copies are still waited for, the step is abandoned with the
    state unchanged, and the next synchronisation reports NB_ETIMEOUT.  With
    the budget restored the same handle steps to the oracle's result."""
    pm, v = nb.seed_plummer(21, 65536)
    rec = nb.records_from_soa(pm, v)
    with direct_sim() as s:
        s.init(rec)
        assert s.get_tune("wait_polls") == 1 << 22
        s.tune("wait_polls", 0)
        s.step(1e-3, 1)
        with pytest.raises(nb.NBodyError) as ei:
            s.synchronize()
        assert ei.value.code == nb.NB_ETIMEOUT
        s.synchronize()                      # the error word was cleared by the report
        out = rec.copy()
        s.write_back(out)
        np.testing.assert_array_equal(out["position"], rec["position"])
        np.testing.assert_array_equal(out["velocity"], rec["velocity"])
        s.tune("wait_polls", 1 << 22)
        s.step(1e-3, 1)
        s.synchronize()
        s.write_back(out)
    # one kick from the initial state: v1 - v0 = F / m dt on sampled bodies
    sub = np.arange(0, 65536, 64)
    F = O.direct_forces_subset(rec, sub.astype(np.int32), G=1.0, S=1e-4)
    dv = out["velocity"][sub] - rec["velocity"][sub]
    dt = float(np.float32(1e-3))
    assert O.rel_l2(dv, F / rec["mass"][sub, None] * dt) < FORCE_TOL


def test_nonfinite_input_rejected_and_handle_reusable():
    rec = nb.records_from_soa(*nb.seed_plummer(6, 100))
    bad = rec.copy()
    bad["position"][17, 1] = np.nan
    with direct_sim() as s:
        with pytest.raises(nb.NBodyError) as ei:
            s.init(bad)
        assert ei.value.code == nb.NB_EINVAL
        s.init(rec)
        s.step(1e-3, 1)
        s.synchronize()


def test_fp64_oracle_gpu_matches_cpu():
    pm, v = nb.seed_plummer(8, 3000)
    targets = np.arange(0, 3000, 7)
    with direct_sim() as s:
        s.init_soa(pm, v)
        F64 = s.fp64_forces(targets)
    ref = O.fp64_forces(pm[:, :3].astype(np.float64), pm[:, 3].astype(np.float64), targets, G=1.0, S=1e-4)
    assert O.rel_l2(F64, ref) < 1e-13


def test_diagnostics_match_cpu_fp64():
    pm, v = nb.seed_plummer(9, 2000)
    with direct_sim() as s:
        s.init_soa(pm, v)
        d = s.diagnostics()
    ref = O.fp64_diagnostics(pm[:, :3], v[:, :3], pm[:, 3], G=1.0, S=1e-4)
    assert abs(d["kinetic"] - ref["kinetic"]) < 1e-12 * abs(ref["kinetic"])
    assert abs(d["potential"] - ref["potential"]) < 1e-6 * abs(ref["potential"])
    np.testing.assert_allclose(d["momentum"], ref["momentum"], atol=1e-12)
    np.testing.assert_allclose(d["angular_momentum"], ref["angular_momentum"], atol=1e-12)


def test_collision_forces_vs_fp64_sampled():
    n = 32768
    pm, v = nb.seed_collision(3, n)
    rng = np.random.default_rng(0)
    targets = np.sort(rng.choice(n, 2048, replace=False))
    with direct_sim() as s:
        s.init_soa(pm, v)
        F = s.compute_forces()
        F64 = s.fp64_forces(targets)
    assert O.rel_l2(F[targets], F64) < FORCE_TOL


def test_uncompensated_flag_runs():
    pm, v = nb.seed_plummer(10, 4096)
    with direct_sim(flags=nb.FLAG_NO_COMPENSATION) as s:
        s.init_soa(pm, v)
        F = s.compute_forces()
        F64 = s.fp64_forces(np.arange(4096))
    assert O.rel_l2(F, F64) < 1e-4


def test_render_vertices_headless():
    pm, v = nb.seed_plummer(12, 777)
    col = np.tile(np.array([[0.2, 0.4, 0.6, 1.0]], np.float32), (777, 1))
    with direct_sim() as s:
        s.init_soa(pm, v)
        rv = s.render_vertices(col, 2.0)
    np.testing.assert_array_equal(rv["position"], pm[:, :3])
    np.testing.assert_array_equal(rv["colour"], col)
    assert np.all(rv["scale"] == 2.0)


def test_full_size_config3_properties():
    """N = 262,144 (two Plummer spheres on a parabolic orbit, eps = 0.01):
    forces within 1e-5 of the FP64 direct sum on sampled targets, Newton's third
    law (net force ~ 0 against the sum of magnitudes) and the energy change of
    a step within the integrator's own error, properties that need no CPU run
    of 6.9e10 interactions."""
    n = 262144
    pm, v = nb.seed_collision(1234, n)
    rng = np.random.default_rng(7)
    targets = np.sort(rng.choice(n, 2048, replace=False)).astype(np.int32)
    with direct_sim(softening2=1e-4) as s:
        s.init_soa(pm, v)
        F = s.compute_forces()
        F64 = s.fp64_forces(targets)
        assert O.rel_l2(F[targets], F64) < FORCE_TOL
        net = np.abs(F.sum(axis=0)).max()          # F is the force m * a on each body
        scale = np.linalg.norm(F, axis=1).sum()
        assert net < 1e-6 * scale, (net, scale)
        # the reference's kick-drift (symplectic Euler) changes the energy by
        # O(dt) per step: 1.05e-5 of it here at dt = 1e-3; a broken force or
        # update would be off by orders of magnitude
        e0 = s.diagnostics(0.0)["total"]
        s.step(1e-3, 1)
        e1 = s.diagnostics(0.5e-3)["total"]
        assert abs(e1 - e0) < 1e-4 * abs(e0), (e0, e1)
