"""The reference's seeders run on the GPU (nb_init_seeded): the same bodies as
the host restatement (nb_seed_reference, up to the last bits of the device's
math functions), and a simulator seeded on the GPU steps exactly like one
initialised from those records."""
import numpy as np
import pytest

import nbody_gb300 as nb

pytestmark = pytest.mark.gpu

REF = dict(G=6.674e-11, softening2=10.0, pos_scale=20 * 1.15e12, theta=0.8)


@pytest.mark.parametrize("seeder", [nb.SEEDER_RANDOM, nb.SEEDER_GALAXY, nb.SEEDER_STAR_SYSTEM])
def test_gpu_seeder_matches_host_restatement(seeder):
    n = 6000
    host = nb.seed_reference(seeder, 21, n)
    with nb.NBodySim(nb.SIM_BARNES_HUT, **REF) as s:
        dev = s.init_seeded(seeder, 21, n)
        assert s.n == n
    for f in ("position", "velocity", "mass", "colour", "original_colour"):
        np.testing.assert_allclose(dev[f], host[f], rtol=2e-6, atol=1e-6 * np.abs(host[f]).max(), err_msg=f)
    assert np.all(dev["forces"] == 0)


def test_gpu_seeded_state_steps_like_uploaded_records():
    n = 4000
    with nb.NBodySim(nb.SIM_BARNES_HUT, **REF) as a, nb.NBodySim(nb.SIM_BARNES_HUT, **REF) as b:
        recs = a.init_seeded(nb.SEEDER_STAR_SYSTEM, 5, n)
        b.init(recs)
        ra, rb = recs.copy(), recs.copy()
        for _ in range(3):
            a.update(0.02 / 60, ra)
            b.update(0.02 / 60, rb)
        assert ra.tobytes() == rb.tobytes()
        assert not np.array_equal(ra["position"], recs["position"])


def test_gpu_seeder_rejects_bad_arguments():
    with nb.NBodySim(nb.SIM_BARNES_HUT) as s:
        with pytest.raises(nb.NBodyError):
            s.init_seeded(5, 0, 10)
        with pytest.raises(nb.NBodyError):
            s.init_seeded(nb.SEEDER_RANDOM, 0, 10, scale=-1.0)


@pytest.mark.parametrize("model,seed,n", [(0, 31, 70000), (0, 32, 3001), (1, 33, 20000), (2, 34, 16384)])
def test_device_generated_galaxy_matches_host_generator(model, seed, n):
    """The workload galaxies generated on the device (nb_batch_add_generated,
    what the served form does at admission) against the host generator
    (nb_seed_*): equal masses; positions and velocities equal up to the
    rounding of the device math functions and of the centre-of-mass sum (a
    float ulp or two on a few bodies)."""
    host = {0: nb.seed_disk, 1: nb.seed_plummer, 2: nb.seed_collision}[model](seed, n)
    with nb.NBodyBatch(bh_threshold=1 << 30) as b:   # direct-sum member: no reordering
        g = b.add_generated(model, seed, n)
        b.commit()
        dev = b.read(g)
    np.testing.assert_array_equal(dev[0][:, 3], host[0][:, 3])          # masses
    for d, h in ((dev[0][:, :3], host[0][:, :3]), (dev[1][:, :3], host[1][:, :3])):
        scale = np.abs(h).max()
        assert np.abs(d - h).max() <= 1e-6 * scale
        assert np.linalg.norm(d - h) <= 1e-7 * np.linalg.norm(h)
        assert np.mean(np.any(d != h, axis=1)) < 0.05
    # the same galaxy again: generation on the device is deterministic
    with nb.NBodyBatch(bh_threshold=1 << 30) as b:
        b.add_generated(2, 99, 1000)            # another galaxy first: a different place in the arrays
        g = b.add_generated(model, seed, n)
        b.commit()
        again = b.read(g)
    np.testing.assert_array_equal(again[0], dev[0])
    np.testing.assert_array_equal(again[1], dev[1])


def test_device_generated_galaxy_rejects_bad_arguments():
    with nb.NBodyBatch() as b:
        with pytest.raises(nb.NBodyError):
            b.add_generated(3, 1, 1000)
        with pytest.raises(nb.NBodyError):
            b.add_generated(0, 1, 1)
