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
