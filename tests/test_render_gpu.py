"""Render hand-off on the GPU: the vertex buffer filled in the kick-drift's
epilogue holds exactly the positions the step produced, with the attached
colours and scale, for both simulators; it follows every step and goes away
on re-initialisation."""
import numpy as np
import pytest

import nbody_gb300 as nb

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind", [nb.SIM_BRUTE_FORCE, nb.SIM_BARNES_HUT])
def test_vertices_follow_the_kick_drift(kind):
    pm, v = nb.seed_plummer(4, 3000)
    colour = np.random.default_rng(1).random((3000, 4)).astype(np.float32)
    with nb.NBodySim(kind=kind, softening2=1e-4, theta=0.5) as s:
        s.init_soa(pm, v)
        ptr = s.render_attach(colour, scale=2.5)
        assert ptr
        first = s.render_read()
        assert np.array_equal(first["position"], pm[:, :3])   # filled at attach time
        for k in range(3):
            s.step(1e-3, 1)
            got = s.render_read()
            want = s.render_vertices(colour, 2.5)   # separate kernel from the current state
            assert got.tobytes() == want.tobytes(), k
        assert not np.array_equal(got["position"], pm[:, :3])
        assert np.all(got["scale"] == np.float32(2.5))
        np.testing.assert_array_equal(got["colour"], colour)
        s.init_soa(pm, v)                                      # a new particle set drops the buffer
        with pytest.raises(nb.NBodyError):
            s.render_read()


def test_default_colour_and_detach():
    pm, v = nb.seed_plummer(5, 1000)
    with nb.NBodySim(kind=nb.SIM_BARNES_HUT, softening2=1e-4) as s:
        s.init_soa(pm, v)
        s.render_attach()
        s.step(1e-3, 2)
        got = s.render_read()
        assert np.all(got["colour"] == 1.0)
        s.render_detach()
        s.step(1e-3, 1)                                        # steps without a buffer still work
        with pytest.raises(nb.NBodyError):
            s.render_read()
