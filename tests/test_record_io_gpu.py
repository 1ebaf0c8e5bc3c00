"""The record boundary on the GPU: kernels that read and write the caller's
104-byte records in place (where the device addresses host memory) give the
same bytes as the staged copies, touch only Position / Velocity / Forces, and
work for pageable as well as pinned buffers."""
import ctypes

import numpy as np
import pytest

import nbody_gb300 as nb

pytestmark = pytest.mark.gpu


def run(kind, rec, flags, steps=3):
    out = rec.copy()
    with nb.NBodySim(kind=kind, softening2=1e-4, theta=0.5, flags=flags) as s:
        s.init(out)
        for _ in range(steps):
            s.update(1e-3, out)
    return out


@pytest.mark.parametrize("kind", [nb.SIM_BRUTE_FORCE, nb.SIM_BARNES_HUT])
def test_in_place_and_staged_records_agree(kind):
    pm, v = nb.seed_plummer(9, 5000)
    rec = nb.records_from_soa(pm, v)
    rec["colour"] = np.random.default_rng(2).random((5000, 4)).astype(np.float32)
    rec["_pad"] = 7.0
    direct = run(kind, rec, nb.FLAG_NONE)
    staged = run(kind, rec, nb.FLAG_STAGED_IO)
    assert direct.tobytes() == staged.tobytes()
    for f in ("colour", "original_colour", "_pad", "mass"):
        assert np.array_equal(direct[f], rec[f]), f
    assert not np.array_equal(direct["position"], rec["position"])


def test_pinned_records():
    import torch
    n = 4096
    pm, v = nb.seed_disk(3, n)
    rec = nb.records_from_soa(pm, v)
    pinned = torch.empty(n * nb.PARTICLE_DTYPE.itemsize, dtype=torch.uint8, pin_memory=True)
    host = np.frombuffer((ctypes.c_char * pinned.numel()).from_address(pinned.data_ptr()),
                         dtype=nb.PARTICLE_DTYPE, count=n)
    host[:] = rec
    with nb.NBodySim(kind=nb.SIM_BARNES_HUT, softening2=0.005 ** 2, theta=0.5) as s:
        s.init(host)
        s.update(5e-4, host)
    with nb.NBodySim(kind=nb.SIM_BARNES_HUT, softening2=0.005 ** 2, theta=0.5, flags=nb.FLAG_STAGED_IO) as s:
        want = rec.copy()
        s.init(want)
        s.update(5e-4, want)
    assert host.tobytes() == want.tobytes()
