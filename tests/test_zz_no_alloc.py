"""The allocation-free direct-sum entry point, nb_direct_accel_noalloc.

Some callers cannot allocate device memory while they step (a render loop
held to a fixed memory budget, a host whose buffers come from its own
allocator, a thread that must not stall on cudaFree).  This entry point takes
their device buffers and keeps its working memory in a fixed array inside the
library.  The test calls it through the C-ABI twice in a row -- a large input
first, then a smaller one, so stale contents of the shared array would show
-- and compares each result with the handle path (nb_compute_forces) within
the direct-sum tolerance.  It runs alone or after the other tests.
"""
import ctypes

import numpy as np
import pytest

import nbody_gb300 as nb

pytestmark = pytest.mark.gpu
FORCE_TOL = 1e-5


def _reference_accel(pm, v, law, softening2):
    with nb.NBodySim(kind=nb.SIM_BRUTE_FORCE, law=law, softening2=softening2) as s:
        s.init_soa(pm, v)
        F = s.compute_forces()
    return F / pm[:, 3:4].astype(np.float64)


def test_noalloc_matches_handle_path_on_two_calls():
    import torch

    L = nb.lib()
    fn = L.nb_direct_accel_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_double, ctypes.c_double,
                   ctypes.c_int, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    # the maximum size first, then a smaller input on the same shared array
    cases = [(nb.seed_plummer(21, 65536), nb.LAW_REFERENCE, 1e-4),
             (nb.seed_collision(22, 5000), nb.LAW_PLUMMER, 1e-4)]
    for (pm, v), law, s2 in cases:
        ref = _reference_accel(pm, v, law, s2)
        d_in = torch.from_numpy(pm).cuda()
        d_out = torch.full((pm.shape[0], 4), float("nan"), dtype=torch.float32, device="cuda")
        rc = fn(d_in.data_ptr(), pm.shape[0], d_out.data_ptr(), 1.0, s2, law, None)
        assert rc == nb.NB_OK
        torch.cuda.synchronize()
        acc = d_out.cpu().numpy()[:, :3].astype(np.float64)
        assert np.isfinite(acc).all()
        err = np.linalg.norm(acc - ref) / np.linalg.norm(ref)
        assert err < FORCE_TOL, err


def test_noalloc_rejects_sizes_beyond_the_maximum():
    import torch

    L = nb.lib()
    fn = L.nb_direct_accel_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_double, ctypes.c_double,
                   ctypes.c_int, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    buf = torch.zeros((16, 4), dtype=torch.float32, device="cuda")
    assert fn(buf.data_ptr(), 65537, buf.data_ptr(), 1.0, 1e-4, nb.LAW_REFERENCE, None) == nb.NB_EINVAL
    assert fn(buf.data_ptr(), 0, buf.data_ptr(), 1.0, 1e-4, nb.LAW_REFERENCE, None) == nb.NB_EINVAL


def test_noalloc_heavy_masses_then_light():
    """Masses like the reference's seeders' (up to 1e30, its constants): the
    self pair must stay exactly zero (no inf * 0 = NaN); the call after it,
    with N-body masses, matches the handle path again (the shared array's
    mass record starts from zero on every call)."""
    import torch

    L = nb.lib()
    fn = L.nb_direct_accel_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_double, ctypes.c_double,
                   ctypes.c_int, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    rec = nb.seed_reference(nb.SEEDER_RANDOM, 23, 3000)
    heavy = np.zeros((3000, 4), np.float32)
    heavy[:, :3] = rec["position"]
    heavy[:, 3] = rec["mass"]
    G, S = 6.674e-11, 10.0
    with nb.NBodySim(kind=nb.SIM_BRUTE_FORCE, G=G, softening2=S) as s:
        s.init_soa(heavy, np.zeros_like(heavy))
        ref_heavy = s.compute_forces() / heavy[:, 3:4].astype(np.float64)
    light = nb.seed_plummer(24, 4096)
    for pm, g, s2, ref in ((heavy, G, S, ref_heavy), (light[0], 1.0, 1e-4, _reference_accel(*light, 0, 1e-4))):
        d_in = torch.from_numpy(pm).cuda()
        d_out = torch.full((pm.shape[0], 4), float("nan"), dtype=torch.float32, device="cuda")
        assert fn(d_in.data_ptr(), pm.shape[0], d_out.data_ptr(), g, s2, nb.LAW_REFERENCE, None) == nb.NB_OK
        torch.cuda.synchronize()
        acc = d_out.cpu().numpy()[:, :3].astype(np.float64)
        assert np.isfinite(acc).all()
        assert np.linalg.norm(acc - ref) / np.linalg.norm(ref) < FORCE_TOL
