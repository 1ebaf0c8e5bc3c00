"""C-ABI checks that need no GPU: the library loads, exports every symbol the
public headers declare, the ctypes structures match the C layout, and the
host-side seeders are deterministic."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

import nbody_gb300 as nb

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")
GOLD = os.path.join(os.path.dirname(__file__), "golden", "nbody_small.npz")


def declared_functions():
    names = set()
    for fn in os.listdir(INCLUDE):
        if not fn.endswith(".h"):
            continue
        text = open(os.path.join(INCLUDE, fn)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b(nb_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    L = nb.lib()
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_struct_layout_matches_c(tmp_path):
    src = tmp_path / "layout.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "nbody_gb300.h"\n'
        "int main(void){\n"
        'printf("%zu %zu %zu %zu %zu\\n", sizeof(nb_particle), offsetof(nb_particle, velocity),'
        " offsetof(nb_particle, forces), offsetof(nb_particle, mass), sizeof(nb_render_vertex));\n"
        'printf("%zu %zu %zu %zu\\n", sizeof(nb_params), offsetof(nb_params, stream), offsetof(nb_params, flags),'
        " sizeof(nb_diag));\n"
        'printf("%zu %zu %zu\\n", sizeof(nb_tree_node), offsetof(nb_tree_node, mass),'
        " offsetof(nb_tree_node, bucket_end));\n"
        "return 0;}\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-I", INCLUDE, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    vals = [int(x) for x in out]
    assert vals[:5] == [104, 48, 72, 96, 32]
    assert nb.PARTICLE_DTYPE.itemsize == 104 and nb.RENDER_DTYPE.itemsize == 32
    assert vals[5] == ctypes.sizeof(nb.nb_params)
    assert vals[6] == nb.nb_params.stream.offset
    assert vals[7] == nb.nb_params.flags.offset
    assert vals[8] == ctypes.sizeof(nb.nb_diag)
    d = nb.TREE_NODE_DTYPE
    assert vals[9:12] == [d.itemsize, d.fields["mass"][1], d.fields["bucket_end"][1]]


def test_default_params_translate_reference_constants():
    p = nb.default_params()
    assert p.kind == nb.SIM_BARNES_HUT      # SimulationState creates Barnes-Hut by default
    assert p.G == 1.0 and p.softening2 == 1e-4 and p.theta == 0.5
    assert p.bounds_half == 4000.0          # src/Sim/BarnesHut.cpp:14-21
    assert p.max_depth == 21 and p.leaf_size == 1


def test_sim_names_match_reference():
    L = nb.lib()
    assert L.nb_sim_name(0) == b"Brute Force CPU"
    assert L.nb_sim_name(1) == b"Brute Force GPU"
    assert L.nb_sim_name(2) == b"Barnes-Hut"
    assert L.nb_sim_name(7) == b"Unknown"


def test_create_rejects_bad_params():
    L = nb.lib()
    h = ctypes.c_void_p()
    for kw in (dict(max_depth=0), dict(max_depth=22), dict(leaf_size=0), dict(kind=5), dict(law=9),
               dict(softening2=-1.0), dict(pos_scale=0.0), dict(law=nb.LAW_PLUMMER, softening2=0.0)):
        p = nb.default_params(**kw)
        assert L.nb_create(ctypes.byref(p), ctypes.byref(h)) == nb.NB_EINVAL, kw
    assert L.nb_create(None, ctypes.byref(h)) == nb.NB_EINVAL


def test_null_handle_calls_fail_cleanly():
    L = nb.lib()
    assert L.nb_step(None, 0.1, 1) == nb.NB_EINVAL
    assert L.nb_destroy(None) == nb.NB_EINVAL
    assert L.nb_init_particles(None, None, 0) == nb.NB_EINVAL
    assert L.nb_last_error(None) == b"null handle"


def test_seeders_deterministic_and_centred():
    a = nb.seed_plummer(42, 3000)
    b = nb.seed_plummer(42, 3000)
    c = nb.seed_plummer(43, 3000)
    np.testing.assert_array_equal(a[0], b[0])
    assert not np.array_equal(a[0], c[0])
    for pm, v in (a, nb.seed_disk(1, 5000), nb.seed_collision(2, 4000)):
        m = pm[:, 3].astype(np.float64)
        com = (pm[:, :3] * m[:, None]).sum(0) / m.sum()
        p = (v[:, :3] * m[:, None]).sum(0)
        assert np.abs(com).max() < 1e-5
        assert np.abs(p).max() < 1e-5
        assert np.isfinite(pm).all() and np.isfinite(v).all()


def test_seeder_distributions():
    pm, v = nb.seed_plummer(7, 20000)
    r = np.linalg.norm(pm[:, :3], axis=1)
    # Plummer half-mass radius a / sqrt(2^(2/3) - 1) = 1.305 a
    assert abs(np.median(r) - 1.305) < 0.05
    assert np.isclose(pm[:, 3].sum(), 1.0, rtol=1e-5)
    # virial ratio of a Plummer sphere: 2K/|W| = 1 (W = -3 pi / 32 for G=M=a=1)
    K = 0.5 * (pm[:, 3] * (v[:, :3] ** 2).sum(1)).sum()
    assert abs(K / (3 * np.pi / 64) - 1.0) < 0.05
    pm, v = nb.seed_disk(3, 20000)
    m = pm[:, 3]
    nb_ = int(round(0.1 * 20000))
    assert np.isclose(m[:-nb_].sum(), 0.9, rtol=1e-4) and np.isclose(m[-nb_:].sum(), 0.1, rtol=1e-4)
    z = pm[:-nb_, 2]
    assert np.std(z) < 0.3
    R = np.linalg.norm(pm[:-nb_, :2], axis=1)
    assert abs(np.mean(R) - 2.0) < 0.1          # exponential disk: <R> = 2 rd
    pm, v = nb.seed_collision(4, 10000)
    left = pm[:5000, 0].mean()
    right = pm[5000:, 0].mean()
    assert abs((right - left) - 10.0) < 0.2


def test_seeders_match_golden_inputs():
    g = np.load(GOLD)
    pm, v = nb.seed_plummer(11, 256)
    np.testing.assert_array_equal(pm, g["plummer256_pos_mass"])
    np.testing.assert_array_equal(v, g["plummer256_vel"])
    pm, v = nb.seed_disk(5, 512)
    np.testing.assert_array_equal(pm, g["disk512_pos_mass"])


def test_server_rejects_jobs_that_can_never_fit():
    """Admission bounds checked at submission, before any device work: a job
    larger than the memory budget or than the batched form's galaxy limit
    (16 Mi bodies) is rejected (state -1) and never queued."""
    import nbody_serve as ns
    with ns.NBodyServer(memory_budget=640 * 10_000) as s:
        small = s.submit(1, 5_000, 10, 1e-3, 0)
        over_budget = s.submit(2, 20_000, 10, 1e-3, 0)
        assert s.status(small)["state"] == 0
        assert s.status(over_budget)["state"] == -1
    with ns.NBodyServer() as s:   # 120 GB budget: 110 M bodies fit it, not one batch's octree
        too_many = s.submit(3, 110 << 20, 10, 1e-3, 0)
        assert s.status(too_many)["state"] == -1
        largest = s.submit(4, 16 << 20, 10, 1e-3, 0)        # one galaxy's limit: queued
        over_galaxy = s.submit(5, (16 << 20) + 1, 10, 1e-3, 0)
        assert s.status(largest)["state"] == 0
        assert s.status(over_galaxy)["state"] == -1


def test_server_release_of_rejected_and_unknown_jobs():
    """A rejected job can be released (it never reaches the device); a queued
    job cannot; an unknown id is an error."""
    import nbody_gb300 as nb
    import nbody_serve as ns
    with ns.NBodyServer(memory_budget=640 * 10_000) as s:
        queued = s.submit(1, 5_000, 10, 1e-3, 0)
        rejected = s.submit(2, 20_000, 10, 1e-3, 0)
        s.release(rejected)
        with pytest.raises(nb.NBodyError):
            s.status(rejected)
        with pytest.raises(nb.NBodyError):
            s.release(queued)
        with pytest.raises(nb.NBodyError):
            s.release(12345)


def test_server_retries_a_failed_batch_build():
    """Host logic of the serving loop: when the batch cannot be built (here,
    on a machine without a usable GPU, nb_batch_create fails) the admitted job
    stays active with no steps done, and the next tick tries the build again
    instead of stepping a batch that does not hold the job."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("the batch builds on a machine with a GPU")
    import nbody_serve as ns
    with ns.NBodyServer() as s:
        j = s.submit(1, 1000, 10, 1e-3, 0)
        for _ in range(2):
            with pytest.raises(nb.NBodyError, match="nb_batch_create"):
                s.tick()
            st = s.status(j)
            assert st["state"] == 1 and st["steps_done"] == 0
