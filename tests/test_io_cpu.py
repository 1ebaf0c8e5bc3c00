""".nbody files, the reference's seeders, the C++ adapter and the headless
driver's host side -- all without a GPU.

Reference behaviour followed: .nbody = raw Particle records
(src/States/Simulation/SimulationState.cpp:229-277, 317-331), re-centred on
load; seeder distributions from src/Sim/RandomSeeder.cpp:12-40,
src/Sim/GalaxySeeder.cpp:43-144, src/Sim/StarSystemSeeder.cpp:17-55."""
import os
import subprocess

import numpy as np
import pytest

import nb_build
import nbody_gb300 as nb

AU, M = 1.15e12, 1000.0
SSS = 20 * AU


def test_file_round_trip_is_byte_exact(tmp_path):
    p = nb.seed_reference(nb.SEEDER_RANDOM, 5, 300)
    f = tmp_path / "a.nbody"
    nb.file_write(str(f), p)
    assert f.stat().st_size == 104 * 300
    assert f.read_bytes() == p.tobytes()
    q = nb.file_read(str(f), recentre=False)
    assert q.tobytes() == p.tobytes()


def test_file_read_recentres_like_the_loader(tmp_path):
    p = nb.seed_reference(nb.SEEDER_GALAXY, 9, 500)
    p["position"] += np.float32(37.5)
    f = tmp_path / "b.nbody"
    nb.file_write(str(f), p)
    q = nb.file_read(str(f))
    # the loader's arithmetic: long double total mass, double moment sums,
    # centre rounded to float, float subtraction
    Mtot = np.longdouble(0)
    c = [0.0, 0.0, 0.0]
    for r in p:
        Mtot += np.longdouble(r["mass"])
        for a in range(3):
            c[a] += float(r["position"][a]) * float(r["mass"])
    centre = np.array([np.float32(ca / float(Mtot)) for ca in c], np.float32)
    expect = (p["position"] - centre).astype(np.float32)
    assert np.array_equal(q["position"], expect)
    # everything but the position is untouched
    for k in ("velocity", "forces", "mass", "colour", "original_colour"):
        assert np.array_equal(q[k], p[k])


def test_file_read_ignores_trailing_partial_record(tmp_path):
    p = nb.seed_reference(nb.SEEDER_STAR_SYSTEM, 1, 3)
    f = tmp_path / "c.nbody"
    f.write_bytes(p.tobytes() + b"\x01" * 50)
    q = nb.file_read(str(f), recentre=False)
    assert q.shape[0] == 3 and q.tobytes() == p.tobytes()


def test_file_edge_cases(tmp_path):
    f = tmp_path / "empty.nbody"
    f.write_bytes(b"")
    assert nb.file_read(str(f)).shape[0] == 0
    with pytest.raises(nb.NBodyError):
        nb.file_read(str(tmp_path / "missing.nbody"))
    nb.file_write(str(tmp_path / "zero.nbody"), np.zeros(0, nb.PARTICLE_DTYPE))
    assert (tmp_path / "zero.nbody").stat().st_size == 0


def test_star_system_seeder_distribution():
    p = nb.seed_reference(nb.SEEDER_STAR_SYSTEM, 3, 2000)
    assert np.all(p[0]["position"] == 0) and p[0]["mass"] == 1e30
    q = p[1:]
    assert np.all(q["position"][:, :2] == 0)
    z = q["position"][:, 2]
    assert z.min() >= np.float32(4 * AU * M / SSS) * (1 - 1e-6)
    assert z.max() <= np.float32(7 * AU * M / SSS) * (1 + 1e-6)
    assert np.all((q["velocity"][:, 0] >= AU * M) & (q["velocity"][:, 0] <= 5 * AU * M))
    assert np.all((q["velocity"][:, 1] >= AU * M / 20) & (q["velocity"][:, 1] <= 5 * AU * M / 20))
    assert np.all(q["velocity"][:, 2] == 0)
    assert np.all((q["mass"] >= 1e10) & (q["mass"] <= 1e26))
    assert np.all(p["colour"] == p["original_colour"])


def test_random_seeder_distribution():
    p = nb.seed_reference(nb.SEEDER_RANDOM, 4, 3000, scale=2.0)
    assert np.abs(p["position"]).max() <= 250.0
    speed = np.linalg.norm(p["velocity"], axis=1)
    assert np.allclose(speed, 1e16, rtol=1e-5)
    assert np.all((p["mass"] >= 1e20) & (p["mass"] <= 1e30))
    assert np.all((p["colour"][:, :3] >= 0.2) & (p["colour"][:, :3] <= 1.0))


def test_galaxy_seeder_split_and_determinism():
    n = 6000
    p = nb.seed_reference(nb.SEEDER_GALAXY, 7, n)
    arms = 2 * 60 * int(n * 0.4 / 60)
    assert np.all(p["mass"][:arms] == 1e20)
    assert np.all((p["mass"][arms:] >= 1e28) & (p["mass"][arms:] <= 1e30))
    # disk bodies lie within radius 720 of the centre (rotation preserves length)
    r = np.linalg.norm(p["position"][arms:].astype(np.float64), axis=1)
    assert np.percentile(r, 50) < 720.0
    assert p.tobytes() == nb.seed_reference(nb.SEEDER_GALAXY, 7, n).tobytes()
    assert p.tobytes() != nb.seed_reference(nb.SEEDER_GALAXY, 8, n).tobytes()


def test_bad_seeder_arguments():
    with pytest.raises(nb.NBodyError):
        nb.seed_reference(7, 0, 10)
    with pytest.raises(nb.NBodyError):
        nb.seed_reference(nb.SEEDER_RANDOM, 0, 10, scale=0.0)


def test_cpp_adapter_header_compiles(tmp_path):
    src = tmp_path / "use.cpp"
    src.write_text(
        '#include "cuda_nbody_sim.hpp"\n'
        "int main() {\n"
        "  std::vector<nbgb::Particle> v(4);\n"
        "  auto s = nbgb::CreateNBodySim(nbgb::ENBodySim::BarnesHut);\n"
        "  s->Init(v); s->Update(0.01f);\n"
        "  return nbgb::NBodySimGetName(nbgb::ENBodySim::BarnesHut).empty();\n"
        "}\n")
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I", nb_build.INCLUDE, str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_driver_builds_and_rejects_bad_usage():
    exe = nb_build.build_driver()
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and "usage" in r.stderr
    r = subprocess.run([exe, "-c", "-p", "0"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2
    r = subprocess.run([exe, "-x"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2
