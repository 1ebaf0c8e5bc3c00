"""The headless precompute driver and the C++ adapter on the GPU: a driver
run must leave exactly the records that the same steps through the Python
binding leave (same library, same kernels), for a seeded star system and for
a re-centred file."""
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

import nb_build
import nbody_gb300 as nb

pytestmark = pytest.mark.gpu

REF = dict(G=6.674e-11, softening2=10.0, pos_scale=20 * 1.15e12, theta=2.0)


def run_driver(cwd, *args):
    exe = nb_build.build_driver()
    r = subprocess.run([exe, "-c", *args], cwd=cwd, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    return json.loads(r.stdout.strip().splitlines()[-1])


def step_python(p, steps, dt, kind=nb.SIM_BARNES_HUT):
    p = p.copy()
    with nb.NBodySim(kind, **REF) as s:
        s.init(p)
        for _ in range(steps):
            s.update(dt, p)
    return p


def test_driver_seeded_run_matches_binding(tmp_path):
    out = run_driver(tmp_path, "-p", "3000", "--steps", "20", "--seed", "4", "--out", "run.nbody")
    assert out["bodies"] == 3000 and out["steps"] == 20
    got = nb.file_read(str(tmp_path / "run.nbody"), recentre=False)
    init = nb.seed_reference(nb.SEEDER_STAR_SYSTEM, 4, 3000)
    want = step_python(init, 20, np.float32(0.02) * np.float32(1.0 / 60.0))
    assert got.tobytes() == want.tobytes()
    assert np.all(np.isfinite(got["position"]))
    assert not np.array_equal(got["position"], init["position"])


def test_driver_file_run_recentres_and_matches_binding(tmp_path):
    src = nb.seed_reference(nb.SEEDER_RANDOM, 2, 1500)
    src["position"] += np.float32(25.0)
    os.makedirs(tmp_path / "data")
    nb.file_write(str(tmp_path / "data" / "in.nbody"), src)
    out = run_driver(tmp_path, "-f", "in.nbody", "--steps", "6", "-s", "0.05", "--out", "o.nbody")
    assert out["bodies"] == 1500
    got = nb.file_read(str(tmp_path / "o.nbody"), recentre=False)
    init = nb.file_read(str(tmp_path / "data" / "in.nbody"))
    want = step_python(init, 6, np.float32(0.05) * np.float32(1.0 / 60.0))
    assert got.tobytes() == want.tobytes()


def test_driver_wall_clock_run_writes_data_file(tmp_path):
    out = run_driver(tmp_path, "-t", "1", "-p", "4000")
    assert out["steps"] >= 1
    assert out["file"].startswith("data/") and out["file"].endswith(".nbody")
    assert (tmp_path / out["file"]).stat().st_size == 4000 * 104


def test_cpp_adapter_program(tmp_path):
    """A program written against the INBodySim-shaped adapter: Init, Update,
    the render hand-off and the octree export."""
    src = tmp_path / "adapter.cpp"
    src.write_text(r'''
#include "cuda_nbody_sim.hpp"
#include <cstdio>
int main() {
    std::vector<nbgb::Particle> v(2048);
    nb_seed_reference(2, 3, 1.0f, v.data(), v.size());
    nb_params p; nb_default_params(&p);
    p.G = 6.674e-11; p.softening2 = 10.0; p.pos_scale = 2.3e13; p.theta = 0.8;
    nbgb::CudaNBodySim sim(nbgb::ENBodySim::BarnesHut, &p);
    sim.Init(v);
    const float x0 = v[100].position[0];
    for (int i = 0; i < 3; ++i) sim.Update(0.01f);
    auto verts = sim.RenderVertices();
    auto nodes = sim.TreeNodes();
    bool ok = verts.size() == v.size() && verts[100].position[0] == v[100].position[0] &&
              v[100].position[0] != x0 && !nodes.empty() && nodes[0].count == (int)v.size();
    std::printf("%s %zu %zu\n", ok ? "OK" : "BAD", verts.size(), nodes.size());
    return ok ? 0 : 1;
}
''')
    lib_dir = os.path.dirname(nb_build.build())
    exe = tmp_path / "adapter"
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I", nb_build.INCLUDE, str(src), "-o", str(exe),
                        "-L", lib_dir, "-lnbody_gb300", "-Wl,-rpath," + lib_dir], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.startswith("OK"), r.stdout + r.stderr
