"""CPU oracle loader -- TEST INFRASTRUCTURE ONLY.

ctypes front end of ``nb_oracle.cpp``, the CPU restatement of the reference's
N-body step (BruteForceCPU, BarnesHut/Octree, Phys::Gravity).  Only the tests,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` import
this module; the product library never does.

Pinned to the reference's own code: oracle/ref/Makefile compiles the
reference's src/Sim/Octree.cpp, BarnesHut.cpp and BruteForceCPU.cpp
unmodified against type-only stand-ins for the DirectXTK / Direct3D headers,
and tests/test_reference_pin_cpu.py finds this restatement bit-identical to
it (every octree node, every force, every updated record) wherever the
depth cap and the remainder-slice fix do not apply; the committed vectors
tests/golden/reference_small.npz come from that build.  Still unpinned: the
DirectXTK SimpleMath arithmetic itself (the stand-in computes each vector
operation in plain float in the documented order).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "nb_oracle.cpp")
# The synthetic workload generator (seeded Plummer spheres, disk + bulge
# galaxies, colliding spheres) is compiled into the oracle from the same
# source file as the product's nb_seed_* so that the CPU arm of the bench
# gets byte-identical initial states without loading the product library.
# Its entry points are renamed orc_seed_* here.
SEED_SRC = os.path.join(os.path.dirname(HERE), "procedural-universe_gb300", "csrc", "nb_seed.cpp")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libnb_oracle.so")

# The 104-byte reference record (src/Render/Misc/Particle.hpp:8-18).
PARTICLE_DTYPE = np.dtype(
    [
        ("position", "<f4", (3,)),
        ("colour", "<f4", (4,)),
        ("original_colour", "<f4", (4,)),
        ("_pad", "<f4"),
        ("velocity", "<f8", (3,)),
        ("forces", "<f8", (3,)),
        ("mass", "<f8"),
    ]
)
assert PARTICLE_DTYPE.itemsize == 104

_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with g++ (-ffp-contract=off: float math as written)."""
    os.makedirs(OUT_DIR, exist_ok=True)
    deps = [SRC, SEED_SRC, os.path.join(os.path.dirname(SEED_SRC), "nb_rng.hpp")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    tmp = LIB + ".tmp.%d" % os.getpid()
    rename = ["-Dnb_seed_plummer=orc_seed_plummer", "-Dnb_seed_disk=orc_seed_disk",
              "-Dnb_seed_collision=orc_seed_collision"]
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-pthread", *rename, "-I", INCLUDE, SRC, SEED_SRC, "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(LIB)
            vp, sz, dbl, i32 = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_double, ctypes.c_int
            L.orc_direct_forces.argtypes = [vp, sz, dbl, dbl, i32, i32, vp]
            L.orc_direct_forces_subset.argtypes = [vp, sz, vp, sz, dbl, dbl, i32, i32, vp]
            L.orc_bh_forces_subset.argtypes = [vp, vp, sz, dbl, dbl, i32, dbl, i32, vp]
            L.orc_direct_step.argtypes = [vp, sz, dbl, dbl, i32, dbl, ctypes.c_float, i32, i32]
            L.orc_tree_build.argtypes = [vp, sz, ctypes.c_float, i32]
            L.orc_tree_build.restype = vp
            L.orc_tree_free.argtypes = [vp]
            L.orc_tree_node_count.argtypes = [vp]
            L.orc_tree_node_count.restype = sz
            L.orc_tree_deeper_buckets.argtypes = [vp]
            L.orc_tree_deeper_buckets.restype = ctypes.c_longlong
            L.orc_tree_nodes.argtypes = [vp, vp, vp, vp, vp]
            L.orc_tree_bucket.argtypes = [vp, sz, vp, i32]
            L.orc_tree_keys.argtypes = [vp, vp, vp]
            L.orc_bh_forces.argtypes = [vp, dbl, dbl, i32, dbl, i32, vp, vp]
            L.orc_bh_step.argtypes = [vp, sz, dbl, dbl, i32, dbl, dbl, ctypes.c_float, i32,
                                      ctypes.c_float, i32, i32]
            L.orc_fp64_forces.argtypes = [vp, vp, sz, vp, sz, dbl, dbl, i32, i32, vp]
            L.orc_fp64_diagnostics.argtypes = [vp, vp, vp, sz, dbl, dbl, i32, i32, vp]
            L.orc_threads_default.restype = i32
            f64 = ctypes.c_double
            L.orc_seed_plummer.argtypes = [ctypes.c_uint64, sz, f64, f64, vp, vp]
            L.orc_seed_disk.argtypes = [ctypes.c_uint64, sz, f64, f64, f64, f64, f64, f64, vp, vp]
            L.orc_seed_collision.argtypes = [ctypes.c_uint64, sz, f64, f64, f64, vp, vp]
            _lib = L
        return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def particles_from_soa(pos_mass: np.ndarray, vel: np.ndarray | None = None) -> np.ndarray:
    """Reference records from (n,4) float32 pos+mass and (n,4) float32 velocity."""
    n = pos_mass.shape[0]
    p = np.zeros(n, dtype=PARTICLE_DTYPE)
    p["position"] = pos_mass[:, :3]
    p["mass"] = pos_mass[:, 3].astype(np.float64)
    if vel is not None:
        p["velocity"] = vel[:, :3].astype(np.float64)
    p["colour"] = 1.0
    p["original_colour"] = 1.0
    return p


# ---- workload generator (the same source as the product's nb_seed_*) -------

def _seeded(fn, seed, n, *args):
    pm = np.zeros((n, 4), np.float32)
    v = np.zeros((n, 4), np.float32)
    rc = fn(seed, n, *args, _ptr(pm), _ptr(v))
    if rc:
        raise RuntimeError("workload generator failed (%d)" % rc)
    return pm, v


def seed_plummer(seed: int, n: int, total_mass=1.0, a=1.0):
    return _seeded(lib().orc_seed_plummer, seed, n, total_mass, a)


def seed_disk(seed: int, n: int, total_mass=1.0, rd=1.0, z0=0.1, bulge_frac=0.1, ab=0.2, dispersion=0.05):
    return _seeded(lib().orc_seed_disk, seed, n, total_mass, rd, z0, bulge_frac, ab, dispersion)


def seed_collision(seed: int, n: int, a=1.0, separation=10.0, pericentre=1.0):
    return _seeded(lib().orc_seed_collision, seed, n, a, separation, pericentre)


def default_threads() -> int:
    return int(lib().orc_threads_default())


def direct_forces(particles: np.ndarray, G=1.0, S=1e-4, law=0, threads=0) -> np.ndarray:
    p = np.ascontiguousarray(particles, dtype=PARTICLE_DTYPE)
    out = np.zeros((p.shape[0], 3), np.float64)
    lib().orc_direct_forces(_ptr(p), p.shape[0], G, S, law, threads, _ptr(out))
    return out


def direct_forces_subset(particles: np.ndarray, targets: np.ndarray, G=1.0, S=1e-4, law=0, threads=0):
    p = np.ascontiguousarray(particles, dtype=PARTICLE_DTYPE)
    t = np.ascontiguousarray(targets, np.int32)
    out = np.zeros((t.shape[0], 3), np.float64)
    lib().orc_direct_forces_subset(_ptr(p), p.shape[0], _ptr(t), t.shape[0], G, S, law, threads, _ptr(out))
    return out


def direct_step(particles: np.ndarray, dt: float, nsteps: int, G=1.0, S=1e-4, law=0, scale=1.0,
                threads=0) -> np.ndarray:
    """Runs BruteForceCPU::Update nsteps times on a copy; returns the records."""
    p = np.array(particles, dtype=PARTICLE_DTYPE, copy=True)
    lib().orc_direct_step(_ptr(p), p.shape[0], G, S, law, scale, dt, nsteps, threads)
    return p


def bh_step(particles: np.ndarray, dt: float, nsteps: int, G=1.0, S=1e-4, law=0, theta=0.5, scale=1.0,
            half=4000.0, max_depth=21, threads=0) -> np.ndarray:
    p = np.array(particles, dtype=PARTICLE_DTYPE, copy=True)
    lib().orc_bh_step(_ptr(p), p.shape[0], G, S, law, theta, scale, half, max_depth, dt, nsteps, threads)
    return p


class OracleTree:
    """The restated reference octree of one particle set."""

    def __init__(self, particles: np.ndarray, half=4000.0, max_depth=21):
        self._p = np.ascontiguousarray(particles, dtype=PARTICLE_DTYPE)
        self.n = self._p.shape[0]
        self.h = lib().orc_tree_build(_ptr(self._p), self.n, half, max_depth)

    def close(self):
        if self.h:
            lib().orc_tree_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def keys(self):
        k = np.zeros(self.n, np.uint64)
        d = np.zeros(self.n, np.int32)
        lib().orc_tree_keys(self.h, _ptr(k), _ptr(d))
        return k, d

    def nodes(self) -> dict:
        m = int(lib().orc_tree_node_count(self.h))
        ints = np.zeros((m, 6), np.int32)
        prefix = np.zeros(m, np.uint64)
        mass = np.zeros(m, np.float64)
        fl = np.zeros((m, 7), np.float32)
        lib().orc_tree_nodes(self.h, _ptr(ints), _ptr(prefix), _ptr(mass), _ptr(fl))
        return dict(level=ints[:, 0], count=ints[:, 1], first_child=ints[:, 2], body=ints[:, 3],
                    bucket_size=ints[:, 4], is_leaf=ints[:, 5], prefix=prefix, mass=mass,
                    com=fl[:, 0:3], side=fl[:, 3], lo=fl[:, 4:7])

    def bucket(self, i: int) -> np.ndarray:
        out = np.zeros(64, np.int32)
        k = lib().orc_tree_bucket(self.h, i, _ptr(out), 64)
        if k > 64:
            out = np.zeros(k, np.int32)
            lib().orc_tree_bucket(self.h, i, _ptr(out), k)
        return out[:k]

    def forces_subset(self, targets, G=1.0, S=1e-4, law=0, theta=0.5, threads=0):
        t = np.ascontiguousarray(targets, np.int32)
        out = np.zeros((t.shape[0], 3), np.float64)
        lib().orc_bh_forces_subset(self.h, _ptr(t), t.shape[0], G, S, law, theta, threads, _ptr(out))
        return out

    def deeper_buckets(self) -> int:
        return int(lib().orc_tree_deeper_buckets(self.h))

    def forces(self, G=1.0, S=1e-4, law=0, theta=0.5, threads=0):
        out = np.zeros((self.n, 3), np.float64)
        inter = ctypes.c_longlong(0)
        lib().orc_bh_forces(self.h, G, S, law, theta, threads, _ptr(out), ctypes.byref(inter))
        return out, int(inter.value)


def fp64_forces(pos3: np.ndarray, mass: np.ndarray, targets: np.ndarray, G=1.0, S=1e-4, law=0,
                threads=0) -> np.ndarray:
    pos3 = np.ascontiguousarray(pos3, np.float64)
    mass = np.ascontiguousarray(mass, np.float64)
    targets = np.ascontiguousarray(targets, np.int32)
    out = np.zeros((targets.shape[0], 3), np.float64)
    lib().orc_fp64_forces(_ptr(pos3), _ptr(mass), pos3.shape[0], _ptr(targets), targets.shape[0], G, S, law,
                          threads, _ptr(out))
    return out


def fp64_diagnostics(pos3, vel3, mass, G=1.0, S=1e-4, law=0, threads=0) -> dict:
    pos3 = np.ascontiguousarray(pos3, np.float64)
    vel3 = np.ascontiguousarray(vel3, np.float64)
    mass = np.ascontiguousarray(mass, np.float64)
    out = np.zeros(11, np.float64)
    lib().orc_fp64_diagnostics(_ptr(pos3), _ptr(vel3), _ptr(mass), pos3.shape[0], G, S, law, threads, _ptr(out))
    return dict(kinetic=out[0], potential=out[1], total=out[2], momentum=out[3:6], angular_momentum=out[6:9],
                mass=out[9])


def rel_l2(a: np.ndarray, b: np.ndarray) -> float:
    """||a - b||_2 / ||b||_2 over all bodies."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
