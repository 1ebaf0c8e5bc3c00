"""The reference's own CPU N-body code, built from its sources -- TEST
INFRASTRUCTURE ONLY.

``oracle/ref/Makefile`` compiles src/Sim/Octree.cpp, BarnesHut.cpp and
BruteForceCPU.cpp of the reference checkout, unmodified, with g++ against the
type-only headers in ``oracle/ref/shim`` (DirectXTK SimpleMath and the
Direct3D type names; no graphics), plus ``oracle/ref/ref_harness.cpp``, into
``oracle/_ref/libnb_ref.so``.  The tests use it to pin the oracle's
restatement and ``tests/golden/make_golden.py`` to generate the golden
vectors.  It exists only where the reference sources do (not on a machine
that only runs the committed tests); ``available()`` says whether it built.

The reference's physics constants are compiled in (src/Sim/Physics.hpp:9-17).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
RECIPE = os.path.join(HERE, "ref")
LIB = os.path.join(HERE, "_ref", "libnb_ref.so")
REFERENCE = os.environ.get("NB_REFERENCE_SRC", "/root/reference")

G = 6.674e-11             # Phys::G
S = 10.0                  # Phys::S (the softener, added to the squared distance)
STAR_SYSTEM_SCALE = 20 * 1.15e12   # Phys::StarSystemScale, the drift divisor
HALF = 4000.0             # BarnesHut's root cube, +-4000

_lock = threading.Lock()
_lib = None
_err = None


def available() -> bool:
    """Whether the reference sources are present and the library builds."""
    try:
        lib()
        return True
    except (OSError, RuntimeError):
        return False


def build() -> str:
    if not os.path.isdir(os.path.join(REFERENCE, "src", "Sim")):
        raise RuntimeError("reference sources not found at %s" % REFERENCE)
    r = subprocess.run(["make", "-s", "-C", RECIPE, "REF=" + REFERENCE], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference build failed:\n" + r.stdout + r.stderr)
    return LIB


def lib():
    global _lib, _err
    with _lock:
        if _lib is None:
            if _err is not None:
                raise RuntimeError(_err)
            try:
                build()
            except RuntimeError as e:
                _err = str(e)
                raise
            L = ctypes.CDLL(LIB)
            vp, sz, dbl, i32 = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_double, ctypes.c_int
            L.ref_workers.restype = i32
            L.ref_octree_build.argtypes = [vp, sz]
            L.ref_octree_build.restype = vp
            L.ref_octree_free.argtypes = [vp]
            L.ref_octree_node_count.argtypes = [vp]
            L.ref_octree_node_count.restype = sz
            L.ref_octree_max_depth.argtypes = [vp]
            L.ref_octree_max_depth.restype = i32
            L.ref_octree_export.argtypes = [vp, vp, vp, vp, vp]
            L.ref_octree_forces.argtypes = [vp, vp, sz, dbl, vp]
            L.ref_bh_update.argtypes = [vp, sz, ctypes.c_float, dbl, i32]
            L.ref_bf_update.argtypes = [vp, sz, ctypes.c_float, i32]
            _lib = L
        return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def workers() -> int:
    """CThreadPool's worker count on this machine (hardware threads - 1)."""
    return int(lib().ref_workers())


class RefOctree:
    """The reference's Octree over BarnesHut's root cube, built by Add in
    array order and CalculateMass."""

    def __init__(self, records: np.ndarray):
        self._p = np.ascontiguousarray(records)
        assert self._p.dtype.itemsize == 104
        self.n = self._p.shape[0]
        self.h = lib().ref_octree_build(_ptr(self._p), self.n)

    def close(self):
        if self.h:
            lib().ref_octree_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def max_depth(self) -> int:
        return int(lib().ref_octree_max_depth(self.h))

    def nodes(self) -> dict:
        """Every node (all eight children of each split), depth first."""
        m = int(lib().ref_octree_node_count(self.h))
        ints = np.zeros((m, 4), np.int32)
        prefix = np.zeros(m, np.uint64)
        mass = np.zeros(m, np.float64)
        fl = np.zeros((m, 10), np.float32)
        lib().ref_octree_export(self.h, _ptr(ints), _ptr(prefix), _ptr(mass), _ptr(fl))
        return dict(level=ints[:, 0], count=ints[:, 1], is_leaf=ints[:, 2], body=ints[:, 3], prefix=prefix,
                    mass=mass, com=fl[:, 0:3], lo=fl[:, 3:6], hi=fl[:, 6:9], side=fl[:, 9])

    def forces(self, targets=None, theta=0.5) -> np.ndarray:
        t = np.arange(self.n, dtype=np.int32) if targets is None else np.ascontiguousarray(targets, np.int32)
        out = np.zeros((t.shape[0], 3), np.float64)
        lib().ref_octree_forces(self.h, _ptr(t), t.shape[0], theta, _ptr(out))
        return out


def bh_update(records: np.ndarray, dt: float, theta: float, steps: int = 1) -> np.ndarray:
    """BarnesHut::Update steps times on a copy of the records."""
    p = np.array(records, copy=True)
    lib().ref_bh_update(_ptr(p), p.shape[0], dt, theta, steps)
    return p


def bf_update(records: np.ndarray, dt: float, steps: int = 1) -> np.ndarray:
    """BruteForceCPU::Update steps times on a copy of the records."""
    p = np.array(records, copy=True)
    lib().ref_bf_update(_ptr(p), p.shape[0], dt, steps)
    return p
