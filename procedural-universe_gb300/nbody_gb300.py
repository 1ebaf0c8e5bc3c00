"""ctypes binding of libnbody_gb300.so (the C-ABI in include/nbody_gb300.h).

This module is the binding a Python caller (tests, bench) uses; it adds no
compute of its own.  ``NBodySim`` mirrors the reference simulator interface
INBodySim (src/Sim/INBodySim.hpp:19-25): ``init(particles)`` and
``update(dt)`` on a caller-owned array of 104-byte Particle records.

The library must exist (built by build.py); there is no fallback: loading
fails loudly when it is missing, and every GPU call raises ``NBodyError``
with the library's message when the CUDA path cannot run.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libnbody_gb300.so")

NB_OK, NB_EINVAL, NB_ENOMEM, NB_ECUDA, NB_ETIMEOUT, NB_EBADSTATE, NB_ENOTSUP = 0, -1, -2, -3, -4, -5, -6
SIM_BRUTE_FORCE, SIM_BRUTE_FORCE_GPU, SIM_BARNES_HUT = 0, 1, 2
LAW_REFERENCE, LAW_PLUMMER = 0, 1
FLAG_NONE, FLAG_NO_COMPENSATION, FLAG_STAGED_IO = 0, 1, 2

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

RENDER_DTYPE = np.dtype([("position", "<f4", (3,)), ("colour", "<f4", (4,)), ("scale", "<f4")])

TREE_NODE_DTYPE = np.dtype(
    [
        ("level", "<i4"),
        ("count", "<i4"),
        ("first_child", "<i4"),
        ("body", "<i4"),
        ("prefix", "<u8"),
        ("mass", "<f8"),
        ("com", "<f4", (3,)),
        ("side", "<f4"),
        ("lo", "<f4", (3,)),
        ("bucket_begin", "<i4"),
        ("bucket_end", "<i4"),
    ],
    align=True,
)
assert TREE_NODE_DTYPE.itemsize == 72


class nb_params(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int),
        ("law", ctypes.c_int),
        ("G", ctypes.c_double),
        ("softening2", ctypes.c_double),
        ("theta", ctypes.c_double),
        ("pos_scale", ctypes.c_double),
        ("bounds_half", ctypes.c_float),
        ("max_depth", ctypes.c_int),
        ("leaf_size", ctypes.c_int),
        ("device", ctypes.c_int),
        ("stream", ctypes.c_void_p),
        ("flags", ctypes.c_int),
    ]


class nb_diag(ctypes.Structure):
    _fields_ = [
        ("kinetic", ctypes.c_double),
        ("potential", ctypes.c_double),
        ("total", ctypes.c_double),
        ("momentum", ctypes.c_double * 3),
        ("angular_momentum", ctypes.c_double * 3),
        ("mass", ctypes.c_double),
        ("centre_of_mass", ctypes.c_double * 3),
    ]


class NBodyError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__("nbody error %d: %s" % (code, msg))
        self.code = code


_lib = None


def lib() -> ctypes.CDLL:
    """Loads the in-tree library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError("libnbody_gb300.so is missing (run __graft_entry__.build())")
        L = ctypes.CDLL(LIB_PATH)
        vp, sz, i32, f32, f64 = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_float, ctypes.c_double
        sig = {
            "nb_default_params": ([vp], i32),
            "nb_create": ([vp, vp], i32),
            "nb_destroy": ([vp], i32),
            "nb_last_error": ([vp], ctypes.c_char_p),
            "nb_sim_name": ([i32], ctypes.c_char_p),
            "nb_init_particles": ([vp, vp, sz], i32),
            "nb_init_soa": ([vp, vp, vp, sz], i32),
            "nb_count": ([vp], sz),
            "nb_step": ([vp, f32, i32], i32),
            "nb_synchronize": ([vp], i32),
            "nb_write_back": ([vp, vp, sz], i32),
            "nb_write_back_direct": ([vp], i32),
            "nb_read_state": ([vp, vp, vp, vp], i32),
            "nb_compute_forces": ([vp, vp], i32),
            "nb_last_interactions": ([vp, vp], i32),
            "nb_fp64_forces": ([vp, vp, sz, vp], i32),
            "nb_diagnostics": ([vp, f32, vp], i32),
            "nb_stream": ([vp], vp),
            "nb_render_vertices": ([vp, vp, f32, vp, sz], i32),
            "nb_tree_keys": ([vp, vp, vp], i32),
            "nb_tree_size": ([vp, vp], i32),
            "nb_tree_nodes": ([vp, vp, sz], i32),
            "nb_tree_order": ([vp, vp], i32),
            "nb_tree_stats": ([vp, vp], i32),
            "nb_profile_enable": ([vp, i32], i32),
            "nb_profile_read": ([vp, i32, vp, vp], i32),
            "nb_launch_count": ([vp, vp], i32),
            "nb_probe_fp32_peak": ([i32, vp], i32),
            "nb_probe_fp32x2_peak": ([i32, vp], i32),
            "nb_tune": ([vp, ctypes.c_char_p, i32], i32),
            "nb_direct_accel_noalloc": ([vp, sz, vp, f64, f64, i32, vp], i32),
            "nb_get_tune": ([vp, ctypes.c_char_p, vp], i32),
            "nb_seed_plummer": ([ctypes.c_uint64, sz, f64, f64, vp, vp], i32),
            "nb_seed_disk": ([ctypes.c_uint64, sz, f64, f64, f64, f64, f64, f64, vp, vp], i32),
            "nb_seed_collision": ([ctypes.c_uint64, sz, f64, f64, f64, vp, vp], i32),
            "nb_seed_reference": ([i32, ctypes.c_uint64, f32, vp, sz], i32),
            "nb_init_seeded": ([vp, i32, ctypes.c_uint64, f32, sz, vp], i32),
            "nb_render_attach": ([vp, vp, f32, vp], i32),
            "nb_render_detach": ([vp], i32),
            "nb_render_read": ([vp, vp, sz], i32),
            "nb_file_write": ([ctypes.c_char_p, vp, sz], i32),
            "nb_file_read": ([ctypes.c_char_p, vp, sz, vp, i32], i32),
        }
        for name, (args, res) in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def default_params(**kw) -> nb_params:
    p = nb_params()
    lib().nb_default_params(ctypes.byref(p))
    for k, v in kw.items():
        if k == "stream":
            v = ctypes.c_void_p(v) if v else None
        setattr(p, k, v)
    return p


# ---- seeders (host C++ in the library; no GPU needed) ----------------------

def seed_plummer(seed: int, n: int, total_mass=1.0, a=1.0):
    pm = np.zeros((n, 4), np.float32)
    v = np.zeros((n, 4), np.float32)
    rc = lib().nb_seed_plummer(seed, n, total_mass, a, _ptr(pm), _ptr(v))
    if rc:
        raise NBodyError(rc, "nb_seed_plummer")
    return pm, v


def seed_disk(seed: int, n: int, total_mass=1.0, rd=1.0, z0=0.1, bulge_frac=0.1, ab=0.2, dispersion=0.05):
    pm = np.zeros((n, 4), np.float32)
    v = np.zeros((n, 4), np.float32)
    rc = lib().nb_seed_disk(seed, n, total_mass, rd, z0, bulge_frac, ab, dispersion, _ptr(pm), _ptr(v))
    if rc:
        raise NBodyError(rc, "nb_seed_disk")
    return pm, v


def seed_collision(seed: int, n: int, a=1.0, separation=10.0, pericentre=1.0):
    pm = np.zeros((n, 4), np.float32)
    v = np.zeros((n, 4), np.float32)
    rc = lib().nb_seed_collision(seed, n, a, separation, pericentre, _ptr(pm), _ptr(v))
    if rc:
        raise NBodyError(rc, "nb_seed_collision")
    return pm, v


SEEDER_RANDOM, SEEDER_GALAXY, SEEDER_STAR_SYSTEM = 0, 1, 2


def seed_reference(seeder: int, seed: int, n: int, scale: float = 1.0) -> np.ndarray:
    """Particle records drawn from the reference's RandomSeeder / GalaxySeeder /
    StarSystemSeeder distributions (src/Sim/*Seeder.cpp)."""
    p = np.zeros(n, dtype=PARTICLE_DTYPE)
    rc = lib().nb_seed_reference(seeder, seed, scale, _ptr(p), n)
    if rc:
        raise NBodyError(rc, "nb_seed_reference")
    return p


def file_write(path: str, particles: np.ndarray) -> None:
    """Writes raw 104-byte Particle records (the reference's .nbody file)."""
    p = np.ascontiguousarray(particles, dtype=PARTICLE_DTYPE)
    rc = lib().nb_file_write(os.fsencode(path), _ptr(p), p.shape[0])
    if rc:
        raise NBodyError(rc, "nb_file_write(%s)" % path)


def file_read(path: str, recentre: bool = True) -> np.ndarray:
    """Reads a .nbody file; recentre=True shifts positions to the centre of
    mass as the reference's file loader does."""
    n = ctypes.c_size_t(0)
    rc = lib().nb_file_read(os.fsencode(path), None, 0, ctypes.byref(n), 0)
    if rc:
        raise NBodyError(rc, "nb_file_read(%s)" % path)
    p = np.zeros(n.value, dtype=PARTICLE_DTYPE)
    rc = lib().nb_file_read(os.fsencode(path), _ptr(p), n.value, ctypes.byref(n), int(recentre))
    if rc:
        raise NBodyError(rc, "nb_file_read(%s)" % path)
    return p[: n.value]


def records_from_soa(pos_mass: np.ndarray, vel: np.ndarray | None = None) -> np.ndarray:
    n = pos_mass.shape[0]
    p = np.zeros(n, dtype=PARTICLE_DTYPE)
    p["position"] = pos_mass[:, :3]
    p["mass"] = pos_mass[:, 3].astype(np.float64)
    if vel is not None:
        p["velocity"] = vel[:, :3].astype(np.float64)
    p["colour"] = 1.0
    p["original_colour"] = 1.0
    return p


class NBodySim:
    """One simulator handle (nb_sim*), shaped like INBodySim."""

    def __init__(self, kind=SIM_BARNES_HUT, **params):
        self._h = ctypes.c_void_p()
        self.params = default_params(kind=kind, **params)
        rc = lib().nb_create(ctypes.byref(self.params), ctypes.byref(self._h))
        if rc:
            raise NBodyError(rc, "nb_create failed (no usable CUDA device?)")
        self.n = 0

    # -- plumbing --
    def _check(self, rc: int, what: str):
        if rc:
            msg = lib().nb_last_error(self._h)
            raise NBodyError(rc, "%s: %s" % (what, msg.decode() if msg else ""))

    def close(self):
        if self._h:
            lib().nb_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    @property
    def stream(self) -> int:
        return lib().nb_stream(self._h) or 0

    # -- INBodySim --
    def init(self, particles: np.ndarray):
        """INBodySim::Init: uploads the caller's 104-byte records."""
        p = np.ascontiguousarray(particles, dtype=PARTICLE_DTYPE)
        self._check(lib().nb_init_particles(self._h, _ptr(p), p.shape[0]), "nb_init_particles")
        self.n = p.shape[0]

    def init_seeded(self, seeder: int, seed: int, n: int, scale: float = 1.0) -> np.ndarray:
        """A reference seeder run on the GPU, then Init; returns the generated records."""
        p = np.zeros(n, dtype=PARTICLE_DTYPE)
        self._check(lib().nb_init_seeded(self._h, seeder, seed, scale, n, _ptr(p)), "nb_init_seeded")
        self.n = n
        return p

    def init_soa(self, pos_mass: np.ndarray, vel: np.ndarray):
        pm = np.ascontiguousarray(pos_mass, np.float32)
        v = np.ascontiguousarray(vel, np.float32)
        assert pm.shape == v.shape and pm.shape[1] == 4
        self._check(lib().nb_init_soa(self._h, _ptr(pm), _ptr(v), pm.shape[0]), "nb_init_soa")
        self.n = pm.shape[0]

    def step(self, dt: float, nsteps: int = 1):
        self._check(lib().nb_step(self._h, dt, nsteps), "nb_step")

    def update(self, dt: float, particles: np.ndarray | None = None):
        """INBodySim::Update: one step, then the records are updated in place."""
        self.step(dt, 1)
        if particles is not None:
            self.write_back(particles)

    def synchronize(self):
        self._check(lib().nb_synchronize(self._h), "nb_synchronize")

    def write_back(self, particles: np.ndarray):
        assert particles.dtype == PARTICLE_DTYPE and particles.flags.c_contiguous
        self._check(lib().nb_write_back(self._h, _ptr(particles), particles.shape[0]), "nb_write_back")

    def write_back_direct(self) -> bool:
        """Whether write_back rewrites the records from the GPU directly (whole records)."""
        return lib().nb_write_back_direct(self._h) == 1

    def read_state(self):
        pos = np.zeros((self.n, 3), np.float32)
        vel = np.zeros((self.n, 3), np.float64)
        force = np.zeros((self.n, 3), np.float64)
        self._check(lib().nb_read_state(self._h, _ptr(pos), _ptr(vel), _ptr(force)), "nb_read_state")
        return pos, vel, force

    def compute_forces(self) -> np.ndarray:
        f = np.zeros((self.n, 3), np.float64)
        self._check(lib().nb_compute_forces(self._h, _ptr(f)), "nb_compute_forces")
        return f

    def last_interactions(self) -> int:
        v = ctypes.c_uint64(0)
        self._check(lib().nb_last_interactions(self._h, ctypes.byref(v)), "nb_last_interactions")
        return int(v.value)

    def fp64_forces(self, targets: np.ndarray) -> np.ndarray:
        t = np.ascontiguousarray(targets, np.int32)
        out = np.zeros((t.shape[0], 3), np.float64)
        self._check(lib().nb_fp64_forces(self._h, _ptr(t), t.shape[0], _ptr(out)), "nb_fp64_forces")
        return out

    def diagnostics(self, half_kick_dt: float = 0.0) -> dict:
        d = nb_diag()
        self._check(lib().nb_diagnostics(self._h, half_kick_dt, ctypes.byref(d)), "nb_diagnostics")
        return dict(kinetic=d.kinetic, potential=d.potential, total=d.total, momentum=np.array(d.momentum[:]),
                    angular_momentum=np.array(d.angular_momentum[:]), mass=d.mass,
                    centre_of_mass=np.array(d.centre_of_mass[:]))

    def tune(self, key: str, value: int):
        self._check(lib().nb_tune(self._h, key.encode(), int(value)), "nb_tune(%s=%d)" % (key, value))

    def get_tune(self, key: str) -> int:
        v = ctypes.c_int(0)
        self._check(lib().nb_get_tune(self._h, key.encode(), ctypes.byref(v)), "nb_get_tune")
        return v.value

    # -- octree export (Barnes-Hut) --
    def tree_keys(self):
        k = np.zeros(self.n, np.uint64)
        d = np.zeros(self.n, np.int32)
        self._check(lib().nb_tree_keys(self._h, _ptr(k), _ptr(d)), "nb_tree_keys")
        return k, d

    def tree_nodes(self) -> np.ndarray:
        m = ctypes.c_size_t(0)
        self._check(lib().nb_tree_size(self._h, ctypes.byref(m)), "nb_tree_size")
        out = np.zeros(m.value, TREE_NODE_DTYPE)
        self._check(lib().nb_tree_nodes(self._h, _ptr(out), m.value), "nb_tree_nodes")
        return out

    def tree_order(self) -> np.ndarray:
        o = np.zeros(self.n, np.int32)
        self._check(lib().nb_tree_order(self._h, _ptr(o)), "nb_tree_order")
        return o

    def tree_stats(self) -> dict:
        st = np.zeros(8, np.int64)
        self._check(lib().nb_tree_stats(self._h, _ptr(st)), "nb_tree_stats")
        return dict(inside=int(st[0]), internal=int(st[1]), nodes=int(st[2]), gaps=int(st[3]),
                    deeper_buckets=int(st[4]), lookup_failures=int(st[5]), outside=int(st[6]))

    def render_vertices(self, colour: np.ndarray | None = None, scale: float = 1.0) -> np.ndarray:
        out = np.zeros(self.n, RENDER_DTYPE)
        c = None if colour is None else np.ascontiguousarray(colour, np.float32)
        self._check(lib().nb_render_vertices(self._h, _ptr(c), scale, _ptr(out), self.n), "nb_render_vertices")
        return out

    def render_attach(self, colour: np.ndarray | None = None, scale: float = 1.0) -> int:
        """Attaches the device vertex buffer filled by every kick-drift; returns its device address."""
        c = None if colour is None else np.ascontiguousarray(colour, np.float32)
        ptr = ctypes.c_void_p()
        self._check(lib().nb_render_attach(self._h, _ptr(c), scale, ctypes.byref(ptr)), "nb_render_attach")
        return ptr.value

    def render_detach(self):
        self._check(lib().nb_render_detach(self._h), "nb_render_detach")

    def render_read(self) -> np.ndarray:
        out = np.zeros(self.n, RENDER_DTYPE)
        self._check(lib().nb_render_read(self._h, _ptr(out), self.n), "nb_render_read")
        return out


class nb_tuning(ctypes.Structure):
    _fields_ = [("direct_block", ctypes.c_int), ("direct_ipt", ctypes.c_int), ("direct_jtile", ctypes.c_int),
                ("leaf_size", ctypes.c_int), ("traverse_block", ctypes.c_int)]


def _bind_batch():
    L = lib()
    if getattr(L, "_batch_bound", False):
        return L
    vp, sz, i32, f32, f64 = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_float, ctypes.c_double
    sig = {
        "nb_batch_create": ([vp, sz, f64, vp], i32),
        "nb_batch_destroy": ([vp], i32),
        "nb_batch_last_error": ([vp], ctypes.c_char_p),
        "nb_batch_add": ([vp, vp, vp, sz, vp], i32),
        "nb_batch_add_generated": ([vp, i32, ctypes.c_uint64, sz, vp], i32),
        "nb_batch_steps_not_run": ([vp, vp], i32),
        "nb_batch_commit": ([vp], i32),
        "nb_batch_set_tuning": ([vp, vp], i32),
        "nb_batch_set_far_field": ([vp, f64], i32),
        "nb_batch_set_far_accuracy": ([vp, f64, f64], i32),
        "nb_batch_get_tuning": ([vp, vp], i32),
        "nb_batch_autotune": ([vp, f32, i32], i32),
        "nb_batch_step": ([vp, f32, i32], i32),
        "nb_batch_read": ([vp, i32, vp, vp], i32),
        "nb_batch_forces": ([vp, i32, vp], i32),
        "nb_batch_info": ([vp, vp, vp, vp], i32),
        "nb_batch_launch_count": ([vp, vp], i32),
        "nb_batch_tree_stats": ([vp, vp], i32),
        "nb_batch_stream": ([vp], vp),
        "nb_batch_write_state": ([vp, vp, vp], i32),
        "nb_batch_read_state": ([vp, vp, vp], i32),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    L._batch_bound = True
    return L


class NBodyBatch:
    """Batched form: many galaxies stepped together (nb_batch*)."""

    def __init__(self, bh_threshold=8192, bh_theta=0.6, **params):
        L = _bind_batch()
        self._h = ctypes.c_void_p()
        p = default_params(**params)
        rc = L.nb_batch_create(ctypes.byref(p), bh_threshold, bh_theta, ctypes.byref(self._h))
        if rc:
            raise NBodyError(rc, "nb_batch_create failed")
        self.sizes = []

    def _check(self, rc, what):
        if rc:
            msg = lib().nb_batch_last_error(self._h)
            raise NBodyError(rc, "%s: %s" % (what, msg.decode() if msg else ""))

    def close(self):
        if self._h:
            lib().nb_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    @property
    def stream(self) -> int:
        return lib().nb_batch_stream(self._h) or 0

    def add(self, pos_mass, vel) -> int:
        pm = np.ascontiguousarray(pos_mass, np.float32)
        v = np.ascontiguousarray(vel, np.float32)
        g = ctypes.c_int32(-1)
        self._check(lib().nb_batch_add(self._h, _ptr(pm), _ptr(v), pm.shape[0], ctypes.byref(g)), "nb_batch_add")
        self.sizes.append(pm.shape[0])
        return g.value

    def add_generated(self, model: int, seed: int, n: int) -> int:
        """A galaxy generated on the device at commit: model 0 disk + bulge,
        1 Plummer sphere, 2 colliding Plummer spheres (the seed_* defaults)."""
        g = ctypes.c_int32(-1)
        self._check(lib().nb_batch_add_generated(self._h, model, seed, n, ctypes.byref(g)), "nb_batch_add_generated")
        self.sizes.append(n)
        return g.value

    def steps_not_run(self) -> int:
        v = ctypes.c_int(0)
        self._check(lib().nb_batch_steps_not_run(self._h, ctypes.byref(v)), "nb_batch_steps_not_run")
        return v.value

    def commit(self):
        self._check(lib().nb_batch_commit(self._h), "nb_batch_commit")

    def step(self, dt, nsteps=1):
        self._check(lib().nb_batch_step(self._h, dt, nsteps), "nb_batch_step")

    def autotune(self, dt, trial_steps=3):
        self._check(lib().nb_batch_autotune(self._h, dt, trial_steps), "nb_batch_autotune")

    def tuning(self) -> dict:
        t = nb_tuning()
        self._check(lib().nb_batch_get_tuning(self._h, ctypes.byref(t)), "nb_batch_get_tuning")
        return {f: getattr(t, f) for f, _ in t._fields_}

    def set_tuning(self, **kw):
        t = nb_tuning()
        self._check(lib().nb_batch_get_tuning(self._h, ctypes.byref(t)), "nb_batch_get_tuning")
        for k, v in kw.items():
            setattr(t, k, v)
        self._check(lib().nb_batch_set_tuning(self._h, ctypes.byref(t)), "nb_batch_set_tuning")

    def set_far_field(self, eta: float):
        self._check(lib().nb_batch_set_far_field(self._h, eta), "nb_batch_set_far_field")

    def set_far_accuracy(self, alpha: float, eta_max: float = 0.5):
        self._check(lib().nb_batch_set_far_accuracy(self._h, alpha, eta_max), "nb_batch_set_far_accuracy")

    def read(self, g):
        n = self.sizes[g]
        pm = np.zeros((n, 4), np.float32)
        v = np.zeros((n, 4), np.float32)
        self._check(lib().nb_batch_read(self._h, g, _ptr(pm), _ptr(v)), "nb_batch_read")
        return pm, v

    def forces(self, g):
        f = np.zeros((self.sizes[g], 3), np.float64)
        self._check(lib().nb_batch_forces(self._h, g, _ptr(f)), "nb_batch_forces")
        return f

    def write_state(self, pos_mass, vel):
        """Uploads every galaxy's state (concatenated in galaxy order)."""
        self._check(lib().nb_batch_write_state(self._h, _ptr(pos_mass), _ptr(vel)), "nb_batch_write_state")

    def read_state(self, pos_mass, vel=None):
        self._check(lib().nb_batch_read_state(self._h, _ptr(pos_mass), _ptr(vel)), "nb_batch_read_state")

    def info(self):
        ng, nb_, it = ctypes.c_size_t(0), ctypes.c_size_t(0), ctypes.c_uint64(0)
        self._check(lib().nb_batch_info(self._h, ctypes.byref(ng), ctypes.byref(nb_), ctypes.byref(it)),
                    "nb_batch_info")
        return dict(galaxies=ng.value, bodies=nb_.value, interactions=it.value)

    def launch_count(self) -> int:
        v = ctypes.c_uint64(0)
        self._check(lib().nb_batch_launch_count(self._h, ctypes.byref(v)), "nb_batch_launch_count")
        return int(v.value)

    def tree_stats(self):
        s = (ctypes.c_int64 * 4)()
        self._check(lib().nb_batch_tree_stats(self._h, s), "nb_batch_tree_stats")
        return dict(groups=s[0], internal=s[1], cells=s[2], bh_bodies=s[3])
