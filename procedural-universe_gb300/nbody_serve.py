"""ctypes binding of the served form (nb_server_* in include/nbody_gb300.h)."""
from __future__ import annotations

import ctypes

import numpy as np

import nbody_gb300 as nb


class nb_server_params(ctypes.Structure):
    _fields_ = [("base", nb.nb_params), ("memory_budget", ctypes.c_size_t), ("max_active", ctypes.c_int),
                ("steps_per_round", ctypes.c_int), ("bh_threshold", ctypes.c_size_t), ("round_seconds", ctypes.c_double)]


class nb_job(ctypes.Structure):
    _fields_ = [("seed", ctypes.c_uint64), ("n", ctypes.c_size_t), ("steps", ctypes.c_int), ("dt", ctypes.c_float),
                ("model", ctypes.c_int)]


class nb_job_status(ctypes.Structure):
    _fields_ = [("id", ctypes.c_uint64), ("state", ctypes.c_int), ("steps_done", ctypes.c_int),
                ("submit_s", ctypes.c_double), ("admit_s", ctypes.c_double), ("done_s", ctypes.c_double),
                ("bytes", ctypes.c_size_t)]


def _bind():
    L = nb.lib()
    if getattr(L, "_server_bound", False):
        return L
    vp, sz, i32 = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int
    sig = {
        "nb_server_default_params": ([vp], i32),
        "nb_server_create": ([vp, vp], i32),
        "nb_server_destroy": ([vp], i32),
        "nb_server_last_error": ([vp], ctypes.c_char_p),
        "nb_server_submit": ([vp, vp, vp], i32),
        "nb_server_tick": ([vp, vp, vp], i32),
        "nb_server_clock": ([vp], ctypes.c_double),
        "nb_server_status": ([vp, ctypes.c_uint64, vp], i32),
        "nb_server_result": ([vp, ctypes.c_uint64, vp, vp, sz], i32),
        "nb_server_release": ([vp, ctypes.c_uint64], i32),
        "nb_server_stats": ([vp, vp, vp], i32),
        "nb_server_timing": ([vp, vp, vp, vp, vp, vp, vp], i32),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    L._server_bound = True
    return L


class NBodyServer:
    """Continuous-batching request loop (nb_server*)."""

    def __init__(self, memory_budget=None, max_active=None, steps_per_round=None, bh_threshold=None,
                 round_seconds=None, **base):
        L = _bind()
        p = nb_server_params()
        L.nb_server_default_params(ctypes.byref(p))
        for k, v in base.items():
            setattr(p.base, k, v)
        if memory_budget is not None:
            p.memory_budget = memory_budget
        if max_active is not None:
            p.max_active = max_active
        if steps_per_round is not None:
            p.steps_per_round = steps_per_round
        if bh_threshold is not None:
            p.bh_threshold = bh_threshold
        if round_seconds is not None:
            p.round_seconds = round_seconds
        self.params = p
        self._h = ctypes.c_void_p()
        rc = L.nb_server_create(ctypes.byref(p), ctypes.byref(self._h))
        if rc:
            raise nb.NBodyError(rc, "nb_server_create failed")
        self.n_of = {}

    def _check(self, rc, what):
        if rc:
            msg = nb.lib().nb_server_last_error(self._h)
            raise nb.NBodyError(rc, "%s: %s" % (what, msg.decode() if msg else ""))

    def close(self):
        if self._h:
            nb.lib().nb_server_destroy(self._h)
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

    def submit(self, seed, n, steps, dt, model=0) -> int:
        j = nb_job(seed=seed, n=n, steps=steps, dt=dt, model=model)
        jid = ctypes.c_uint64(0)
        self._check(nb.lib().nb_server_submit(self._h, ctypes.byref(j), ctypes.byref(jid)), "nb_server_submit")
        self.n_of[jid.value] = n
        return jid.value

    def tick(self):
        a, q = ctypes.c_int(0), ctypes.c_int(0)
        self._check(nb.lib().nb_server_tick(self._h, ctypes.byref(a), ctypes.byref(q)), "nb_server_tick")
        return a.value, q.value

    def clock(self) -> float:
        return nb.lib().nb_server_clock(self._h)

    def status(self, jid) -> dict:
        st = nb_job_status()
        self._check(nb.lib().nb_server_status(self._h, jid, ctypes.byref(st)), "nb_server_status")
        return {f: getattr(st, f) for f, _ in st._fields_}

    def result(self, jid):
        n = self.n_of[jid]
        pm = np.zeros((n, 4), np.float32)
        v = np.zeros((n, 4), np.float32)
        self._check(nb.lib().nb_server_result(self._h, jid, nb._ptr(pm), nb._ptr(v), n), "nb_server_result")
        return pm, v

    def release(self, jid):
        """Forgets a finished or rejected job (frees its result)."""
        self._check(nb.lib().nb_server_release(self._h, jid), "nb_server_release")
        self.n_of.pop(jid, None)

    def stats(self):
        bs, r = ctypes.c_uint64(0), ctypes.c_uint64(0)
        self._check(nb.lib().nb_server_stats(self._h, ctypes.byref(bs), ctypes.byref(r)), "nb_server_stats")
        return dict(body_steps=bs.value, rounds=r.value)

    def timing(self):
        """Rebuilds (count, seconds), batch steps (count, seconds) and host generation seconds."""
        nr, ns_, nl = ctypes.c_uint64(0), ctypes.c_uint64(0), ctypes.c_uint64(0)
        rs, ss, gs = ctypes.c_double(0), ctypes.c_double(0), ctypes.c_double(0)
        self._check(nb.lib().nb_server_timing(self._h, ctypes.byref(nr), ctypes.byref(rs), ctypes.byref(ns_),
                                              ctypes.byref(ss), ctypes.byref(gs), ctypes.byref(nl)),
                    "nb_server_timing")
        return dict(rebuilds=nr.value, rebuild_s=rs.value, batch_steps=ns_.value, step_s=ss.value,
                    generate_s=gs.value, step_launches=nl.value)
