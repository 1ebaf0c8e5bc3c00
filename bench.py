"""Benchmark of the GB300 N-body step.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]

A step is one pass of the hot path over one galaxy: Barnes-Hut (octree keys,
radix sort, topology, mass pass, traversal, kick-drift) or direct sum (force
kernel + kick-drift).  `value` is body-steps/s with the particle state
resident in HBM; `e2e` is the same metric through the reference-facing C-ABI
(nb_init_particles from pinned host records, nb_step, nb_write_back into the
records) with the host<->device copies inside the timed region.

Workloads (seeded synthetic galaxies; no dataset is involved):
  bh1m        Barnes-Hut, N=1,048,576 exponential disk (90%) + Hernquist bulge
              (10%), theta=0.5, eps=0.005, dt=5e-4              [default]
  direct262k  direct sum, N=262,144, two Plummer spheres on a parabolic orbit,
              eps=0.01, dt=1e-3
  direct4096  direct sum, N=4096 Plummer sphere, eps=0.01, dt=1e-3

  batch512    512 galaxies, n log-uniform in [256, 65,536] (batched form)
  served      Poisson stream of 200 galaxy jobs (200 per second; --requests),
              n log-uniform in [1,024, 1,048,576] (served form: continuous
              batching under a memory budget)
  bh1m_batched  the batched form (group traversal, quadrupoles) on the bh1m galaxy

The default line (bh1m, one GPU) also carries
  "direct": the two direct-sum configurations, direct262k (20 steps) and
            direct4096 (100 steps), each with its own roofline against the
            FP32 FMA peak, FP64 force error, drift, CPU baseline and e2e
            (--no-direct leaves them out);
  "forms":  the batched and the served form on their workloads, each against
            sequential plain-path launches at the plain path's own theta and
            at equal accuracy (force error <= 1e-3 against the FP64 direct
            sum) (--no-forms leaves them out).

--impl reference times the reference's CPU algorithm (the oracle's
restatement of BruteForceCPU / BarnesHut on all host cores) on the same
workload, a bounded sample per step.  That arm loads only the oracle's
library: its initial states come from the oracle's copy of the workload
generator (the same source as the product's nb_seed_*, byte-identical
output), and it does not build or load the CUDA library.
Multi-GPU: the step does not shard across GPUs; --gpus N runs N
independent replicas (one galaxy per rank, different seeds) and reports the
aggregate.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "procedural-universe_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

WORKLOADS = {
    "bh1m": dict(kind=2, n=1 << 20, model="disk", eps=0.005, dt=5e-4, theta=0.5,
                 desc="Barnes-Hut, N=1,048,576 disk (rd=1, z0=0.1, 5% dispersion) + 10% Hernquist bulge (a=0.2), "
                      "theta=0.5, eps=0.005, dt=5e-4"),
    "direct262k": dict(kind=0, n=262144, model="collision", eps=0.01, dt=1e-3, theta=0.5,
                       desc="direct sum, N=262,144, two Plummer spheres (a=1, M=1 each) on a parabolic orbit "
                            "10 apart (pericentre 1), eps=0.01, dt=1e-3"),
    "direct4096": dict(kind=0, n=4096, model="plummer", eps=0.01, dt=1e-3, theta=0.5,
                       desc="direct sum, N=4096 Plummer sphere (a=1, M=1), eps=0.01, dt=1e-3"),
}
METRIC = "body-steps/s"
L2_FLUSH_BYTES = 512 << 20       # > 129 MB L2
FLOP_PER_INTERACTION = 20


# the step count each configuration is specified with (its sub-line in the default run)
CONFIG_STEPS = {"bh1m": 50, "direct262k": 20, "direct4096": 100}


def seed_workload(w, seed, gen=None):
    """Initial state (pos+mass, velocity) of workload w.  gen is the module
    whose seeders are used: the product binding for the GPU arm, the oracle
    for the CPU arm; both compile the same generator source."""
    if gen is None:
        import nbody_gb300 as gen
    if w["model"] == "disk":
        return gen.seed_disk(seed, w["n"])
    if w["model"] == "collision":
        return gen.seed_collision(seed, w["n"])
    return gen.seed_plummer(seed, w["n"])


def workload_config(name, w, world):
    """The line's config object; identical for both arms of the same run."""
    return {"workload": name, "desc": w["desc"], "n": w["n"],
            "parallelism": "replicas" if world > 1 else "1 GPU",
            "l2": "flushed (512 MB write) before every timed step"}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


# ---- replicas: one independent galaxy per rank, no data-path collective ----
def replica_seed(rank: int) -> int:
    """Seed of rank's galaxy: every replica steps a different galaxy."""
    return 1234 + rank


def max_over_ranks(x: float, device="cpu") -> float:
    """The largest x over the ranks of the process group (x itself without one)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replicas_value(world: int, n: int, steps: int, max_total_ms: float) -> float:
    """Body-steps/s of all replicas together, timed by the slowest rank."""
    return world * n * steps / (max_total_ms * 1e-3)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, device: int):
        self.device = device
        self.samples = []
        self._stop = threading.Event()
        self._proc = None
        self._thread = None

    def start(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self._proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + q, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self._proc = None
            return
        self._thread = threading.Thread(target=self._read, daemon=True)
        self._thread.start()

    def _read(self):
        for line in self._proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def stop(self) -> dict:
        if self._proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self._proc.terminate()
        try:
            self._proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self._proc.kill()
        if self._thread:
            self._thread.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            try:
                sm.append(float(s[0]))
                mx.append(float(s[1]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if s[3 + k].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


# --------------------------------------------------------------------------
# CPU baseline: the reference's CPU algorithm (oracle restatement), bounded.
# --------------------------------------------------------------------------
def cpu_baseline(w, pm, v, budget_s=12.0, F_gpu=None):
    """Times the reference's algorithm (oracle restatement) on a bounded sample
    of the workload; with F_gpu (the GPU forces of the same initial state) it
    also reports their relative L2 difference on the sampled bodies."""
    from oracle import oracle as O
    threads = O.default_threads()
    cores = threads + 1                 # workers + the calling thread (CThreadPool layout)
    rec = O.particles_from_soa(pm, v)
    n = w["n"]
    S = w["eps"] ** 2
    rng = np.random.default_rng(0)
    if w["kind"] == 2:
        t0 = time.perf_counter()
        tree = O.OracleTree(rec)
        t_build = time.perf_counter() - t0
        m = 4096
        while True:
            targets = np.sort(rng.choice(n, m, replace=False))
            t0 = time.perf_counter()
            Fo = tree.forces_subset(targets, G=1.0, S=S, theta=w["theta"])
            t_walk = time.perf_counter() - t0
            if t_walk > 2.0 or m >= n:
                break
            m = min(n, m * 4)
        tree.close()
        step_s = t_build + t_walk * n / m
        sample = ("serial octree build of all %d bodies (%.2f s) + traversal of %d sampled bodies on %d threads "
                  "(%.2f s), extrapolated to one step of %d bodies" % (n, t_build, m, threads, t_walk, n))
    else:
        m = min(n, 1024)
        while True:
            targets = np.sort(rng.choice(n, m, replace=False))
            t0 = time.perf_counter()
            Fo = O.direct_forces_subset(rec, targets, G=1.0, S=S)
            t_f = time.perf_counter() - t0
            if t_f > min(2.0, budget_s) or m >= n:
                break
            m = min(n, m * 4)
        step_s = t_f * n / m
        sample = ("direct-sum forces of %d sampled target bodies against all %d sources on %d threads (%.2f s), "
                  "extrapolated to one step of %d bodies" % (m, n, threads, t_f, n))
    out = {"value": n / step_s, "unit": METRIC, "cores": cores, "kind": "port", "sample": sample, "step_s": step_s}
    if F_gpu is not None:
        out["force_rel_l2_gpu_vs_port"] = float(O.rel_l2(F_gpu[targets], Fo))
        out["force_compared_bodies"] = int(len(targets))
    return out


def run_reference(args, name, w):
    """The reference arm: the oracle's restatement of the reference's CPU
    algorithm on all host cores, a bounded sample of the workload per step.
    Loads only oracle/_build/libnb_oracle.so (no CUDA library)."""
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    from oracle import oracle as O
    pm, v = seed_workload(w, replica_seed(0), gen=O)
    vals = []
    base = None
    for i in range(args.warmup + args.steps):
        b = cpu_baseline(w, pm, v)
        if i >= args.warmup:
            vals.append(b["value"])
            base = b
    val = float(np.median(vals)) if vals else 0.0
    out = {"metric": METRIC, "value": val, "unit": METRIC, "impl": "reference", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * w["n"] / val if val else None,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
           "data": "synthetic (seeded galaxies)", "config": workload_config(name, w, args.gpus),
           "cpu_baseline": {"value": val, "unit": METRIC, "cores": base["cores"] if base else None,
                            "kind": "port", "sample": base["sample"] if base else ""},
           "e2e": {"value": val, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))
    return 0


# DRAM bytes per launch of the dominant kernels, from one ncu capture each
# (dram__bytes_read.sum + dram__bytes_write.sum); the summaries under
# profiles/ give the command and the figures.
NCU_TRAFFIC = {
    ("bh1m", "k_traverse"): (86.4e6, "profiles/k_traverse_bh1m.md"),
    ("direct262k", "k_direct_force"): (267.1e6, "profiles/k_direct_force_direct262k.md"),
}


def measure(args, name, w, steps, warmup, world, rank, dev, with_cpu=True, with_e2e=True):
    """One workload on the plain path: K timed steps with the state resident
    (CUDA events on the simulator's stream, L2 flushed before each step), the
    dominant kernel's roofline, FP64 force error and drift, e2e through the
    C-ABI with pinned host records, and the CPU baseline (rank 0).  Returns
    the line's fields."""
    import torch
    import nbody_gb300 as nb

    n = w["n"]
    pm, v = seed_workload(w, replica_seed(rank))
    stream = torch.cuda.Stream(device=dev)
    sim = nb.NBodySim(kind=w["kind"], device=dev, softening2=w["eps"] ** 2, theta=w["theta"],
                      stream=stream.cuda_stream)
    rec_host = nb.records_from_soa(pm, v)
    sim.init(rec_host)
    F_init = sim.compute_forces()      # forces of the initial state, compared with the CPU port below
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    dt = w["dt"]

    diag0 = sim.diagnostics(0.0)       # FP64 energy and angular momentum of the initial state

    # warm-up (untimed)
    for _ in range(warmup):
        sim.step(dt, 1)
    sim.synchronize()

    # ---- device-resident timed region ----
    lib = nb.lib()
    launches0 = ctypes.c_uint64(0)
    lib.nb_launch_count(sim.handle, ctypes.byref(launches0))
    lib.nb_profile_enable(sim.handle, 1)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    clocks = ClockSampler(dev)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    t_wall0 = time.perf_counter()
    with torch.cuda.stream(stream):
        for k in range(steps):
            flush.zero_()                       # L2 flush between timed steps (untimed)
            evs[k][0].record(stream)
            sim.step(dt, 1)
            evs[k][1].record(stream)
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall0
    clk = clocks.stop()
    step_ms = [a.elapsed_time(b) for a, b in evs]
    total_ms = float(sum(step_ms))
    inter_last = sim.last_interactions()
    launches1 = ctypes.c_uint64(0)
    lib.nb_launch_count(sim.handle, ctypes.byref(launches1))
    phases = {}
    names = ["direct_force", "direct_update", "keys", "sort", "topology", "mass", "traverse", "update"]
    for ph, nm in enumerate(names):
        ms = ctypes.c_double(0)
        cnt = ctypes.c_uint64(0)
        lib.nb_profile_read(sim.handle, ph, ctypes.byref(ms), ctypes.byref(cnt))
        if cnt.value:
            phases[nm] = {"ms_total": ms.value, "launches": int(cnt.value), "ms_avg": ms.value / cnt.value}
    lib.nb_profile_enable(sim.handle, 0)
    total_ms = max_over_ranks(total_ms, device="cuda")
    value = replicas_value(world, n, steps, total_ms)
    # drift over the warm-up and timed steps (kick-drift velocities synchronised by half a kick)
    diag1 = sim.diagnostics(0.5 * dt)
    L0, L1 = diag0["angular_momentum"], diag1["angular_momentum"]
    drift = {"energy_rel": (diag1["total"] - diag0["total"]) / abs(diag0["total"]),
             "angular_momentum_rel": float(np.linalg.norm(L1 - L0) / max(np.linalg.norm(L0), 1e-300)),
             "energy_initial": diag0["total"], "steps": warmup + steps, "dt": dt,
             "how": "FP64 reductions on the GPU (kinetic + pairwise potential, L = sum m x × v)"}

    # ---- roofline of the dominant kernel ----
    # Both kernels are bounded by FP32 arithmetic issue, not by HBM: the
    # achieved figure is the interaction arithmetic (20 flops per interaction)
    # per launch over the launch's average CUDA-event time, against the FP32
    # FMA peak measured on this GPU.  The traversal's HBM side is reported
    # beside it: its algorithmic bytes (body read + acceleration write, 32 B
    # per body, plus one read of every tree cell) against the measured copy
    # bandwidth.
    peaks, peak_src = measured_peaks()
    fp32 = ctypes.c_double(0)
    lib.nb_probe_fp32_peak(dev, ctypes.byref(fp32))
    flops = FLOP_PER_INTERACTION * float(inter_last)
    dom = "traverse" if w["kind"] == 2 else "direct_force"
    kname = "k_traverse" if w["kind"] == 2 else "k_direct_force"
    ph = phases.get(dom, {})
    t_launch = ph.get("ms_avg", float("nan")) * 1e-3
    achieved = flops / t_launch / 1e12
    traffic = NCU_TRAFFIC.get((name, kname))
    roof = {"kernel": kname, "bound": "fp32", "achieved": achieved,
            "peak": fp32.value, "unit": "TFLOP/s", "frac": achieved / fp32.value if fp32.value else None,
            "traffic": traffic[0] if traffic else None,
            "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum per launch, " + traffic[1])
            if traffic else None,
            "peak_source": "measured on this GPU by an FMA-chain probe (nb_probe_fp32_peak)",
            "flops_per_launch": flops, "interactions_per_launch": float(inter_last),
            "launch_ms": t_launch * 1e3}
    if w["kind"] == 2:
        stats = sim.tree_stats()
        alg_bytes = 32.0 * n + 48.0 * stats["nodes"]
        roof["hbm"] = {"achieved": alg_bytes / t_launch / 1e9, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                       "frac": alg_bytes / t_launch / 1e9 / peaks["hbm_gbs"], "peak_source": peak_src + " hbm_gbs",
                       "algorithmic_bytes_per_launch": alg_bytes,
                       "logical_node_bytes_per_launch": 16.0 * float(inter_last),
                       "note": "the per-interaction node reads are served from L1/L2"}

    # ---- end-to-end through the C-ABI with pinned host records ----
    e2e = None
    if with_e2e:
        nbytes = n * nb.PARTICLE_DTYPE.itemsize
        pinned = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
        buf = (ctypes.c_char * nbytes).from_address(pinned.data_ptr())
        host = np.frombuffer(buf, dtype=nb.PARTICLE_DTYPE, count=n)
        host[:] = rec_host
        e2e_steps = max(1, min(steps, 5))
        sim.init(host)
        sim.step(dt, 1)
        sim.write_back(host)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            sim.init(host)            # H2D of this step's inputs (104-B records)
            sim.step(dt, 1)
            sim.write_back(host)      # D2H of the result into the records
        torch.cuda.synchronize()
        t_e2e = max_over_ranks(time.perf_counter() - t0, device="cuda")
        e2e = {"value": replicas_value(world, n, e2e_steps, t_e2e * 1e3), "unit": METRIC,
               "h2d_bytes_per_step": n * 104,
               "d2h_bytes_per_step": n * (104 if sim.write_back_direct() else 64), "steps": e2e_steps}

    # ---- force error vs the FP64 oracle on the GPU (sampled targets) ----
    rng = np.random.default_rng(1)
    targets = np.sort(rng.choice(n, min(n, 4096), replace=False)).astype(np.int32)
    F = sim.compute_forces()
    F64 = sim.fp64_forces(targets)
    ferr = float(np.linalg.norm(F[targets] - F64) / np.linalg.norm(F64))
    sim.close()

    cpu = None
    if with_cpu and rank == 0:
        cpu = cpu_baseline(w, pm, v, F_gpu=F_init)
        cpu.pop("step_s", None)
    out = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": steps,
        "warmup": warmup, "ms_per_step": total_ms / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (Kahan-compensated) + f64 diagnostics",
        "data": "synthetic (seeded galaxies)",
        "config": workload_config(name, w, world),
        "roofline": roof, "cpu_baseline": cpu, "e2e": e2e,
        "gpu_launches": int(launches1.value - launches0.value),
        "clocks": clk,
        "interactions_per_step": inter_last,
        "force_rel_l2_vs_fp64": ferr, "force_err_sample": int(len(targets)),
    }
    # The contract's tolerance: direct sum within 1e-5 of the FP64 direct sum;
    # Barnes-Hut within 1e-3 of the reference's own CPU algorithm at the same
    # theta and softening (its monopole, per-body rule errs by a few 1e-3
    # against FP64 at theta = 0.5, which force_rel_l2_vs_fp64 shows).
    if w["kind"] == 2:
        vs_port = cpu.get("force_rel_l2_gpu_vs_port") if cpu else None
        out["force_rel_l2_vs_reference_port"] = vs_port
        out["force_tolerance"] = {
            "against": "the reference's CPU Barnes-Hut (oracle restatement), same theta and softening, "
                       "initial state, sampled bodies", "limit": 1e-3, "value": vs_port,
            "met": (vs_port is not None and vs_port <= 1e-3),
            "fp64_error_of_the_reference_algorithm": ferr}
    else:
        out["force_tolerance"] = {"against": "FP64 direct sum on the GPU, sampled bodies", "limit": 1e-5,
                                  "value": ferr, "met": ferr <= 1e-5}
    out["drift"] = drift
    out["phases_ms_avg"] = {k: v_["ms_avg"] for k, v_ in phases.items()}
    out["wall_s_timed_region"] = t_wall
    return out


def run_ours(args, name, w):
    import torch

    world, rank, local = dist_env()
    dev = local if world > 1 else 0
    torch.cuda.set_device(dev)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    out = measure(args, name, w, args.steps, args.warmup, world, rank, dev,
                  with_cpu=not args.no_cpu_baseline, with_e2e=not args.no_e2e)
    if rank == 0:
        if world == 1 and not args.no_direct and name == "bh1m":
            # the direct-sum configurations, each over its configured step count
            out["direct"] = {}
            for sub in ("direct262k", "direct4096"):
                d = measure(args, sub, WORKLOADS[sub], CONFIG_STEPS[sub], args.warmup, 1, 0, dev,
                            with_cpu=not args.no_cpu_baseline, with_e2e=not args.no_e2e)
                for k in ("metric", "unit", "n_gpus", "higher_is_better", "scaling", "vs_baseline", "data"):
                    d.pop(k, None)
                out["direct"][sub] = d
        out["forms"] = None
        if world == 1 and not args.no_forms:
            out["forms"] = run_forms(args)
        print(json.dumps(out))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_forms(args):
    """The batched (512 galaxies) and served (Poisson stream) forms beside the
    plain path, each against sequential plain launches: at the plain path's
    own theta and at equal accuracy (force error <= 1e-3)."""
    import torch
    import nbody_gb300 as nb
    import bench_forms

    # each form over its configured step count: 100 steps of the 512-galaxy
    # batch, 200 steps per served job
    fargs = argparse.Namespace(steps=bench_forms.BATCH_STEPS, warmup=3, no_cpu_baseline=True)
    out = {}
    b = bench_forms.run_batch(fargs, nb, torch)
    s = bench_forms.run_served(fargs, nb, torch)
    for name, r in (("batch512", b), ("served", s)):
        out[name] = {
            "value": r["value"], "unit": r["unit"], "steps": r["steps"], "config": r["config"],
            "force_rel_l2_vs_fp64": r.get("force_rel_l2_vs_fp64_max", r.get("force_rel_l2_vs_fp64_largest")),
            "sequential_plain": {k: r["sequential_plain"][k] for k in
                                 ("value", "theta", "force_rel_l2_vs_fp64_largest")},
            "speedup_vs_sequential_plain": r["speedup_vs_sequential_plain"],
            "sequential_plain_equal_accuracy": {k: r["sequential_plain_equal_accuracy"][k] for k in
                                                ("value", "theta", "force_rel_l2_vs_fp64_largest")},
            "speedup_vs_sequential_plain_equal_accuracy": r["speedup_vs_sequential_plain_equal_accuracy"],
        }
        for k in ("latency_s", "e2e", "tuning", "makespan_s", "server_timing", "served_equal_accuracy", "gpu_launches"):
            if r.get(k) is not None:
                out[name][k] = r[k]
    out["served"]["sequential_plain_equal_accuracy"]["latency_s"] = \
        s["sequential_plain_equal_accuracy"]["latency_s"]
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="bh1m", choices=sorted(WORKLOADS) + ["batch512", "served", "bh1m_batched"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--requests", type=int, default=200,
                    help="jobs in the served workload's Poisson stream (--workload served)")
    ap.add_argument("--no-forms", action="store_true",
                    help="skip the batched and served forms reported beside the plain-path line")
    ap.add_argument("--no-direct", action="store_true",
                    help="skip the direct-sum configurations reported beside the plain-path line")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    if args.impl == "reference":
        # the CPU arm: the oracle only, neither built nor loaded CUDA library
        if dist_env()[1] != 0:
            return 0
        if args.workload in ("batch512", "served"):
            import bench_forms
            from oracle import oracle as O
            print(json.dumps(bench_forms.reference_line(args, O, args.workload)))
            return 0
        name = "bh1m" if args.workload == "bh1m_batched" else args.workload
        return run_reference(args, name, WORKLOADS[name])
    import nb_build
    nb_build.build()
    if args.workload in ("batch512", "served", "bh1m_batched"):
        import torch
        import nbody_gb300 as nb
        import bench_forms
        if dist_env()[1] != 0:
            return 0
        fn = {"batch512": bench_forms.run_batch, "served": bench_forms.run_served,
              "bh1m_batched": bench_forms.run_batch_single}[args.workload]
        print(json.dumps(fn(args, nb, torch)))
        return 0
    return run_ours(args, args.workload, WORKLOADS[args.workload])


if __name__ == "__main__":
    sys.exit(main())
