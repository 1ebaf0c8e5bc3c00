"""Batched and served forms of the N-body step, measured for bench.py.

batch512: 512 independent galaxies, particle counts log-uniform in
[256, 65,536], each a Plummer sphere or an exponential disk (coin flip) from
its own seed; Barnes-Hut (group opening test, theta=0.6, quadrupoles) for
n >= 8192, direct sum below; eps=0.01, dt=1e-3.  One launch per phase, the
step replayed from a CUDA graph, tiles and leaf size from the autotuner.
Compared with sequential plain-path launches (one handle per galaxy, the
reference's per-body Barnes-Hut at the same theta, or direct sum) on the
same GPU, and with the CPU restatement of the reference on a 16-galaxy
sample.

served: Poisson arrivals (seeded, 200 per second) of 200 galaxy-generation jobs,
n log-uniform in [1,024, 1,048,576], disk + bulge as in the 1M-body workload, 200 steps each,
Barnes-Hut theta=0.5, admitted against a 120 GB device-memory budget and
stepped together by continuous batching (see nb_server_* in the C-ABI).
"""
from __future__ import annotations

import ctypes
import time

import numpy as np

METRIC = "body-steps/s"
SERVED_REQUESTS = 200   # jobs in the served stream (mean n about 154,000, arrivals over about 1 s)
BATCH_STEPS = 100       # steps of the 512-galaxy batch, as the workload specifies
BATCH = dict(eps2=1e-4, dt=1e-3, theta=0.6, threshold=8192)
SERVED = dict(rate=200.0, steps=200, dt=5e-4, theta=0.5, eps=0.005, max_active=64, steps_per_round=25,
              round_seconds=0.1)


def batch_config(gals):
    """config object of the batch512 lines (both arms)."""
    n_real = sum(pm.shape[0] for pm, _ in gals)
    bh = sum(1 for pm, _ in gals if pm.shape[0] >= BATCH["threshold"])
    return {"workload": "batch512", "galaxies": len(gals), "bodies": n_real,
            "barnes_hut_members": bh, "theta": BATCH["theta"], "eps": 0.01, "dt": BATCH["dt"],
            "l2": "inputs (%.0f MB of state) larger than L2" % (n_real * 64 / 1e6)}


def served_config(requests, sizes, round_seconds):
    """config object of the served lines (both arms)."""
    c = SERVED
    return {"workload": "served", "requests": requests, "rate_per_s": c["rate"], "n_range": [1024, 1 << 20],
            "mean_n": float(sizes.mean()), "steps_per_job": c["steps"], "theta": c["theta"], "eps": c["eps"],
            "dt": c["dt"], "memory_budget_gb": 120, "max_active": c["max_active"],
            "steps_per_round": c["steps_per_round"], "round_seconds": round_seconds,
            "warmup": "one server run of two small jobs (4,096 and 512 bodies, 3 steps) before the stream"}


def batch_galaxies(nb, seed=2024, count=512, lo=256, hi=65536):
    rng = np.random.default_rng(seed)
    ns = np.round(np.exp(rng.uniform(np.log(lo), np.log(hi), count))).astype(int)
    models = rng.integers(0, 2, count)
    gals = []
    for k, (n, m) in enumerate(zip(ns, models)):
        if m == 0:
            gals.append(nb.seed_plummer(seed * 1000 + k, int(n)))
        else:
            gals.append(nb.seed_disk(seed * 1000 + k, int(n), bulge_frac=0.0))
    return gals


PLAIN_THETAS = (0.5, 0.4, 0.35, 0.3, 0.28, 0.26, 0.24, 0.22, 0.2, 0.18, 0.16)


def batched_forces(b, g):
    """Forces of galaxy g as the batched form's steps see them: after one
    evaluation, so that the far field's relative rule (which reads the
    previous accelerations) decides, as it does in every step after the first."""
    b.forces(g)
    return b.forces(g)


def force_error(nb, F, pm, v, eps2, samples=1024, seed=3):
    """Relative L2 error of forces F against the FP64 direct sum on sampled bodies."""
    n = pm.shape[0]
    t = np.sort(np.random.default_rng(seed).choice(n, min(n, samples), replace=False)).astype(np.int32)
    with nb.NBodySim(kind=nb.SIM_BRUTE_FORCE, softening2=eps2) as s:
        s.init_soa(pm, v)
        F64 = s.fp64_forces(t)
    return float(np.linalg.norm(F[t] - F64) / np.linalg.norm(F64))


def plain_theta_for(nb, pm, v, eps2, target=1e-3, refine=4):
    """Largest theta of the plain path (the reference's per-body opening rule)
    whose force error on this galaxy is within target: the first grid value
    that meets it, then bisection towards the next larger grid value (refine
    halvings, so the comparator is not flattered by the grid's spacing)."""
    def err_at(th):
        with nb.NBodySim(kind=nb.SIM_BARNES_HUT, softening2=eps2, theta=th) as s:
            s.init_soa(pm, v)
            return force_error(nb, s.compute_forces(), pm, v, eps2)

    prev = None
    for th in PLAIN_THETAS:
        e = err_at(th)
        if e <= target:
            lo, e_lo, hi = th, e, prev
            for _ in range(refine if hi is not None else 0):
                mid = round(0.5 * (lo + hi), 4)
                e_mid = err_at(mid)
                if e_mid <= target:
                    lo, e_lo = mid, e_mid
                else:
                    hi = mid
            return lo, e_lo
        prev = th
    return PLAIN_THETAS[-1], e


def batched_theta_for(nb, pm, v, eps2, thetas, target=1e-3, refine=3):
    """Largest opening angle of the batched form (group rule, quadrupoles, far
    field) whose force error on this galaxy is within target: the first of the
    descending thetas that meets it, then bisection towards the next larger one."""
    def err_at(th):
        with nb.NBodyBatch(bh_threshold=1024, bh_theta=th, softening2=eps2) as b:
            b.add(pm, v)
            b.commit()
            return force_error(nb, batched_forces(b, 0), pm, v, eps2)

    prev = None
    for th in thetas:
        e = err_at(th)
        if e <= target:
            lo, e_lo, hi = th, e, prev
            for _ in range(refine if hi is not None else 0):
                mid = round(0.5 * (lo + hi), 4)
                e_mid = err_at(mid)
                if e_mid <= target:
                    lo, e_lo = mid, e_mid
                else:
                    hi = mid
            return lo, e_lo
        prev = th
    return thetas[-1], e


def sequential_plain(nb, gals, eps2, dt, theta, threshold, steps=2):
    """Body-steps/s of stepping every galaxy with its own plain handle, one after another."""
    total_t = 0.0
    total_n = 0
    for pm, v in gals:
        n = pm.shape[0]
        kind = nb.SIM_BARNES_HUT if n >= threshold else nb.SIM_BRUTE_FORCE
        with nb.NBodySim(kind=kind, softening2=eps2, theta=theta) as s:
            s.init_soa(pm, v)
            s.step(dt, 1)
            s.synchronize()
            t0 = time.perf_counter()
            s.step(dt, steps)
            s.synchronize()
            total_t += (time.perf_counter() - t0) / steps
        total_n += n
    return total_n / total_t


def cpu_sample(gals, eps2, theta, threshold, count=16, seed=7, budget_s=20.0):
    """The reference's CPU algorithms (oracle restatement) on a galaxy sample
    (at most count galaxies, stopping once budget_s of CPU work is done)."""
    from oracle import oracle as O
    rng = np.random.default_rng(seed)
    pick = rng.choice(len(gals), min(count, len(gals)), replace=False)
    t_tot = 0.0
    n_tot = 0
    done = []
    for g in pick:
        if t_tot > budget_s:
            break
        done.append(g)
        pm, v = gals[g]
        rec = O.particles_from_soa(pm, v)
        t0 = time.perf_counter()
        if pm.shape[0] >= threshold:
            tree = O.OracleTree(rec)
            tree.forces(G=1.0, S=eps2, theta=theta)
            tree.close()
        else:
            O.direct_forces(rec, G=1.0, S=eps2)
        t_tot += time.perf_counter() - t0
        n_tot += pm.shape[0]
    return {"value": n_tot / t_tot, "unit": METRIC, "cores": O.default_threads() + 1, "kind": "port",
            "sample": "%d of the galaxies (%d bodies), one force pass each (Barnes-Hut per-body rule at theta=%.1f "
                      "for n >= %d, direct sum below) on all host cores" % (len(done), n_tot, theta, threshold)}


def served_stream(requests=SERVED_REQUESTS, rate=200.0):
    """Seeded Poisson arrivals and log-uniform job sizes in [1,024, 1,048,576]."""
    rng = np.random.default_rng(5)
    gaps = rng.exponential(1.0 / rate, requests)
    arrivals = np.cumsum(gaps) - gaps[0]
    sizes = np.round(np.exp(rng.uniform(np.log(1024), np.log(1 << 20), requests))).astype(int)
    return arrivals, sizes


def reference_line(args, gen, workload):
    """The reference's CPU algorithms (oracle restatement) on a bounded sample
    of the batched or served workload, as the reference arm's JSON line.  gen
    is the oracle module: its copy of the workload generator gives the same
    galaxies as the GPU arm's."""
    if workload == "batch512":
        gals = batch_galaxies(gen)
        cpu = cpu_sample(gals, BATCH["eps2"], BATCH["theta"], BATCH["threshold"])
        cfg = batch_config(gals)
    else:
        requests = getattr(args, "requests", SERVED_REQUESTS)
        _, sizes = served_stream(requests, SERVED["rate"])
        gals = [gen.seed_disk(10_000 + k, int(n)) for k, n in enumerate(sizes)]
        cpu = cpu_sample(gals, SERVED["eps"] ** 2, SERVED["theta"], 1024, count=len(gals))
        cfg = served_config(requests, sizes, SERVED["round_seconds"])
    return {"metric": METRIC, "value": cpu["value"], "unit": METRIC, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic (seeded)", "config": cfg,
            "cpu_baseline": cpu,
            "e2e": {"value": cpu["value"], "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def run_served(args, nb, torch, requests=None, rate=SERVED["rate"], steps=SERVED["steps"], dt=SERVED["dt"],
               theta=SERVED["theta"], eps=SERVED["eps"]):
    import nbody_serve as ns
    if requests is None:
        requests = getattr(args, "requests", SERVED_REQUESTS)
    arrivals, sizes = served_stream(requests, rate)
    # warm-up: one small Barnes-Hut job and one direct-sum job through a server of
    # the same settings, so that first-use module loading is not in the stream
    with ns.NBodyServer(max_active=64, steps_per_round=25, bh_threshold=1024, softening2=eps * eps,
                        theta=theta) as warm:
        warm.submit(1, 4096, 3, dt, 0)
        warm.submit(2, 512, 3, dt, 0)
        while warm.tick() != (0, 0):
            pass
    def serve(th):
        """The stream through one server at opening angle th: (body-steps/s,
        latencies, makespan, rounds, timing, round seconds)."""
        server = ns.NBodyServer(max_active=64, steps_per_round=25, bh_threshold=1024, softening2=eps * eps, theta=th)
        round_s = server.params.round_seconds
        ids = []
        submitted = 0
        t0 = server.clock()
        while True:
            now = server.clock() - t0
            while submitted < requests and arrivals[submitted] <= now:
                ids.append(server.submit(10_000 + submitted, int(sizes[submitted]), steps, dt, 0))
                submitted += 1
            a, q = server.tick()
            if submitted == requests and a == 0 and q == 0:
                break
            if a == 0 and q == 0:
                time.sleep(max(0.0, arrivals[submitted] - (server.clock() - t0)))
        st = [server.status(i) for i in ids]
        lat = np.array([s["done_s"] - s["submit_s"] for s in st])
        makespan = max(s["done_s"] for s in st) - min(s["submit_s"] for s in st)
        rounds = server.stats()["rounds"]
        timing = server.timing()
        server.close()
        return total / makespan, lat, makespan, rounds, timing, round_s

    total = float(sizes.sum()) * steps
    value, lat, makespan, rounds, timing, server_round_s = serve(theta)
    # sequential plain path: one handle per job (reference per-body Barnes-Hut), FIFO
    def replay(th):
        service = []
        for k, n in enumerate(sizes):
            t0 = time.perf_counter()
            pm, v = nb.seed_disk(10_000 + k, int(n))
            t_gen = time.perf_counter() - t0
            # the job's whole life on its own handle: set-up and first step, the
            # remaining steps (timed over two), and the read-back of its result
            t0 = time.perf_counter()
            with nb.NBodySim(kind=nb.SIM_BARNES_HUT, softening2=eps * eps, theta=th) as s:
                s.init_soa(pm, v)
                s.step(dt, 1)
                s.synchronize()
                t1 = time.perf_counter()
                s.step(dt, 2)
                s.synchronize()
                t2 = time.perf_counter()
                s.read_state()
                t3 = time.perf_counter()
            t_step = (t2 - t1) / 2
            service.append(t_gen + (t1 - t0) + (steps - 1) * t_step + (t3 - t2))
        done, t = [], 0.0
        for arr, sv in zip(arrivals, service):
            t = max(t, arr) + sv
            done.append(t)
        lat = np.array(done) - arrivals
        return total / (done[-1] - arrivals[0]), lat

    seq_value, seq_lat = replay(theta)
    big = int(np.argmax(sizes))
    pm, v = nb.seed_disk(10_000 + big, int(sizes[big]))
    with nb.NBodySim(kind=nb.SIM_BARNES_HUT, softening2=eps * eps, theta=theta) as s:
        s.init_soa(pm, v)
        plain_err = force_error(nb, s.compute_forces(), pm, v, eps * eps)
    with nb.NBodyBatch(bh_threshold=1024, bh_theta=theta, softening2=eps * eps) as b:
        b.add(pm, v)
        b.commit()
        served_err = force_error(nb, batched_forces(b, 0), pm, v, eps * eps)
    th_eq, err_eq = plain_theta_for(nb, pm, v, eps * eps)
    eq_value, eq_lat = replay(th_eq)
    # the served form at equal accuracy too: its opening angle chosen by the same
    # rule as the plain path's (largest job's force error <= 1e-3)
    th_b, err_b = batched_theta_for(nb, pm, v, eps * eps, thetas=(0.65, 0.6, 0.55, 0.5))
    served_eq = None
    if th_b > theta:
        v_b, lat_b, mk_b, _, _, _ = serve(th_b)
        served_eq = {"value": v_b, "unit": METRIC, "theta": th_b, "force_rel_l2_vs_fp64_largest": err_b,
                     "makespan_s": mk_b,
                     "latency_s": {"p50": float(np.percentile(lat_b, 50)), "p99": float(np.percentile(lat_b, 99))},
                     "speedup_vs_sequential_plain_equal_accuracy": v_b / eq_value,
                     "how": "the same stream and server at the largest theta whose batched force error on the "
                            "largest job is <= 1e-3 (grid, then bisection), against sequential_plain_equal_accuracy"}
    return {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": 1, "steps": steps,
        "warmup": 1, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (Kahan-compensated)", "data": "synthetic (seeded galaxies, Poisson arrivals)",
        "config": served_config(requests, sizes, server_round_s),
        "offered": {"value": rate * float(sizes.mean()) * steps, "unit": METRIC},
        "latency_s": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                      "max": float(lat.max())},
        "makespan_s": makespan, "rounds": rounds, "server_timing": timing,
        "gpu_launches": timing["step_launches"],
        "force_rel_l2_vs_fp64_largest": served_err,
        "sequential_plain": {"value": seq_value, "unit": METRIC, "theta": theta,
                             "force_rel_l2_vs_fp64_largest": plain_err,
                             "latency_s": {"p50": float(np.percentile(seq_lat, 50)),
                                           "p99": float(np.percentile(seq_lat, 99))},
                             "how": "each job generated, then created, initialised and stepped once on its own "
                                    "plain Barnes-Hut handle (timed), its other %d steps timed over 2 and scaled, "
                                    "its result read back (timed); FIFO, the same arrivals" % (steps - 1)},
        "speedup_vs_sequential_plain": value / seq_value,
        "sequential_plain_equal_accuracy": {
            "value": eq_value, "unit": METRIC, "theta": th_eq, "force_rel_l2_vs_fp64_largest": err_eq,
            "latency_s": {"p50": float(np.percentile(eq_lat, 50)), "p99": float(np.percentile(eq_lat, 99))},
            "how": "as sequential_plain, at the largest theta whose force error on the largest job is <= 1e-3 "
                   "(grid, then bisection to 0.00125)"},
        "speedup_vs_sequential_plain_equal_accuracy": value / eq_value,
        "served_equal_accuracy": served_eq,
        "cpu_baseline": None,
        "cpu_baseline_note": "not timed for the served stream (hours of CPU work); see the bh1m workload",
    }


def run_batch_single(args, nb, torch, n=1 << 20, theta=0.5, eps=0.005, dt=5e-4):
    """The batched form on the 1M-body disk + bulge galaxy of the plain-path
    workload: the same galaxy, theta and softening, stepped by the group-wise
    traversal with quadrupoles from a CUDA graph."""
    eps2 = eps * eps
    pm, v = nb.seed_disk(1234, n)
    flush = torch.empty((512 << 20) // 4, dtype=torch.float32, device="cuda")

    def timed(th):
        """ms per step (CUDA events, L2 flushed before each step), force error, info, tree stats."""
        stream = torch.cuda.Stream()
        b = nb.NBodyBatch(bh_threshold=1024, bh_theta=th, softening2=eps2, stream=stream.cuda_stream)
        b.add(pm, v)
        b.commit()
        e = force_error(nb, batched_forces(b, 0), pm, v, eps2)
        b.step(dt, args.warmup)
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(args.steps)]
        torch.cuda.synchronize()
        l0 = b.launch_count()
        with torch.cuda.stream(stream):
            for k in range(args.steps):
                flush.zero_()
                evs[k][0].record(stream)
                b.step(dt, 1)
                evs[k][1].record(stream)
        torch.cuda.synchronize()
        t = float(sum(a.elapsed_time(c) for a, c in evs)) / args.steps
        inf, st = b.info(), b.tree_stats()
        inf["launches"] = b.launch_count() - l0
        b.close()
        return t, e, inf, st

    ms, err, info, stats = timed(theta)
    plain = sequential_plain(nb, [(pm, v)], eps2, dt, theta, 2)
    with nb.NBodySim(kind=nb.SIM_BARNES_HUT, softening2=eps2, theta=theta) as s:
        s.init_soa(pm, v)
        plain_err = force_error(nb, s.compute_forces(), pm, v, eps2)
    th_eq, err_eq = plain_theta_for(nb, pm, v, eps2)
    plain_eq = sequential_plain(nb, [(pm, v)], eps2, dt, th_eq, 2)
    # the batched form at equal accuracy too: its theta by the same rule as the plain path's
    th_b, _ = batched_theta_for(nb, pm, v, eps2, thetas=(0.65, 0.6, 0.55, 0.5))
    batched_eq = None
    if th_b > theta:
        ms_b, err_b, _, _ = timed(th_b)
        batched_eq = {"value": n / (ms_b * 1e-3), "unit": METRIC, "theta": th_b, "ms_per_step": ms_b,
                      "force_rel_l2_vs_fp64": err_b, "speedup_vs_plain_equal_accuracy": n / (ms_b * 1e-3) / plain_eq}
    return {
        "metric": METRIC, "value": n / (ms * 1e-3), "unit": METRIC, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (Kahan-compensated)", "data": "synthetic (seeded galaxy)",
        "config": {"workload": "bh1m_batched", "n": n, "theta": theta, "eps": eps, "dt": dt,
                   "l2": "flushed (512 MB write) before every timed step"},
        "gpu_launches": info["launches"],
        "force_rel_l2_vs_fp64": err, "interactions_per_body": info["interactions"] / n,
        "groups": stats["groups"], "bodies_per_group": n / max(1, stats["groups"]),
        "plain": {"value": plain, "theta": theta, "force_rel_l2_vs_fp64": plain_err},
        "plain_equal_accuracy": {"value": plain_eq, "theta": th_eq, "force_rel_l2_vs_fp64": err_eq},
        "speedup_vs_plain": n / (ms * 1e-3) / plain,
        "speedup_vs_plain_equal_accuracy": n / (ms * 1e-3) / plain_eq,
        "batched_equal_accuracy": batched_eq,
    }


def run_batch(args, nb, torch):
    eps2, dt, theta, threshold = BATCH["eps2"], BATCH["dt"], BATCH["theta"], BATCH["threshold"]
    gals = batch_galaxies(nb)
    n_real = sum(pm.shape[0] for pm, _ in gals)
    stream = torch.cuda.Stream()
    b = nb.NBodyBatch(bh_threshold=threshold, bh_theta=theta, softening2=eps2, stream=stream.cuda_stream)
    for pm, v in gals:
        b.add(pm, v)
    t0 = time.perf_counter()
    b.commit()
    t_commit = time.perf_counter() - t0
    t0 = time.perf_counter()
    b.autotune(dt, 2)
    t_tune = time.perf_counter() - t0
    b.step(dt, args.warmup)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    torch.cuda.synchronize()
    launches0 = b.launch_count()
    for k in range(args.steps):
        evs[k][0].record(stream)
        b.step(dt, 1)
        evs[k][1].record(stream)
    torch.cuda.synchronize()
    gpu_launches = b.launch_count() - launches0
    ms = float(sum(a.elapsed_time(c) for a, c in evs))
    value = n_real * args.steps / (ms * 1e-3)
    info = b.info()
    # end to end: whole-batch state from pinned host memory, step, positions back
    pin_pos = torch.empty((n_real, 4), dtype=torch.float32, pin_memory=True)
    pin_vel = torch.empty((n_real, 4), dtype=torch.float32, pin_memory=True)
    hp = pin_pos.numpy()
    hv = pin_vel.numpy()
    b.read_state(hp, hv)
    e2e_steps = max(1, min(args.steps, 5))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        b.write_state(hp, hv)
        b.step(dt, 1)
        b.read_state(hp, None)
    torch.cuda.synchronize()
    t_e2e = time.perf_counter() - t0
    # force error of the Barnes-Hut members vs the FP64 direct sum
    errs = []
    bh_ids = [g for g, (pm, _) in enumerate(gals) if pm.shape[0] >= threshold]
    for g in bh_ids[:8]:
        pm, v = gals[g]
        cur_pm, cur_v = b.read(g)
        F = b.forces(g)
        t = np.arange(0, pm.shape[0], max(1, pm.shape[0] // 1024)).astype(np.int32)
        with nb.NBodySim(kind=nb.SIM_BRUTE_FORCE, softening2=eps2) as s:
            s.init_soa(cur_pm, cur_v)
            F64 = s.fp64_forces(t)
        errs.append(float(np.linalg.norm(F[t] - F64) / np.linalg.norm(F64)))
    tune = b.tuning()
    b.close()
    seq = sequential_plain(nb, gals, eps2, dt, theta, threshold)
    big = max(range(len(gals)), key=lambda g: gals[g][0].shape[0])
    with nb.NBodySim(kind=nb.SIM_BARNES_HUT, softening2=eps2, theta=theta) as s:
        s.init_soa(*gals[big])
        plain_err = force_error(nb, s.compute_forces(), *gals[big], eps2)
    th_eq, err_eq = plain_theta_for(nb, *gals[big], eps2)
    seq_eq = sequential_plain(nb, gals, eps2, dt, th_eq, threshold)
    cpu = None if args.no_cpu_baseline else cpu_sample(gals, eps2, theta, threshold)
    return {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (Kahan-compensated)", "data": "synthetic (seeded galaxies)", "gpu_launches": gpu_launches,
        "config": batch_config(gals),
        "sequential_plain": {"value": seq, "unit": METRIC, "theta": theta,
                             "force_rel_l2_vs_fp64_largest": plain_err,
                             "how": "one plain handle per galaxy, stepped one galaxy after another (2 steps each)"},
        "speedup_vs_sequential_plain": value / seq,
        "sequential_plain_equal_accuracy": {
            "value": seq_eq, "unit": METRIC, "theta": th_eq, "force_rel_l2_vs_fp64_largest": err_eq,
            "how": "as sequential_plain, at the largest theta whose force error on the largest galaxy is <= 1e-3 "
                   "(grid, then bisection to 0.00125)"},
        "speedup_vs_sequential_plain_equal_accuracy": value / seq_eq,
        "force_rel_l2_vs_fp64_max": max(errs) if errs else None, "force_err_galaxies": len(errs),
        "interactions_per_step": info["interactions"], "tuning": tune,
        "e2e": {"value": n_real * e2e_steps / t_e2e, "unit": METRIC, "h2d_bytes_per_step": n_real * 32,
                "d2h_bytes_per_step": n_real * 16, "steps": e2e_steps},
        "cpu_baseline": cpu, "setup_s": {"commit": t_commit, "autotune": t_tune},
    }
