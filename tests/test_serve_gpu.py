"""GPU tests of the served form: continuous batching with admission by a
device-memory budget.  A job's result is the same alone and in the mix
(bit for bit: its state never leaves the device and the batched kernels treat
each galaxy independently), queued jobs enter as slots and memory free up,
and a job that can never fit is rejected."""
import numpy as np
import pytest

import nbody_gb300 as nb
import nbody_serve as ns

pytestmark = pytest.mark.gpu
DT = 5e-4
JOBS = [(11, 3000, 0), (12, 9000, 1), (13, 20000, 0), (14, 1500, 1), (15, 40000, 0), (16, 6000, 0)]


def run_all(server, jobs, steps):
    ids = [server.submit(seed, n, steps, DT, model) for seed, n, model in jobs]
    max_active = 0
    for _ in range(10000):
        a, q = server.tick()
        max_active = max(max_active, a)
        if a == 0 and q == 0:
            break
    return ids, max_active


def test_alone_equals_in_the_mix():
    with ns.NBodyServer(max_active=8, steps_per_round=7, bh_threshold=8192) as mix:
        ids, _ = run_all(mix, JOBS, 30)
        mixed = [mix.result(i) for i in ids]
        for i in ids:
            st = mix.status(i)
            assert st["state"] == 2 and st["steps_done"] == 30
            assert st["submit_s"] <= st["admit_s"] <= st["done_s"]
    for k in (0, 2, 4):
        with ns.NBodyServer(max_active=8, steps_per_round=30, bh_threshold=8192) as alone:
            (i,), _ = run_all(alone, [JOBS[k]], 30)
            pa, va = alone.result(i)
        np.testing.assert_array_equal(pa, mixed[k][0])
        np.testing.assert_array_equal(va, mixed[k][1])


def test_admission_by_memory_budget_and_slots():
    with ns.NBodyServer() as probe:
        per_body = probe.status(probe.submit(1, 1000, 1, DT, 0))["bytes"] / 1000
    budget = int(per_body * 23000)  # room for the 20000-body job plus a small one at a time
    with ns.NBodyServer(memory_budget=budget, max_active=3, steps_per_round=5, bh_threshold=8192) as s:
        ids = [s.submit(seed, n, 10, DT, model) for seed, n, model in JOBS]
        seen = []
        for _ in range(10000):
            a, q = s.tick()
            active_bytes = sum(s.status(i)["bytes"] for i in ids if s.status(i)["state"] == 1)
            assert active_bytes <= budget
            assert a <= 3
            seen.append(a)
            if a == 0 and q == 0:
                break
        states = [s.status(i)["state"] for i in ids]
        assert states[4] == -1                       # 40000 bodies can never fit this budget
        assert all(st == 2 for k, st in enumerate(states) if k != 4)
        assert max(seen) >= 2                        # jobs did share rounds


def test_result_matches_batched_form():
    """A served job is the batched form's galaxy of the same (model, seed, n),
    generated on the device, stepped the same number of steps."""
    seed, n, model = JOBS[2]
    with ns.NBodyServer(max_active=4, steps_per_round=4, bh_threshold=8192) as s:
        (i,), _ = run_all(s, [(seed, n, model)], 12)
        pr, vr = s.result(i)
        assert s.timing()["generate_s"] == 0.0   # nothing of the job was made on the host
        s.release(i)                        # the result is taken: the server forgets the job
        with pytest.raises(nb.NBodyError):
            s.status(i)
    with nb.NBodyBatch(bh_threshold=8192, bh_theta=0.5, softening2=0.005 ** 2) as b:
        b.add_generated(model, seed, n)
        b.commit()
        b.step(DT, 12)
        pb, vb = b.read(0)
    np.testing.assert_array_equal(pr, pb)
    np.testing.assert_array_equal(vr, vb)


def test_round_length_by_time_budget():
    """round_seconds 0: rounds of steps_per_round; a budget below one step:
    one step per round; a large budget: one measuring step, then full rounds."""
    for secs, rounds in ((0.0, 3), (1e-9, 10), (100.0, 4)):
        with ns.NBodyServer(max_active=2, steps_per_round=4, bh_threshold=8192, round_seconds=secs) as s:
            (i,), _ = run_all(s, [JOBS[0]], 10)
            assert s.status(i)["steps_done"] == 10
            assert s.stats()["rounds"] == rounds, (secs, s.stats())
