"""Device memory of the library comes from a pool per device that keeps
freed memory for the next allocation.  Creating and destroying the same
handles again must reuse it: the device's free memory settles after the
first round instead of falling round after round (no leak), and a served
server that rebuilds its batch many times stays within the same footprint."""
import numpy as np
import pytest
import torch

import nbody_gb300 as nb
import nbody_serve as ns

pytestmark = pytest.mark.gpu


def free_bytes():
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


def test_handles_reuse_pool_memory():
    pm, v = nb.seed_disk(3, 300_000)
    small = [nb.seed_plummer(10 + k, 3000 + 500 * k) for k in range(6)]
    seen = []
    for _ in range(4):
        with nb.NBodySim(kind=nb.SIM_BARNES_HUT, softening2=0.005 ** 2) as s:
            s.init_soa(pm, v)
            s.step(5e-4, 2)
        with nb.NBodyBatch(bh_threshold=1024, bh_theta=0.5, softening2=0.005 ** 2) as b:
            b.add(pm, v)
            for p, w in small:
                b.add(p, w)
            b.commit()
            b.step(5e-4, 2)
        seen.append(free_bytes())
    # after the first round the pool holds what the handles need: later rounds
    # take no new device memory (64 MB of slack for the runtime)
    assert min(seen[1:]) >= seen[0] - (64 << 20), [x >> 20 for x in seen]


def test_server_rebuilds_stay_within_footprint():
    seen = []
    with ns.NBodyServer(max_active=3, steps_per_round=2, bh_threshold=8192) as s:
        ids = [s.submit(100 + k, 20_000 + 1000 * (k % 4), 4, 5e-4, k % 2) for k in range(12)]
        for _ in range(10000):
            a, q = s.tick()
            seen.append(free_bytes())
            if a == 0 and q == 0:
                break
        assert all(s.status(i)["state"] == 2 for i in ids)
        assert s.timing()["rebuilds"] >= 4
    half = len(seen) // 2
    assert min(seen[half:]) >= min(seen[:half]) - (64 << 20), (min(seen[:half]) >> 20, min(seen[half:]) >> 20)
