"""The bench's two arms see the same workload.

The reference arm (`bench.py --impl reference`) times the oracle's
restatement of the reference's CPU algorithm.  It must not build or load the
CUDA library, and it must step the same initial state as the GPU arm: the
oracle carries its own copy of the workload generator, compiled from the same
source file, and the two copies must agree byte for byte.  Its config object
must equal the GPU arm's.
"""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

import nbody_gb300 as nb
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("model,seed,n", [("plummer", 1234, 4096), ("collision", 1234, 262144),
                                          ("disk", 1234, 100_000), ("disk", 10_017, 3000)])
def test_workload_generators_byte_identical(model, seed, n):
    a = getattr(O, "seed_" + model)(seed, n)
    b = getattr(nb, "seed_" + model)(seed, n)
    for x, y in zip(a, b):
        assert x.dtype == y.dtype == np.float32 and x.shape == y.shape == (n, 4)
        np.testing.assert_array_equal(x.view(np.uint32), y.view(np.uint32))


def test_batch_galaxies_identical_through_either_generator():
    import bench_forms
    ga = bench_forms.batch_galaxies(O, count=24)
    gb = bench_forms.batch_galaxies(nb, count=24)
    for (pa, va), (pb, vb) in zip(ga, gb):
        np.testing.assert_array_equal(pa.view(np.uint32), pb.view(np.uint32))
        np.testing.assert_array_equal(va.view(np.uint32), vb.view(np.uint32))
    assert bench_forms.batch_config(ga) == bench_forms.batch_config(gb)


def test_reference_arm_loads_only_the_oracle():
    code = ("import sys; sys.path.insert(0, %r); sys.argv = ['bench.py', '--impl', 'reference', '--workload', "
            "'direct4096', '--steps', '1', '--warmup', '3']\n"
            "import bench\n"
            "bench.main()\n"
            "maps = open('/proc/self/maps').read()\n"
            "print(json.dumps({'product': 'libnbody_gb300' in maps, 'oracle': 'libnb_oracle' in maps}))\n"
            % ROOT).replace("import bench\n", "import bench, json\n")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(x) for x in r.stdout.strip().splitlines()]
    line, maps = lines[0], lines[1]
    assert maps == {"product": False, "oracle": True}
    import bench
    assert line["impl"] == "reference"
    assert line["config"] == bench.workload_config("direct4096", bench.WORKLOADS["direct4096"], 1)
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["value"] > 0
