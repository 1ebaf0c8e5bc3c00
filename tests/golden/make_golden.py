"""Generates the committed golden fixtures of the N-body step.

The reference holds no golden vectors for this path and cannot run here, so
these fixtures are outputs of the CPU oracle (oracle/nb_oracle.cpp, the
restatement of the reference's BruteForceCPU / BarnesHut / Octree) on small
seeded inputs from this library's seeders.  They pin the oracle and the
seeders against regressions and give the GPU tests fixed expected values.

Run:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "procedural-universe_gb300"))

from oracle import oracle as O  # noqa: E402
import nbody_gb300 as nb  # noqa: E402


def main():
    out = {}
    # Plummer sphere, 256 bodies: direct-sum forces and 10 kick-drift steps.
    pm, v = nb.seed_plummer(11, 256)
    out["plummer256_pos_mass"] = pm
    out["plummer256_vel"] = v
    rec = O.particles_from_soa(pm, v)
    out["plummer256_direct_forces"] = O.direct_forces(rec, G=1.0, S=1e-4)
    after = O.direct_step(rec, 1e-3, 10, G=1.0, S=1e-4)
    out["plummer256_direct_10_pos"] = after["position"]
    out["plummer256_direct_10_vel"] = after["velocity"]

    # Disk + bulge, 512 bodies: octree keys, topology and forces at theta 0.5.
    pm, v = nb.seed_disk(5, 512)
    out["disk512_pos_mass"] = pm
    out["disk512_vel"] = v
    rec = O.particles_from_soa(pm, v)
    t = O.OracleTree(rec)
    keys, depth = t.keys()
    nodes = t.nodes()
    out["disk512_keys"] = keys
    out["disk512_depth"] = depth
    for k in ("level", "count", "first_child", "body", "prefix", "mass", "com", "side", "lo"):
        out["disk512_node_" + k] = nodes[k]
    f, inter = t.forces(G=1.0, S=0.005 ** 2, theta=0.5)
    out["disk512_bh_forces"] = f
    out["disk512_bh_interactions"] = np.array([inter], np.int64)
    t.close()

    np.savez_compressed(os.path.join(HERE, "nbody_small.npz"), **out)
    print("wrote", os.path.join(HERE, "nbody_small.npz"), len(out), "arrays")


if __name__ == "__main__":
    main()
