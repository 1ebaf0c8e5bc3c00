"""Generates the committed golden fixtures of the N-body step.

reference_small.npz -- outputs of the reference's own CPU code: its
  src/Sim/Octree.cpp, BarnesHut.cpp and BruteForceCPU.cpp compiled unmodified
  (oracle/ref/Makefile, type-only stand-ins for the DirectXTK / Direct3D
  headers) and run through oracle/ref/ref_harness.cpp.  The reference holds
  no golden vectors of its own for this path; these are made by running it.
  Inputs come from this library's restatement of the reference's seeders
  (Galaxy and Random distributions, masses rounded to float); constants are
  the reference's (G = 6.674e-11, S = 10, drift divisor 2.3e13, root cube
  +-4000).  Contents: the octree of a 2,100-body galaxy (every node, depth
  first) and of the 512-body disk of nbody_small.npz, CalculateForce of every
  body at theta 0.5 and 1.0, one BarnesHut::Update, two BruteForceCPU::Update
  of a 2,100-body random cloud.  2,100 is a multiple of the reference thread
  pool's worker count on the generating machine (7), so the pool's
  remainder slice is empty and every body's force is computed.
nbody_small.npz -- outputs of the CPU oracle (oracle/nb_oracle.cpp) at the
  N-body units of the workloads (G = 1, S = eps^2); the oracle is pinned to
  the reference build by tests/test_reference_pin_cpu.py.

Run:  python tests/golden/make_golden.py   (needs the reference sources)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "procedural-universe_gb300"))

from oracle import oracle as O  # noqa: E402
from oracle import reference_build as R  # noqa: E402
import nbody_gb300 as nb  # noqa: E402

REF_N = 2100
REF_DT = 1.0


def reference_inputs():
    """The two reference-unit inputs, masses rounded to float."""
    gal = nb.seed_reference(nb.SEEDER_GALAXY, 21, REF_N)
    rnd = nb.seed_reference(nb.SEEDER_RANDOM, 22, REF_N)
    for r in (gal, rnd):
        r["mass"] = r["mass"].astype(np.float32).astype(np.float64)
        r["forces"] = 0.0
    return gal, rnd


def reference_fixture(disk512_pm, disk512_vel):
    """Every array of reference_small.npz, computed by the reference build."""
    out = {}
    gal, rnd = reference_inputs()
    out["galaxy_records"] = gal
    t = R.RefOctree(gal)
    for k, v in t.nodes().items():
        out["galaxy_node_" + k] = v
    out["galaxy_forces_t05"] = t.forces(theta=0.5)
    out["galaxy_forces_t10"] = t.forces(theta=1.0)
    out["galaxy_max_depth"] = np.array([t.max_depth()], np.int32)
    t.close()
    out["galaxy_bh_update"] = R.bh_update(gal, REF_DT, 0.5, 1)
    out["random_records"] = rnd
    out["random_bf_update2"] = R.bf_update(rnd, REF_DT, 2)
    d = O.particles_from_soa(disk512_pm, disk512_vel)
    t = R.RefOctree(d)
    for k, v in t.nodes().items():
        out["disk512_node_" + k] = v
    out["disk512_max_depth"] = np.array([t.max_depth()], np.int32)
    t.close()
    out["meta"] = np.array([R.G, R.S, R.STAR_SYSTEM_SCALE, REF_DT, R.workers()], np.float64)
    return out


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

    if REF_N % R.workers() != 0:
        raise SystemExit("the reference pool here has %d workers; REF_N must be a multiple" % R.workers())
    ref = reference_fixture(out["disk512_pos_mass"], out["disk512_vel"])
    np.savez_compressed(os.path.join(HERE, "reference_small.npz"), **ref)
    print("wrote", os.path.join(HERE, "reference_small.npz"), len(ref), "arrays")


if __name__ == "__main__":
    main()
