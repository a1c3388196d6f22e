"""Digest of the PRM roadmap of the 7-DoF DH arm among 16,384 spheres (the large-roadmap workload of
ompl_gb300.workloads.config4), computed on the CPU with the oracle restatement (oracle/port), at
200,000 and at 2,000,000 uniform samples. Writes tests/golden/prm_dh_arm7_digest.json:

  milestones, candidates (connection attempts), edges (accepted), and SHA-256 digests of
  sample_index (int64, little-endian) and of the accepted edges in attempt order, as an (E, 2) int64
  array of (src = neighbour n, dst = new milestone m), following PRM.cpp:570-604.

The GPU roadmap (ompl_gb300.prm.construct_roadmap) must reproduce these digests exactly
(tests/test_gpu_prm.py). Run: python tests/golden/make_prm_digest.py [--threads N]
(about 5 minutes on 8 cores for both sizes)."""
import argparse
import hashlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from ompl_gb300 import workloads as W  # noqa: E402
from oracle.oracle import CheckerDesc, Oracle, SpaceDesc  # noqa: E402

SIZES = (200_000, 2_000_000)


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<i8").tobytes()).hexdigest()


def roadmap_digest(sample_index, edge_src, edge_dst, candidates):
    edges = np.stack([np.asarray(edge_src, dtype=np.int64), np.asarray(edge_dst, dtype=np.int64)], axis=1)
    return {"milestones": int(len(sample_index)), "candidates": int(candidates), "edges": int(len(edges)),
            "sample_index_sha256": digest(sample_index), "edges_sha256": digest(edges)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    args = ap.parse_args()
    port = Oracle.port()
    port.set_threads(args.threads)
    w = W.config4()
    sd = SpaceDesc(w.space_kind, w.dim, lvs_fraction=w.lvs_fraction)
    cd = CheckerDesc(w.checker_kind, w.obstacles, w.dh, w.spheres_per_link, w.sphere_radius)
    out = {"workload": "prm_dh_arm7: 7-DoF DH arm (8 spheres of r 0.05 per link) among 16,384 spheres, wrap-L2 "
                       "joint space, k = 10, segment length 0.01 rad", "seed": int(w.extra["sampler_seed"]),
           "k": 10, "sizes": {}}
    for n in SIZES:
        t = time.time()
        r = port.prm_roadmap(sd, cd, int(w.extra["sampler_seed"]), n, 10)
        out["sizes"][str(n)] = roadmap_digest(r["sample_index"], r["edge_src"], r["edge_dst"], r["candidates"])
        print(n, out["sizes"][str(n)], f"{time.time() - t:.1f} s", flush=True)
    with open(os.path.join(HERE, "prm_dh_arm7_digest.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
