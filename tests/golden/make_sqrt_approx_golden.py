"""Golden fixture for NearestNeighborsSqrtApprox::nearest, produced by OMPL's own class compiled from the
OMPL source tree (oracle/_ref, built by oracle/ref/Makefile): for RealVector(2), the 10-link kinematic
chain and the wrapped 7-joint space, 1,500 seeded points (added in one call), 120 of them removed one at
a time, then 400 seeded queries made in order. Writes tests/golden/sqrt_approx.npz with the inputs, the
returned rows and distances, and the structure's offset after the queries.

Run: python tests/golden/make_sqrt_approx_golden.py <OMPL source tree>   (or set OMPL_SOURCE_TREE)"""
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle.oracle import (SPACE_KINEMATIC_CHAIN, SPACE_REAL_VECTOR, SPACE_WRAP_L2, Oracle,  # noqa: E402
                           SpaceDesc, build_reference)

CASES = {"rv2": (SPACE_REAL_VECTOR, 2, 0.0), "chain10": (SPACE_KINEMATIC_CHAIN, 10, 0.1),
         "wrap7": (SPACE_WRAP_L2, 7, 0.0)}


def space(kind, dim, link):
    if kind == SPACE_REAL_VECTOR:
        return SpaceDesc(kind, dim, np.zeros(dim), np.ones(dim))
    if kind == SPACE_KINEMATIC_CHAIN:
        return SpaceDesc(kind, dim, link_length=link)
    return SpaceDesc(kind, dim)


def main(tree):
    if build_reference(tree) is None:
        sys.exit("no OMPL source tree at " + str(tree))
    ref = Oracle.reference()
    out = {}
    for i, (name, (kind, dim, link)) in enumerate(CASES.items()):
        rng = np.random.default_rng(40 + i)
        lo, hi = (0.0, 1.0) if kind == SPACE_REAL_VECTOR else (-math.pi, math.pi)
        pts = rng.uniform(lo, hi, size=(1500, dim))
        q = rng.uniform(lo, hi, size=(400, dim))
        rem = rng.choice(1500, size=120, replace=False).astype(np.int64)
        idx, dist, off = ref.nn_sqrt_approx(space(kind, dim, link), pts, q, rem)
        out.update({f"{name}_pts": pts, f"{name}_q": q, f"{name}_remove": rem, f"{name}_idx": idx,
                    f"{name}_dist": dist, f"{name}_offset": np.int64(off)})
    np.savez_compressed(os.path.join(HERE, "sqrt_approx.npz"), **out)
    print("wrote", os.path.join(HERE, "sqrt_approx.npz"))


if __name__ == "__main__":
    tree = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("OMPL_SOURCE_TREE")
    if not tree:
        sys.exit("usage: make_sqrt_approx_golden.py <OMPL source tree> (or set OMPL_SOURCE_TREE)")
    main(tree)
