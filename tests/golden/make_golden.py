"""Generate the golden fixtures in tests/golden/ by running OMPL's OWN code.

Requires the OMPL source tree (argv[1], or $OMPL_SOURCE_TREE): the script builds
oracle/_ref/libompl_ref.so from those sources (oracle/ref/Makefile) and records inputs and the
reference's outputs as small .npz files. The CPU restatement (oracle/liboracle.so) is then pinned
against these files by tests/test_oracle_golden.py on every machine, including ones without the
source tree.

Inputs are seeded numpy draws, plus two of OMPL's own test/demo worlds read from the tree:
tests/resources/circle_obstacles.txt + circle_queries.txt (the 2D circles planning tests) and the
"horn" segment world that demos/KinematicChain.h:279-315 builds (obtained by calling the compiled
demo header).
"""
from __future__ import annotations

import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.oracle import (CHECK_CHAIN_SEGMENTS, CHECK_CIRCLES, CHECK_DH_SPHERES, NN_REF_GNAT,  # noqa: E402
                           NN_REF_GNAT_NTS, NN_REF_LINEAR, NN_REF_SQRT_APPROX, SPACE_KINEMATIC_CHAIN,
                           SPACE_REAL_VECTOR, SPACE_SO2, SPACE_WRAP_L2, CheckerDesc, Oracle, SpaceDesc,
                           build_reference)
from ompl_gb300 import workloads as W  # noqa: E402

PI = math.pi


def space_dict(sp: SpaceDesc):
    return dict(space_kind=sp.kind, dim=sp.dim, low=np.asarray(sp.low if sp.low is not None else np.zeros(sp.dim)),
                high=np.asarray(sp.high if sp.high is not None else np.zeros(sp.dim)), link_length=sp.link_length,
                lvs_fraction=sp.lvs_fraction, factor=sp.factor)


def checker_dict(ck: CheckerDesc):
    return dict(checker_kind=ck.kind, obstacles=np.asarray(ck.obstacles),
                dh=np.asarray(ck.dh if ck.dh is not None else np.zeros((0, 3))),
                spheres_per_link=ck.spheres_per_link, sphere_radius=ck.sphere_radius)


def load_circles(tree):
    rows = []
    with open(os.path.join(tree, "tests/resources/circle_obstacles.txt")) as f:
        lines = f.read().split("\n")[2:]
    for ln in lines:
        p = ln.split()
        if len(p) == 4:
            rows.append([float(p[1]), float(p[2]), float(p[3])])
    circles = np.array(rows)
    q = []
    with open(os.path.join(tree, "tests/resources/circle_queries.txt")) as f:
        toks = f.read().split()
    for i in range(0, len(toks) - 7, 8):
        q.append([float(toks[i + 2]), float(toks[i + 3]), float(toks[i + 6]), float(toks[i + 7])])
    return circles, np.array(q)


def horn_environment(R, d, eps):
    """createHornEnvironment(d, eps) of demos/KinematicChain.h:279-315, run from the compiled demo header
    (it also writes environment_<d>.dat, so it runs inside a temporary directory)."""
    import ctypes as C
    import tempfile
    fn = R.lib.ora_ref_horn_environment
    fn.restype = C.c_long
    buf = np.zeros((4 * d, 4))
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as tmp:
        os.chdir(tmp)
        try:
            n = fn(C.c_uint(d), C.c_double(eps), buf.ctypes.data_as(C.POINTER(C.c_double)), C.c_long(buf.shape[0]))
        finally:
            os.chdir(cwd)
    return np.ascontiguousarray(buf[:n])


def motion_case(R, sp, ck, s1, s2):
    m = R.check_motion(sp, ck, s1, s2)
    return dict(s1=s1, s2=s2, ok=m["ok"], ok_bisect=m["ok_bisect"], last_t=m["last_t"], last_state=m["last_state"],
                nd=m["nd"], first_j=m["first_j"])


def main(tree):
    if build_reference(tree) is None:
        raise SystemExit(f"OMPL source tree not found at {tree}")
    R = Oracle.reference()
    rng = np.random.default_rng(12345)
    out = {}

    # RNG / samplers (RandomNumbers.h:66-76, RealVectorStateSpace.cpp:45-65, SO2StateSpace.cpp:46-56)
    seeds = np.array([1, 42, 1000000000, 4294967295], dtype=np.uint64)
    out["rng"] = dict(seeds=seeds, u01=np.stack([R.rng_uniform(int(s), 2000) for s in seeds]),
                      upi=np.stack([R.rng_uniform(int(s), 2000, -PI, PI) for s in seeds]))
    spaces = {
        "rv2": SpaceDesc(SPACE_REAL_VECTOR, 2, np.zeros(2), np.ones(2), lvs_fraction=0.01),
        "rv7": SpaceDesc(SPACE_REAL_VECTOR, 7, np.array([-3, -2, -1, 0, -0.5, -PI, 1.0]),
                         np.array([3, 2, 1, 5, 0.5, PI, 1.5]), lvs_fraction=0.003, factor=2),
        "so2": SpaceDesc(SPACE_SO2, 1, lvs_fraction=0.05),
        "chain10": SpaceDesc(SPACE_KINEMATIC_CHAIN, 10, link_length=0.1, lvs_fraction=0.005),
        "wrap7": SpaceDesc(SPACE_WRAP_L2, 7, lvs_fraction=0.01 / math.sqrt(7 * PI * PI)),
    }
    # sampleGaussian calls interleaved with sampleUniform on one RNG (RealVectorStateSpace.cpp:67-82,
    # SO2StateSpace.cpp:58-62, RandomNumbers.h:98-101): odd call sizes carry the cached normal value
    gauss_ops = [("gaussian", 151), ("uniform", 3), ("gaussian", 100), ("gaussian", 1), ("uniform", 2),
                 ("gaussian", 147)]
    grng = np.random.default_rng(777)
    for name, sp in spaces.items():
        lo = np.asarray(sp.low) if sp.kind == SPACE_REAL_VECTOR else np.full(sp.dim, -PI)
        hi = np.asarray(sp.high) if sp.kind == SPACE_REAL_VECTOR else np.full(sp.dim, PI)
        a = rng.uniform(lo, hi, size=(600, sp.dim))
        b = rng.uniform(lo, hi, size=(600, sp.dim))
        b[:20] = a[:20]                      # identical endpoints: distance 0, nd 0
        t = rng.uniform(0, 1, size=600)
        t[:5] = [0.0, 1.0, 0.5, 0.25, 1.0 / 3.0]
        near = rng.uniform(lo, hi, size=(300, sp.dim))
        wide = (hi - lo) * 3.0 if sp.kind != SPACE_SO2 else np.full(1, 20.0)
        out_of_bounds = rng.uniform(lo - wide, hi + wide, size=(300, sp.dim))
        out[f"space_{name}"] = dict(
            **space_dict(sp), extent=R.extent(sp), lvs=R.lvs(sp), a=a, b=b, t=t,
            distance=R.distance(sp, a, b), interpolate=R.interpolate(sp, a, b, t),
            valid_segment_count=R.valid_segment_count(sp, a, b),
            sample_seed=7, sample=R.sample_uniform(sp, 7, 700),
            near=near, near_distance=0.3, sample_near=R.sample_uniform_near(sp, 11, near, 0.3),
            oob=out_of_bounds, enforce=R.enforce_bounds(sp, out_of_bounds))
        gmean = grng.uniform(lo, hi, size=(399, sp.dim))
        out[f"space_{name}"].update(
            gauss_kinds=np.array([1 if k == "gaussian" else 0 for k, _ in gauss_ops]),
            gauss_counts=np.array([c for _, c in gauss_ops]), gauss_seed=5, gauss_mean=gmean, gauss_stddev=0.4,
            gauss_out=R.sample_script(sp, 5, gauss_ops, gmean, 0.4))

    # Workload-0 circles world (seeded), checked with the reference DiscreteMotionValidator.
    w0 = W.config0(seed=0, n_states=3000, n_edges=3000, n_queries=300)
    sp0 = SpaceDesc(w0.space_kind, 2, w0.low, w0.high, lvs_fraction=w0.lvs_fraction)
    ck0 = CheckerDesc(CHECK_CIRCLES, w0.obstacles)
    out["circles_seeded"] = dict(**space_dict(sp0), **checker_dict(ck0), states=w0.states,
                                 valid=R.is_valid(sp0, ck0, w0.states), **motion_case(R, sp0, ck0, w0.s1, w0.s2))

    # OMPL's own 2D circles test world and queries (tests/resources, 2DcirclesSetup.h:78-88:
    # bounds = the circles' bounding box, resolution 0.002).
    circles, queries = load_circles(tree)
    lo = np.array([np.min(circles[:, 0] - circles[:, 2]), np.min(circles[:, 1] - circles[:, 2])])
    hi = np.array([np.max(circles[:, 0] + circles[:, 2]), np.max(circles[:, 1] + circles[:, 2])])
    spc = SpaceDesc(SPACE_REAL_VECTOR, 2, lo, hi, lvs_fraction=0.002)
    ckc = CheckerDesc(CHECK_CIRCLES, circles)
    st = rng.uniform(lo, hi, size=(2000, 2))
    out["circles_ompl_tests"] = dict(**space_dict(spc), **checker_dict(ckc), states=st, valid=R.is_valid(spc, ckc, st),
                                     **motion_case(R, spc, ckc, queries[:, :2].copy(), queries[:, 2:].copy()))

    # Workload-1 kinematic chain (seeded segment world) and the demo's horn world.
    w1 = W.config1(seed=1, n_states=200_000, n_edges=10, n_queries=10)
    sp1 = SpaceDesc(SPACE_KINEMATIC_CHAIN, 10, link_length=0.1, lvs_fraction=0.005)
    ck1 = CheckerDesc(CHECK_CHAIN_SEGMENTS, w1.obstacles)
    v1 = R.is_valid(sp1, ck1, w1.states[:4000])
    full_valid = R.is_valid(sp1, ck1, w1.states)
    vs = w1.states[full_valid == 1]
    i = rng.integers(0, len(vs), 600)
    j = rng.integers(0, len(vs), 600)
    s1 = np.vstack([vs[i], w1.states[:200]])
    s2 = np.vstack([vs[j], w1.states[200:400]])
    out["chain_seeded"] = dict(**space_dict(sp1), **checker_dict(ck1), states=w1.states[:4000], valid=v1,
                               valid_states=vs, **motion_case(R, sp1, ck1, s1, s2))
    horn = horn_environment(R, 10, math.log(10.0) / 10.0)
    sph = SpaceDesc(SPACE_KINEMATIC_CHAIN, 10, link_length=0.1, lvs_fraction=0.01)
    ckh = CheckerDesc(CHECK_CHAIN_SEGMENTS, horn)
    # start/goal of demos/KinematicChainBenchmark.cpp:53-58 plus random states
    start = np.full(10, PI / 10.0)
    start[0] = 0.0
    goal = np.zeros(10)
    goal[0] = PI - 0.001
    sth = np.vstack([start, goal, rng.uniform(-0.6, 0.6, size=(1998, 10))])
    e1 = np.vstack([start, sth[2:300]])
    e2 = np.vstack([goal, sth[300:598]])
    out["chain_horn"] = dict(**space_dict(sph), **checker_dict(ckh), states=sth, valid=R.is_valid(sph, ckh, sth),
                             **motion_case(R, sph, ckh, e1, e2))

    # DH sphere arm (definition shared by both oracle builds).
    w2 = W.config2(seed=2, n_edges=120, n_world=512)
    sp2 = SpaceDesc(SPACE_REAL_VECTOR, 7, w2.low, w2.high, lvs_fraction=0.02)
    ck2 = CheckerDesc(CHECK_DH_SPHERES, w2.obstacles, dh=w2.dh, spheres_per_link=8, sphere_radius=0.05)
    st2 = rng.uniform(-PI, PI, size=(600, 7))
    out["dh_arm"] = dict(**space_dict(sp2), **checker_dict(ck2), states=st2, valid=R.is_valid(sp2, ck2, st2),
                         **motion_case(R, sp2, ck2, st2[:120], st2[120:240]))

    # Nearest neighbours: reference Linear (exact) + GNAT, nearestK and nearestR.
    for name, sp, n, nq, k, r in (("rv2", spaces["rv2"], 3000, 200, 10, 0.05),
                                  ("chain10", spaces["chain10"], 2000, 60, 16, 1.2),
                                  ("wrap7", spaces["wrap7"], 3000, 100, 10, 3.0)):
        lo = np.asarray(sp.low) if sp.kind == SPACE_REAL_VECTOR else np.full(sp.dim, -PI)
        hi = np.asarray(sp.high) if sp.kind == SPACE_REAL_VECTOR else np.full(sp.dim, PI)
        pts = rng.uniform(lo, hi, size=(n, sp.dim))
        q = np.vstack([rng.uniform(lo, hi, size=(nq - 5, sp.dim)), pts[:5]])  # 5 queries hit a point exactly
        li, ld = R.knn(sp, pts, q, k, NN_REF_LINEAR)
        gi, gd = R.knn(sp, pts, q, k, NN_REF_GNAT)
        ni, nd_ = R.knn(sp, pts, q, k, NN_REF_GNAT_NTS)
        si, sd = R.knn(sp, pts, q, k, NN_REF_SQRT_APPROX)
        big_i, big_d = R.knn(sp, pts[:50], q[:10], 80, NN_REF_LINEAR)   # k > size: everything, sorted
        rc, ri, rd = R.radius(sp, pts, q, r, NN_REF_LINEAR)
        grc, gri, grd = R.radius(sp, pts, q, r, NN_REF_GNAT)
        limit = np.sort(rng.integers(0, n, size=nq))
        pi_, pd_ = R.knn_prefix(sp, pts, q, limit, k)
        out[f"knn_{name}"] = dict(**space_dict(sp), pts=pts, q=q, k=k, r=r, linear_idx=li, linear_dist=ld,
                                  gnat_idx=gi, gnat_dist=gd, gnat_nts_dist=nd_, sqrt_dist=sd, big_idx=big_i,
                                  big_dist=big_d, radius_counts=rc, radius_idx=ri, radius_dist=rd,
                                  gnat_radius_counts=grc, gnat_radius_dist=grd, prefix_limit=limit,
                                  prefix_idx=pi_, prefix_dist=pd_)

    # SpaceInformation::checkMotion(states, count, firstInvalid) and getMotionStates.
    ms = []
    for c in range(40):
        count = int(rng.integers(0, 40))
        a = rng.uniform(0, 1, size=(1, 2))
        b = rng.uniform(0, 1, size=(1, 2))
        for endpoints in (0, 1):
            ms.append((a, b, count, endpoints, R.get_motion_states(sp0, a, b, count, endpoints)))
    states_list = [m[4] for m in ms]
    cm = [R.check_motion_states(sp0, ck0, s) for s in states_list]
    out["motion_states"] = dict(
        **space_dict(sp0), **checker_dict(ck0), a=np.vstack([m[0] for m in ms]), b=np.vstack([m[1] for m in ms]),
        count=np.array([m[2] for m in ms]), endpoints=np.array([m[3] for m in ms]),
        lengths=np.array([len(s) for s in states_list]), states=np.vstack(states_list),
        ok=np.array([c[0] for c in cm]), first_invalid=np.array([c[1] for c in cm]), ok_bisect=np.array([c[2] for c in cm]))

    for name, d in out.items():
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **d)
    print("wrote", len(out), "fixtures to", HERE)


if __name__ == "__main__":
    tree = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("OMPL_SOURCE_TREE")
    if not tree:
        sys.exit("usage: make_golden.py <OMPL source tree> (or set OMPL_SOURCE_TREE)")
    main(tree)
