"""RRTConnect-shaped clients of the request loop (ompl_gb300/rrt.py, RRTConnect.cpp:116-330): each client's
trees, requests and solution are the same when the clients run one after the other as when they run
together (their requests overlapping in the request loop), and the same as a replay of the algorithm on
the CPU with the oracle's nearest neighbour, isValid and checkMotion."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from ompl_gb300 import base as B  # noqa: E402
from ompl_gb300 import rrt  # noqa: E402
from ompl_gb300 import serve  # noqa: E402
from ompl_gb300 import workloads as W  # noqa: E402
from oracle.oracle import CheckerDesc, SpaceDesc  # noqa: E402

LVS_FRACTION = 1.0 / 2500.0
DH = W.dh_arm(np.random.default_rng(2))
LO, HI = np.full(7, -math.pi), np.full(7, math.pi)
RANGE = 0.2 * math.sqrt(7 * (2 * math.pi) ** 2)  # SelfConfig's default range: 0.2 of the space's extent


def client_setup(c, port):
    crng = np.random.default_rng(900 + c)
    world = W.sphere_world(crng, int(crng.integers(1024, 4097)))
    sd = SpaceDesc(0, 7, LO, HI, lvs_fraction=LVS_FRACTION)
    cd = CheckerDesc(3, world, DH, 8, 0.05)
    cand = crng.uniform(-math.pi, math.pi, size=(400, 7))
    ok = port.is_valid(sd, cd, cand).astype(bool)
    start, goal = cand[ok][0], cand[ok][1]
    return world, sd, cd, start, goal


def make_clients(srv, setups, seeds):
    out = []
    for (world, _, _, start, goal), seed in zip(setups, seeds):
        space = B.RealVectorStateSpace(7, LO, HI)
        space.setLongestValidSegmentFraction(LVS_FRACTION)
        ck = B.DHSphereArmValidityChecker(space, DH, world, 8, 0.05)
        ck.setPrecision("fp32_guarded")
        out.append(rrt.RRTConnectClient(srv, ck, start, goal, seed, RANGE))
    return out


def oracle_replay(port, sd, cd, start, goal, seed, max_iterations):
    """The client's algorithm on the CPU: nearest = oracle nearestK(1) over the tree's states."""
    rng = np.random.default_rng(seed)
    trees = {True: [start.copy()], False: [goal.copy()]}
    trace = []

    def grow(is_start, rstate):
        pts = np.array(trees[is_start])
        idx, dist = port.knn(sd, pts, rstate.reshape(1, -1), 1)
        nk, d = int(idx[0, 0]), float(dist[0, 0])
        nstate = pts[nk]
        reach, dstate = True, rstate
        if d > RANGE:
            dstate = nstate + (rstate - nstate) * (RANGE / d)
            if np.array_equal(dstate, nstate):
                trace.append((is_start, nk, None, rrt.TRAPPED))
                return rrt.TRAPPED, -1
            reach = False
        if is_start:
            ok = bool(port.check_motion(sd, cd, nstate, dstate, want_state=False, want_bisect=False)["ok"][0])
        else:
            ok = bool(port.is_valid(sd, cd, dstate)[0]) and \
                bool(port.check_motion(sd, cd, dstate, nstate, want_state=False, want_bisect=False)["ok"][0])
        if not ok:
            trace.append((is_start, nk, None, rrt.TRAPPED))
            return rrt.TRAPPED, -1
        trees[is_start].append(dstate.copy())
        trace.append((is_start, nk, dstate.copy(), rrt.REACHED if reach else rrt.ADVANCED))
        return (rrt.REACHED if reach else rrt.ADVANCED), len(trees[is_start]) - 1

    start_tree = True
    for _ in range(max_iterations):
        is_start = start_tree
        start_tree = not start_tree
        rstate = (HI - LO) * rng.random(7) + LO
        gs, key = grow(is_start, rstate)
        if gs == rrt.TRAPPED:
            continue
        target = trees[is_start][key]
        gsc, _ = grow(not is_start, target)
        while gsc == rrt.ADVANCED:
            gsc, _ = grow(not is_start, target)
        if gsc == rrt.REACHED:
            break
    return trace


def same_trace(a, b):
    return len(a) == len(b) and all(x[0] == y[0] and x[1] == y[1] and x[3] == y[3] and
                                    ((x[2] is None and y[2] is None) or np.array_equal(x[2], y[2]))
                                    for x, y in zip(a, b))


def test_rrtconnect_clients_alone_equal_mix_and_oracle(port):
    port.set_threads(16)
    n, iters = 16, 60
    setups = [client_setup(c, port) for c in range(n)]
    seeds = [7000 + c for c in range(n)]
    srv = serve.Server(n_streams=16, arena_bytes=1 << 30)
    alone = make_clients(srv, setups, seeds)
    rrt.run_clients(alone, iters, concurrent=False)
    mix = make_clients(srv, setups, seeds)
    rrt.run_clients(mix, iters, concurrent=True)
    assert srv.stats()["max_concurrent"] > 1
    srv.close()
    for a, m in zip(alone, mix):
        assert same_trace(a.trace, m.trace)
        assert a.solution == m.solution
    assert sum(c.solution is not None for c in alone) > 0
    for c in range(3):
        _, sd, cd, start, goal = setups[c]
        ref = oracle_replay(port, sd, cd, start, goal, seeds[c], iters)
        assert same_trace(alone[c].trace, ref), c
