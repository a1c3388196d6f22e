"""RRTConnect-shaped planner clients of the request loop (geometric/planners/rrt/src/RRTConnect.cpp).

Each client keeps two trees (start and goal), each a device-resident NearestNeighborsGPU index plus the
host-side parent links, and runs RRTConnect::solve's iteration (RRTConnect.cpp:247-330): sample a state,
grow the current tree towards it (growTree, :116-196), and when that tree advanced, try to connect the
other tree to the new state by growing it until it is trapped or reaches the state. Every growTree is
served by the request loop: one nearestK request (k = 1: `tree->nearest`, the nearest element with the
smallest index among equals, as NearestNeighborsLinear's first minimum), and, for the start tree, one
checkMotion(nearest, new) request; for the goal tree one isValid(new) request and, when valid, one
checkMotion(new, nearest) request (:146-147). The new motion is added to its tree with a synchronous
host-memory call before the client's next request, so a client's requests never overlap each other;
many clients overlap on the device.

Deviations from RRTConnect, stated: states are drawn with numpy's PCG64 from the client's seed, not
with OMPL's sampler stream; the `addIntermediateStates_` option is not provided (its default, off, is
what runs); the host computes interpolate (RealVectorStateSpace.cpp:257-265, from + (to - from) t) and
takes the distance d from the nearestK answer (distance(element, query), the same FP64 value as
si_->distance(nmotion, rmotion) since the L2 sum is symmetric in its arguments).
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

from . import base as B
from . import capi
from .capi import check, lib

TRAPPED, ADVANCED, REACHED = 0, 1, 2


class Tree:
    """One RRTConnect tree: its states (rows, insertion order = nearestK key) and parent links."""

    def __init__(self, space, capacity):
        self.nn = B.NearestNeighborsGPU(space, capacity=capacity)
        self.states = []
        self.parent = []
        self.dim = space.dim

    def add(self, state, parent):
        row = np.ascontiguousarray(state, dtype=np.float64).reshape(1, self.dim)
        first = C.c_int64()
        check(lib().gbo_nn_add_host(self.nn._h, row.ctypes.data_as(C.c_void_p), 1, C.byref(first)))
        self.states.append(row[0].copy())
        self.parent.append(parent)
        return first.value


class RRTConnectClient:
    """RRTConnect over the request loop for one planning query (start, goal) with a GPU checker in a
    RealVectorStateSpace. `range_` is RRTConnect's maxDistance_."""

    def __init__(self, server, checker, start, goal, seed, range_, capacity=4096):
        self.server = server
        self.checker = checker
        self.space = checker.space
        self.dim = self.space.dim
        self.low = np.asarray(self.space.low, dtype=np.float64)
        self.high = np.asarray(self.space.high, dtype=np.float64)
        self.rng = np.random.default_rng(seed)
        self.range = float(range_)
        self.t_start = Tree(self.space, capacity)
        self.t_goal = Tree(self.space, capacity)
        self.t_start.add(start, -1)
        self.t_goal.add(goal, -1)
        self.start_tree = True
        self.log = []           # (kind, latency s) of every request
        self.trace = []         # per growTree: (tree, nearest key, new state or None, outcome)
        self.solution = None

    # the request loop's answers
    def _nearest(self, tree, q):
        t = self.server.submit_knn(tree.nn, q.reshape(1, -1), 1, want_dist=True)
        res, lat = self.server.wait(t)
        self.log.append(("knn", lat))
        return int(res["idx"][0, 0]), float(res["dist"][0, 0])

    def _motion(self, a, b):
        t = self.server.submit_motion(self.checker, a.reshape(1, -1), b.reshape(1, -1))
        res, lat = self.server.wait(t)
        self.log.append(("motion", lat))
        return bool(res["ok"][0])

    def _valid(self, s):
        t = self.server.submit_validity(self.checker, s.reshape(1, -1))
        res, lat = self.server.wait(t)
        self.log.append(("validity", lat))
        return bool(res["ok"][0])

    def _grow(self, tree, is_start, rstate):
        """growTree (RRTConnect.cpp:116-196) without intermediate states: returns (outcome, new key)."""
        nk, d = self._nearest(tree, rstate)
        nstate = tree.states[nk]
        reach = True
        dstate = rstate
        if d > self.range:
            t = self.range / d
            dstate = nstate + (rstate - nstate) * t
            if np.array_equal(dstate, nstate):
                self.trace.append((is_start, nk, None, TRAPPED))
                return TRAPPED, -1
            reach = False
        ok = self._motion(nstate, dstate) if is_start else (self._valid(dstate) and self._motion(dstate, nstate))
        if not ok:
            self.trace.append((is_start, nk, None, TRAPPED))
            return TRAPPED, -1
        key = tree.add(dstate, nk)
        self.trace.append((is_start, nk, dstate.copy(), REACHED if reach else ADVANCED))
        return (REACHED if reach else ADVANCED), key

    def step(self):
        """One iteration of RRTConnect::solve's loop (RRTConnect.cpp:247-330); True once solved."""
        if self.solution is not None:
            return True
        is_start = self.start_tree
        tree, other = (self.t_start, self.t_goal) if is_start else (self.t_goal, self.t_start)
        self.start_tree = not self.start_tree
        rstate = (self.high - self.low) * self.rng.random(self.dim) + self.low  # uniformReal(low, high)
        gs, key = self._grow(tree, is_start, rstate)
        if gs == TRAPPED:
            return False
        target = tree.states[key]
        gsc, okey = self._grow(other, not is_start, target)
        while gsc == ADVANCED:
            gsc, okey = self._grow(other, not is_start, target)
        if gsc == REACHED:
            s_key, g_key = (key, okey) if is_start else (okey, key)
            self.solution = (s_key, g_key)
            return True
        return False

    def path(self):
        """Start-to-goal states of the solution (tree paths joined at the connection)."""
        if self.solution is None:
            return None
        s_key, g_key = self.solution
        a = []
        k = s_key
        while k >= 0:
            a.append(self.t_start.states[k])
            k = self.t_start.parent[k]
        b = []
        k = g_key
        while k >= 0:
            b.append(self.t_goal.states[k])
            k = self.t_goal.parent[k]
        return np.array(a[::-1] + b)

    def run(self, max_iterations):
        t = time.perf_counter()
        it = 0
        while it < max_iterations and not self.step():
            it += 1
        return it, time.perf_counter() - t


def run_clients(clients, max_iterations, concurrent=True):
    """Runs every client to a solution or max_iterations, concurrently (one thread each: requests from
    all clients overlap in the request loop) or one after the other."""
    import threading

    if not concurrent:
        for c in clients:
            c.run(max_iterations)
        return
    threads = [threading.Thread(target=c.run, args=(max_iterations,)) for c in clients]
    for t in threads:
        t.start()
    for t in threads:
        t.join()


def request_percentiles(clients, kind=None, qs=(50, 99)):
    xs = [lat for c in clients for k, lat in c.log if kind in (None, k)]
    return {q: float(np.percentile(xs, q) * 1e3) for q in qs} if xs else {}
