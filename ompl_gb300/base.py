"""Python mirror of OMPL's plugin interfaces for the sampling / validity / motion / kNN path, backed
by libgbompl.so. Class and method names follow OMPL (ompl::base::*, ompl::NearestNeighbors<T>).

Batches are torch CUDA tensors (device-resident, no copies) or numpy arrays (copied in and out).
A batch of n states is an (n, dim) array (OMPL's per-state layout, passed as AoS) or, with
``soa=True``, a (dim, n) array (the coalesced layout the kernels prefer).
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import torch

from . import capi
from .capi import check, lib

PI = math.pi


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _stream(stream):
    if stream is None:
        return C.c_void_p(torch.cuda.current_stream().cuda_stream)
    return C.c_void_p(stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream))


def _dev(x, dtype=torch.float64):
    if isinstance(x, torch.Tensor):
        t = x.to(device="cuda", dtype=dtype)
    else:
        t = torch.as_tensor(np.ascontiguousarray(x), dtype=dtype, device="cuda")
    return t.contiguous()


def _batch(states, dim, soa):
    """Returns (tensor, n, ld, layout) for a batch of states."""
    t = _dev(states)
    if soa:
        t = t.reshape(dim, -1)
        return t, t.shape[1], t.shape[1], capi.LAYOUT_SOA
    t = t.reshape(-1, dim)
    return t, t.shape[0], dim, capi.LAYOUT_AOS


def _host(t):
    return t.cpu().numpy()


class StateSpace:
    """Common part of the spaces (StateSpace.cpp:237-249, 820-854)."""

    kind = capi.SPACE_REAL_VECTOR

    def __init__(self, dim, low=None, high=None, param=0.0):
        self.dim = dim
        self.low = None if low is None else np.array(np.broadcast_to(np.asarray(low, dtype=np.float64), (dim,)))
        self.high = None if high is None else np.array(np.broadcast_to(np.asarray(high, dtype=np.float64), (dim,)))
        self.param = param
        self.fraction = 0.01
        self.factor = 1
        self.lvs = None  # set to take the segment length from an OMPL space as-is
        self._h = None

    # OMPL-style configuration
    def setLongestValidSegmentFraction(self, f):
        if f < np.finfo(float).eps or f > 1.0 - np.finfo(float).eps:
            raise capi.GboError(capi.ERR_INVALID_ARGUMENT, "The fraction of the extent must be larger than 0 and less than 1")
        self.fraction = f
        self._h = None

    def setValidSegmentCountFactor(self, k):
        if k < 1:
            raise capi.GboError(capi.ERR_INVALID_ARGUMENT, "The multiplicative factor for the valid segment count "
                                                           "between two states must be strictly positive")
        self.factor = int(k)
        self._h = None

    def handle(self):
        if self._h is None:
            h = C.c_void_p()
            low = self.low.ctypes.data_as(C.POINTER(C.c_double)) if self.low is not None else None
            high = self.high.ctypes.data_as(C.POINTER(C.c_double)) if self.high is not None else None
            check(lib().gbo_space_create(self.kind, self.dim, low, high, self.param,
                                         -1.0 if self.lvs is None else self.lvs, self.fraction, self.factor,
                                         C.byref(h)))
            self._h = h
        return self._h

    def setup(self):
        self._h = None
        self.handle()

    def getMaximumExtent(self):
        e, l_ = C.c_double(), C.c_double()
        check(lib().gbo_space_info(self.handle(), C.byref(e), C.byref(l_)))
        return e.value

    def getLongestValidSegmentLength(self):
        e, l_ = C.c_double(), C.c_double()
        check(lib().gbo_space_info(self.handle(), C.byref(e), C.byref(l_)))
        return l_.value

    def getDimension(self):
        return self.dim

    def distance(self, a, b, soa=False, stream=None):
        ta, n, ld, lay = _batch(a, self.dim, soa)
        tb, _, _, _ = _batch(b, self.dim, soa)
        out = torch.empty(n, dtype=torch.float64, device="cuda")
        check(lib().gbo_space_distance(self.handle(), _ptr(ta), _ptr(tb), n, ld, lay, _ptr(out), _stream(stream)))
        return out if isinstance(a, torch.Tensor) else _host(out)

    def interpolate(self, a, b, t, soa=False, stream=None):
        ta, n, ld, lay = _batch(a, self.dim, soa)
        tb, _, _, _ = _batch(b, self.dim, soa)
        tt = _dev(np.broadcast_to(np.asarray(t, dtype=np.float64), (n,)).copy() if not isinstance(t, torch.Tensor)
                  else t)
        out = torch.empty_like(ta)
        check(lib().gbo_space_interpolate(self.handle(), _ptr(ta), _ptr(tb), _ptr(tt), n, ld, lay, _ptr(out),
                                          _stream(stream)))
        return out if isinstance(a, torch.Tensor) else _host(out)

    def getMotionStates(self, s1, s2, count, endpoints=True, stream=None):
        """SpaceInformation::getMotionStates(s1, s2, states, count, endpoints, alloc=true) for a batch
        of edges (AoS rows): returns (n, m, dim) with m = count + 2 (endpoints) or count."""
        t1, n, ld, lay = _batch(s1, self.dim, False)
        t2, _, _, _ = _batch(s2, self.dim, False)
        m = count + 2 if endpoints else count
        out = torch.empty((n * m, self.dim), dtype=torch.float64, device="cuda")
        check(lib().gbo_get_motion_states(self.handle(), _ptr(t1), _ptr(t2), n, ld, lay, int(count),
                                          1 if endpoints else 0, _ptr(out), self.dim, _stream(stream)))
        out = out.reshape(n, m, self.dim)
        return out if isinstance(s1, torch.Tensor) else _host(out)


class RealVectorStateSpace(StateSpace):
    kind = capi.SPACE_REAL_VECTOR

    def __init__(self, dim, low, high):
        super().__init__(dim, low, high)


class SO2StateSpace(StateSpace):
    kind = capi.SPACE_SO2

    def __init__(self):
        super().__init__(1)


class KinematicChainSpace(StateSpace):
    """KinematicChainSpace of demos/KinematicChain.h:88-191 (joints in [-pi, pi], workspace metric)."""
    kind = capi.SPACE_KINEMATIC_CHAIN

    def __init__(self, num_links, link_length):
        super().__init__(num_links, param=link_length)
        self.linkLength = link_length


class WrapL2StateSpace(StateSpace):
    """Joint space [-pi, pi]^dim with L2 over per-joint wrapped differences (no OMPL counterpart)."""
    kind = capi.SPACE_WRAP_L2

    def __init__(self, dim):
        super().__init__(dim)


class StateValidityChecker:
    """GPU-backed StateValidityChecker (StateValidityChecker.h:111). Subclasses bind a world."""

    kind = capi.CHECK_ALL_VALID

    def __init__(self, space: StateSpace, world=None, dh=None, spheres_per_link=0, sphere_radius=0.0):
        self.space = space
        w = np.ascontiguousarray(np.zeros((0, 4)) if world is None else world, dtype=np.float64)
        d = None if dh is None else np.ascontiguousarray(dh, dtype=np.float64)
        h = C.c_void_p()
        check(lib().gbo_checker_create(space.handle(), self.kind, w.ctypes.data_as(C.POINTER(C.c_double)),
                                       w.shape[0], None if d is None else d.ctypes.data_as(C.POINTER(C.c_double)),
                                       0 if d is None else d.shape[0], spheres_per_link, sphere_radius, C.byref(h)))
        self._h = h
        self.precision = capi.PRECISION_FP64

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                lib().gbo_checker_destroy(self._h)
        except Exception:
            pass

    def setPrecision(self, precision):
        p = {"fp64": capi.PRECISION_FP64, "fp32_guarded": capi.PRECISION_FP32_GUARDED}.get(precision, precision)
        check(lib().gbo_checker_set_precision(self._h, p))
        self.precision = p

    def stats(self):
        """Counters of the last call: states evaluated, states re-checked in FP64, one-ulp hazards of
        the FP64 decisions (gbo_checker_counters)."""
        e, r, h = C.c_uint64(), C.c_uint64(), C.c_uint64()
        check(lib().gbo_checker_counters(self._h, C.byref(e), C.byref(r), C.byref(h)))
        return {"evaluated": e.value, "rechecked": r.value, "hazards": h.value}

    def precisionStats(self, states, soa=False, stream=None):
        """Flip rate of the FP32 form (face-value FP32 verdict vs FP64 verdict), the guarded form's
        ambiguous states and the largest |FP32 - FP64| of the compared quantities, on a batch of states."""
        t, n, ld, lay = _batch(states, self.space.dim, soa)
        out = capi.PrecisionStats()
        check(lib().gbo_checker_precision_stats(self._h, _ptr(t), n, ld, lay, C.byref(out), _stream(stream)))
        return {"states": out.states, "flips": out.flips, "flip_rate": out.flips / max(out.states, 1),
                "ambiguous": out.ambiguous, "ambiguous_rate": out.ambiguous / max(out.states, 1),
                "max_abs_err": out.max_abs_err}

    def isValid(self, states, soa=False, stream=None):
        t, n, ld, lay = _batch(states, self.space.dim, soa)
        out = torch.empty(n, dtype=torch.uint8, device="cuda")
        check(lib().gbo_is_valid(self._h, _ptr(t), n, ld, lay, _ptr(out), _stream(stream)))
        return out if isinstance(states, torch.Tensor) else _host(out).astype(bool)

    def isValidHost(self, states):
        a = np.ascontiguousarray(states, dtype=np.float64).reshape(-1, self.space.dim)
        out = np.empty(a.shape[0], dtype=np.uint8)
        check(lib().gbo_is_valid_host(self._h, a.ctypes.data_as(C.c_void_p), a.shape[0],
                                      out.ctypes.data_as(C.c_void_p)))
        return out.astype(bool)


class AllValidStateValidityChecker(StateValidityChecker):
    kind = capi.CHECK_ALL_VALID

    def __init__(self, space):
        super().__init__(space)


class CirclesValidityChecker(StateValidityChecker):
    """Point robot vs circles (tests/resources/circles2D.h:141-151); world rows (x, y, r)."""
    kind = capi.CHECK_CIRCLES

    def __init__(self, space, circles):
        super().__init__(space, world=np.asarray(circles).reshape(-1, 3))


class KinematicChainValidityChecker(StateValidityChecker):
    """demos/KinematicChain.h:193-277; world rows (x0, y0, x1, y1)."""
    kind = capi.CHECK_CHAIN_SEGMENTS

    def __init__(self, space, segments):
        super().__init__(space, world=np.asarray(segments).reshape(-1, 4))


class DHSphereArmValidityChecker(StateValidityChecker):
    """Serial DH arm covered by spheres vs world spheres (x, y, z, r) on a uniform grid."""
    kind = capi.CHECK_DH_SPHERES

    def __init__(self, space, dh, world, spheres_per_link=8, sphere_radius=0.05):
        super().__init__(space, world=np.asarray(world).reshape(-1, 4), dh=dh, spheres_per_link=spheres_per_link,
                         sphere_radius=sphere_radius)


class DHBoxArmValidityChecker(StateValidityChecker):
    """The serial DH arm covered by spheres vs axis-aligned world boxes, rows (cx, cy, cz, hx, hy, hz):
    a robot sphere hits a box when its centre is closer to the box than its radius (oracle/dh_arm.h
    states the operation order)."""
    kind = capi.CHECK_DH_BOXES

    def __init__(self, space, dh, boxes, spheres_per_link=8, sphere_radius=0.05):
        super().__init__(space, world=np.asarray(boxes).reshape(-1, 6), dh=dh, spheres_per_link=spheres_per_link,
                         sphere_radius=sphere_radius)


class DiscreteMotionValidator:
    """DiscreteMotionValidator (DiscreteMotionValidator.cpp:48-145) over a GPU checker."""

    def __init__(self, checker: StateValidityChecker):
        self.checker = checker
        self.space = checker.space
        self.valid_ = 0
        self.invalid_ = 0

    def getValidMotionCount(self):
        return self.valid_

    def getInvalidMotionCount(self):
        return self.invalid_

    def checkMotions(self, s1, s2, schedule=capi.SCHEDULE_PLAIN, soa=False, last_valid=False, stream=None):
        """Batch checkMotion: dict(ok, first_j, nd[, last_t, last_state]) as tensors or numpy arrays."""
        dim = self.space.dim
        t1, n, ld, lay = _batch(s1, dim, soa)
        t2, _, _, _ = _batch(s2, dim, soa)
        ok = torch.empty(n, dtype=torch.uint8, device="cuda")
        fj = torch.empty(n, dtype=torch.int32, device="cuda")
        nd = torch.empty(n, dtype=torch.int32, device="cuda")
        st = _stream(stream)
        check(lib().gbo_check_motion(self.checker._h, _ptr(t1), _ptr(t2), n, ld, lay, schedule, _ptr(ok), _ptr(fj),
                                     _ptr(nd), st))
        res = {"ok": ok, "first_j": fj, "nd": nd}
        if last_valid:
            lt = torch.empty(n, dtype=torch.float64, device="cuda")
            ls = torch.empty_like(t1)
            check(lib().gbo_last_valid(self.space.handle(), _ptr(t1), _ptr(t2), _ptr(fj), _ptr(nd), n, ld, lay,
                                       _ptr(lt), _ptr(ls), st))
            res["last_t"] = lt
            res["last_state"] = ls
        if not isinstance(s1, torch.Tensor):
            res = {k: _host(v) for k, v in res.items()}
            nv = int(res["ok"].sum())
            self.valid_ += nv
            self.invalid_ += n - nv
        return res

    def checkMotion(self, s1, s2, lastValid=None):
        """Single-edge drop-in: returns bool; with lastValid=[state or None, t] fills it like OMPL."""
        r = self.checkMotions(np.asarray(s1).reshape(1, -1), np.asarray(s2).reshape(1, -1),
                              last_valid=lastValid is not None)
        ok = bool(r["ok"][0])
        if lastValid is not None and not ok:
            lastValid[1] = float(r["last_t"][0])
            lastValid[0] = r["last_state"][0].copy()
        return ok

    def checkMotionHost(self, s1, s2, last_valid=True):
        a = np.ascontiguousarray(s1, dtype=np.float64).reshape(-1, self.space.dim)
        b = np.ascontiguousarray(s2, dtype=np.float64).reshape(-1, self.space.dim)
        n = a.shape[0]
        ok = np.empty(n, dtype=np.uint8)
        lt = np.empty(n) if last_valid else None
        ls = np.empty_like(a) if last_valid else None
        vp = C.c_void_p
        check(lib().gbo_check_motion_host(self.checker._h, a.ctypes.data_as(vp), b.ctypes.data_as(vp), n,
                                          ok.ctypes.data_as(vp), lt.ctypes.data_as(vp) if last_valid else None,
                                          ls.ctypes.data_as(vp) if last_valid else None))
        return ok.astype(bool), lt, ls

    def checkMotionStates(self, states, stream=None):
        """SpaceInformation::checkMotion(states, count, firstInvalidStateIndex)."""
        t, n, ld, lay = _batch(states, self.space.dim, False)
        ok = torch.empty(1, dtype=torch.uint8, device="cuda")
        fi = torch.empty(1, dtype=torch.int64, device="cuda")
        check(lib().gbo_check_motion_states(self.checker._h, _ptr(t), n, ld, lay, _ptr(ok), _ptr(fi),
                                            _stream(stream)))
        return bool(ok.item()), int(fi.item())


class StateSampler:
    """The space's default sampler (RealVectorStateSampler / SO2StateSampler) with its RNG seeded as
    RNG::setLocalSeed(seed); consecutive calls continue the same stream."""

    def __init__(self, space: StateSpace, seed: int):
        self.space = space
        h = C.c_void_p()
        check(lib().gbo_sampler_create(space.handle(), seed & 0xFFFFFFFF, C.byref(h)))
        self._h = h

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                lib().gbo_sampler_destroy(self._h)
        except Exception:
            pass

    def sampleUniform(self, n, soa=False, stream=None, host=True):
        dim = self.space.dim
        out = torch.empty((dim, n) if soa else (n, dim), dtype=torch.float64, device="cuda")
        ld, lay = (n, capi.LAYOUT_SOA) if soa else (dim, capi.LAYOUT_AOS)
        check(lib().gbo_sample_uniform(self._h, n, _ptr(out), ld, lay, _stream(stream)))
        return _host(out) if host else out

    def sampleUniformNear(self, near, distance, stream=None):
        t, n, ld, lay = _batch(near, self.space.dim, False)
        out = torch.empty_like(t)
        check(lib().gbo_sample_uniform_near(self._h, _ptr(t), float(distance), n, ld, lay, _ptr(out),
                                            _stream(stream)))
        return out if isinstance(near, torch.Tensor) else _host(out)

    def sampleGaussian(self, mean, stddev, stream=None):
        """StateSampler::sampleGaussian for each row of `mean` (RealVectorStateSpace.cpp:67-82,
        SO2StateSpace.cpp:58-62); the cached second normal value carries across calls."""
        t, n, ld, lay = _batch(mean, self.space.dim, False)
        out = torch.empty_like(t)
        check(lib().gbo_sample_gaussian(self._h, _ptr(t), float(stddev), n, ld, lay, _ptr(out), _stream(stream)))
        return out if isinstance(mean, torch.Tensor) else _host(out)

    def sampleValid(self, checker, n, attempts=100, stream=None, host=True):
        """UniformValidStateSampler::sample called n times on this sampler's stream: (states, ok)."""
        dim = self.space.dim
        out = torch.empty((n, dim), dtype=torch.float64, device="cuda")
        ok = torch.empty(n, dtype=torch.uint8, device="cuda")
        check(lib().gbo_sample_valid(self._h, checker._h, n, int(attempts), _ptr(out), dim, capi.LAYOUT_AOS,
                                     _ptr(ok), _stream(stream)))
        return (_host(out), _host(ok).astype(bool)) if host else (out, ok)


RealVectorStateSampler = StateSampler


class NearestNeighborsGPU:
    """ompl::NearestNeighbors<T> over a device-resident index. Elements are identified by their
    insertion index (key); results are ordered by (distance, key)."""

    def __init__(self, space: StateSpace, capacity: int, precision="fp32_guarded"):
        self.space = space
        h = C.c_void_p()
        check(lib().gbo_nn_create(space.handle(), int(capacity), C.byref(h)))
        self._h = h
        self.setPrecision(precision)

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                lib().gbo_nn_destroy(self._h)
        except Exception:
            pass

    def setPrecision(self, precision):
        p = {"fp64": capi.PRECISION_FP64, "fp32_guarded": capi.PRECISION_FP32_GUARDED}.get(precision, precision)
        check(lib().gbo_nn_set_precision(self._h, p))

    def reportsSortedResults(self):
        return True

    def add(self, states, soa=False, stream=None):
        t, n, ld, lay = _batch(states, self.space.dim, soa)
        first = C.c_int64()
        check(lib().gbo_nn_add(self._h, _ptr(t), n, ld, lay, C.byref(first), _stream(stream)))
        if not isinstance(states, torch.Tensor):
            torch.cuda.synchronize()
        return np.arange(first.value, first.value + n)

    def remove(self, keys, stream=None):
        k = _dev(np.atleast_1d(keys), torch.int64)
        check(lib().gbo_nn_remove(self._h, _ptr(k), k.numel(), _stream(stream)))
        torch.cuda.synchronize()
        return True

    def clear(self):
        check(lib().gbo_nn_clear(self._h))
        self._sqrt_offset = 0

    def size(self):
        s = C.c_int64()
        check(lib().gbo_nn_size(self._h, C.byref(s)))
        return s.value

    def stats(self):
        q, r, f = C.c_uint64(), C.c_uint64(), C.c_uint64()
        check(lib().gbo_nn_stats(self._h, C.byref(q), C.byref(r), C.byref(f)))
        e, b = C.c_float(), C.c_float()
        check(lib().gbo_nn_error_stats(self._h, C.byref(e), C.byref(b)))
        nb = C.c_uint64()
        check(lib().gbo_nn_search_bytes(self._h, C.byref(nb)))
        return {"queries": q.value, "rechecked": r.value, "fallbacks": f.value, "max_fp32_error": e.value,
                "fp32_error_bound": b.value, "search_bytes": nb.value}

    def nearestK(self, queries, k, prefix=None, soa=False, want_dist=True, stream=None):
        t, n, ld, lay = _batch(queries, self.space.dim, soa)
        idx = torch.empty((n, k), dtype=torch.int64, device="cuda")
        dist = torch.empty((n, k), dtype=torch.float64, device="cuda") if want_dist else None
        pre = None if prefix is None else _dev(prefix, torch.int64)
        check(lib().gbo_nn_nearest_k(self._h, _ptr(t), n, ld, lay, int(k), _ptr(pre), _ptr(idx), _ptr(dist),
                                     _stream(stream)))
        if isinstance(queries, torch.Tensor):
            return idx, dist
        return _host(idx), (_host(dist) if want_dist else None)

    def nearestSqrtApprox(self, queries, soa=False, stream=None):
        """NearestNeighborsSqrtApprox::nearest (NearestNeighborsSqrtApprox.h:91-115) for each query in
        order, over the present elements: (keys, distances). The structure's offset carries across calls
        and restarts at clear()."""
        t, n, ld, lay = _batch(queries, self.space.dim, soa)
        idx = torch.empty(n, dtype=torch.int64, device="cuda")
        dist = torch.empty(n, dtype=torch.float64, device="cuda")
        off = C.c_uint64(getattr(self, "_sqrt_offset", 0))
        check(lib().gbo_nn_nearest_sqrt_approx(self._h, _ptr(t), n, ld, lay, C.byref(off), _ptr(idx), _ptr(dist),
                                               _stream(stream)))
        self._sqrt_offset = off.value
        if isinstance(queries, torch.Tensor):
            return idx, dist
        return _host(idx), _host(dist)

    def nearestR(self, queries, radius, soa=False, stream=None):
        t, n, ld, lay = _batch(queries, self.space.dim, soa)
        counts = torch.empty(n, dtype=torch.int64, device="cuda")
        st = _stream(stream)
        check(lib().gbo_nn_nearest_r_count(self._h, _ptr(t), n, ld, lay, float(radius), _ptr(counts), st))
        offsets = torch.zeros(n, dtype=torch.int64, device="cuda")
        if n > 1:
            offsets[1:] = torch.cumsum(counts, 0)[:-1]
        total = int(counts.sum().item())
        idx = torch.empty(max(total, 1), dtype=torch.int64, device="cuda")
        dist = torch.empty(max(total, 1), dtype=torch.float64, device="cuda")
        check(lib().gbo_nn_nearest_r_fill(self._h, _ptr(t), n, ld, lay, float(radius), _ptr(offsets), _ptr(idx),
                                          _ptr(dist), st))
        return _host(counts), _host(idx)[:total], _host(dist)[:total]


def measure_fp32_peak():
    f = C.c_double()
    check(lib().gbo_measure_fp32_peak(C.byref(f), _stream(None)))
    return f.value


def measure_fp64_peak():
    f = C.c_double()
    check(lib().gbo_measure_fp64_peak(C.byref(f), _stream(None)))
    return f.value


def launch_count():
    return int(lib().gbo_launch_count())
