"""ORACLE (test infrastructure only): ctypes wrapper over the oracle C API (oracle/oracle_api.h).

The same wrapper drives both implementations of that API:
  * ``Oracle.port()``      -> oracle/liboracle.so, the CPU restatement (builds anywhere);
  * ``Oracle.reference()`` -> oracle/_ref/libompl_ref.so, OMPL's own sources compiled unmodified
                              (only where the OMPL source tree was available at build time).

Only tests/, the smoke check and the benchmark's CPU-baseline leg may import this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libompl_ref.so")

SPACE_REAL_VECTOR, SPACE_SO2, SPACE_KINEMATIC_CHAIN, SPACE_WRAP_L2 = 0, 1, 2, 3
CHECK_ALL_VALID, CHECK_CIRCLES, CHECK_CHAIN_SEGMENTS, CHECK_DH_SPHERES, CHECK_DH_BOXES = 0, 1, 2, 3, 4
NN_EXACT, NN_REF_LINEAR, NN_REF_GNAT, NN_REF_GNAT_NTS, NN_REF_SQRT_APPROX = 0, 1, 2, 3, 4


def build_port(verbose: bool = False) -> str:
    """Compile the CPU restatement into oracle/liboracle.so (no -march: same FP64 on x86 and Arm)."""
    src = os.path.join(HERE, "port", "oracle.cpp")
    deps = [src, os.path.join(HERE, "oracle_api.h"), os.path.join(HERE, "dh_arm.h")]
    if os.path.exists(PORT_SO) and all(os.path.getmtime(PORT_SO) >= os.path.getmtime(d) for d in deps):
        return PORT_SO
    cmd = ["g++", "-std=c++17", "-O3", "-ffp-contract=off", "-fPIC", "-shared", src, "-o", PORT_SO, "-lpthread"]
    subprocess.run(cmd, check=True, capture_output=not verbose)
    return PORT_SO


def build_reference(tree: str | None = None, jobs: int = 8) -> str | None:
    """Compile OMPL's own sources from the OMPL source tree `tree` (else $OMPL_SOURCE_TREE) into
    oracle/_ref/; None when neither names a source tree."""
    tree = tree or os.environ.get("OMPL_SOURCE_TREE")
    if not tree or not os.path.isdir(os.path.join(tree, "src", "ompl")):
        return None
    subprocess.run(["make", "-s", "-C", os.path.join(HERE, "ref"), f"-j{jobs}", f"REF={tree}"], check=True,
                   capture_output=True)
    return REF_SO


class _Space(C.Structure):
    _fields_ = [("kind", C.c_int), ("dim", C.c_int), ("low", C.POINTER(C.c_double)),
                ("high", C.POINTER(C.c_double)), ("link_length", C.c_double), ("lvs_fraction", C.c_double),
                ("factor", C.c_uint)]


class _Checker(C.Structure):
    _fields_ = [("kind", C.c_int), ("obstacles", C.POINTER(C.c_double)), ("n_obstacles", C.c_long),
                ("dh", C.POINTER(C.c_double)), ("n_joints", C.c_int), ("spheres_per_link", C.c_int),
                ("sphere_radius", C.c_double)]


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


@dataclass
class SpaceDesc:
    kind: int
    dim: int
    low: np.ndarray | None = None
    high: np.ndarray | None = None
    link_length: float = 0.0
    lvs_fraction: float = 0.01
    factor: int = 1
    _keep: list = field(default_factory=list, repr=False)

    def c(self):
        low = np.ascontiguousarray(self.low if self.low is not None else np.zeros(self.dim), dtype=np.float64)
        high = np.ascontiguousarray(self.high if self.high is not None else np.zeros(self.dim), dtype=np.float64)
        self._keep = [low, high]
        return _Space(self.kind, self.dim, _dp(low), _dp(high), self.link_length, self.lvs_fraction, self.factor)


@dataclass
class CheckerDesc:
    kind: int
    obstacles: np.ndarray | None = None
    dh: np.ndarray | None = None
    spheres_per_link: int = 0
    sphere_radius: float = 0.0
    _keep: list = field(default_factory=list, repr=False)

    def c(self):
        obs = np.ascontiguousarray(self.obstacles if self.obstacles is not None else np.zeros((0, 4)),
                                   dtype=np.float64)
        if obs.ndim == 1:
            obs = obs.reshape(1, -1)
        dh = np.ascontiguousarray(self.dh if self.dh is not None else np.zeros((0, 3)), dtype=np.float64)
        self._keep = [obs, dh]
        return _Checker(self.kind, _dp(obs), obs.shape[0], _dp(dh), dh.shape[0], self.spheres_per_link,
                        self.sphere_radius)


def _rows(a, dim):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(-1, dim))


class Oracle:
    def __init__(self, path: str):
        self.path = path
        self.lib = C.CDLL(path)
        L = self.lib
        L.ora_space_extent.restype = C.c_double
        L.ora_space_lvs.restype = C.c_double
        L.ora_get_motion_states.restype = C.c_long
        L.ora_radius.restype = C.c_long
        L.ora_check_motion_states.restype = C.c_int
        L.ora_set_threads.restype = C.c_int

    @classmethod
    def port(cls) -> "Oracle":
        return cls(build_port())

    @classmethod
    def reference(cls) -> "Oracle | None":
        return cls(REF_SO) if os.path.exists(REF_SO) else None

    def set_threads(self, n: int) -> int:
        return self.lib.ora_set_threads(int(n))

    def extent(self, sp: SpaceDesc) -> float:
        s = sp.c()
        return self.lib.ora_space_extent(C.byref(s))

    def lvs(self, sp: SpaceDesc) -> float:
        s = sp.c()
        return self.lib.ora_space_lvs(C.byref(s))

    def distance(self, sp, a, b):
        a, b = _rows(a, sp.dim), _rows(b, sp.dim)
        out = np.empty(a.shape[0])
        s = sp.c()
        self.lib.ora_distance(C.byref(s), _dp(a), _dp(b), C.c_long(a.shape[0]), _dp(out))
        return out

    def interpolate(self, sp, a, b, t):
        a, b = _rows(a, sp.dim), _rows(b, sp.dim)
        t = np.ascontiguousarray(np.broadcast_to(np.asarray(t, dtype=np.float64), (a.shape[0],)))
        out = np.empty_like(a)
        s = sp.c()
        self.lib.ora_interpolate(C.byref(s), _dp(a), _dp(b), _dp(t), C.c_long(a.shape[0]), _dp(out))
        return out

    def valid_segment_count(self, sp, a, b):
        a, b = _rows(a, sp.dim), _rows(b, sp.dim)
        out = np.empty(a.shape[0], dtype=np.uint32)
        s = sp.c()
        self.lib.ora_valid_segment_count(C.byref(s), _dp(a), _dp(b), C.c_long(a.shape[0]),
                                         out.ctypes.data_as(C.POINTER(C.c_uint)))
        return out

    def enforce_bounds(self, sp, states):
        st = _rows(states, sp.dim).copy()
        s = sp.c()
        self.lib.ora_enforce_bounds(C.byref(s), _dp(st), C.c_long(st.shape[0]))
        return st

    def rng_uniform(self, seed, n, lo=None, hi=None):
        out = np.empty(n)
        kind = 0 if lo is None else 1
        self.lib.ora_rng_uniform(C.c_uint(seed), kind, C.c_double(lo or 0.0), C.c_double(hi or 0.0), C.c_long(n),
                                 _dp(out))
        return out

    def sample_uniform(self, sp, seed, n):
        out = np.empty((n, sp.dim))
        s = sp.c()
        self.lib.ora_sample_uniform(C.byref(s), C.c_uint(seed), C.c_long(n), _dp(out))
        return out

    def sample_uniform_near(self, sp, seed, near, distance):
        near = _rows(near, sp.dim)
        out = np.empty_like(near)
        s = sp.c()
        self.lib.ora_sample_uniform_near(C.byref(s), C.c_uint(seed), _dp(near), C.c_double(distance),
                                         C.c_long(near.shape[0]), _dp(out))
        return out

    def sample_script(self, sp, seed, ops, mean=None, stddev=0.0, log_mode=0):
        """ops: list of ("uniform" | "gaussian", count); gaussian calls take the next rows of mean."""
        kinds = np.array([1 if k == "gaussian" else 0 for k, _ in ops], dtype=np.int32)
        counts = np.array([c for _, c in ops], dtype=np.int64)
        mean = np.zeros((1, sp.dim)) if mean is None else _rows(mean, sp.dim)
        out = np.empty((int(counts.sum()), sp.dim))
        s = sp.c()
        self.lib.ora_sample_script(C.byref(s), C.c_uint(seed), kinds.ctypes.data_as(C.POINTER(C.c_int)),
                                   counts.ctypes.data_as(C.POINTER(C.c_long)), C.c_int(len(ops)), _dp(mean),
                                   C.c_double(stddev), C.c_int(log_mode), _dp(out))
        return out

    def log_rn(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = np.empty_like(x)
        self.lib.ora_log_rn(_dp(x), C.c_long(x.size), _dp(out))
        return out

    def is_valid(self, sp, ck, states):
        st = _rows(states, sp.dim)
        out = np.empty(st.shape[0], dtype=np.uint8)
        s, c = sp.c(), ck.c()
        self.lib.ora_is_valid(C.byref(s), C.byref(c), _dp(st), C.c_long(st.shape[0]),
                              out.ctypes.data_as(C.POINTER(C.c_ubyte)))
        return out

    def check_motion(self, sp, ck, s1, s2, want_state=True, want_bisect=True):
        s1, s2 = _rows(s1, sp.dim), _rows(s2, sp.dim)
        n = s1.shape[0]
        ok = np.empty(n, dtype=np.uint8)
        okb = np.empty(n, dtype=np.uint8) if want_bisect else None
        lt = np.empty(n)
        ls = np.empty((n, sp.dim)) if want_state else None
        nd = np.empty(n, dtype=np.int32)
        fj = np.empty(n, dtype=np.int32)
        s, c = sp.c(), ck.c()
        u8 = C.POINTER(C.c_ubyte)
        i32 = C.POINTER(C.c_int)
        self.lib.ora_check_motion(C.byref(s), C.byref(c), _dp(s1), _dp(s2), C.c_long(n), ok.ctypes.data_as(u8),
                                  okb.ctypes.data_as(u8) if okb is not None else None, _dp(lt), _dp(ls),
                                  nd.ctypes.data_as(i32), fj.ctypes.data_as(i32))
        return dict(ok=ok, ok_bisect=okb, last_t=lt, last_state=ls, nd=nd, first_j=fj)

    def check_motion_states(self, sp, ck, states):
        st = _rows(states, sp.dim)
        fi = C.c_long(-1)
        okb = C.c_int(0)
        s, c = sp.c(), ck.c()
        r = self.lib.ora_check_motion_states(C.byref(s), C.byref(c), _dp(st), C.c_long(st.shape[0]), C.byref(fi),
                                             C.byref(okb))
        return bool(r), (fi.value if not r else -1), bool(okb.value)

    def get_motion_states(self, sp, s1, s2, count, endpoints):
        s1, s2 = _rows(s1, sp.dim), _rows(s2, sp.dim)
        out = np.empty((count + 2, sp.dim))
        s = sp.c()
        m = self.lib.ora_get_motion_states(C.byref(s), _dp(s1), _dp(s2), C.c_uint(count), int(endpoints), _dp(out))
        return out[:m]

    def knn(self, sp, pts, q, k, algo=NN_EXACT):
        pts, q = _rows(pts, sp.dim), _rows(q, sp.dim)
        idx = np.empty((q.shape[0], k), dtype=np.int64)
        dist = np.empty((q.shape[0], k))
        s = sp.c()
        self.lib.ora_knn(C.byref(s), algo, _dp(pts), C.c_long(pts.shape[0]), _dp(q), C.c_long(q.shape[0]), k,
                         idx.ctypes.data_as(C.POINTER(C.c_long)), _dp(dist))
        return idx, dist

    def nn_sqrt_approx(self, sp, pts, queries, remove=()):
        """NearestNeighborsSqrtApprox::nearest for each query in order, after removing `remove` rows one
        at a time: (idx, dist, offset after the queries)."""
        p = _rows(pts, sp.dim)
        qq = _rows(queries, sp.dim)
        rem = np.ascontiguousarray(np.asarray(remove, dtype=np.int64))
        idx = np.empty(qq.shape[0], dtype=np.int64)
        dist = np.empty(qq.shape[0])
        s = sp.c()
        lp = C.POINTER(C.c_long)
        self.lib.ora_nn_sqrt_approx.restype = C.c_ulong
        off = self.lib.ora_nn_sqrt_approx(C.byref(s), _dp(p), C.c_long(p.shape[0]), rem.ctypes.data_as(lp),
                                          C.c_long(rem.size), _dp(qq), C.c_long(qq.shape[0]), idx.ctypes.data_as(lp),
                                          _dp(dist))
        return idx, dist, int(off)

    def knn_prefix(self, sp, pts, q, limit, k):
        pts, q = _rows(pts, sp.dim), _rows(q, sp.dim)
        limit = np.ascontiguousarray(limit, dtype=np.int64)
        idx = np.empty((q.shape[0], k), dtype=np.int64)
        dist = np.empty((q.shape[0], k))
        s = sp.c()
        self.lib.ora_knn_prefix(C.byref(s), _dp(pts), C.c_long(pts.shape[0]), _dp(q),
                                limit.ctypes.data_as(C.POINTER(C.c_long)), C.c_long(q.shape[0]), k,
                                idx.ctypes.data_as(C.POINTER(C.c_long)), _dp(dist))
        return idx, dist

    def radius(self, sp, pts, q, r, algo=NN_EXACT):
        pts, q = _rows(pts, sp.dim), _rows(q, sp.dim)
        nq = q.shape[0]
        counts = np.empty(nq, dtype=np.int64)
        s = sp.c()
        lp = C.POINTER(C.c_long)
        total = self.lib.ora_radius(C.byref(s), algo, _dp(pts), C.c_long(pts.shape[0]), _dp(q), C.c_long(nq),
                                    C.c_double(r), counts.ctypes.data_as(lp), None, None, C.c_long(0))
        idx = np.empty(max(total, 1), dtype=np.int64)
        dist = np.empty(max(total, 1))
        self.lib.ora_radius(C.byref(s), algo, _dp(pts), C.c_long(pts.shape[0]), _dp(q), C.c_long(nq), C.c_double(r),
                            counts.ctypes.data_as(lp), idx.ctypes.data_as(lp), _dp(dist), C.c_long(total))
        return counts, idx[:total], dist[:total]

    # ---- restatement-only entry points (absent from the reference build)
    def is_valid_brute(self, sp, ck, states):
        """isValid with every robot sphere tested against every world sphere (no grid)."""
        st = _rows(states, sp.dim)
        out = np.empty(st.shape[0], dtype=np.uint8)
        s, c = sp.c(), ck.c()
        self.lib.ora_is_valid_brute(C.byref(s), C.byref(c), _dp(st), C.c_long(st.shape[0]),
                                    out.ctypes.data_as(C.POINTER(C.c_ubyte)))
        return out

    def sincos_rn(self, x):
        """Correctly rounded sin and cos (double-double evaluation); returns (sin, cos, undecided)."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        s, c = np.empty_like(x), np.empty_like(x)
        self.lib.ora_sincos_rn.restype = C.c_long
        hard = self.lib.ora_sincos_rn(_dp(x), C.c_long(x.size), _dp(s), _dp(c))
        return s, c, int(hard)

    def trig_rounding(self, x):
        """The C library's sin/cos against the correctly rounded values on x: dict(sin_misrounded,
        cos_misrounded, undecided, max_ulps)."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        counts = np.zeros(4, dtype=np.int64)
        self.lib.ora_trig_rounding(_dp(x), C.c_long(x.size), counts.ctypes.data_as(C.POINTER(C.c_long)))
        return dict(sin_misrounded=int(counts[0]), cos_misrounded=int(counts[1]), undecided=int(counts[2]),
                    max_ulps=int(counts[3]))

    def prm_roadmap(self, sp, ck, seed, n_samples, k=10, edge_cap=None):
        """PRM roadmap (restatement): dict(sample_index, edge_src, edge_dst, candidates)."""
        cap = int(edge_cap if edge_cap is not None else n_samples * k)
        si = np.empty(n_samples, dtype=np.int64)
        es = np.empty(max(cap, 1), dtype=np.int64)
        ed = np.empty(max(cap, 1), dtype=np.int64)
        nm, cand = C.c_long(0), C.c_long(0)
        s, c = sp.c(), ck.c()
        lp = C.POINTER(C.c_long)
        self.lib.ora_prm_roadmap.restype = C.c_long
        ne = self.lib.ora_prm_roadmap(C.byref(s), C.byref(c), C.c_uint(seed), C.c_long(n_samples), C.c_int(k),
                                      C.byref(nm), si.ctypes.data_as(lp), es.ctypes.data_as(lp),
                                      ed.ctypes.data_as(lp), C.c_long(cap), C.byref(cand))
        if ne > cap:
            raise RuntimeError(f"edge capacity {cap} < {ne}")
        return dict(sample_index=si[:nm.value], edge_src=es[:ne], edge_dst=ed[:ne], candidates=int(cand.value))
