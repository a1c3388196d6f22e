"""Python wrapper of the request loop (gbo_server_* in include/gbompl.h): concurrent planner
instances submit validity, motion and nearestK requests over their own device-resident worlds and
roadmaps; the server admits them by stream slot and device footprint and overlaps them on the GPU."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .capi import check, lib


class Server:
    def __init__(self, n_streams=16, arena_bytes=4 << 30):
        h = C.c_void_p()
        check(lib().gbo_server_create(int(n_streams), int(arena_bytes), C.byref(h)))
        self._h = h
        self._live = {}

    def close(self):
        if self._h:
            lib().gbo_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _submit(self, req, keep):
        t = C.c_uint64()
        check(lib().gbo_server_submit(self._h, C.byref(req), C.byref(t)))
        self._live[t.value] = (req, keep)
        return t.value

    @staticmethod
    def _rows(x, dim):
        return np.ascontiguousarray(x, dtype=np.float64).reshape(-1, dim)

    def submit_validity(self, checker, states):
        st = self._rows(states, checker.space.dim)
        ok = np.empty(st.shape[0], dtype=np.uint8)
        req = capi.Request(kind=capi.REQ_VALIDITY, checker=checker._h.value, states=st.ctypes.data, n=st.shape[0],
                           ok=ok.ctypes.data)
        return self._submit(req, {"states": st, "ok": ok})

    def submit_motion(self, checker, s1, s2, schedule=capi.SCHEDULE_AUTO):
        a = self._rows(s1, checker.space.dim)
        b = self._rows(s2, checker.space.dim)
        n = a.shape[0]
        ok = np.empty(n, dtype=np.uint8)
        fj = np.empty(n, dtype=np.int32)
        nd = np.empty(n, dtype=np.int32)
        req = capi.Request(kind=capi.REQ_MOTION, checker=checker._h.value, states=a.ctypes.data,
                           states2=b.ctypes.data, n=n, schedule=schedule, ok=ok.ctypes.data, first_j=fj.ctypes.data,
                           nd=nd.ctypes.data)
        return self._submit(req, {"s1": a, "s2": b, "ok": ok, "first_j": fj, "nd": nd})

    def submit_knn(self, nn, queries, k, want_dist=True):
        q = self._rows(queries, nn.space.dim)
        n = q.shape[0]
        idx = np.empty((n, k), dtype=np.int64)
        dist = np.empty((n, k)) if want_dist else None
        req = capi.Request(kind=capi.REQ_KNN, nn=nn._h.value, states=q.ctypes.data, n=n, k=k, idx=idx.ctypes.data,
                           dist=dist.ctypes.data if want_dist else None)
        return self._submit(req, {"q": q, "idx": idx, "dist": dist})

    def wait(self, ticket, timeout_s=-1.0):
        """Returns (result dict, latency seconds); raises GboError if the request failed."""
        lat = C.c_double()
        st = lib().gbo_server_wait(self._h, C.c_uint64(ticket), C.c_double(timeout_s), C.byref(lat))
        _, keep = self._live.pop(ticket)
        check(st)
        return keep, lat.value

    def stats(self):
        s, c, a, m = C.c_uint64(), C.c_uint64(), C.c_int64(), C.c_int()
        check(lib().gbo_server_stats(self._h, C.byref(s), C.byref(c), C.byref(a), C.byref(m)))
        return {"submitted": s.value, "completed": c.value, "arena_in_use": a.value, "max_concurrent": m.value}
