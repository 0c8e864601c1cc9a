"""Serving: continuous-batching fixed-centroid transport solves (d2g_server_*).

Each request is a query distribution (m_q supports in R^d, weights) solved
against all resident centroids with B-ADMM (centroid weights held fixed);
the answer is the transport cost to every centroid and the argmin.  The
server admits requests by HBM budget and queue bound and batches whatever
has arrived whenever a batch slot frees up.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

from . import _lib as L


class Server:
    def __init__(self, c_w, c_supp, iters=200, rho_coeff=2.0, hbm_budget_bytes=1 << 30,
                 max_queue=4096, max_batch_entries=0):
        self.lib = L.load()
        c_w = np.ascontiguousarray(c_w, np.float64)
        self.k, self.m = c_w.shape
        c_supp = np.ascontiguousarray(c_supp, np.float64).reshape(self.k, self.m, -1)
        self.dim = c_supp.shape[2]
        d = L.d2g_server_desc()
        d.num_of_labels, d.str, d.dim = self.k, self.m, self.dim
        d.c_w, d.c_supp = c_w.ctypes.data, c_supp.ctypes.data
        d.iters, d.rhoCoeff = int(iters), float(rho_coeff)
        d.hbm_budget_bytes, d.max_queue = int(hbm_budget_bytes), int(max_queue)
        d.max_batch_entries = int(max_batch_entries)
        h = C.c_void_p()
        L.check(self.lib.d2g_server_create(C.byref(d), C.byref(h)), "d2g_server_create")
        self.h = h
        self._costs = np.empty(self.k)

    def close(self):
        if getattr(self, "h", None):
            self.lib.d2g_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def try_submit(self, w, supp):
        """Ticket, or None when admission control refuses the request."""
        w = np.ascontiguousarray(w, np.float64)
        supp = np.ascontiguousarray(supp, np.float64)
        t = C.c_longlong()
        rc = self.lib.d2g_server_submit(self.h, w.size, w.ctypes.data, supp.ctypes.data, C.byref(t))
        if rc == L.D2G_E_ADMISSION:
            return None
        L.check(rc, "d2g_server_submit")
        return t.value

    def submit(self, w, supp):
        t = self.try_submit(w, supp)
        if t is None:
            raise L.D2GError(L.D2G_E_ADMISSION, "d2g_server_submit")
        return t

    def result(self, ticket, costs=True):
        """None while pending, else (label, costs or None, latency_ms); collects the ticket."""
        lab = C.c_int()
        lat = C.c_double()
        rc = self.lib.d2g_server_result(self.h, ticket, C.byref(lab),
                                        self._costs.ctypes.data if costs else None, C.byref(lat))
        if rc < 0:
            L.check(rc, "d2g_server_result")
        if rc == 0:
            return None
        return lab.value, (self._costs.copy() if costs else None), lat.value

    def wait(self):
        rc = self.lib.d2g_server_progress(self.h, 1)
        if rc < 0:
            L.check(rc, "d2g_server_progress")
        return rc

    def solve(self, w, supp):
        """One request, waited for."""
        t = self.submit(w, supp)
        while True:
            r = self.result(t)
            if r is not None:
                return r
            self.wait()


def poisson_run(server: Server, queries, rate: float, seed: int = 0, costs: bool = False):
    """Offer `queries` with Poisson arrivals at `rate` req/s; returns latency
    percentiles, throughput and refusals.  Arrivals are paced by busy-waiting
    on the host clock; results are collected as they complete."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=len(queries))
    arrive = np.cumsum(gaps)
    pending = {}
    lat, refused, done = [], 0, {}
    t0 = time.perf_counter()

    def collect():
        for i, t in list(pending.items()):
            r = server.result(t, costs)
            if r is not None:
                done[i] = r
                lat.append(r[2])
                del pending[i]
    for i, (w, s) in enumerate(queries):
        while time.perf_counter() - t0 < arrive[i]:
            if pending and (i & 7) == 0:
                collect()
        t = server.try_submit(w, s)
        if t is None:
            refused += 1
        else:
            pending[i] = t
        if len(pending) > 64 and (i & 15) == 0:
            collect()
    while pending:
        server.wait()
        collect()
    wall = time.perf_counter() - t0
    lat = np.array(lat)
    return {"rate_offered": rate, "requests": len(queries), "completed": int(lat.size),
            "refused": refused, "throughput": lat.size / wall if wall > 0 else 0.0,
            "p50_ms": float(np.percentile(lat, 50)) if lat.size else None,
            "p99_ms": float(np.percentile(lat, 99)) if lat.size else None,
            "wall_s": wall, "results": done}
