"""Python driver of the native solve-request loop (qllg_server_* in
libqll_gb300): resident lattices, continuous batching of solve requests
(lattice, mass, shifts, tolerance, source), HBM admission, latency records.

The scheduling itself is native; this module owns the host buffers of the
requests (sources and solutions must stay alive until a request completes)
and gives a Poisson load generator for the serving benchmark."""
import ctypes
import time
from ctypes import POINTER, Structure, c_double, c_int, c_longlong, c_size_t, c_void_p

import numpy as np

from . import qll


class RequestInfo(Structure):
    _fields_ = [("status", c_int), ("ncol", c_int), ("iters", c_int*16),
                ("true_rsq", c_double*16), ("seconds_queued", c_double),
                ("seconds_total", c_double)]


class ServerInfo(Structure):
    _fields_ = [("budget_bytes", c_size_t), ("used_bytes", c_size_t), ("batches", c_int),
                ("busy_columns", c_int), ("requests", c_int), ("pending", c_int),
                ("admitted_columns", c_longlong), ("chunks", c_longlong)]


_declared = False


def _lib():
    global _declared
    L = qll.load()
    if not _declared:
        L.qllg_server_create.restype = c_void_p
        L.qllg_server_create.argtypes = [c_size_t, c_int, c_int]
        L.qllg_server_add_lattice.argtypes = [c_void_p, c_void_p]
        L.qllg_server_submit.argtypes = [c_void_p, c_int, c_double, c_int, POINTER(c_double),
                                         c_double, c_void_p, POINTER(c_void_p)]
        L.qllg_server_step.argtypes = [c_void_p]
        L.qllg_server_pending.argtypes = [c_void_p]
        L.qllg_server_request.argtypes = [c_void_p, c_int, POINTER(RequestInfo)]
        L.qllg_server_stats.argtypes = [c_void_p, POINTER(ServerInfo)]
        L.qllg_server_destroy.argtypes = [c_void_p]
        L.qllg_server_destroy.restype = None
        for fn in (L.qllg_stag_create_asqtad, L.qllg_stag_create_asqtad_fb):
            fn.restype = c_void_p
            fn.argtypes = [POINTER(c_int), POINTER(c_void_p), POINTER(qll.Fat7Coeffs)]
        L.qllg_stag_destroy.argtypes = [c_void_p]
        L.qllg_stag_destroy.restype = None
        _declared = True
    return L


def asqtad_operator(dims, seed, eps, single_store=False):
    """resident asqtad operator from seeded thin links (fat7 on the GPU);
    single_store keeps the forward links only (half the link memory)"""
    L = _lib()
    thin = qll.gen_gauge(tuple(dims), seed, eps, ks=True)
    coef = qll.asqtad_coeffs()
    create = L.qllg_stag_create_asqtad_fb if single_store else L.qllg_stag_create_asqtad
    S = create(qll.dims_c(tuple(dims)), qll.vp_array(thin), ctypes.byref(coef))
    if not S:
        raise RuntimeError(qll.last_error())
    return c_void_p(S)


class Server:
    def __init__(self, hbm_budget, chunk=20, max_batches=2):
        self.L = _lib()
        p = self.L.qllg_server_create(int(hbm_budget), int(chunk), int(max_batches))
        if not p:
            raise RuntimeError(qll.last_error())
        self.p = c_void_p(p)
        self.vh = []
        self.bufs = {}

    def add_lattice(self, S, dims):
        lid = self.L.qllg_server_add_lattice(self.p, S)
        if lid < 0:
            raise RuntimeError(qll.last_error())
        self.vh.append(int(np.prod(dims))//2)
        return lid

    def submit(self, lattice, mass, shifts, tol, src):
        """src: [V/2, 6] float64 (even sites); returns the request id, or -1
        with qll.last_error() set when the request is refused"""
        src = np.ascontiguousarray(src, dtype=np.float64)
        n = max(1, len(shifts))
        vh = self.vh[lattice] if 0 <= lattice < len(self.vh) else 1
        outs = [np.zeros((vh, 6)) for _ in range(n)]
        sh = (c_double*max(1, len(shifts)))(*(shifts if shifts else [0.0]))
        op = (c_void_p*n)(*[o.ctypes.data for o in outs])
        rid = self.L.qllg_server_submit(self.p, lattice, mass, len(shifts), sh, tol,
                                        src.ctypes.data, op)
        if rid >= 0:
            self.bufs[rid] = (src, outs)
        return rid

    def step(self):
        n = self.L.qllg_server_step(self.p)
        if n < 0:
            raise RuntimeError(qll.last_error())
        return n

    def pending(self):
        return self.L.qllg_server_pending(self.p)

    def info(self, rid):
        inf = RequestInfo()
        if self.L.qllg_server_request(self.p, rid, ctypes.byref(inf)):
            raise RuntimeError(qll.last_error())
        return inf

    def result(self, rid):
        return self.bufs[rid][1]

    def stats(self):
        s = ServerInfo()
        self.L.qllg_server_stats(self.p, ctypes.byref(s))
        return s

    def drain(self, timeout=600.0, on_step=None):
        t0 = time.perf_counter()
        while self.pending():
            self.step()
            if on_step:
                on_step(self)
            if time.perf_counter() - t0 > timeout:
                raise RuntimeError("server did not drain in %.0f s" % timeout)

    def close(self):
        if self.p:
            self.L.qllg_server_destroy(self.p)
            self.p = None


def poisson_load(server, lattices, rate, nreq, seed=7, tol_choices=(1e-8, 1e-10),
                 mass_range=(0.005, 0.1), max_shifts=16, src_seed=6000):
    """drive server with nreq requests arriving as a Poisson process of the
    given rate (per second): each picks a lattice uniformly, m ~ U[mass_range],
    1..max_shifts shifts log-spaced in [1e-4, 1], a Gaussian even-site source
    and a tolerance from tol_choices.  Returns per-request records."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0/rate, size=nreq)
    arrive = np.cumsum(gaps)
    plan = []
    for i in range(nreq):
        lat = int(rng.integers(len(lattices)))
        m = float(rng.uniform(*mass_range))
        ns = int(rng.integers(1, max_shifts + 1))
        shifts = list(np.logspace(-4, 0, ns)) if ns > 1 else [1e-4]
        tol = float(tol_choices[int(rng.integers(len(tol_choices)))])
        plan.append((arrive[i], lat, m, shifts, tol))
    # a few Gaussian sources per lattice, made before the clock starts
    nsrc = 4
    srcs = [[qll.gen_source(tuple(d), src_seed + 100*li + j, 6, "even")[:int(np.prod(d))//2]
             for j in range(nsrc)] for li, d in enumerate(lattices)]
    recs = []
    t0 = time.perf_counter()
    k = 0
    while k < nreq or server.pending():
        now = time.perf_counter() - t0
        while k < nreq and plan[k][0] <= now:
            _, lat, m, shifts, tol = plan[k]
            rid = server.submit(lat, m, shifts, tol, srcs[lat][k % nsrc])
            if rid < 0:
                raise RuntimeError(qll.last_error())
            recs.append({"id": rid, "lattice": lat, "mass": m, "nshift": len(shifts), "tol": tol})
            k += 1
        server.step()
    for r in recs:
        inf = server.info(r["id"])
        r["status"] = inf.status
        r["latency_s"] = inf.seconds_total
        r["queued_s"] = inf.seconds_queued
        r["iters"] = max(inf.iters[:inf.ncol])
        r["max_true_rsq_over_tol2"] = max(inf.true_rsq[j]/r["tol"]**2 for j in range(inf.ncol))
    return recs, time.perf_counter() - t0
