"""The solve-request loop (qllg_server_*): continuous batching, HBM
admission and the invariance of a request's result to the requests running
beside it.

Tolerance of the invariance test: bitwise.  A column's arithmetic never
involves another column, so a request must give exactly the same solution
and iteration counts alone and in the mix (whatever column it lands in and
whenever it is admitted).  Accuracy: every shift reaches the requested
true residual, and one shift is compared with the oracle's FP64 CG."""
import ctypes

import numpy as np
import pytest

import oracle_lib as orc
from inputs import relerr
from qll_gb300 import qll
from qll_gb300 import serve

pytestmark = pytest.mark.gpu

LATS = [(8, 8, 8, 8), (8, 8, 8, 12)]
BIG = 64 << 30


def _server(budget=BIG, chunk=7, max_batches=2):
    V = serve.Server(budget, chunk=chunk, max_batches=max_batches)
    ops = []
    for i, d in enumerate(LATS):
        S = serve.asqtad_operator(d, 5001 + i, 0.3)
        ops.append(S)
        V.add_lattice(S, d)
    return V, ops


def _close(V, ops):
    V.close()
    for S in ops:
        serve._lib().qllg_stag_destroy(S)


def _src(d, seed):
    return qll.gen_source(d, seed, 6, "even")[:int(np.prod(d))//2].copy()


PROBE = dict(lattice=1, mass=0.05, shifts=[0.0, 1e-3, 0.1], tol=1e-8)


def test_request_same_alone_and_in_the_mix():
    src = _src(LATS[1], 7100)
    V, ops = _server()
    rid = V.submit(PROBE["lattice"], PROBE["mass"], PROBE["shifts"], PROBE["tol"], src)
    assert rid >= 0, qll.last_error()
    V.drain()
    alone = [x.copy() for x in V.result(rid)]
    inf = V.info(rid)
    its_alone = list(inf.iters[:inf.ncol])
    for k in range(inf.ncol):
        assert inf.true_rsq[k] < PROBE["tol"]**2, (k, inf.true_rsq[k])
    _close(V, ops)

    # the same request admitted into running batches, between others
    V, ops = _server()
    rng = np.random.default_rng(3)
    others = []
    for j in range(5):
        lat = j % 2
        ns = int(rng.integers(1, 6))
        others.append(V.submit(lat, float(rng.uniform(0.02, 0.2)),
                               list(np.logspace(-4, 0, ns)), 1e-8, _src(LATS[lat], 7200 + j)))
    for _ in range(3):
        V.step()
    rid = V.submit(PROBE["lattice"], PROBE["mass"], PROBE["shifts"], PROBE["tol"], src)
    for j in range(5, 9):
        lat = j % 2
        others.append(V.submit(lat, 0.03 + 0.01*j, [0.0, 0.01], 1e-10, _src(LATS[lat], 7200 + j)))
        V.step()
    stats = []
    V.drain(on_step=lambda s: stats.append(s.stats().busy_columns))
    assert max(stats) > len(PROBE["shifts"])          # it really ran beside others
    inf = V.info(rid)
    assert list(inf.iters[:inf.ncol]) == its_alone
    for k, x in enumerate(V.result(rid)):
        assert np.array_equal(x, alone[k]), k
    for o in others:
        oi = V.info(o)
        assert oi.status == 2
        tol = 1e-8 if o < 5 else 1e-10
        for k in range(oi.ncol):
            assert oi.true_rsq[k] < tol**2*1.0001, (o, k, oi.true_rsq[k])
    _close(V, ops)

    # shift 0 against the oracle's FP64 CG (normalised system, no mass scaling)
    d = LATS[1]
    thin = qll.gen_gauge(d, 5002, 0.3, ks=True)
    fl, ll = orc.smear_fat7(d, thin, qll.asqtad_coeffs())
    u, u3 = [None]*8, [None]*8
    for mu in range(4):
        u[2*mu], u[2*mu+1] = fl[mu], orc.negadj_back(d, fl[mu], mu, 1)
        u3[2*mu], u3[2*mu+1] = ll[mu], orc.negadj_back(d, ll[mu], mu, 3)
    b = np.zeros((int(np.prod(d)), 6))
    b[:src.shape[0]] = src
    its_o, xo, _ = orc.solve2(d, u, u3, PROBE["mass"], b, 1e-16, 5000, noscale=1)
    assert relerr(alone[0], xo[:src.shape[0]]) < 1e-7


def test_admission_within_the_hbm_budget():
    """a budget with room for the links and one batch: requests of the two
    lattices take turns in one batch slot, and all complete"""
    V0, ops0 = _server()
    links = V0.stats().used_bytes
    _close(V0, ops0)
    # one 16-column batch of the larger lattice, plus slack below a second
    Vh = int(np.prod(LATS[1]))//2
    batch = 16*Vh*(4*24 + 5*48) + 48*Vh + (1 << 20)
    V, ops = _server(budget=links + batch + batch//2, max_batches=1)
    ids = []
    for j in range(6):
        lat = j % 2
        ids.append(V.submit(lat, 0.05, [0.0, 1e-2], 1e-8, _src(LATS[lat], 7300 + j)))
    most = []
    V.drain(on_step=lambda s: most.append(s.stats().batches))
    assert max(most) == 1
    for i in ids:
        inf = V.info(i)
        assert inf.status == 2 and all(inf.true_rsq[k] < 1e-16 for k in range(inf.ncol))
    _close(V, ops)


def test_refused_requests():
    V, ops = _server()
    src = _src(LATS[0], 7400)
    assert V.submit(0, 0.05, list(np.logspace(-4, 0, 17)), 1e-8, src) == -1
    assert "shifts" in qll.last_error()
    qll.load().qllg_clear_error()
    assert V.submit(5, 0.05, [], 1e-8, src) == -1
    assert "lattice" in qll.last_error()
    qll.load().qllg_clear_error()
    assert V.submit(0, 0.0, [], 1e-8, src) == -1
    qll.load().qllg_clear_error()
    _close(V, ops)


def test_nan_request_fails_alone():
    """a request whose host source holds a NaN ends FAILED (status 3) while
    the request sharing its batch converges bitwise as it does alone"""
    src = _src(LATS[1], 7100)
    V, ops = _server()
    rid = V.submit(PROBE["lattice"], PROBE["mass"], PROBE["shifts"], PROBE["tol"], src)
    V.drain()
    alone = [x.copy() for x in V.result(rid)]
    its_alone = list(V.info(rid).iters[:V.info(rid).ncol])
    _close(V, ops)

    V, ops = _server()
    bad = _src(LATS[1], 7101)
    bad[17, 3] = np.nan
    rbad = V.submit(PROBE["lattice"], 0.07, [0.0, 1e-2], 1e-8, bad)
    rid = V.submit(PROBE["lattice"], PROBE["mass"], PROBE["shifts"], PROBE["tol"], src)
    assert rbad >= 0 and rid >= 0, qll.last_error()
    busy = []
    V.drain(on_step=lambda s: busy.append(s.stats().busy_columns))
    assert max(busy) >= len(PROBE["shifts"]) + 1         # they shared a batch
    assert V.info(rbad).status == 3
    inf = V.info(rid)
    assert inf.status == 2
    assert list(inf.iters[:inf.ncol]) == its_alone
    for k, x in enumerate(V.result(rid)):
        assert np.array_equal(x, alone[k]), k
    _close(V, ops)


def test_allocation_failure_at_batch_creation_keeps_the_queue():
    """a device allocation that fails while the first batch is made (an
    injected cudaMalloc failure) fails that scheduling pass with an error
    and leaves every request queued; the next passes admit and finish them"""
    L = serve._lib()
    L.qllg_set_param.argtypes = [ctypes.c_char_p, ctypes.c_double]
    L.qllg_device_alloc_count.restype = ctypes.c_ulonglong
    V, ops = _server()
    ids = [V.submit(j % 2, 0.05 + 0.01*j, [0.0, 1e-2], 1e-8, _src(LATS[j % 2], 7500 + j))
           for j in range(3)]
    L.qllg_set_param(b"fail_alloc_at", float(L.qllg_device_alloc_count() + 1))
    try:
        with pytest.raises(RuntimeError, match="injected failure"):
            V.step()
    finally:
        L.qllg_set_param(b"fail_alloc_at", 0.0)
    L.qllg_clear_error()
    assert V.pending() == 3
    assert all(V.info(i).status == 0 for i in ids)
    assert V.stats().batches == 0
    V.drain()
    for i in ids:
        inf = V.info(i)
        assert inf.status == 2
        assert all(inf.true_rsq[k] < 1e-16 for k in range(inf.ncol))
    _close(V, ops)
