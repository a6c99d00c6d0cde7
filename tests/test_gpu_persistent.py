"""The persistent CG (one cooperative launch for the whole loop on small
lattices) against the multi-launch graph loop and the oracle: same
iteration counts (FP64 within 1; mixed within 3: its intermediate reliable
updates are FP64 where the loop's are double-float), solutions within the
solver tolerance of each other and within 1e-7 of the oracle's FP64
solve2; and its bounded grid-barrier waits: a barrier that can never be
passed (one arrival more than the grid) makes the solve fail with an
error after the poll limit instead of hanging, and the next solve works."""
import ctypes
from ctypes import byref, c_double

import numpy as np
import pytest

import oracle_lib as orc
from inputs import asqtad_links, relerr
from qll_gb300 import qll

pytestmark = pytest.mark.gpu

DIMS = (8, 8, 8, 8)


def _op():
    L = qll.load()
    L.qllg_set_param.argtypes = [ctypes.c_char_p, c_double]
    L.qllg_stag_last_solve_persistent.argtypes = [ctypes.c_void_p]
    u, u3 = asqtad_links(DIMS)
    S = L.qllg_stag_create(qll.dims_c(DIMS), qll.vp_array(u), qll.vp_array(u3))
    assert S, qll.last_error()
    return L, ctypes.c_void_p(S), u, u3


def _solve(L, S, bs, masses, mode, persistent):
    L.qllg_set_param(b"persistent", persistent)
    n = len(bs)
    xs = [np.zeros_like(bs[0]) for _ in range(n)]
    info = qll.SolveInfo()
    its = L.qllg_stag_solve(S, n, qll.vp_array(xs), qll.vp_array(bs), (c_double*n)(*masses), 1e-16,
                            5000, mode, byref(info))
    L.qllg_set_param(b"persistent", 1)
    assert its > 0, qll.last_error()
    assert L.qllg_stag_last_solve_persistent(S) == persistent
    return xs, info


@pytest.mark.parametrize("mode", [qll.SOLVE_DOUBLE, qll.SOLVE_MIXED_SINGLE])
@pytest.mark.parametrize("nrhs", [1, 4])
def test_persistent_matches_graph_loop_and_oracle(mode, nrhs):
    L, S, u, u3 = _op()
    try:
        masses = [0.1 + 0.03*k for k in range(nrhs)]
        bs = [qll.gen_source(DIMS, 2100 + k, 6, "even") for k in range(nrhs)]
        xp, ip = _solve(L, S, bs, masses, mode, 1)
        xg, ig = _solve(L, S, bs, masses, mode, 0)
        Vh = bs[0].shape[0]//2
        for k in range(nrhs):
            assert abs(ip.iters[k] - ig.iters[k]) <= (1 if mode == qll.SOLVE_DOUBLE else 3), \
                (k, ip.iters[k], ig.iters[k])
            assert ip.true_rsq[k] < 1e-16*1.0001, (k, ip.true_rsq[k])
            assert relerr(xp[k][:Vh], xg[k][:Vh]) < 1e-7
            its_o, xo, _ = orc.solve2(DIMS, u, u3, masses[k], bs[k], 1e-16, 5000, noscale=1)
            assert relerr(xp[k][:Vh], xo[:Vh]) < 1e-7
            if mode == qll.SOLVE_DOUBLE:
                assert abs(ip.iters[k] - its_o) <= 1
        if mode == qll.SOLVE_MIXED_SINGLE:
            assert ip.reliable_updates > 0
    finally:
        L.qllg_stag_destroy(S)


def test_barrier_wait_runs_out_with_an_error():
    L, S, u, u3 = _op()
    try:
        b = qll.gen_source(DIMS, 2100, 6, "even")
        x = np.zeros_like(b)
        info = qll.SolveInfo()
        L.qllg_set_param(b"cg_barrier_extra", 1)       # an arrival that never comes
        L.qllg_set_param(b"wait_polls", 2000)
        try:
            its = L.qllg_stag_solve(S, 1, qll.vp_array([x]), qll.vp_array([b]), (c_double*1)(0.1),
                                    1e-16, 5000, qll.SOLVE_DOUBLE, byref(info))
        finally:
            L.qllg_set_param(b"cg_barrier_extra", 0)
            L.qllg_set_param(b"wait_polls", 2e7)
        assert its < 0
        assert "barrier wait ran out" in qll.last_error()
        L.qllg_clear_error()
        # the context is still usable: the same solve now runs to the end
        xs, inf = _solve(L, S, [b], [0.1], qll.SOLVE_DOUBLE, 1)
        assert inf.true_rsq[0] < 1e-16*1.0001
    finally:
        L.qllg_stag_destroy(S)


@pytest.mark.parametrize("pipeline", [11, 20, 22])
def test_bulk_pipeline_wait_runs_out_with_an_error(pipeline):
    """the copy pipelines' waits (the bulk-copy kernel, variant 11, and the
    per-warp tensor-copy kernels, variants 20 and 22) take the same limit: with
    their copies not issued (bulk_wait_test) the first waits run out after
    the limit, the launch records the error flag and returns; with copies
    issued again the same launch is bitwise the register kernel's"""
    torch = pytest.importorskip("torch")
    L, S, u, u3 = _op()
    try:
        L.qllg_stag_vec_bytes.restype = ctypes.c_size_t
        L.qllg_stag_vec_bytes.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        L.qllg_stag_dslash_device.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                              ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        n = L.qllg_stag_vec_bytes(S, 1, 16)//4
        g = torch.Generator(device="cuda").manual_seed(5)
        src = torch.randn(n, dtype=torch.float32, device="cuda", generator=g)
        outs = []
        assert L.qllg_k_bulk_error(1) >= 0
        for variant, test in ((pipeline, 1), (pipeline, 0), (10, 0)):
            L.qllg_set_param(b"dslash_variant", variant)
            L.qllg_set_param(b"bulk_wait_test", test)
            L.qllg_set_param(b"wait_polls", 2e5 if test else 2e7)
            dst = torch.zeros_like(src)
            torch.cuda.synchronize()
            rc = L.qllg_stag_dslash_device(S, 1, 16, 1, ctypes.c_void_p(dst.data_ptr()),
                                           ctypes.c_void_p(src.data_ptr()))
            torch.cuda.synchronize()
            L.qllg_set_param(b"dslash_variant", -1)
            L.qllg_set_param(b"bulk_wait_test", 0)
            L.qllg_set_param(b"wait_polls", 2e7)
            assert rc == 0, qll.last_error()
            outs.append((L.qllg_k_bulk_error(1), dst))
        assert outs[0][0] == 1           # the waits ran out
        assert outs[1][0] == 0 and outs[2][0] == 0
        assert torch.equal(outs[1][1], outs[2][1])
    finally:
        L.qllg_stag_destroy(S)


def _wilson(dims):
    from inputs import wilson_links
    L = qll.load()
    L.qllg_set_param.argtypes = [ctypes.c_char_p, c_double]
    L.qllg_wilson_create.restype = ctypes.c_void_p
    L.qllg_wilson_create.argtypes = [ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_void_p)]
    L.qllg_wilson_solve.restype = ctypes.c_int
    L.qllg_wilson_solve.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, c_double,
                                    c_double, ctypes.c_int, ctypes.c_int, ctypes.POINTER(qll.SolveInfo)]
    L.qllg_wilson_destroy.argtypes = [ctypes.c_void_p]
    W = L.qllg_wilson_create(qll.dims_c(dims), qll.vp_array(list(wilson_links(dims))))
    assert W, qll.last_error()
    return L, ctypes.c_void_p(W)


def _wsolve(L, W, b, persistent):
    L.qllg_set_param(b"wilson_persistent", persistent)
    x = np.zeros_like(b)
    info = qll.SolveInfo()
    try:
        its = L.qllg_wilson_solve(W, x.ctypes.data, b.ctypes.data, 1/(2*0.12) - 4, 1e-17, 5000,
                                  qll.SOLVE_MIXED_SINGLE, byref(info))
    finally:
        L.qllg_set_param(b"wilson_persistent", 1)
    return its, x, info


@pytest.mark.parametrize("dims", [(8, 8, 8, 8), (8, 8, 8, 16)])
def test_wilson_persistent_matches_graph_loop(dims):
    """the persistent FP32 iterations of the mixed Wilson CGNR (cooperative
    launches between the reliable updates) against the graph loop: their
    sums are reduced in another order, so reliable updates and iterations
    agree within one, solutions within 1e-6
    of each other and the true residual of S x = b below 1e-8 in both"""
    L, W = _wilson(dims)
    try:
        b = qll.gen_source(dims, 77, 24, "even")
        itp, xp, ip = _wsolve(L, W, b, 1)
        itg, xg, ig = _wsolve(L, W, b, 0)
        assert itp > 0 and itg > 0, qll.last_error()
        assert abs(itp - itg) <= 1, (itp, itg)
        assert ip.reliable_updates >= 1 and abs(ip.reliable_updates - ig.reliable_updates) <= 1
        assert ip.true_rsq[0] < 1e-16 and ig.true_rsq[0] < 1e-16
        assert relerr(xp, xg) < 1e-6
    finally:
        L.qllg_wilson_destroy(W)


def test_wilson_persistent_barrier_wait_runs_out_with_an_error():
    """a barrier of the persistent CGNR that can never be passed ends the
    solve with an error after the poll limit; the next solve works"""
    dims = (8, 8, 8, 8)
    L, W = _wilson(dims)
    try:
        b = qll.gen_source(dims, 78, 24, "even")
        L.qllg_set_param(b"cg_barrier_extra", 1)
        L.qllg_set_param(b"wait_polls", 2000)
        try:
            its, _, _ = _wsolve(L, W, b, 1)
        finally:
            L.qllg_set_param(b"cg_barrier_extra", 0)
            L.qllg_set_param(b"wait_polls", 2e7)
        assert its < 0
        assert "barrier wait ran out" in qll.last_error()
        L.qllg_clear_error()
        its, _, info = _wsolve(L, W, b, 1)
        assert its > 0 and info.true_rsq[0] < 1e-16
    finally:
        L.qllg_wilson_destroy(W)


def test_wilson_persistent_stops_at_maxits():
    """a solve capped below convergence stops at the cap in the persistent
    loop as in the graph loop, with its FP64 residual reported"""
    dims = (8, 8, 8, 8)
    L, W = _wilson(dims)
    try:
        b = qll.gen_source(dims, 79, 24, "even")
        out = {}
        for persistent in (1, 0):
            L.qllg_set_param(b"wilson_persistent", persistent)
            x = np.zeros_like(b)
            info = qll.SolveInfo()
            try:
                its = L.qllg_wilson_solve(W, x.ctypes.data, b.ctypes.data, 1/(2*0.12) - 4, 1e-17, 7,
                                          qll.SOLVE_MIXED_SINGLE, byref(info))
            finally:
                L.qllg_set_param(b"wilson_persistent", 1)
            assert its == 7, (persistent, its, qll.last_error())
            assert info.true_rsq[0] > 1e-16
            out[persistent] = x
        assert relerr(out[1], out[0]) < 1e-5
    finally:
        L.qllg_wilson_destroy(W)
