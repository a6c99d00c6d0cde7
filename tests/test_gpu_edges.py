"""Edge cases of the GPU path: zero right-hand sides inside a batch, the
iteration limit, the smallest lattice, refused geometries and batch sizes.

Tolerances as elsewhere: FP64 Dslash 1e-12 relative to the oracle, solves
to the requested FP64 true residual."""
import ctypes
from ctypes import byref, c_double

import numpy as np
import pytest

import oracle_lib as orc
from inputs import asqtad_links, relerr
from qll_gb300 import qll

pytestmark = pytest.mark.gpu


def _op(dims, seed=1001):
    L = qll.load()
    u, u3 = asqtad_links(dims, seed)
    S = L.qllg_stag_create(qll.dims_c(dims), qll.vp_array(u), qll.vp_array(u3))
    assert S, qll.last_error()
    return L, ctypes.c_void_p(S), u, u3


@pytest.mark.parametrize("mode", [qll.SOLVE_DOUBLE, qll.SOLVE_MIXED_SINGLE, qll.SOLVE_MIXED_HALF])
def test_zero_rhs_in_a_batch(mode):
    """b = 0 (the reference's cgSolve divides by |b|^2 = 0) starts inactive:
    x stays 0 and takes no iterations, the other rhs converge as usual"""
    dims = (4, 4, 6, 8)
    L, S, u, u3 = _op(dims)
    nrhs = 4
    bs = [qll.gen_source(dims, 9300 + k, 6, "even") for k in range(nrhs)]
    bs[2][:] = 0
    xs = [np.full_like(bs[0], 7.0) for _ in range(nrhs)]
    info = qll.SolveInfo()
    its = L.qllg_stag_solve(S, nrhs, qll.vp_array(xs), qll.vp_array(bs),
                            (c_double*nrhs)(0.1, 0.1, 0.1, 0.1), 1e-16, 5000, mode, byref(info))
    assert its > 0, qll.last_error()
    Vh = bs[0].shape[0]//2
    assert info.iters[2] == 0
    assert np.all(xs[2][:Vh] == 0)
    for k in (0, 1, 3):
        assert np.all(np.isfinite(xs[k]))
        assert info.true_rsq[k] < 1e-16*1.0001
    L.qllg_stag_destroy(S)


@pytest.mark.parametrize("mode", [qll.SOLVE_DOUBLE, qll.SOLVE_MIXED_SINGLE])
def test_iteration_limit(mode):
    """maxits stops every rhs there; the solution so far is returned and the
    reported true residual says it has not converged"""
    dims = (4, 4, 6, 8)
    L, S, u, u3 = _op(dims)
    nrhs = 2
    bs = [qll.gen_source(dims, 9400 + k, 6, "even") for k in range(nrhs)]
    xs = [np.zeros_like(bs[0]) for _ in range(nrhs)]
    info = qll.SolveInfo()
    its = L.qllg_stag_solve(S, nrhs, qll.vp_array(xs), qll.vp_array(bs), (c_double*nrhs)(0.01, 0.02),
                            1e-30, 12, mode, byref(info))
    assert its == 12, (its, qll.last_error())
    for k in range(nrhs):
        assert info.iters[k] == 12
        assert np.all(np.isfinite(xs[k]))
        # not converged (CG minimises the A-norm of the error, so early
        # residuals may even exceed |b|)
        assert np.isfinite(info.true_rsq[k]) and info.true_rsq[k] > 1e-16
    if mode == qll.SOLVE_DOUBLE:
        # the oracle's cgSolveT stopped at the same place
        its_o, xo, _ = orc.solve2(dims, u, u3, 0.01, bs[0], 1e-30, 12, noscale=1)
        assert its_o == 12
        assert relerr(xs[0][:bs[0].shape[0]//2], xo[:bs[0].shape[0]//2]) < 1e-10
    L.qllg_stag_destroy(S)


def test_smallest_lattice():
    """4^4, the smallest extents the three-hop Naik term allows: the Dslash
    against the oracle and a solve to the true residual"""
    dims = (4, 4, 4, 4)
    L, S, u, u3 = _op(dims, 1007)
    y = qll.gen_source(dims, 9500, 6, "all")
    x = np.zeros_like(y)
    assert L.qllg_stag_dslash(S, x.ctypes.data, 0.3, y.ctypes.data, b"all") == 0, qll.last_error()
    assert relerr(x, orc.dslash(dims, u, u3, 0.3, y, "all")) < 1e-12
    b = qll.gen_source(dims, 9501, 6, "even")
    xs = [np.zeros_like(b)]
    info = qll.SolveInfo()
    assert L.qllg_stag_solve(S, 1, qll.vp_array(xs), qll.vp_array([b]), (c_double*1)(0.05), 1e-16,
                             5000, qll.SOLVE_MIXED_SINGLE, byref(info)) > 0, qll.last_error()
    assert info.true_rsq[0] < 1e-16*1.0001
    L.qllg_stag_destroy(S)


@pytest.mark.parametrize("dims", [(4, 4, 4, 5), (2, 4, 4, 4), (4, 4, 4, 0)])
def test_refused_geometry(dims):
    L = qll.load()
    V = max(1, int(np.prod(dims)))
    u = [np.zeros((V, 18)) for _ in range(8)]
    S = L.qllg_stag_create(qll.dims_c(dims), qll.vp_array(u), qll.vp_array(u))
    assert not S
    assert qll.last_error()
    L.qllg_clear_error()


def test_refused_batch_sizes():
    dims = (4, 4, 6, 8)
    L, S, u, u3 = _op(dims)
    b = qll.gen_source(dims, 9600, 6, "even")
    info = qll.SolveInfo()
    for n in (0, 17):
        xs = [np.zeros_like(b) for _ in range(max(n, 1))]
        bs = [b]*max(n, 1)
        rc = L.qllg_stag_solve(S, n, qll.vp_array(xs), qll.vp_array(bs),
                               (c_double*max(n, 1))(*[0.1]*max(n, 1)), 1e-16, 100,
                               qll.SOLVE_DOUBLE, byref(info))
        assert rc == -1
        assert "nrhs" in qll.last_error()
        L.qllg_clear_error()
    L.qllg_stag_destroy(S)


@pytest.mark.parametrize("mode", [qll.SOLVE_MIXED_SINGLE, qll.SOLVE_MIXED_HALF, qll.SOLVE_DOUBLE])
def test_true_residual_is_that_of_the_returned_x(mode):
    """true_rsq equals |b - A x|^2/|b|^2 of the returned x, computed by the
    oracle's dslashp2 (the mixed modes report the residual of their final
    FP64 reliable update, the FP64 mode recomputes it)"""
    dims = (4, 4, 6, 8)
    L, S, u, u3 = _op(dims)
    nrhs = 4
    masses = [0.05, 0.07, 0.1, 0.2]
    bs = [qll.gen_source(dims, 9700 + k, 6, "even") for k in range(nrhs)]
    xs = [np.zeros_like(bs[0]) for _ in range(nrhs)]
    info = qll.SolveInfo()
    its = L.qllg_stag_solve(S, nrhs, qll.vp_array(xs), qll.vp_array(bs), (c_double*nrhs)(*masses),
                            1e-16, 5000, mode, byref(info))
    assert its > 0, qll.last_error()
    Vh = bs[0].shape[0]//2
    for k in range(nrhs):
        Ax, _ = orc.dslashp2(dims, u, u3, masses[k], xs[k])
        r = bs[k][:Vh] - Ax[:Vh]
        tr = float(np.sum(r*r)/np.sum(bs[k][:Vh]*bs[k][:Vh]))
        assert tr < 1e-16*1.0001
        # FP64 roundings of A x differ between the two computations at about
        # 1e-16 |b|, a relative 1e-8 of |r| = 1e-8 |b|
        assert abs(info.true_rsq[k] - tr) <= 1e-6*tr, (k, info.true_rsq[k], tr)
    L.qllg_stag_destroy(S)


def _to_df(x):
    """float64 array -> the library's double-float layout: each real as the
    pair (float32(x), float32(x - float32(x)))"""
    hi = x.astype(np.float32)
    lo = (x - hi.astype(np.float64)).astype(np.float32)
    return np.stack([hi, lo], axis=-1).reshape(-1)


def test_double_float_dslash_against_fp64():
    """the double-float Dslash of the reliable updates (precision 4, FP32
    instructions) against the FP64 one on the same input: relative error at
    the double-float precision, about 2^-47 per operation"""
    torch = pytest.importorskip("torch")
    L = qll.load()
    vp = ctypes.c_void_p
    L.qllg_stag_vec_bytes.restype = ctypes.c_size_t
    L.qllg_stag_vec_bytes.argtypes = [vp, ctypes.c_int, ctypes.c_int]
    L.qllg_stag_dslash_device.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp, vp]
    for fb in (0, 1):
        dims = (4, 4, 6, 8)
        th = qll.gen_gauge(dims, 1009, 0.3, ks=True)
        c = qll.asqtad_coeffs()
        fn = L.qllg_stag_create_asqtad_fb if fb else L.qllg_stag_create_asqtad
        fn.restype = vp
        fn.argtypes = [ctypes.POINTER(ctypes.c_int), ctypes.POINTER(vp), ctypes.POINTER(qll.Fat7Coeffs)]
        S = vp(fn(qll.dims_c(dims), qll.vp_array(th), byref(c)))
        assert S.value, qll.last_error()
        for nrhs in (1, 4, 16):
            n = L.qllg_stag_vec_bytes(S, 0, nrhs)//8
            assert L.qllg_stag_vec_bytes(S, 4, nrhs) == 8*n
            x = np.random.default_rng(nrhs + 10*fb).standard_normal(n)
            src64 = torch.from_numpy(x).cuda()
            srcdf = torch.from_numpy(_to_df(x)).cuda()
            for parity in (0, 1):
                o64 = torch.zeros_like(src64)
                odf = torch.zeros_like(srcdf)
                torch.cuda.synchronize()
                assert L.qllg_stag_dslash_device(S, 0, nrhs, parity, vp(o64.data_ptr()),
                                                 vp(src64.data_ptr())) == 0, qll.last_error()
                assert L.qllg_stag_dslash_device(S, 4, nrhs, parity, vp(odf.data_ptr()),
                                                 vp(srcdf.data_ptr())) == 0, qll.last_error()
                torch.cuda.synchronize()
                pair = odf.cpu().numpy().reshape(-1, 2).astype(np.float64)
                got = pair[:, 0] + pair[:, 1]
                ref = o64.cpu().numpy()
                assert relerr(got, ref) < 1e-13, (fb, nrhs, parity, relerr(got, ref))
        L.qllg_stag_destroy(S)


def test_double_float_reliable_updates():
    """the mixed solve with its intermediate reliable updates in double-float
    (ru_df 1) and in FP64 (0): both reach the FP64 true residual, with
    iteration counts within a few of each other (and within the FP32 sloppy
    slowdown of the oracle's FP64 CG), and solutions that agree to the
    tolerance"""
    dims = (4, 4, 6, 8)
    L, S, u, u3 = _op(dims)
    L.qllg_set_param.argtypes = [ctypes.c_char_p, c_double]
    nrhs = 4
    masses = [0.02, 0.05, 0.1, 0.3]
    bs = [qll.gen_source(dims, 9800 + k, 6, "even") for k in range(nrhs)]
    Vh = bs[0].shape[0]//2
    res = {}
    for ru_df in (1, 0):
        L.qllg_set_param(b"ru_df", ru_df)
        xs = [np.zeros_like(bs[0]) for _ in range(nrhs)]
        info = qll.SolveInfo()
        its = L.qllg_stag_solve(S, nrhs, qll.vp_array(xs), qll.vp_array(bs),
                                (c_double*nrhs)(*masses), 1e-20, 5000, qll.SOLVE_MIXED_SINGLE,
                                byref(info))
        assert its > 0, qll.last_error()
        assert info.reliable_updates > nrhs
        res[ru_df] = (xs, [info.iters[k] for k in range(nrhs)], [info.true_rsq[k] for k in range(nrhs)])
    L.qllg_set_param(b"ru_df", 1)
    for k in range(nrhs):
        its_o, xo, _ = orc.solve2(dims, u, u3, masses[k], bs[k], 1e-20, 5000, noscale=1)
        for ru_df in (1, 0):
            xs, iters, tr = res[ru_df]
            assert tr[k] < 1e-20*1.0001, (ru_df, k, tr[k])
            # FP32 sloppy iterations converge more slowly at 1e-10 than FP64
            # CG (measured: 493 against 376 at m = 0.02)
            assert its_o - 5 <= iters[k] <= its_o*3//2 + 5, (ru_df, k, iters[k], its_o)
            # |x - x*| <= cond(A) |r|/|b|, cond about 10/m^2
            assert relerr(xs[k][:Vh], xo[:Vh]) < 1e-5, (ru_df, k)
        assert abs(res[1][1][k] - res[0][1][k]) <= 2, (k, res[1][1][k], res[0][1][k])
        assert relerr(res[1][0][k][:Vh], res[0][0][k][:Vh]) < 1e-6
    L.qllg_stag_destroy(S)
