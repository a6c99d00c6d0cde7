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
