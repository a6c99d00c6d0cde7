"""GPU: the host-array transfers of the solver API.  Copies of at least
1 MiB between page-locked host arrays and the device run on the SMs
(parameter host_copy_sm); pageable arrays, small or unaligned ones take a
copy engine.  Both paths must move the same bytes."""
import ctypes
from ctypes import POINTER, byref, c_int, c_void_p

import numpy as np
import pytest

from qll_gb300 import qll

pytestmark = pytest.mark.gpu


def _pinned_views(torch, nblk, n, offset_bytes):
    """nblk float64 arrays of n elements inside one page-locked buffer, the
    first starting offset_bytes past the buffer's start"""
    extra = (offset_bytes + 7)//8
    buf = torch.empty(nblk*n + extra + 2, dtype=torch.float64, pin_memory=True)
    raw = buf.numpy().view(np.uint8)
    views = [raw[offset_bytes + 8*n*k: offset_bytes + 8*n*(k + 1)].view(np.float64) for k in range(nblk)]
    return buf, views


def test_host_copies_sm_and_copy_engine_agree():
    torch = pytest.importorskip("torch")
    dims = (16, 16, 16, 32)
    L = qll.load()
    L.qllg_stag_create_asqtad.restype = c_void_p
    L.qllg_stag_create_asqtad.argtypes = [POINTER(c_int), POINTER(c_void_p), POINTER(qll.Fat7Coeffs)]
    L.qllg_set_param.argtypes = [ctypes.c_char_p, ctypes.c_double]
    L.qllg_stag_vec_alloc.restype = c_void_p
    L.qllg_launch_count.restype = ctypes.c_ulonglong
    thin = qll.gen_gauge(dims, 1007, 0.3, ks=True)
    S = c_void_p(L.qllg_stag_create_asqtad(qll.dims_c(dims), qll.vp_array(thin), byref(qll.asqtad_coeffs())))
    assert S.value, qll.last_error()
    nrhs = 4
    srcs = [qll.gen_source(dims, 9100 + k, 6, "even") for k in range(nrhs)]
    n = srcs[0].size                               # [V][6]; the vectors hold the even half
    nh = n//2
    assert 8*nh >= 1 << 20                         # large enough for the SM copy
    dev = c_void_p(L.qllg_stag_vec_alloc(S, nrhs))
    assert dev.value, qll.last_error()

    def upload(arrs):
        c0 = L.qllg_launch_count()
        assert L.qllg_stag_vec_upload(S, dev, nrhs, qll.vp_array(arrs)) == 0, qll.last_error()
        torch.cuda.synchronize()
        return L.qllg_launch_count() - c0

    def download(arrs):
        c0 = L.qllg_launch_count()
        assert L.qllg_stag_vec_download(S, dev, nrhs, qll.vp_array(arrs)) == 0, qll.last_error()
        return L.qllg_launch_count() - c0

    # the reference: pageable arrays, copy engine
    L.qllg_set_param(b"host_copy_sm", 1)
    base_up = upload(srcs)
    outs = [np.full_like(s, np.nan) for s in srcs]
    base_down = download(outs)
    for o, s in zip(outs, srcs):
        assert np.array_equal(o.reshape(-1)[:nh], s.reshape(-1)[:nh])
    for sm in (1, 0):
        L.qllg_set_param(b"host_copy_sm", sm)
        for off in (0, 16, 8):
            buf_in, vin = _pinned_views(torch, nrhs, n, off)
            for v, s in zip(vin, srcs):
                v[:] = s.reshape(-1)
            up = upload([v.reshape(srcs[0].shape) for v in vin])
            buf_out, vout = _pinned_views(torch, nrhs, n, off)
            for v in vout:
                v[:] = np.nan
            down = download(vout)
            for v, s in zip(vout, srcs):
                assert np.array_equal(v[:nh], s.reshape(-1)[:nh]), (sm, off)
            # the SM copy ran (one launch a rhs each way) exactly where it applies
            sm_path = sm == 1 and off % 16 == 0
            assert up - base_up == (nrhs if sm_path else 0), (sm, off, up, base_up)
            assert down - base_down == (nrhs if sm_path else 0), (sm, off, down, base_down)
            del buf_in, buf_out
    L.qllg_set_param(b"host_copy_sm", 1)
    # a solve through the host-array API from page-locked arrays gives
    # bitwise the solution of the same solve from pageable arrays
    masses = (ctypes.c_double*nrhs)(*[0.05 + 0.01*k for k in range(nrhs)])
    xs_a = [np.zeros_like(s) for s in srcs]
    info = qll.SolveInfo()
    assert L.qllg_stag_solve(S, nrhs, qll.vp_array(xs_a), qll.vp_array(srcs), masses, 1e-14, 4000,
                             qll.SOLVE_MIXED_SINGLE, byref(info)) > 0, qll.last_error()
    buf_b, bp = _pinned_views(torch, nrhs, n, 0)
    buf_x, xp = _pinned_views(torch, nrhs, n, 0)
    for v, s in zip(bp, srcs):
        v[:] = s.reshape(-1)
    for v in xp:
        v[:] = 0
    assert L.qllg_stag_solve(S, nrhs, qll.vp_array(xp), qll.vp_array(bp), masses, 1e-14, 4000,
                             qll.SOLVE_MIXED_SINGLE, byref(info)) > 0, qll.last_error()
    for a, b in zip(xs_a, xp):
        assert np.array_equal(a.reshape(-1)[:nh], b[:nh])
    del buf_b, buf_x
    L.qllg_stag_vec_free(dev)
    L.qllg_stag_destroy(S)
