"""qllg_stag_dslash_norm2_noalloc -- the Dslash + |out|^2 entry point that
allocates no device memory (its reduction scratch is a fixed file-scope
__device__ array) -- against the allocating qllg_stag_dslash_device on the
same inputs.

Tolerances: the output is produced by the same kernel instantiation as the
allocating call, so it must be bit-identical; the per-rhs norms must match
|out|^2 recomputed here in float64 to 1e-12 relative for FP64 spinors, to
1e-6 for FP32 spinors (each thread sums its squares in FP32 with Kahan
compensation before the FP64 grid reduction) and to 2e-4 for the 16-bit
layout (the kernel sums the values before they are rounded to 16 bits).  Two calls in a row are checked, so a counter or
partial left over by the first call would show in the second.  Every call
is also checked to allocate nothing: the library's count of device
allocations stays put and the device's free memory does not drop.

The file sorts last so it runs after every other test; it also passes
alone in a fresh process."""
import ctypes

import pytest

from qll_gb300 import qll

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

DIMS = (8, 8, 8, 16)
VP, I = ctypes.c_void_p, ctypes.c_int


def _lib():
    L = qll.load()
    L.qllg_stag_create_asqtad.restype = VP
    L.qllg_stag_create_asqtad.argtypes = [ctypes.POINTER(ctypes.c_int), ctypes.POINTER(VP),
                                          ctypes.POINTER(qll.Fat7Coeffs)]
    L.qllg_stag_vec_bytes.restype = ctypes.c_size_t
    L.qllg_stag_vec_bytes.argtypes = [VP, I, I]
    L.qllg_stag_dslash_device.argtypes = [VP, I, I, I, VP, VP]
    L.qllg_stag_dslash_norm2_noalloc.argtypes = [VP, I, I, I, VP, VP, VP]
    L.qllg_device_alloc_count.restype = ctypes.c_ulonglong
    return L


def _call_without_allocating(L, *args):
    """one no-allocation call, checked to allocate nothing: the library's
    own allocation count stays put, and so does the device's free memory
    (which would drop if the call loaded a kernel or the scratch)"""
    torch.cuda.synchronize()
    n0 = L.qllg_device_alloc_count()
    free0 = torch.cuda.mem_get_info()[0]
    rc = L.qllg_stag_dslash_norm2_noalloc(*args)
    torch.cuda.synchronize()
    assert L.qllg_device_alloc_count() == n0, "the no-allocation call allocated device memory"
    assert torch.cuda.mem_get_info()[0] >= free0, "device free memory dropped during the call"
    return rc


@pytest.fixture(scope="module")
def op():
    L = _lib()
    thin = qll.gen_gauge(DIMS, 1001, 0.3, ks=True)
    coef = qll.asqtad_coeffs()
    S = L.qllg_stag_create_asqtad(qll.dims_c(DIMS), qll.vp_array(thin), ctypes.byref(coef))
    assert S, qll.last_error()
    yield L, VP(S)
    L.qllg_stag_destroy(VP(S))


def _input(L, S, prec, nrhs, seed):
    nb = L.qllg_stag_vec_bytes(S, prec, nrhs)
    g = torch.Generator(device="cuda").manual_seed(seed)
    if prec == 0:
        return torch.randn(nb//8, dtype=torch.float64, device="cuda", generator=g)
    src = torch.randn(nb//4, dtype=torch.float32, device="cuda", generator=g)
    if prec == 2:
        # six int16 from random bits, then a per-(site, rhs) scale of 1
        src = src.view(-1, 4)
        src[:, 3] = 1.0
        src = src.reshape(-1)
    return src


def _norm2(out, prec, nrhs):
    """|out|^2 per rhs in float64 from the library layouts: [3][Vh][nrhs]
    complex for FP64/FP32, one int4 (six int16 + float scale) per (site,
    rhs) for the 16-bit layout."""
    if prec in (0, 1):
        v = out.to(torch.float64).view(3, -1, nrhs, 2)
        return (v*v).sum(dim=(0, 1, 3))
    w = out.view(torch.int32).view(-1, 4)
    lo = ((w[:, :3] & 0xFFFF) ^ 0x8000) - 0x8000
    hi = w[:, :3] >> 16
    s = w[:, 3].contiguous().view(torch.float32).to(torch.float64)/32767.0
    vals = torch.cat([lo, hi], dim=1).to(torch.float64)*s[:, None]
    return (vals*vals).sum(dim=1).view(-1, nrhs).sum(dim=0)


@pytest.mark.parametrize("prec", [0, 1, 2])
@pytest.mark.parametrize("nrhs", [1, 4, 16])
def test_noalloc_matches_dslash_device(op, prec, nrhs):
    L, S = op
    tol = {0: 1e-12, 1: 1e-6, 2: 2e-4}[prec]
    for parity in (0, 1):
        src = _input(L, S, prec, nrhs, 17 + 3*prec + nrhs + parity)
        ref = torch.zeros_like(src)
        torch.cuda.synchronize()
        # the allocating entry point (also creates the links of this
        # precision, which the no-allocation call requires)
        assert L.qllg_stag_dslash_device(S, prec, nrhs, parity, VP(ref.data_ptr()),
                                         VP(src.data_ptr())) == 0, qll.last_error()
        torch.cuda.synchronize()
        want = _norm2(ref, prec, nrhs)
        for call in range(2):
            out = torch.full_like(src, float("nan"))
            nrm = torch.full((nrhs,), float("nan"), dtype=torch.float64, device="cuda")
            rc = _call_without_allocating(L, S, prec, nrhs, parity, VP(out.data_ptr()),
                                          VP(src.data_ptr()), VP(nrm.data_ptr()))
            assert rc == 0, qll.last_error()
            torch.cuda.synchronize()
            assert torch.equal(out.view(torch.uint8), ref.view(torch.uint8)), \
                f"output differs (prec {prec}, nrhs {nrhs}, parity {parity}, call {call})"
            rel = ((nrm - want).abs()/want).max().item()
            assert rel < tol, f"norm rel err {rel} (prec {prec}, nrhs {nrhs}, call {call})"


def test_noalloc_with_the_grid_at_its_block_cap():
    """24^3x48 at one rhs needs more blocks than the scratch's 1024; the
    launch is capped there and the grid-stride loop covers the rest"""
    L = _lib()
    dims = (24, 24, 24, 48)
    thin = qll.gen_gauge(dims, 1003, 0.3, ks=True)
    coef = qll.asqtad_coeffs()
    S = VP(L.qllg_stag_create_asqtad(qll.dims_c(dims), qll.vp_array(thin), ctypes.byref(coef)))
    assert S.value, qll.last_error()
    try:
        for prec in (0, 1):
            src = _input(L, S, prec, 1, 99 + prec)
            ref = torch.zeros_like(src)
            torch.cuda.synchronize()
            assert L.qllg_stag_dslash_device(S, prec, 1, 1, VP(ref.data_ptr()),
                                             VP(src.data_ptr())) == 0, qll.last_error()
            torch.cuda.synchronize()
            want = _norm2(ref, prec, 1)
            for call in range(2):
                out = torch.full_like(src, float("nan"))
                nrm = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
                assert _call_without_allocating(L, S, prec, 1, 1, VP(out.data_ptr()),
                                                VP(src.data_ptr()),
                                                VP(nrm.data_ptr())) == 0, qll.last_error()
                torch.cuda.synchronize()
                assert torch.equal(out.view(torch.uint8), ref.view(torch.uint8))
                assert abs(nrm.item() - want.item())/want.item() < (1e-12 if prec == 0 else 1e-6)
    finally:
        L.qllg_stag_destroy(S)


def test_noalloc_refuses_what_it_cannot_do_without_allocating():
    L = _lib()
    thin = qll.gen_gauge(DIMS, 1002, 0.3, ks=True)
    coef = qll.asqtad_coeffs()
    S = VP(L.qllg_stag_create_asqtad(qll.dims_c(DIMS), qll.vp_array(thin), ctypes.byref(coef)))
    assert S.value, qll.last_error()
    try:
        nb = L.qllg_stag_vec_bytes(S, 1, 4)
        src = torch.zeros(nb//4, dtype=torch.float32, device="cuda")
        out = torch.empty_like(src)
        nrm = torch.empty(16, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        # FP32 links were never created on this operator
        assert L.qllg_stag_dslash_norm2_noalloc(S, 1, 4, 0, VP(out.data_ptr()),
                                                VP(src.data_ptr()), VP(nrm.data_ptr())) == -1
        assert "not created" in qll.last_error()
        L.qllg_clear_error()
        # more rhs than the fixed scratch holds, and a batch size the kernels
        # do not have
        for bad in (32, 3):
            assert L.qllg_stag_dslash_norm2_noalloc(S, 0, bad, 0, VP(out.data_ptr()),
                                                    VP(src.data_ptr()),
                                                    VP(nrm.data_ptr())) == -1
            assert "nrhs" in qll.last_error()
            L.qllg_clear_error()
    finally:
        L.qllg_stag_destroy(S)
