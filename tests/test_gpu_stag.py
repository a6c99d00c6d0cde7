"""GPU parity of the asqtad staggered path against the CPU oracle, through
the C-ABI: neighbour tables (bit-exact), dslash2 (FP64 1e-12, FP32 1e-5
relative), solve2 (same iteration count in FP64; solutions within 10x the
solver tolerance), multi-rhs and mixed-precision solves (true residual
1e-8 in FP64)."""
import ctypes
from ctypes import byref, c_double, c_float, c_int

import numpy as np
import pytest

import oracle_lib as orc
from inputs import as_dtype, asqtad_links, relerr
from qll_gb300 import qll

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _multi_launch_loop():
    """these tests are about the multi-launch solver loop (fused Dslash
    epilogues, graph capture, reliable-update kernels, launch shapes): on
    their small lattices the persistent CG would take the solves, so it is
    off here (tests/test_gpu_persistent.py covers it)"""
    L = qll.load()
    L.qllg_set_param.argtypes = [ctypes.c_char_p, ctypes.c_double]
    L.qllg_set_param(b"persistent", 0)
    yield
    L.qllg_set_param(b"persistent", 1)

DIMS = (4, 4, 6, 8)
TOL = {"D": 1e-12, "F": 1e-5}
DT = {"D": np.float64, "F": np.float32}
CT = {"D": c_double, "F": c_float}


def _links(prec, dims=DIMS):
    u, u3 = asqtad_links(dims)
    return as_dtype(u, DT[prec]), as_dtype(u3, DT[prec])


@pytest.mark.parametrize("dims", [(4, 4, 6, 8), (8, 4, 4, 6)])
def test_neighbour_tables_bit_exact(dims):
    L = qll.load()
    V = int(np.prod(dims))
    Vh = V//2
    for parity in (0, 1):
        for slot in range(16):
            out = np.zeros(Vh, dtype=np.int32)
            rc = L.qllg_stag_nbr_table(qll.dims_c(dims), parity, slot, qll.ptr(out))
            assert rc == 0, qll.last_error()
            ref = orc.stag_slot_table(dims, slot, 1, parity)
            assert np.array_equal(out, ref[parity*Vh:(parity+1)*Vh]), (parity, slot)


@pytest.mark.parametrize("prec", ["D", "F"])
@pytest.mark.parametrize("sub", ["all", "even", "odd"])
def test_dslash2_matches_oracle(prec, sub):
    L = qll.load()
    lay = qll.setup_layout(DIMS, prec)
    u, u3 = _links(prec)
    S = qll.D if prec == "D" else qll.F
    sl = S["StaggeredLinks"]()
    getattr(L, "createStaggeredLinks" + prec)(byref(sl), byref(lay), qll.ptr_array(u, CT[prec]),
                                              qll.ptr_array(u3, CT[prec]), sub.encode())
    assert sl.t, qll.last_error()
    y = qll.gen_source(DIMS, 31, 6, "all").astype(DT[prec])
    x = np.full_like(y, 7.0)
    getattr(L, "dslash2" + prec)(byref(sl), qll.ptr(x), CT[prec](0.25), qll.ptr(y))
    assert not qll.last_error(), qll.last_error()
    ref = orc.dslash(DIMS, u, u3, 0.25, y, sub)
    Vh = x.shape[0]//2
    rng = {"all": slice(0, 2*Vh), "even": slice(0, Vh), "odd": slice(Vh, 2*Vh)}[sub]
    assert relerr(x[rng], ref[rng]) < TOL[prec]
    # sites outside the subset are not written
    if sub != "all":
        other = slice(Vh, 2*Vh) if sub == "even" else slice(0, Vh)
        assert np.all(x[other] == 7.0)
    getattr(L, "freeStaggeredLinks" + prec)(byref(sl))


def _make_solver(prec, dims=DIMS):
    L = qll.load()
    lay = qll.setup_layout(dims, prec)
    u, u3 = _links(prec, dims)
    S = qll.D if prec == "D" else qll.F
    ss = S["StaggeredSolver"]()
    getattr(L, "createStaggeredSolver" + prec)(byref(ss), byref(lay), qll.ptr_array(u, CT[prec]),
                                               qll.ptr_array(u3, CT[prec]), b"even")
    assert ss.sle.t, qll.last_error()
    return L, lay, ss, u, u3


@pytest.mark.parametrize("prec", ["D", "F"])
def test_solve2_matches_oracle(prec):
    L, lay, ss, u, u3 = _make_solver(prec)
    b = qll.gen_source(DIMS, 2001, 6, "even").astype(DT[prec])
    rsq = 1e-16 if prec == "D" else 1e-10
    x = np.zeros_like(b)
    its = getattr(L, "solve2" + prec)(byref(ss), qll.ptr(x), CT[prec](0.1), qll.ptr(b), rsq,
                                      2000, b"even")
    assert its > 0, qll.last_error()
    assert ss.its == its
    its_o, xo, _ = orc.solve2(DIMS, u, u3, 0.1, b, rsq, 2000)
    Vh = b.shape[0]//2
    if prec == "D":
        assert abs(its - its_o) <= 1
        assert relerr(x[:Vh], xo[:Vh]) < 10*np.sqrt(rsq)
    else:
        assert abs(its - its_o) <= 3
        assert relerr(x[:Vh], xo[:Vh]) < 1e-4
    assert np.all(x[Vh:] == 0)
    getattr(L, "freeStaggeredSolver" + prec)(byref(ss))


def test_solve2_mixed_switch():
    """solve2_mixed 1: the drop-in solve2D runs the FP32 mixed solver; the
    solution reaches the same tolerance as the oracle's FP64 CG, with the
    reference's mass scaling"""
    L, lay, ss, u, u3 = _make_solver("D")
    L.qllg_set_param.argtypes = [ctypes.c_char_p, c_double]
    b = qll.gen_source(DIMS, 2003, 6, "even")
    x = np.zeros_like(b)
    L.qllg_set_param(b"solve2_mixed", 1)
    its = L.solve2D(byref(ss), qll.ptr(x), c_double(0.1), qll.ptr(b), 1e-16, 2000, b"even")
    L.qllg_set_param(b"solve2_mixed", 0)
    assert its > 0, qll.last_error()
    its_o, xo, _ = orc.solve2(DIMS, u, u3, 0.1, b, 1e-16, 2000)
    Vh = b.shape[0]//2
    # both are within the tolerance of the exact solution: |x - x*| <= cond |r|/|b|
    assert relerr(x[:Vh], xo[:Vh]) < 1e-5
    assert np.all(x[Vh:] == 0)
    L.freeStaggeredSolverD(byref(ss))


def test_solve2_noscale_and_mass_zero_scaling():
    L, lay, ss, u, u3 = _make_solver("D")
    b = qll.gen_source(DIMS, 2002, 6, "even")
    x1 = np.zeros_like(b)
    ss.noscale = 1
    L.solve2D(byref(ss), qll.ptr(x1), 0.2, qll.ptr(b), 1e-18, 2000, b"even")
    ss.noscale = 0
    x2 = np.zeros_like(b)
    L.solve2D(byref(ss), qll.ptr(x2), 0.2, qll.ptr(b), 1e-18, 2000, b"even")
    Vh = b.shape[0]//2
    assert relerr(x2[:Vh], 0.2*x1[:Vh]) < 1e-14
    L.freeStaggeredSolverD(byref(ss))


def _native(dims=DIMS):
    L = qll.load()
    u, u3 = asqtad_links(dims)
    S = L.qllg_stag_create(qll.dims_c(dims), qll.vp_array(u), qll.vp_array(u3))
    assert S, qll.last_error()
    return L, S, u, u3


@pytest.mark.parametrize("nrhs", [1, 3, 4, 16])
def test_multi_rhs_double_matches_single(nrhs):
    L, S, u, u3 = _native()
    masses = [0.1 + 0.05*k for k in range(nrhs)]
    bs = [qll.gen_source(DIMS, 3000 + k, 6, "even") for k in range(nrhs)]
    xs = [np.zeros_like(bs[0]) for _ in range(nrhs)]
    info = qll.SolveInfo()
    its = L.qllg_stag_solve(S, nrhs, qll.vp_array(xs), qll.vp_array(bs),
                            (c_double*nrhs)(*masses), 1e-16, 3000, qll.SOLVE_DOUBLE, byref(info))
    assert its > 0, qll.last_error()
    Vh = bs[0].shape[0]//2
    for k in range(nrhs):
        its_o, xo, _ = orc.solve2(DIMS, u, u3, masses[k], bs[k], 1e-16, 3000, noscale=1)
        assert abs(info.iters[k] - its_o) <= 1
        assert relerr(xs[k][:Vh], xo[:Vh]) < 1e-7
        assert info.true_rsq[k] < 1e-15
    L.qllg_stag_destroy(S)


@pytest.mark.parametrize("mode", [qll.SOLVE_MIXED_HALF, qll.SOLVE_MIXED_SINGLE])
@pytest.mark.parametrize("nrhs", [1, 8])
def test_mixed_precision_reaches_fp64_residual(mode, nrhs):
    L, S, u, u3 = _native()
    masses = [0.05 + 0.01*k for k in range(nrhs)]
    bs = [qll.gen_source(DIMS, 4000 + k, 6, "even") for k in range(nrhs)]
    xs = [np.zeros_like(bs[0]) for _ in range(nrhs)]
    info = qll.SolveInfo()
    its = L.qllg_stag_solve(S, nrhs, qll.vp_array(xs), qll.vp_array(bs),
                            (c_double*nrhs)(*masses), 1e-16, 5000, mode, byref(info))
    assert its > 0, qll.last_error()
    assert info.reliable_updates > 0
    Vh = bs[0].shape[0]//2
    for k in range(nrhs):
        # true residual of the FP64 operator, recomputed in FP64
        assert info.true_rsq[k] < 1e-16*1.0001, (k, info.true_rsq[k])
        its_o, xo, _ = orc.solve2(DIMS, u, u3, masses[k], bs[k], 1e-16, 5000, noscale=1)
        assert relerr(xs[k][:Vh], xo[:Vh]) < 1e-7
    L.qllg_stag_destroy(S)


@pytest.mark.parametrize("mode", [qll.SOLVE_DOUBLE, qll.SOLVE_MIXED_SINGLE])
def test_graph_loop_matches_host_loop(mode):
    """the CUDA-graph solver loop (conditional WHILE node) and the
    host-polled loop launch the same kernels: identical iterations and
    bitwise identical solutions"""
    L, S, u, u3 = _native()
    L.qllg_set_param.argtypes = [ctypes.c_char_p, ctypes.c_double]
    nrhs = 4
    masses = (c_double*nrhs)(0.05, 0.07, 0.1, 0.2)
    bs = [qll.gen_source(DIMS, 5000 + k, 6, "even") for k in range(nrhs)]
    out = {}
    for graph in (1, 0):
        L.qllg_set_param(b"graph", graph)
        xs = [np.zeros_like(bs[0]) for _ in range(nrhs)]
        info = qll.SolveInfo()
        its = L.qllg_stag_solve(S, nrhs, qll.vp_array(xs), qll.vp_array(bs), masses, 1e-16, 5000,
                                mode, byref(info))
        assert its > 0, qll.last_error()
        out[graph] = (list(info.iters[:nrhs]), xs)
    L.qllg_set_param(b"graph", 1)
    assert out[0][0] == out[1][0]
    for k in range(nrhs):
        assert np.array_equal(out[0][1][k], out[1][1][k])
    L.qllg_stag_destroy(S)


@pytest.mark.parametrize("mode", [qll.SOLVE_MIXED_SINGLE, qll.SOLVE_MIXED_HALF])
def test_compact_reliable_update_matches_masked(mode):
    """the reliable update over the flagged rhs only (threads compacted onto
    them) and the masked multi-rhs launch compute the same FP64 residuals:
    identical iterations and bitwise identical solutions (every update in
    FP64: ru_df 0)"""
    L, S, u, u3 = _native()
    L.qllg_set_param.argtypes = [ctypes.c_char_p, ctypes.c_double]
    L.qllg_set_param(b"ru_df", 0)
    nrhs = 8
    masses = (c_double*nrhs)(*[0.05 + 0.02*k for k in range(nrhs)])
    bs = [qll.gen_source(DIMS, 5100 + k, 6, "even") for k in range(nrhs)]
    out = {}
    for compact in (1, 0):
        L.qllg_set_param(b"ru_compact", compact)
        xs = [np.zeros_like(bs[0]) for _ in range(nrhs)]
        info = qll.SolveInfo()
        its = L.qllg_stag_solve(S, nrhs, qll.vp_array(xs), qll.vp_array(bs), masses, 1e-16, 5000,
                                mode, byref(info))
        assert its > 0, qll.last_error()
        assert info.reliable_updates > 0
        out[compact] = (list(info.iters[:nrhs]), xs)
    L.qllg_set_param(b"ru_compact", 1)
    L.qllg_set_param(b"ru_df", 1)
    assert out[0][0] == out[1][0]
    for k in range(nrhs):
        assert np.array_equal(out[0][1][k], out[1][1][k])
    L.qllg_stag_destroy(S)


@pytest.mark.parametrize("nrhs", [4, 16])
def test_vectorised_dslash_matches_per_rhs_loads(nrhs):
    """FP32 multi-rhs Dslash with 16-byte spinor access, with per-rhs
    access (parameter off), and on buffers offset by 8 bytes (the launcher
    then falls back to per-rhs access): bitwise identical outputs"""
    torch = pytest.importorskip("torch")
    L, S, u, u3 = _native()
    L.qllg_set_param.argtypes = [ctypes.c_char_p, ctypes.c_double]
    L.qllg_stag_vec_bytes.restype = ctypes.c_size_t
    L.qllg_stag_vec_bytes.argtypes = [ctypes.c_void_p, c_int, c_int]
    L.qllg_stag_dslash_device.argtypes = [ctypes.c_void_p, c_int, c_int, c_int,
                                          ctypes.c_void_p, ctypes.c_void_p]
    n = L.qllg_stag_vec_bytes(S, 1, nrhs)//4
    g = torch.Generator(device="cuda").manual_seed(77 + nrhs)
    src = torch.randn(n + 2, dtype=torch.float32, device="cuda", generator=g)
    outs = []
    for vec4, off in ((1, 0), (0, 0), (1, 2)):
        L.qllg_set_param(b"dslash_vec4", vec4)
        dst = torch.zeros(n + 2, dtype=torch.float32, device="cuda")
        if off:
            src[off:].copy_(src[:n].clone())
        torch.cuda.synchronize()
        for parity in (0, 1):
            rc = L.qllg_stag_dslash_device(S, 1, nrhs, parity,
                                           ctypes.c_void_p(dst[off:].data_ptr() + 0),
                                           ctypes.c_void_p(src[off:].data_ptr()))
            assert rc == 0, qll.last_error()
            torch.cuda.synchronize()
            outs.append(dst[off:off + n].clone())
    L.qllg_set_param(b"dslash_vec4", 1)
    assert torch.equal(outs[0], outs[2]) and torch.equal(outs[1], outs[3])
    assert torch.equal(outs[0], outs[4]) and torch.equal(outs[1], outs[5])
    L.qllg_stag_destroy(S)


@pytest.mark.parametrize("mode", [qll.SOLVE_DOUBLE, qll.SOLVE_MIXED_SINGLE])
def test_multishift_multi_rhs_matches_oracle(mode):
    """every (rhs, shift) pair reaches the FP64 true residual and agrees
    with the oracle's solveMulti2 (FP64 multishift CG) within 10x the
    tolerance; 4 rhs x 5 shifts = 20 pairs, two batches in the mixed mode"""
    L, S, u, u3 = _native()
    L.qllg_stag_solve_multishift.argtypes = [ctypes.c_void_p, c_int, ctypes.c_void_p,
                                             ctypes.c_void_p, c_double, c_int, ctypes.c_void_p,
                                             c_double, c_int, c_int, ctypes.c_void_p,
                                             ctypes.c_void_p]
    nrhs, mass = 4, 0.05
    shifts = [1e-2, 1e-4, 1.0, 1e-3, 0.1]       # unsorted, none zero
    ns = len(shifts)
    bs = [qll.gen_source(DIMS, 6100 + r, 6, "even") for r in range(nrhs)]
    xs = [np.zeros_like(bs[0]) for _ in range(nrhs*ns)]
    its = (c_int*(nrhs*ns))()
    tr = (c_double*(nrhs*ns))()
    rc = L.qllg_stag_solve_multishift(S, nrhs, qll.vp_array(xs), qll.vp_array(bs), mass, ns,
                                      (c_double*ns)(*shifts), 1e-16, 5000, mode, its, tr)
    assert rc > 0, qll.last_error()
    Vh = bs[0].shape[0]//2
    srt = sorted(range(ns), key=lambda k: shifts[k])   # the oracle's base is its first mass
    for r in range(nrhs):
        its_o, xo = orc.solve_multi2(DIMS, u, u3, [np.sqrt(mass**2 + shifts[k]) for k in srt],
                                     bs[r], 1e-16, 5000, noscale=1)
        for j, k in enumerate(srt):
            assert tr[r*ns + k] < (1e-16*1.0001 if mode == qll.SOLVE_MIXED_SINGLE else 1e-15), \
                (r, k, tr[r*ns + k])
            assert relerr(xs[r*ns + k][:Vh], xo[j][:Vh]) < 1e-7, (r, k)
            assert np.all(xs[r*ns + k][Vh:] == 0)
    L.qllg_stag_destroy(S)


@pytest.mark.parametrize("nrhs", [4, 16])
def test_dslash_variants_agree(nrhs):
    """the autotuner's candidates (4, 2, 1 rhs per thread, shared-memory
    staging, the other launch shapes of the 4-rhs kernel, the bulk-copy
    pipeline) compute bitwise the same FP32 Dslash"""
    torch = pytest.importorskip("torch")
    L, S, u, u3 = _native()
    L.qllg_set_param.argtypes = [ctypes.c_char_p, ctypes.c_double]
    L.qllg_stag_vec_bytes.restype = ctypes.c_size_t
    L.qllg_stag_vec_bytes.argtypes = [ctypes.c_void_p, c_int, c_int]
    L.qllg_stag_dslash_device.argtypes = [ctypes.c_void_p, c_int, c_int, c_int,
                                          ctypes.c_void_p, ctypes.c_void_p]
    n = L.qllg_stag_vec_bytes(S, 1, nrhs)//4
    g = torch.Generator(device="cuda").manual_seed(91 + nrhs)
    src = torch.randn(n, dtype=torch.float32, device="cuda", generator=g)
    outs = []
    for v in range(24):
        L.qllg_set_param(b"dslash_variant", v)
        for parity in (0, 1):
            dst = torch.full_like(src, float("nan"))
            torch.cuda.synchronize()
            assert L.qllg_stag_dslash_device(S, 1, nrhs, parity, ctypes.c_void_p(dst.data_ptr()),
                                             ctypes.c_void_p(src.data_ptr())) == 0, qll.last_error()
            torch.cuda.synchronize()
            outs.append(dst)
    L.qllg_set_param(b"dslash_variant", -1)
    for k in range(2, len(outs)):
        assert torch.equal(outs[k], outs[k % 2]), k
    # no bounded wait of the bulk-copy pipeline ran out
    assert L.qllg_k_bulk_error(1) == 0
    L.qllg_stag_destroy(S)


def test_warp_pipeline_over_several_passes():
    """the per-warp cp.async pipelines (variants 17-19) and tensor-copy
    pipelines (20-23) on a lattice where every warp takes several groups
    of sites, so that its ring prefetches across the group boundary:
    bitwise the register kernel's Dslash, and a 16-rhs mixed solve (fused
    CG epilogue, norms, rhs dropping out as they converge) to the same FP64
    true residual in the same iterations"""
    torch = pytest.importorskip("torch")
    from ctypes import POINTER, c_void_p
    dims = (16, 16, 16, 32)
    L = qll.load()
    L.qllg_stag_create_asqtad.restype = c_void_p
    L.qllg_stag_create_asqtad.argtypes = [POINTER(c_int), POINTER(c_void_p), POINTER(qll.Fat7Coeffs)]
    L.qllg_set_param.argtypes = [ctypes.c_char_p, ctypes.c_double]
    L.qllg_stag_vec_bytes.restype = ctypes.c_size_t
    L.qllg_stag_vec_bytes.argtypes = [ctypes.c_void_p, c_int, c_int]
    L.qllg_stag_dslash_device.argtypes = [ctypes.c_void_p, c_int, c_int, c_int,
                                          ctypes.c_void_p, ctypes.c_void_p]
    thin = qll.gen_gauge(dims, 1005, 0.3, ks=True)
    S = c_void_p(L.qllg_stag_create_asqtad(qll.dims_c(dims), qll.vp_array(thin),
                                           byref(qll.asqtad_coeffs())))
    assert S.value, qll.last_error()
    n = L.qllg_stag_vec_bytes(S, 1, 16)//4
    g = torch.Generator(device="cuda").manual_seed(77)
    src = torch.randn(n, dtype=torch.float32, device="cuda", generator=g)
    want = {}
    for v in (10, 17, 18, 19, 20, 21, 22, 23):
        L.qllg_set_param(b"dslash_variant", v)
        for parity in (0, 1):
            dst = torch.full_like(src, float("nan"))
            torch.cuda.synchronize()
            assert L.qllg_stag_dslash_device(S, 1, 16, parity, ctypes.c_void_p(dst.data_ptr()),
                                             ctypes.c_void_p(src.data_ptr())) == 0, qll.last_error()
            torch.cuda.synchronize()
            if parity not in want:
                want[parity] = dst
            assert torch.equal(dst, want[parity]), (v, parity)
    nrhs = 16
    masses = [0.02 + 0.01*k for k in range(nrhs)]
    bs = [qll.gen_source(dims, 8100 + k, 6, "even") for k in range(nrhs)]
    iters = {}
    for v in (10, 19, 20, 22):
        L.qllg_set_param(b"dslash_variant", v)
        xs = [np.zeros_like(bs[0]) for _ in range(nrhs)]
        info = qll.SolveInfo()
        its = L.qllg_stag_solve(S, nrhs, qll.vp_array(xs), qll.vp_array(bs), (c_double*nrhs)(*masses),
                                1e-16, 5000, qll.SOLVE_MIXED_SINGLE, byref(info))
        assert its > 0, qll.last_error()
        assert max(info.true_rsq[k] for k in range(nrhs)) < 1e-16*1.0001, v
        iters[v] = [info.iters[k] for k in range(nrhs)]
    L.qllg_set_param(b"dslash_variant", -1)
    # the per-rhs sums are folded in a different order: iterations within 2
    for v in (19, 20, 22):
        assert all(abs(a - b) <= 2 for a, b in zip(iters[10], iters[v])), iters
    assert L.qllg_k_bulk_error(1) == 0
    L.qllg_stag_destroy(S)


@pytest.mark.parametrize("variant", range(24))
def test_mixed_solve_with_each_dslash_variant(variant):
    """the fused CG epilogue and the norms of every variant: the 16-rhs
    mixed solve reaches the FP64 true residual and matches the oracle"""
    L, S, u, u3 = _native()
    L.qllg_set_param.argtypes = [ctypes.c_char_p, ctypes.c_double]
    L.qllg_set_param(b"dslash_variant", variant)
    nrhs = 16
    masses = [0.05 + 0.01*k for k in range(nrhs)]
    bs = [qll.gen_source(DIMS, 8000 + k, 6, "even") for k in range(nrhs)]
    xs = [np.zeros_like(bs[0]) for _ in range(nrhs)]
    info = qll.SolveInfo()
    its = L.qllg_stag_solve(S, nrhs, qll.vp_array(xs), qll.vp_array(bs), (c_double*nrhs)(*masses),
                            1e-16, 5000, qll.SOLVE_MIXED_SINGLE, byref(info))
    L.qllg_set_param(b"dslash_variant", -1)
    assert its > 0, qll.last_error()
    Vh = bs[0].shape[0]//2
    for k in (0, 7, 15):
        assert info.true_rsq[k] < 1e-16*1.0001
        its_o, xo, _ = orc.solve2(DIMS, u, u3, masses[k], bs[k], 1e-16, 5000, noscale=1)
        assert relerr(xs[k][:Vh], xo[:Vh]) < 1e-7
    L.qllg_stag_destroy(S)


def test_foreign_layout_adapters():
    """links and vectors in an embedding code's layout (a shuffled site
    order, row-major matrices) reordered on the GPU give bitwise the
    operator and the solution of the reference-ordered arrays"""
    L, S, u, u3 = _native()
    vp = ctypes.c_void_p
    L.qllg_stag_create_foreign.restype = vp
    L.qllg_stag_create_foreign.argtypes = [ctypes.POINTER(c_int), ctypes.POINTER(vp),
                                           ctypes.POINTER(vp), ctypes.POINTER(c_int), c_int]
    for fn in ("qllg_stag_vec_upload_foreign", "qllg_stag_vec_download_foreign"):
        getattr(L, fn).argtypes = [vp, vp, c_int, ctypes.POINTER(vp), ctypes.POINTER(c_int)]
    V = int(np.prod(DIMS))
    rng = np.random.default_rng(12)
    perm = rng.permutation(V).astype(np.int32)          # foreign site s is QLL site perm[s]

    def foreign(a, n):
        f = np.empty_like(a)
        f[np.arange(V)] = a[perm]
        if n == 18:                                       # column-major -> row-major
            f = f.reshape(V, 3, 3, 2).transpose(0, 2, 1, 3).reshape(V, 18)
        return np.ascontiguousarray(f)

    fu = [foreign(a, 18) for a in u]
    fu3 = [foreign(a, 18) for a in u3]
    pp = perm.ctypes.data_as(ctypes.POINTER(c_int))
    F = vp(L.qllg_stag_create_foreign(qll.dims_c(DIMS), qll.vp_array(fu), qll.vp_array(fu3), pp, 1))
    assert F.value, qll.last_error()
    nrhs = 4
    masses = (c_double*nrhs)(0.05, 0.1, 0.2, 0.5)
    bs = [qll.gen_source(DIMS, 9100 + k, 6, "even") for k in range(nrhs)]
    # reference-ordered solve on the reference-ordered operator
    xs = [np.zeros_like(bs[0]) for _ in range(nrhs)]
    info = qll.SolveInfo()
    assert L.qllg_stag_solve(S, nrhs, qll.vp_array(xs), qll.vp_array(bs), masses, 1e-16, 5000,
                             qll.SOLVE_DOUBLE, byref(info)) > 0, qll.last_error()
    # foreign-ordered arrays through the adapters
    fb = [foreign(b, 6) for b in bs]
    bd, xd = vp(L.qllg_stag_vec_alloc(F, nrhs)), vp(L.qllg_stag_vec_alloc(F, nrhs))
    assert L.qllg_stag_vec_upload_foreign(F, bd, nrhs, qll.vp_array(fb), pp) == 0, qll.last_error()
    info2 = qll.SolveInfo()
    assert L.qllg_stag_solve_device(F, nrhs, xd, bd, masses, 1e-16, 5000, qll.SOLVE_DOUBLE,
                                    byref(info2)) > 0, qll.last_error()
    fx = [np.full_like(bs[0], np.nan) for _ in range(nrhs)]
    assert L.qllg_stag_vec_download_foreign(F, xd, nrhs, qll.vp_array(fx), pp) == 0
    assert list(info.iters[:nrhs]) == list(info2.iters[:nrhs])
    Vh = V//2
    for k in range(nrhs):
        back = np.empty_like(fx[k])
        back[perm] = fx[k]                                # to the reference order
        assert np.array_equal(back[:Vh], xs[k][:Vh]), k
        assert np.all(back[Vh:] == 0)
    L.qllg_stag_vec_free(bd)
    L.qllg_stag_vec_free(xd)
    L.qllg_stag_destroy(F)
    L.qllg_stag_destroy(S)


@pytest.mark.parametrize("single_store", [0, 1])
def test_reconstruct12_links(single_store):
    """Naik links held as two rows + a sign (the long links of fat7 are
    -1/24 times products of SU(3) links): the Dslash agrees with FP64 to FP32
    rounding, and the mixed solve reaches the same FP64 true residual and
    solution as with 18-real links"""
    torch = pytest.importorskip("torch")
    L = qll.load()
    vp = ctypes.c_void_p
    fn = L.qllg_stag_create_asqtad_fb if single_store else L.qllg_stag_create_asqtad
    fn.restype = vp
    fn.argtypes = [ctypes.POINTER(c_int), ctypes.POINTER(vp), ctypes.POINTER(qll.Fat7Coeffs)]
    L.qllg_set_param.argtypes = [ctypes.c_char_p, c_double]
    L.qllg_stag_recon12.argtypes = [vp]
    L.qllg_stag_vec_bytes.restype = ctypes.c_size_t
    L.qllg_stag_vec_bytes.argtypes = [vp, c_int, c_int]
    L.qllg_stag_dslash_device.argtypes = [vp, c_int, c_int, c_int, vp, vp]
    th = qll.gen_gauge(DIMS, 1009, 0.3, ks=True)
    c = qll.asqtad_coeffs()
    S = vp(fn(qll.dims_c(DIMS), qll.vp_array(th), byref(c)))
    assert S.value, qll.last_error()
    L.qllg_set_param(b"links_recon12", 1)
    assert L.qllg_stag_recon12(S) == 1, qll.last_error()
    for nrhs in (1, 16):
        n = L.qllg_stag_vec_bytes(S, 1, nrhs)//4
        g = torch.Generator(device="cuda").manual_seed(31 + nrhs)
        src = torch.randn(n, dtype=torch.float32, device="cuda", generator=g)
        src64 = src.to(torch.float64)
        for parity in (0, 1):
            outs = {}
            for prec, inp in ((0, src64), (1, src), (3, src)):
                o = torch.zeros_like(inp)
                torch.cuda.synchronize()
                assert L.qllg_stag_dslash_device(S, prec, nrhs, parity, vp(o.data_ptr()),
                                                 vp(inp.data_ptr())) == 0, qll.last_error()
                torch.cuda.synchronize()
                outs[prec] = o.to(torch.float64)
            ref = outs[0]
            for prec in (1, 3):
                err = ((outs[prec] - ref).norm()/ref.norm()).item()
                assert err < 2e-6, (prec, nrhs, parity, err)
    nrhs = 4
    masses = (c_double*nrhs)(0.05, 0.07, 0.1, 0.2)
    bs = [qll.gen_source(DIMS, 9700 + k, 6, "even") for k in range(nrhs)]
    sol = {}
    for recon in (1, 0):
        L.qllg_set_param(b"links_recon12", recon)
        xs = [np.zeros_like(bs[0]) for _ in range(nrhs)]
        info = qll.SolveInfo()
        assert L.qllg_stag_solve(S, nrhs, qll.vp_array(xs), qll.vp_array(bs), masses, 1e-16, 5000,
                                 qll.SOLVE_MIXED_SINGLE, byref(info)) > 0, qll.last_error()
        for k in range(nrhs):
            assert info.true_rsq[k] < 1e-16*1.0001
        sol[recon] = xs
    L.qllg_set_param(b"links_recon12", 0)
    Vh = bs[0].shape[0]//2
    for k in range(nrhs):
        assert relerr(sol[1][k][:Vh], sol[0][k][:Vh]) < 1e-7
    L.qllg_stag_destroy(S)


def test_reconstruct12_refused_for_general_links():
    """Naik links that are not real multiples of SU(3) matrices: no
    reconstruct-12 copy, the mixed FP32 solve falls back to 18-real links"""
    L, S, u, u3 = _native()
    L.qllg_stag_destroy(S)
    rng = np.random.default_rng(4)
    u3b = [a + 1e-3*rng.standard_normal(a.shape) for a in u3]
    S = ctypes.c_void_p(L.qllg_stag_create(qll.dims_c(DIMS), qll.vp_array(u), qll.vp_array(u3b)))
    assert S.value, qll.last_error()
    L.qllg_stag_recon12.argtypes = [ctypes.c_void_p]
    L.qllg_set_param.argtypes = [ctypes.c_char_p, c_double]
    L.qllg_set_param(b"links_recon12", 1)
    assert L.qllg_stag_recon12(S) == 0
    nrhs = 2
    bs = [qll.gen_source(DIMS, 9800 + k, 6, "even") for k in range(nrhs)]
    xs = [np.zeros_like(bs[0]) for _ in range(nrhs)]
    info = qll.SolveInfo()
    assert L.qllg_stag_solve(S, nrhs, qll.vp_array(xs), qll.vp_array(bs), (c_double*nrhs)(0.1, 0.2),
                             1e-16, 5000, qll.SOLVE_MIXED_SINGLE, byref(info)) > 0, qll.last_error()
    L.qllg_set_param(b"links_recon12", 0)
    assert max(info.true_rsq[k] for k in range(nrhs)) < 1e-16*1.0001
    L.qllg_stag_destroy(S)


def test_unknown_parameter_is_refused():
    L = qll.load()
    L.qllg_set_param.argtypes = [ctypes.c_char_p, ctypes.c_double]
    assert L.qllg_set_param(b"no_such_knob", 1.0) == -1
    assert "no_such_knob" in qll.last_error()
