"""GPU parity, through the C ABI, of the rest of the hot path: multishift
CG, fat7 smearing, plaquette, double-stored links, the single-stored (Fb)
link variant, cgSolve/cgmsSolve with the library's Linop, fields, shift
and transporter (with the reference's stress.c and fieldtest.c known
answers), and the Wilson operator and solvers."""
import ctypes
from ctypes import byref, c_double, c_float, c_int

import numpy as np
import pytest

import oracle_lib as orc
from inputs import as_dtype, asqtad_links, relerr, wilson_links
from qll_gb300 import qll

pytestmark = pytest.mark.gpu

DIMS = (4, 4, 6, 8)
DT = {"D": np.float64, "F": np.float32}
CT = {"D": c_double, "F": c_float}
TOL = {"D": 1e-12, "F": 1e-5}


def _solver(prec, dims=DIMS):
    L = qll.load()
    lay = qll.setup_layout(dims, prec)
    u, u3 = asqtad_links(dims)
    u, u3 = as_dtype(u, DT[prec]), as_dtype(u3, DT[prec])
    S = qll.D if prec == "D" else qll.F
    ss = S["StaggeredSolver"]()
    getattr(L, "createStaggeredSolver" + prec)(byref(ss), byref(lay), qll.ptr_array(u, CT[prec]),
                                               qll.ptr_array(u3, CT[prec]), b"even")
    assert ss.sle.t, qll.last_error()
    return L, lay, ss, u, u3


def _ptrs(arrs, prec):
    return qll.ptr_array(arrs, CT[prec])


@pytest.mark.parametrize("prec", ["D", "F"])
def test_solve_multi2_matches_oracle(prec):
    L, lay, ss, u, u3 = _solver(prec)
    fn = getattr(L, "solveMulti2" + prec)
    fn.restype = c_int
    masses = [0.1, 0.14, 0.196, 0.2744, 0.38416]
    b = qll.gen_source(DIMS, 77, 6, "even").astype(DT[prec])
    xs = [np.zeros_like(b) for _ in masses]
    rsq = 1e-14 if prec == "D" else 1e-8
    its = fn(byref(ss), _ptrs(xs, prec), (c_double*5)(*masses), 5, qll.ptr(b), c_double(rsq),
             c_int(3000), b"even")
    assert its > 0, qll.last_error()
    its_o, xo = orc.solve_multi2(DIMS, u, u3, masses, b, rsq, 3000)
    Vh = b.shape[0]//2
    assert abs(its - its_o) <= (1 if prec == "D" else 3)
    for k in range(5):
        assert relerr(xs[k][:Vh], xo[k][:Vh]) < (1e-6 if prec == "D" else 1e-3), k
    getattr(L, "freeStaggeredSolver" + prec)(byref(ss))


def test_cgsolve_and_cgmssolve_with_library_linop():
    L, lay, ss, u, u3 = _solver("D")
    L.cgSolveD.restype = c_int
    L.cgmsSolveD.restype = c_int
    b = qll.gen_source(DIMS, 78, 6, "even")
    x = np.zeros_like(b)
    ss.mass = 0.12
    lin = ctypes.cast(L.stagLinopD, ctypes.c_void_p)
    its = L.cgSolveD(byref(ss.cgls), qll.ptr(x), qll.ptr(b), lin, ctypes.cast(byref(ss), ctypes.c_void_p),
                     None, None, c_double(1e-16), c_int(2000))
    assert its > 0, qll.last_error()
    its_o, xo, _ = orc.solve2(DIMS, u, u3, 0.12, b, 1e-16, 2000, noscale=1)
    Vh = b.shape[0]//2
    assert abs(its - its_o) <= 1
    assert relerr(x[:Vh], xo[:Vh]) < 1e-7
    # an operator that is not the library's is refused, with a message
    bad = ctypes.cast(L.dslash2D, ctypes.c_void_p)
    assert L.cgSolveD(byref(ss.cgls), qll.ptr(x), qll.ptr(b), bad, None, None, None,
                      c_double(1e-10), c_int(10)) == -1
    assert "stagLinop" in qll.last_error()
    L.freeStaggeredSolverD(byref(ss))


@pytest.mark.parametrize("prec", ["D", "F"])
def test_fat7_plaquette_doublestore(prec):
    L = qll.load()
    lay = qll.setup_layout(DIMS, prec)
    th = [a.astype(DT[prec]) for a in qll.gen_gauge(DIMS, 1001, 0.3, ks=True)]
    F = (qll.D if prec == "D" else qll.F)["Field"]
    V = th[0].shape[0]

    def fields(arrs):
        fs = [F() for _ in arrs]
        for f, a in zip(fs, arrs):
            f.l = ctypes.pointer(lay)
            f.f = qll.ptr(a)
            f.nelem = 18
        arr = (ctypes.POINTER(F)*len(fs))(*[ctypes.pointer(f) for f in fs])
        return fs, arr

    fl = [np.zeros((V, 18), DT[prec]) for _ in range(4)]
    ll = [np.zeros((V, 18), DT[prec]) for _ in range(4)]
    fk, fa = fields(fl)
    lk, la = fields(ll)
    uk, ua = fields(th)
    c = qll.asqtad_coeffs()
    getattr(L, "smearFat7" + prec)(fa, la, byref(c), ua, ua)
    assert not qll.last_error(), qll.last_error()
    flo, llo = orc.smear_fat7(DIMS, th, c)
    for mu in range(4):
        assert relerr(fl[mu], flo[mu]) < TOL[prec]
        assert relerr(ll[mu], llo[mu]) < TOL[prec]
    plaq = (c_double*6)()
    getattr(L, "gaugePlaq" + prec)(plaq, ua)
    po = orc.plaq(DIMS, th)
    assert np.allclose(plaq[:], po, rtol=0, atol=(1e-13 if prec == "D" else 1e-6))
    out = [np.zeros((V, 18), DT[prec]) for _ in range(4)]
    ok, oa = fields(out)
    getattr(L, "gaugeDoublestore" + prec)(oa, ua, (c_int*4)(0, 1, 2, 3), (c_int*4)(-1, 1, -1, 1), 4)
    for mu, ln in zip(range(4), (-1, 1, -1, 1)):
        assert np.array_equal(out[mu], orc.doublestore(DIMS, th[mu], mu, ln))


def test_stag_create_asqtad_matches_host_links():
    """thin links -> GPU fat7 -> resident operator equals the operator built
    from oracle-smeared host links"""
    L = qll.load()
    L.qllg_stag_create_asqtad.restype = ctypes.c_void_p
    L.qllg_stag_create_asqtad.argtypes = [ctypes.POINTER(c_int), ctypes.POINTER(ctypes.c_void_p),
                                          ctypes.POINTER(qll.Fat7Coeffs)]
    th = qll.gen_gauge(DIMS, 1001, 0.3, ks=True)
    c = qll.asqtad_coeffs()
    S = L.qllg_stag_create_asqtad(qll.dims_c(DIMS), qll.vp_array(th), byref(c))
    assert S, qll.last_error()
    u, u3 = asqtad_links(DIMS, 1001, 0.3)
    y = qll.gen_source(DIMS, 5, 6, "all")
    x = np.zeros_like(y)
    assert L.qllg_stag_dslash(S, x.ctypes.data, 0.2, y.ctypes.data, b"all") == 0
    assert relerr(x, orc.dslash(DIMS, u, u3, 0.2, y, "all")) < 1e-12
    L.qllg_stag_destroy(S)


@pytest.mark.parametrize("sub", ["all", "even"])
def test_fb_links_match_oracle(sub):
    L = qll.load()
    lay = qll.setup_layout(DIMS)
    u, u3 = asqtad_links(DIMS)
    fwd = [u[i] if i % 2 == 0 else np.full_like(u[i], np.nan) for i in range(8)]
    fwd3 = [u3[i] if i % 2 == 0 else np.full_like(u3[i], np.nan) for i in range(8)]
    sl = qll.D["StaggeredLinks"]()
    L.createStaggeredLinksFbD(byref(sl), byref(lay), _ptrs(fwd, "D"), _ptrs(fwd3, "D"), sub.encode())
    assert sl.t and sl.fb == 1, qll.last_error()
    y = qll.gen_source(DIMS, 9, 6, "all")
    x = np.zeros_like(y)
    L.dslash2D(byref(sl), qll.ptr(x), 0.3, qll.ptr(y))
    ref = orc.dslash(DIMS, u, u3, 0.3, y, sub)
    rng = slice(0, x.shape[0]) if sub == "all" else slice(0, x.shape[0]//2)
    assert relerr(x[rng], ref[rng]) < 1e-12
    L.freeStaggeredLinksD(byref(sl))


def test_fields_shift_transport_and_reference_kats():
    L = qll.load()
    dims = (4, 4, 6, 4)
    lay = qll.setup_layout(dims)
    V = int(np.prod(dims))
    F = qll.D["Field"]
    y = qll.gen_source(dims, 3, 6, "all")
    f = F()
    f.l = ctypes.pointer(lay)
    f.f = qll.ptr(y)
    f.nelem = 6
    for sub in ("all", "even", "odd"):
        s = qll.Subset()
        L.layoutSubset(byref(s), byref(lay), sub.encode())
        L.fieldNorm2D.restype = c_double
        L.fieldSumElemD.restype = c_double
        n2 = L.fieldNorm2D(byref(f), byref(s))
        se = L.fieldSumElemD(byref(f), byref(s))
        assert abs(n2 - np.sum(y[s.begin:s.end]**2)) < 1e-10*n2
        assert abs(se - np.sum(y[s.begin:s.end])) < 1e-10*np.sum(np.abs(y))
    for d in (1, -2, 3, -4):
        for ln in (1, 3):
            x = np.zeros_like(y)
            L.shiftD(qll.ptr(x), qll.ptr(y), 6, d, ln)
            assert np.array_equal(x, orc.shift(dims, y, 6, d, ln))
    # fieldtest.c known answer: forward transport then backward transport
    # with the double-stored adjoint returns the field
    th = qll.gen_gauge(dims, 4, 0.5, ks=False)[3]
    ua = orc.doublestore(dims, th, 3, -1)
    T = qll.D["Transporter"]
    t0, tb = T(), T()
    alls = qll.Subset()
    L.layoutSubset(byref(alls), byref(lay), b"all")
    L.getShiftD.restype = ctypes.POINTER(qll.ShiftIndices)
    L.transporterNewD(byref(t0), qll.ptr(th), L.getShiftD(3, 1, b"all"), byref(alls), 6, 3)
    L.transporterNewD(byref(tb), qll.ptr(ua), L.getShiftD(3, -1, b"all"), byref(alls), 6, 3)
    v2 = np.zeros_like(y)
    v3 = np.zeros_like(y)
    L.transporterDoD(byref(t0), qll.ptr(v2), qll.ptr(y), 2)
    L.transporterDoD(byref(tb), qll.ptr(v3), qll.ptr(v2), 2)
    assert np.sum((v3 - y)**2) < 1e-26*np.sum(y**2)
    assert relerr(v2, orc.transport(dims, np.zeros_like(y), th, y, 6, 3, 1)) < 1e-14
    # stress.c known answer: 8 constant-link transports of a constant field
    u0 = np.tile(np.arange(1, 19, dtype=np.float64), (V, 1))
    orc.lib().or_makeUD(qll.ptr(u0), V)
    v1 = np.tile(np.arange(1, 7, dtype=np.float64), (V, 1))
    Ts = [T() for _ in range(8)]
    for d in range(8):
        L.transporterNewD(byref(Ts[d]), qll.ptr(u0), L.getShiftD(d//2, 1 - 2*(d & 1), b"all"),
                          byref(alls), 6, 3)
    nrep = 3
    norms = []
    for its in range(3):
        v2 = np.zeros_like(v1)
        for _ in range(nrep):
            for d in range(8):
                L.transporterDoD(byref(Ts[d]), qll.ptr(v2), qll.ptr(v1), 2)
        norms.append(float(np.sum(v2**2)))
    m = u0[0, 0::2] + 1j*u0[0, 1::2]
    M = m.reshape(3, 3).T
    check = float(np.sum(np.abs(M @ (v1[0, 0::2] + 1j*v1[0, 1::2]))**2))
    assert abs(norms[0]/check/V/nrep**2/64 - 1) < 1e-10
    assert norms[1] == norms[0] and norms[2] == norms[0]


# ----------------------------------------------------------------- Wilson
@pytest.mark.parametrize("prec", ["D", "F"])
@pytest.mark.parametrize("sub", ["all", "even", "odd"])
def test_wilson_dslash_matches_oracle(prec, sub):
    L = qll.load()
    lay = qll.setup_layout(DIMS, prec)
    u = as_dtype(wilson_links(DIMS), DT[prec])
    S = qll.D if prec == "D" else qll.F
    wl = S["WilsonLinks"]()
    getattr(L, "createWilsonLinks" + prec)(byref(wl), byref(lay), _ptrs(u, prec), sub.encode())
    assert wl.t, qll.last_error()
    y = qll.gen_source(DIMS, 21, 24, "all").astype(DT[prec])
    x = np.full_like(y, 3.0)
    getattr(L, "wilsonDslash" + prec)(byref(wl), qll.ptr(x), CT[prec](0.1667), 1, qll.ptr(y))
    ref = orc.wilson_dslash(DIMS, u, 0.1667, y, sub)
    Vh = y.shape[0]//2
    rng = {"all": slice(0, 2*Vh), "even": slice(0, Vh), "odd": slice(Vh, 2*Vh)}[sub]
    assert relerr(x[rng], ref[rng]) < TOL[prec]
    getattr(L, "freeWilsonLinks" + prec)(byref(wl))


@pytest.mark.parametrize("prec", ["F", "D"])
@pytest.mark.parametrize("sub", ["all", "even", "odd"])
def test_wilson_small_launch_kernels(sub, prec):
    """the small-launch Wilson kernels (three threads per site, one per
    output colour: wilson_c3, wilson_f64_c3; two threads per site split by
    direction: wilson_f32_dir2, wilson_f64_dir2) each against the one-
    thread-per-site kernel: the same sums in another order, so rounding
    apart"""
    L = qll.load()
    L.qllg_set_param.argtypes = [ctypes.c_char_p, c_double]
    L.qllg_get_param.argtypes = [ctypes.c_char_p]
    L.qllg_get_param.restype = c_double
    knobs = [b"wilson_c3", b"wilson_f32_dir2"] if prec == "F" else [b"wilson_f64_c3", b"wilson_f64_dir2"]
    saved = {k: L.qllg_get_param(k) for k in knobs}
    lay = qll.setup_layout(DIMS, prec)
    u = as_dtype(wilson_links(DIMS), DT[prec])
    wl = qll.F["WilsonLinks"]() if prec == "F" else qll.D["WilsonLinks"]()
    getattr(L, "createWilsonLinks" + prec)(byref(wl), byref(lay), _ptrs(u, prec), sub.encode())
    assert wl.t, qll.last_error()
    y = qll.gen_source(DIMS, 24, 24, "all").astype(DT[prec])

    def run(on):
        for k in knobs:
            L.qllg_set_param(k, 1 if k == on else 0)
        x = np.full_like(y, 3.0)
        getattr(L, "wilsonDslash" + prec)(byref(wl), qll.ptr(x), CT[prec](0.1667), 1, qll.ptr(y))
        return x
    try:
        base = run(None)
        for k in knobs:
            assert relerr(run(k), base) < (1e-6 if prec == "F" else 1e-14), k
    finally:
        for k in knobs:
            L.qllg_set_param(k, saved[k])
        getattr(L, "freeWilsonLinks" + prec)(byref(wl))


def test_wilson_reference_solve_iterates_match():
    """wilsonSolve is the reference's algorithm (not a convergent solver for
    the Wilson matrix); a fixed number of iterations must match the oracle"""
    L = qll.load()
    lay = qll.setup_layout(DIMS)
    u = list(wilson_links(DIMS))
    ws = qll.D["WilsonSolver"]()
    L.createWilsonSolverD(byref(ws), byref(lay), _ptrs(u, "D"), b"even")
    assert ws.sle.t, qll.last_error()
    b = qll.gen_source(DIMS, 22, 24, "even")
    x = np.zeros_like(b)
    L.wilsonSolveD.restype = c_int
    its = L.wilsonSolveD(byref(ws), qll.ptr(x), c_double(0.5), qll.ptr(b), c_double(1e-30),
                         c_int(6), b"even")
    assert its == 6, qll.last_error()
    its_o, xo = orc.wilson_solve_ref(DIMS, u, 0.5, b, 1e-30, 6)
    Vh = b.shape[0]//2
    assert its_o == 6
    assert relerr(x[:Vh], xo[:Vh]) < 1e-10
    L.freeWilsonSolverD(byref(ws))


@pytest.mark.parametrize("mode", [qll.SOLVE_DOUBLE, qll.SOLVE_MIXED_SINGLE])
def test_wilson_cgnr_matches_oracle(mode):
    L = qll.load()
    L.qllg_wilson_create.restype = ctypes.c_void_p
    L.qllg_wilson_create.argtypes = [ctypes.POINTER(c_int), ctypes.POINTER(ctypes.c_void_p)]
    L.qllg_wilson_solve.restype = c_int
    L.qllg_wilson_solve.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, c_double,
                                    c_double, c_int, c_int, ctypes.POINTER(qll.SolveInfo)]
    u = list(wilson_links(DIMS))
    W = L.qllg_wilson_create(qll.dims_c(DIMS), qll.vp_array(u))
    assert W, qll.last_error()
    b = qll.gen_source(DIMS, 23, 24, "even")
    x = np.zeros_like(b)
    info = qll.SolveInfo()
    mass = 1/(2*0.12) - 4
    its = L.qllg_wilson_solve(W, x.ctypes.data, b.ctypes.data, mass, 1e-16, 5000, mode, byref(info))
    assert its > 0, qll.last_error()
    its_o, xo, _ = orc.wilson_cgnr(DIMS, u, mass, b, 1e-16, 5000)
    Vh = b.shape[0]//2
    assert relerr(x[:Vh], xo[:Vh]) < 1e-6
    assert info.true_rsq[0] < 1e-12
    if mode == qll.SOLVE_DOUBLE:
        assert abs(its - its_o) <= 2
    else:
        assert info.reliable_updates > 0
    L.qllg_wilson_destroy(ctypes.c_void_p(W))


def test_wilson_double_float_reliable_updates():
    """the mixed CGNR with its intermediate reliable updates in double-float
    (wilson_ru_df 1, the Wilson kernel on (hi, lo) float pairs, with three
    threads or one thread per site) and in FP64 (0): each reaches the FP64
    true residual in about the same iterations, with solutions that agree
    with each other and with the oracle's CGNR"""
    L = qll.load()
    L.qllg_set_param.argtypes = [ctypes.c_char_p, c_double]
    L.qllg_wilson_create.restype = ctypes.c_void_p
    L.qllg_wilson_create.argtypes = [ctypes.POINTER(c_int), ctypes.POINTER(ctypes.c_void_p)]
    L.qllg_wilson_solve.restype = c_int
    L.qllg_wilson_solve.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, c_double,
                                    c_double, c_int, c_int, ctypes.POINTER(qll.SolveInfo)]
    u = list(wilson_links(DIMS))
    W = L.qllg_wilson_create(qll.dims_c(DIMS), qll.vp_array(u))
    assert W, qll.last_error()
    b = qll.gen_source(DIMS, 29, 24, "even")
    Vh = b.shape[0]//2
    mass = 1/(2*0.12) - 4
    res = {}
    for ru_df, c3 in ((1, 1), (1, 0), (0, 1)):
        L.qllg_set_param(b"wilson_ru_df", ru_df)
        L.qllg_set_param(b"wilson_df_c3", c3)
        x = np.zeros_like(b)
        info = qll.SolveInfo()
        its = L.qllg_wilson_solve(W, x.ctypes.data, b.ctypes.data, mass, 1e-20, 5000,
                                  qll.SOLVE_MIXED_SINGLE, byref(info))
        assert its > 0, qll.last_error()
        assert info.reliable_updates > 1
        res[ru_df, c3] = (x, its, info.true_rsq[0])
    L.qllg_set_param(b"wilson_ru_df", 2)
    L.qllg_set_param(b"wilson_df_c3", 1)
    its_o, xo, _ = orc.wilson_cgnr(DIMS, u, mass, b, 1e-20, 5000)
    for key, (x, its, tr) in res.items():
        assert tr < 1e-16, (key, tr)
        assert relerr(x[:Vh], xo[:Vh]) < 1e-7, key
        assert abs(its - res[0, 1][1]) <= 2, (key, its, res[0, 1][1])
        assert relerr(x[:Vh], res[0, 1][0][:Vh]) < 1e-7, key
    L.qllg_wilson_destroy(ctypes.c_void_p(W))


def test_single_stored_operator_matches_double_stored():
    """qllg_stag_create_asqtad_fb holds the 8 forward slots only and makes
    the backward links in the kernels: the Dslash (every precision and rhs
    count), the links it reports and a mixed solve are bitwise those of the
    double-stored operator, at about half the resident link bytes"""
    torch = pytest.importorskip("torch")
    L = qll.load()
    vp = ctypes.c_void_p
    for fn in ("qllg_stag_create_asqtad", "qllg_stag_create_asqtad_fb"):
        getattr(L, fn).restype = vp
        getattr(L, fn).argtypes = [ctypes.POINTER(c_int), ctypes.POINTER(vp),
                                   ctypes.POINTER(qll.Fat7Coeffs)]
    L.qllg_stag_vec_bytes.restype = ctypes.c_size_t
    L.qllg_stag_vec_bytes.argtypes = [vp, c_int, c_int]
    L.qllg_stag_dslash_device.argtypes = [vp, c_int, c_int, c_int, vp, vp]
    L.qllg_stag_device_bytes.restype = ctypes.c_size_t
    L.qllg_stag_device_bytes.argtypes = [vp]
    L.qllg_stag_get_links.argtypes = [vp, ctypes.POINTER(vp)]
    dims = (8, 8, 8, 8)
    th = qll.gen_gauge(dims, 1005, 0.3, ks=True)
    c = qll.asqtad_coeffs()
    S2 = vp(L.qllg_stag_create_asqtad(qll.dims_c(dims), qll.vp_array(th), byref(c)))
    S1 = vp(L.qllg_stag_create_asqtad_fb(qll.dims_c(dims), qll.vp_array(th), byref(c)))
    assert S2.value and S1.value, qll.last_error()
    assert L.qllg_stag_device_bytes(S1)*2 == L.qllg_stag_device_bytes(S2)
    V = int(np.prod(dims))
    l2 = [np.zeros((V, 18)) for _ in range(16)]
    l1 = [np.zeros((V, 18)) for _ in range(16)]
    assert L.qllg_stag_get_links(S2, qll.vp_array(l2)) == 0
    assert L.qllg_stag_get_links(S1, qll.vp_array(l1)) == 0
    for k in range(16):
        assert np.array_equal(l1[k], l2[k]), k
    g = torch.Generator(device="cuda").manual_seed(5)
    for prec in (0, 1, 2):
        for nrhs in (1, 4, 16):
            n = L.qllg_stag_vec_bytes(S2, prec, nrhs)
            if prec == 0:
                src = torch.randn(n//8, dtype=torch.float64, device="cuda", generator=g)
            else:
                src = torch.randn(n//4, dtype=torch.float32, device="cuda", generator=g)
                if prec == 2:
                    src = src.view(-1, 4)
                    src[:, 3] = 1.0
                    src = src.reshape(-1)
            for parity in (0, 1):
                o2, o1 = torch.zeros_like(src), torch.zeros_like(src)
                torch.cuda.synchronize()
                assert L.qllg_stag_dslash_device(S2, prec, nrhs, parity, vp(o2.data_ptr()),
                                                 vp(src.data_ptr())) == 0, qll.last_error()
                assert L.qllg_stag_dslash_device(S1, prec, nrhs, parity, vp(o1.data_ptr()),
                                                 vp(src.data_ptr())) == 0, qll.last_error()
                torch.cuda.synchronize()
                assert torch.equal(o1.view(torch.uint8), o2.view(torch.uint8)), (prec, nrhs, parity)
    # every autotuner candidate of the 16-rhs FP32 kernel, single-stored
    # against double-stored
    L.qllg_set_param.argtypes = [ctypes.c_char_p, c_double]
    n = L.qllg_stag_vec_bytes(S2, 1, 16)
    src = torch.randn(n//4, dtype=torch.float32, device="cuda", generator=g)
    for v in range(24):
        L.qllg_set_param(b"dslash_variant", v)
        o2, o1 = torch.zeros_like(src), torch.zeros_like(src)
        torch.cuda.synchronize()
        assert L.qllg_stag_dslash_device(S2, 1, 16, 1, vp(o2.data_ptr()), vp(src.data_ptr())) == 0
        assert L.qllg_stag_dslash_device(S1, 1, 16, 1, vp(o1.data_ptr()), vp(src.data_ptr())) == 0
        torch.cuda.synchronize()
        assert torch.equal(o1.view(torch.uint8), o2.view(torch.uint8)), v
    L.qllg_set_param(b"dslash_variant", -1)
    nrhs = 8
    masses = (c_double*nrhs)(*[0.05 + 0.01*k for k in range(nrhs)])
    bs = [qll.gen_source(dims, 9000 + k, 6, "even") for k in range(nrhs)]
    sol = []
    # 18-real links (reconstruct-12 rebuilds a backward Naik link from its
    # own two rows when double-stored, from the forward one when single-
    # stored: equal to FP32 rounding, not bitwise)
    L.qllg_set_param.argtypes = [ctypes.c_char_p, c_double]
    L.qllg_set_param(b"links_recon12", 0)
    for S in (S2, S1):
        xs = [np.zeros_like(bs[0]) for _ in range(nrhs)]
        info = qll.SolveInfo()
        its = L.qllg_stag_solve(S, nrhs, qll.vp_array(xs), qll.vp_array(bs), masses, 1e-16, 5000,
                                qll.SOLVE_MIXED_SINGLE, byref(info))
        assert its > 0, qll.last_error()
        sol.append((list(info.iters[:nrhs]), xs))
    L.qllg_set_param(b"links_recon12", 0)
    assert sol[0][0] == sol[1][0]
    for k in range(nrhs):
        assert np.array_equal(sol[0][1][k], sol[1][1][k])
    L.qllg_stag_destroy(S1)
    L.qllg_stag_destroy(S2)


@pytest.mark.parametrize("mode", [qll.SOLVE_DOUBLE, qll.SOLVE_MIXED_SINGLE])
def test_wilson_cgnr_graph_matches_host_loop(mode):
    """the CGNR loop captured as one CUDA-graph launch runs the same kernels
    in the same order as the host-polled loop: bitwise the same solution
    and iteration count"""
    L = qll.load()
    L.qllg_set_param.argtypes = [ctypes.c_char_p, c_double]
    L.qllg_wilson_create.restype = ctypes.c_void_p
    L.qllg_wilson_create.argtypes = [ctypes.POINTER(c_int), ctypes.POINTER(ctypes.c_void_p)]
    L.qllg_wilson_solve.restype = c_int
    L.qllg_wilson_solve.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, c_double,
                                    c_double, c_int, c_int, ctypes.POINTER(qll.SolveInfo)]
    dims = (8, 8, 8, 8)
    u = list(wilson_links(dims))
    W = L.qllg_wilson_create(qll.dims_c(dims), qll.vp_array(u))
    assert W, qll.last_error()
    b = qll.gen_source(dims, 24, 24, "even")
    mass = 1/(2*0.12) - 4
    out = []
    L.qllg_set_param(b"wilson_persistent", 0)     # the graph loop, not the persistent one
    for graph in (1, 0, 1):
        L.qllg_set_param(b"graph", graph)
        x = np.zeros_like(b)
        info = qll.SolveInfo()
        its = L.qllg_wilson_solve(W, x.ctypes.data, b.ctypes.data, mass, 1e-16, 5000, mode,
                                  byref(info))
        assert its > 0, qll.last_error()
        out.append((its, x))
    L.qllg_set_param(b"graph", 1)
    L.qllg_set_param(b"wilson_persistent", 1)
    assert out[0][0] == out[1][0] == out[2][0]
    assert np.array_equal(out[0][1], out[1][1]) and np.array_equal(out[0][1], out[2][1])
    L.qllg_wilson_destroy(ctypes.c_void_p(W))


def test_wilson_fused_update_matches_separate_kernels():
    """the FP32 CGNR with the CG update in the last half Dslash's epilogue
    (wilson_fused_update) against the separate update kernel: the |r|^2
    sums are reduced in a different order, so the two agree to the solver's
    accuracy (iterations within one, solutions within 1e-6), and both reach
    the true residual target; the reliable-update block as a graph
    conditional (graph_ru_if) changes nothing, bitwise"""
    L = qll.load()
    L.qllg_set_param.argtypes = [ctypes.c_char_p, c_double]
    L.qllg_wilson_create.restype = ctypes.c_void_p
    L.qllg_wilson_create.argtypes = [ctypes.POINTER(c_int), ctypes.POINTER(ctypes.c_void_p)]
    L.qllg_wilson_solve.restype = c_int
    L.qllg_wilson_solve.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, c_double,
                                    c_double, c_int, c_int, ctypes.POINTER(qll.SolveInfo)]
    dims = (8, 8, 8, 16)
    u = list(wilson_links(dims))
    W = L.qllg_wilson_create(qll.dims_c(dims), qll.vp_array(u))
    assert W, qll.last_error()
    b = qll.gen_source(dims, 31, 24, "even")
    mass = 1/(2*0.12) - 4
    runs = {}
    L.qllg_set_param(b"wilson_persistent", 0)     # the graph loop, not the persistent one
    for fused in (1, 0):
        for ru_if in (1, 0):
            L.qllg_set_param(b"wilson_fused_update", fused)
            L.qllg_set_param(b"graph_ru_if", ru_if)
            x = np.zeros_like(b)
            info = qll.SolveInfo()
            its = L.qllg_wilson_solve(W, x.ctypes.data, b.ctypes.data, mass, 1e-17, 5000,
                                      qll.SOLVE_MIXED_SINGLE, byref(info))
            assert its > 0, qll.last_error()
            assert info.true_rsq[0] < 1e-16
            runs[(fused, ru_if)] = (its, info.reliable_updates, x)
    L.qllg_set_param(b"wilson_fused_update", 1)
    L.qllg_set_param(b"graph_ru_if", 1)
    L.qllg_set_param(b"wilson_persistent", 1)
    # the IF node changes nothing: bitwise the same per fused setting
    for fused in (1, 0):
        a, c = runs[(fused, 1)], runs[(fused, 0)]
        assert a[0] == c[0] and a[1] == c[1] and np.array_equal(a[2], c[2])
    f, s = runs[(1, 1)], runs[(0, 1)]
    assert abs(f[0] - s[0]) <= 1
    assert relerr(f[2], s[2]) < 1e-6
    L.qllg_wilson_destroy(ctypes.c_void_p(W))
