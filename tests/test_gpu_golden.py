"""The GPU path against the reference's own outputs (tests/golden/
ref_4x4x4x4.npz, made from the reference library compiled from its
sources), through the drop-in C API: fat7 from the stored thin links,
dslash2, solve2, solveMulti2 and wilsonDslash on the stored inputs.
Tolerances: FP64 operators 1e-12 relative, FP32 1e-5; solves to the
reference's iteration count within 1 and solutions within 1e-7 (10x the
solver tolerance 1e-8)."""
import ctypes
import os
from ctypes import byref, c_double, c_float, c_int

import numpy as np
import pytest

from inputs import relerr
from qll_gb300 import qll
from test_golden import DIMS, G, golden_links, golden_wilson_links

pytestmark = pytest.mark.gpu

DT = {"D": np.float64, "F": np.float32}
CT = {"D": c_double, "F": c_float}


def test_fat7_on_gpu_matches_reference():
    L = qll.load()
    L.qllg_stag_create_asqtad.restype = ctypes.c_void_p
    L.qllg_stag_create_asqtad.argtypes = [ctypes.POINTER(c_int), ctypes.POINTER(ctypes.c_void_p),
                                          ctypes.POINTER(qll.Fat7Coeffs)]
    L.qllg_stag_get_links.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]
    thin = [np.ascontiguousarray(G["thin"][mu]) for mu in range(4)]
    S = L.qllg_stag_create_asqtad(qll.dims_c(DIMS), qll.vp_array(thin), byref(qll.asqtad_coeffs()))
    assert S, qll.last_error()
    V = int(np.prod(DIMS))
    links = [np.zeros((V, 18)) for _ in range(16)]
    assert L.qllg_stag_get_links(ctypes.c_void_p(S), qll.vp_array(links)) == 0
    L.qllg_stag_destroy(ctypes.c_void_p(S))
    for mu in range(4):
        assert relerr(links[4*mu], G["fat"][mu]) < 1e-12, mu
        assert relerr(links[4*mu + 1], G["long"][mu]) < 1e-12, mu


@pytest.mark.parametrize("prec", ["D", "F"])
@pytest.mark.parametrize("sub", ["all", "even", "odd"])
def test_dslash2_matches_reference(prec, sub):
    L = qll.load()
    lay = qll.setup_layout(DIMS, prec)
    u, u3 = golden_links()
    u = [a.astype(DT[prec]) for a in u]
    u3 = [a.astype(DT[prec]) for a in u3]
    St = qll.D if prec == "D" else qll.F
    sl = St["StaggeredLinks"]()
    getattr(L, "createStaggeredLinks" + prec)(byref(sl), byref(lay), qll.ptr_array(u, CT[prec]),
                                              qll.ptr_array(u3, CT[prec]), sub.encode())
    assert sl.t, qll.last_error()
    y = np.ascontiguousarray(G["y"], dtype=DT[prec])
    x = np.zeros_like(y)
    getattr(L, "dslash2" + prec)(byref(sl), qll.ptr(x), CT[prec](0.25), qll.ptr(y))
    getattr(L, "freeStaggeredLinks" + prec)(byref(sl))
    want = G["d_" + sub]
    Vh = x.shape[0]//2
    rng = {"all": slice(0, 2*Vh), "even": slice(0, Vh), "odd": slice(Vh, 2*Vh)}[sub]
    assert relerr(x[rng], want[rng]) < (1e-12 if prec == "D" else 1e-5)


def test_solve2_and_solve_multi2_match_reference():
    L = qll.load()
    lay = qll.setup_layout(DIMS, "D")
    u, u3 = golden_links()
    ss = qll.D["StaggeredSolver"]()
    L.createStaggeredSolverD(byref(ss), byref(lay), qll.ptr_array(u, c_double),
                             qll.ptr_array(u3, c_double), b"even")
    assert ss.sle.t, qll.last_error()
    ss.noscale = 1
    b = np.ascontiguousarray(G["b"])
    Vh = b.shape[0]//2
    x = np.zeros_like(b)
    L.solve2D.restype = c_int
    its = L.solve2D(byref(ss), qll.ptr(x), c_double(0.1), qll.ptr(b), c_double(1e-16), c_int(5000),
                    b"even")
    assert abs(its - int(G["its_solve2"])) <= 1, (its, int(G["its_solve2"]))
    assert relerr(x[:Vh], G["x_solve2"][:Vh]) < 1e-7
    masses = [float(m) for m in G["masses"]]
    xs = [np.zeros_like(b) for _ in masses]
    L.solveMulti2D.restype = c_int
    its = L.solveMulti2D(byref(ss), qll.ptr_array(xs, c_double),
                         (c_double*len(masses))(*masses), len(masses), qll.ptr(b),
                         c_double(1e-16), c_int(5000), b"even")
    assert abs(its - int(G["its_multi"])) <= 1, (its, int(G["its_multi"]))
    for k in range(len(masses)):
        assert relerr(xs[k][:Vh], G["x_multi"][k][:Vh]) < 1e-7, k
    L.freeStaggeredSolverD(byref(ss))


@pytest.mark.parametrize("prec", ["D", "F"])
@pytest.mark.parametrize("sub", ["all", "even", "odd"])
def test_wilson_dslash_matches_reference(prec, sub):
    L = qll.load()
    lay = qll.setup_layout(DIMS, prec)
    u = [a.astype(DT[prec]) for a in golden_wilson_links()]
    St = qll.D if prec == "D" else qll.F
    wl = St["WilsonLinks"]()
    getattr(L, "createWilsonLinks" + prec)(byref(wl), byref(lay), qll.ptr_array(u, CT[prec]),
                                           sub.encode())
    assert wl.t, qll.last_error()
    y = np.ascontiguousarray(G["yw"], dtype=DT[prec])
    x = np.zeros_like(y)
    getattr(L, "wilsonDslash" + prec)(byref(wl), qll.ptr(x), CT[prec](0.1667), 1, qll.ptr(y))
    getattr(L, "freeWilsonLinks" + prec)(byref(wl))
    want = G["w_" + sub]
    Vh = x.shape[0]//2
    rng = {"all": slice(0, 2*Vh), "even": slice(0, Vh), "odd": slice(Vh, 2*Vh)}[sub]
    assert relerr(x[rng], want[rng]) < (1e-12 if prec == "D" else 1e-5)
