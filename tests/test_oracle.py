"""The CPU oracle against the known-answer tests of the reference's own test
programs (stress.c, fieldtest.c) and against analytic properties of the
operators.  No GPU."""
import ctypes

import numpy as np
import pytest

import oracle_lib as orc
from inputs import asqtad_links, relerr
from qll_gb300 import qll

DIMS = (4, 4, 4, 4)


def test_stress_kat():
    # stress.c:218-234: first pass within 1e-10 of the analytic norm, later
    # passes bitwise identical
    ok = ctypes.c_int()
    r = orc.lib().or_stress_kat(orc.dims_c((4, 4, 6, 4)), 3, 4, ctypes.byref(ok))
    assert abs(r - 1) < 1e-10
    assert ok.value == 1


def test_fieldtest_kat():
    # fieldtest.c:183-191: forward then backward transport with the
    # double-stored adjoint is the identity
    d = (4, 4, 4, 6)
    v = orc.lib().or_fieldtest_kat(orc.dims_c(d))
    V = np.prod(d)
    norm_v1 = sum(float(i)**2 for i in range(6*V))
    assert v < 1e-28*norm_v1


@pytest.mark.parametrize("dims", [(4, 4, 4, 4), (4, 6, 4, 8), (8, 4, 6, 4)])
def test_layout_index_matches_library(dims):
    lay = qll.setup_layout(dims)
    L = qll.load()
    V = int(np.prod(dims))
    for i in range(V):
        x = orc.site_coord(dims, i)
        assert orc.site_index(dims, x) == i
        li = qll.LayoutIndex()
        xc = (ctypes.c_int*4)(*x)
        L.layoutIndex(ctypes.byref(lay), ctypes.byref(li), xc)
        assert li.index == i
        yc = (ctypes.c_int*4)()
        L.layoutCoord(ctypes.byref(lay), yc, ctypes.byref(li))
        assert tuple(yc) == x


def test_shift_tables_match_library():
    dims = (4, 6, 4, 8)
    qll.setup_layout(dims)
    L = qll.load()
    V = int(np.prod(dims))
    for mu in range(4):
        for ln in (1, -1, 3, -3):
            for sub, par in (("all", -1), ("even", 0), ("odd", 1)):
                si = L.getShiftD(mu, ln, sub.encode())
                lib_t = np.ctypeslib.as_array(si.contents.pidx, shape=(V,))
                disp = [0, 0, 0, 0]
                disp[mu] = -ln
                assert np.array_equal(lib_t, orc.shift_table(dims, disp, par))


def _cdot(a, b):
    ac = a[:, 0::2] + 1j*a[:, 1::2]
    bc = b[:, 0::2] + 1j*b[:, 1::2]
    return np.vdot(ac, bc)


def test_dslash_antihermitian():
    u, u3 = asqtad_links(DIMS)
    a = qll.gen_source(DIMS, 7, 6, "all")
    b = qll.gen_source(DIMS, 8, 6, "all")
    Db = orc.dslash(DIMS, u, u3, 0.0, b, "all")
    Da = orc.dslash(DIMS, u, u3, 0.0, a, "all")
    lhs, rhs = _cdot(a, Db), -_cdot(Da, b)
    assert abs(lhs - rhs) < 1e-12*abs(lhs)


def _random_su3(V, seed):
    g = qll.gen_gauge((4, 4, 4, 4), seed, 2.0, ks=False)[0]
    assert g.shape[0] == V
    m = g[:, 0::2] + 1j*g[:, 1::2]
    return m.reshape(V, 3, 3).transpose(0, 2, 1)   # [site][row][col]


def _to_mat(u):
    V = u.shape[0]
    return (u[:, 0::2] + 1j*u[:, 1::2]).reshape(V, 3, 3).transpose(0, 2, 1)


def _from_mat(m):
    V = m.shape[0]
    c = m.transpose(0, 2, 1).reshape(V, 9)
    out = np.empty((V, 18))
    out[:, 0::2] = c.real
    out[:, 1::2] = c.imag
    return out


def _shift_idx(dims, mu, ln):
    disp = [0, 0, 0, 0]
    disp[mu] = -ln
    return orc.shift_table(dims, disp, -1)


def test_fat7_and_dslash_gauge_covariance():
    dims = DIMS
    V = int(np.prod(dims))
    th = qll.gen_gauge(dims, 1001, 0.3, ks=True)
    g = _random_su3(V, 4242)
    gd = g.conj().transpose(0, 2, 1)
    thg = []
    for mu in range(4):
        fw = _shift_idx(dims, mu, 1)
        thg.append(_from_mat(g @ _to_mat(th[mu]) @ gd[fw]))
    c = qll.asqtad_coeffs()
    fl, ll = orc.smear_fat7(dims, th, c)
    flg, llg = orc.smear_fat7(dims, thg, c)
    for mu in range(4):
        f1 = _shift_idx(dims, mu, 1)
        f3 = _shift_idx(dims, mu, 3)
        assert relerr(_to_mat(flg[mu]), g @ _to_mat(fl[mu]) @ gd[f1]) < 1e-13
        assert relerr(_to_mat(llg[mu]), g @ _to_mat(ll[mu]) @ gd[f3]) < 1e-13
    # Dslash with transformed links on a transformed field
    u, u3 = [None]*8, [None]*8
    ug, u3g = [None]*8, [None]*8
    for mu in range(4):
        u[2*mu], u[2*mu+1] = fl[mu], orc.negadj_back(dims, fl[mu], mu, 1)
        u3[2*mu], u3[2*mu+1] = ll[mu], orc.negadj_back(dims, ll[mu], mu, 3)
        ug[2*mu], ug[2*mu+1] = flg[mu], orc.negadj_back(dims, flg[mu], mu, 1)
        u3g[2*mu], u3g[2*mu+1] = llg[mu], orc.negadj_back(dims, llg[mu], mu, 3)
    psi = qll.gen_source(dims, 9, 6, "all")
    pc = psi[:, 0::2] + 1j*psi[:, 1::2]
    gpsi_c = np.einsum("sij,sj->si", g, pc)
    gpsi = np.empty_like(psi)
    gpsi[:, 0::2], gpsi[:, 1::2] = gpsi_c.real, gpsi_c.imag
    out = orc.dslash(dims, ug, u3g, 0.3, gpsi, "all")
    ref = orc.dslash(dims, u, u3, 0.3, psi, "all")
    rc = np.einsum("sij,sj->si", g, ref[:, 0::2] + 1j*ref[:, 1::2])
    assert relerr(out[:, 0::2] + 1j*out[:, 1::2], rc) < 1e-13


def test_plaquette():
    dims = DIMS
    V = int(np.prod(dims))
    unit = np.zeros((V, 18))
    unit[:, [0, 8, 16]] = 1.0
    assert np.allclose(orc.plaq(dims, [unit]*4), 1.0, atol=1e-15)
    th = qll.gen_gauge(dims, 55, 0.3, ks=False)
    p = orc.plaq(dims, th)
    assert np.all(p < 1) and np.all(p > 0.5)
    # gauge invariance
    g = _random_su3(V, 77)
    gd = g.conj().transpose(0, 2, 1)
    thg = [_from_mat(g @ _to_mat(th[mu]) @ gd[_shift_idx(dims, mu, 1)]) for mu in range(4)]
    assert np.allclose(orc.plaq(dims, thg), p, atol=1e-13)


def test_fat7_one_link_only():
    th = qll.gen_gauge(DIMS, 3, 0.3, ks=True)
    c = qll.Fat7Coeffs(0.7, 0, 0, 0, 0, 0)
    fl, ll = orc.smear_fat7(DIMS, th, c, want_long=False)
    for mu in range(4):
        assert np.allclose(fl[mu], 0.7*th[mu], atol=1e-15)


def test_cg_true_residual_and_cgms_consistency():
    dims = DIMS
    u, u3 = asqtad_links(dims)
    b = qll.gen_source(dims, 2001, 6, "even")
    V = int(np.prod(dims))
    Vh = V//2
    its, x, frsq = orc.solve2(dims, u, u3, 0.1, b, 1e-20, 1000, noscale=1)
    assert frsq < 1e-20
    Ax, _ = orc.dslashp2(dims, u, u3, 0.1, x)
    r = b[:Vh] - Ax[:Vh]
    assert np.linalg.norm(r)**2 < 1e-18*np.linalg.norm(b[:Vh])**2
    masses = [0.1, 0.14, 0.2]
    itm, xs = orc.solve_multi2(dims, u, u3, masses, b, 1e-20, 1000, noscale=1)
    for m, xm in zip(masses, xs):
        _, xr, _ = orc.solve2(dims, u, u3, m, b, 1e-22, 1000, noscale=1)
        assert relerr(xm[:Vh], xr[:Vh]) < 1e-8


def test_gamma_algebra_and_wilson_gamma5_hermiticity():
    g = [orc.gamma(d) for d in range(5)]
    I4 = np.eye(4)
    for a in range(4):
        for b in range(4):
            assert np.allclose(g[a] @ g[b] + g[b] @ g[a], 2*I4*(a == b))
    assert np.allclose(g[4], g[0] @ g[1] @ g[2] @ g[3])
    # Wilson links u[2mu] = U/2, u[2mu+1] = +U(x-mu)^dagger/2
    dims = DIMS
    th = qll.gen_gauge(dims, 12, 0.3, ks=False)
    u = [None]*8
    for mu in range(4):
        u[2*mu] = 0.5*th[mu]
        u[2*mu+1] = 0.5*orc.doublestore(dims, th[mu], mu, -1)
    a = qll.gen_source(dims, 1, 24, "even")
    b = qll.gen_source(dims, 2, 24, "even")
    Sb = orc.wilson_schur(dims, u, 0.1667, b, 0)
    Sda = orc.wilson_schur(dims, u, 0.1667, a, 1)
    Vh = int(np.prod(dims))//2
    lhs = _cdot(a[:Vh], Sb[:Vh])
    rhs = _cdot(Sda[:Vh], b[:Vh])
    assert abs(lhs - rhs) < 1e-12*abs(lhs)
