"""The oracle pinned to the reference itself: the reference library compiled
from its own sources (oracle/ref_build.py, one-lane -DC1 build) and the
oracle's C restatement run on the same seeded inputs.

Expected agreement: the Dslash, fat7 smearing, plaquette and Wilson
Dslash keep the reference's operation order site by site, so they agree
bit for bit; the solvers' global sums are folded in a different order
(the reference sums per OpenMP thread, then over threads), so CG and cgms
iterates agree to rounding: CG solutions within 1e-12 relative, cgms
solutions within 1e-10 (the small-mass system amplifies rounding), and
iteration counts within 1.

Skipped where the reference was not built (no reference tree and no staged
sources on this machine)."""
import numpy as np
import pytest

import oracle_lib as orc
import ref_lib as ref
from inputs import asqtad_links, relerr, wilson_links
from qll_gb300 import qll

pytestmark = pytest.mark.skipif(not ref.available(), reason="reference library not built")

DIMS = [(4, 4, 6, 8), (8, 8, 8, 8)]


@pytest.mark.parametrize("dims", DIMS)
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("sub", ["all", "even", "odd"])
def test_dslash2_bitwise(dims, dtype, sub):
    u, u3 = asqtad_links(dims)
    u = [np.ascontiguousarray(a, dtype=dtype) for a in u]
    u3 = [np.ascontiguousarray(a, dtype=dtype) for a in u3]
    y = qll.gen_source(dims, 31, 6, "all").astype(dtype)
    got = orc.dslash(dims, u, u3, 0.25, y, sub)
    want = ref.dslash(dims, u, u3, 0.25, y, sub)
    assert np.array_equal(got, want), relerr(got, want)


@pytest.mark.parametrize("dims", DIMS)
def test_fat7_and_plaquette_bitwise(dims):
    thin = qll.gen_gauge(dims, 1001, 0.3, ks=True)
    coef = qll.asqtad_coeffs()
    fl, ll = orc.smear_fat7(dims, thin, coef)
    rfl, rll = ref.smear_fat7(dims, thin, coef)
    for mu in range(4):
        assert np.array_equal(fl[mu], rfl[mu]), (mu, relerr(fl[mu], rfl[mu]))
        assert np.array_equal(ll[mu], rll[mu]), (mu, relerr(ll[mu], rll[mu]))
    th = qll.gen_gauge(dims, 1001, 0.3, ks=False)
    assert np.allclose(orc.plaq(dims, th), ref.plaq(dims, th), rtol=1e-14, atol=0)


def test_fat7_general_coefficients():
    """every path of smearFat7 with distinct weights (the reference's own
    test coefficients of testdslash.c:306-312), so that a swapped staple
    term would show"""
    dims = (4, 4, 6, 8)
    thin = qll.gen_gauge(dims, 77, 0.5, ks=True)

    class C:
        one_link = 0.3 - (0.1*15)/16
        three_staple = 0.2/(4*6)
        five_staple = 0.2/(16*24)
        seven_staple = 0.2/(64*48)
        lepage = 0.1/(16*6)
        naik = 0.2
    fl, ll = orc.smear_fat7(dims, thin, C)
    rfl, rll = ref.smear_fat7(dims, thin, C)
    for mu in range(4):
        assert np.array_equal(fl[mu], rfl[mu])
        assert np.array_equal(ll[mu], rll[mu])


@pytest.mark.parametrize("dims,mass", [((4, 4, 6, 8), 0.1), ((8, 8, 8, 8), 0.1)])
def test_solve2(dims, mass):
    u, u3 = asqtad_links(dims)
    b = qll.gen_source(dims, 2100, 6, "even")
    its_o, xo, _ = orc.solve2(dims, u, u3, mass, b, 1e-16, 5000, noscale=0)
    its_r, xr = ref.solve2(dims, u, u3, mass, b, 1e-16, 5000, noscale=0)
    assert abs(its_o - its_r) <= 1, (its_o, its_r)
    assert relerr(xo, xr) < 1e-12


def test_solve_multi2():
    dims = (4, 4, 6, 8)
    u, u3 = asqtad_links(dims)
    b = qll.gen_source(dims, 2300, 6, "even")
    masses = [0.05, 0.08, 0.2, 0.5]
    its_o, xo = orc.solve_multi2(dims, u, u3, masses, b, 1e-16, 5000, noscale=1)
    its_r, xr = ref.solve_multi2(dims, u, u3, masses, b, 1e-16, 5000, noscale=1)
    assert abs(its_o - its_r) <= 1, (its_o, its_r)
    for k in range(len(masses)):
        # the smallest mass (condition number ~ 1e3 here) amplifies the
        # rounding of the differently ordered sums to a few 1e-12
        assert relerr(xo[k], xr[k]) < 1e-10, k


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("sub", ["all", "even", "odd"])
def test_wilson_dslash_bitwise(dtype, sub):
    dims = (4, 4, 6, 8)
    u = [np.ascontiguousarray(a, dtype=dtype) for a in wilson_links(dims)]
    y = qll.gen_source(dims, 22, 24, "all").astype(dtype)
    got = orc.wilson_dslash(dims, u, 0.1667, y, sub)
    want = ref.wilson_dslash(dims, u, 0.1667, y, sub)
    assert np.array_equal(got, want), relerr(got, want)


def test_shift_doublestore_and_backward_links():
    """the reference's shift and gaugeDoublestore against the oracle's, and
    the negative-adjoint backward links the tests and the benchmark feed to
    createStaggeredLinks (-F(x-mu)^dagger, -L(x-3mu)^dagger) against
    minus the reference's doublestore"""
    dims = (4, 4, 6, 8)
    th = qll.gen_gauge(dims, 1001, 0.3, ks=True)
    v = qll.gen_source(dims, 5, 6, "all")
    for mu in range(4):
        for d in (mu + 1, -(mu + 1)):
            for ln in (1, 3):
                assert np.array_equal(orc.shift(dims, v, 6, d, ln), ref.shift(dims, v, 6, d, ln))
        for ln in (1, 3):
            want = ref.doublestore(dims, th[mu], mu, -ln)
            assert np.array_equal(orc.doublestore(dims, th[mu], mu, -ln), want)
            assert np.array_equal(orc.negadj_back(dims, th[mu], mu, ln), -want)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_make_u_bitwise(dtype):
    """makeU (lib/vla.c:1635-1665) is site-local: the oracle's restatement
    equals the reference's result bit for bit on seeded random matrices"""
    rng = np.random.default_rng(1656)
    m = rng.standard_normal((2048, 18)).astype(dtype)
    want = ref.make_u(m.copy())
    got = orc.make_u(m.copy())
    assert np.array_equal(got, want), relerr(got, want)
