"""The oracle against the reference's own outputs stored in
tests/golden/ref_4x4x4x4.npz (made by tests/golden/make_golden.py from the
reference library compiled from its sources): runs on any machine, with or
without the reference tree.  Dslash, fat7 and Wilson Dslash bit for bit;
solves to 1e-10 (the global sums are folded in another order, and the
solution error is that rounding times the condition number)."""
import os

import numpy as np
import pytest

import oracle_lib as orc
from inputs import relerr
from qll_gb300 import qll

G = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_4x4x4x4.npz"))
DIMS = tuple(int(v) for v in G["dims"])


def golden_links():
    """the reference's fat and Naik links with the oracle's negative-adjoint
    backward links (bit for bit the reference's, tests/test_ref_pin.py)"""
    u, u3 = [None]*8, [None]*8
    for mu in range(4):
        u[2*mu] = np.ascontiguousarray(G["fat"][mu])
        u[2*mu + 1] = orc.negadj_back(DIMS, u[2*mu], mu, 1)
        u3[2*mu] = np.ascontiguousarray(G["long"][mu])
        u3[2*mu + 1] = orc.negadj_back(DIMS, u3[2*mu], mu, 3)
    return u, u3


def golden_wilson_links():
    th = [np.ascontiguousarray(G["thin"][mu]) for mu in range(4)]
    u = []
    for mu in range(4):
        u += [0.5*th[mu], 0.5*orc.doublestore(DIMS, th[mu], mu, -1)]
    return u


def test_fat7_matches_reference():
    thin = [np.ascontiguousarray(G["thin"][mu]) for mu in range(4)]
    fl, ll = orc.smear_fat7(DIMS, thin, qll.asqtad_coeffs())
    for mu in range(4):
        assert np.array_equal(fl[mu], G["fat"][mu])
        assert np.array_equal(ll[mu], G["long"][mu])


@pytest.mark.parametrize("sub", ["all", "even", "odd"])
def test_dslash2_matches_reference(sub):
    u, u3 = golden_links()
    got = orc.dslash(DIMS, u, u3, 0.25, np.ascontiguousarray(G["y"]), sub)
    assert np.array_equal(got, G["d_" + sub])


def test_solves_match_reference():
    u, u3 = golden_links()
    b = np.ascontiguousarray(G["b"])
    its, x, _ = orc.solve2(DIMS, u, u3, 0.1, b, 1e-16, 5000, noscale=1)
    assert abs(its - int(G["its_solve2"])) <= 1
    assert relerr(x, G["x_solve2"]) < 1e-10
    masses = [float(m) for m in G["masses"]]
    its, xs = orc.solve_multi2(DIMS, u, u3, masses, b, 1e-16, 5000, noscale=1)
    assert abs(its - int(G["its_multi"])) <= 1
    for k in range(len(masses)):
        assert relerr(xs[k], G["x_multi"][k]) < 1e-10


@pytest.mark.parametrize("sub", ["all", "even", "odd"])
def test_wilson_dslash_matches_reference(sub):
    got = orc.wilson_dslash(DIMS, golden_wilson_links(), 0.1667, np.ascontiguousarray(G["yw"]),
                            sub)
    assert np.array_equal(got, G["w_" + sub])
