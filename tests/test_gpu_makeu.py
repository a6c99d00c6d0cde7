"""GPU: makeUD/makeUF (include/vla.h), QLL's re-unitarisation of matrix
sites (lib/vla.c:1635-1665), against the oracle's restatement: the same
vectors within rounding (the GPU fuses its multiply-adds), as unitary as
the oracle's result, sites outside [i0, i1) untouched, and nc 1 and 2
against the same Gram-Schmidt written here."""
import ctypes

import numpy as np
import pytest

import oracle_lib as orc
from qll_gb300 import qll

pytestmark = pytest.mark.gpu


def _call(a, nc, i0, i1):
    L = qll.load()
    f = L.makeUD if a.dtype == np.float64 else L.makeUF
    ct = ctypes.c_double if a.dtype == np.float64 else ctypes.c_float
    f.argtypes = [ctypes.POINTER(ct), ctypes.c_int, ctypes.c_int, ctypes.c_int]
    f.restype = None
    L.qllg_clear_error()
    f(a.ctypes.data_as(ctypes.POINTER(ct)), nc, i0, i1)
    assert not qll.last_error(), qll.last_error()


def _gram_schmidt(m, nc):
    """the reference's order: normalise v_i, then for each j < i remove
    <v_j, v_i> v_j and normalise again"""
    v = [m[2*nc*i:2*nc*(i + 1)].astype(np.float64) for i in range(nc)]
    c = [x[0::2] + 1j*x[1::2] for x in v]
    for i in range(nc):
        c[i] = c[i]/np.sqrt(np.vdot(c[i], c[i]).real)
        for j in range(i):
            c[i] = c[i] - np.vdot(c[j], c[i])*c[j]
            c[i] = c[i]/np.sqrt(np.vdot(c[i], c[i]).real)
    out = np.empty(2*nc*nc)
    for i in range(nc):
        out[2*nc*i:2*nc*(i + 1):2] = c[i].real
        out[2*nc*i + 1:2*nc*(i + 1):2] = c[i].imag
    return out


@pytest.mark.parametrize("dt", [np.float64, np.float32])
def test_make_u_matches_oracle(dt):
    rng = np.random.default_rng(1635)
    n = 5000
    m = rng.standard_normal((n, 18)).astype(dt)
    want = orc.make_u(m.copy())
    got = m.copy()
    _call(got, 3, 0, n)
    tol = 1e-13 if dt == np.float64 else 1e-5
    assert np.max(np.abs(got - want)) < tol
    # unitary to the rounding of a single Gram-Schmidt pass, as the
    # oracle's (random matrices include badly conditioned ones)
    def unitarity(a):
        U = (a[:, 0::2].astype(np.float64) + 1j*a[:, 1::2].astype(np.float64)).reshape(n, 3, 3)
        return np.max(np.abs(np.einsum("sik,sjk->sij", U, U.conj()) - np.eye(3)))
    assert unitarity(got) < (1e-12 if dt == np.float64 else 1e-4)
    assert unitarity(got) < 10*unitarity(want) + (1e-15 if dt == np.float64 else 1e-7)
    # a sub-range: the other sites stay as they were
    part = m.copy()
    _call(part, 3, 100, 2100)
    assert np.array_equal(part[:100], m[:100]) and np.array_equal(part[2100:], m[2100:])
    assert np.array_equal(part[100:2100], got[100:2100])
    # an empty range changes nothing
    same = m.copy()
    _call(same, 3, 7, 7)
    assert np.array_equal(same, m)


@pytest.mark.parametrize("nc", [1, 2])
def test_make_u_smaller_matrices(nc):
    rng = np.random.default_rng(1657 + nc)
    n = 64
    m = rng.standard_normal((n, 2*nc*nc))
    got = m.copy()
    _call(got, nc, 0, n)
    for s in range(n):
        assert np.max(np.abs(got[s] - _gram_schmidt(m[s], nc))) < 1e-14
