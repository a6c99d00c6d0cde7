"""ctypes access to the reference library compiled by oracle/ref_build.py
(oracle/_ref/libqllref.so, one-lane -DC1 build), for tests.  available()
is False where it was not built (no reference tree and no staged sources)."""
import ctypes
import os
from ctypes import POINTER, c_char_p, c_double, c_float, c_int

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PATH = os.path.join(ROOT, "oracle", "_ref", "libqllref.so")
_L = None
_dims = None


def available():
    return os.path.exists(PATH)


def lib():
    global _L
    if _L is None:
        _L = ctypes.CDLL(PATH)
        for s in "DF":
            getattr(_L, "refh_solve2" + s).restype = c_int
            getattr(_L, "refh_solveMulti2" + s).restype = c_int
    return _L


def setup(dims):
    """the reference's layout and shift tables for dims (both precisions);
    one OpenMP thread, since the reference's smearFat7 races with many
    threads on 4^4 lattices"""
    global _dims
    if _dims != tuple(dims):
        lib().refh_set_threads(1)
        assert lib().refh_setup((c_int*4)(*dims)) == 0
        _dims = tuple(dims)


def _ct(a):
    return c_double if a.dtype == np.float64 else c_float


def _sfx(a):
    return "D" if a.dtype == np.float64 else "F"


def _P(a):
    return a.ctypes.data_as(POINTER(_ct(a)))


def _PA(arrs):
    ct = _ct(arrs[0])
    return (POINTER(ct)*len(arrs))(*[a.ctypes.data_as(POINTER(ct)) for a in arrs])


def dslash(dims, u, u3, mass, y, sub):
    setup(dims)
    x = np.zeros_like(y)
    getattr(lib(), "refh_dslash" + _sfx(y))(_P(x), _PA(u), _PA(u3), c_double(mass), _P(y),
                                            sub.encode())
    return x


def solve2(dims, u, u3, mass, y, rsq, maxits, noscale=0):
    setup(dims)
    x = np.zeros_like(y)
    its = getattr(lib(), "refh_solve2" + _sfx(y))(_P(x), _PA(u), _PA(u3), c_double(mass), _P(y),
                                                  c_double(rsq), maxits, noscale)
    return its, x


def solve_multi2(dims, u, u3, masses, y, rsq, maxits, noscale=0):
    setup(dims)
    xs = [np.zeros_like(y) for _ in masses]
    its = getattr(lib(), "refh_solveMulti2" + _sfx(y))(
        _PA(xs), _PA(u), _PA(u3), (c_double*len(masses))(*masses), len(masses), _P(y),
        c_double(rsq), maxits, noscale)
    return its, xs


def smear_fat7(dims, thin, coef, want_long=True):
    setup(dims)
    fl = [np.zeros_like(thin[0]) for _ in range(4)]
    ll = [np.zeros_like(thin[0]) for _ in range(4)] if want_long else None
    c = (c_double*6)(coef.one_link, coef.three_staple, coef.five_staple, coef.seven_staple,
                     coef.lepage, coef.naik)
    getattr(lib(), "refh_smearFat7" + _sfx(thin[0]))(_PA(fl), _PA(ll) if ll else None, c,
                                                     _PA(list(thin)))
    return fl, ll


def plaq(dims, u):
    setup(dims)
    out = (c_double*6)()
    getattr(lib(), "refh_plaq" + _sfx(u[0]))(out, _PA(list(u)))
    return np.array(out[:])


def wilson_dslash(dims, u, mass, y, sub, sign=1):
    setup(dims)
    x = np.zeros_like(y)
    getattr(lib(), "refh_wilson_dslash" + _sfx(y))(_P(x), _PA(list(u)), c_double(mass), sign,
                                                   _P(y), sub.encode())
    return x


def shift(dims, y, nelem, d, length):
    """the reference's shift: x(s) = y(s + length * sign(d) * e_{|d|-1})"""
    setup(dims)
    x = np.zeros_like(y)
    getattr(lib(), "refh_shift" + _sfx(y))(_P(x), _P(y), nelem, d, length)
    return x


def doublestore(dims, u, mu, length):
    """gaugeDoublestore of one field: the shift by (mu, length), then the
    adjoint of each matrix"""
    setup(dims)
    out = np.zeros_like(u)
    getattr(lib(), "refh_doublestore" + _sfx(u))(_PA([out]), _PA([u]), (c_int*1)(mu),
                                                 (c_int*1)(length), 1)
    return out


def make_u(m, nc=3):
    """the reference's makeU on every site of m ([nsites][2 nc^2] reals), in place"""
    getattr(lib(), "refh_makeU" + _sfx(m))(_P(m), nc, int(m.size//(2*nc*nc)))
    return m
