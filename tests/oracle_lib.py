"""ctypes access to the CPU oracle (oracle/_build/liboracle.so) for tests."""
import ctypes
import os
from ctypes import POINTER, c_char_p, c_double, c_float, c_int

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
_L = None


class OrFat7(ctypes.Structure):
    _fields_ = [(n, c_double) for n in ("one_link", "three_staple", "five_staple",
                                         "seven_staple", "lepage", "naik")]


def lib():
    global _L
    if _L is None:
        _L = ctypes.CDLL(os.path.join(ROOT, "oracle", "_build", "liboracle.so"))
        _L.or_stress_kat.restype = c_double
        _L.or_fieldtest_kat.restype = c_double
        for S in "DF":
            getattr(_L, "or_dslashp2" + S).restype = c_double
            getattr(_L, "or_norm2" + S).restype = c_double
    return _L


def dims_c(dims):
    return (c_int*4)(*dims)


def _ct(a):
    return c_double if a.dtype == np.float64 else c_float


def P(a):
    return a.ctypes.data_as(POINTER(_ct(a)))


def PA(arrs, ct):
    arr = (POINTER(ct)*len(arrs))()
    for i, a in enumerate(arrs):
        arr[i] = a.ctypes.data_as(POINTER(ct)) if a is not None else POINTER(ct)()
    return arr


def sfx(a):
    return "D" if a.dtype == np.float64 else "F"


def realtype(dtype):
    return c_double if dtype == np.float64 else c_float


def dslash(dims, u, u3, mass, y, sub):
    s = sfx(y)
    ct = realtype(y.dtype)
    x = np.zeros_like(y)
    getattr(lib(), "or_dslash" + s)(dims_c(dims), P(x), PA(u, ct),
                                    PA(u3, ct) if u3 is not None else None,
                                    ct(mass), P(y), sub.encode())
    return x


def solve2(dims, u, u3, mass, y, rsq, maxits, noscale=0):
    s = sfx(y)
    ct = realtype(y.dtype)
    x = np.zeros_like(y)
    fr = c_double()
    its = getattr(lib(), "or_solve2" + s)(dims_c(dims), P(x), PA(u, ct), PA(u3, ct),
                                          ct(mass), P(y), c_double(rsq), maxits, noscale,
                                          ctypes.byref(fr))
    return its, x, fr.value


def solve_multi2(dims, u, u3, masses, y, rsq, maxits, noscale=0):
    s = sfx(y)
    ct = realtype(y.dtype)
    xs = [np.zeros_like(y) for _ in masses]
    m = (c_double*len(masses))(*masses)
    its = getattr(lib(), "or_solveMulti2" + s)(dims_c(dims), PA(xs, ct), PA(u, ct), PA(u3, ct),
                                               m, len(masses), P(y), c_double(rsq), maxits,
                                               noscale)
    return its, xs


def dslashp2(dims, u, u3, mass, x):
    s = sfx(x)
    ct = realtype(x.dtype)
    Ax = np.zeros_like(x)
    v = np.zeros_like(x)
    pAp = getattr(lib(), "or_dslashp2" + s)(dims_c(dims), P(Ax), P(x), PA(u, ct), PA(u3, ct),
                                            c_double(mass), P(v))
    return Ax, pAp


def smear_fat7(dims, u, coef, want_long=True):
    s = sfx(u[0])
    ct = realtype(u[0].dtype)
    fl = [np.zeros_like(u[0]) for _ in range(4)]
    ll = [np.zeros_like(u[0]) for _ in range(4)] if want_long else None
    c = OrFat7(coef.one_link, coef.three_staple, coef.five_staple, coef.seven_staple,
               coef.lepage, coef.naik)
    getattr(lib(), "or_smearFat7" + s)(dims_c(dims), PA(fl, ct),
                                       PA(ll, ct) if ll is not None else None,
                                       ctypes.byref(c), PA(u, ct), PA(u, ct))
    return fl, ll


def negadj_back(dims, u, mu, length):
    s = sfx(u)
    out = np.zeros_like(u)
    getattr(lib(), "or_negadj_back" + s)(dims_c(dims), P(out), P(u), mu, length)
    return out


def doublestore(dims, u, mu, length):
    s = sfx(u)
    out = np.zeros_like(u)
    getattr(lib(), "or_doublestore" + s)(dims_c(dims), P(out), P(u), mu, length)
    return out


def plaq(dims, u):
    s = sfx(u[0])
    out = (c_double*6)()
    getattr(lib(), "or_plaq" + s)(dims_c(dims), out, PA(u, realtype(u[0].dtype)))
    return np.array(out[:])


def shift_table(dims, disp, parity):
    V = int(np.prod(dims))
    t = np.zeros(V, dtype=np.int32)
    lib().or_shift_table(dims_c(dims), (c_int*4)(*disp), parity,
                         t.ctypes.data_as(POINTER(c_int)))
    return t


def stag_slot_table(dims, slot, naik, parity):
    V = int(np.prod(dims))
    t = np.zeros(V, dtype=np.int32)
    lib().or_stag_slot_table(dims_c(dims), slot, naik, parity, t.ctypes.data_as(POINTER(c_int)))
    return t


def site_coord(dims, idx):
    x = (c_int*4)()
    lib().or_site_coord(dims_c(dims), idx, x)
    return tuple(x)


def site_index(dims, x):
    return lib().or_site_index(dims_c(dims), (c_int*4)(*x))


def wilson_dslash(dims, u, mass, y, sub):
    s = sfx(y)
    ct = realtype(y.dtype)
    x = np.zeros_like(y)
    getattr(lib(), "or_wilson_dslash" + s)(dims_c(dims), P(x), PA(u, ct), ct(mass), 1, P(y),
                                           sub.encode())
    return x


def wilson_cgnr(dims, u, mass, b, rsq, maxits):
    s = sfx(b)
    x = np.zeros_like(b)
    fr = c_double()
    its = getattr(lib(), "or_wilson_cgnr" + s)(dims_c(dims), P(x), PA(u, realtype(b.dtype)),
                                               c_double(mass), P(b), c_double(rsq), maxits,
                                               ctypes.byref(fr))
    return its, x, fr.value


def wilson_schur(dims, u, mass, y, dag):
    s = sfx(y)
    out = np.zeros_like(y)
    tmp = np.zeros_like(y)
    getattr(lib(), "or_wilson_schur" + s)(dims_c(dims), P(out), PA(u, realtype(y.dtype)),
                                          c_double(mass), P(y), dag, P(tmp))
    return out


def wilson_solve_ref(dims, u, mass, b, rsq, maxits, noscale=0):
    s = sfx(b)
    ct = realtype(b.dtype)
    x = np.zeros_like(b)
    its = getattr(lib(), "or_wilson_solve" + s)(dims_c(dims), P(x), PA(u, ct), ct(mass), P(b),
                                                c_double(rsq), maxits, noscale)
    return its, x


def transport(dims, dest, u, src, nelem, mu, fwd):
    s = sfx(src)
    getattr(lib(), "or_transport" + s)(dims_c(dims), P(dest), P(u), P(src), nelem, mu, fwd)
    return dest


def shift(dims, y, nelem, d, length):
    s = sfx(y)
    x = np.zeros_like(y)
    getattr(lib(), "or_shift" + s)(dims_c(dims), P(x), P(y), nelem, d, length)
    return x


def gamma(d):
    g = (c_double*32)()
    lib().or_gamma(d, g)
    a = np.array(g[:]).reshape(4, 4, 2)
    return a[..., 0] + 1j*a[..., 1]


def make_u(m):
    """or_makeU (lib/vla.c:1635-1665) in place on [nsites][18] reals"""
    s = "D" if m.dtype == np.float64 else "F"
    getattr(lib(), "or_makeU" + s)(P(m), int(m.size//18))
    return m
