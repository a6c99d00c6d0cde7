"""ctypes mirror of the C API of libqll_gb300.

The structures below mirror include/layout.h, include/qllP.h,
include/solversP.h and include/qll_gb300.h member for member, so Python code
drives the library through the same entry points a C caller of QLL uses
(stagDslashSetupD, createStaggeredSolverD, solve2D, ...).  Fields are numpy
arrays in the one-lane QLL host layout: float64/float32 of shape
(nSites, nelem), even sites first.
"""
import ctypes
import os
from ctypes import (POINTER, Structure, byref, c_char_p, c_double, c_float, c_int,
                    c_size_t, c_uint, c_ulonglong, c_void_p)

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "libqll_gb300.so")

_lib = None


def load():
    """Load the in-tree libqll_gb300.so; fails loudly when it is not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIBPATH):
        raise RuntimeError("libqll_gb300.so is not built (run __graft_entry__.build())")
    _lib = ctypes.CDLL(LIBPATH)
    _declare(_lib)
    return _lib


# ------------------------------------------------------------ structures
class Layout(Structure):
    _fields_ = [("nDim", c_int), ("physGeom", POINTER(c_int)), ("rankGeom", POINTER(c_int)),
                ("innerGeom", POINTER(c_int)), ("outerGeom", POINTER(c_int)),
                ("localGeom", POINTER(c_int)), ("physVol", c_int), ("nEven", c_int),
                ("nOdd", c_int), ("nSites", c_int), ("nEvenOuter", c_int),
                ("nOddOuter", c_int), ("nSitesOuter", c_int), ("nSitesInner", c_int),
                ("innerCb", c_int), ("innerCbDir", c_int), ("shifts", c_void_p),
                ("nranks", c_int), ("myrank", c_int)]


class LayoutIndex(Structure):
    _fields_ = [("rank", c_int), ("index", c_int)]


class Subset(Structure):
    _fields_ = [("begin", c_int), ("end", c_int), ("beginOuter", c_int), ("endOuter", c_int)]


_IP = POINTER(c_int)


class ShiftIndices(Structure):
    _fields_ = [("gi", c_void_p), ("disp", _IP), ("sidx", _IP), ("pidx", _IP),
                ("nRecvRanks", c_int), ("recvRanks", _IP), ("recvRankSizes", _IP),
                ("recvRankSizes1", _IP), ("recvRankOffsets", _IP), ("recvRankOffsets1", _IP),
                ("nRecvSites", c_int), ("nRecvSites1", c_int), ("nRecvDests", c_int),
                ("recvDests", _IP), ("recvLocalSrcs", _IP), ("recvRemoteSrcs", _IP),
                ("nSendRanks", c_int), ("sendRanks", _IP), ("sendRankSizes", _IP),
                ("sendRankSizes1", _IP), ("sendRankOffsets", _IP), ("sendRankOffsets1", _IP),
                ("nSendSites", c_int), ("nSendSites1", c_int), ("sendSites", _IP),
                ("vv", c_int), ("offr", c_int), ("lenr", c_int), ("nthreads", c_int),
                ("perm", c_int), ("pack", c_int), ("blend", c_int),
                ("sqmpmem", c_void_p), ("smsg", c_void_p), ("rqmpmem", c_void_p),
                ("rmsg", c_void_p), ("pairmsg", c_void_p)]


class ShiftBuf(Structure):
    _fields_ = [("sqmpmem", c_void_p), ("smsg", c_void_p), ("rqmpmem", c_void_p),
                ("rmsg", c_void_p), ("pairmsg", c_void_p), ("sbuf", c_void_p),
                ("rbuf", c_void_p), ("sbufSize", c_int), ("rbufSize", c_int),
                ("first", c_int), ("offr", _IP), ("lenr", _IP)]


class Fat7Coeffs(Structure):
    _fields_ = [("one_link", c_double), ("three_staple", c_double), ("five_staple", c_double),
                ("seven_staple", c_double), ("lepage", c_double), ("naik", c_double)]


def _prec_structs(real):
    class Field(Structure):
        _fields_ = [("l", POINTER(Layout)), ("f", POINTER(real)), ("nelem", c_int)]

    class Transporter(Structure):
        _fields_ = [("u", POINTER(real)), ("si", ShiftIndices), ("nelem", c_int), ("nc", c_int),
                    ("td", c_int), ("sb", ShiftBuf), ("sub", Subset), ("backward", c_int),
                    ("dest", POINTER(real)), ("src", POINTER(real))]

    class StaggeredLinks(Structure):
        _fields_ = [("massFac", c_double), ("t", POINTER(Transporter)), ("n", c_int),
                    ("fb", c_int)]

    class Cgls(Structure):
        _fields_ = [("r1", POINTER(real)), ("r2", POINTER(real)), ("z", POINTER(real)),
                    ("p", POINTER(real)), ("Ap", POINTER(real)), ("Adr2", POINTER(real)),
                    ("nelem", c_int), ("verbose", c_int), ("indent", c_int)]

    class StaggeredSolver(Structure):
        _fields_ = [("sle", StaggeredLinks), ("slo", StaggeredLinks), ("mass", c_double),
                    ("v", POINTER(real)), ("cgls", Cgls), ("its", c_int), ("noscale", c_int),
                    ("flops", c_double), ("secs", c_double), ("sube", Subset), ("subo", Subset)]

    WilsonLinks = type("WilsonLinks", (Structure,), {"_fields_": StaggeredLinks._fields_})

    class WilsonSolver(Structure):
        _fields_ = [("sle", WilsonLinks), ("slo", WilsonLinks), ("mass", c_double),
                    ("v", POINTER(real)), ("cgls", Cgls), ("its", c_int), ("noscale", c_int),
                    ("flops", c_double), ("secs", c_double), ("sube", Subset), ("subo", Subset)]

    return dict(Field=Field, Transporter=Transporter, StaggeredLinks=StaggeredLinks,
                Cgls=Cgls, StaggeredSolver=StaggeredSolver, WilsonLinks=WilsonLinks,
                WilsonSolver=WilsonSolver)


D = _prec_structs(c_double)
F = _prec_structs(c_float)


class SolveInfo(Structure):
    _fields_ = [("iters", c_int*16), ("rsq", c_double*16), ("true_rsq", c_double*16),
                ("reliable_updates", c_int), ("total_iters", c_int), ("seconds", c_double)]


SOLVE_DOUBLE, SOLVE_SINGLE, SOLVE_MIXED_HALF, SOLVE_MIXED_SINGLE = 0, 1, 2, 3


def _declare(L):
    vp, i, d = c_void_p, c_int, c_double
    sig = {
        "qllg_last_error": (c_char_p, []),
        "qllg_clear_error": (None, []),
        "qllg_version": (c_char_p, []),
        "qllg_init": (i, []),
        "qllg_set_stream": (i, [vp]),
        "qllg_get_stream": (vp, []),
        "qllg_gen_gauge": (i, [POINTER(c_int), c_ulonglong, d, i, POINTER(vp)]),
        "qllg_gen_source": (i, [POINTER(c_int), c_ulonglong, i, c_char_p, vp]),
        "qllg_asqtad_coeffs": (None, [POINTER(Fat7Coeffs)]),
        "qllg_stag_create": (vp, [POINTER(c_int), POINTER(vp), POINTER(vp)]),
        "qllg_stag_create_f": (vp, [POINTER(c_int), POINTER(vp), POINTER(vp)]),
        "qllg_stag_destroy": (None, [vp]),
        "qllg_stag_device_bytes": (c_size_t, [vp]),
        "qllg_stag_dslash": (i, [vp, vp, d, vp, c_char_p]),
        "qllg_stag_solve": (i, [vp, i, POINTER(vp), POINTER(vp), POINTER(c_double), d, i, i,
                                POINTER(SolveInfo)]),
        "qllg_stag_solve_device": (i, [vp, i, vp, vp, POINTER(c_double), d, i, i,
                                       POINTER(SolveInfo)]),
        "qllg_stag_vec_alloc": (vp, [vp, i]),
        "qllg_stag_vec_free": (None, [vp]),
        "qllg_stag_vec_upload": (i, [vp, vp, i, POINTER(vp)]),
        "qllg_stag_vec_download": (i, [vp, vp, i, POINTER(vp)]),
        "qllg_stag_nbr_table": (i, [POINTER(c_int), i, i, POINTER(c_int)]),
        "qllg_timing_enable": (None, [i]),
        "qllg_timing_reset": (None, []),
        "qllg_timing_read": (i, [c_char_p, POINTER(c_int), POINTER(c_double)]),
        "layoutSetup": (None, [POINTER(Layout)]),
        "layoutIndex": (None, [POINTER(Layout), POINTER(LayoutIndex), POINTER(c_int)]),
        "layoutCoord": (None, [POINTER(Layout), POINTER(c_int), POINTER(LayoutIndex)]),
        "layoutSubset": (None, [POINTER(Subset), POINTER(Layout), c_char_p]),
        "stagDslashSetupD": (None, [POINTER(Layout), i, POINTER(c_int), POINTER(c_int)]),
        "stagDslashSetupF": (None, [POINTER(Layout), i, POINTER(c_int), POINTER(c_int)]),
        "getShiftD": (POINTER(ShiftIndices), [i, i, c_char_p]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    for P, S, real in (("D", D, c_double), ("F", F, c_float)):
        RP = POINTER(real)
        RPP = POINTER(RP)
        psig = {
            "createStaggeredLinks": (None, [POINTER(S["StaggeredLinks"]), POINTER(Layout), RPP,
                                            RPP, c_char_p]),
            "freeStaggeredLinks": (None, [POINTER(S["StaggeredLinks"])]),
            "dslash2": (None, [POINTER(S["StaggeredLinks"]), RP, real, RP]),
            "createStaggeredSolver": (None, [POINTER(S["StaggeredSolver"]), POINTER(Layout),
                                             RPP, RPP, c_char_p]),
            "freeStaggeredSolver": (None, [POINTER(S["StaggeredSolver"])]),
            "solve2": (c_int, [POINTER(S["StaggeredSolver"]), RP, real, RP, c_double, c_int,
                               c_char_p]),
        }
        for name, (res, args) in psig.items():
            fn = getattr(L, name + P)
            fn.restype = res
            fn.argtypes = args


def last_error():
    return load().qllg_last_error().decode()


# ----------------------------------------------------------- helpers
def ptr(a):
    """ctypes pointer to the data of a contiguous numpy array."""
    assert a.flags["C_CONTIGUOUS"]
    ct = c_double if a.dtype == np.float64 else (c_float if a.dtype == np.float32 else c_int)
    return a.ctypes.data_as(POINTER(ct))


def ptr_array(arrs, ct):
    """array of real* for a list of numpy arrays (None entries give NULL)."""
    P = POINTER(ct)
    out = (P*len(arrs))()
    for k, a in enumerate(arrs):
        out[k] = ptr(a) if a is not None else P()
    return out


def vp_array(arrs):
    out = (c_void_p*len(arrs))()
    for k, a in enumerate(arrs):
        out[k] = a.ctypes.data if a is not None else None
    return out


def dims_c(dims):
    return (c_int*4)(*dims)


def setup_layout(dims, prec="D"):
    """stagDslashSetup for one rank; returns the Layout (keep it alive)."""
    L = load()
    lay = Layout()
    lay.nranks = 1
    lay.myrank = 0
    getattr(L, "stagDslashSetup" + prec)(byref(lay), 4, dims_c(dims), None)
    if lay.nSites == 0:
        raise RuntimeError("stagDslashSetup failed: " + last_error())
    return lay


def gen_gauge(dims, seed, eps, ks=True):
    """four [V,18] float64 SU(3) link fields (KS phases folded in when ks)."""
    L = load()
    V = int(np.prod(dims))
    u = [np.zeros((V, 18)) for _ in range(4)]
    rc = L.qllg_gen_gauge(dims_c(dims), seed, eps, int(ks), vp_array(u))
    if rc:
        raise RuntimeError(last_error())
    return u


def gen_source(dims, seed, nelem=6, sub="even"):
    L = load()
    V = int(np.prod(dims))
    v = np.zeros((V, nelem))
    if L.qllg_gen_source(dims_c(dims), seed, nelem, sub.encode(), v.ctypes.data):
        raise RuntimeError(last_error())
    return v


def asqtad_coeffs():
    c = Fat7Coeffs()
    load().qllg_asqtad_coeffs(byref(c))
    return c
