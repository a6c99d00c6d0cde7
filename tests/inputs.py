"""Seeded test inputs shared by the oracle and the GPU library: thin links
from the library's host generator (KS phases folded in), fat7/asqtad
smearing and negative-adjoint backward links from the CPU oracle."""
import functools

import numpy as np

import oracle_lib as orc
from qll_gb300 import qll


@functools.lru_cache(maxsize=8)
def asqtad_links(dims, seed=1001, eps=0.3):
    """(u, u3): 8 fat and 8 Naik float64 [V,18] arrays in createStaggeredLinks
    order: u[2mu] forward, u[2mu+1] = -F_mu(x-mu)^dagger, and for Naik the
    same with three hops."""
    th = qll.gen_gauge(dims, seed, eps, ks=True)
    fl, ll = orc.smear_fat7(dims, th, qll.asqtad_coeffs())
    u, u3 = [None]*8, [None]*8
    for mu in range(4):
        u[2*mu] = fl[mu]
        u[2*mu+1] = orc.negadj_back(dims, fl[mu], mu, 1)
        u3[2*mu] = ll[mu]
        u3[2*mu+1] = orc.negadj_back(dims, ll[mu], mu, 3)
    return tuple(u), tuple(u3)


def as_dtype(arrs, dtype):
    return [np.ascontiguousarray(a, dtype=dtype) for a in arrs]


def relerr(a, b):
    n = np.linalg.norm(b)
    return np.linalg.norm(a - b)/(n if n > 0 else 1.0)


@functools.lru_cache(maxsize=4)
def wilson_links(dims, seed=1201, eps=0.3, half=True):
    """8 Wilson links: u[2mu] = c U_mu(x), u[2mu+1] = c U_mu(x-mu)^dagger with
    c = 1/2 (the hopping normalisation of the standard Wilson matrix)."""
    th = qll.gen_gauge(dims, seed, eps, ks=False)
    c = 0.5 if half else 1.0
    u = [None]*8
    for mu in range(4):
        u[2*mu] = c*th[mu]
        u[2*mu+1] = c*orc.doublestore(dims, th[mu], mu, -1)
    return tuple(u)
