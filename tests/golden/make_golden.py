"""Generates tests/golden/ref_4x4x4x4.npz: outputs of the reference library
itself (compiled from its sources by oracle/ref_build.py) on seeded inputs
that are stored beside them, so that machines without the reference (the
GPU host) can check against the reference's own numbers.

Lattice 4^4.  Inputs: thin links (eps 0.3, gauge seed 1001, staggered
phases folded in) and Gaussian sources.  Reference outputs:
  fat, long   smearFat7 with the asqtad coefficients (u0 = 1)
  d_<sub>     dslash2 on those links with the negative-adjoint backward
              links -F(x-mu)^dagger, -L(x-3mu)^dagger (minus the
              reference's gaugeDoublestore; not stored: the oracle's
              negadj_back makes them bit for bit), mass 0.25, of source y,
              for the output sites of sub (all, even, odd)
  x_solve2    solve2, mass 0.1, rsq 1e-16, noscale (iterations its_solve2)
  x_multi     solveMulti2, masses 0.1 0.15 0.3, rsq 1e-16, noscale
  w_<sub>     wilsonDslash with links u[2mu] = 1/2 U_mu, u[2mu+1] =
              1/2 U_mu(x-mu)^dagger (the reference's gaugeDoublestore), U the
              thin links above, mass 0.1667, of source yw
Run: python tests/golden/make_golden.py (needs oracle/_ref/libqllref.so and
the GPU library for the input generator)."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import ref_lib as ref          # noqa: E402
from qll_gb300 import qll      # noqa: E402

DIMS = (4, 4, 4, 4)


def main():
    thin = qll.gen_gauge(DIMS, 1001, 0.3, ks=True)
    coef = qll.asqtad_coeffs()
    fat, lng = ref.smear_fat7(DIMS, thin, coef)
    bfat = [-ref.doublestore(DIMS, fat[mu], mu, -1) for mu in range(4)]
    blng = [-ref.doublestore(DIMS, lng[mu], mu, -3) for mu in range(4)]
    u = [a for mu in range(4) for a in (fat[mu], bfat[mu])]
    u3 = [a for mu in range(4) for a in (lng[mu], blng[mu])]
    out = {"dims": np.array(DIMS), "thin": np.array(thin), "fat": np.array(fat),
           "long": np.array(lng)}
    y = qll.gen_source(DIMS, 31, 6, "all")
    out["y"] = y
    for sub in ("all", "even", "odd"):
        out["d_" + sub] = ref.dslash(DIMS, u, u3, 0.25, y, sub)
    b = qll.gen_source(DIMS, 2100, 6, "even")
    out["b"] = b
    its, x = ref.solve2(DIMS, u, u3, 0.1, b, 1e-16, 5000, noscale=1)
    out["x_solve2"], out["its_solve2"] = x, np.array(its)
    masses = [0.1, 0.15, 0.3]
    its, xs = ref.solve_multi2(DIMS, u, u3, masses, b, 1e-16, 5000, noscale=1)
    out["masses"], out["x_multi"], out["its_multi"] = np.array(masses), np.array(xs), np.array(its)
    wu = []
    for mu in range(4):
        wu += [0.5*thin[mu], 0.5*ref.doublestore(DIMS, thin[mu], mu, -1)]
    yw = qll.gen_source(DIMS, 22, 24, "all")
    out["yw"] = yw
    for sub in ("all", "even", "odd"):
        out["w_" + sub] = ref.wilson_dslash(DIMS, wu, 0.1667, yw, sub)
    np.savez_compressed(os.path.join(HERE, "ref_4x4x4x4.npz"), **out)


if __name__ == "__main__":
    main()
