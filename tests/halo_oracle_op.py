"""The CPU oracle as the per-rank operator of qll_gb300.halo (test
infrastructure): its half Dslash on a rank's padded lattice, vectors as
numpy arrays [Vh][6] of one parity."""
import numpy as np

import oracle_lib as orc


class OracleOp:
    def __init__(self, slab, u, u3):
        self.s = slab
        self.u = [slab.local_field(a) for a in u]
        self.u3 = [slab.local_field(a) for a in u3]

    def zeros(self):
        return np.zeros((self.s.vhp, 6))

    def hop(self, out_parity, out, inp):
        """out = D inp on the output parity (the hop term alone)"""
        full = np.zeros((2*self.s.vhp, 6))
        full[(1 - out_parity)*self.s.vhp:(2 - out_parity)*self.s.vhp] = inp
        res = orc.dslash(self.s.pdims, self.u, self.u3, 0.0, full, "odd" if out_parity else "even")
        out[:] = res[out_parity*self.s.vhp:(out_parity + 1)*self.s.vhp]

    def slices(self, v, a, b):
        return v[a*self.s.s2:b*self.s.s2]

    def dot_own(self, a, b):
        o = self.s.own
        return float(np.sum(a[o]*b[o]))

    def own(self, v):
        return v[self.s.own]
