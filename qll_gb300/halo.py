"""Domain decomposition of the asqtad operator and CG along the time
direction: the reference's multi-rank path (the lattice split over ranks by
partitionGeom, lib/stagDslash.c:754-801; halo exchange through
lib/shifts.c:7-304 and lib/gather.c; the CG's global sums through gsum and
QMP_sum_double_array, lib/common.c:52-72), for one GPU per rank.

Each rank owns L3/R consecutive time slices.  It holds them in a padded
local lattice of L3/R + 2*PAD slices (PAD = 4, an even number so that the
local checkerboard is the global one; the three-hop Naik term needs 3), a
full periodic lattice to the GPU library, whose links are the global links
of those sites.  Before every half Dslash the PAD slices next to each face
of the input vector are exchanged with the neighbouring ranks; the
library's kernel then runs over the whole padded lattice and its output is
exact on the owned slices (no hop from an owned site reaches past the
halo).  A t-slice of one parity is one contiguous run of sites in the
library layout, so a face is three contiguous copies (one per colour).

Transports: LocalComm runs several ranks in one process (on one GPU, or,
in the tests, on the CPU with the oracle as the operator) with direct
copies between their buffers; DistComm runs one rank per process over
torch.distributed (NCCL between GPUs, gloo between CPU processes), faces by
point-to-point send and receive, global sums by all_reduce.  The CG is cgSolveT's scaled form
(lib/cg.c:77-115) in FP64 with vector updates on the owned sites.
"""
import ctypes

import numpy as np

PAD = 4


def coords_all(dims):
    """coordinates (V, 4) of the sites in the one-lane order (even sites
    first, each parity lexicographic with x0 fastest, halved)"""
    L0, L1, L2, L3 = dims
    V = L0*L1*L2*L3
    idx = np.arange(V)
    par = (idx >= V//2).astype(np.int64)
    i = idx - par*(V//2)
    x0h = i % (L0//2)
    r = i // (L0//2)
    x1 = r % L1
    r = r // L1
    x2 = r % L2
    x3 = r // L2
    x0 = 2*x0h + ((par + x1 + x2 + x3) & 1)
    return np.stack([x0, x1, x2, x3], axis=1)


def site_index(dims, x):
    L0, L1, L2, L3 = dims
    V = L0*L1*L2*L3
    lex = x[:, 0] + L0*(x[:, 1] + L1*(x[:, 2] + L2*x[:, 3]))
    par = (x[:, 0] + x[:, 1] + x[:, 2] + x[:, 3]) & 1
    return par*(V//2) + lex//2


class Slab:
    """rank `rank` of `nranks` along t: its padded lattice and the map from
    its sites to the global ones"""

    def __init__(self, dims, rank, nranks):
        L0, L1, L2, L3 = dims
        if L3 % nranks or (L3//nranks) % 2 or L3//nranks < PAD:
            raise ValueError("t extent %d does not split into %d even slabs of at least %d"
                             % (L3, nranks, PAD))
        self.dims, self.rank, self.nranks = tuple(dims), rank, nranks
        self.lt = L3//nranks
        self.t0 = rank*self.lt
        self.pdims = (L0, L1, L2, self.lt + 2*PAD)
        self.s2 = L0*L1*L2//2                 # sites of one parity in one t-slice
        self.vhp = int(np.prod(self.pdims))//2
        x = coords_all(self.pdims)
        x[:, 3] = (self.t0 - PAD + x[:, 3]) % L3
        self.gidx = site_index(dims, x)       # global site of each padded site
        self.own = slice(PAD*self.s2, (PAD + self.lt)*self.s2)   # owned half-sites

    def local_field(self, f):
        """a global [V][n] field on this rank's padded lattice"""
        return np.ascontiguousarray(f[self.gidx])


# ------------------------------------------------------------- operators
# An operator object holds one rank's padded lattice: zeros() makes a vector
# of one parity, hop(out_parity, out, in) applies the half Dslash, and
# slices/own/dot_own address its t-slices and owned sites.

class GpuOp:
    """the GPU library's FP64 half Dslash on a rank's padded lattice;
    vectors are CUDA tensors [3][Vh][2] (the library layout, one rhs)"""

    def __init__(self, slab, u, u3):
        import torch
        from . import qll
        self.torch = torch
        self.s = slab
        self.L = qll.load()
        self.L.qllg_stag_dslash_device.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                                   ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        # the library's kernels on torch's current stream, in order with the
        # face copies and vector updates made through torch
        self.L.qllg_set_stream(ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        ul = [slab.local_field(a) for a in u]
        u3l = [slab.local_field(a) for a in u3]
        S = self.L.qllg_stag_create(qll.dims_c(slab.pdims), qll.vp_array(ul), qll.vp_array(u3l))
        if not S:
            raise RuntimeError(qll.last_error())
        self.S = ctypes.c_void_p(S)

    def zeros(self):
        return self.torch.zeros((3, self.s.vhp, 2), dtype=self.torch.float64, device="cuda")

    def hop(self, out_parity, out, inp):
        if self.L.qllg_stag_dslash_device(self.S, 0, 1, out_parity, ctypes.c_void_p(out.data_ptr()),
                                          ctypes.c_void_p(inp.data_ptr())):
            from . import qll
            raise RuntimeError(qll.last_error())

    def slices(self, v, a, b):
        return v[:, a*self.s.s2:b*self.s.s2, :]

    def dot_own(self, a, b):
        o = self.s.own
        return float((a[:, o, :]*b[:, o, :]).sum().item())

    def own(self, v):
        return v[:, self.s.own, :]

    def from_host(self, h):
        """[Vh][6] host array of one parity -> library layout"""
        return self.torch.from_numpy(np.ascontiguousarray(
            h.reshape(-1, 3, 2).transpose(1, 0, 2))).cuda()

    def to_host(self, v):
        return v.cpu().numpy().transpose(1, 0, 2).reshape(-1, 6)

    def close(self):
        self.L.qllg_stag_destroy(self.S)


# ------------------------------------------------------------ transports

class LocalComm:
    """all ranks in this process: faces by direct copies"""

    def exchange(self, ops, vecs):
        R = len(ops)
        lt = ops[0].s.lt
        lows = [ops[r].slices(vecs[r], lt, lt + PAD) for r in range(R)]        # top owned slices
        highs = [ops[r].slices(vecs[r], PAD, 2*PAD) for r in range(R)]         # bottom owned slices
        lows = [x.copy() if isinstance(x, np.ndarray) else x.clone() for x in lows]
        highs = [x.copy() if isinstance(x, np.ndarray) else x.clone() for x in highs]
        for r in range(R):
            ops[r].slices(vecs[r], 0, PAD)[...] = lows[(r - 1) % R]
            ops[r].slices(vecs[r], lt + PAD, lt + 2*PAD)[...] = highs[(r + 1) % R]

    def allsum(self, xs):
        return float(sum(xs))


class DistComm:
    """one rank per process over torch.distributed (the process group must
    be initialised: NCCL for GPU tensors, gloo for CPU ones)"""

    def __init__(self):
        import torch.distributed as dist
        self.dist = dist
        self.rank = dist.get_rank()
        self.size = dist.get_world_size()

    def _t(self, x):
        import torch
        return x if isinstance(x, torch.Tensor) else torch.from_numpy(x)

    def exchange(self, ops, vecs):
        import torch
        op, v = ops[0], vecs[0]
        lt = op.s.lt
        dn, up = (self.rank - 1) % self.size, (self.rank + 1) % self.size
        send_up = self._t(op.slices(v, lt, lt + PAD)).contiguous()       # to the rank above
        send_dn = self._t(op.slices(v, PAD, 2*PAD)).contiguous()         # to the rank below
        recv_dn = torch.empty_like(send_up)
        recv_up = torch.empty_like(send_dn)
        reqs = [self.dist.isend(send_up, up, tag=1), self.dist.isend(send_dn, dn, tag=2),
                self.dist.irecv(recv_dn, dn, tag=1), self.dist.irecv(recv_up, up, tag=2)]
        for q in reqs:
            q.wait()
        lo, hi = op.slices(v, 0, PAD), op.slices(v, lt + PAD, lt + 2*PAD)
        if isinstance(v, np.ndarray):
            lo[...] = recv_dn.numpy()
            hi[...] = recv_up.numpy()
        else:
            lo[...] = recv_dn
            hi[...] = recv_up

    def allsum(self, xs):
        import torch
        t = torch.tensor([float(sum(xs))], dtype=torch.float64)
        if self.dist.get_backend() == "nccl":
            t = t.cuda()
        self.dist.all_reduce(t)
        return float(t.item())


# --------------------------------------------------------- Dslash and CG

def hop(comm, ops, out_parity, outs, ins):
    """the decomposed half Dslash: faces of the inputs, then each rank's
    padded-lattice Dslash (exact on its owned sites)"""
    comm.exchange(ops, ins)
    for op, o, i in zip(ops, outs, ins):
        op.hop(out_parity, o, i)


def cg(comm, ops, bs, mass, rsq, maxits):
    """cgSolveT on (m^2 - D_eo D_oe) x = b over the decomposed lattice, FP64,
    vector updates on the owned sites; bs: each rank's even-site source.
    Returns (iterations, per-rank solutions, final |r|^2/|b|^2)."""
    m2 = mass*mass
    xs = [op.zeros() for op in ops]
    ps = [op.zeros() for op in ops]
    vs = [op.zeros() for op in ops]
    ts = [op.zeros() for op in ops]
    rs = []
    for op, b in zip(ops, bs):
        r = op.zeros()
        op.own(r)[...] = op.own(b)
        rs.append(r)
    r2 = comm.allsum([op.dot_own(r, r) for op, r in zip(ops, rs)])
    b2 = r2
    stop = rsq*b2
    its = 0
    while r2 >= stop and its < maxits and b2 > 0:
        its += 1
        beta = 1.0/r2
        for op, p, r in zip(ops, ps, rs):
            op.own(p)[...] += beta*op.own(r)
        hop(comm, ops, 1, vs, ps)
        hop(comm, ops, 0, ts, vs)
        pap = comm.allsum([m2*op.dot_own(p, p) + op.dot_own(v, v)
                           for op, p, v in zip(ops, ps, vs)])
        alpha = 1.0/pap
        for op, x, p, r, t in zip(ops, xs, ps, rs, ts):
            ap = m2*op.own(p) - op.own(t)
            op.own(x)[...] += alpha*op.own(p)
            op.own(r)[...] -= alpha*ap
        r2 = comm.allsum([op.dot_own(r, r) for op, r in zip(ops, rs)])
    return its, xs, (r2/b2 if b2 > 0 else 0.0)
