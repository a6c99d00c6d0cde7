"""The time-direction domain decomposition (qll_gb300.halo): faces
exchanged between ranks, each rank's padded-lattice Dslash, global sums.

CPU: the oracle as each rank's operator, ranks in one process (1, 2 and 4
of them) and two gloo processes: the decomposed half Dslash equals the
global one bit for bit on every owned site (the same arithmetic per site),
and the decomposed CG takes the global CG's iterations (within 1: the sums
are folded in another order) with solutions within 1e-10.
GPU: two ranks on one GPU (in-process transport, the library's kernels):
the decomposed Dslash bitwise equal to the global GPU Dslash, the CG
against the library's global FP64 solve.  The multi-GPU transport (NCCL) is
the gloo test's code path with GPU tensors; this run has one GPU, so it is
not measured on hardware."""
import os
import socket

import numpy as np
import pytest

import oracle_lib as orc
from halo_oracle_op import OracleOp
from inputs import asqtad_links, relerr
from qll_gb300 import halo, qll

DIMS = (4, 4, 4, 16)
MASS = 0.1


def _global(dims=DIMS):
    u, u3 = asqtad_links(dims)
    return list(u), list(u3)


def _owned_rows(slab, parity):
    """global half-site indices (within a parity) of a rank's owned sites"""
    Vh = int(np.prod(slab.dims))//2
    rows = slab.gidx[parity*slab.vhp:(parity + 1)*slab.vhp][slab.own]
    return rows - parity*Vh


@pytest.mark.parametrize("nranks", [1, 2, 4])
def test_decomposed_dslash_and_cg_in_process(nranks):
    u, u3 = _global()
    Vh = int(np.prod(DIMS))//2
    slabs = [halo.Slab(DIMS, r, nranks) for r in range(nranks)]
    ops = [OracleOp(s, u, u3) for s in slabs]
    comm = halo.LocalComm()
    # the half Dslash D_oe of an even vector
    y = qll.gen_source(DIMS, 31, 6, "even")
    want = orc.dslash(DIMS, u, u3, 0.0, y, "odd")[Vh:]
    ins = [op.zeros() for op in ops]
    for s, v in zip(slabs, ins):
        v[s.own] = y[:Vh][_owned_rows(s, 0)]
    outs = [op.zeros() for op in ops]
    halo.hop(comm, ops, 1, outs, ins)
    for s, o in zip(slabs, outs):
        assert np.array_equal(o[s.own], want[_owned_rows(s, 1)])
    # the CG
    b = qll.gen_source(DIMS, 2100, 6, "even")
    bs = []
    for s, op in zip(slabs, ops):
        v = op.zeros()
        v[s.own] = b[:Vh][_owned_rows(s, 0)]
        bs.append(v)
    its, xs, rr = halo.cg(comm, ops, bs, MASS, 1e-16, 5000)
    its_o, xo, _ = orc.solve2(DIMS, u, u3, MASS, b, 1e-16, 5000, noscale=1)
    assert abs(its - its_o) <= 1, (its, its_o)
    assert rr < 1e-16
    x = np.zeros((Vh, 6))
    for s, v in zip(slabs, xs):
        x[_owned_rows(s, 0)] = v[s.own]
    assert relerr(x, xo[:Vh]) < 1e-10


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        u, u3 = _global()
        Vh = int(np.prod(DIMS))//2
        slab = halo.Slab(DIMS, rank, world)
        op = OracleOp(slab, u, u3)
        comm = halo.DistComm()
        y = qll.gen_source(DIMS, 31, 6, "even")
        v = op.zeros()
        v[slab.own] = y[:Vh][_owned_rows(slab, 0)]
        o = op.zeros()
        halo.hop(comm, [op], 1, [o], [v])
        want = orc.dslash(DIMS, u, u3, 0.0, y, "odd")[Vh:]
        ok_dslash = bool(np.array_equal(o[slab.own], want[_owned_rows(slab, 1)]))
        b = qll.gen_source(DIMS, 2100, 6, "even")
        bv = op.zeros()
        bv[slab.own] = b[:Vh][_owned_rows(slab, 0)]
        its, xs, rr = halo.cg(comm, [op], [bv], MASS, 1e-16, 5000)
        its_o, xo, _ = orc.solve2(DIMS, u, u3, MASS, b, 1e-16, 5000, noscale=1)
        mine = xo[:Vh][_owned_rows(slab, 0)]
        err = float(np.linalg.norm(xs[0][slab.own] - mine))
        q.put((rank, ok_dslash, its, its_o, rr, err, float(np.linalg.norm(mine))))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_decomposed_dslash_and_cg_over_gloo():
    """two processes, one rank each, faces and sums over gloo"""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    err2 = sum(r[5]**2 for r in res)
    nrm2 = sum(r[6]**2 for r in res)
    for rank, ok_dslash, its, its_o, rr, _, _ in res:
        assert ok_dslash, rank
        assert abs(its - its_o) <= 1, (rank, its, its_o)
        assert rr < 1e-16
    assert np.sqrt(err2/nrm2) < 1e-10


@pytest.mark.gpu
def test_decomposed_on_one_gpu_matches_global():
    torch = pytest.importorskip("torch")
    import ctypes
    dims = (8, 8, 8, 16)
    u, u3 = _global(dims)
    Vh = int(np.prod(dims))//2
    L = qll.load()
    L.qllg_stag_dslash_device.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    G = ctypes.c_void_p(L.qllg_stag_create(qll.dims_c(dims), qll.vp_array(u), qll.vp_array(u3)))
    assert G.value, qll.last_error()
    slabs = [halo.Slab(dims, r, 2) for r in range(2)]
    ops = [halo.GpuOp(s, u, u3) for s in slabs]
    comm = halo.LocalComm()
    try:
        y = qll.gen_source(dims, 31, 6, "even")[:Vh]
        yg = ops[0].from_host(y)                       # the global vector, library layout
        og = torch.zeros_like(yg)
        assert L.qllg_stag_dslash_device(G, 0, 1, 1, ctypes.c_void_p(og.data_ptr()),
                                         ctypes.c_void_p(yg.data_ptr())) == 0
        torch.cuda.synchronize()
        want = ops[0].to_host(og)
        ins = []
        for s, op in zip(slabs, ops):
            h = np.zeros((s.vhp, 6))
            h[s.own] = y[_owned_rows(s, 0)]
            ins.append(op.from_host(h))
        outs = [op.zeros() for op in ops]
        halo.hop(comm, ops, 1, outs, ins)
        torch.cuda.synchronize()
        for s, op, o in zip(slabs, ops, outs):
            assert np.array_equal(op.to_host(o)[s.own], want[_owned_rows(s, 1)])
        b = qll.gen_source(dims, 2100, 6, "even")
        bs = []
        for s, op in zip(slabs, ops):
            h = np.zeros((s.vhp, 6))
            h[s.own] = b[:Vh][_owned_rows(s, 0)]
            bs.append(op.from_host(h))
        its, xs, rr = halo.cg(comm, ops, bs, MASS, 1e-16, 5000)
        x = np.zeros((Vh, 6))
        for s, op, v in zip(slabs, ops, xs):
            x[_owned_rows(s, 0)] = op.to_host(v)[s.own]
        its_o, xo, _ = orc.solve2(dims, u, u3, MASS, b, 1e-16, 5000, noscale=1)
        assert abs(its - its_o) <= 1, (its, its_o)
        assert rr < 1e-16
        assert relerr(x, xo[:Vh]) < 1e-10
    finally:
        for op in ops:
            op.close()
        L.qllg_stag_destroy(G)
