"""Benchmark of the asqtad CG hot path on GB300.

Workload (the configuration the headline metric is quoted on): 32^3 x 64
lattice, SU(3) links exp(i 0.4 H) with staggered phases, fat7/asqtad
smearing on the GPU, m = 0.01, a block of 16 Gaussian sources solved
together to |r|^2 < 1e-16 |b|^2 (true residual 1e-8) by the mixed-precision
CG: FP32 Krylov vectors and links in the sloppy iterations, FP64 reliable
updates (true residual recomputed from the FP64 operator, solution
accumulated in FP64), multi-rhs Dslash reusing each link load across the 16
sources.  A step is one such 16-source solve; value = solves per second.
The 16-bit-storage mode (per-site scale) is also run once and reported: at
m = 0.01 its quantisation noise swamps the low modes and it needs about 3x
the iterations, so FP32 sloppy storage is the faster choice here.

--impl reference times the reference's own FP64 solve2 on the host CPU
cores: the reference library compiled from its sources (oracle/_ref, its
4-site SIMD layout, host-native flags), or, where it was not built, the CPU
oracle's C restatement of it; one converged solve of one source per step,
on inputs made on the host without loading the GPU library.

Run: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
For N > 1 each rank solves its own block (replicas; no collective in the
data path); the timed region is bracketed by a barrier and the max over
ranks is reported.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

DIMS = (32, 32, 32, 64)
EPS = 0.4
MASS = 0.01
NRHS = 16
RSQ = 1e-16
MAXITS = 20000
SEED_GAUGE = 1004
SEED_SRC = 2400
WORKLOAD = "asqtad_cg_32^3x64_m0.01_eps0.4_16rhs_mixed_fp32_fp64_tol1e-8"
METRIC = "mixed-precision multi-RHS asqtad CG solves/s at 1e-8 true residual"
# the workload's description, identical in both arms
CONFIG = {"workload": WORKLOAD, "lattice": list(DIMS), "mass": MASS, "eps": EPS, "nrhs": NRHS,
          "tol_true_residual": 1e-8, "parallelism": "replicas (one process per GPU, no collective)",
          "l2": "inputs larger than L2 (links 2.4 GB FP32 + 4.8 GB FP64)"}
# DRAM bytes (read + write) per even site of one 16-rhs FP32 half Dslash
# (the autotuned launch shape, the per-warp cp.async pipeline with 4
# stages), ncu capture at 24^3x48: 531.2 MB + 112.1 MB over 331,776 sites
TRAFFIC_PER_SITE_BYTES = (531.186176e6 + 112.13824e6)/331776


def apply_params(L, args):
    """library parameters given as --param name=value"""
    from qll_gb300 import qll
    L.qllg_set_param.argtypes = [ctypes.c_char_p, ctypes.c_double]
    for kv in args.param:
        k, v = kv.split("=")
        if L.qllg_set_param(k.encode(), float(v)) != 0:
            raise SystemExit(qll.last_error())


def tuned_choice(L):
    """the launch shape the autotuner chose for the 16-rhs FP32 half Dslash
    of the headline lattice (plain launch)"""
    key = "stag_dslash p1/1 s16 n16 V%d (%d %d %d %d)" % ((int(np.prod(DIMS)),) + tuple(DIMS))
    for line in autotune_report(L):
        if line.startswith(key + ":"):
            return line[len(key) + 1:].split("|")[0].strip()
    return "untuned"


def autotune_report(L):
    """the Dslash variant the autotuner chose per launch shape, with times"""
    buf = ctypes.create_string_buffer(16384)
    L.qllg_autotune_report.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
    L.qllg_autotune_report(buf, len(buf))
    return [ln for ln in buf.value.decode().splitlines() if ln]


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x, ws, device="cuda"):
    """the largest x over the ranks of the job (the slowest rank's time)"""
    if ws == 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_seeds(rank):
    """gauge and source seeds of one replica: every rank solves its own
    configuration and sources (replicas, no collective in the data path)"""
    return SEED_GAUGE + 17*rank, SEED_SRC + 100*rank


class Clocks:
    """nvidia-smi sampling of SM clock and throttle reasons during a region"""

    def __init__(self, out):
        self.out = out
        self.p = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.out, "w")
            self.p = subprocess.Popen(["nvidia-smi", "--query-gpu=" + q, "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()
            self.f.close()

    def summary(self, gpu_index=0):
        try:
            rows = [r.split(",") for r in open(self.out).read().strip().splitlines()]
        except OSError:
            return None
        rows = [[c.strip() for c in r] for r in rows if len(r) >= 9]
        rows = [r for r in rows if r[0] == str(gpu_index)] or rows
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return {}


# ------------------------------------------------------------- GPU arm
def run_gpu(args):
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from qll_gb300 import qll
    L = qll.load()
    L.qllg_stag_create_asqtad.restype = ctypes.c_void_p
    L.qllg_stag_create_asqtad.argtypes = [ctypes.POINTER(ctypes.c_int),
                                          ctypes.POINTER(ctypes.c_void_p),
                                          ctypes.POINTER(qll.Fat7Coeffs)]
    L.qllg_launch_count.restype = ctypes.c_ulonglong
    L.qllg_stag_get_links.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]
    L.qllg_stag_device_bytes.restype = ctypes.c_size_t
    stream = torch.cuda.current_stream()
    L.qllg_set_stream(ctypes.c_void_p(stream.cuda_stream))
    apply_params(L, args)

    t0 = time.time()
    seed_gauge, seed_src = replica_seeds(rank)
    thin = qll.gen_gauge(DIMS, seed_gauge, EPS, ks=True)
    coef = qll.asqtad_coeffs()
    S = L.qllg_stag_create_asqtad(qll.dims_c(DIMS), qll.vp_array(thin), ctypes.byref(coef))
    if not S:
        raise RuntimeError(qll.last_error())
    S = ctypes.c_void_p(S)
    del thin
    srcs = [qll.gen_source(DIMS, seed_src + r, 6, "even") for r in range(NRHS)]
    xs = [np.zeros_like(srcs[0]) for _ in range(NRHS)]
    masses = (ctypes.c_double*NRHS)(*([MASS]*NRHS))
    b_dev = L.qllg_stag_vec_alloc(S, NRHS)
    x_dev = L.qllg_stag_vec_alloc(S, NRHS)
    if L.qllg_stag_vec_upload(S, b_dev, NRHS, qll.vp_array(srcs)):
        raise RuntimeError(qll.last_error())
    log("setup %.1fs (gauge, GPU fat7, sources)" % (time.time() - t0))

    info = qll.SolveInfo()

    def solve(mode=qll.SOLVE_MIXED_SINGLE, nrhs=NRHS, x=x_dev, b=b_dev, rsq=RSQ):
        its = L.qllg_stag_solve_device(S, nrhs, x, b, masses, rsq, MAXITS, mode,
                                       ctypes.byref(info))
        if its < 0:
            raise RuntimeError(qll.last_error())
        return its

    # plain FP64 single-rhs GPU CG: the comparison the target is stated on
    b1 = L.qllg_stag_vec_alloc(S, 1)
    x1 = L.qllg_stag_vec_alloc(S, 1)
    L.qllg_stag_vec_upload(S, b1, 1, qll.vp_array(srcs[:1]))
    torch.cuda.synchronize()
    t1 = time.time()
    its64 = solve(qll.SOLVE_DOUBLE, 1, x1, b1)
    torch.cuda.synchronize()
    fp64_s = time.time() - t1
    fp64_true = info.true_rsq[0]
    log("FP64 single-rhs CG: %d iterations, %.3fs, true rsq %.2e" % (its64, fp64_s, fp64_true))

    for _ in range(args.warmup):
        solve()
    torch.cuda.synchronize()
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    # the timed region runs the production path: each solve's iterations are
    # one CUDA-graph launch (per-kernel event timing is off, it would force
    # the host-polled loop); the kernel counter includes the kernels the
    # graph trips ran
    n0 = L.qllg_launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    iters, truer = [], []
    with Clocks(os.path.join(os.environ.get("QLLG_CLOCKS_DIR", "/tmp"),
                             "bench_clocks_r%d.csv" % rank)) as clk:
        torch.cuda.nvtx.range_push("timed")
        ev0.record(stream)
        for _ in range(args.steps):
            iters.append(solve())
            truer.append(max(info.true_rsq[r] for r in range(NRHS)))
        ev1.record(stream)
        torch.cuda.nvtx.range_pop()
        torch.cuda.synchronize()
    nlaunch = int(L.qllg_launch_count() - n0)
    ms = ev0.elapsed_time(ev1)
    # one more solve, untimed, with per-kernel CUDA events on the library
    # stream: the average launch times of the roofline
    L.qllg_timing_enable(1)
    L.qllg_timing_reset()
    its_timed = solve()
    torch.cuda.synchronize()
    cnt, tot = ctypes.c_int(), ctypes.c_double()
    L.qllg_timing_read(b"stag_dslash_f32_n16", ctypes.byref(cnt), ctypes.byref(tot))
    fcnt, ftot = ctypes.c_int(), ctypes.c_double()
    L.qllg_timing_read(b"stag_cg_fused_f32_n16", ctypes.byref(fcnt), ctypes.byref(ftot))
    L.qllg_timing_enable(0)
    t_max = max_over_ranks(ms, ws)
    value = ws*NRHS*args.steps/(t_max*1e-3)

    # end to end through the host-array API: H2D of the sources and D2H of
    # the solutions are inside the timed region; the host arrays are in
    # pinned (page-locked) memory
    def pinned(a):
        t = torch.empty(a.size, dtype=torch.float64, pin_memory=True).numpy()
        t[:] = a.reshape(-1)
        return t
    srcs_p = [pinned(s) for s in srcs]
    xs_p = [pinned(x) for x in xs]
    e2e_steps = max(1, min(args.steps, 3))
    # one untimed warm-up through the same call (its device buffers differ
    # from the device-API solves above, so it captures its own solver graph)
    if L.qllg_stag_solve(S, NRHS, qll.vp_array(xs_p), qll.vp_array(srcs_p), masses, RSQ,
                         MAXITS, qll.SOLVE_MIXED_SINGLE, ctypes.byref(info)) < 0:
        raise RuntimeError(qll.last_error())
    torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    te = time.time()
    for _ in range(e2e_steps):
        its = L.qllg_stag_solve(S, NRHS, qll.vp_array(xs_p), qll.vp_array(srcs_p), masses, RSQ,
                                MAXITS, qll.SOLVE_MIXED_SINGLE, ctypes.byref(info))
        if its < 0:
            raise RuntimeError(qll.last_error())
    torch.cuda.synchronize()
    te = max_over_ranks(time.time() - te, ws)
    e2e = ws*NRHS*e2e_steps/te
    Vh = srcs[0].shape[0]//2
    bytes_io = NRHS*Vh*6*8

    # roofline of the dominant kernel: the 16-rhs FP32 asqtad half-Dslash
    # (D_oe p).  Algorithmic bytes per output site and rhs (the lattice
    # convention: 16 neighbour spinor loads + 1 store, links shared by the
    # 16 rhs; Naik links 12 reals with reconstruct-12, else 18):
    # (8*18*4 + 8*naik*4)/16 + 17*(6*4) = 480 B (18) or 468 B (12)
    L.qllg_stag_recon12.argtypes = [ctypes.c_void_p]
    recon = bool(L.qllg_stag_recon12(S))
    naik = 12 if recon else 18
    per_site_rhs = (8*18*4 + 8*naik*4)/16 + 17*(6*4)
    launch_bytes = per_site_rhs*Vh*NRHS
    # the host-polled loop of the timing solve issues its iterations in
    # growing batches and checks for convergence between batches, so the last
    # batch can hold launches after the final iteration, which return at once
    # (the done flag): the per-launch time is the total over the launches
    # that did work, one per iteration (the idle ones add microseconds)
    work = min(cnt.value, its_timed)
    avg_ms = tot.value/max(work, 1)
    achieved = launch_bytes/(avg_ms*1e-3)/1e9
    pk = peaks()
    peak = pk.get("hbm_gbs")
    compulsory = (8*18*4 + 8*naik*4)/16 + 2*(6*4)
    achieved_dram = compulsory*Vh*NRHS/(avg_ms*1e-3)/1e9
    # the fused D_eo + CG update: links + 16 neighbours + self + x and r
    # read and written
    fused_bytes = ((8*18*4 + 8*naik*4)/16 + 17*(6*4) + 4*(6*4))*Vh*NRHS
    # its compulsory DRAM bytes: links, v in, p (self) in, x and r in and out
    fused_compulsory = ((8*18*4 + 8*naik*4)/16 + 6*(6*4))*Vh*NRHS
    favg = ftot.value/max(min(fcnt.value, its_timed), 1)

    # the 16-bit-storage mode, once (not timed in the headline)
    t_h = time.time()
    its_half = solve(qll.SOLVE_MIXED_HALF)
    torch.cuda.synchronize()
    t_h = time.time() - t_h

    # the same 16-rhs mixed solve to true residual 1e-10 (|r|^2 < 1e-20 |b|^2),
    # the tighter tolerance of the same workload, once
    t_t = time.time()
    its_tight = solve(rsq=1e-20)
    torch.cuda.synchronize()
    t_t = time.time() - t_t
    tight_true = max(info.true_rsq[r] for r in range(NRHS))

    out = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_max/args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32 (sloppy vectors and links) / fp64 (reliable updates, solution)",
        "data": "synthetic (seeded SU(3) gauge, fat7 on GPU, Gaussian sources)",
        "config": CONFIG,
        "iters_per_solve": iters, "max_true_rsq": max(truer),
        "mixed_16bit_storage": {"solves_per_s": ws*NRHS/t_h, "iters": its_half,
                                "note": "16-bit Krylov vectors with per-site scale; slower at m=0.01"},
        "tol_1e-10": {"solves_per_s": ws*NRHS/t_t, "iters": its_tight, "max_true_rsq": tight_true,
                      "note": "the same mixed 16-rhs solve to true residual 1e-10, once, untimed by events"},
        "fp64_single_rhs": {"solves_per_s": 1/fp64_s, "iters": its64, "true_rsq": fp64_true,
                            "speedup_of_value": value/ws*fp64_s},
        "e2e": {"value": e2e, "unit": "solves/s", "h2d_bytes_per_step": bytes_io,
                "d2h_bytes_per_step": bytes_io, "host_memory": "pinned",
                "api": "qllg_stag_solve (host arrays)"},
        "fused_cg_kernel": {"avg_launch_ms": favg, "launches": fcnt.value,
                            "gbs": fused_bytes/(favg*1e-3)/1e9 if favg > 0 else None,
                            "compulsory_gbs": fused_compulsory/(favg*1e-3)/1e9 if favg > 0 else None,
                            "frac_of_hbm": (fused_compulsory/(favg*1e-3)/1e9/peak) if (favg > 0 and peak) else None,
                            "basis": "compulsory DRAM bytes per launch: links, v, p (the mass term), x and r "
                                     "read, x and r written (216 B per site and rhs)"},
        "roofline": {"kernel": "stag_dslash_mr<f32,%s,16 slots,16 rhs>, %s"
                               % ("f32 reconstruct-12" if recon else "f32", tuned_choice(L)),
                     "bound": "hbm",
                     "achieved": achieved_dram, "peak": peak, "unit": "GB/s",
                     "frac": achieved_dram/peak if peak else None,
                     "basis": "compulsory DRAM bytes per launch: the links (shared by the 16 rhs) "
                              "plus one load and one store of each spinor (%.0f B per site and "
                              "rhs), over the event-timed launch duration" % compulsory,
                     "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if peak else None,
                     "bytes_per_launch": compulsory*Vh*NRHS,
                     "avg_launch_ms": avg_ms, "launches_event_timed": cnt.value,
                     "launches_with_work": work,
                     "timing_note": "avg launch time from CUDA events over one extra 16-rhs solve after the timed "
                                    "region: total event time over the launches that did work (one per iteration; "
                                    "the launches after convergence return at once)",
                     # dram read+write of one launch from an ncu capture at
                     # 24^3x48, scaled by sites to this lattice
                     "traffic": TRAFFIC_PER_SITE_BYTES*Vh,
                     "traffic_source": "ncu dram__bytes_read+write of one launch at 24^3x48, "
                                       "scaled by sites (captured separately; not measured in this run)",
                     "lattice_convention": {
                         "gbs": achieved, "bytes_per_launch": launch_bytes,
                         "note": "16 neighbour spinor loads + 1 store per site and rhs, links "
                                 "shared by the 16 rhs (%.0f B): neighbour reuse through L1/L2 "
                                 "is what lets this figure exceed the HBM peak" % per_site_rhs}},
        "autotune": autotune_report(L),
        "gpu_launches": nlaunch,
        "clocks": clk.summary(local),
        "device_bytes": int(L.qllg_stag_device_bytes(S)),
    }
    if rank == 0 and not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(L, S)
    L.qllg_stag_vec_free(b_dev)
    L.qllg_stag_vec_free(x_dev)
    L.qllg_stag_vec_free(b1)
    L.qllg_stag_vec_free(x1)
    L.qllg_stag_destroy(S)
    if rank == 0 and not args.no_serve:
        ts = time.time()
        out["c1"] = run_c1(args)
        out["wilson"] = run_wilson(args)
        out["multishift"] = run_multishift(args)
        out["serving"] = run_serving(args)
        log("multishift and serving %.1fs" % (time.time() - ts))
    if rank == 0:
        print(json.dumps(out), flush=True)
    if ws > 1:
        dist.destroy_process_group()


# ---------------------------------------------------------------- Wilson
def site_index(dims, x):
    """QLL's one-lane site index (layoutIndex): even sites first, each parity
    lexicographic with x0 fastest, halved"""
    L0, L1, L2, _ = dims
    lex = x[0] + L0*(x[1] + L1*(x[2] + L2*x[3]))
    par = (x[0] + x[1] + x[2] + x[3]) % 2
    return lex//2 + par*(int(np.prod(dims))//2)


def wilson_links_host(dims, seed, eps, c=0.5):
    """u[2mu] = c U_mu(x), u[2mu+1] = c U_mu(x-mu)^dagger (host [V][18],
    entry 3*column + row)"""
    from qll_gb300 import qll
    V = int(np.prod(dims))
    th = qll.gen_gauge(tuple(dims), seed, eps, ks=False)
    x = np.array(np.meshgrid(*[np.arange(n) for n in dims], indexing="ij")).reshape(4, -1)
    here = site_index(dims, x)
    u = []
    for mu in range(4):
        y = x.copy()
        y[mu] = (y[mu] - 1) % dims[mu]
        nb = np.empty(V, dtype=np.int64)
        nb[here] = site_index(dims, y)
        m = th[mu].reshape(V, 3, 3, 2)[nb]            # [site, col, row, re/im] at x-mu
        adj = np.stack([m[..., 0].transpose(0, 2, 1), -m[..., 1].transpose(0, 2, 1)], axis=-1)
        u += [np.ascontiguousarray(c*th[mu]), np.ascontiguousarray(c*adj.reshape(V, 18))]
    return u


def wilson_dslash_timing(L, W, dims, prec, launches=50):
    """event-timed half Wilson Dslash (the hop term, odd output sites) on
    random device vectors: ms per launch and GB/s on two byte bases per
    output site, compulsory (8 links + 1 spinor load + 1 store: the bytes
    DRAM must move when neighbours come from cache) and the lattice
    convention (8 links + 8 neighbour loads + 1 store)"""
    import torch
    from qll_gb300 import qll
    L.qllg_wilson_vec_bytes.restype = ctypes.c_size_t
    L.qllg_wilson_vec_bytes.argtypes = [ctypes.c_void_p, ctypes.c_int]
    L.qllg_wilson_dslash_device.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_void_p, ctypes.c_void_p]
    stream = torch.cuda.current_stream()
    L.qllg_set_stream(ctypes.c_void_p(stream.cuda_stream))
    nb = L.qllg_wilson_vec_bytes(W, prec)
    dt = torch.float64 if prec == 0 else torch.float32
    src = torch.randn(nb//(8 if prec == 0 else 4), dtype=dt, device="cuda")
    dst = torch.empty_like(src)
    for _ in range(3):
        if L.qllg_wilson_dslash_device(W, prec, 1, ctypes.c_void_p(dst.data_ptr()),
                                       ctypes.c_void_p(src.data_ptr())):
            raise RuntimeError(qll.last_error())
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(launches):
        L.qllg_wilson_dslash_device(W, prec, 1, ctypes.c_void_p(dst.data_ptr()),
                                    ctypes.c_void_p(src.data_ptr()))
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)/launches
    b = 8 if prec == 0 else 4
    Vh = int(np.prod(dims))//2
    comp = (8*18*b + 2*24*b)*Vh
    conv = (8*18*b + 9*24*b)*Vh
    return {"dims": list(dims), "prec": "f64" if prec == 0 else "f32", "ms": ms,
            "compulsory_gbs": comp/(ms*1e-3)/1e9, "lattice_convention_gbs": conv/(ms*1e-3)/1e9,
            "gflops": 1344*Vh/(ms*1e-3)/1e9, "bytes_compulsory": comp}


def run_wilson(args):
    """C2: Wilson even-odd CGNR at 16^3x32 (--wilson-dims for another lattice), eps=0.3, kappa=0.12 (QLL mass
    1/(2 kappa) - 4), Gaussian 4x3 source, tolerance 1e-8: FP32 iterations
    with FP64 reliable updates against the plain FP64 CG, each solve one
    CUDA-graph launch; and the half Wilson Dslash timed alone at C2 and at
    32^3x64, with its roofline"""
    from qll_gb300 import qll
    L = qll.load()
    apply_params(L, args)
    L.qllg_wilson_create.restype = ctypes.c_void_p
    L.qllg_wilson_create.argtypes = [ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_void_p)]
    L.qllg_wilson_solve.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_void_p]
    L.qllg_wilson_destroy.argtypes = [ctypes.c_void_p]
    dims, kappa = tuple(int(v) for v in args.wilson_dims.split(",")), 0.12
    mass = 1/(2*kappa) - 4
    u = wilson_links_host(dims, 1002, 0.3)
    W = ctypes.c_void_p(L.qllg_wilson_create(qll.dims_c(dims), qll.vp_array(u)))
    if not W.value:
        raise RuntimeError(qll.last_error())
    b = pinned_like(qll.gen_source(dims, 2200, 24, "even"))
    out = {"workload": "C2: Wilson e/o CGNR %s, eps=0.3, kappa=0.12, true residual 1e-8 "
                       "(normal-equation rsq 1e-17)" % "x".join(map(str, dims)),
           "host_arrays": "pinned; seconds: host clock around qllg_wilson_solve (upload of b, the CGNR, the "
                          "FP64 true residual of S x = b, download of x); device_seconds: the CGNR alone "
                          "(CUDA events)"}
    x = pinned_like(np.zeros_like(b))

    def solve(mode, timing):
        x[...] = 0
        info = qll.SolveInfo()
        L.qllg_timing_enable(1 if timing else 0)
        L.qllg_timing_reset()
        t = time.time()
        # CGNR stops on the normal-equation residual |S^+ r|^2 < rsq |S^+ b|^2;
        # 1e-17 there puts the true residual |b - S x|/|b| below 1e-8
        its = L.qllg_wilson_solve(W, x.ctypes.data, b.ctypes.data, mass, 1e-17, MAXITS, mode,
                                  ctypes.byref(info))
        dt = time.time() - t
        cnt, tot = ctypes.c_int(), ctypes.c_double()
        L.qllg_timing_read(b"wilson_dslash", ctypes.byref(cnt), ctypes.byref(tot))
        L.qllg_timing_enable(0)
        if its < 0:
            raise RuntimeError(qll.last_error())
        return dt, its, info, cnt.value, tot.value

    L.qllg_get_param.restype = ctypes.c_double
    L.qllg_get_param.argtypes = [ctypes.c_char_p]

    def loop_kind(mode):
        # the library's choice: persistent FP32 iterations on small lattices
        vh = b.shape[0]//2
        if (mode == qll.SOLVE_MIXED_SINGLE and L.qllg_get_param(b"wilson_persistent") != 0 and
                vh <= L.qllg_get_param(b"persistent_max")):
            return "persistent cooperative launches of the FP32 iterations between the reliable updates"
        return "one CUDA-graph launch"

    for name, mode in (("mixed", qll.SOLVE_MIXED_SINGLE), ("fp64", qll.SOLVE_DOUBLE)):
        best = None
        for rep in range(3):
            dt, its, info, _, _ = solve(mode, False)
            if best is None or dt < best["seconds"]:
                best = {"seconds": dt, "solves_per_s": 1/dt, "iters": its,
                        "device_seconds": info.seconds, "reliable_updates": info.reliable_updates,
                        "true_rsq": info.true_rsq[0], "loop": loop_kind(mode)}
        # the half-Dslash launches of one more solve, event-timed (a host-
        # polled loop: events cannot sit in a graph's conditional body)
        _, _, _, cnt, tot = solve(mode, True)
        best["dslash_launches"] = cnt
        best["dslash_avg_ms"] = tot/max(cnt, 1)
        out[name] = best
    out["mixed"]["dslash_note"] = "avg over the solve's FP32 and FP64 half-Dslash launches"
    out["speedup_mixed_over_fp64"] = out["fp64"]["seconds"]/out["mixed"]["seconds"]
    # the half Dslash alone: C2 in FP32 and FP64, and FP32 at 32^3x64
    out["dslash_c2_f32"] = wilson_dslash_timing(L, W, dims, 1)
    out["dslash_c2_f64"] = wilson_dslash_timing(L, W, dims, 0)
    L.qllg_wilson_destroy(W)
    big = (32, 32, 32, 64)
    ub = wilson_links_host(big, 1004, 0.3)
    W = ctypes.c_void_p(L.qllg_wilson_create(qll.dims_c(big), qll.vp_array(ub)))
    del ub
    if not W.value:
        raise RuntimeError(qll.last_error())
    d32 = wilson_dslash_timing(L, W, big, 1)
    L.qllg_wilson_destroy(W)
    out["dslash_32x32x32x64_f32"] = d32
    pk = peaks().get("hbm_gbs")
    out["roofline"] = {"kernel": "wilson_dslash<f32> half Dslash, 32^3x64 (inputs larger than L2)",
                       "bound": "hbm", "achieved": d32["compulsory_gbs"], "peak": pk, "unit": "GB/s",
                       "frac": d32["compulsory_gbs"]/pk if pk else None,
                       "basis": "compulsory bytes per output site: 8 links + 1 spinor load + "
                                "1 store (768 B in FP32)",
                       "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if pk else None,
                       "c2_note": "at 16^3x32 the links and spinors (66 MB FP32) fit in L2, so "
                                  "its GB/s are not an HBM figure"}
    return out


# ---------------------------------------------------------------------- C1
def run_c1(args):
    """C1: 8^4, eps=0.3, m=0.1, one source, FP64 CG to true residual 1e-8
    (rsq 1e-16): the GPU FP64 and mixed solves (time and iterations; no
    roofline claim, 8^4 fits in L2) beside the oracle's FP64 CG (cgSolveT
    restated) on the host cores on the same links; equal FP64 iteration
    counts are the parity check"""
    from ctypes import POINTER
    from qll_gb300 import qll
    L = qll.load()
    apply_params(L, args)
    L.qllg_stag_create_asqtad.restype = ctypes.c_void_p
    L.qllg_stag_create_asqtad.argtypes = [ctypes.POINTER(ctypes.c_int),
                                          ctypes.POINTER(ctypes.c_void_p),
                                          ctypes.POINTER(qll.Fat7Coeffs)]
    L.qllg_stag_get_links.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]
    dims, mass, rsq = (8, 8, 8, 8), 0.1, 1e-16
    thin = qll.gen_gauge(dims, 1001, 0.3, ks=True)
    S = ctypes.c_void_p(L.qllg_stag_create_asqtad(qll.dims_c(dims), qll.vp_array(thin),
                                                  ctypes.byref(qll.asqtad_coeffs())))
    if not S.value:
        raise RuntimeError(qll.last_error())
    src = qll.gen_source(dims, 2100, 6, "even")
    out = {"workload": "C1: asqtad CG 8^4, eps=0.3, m=0.1, 1 rhs, true residual 1e-8"}
    for name, mode in (("fp64", qll.SOLVE_DOUBLE), ("mixed", qll.SOLVE_MIXED_SINGLE)):
        best = None
        for _ in range(3):
            x = np.zeros_like(src)
            info = qll.SolveInfo()
            t = time.time()
            its = L.qllg_stag_solve(S, 1, qll.vp_array([x]), qll.vp_array([src]),
                                    (ctypes.c_double*1)(mass), rsq, MAXITS, mode, ctypes.byref(info))
            dt = time.time() - t
            if its < 0:
                raise RuntimeError(qll.last_error())
            if best is None or dt < best["seconds"]:
                best = {"seconds": dt, "iters": its, "true_rsq": info.true_rsq[0],
                        "api": "qllg_stag_solve (host arrays)"}
        out[name] = best
    V = int(np.prod(dims))
    links = [np.zeros((V, 18)) for _ in range(16)]
    if L.qllg_stag_get_links(S, qll.vp_array(links)):
        raise RuntimeError(qll.last_error())
    L.qllg_stag_destroy(S)
    sec, its, cores = cpu_solve(links, src, dims=dims, mass=mass, rsq=rsq)
    out["cpu_oracle_fp64"] = {"seconds": sec, "iters": its, "cores": cores, "kind": "port"}
    return out


# ------------------------------------------------------------- multishift
def pinned_like(a):
    """a page-locked copy of host array a (the library moves page-locked
    arrays of 1 MiB or more on the SMs rather than the copy engines)"""
    import torch
    t = torch.empty(a.size, dtype=torch.float64, pin_memory=True).numpy().reshape(a.shape)
    t[...] = a
    return t


def run_multishift(args):
    """C3: 24^3x48, m=0.02, 12 shifts log-spaced over 1e-4..1, 8 Gaussian
    rhs, tolerance 1e-8 on every shift: the mixed multi-rhs solve (FP32
    multishift CG for the 8 rhs at once, then every (rhs, shift) pair
    refined by the FP32 mixed CG with FP64 reliable updates) against the
    reference's FP64 multishift CG run rhs after rhs"""
    from qll_gb300 import qll, serve
    L = serve._lib()
    L.qllg_stag_solve_multishift.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                             ctypes.c_void_p, ctypes.c_double, ctypes.c_int,
                                             ctypes.c_void_p, ctypes.c_double, ctypes.c_int,
                                             ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    apply_params(L, args)
    dims, nrhs, mass = (24, 24, 24, 48), 8, 0.02
    shifts = [10**(-4 + 4*k/11) for k in range(12)]
    ns = len(shifts)
    S = serve.asqtad_operator(dims, 1003, 0.3)
    bs = [pinned_like(qll.gen_source(dims, 2300 + r, 6, "even")) for r in range(nrhs)]
    out = {"workload": "C3: asqtad multishift 24^3x48, m=0.02, eps=0.3, 12 shifts 1e-4..1, "
                       "8 rhs, tolerance 1e-8 on every shift", "dims": list(dims),
           "host_arrays": "pinned; seconds: host clock around qllg_stag_solve_multishift (sources in, "
                          "96 solutions out)"}
    xs = [pinned_like(np.zeros_like(bs[0])) for _ in range(nrhs*ns)]
    for name, mode in (("mixed", qll.SOLVE_MIXED_SINGLE), ("fp64_cgms", qll.SOLVE_DOUBLE)):
        for x in xs:
            x[...] = 0
        its = (ctypes.c_int*(nrhs*ns))()
        tr = (ctypes.c_double*(nrhs*ns))()
        reps = 1 if mode == qll.SOLVE_DOUBLE else 2
        best = None
        for _ in range(reps):
            t = time.time()
            rc = L.qllg_stag_solve_multishift(S, nrhs, qll.vp_array(xs), qll.vp_array(bs), mass, ns,
                                              (ctypes.c_double*ns)(*shifts), 1e-16, MAXITS, mode,
                                              its, tr)
            dt = time.time() - t
            if rc < 0:
                raise RuntimeError(qll.last_error())
            best = dt if best is None else min(best, dt)
        out[name] = {"seconds": best, "rhs_per_s": nrhs/best, "shift_solves_per_s": nrhs*ns/best,
                     "max_iters": max(its), "max_true_rsq": max(tr[:]),
                     "note": ("FP32 multishift CG of the 8 rhs at once, then the pairs refined "
                              "16 per launch with FP64 reliable updates"
                              if mode == qll.SOLVE_MIXED_SINGLE else
                              "reference algorithm (cgmsSolveT) in FP64, one rhs per call")}
    out["speedup_mixed_over_fp64"] = out["fp64_cgms"]["seconds"]/out["mixed"]["seconds"]
    L.qllg_stag_destroy(S)
    return out


# ---------------------------------------------------------------- serving
SERVE_LATTICES = [(16, 16, 16, 16), (24, 24, 24, 48), (32, 32, 32, 64)]
SERVE_SEEDS = [5001, 5002, 5003]
SERVE_EPS = [0.3, 0.3, 0.4]


def run_serving(args):
    """the request loop on the three resident lattices: the capacity with
    every request queued at once, then Poisson arrivals at 70% of it
    (seed 7): p50/p99 latency and solves/s; beside it the same kind of
    requests solved one shift at a time by the plain FP64 single-rhs CG"""
    from qll_gb300 import qll, serve
    L = serve._lib()
    apply_params(L, args)
    # single-stored links: half the resident link bytes per lattice
    ops = [serve.asqtad_operator(d, s, e, single_store=True)
           for d, s, e in zip(SERVE_LATTICES, SERVE_SEEDS, SERVE_EPS)]

    def server():
        V = serve.Server(int(args.serve_budget*(1 << 30)), chunk=args.serve_chunk, max_batches=2)
        for S, d in zip(ops, SERVE_LATTICES):
            V.add_lattice(S, d)
        return V

    # capacity: all requests queued at t = 0
    V = server()
    recs, t_sat = serve.poisson_load(V, SERVE_LATTICES, rate=1e9,
                                     nreq=min(60, args.serve_requests//2), seed=11)
    cap = len(recs)/t_sat
    V.close()
    # Poisson arrivals at 70% of the capacity
    rate = 0.7*cap
    V = server()
    recs, t_run = serve.poisson_load(V, SERVE_LATTICES, rate=rate, nreq=args.serve_requests, seed=7)
    st = V.stats()
    V.close()
    lat = np.array([r["latency_s"] for r in recs])
    cols = sum(r["nshift"] for r in recs)
    worst = max(r["max_true_rsq_over_tol2"] for r in recs)

    # serial plain FP64 baseline on a sample: one request per lattice, each
    # shift a separate single-rhs FP64 CG
    info = qll.SolveInfo()
    rng = np.random.default_rng(7)
    t_serial, n_serial = 0.0, 0
    for li, (S, d) in enumerate(zip(ops, SERVE_LATTICES)):
        m = float(rng.uniform(0.005, 0.1))
        ns = int(rng.integers(1, 17))
        shifts = list(np.logspace(-4, 0, ns)) if ns > 1 else [1e-4]
        b = qll.gen_source(d, 6000 + 100*li, 6, "even")
        x = np.zeros_like(b)
        t = time.time()
        for sh in shifts:
            ms = (ctypes.c_double*1)(float(np.sqrt(m*m + sh)))
            if L.qllg_stag_solve(S, 1, qll.vp_array([x]), qll.vp_array([b]), ms, 1e-16, MAXITS,
                                 qll.SOLVE_DOUBLE, ctypes.byref(info)) < 0:
                raise RuntimeError(qll.last_error())
        t_serial += time.time() - t
        n_serial += 1
    for S in ops:
        L.qllg_stag_destroy(S)
    return {
        "workload": "C5: 16^4 + 24^3x48 + 32^3x64 resident (single-stored links); Poisson "
                    "arrivals (seed 7) at 70% "
                    "of the measured capacity; per request m~U[0.005,0.1], 1-16 shifts "
                    "log-spaced in [1e-4,1], tolerance 1e-8 or 1e-10",
        "requests": len(recs), "shift_solves": cols, "seconds": t_run,
        "requests_per_s": len(recs)/t_run, "shift_solves_per_s": cols/t_run,
        "capacity_requests_per_s": cap, "arrival_rate_per_s": rate,
        "latency_p50_s": float(np.percentile(lat, 50)),
        "latency_p99_s": float(np.percentile(lat, 99)),
        "latency_max_s": float(lat.max()),
        "failed_requests": int(sum(1 for r in recs if r["status"] != 2)),
        "max_true_rsq_over_tol2": worst,
        "hbm_budget_bytes": st.budget_bytes, "hbm_used_bytes_end": st.used_bytes,
        "chunk_iters": args.serve_chunk,
        "autotune": autotune_report(L),
        "serial_fp64_baseline": {"requests_per_s": n_serial/t_serial, "sample": "%d requests, "
                                 "one per lattice, each shift a separate FP64 single-rhs CG"
                                 % n_serial},
    }


# ---------------------------------------------------------- CPU baseline
def host_threads():
    """the host cores this process may run on"""
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def _oracle(fast=True):
    """the CPU oracle: the timing build (host-native flags) or the parity
    build, with its thread count set to every host core this process may
    use (an OpenMP runtime shared with other code in the process may have
    been set to fewer)"""
    from ctypes import POINTER
    name = "liboracle_fast.so" if fast else "liboracle.so"
    lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_build", name))
    lib.or_solve2D.restype = ctypes.c_int
    lib.or_num_threads.restype = ctypes.c_int
    lib.or_set_num_threads(host_threads())
    return lib, POINTER


def cpu_solve(u16, src, dims=None, mass=MASS, rsq=RSQ, maxits=MAXITS):
    """one converged FP64 CG solve (solve2D: cgSolveT with dslash2, the
    reference's algorithm restated) of one source on the host cores, timed
    whole; u16 are the 16 link slots 4mu+2b+naik.  Returns (seconds,
    iterations, threads)."""
    dims = tuple(dims or DIMS)
    lib, POINTER = _oracle()
    PA = (POINTER(ctypes.c_double)*8)
    u = PA(*[u16[2*i].ctypes.data_as(POINTER(ctypes.c_double)) for i in range(8)])
    u3 = PA(*[u16[2*i+1].ctypes.data_as(POINTER(ctypes.c_double)) for i in range(8)])
    x = np.zeros_like(src)
    fr = ctypes.c_double()
    args = lambda its: (dims_ct(dims), x.ctypes.data_as(POINTER(ctypes.c_double)), u, u3,
                        ctypes.c_double(mass), src.ctypes.data_as(POINTER(ctypes.c_double)),
                        ctypes.c_double(rsq), its, 1, ctypes.byref(fr))
    lib.or_solve2D(*args(2))                            # first touch, thread start-up
    x[:] = 0
    t = time.time()
    its = lib.or_solve2D(*args(maxits))
    return time.time() - t, its, lib.or_num_threads()


def dims_ct(dims):
    return (ctypes.c_int*4)(*dims)


REF_FAST = os.path.join(ROOT, "oracle", "_ref", "libqllref_fast.so")


def _aligned(shape):
    """a zeroed float64 array on a 64-byte boundary (the reference's
    vector loads assume its own 64-byte-aligned allocations)"""
    n = int(np.prod(shape))
    buf = np.zeros(n + 16)
    off = (-buf.ctypes.data % 64)//8
    return buf[off:off + n].reshape(shape)


def ref_cpu_solve(u16, src, dims=None, mass=MASS, rsq=RSQ, maxits=MAXITS):
    """one converged FP64 solve2 of the reference library itself
    (oracle/_ref/libqllref_fast.so: the reference's sources, its 4-site SIMD
    layout, host-native flags) on the host cores, timed whole; the links and
    the source are moved into the reference's layout first, untimed.
    Returns (seconds, iterations, threads)."""
    from ctypes import POINTER, c_double, c_int
    dims = tuple(dims or DIMS)
    R = ctypes.CDLL(REF_FAST)
    R.refh_solve2D.restype = c_int
    n = host_threads()
    R.refh_set_threads(n)
    if R.refh_setup(dims_ct(dims)):
        raise RuntimeError("reference setup failed")
    P = lambda a: a.ctypes.data_as(POINTER(c_double))

    def to_layout(a):
        out = _aligned(a.shape)
        R.refh_convertD(P(out), P(np.ascontiguousarray(a)), a.shape[1], 1)
        return out
    # slot 4mu+2b+naik -> u[2mu+b] (fat), u3[2mu+b] (Naik)
    u = [to_layout(u16[4*mu + 2*b]) for mu in range(4) for b in range(2)]
    u3 = [to_layout(u16[4*mu + 2*b + 1]) for mu in range(4) for b in range(2)]
    PA = lambda arrs: (POINTER(c_double)*8)(*[P(a) for a in arrs])
    b = to_layout(src)
    x = _aligned(src.shape)
    R.refh_solve2D(P(x), PA(u), PA(u3), c_double(mass), P(b), c_double(rsq), 2, 1)   # warm
    x[:] = 0
    t = time.time()
    its = R.refh_solve2D(P(x), PA(u), PA(u3), c_double(mass), P(b), c_double(rsq), maxits, 1)
    return time.time() - t, its, n


def timed_cpu_solve(u16, src, **kw):
    """the CPU baseline's converged solve: the reference library itself
    where it was built here (kind "reference"), else the oracle's
    restatement of it (kind "port")"""
    if os.path.exists(REF_FAST):
        sec, its, cores = ref_cpu_solve(u16, src, **kw)
        return sec, its, cores, "reference", ("the reference's own solve2D/cgSolveT/dslash2, "
                                              "compiled from its sources with its 4-site SIMD "
                                              "layout (-DC4) and host-native flags")
    sec, its, cores = cpu_solve(u16, src, **kw)
    return sec, its, cores, "port", ("the oracle's restatement of solve2D/cgSolveT/dslash2, "
                                     "host-native build")


def cpu_baseline(L, S):
    """the GPU arm's CPU baseline: one converged FP64 solve of one source
    by the oracle on the host cores, on the operator's own links"""
    from qll_gb300 import qll
    V = int(np.prod(DIMS))
    links = [np.zeros((V, 18)) for _ in range(16)]
    if L.qllg_stag_get_links(S, qll.vp_array(links)):
        raise RuntimeError(qll.last_error())
    src = qll.gen_source(DIMS, SEED_SRC, 6, "even")
    sec, its, cores, kind, what = timed_cpu_solve(links, src)
    return {"value": 1.0/sec, "unit": "solves/s", "cores": cores, "kind": kind,
            "sample": "one converged FP64 CG solve of one source (%d iterations, %.1f s; %s, "
                      "OpenMP on %d threads) on the 32^3x64 links" % (its, sec, what, cores)}


def cpu_inputs():
    """the headline inputs made on the host by the oracle alone (no GPU
    library loaded): thin links by the shared generator, fat7 and Naik
    links by the oracle's smearFat7, negative-adjoint backward links; in
    slot order 4mu+2b+naik"""
    lib, POINTER = _oracle(fast=False)
    V = int(np.prod(DIMS))
    thin = [np.zeros((V, 18)) for _ in range(4)]
    pa = (ctypes.c_void_p*4)(*[t.ctypes.data for t in thin])
    if lib.or_gen_gauge(dims_ct(DIMS), ctypes.c_ulonglong(SEED_GAUGE), ctypes.c_double(EPS), 1, pa):
        raise RuntimeError("or_gen_gauge failed")
    src = np.zeros((V, 6))
    lib.or_gen_source(dims_ct(DIMS), ctypes.c_ulonglong(SEED_SRC), 6, b"even",
                      ctypes.c_void_p(src.ctypes.data))
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib as orc

    class Coef:
        one_link, three_staple, five_staple = 5/8, -1/16, 1/64
        seven_staple, lepage, naik = -1/384, -1/16, -1/24
    fl, ll = orc.smear_fat7(DIMS, thin, Coef)
    del thin
    links = []
    for mu in range(4):
        links += [fl[mu], ll[mu], orc.negadj_back(DIMS, fl[mu], mu, 1),
                  orc.negadj_back(DIMS, ll[mu], mu, 3)]
    return links, src


def run_reference(args):
    """the reference arm: the reference's own CPU solve on the host cores
    (the reference library compiled from its sources, SIMD layout,
    host-native flags; the oracle's restatement of it where the reference
    was not built), one converged FP64 solve of one source per step, on
    inputs made on the host without the GPU library.  Timed steps are
    capped so that the run stays within a few minutes; the line reports the
    steps actually timed."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    links, src = cpu_inputs()
    budget_s = args.cpu_budget
    secs, its = [], 0
    for _ in range(min(args.warmup, 1)):
        timed_cpu_solve(links, src, maxits=20)           # warm-up: a short solve
    t0 = time.time()
    for k in range(args.steps):
        sec, its, cores, kind, what = timed_cpu_solve(links, src)
        secs.append(sec)
        if time.time() - t0 + sec > budget_s:
            break
    value = len(secs)/sum(secs)
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s",
           "n_gpus": ws, "steps": len(secs), "steps_requested": args.steps, "warmup": args.warmup,
           "ms_per_step": 1e3*sum(secs)/len(secs),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded SU(3) gauge, oracle fat7, Gaussian source)",
           "config": CONFIG,
           "cpu_baseline": {"value": value, "unit": "solves/s", "cores": cores, "kind": kind,
                            "sample": "%d converged FP64 CG solves of one source (%d iterations "
                                      "each; %s, OpenMP on %d threads)"
                                      % (len(secs), its, what, cores)},
           "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def run_wilson_dslash_only(args):
    """launches of the Wilson half Dslash alone on a chosen lattice (FP32,
    random device input), for profiling"""
    from qll_gb300 import qll
    L = qll.load()
    apply_params(L, args)
    L.qllg_wilson_create.restype = ctypes.c_void_p
    L.qllg_wilson_create.argtypes = [ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_void_p)]
    L.qllg_wilson_destroy.argtypes = [ctypes.c_void_p]
    dims = tuple(int(v) for v in args.dims.split(","))
    u = wilson_links_host(dims, 1004, 0.3)
    W = ctypes.c_void_p(L.qllg_wilson_create(qll.dims_c(dims), qll.vp_array(u)))
    del u
    if not W.value:
        raise SystemExit(qll.last_error())
    prec = {"f64": 0, "f32": 1}[args.prec]
    out = wilson_dslash_timing(L, W, dims, prec, launches=args.launches)
    L.qllg_wilson_destroy(W)
    print(json.dumps({"wilson_dslash_only": out}), flush=True)


def run_dslash_only(args):
    """a few launches of the headline Dslash kernel on a chosen lattice, for
    profiling: FP32, 16 rhs, device-resident random input"""
    import torch
    from qll_gb300 import qll
    L = qll.load()
    L.qllg_stag_create_asqtad.restype = ctypes.c_void_p
    L.qllg_stag_create_asqtad.argtypes = [ctypes.POINTER(ctypes.c_int),
                                          ctypes.POINTER(ctypes.c_void_p),
                                          ctypes.POINTER(qll.Fat7Coeffs)]
    L.qllg_stag_vec_bytes.restype = ctypes.c_size_t
    L.qllg_stag_vec_bytes.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
    L.qllg_stag_dslash_device.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    L.qllg_set_param.argtypes = [ctypes.c_char_p, ctypes.c_double]
    for kv in args.param:
        k, v = kv.split("=")
        if L.qllg_set_param(k.encode(), float(v)) != 0:
            raise SystemExit(qll.last_error())
    stream = torch.cuda.current_stream()
    L.qllg_set_stream(ctypes.c_void_p(stream.cuda_stream))
    dims = tuple(int(v) for v in args.dims.split(","))
    prec = {"f64": 0, "f32": 1, "i16": 2, "f32r": 3, "df": 4}[args.prec]
    thin = qll.gen_gauge(dims, SEED_GAUGE, EPS, ks=True)
    coef = qll.asqtad_coeffs()
    S = ctypes.c_void_p(L.qllg_stag_create_asqtad(qll.dims_c(dims), qll.vp_array(thin),
                                                  ctypes.byref(coef)))
    nb = L.qllg_stag_vec_bytes(S, prec, args.nrhs)
    # random 4-byte words are valid input for FP32 layouts; the 16-bit layout
    # gets scales of 1
    src = torch.randn(nb//4, dtype=torch.float32, device="cuda")
    if prec == 2:
        src = src.view(-1, 4)
        src[:, 3] = 1.0
        src = src.reshape(-1)
    if prec == 0:
        src = torch.randn(nb//8, dtype=torch.float64, device="cuda")
    dst = torch.empty_like(src)
    for _ in range(3):
        L.qllg_stag_dslash_device(S, prec, args.nrhs, 1, ctypes.c_void_p(dst.data_ptr()),
                                  ctypes.c_void_p(src.data_ptr()))
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.launches):
        L.qllg_stag_dslash_device(S, prec, args.nrhs, 1, ctypes.c_void_p(dst.data_ptr()),
                                  ctypes.c_void_p(src.data_ptr()))
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)/args.launches
    Vh = int(np.prod(dims))//2
    bs = {0: 8, 1: 4, 2: 2, 3: 4, 4: 8}[prec]
    ns = 4 if prec == 2 else 0
    naik_reals = 12 if prec == 3 else 18
    per = (8*18*bs + 8*naik_reals*bs)/args.nrhs + 17*(6*bs + ns)
    print(json.dumps({"dslash_only": {"dims": dims, "nrhs": args.nrhs, "prec": args.prec,
                                      "params": args.param, "autotune": autotune_report(L),
                                      "ms": ms, "algorithmic_gbs": per*Vh*args.nrhs/(ms*1e-3)/1e9,
                                      "bulk_error": L.qllg_k_bulk_error(1),
                                      "error": qll.last_error()}}), flush=True)
    L.qllg_stag_destroy(S)


def run_solve_only(args):
    """a few multi-rhs solves of a chosen mode on a chosen lattice, for
    profiling the solver's kernels (and sweeping its parameters with
    --param name=value): prints iterations, reliable updates and time"""
    from qll_gb300 import qll
    L = qll.load()
    L.qllg_stag_create_asqtad.restype = ctypes.c_void_p
    L.qllg_stag_create_asqtad.argtypes = [ctypes.POINTER(ctypes.c_int),
                                          ctypes.POINTER(ctypes.c_void_p),
                                          ctypes.POINTER(qll.Fat7Coeffs)]
    L.qllg_set_param.argtypes = [ctypes.c_char_p, ctypes.c_double]
    for kv in args.param:
        k, v = kv.split("=")
        if L.qllg_set_param(k.encode(), float(v)) != 0:
            raise SystemExit(qll.last_error())
    dims = tuple(int(v) for v in args.dims.split(","))
    mode = {"double": qll.SOLVE_DOUBLE, "single": qll.SOLVE_SINGLE,
            "mixed_half": qll.SOLVE_MIXED_HALF, "mixed_single": qll.SOLVE_MIXED_SINGLE}[args.mode]
    thin = qll.gen_gauge(dims, SEED_GAUGE, EPS, ks=True)
    coef = qll.asqtad_coeffs()
    S = ctypes.c_void_p(L.qllg_stag_create_asqtad(qll.dims_c(dims), qll.vp_array(thin),
                                                  ctypes.byref(coef)))
    if not S.value:
        raise SystemExit(qll.last_error())
    nrhs = args.nrhs
    srcs = [qll.gen_source(dims, SEED_SRC + r, 6, "even") for r in range(nrhs)]
    b = L.qllg_stag_vec_alloc(S, nrhs)
    x = L.qllg_stag_vec_alloc(S, nrhs)
    L.qllg_stag_vec_upload(S, b, nrhs, qll.vp_array(srcs))
    masses = (ctypes.c_double*nrhs)(*([MASS]*nrhs))
    info = qll.SolveInfo()
    fams = ["stag_dslash_f32_n%d" % nrhs, "stag_cg_fused_f32_n%d" % nrhs,
            "stag_dslash_f64_n%d" % nrhs, "stag_dslash_df_n%d" % nrhs]
    for k in range(args.launches):
        timed = args.timing and k == args.launches - 1
        if timed:
            # per-kernel-family CUDA events (the host-polled loop, no graph)
            L.qllg_timing_enable(1)
            L.qllg_timing_reset()
        t = time.time()
        its = L.qllg_stag_solve_device(S, nrhs, x, b, masses, RSQ, MAXITS, mode, ctypes.byref(info))
        dt = time.time() - t
        if timed:
            L.qllg_timing_enable(0)
            tm = {}
            for f in fams:
                cnt, tot = ctypes.c_int(), ctypes.c_double()
                L.qllg_timing_read(f.encode(), ctypes.byref(cnt), ctypes.byref(tot))
                tm[f] = {"launches": cnt.value, "ms": tot.value}
            print(json.dumps({"timing": tm}), flush=True)
        print(json.dumps({"solve_only": {"dims": dims, "nrhs": nrhs, "mode": args.mode,
                                         "params": args.param, "iters": its,
                                         "reliable_updates": info.reliable_updates,
                                         "seconds": dt,
                                         "max_true_rsq": max(info.true_rsq[r] for r in range(nrhs)),
                                         "error": qll.last_error()}}), flush=True)
    L.qllg_stag_vec_free(b)
    L.qllg_stag_vec_free(x)
    L.qllg_stag_destroy(S)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-budget", type=float, default=150.0,
                    help="--impl reference: stop timing further solves after this many seconds")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--dslash-only", action="store_true")
    ap.add_argument("--wilson-dslash-only", action="store_true",
                    help="the Wilson half Dslash alone on --dims, --prec f32 or f64")
    ap.add_argument("--dims", default="32,32,32,64")
    ap.add_argument("--prec", default="f32", choices=["f64", "f32", "i16", "f32r", "df"])
    ap.add_argument("--nrhs", type=int, default=16)
    ap.add_argument("--launches", type=int, default=20)
    ap.add_argument("--solve-only", action="store_true")
    ap.add_argument("--mode", default="mixed_single",
                    choices=["double", "single", "mixed_half", "mixed_single"])
    ap.add_argument("--param", action="append", default=[])
    ap.add_argument("--serve", action="store_true", help="only the serving benchmark")
    ap.add_argument("--timing", action="store_true",
                    help="--solve-only: per-kernel-family event times of the last solve")
    ap.add_argument("--no-serve", action="store_true",
                    help="skip the Wilson, multishift and serving legs")
    ap.add_argument("--multishift", action="store_true", help="only the multishift benchmark")
    ap.add_argument("--wilson", action="store_true", help="only the Wilson benchmark")
    ap.add_argument("--wilson-dims", default="16,16,16,32", help="lattice of the Wilson benchmark")
    ap.add_argument("--serve-requests", type=int, default=300)
    ap.add_argument("--serve-budget", type=float, default=48.0, help="GiB")
    ap.add_argument("--serve-chunk", type=int, default=20)
    args = ap.parse_args()
    if args.wilson_dslash_only:
        run_wilson_dslash_only(args)
    elif args.dslash_only:
        run_dslash_only(args)
    elif args.solve_only:
        run_solve_only(args)
    elif args.serve:
        print(json.dumps({"serving": run_serving(args)}), flush=True)
    elif args.multishift:
        print(json.dumps({"multishift": run_multishift(args)}), flush=True)
    elif args.wilson:
        print(json.dumps({"wilson": run_wilson(args)}), flush=True)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
