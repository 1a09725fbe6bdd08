"""Benchmark: converged eigenpairs per second on the three-mode leaf (N = 671,744, m = 12, block 16).

A step is one eigen-solve of the leaf Hamiltonian
    H = 4E_C1 n1^2 - E_C2 d2^2 - E_C3 d3^2 + E_L/2 (phi2^2 + phi3^2) - 2E_J cos phi1 cos phi2 - E_J' cos(phi2 - phi3)
on a 41 x 256 x 64 charge x grid x grid basis for one synthetic theta drawn from the stated
uniform ranges (seeded; the draws cycle), lowest 12 eigenpairs with LOBPCG (block 16, product
seed), every pair accepted at ||H x - lambda x|| <= 1e-8 ||H|| (||H|| = Gershgorin bound) by a
fresh FP64 application.

  value            converged pairs / s of the mixed-precision solver (FP32 bulk, FP64 Rayleigh-Ritz
                   and refinement), operators already on the device when the timed region starts
  plain_f64        the same for the plain FP64 solver (the metric's denominator)
  e2e              the public API end to end with host buffers: kf_op_create from the host term
                   list, solve (product seed built by the library), host eigenpairs out, kf_op_destroy,
                   every step
  roofline         the dominant kernel of a warm solve by the ncu launch list (its template
                   instantiations summed), the fused stencil apply k_apply_fused<float>: algorithmic
                   bytes 2 N b 4 per launch (16 columns) over its CUDA-event time, against the measured
                   HBM copy bandwidth; roofline_update / roofline_mode / roofline_gram: the tcgen05
                   FP32 block update on the fused X/P Rayleigh-Ritz shape ([X_a Q] C, 18 + 36 -> 36
                   columns, (54 + 36) N 4), the separable preconditioner's tcgen05 mode product
                   (256-point axis, 18 columns, 2 N b 4) and the tensor-core Gram of the
                   orthogonalisation ([X Z]'Z, 18 + 36 columns, N b 4)
  cpu_baseline     the oracle's restatement of the reference CPU path (C/OpenMP mul! + NumPy LOBPCG)
                   on the host cores, a bounded sample

`--impl reference` times the reference's CPU path (the oracle port: the reference is Julia and
cannot run here) on the same workload and metric.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "kronfreecircuits.jl_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

M_PAIRS = 12
SEED = 20261205          # theta draws of the three-mode leaf workload
NDRAWS = 64
# ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch (profiles/*.md), N = 671,744: the
# FP32 16-column fused apply (written Y stays in L2: reads 45.7 MB, writes 9.9 MB); the pipelined
# tcgen05 mode product, 256-point axis, 18 columns (reads 48.6 MB = X once, writes 1.9 MB: Y stays
# in L2);
# the tensor-core Gram of [X Z]'Z at 18 + 36 columns (reads 145.2 MB = every element once, writes
# 0.1 MB of partials)
APPLY_TRAFFIC_BYTES = 55641088
MODE_TRAFFIC_BYTES = 50463488
UPDATE_TRAFFIC_BYTES = 200817152   # ncu dram bytes read + written, one launch (the rest of Y stays in L2)
GRAM_TC_TRAFFIC_BYTES = 145235200


def thetas():
    from kfgpu import circuits
    rng = np.random.default_rng(SEED)
    return [circuits.three_mode_theta(rng) for _ in range(NDRAWS)]


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Dist:
    """Replicas, one process per GPU (torchrun's RANK / LOCAL_RANK / WORLD_SIZE): the path has no
    exchange step, so each rank solves its own theta draws on its own GPU and only host-side
    scalars meet, over a gloo process group -- a barrier around the timed region, the largest
    time over ranks, sums of the work done."""

    def __init__(self):
        self.rank = int(os.environ.get("RANK", "0"))
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.dist = None
        if self.world > 1:
            import torch.distributed as dist
            if not dist.is_initialized():
                dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.dist is not None:
            self.dist.barrier()

    def _reduce(self, x, op):
        if self.dist is None:
            return float(x)
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self.dist.all_reduce(t, op=op)
        return float(t.item())

    def max(self, x):
        return self._reduce(x, self.dist.ReduceOp.MAX if self.dist else None)

    def sum(self, x):
        return self._reduce(x, self.dist.ReduceOp.SUM if self.dist else None)

    def close(self):
        if self.dist is not None and self.dist.is_initialized():
            self.dist.destroy_process_group()


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self, gpu=0):
        self.rows, self._stop, self._t, self.gpu = [], threading.Event(), None, gpu

    def start(self):
        def run():
            q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
            while not self._stop.is_set():
                try:
                    out = subprocess.run(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits"],
                                         capture_output=True, text=True, timeout=5).stdout.strip()
                    if out:
                        self.rows.append([x.strip() for x in out.split(",")])
                except Exception:
                    pass
                self._stop.wait(0.2)
        self._t = threading.Thread(target=run, daemon=True)
        self._t.start()
        return self

    def stop(self):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)
        sm = [float(r[0]) for r in self.rows if r and r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if len(r) > 1 and r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if len(r) > 2 + i and r[2 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def measure_apply(torch, H, f32, b=16, reps=20):
    """CUDA-event time of one fused apply launch (inputs larger than L2 rotate between launches)."""
    dt = torch.float32 if f32 else torch.float64
    nbuf = 3
    Xs = [torch.randn(b, H.N, dtype=dt, device="cuda") for _ in range(nbuf)]
    Ys = [torch.empty_like(Xs[0]) for _ in range(nbuf)]
    s = torch.cuda.Stream()
    H.set_stream(s.cuda_stream)
    for i in range(3):
        H.apply_device(Xs[i % nbuf].data_ptr(), Ys[i % nbuf].data_ptr(), b, f32=f32)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for i in range(reps):
        H.apply_device(Xs[i % nbuf].data_ptr(), Ys[i % nbuf].data_ptr(), b, f32=f32)
    e1.record(s)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps / 1e3


def run_ours(args, D):
    import torch
    from kfgpu import KronFreeOperator, LOBPCG, circuits, solve
    from kfgpu._abi import launch_count
    from kfgpu.build import build_library

    assert torch.cuda.is_available(), "bench.py needs a CUDA device"
    torch.cuda.set_device(D.local)
    if D.rank == 0:
        build_library()
    D.barrier()
    ths = thetas()
    K, W = args.steps, args.warmup
    # each replica solves its own draws (weak scaling: K solves per GPU)
    idx = [(W + D.rank * K + k) % NDRAWS for k in range(K)]
    # operators prepared before the timed region (inputs resident); each solve builds its product
    # seed on the device, as the reference's solve builds it (src/lobpcg.jl:247)
    ops = {}
    for i in sorted(set(idx) | set(range(W))):
        dims, terms = circuits.three_mode_leaf(ths[i])
        H = KronFreeOperator(dims, terms)
        ops[i] = (H, None)
    stream = torch.cuda.Stream()
    for H, _ in ops.values():
        H.set_stream(stream.cuda_stream)

    def one(i, precision, precond=None):
        H, seedb = ops[i]
        tol = 1e-8 * H.gershgorin_bound()
        pc = precond or ("separable" if precision == "mixed" else "ritz")
        buf = args.buffer if precision == "mixed" else None
        E, V, st = solve(LOBPCG(tol=tol, precision=precision, preconditioner=pc, buffer=buf), H, M_PAIRS,
                         seed_block=seedb)
        return st["converged"], st

    for w in range(W):
        one(w, "mixed")
    torch.cuda.synchronize()
    n0 = launch_count()
    clocks = Clocks(D.local).start()
    D.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    conv, stats = 0, []
    for i in idx:
        c, st = one(i, "mixed")
        conv += c
        stats.append(st)
    e1.record(stream)
    torch.cuda.synchronize()
    D.barrier()
    clk = clocks.stop()
    # the job's time is the slowest replica's; its work is every replica's
    t_mixed = D.max(e0.elapsed_time(e1) / 1e3)
    conv_all = D.sum(conv)
    launches = int(D.sum(launch_count() - n0))
    value = conv_all / t_mixed
    # plain FP64 on a subset of the same draws (the metric's denominator)
    kp = max(1, min(args.plain_steps, K))
    D.barrier()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    conv64, st64 = 0, []
    for i in idx[:kp]:
        c, st = one(i, "f64")
        conv64 += c
        st64.append(st)
    f1.record(stream)
    torch.cuda.synchronize()
    t64 = D.max(f0.elapsed_time(f1) / 1e3)
    plain = D.sum(conv64) / t64
    # the same FP64 solver with the separable preconditioner (what precision alone buys)
    g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    g0.record(stream)
    c_sep, st_sep = one(idx[0], "f64", "separable")
    g1.record(stream)
    torch.cuda.synchronize()
    t_sep = g0.elapsed_time(g1) / 1e3
    # end to end through the public API with host buffers
    ke = max(1, min(args.e2e_steps, K))
    h2d = d2h = 0
    torch.cuda.synchronize()
    D.barrier()
    t0 = time.perf_counter()
    conv_e = 0
    for i in idx[:ke]:
        dims, terms = circuits.three_mode_leaf(ths[i])
        H = KronFreeOperator(dims, terms)
        tol = 1e-8 * H.gershgorin_bound()
        E, V, st = solve(LOBPCG(tol=tol, precision="mixed", preconditioner="separable", buffer=args.buffer), H,
                         M_PAIRS)
        conv_e += st["converged"]
        h2d += H.N * 8 + sum(op.n * 8 * 5 for _, fs in terms for _, op in fs)
        d2h += V.nbytes + E.nbytes
        H.close()
    torch.cuda.synchronize()
    te = D.max(time.perf_counter() - t0)
    conv_e = D.sum(conv_e)
    # roofline of the dominant kernel of a warm solve (by the ncu launch list: the fused stencil
    # apply), of the tcgen05 block update on the fused X/P Rayleigh-Ritz shape, of the
    # preconditioner's mode product and of the tensor-core Gram
    H0 = ops[idx[0]][0]
    peak, kind = peaks()
    t_upd = time_update(torch, 1, 18, 36, 36, H0.N)
    alg_upd = (18 + 36 + 36) * H0.N * 4
    t_mode = time_mode_product(torch, 1, (41, 256, 64), 1, b=MODE_COLS)
    alg_mode = 2 * H0.N * MODE_COLS * 4
    t_gram = time_gram_tc(torch, (18, 36), (0, 2, 1, 2), H0.N)
    alg_gram = (18 + 36) * H0.N * 4
    t_apply = measure_apply(torch, H0, True)
    alg = 2 * H0.N * 16 * 4
    achieved = alg / t_apply / 1e9
    line = {
        "metric": "converged eigenpairs/s at 1e-8 resid: warm-start mixed vs plain FP64, 1 GB300",
        "value": value, "unit": "eigenpairs/s", "n_gpus": D.world, "steps": K, "warmup": W,
        "ms_per_step": 1e3 * t_mixed / K, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 bulk + f64 refinement", "data": "synthetic",
        "config": {"workload": "three-mode leaf 41x256x64 (N=671,744), LOBPCG m=12 block=16, product seed, "
                               "tol 1e-8*||H||, theta ~ U(ranges) seed 20261205",
                   "buffer_columns": "library default (2, mixed only)" if args.buffer is None else args.buffer,
                   "l2": "inputs larger than L2 (a 16-column FP32 block is 43 MB; a solve streams ~10 GB)"},
        "replicas": D.world,
        "plain_f64": {"value": plain, "steps": kp, "ms_per_step": 1e3 * t64 / kp,
                      "iterations": [s["iterations"] for s in st64]},
        "speedup_mixed_vs_f64": value / plain if plain > 0 else None,
        "f64_separable": {"value": c_sep / t_sep, "iterations": st_sep["iterations"], "ms_per_step": 1e3 * t_sep},
        "iterations": [s["iterations"] for s in stats], "iterations_f64_phase": [s["iterations_f64"] for s in stats],
        "max_residual_rel": max(s["max_residual"] / s["hnorm"] for s in stats),
        "e2e": {"value": conv_e / te, "unit": "eigenpairs/s", "h2d_bytes_per_step": int(h2d / ke),
                "d2h_bytes_per_step": int(d2h / ke), "steps": ke},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": APPLY_TRAFFIC_BYTES, "kernel": "k_apply_fused<float> (fused stencil apply, 16 columns, the tuned variant)",
                     "algorithmic_bytes": alg, "launch_us": t_apply * 1e6, "peak_kind": kind},
        "roofline_update": {"bound": "hbm", "achieved": alg_upd / t_upd / 1e9, "peak": peak, "unit": "GB/s",
                            "frac": alg_upd / t_upd / 1e9 / peak, "traffic": UPDATE_TRAFFIC_BYTES,
                            "kernel": "k_update_tc<3> (tcgen05 FP32 block update, TF32 hi / lo, 3-tile staging ring: "
                                      "[X_a Q] C, 18 + 36 -> 36 columns, the fused X/P Rayleigh-Ritz update)",
                            "algorithmic_bytes": alg_upd, "launch_us": t_upd * 1e6, "peak_kind": kind},
        "roofline_mode": {"bound": "hbm", "achieved": alg_mode / t_mode / 1e9, "peak": peak, "unit": "GB/s",
                          "frac": alg_mode / t_mode / 1e9 / peak, "traffic": MODE_TRAFFIC_BYTES,
                          "kernel": f"k_mode_pipe<64> (pipelined tcgen05 BF16 mode product, 256-point axis, "
                                    f"{MODE_COLS} columns)",
                          "algorithmic_bytes": alg_mode, "launch_us": t_mode * 1e6, "peak_kind": kind},
        "roofline_gram": {"bound": "hbm", "achieved": alg_gram / t_gram / 1e9, "peak": peak, "unit": "GB/s",
                          "frac": alg_gram / t_gram / 1e9 / peak, "traffic": GRAM_TC_TRAFFIC_BYTES,
                          "kernel": "k_gram_tc + k_reduce_partials_f32 ([X Z]'Z, 18 + 36 FP32 columns)",
                          "algorithmic_bytes": alg_gram, "launch_us": t_gram * 1e6, "peak_kind": kind},
        "clocks": clk, "gpu_launches": launches,
    }
    if not args.no_cpu and D.world == 1:
        line["cpu_baseline"] = cpu_baseline(ths[idx[0]], bounded=True,
                                            iters=int(round(np.mean([s["iterations"] for s in st64]))))
    return line if D.rank == 0 else None


def profile_one(args):
    """One mixed-precision solve (the timed step's work) for a profiler's launch list: a first solve
    on another draw tunes the fused apply (as the bench's warm-up does), then the measured solve
    runs inside the NVTX range "measured_solve" (ncu --nvtx --nvtx-include "measured_solve/")."""
    import torch
    from kfgpu import KronFreeOperator, LOBPCG, circuits, solve
    from kfgpu._abi import launch_count
    ths = thetas()

    def one(th):
        dims, terms = circuits.three_mode_leaf(th)
        H = KronFreeOperator(dims, terms)
        return H, solve(LOBPCG(tol=1e-8 * H.gershgorin_bound(), precision="mixed", preconditioner="separable",
                               buffer=args.buffer), H, M_PAIRS)

    one(ths[(args.warmup + 1) % len(ths)])
    torch.cuda.synchronize()
    n0 = launch_count()
    t0 = time.perf_counter()
    torch.cuda.nvtx.range_push("measured_solve")
    H, (E, V, st) = one(ths[args.warmup])
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    return {"seconds": time.perf_counter() - t0, "launches": launch_count() - n0, "iterations": st["iterations"],
            "iterations_f64": st["iterations_f64"], "seconds_f64": st["seconds_f64"]}


def run_apply_workload(args):
    """The fused stencil apply alone on the three-mode leaf: 3 launches per precision after the
    autotuner's first call (16 columns, inputs rotating over three blocks larger than L2)."""
    import torch
    from kfgpu import KronFreeOperator, circuits
    ths = thetas()
    dims, terms = circuits.three_mode_leaf(ths[args.warmup])
    H = KronFreeOperator(dims, terms)
    out = {"workload": "fused apply, three-mode leaf 41x256x64 (N=671,744), 16 columns"}
    for f32 in (True, False):
        t = measure_apply(torch, H, f32, b=16, reps=3)
        by = 2 * H.N * 16 * (4 if f32 else 8)
        out["apply_%s_us" % ("f32" if f32 else "f64")] = t * 1e6
        out["apply_%s_gbs" % ("f32" if f32 else "f64")] = by / t / 1e9
    # every kernel variant forced (0-4, 6: point per thread, 5: plane-marching through shared memory)
    import ctypes as C
    from kfgpu import _abi
    for f32 in (True, False):
        dt = torch.float32 if f32 else torch.float64
        X = torch.randn(16, H.N, dtype=dt, device="cuda")
        Y = torch.empty_like(X)
        flags = _abi.KF_DEVICE | (_abi.KF_F32 if f32 else _abi.KF_F64)
        for v in range(7):
            ms = C.c_float(0)
            _abi.check(_abi.lib().kf_test_apply_variant(H.handle, v, C.c_void_p(X.data_ptr()), C.c_void_p(Y.data_ptr()),
                                                        H.N, 16, flags, 10, C.byref(ms)))
            out["variant%d_%s_us" % (v, "f32" if f32 else "f64")] = ms.value * 1e3
    return out


def time_mode_product(torch, path, dims, axis, b=16, reps=10):
    """Mean device time of one mode product launch (the library's test-only timing entry point:
    operator image built once, CUDA events around `reps` launches); X and Y are b-column FP32
    blocks of the given grid (the 16-column three-mode block is 43 MB, so X and Y together exceed
    L2 only partly; the launches read the same X)."""
    import ctypes as C
    from kfgpu import _abi
    N = int(np.prod(dims))
    d = dims[axis]
    left = int(np.prod(dims[:axis])) if axis > 0 else 1
    rng = np.random.default_rng(1)
    A = np.ascontiguousarray(np.linalg.qr(rng.standard_normal((d, d)))[0].T)
    X = torch.randn(b, N, dtype=torch.float32, device="cuda")
    Y = torch.empty_like(X)
    ms = C.c_float(0)
    _abi.check(_abi.lib().kf_test_time_mode_product(path, C.c_void_p(X.data_ptr()), C.c_void_p(Y.data_ptr()),
                                                    A.ctypes.data_as(C.c_void_p), d, left, N, b, reps, None,
                                                    C.byref(ms)))
    return ms.value / 1e3


def time_gram(torch, ka, kb, N, reps=10, path=0):
    """Mean device time of one FP32 Gram product A'B (A: N x ka, B: N x kb; the Gram kernel with its
    fixed-order partial reduction), through the library's test-only timing entry point.  path 0:
    the solvers' choice (tcgen05 where the shapes fit), 1: the SIMT kernel."""
    import ctypes as C
    from kfgpu import _abi
    A = torch.randn(ka, N, dtype=torch.float32, device="cuda")
    B = torch.randn(kb, N, dtype=torch.float32, device="cuda")
    ms = C.c_float(0)
    _abi.check(_abi.lib().kf_test_time_gram(path, C.c_void_p(A.data_ptr()), N, ka, C.c_void_p(B.data_ptr()), N, kb,
                                            N, reps, None, C.byref(ms), None))
    return ms.value / 1e3


GRAM_SHAPES = ((16, 32), (32, 32), (16, 16), (16, 2), (2, 4))


def time_gram_tc(torch, widths, rr, N, reps=10):
    """Mean device time of one tensor-core Gram of a pool of FP32 blocks (the sources `widths`; rows
    of G from sources rr[0]..rr[1]-1, columns from rr[2]..rr[3]-1), with its reduction."""
    import ctypes as C
    from kfgpu import _abi
    blocks = [torch.randn(k, N, dtype=torch.float32, device="cuda") for k in widths]
    ns = len(blocks)
    ptrs = (C.c_void_p * ns)(*[b.data_ptr() for b in blocks])
    lds = (C.c_int64 * ns)(*[N] * ns)
    ks = (C.c_int32 * ns)(*widths)
    ms = C.c_float(0)
    _abi.check(_abi.lib().kf_test_gram_tc(C.cast(ptrs, C.c_void_p), C.cast(lds, C.c_void_p), C.cast(ks, C.c_void_p),
                                          ns, rr[0], rr[1], rr[2], rr[3], N, reps, None, C.byref(ms), None))
    return ms.value / 1e3


def time_update(torch, path, kx0, kx1, ky, N, reps=10):
    """Mean device time of one FP32 block update Y = [X0 X1] C (path 0: SIMT, 1: tcgen05, 2-4: tcgen05
    with the register gather, a two- or a three-tile staging ring), through the library's test-only
    timing entry point."""
    import ctypes as C
    from kfgpu import _abi
    X0 = torch.randn(kx0, N, dtype=torch.float32, device="cuda")
    X1 = torch.randn(max(kx1, 1), N, dtype=torch.float32, device="cuda")
    Y = torch.empty(ky, N, dtype=torch.float32, device="cuda")
    Cm = np.asfortranarray(np.random.default_rng(0).standard_normal((kx0 + kx1, ky)))
    ms = C.c_float(0)
    _abi.check(_abi.lib().kf_test_update(path, C.c_void_p(Y.data_ptr()), N, ky, C.c_void_p(X0.data_ptr()), N, kx0,
                                         C.c_void_p(X1.data_ptr()), N, kx1, Cm.ctypes.data_as(C.c_void_p), kx0 + kx1,
                                         1.0, 0.0, N, reps, None, C.byref(ms)))
    return ms.value / 1e3


UPDATE_SHAPES = ((32, 16, 32), (36, 18, 36), (18, 36, 36), (18, 36, 18), (16, 32, 16), (16, 0, 16), (2, 0, 1))


def time_update_f64(torch, path, kx, ky, N, reps=10):
    """Mean device time of one FP64 block update Y = X C (path 0: the FP64 kernel, 1: double-float
    arithmetic on the FP32 pipes), through the library's test-only timing entry point."""
    import ctypes as C
    from kfgpu import _abi
    X = torch.randn(kx, N, dtype=torch.float64, device="cuda")
    Y = torch.empty(ky, N, dtype=torch.float64, device="cuda")
    Cm = np.asfortranarray(np.random.default_rng(0).standard_normal((kx, ky)))
    ms = C.c_float(0)
    _abi.check(_abi.lib().kf_test_update_f64(path, C.c_void_p(Y.data_ptr()), C.c_void_p(X.data_ptr()), kx, ky,
                                             Cm.ctypes.data_as(C.c_void_p), N, reps, None, C.byref(ms)))
    return ms.value / 1e3


def run_update_workload(args):
    """The FP32 block updates of LOBPCG on N = 671,744 rows: tcgen05 (TF32 hi / lo) and SIMT."""
    import torch
    N = 671744
    peak, kind = peaks()
    out = {"workload": "FP32 block update Y = [X0 X1] C, N=671,744 rows", "hbm_peak_gbs": peak, "peak_kind": kind}
    from kfgpu._abi import ArgumentError
    for kx0, kx1, ky in UPDATE_SHAPES:
        for path, name in ((1, "tc"), (2, "tc_gather"), (3, "tc_ring2"), (4, "tc_ring3"), (0, "simt")):
            try:
                t = time_update(torch, path, kx0, kx1, ky, N)
            except ArgumentError:
                continue   # the shape does not fit that producer mode
            key = f"update_{kx0}+{kx1}_to_{ky}_{name}"
            out[key + "_us"] = t * 1e6
            out[key + "_gbs"] = (kx0 + kx1 + ky) * N * 4 / t / 1e9
    for path, name in ((0, "f64"), (1, "double_float")):
        t = time_update_f64(torch, path, 18, 18, N)
        out[f"update_f64_18_to_18_{name}_us"] = t * 1e6
        out[f"update_f64_18_to_18_{name}_gbs"] = 36 * N * 8 / t / 1e9
    return out


def run_gram_workload(args):
    """The FP32 Gram products of LOBPCG's orthogonalisation and Rayleigh-Ritz on N = 671,744 rows."""
    import torch
    N = 671744
    peak, kind = peaks()
    out = {"workload": "FP32 Gram A'B, N=671,744 rows", "hbm_peak_gbs": peak, "peak_kind": kind}
    for ka, kb in GRAM_SHAPES + ((20, 40), (48, 48)):
        for path, name in ((0, "gram"), (1, "simt")):
            t = time_gram(torch, ka, kb, N, path=path)
            out[f"{name}_{ka}x{kb}_us"] = t * 1e6
            out[f"{name}_{ka}x{kb}_gbs"] = (ka + kb) * N * 4 / t / 1e9
    # the solve's tensor-core pools: [X Z]'Z of the orthogonalisation and the merged Rayleigh-Ritz
    # [X_a Q]'[HX_a HZ] (block 18 = 12 + 4 guards + 2 buffer columns)
    for name, widths, rr in (("xz", (18, 36), (0, 2, 1, 2)), ("rr", (18, 36, 18, 36), (0, 2, 2, 4))):
        t = time_gram_tc(torch, widths, rr, N)
        out[f"tc_pool_{name}_us"] = t * 1e6
        out[f"tc_pool_{name}_gbs"] = sum(widths) * N * 4 / t / 1e9
    return out


MODE_COLS = 18   # the active block of a solve with m = 12, 4 guards, 2 buffer columns


def run_mode_workload(args):
    """The separable preconditioner's mode products on the three-mode leaf grid (18 FP32 columns, the
    active block of a solve): tensor cores (tcgen05, BF16 operands) and the SIMT FP32 kernel, per
    non-diagonal axis."""
    import torch
    dims = (41, 256, 64)
    N = int(np.prod(dims))
    peak, kind = peaks()
    out = {"workload": f"mode products, three-mode grid 41x256x64 (N=671,744), {MODE_COLS} FP32 columns"}
    for axis in (1, 2):
        for path, name in ((1, "tc"), (0, "simt")):
            t = time_mode_product(torch, path, dims, axis, b=MODE_COLS)
            by = 2 * N * MODE_COLS * 4
            out[f"axis{axis}_{name}_us"] = t * 1e6
            out[f"axis{axis}_{name}_gbs"] = by / t / 1e9
            out[f"axis{axis}_{name}_tflops"] = 2 * N * dims[axis] * MODE_COLS / t / 1e12
    out["hbm_peak_gbs"] = peak
    out["peak_kind"] = kind
    return out


def run_batch_workload(args):
    """Batched theta sweep: 512 fluxonium leaves (n ~ U{200..1600} on [-5 pi, 5 pi], 5-point stencil,
    keep 10) plus 64 chains of 2-4 leaves (g ~ U[0.01, 0.1] n_i n_{i+1}, parents keep 20), all leaves
    in one persistent graph-captured launch (CTA size from the autotuner), then the parents."""
    import torch
    from kfgpu import KronFreeOperator, LOBPCG, circuits, ops as P, solve
    from kfgpu.batch import autotune, batch_solve
    from kfgpu.ops import PhaseGrid, localop
    rng = np.random.default_rng(SEED + 2)
    leaves = []
    for _ in range(512):
        th = circuits.fluxonium_theta(rng)
        leaves.append((th, int(rng.integers(200, 1601))))
    chains = []
    for _ in range(64):
        k = int(rng.integers(2, 5))
        chains.append(([(circuits.fluxonium_theta(rng), int(rng.integers(200, 1601))) for _ in range(k)],
                       [rng.uniform(0.01, 0.1) for _ in range(k - 1)]))
    all_leaves = leaves + [lf for c, _ in chains for lf in c]
    ops = []
    for th, n in all_leaves:
        dims, terms = circuits.fluxonium_leaf(th, n)
        ops.append((dims, terms, 0.0))
    m = [10] * len(ops)
    tol = 1e-8 * 2e3            # 1e-8 ||H|| for the coarsest leaves' Gershgorin bound scale
    tile = autotune(ops[:64], m[:64], tol)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    Es, Vs, iters, resid = batch_solve(ops, m, tol)
    t_leaves = time.perf_counter() - t0
    # parents of the chains
    t1 = time.perf_counter()
    k0 = len(leaves)
    nparent_pairs = 0
    for c, gs in chains:
        idx = list(range(k0, k0 + len(c)))
        k0 += len(c)
        dims = [10] * len(c)
        terms = [(1.0, [(a, P.DiagonalOp(Es[i]))]) for a, i in enumerate(idx)]
        ports = []
        for i in idx:
            n = all_leaves[i][1]
            A = localop(PhaseGrid(-5 * np.pi, 5 * np.pi, n, 4), "n", part="im").dense()
            ports.append(Vs[i].T @ A @ Vs[i])
        for a in range(len(c) - 1):
            terms.append((-gs[a], [(a, P.DenseOp(ports[a])), (a + 1, P.DenseOp(ports[a + 1]))]))
        H = KronFreeOperator(dims, terms, block_capacity=24)
        Ep, Vp, st = solve(LOBPCG(tol=1e-8 * H.gershgorin_bound(), precision="mixed"), H, 20)
        nparent_pairs += 20
        H.close()
    t_parents = time.perf_counter() - t1
    return {"workload": "batched theta sweep: 512 fluxonium leaves + 64 chains of 2-4 (704 leaves in one launch)",
            "leaves": len(ops), "leaf_pairs_per_s": 10 * len(ops) / t_leaves, "leaf_seconds": t_leaves,
            "parents": len(chains), "parent_seconds": t_parents,
            "pairs_per_s_total": (10 * len(ops) + nparent_pairs) / (t_leaves + t_parents),
            "tuned_threads_per_cta": tile, "max_leaf_iterations": int(iters.max()),
            "mean_leaf_iterations": float(iters.mean()), "max_residual": float(resid.max())}


def run_warmstart_workload(args):
    """Learned warm start on the two-transmon circuit (flat 61 x 61): label n_train theta with the
    plain solver, POD 128, train 7 -> 256 -> 256 -> 1536 with the library's kernels, then LOBPCG on
    n_test held-out theta: warm-started vs random start."""
    from kfgpu import warmstart as W
    t0 = time.perf_counter()
    train = W.sample_thetas(args.n_train, seed=SEED + 3)
    Vs, _ = W.label(train)
    t_label = time.perf_counter() - t0
    POD = W.pod_basis(Vs, k=128)
    ws = W.WarmStart(POD, 12, hidden=256, seed=1)
    t1 = time.perf_counter()
    losses = ws.fit(train, W.targets(Vs, POD), epochs=args.epochs, batch=256, lr=1e-3)
    t_train = time.perf_counter() - t1
    rows = W.evaluate(ws, W.sample_thetas(args.n_test, seed=SEED + 4))
    wi = np.array([r["warm_iters"] for r in rows]); ri = np.array([r["random_iters"] for r in rows])
    wt = np.array([r["warm_s"] for r in rows]); rt = np.array([r["random_s"] for r in rows])
    return {"workload": "learned warm start, two transmons flat 61x61 (N=3,721), m=12",
            "n_train": args.n_train, "n_test": args.n_test, "label_seconds": t_label, "train_seconds": t_train,
            "loss_first_last": [float(losses[0]), float(losses[-1])],
            "warm_mean_iterations": float(wi.mean()), "random_mean_iterations": float(ri.mean()),
            "warm_mean_seconds": float(wt.mean()), "random_mean_seconds": float(rt.mean()),
            "warm_pairs_per_s": 12 / float(wt.mean()), "random_pairs_per_s": 12 / float(rt.mean()),
            "fell_back": int(sum(r["fell_back"] for r in rows)),
            "max_abs_dE": float(max(r["max_dE"] for r in rows))}


def run_dense_workload(args):
    """Three children of 48 kept states (N = 110,592) with dense pairwise port couplings; the lowest
    30 pairs, mixed vs FP64 (eigenvalue differences and FP64 residuals)."""
    import torch
    from kfgpu import KronFreeOperator, LOBPCG, circuits, solve
    out = {"workload": "dense parent 48^3 (N=110,592), 3 dense pair couplings, m=30 block 32"}
    rng = np.random.default_rng(SEED + 5)
    dims, terms = circuits.dense_parent(rng, d=48)
    H = KronFreeOperator(dims, terms, block_capacity=32)
    tol = 1e-8 * H.gershgorin_bound()
    res = {}
    for prec in ("mixed", "f64"):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        E, V, st = solve(LOBPCG(tol=tol, precision=prec, guard=2), H, 30)
        res[prec] = (E, time.perf_counter() - t0, st)
    out.update({"mixed_pairs_per_s": 30 / res["mixed"][1], "f64_pairs_per_s": 30 / res["f64"][1],
                "mixed_iterations": res["mixed"][2]["iterations"], "f64_iterations": res["f64"][2]["iterations"],
                "max_rel_dE_mixed_vs_f64": float(np.max(np.abs(res["mixed"][0] - res["f64"][0]) / np.abs(res["f64"][0]))),
                "max_residual_rel": float(res["mixed"][2]["max_residual"] / H.gershgorin_bound())})
    # the dense apply alone (32 columns, FP32 and FP64): flops counted as 6 mode products per column
    for f32 in (True, False):
        t = measure_apply(torch, H, f32, b=32)
        flops = 6 * 2 * 48 * H.N * 32
        out["apply_%s_us" % ("f32" if f32 else "f64")] = t * 1e6
        out["apply_%s_tflops" % ("f32" if f32 else "f64")] = flops / t / 1e12
    return out


def cpu_baseline(theta, bounded=True, iters=None):
    """The oracle's restatement of the reference CPU path on the host cores: a bounded sample of
    LOBPCG iterations of the same solve (C/OpenMP mul! + NumPy LOBPCG), extrapolated to the
    iteration count the same algorithm needs (measured here on the GPU's FP64 run when given,
    else the sample's own count)."""
    from oracle import capply, circuits as oc, solvers as osol
    H = oc.three_mode_operator(theta)
    CA = capply.CApply(H)

    class Fast:
        N, dtype = H.N, H.dtype

        def matvec(self, X):
            return CA.matvec(X)

        def full_diagonal(self):
            return H.full_diagonal()

    tol = 1e-8 * H.gershgorin_bound()
    X0 = osol.perturbed_seed(H.product_seed(M_PAIRS + 4))
    D = H.full_diagonal()
    n_it = 8 if bounded else 100000
    t0 = time.perf_counter()
    r = osol.lobpcg_core(Fast(), X0, D, tol, n_it, "ritz", 0.01)
    dt = time.perf_counter() - t0
    per_it = dt / max(r["iters"], 1)
    need = iters if iters else r["iters"]
    cores = os.cpu_count()
    return {"value": M_PAIRS / (per_it * need), "unit": "eigenpairs/s", "cores": cores, "kind": "port",
            "sample": f"{r['iters']} LOBPCG iterations of the N=671,744 solve in {dt:.1f} s "
                      f"({per_it:.2f} s/iteration, OpenMP threads={cores}), extrapolated to {need} iterations"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return None
    ths = thetas()
    K, W = args.steps, args.warmup
    vals = []
    for k in range(W + K):
        cb = cpu_baseline(ths[k % NDRAWS], bounded=True, iters=args.ref_iters)
        if k >= W:
            vals.append(cb)
    v = float(np.mean([c["value"] for c in vals]))
    return {"metric": "converged eigenpairs/s at 1e-8 resid: warm-start mixed vs plain FP64, 1 GB300",
            "impl": "reference", "value": v, "unit": "eigenpairs/s", "n_gpus": 0, "steps": K, "warmup": W,
            "higher_is_better": True, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "three-mode leaf 41x256x64 (N=671,744), LOBPCG m=12 block=16, product seed"},
            "cpu_baseline": {"value": v, "unit": "eigenpairs/s", "cores": vals[0]["cores"], "kind": "port",
                             "sample": vals[0]["sample"]},
            "e2e": {"value": v, "unit": "eigenpairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--plain-steps", type=int, default=2)
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--ref-iters", type=int, default=868,
                    help="LOBPCG iterations the plain FP64 solve of this workload takes, for the reference arm's "
                         "extrapolation (868: the mean over the first two timed draws measured on GB300)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--buffer", type=int, default=None,
                    help="unchecked LOBPCG columns beyond the guards in the mixed solves (default: the library's)")
    ap.add_argument("--workload", default="leaf3",
                    choices=["leaf3", "batch", "warmstart", "dense", "apply", "mode", "gram", "update"],
                    help="leaf3 (the benchmarked workload) or one of the other measured configurations")
    ap.add_argument("--n-train", type=int, default=4096)
    ap.add_argument("--n-test", type=int, default=1024)
    ap.add_argument("--epochs", type=int, default=200)
    ap.add_argument("--profile", action="store_true",
                    help="one mixed-precision solve of the first timed draw, no warm-up (for the ncu launch list)")
    args = ap.parse_args()
    if args.profile:
        print(json.dumps(profile_one(args)), flush=True)
        return
    if args.workload != "leaf3":
        fn = {"batch": run_batch_workload, "warmstart": run_warmstart_workload, "dense": run_dense_workload,
              "apply": run_apply_workload, "mode": run_mode_workload, "gram": run_gram_workload,
              "update": run_update_workload}
        print(json.dumps(fn[args.workload](args)), flush=True)
        return
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        line = run_reference(args)
    else:
        D = Dist()
        try:
            line = run_ours(args, D)
        finally:
            D.close()
    if line is not None:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
