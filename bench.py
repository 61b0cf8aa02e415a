#!/usr/bin/env python
"""Benchmark: HODLR factor + solve at N = 2^20 (leaf 128, 13 levels, rank 32,
64 right-hand sides) on one GB300.

Our arm (default): the mixed-precision path (FP32 leaf LU / low-rank GEMMs,
FP64 capacitance LU, FP64-accurate residual + iterative refinement to a
relative residual of 1e-12) on the ill-conditioned Gaussian workload
(orthonormalised factors, s_i = 10^(-6 i / r), leaf shift 1.5), timed per
step = factor + solve with inputs resident in HBM.  The plain FP64 GPU path is
timed on the same inputs beside it.  One JSON line on stdout.

--impl reference: the reference's own CPU algorithm on the host cores --
fastSolver2's hsolve with its dgemm_/dgesv_ calls on single-threaded OpenBLAS,
threaded the way its Legion index launch splits subtrees -- solving the whole
N = 2^20 system in every one of the K + W steps.

Multi-GPU (torchrun): the solve does not shard in this build, so each rank
solves its own independent system (replicas); the line reports the max over
ranks.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "HODLR factor+solve ms at N=2^20 (mixed vs FP64 on GPU, rel. resid ≤1e-12)"
WORKLOAD = dict(n=1 << 20, leaf=128, levels=13, rank=32, nrhs=64)
SMALL = dict(n=1 << 14, leaf=128, levels=7, rank=32, nrhs=64)
SEED = 20261203


def algo_flops(n, m, L, r, k):
    """Algorithmic FP64 flop counts of factor and solve (the hsolve one-shot count)."""
    F = (2 / 3) * n * m * m + 2 * n * m * L * r + sum(
        2 * n * r * r + 4 * n * r * r * l + (2 ** l) * ((16 / 3) * r ** 3 + 8 * r ** 3 * l) for l in range(L))
    S = 2 * n * m * k + sum(4 * n * r * k + 8 * (2 ** l) * r * r * k for l in range(L))
    return F, S


def algo_bytes(n, m, L, r, k, w=8):
    """Compulsory traffic of factor and solve at element width w."""
    caps = (2 ** L) * (2 * r) ** 2 * w
    return (2 * n * m + 3 * n * r * L) * w + caps, (n * m + 2 * n * r * L + 2 * n * k) * w + caps


def ragged_systems(count=512, seed=SEED):
    """Ragged batch: N log-uniform in [2^10, 2^16] rounded to a power of two,
    leaf m in {64, 128, 256} with m <= N/2, rank r in {8, 16, 32, 64} with
    r < m, 1..8 right-hand sides.  Returns [(n, leaf, levels, rank, nrhs)]."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        e = int(round(rng.uniform(10.0, 16.0)))
        n = 1 << e
        m = int(rng.choice([x for x in (64, 128, 256) if x <= n // 2]))
        r = int(rng.choice([x for x in (8, 16, 32, 64) if x < m]))
        k = int(rng.integers(1, 9))
        L = (n // m).bit_length() - 1
        out.append((n, m, L, r, k))
    return out


def ragged_flops(systems):
    return sum(sum(algo_flops(n, m, L, r, k)) for n, m, L, r, k in systems)


def resid_flops(n, m, L, r, k):
    return 2 * n * m * k + 4 * n * r * k * L


# ---------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, ValueError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------- CPU leg
def workload_config(wl, world):
    """The config dict both arms print (the workload, not the implementation)."""
    return {"workload": "HODLR N=%d leaf %d L=%d rank %d nrhs %d, orthonormal-class factors s_i=10^(-6i/%d), "
                        "leaf shift 1.5; factor+solve to rel. resid <=1e-12"
                        % (wl["n"], wl["leaf"], wl["levels"], wl["rank"], wl["nrhs"], wl["rank"]),
            **wl, "parallelism": "replicas" if world > 1 else "one system per device",
            "l2": "inputs larger than L2 (>4 GB touched per step)"}


def cpu_problem(wl, seed, threads):
    """Host inputs of the workload for the CPU leg: leaf blocks G/sqrt(m) + 1.5 I,
    per-level U, V Gaussian / sqrt(block rows) (the scale of orthonormal
    blocks; the solve's flops do not depend on the values), s_i = 10^(-6 i/r)
    folded into V, b Gaussian.  Returns (K0, W0 = [b | U^(0) | ...], Vs)."""
    from oracle import oracle as O
    n, m, L, r, k = wl["n"], wl["leaf"], wl["levels"], wl["rank"], wl["nrhs"]
    K0 = np.empty((n, m), order="F")
    O.fill_gaussian(K0, seed, 1.0 / np.sqrt(m), 1.5, m, threads)
    W0 = np.empty((n, k + L * r), order="F")
    O.fill_gaussian(W0[:, :k], seed + 1, 1.0, 0.0, 0, threads)
    sv = 10.0 ** (-6.0 * np.arange(r) / r)
    Vs = []
    for l in range(L):
        nb = n >> (l + 1)
        O.fill_gaussian(W0[:, k + l * r:k + (l + 1) * r], seed + 2 + 2 * l, 1.0 / np.sqrt(nb), 0.0, 0, threads)
        V = np.empty((n, r), order="F")
        O.fill_gaussian(V, seed + 3 + 2 * l, 1.0 / np.sqrt(nb), 0.0, 0, threads)
        V *= sv[None, :]
        Vs.append(V)
    return K0, W0, Vs


def cpu_solve_runs(wl, steps, warmup, threads=None, seed=SEED):
    """Full-size solves of the reference algorithm on the host cores: fastSolver2's
    hsolve (src/tasks/leaf_solve.cc:73-154) with its dgemm_/dgesv_ calls on
    single-threaded OpenBLAS (bitwise the reference's own build on the same BLAS),
    the 2^p subtrees under depth p on P = 2^p threads and the top p levels as
    row-chunked reduce / capacitance / update steps (the reference's index
    launch).  Every step solves the whole N; the in-place inputs are restored
    between steps outside the timing.  Returns (ms per step list, threads
    used, relative residual of the last solution, kind, sample text)."""
    from oracle import oracle as O
    threads = threads or (os.cpu_count() or 1)
    P = 1
    while P * 2 <= threads and P * 2 <= (1 << wl["levels"]):
        P *= 2
    n, m, L, r, k = wl["n"], wl["leaf"], wl["levels"], wl["rank"], wl["nrhs"]
    if O.blas_lib() is None:
        raise RuntimeError("scipy's OpenBLAS is not available for the CPU leg")
    K0, W0, Vs = cpu_problem(wl, seed, threads)
    K, W = np.empty_like(K0, order="F"), np.empty_like(W0, order="F")
    times = []
    for i in range(warmup + steps):
        O.copy_mt(K, K0, threads)
        O.copy_mt(W, W0, threads)
        t0 = time.perf_counter()
        info = O.blas_hsolve_mt(m, L, r, K, Vs, W, k, P)
        dt = time.perf_counter() - t0
        if info != 0:
            raise RuntimeError("reference hsolve failed: info %d" % info)
        if i >= warmup:
            times.append(dt * 1e3)
    X = np.asfortranarray(W[:, :k])
    Us = [W0[:, k + l * r:k + (l + 1) * r] for l in range(L)]
    Y = O.blas_matvec(m, L, r, K0, Us, Vs, None, X, threads)
    B = W0[:, :k]
    resid = float((np.linalg.norm(B - Y, axis=0) / np.linalg.norm(B, axis=0)).max())
    sample = ("fastSolver2's hsolve restated with its dgemm_/dgesv_ calls on single-threaded OpenBLAS (bitwise the "
              "reference's own build on that BLAS), whole N=%d system every step, %d subtrees on %d threads + the "
              "top %d levels row-chunked over them; %d steps after %d warm-up" %
              (n, P, P, P.bit_length() - 1, steps, warmup))
    return times, P, resid, "port", sample


def run_reference(args, wl):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return 0
    t_wall = time.perf_counter()
    times, threads, resid, kind, sample = cpu_solve_runs(wl, args.steps, args.warmup)
    wall = time.perf_counter() - t_wall
    value = float(np.mean(times))
    line = {"metric": METRIC, "value": value, "unit": "ms", "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": value, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Gaussian)",
            "config": workload_config(wl, world),
            "cpu_baseline": {"value": value, "unit": "ms", "cores": threads, "kind": kind, "sample": sample},
            "e2e": {"value": value, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "step_ms": {"median": float(np.median(times)), "min": float(np.min(times)),
                        "max": float(np.max(times))},
            "rel_resid": resid, "host_cores": os.cpu_count(), "wall_s": wall}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------- GPU arm
def run_ours(args, wl):
    import torch
    import fastsolver2_gb300 as fs

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    fs.lib()

    n, m, L, r, k = wl["n"], wl["leaf"], wl["levels"], wl["rank"], wl["nrhs"]
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    dev = "cuda"

    def colmajor(rows, cols):
        return torch.empty((cols, rows), dtype=torch.float64, device=dev).t()

    launches0 = fs.kernel_launches()
    ffma_tf, dfma_tf, mma_tf = probe_peaks()   # live FMA-pipe and warp-level bf16 MMA rates
    with torch.cuda.stream(stream):
        # FLAG_STREAM_INPUTS: in the e2e leg the host V of each level is copied
        # by the factorisation, beside the levels below it
        mixed = fs.Solver(n, m, L, r, nrhs_max=k, precision=fs.PREC_MIXED, residual=args.resid,
                          refine_tol=1e-12, refine_max_iter=10, stream=sp,
                          flags=0 if args.plain_inputs else fs.FLAG_STREAM_INPUTS)
        B0 = colmajor(n, k)
        mixed.generate(SEED + rank, shift=1.5, orthonormal=True, decay=6.0, B=B0)
        B = colmajor(n, k)
        tuning = None if args.no_tune else mixed.autotune(nrhs=k)

        def step():
            B.copy_(B0)
            mixed.factor()
            return mixed.solve(B)

        # the timed region: the graphs as a user runs them (no per-phase event nodes)
        mixed.profile(0)
        for _ in range(args.warmup):
            step()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        clocks = ClockSampler(local)
        clocks.start()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0 = fs.kernel_launches()
        t_wall = time.perf_counter()
        e0.record(stream)
        iters = []
        for _ in range(args.steps):
            info = step()
            iters.append(info.iterations)
        e1.record(stream)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        wall = time.perf_counter() - t_wall
        launches = fs.kernel_launches() - l0
        clk = clocks.stop()
        ms = e0.elapsed_time(e1) / args.steps
        final_resid_dev = info.rel_residual
        # a second pass of the same steps with per-phase CUDA events recorded
        # as event nodes inside the graphs (captured outside this pass): the
        # per-phase times of the roofline
        ms_events = None
        phases = {}
        if not args.no_phase_timing:
            mixed.profile(1)
            for _ in range(2):
                step()
            mixed.profile(-1, read=True)
            torch.cuda.synchronize()
            p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            p0.record(stream)
            for _ in range(args.steps):
                step()
            p1.record(stream)
            torch.cuda.synchronize()
            ms_events = p0.elapsed_time(p1) / args.steps
            phases = mixed.profile(0, read=True)

        # independent FP64 check of the mixed result: max_j ||b_j - A x_j|| / ||b_j||
        fp64 = fs.Solver(n, m, L, r, nrhs_max=k, precision=fs.PREC_FP64, stream=sp)
        fp64.generate(SEED + rank, shift=1.5, orthonormal=True, decay=6.0, B=None)
        AX = colmajor(n, k)
        fp64.matvec(B, AX)
        torch.cuda.synchronize()
        check = ((B0 - AX).norm(dim=0) / B0.norm(dim=0)).max().item()

        # the plain FP64 GPU path on the same inputs
        Bd = colmajor(n, k)
        fp64_ms = [float("nan")] if args.no_fp64 else []
        for i in range(0 if args.no_fp64 else args.fp64_steps + 1):
            Bd.copy_(B0)
            f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            f0.record(stream)
            fp64.factor()
            fp64.solve(Bd)
            f1.record(stream)
            torch.cuda.synchronize()
            if i > 0:
                fp64_ms.append(f0.elapsed_time(f1))
        fp64_factor_ms, fp64_solve_ms = fp64.timings()
        fp64_resid = None
        if not args.no_fp64:
            fp64_AX = colmajor(n, k)
            fp64.matvec(Bd, fp64_AX)
            torch.cuda.synchronize()
            fp64_resid = ((B0 - fp64_AX).norm(dim=0) / B0.norm(dim=0)).max().item()
            del fp64_AX
        del fp64, AX, Bd

        # end to end through the C ABI with host buffers: H2D of the problem and
        # the right-hand sides, factor, solve, D2H of the solution
        e2e = None
        if not args.no_e2e:
            nleaf = 1 << L
            # pinned host buffers on the GPU's NUMA node: cudaHostAlloc touches
            # the pages from the calling thread, so it runs on that node's CPUs
            numa = host_numa_binding(local)
            pin = dict(dtype=torch.float64, pin_memory=True)
            hD = torch.empty(nleaf * m * m, **pin)
            hU = torch.empty(L * n * r, **pin)
            hV = torch.empty(L * n * r, **pin)
            hs = torch.empty(max(L, 1) * r, **pin)
            hB = torch.empty((k, n), **pin).t()
            hX = torch.empty((k, n), **pin).t()
            numa["host_buffer_nodes"] = numa_nodes_of([hD, hU, hV, hB, hX])
            restore_affinity(numa)
            mixed.get_inputs(D=hD, U=hU, V=hV, s=hs)
            hB.copy_(B0)
            torch.cuda.synchronize()
            lib = fs.lib()
            Be = colmajor(n, k)

            # events between the parts of each step: inputs set (host copies
            # + preparation), factor, solve, read-back
            pev = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(args.e2e_steps)]

            def e2e_step(ev=None):
                fs.check(lib.hodlr_set_leaf_blocks(mixed.h, hD.data_ptr(), m, m * m))
                for l in range(L):
                    off = l * n * r * 8
                    fs.check(lib.hodlr_set_lowrank(mixed.h, l, hU.data_ptr() + off, n, hV.data_ptr() + off, n,
                                                   hs.data_ptr() + l * r * 8))
                Be.copy_(hB, non_blocking=True)
                if ev:
                    ev[0].record(stream)
                mixed.factor()
                if ev:
                    ev[1].record(stream)
                mixed.solve(Be)
                if ev:
                    ev[2].record(stream)
                hX.copy_(Be, non_blocking=True)
                if ev:
                    ev[3].record(stream)
                stream.synchronize()

            # warm-up: the first factor and solve after the phase pass run
            # eagerly, the second capture their graphs -- both outside the timing
            for _ in range(max(2, args.warmup)):
                e2e_step()
            torch.cuda.synchronize()
            g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            g0.record(stream)
            for i in range(args.e2e_steps):
                e2e_step(pev[i])
            g1.record(stream)
            torch.cuda.synchronize()
            h2d = (hD.numel() + hU.numel() + hV.numel() + L * r + n * k) * 8
            e2e = {"value": g0.elapsed_time(g1) / args.e2e_steps, "unit": "ms", "h2d_bytes_per_step": h2d,
                   "d2h_bytes_per_step": n * k * 8, "steps": args.e2e_steps}
            # per step (medians): inputs set (host copies + preparation, from the
            # previous step's end), factor, solve, read-back of the solution
            starts = [g0] + [ev[3] for ev in pev[:-1]]
            parts = [[a.elapsed_time(b) for a, b in zip([st] + ev[:3], ev)] for st, ev in zip(starts, pev)]
            names = ("set_inputs", "factor", "solve", "readback")
            e2e["parts_ms"] = {name: {"median": float(np.median([p[i] for p in parts])),
                                      "min": float(np.min([p[i] for p in parts])),
                                      "max": float(np.max([p[i] for p in parts]))}
                               for i, name in enumerate(names)}
            per_step = [float(sum(p)) for p in parts]
            e2e["per_step_ms"] = per_step
            e2e["step_ms"] = {"mean": float(np.mean(per_step)), "median": float(np.median(per_step)),
                              "min": float(np.min(per_step)), "max": float(np.max(per_step))}
            # the bare host-to-device copies of the same buffers, in the same
            # run: the host link's share of the set_inputs part
            dD, dU, dV = torch.empty_like(hD, device=dev), torch.empty_like(hU, device=dev), \
                torch.empty_like(hV, device=dev)
            bare = []
            for _ in range(5):
                c0, c1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                c0.record(stream)
                dD.copy_(hD, non_blocking=True)
                dU.copy_(hU, non_blocking=True)
                dV.copy_(hV, non_blocking=True)
                Be.copy_(hB, non_blocking=True)
                c1.record(stream)
                stream.synchronize()
                bare.append(c0.elapsed_time(c1))
            e2e["bare_h2d_ms"] = {"median": float(np.median(bare)), "min": float(np.min(bare)),
                                  "max": float(np.max(bare)),
                                  "gb_per_s": h2d / (float(np.median(bare)) * 1e-3) / 1e9}
            e2e["numa"] = numa
            # the same set calls from device buffers: device copies plus the
            # preparation of the derived copies (FP32 V, digit slices), which
            # runs on the handle's side stream -- timed on the host around a
            # device-wide synchronisation
            torch.cuda.synchronize()

            def set_from_device():
                fs.check(lib.hodlr_set_leaf_blocks(mixed.h, dD.data_ptr(), m, m * m))
                for l in range(L):
                    off = l * n * r * 8
                    fs.check(lib.hodlr_set_lowrank(mixed.h, l, dU.data_ptr() + off, n, dV.data_ptr() + off, n,
                                                   hs.data_ptr() + l * r * 8))
                torch.cuda.synchronize()

            set_from_device()
            sd = []
            for _ in range(3):
                t0 = time.perf_counter()
                set_from_device()
                sd.append((time.perf_counter() - t0) * 1e3)
            e2e["set_from_device_buffers_ms"] = float(np.median(sd))
            del dD, dU, dV

        # the same tree with the plain Gaussian generators (leaf shift 4): FP64 and mixed
        gauss = None
        if not args.no_fp64:
            del mixed
            gauss = {"workload": "N=2^20 leaf 128 L=13 rank 32 nrhs 64, Gaussian U, V / sqrt(block rows), "
                                 "leaves G/sqrt(128) + 4I"}
            Bg0 = colmajor(n, k)
            for prec, name in ((fs.PREC_FP64, "fp64"), (fs.PREC_MIXED, "mixed")):
                g = fs.Solver(n, m, L, r, nrhs_max=k, precision=prec, residual=args.resid, stream=sp)
                g.generate(SEED + 1, shift=4.0, orthonormal=False, decay=0.0, B=Bg0)
                Bg = colmajor(n, k)
                times = []
                for i in range(3):
                    Bg.copy_(Bg0)
                    h0, h1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    h0.record(stream)
                    g.factor()
                    ginfo = g.solve(Bg)
                    h1.record(stream)
                    torch.cuda.synchronize()
                    if i > 0:
                        times.append(h0.elapsed_time(h1))
                gauss[name] = {"ms_per_step": float(np.mean(times)), "refine_iterations": ginfo.iterations}
                if prec == fs.PREC_FP64:
                    GX = colmajor(n, k)
                    g.matvec(Bg, GX)
                    torch.cuda.synchronize()
                    gauss[name]["rel_resid"] = ((Bg0 - GX).norm(dim=0) / Bg0.norm(dim=0)).max().item()
                    del GX
                else:
                    gauss[name]["rel_resid"] = ginfo.rel_residual
                g.close()
            del Bg0, Bg
        dense_check = small_config_dense_check(fs, torch)
        adjoint = run_adjoint(fs, torch, stream, colmajor)
        ragged = None if args.no_ragged else run_ragged(args, fs, torch, stream, colmajor)

    # ---- report (max over ranks)
    ms = max_over_ranks(ms, dev)
    if e2e is not None:
        e2e["value"] = max_over_ranks(e2e["value"], dev)
    F, S = algo_flops(n, m, L, r, k)
    nres = float(np.mean(iters)) + 1.0
    total_ms = sum(v[0] for v in phases.values())
    # per-phase algorithmic work of one mixed step, split by the pipe that
    # bounds it: (FP64 flops at this GPU's DFMA rate, FP32 flops at its FFMA
    # rate, FP64-equivalent flops of the digit-product residual at the bf16
    # MMA rate / 28 digit pairs); frac = that roofline time / the measured
    # time, so a phase that mixes pipes (the capacitance step: FP64 LU, FP32
    # inverse and application) is rated against each pipe for its own part
    nsw = float(np.mean(iters)) + 1.0        # sweeps = residual evaluations per solve
    cap_lu = sum((2 ** l) * (2 / 3) * (2 * r) ** 3 for l in range(L))
    cap_fp32 = (sum((2 ** l) * (2 * (2 * r) ** 3 + 2 * (2 * r) ** 2 * l * r) for l in range(L))
                + nsw * sum((2 ** l) * 2 * (2 * r) ** 2 * k for l in range(L)))
    resid_pipe = {0: "fp64", 1: "dw", 2: "mma"}[args.resid]
    work = {  # name: {pipe: flops}
        "leaf_lu": {"fp32": (2 / 3) * n * m * m + 2 * n * m * m},
        # the factorisation's application D^-1 U runs on the tensor cores and
        # is bounded by its bytes (U in FP64, Utilde in FP32, Dinv); the
        # solve's applications to the right-hand sides by the FFMA rate
        "leaf_solve": {"hbm": n * L * r * (8 + 4) + n * m * 4, "fp32": nsw * 2 * n * m * k},
        "reduce": {"fp32": sum(2 * n * r * (l + 1) * r for l in range(L)) + nsw * 2 * n * r * k * L},
        "update": {"fp32": sum(2 * n * r * l * r for l in range(L)) + nsw * 2 * n * r * k * L},
        "capacitance": {"fp64": cap_lu, "fp32": cap_fp32},
        "resid_leaf": {resid_pipe: nsw * 2 * n * m * k},
        "resid_reduce": {resid_pipe: nsw * 2 * n * r * k * L},
        "resid_update": {resid_pipe: nsw * 2 * n * r * k * L},
    }
    dw_tf = ffma_tf / 12.0   # a double-word FMA is 12 FP32 instructions
    # "hbm" work is bytes and its peak TB/s (10^12 bytes / s), the others flops and TFLOP/s
    pipe_peak = {"fp64": dfma_tf, "fp32": ffma_tf, "dw": dw_tf, "mma": mma_tf / OZ_PAIRS,
                 "hbm": (_measured_peak("hbm_gbs") or 6800.0) / 1e3}
    phase_report = {}
    for name, (pms, pn) in phases.items():
        per_step = pms / args.steps
        ent = {"ms_per_step": per_step, "launches_per_step": pn / args.steps}
        if name in work and per_step > 0:
            w = work[name]
            t_bound = sum(f / (pipe_peak[pp] * 1e12) for pp, f in w.items()) * 1e3
            ent.update(tflops=sum(f for pp, f in w.items() if pp != "hbm") / (per_step * 1e-3) / 1e12,
                       bound_ms=t_bound, frac=t_bound / per_step,
                       pipes={pp: pipe_peak[pp] for pp in w})
        phase_report[name] = ent
    # the kernels of the dominant phases: (phases, bound, peak, native work
    # factor, ncu DRAM bytes per launch)
    bf16_peak = _measured_peak("bf16_tflops")
    if args.resid == 2:
        # tcgen05: the residual (leaf term and every level's update in one
        # pass) and the reductions of every level in one pass
        resid_kernels = {
            "oz_tc_kernel<0>": (("resid_leaf", "resid_update"), "tensor", bf16_peak, OZ_PAIRS,
                                TRAFFIC.get("oz_tc_kernel<0>")),
            "oz_tc_kernel<1>": (("resid_reduce",), "tensor", bf16_peak, OZ_PAIRS, TRAFFIC.get("oz_tc_kernel<1>")),
        }
    else:
        resid_kernels = {
            "dw_update_kernel": (("resid_leaf", "resid_update"), "fp32_fma_pipe", dw_tf, 1.0,
                                 8 * (100.77e6 + 16.15e6)),
            "dw_reduce_kernel": (("resid_reduce",), "fp32_fma_pipe", dw_tf, 1.0, 8 * (100.69e6 + 3.11e6)),
        }
    kernels = dict(resid_kernels)
    # the FP32 low-rank GEMMs move 4-8 bytes per 2 r flops: HBM-bound, rated
    # by their algorithmic bytes (each operand read once, C read and written)
    hbm_peak = _measured_peak("hbm_gbs")
    upd_bytes = (sum(n * r * 4 + 2 * n * l * r * 4 for l in range(1, L))
                 + nsw * sum(n * r * 4 + 2 * n * k * 4 for l in range(L)))
    red_bytes = sum(n * r * 4 + n * (l + 1) * r * 4 for l in range(L)) + nsw * L * (n * r * 4 + n * k * 4)
    red_name = "reduce_tma_kernel" if os.environ.get("HODLR_NO_TCGEN05") == "1" else "reduce_tc_kernel"
    kernels[red_name] = (("reduce",), "hbm", hbm_peak, red_bytes, TRAFFIC.get(red_name))
    # the update runs on the tcgen05 tensor cores (exact bf16x3 split) unless
    # HODLR_NO_TCGEN05=1 selects the FP32-FMA TMA kernel; both are HBM-bound
    upd_name = "update_tma_kernel" if os.environ.get("HODLR_NO_TCGEN05") == "1" else "update_tc_kernel"
    kernels[upd_name] = (("update",), "hbm", hbm_peak, upd_bytes, TRAFFIC.get(upd_name))
    roof = None
    best = None
    for kname, spec in kernels.items():
        kms = sum(phase_report.get(ph, {}).get("ms_per_step", 0.0) for ph in spec[0])
        if best is None or kms > best[1]:
            best = (kname, kms, spec)
    if best and best[1] > 0:
        kname, kms, (phs, bound, pk, factor, traffic) = best
        nl = sum(phase_report[ph]["launches_per_step"] for ph in phs)
        if bound == "hbm":  # factor = algorithmic bytes per step
            ach = factor / (kms * 1e-3) / 1e9
            roof = {"kernel": kname, "bound": "hbm", "achieved": ach, "peak": pk, "unit": "GB/s",
                    "frac": ach / pk if pk else None, "traffic": traffic,
                    "algorithmic_bytes_per_launch": factor / max(nl, 1),
                    "avg_launch_ms": kms / max(nl, 1), "launches_per_step": nl}
        else:
            kwork = factor * sum(sum(work[ph].values()) for ph in phs)
            ach = kwork / (kms * 1e-3) / 1e12
            roof = {"kernel": kname, "bound": bound, "achieved": ach, "peak": pk, "unit": "TFLOP/s",
                    "frac": ach / pk if pk else None, "traffic": traffic,
                    "avg_launch_ms": kms / max(nl, 1), "launches_per_step": nl}
        if bound == "tensor":
            roof["note"] = ("bf16 digit-product flops (%d digit pairs per FP64 product) of the kernel's phases / "
                            "their CUDA-event time in the timed graphs; peak = the driver-measured dense bf16 "
                            "GEMM rate (MEASURED_PEAKS.json)" % OZ_PAIRS)
        elif bound == "hbm":
            roof["note"] = ("algorithmic bytes of the kernel's launches in one step (FP32 operands read once, the "
                            "updated columns read and written once) / their CUDA-event time in the timed graphs; "
                            "peak = the driver-measured HBM copy bandwidth (MEASURED_PEAKS.json); traffic = ncu "
                            "DRAM bytes (read + write) per launch, averaged over one step's launches")
        else:
            roof["note"] = ("FP64-equivalent algorithmic flops of the kernel's phases / their CUDA-event time in "
                            "the timed graphs; peak = this GPU's FFMA rate measured live (bench_peaks.cu), "
                            "/12 for double-word arithmetic; traffic = ncu DRAM bytes per launch of the N=2^17 "
                            "capture x 8")
    line = {
        "metric": METRIC, "value": ms, "unit": "ms", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (device counter-based Gaussian generator, seeded)",
        "config": workload_config(wl, world),
        "method": "mixed precision (FP32 leaf LU / low-rank GEMMs, FP64 capacitance LU) + FP64 iterative "
                  "refinement; orthonormal factors (CholeskyQR2 on the device)",
        "residual": {0: "native fp64", 1: "fp64-accurate double-word (FP32 pipes)",
                     2: "fp64-accurate bf16 digit products (tcgen05 tensor cores)"}[args.resid],
        "ms_per_step_with_phase_events": ms_events,
        "fp_peaks_measured_tflops": {"ffma": ffma_tf, "dfma": dfma_tf, "mma_sync_bf16": mma_tf,
                                     "hbm_gbs_measured_peaks_json": _measured_peak("hbm_gbs"),
                                     "bf16_gemm_measured_peaks_json": _measured_peak("bf16_tflops")},
        "tuning": tuning,
        "refine_iterations": float(np.mean(iters)), "rel_resid_device": final_resid_dev,
        "rel_resid_fp64_check": check,
        "fp64_ms": float(np.mean(fp64_ms)), "fp64_factor_ms": fp64_factor_ms, "fp64_solve_ms": fp64_solve_ms,
        "fp64_rel_resid": fp64_resid,
        "speedup_vs_fp64": float(np.mean(fp64_ms)) / ms,
        "algorithmic_gflop_per_step": (F + S) / 1e9,
        "phases": phase_report,
        "phase_timing_note": ("value = the steps without instrumentation; phases = a second pass of the same "
                              "steps with per-phase CUDA events recorded as event nodes inside the graphs "
                              "(ms_per_step_with_phase_events)"),
        "roofline": roof,
        "clocks": clk, "gpu_launches": launches, "wall_s": wall,
        "e2e": e2e,
    }
    if gauss is not None:
        line["gaussian_generators"] = gauss
    line["small_config_vs_dense_lu"] = dense_check
    line["adjoint"] = adjoint
    if ragged is not None:
        line["ragged_batch"] = ragged
    # CPU baseline last (rank 0, N = 1): its ~12 GB of host arrays and busy
    # cores then cannot disturb the host-link part of the e2e measurement
    if rank == 0 and world == 1 and not args.no_cpu:
        ctimes, cthreads, cresid, ckind, csample = cpu_solve_runs(wl, steps=args.cpu_steps, warmup=1)
        line["cpu_baseline"] = {"value": float(np.median(ctimes)), "unit": "ms", "cores": cthreads, "kind": ckind,
                                "sample": csample, "step_ms": ctimes, "rel_resid": cresid}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_adjoint(fs, torch, stream, colmajor, reps=3):
    """The adjoint configuration: N = 2^18, leaf 128, 11 levels, rank 24, one
    right-hand side, FP64, loss 0.5 ||x||^2 (so dLoss/dx = x).  Forward =
    factor + solve; adjoint = hodlr_adjoint (the transpose solve on the kept
    factorisation, then every gradient as rank-1 outer-product kernels).
    CUDA events on the handle's stream; the median of `reps` after one warm-up."""
    m, L, r, k = 128, 11, 24, 1
    n = m << L
    sp = stream.cuda_stream
    s = fs.Solver(n, m, L, r, nrhs_max=k, precision=fs.PREC_FP64, stream=sp)
    dd = dict(dtype=torch.float64, device="cuda")
    b0 = colmajor(n, k)
    s.generate(SEED + 4, shift=4.0, orthonormal=False, decay=2.0, B=b0)
    x, g, db = colmajor(n, k), colmajor(n, k), colmajor(n, k)
    dD = torch.empty((n // m) * m * m, **dd)
    dU = torch.empty(L * n * r, **dd)
    dV = torch.empty(L * n * r, **dd)
    ds = torch.empty(L * r, **dd)
    fwd, adj = [], []
    for i in range(reps + 1):
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        x.copy_(b0)
        e[0].record(stream)
        s.factor()
        s.solve(x)
        e[1].record(stream)
        g.copy_(x)
        stream.synchronize()
        t = torch.cuda.Event(enable_timing=True)
        t.record(stream)
        s.adjoint(x, g, db=db, dD=dD, dU=dU, dV=dV, ds=ds)
        e[2].record(stream)
        torch.cuda.synchronize()
        if i > 0:
            fwd.append(e[0].elapsed_time(e[1]))
            adj.append(t.elapsed_time(e[2]))
    s.close()
    f, a = float(np.median(fwd)), float(np.median(adj))
    return {"workload": "N=2^18 leaf 128 L=11 rank 24 nrhs 1, FP64, loss 0.5||x||^2; gradients wrt b, D_leaf, "
                        "U, V, s", "forward_ms": f, "adjoint_ms": a, "adjoint_over_forward": a / f}


def dense_from_handle(solver, n, m, L, r):
    """The dense N x N matrix of a handle's inputs (small N only)."""
    import torch
    D = torch.empty((n // m) * m * m, dtype=torch.float64)
    U = torch.empty(max(L, 1) * n * r, dtype=torch.float64)
    V = torch.empty_like(U)
    sv = torch.empty(max(L, 1) * r, dtype=torch.float64)
    solver.get_inputs(D=D, U=U, V=V, s=sv)
    D, U, V, sv = D.numpy(), U.numpy(), V.numpy(), sv.numpy()
    A = np.zeros((n, n))
    for i in range(n // m):
        A[i * m:(i + 1) * m, i * m:(i + 1) * m] = D[i * m * m:(i + 1) * m * m].reshape(m, m).T
    for l in range(L):
        Ul = U[l * n * r:(l + 1) * n * r].reshape(r, n).T * sv[l * r:(l + 1) * r]
        Vl = V[l * n * r:(l + 1) * n * r].reshape(r, n).T
        rows = n >> (l + 1)
        for p in range(1 << l):
            c0, c1 = slice(2 * p * rows, (2 * p + 1) * rows), slice((2 * p + 1) * rows, (2 * p + 2) * rows)
            A[c0, c1] = Ul[c0] @ Vl[c1].T
            A[c1, c0] = Ul[c1] @ Vl[c0].T
    return A


def small_config_dense_check(fs, torch):
    """N = 4096, leaf 256, 4 levels, rank 16, 1 rhs (leaves G/sqrt(256) + 4I,
    Gaussian U, V): both precisions against a dense FP64 LU (scipy)."""
    import scipy.linalg as sla
    n, m, L, r, k = 4096, 256, 4, 16, 1
    out = {"workload": "N=4096 leaf 256 L=4 rank 16 nrhs 1, Gaussian generators, leaf shift 4"}
    for prec, name in ((fs.PREC_FP64, "fp64"), (fs.PREC_MIXED, "mixed")):
        s = fs.Solver(n, m, L, r, nrhs_max=k, precision=prec)
        B = torch.empty((k, n), dtype=torch.float64, device="cuda").t()
        s.generate(SEED, shift=4.0, orthonormal=False, decay=0.0, B=B)
        A = dense_from_handle(s, n, m, L, r)
        b = B.cpu().numpy()
        x_ref = sla.lu_solve(sla.lu_factor(A), b)
        s.factor()
        s.solve(B)
        x = B.cpu().numpy()
        out[name] = {"rel_err_vs_dense_lu": float(np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref)),
                     "rel_resid": float(np.linalg.norm(b - A @ x) / np.linalg.norm(b))}
        s.close()
    return out


def run_ragged(args, fs, torch, stream, colmajor):
    """The ragged batch of 512 systems: batched factor + solve (one graph
    launch each), FP64 and mixed; each batch solution checked by the FP64
    product of its own system; and the same systems as 512 separate handles
    (FP64) for comparison."""
    systems = ragged_systems(512, SEED)
    sp = stream.cuda_stream
    total = sum(n * k for n, m, L, r, k in systems)
    out = {"systems": len(systems), "workload": "512 systems, N log-uniform in [2^10, 2^16], leaf {64,128,256}, "
           "rank {8,16,32,64} < leaf, 1-8 rhs; leaves G/sqrt(m)+4I, Gaussian U, V (seeded)",
           "rows": int(sum(s[0] for s in systems)), "algorithmic_gflop": ragged_flops(systems) / 1e9}
    big0 = torch.empty(total, dtype=torch.float64, device="cuda")
    big = torch.empty_like(big0)

    def views(buf):
        vs, off = [], 0
        for n, m, L, r, k in systems:
            vs.append(buf[off:off + n * k].view(k, n).t())
            off += n * k
        return vs

    V0, V = views(big0), views(big)
    solutions = {}
    for prec, name in ((fs.PREC_FP64, "fp64"), (fs.PREC_MIXED, "mixed")):
        b = fs.Batch(systems, precision=prec, residual=args.resid, refine_tol=1e-12, stream=sp)
        b.generate(SEED, shift=4.0, Bs=V0)
        # per-forest launch shapes (mixed only: an FP64 tuning pass would take a minute)
        tunes = b.autotune() if (prec == fs.PREC_MIXED and not args.no_tune) else None
        infos = []

        def step():
            big.copy_(big0)
            b.factor()
            infos[:] = b.solve(V)

        nsteps = min(args.steps, 3)   # an FP64 step of this batch takes seconds
        for _ in range(2):            # eager run, then graph capture
            step()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(nsteps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / nsteps
        nf, fms, sms = b.stats()
        out[name] = {"ms_per_step": ms, "steps": nsteps, "factor_ms": fms, "solve_ms": sms, "forests": nf,
                     "tuning": tunes,
                     "max_rel_residual_device": (max(i.rel_residual for i in infos)
                                                 if prec == fs.PREC_MIXED else None),
                     "max_iterations": max(i.iterations for i in infos)}
        solutions[name] = big.clone()
        b.close()
    # the same systems as separate FP64 handles: their FP64 products check the
    # batch's solutions, then they run one after another for comparison
    handles = []
    for i, (n, m, L, r, k) in enumerate(systems):
        h = fs.Solver(n, m, L, r, nrhs_max=k, precision=fs.PREC_FP64, stream=sp)
        h.generate(SEED + i, shift=4.0, B=None)
        handles.append(h)
    for name, xs in solutions.items():
        worst = 0.0
        with torch.cuda.stream(stream):
            for h, x, b0 in zip(handles, views(xs), V0):
                y = torch.empty_like(x.t()).t()
                h.matvec(x, y)
                worst = max(worst, ((b0 - y).norm(dim=0) / b0.norm(dim=0)).max().item())
        out[name]["max_rel_residual"] = worst
    del solutions
    out["residual_note"] = ("max over systems and columns of ||b - A x|| / ||b||, A x by each system's own FP64 "
                            "handle (hodlr_matvec, native FP64)")
    for rep in range(2):   # the first pass loads and captures, the second is timed
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for h, x in zip(handles, V):
            h.factor()
            h.solve(x)
        torch.cuda.synchronize()
        loop_ms = (time.perf_counter() - t0) * 1e3
    out["fp64_separate_handles_ms"] = loop_ms
    for h in handles:
        h.close()
    return out


OZ_PAIRS = 28   # digit pairs (s + t <= 6 of 7 x 7) per FP64 product in the tensor-core residual
# ncu DRAM bytes (read + write) per launch, averaged over the launches of one
# mixed step at N=2^20 (a dram__bytes capture of this benchmark's kernels)
TRAFFIC = {"update_tc_kernel": 38.775e9 / 155, "update_tma_kernel": 38.804e9 / 155,
           "reduce_tma_kernel": 25.553e9 / 156,
           # ncu DRAM bytes of one step's tensor-core reductions at N=2^17 were 1.0177 x their algorithmic
           # bytes (2.134 GB of 2.097 GB); the same ratio applied to the N=2^20 step's 24.43 GB / 156 launches
           "reduce_tc_kernel": 1.0177 * 156.587e6,
           "oz_tc_kernel<0>": 21.130e9 / 11, "oz_tc_kernel<1>": (20.116e9 + 0.134e9) / 11}


def host_numa_binding(local):
    """Pin the calling thread to the CPUs of the GPU's NUMA node (when the
    node is known and those CPUs are ours), so pinned buffers allocated next
    land there.  Returns a record (node, CPUs, the previous affinity)."""
    rec = {"gpu_numa_node": None, "bound_cpus": None}
    try:
        bus = subprocess.run(["nvidia-smi", "-i", str(local), "--query-gpu=pci.bus_id", "--format=csv,noheader"],
                             capture_output=True, text=True, timeout=20).stdout.strip()
        dom, rest = bus.split(":", 1)
        path = "/sys/bus/pci/devices/%04x:%s/numa_node" % (int(dom, 16), rest.lower())
        with open(path) as f:
            node = int(f.read().strip())
        rec["gpu_numa_node"] = node
        rec["pci_bus_id"] = bus
        if node >= 0 and hasattr(os, "sched_setaffinity"):
            with open("/sys/devices/system/node/node%d/cpulist" % node) as f:
                cpus = set()
                for part in f.read().strip().split(","):
                    if "-" in part:
                        a, b = part.split("-")
                        cpus.update(range(int(a), int(b) + 1))
                    elif part:
                        cpus.add(int(part))
            old = os.sched_getaffinity(0)
            use = cpus & old
            if use:
                os.sched_setaffinity(0, use)
                rec["bound_cpus"] = len(use)
                rec["_old"] = sorted(old)
    except (OSError, ValueError, subprocess.SubprocessError):
        pass
    return rec


def restore_affinity(rec):
    old = rec.pop("_old", None)
    if old:
        os.sched_setaffinity(0, set(old))


def numa_nodes_of(tensors):
    """Pages per NUMA node of the mappings that overlap the given host
    tensors (/proc/self/maps for the extents, /proc/self/numa_maps for the
    per-node page counts)."""
    spans = [(t.data_ptr(), t.data_ptr() + t.numel() * t.element_size()) for t in tensors]
    out = {}
    try:
        ends = {}
        with open("/proc/self/maps") as f:
            for line in f:
                a, b = line.split()[0].split("-")
                ends[int(a, 16)] = int(b, 16)
        with open("/proc/self/numa_maps") as f:
            for line in f:
                fields = line.split()
                start = int(fields[0], 16)
                end = ends.get(start, start)
                if not any(start < hi and lo < end for lo, hi in spans):
                    continue
                for fld in fields[1:]:
                    if fld.startswith("N") and "=" in fld:
                        nd, cnt = fld[1:].split("=")
                        out["node" + nd] = out.get("node" + nd, 0) + int(cnt)
    except (OSError, ValueError, IndexError):
        return None
    return out


def max_over_ranks(value, device):
    """The maximum of a per-rank time over every rank of the initialised
    process group (the value itself without one, or with one rank)."""
    import torch
    import torch.distributed as dist
    if value is None or not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return value
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.item()


PEAKS_SO = os.path.join(ROOT, "bench_peaks.so")


def build_peak_probe():
    """Compile bench_peaks.cu (the FMA / MMA rate probe of this benchmark,
    not part of the solver library) into bench_peaks.so for sm_103a."""
    src = os.path.join(ROOT, "bench_peaks.cu")
    if os.path.exists(PEAKS_SO) and os.path.getmtime(PEAKS_SO) >= os.path.getmtime(src):
        return PEAKS_SO
    nvcc = "/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else "nvcc"
    subprocess.check_call([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-shared",
                           "-Xcompiler", "-fPIC", src, "-o", PEAKS_SO + ".tmp"])
    os.replace(PEAKS_SO + ".tmp", PEAKS_SO)
    return PEAKS_SO


def probe_peaks():
    """(FFMA, DFMA, mma.sync bf16) TFLOP/s of the current GPU, measured live."""
    import ctypes
    lib = ctypes.CDLL(build_peak_probe())
    f, d, t = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    if lib.bench_probe_fp_peaks(ctypes.byref(f), ctypes.byref(d)) or lib.bench_probe_mma_bf16(ctypes.byref(t)):
        raise RuntimeError("peak probe failed")
    return f.value, d.value, t.value


def _measured_peak(key):
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f).get(key)
    except (OSError, ValueError):
        return None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--resid", type=int, default=2,
                    help="0 native FP64 residual, 1 double-word FP32 pipes, 2 tensor-core digit products")
    ap.add_argument("--fp64-steps", type=int, default=3)
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--cpu-steps", type=int, default=3, help="full-size CPU solves timed for cpu_baseline")
    ap.add_argument("--small", action="store_true", help="N=2^14 smoke-sized workload")
    ap.add_argument("--levels", type=int, default=None, help="override the tree depth (N = 128 * 2^levels)")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 comparator")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--plain-inputs", action="store_true",
                    help="e2e: copy every input when it is set (no V streamed in by the factorisation)")
    ap.add_argument("--no-ragged", action="store_true", help="skip the 512-system ragged batch")
    ap.add_argument("--no-tune", action="store_true", help="default launch shapes (no autotuning pass)")
    ap.add_argument("--no-phase-timing", action="store_true",
                    help="no per-phase CUDA events in the timed graphs (for profiler runs)")
    args = ap.parse_args()
    wl = dict(SMALL if args.small else WORKLOAD)
    if args.levels is not None:
        wl.update(levels=args.levels, n=wl["leaf"] << args.levels)
    if args.impl == "reference":
        return run_reference(args, wl)
    return run_ours(args, wl)


if __name__ == "__main__":
    sys.exit(main())
