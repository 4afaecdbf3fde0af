#!/usr/bin/env python
"""Benchmark: CASCI(12e,12o) time-to-energy on one GB300.

Workload: 853,776 determinants (n_alpha = n_beta = 6 in 12 orbitals), seeded
synthetic integrals (h1 = diag(-2 + 0.25 p) + N(0, 0.05^2) off-diagonal,
V = sum over 24 symmetric Cholesky vectors with N(0, 0.1^2) entries).
One step = the hot path from integrals and determinants resident in HBM to
the ground-state energy: the operator (qdkgb_build_operator: for this
complete space of 1.55e9 matrix elements the direct sigma, nothing stored) +
Davidson to a full-precision residual norm of 1e-8, in the mixed-precision
form (FP32 sigma, double-float subspace, FP64 refinement).  The plain FP64
path (the matrix stored in the slab layout) is timed beside it.

The stored matrix (6.2 GB FP32 + 6.2 GB low parts, or 12.4 GB FP64) is far
larger than L2 (129 MB), so no L2 flush is needed between steps.

  python bench.py [--steps K] [--warmup W] [--impl ours|reference]
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NORB, NEL, NCHOL, SEED = 12, 12, 24, 20261203  # the headline workload (--norb/--nel/--nchol shrink it for profiling)
RES_TOL = 1e-8
WORKLOAD = "CASCI(12e,12o) FP64 integrals, 853,776 determinants, H build + Davidson to |r| < 1e-8"
METRIC = "casci_12e12o_time_to_energy"


def set_workload(norb, nel, nchol):
    """Smaller CASCI(nel, norb) cases of the same recipe (profiling captures)."""
    global NORB, NEL, NCHOL, WORKLOAD, METRIC
    if (norb, nel, nchol) == (NORB, NEL, NCHOL):
        return
    NORB, NEL, NCHOL = norb, nel, nchol
    WORKLOAD = "CASCI(%de,%do) FP64 integrals, H build + Davidson to |r| < 1e-8" % (nel, norb)
    METRIC = "casci_%de%do_time_to_energy" % (nel, norb)


def _package():
    import __graft_entry__ as g

    return g._package()


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _bf16_peak():
    """Dense bf16 tensor TFLOP/s: the measured burst figure, else the
    fallback 1900."""
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        return float(json.load(open(p))["bf16_tflops"])
    return 1900.0


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = str(gpu_index)
        self.lines = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", self.gpu, "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ CPU baseline
def cpu_full_run(T, V, a, b):
    """One full CPU time-to-energy of the reference's algorithm (the oracle's
    restatement of MACIS, OpenMP on every host core): the sorted-double-loop
    H build with all its passes (count, fill, mirror, per-row column sort,
    threshold; sorted_double_loop.hpp:86-451) into an int64 CSR, then
    selected_ci_diag's Davidson (diagonal guess, CGS2, Rayleigh-Ritz, to
    |r| < 1e-8; davidson.hpp:259-372), timed end to end."""
    import oracle

    oracle.build()
    t0 = time.perf_counter()
    M = oracle.build_csr(oracle.Hamiltonian(T, V), a, b)
    t1 = time.perf_counter()
    E, _, it = M.selected_ci_diag(tol=RES_TOL)
    t2 = time.perf_counter()
    del M
    return {"value": t2 - t0, "unit": "s", "cores": oracle.num_threads(), "kind": "port",
            "sample": "full: SDL H build (count, fill, mirror, row sort, threshold) + Davidson to |r| < 1e-8, "
                      "end to end, no extrapolation",
            "build_s": t1 - t0, "davidson_s": t2 - t1, "iterations": int(it), "energy": float(E)}


def run_reference(args):
    """The reference arm: full CPU time-to-energy runs of the reference's
    algorithm on the host cores (cpu_full_run).  A run takes tens of seconds,
    so the arm makes as many full runs as fit in about three minutes (at most
    --steps, at least one) and reports their mean; no warm-up run (a CPU run
    has nothing to compile or page in twice)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    pkg = _package()
    T, V, _ = pkg.integrals.synthetic_integrals(NORB, NCHOL, SEED)
    a, b = pkg.determinants.fci_space(NORB, NEL // 2, NEL // 2)
    budget = 180.0
    runs = []
    t_start = time.perf_counter()
    while len(runs) < max(1, args.steps):
        runs.append(cpu_full_run(T, V, a, b))
        spent = time.perf_counter() - t_start
        if spent + spent / len(runs) > budget:
            break
    v = float(np.mean([r["value"] for r in runs]))
    cb = dict(runs[-1])
    cb["value"] = v
    cb["runs"] = len(runs)
    cb["run_values"] = [r["value"] for r in runs]
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "s", "n_gpus": args.gpus,
            "steps": len(runs), "warmup": 0, "steps_requested": args.steps, "warmup_requested": args.warmup,
            "ms_per_step": v * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "norb": NORB, "nalpha": NEL // 2, "nbeta": NEL // 2,
                       "n_chol": NCHOL, "seed": SEED, "res_tol": RES_TOL},
            "cpu_baseline": cb, "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_reference_batched(args):
    """The reference's per-instance CPU path (oracle restatement of the SDL
    build + Davidson, OpenMP on all host cores) over a bounded sample of the
    512 instances (every 32nd), scaled to the batch."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import oracle

    oracle.build()
    pkg = _package()
    inst = batch_instances(pkg)
    sample = inst[::32]
    vals = []
    for step in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        for no, na, nb, T, V in sample:
            a, b = pkg.determinants.fci_space(no, na, nb)
            M = oracle.build_csr(oracle.Hamiltonian(T, V), a, b)
            M.selected_ci_diag(tol=RES_TOL)
        dt = (time.perf_counter() - t0) * len(inst) / len(sample)
        if step >= args.warmup:
            vals.append(len(inst) / dt)
    v = float(np.mean(vals))
    cb = {"value": v, "unit": "instances/s", "cores": oracle.num_threads(), "kind": "port",
          "sample": "every 32nd instance (%d of %d): SDL CSR build + Davidson to |r| < 1e-8, scaled"
                    % (len(sample), len(inst))}
    line = {"impl": "reference", "metric": "casci_batch512_instances_per_s", "value": v, "unit": "instances/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": len(inst) / v * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": "512 CASCI instances, norb in {6,8,10}", "seed": BATCH_SEED},
            "cpu_baseline": cb, "e2e": {"value": v, "unit": "instances/s", "h2d_bytes_per_step": 0,
                                        "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ------------------------------------------------------------------ GPU arm
def max_over_ranks(value, world):
    """The largest of the ranks' values (a job's step time is its slowest
    replica's); the value itself on one rank.  Host tensors: the gloo group."""
    if world <= 1:
        return float(value)
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(value)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_ours(args):
    import torch

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
    torch.cuda.set_device(local)
    pkg = _package()
    pkg.build.build()
    capi = pkg.capi
    T, V, _ = pkg.integrals.synthetic_integrals(NORB, NCHOL, SEED)
    a, b = capi.fci_dets(NORB, NEL // 2, NEL // 2)
    N = len(a)
    # a real stream (torch's default stream has handle 0, which the library reads as 'use your own')
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = capi.Context(local)
    ctx.set_stream(stream.cuda_stream)
    ctx.set_integrals(T, V)
    ctx.set_dets(a, b)

    def ev():
        e = torch.cuda.Event(enable_timing=True)
        e.record(stream)
        return e

    def step(storage, precision):
        # the FP64 path stores the matrix (the reference's form); the mixed
        # path takes the operator qdkgb_build_operator picks, as qdkgb_casci
        # does (for this complete space the direct sigma in both precisions)
        e0 = ev()
        if precision == capi.PREC_FP64:
            ctx.build_hamiltonian(storage=storage)
        else:
            ctx.build_operator(storage=storage)
        e1 = ev()
        E, _, info = ctx.davidson(tol=RES_TOL, precision=precision, want_vector=False)
        e2 = ev()
        torch.cuda.synchronize()
        return E, info, e0.elapsed_time(e1) / 1e3, e1.elapsed_time(e2) / 1e3

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    # plain FP64 path (the reference's precision) for the comparison
    E64, info64, hb64, dv64 = step(capi.H_FP64, capi.PREC_FP64)
    nnz = ctx.nnz
    lay64, stored64 = ctx.operator_layout()
    # FP64 SpMV roofline (FP64 values + int32 columns)
    x64 = torch.randn(N, dtype=torch.float64, device="cuda")
    y64 = torch.empty_like(x64)
    t_spmv64 = time_spmv(ctx, capi.PREC_FP64, x64, y64, stream)
    # the first FP64 step above is cold (it also times the FP64 sigma's
    # segment candidates); the reported split comes from the later steps
    fp64_times, hb64s, dv64s = [], [], []
    for _ in range(max(1, min(args.steps, 2))):
        _, _, h, d = step(capi.H_FP64, capi.PREC_FP64)
        fp64_times.append(h + d)
        hb64s.append(h)
        dv64s.append(d)
    hb64, dv64 = float(np.mean(hb64s)), float(np.mean(dv64s))
    # mixed path: warm-up, then the timed steps
    for _ in range(args.warmup):
        step(capi.H_SPLIT32, capi.PREC_MIXED)
    barrier()
    launches0 = capi.kernel_launches()
    times, hbs, dvs, infos, Es = [], [], [], [], []
    with ClockSampler(local) as clk:
        barrier()
        t_wall = time.perf_counter()
        for _ in range(args.steps):
            E, info, h, d = step(capi.H_SPLIT32, capi.PREC_MIXED)
            times.append(h + d)
            hbs.append(h)
            dvs.append(d)
            infos.append(info)
            Es.append(E)
        barrier()
        t_wall = time.perf_counter() - t_wall
    launches = capi.kernel_launches() - launches0
    t_step = float(np.mean(times))
    t_step = max_over_ranks(t_step, world)
    # FP32 SpMV roofline on the split storage (FP32 values + int32 columns)
    x32 = torch.randn(N, dtype=torch.float32, device="cuda")
    y32 = torch.empty_like(x32)
    t_spmv32 = time_spmv(ctx, capi.PREC_MIXED, x32, y32, stream)
    lay32, stored32 = ctx.operator_layout()
    peak, peak_kind = _peaks()
    # algorithmic bytes of one sigma: the stored values once, x once (L2
    # resident), y once; the CSR layout adds int32 columns and int64 rowptr
    if lay32 == capi.OP_SLAB:
        bytes32 = stored32 * 4 + N * 4 + N * 4
        # the slab sigma's variant follows the number of beta strings (and
        # 16-byte alignment, which device allocations have): 4 or 2 strings per
        # thread when it divides, else one
        nbs = math.comb(NORB, NEL // 2)
        vec = 4 if nbs % 4 == 0 else (2 if nbs % 2 == 0 else 1)
        kern32 = ("k_slab_sigma32v<%d> (FP32 sigma, slab layout: values only, %d beta strings per thread)"
                  % (vec, vec) if vec > 1 else "k_slab_sigma<0> (FP32 sigma, slab layout: values only)")
        used32 = ctx.sigma_plan(capi.PREC_MIXED, with_kernel=True)[2]
        if used32 == "tma":
            kern32 = ("k_slab_sigma32t (FP32 sigma, slab layout: values only; rows streamed into shared memory "
                      "by TMA bulk copies, 4 beta strings per thread)")
        elif used32 in ("register8", "register16"):
            kern32 = ("k_slab_sigma32v<4, %d> (FP32 sigma, slab layout: values only, 4 beta strings per thread, "
                      "%d positions in flight)" % ((8, 8) if used32 == "register8" else (16, 16)))
    elif lay32 in (capi.OP_SLAB_DIRECT32, capi.OP_DIRECT):
        bytes32 = None
        kern32 = ("FP32 direct sigma: k_ds_opposite_mm (opposite-spin doubles and every single excitation as one "
                  "contraction per alpha string, FMA pipe) + the same-spin string-only part")
    else:
        bytes32 = nnz * 8 + (N + 1) * 8 + N * 4 + N * 4
        kern32 = "k_spmv_csr<float> (FP32 sigma, CSR)"
    if lay64 == capi.OP_SLAB:
        bytes64 = stored64 * 8 + N * 8 + N * 8
        kern64 = "k_slab_sigma<1> (FP64 sigma, slab layout; FP64-pipe bound)"
    else:
        bytes64 = nnz * 12 + (N + 1) * 8 + N * 8 + N * 8
        kern64 = "k_spmv_csr<double> (FP64 sigma, CSR)"
    roof = None
    if lay32 in (capi.OP_SLAB_DIRECT32, capi.OP_DIRECT):
        # FLOPs of one FP32 direct sigma as formulated: the contraction forms
        # E (rows: the n(n-1) pairs, n W rows, one string row; K: the alpha
        # singles and the own row) for every beta string; the same-spin part
        # as two dense products (or the element-wise kernels, fewer FLOPs)
        ka = NEL // 2
        na_s = math.comb(NORB, ka)
        nsa = ka * (NORB - ka)
        rows = NORB * (NORB - 1) + NORB + 1
        flops = 2.0 * na_s * rows * (nsa + 1) * na_s
        plan = ctx.direct_plan()
        if plan.get("dense"):
            flops += 2.0 * 2 * na_s ** 3
        if plan.get("contraction") == "tensor":
            # TF32 x 3 on tcgen05: the tensor pipe runs three TF32 products per
            # FP32 product; its dense TF32 rate is half the measured bf16 rate
            tf32_peak = _bf16_peak() / 2
            achieved = 3 * flops / t_spmv32 / 1e12
            kern32 = ("FP32 direct sigma on the tensor cores: k_ds_opposite_tc (opposite-spin doubles and every "
                      "single excitation as one tcgen05 TF32x3 contraction per alpha string) + k_tc_gemm2b (the "
                      "same-spin string-only part as two dense tcgen05 TF32x3 products)")
            roof = {"bound": "tensor", "kernel": kern32, "achieved": achieved, "peak": tf32_peak,
                    "unit": "TFLOP/s", "frac": achieved / tf32_peak,
                    "peak_source": "measured bf16 dense rate / 2 (TF32), of measured", "traffic": None,
                    "algorithmic_flops": flops, "tensor_flops": 3 * flops, "launch_ms": t_spmv32 * 1e3,
                    "plan": plan}
        else:
            fp32_peak = 152 * 128 * 2 * 2.07e9 / 1e12
            achieved = flops / t_spmv32 / 1e12
            roof = {"bound": "fp32", "kernel": kern32, "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                    "frac": achieved / fp32_peak, "peak_source": "nominal FP32 FMA rate (152 SMs x 128 lanes x 2 x "
                    "2.07 GHz; no measured FP32 figure)", "traffic": None, "algorithmic_flops": flops,
                    "launch_ms": t_spmv32 * 1e3, "plan": plan}
        achieved32 = None
    else:
        achieved32 = bytes32 / t_spmv32 / 1e9
    achieved64 = bytes64 / t_spmv64 / 1e9
    traffic = None
    tp = os.path.join(ROOT, "profiles", "spmv_traffic.json")
    if os.path.exists(tp) and lay32 == capi.OP_SLAB:
        per_el = json.load(open(tp)).get("slab_fp32_dram_bytes_per_element")
        if per_el:
            traffic = int(round(per_el * stored32))

    # end to end through the C ABI with host buffers: integrals in, energy and
    # CI vector out (host->device copies of T, V and the determinant list inside)
    ctx_e2e = capi.Context(local)
    e2e_times = []
    for i in range(1 + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        Ee, Ce, _ = ctx_e2e.casci(T, V, NEL // 2, NEL // 2, tol=RES_TOL, precision=capi.PREC_MIXED)
        torch.cuda.synchronize()
        if i > 0:
            e2e_times.append(time.perf_counter() - t0)
    ctx_e2e.close()
    # per call: the integrals in (the complete space of an unchanged shape
    # stays on the device), the energy and CI vector out
    h2d = T.nbytes + V.nbytes
    d2h = N * 8 + 8

    cb = None
    if rank == 0 and not args.no_cpu:
        cb = cpu_full_run(T, V, np.asarray(a), np.asarray(b))
        # parity inside the bench: the plain FP64 GPU energy against the CPU
        # restatement of the reference on the same integrals (bar 1e-10 Eh)
        cb["energy_error_vs_gpu_fp64"] = abs(cb["energy"] - E64)
        cb["iterations_gpu_fp64"] = int(info64["iterations"])
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": t_step, "unit": "s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 sigma / double-float subspace / f64 refinement", "data": "synthetic",
        "config": {"workload": WORKLOAD, "norb": NORB, "nalpha": NEL // 2, "nbeta": NEL // 2, "ndets": N,
                   "nnz": nnz, "n_chol": NCHOL, "seed": SEED, "res_tol": RES_TOL, "precision": "mixed",
                   "l2": (("working set larger than L2: Davidson subspace columns of %.1f MB (V and A V, tens of "
                           "columns per solve), no stored matrix; no flush" % (N * 8 / 1e6))
                          if lay32 == capi.OP_DIRECT else
                          "inputs larger than L2 (stored H %.1f GB), no flush" % (stored32 * 8 / 1e9)),
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "roofline": roof or {"bound": "hbm", "kernel": kern32, "achieved": achieved32,
                             "peak": peak, "unit": "GB/s", "frac": achieved32 / peak, "peak_source": peak_kind,
                             "traffic": traffic, "algorithmic_bytes": bytes32, "launch_ms": t_spmv32 * 1e3},
        "operator_mixed": capi.LAYOUT_NAMES.get(lay32),
        "spmv_fp64": {"kernel": kern64, "achieved_gbs": achieved64, "frac": achieved64 / peak,
                      "launch_ms": t_spmv64 * 1e3, "algorithmic_bytes": bytes64},
        "sigma_autotune": {"fp32": dict(zip(("segments", "candidates_ms", "kernel", "kernel_candidates_ms"),
                                            ctx.sigma_plan(capi.PREC_MIXED, with_kernel=True))),
                           "fp64": dict(zip(("segments", "candidates_ms"), ctx.sigma_plan(capi.PREC_FP64)))},
        "hbuild_s": float(np.mean(hbs)), "davidson_s": float(np.mean(dvs)),
        "davidson": {k: infos[-1][k] for k in ("iterations", "spmv_fp64", "spmv_fp32", "restarts", "residual_norm")},
        "fp64_path": {"time_to_energy_s": float(np.mean(fp64_times)), "hbuild_s": hb64, "davidson_s": dv64,
                      "iterations": info64["iterations"], "energy": E64},
        "mixed_speedup_vs_fp64": float(np.mean(fp64_times)) / t_step,
        "energy": Es[-1], "energy_error_vs_fp64": abs(Es[-1] - E64),
        "e2e": {"value": float(np.mean(e2e_times)), "unit": "s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "energy_error_vs_fp64": abs(Ee - E64)},
        "gpu_launches": launches, "wall_s_timed": t_wall,
        "clocks": clk.summary(),
        "cpu_baseline": cb,
    }
    print(json.dumps(line))


# ------------------------------------------------------------------ batched CASCI
BATCH_N, BATCH_SEED, BATCH_SIZES = 512, 20261204, (6, 8, 10)


def batch_instances(pkg, n=BATCH_N, seed=BATCH_SEED):
    """512 instances, norb drawn uniformly from {6, 8, 10} (seeded), n_alpha =
    n_beta = norb / 2, integrals of the same recipe with 2 norb Cholesky
    vectors and a per-instance seed."""
    rng = np.random.default_rng(seed)
    norbs = rng.choice(BATCH_SIZES, size=n)
    out = []
    for i, no in enumerate(norbs):
        no = int(no)
        T, V, _ = pkg.integrals.synthetic_integrals(no, 2 * no, seed + 1 + i)
        out.append((no, no // 2, no // 2, T, V))
    return out


def _slab_elements(no, na, nb):
    """Stored values of one complete (norb, na, nb) space in the slab layout:
    determinants x row length."""
    from math import comb

    ga, gb = comb(no, na), comb(no, nb)
    ka, kb = na * (no - na), nb * (no - nb)
    n1b = 1 + kb
    n2b = 1 + kb + comb(nb, 2) * comb(no - nb, 2)
    c2a = comb(na, 2) * comb(no - na, 2)
    return ga * gb * (n2b + ka * n1b + c2a)


def _batch_bytes(inst):
    """Stored values read by one FP32 sigma over every instance (slab: rowlen
    per determinant) plus x and y."""
    from math import comb

    tot = 0
    for no, na, nb, _, _ in inst:
        ga, gb = comb(no, na), comb(no, nb)
        ka, kb = na * (no - na), nb * (no - nb)
        n1a, n1b = 1 + ka, 1 + kb
        n2b = 1 + kb + comb(nb, 2) * comb(no - nb, 2)
        c2a = comb(na, 2) * comb(no - na, 2)
        rowlen = n2b + ka * n1b + c2a
        nd = ga * gb
        tot += nd * rowlen * 4 + nd * 8
    return tot


def run_batched(args):
    import torch

    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    pkg = _package()
    pkg.build.build()
    capi = pkg.capi
    inst = batch_instances(pkg)
    # a sub-batch for profiling: one shape (--batch-norb), the first
    # --batch-count instances; --persistent / --cluster select the solver
    if args.batch_norb:
        inst = [x for x in inst if x[0] == args.batch_norb]
    if args.batch_count:
        inst = inst[:args.batch_count]
    solver = {"persistent": args.persistent, "cluster": args.cluster}
    ctx = capi.Context(local)
    for _ in range(max(1, args.warmup)):
        capi.casci_batch(ctx, inst, res_tol=RES_TOL, **solver)
    launches0 = capi.kernel_launches()
    times, infos = [], []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            E, R, its, info = capi.casci_batch(ctx, inst, res_tol=RES_TOL, **solver)
            torch.cuda.synchronize()
            times.append(time.perf_counter() - t0)
            infos.append(info)
    launches = capi.kernel_launches() - launches0
    t = float(np.mean(times))
    its_last = np.asarray(its)
    # the persistent cluster solver (one launch per shape, tuned cluster
    # size) on the same batch, beside the default lockstep path
    t_pers = None
    if not args.no_cpu and not args.persistent:
        capi.casci_batch(ctx, inst, res_tol=RES_TOL, persistent=1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        capi.casci_batch(ctx, inst, res_tol=RES_TOL, persistent=1)
        torch.cuda.synchronize()
        t_pers = time.perf_counter() - t0
    plan = capi.batch_plan(ctx)
    # plain per-instance FP64 GPU path on a sample (every 8th instance), scaled
    sample = inst[::8]
    ctx1 = capi.Context(local)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    dE = []
    for j, (no, na, nb, T, V) in enumerate(sample):
        E64, _, _ = ctx1.casci(T, V, na, nb, tol=RES_TOL, want_vector=False)
        dE.append(abs(E64 - E[8 * j]))
    torch.cuda.synchronize()
    t_loop = (time.perf_counter() - t0) * len(inst) / len(sample)
    ctx1.close()
    ctx.close()
    if rank != 0:
        return
    counts = {str(k): int(sum(1 for x in inst if x[0] == k)) for k in BATCH_SIZES}
    # whole-solve sigma traffic: every sigma application streams the
    # instance's stored values once (4 bytes each; the full-precision refresh
    # reads 8, so this is a lower bound) - against the measured HBM peak
    stored = [_slab_elements(x[0], x[1], x[2]) for x in inst]
    sigma_bytes = float(sum(int(n_it) * st * 4 for n_it, st in zip(its_last, stored)))
    peak, peak_kind = _peaks()
    achieved = sigma_bytes / t / 1e9
    h2d = int(sum(x[3].nbytes + x[4].nbytes for x in inst))
    d2h = int(sum(8 + x[0] ** 2 * 8 for x in inst))
    line = {
        "metric": ("casci_batch512_instances_per_s" if not (args.batch_norb or args.batch_count)
                   else "casci_batch_subset_instances_per_s"), "value": len(inst) / t, "unit": "instances/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 sigma / f64 subspace+refinement",
        "data": "synthetic",
        "config": {"workload": "512 independent CASCI instances, norb uniform in {6,8,10} (n_alpha = n_beta = "
                               "norb/2: 400 / 4,900 / 63,504 determinants), seeded integrals of the same recipe "
                               "with 2 norb Cholesky vectors; energy to |r| < 1e-8 and spin-summed 1-RDM per "
                               "instance", "instances": counts, "seed": BATCH_SEED, "res_tol": RES_TOL,
                   "l2": "stored matrices %.1f GB, larger than L2; no flush" % (_batch_bytes(inst) * 2 / 1e9),
                   "subset": ({"norb": args.batch_norb or None, "count": args.batch_count or None}
                              if (args.batch_norb or args.batch_count) else None),
                   "solver": "persistent" if args.persistent else "lockstep"},
        "per_instance_fp64_gpu": {"instances_per_s": len(inst) / t_loop,
                                  "sample": "every 8th instance (%d) through qdkgb_casci FP64, scaled" % len(sample),
                                  "max_abs_energy_diff_vs_batch": float(max(dE))},
        "batch_speedup_vs_per_instance_fp64": t_loop / t,
        "roofline": {"bound": "hbm", "kernel": "the lockstep solve: new directions through the direct contraction "
                                               "(k_ds_opposite_mm or k_ds_opposite_tc + k_tc_gemm2b tcgen05 same-spin products, "
                                               "instance grid axis), full-precision refreshes through the stored "
                                               "split slab (k_slab_sigma<2>), batched vector kernels",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind, "traffic": None,
                     "algorithmic_bytes": sigma_bytes,
                     "note": "slab-equivalent sigma bytes of the whole solve (iterations x stored values x 4 B per "
                             "instance) over the call's wall time, which also holds emission, vector work and the "
                             "eigensolves; the FP32 sigmas no longer stream the stored values "
                             "(QDKGB_BATCH_DIRECT=0 restores the slab sigma), so this is an equivalent rate"},
        "persistent_s": t_pers, "persistent_plan": plan,
        "sigma_gbs_per_fp32_sweep_bytes": _batch_bytes(inst),
        "max_sigma_applications": max(i["iterations"] for i in infos),
        "graph_replays": infos[-1]["graph_replays"],
        "e2e": {"value": len(inst) / t, "unit": "instances/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "note": "the call takes host integrals and returns host energies and 1-RDMs"},
        "gpu_launches": launches, "clocks": clk.summary(),
    }
    print(json.dumps(line))


# ------------------------------------------------------------------ CASCI(14e,14o), direct sigma
def run_cas14(args):
    """CASCI(14e,14o): 11,778,624 determinants, 3.98e10 matrix elements per
    sigma (no storable matrix: the sigma is recomputed on the fly), FP64 and
    mixed Davidson to |r| < 1e-8, then the spin-resolved RDMs of the mixed
    vector (the backward of the differentiable energy)."""
    import torch

    local = int(os.environ.get("LOCAL_RANK", "0"))
    rank = int(os.environ.get("RANK", "0"))
    torch.cuda.set_device(local)
    pkg = _package()
    pkg.build.build()
    capi = pkg.capi
    norb, nel, nchol = 14, 14, 28
    T, V, _ = pkg.integrals.synthetic_integrals(norb, nchol, SEED)
    a, b = capi.fci_dets(norb, nel // 2, nel // 2)
    N = len(a)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = capi.Context(local)
    ctx.set_stream(stream.cuda_stream)
    ctx.set_integrals(T, V)
    ctx.set_dets(a, b)
    ctx.build_direct_sigma()

    def solve(prec):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        E, C, info = ctx.davidson(tol=RES_TOL, precision=prec)
        torch.cuda.synchronize()
        return E, C, info, time.perf_counter() - t0

    x64 = torch.randn(N, dtype=torch.float64, device="cuda")
    y64 = torch.empty_like(x64)
    x32 = torch.randn(N, dtype=torch.float32, device="cuda")
    y32 = torch.empty_like(x32)
    t_s64 = time_spmv(ctx, capi.PREC_FP64, x64, y64, stream, reps=3)
    t_s32 = time_spmv(ctx, capi.PREC_MIXED, x32, y32, stream, reps=5)
    launches0 = capi.kernel_launches()
    with ClockSampler(local) as clk:
        Em, Cm, infom, tm = solve(capi.PREC_MIXED)
        E64, _, info64, t64 = solve(capi.PREC_FP64)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    R = ctx.rdms_spin_dep(Cm)
    torch.cuda.synchronize()
    t_rdm = time.perf_counter() - t0
    launches = capi.kernel_launches() - launches0
    ctx.close()
    # the drop-in path: create("multi_configuration_calculator", "gb300_cas")
    # .run(H, 7, 7) from host integrals to energy + CI vector + 1-RDMs; it
    # picks the direct sigma because the stored matrix exceeds the device
    calc = pkg.calculators.create("multi_configuration_calculator", "gb300_cas")
    calc.settings().set("precision", "mixed")
    calc.settings().set("calculate_one_rdm", True)
    calc.settings().set("device", local)
    t0 = time.perf_counter()
    Ep, wfn = calc.run(pkg.calculators.Hamiltonian(T, V, 0.0), nel // 2, nel // 2)
    t_plugin = time.perf_counter() - t0
    if rank != 0:
        return
    elems = 3.98e10
    line = {
        "metric": "casci_14e14o_time_to_energy", "value": tm, "unit": "s", "n_gpus": 1, "steps": 1, "warmup": 0,
        "ms_per_step": tm * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 sigma / double-float subspace / f64 refinement", "data": "synthetic",
        "config": {"workload": "CASCI(14e,14o) direct sigma, 11,778,624 determinants, Davidson to |r| < 1e-8",
                   "norb": norb, "nalpha": nel // 2, "nbeta": nel // 2, "ndets": N, "n_chol": nchol, "seed": SEED},
        "mixed": {"seconds": tm, "iterations": infom["iterations"], "spmv_fp32": infom["spmv_fp32"],
                  "spmv_fp64": infom["spmv_fp64"], "energy": Em},
        "fp64": {"seconds": t64, "iterations": info64["iterations"], "energy": E64},
        "mixed_speedup_vs_fp64": t64 / tm, "energy_error_vs_fp64": abs(Em - E64),
        "sigma": {"fp64_ms": t_s64 * 1e3, "fp32_ms": t_s32 * 1e3,
                  "elements_per_s_fp32": elems / t_s32, "elements_per_s_fp64": elems / t_s64,
                  "csr_equivalent_gbs_fp32": 478e9 / t_s32 / 1e9,
                  "note": "no stored matrix: 3.98e10 elements recomputed per sigma; CSR-equivalent GB/s = "
                          "478 GB (FP64 CSR with int32 columns) / sigma time"},
        "rdms_spin_dep_s": t_rdm, "rdm_trace": float(np.trace(R["aa"] + R["bb"])),
        "plugin": {"call": 'create("multi_configuration_calculator", "gb300_cas").run(H, 7, 7), mixed, 1-RDMs',
                   "seconds": t_plugin, "operator": wfn.info.get("operator"), "energy": Ep,
                   "energy_error_vs_fp64": abs(Ep - E64), "iterations": wfn.info.get("iterations")},
        "gpu_launches": launches, "clocks": clk.summary(),
    }
    print(json.dumps(line))


# ------------------------------------------------------------------ kernels of complete spaces
def run_rdm(args):
    """Spin-resolved RDMs (all five blocks) of a normalised random vector over
    the complete CASCI(nel, norb) space (default CASCI(14e,14o), 11,778,624
    determinants): seconds per call and the opposite-spin sweep's FP64
    multiply-adds (one per (alpha transition, beta transition) pair, with the
    reversed alpha transitions folded)."""
    import torch

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    pkg = _package()
    pkg.build.build()
    capi = pkg.capi
    norb, nel = args.norb, args.nel
    T, V, _ = pkg.integrals.synthetic_integrals(norb, args.nchol, SEED)
    a, b = capi.fci_dets(norb, nel // 2, nel // 2)
    C = np.random.default_rng(3).normal(size=len(a))
    C /= np.linalg.norm(C)
    with capi.Context(local) as ctx:
        ctx.set_integrals(T, V)
        ctx.set_dets(a, b)
        for _ in range(args.warmup):
            ctx.rdms_spin_dep(C)
        times = []
        for _ in range(args.steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            R = ctx.rdms_spin_dep(C)
            torch.cuda.synchronize()
            times.append(time.perf_counter() - t0)
    k = nel // 2
    na = math.comb(norb, k)
    # alpha transitions with k >= l: off-diagonal classes C(n-2, k-1) each, diagonal C(n-1, k-1)
    n_off, n_diag = math.comb(norb - 2, k - 1), math.comb(norb - 1, k - 1)
    alpha_tr = (norb * (norb - 1) // 2) * n_off + norb * n_diag
    beta_el = norb * (norb - 1) * n_off + norb * n_diag
    dfma = alpha_tr * beta_el
    t = float(np.median(times))
    print(json.dumps({"metric": "rdm_spin_dep_seconds", "value": t, "unit": "s", "n_gpus": 1, "steps": args.steps,
                      "warmup": args.warmup, "higher_is_better": False, "dtype": "f64", "data": "synthetic",
                      "config": {"workload": "spin-resolved RDMs, CASCI(%de,%do), %d determinants" % (nel, norb, na * na),
                                 "norb": norb, "nalpha": k, "nbeta": k},
                      "opposite_spin_dfma": dfma, "dfma_per_s": dfma / t, "trace": float(np.trace(R["aa"] + R["bb"]))}))


def run_direct(args):
    """The direct (recompute-on-the-fly) sigma of the complete CASCI(nel, norb)
    space: milliseconds per FP64 and FP32 application and elements per
    second (elements = determinants x stored row length)."""
    import torch

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    pkg = _package()
    pkg.build.build()
    capi = pkg.capi
    norb, nel = args.norb, args.nel
    T, V, _ = pkg.integrals.synthetic_integrals(norb, args.nchol, SEED)
    a, b = capi.fci_dets(norb, nel // 2, nel // 2)
    N = len(a)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    with capi.Context(local) as ctx:
        ctx.set_stream(stream.cuda_stream)
        ctx.set_integrals(T, V)
        ctx.set_dets(a, b)
        ctx.build_direct_sigma()
        x64 = torch.randn(N, dtype=torch.float64, device="cuda")
        y64 = torch.empty_like(x64)
        x32 = torch.randn(N, dtype=torch.float32, device="cuda")
        y32 = torch.empty_like(x32)
        t64 = time_spmv(ctx, capi.PREC_FP64, x64, y64, stream, reps=max(1, args.steps))
        t32 = time_spmv(ctx, capi.PREC_MIXED, x32, y32, stream, reps=max(1, args.steps))
    k = nel // 2
    s1 = k * (norb - k)
    rowlen = 1 + 2 * s1 + 2 * math.comb(k, 2) * math.comb(norb - k, 2) + s1 * s1
    elems = N * rowlen
    print(json.dumps({"metric": "direct_sigma_ms", "value": t32 * 1e3, "unit": "ms", "n_gpus": 1, "steps": args.steps,
                      "warmup": 0, "higher_is_better": False, "dtype": "f32", "data": "synthetic",
                      "config": {"workload": "direct sigma, CASCI(%de,%do), %d determinants" % (nel, norb, N),
                                 "norb": norb, "nalpha": k, "nbeta": k},
                      "fp32_ms": t32 * 1e3, "fp64_ms": t64 * 1e3, "elements": elems,
                      "elements_per_s_fp32": elems / t32, "elements_per_s_fp64": elems / t64}))


# ------------------------------------------------------------------ ASCI, 40 orbitals
def run_asci(args):
    """ASCI selected CI over 40 orbitals, n_alpha = n_beta = 8, integrals of
    the same recipe with diagonal spacing 0.1 and 80 Cholesky vectors; grown
    from the lowest-diagonal determinant (core Fixed 10,000, grow factor 8) to
    `--asci-dets` determinants (2,000,000 by default), then refined; FP64 H
    build + Davidson for the lowest root at every step, then the two lowest
    roots of the final space (FP64 H build + block Davidson)."""
    import torch

    local = int(os.environ.get("LOCAL_RANK", "0"))
    rank = int(os.environ.get("RANK", "0"))
    torch.cuda.set_device(local)
    pkg = _package()
    pkg.build.build()
    capi = pkg.capi
    norb, nel, nchol = 40, 16, 80
    T, V, _ = pkg.integrals.synthetic_integrals(norb, nchol, SEED, diag_spacing=0.1)
    ctx = capi.Context(local)
    ctx.set_integrals(T, V)
    a0, b0 = pkg.determinants.canonical_hf(nel // 2, nel // 2)
    ctx.set_dets(np.array([a0], dtype=np.uint64), np.array([b0], dtype=np.uint64))
    ctx.build_hamiltonian()
    E0 = float(ctx.diagonal()[0])
    kw = dict(ntdets_max=args.asci_dets, core_selection_fixed=1, ncdets_max=10000, grow_factor=8)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    Eg, a, b, c, _ = capi.asci(ctx, [a0], [b0], [1.0], E0, grow=True, refine=False, **kw)
    torch.cuda.synchronize()
    t_grow = time.perf_counter() - t0
    phases_grow = capi.asci_phase_times(ctx)
    t0 = time.perf_counter()
    refined = True
    try:
        E, a, b, c, _ = capi.asci(ctx, a, b, c, Eg, grow=False, refine=True, **kw)
    except capi.NotConverged:
        refined = False  # the reference's asci_refine stops the same way after max_refine_iter
        E = Eg
    torch.cuda.synchronize()
    t_ref = time.perf_counter() - t0
    phases_refine = capi.asci_phase_times(ctx)
    # the configuration's two roots: FP64 H build + block Davidson on the final space
    t0 = time.perf_counter()
    ctx.set_dets(a, b)
    ctx.build_hamiltonian()
    E2, _, info2 = ctx.davidson(tol=RES_TOL, nroots=2, max_m=64, want_vector=False)
    torch.cuda.synchronize()
    t_roots = time.perf_counter() - t0
    t = t_grow + t_ref + t_roots
    if rank != 0:
        return
    line = {"metric": "asci_40o_16e_time", "value": t, "unit": "s", "n_gpus": 1, "steps": 1, "warmup": 0,
            "ms_per_step": t * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": "ASCI grow + refine, 40 orbitals, 8 alpha + 8 beta electrons, core Fixed 10,000, "
                                   "grow factor 8, FP64 H build + Davidson (lowest root)",
                       "ntdets_max": args.asci_dets, "n_chol": nchol, "diag_spacing": 0.1, "seed": SEED},
            "grow_s": t_grow, "refine_s": t_ref, "refine_converged": refined,
            "phases": {"grow": phases_grow, "refine": phases_refine,
                       "note": "seconds per phase (determinant search, determinant-space set-up, H build, "
                               "Davidson), host-synchronised"},
            "two_roots": {"seconds": t_roots, "energies": [float(x) for x in E2],
                          "iterations": info2["iterations"], "sigma_applications": info2["spmv_fp64"],
                          "residual_norm": info2["residual_norm"], "nnz": int(ctx.nnz)},
            "ndets": int(len(a)), "energy_after_grow": Eg, "energy": E, "norm_c": float(np.linalg.norm(c))}
    print(json.dumps(line))


def run_pt2(args):
    """ASCI-PT2 in the reference's own test configuration (external/macis/
    tests/asci.cxx:488-570): water cc-pVDZ (24 orbitals, 5 + 5 electrons, the
    FCIDUMP committed under tests/golden), ASCI grown and refined to 10,000
    determinants (core Fixed) by the GPU, then E_PT2 of that wavefunction
    (pinned at -5.701535028967e-3).  A step is one qdkgb_asci_pt2 call from
    host determinants and coefficients to the host energy; the CPU baseline
    runs the oracle's PT2 on the same wavefunction with every host core."""
    import torch

    local = int(os.environ.get("LOCAL_RANK", "0"))
    rank = int(os.environ.get("RANK", "0"))
    torch.cuda.set_device(local)
    pkg = _package()
    pkg.build.build()
    capi = pkg.capi
    d = np.load(os.path.join(ROOT, "tests", "golden", "h2o_ccpvdz_fcidump.npz"))
    f = pkg.integrals.integrals_from_lines(int(d["norb"]), d["idx"], d["vals"], int(d["nelec"]), int(d["ms2"]))
    ctx = capi.Context(local)
    ctx.set_integrals(f["T"], f["V"])
    a0, b0 = pkg.determinants.canonical_hf(5, 5)
    ctx.set_dets(np.array([a0], dtype=np.uint64), np.array([b0], dtype=np.uint64))
    ctx.build_hamiltonian()
    E0 = float(ctx.diagonal()[0])
    E, a, b, c, _ = capi.asci(ctx, [a0], [b0], [1.0], E0, grow=True, refine=True, ntdets_max=10000,
                              core_selection_fixed=1)
    for _ in range(max(3, args.warmup)):
        capi.asci_pt2(ctx, a, b, c, E)
    torch.cuda.synchronize()
    launches0 = capi.kernel_launches()
    times = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            t0 = time.perf_counter()
            ept2, next_ = capi.asci_pt2(ctx, a, b, c, E)
            times.append(time.perf_counter() - t0)
    launches = capi.kernel_launches() - launches0
    t = float(np.mean(times))
    if rank != 0:
        return
    contribs = 0
    for x, y in zip(a, b):
        ka, kb = bin(int(x)).count("1"), bin(int(y)).count("1")
        sa, sb = ka * (24 - ka), kb * (24 - kb)
        contribs += 1 + sa + sb + sa * sb + (ka * (ka - 1) // 2) * ((24 - ka) * (23 - ka) // 2) + \
            (kb * (kb - 1) // 2) * ((24 - kb) * (23 - kb) // 2)
    line = {"metric": "asci_pt2_h2o_10k_time", "value": t, "unit": "s", "n_gpus": 1, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": t * 1e3, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "water cc-pVDZ FCIDUMP (tests/golden)",
            "config": {"workload": "ASCI-PT2 of the 10,000-determinant water cc-pVDZ ASCI wavefunction "
                                   "(asci.cxx:488-570), pt2_tol 1e-16", "ndets": int(len(a)),
                       "contributions": contribs, "l2": "hash table larger than L2"},
            "ept2": ept2, "ept2_reference": -5.701535028967e-03, "ept2_error": ept2 + 5.701535028967e-03,
            "external_determinants": int(next_), "contributions_per_s": contribs / t,
            "e2e": {"value": t, "unit": "s", "h2d_bytes_per_step": int(len(a)) * 24, "d2h_bytes_per_step": 16 + 8 * 2},
            "gpu_launches": launches // max(1, args.steps), "clocks": clk.summary()}
    if not args.no_cpu:
        import oracle

        oracle.build()
        H = oracle.Hamiltonian(f["T"], f["V"])
        t0 = time.perf_counter()
        e_orc, n_orc = oracle.asci_pt2(H, a, b, c, E)
        tc = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": tc, "unit": "s", "cores": oracle.num_threads(), "kind": "port",
                                "sample": "the full workload (one PT2 of the same wavefunction)",
                                "ept2": e_orc, "external_determinants": int(n_orc)}
    print(json.dumps(line))


def run_entropies(args):
    """Orbital entropies and mutual information (form_entropies) of the
    CASCI(10e,10o) ground state (63,504 determinants, synthetic integrals of
    the bench's recipe): a step is one qdkgb_orbital_entropies call from the
    host CI vector to the host s1 / s2 / I matrices; the CPU baseline runs the
    oracle's form_entropies on the same vector with every host core."""
    import torch

    local = int(os.environ.get("LOCAL_RANK", "0"))
    rank = int(os.environ.get("RANK", "0"))
    torch.cuda.set_device(local)
    pkg = _package()
    pkg.build.build()
    capi = pkg.capi
    norb, na = 10, 5
    T, V, _ = pkg.integrals.synthetic_integrals(norb, 2 * norb, SEED)
    ctx = capi.Context(local)
    E, C, _ = ctx.casci(T, V, na, na, tol=1e-8)
    a, b = capi.fci_dets(norb, na, na)
    ctx.set_integrals(T, V)
    ctx.set_dets(a, b)
    for _ in range(max(3, args.warmup)):
        ctx.orbital_entropies(C)
    torch.cuda.synchronize()
    launches0 = capi.kernel_launches()
    times = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            t0 = time.perf_counter()
            s1, s2, mi = ctx.orbital_entropies(C)
            times.append(time.perf_counter() - t0)
    launches = capi.kernel_launches() - launches0
    t = float(np.mean(times))
    if rank != 0:
        return
    line = {"metric": "orbital_entropies_casci10_time", "value": t, "unit": "s", "n_gpus": 1, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": t * 1e3, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "single-/two-orbital entropies and mutual information of the CASCI(10e,10o) "
                                   "ground state, 63,504 determinants", "seed": SEED},
            "s1_sum": float(s1.sum()), "mi_max": float(mi.max()),
            "e2e": {"value": t, "unit": "s", "h2d_bytes_per_step": int(len(C)) * 8,
                    "d2h_bytes_per_step": 8 * (norb + 2 * norb * norb)},
            "gpu_launches": launches // max(1, args.steps), "clocks": clk.summary()}
    if not args.no_cpu:
        import oracle

        oracle.build()
        t0 = time.perf_counter()
        o1, o2, om = oracle.entropies(norb, a, b, C)
        tc = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": tc, "unit": "s", "cores": oracle.num_threads(), "kind": "port",
                                "sample": "the full workload (one form_entropies of the same vector)",
                                "max_abs_diff_s2": float(np.abs(o2 - s2).max())}
    print(json.dumps(line))


def run_casscf(args):
    """CASSCF in the reference's own test configuration (external/macis/tests/
    mcscf.cxx:26-66): water cc-pVDZ (FCIDUMP under tests/golden), 1 inactive +
    8 active orbitals, 4 + 4 active electrons, from the start orbitals; a step
    is one qdkgb_casscf call (device CASCI, RDMs and integral transform per
    macro iteration).  The CPU baseline runs the oracle's casscf_diis on the
    same integrals with every host core."""
    import torch

    local = int(os.environ.get("LOCAL_RANK", "0"))
    rank = int(os.environ.get("RANK", "0"))
    torch.cuda.set_device(local)
    pkg = _package()
    pkg.build.build()
    capi = pkg.capi
    d = np.load(os.path.join(ROOT, "tests", "golden", "h2o_ccpvdz_fcidump.npz"))
    f = pkg.integrals.integrals_from_lines(int(d["norb"]), d["idx"], d["vals"], int(d["nelec"]), int(d["ms2"]))
    ctx = capi.Context(local)
    for _ in range(max(1, args.warmup)):
        capi.casscf(ctx, f["T"], f["V"], f["E_core"], 4, 4, 1, 8)
    torch.cuda.synchronize()
    launches0 = capi.kernel_launches()
    times = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            t0 = time.perf_counter()
            E, g, _, U, iters, conv = capi.casscf(ctx, f["T"], f["V"], f["E_core"], 4, 4, 1, 8)
            times.append(time.perf_counter() - t0)
    launches = capi.kernel_launches() - launches0
    t = float(np.mean(times))
    if rank != 0:
        return
    line = {"metric": "casscf_h2o_ccpvdz_8e8o_time", "value": t, "unit": "s", "n_gpus": 1, "steps": args.steps,
            "warmup": max(1, args.warmup), "ms_per_step": t * 1e3, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "water cc-pVDZ FCIDUMP (tests/golden)",
            "config": {"workload": "CASSCF, water cc-pVDZ, 1 inactive + CAS(8e,8o), 24 orbitals (mcscf.cxx:26-66)"},
            "energy": E, "energy_reference": -76.1114493227, "energy_error": E + 76.1114493227,
            "macro_iterations": iters, "converged": conv,
            "e2e": {"value": t, "unit": "s", "h2d_bytes_per_step": 8 * (24 ** 2 + 24 ** 4),
                    "d2h_bytes_per_step": 8 * (1 + 64 + 8 ** 4 + 24 ** 2)},
            "gpu_launches": launches // max(1, args.steps), "clocks": clk.summary()}
    if not args.no_cpu:
        import oracle

        oracle.build()
        t0 = time.perf_counter()
        Eo, _, _, it_o, _ = oracle.casscf(f["T"], f["V"], f["E_core"], 4, 4, 1, 8)
        tc = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": tc, "unit": "s", "cores": oracle.num_threads(), "kind": "port",
                                "sample": "the full workload (one casscf_diis of the same integrals)",
                                "energy": Eo, "macro_iterations": it_o}
    print(json.dumps(line))


def time_spmv(ctx, precision, x, y, stream, reps=20):
    import torch

    for _ in range(3):
        ctx.spmv_device(x.data_ptr(), y.data_ptr(), precision)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        ctx.spmv_device(x.data_ptr(), y.data_ptr(), precision)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / 1e3 / reps


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--norb", type=int, default=NORB)
    ap.add_argument("--nel", type=int, default=NEL)
    ap.add_argument("--nchol", type=int, default=NCHOL)
    ap.add_argument("--asci-dets", type=int, default=2000000)
    ap.add_argument("--batch-norb", type=int, default=0, help="batched: only the instances of this norb")
    ap.add_argument("--batch-count", type=int, default=0, help="batched: only the first N instances")
    ap.add_argument("--persistent", type=int, default=0, help="batched: 1 = the persistent cluster solver")
    ap.add_argument("--cluster", type=int, default=0, help="batched, persistent: CTAs per instance (0: tuned)")
    ap.add_argument("--workload", default="cas12",
                    choices=["cas12", "batched", "cas14", "asci", "pt2", "entropies", "casscf", "rdm", "direct"],
                    help="cas12: the headline CASCI(12e,12o); batched: 512 small instances; "
                         "cas14: CASCI(14e,14o) with the direct sigma")
    args = ap.parse_args()
    set_workload(args.norb, args.nel, args.nchol)
    if args.workload == "cas14":
        run_cas14(args)
    elif args.workload == "rdm":
        run_rdm(args)
    elif args.workload == "direct":
        run_direct(args)
    elif args.workload == "asci":
        run_asci(args)
    elif args.workload == "pt2":
        run_pt2(args)
    elif args.workload == "entropies":
        run_entropies(args)
    elif args.workload == "casscf":
        run_casscf(args)
    elif args.workload == "batched":
        if args.impl == "reference":
            run_reference_batched(args)
        else:
            run_batched(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
