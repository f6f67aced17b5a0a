#!/usr/bin/env python
"""Benchmark: time-to-gain of the symmetric-BEM forward path on one GB300.

Workload (config1, all data seeded and synthetic): 3 nested ico4 surfaces
(2562 vertices / 5120 triangles each, radii .87/.92/1 perturbed by a 2%
degree<=4 spherical-harmonic field), conductivities 1/.0125/1, HeadMat size
17926, 2000 dipoles, 64 EEG electrodes, 151 radial magnetometers at r=1.2.

One step = one full forward gain (HeadMat assembly, DipSourceMat, Head2EEG /
Head2MEG / DipSource2MEG, factorization, adjoint solves, gain products) in the
mixed-precision mode, geometry and sensor arrays already resident on the
device.  `value` is seconds per step (lower is better).  The FP64 drop-in is
timed on the same box in the same run, and the mixed result's relative error
against it is reported (target <= 1e-6).

`--impl reference` runs the reference CPU pipeline restated by the oracle
port (HeadMat, sensor matrices, the DSPTRF/DSPTRS adjoint solve, DipSourceMat,
contraction) once on the full workload, unscaled, on all host threads.

Inputs exceed the 129 MB L2 (the 2.6 GB head matrix is rebuilt every step),
so no explicit L2 flush is done between steps.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "time-to-gain (s) ico4-ico5, mixed-prec vs FP64 on same GB300 at rel err <=1e-6"


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), float(d["bf16_tflops"]), float(d.get("bf16_tflops_sustained", d["bf16_tflops"])), \
            "measured"
    return 6800.0, 1900.0, 1700.0, "fallback"


# ---------------------------------------------------------------------------
# clocks sampler
# ---------------------------------------------------------------------------
class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap,memory.used")

    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.device)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out = ""
        sm, mx, reasons, mem = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in out.splitlines():
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
                if len(f) > 9:
                    mem.append(float(f[9]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm),
                "memory_used_max_mib": max(mem) if mem else None}


# ---------------------------------------------------------------------------
# CPU baseline: the reference's pipeline restated by the oracle port
# ---------------------------------------------------------------------------
def workload_config(name: str, N: int, nd: int, ne: int, nm: int) -> dict:
    """The `config` object of the bench line; both arms print the same one for the same workload."""
    shape = {"config0": "3-layer ico3 head", "config1": "3-layer ico4 SH-perturbed head"}.get(name, name)
    return {"workload": f"{name}: {shape}, N={N}, {nd} dipoles, {ne} EEG, {nm} MEG", "N": N, "dipoles": nd,
            "eeg": ne, "meg": nm, "parallelism": "none (one head model per process; replicas under torchrun)",
            "l2": "inputs > L2 (the head matrix, 8 N^2 bytes, is rebuilt every step); no flush"}


def cpu_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def reference_cache_path(config: str) -> str:
    import tempfile
    return os.path.join(tempfile.gettempdir(), f"omg_bench_reference_{config}.json")


def cpu_pipeline(w, threads: int):
    """The reference's time-to-gain pipeline on the CPU at full size
    (oracle.forward_pipeline: HeadMat, H2EM, H2MM, DS2MM, then the
    GainEEGMEGadjoint solve by DSPTRF/DSPTRS, DipSourceMat and the
    contraction), all host threads.  Returns (seconds without the geometry
    set-up, per-stage seconds)."""
    from oracle import oracle
    oracle.set_threads(threads)
    oracle.openblas_threads(threads)
    _, _, t = oracle.forward_pipeline(w.head, w.dipoles, w.electrodes, w.squids if len(w.squids) else None)
    return sum(v for k, v in t.items() if k != "geometry"), t


def cpu_sample_time(config: str, threads: int):
    """Bounded CPU sample for the GPU line: the whole pipeline measured on the
    config0 head (N = 4486, 200 dipoles, 64 EEG, 32 MEG; ~10-20 s of CPU work)
    and each measured stage scaled to the bench workload by its operation count
    (pair integrals ~ T^2, the DSPTRF factorization ~ N^3, solves ~ N^2 k,
    DipSourceMat ~ dipoles x triangles, contraction ~ k N dipoles, sensor
    matrices ~ sensors x N)."""
    from openmeeg_gb300 import workloads
    w0 = workloads.config0()
    w1 = getattr(workloads, config)()
    _, t0 = cpu_pipeline(w0, threads)
    T0 = sum(t.shape[0] for t in w0.head.triangles)
    T1 = sum(t.shape[0] for t in w1.head.triangles)
    N0 = sum(v.shape[0] for v in w0.head.vertices) + T0 - w0.head.triangles[-1].shape[0]
    N1 = sum(v.shape[0] for v in w1.head.vertices) + T1 - w1.head.triangles[-1].shape[0]
    k0 = w0.electrodes.shape[0] + w0.squids.shape[0]
    k1 = w1.electrodes.shape[0] + w1.squids.shape[0]
    nd0, nd1 = w0.dipoles.shape[0], w1.dipoles.shape[0]
    scale = {"headmat": (T1 / T0) ** 2, "factor_solve": (N1 / N0) ** 3, "dsm": (nd1 / nd0) * (T1 / T0),
             "contract": (k1 * N1 * nd1) / (k0 * N0 * nd0), "h2em": N1 / N0,
             "h2mm": (w1.squids.shape[0] * N1) / max(1, w0.squids.shape[0] * N0),
             "ds2mm": (w1.squids.shape[0] * nd1) / max(1, w0.squids.shape[0] * nd0)}
    parts = {k: v * scale[k] for k, v in t0.items() if k in scale}
    sample = (f"the whole pipeline on the config0 head (N={N0}, {nd0} dipoles, {k0} sensor rows) measured stage by "
              f"stage ({sum(v for k, v in t0.items() if k != 'geometry'):.1f} s), each stage scaled to {config} by "
              f"its operation count (pair integrals T^2, DSPTRF N^3, DSM dipoles x T, contraction k N dipoles)")
    return sum(parts.values()), parts, sample


def read_reference_cache(config: str, cfg: dict):
    """The measurement an earlier `--impl reference` run of the same workload left in this
    machine's temp directory (within the last 12 hours), or None."""
    p = reference_cache_path(config)
    try:
        d = json.load(open(p))
    except (OSError, ValueError):
        return None
    if d.get("config") != cfg or time.time() - d.get("when", 0) > 12 * 3600:
        return None
    return d


def run_reference(args):
    """The reference arm: the reference's CPU pipeline for the bench workload,
    restated by the oracle port (C restatement of the assembly, LAPACK DSPTRF/
    DSPTRS for the solve), at full size and unscaled, on all host threads.  One
    full pipeline is several minutes of CPU work, so each invocation runs it
    once: the line reports the single step it ran (steps 1, warmup 0) beside the
    requested counts."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from openmeeg_gb300 import workloads
    from oracle import oracle
    w = getattr(workloads, args.config)()
    g = oracle.digest(w.head)
    nd, ne, nm = w.dipoles.shape[0], w.electrodes.shape[0], w.squids.shape[0]
    cfg = workload_config(args.config, g.N, nd, ne, nm)
    threads = cpu_threads()
    t_wall0 = time.perf_counter()
    v, parts = cpu_pipeline(w, threads)
    wall = time.perf_counter() - t_wall0
    sample = (f"the whole {args.config} workload, unscaled: one run of the reference pipeline (HeadMat, H2EM, "
              f"H2MM, DS2MM, GainEEGMEGadjoint with DSPTRF/DSPTRS on the packed head matrix, DipSourceMat of all "
              f"{nd} dipoles, contraction) by the oracle port")
    cpu = {"value": v, "unit": "s", "cores": threads, "kind": "port", "sample": sample,
           "stages_s": {k: round(x, 3) for k, x in parts.items()}}
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "s", "n_gpus": args.gpus, "steps": 1,
        "warmup": 0, "steps_requested": args.steps, "warmup_requested": args.warmup, "ms_per_step": v * 1e3,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded nested icosphere heads, dipoles, Fibonacci sensors)",
        "config": cfg, "cpu_baseline": cpu,
        "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "timed_wall_s": wall,
        "note": "one full, unscaled pipeline per invocation (several minutes of CPU work); no warm-up: the CPU "
                "path has no device state to warm",
    }
    try:
        with open(reference_cache_path(args.config), "w") as f:
            json.dump({"config": cfg, "value": v, "cores": threads, "stages_s": line["cpu_baseline"]["stages_s"],
                       "when": time.time()}, f)
    except OSError:
        pass
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
# executed FP64 flops per near pair (DADD + DMUL + 2 DFMA thread instructions) of near_pairs_kernel, ncu at config1
# (launch 3: 93,224 pairs, 1.735 GFLOP)
FP64_FLOPS_PER_NEAR_PAIR = 1.735e9 / 93224

# DRAM bytes per launch measured by ncu (dram__bytes_read.sum + dram__bytes_write.sum)
# on a smaller head, per unit of the kernel's size (the summaries in profiles/ give
# the command and the raw figures); scaled to the bench workload by that unit.
NCU_TRAFFIC_PER_UNIT = {
    # near pairs: DRAM bytes per near pair (ncu at config1, launch 3: 6.49 MB for 93,224 pairs)
    "near_pairs": 6.49e6 / 93224,
    # residual B - A X (double-float): bytes per N^2 element of the float-pair head matrix
    # (ncu at N = 17926: 3.205 GB per launch)
    "residual_df64": 9.97,
    # residual from digits: DRAM bytes per launch at config1 (N = 17926, 215 right-hand sides, tiles of
    # 128 x 224, one level group; ncu dram__bytes_read.sum + dram__bytes_write.sum of the first residual
    # launch: 14.01 GB + 157.5 MB), per byte of the 21 digit-plane reads the kernel structure implies
    # (21 x N x ld x 2 B = 13.54 GB)
    "residual_tc": (14.01e9 + 0.1575e9) / (21 * 17926 * 17984 * 2.0),   # 14.17 GB per launch; 1.05
    # grouped fold of the diagonal-block inverses: DRAM bytes per algorithmic byte (ncu at config1:
    # 2.72 GB read + 2.49 GB written for 2048 x 140 x 17926 B)
    "fold": (2.72e9 + 2.49e9) / (2048.0 * 140 * 17926),
}


def digit_tiles(n, k, n_sm=152):
    """The digit GEMM's tile width (columns per tile, a multiple of 16) and column-block count for an
    n x k output, as the library picks them (tc_residual.cu, digit_gemm)."""
    nrb = (n + 127) // 128
    ncb = (k + 255) // 256
    width = lambda nc: ((k + nc - 1) // nc + 15) // 16 * 16
    while 2 * nrb * ncb < n_sm and width(ncb + 1) >= 64:
        ncb += 1
    return width(ncb), ncb


def pipe_peaks():
    """Measured FMA instruction rates (per lane per second) of the FP32 and FP64
    pipes of this GPU (the library's probe kernel: 8 independent FMA chains per
    thread, 8 CTAs of 256 threads per SM, CUDA events); the rooflines of the
    CUDA-core kernels are taken against these."""
    import ctypes
    from openmeeg_gb300 import _lib
    lib = _lib.load()
    lib.omg_internal_pipe_peak.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    out = []
    for kind in (0, 1):
        v = ctypes.c_double()
        if lib.omg_internal_pipe_peak(kind, ctypes.byref(v)) != 0:
            raise RuntimeError("pipe peak probe failed")
        out.append(v.value)
    return {"fp32_fma_per_s": out[0], "fp64_fma_per_s": out[1]}


def assembly_evaluations(head):
    """Kernel evaluations of one head matrix (16-point rule): E_S = 16 (L T^2 / 2 + (L - 1) T^2) OperatorS and
    E_D = 16 (3 L - 4) T^2 P1 single-layer evaluations for L nested meshes of T triangles each (self pairs,
    adjacent pairs, barrier temporaries)."""
    L = len(head.triangles)
    T = head.triangles[0].shape[0]
    return 16 * (L * T * T // 2 + (L - 1) * T * T), 16 * (3 * L - 4) * T * T


def roofline_entry(name, launches, ms, steps, N, k, nd, stats, peaks_, pipes):
    """Roofline of one kernel over the timed region: achieved = algorithmic work
    per launch / mean launch duration (CUDA events around each launch on the
    library's stream).

    Algorithmic work:
      residual_tc -- R = B - A X from fixed-point digits on the tensor cores: 6 + 6 bf16
        digit planes, 21 digit pairs up to level 7, each an N x N x k_pad integer GEMM
        (k_pad = k rounded up to 128); the FP64-equivalent work is 2 N^2 k.
      residual_df64 -- R = B - A X in double-float arithmetic: reads the float-pair
        head matrix (8 N^2 bytes), X pairs (8 N k), B (8 N k), writes R (8 N k);
        N^2 k multiply-adds at 12 FP32 operations each (exact product + TwoSum).
      gemm_syrk -- tcgen05 3xTF32 trailing updates of the FP32 LDL^T: N^3/3
        algorithmic flops per factorization; executed tensor flops are 3x
        (hi*hi, hi*lo, lo*hi), against the TF32 dense rate (half of bf16).
    """
    if launches == 0:
        return None
    hbm, bf16, bf16_sus, kind = peaks_
    t_launch = ms / 1e3 / launches
    per_step = launches / steps
    info = {"kernel": name, "launches_per_step": per_step, "mean_launch_ms": ms / launches}
    if name == "residual_tc":
        # R = B - A X from 6 + 6 bf16 digit planes, 21 digit pairs (levels <= 7): every pair is a full
        # N x N x k integer GEMM on the tensor cores, k padded to the tiles' width (a multiple of 16)
        pairs = 21
        width, ncb = digit_tiles(N, k)
        kexec = width * ncb
        flops = 2.0 * N * N * kexec * pairs
        achieved = flops / t_launch / 1e12
        ld = (N + 63) // 64 * 64
        plane_reads = pairs * (N * ld * 2.0) * ncb     # each pair streams one A plane per column block
        measured = NCU_TRAFFIC_PER_UNIT["residual_tc"]
        info.update({"bound": "tensor", "achieved": achieved, "peak": bf16, "unit": "TFLOP/s",
                     "frac": achieved / bf16, "traffic": measured * plane_reads if measured else None,
                     "digit_plane_reads_per_launch": plane_reads,
                     "hbm_frac_if_plane_reads": plane_reads / t_launch / 1e9 / hbm,
                     "traffic_note": "DRAM bytes per launch from an ncu capture of the config1 residual, scaled by "
                                     "the plane reads (null when not captured)",
                     "algorithmic_fp64_equivalent_flops_per_launch": 2.0 * N * N * k,
                     "executed_bf16_flops_per_launch": flops,
                     "note": f"executed bf16 tensor flops (21 exact digit-pair GEMMs, {ncb} tile(s) of {width} "
                             f"columns) vs {kind} bf16 burst peak"})
    elif name == "residual_df64":
        nbytes = 8.0 * N * N + 24.0 * N * k
        achieved = nbytes / t_launch / 1e9
        tr = NCU_TRAFFIC_PER_UNIT.get(name)
        fp32_ops = 12.0 * N * N * k
        info.update({"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": (tr * N * N) if tr else None,
                     "algorithmic_bytes_per_launch": nbytes,
                     "fp32_issue_frac_of_measured": fp32_ops / t_launch / pipes["fp32_fma_per_s"],
                     "note": f"HBM fraction of {kind} copy bandwidth; the kernel is FP32-issue bound "
                             f"(12 FP32 ops per multiply-add), see fp32_issue_frac_of_measured"})
    elif name == "solve_sweep":
        # one triangular sweep per launch (2 sweeps per solve, 2 solves per gain): nrhs N^2 algorithmic FP32
        # flops per sweep (sum over blocks of 2 x 128 x rows below x nrhs), executed 3x as TF32 products;
        # bounded by its dependency chain (one 128-row block product + epilogue + flag hand-over per block)
        flops = k * N ** 2
        achieved = flops / t_launch / 1e12
        tf32_peak = bf16 / 2.0
        info.update({"bound": "tensor (dependency chain)", "achieved": 3 * achieved, "peak": tf32_peak,
                     "unit": "TFLOP/s", "frac": 3 * achieved / tf32_peak, "traffic": None,
                     "algorithmic_fp32_tflops": achieved,
                     "chain_us_per_block": t_launch * 1e6 / ((N + 127) // 128),
                     "note": f"persistent sweep: executed TF32 tensor flops vs half the {kind} bf16 burst peak; the "
                             f"141-block dependency chain bounds it (chain_us_per_block)"})
    elif name == "gemm_solve":
        # the FP32 solves: a dependent chain of tensor-core updates per sweep (one per 128-row block), each
        # sweep nrhs N^2 algorithmic flops (forward: sum over blocks of 2 (N - k1) nrhs 128), executed TF32
        # tensor flops 3x; latency-bound (each update waits for the previous one's band copy)
        flops = 4.0 * k * N ** 2 / per_step   # two solves of two sweeps each per gain
        achieved = flops / t_launch / 1e12
        tf32_peak = bf16 / 2.0
        info.update({"bound": "tensor", "achieved": 3 * achieved, "peak": tf32_peak, "unit": "TFLOP/s",
                     "frac": 3 * achieved / tf32_peak, "traffic": None, "algorithmic_fp32_tflops": achieved,
                     "note": "dependent chain of 128-deep updates (141 per sweep at config1): latency-bound, "
                             f"executed TF32 tensor flops vs half the {kind} bf16 burst peak"})
    elif name == "gemm_syrk":
        # trailing updates of the FP32 LDL^T on the tensor cores: sum over panels of
        # 2 (N - k1)^2 / 2 * 128 = ~N^3/3 algorithmic flops per factorization (lower triangle only);
        # executed TF32 tensor flops are 3x (hi*hi, hi*lo, lo*hi)
        flops = (N ** 3 / 3.0) / per_step
        achieved = flops / t_launch / 1e12
        tf32_peak = bf16 / 2.0
        info.update({"bound": "tensor", "achieved": 3 * achieved, "peak": tf32_peak, "unit": "TFLOP/s",
                     "frac": 3 * achieved / tf32_peak, "traffic": None, "algorithmic_fp32_tflops": achieved,
                     "note": f"executed TF32 tensor flops (3 per FP32-accurate product) vs half the {kind} bf16 "
                             f"burst peak (the TF32 dense rate is half the bf16 rate)"})
    elif name == "ff_block":
        # far-field FP32 Gauss products: 16 x 16 point pairs per triangle pair below 6 max edges, 7 x 7 from
        # there on; S and both D from the same distances, 12 FP32 operations per point pair (3 differences,
        # 3 for r^2, rsqrt, 2 for r^-3, 3 accumulations: the normal components r.n fold into per-point weights
        # since the points lie in their triangles' planes)
        n16 = stats.get("_pairs_6", 0) - stats.get("_near_pairs", 0)
        n7 = stats.get("_tri_pairs", 0) - stats.get("_pairs_6", 0)
        ops = 12.0 * (256 * n16 + 49 * n7) / per_step
        achieved = ops / t_launch
        peak = pipes["fp32_fma_per_s"]
        info.update({"bound": "fp32", "achieved": achieved / 1e12, "peak": peak / 1e12,
                     "unit": "T FP32 op/s", "frac": achieved / peak, "traffic": None,
                     "note": "FP32-pipe bound (rsqrt + FMA); peak: measured FP32 FMA instruction rate of this GPU"})
    elif name == "near_pairs":
        # FP64 analytic near-pair integrals (OperatorS, P1 single layer both ways at the 16 points of the rule):
        # FP64 operations executed per near pair from an ncu capture (thread-level DADD + DMUL + 2 DFMA, the
        # library's log/atan2/sqrt/division sequences included) against the nominal FP64 rate
        pairs = stats.get("_near_pairs", 0)
        flops = FP64_FLOPS_PER_NEAR_PAIR * pairs / per_step
        achieved = flops / t_launch
        peak = 2.0 * pipes["fp64_fma_per_s"]
        info.update({"bound": "fp64", "achieved": achieved / 1e12, "peak": peak / 1e12, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": NCU_TRAFFIC_PER_UNIT["near_pairs"] * pairs / per_step,
                     "near_pairs_per_launch": pairs / per_step,
                     "evals_per_s": 16 * 3 * pairs / per_step / t_launch,
                     "note": "executed FP64 flops (ncu op counts per near pair) vs the measured FP64 FMA rate of "
                             "this GPU (x2 flops); evals_per_s counts the 16 OperatorS + 32 P1 single-layer "
                             "evaluations of each near pair"})
    elif name == "dsm":
        # DipSourceMat: the first adaptive level of every (dipole, triangle) pair in FP32 (both integrands at
        # the 16 rule points of the triangle and of its 4 halves: 80 points), the pairs that level does not
        # settle by the FP64 recursion; runs on the second stream under the solves
        T = stats.get("_triangles", 0)
        evals = 80.0 * nd * T / per_step
        info.update({"bound": "fp32 (FP64 on the unsettled pairs)", "achieved": None, "peak": None, "unit": None,
                     "frac": None, "traffic": None, "evals_per_s": evals / t_launch,
                     "note": "first-level integrand evaluations (80 points per dipole-triangle pair) per second; "
                             "the launch overlaps the solves on the second stream, so its event time includes "
                             "waiting for SMs"})
    elif name == "fold":
        # the folds of the diagonal-block inverses into the solve operators after the factorization, one grouped
        # launch: every element of the panels below the blocks and of the block rows left of them (N - nk_b rows
        # or columns of 128 per block b) is read and written as TF32 head + remainder, 16 bytes, so
        # 2048 (nblocks - 1) N bytes in all; the inverses themselves (64 KB each) stay in L2
        nblk = (N + 127) // 128
        nbytes = 2048.0 * (nblk - 1) * N / per_step
        achieved = nbytes / t_launch / 1e9
        tr = NCU_TRAFFIC_PER_UNIT.get(name)
        info.update({"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": tr * nbytes if tr else None, "algorithmic_bytes_per_launch": nbytes,
                     "note": f"280 3xTF32 products at config1 in one persistent launch; HBM fraction of {kind} copy "
                             f"bandwidth"})
    elif name in ("potrf_inv", "apply_inv"):
        info.update({"bound": "latency", "achieved": None, "peak": None, "unit": None, "frac": None, "traffic": None,
                     "note": "one diagonal block per launch (128 x 128, one CTA), sequential over the blocks: "
                             "latency bound, no bandwidth or tensor roofline applies"})
    else:
        info.update({"bound": None, "achieved": None, "peak": None, "unit": None, "frac": None, "traffic": None})
    return info


def max_over_ranks(value: float, device) -> float:
    """The slowest rank's time: every rank contributes its own value, all receive the maximum
    (replicas share no data; this is the only collective of the multi-GPU bench)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.barrier()
    return float(t.item())


def whole_job_rate(units_per_rank: float, world: int, t_max: float) -> float:
    """Units all ranks processed per second of the slowest rank (weak scaling: fixed work per rank)."""
    return units_per_rank * world / t_max


def tri_pairs(head):
    """Triangle pairs the head matrix integrates (S for non-barrier pairs, D and D* both ways): the pair
    loop of the symmetric BEM over nested meshes (self pairs and adjacent pairs)."""
    T = [t.shape[0] for t in head.triangles]
    L = len(T)
    pairs = 0
    for m in range(L):
        pairs += T[m] * (T[m] + 1) // 2                 # self pair (upper triangle)
        if m > 0:
            pairs += T[m] * T[m - 1]                     # adjacent pair
    return pairs


def near_pairs_count(head, rho=1.5):
    """Near triangle pairs of the mixed head matrix (those integrated by the FP64 analytic kernels): centroid
    distance below rho times the larger of the two triangles' longest edges, over the self pairs (j >= i) and
    the adjacent mesh pairs, as the far-field kernel lists them."""
    from scipy.spatial import cKDTree
    cen, hmax = [], []
    for V, T in zip(head.vertices, head.triangles):
        P = V[T]
        cen.append(P.mean(axis=1))
        e = np.stack([np.linalg.norm(P[:, 1] - P[:, 0], axis=1), np.linalg.norm(P[:, 2] - P[:, 1], axis=1),
                      np.linalg.norm(P[:, 0] - P[:, 2], axis=1)], axis=1)
        hmax.append(e.max(axis=1))
    count = 0
    for m in range(len(cen)):
        for m2 in ([m] if m == 0 else [m - 1, m]):
            r = rho * max(hmax[m].max(), hmax[m2].max())
            pairs = cKDTree(cen[m]).query_ball_tree(cKDTree(cen[m2]), r)
            for i, js in enumerate(pairs):
                if not js:
                    continue
                js = np.asarray(js)
                if m2 == m:
                    js = js[js >= i]
                d = np.linalg.norm(cen[m2][js] - cen[m][i], axis=1)
                count += int(np.count_nonzero(d < rho * np.maximum(hmax[m][i], hmax[m2][js])))
    return count


def run_gpu(args):
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    __import__("__graft_entry__").build()
    from openmeeg_gb300 import _lib, api, workloads

    w = getattr(workloads, args.config)()
    ctx = api.Context(local)
    ctx.bind_current_stream()
    geo = api.Geometry.from_head(w.head, ctx)
    dev = torch.device("cuda", local)
    dip = torch.as_tensor(w.dipoles, dtype=torch.float64, device=dev)
    el = torch.as_tensor(w.electrodes, dtype=torch.float64, device=dev)
    sq = torch.as_tensor(w.squids, dtype=torch.float64, device=dev) if len(w.squids) else None
    N = geo.size
    nd, ne, nm = dip.shape[0], el.shape[0], (0 if sq is None else sq.shape[0])

    def step(prec):
        return api.forward_gain(geo, dip, el, sq, precision=prec)

    if args.only_mixed or args.only_fp64:
        for _ in range(args.warmup + args.steps):
            step("mixed" if args.only_mixed else "fp64")
        torch.cuda.synchronize()
        print(json.dumps({"only": "mixed" if args.only_mixed else "fp64", "config": args.config, "steps": args.steps}))
        return 0
    # FP64 drop-in on the same box (its result is the accuracy reference)
    step("fp64")
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f64_times = []
    for _ in range(max(1, args.fp64_steps)):
        e0.record()
        ge64, gm64, st64 = step("fp64")
        e1.record()
        torch.cuda.synchronize()
        f64_times.append(e0.elapsed_time(e1) / 1e3)
    t_fp64 = float(np.median(f64_times))

    for _ in range(args.warmup):
        step("mixed")
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clocks = Clocks(local)
    clocks.start()
    launches0 = ctx.launches()
    torch.cuda.synchronize()
    e0.record()
    for _ in range(args.steps):
        gex, gmx, stx = step("mixed")
    e1.record()
    torch.cuda.synchronize()
    launches = ctx.launches() - launches0
    ck = clocks.stop()
    # per-kernel breakdown from separate profiled steps (events around every launch), outside the timed region
    _lib.profile_enable(True)
    _lib.profile_read()
    for _ in range(args.profile_steps):
        step("mixed")
    torch.cuda.synchronize()
    _lib.profile_enable(False)
    prof = _lib.profile_read()
    t_step = e0.elapsed_time(e1) / 1e3 / args.steps
    t_max = max_over_ranks(t_step, dev) if world > 1 else t_step

    def relerr(a, b):
        return float(torch.linalg.norm(a - b) / torch.linalg.norm(b))

    err_eeg = relerr(gex, ge64)
    err_meg = relerr(gmx, gm64) if gm64 is not None else None

    # end to end through the C ABI with host buffers: geometry from host arrays + gain_host, the sources and
    # the gains in pinned host memory
    def pinned(a):
        t = torch.empty(a.shape, dtype=torch.float64, pin_memory=True).numpy()
        t[...] = a
        return t
    dip_h = pinned(np.ascontiguousarray(np.asarray(w.dipoles, np.float64)[:, :6]))
    el_h = pinned(np.ascontiguousarray(np.asarray(w.electrodes, np.float64)[:, :3]))
    sq_h = pinned(np.ascontiguousarray(np.asarray(w.squids, np.float64)[:, :6])) if nm else None
    out_h = (pinned(np.zeros((nd, ne))), pinned(np.zeros((nd, nm))))
    e2e_times = []
    for _ in range(max(1, args.e2e_steps)):
        torch.cuda.synchronize()
        s = time.perf_counter()
        g2 = api.Geometry.from_head(w.head, ctx)
        api.forward_gain(g2, dip_h, el_h, sq_h, precision="mixed", host=True, out=out_h)
        e2e_times.append(time.perf_counter() - s)
        del g2
    t_e2e = float(np.median(e2e_times))
    h2d = sum(a.nbytes for a in w.head.vertices) + sum(a.nbytes for a in w.head.triangles) + \
        w.dipoles.nbytes + w.electrodes.nbytes + (w.squids.nbytes if nm else 0)
    d2h = 8 * nd * (ne + nm)

    # roofline of the dominant kernel over the timed region: the largest kernel on the main streams
    # (DipSourceMat runs on the second stream under the solves; its event time includes waiting for SMs)
    pk = peaks()
    pipes = pipe_peaks()
    main = {n: v for n, v in prof.items() if n != "dsm"}
    dom = max(main.items(), key=lambda kv: kv[1][1]) if main else ("none", (0, 0.0))
    dname, (dl, dms) = dom
    total_prof_ms = sum(v[1] for v in prof.values())
    stx_r = dict(stx)
    stx_r["_tri_pairs"] = tri_pairs(w.head)
    stx_r["_near_pairs"] = near_pairs_count(w.head)
    stx_r["_pairs_6"] = near_pairs_count(w.head, 6.0)   # pairs below the 7-point far-field tier
    stx_r["_triangles"] = sum(t.shape[0] for t in w.head.triangles)
    roof = roofline_entry(dname, dl, dms, args.profile_steps, N, ne + nm, nd, stx_r, pk, pipes)
    roof["dominant_rule"] = "largest profiled kernel on the main streams (DipSourceMat overlaps on the second one)"
    others = {n: roofline_entry(n, v[0], v[1], args.profile_steps, N, ne + nm, nd, stx_r, pk, pipes)
              for n, v in prof.items() if n in ("residual_tc", "residual_df64", "gemm_syrk", "ff_block", "near_pairs",
                                                 "solve_sweep", "dsm", "fold")
              and n != dname}
    e_s, e_d = assembly_evaluations(w.head)
    assembly = {"evaluations_per_headmat": {"E_S": e_s, "E_D": e_d},
                "mixed_evals_per_s": (e_s + e_d) / (stx["t_headmat_ms"] / 1e3),
                "fp64_evals_per_s": (e_s + e_d) / (st64["t_headmat_ms"] / 1e3),
                "note": "E_S + E_D kernel evaluations of the 16-point rule per head matrix over the head-matrix "
                        "stage time (mixed: FP32 far pairs, FP64 analytic near pairs; FP64: all analytic)"}

    cfg = workload_config(args.config, N, nd, ne, nm)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cached = read_reference_cache(args.config, cfg)
        if cached:
            cpu = {"value": cached["value"], "unit": "s", "cores": cached["cores"], "kind": "port",
                   "sample": "the whole workload, unscaled: measured by this machine's bench.py --impl reference "
                             f"run {int(time.time() - cached['when'])} s before this line",
                   "stages_s": cached["stages_s"]}
        else:
            threads = cpu_threads()
            total, parts, sample = cpu_sample_time(args.config, threads)
            cpu = {"value": total, "unit": "s", "cores": threads, "kind": "port", "sample": sample,
                   "stages_s": {k: round(x, 3) for k, x in parts.items()}}

    if rank == 0:
        line = {
            "metric": METRIC, "value": t_max / world, "unit": "s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max * 1e3, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64 (mixed); f64 drop-in timed beside it",
            "data": "synthetic (seeded nested icosphere heads, dipoles, Fibonacci sensors)",
            "config": cfg,
            "mixed_stats": {k: (round(v, 3) if isinstance(v, float) else v) for k, v in stx.items()},
            "fp64_stats": {k: (round(v, 3) if isinstance(v, float) else v) for k, v in st64.items()},
            "e2e": {"value": t_e2e, "unit": "s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                    "path": "omg_geometry_create + omg_gain_host (pinned host buffers, mixed; median of "
                            f"{max(1, args.e2e_steps)} steps)"},
            "gpu_launches": int(launches),
            "kernels_ms_per_step": {k: round(v[1] / args.profile_steps, 3) for k, v in
                                    sorted(prof.items(), key=lambda kv: -kv[1][1])},
            "profiled_ms_per_step": round(total_prof_ms / args.profile_steps, 3),
            "profile_note": "per-kernel CUDA-event times from separate profiled steps (not the timed ones)",
            "roofline": roof,
            "roofline_other": others,
            "assembly": assembly,
            "pipe_peaks_measured": pipes,
            "clocks": ck,
            "cpu_baseline": cpu,
            # last, so that the end of the line carries the metric's own comparison
            "fp64_s": t_fp64, "fp64_steps": len(f64_times),
            "rel_err_vs_fp64": {"eeg": err_eeg, "meg": err_meg},
            "speedup_vs_fp64": t_fp64 / t_step,
        }
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()
    return 0


def run_batch(args):
    """config3: 32 uneven heads as one captured graph (mixed precision), models/s,
    next to the sequential per-model FP64 loop on the same GPU."""
    import torch
    local = int(os.environ.get("LOCAL_RANK", "0"))
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    torch.cuda.set_device(local)
    __import__("__graft_entry__").build()
    from openmeeg_gb300 import api, workloads
    import tempfile
    os.environ.setdefault("OMG_TUNE_CACHE", os.path.join(tempfile.gettempdir(), "omg_tune_cache.txt"))
    ws = workloads.config3_models()
    ctx = api.Context(local)
    geos = [api.Geometry.from_head(w.head, ctx) for w in ws]
    sizes = [g.size for g in geos]
    nd_tot = sum(w.dipoles.shape[0] for w in ws)
    ev = lambda: torch.cuda.Event(enable_timing=True)

    # sequential per-model FP64 loop (the reference shape of the computation)
    ref = []
    torch.cuda.synchronize()
    e0, e1 = ev(), ev()
    t0 = time.perf_counter()
    e0.record(torch.cuda.current_stream())
    for g, w in zip(geos, ws):
        ge, _, _ = api.forward_gain(g, w.dipoles, w.electrodes, None, precision="fp64")
        ref.append(ge)
    e1.record(torch.cuda.current_stream())
    torch.cuda.synchronize()
    t_seq64 = time.perf_counter() - t0

    # sequential per-model mixed loop (the same precision as the batch, no graph)
    t0 = time.perf_counter()
    for g, w in zip(geos, ws):
        api.forward_gain(g, w.dipoles, w.electrodes, None, precision="mixed")
    torch.cuda.synchronize()
    t_seqmx = time.perf_counter() - t0

    # batched: plan + tune + capture, then replays
    t0 = time.perf_counter()
    b = api.BatchForward([(g, w.dipoles, w.electrodes, None) for g, w in zip(geos, ws)], precision="mixed",
                         n_branches=args.branches)
    t_create = time.perf_counter() - t0
    for _ in range(args.warmup):
        b.run()
    clocks = Clocks(local)
    clocks.start()
    s = torch.cuda.current_stream()
    torch.cuda.synchronize()
    e0, e1 = ev(), ev()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        b.run()          # blocking: replays on the context stream and checks every model
    t_wall = (time.perf_counter() - t0) / args.steps
    ck = clocks.stop()
    info = b.info()
    errs = []
    for i in range(len(ws)):
        ge, _ = b.gains(i)
        errs.append(float(torch.linalg.norm(ge - ref[i]) / torch.linalg.norm(ref[i])))

    # end to end through the public API with host buffers: geometries from host
    # arrays, batch creation (plan, cached branch count, capture), one run, gains to host
    t0 = time.perf_counter()
    geos2 = [api.Geometry.from_head(w.head, ctx) for w in ws]
    b2 = api.BatchForward([(g, w.dipoles, w.electrodes, None) for g, w in zip(geos2, ws)], precision="mixed",
                          n_branches=info["n_branches"])
    b2.run()
    host = [b2.gains(i)[0].cpu() for i in range(len(ws))]
    t_e2e = time.perf_counter() - t0
    del b2, geos2, host
    h2d = sum(sum(a.nbytes for a in w.head.vertices) + sum(a.nbytes for a in w.head.triangles) + w.dipoles.nbytes +
              w.electrodes.nbytes for w in ws)
    d2h = sum(8 * w.dipoles.shape[0] * w.electrodes.shape[0] for w in ws)
    if rank == 0:
        line = {
            "metric": "batched forward throughput (models/s), 32 uneven heads, mixed precision, graph replay",
            "value": len(ws) / t_wall * world, "unit": "models/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_wall * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64 (mixed)", "data": "synthetic (seeded nested icosphere heads)",
            "config": {"workload": "config3: 32 heads, ico3/ico4 surfaces, 3-4 layers, inner radii +-3%, "
                                   "100-1000 dipoles, 64 EEG", "N_min": min(sizes), "N_max": max(sizes),
                       "N_sum": sum(sizes), "dipoles": nd_tot, "parallelism": "single GPU, graph branches",
                       "l2": "inputs > L2 (every head matrix rebuilt each step); no flush"},
            "sequential_fp64_s": t_seq64, "sequential_fp64_models_per_s": len(ws) / t_seq64,
            "speedup_vs_sequential_fp64": t_seq64 / t_wall,
            "sequential_mixed_s": t_seqmx, "speedup_vs_sequential_mixed": t_seqmx / t_wall,
            "batch_create_s": t_create, "batch_info": info,
            "rel_err_vs_fp64": {"max": max(errs), "median": float(np.median(errs))},
            "e2e": {"value": len(ws) / t_e2e, "unit": "models/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h),
                    "path": "Geometry.from_head x32 + BatchForward (plan, cached tune, capture) + run + gains to host"},
            "gpu_launches": int(info["launches_per_run"]) * args.steps,
            "clocks": ck,
        }
        print(json.dumps(line))
    return 0


def run_large(args):
    """config4: 4 layers ico5 (N = 102408), 10000 dipoles, 256 EEG + 306 MEG.  One FP64 drop-in and one
    mixed-precision time-to-gain on the same GPU, the memory each needed, the mixed result's error against
    the FP64 one, and both against the analytic nested-sphere series (EEG) and Sarvas's formula (MEG) on a
    sample of the dipoles."""
    import torch
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    __import__("__graft_entry__").build()
    from oracle import analytic as an
    from openmeeg_gb300 import api, workloads
    w = workloads.config4()
    ctx = api.Context(local)
    geo = api.Geometry.from_head(w.head, ctx)
    N = geo.size
    dev = torch.device("cuda", local)
    dip = torch.as_tensor(w.dipoles, dtype=torch.float64, device=dev)
    el = torch.as_tensor(w.electrodes, dtype=torch.float64, device=dev)
    sq = torch.as_tensor(w.squids, dtype=torch.float64, device=dev)
    out, res = {}, {}
    for prec in args.large_precisions.split(","):
        clocks = Clocks(local)
        clocks.start()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ge, gm, st = api.forward_gain(geo, dip, el, sq, precision=prec)
        torch.cuda.synchronize()
        t = time.perf_counter() - t0
        ck = clocks.stop()
        out[prec] = (ge.cpu().numpy(), gm.cpu().numpy())
        del ge, gm
        res[prec] = {"time_to_gain_s": t, "stats": {k: (round(v, 3) if isinstance(v, float) else v)
                                                    for k, v in st.items()},
                     "library_peak_bytes": int(st["device_bytes"]), "clocks": ck}
    ns = min(args.analytic_dipoles, w.dipoles.shape[0])
    radii = [float(np.linalg.norm(v, axis=1).mean()) for v in w.head.vertices]
    sig = [d[2] for d in w.head.domains if d[2] > 0]
    Va = an.eeg_sphere(radii, sig, w.dipoles[:ns], w.electrodes)
    Ba = an.sarvas(w.dipoles[:ns], w.squids)
    for prec, (ge, gm) in out.items():
        res[prec]["analytic_eeg"] = {"rdm_max": float(an.rdm(ge[:, :ns], Va).max()),
                                     "mag_max": float(an.mag(ge[:, :ns], Va).max()),
                                     "rdm_median": float(np.median(an.rdm(ge[:, :ns], Va)))}
        res[prec]["analytic_meg"] = {"rdm_max": float(an.rdm(gm[:, :ns], Ba).max()),
                                     "mag_max": float(an.mag(gm[:, :ns], Ba).max())}
    line = {"metric": "time-to-gain (s), config4 large head", "unit": "s", "n_gpus": 1,
            "config": {"workload": "config4: 4 nested ico5 spheres r .85/.88/.92/1, sigma .33/1.79/.0042/.33, "
                                   "N=%d, 10000 dipoles r<0.8, 256 EEG, 306 radial MEG at r=1.15" % N, "N": N,
                       "analytic_sample_dipoles": ns},
            "results": res}
    if "fp64" in out and "mixed" in out:
        e64, m64 = out["fp64"]
        emx, mmx = out["mixed"]
        line["value"] = res["mixed"]["time_to_gain_s"]
        line["speedup_vs_fp64"] = res["fp64"]["time_to_gain_s"] / res["mixed"]["time_to_gain_s"]
        line["rel_err_vs_fp64"] = {"eeg": float(np.linalg.norm(emx - e64) / np.linalg.norm(e64)),
                                   "meg": float(np.linalg.norm(mmx - m64) / np.linalg.norm(m64))}
    print(json.dumps(line))
    return 0


def run_adjoint(args):
    """config2: config1 geometry, 500 dipoles, conductivities sampled log-uniformly within x[0.5, 2].
    Gain + gradient (d gain / d conductivities and d gain / d dipoles through the torch.autograd.Function)
    in FP64 and mixed precision; checked against central finite differences (FP64, relative step 1e-6)
    for the 3 conductivities and a sample of dipole coordinates, and mixed against FP64."""
    import torch
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    __import__("__graft_entry__").build()
    from openmeeg_gb300 import adjoint, api, workloads
    w = workloads.config2(base=args.head)
    ctx = api.Context(local)
    geo = api.Geometry.from_head(w.head, ctx)
    dev = torch.device("cuda", local)
    sig0 = torch.tensor([d[2] for d in w.head.domains], dtype=torch.float64)
    dip0 = torch.as_tensor(w.dipoles, dtype=torch.float64, device=dev)
    k = w.electrodes.shape[0] + w.squids.shape[0]
    Gbar = torch.randn(k, dip0.shape[0], generator=torch.Generator().manual_seed(11), dtype=torch.float64).to(dev)

    def loss(sig, dip, prec):
        return (adjoint.gain(sig, dip, geo, w.head.domains, w.electrodes, w.squids, precision=prec) * Gbar).sum()

    res, grads = {}, {}
    for prec in ("fp64", "mixed"):
        sig = sig0.clone().requires_grad_(True)
        dip = dip0.clone().requires_grad_(True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        L = loss(sig, dip, prec)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        gs, gd = torch.autograd.grad(L, [sig, dip])
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        grads[prec] = (gs.detach().cpu().numpy(), gd.detach().cpu().numpy())
        res[prec] = {"forward_s": t1 - t0, "backward_s": t2 - t1}
    # central differences (FP64) for the conductivities
    gs64 = grads["fp64"][0]
    fd = np.zeros_like(gs64)
    with torch.no_grad():
        for kd in range(len(sig0)):
            if sig0[kd] == 0:
                continue
            h = 1e-6 * float(sig0[kd])
            sp, sm = sig0.clone(), sig0.clone()
            sp[kd] += h
            sm[kd] -= h
            fd[kd] = (float(loss(sp, dip0, "fp64")) - float(loss(sm, dip0, "fp64"))) / (2 * h)
    nz = sig0.numpy() > 0
    sig_err = float(np.max(np.abs(gs64[nz] - fd[nz]) / np.abs(fd[nz])))
    # central differences for a sample of dipole coordinates: the head matrix and its solves do not
    # depend on the dipoles, so each difference re-evaluates the full gain at two perturbed dipole sets
    rng = np.random.default_rng(3)
    sample = [(int(j), int(c)) for j, c in zip(rng.integers(0, dip0.shape[0], args.fd_dipoles),
                                               rng.integers(0, 6, args.fd_dipoles))]
    gd64 = grads["fp64"][1]
    dip_err = 0.0
    with torch.no_grad():
        for j, c in sample:
            h = 1e-6
            dp, dm = dip0.clone(), dip0.clone()
            dp[j, c] += h
            dm[j, c] -= h
            f = (float(loss(sig0, dp, "fp64")) - float(loss(sig0, dm, "fp64"))) / (2 * h)
            dip_err = max(dip_err, abs(gd64[j, c] - f) / max(abs(f), 1e-30))
    mix_sig = float(np.linalg.norm(grads["mixed"][0] - gs64) / np.linalg.norm(gs64))
    mix_dip = float(np.linalg.norm(grads["mixed"][1] - gd64) / np.linalg.norm(gd64))
    line = {"metric": "gain + gradient time (s), config2", "unit": "s", "n_gpus": 1,
            "value": res["mixed"]["forward_s"] + res["mixed"]["backward_s"], "higher_is_better": False,
            "config": {"workload": "config2: %s geometry (N=%d), 500 dipoles, sigma sampled x[0.5,2]" % (args.head,
                                                                                                      geo.size),
                       "fd_step": "1e-6 relative (conductivities), 1e-6 absolute (dipoles)",
                       "fd_dipole_coordinates": len(sample)},
            "results": res,
            "fd_rel_err": {"conductivities_max": sig_err, "dipole_coordinates_max": dip_err},
            "mixed_vs_fp64_gradient_rel_err": {"conductivities": mix_sig, "dipoles": mix_dip}}
    print(json.dumps(line))
    return 0


def run_next(args):
    """The rows beside the forward path on the config1 head (ico4, N=17926):
    SurfSourceMat and SurfSource2MEGMat (an ico3 source surface, 642 vertices,
    in the brain), Surf2VolMat and DipSource2InternalPotMat (5000 points over
    the whole head and its surroundings, 2000 dipoles), EITSourceMat (64
    electrodes of radius 0.05).  Per row: CUDA-event time per call over
    --steps calls after --warmup, kernel launches, the analytic-kernel
    evaluations of the call and their rate, and, where the oracle restates
    the row, the oracle's CPU time on a bounded sample scaled to the call."""
    import torch
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    __import__("__graft_entry__").build()
    from openmeeg_gb300 import api, workloads
    from openmeeg_gb300 import synthetic as syn
    w = getattr(workloads, args.head)()
    ctx = api.Context(local)
    ctx.bind_current_stream()
    geo = api.Geometry.from_head(w.head, ctx)
    dev = torch.device("cuda", local)
    rng = np.random.default_rng(17)
    Vs, Ts = syn.icosphere(3, inward=False)
    Vs = Vs * 0.5 + np.array([0.03, -0.02, 0.01])
    u = rng.standard_normal((5000, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    pts = u * (rng.random(5000) ** (1.0 / 3.0) * 1.1)[:, None]
    dip = w.dipoles
    el = np.hstack([w.electrodes[:, :3], np.full((w.electrodes.shape[0], 1), 0.05)])
    pts_d = torch.as_tensor(pts, device=dev)
    dip_d = torch.as_tensor(dip, device=dev)
    el_d = torch.as_tensor(el, device=dev)
    sq_d = torch.as_tensor(w.squids, device=dev)
    T_in = w.head.triangles[0].shape[0]
    Ttot = sum(t.shape[0] for t in w.head.triangles)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn):
        out = None
        for _ in range(args.warmup):
            out = fn()
        torch.cuda.synchronize()
        l0 = ctx.launches()
        e0.record()
        for _ in range(args.steps):
            out = fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / args.steps, (ctx.launches() - l0) / args.steps, out

    rows = {}
    clocks = Clocks(local)
    clocks.start()
    ms, nl, A = timed(lambda: api.SurfSourceMat(geo, Vs, Ts))
    ev = 2 * 16 * T_in * Ts.shape[0]            # S and D pair integrals of the brain's boundary vs the source
    rows["SurfSourceMat"] = {"ms": ms, "launches": nl, "shape": list(A.shape), "evaluations": ev,
                             "evals_per_s": ev / (ms / 1e3), "cpu": None,
                             "note": "16-point S and D pair integrals (brain boundary x source triangles)"}
    ms, nl, A = timed(lambda: api.SurfSource2MEGMat(Vs, Ts, sq_d, ctx))
    rows["SurfSource2MEGMat"] = {"ms": ms, "launches": nl, "shape": list(A.shape),
                                 "evaluations": sq_d.shape[0] * Ts.shape[0],
                                 "evals_per_s": sq_d.shape[0] * Ts.shape[0] / (ms / 1e3), "cpu": None}
    ms, nl, A = timed(lambda: api.Surf2VolMat(geo, pts_d))
    kept = A.shape[0]
    rows["Surf2VolMat"] = {"ms": ms, "launches": nl, "shape": list(A.shape), "points": pts.shape[0],
                           "evaluations": kept * Ttot, "evals_per_s": kept * Ttot / (ms / 1e3),
                           "note": "upper bound: P1 + S per (kept point, triangle of its domain's boundary); "
                                   "one thread per (point, triangle) of the whole head"}
    ms, nl, A = timed(lambda: api.DipSource2InternalPotMat(geo, dip_d, pts_d))
    rows["DipSource2InternalPotMat"] = {"ms": ms, "launches": nl, "shape": list(A.shape),
                                        "evaluations": kept * dip.shape[0],
                                        "evals_per_s": kept * dip.shape[0] / (ms / 1e3)}
    ms, nl, A = timed(lambda: api.EITSourceMat(geo, el_d))
    rows["EITSourceMat"] = {"ms": ms, "launches": nl, "shape": list(A.shape)}
    # CorticalMat / CorticalMat2 on the config0 head (N = 4486, 64 electrodes, cortex = the brain's boundary): one
    # KKT system each (N + rows outside the cortex [+ electrodes] unknowns), FP64 LU with partial pivoting
    w0 = workloads.config0()
    geo0 = api.Geometry.from_head(w0.head, ctx)
    M0 = api.Head2EEGMat(geo0, torch.as_tensor(w0.electrodes[:, :3], device=dev), sparse=True)
    ncx = w0.head.vertices[0].shape[0] + w0.head.triangles[0].shape[0]
    for name, fn, extra in (("CorticalMat", lambda: api.CorticalMat(geo0, M0, "Brain", 1e-4, 1.58e-2), 0),
                            ("CorticalMat2", lambda: api.CorticalMat2(geo0, M0, "Brain", 12.4), M0[1].shape[0])):
        ms, nl, A = timed(fn)
        nk = 2 * geo0.size - ncx + extra
        rows[name] = {"ms": ms, "launches": nl, "shape": list(A.shape), "kkt_unknowns": nk,
                      "lu_gflop": 2.0 * nk ** 3 / 3 / 1e9, "fp64_tflops": 2.0 * nk ** 3 / 3 / (ms / 1e3) / 1e12,
                      "cpu": None, "note": "config0 head; alpha 1e-4 / beta 1.58e-2 and gamma 12.4 as in the "
                                           "reference's tests (TestHead.cmake:94-96)"}
    ck = clocks.stop()
    if not args.no_cpu:
        from oracle import oracle
        g = oracle.digest(w.head)
        nthr = oracle.num_threads()
        for name, fn, n_sample, n_full in (
                ("Surf2VolMat", lambda k: oracle.surf2volmat(g, pts[:k]), 400, pts.shape[0]),
                ("DipSource2InternalPotMat", lambda k: oracle.dipsource2internalpotmat(g, dip[:20], pts[:k]), 200,
                 pts.shape[0] * dip.shape[0] / 20),
                ("EITSourceMat", lambda k: oracle.eitsourcemat(g, el[:k]), 8, el.shape[0])):
            s = time.perf_counter()
            fn(n_sample)
            t = (time.perf_counter() - s) * n_full / n_sample
            rows[name]["cpu"] = {"value_ms": t * 1e3, "cores": nthr, "kind": "port",
                                 "sample": f"{n_sample} of the call's units, scaled linearly"}
            rows[name]["speedup_vs_cpu"] = t * 1e3 / rows[name]["ms"]
        # the reference's CorticalMat (SVD projector, SVD pseudo-inverse) as the oracle restates it, whole call
        g0 = oracle.digest(w0.head)
        Md = oracle.h2em(g0, w0.electrodes)
        s = time.perf_counter()
        oracle.corticalmat(g0, Md, "Brain", 1e-4, 1.58e-2)
        t = time.perf_counter() - s
        rows["CorticalMat"]["cpu"] = {"value_ms": t * 1e3, "cores": os.cpu_count(), "kind": "port",
                                      "sample": "the whole call (LAPACK SVDs through numpy on all host cores)"}
        rows["CorticalMat"]["speedup_vs_cpu"] = t * 1e3 / rows["CorticalMat"]["ms"]
    line = {"metric": "time per call (ms) of the rows beside the forward path, config1 head", "unit": "ms",
            "higher_is_better": False, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": f"{args.head} head (N={geo.size}); ico3 source surface (642 vertices) in the brain; "
                                   f"5000 points (r < 1.1), {dip.shape[0]} dipoles, 64 EIT electrodes (r = 0.05), "
                                   f"{sq_d.shape[0]} magnetometers"},
            "rows": rows, "clocks": ck}
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="config1")
    ap.add_argument("--branches", type=int, default=0, help="config3: graph branches (0 = autotune)")
    ap.add_argument("--large-precisions", default="mixed,fp64", help="config4: precisions to run, in order")
    ap.add_argument("--fd-dipoles", type=int, default=4, help="config2: dipole coordinates checked by differences")
    ap.add_argument("--analytic-dipoles", type=int, default=500, help="config4: dipoles checked analytically")
    ap.add_argument("--head", default="config1", choices=["config0", "config1"],
                    help="config2 / next: the head the rows run on (config0: a small profiling case)")
    ap.add_argument("--fp64-steps", type=int, default=3)
    ap.add_argument("--profile-steps", type=int, default=1)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--only-mixed", action="store_true",
                    help="profiling aid: run the mixed-precision steps only (no FP64 reference, e2e or CPU leg)")
    ap.add_argument("--only-fp64", action="store_true", help="profiling aid: run FP64 drop-in steps only")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.config == "config3":
        return run_batch(args)
    if args.config == "config4":
        return run_large(args)
    if args.config == "config2":
        return run_adjoint(args)
    if args.config == "next":
        return run_next(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
