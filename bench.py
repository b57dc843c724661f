"""Benchmark: seconds per symmetry-adapted GW iteration on one GB300.

Workload: the C2 crystal (Fm-3m, 3x3x3 k mesh = 27 k / 4 irreducible,
nao=26, naux=120, nts=100, beta=100, ns=1, V stored for all 729 k pairs),
synthetic seeded data (see mbsymmetry_gb300/crystal.py).  One step = one GW
iteration P0 -> P~ (W~ solve) -> Sigma -> Dyson with all tau <-> i omega
transforms, replayed as one CUDA graph, with the P0 and Sigma contractions on
the sliced split-precision path (BF16 fixed-point slices on tcgen05, Sigma
within 1e-7 Ha of FP64: the error is measured and reported in the line); the
FP64 drop-in, the FP32-class split paths, mixed-vs-FP64 blocks for C3, C4 and
C2's sizes built from Gaussian orbitals, and the self-consistent loop are
reported beside it.

  value  device time of the iteration (CUDA events recorded on the engine's
         stream), inputs resident in HBM, L2 flushed before every iteration.
  e2e    the same iteration through the public C ABI with host buffers:
         gwgb_set_G (H2D) + gwgb_iteration + gwgb_get_sigma + gwgb_get_G (D2H).

--impl reference times whole iterations of the FP64 CPU oracle (the
restatement of the reference's CPU algorithm) on all host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

CONFIG = "C2"
WORKLOADS = {
    "C2": ("C2: Fm-3m 3x3x3 k mesh (27 k, 4 irreducible), nao=26, naux=120, nts=100, beta=100, "
           "ns=1, V stored for all 729 k pairs, irrep blocks 1-8 (AO) / 2-40 (aux)"),
    "C3": ("C3: Fm-3m 4x4x4 k mesh (64 k, 8 irreducible), nao=52, naux=250, nts=120, beta=100, "
           "ns=1, V stored for all 4096 k pairs (12.2 GB), irrep blocks 2-16 (AO) / 4-64 (aux)"),
    "C3m": ("C3m (profiling case): C3's nao=52, naux=250, nts=120, beta=100 and block sizes 2-16 / 4-64 "
            "on the Fm-3m 3x3x3 mesh (27 k)"),
}
WORKLOAD = WORKLOADS[CONFIG]
METRIC = "s/GW iteration + tensor TFLOP/s: mixed vs FP64 GPU at Sigma err<=1e-7 Ha; CPU ref"
# dram__bytes_read.sum + dram__bytes_write.sum summed over one iteration's launches of
# each sliced-path GEMM kernel on C2, from one ncu capture of `bench.py --profile`.
OZ_TRAFFIC = {"oz_gemm_kernel": 8.629e9, "oz_simt_kernel": 21.484e9}
L2_BYTES = 129 * 1024 * 1024


def _rank_info():
    from mbsymmetry_gb300.replicas import rank_info
    return rank_info()


def _load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except OSError:
        return {}


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"gwgb_clocks_{os.getpid()}_dev{device}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for n, v in zip(names, parts[5:9]):
                    if v.lower() == "active":
                        reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def _setup():
    from mbsymmetry_gb300.crystal import CONFIGS, load_ir, make_crystal
    from mbsymmetry_gb300.transformer import build_transforms
    spec = CONFIGS[CONFIG]
    cr = make_crystal(spec)
    tr = build_transforms(load_ir(spec.nts), spec.beta)
    return cr, tr


def _host_cores():
    """Cores this process may run on (torchrun sets OMP_NUM_THREADS=1 for its
    ranks; the CPU timings use every core they have)."""
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def _cpu_reference(cr, tr, steps, threads=None, with_numpy=False):
    """Time whole GW iterations of the FP64 CPU oracle (the C restatement of the
    reference's CPU path: G rotation, P0 over all nts/2 tau, W~ solve, P~
    rotation, Sigma over all nts tau, Dyson) on all host cores; per step one
    full iteration, nothing sampled or scaled.  with_numpy: also time the
    numpy/BLAS restatement of the two contractions once (second figure)."""
    threads = _host_cores() if threads is None else threads
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from oracle import Oracle  # the CPU baseline (restatement of the reference's CPU path)
    L, nts, ns = cr.layout, tr.nts, cr.ns
    orc = Oracle(L, ns, nts, threads=threads)
    zero = np.zeros(nts * ns * L.flat_ao_size, np.complex128)
    G, _ = orc.dyson(zero, cr.F, cr.S, tr, cr.mu)
    per_step = []
    for _ in range(steps):
        t0 = time.perf_counter()
        Gf = orc.rotate_G(G)
        P0 = orc.p0(Gf, cr.V)
        Pf = orc.rotate_P(orc.p_tilde(P0, tr))
        S = orc.sigma(Gf, Pf, cr.V)
        orc.dyson(S, cr.F, cr.S, tr, cr.mu)
        per_step.append(time.perf_counter() - t0)
    sample = (f"{CONFIG}: whole GW iterations (G rotation, P0 for all {nts // 2} tau, W~ solve, P~ rotation, "
              f"Sigma for all {nts} tau, Dyson), C restatement with OpenMP; per step one iteration")
    out = {"value": float(np.mean(per_step)), "cores": orc.threads(), "sample": sample}
    if with_numpy:
        import np_baseline  # numpy/BLAS restatement of the contractions
        t0 = time.perf_counter()
        np_baseline.p0(L, ns, nts, Gf, cr.V)
        np_baseline.sigma(L, ns, nts, Gf, Pf, cr.V)
        out["numpy_contractions_s"] = time.perf_counter() - t0
        out["numpy_note"] = ("numpy/BLAS restatement of P0 and Sigma (tau batched into matmuls per V block), "
                             "contractions only; the C figure is the whole iteration")
    return out


def run_reference(args):
    rank, world, _ = _rank_info()
    if rank != 0:
        return
    cr, tr = _setup()
    for _ in range(max(0, min(args.warmup, 1))):
        _cpu_reference(cr, tr, 1)
    ref = _cpu_reference(cr, tr, args.steps)
    v, cores, sample = ref["value"], ref["cores"], ref["sample"]
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": v * 1e3, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD}, "precision": "fp64 (CPU restatement)",
        "cpu_baseline": {"value": v, "unit": "s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def _peaks(dev):
    """Roofline denominators measured in this run (peaks/peaks.cu) and the driver's file."""
    import ctypes
    probe = ctypes.CDLL(os.path.join(ROOT, "peaks", "libgwgb_peaks.so"))
    for fn in ("gwgb_probe_fp64_tflops", "gwgb_probe_dmma_tflops"):
        getattr(probe, fn).restype = ctypes.c_double
        getattr(probe, fn).argtypes = [ctypes.c_int]
    probe.gwgb_probe_tc_tflops.restype = ctypes.c_double
    probe.gwgb_probe_tc_tflops.argtypes = [ctypes.c_int, ctypes.c_int]
    probe.gwgb_probe_fp32_tflops.restype = ctypes.c_double
    probe.gwgb_probe_fp32_tflops.argtypes = [ctypes.c_int]
    pk = _load_peaks()
    return {"hbm_gbs": pk.get("hbm_gbs"), "bf16_tflops_cublas": pk.get("bf16_tflops"),
            "fp64_fma_tflops": probe.gwgb_probe_fp64_tflops(dev), "fp64_dmma_tflops": probe.gwgb_probe_dmma_tflops(dev),
            "fp32_fma_tflops": probe.gwgb_probe_fp32_tflops(dev),
            "tcgen05_tf32_tflops": probe.gwgb_probe_tc_tflops(dev, 0),
            "tcgen05_bf16_tflops": probe.gwgb_probe_tc_tflops(dev, 1)}


STAGE_KEYS = ("rotate_G_ms", "p0_ms", "pq_ms", "sigma_ms", "dyson_ms", "transform_ms", "solve_ms")
PREC_LABEL = {
    "ozaki": ("bf16 x4 fixed-point slices per operand row (Ozaki scheme) on tcgen05 kind::f16, 10 products, "
              "exact FP32 partial sums, float-float accumulation and intermediates; FP64 W~ solve, Dyson, "
              "transforms, mu search, energies"),
    "fp64": "complex128 contractions on CUDA cores (the drop-in)",
    "tf32x3": ("tf32x3 (tcgen05 kind::tf32, 2 planes, 3 products, FP32 accumulate within an aux block or "
               "aux-row chunk, FP64 across): FP32-class error, no 1e-7 claim"),
    "bf16x3": ("bf16x3 (tcgen05 kind::f16, 3 BF16 planes, 6 products, FP32 accumulate within an aux block or "
               "aux-row chunk, FP64 across): FP32-class error, no 1e-7 claim"),
}


def _timed(s, G0, mu, prec, steps, warmup, flush, sync):
    """Device time of `steps` graph-launched iterations from G0 (L2 flushed before each)."""
    s.single_prec_run(prec != "fp64", prec)
    for _ in range(warmup):
        s.set_G(G0)
        s.iteration(mu)
    times, stg = [], {}
    for _ in range(steps):
        s.set_G(G0)
        flush.zero_()
        sync()
        s.iteration(mu)
        st = s.stats()
        times.append(st["total_ms"])
        for k in STAGE_KEYS:
            stg[k] = stg.get(k, 0.0) + st[k] / steps
    return float(np.mean(times)), stg, st


def _launch_profile(s, G0, mu, steps):
    """Per-launch CUDA-event times of the sliced path (gwgb_set_launch_timing)
    over `steps` iterations from G0, summed per kernel and per stage (per
    iteration).  A separate pass after the headline timing: the events add a
    few microseconds per launch."""
    s.launch_timing(True)
    s.set_G(G0)
    s.iteration(mu)  # captures the graph with the event records
    kern, stage = {}, {}
    for _ in range(steps):
        s.set_G(G0)
        s.iteration(mu)
        for x in s.launch_stats():
            if not x["ran"]:
                continue
            k = kern.setdefault(x["kernel"], {"ms": 0.0, "flops": 0.0, "mma_flops": 0.0, "bytes": 0.0, "launches": 0})
            g = stage.setdefault(x["stage"], {"ms": 0.0, "flops": 0.0})
            for d in (k, g):
                d["ms"] += x["ms"] / steps
                d["flops"] += x["flops"] / steps
            k["mma_flops"] += x["mma_flops"] / steps
            k["bytes"] += x["bytes"] / steps
            k["launches"] += 1
    s.launch_timing(False)
    for k in kern.values():
        k["launches"] //= steps
    return kern, stage


def _kernel_roofline(kern, peaks, traffic):
    """Roofline of the sliced path's dominant kernel (largest summed launch time)."""
    name = max(kern, key=lambda n: kern[n]["ms"])
    k = kern[name]
    t = k["ms"] * 1e-3
    if name == "oz_gemm_kernel":
        peak = peaks["tcgen05_bf16_tflops"]
        alg = k["flops"] / t / 1e12
        exe = k["mma_flops"] / t / 1e12
        return {"bound": "tensor", "kernel": name, "achieved": alg, "peak": peak, "unit": "TFLOP/s",
                "frac": alg / peak, "executed_tflops": exe, "frac_executed": exe / peak,
                "peak_source": "tcgen05 kind::f16 (BF16) rate measured in this run (peaks/peaks.cu), of measured",
                "achieved_note": "algorithmic complex FLOPs (8 M N K per block GEMM) of its launches / their summed "
                                 "CUDA-event time; executed = BF16 MMA FLOPs issued (10 slice products, real "
                                 "embedding, 128-row tiles, N and K padded to the MMA shape)",
                "launches_per_step": k["launches"], "ms_per_step": k["ms"], "traffic": traffic.get(name),
                "traffic_unit": "bytes per step, all launches of the kernel (ncu)"}
    if name == "oz_simt_kernel":
        peak = peaks["fp32_fma_tflops"]
        alg = k["flops"] / t / 1e12
        ins = k["mma_flops"] / t / 1e12  # FP32 instructions (48 per complex MAC) per second, in T/s
        return {"bound": "fp32 (CUDA-core float-float)", "kernel": name, "achieved": alg, "peak": peak,
                "unit": "TFLOP/s", "frac": alg / peak, "fp32_instr_per_s_T": ins,
                "frac_fp32_issue": 2.0 * ins / peak,
                "peak_source": "FP32 FMA rate measured in this run (peaks/peaks.cu, 2 flops per FMA), of measured",
                "achieved_note": "algorithmic complex FLOPs / summed launch time; each complex MAC costs 48 FP32 "
                                 "instructions in float-float, so frac_fp32_issue = instructions / FMA issue rate",
                "launches_per_step": k["launches"], "ms_per_step": k["ms"], "traffic": traffic.get(name),
                "traffic_unit": "bytes per step, all launches of the kernel (ncu)"}
    gbs = k["bytes"] / t / 1e9
    return {"bound": "hbm", "kernel": name, "achieved": gbs, "peak": peaks["hbm_gbs"], "unit": "GB/s",
            "frac": gbs / peaks["hbm_gbs"] if peaks.get("hbm_gbs") else None, "traffic": traffic.get(name)}


CONFIG_BLOCKS = {
    "C3": "C3 (the mixed-precision config): Fm-3m 4x4x4 k mesh (64 k, 8 irreducible), nao=52, naux=250, nts=120, "
          "beta=100, irrep blocks 2-16 (AO) / 4-64 (aux), V for all k pairs (12.2 GB)",
    "C4": "C4: hexagonal 4x4x3 k mesh (48 k, 8 irreducible), nao=72, naux=350, nts=120, beta=200, irrep blocks "
          "2-30, V for all k pairs",
    "C2-orbital": "C2's sizes (Fm-3m 3x3x3 k mesh, 4 irreducible, nao=26, naux=120, nts=100, beta=100) as a "
                  "tight-binding crystal from Gaussian orbitals: Slater-Koster F, V from three-centre overlaps of "
                  "Gaussian auxiliary functions (exponents 0.3-3.0), irrep blocks (AO 2-12, aux 12-56), rotations "
                  "and V selection rule from O_h",
}


def _config_block(name, dev, warmup):
    """Mixed vs FP64 on another crystal (C3, C4, or C2's sizes built from
    Gaussian orbitals): one timed iteration each after warm-up, Sigma and G
    error of the sliced path against FP64."""
    from mbsymmetry_gb300.crystal import CONFIGS, load_ir, make_crystal
    from mbsymmetry_gb300.solver import GWSolver
    from mbsymmetry_gb300.transformer import build_transforms
    if name == "C2-orbital":
        from mbsymmetry_gb300.orbitals import make_orbital_crystal
        spec = CONFIGS["C2"]
        cr = make_orbital_crystal(spec)
    else:
        spec = CONFIGS[name]
        cr = make_crystal(spec)
    tr = build_transforms(load_ir(spec.nts), spec.beta)
    s = GWSolver(cr.layout, cr.ns, tr, device=dev)
    s.set_shared_Coulomb(cr.V)
    s.set_fock(cr.F, cr.S)
    s.set_Selfenergy(np.zeros(s.g_size, np.complex128))
    s.dyson(cr.mu)
    G0 = s.G_tau()
    out, res = {"workload": CONFIG_BLOCKS[name]}, {}
    for prec in ("fp64", "ozaki"):
        s.single_prec_run(prec != "fp64", prec)
        for _ in range(1 + (prec != "fp64") * max(0, min(warmup, 1))):
            s.set_G(G0)
            s.iteration(cr.mu)
        st = s.stats()
        res[prec] = (s.Selfenergy(), s.G_tau())
        out[prec] = {"s_per_iteration": st["total_ms"] / 1e3, "p0_s": st["p0_ms"] / 1e3,
                     "sigma_s": st["sigma_ms"] / 1e3,
                     "contraction_tflops_alg": {k: st[f"{k}_flops"] / (st[f"{k}_ms"] * 1e-3) / 1e12
                                                for k in ("p0", "sigma")}}
    kern, stage = _launch_profile(s, G0, cr.mu, 1)
    out["ozaki"]["kernels"] = kern
    out["ozaki"]["stages_ms"] = {k: v["ms"] for k, v in stage.items()}
    s.close()
    out["speedup"] = out["fp64"]["s_per_iteration"] / out["ozaki"]["s_per_iteration"]
    out["sigma_max_abs_err"] = float(np.abs(res["ozaki"][0] - res["fp64"][0]).max())
    out["G_max_abs_err"] = float(np.abs(res["ozaki"][1] - res["fp64"][1]).max())
    out["sigma_max_abs"] = float(np.abs(res["fp64"][0]).max())
    return out


def run_gpu(args):
    rank, world, local = _rank_info()
    import torch
    from mbsymmetry_gb300.replicas import Replicas
    dev = local
    torch.cuda.set_device(dev)
    reps = Replicas(device=f"cuda:{dev}")  # independent replicas: max-over-ranks timing, rank 0 reports
    from mbsymmetry_gb300.solver import GWSolver
    from mbsymmetry_gb300 import _abi
    import ctypes

    cr, tr = _setup()
    L = cr.layout
    s = GWSolver(L, cr.ns, tr, device=dev)
    s.set_shared_Coulomb(cr.V)
    s.set_fock(cr.F, cr.S)
    s.set_Selfenergy(np.zeros(s.g_size, np.complex128))
    s.dyson(cr.mu)                          # G0: the input of every timed iteration
    G0 = s.G_tau()
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=f"cuda:{dev}")
    sync = torch.cuda.synchronize

    clocks = ClockSampler(dev)
    with clocks:  # clocks sampled over both timed regions (FP64, then the headline)
        # ---- FP64 drop-in (the accuracy reference of the split paths) -------
        ms64, st64, s64 = _timed(s, G0, cr.mu, "fp64", args.steps, args.warmup, flush, sync)
        sig64, g64 = s.Selfenergy(), s.G_tau()

        # ---- headline: the sliced split-precision path -----------------------
        s.single_prec_run(True, "ozaki")
        for _ in range(args.warmup):
            s.set_G(G0)
            s.iteration(cr.mu)
        reps.barrier()
        ms, stages, st = _timed(s, G0, cr.mu, "ozaki", args.steps, 0, flush, sync)
        reps.barrier()
    launches = int(st["kernel_launches"]) * args.steps
    ms = reps.max_over_ranks(ms)
    sig_oz, g_oz = s.Selfenergy(), s.G_tau()

    # ---- e2e through the C ABI with pinned host buffers (sliced path) -------
    g_host = torch.from_numpy(G0.view(np.float64)).pin_memory()
    sig_host = torch.empty(2 * s.g_size, dtype=torch.float64).pin_memory()
    g_out = torch.empty(2 * s.g_size, dtype=torch.float64).pin_memory()
    lib = _abi.load()
    h = s.h
    vp = ctypes.c_void_p
    for _ in range(2):
        _abi.check(lib.gwgb_set_G(h, vp(g_host.data_ptr())))
        _abi.check(lib.gwgb_iteration(h, cr.mu))
    e2e = []
    reps.barrier()
    for _ in range(args.steps):
        flush.zero_()
        sync()
        t0 = time.perf_counter()
        _abi.check(lib.gwgb_set_G(h, vp(g_host.data_ptr())))
        _abi.check(lib.gwgb_iteration(h, cr.mu))
        _abi.check(lib.gwgb_get_sigma(h, vp(sig_host.data_ptr())))
        _abi.check(lib.gwgb_get_G(h, vp(g_out.data_ptr())))
        e2e.append(time.perf_counter() - t0)
    reps.barrier()
    e2e_s = reps.max_over_ranks(float(np.mean(e2e)))
    gbytes = s.g_size * 16

    # ---- rooflines ------------------------------------------------------------
    peaks = _peaks(dev)
    fp64_peak = peaks["fp64_fma_tflops"]
    kern, lstages = _launch_profile(s, G0, cr.mu, args.steps)
    roofline = _kernel_roofline(kern, peaks, OZ_TRAFFIC)
    roofline["kernels"] = kern
    roofline["stages_ms"] = {k: v["ms"] for k, v in lstages.items()}
    # the same figures for every sliced-path kernel (the tcgen05 one beside the dominant one)
    roofline["per_kernel"] = {n: {k: v for k, v in _kernel_roofline({n: kern[n]}, peaks, OZ_TRAFFIC).items()
                                  if k not in ("achieved_note", "peak_source")} for n in kern}
    dom64 = "sigma" if st64["sigma_ms"] >= st64["p0_ms"] else "p0"
    a64 = s64[f"{dom64}_flops"] / (st64[f"{dom64}_ms"] * 1e-3) / 1e12
    fp64 = {"precision": PREC_LABEL["fp64"], "s_per_iteration": ms64 / 1e3, "stages_ms": st64,
            "contraction_tflops": {k: s64[f"{k}_flops"] / (st64[f"{k}_ms"] * 1e-3) / 1e12 for k in ("p0", "sigma")},
            "roofline": {"bound": "fp64 (CUDA-core FMA)", "kernel": f"{dom64}_fp64_kernel", "achieved": a64,
                         "peak": fp64_peak, "unit": "TFLOP/s", "frac": a64 / fp64_peak if fp64_peak > 0 else None,
                         "traffic": {"sigma": 0.0703e9, "p0": 0.0563e9}[dom64],
                         "traffic_unit": "bytes per launch (ncu)",
                         "note": "FP64 FMA on CUDA cores: the FP64 tensor path (DMMA) measures slower on this "
                                 "GPU (peaks.fp64_dmma_tflops)"},
            "transforms": {"ms": st64["transform_ms"], "bytes_alg": s64["transform_bytes"],
                           "achieved_gbs": s64["transform_bytes"] / (st64["transform_ms"] * 1e-3) / 1e9,
                           "flops_alg": s64["transform_flops"],
                           "frac_fp64": s64["transform_flops"] / (st64["transform_ms"] * 1e-3) / 1e12 / fp64_peak
                                        if fp64_peak > 0 else None},
            "solves": {"ms": st64["solve_ms"], "gflops": s64["solve_flops"] / (st64["solve_ms"] * 1e-3) / 1e9}}

    # ---- FP32-class split precisions on the same input ----------------------
    def run_split(kind):
        m, stg, stk = _timed(s, G0, cr.mu, kind, args.steps, args.warmup, flush, sync)
        return {"precision": PREC_LABEL[kind], "s_per_iteration": m / 1e3, "speedup_vs_fp64": ms64 / m,
                "sigma_max_abs_err_vs_fp64": float(np.abs(s.Selfenergy() - sig64).max()),
                "G_max_abs_err_vs_fp64": float(np.abs(s.G_tau() - g64).max()), "stages_ms": stg}

    split_tf32 = run_split("tf32x3")
    split_bf16 = run_split("bf16x3")
    s.single_prec_run(False)

    # ---- autotuner (mbsymmetry_gb300/autotune.py): the sliced path's width-class
    # boundary between tcgen05 and the CUDA-core kernel, on this workload
    from mbsymmetry_gb300 import autotune as _autotune
    tune = _autotune.autotune(L, cr.ns, tr, cr.V, cr.F, cr.S, cr.mu, G=G0, precision="ozaki", reps=2)

    # ---- the reference's cuBLAS call sequence on this GPU (measurement only) --
    s.set_G(G0)
    s.solve()
    s.refproxy(nt_batch=4, nstreams=16)  # warm-up: cuBLAS handle and kernel loading
    px = s.refproxy(nt_batch=4, nstreams=16)
    _, sig_px = s.refproxy_results()
    px_s = (px["p0_ms"] + px["sigma_ms"]) / 1e3
    proxy = {"what": "SymmetryMBPT's cuBLAS call sequence (cugw_routines_block.cu, cugw_qkpt_block.cu) replayed "
                     "on this GPU: G rotation, per-pair V transposes and ZGEMM_SB chains of P0 and Sigma; "
                     "V resident in HBM, per-stream accumulators instead of locks",
             "nt_batch": 4, "streams": 16, "p0_s": px["p0_ms"] / 1e3, "sigma_s": px["sigma_ms"] / 1e3,
             "contractions_s": px_s, "gemm_calls": int(px["gemm_calls"]), "other_calls": int(px["other_calls"]),
             "sigma_max_abs_diff_vs_fp64_kernels": float(np.abs(sig_px - sig64).max()),
             "speedup_fp64_kernels": px_s / ((st64["p0_ms"] + st64["sigma_ms"]) / 1e3),
             "speedup_sliced_kernels": px_s / ((stages["p0_ms"] + stages["sigma_ms"]) / 1e3)}

    # ---- self-consistent loop: 10 graph-launched iterations, alpha = 0.5 ----
    # Each iteration: GW Sigma, linear mixing, device-side mu search (half
    # filling, N = nao), Dyson, energies.  FP64 and the sliced path; per
    # iteration mu and E_corr and the final Sigma are compared.
    zeros = np.zeros(s.g_size, np.complex128)
    sc = {"iterations": 10, "alpha": 0.5, "n_electrons": float(L.nao),
          "note": "graph launches back to back (no L2 flush between iterations)"}
    finals = {}
    for prec in ("fp64", "ozaki"):
        s.single_prec_run(prec != "fp64", prec)
        s.set_G(G0)
        s.set_Selfenergy(zeros)
        recs = s.sc_loop(10, 0.5, float(L.nao), cr.mu, step=0.05, tol=1e-10, max_evals=24)
        stl = s.stats()
        finals[prec] = (s.Selfenergy(), recs)
        sc[prec] = {"s_per_iteration": stl["total_ms"] / 1e3, "mu": [r["mu"] for r in recs],
                    "e_corr": [r["e_corr"] for r in recs], "mu_evals": [r["mu_evals"] for r in recs],
                    "n_final": recs[-1]["n_electrons"], "leakage_final": recs[-1]["leakage"]}
    s.single_prec_run(False)
    sc["per_iteration_e_corr_abs_diff"] = [abs(a["e_corr"] - b["e_corr"])
                                           for a, b in zip(finals["fp64"][1], finals["ozaki"][1])]
    sc["per_iteration_mu_abs_diff"] = [abs(a["mu"] - b["mu"]) for a, b in zip(finals["fp64"][1], finals["ozaki"][1])]
    sc["final_sigma_max_abs_diff"] = float(np.abs(finals["fp64"][0] - finals["ozaki"][0]).max())
    sc["speedup"] = sc["fp64"]["s_per_iteration"] / sc["ozaki"]["s_per_iteration"]
    s.close()
    def guarded(name):  # a failing block is reported in its own key, the line still prints
        try:
            return _config_block(name, dev, args.warmup)
        except Exception as e:  # noqa: BLE001
            return {"workload": CONFIG_BLOCKS[name], "error": f"{type(e).__name__}: {e}"}
    big = {} if args.no_c4 or world > 1 else {n: guarded(n) for n in ("C2-orbital", "C3", "C4")}

    line = {
        "metric": METRIC, "value": reps.seconds_per_iteration(ms), "unit": "s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "bf16x4 slices (c128 in/out, fp64 solves)",
        "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD},
        "precision": "ozaki: " + PREC_LABEL["ozaki"], "l2": "flushed (256 MiB write) before each step",
        "parallelism": "replicas" if world > 1 else "1 GPU",
        "replica_iterations_per_s": reps.replica_throughput(ms) if world > 1 else None,
        "sigma_max_abs_err_vs_fp64": float(np.abs(sig_oz - sig64).max()),
        "G_max_abs_err_vs_fp64": float(np.abs(g_oz - g64).max()),
        "sigma_max_abs": float(np.abs(sig64).max()),
        "speedup_vs_fp64": ms64 / ms,
        "e2e": {"value": e2e_s, "unit": "s", "h2d_bytes_per_step": gbytes, "d2h_bytes_per_step": 2 * gbytes},
        "gpu_launches": launches,
        "stages_ms": stages,
        "contraction_tflops_alg": {k: st[f"{k}_flops"] / (stages[f"{k}_ms"] * 1e-3) / 1e12 for k in ("p0", "sigma")},
        "roofline": roofline,
        "clocks": clocks.summary(),
        "fp64": fp64,
        "split_tf32x3": split_tf32,
        "split_bf16x3": split_bf16,
        "c3_mixed_vs_fp64": big.get("C3"),
        "c4_mixed_vs_fp64": big.get("C4"),
        "c2_orbital_mixed_vs_fp64": big.get("C2-orbital"),
        "reference_gpu_proxy": proxy,
        "autotune": {"precision": "ozaki", "metric": tune["metric"], "best": tune["best"],
                     "default": _autotune.OZAKI_CANDIDATES[0], "trials": tune["trials"]},
        "sc_loop": sc,
        "peaks": peaks,
    }
    if reps.reports and world == 1 and not args.no_cpu_baseline:  # rank 0 at N = 1 only
        ref = _cpu_reference(cr, tr, 1, with_numpy=True)
        line["cpu_baseline"] = {"value": ref["value"], "unit": "s", "cores": ref["cores"], "kind": "port",
                                "sample": ref["sample"], "numpy_contractions_s": ref["numpy_contractions_s"],
                                "numpy_note": ref["numpy_note"]}
    if reps.reports:
        print(json.dumps(line))
    reps.close()


def run_profile(args):
    """One FP64 and one sliced-path iteration of the workload (each after one
    warm-up iteration): the command that ncu captures (a plain run of it must
    exit 0 first).  The sliced path's six oz_gemm_kernel launches of the second
    iteration are the stages Z1, Z, P0, W, U, Sigma in that order."""
    import torch
    from mbsymmetry_gb300.solver import GWSolver
    torch.cuda.set_device(0)
    cr, tr = _setup()
    s = GWSolver(cr.layout, cr.ns, tr, device=0)
    s.set_shared_Coulomb(cr.V)
    s.set_fock(cr.F, cr.S)
    s.set_Selfenergy(np.zeros(s.g_size, np.complex128))
    s.dyson(cr.mu)
    G0 = s.G_tau()
    s.set_G(G0)
    s.iteration(cr.mu)
    s.single_prec_run(True, "ozaki")
    for _ in range(2):
        s.set_G(G0)
        s.iteration(cr.mu)
    st = s.stats()
    s.close()
    print(f"profile run: {CONFIG}, one FP64 and two sliced-path iterations (last {st['total_ms']:.2f} ms)")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-c4", action="store_true", help="skip the mixed-vs-FP64 blocks (orbital C2, C3, C4)")
    ap.add_argument("--config", default="C2", choices=sorted(WORKLOADS),
                    help="workload (C2 is the benchmark; C3 is for profiling and manual runs)")
    ap.add_argument("--profile", action="store_true",
                    help="one FP64 and two sliced-path iterations only (the command for ncu captures)")
    args = ap.parse_args()
    global CONFIG, WORKLOAD
    CONFIG, WORKLOAD = args.config, WORKLOADS[args.config]
    if args.profile:
        run_profile(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
