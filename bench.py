"""Benchmark: seconds per symmetry-adapted GW iteration on one GB300.

Workload: the C2 crystal (Fm-3m, 3x3x3 k mesh = 27 k / 4 irreducible,
nao=26, naux=120, nts=100, beta=100, ns=1, V stored for all 729 k pairs),
synthetic seeded data (see mbsymmetry_gb300/crystal.py).  One step = one GW
iteration P0 -> P~ (W~ solve) -> Sigma -> Dyson with all tau <-> i omega
transforms, FP64 (the drop-in path), replayed as one CUDA graph.

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
METRIC = "s/GW iteration (FP64 drop-in, P0 -> W~ -> Sigma -> Dyson)"
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
                                          "--format=csv,noheader,nounits", "-lms", "200"],
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
        "config": {"workload": WORKLOAD, "precision": "fp64"},
        "cpu_baseline": {"value": v, "unit": "s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


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

    barrier = reps.barrier

    for _ in range(args.warmup):
        s.set_G(G0)
        s.iteration(cr.mu)
    stage_tot = {}
    times = []
    with ClockSampler(dev) as clocks:
        barrier()
        for _ in range(args.steps):
            s.set_G(G0)                     # same input each step (not timed)
            flush.zero_()                   # L2 flush between timed iterations
            torch.cuda.synchronize()
            s.iteration(cr.mu)              # events inside the engine's graph
            st = s.stats()
            times.append(st["total_ms"])
            for k in ("rotate_G_ms", "p0_ms", "pq_ms", "rotate_P_ms", "sigma_ms", "dyson_ms", "transform_ms",
                      "solve_ms"):
                stage_tot[k] = stage_tot.get(k, 0.0) + st[k]
        barrier()
    launches = int(st["kernel_launches"]) * args.steps
    ms = reps.max_over_ranks(float(np.mean(times)))
    stages = {k: v / args.steps for k, v in stage_tot.items()}

    # ---- e2e through the C ABI with pinned host buffers ------------------
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
    barrier()
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        _abi.check(lib.gwgb_set_G(h, vp(g_host.data_ptr())))
        _abi.check(lib.gwgb_iteration(h, cr.mu))
        _abi.check(lib.gwgb_get_sigma(h, vp(sig_host.data_ptr())))
        _abi.check(lib.gwgb_get_G(h, vp(g_out.data_ptr())))
        e2e.append(time.perf_counter() - t0)
    barrier()
    e2e_s = reps.max_over_ranks(float(np.mean(e2e)))
    gbytes = s.g_size * 16

    # ---- roofline of the dominant kernel ---------------------------------
    peaks = _load_peaks()
    probe = ctypes.CDLL(os.path.join(ROOT, "peaks", "libgwgb_peaks.so"))
    for fn in ("gwgb_probe_fp64_tflops", "gwgb_probe_dmma_tflops"):
        getattr(probe, fn).restype = ctypes.c_double
        getattr(probe, fn).argtypes = [ctypes.c_int]
    probe.gwgb_probe_tc_tflops.restype = ctypes.c_double
    probe.gwgb_probe_tc_tflops.argtypes = [ctypes.c_int, ctypes.c_int]
    fp64_peak = probe.gwgb_probe_fp64_tflops(dev)
    dmma_peak = probe.gwgb_probe_dmma_tflops(dev)
    tf32_peak = probe.gwgb_probe_tc_tflops(dev, 0)
    bf16_tc_peak = probe.gwgb_probe_tc_tflops(dev, 1)
    dom = "sigma" if stages["sigma_ms"] >= stages["p0_ms"] else "p0"
    flops = st[f"{dom}_flops"]
    dom_ms = stages[f"{dom}_ms"]
    achieved = flops / (dom_ms * 1e-3) / 1e12
    # DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) of the same
    # kernel on this workload from one ncu capture; the kernels are FP64-pipe bound.
    traffic = {"sigma": 0.0703e9, "p0": 0.0563e9}[dom]
    roofline = {"bound": "tensor", "kernel": f"{dom}_fp64_kernel", "achieved": achieved, "peak": fp64_peak,
                "unit": "TFLOP/s", "frac": achieved / fp64_peak if fp64_peak > 0 else None, "traffic": traffic,
                "traffic_unit": "bytes per launch (ncu)",
                "peak_source": "FP64 FMA microbenchmark measured in this run (MEASURED_PEAKS.json has no FP64 "
                               "figure); contraction FLOPs = 8MNK per complex GEMM of the block layout",
                "flop_alg_per_launch": flops, "kernel_ms": dom_ms}

    # ---- split tensor-core precisions on the same input ---------------------
    sig64 = s.Selfenergy()
    g64 = s.G_tau()

    def run_mixed(kind, label):
        s.single_prec_run(True, kind)
        for _ in range(args.warmup):
            s.set_G(G0)
            s.iteration(cr.mu)
        mtimes, mstage = [], {}
        for _ in range(args.steps):
            s.set_G(G0)
            flush.zero_()
            torch.cuda.synchronize()
            s.iteration(cr.mu)
            stm = s.stats()
            mtimes.append(stm["total_ms"])
            for k in ("p0_ms", "sigma_ms", "pq_ms", "rotate_P_ms", "dyson_ms"):
                mstage[k] = mstage.get(k, 0.0) + stm[k] / args.steps
        sig32 = s.Selfenergy()
        g32 = s.G_tau()
        s.single_prec_run(False)
        return {"precision": label,
                "s_per_iteration": float(np.mean(mtimes)) / 1e3,
                "speedup_vs_fp64": ms / float(np.mean(mtimes)),
                "sigma_max_abs_err_vs_fp64": float(np.abs(sig32 - sig64).max()),
                "sigma_max_abs": float(np.abs(sig64).max()),
                "G_max_abs_err_vs_fp64": float(np.abs(g32 - g64).max()),
                "stages_ms": mstage,
                "contraction_tflops_alg": {"p0": stm["p0_flops"] / (mstage["p0_ms"] * 1e-3) / 1e12,
                                           "sigma": stm["sigma_flops"] / (mstage["sigma_ms"] * 1e-3) / 1e12}}

    mixed = run_mixed("tf32x3", "tf32x3 (tcgen05 kind::tf32, 2 planes, 3 products, FP32 accumulate within an aux "
                                "block or aux-row chunk, FP64 across)")
    mixed_bf16 = run_mixed("bf16x3", "bf16x3 (tcgen05 kind::f16, 3 BF16 planes, 6 products, FP32 accumulate within "
                                     "an aux block or aux-row chunk, FP64 across)")

    # ---- tile-shape autotuner (mbsymmetry_gb300/autotune.py) on this workload ---
    from mbsymmetry_gb300 import autotune as _autotune
    tune = _autotune.autotune(L, cr.ns, tr, cr.V, cr.F, cr.S, cr.mu, G=G0, precision="tf32x3", reps=2)

    # ---- the reference's cuBLAS call sequence on this GPU (measurement only) --
    # G rotation + per-pair strided-batched ZGEMM chains of P0 and Sigma, 16
    # streams, 4 tau per batch (the reference's nqkpt streams and test nt_batch);
    # P0 from G0, Sigma from G0 and the FP64 P~ of the same solve.
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
             "speedup_fp64_kernels": px_s / ((stages["p0_ms"] + stages["sigma_ms"]) / 1e3),
             "speedup_tf32x3_kernels": px_s / ((mixed["stages_ms"]["p0_ms"] + mixed["stages_ms"]["sigma_ms"]) / 1e3)}

    # ---- self-consistent loop: 10 graph-launched iterations, alpha = 0.5 ----
    # Each iteration: GW Sigma, linear mixing, device-side mu search (half
    # filling, N = nao), Dyson, energies.  FP64 throughout, and TF32x3 with the
    # last iteration in FP64; the final Sigma / energy of the two are compared.
    zeros = np.zeros(s.g_size, np.complex128)
    sc = {"iterations": 10, "alpha": 0.5, "n_electrons": float(L.nao),
          "note": "graph launches back to back (no L2 flush between iterations)"}
    finals = {}
    for label, prec, final in (("fp64", "fp64", False), ("tf32x3_final_fp64", "tf32x3", True)):
        s.single_prec_run(prec != "fp64", "tf32x3")
        s.set_G(G0)
        s.set_Selfenergy(zeros)
        recs = s.sc_loop(10, 0.5, float(L.nao), cr.mu, step=0.05, tol=1e-10, max_evals=24, final_fp64=final)
        stl = s.stats()
        finals[label] = (s.Selfenergy(), recs[-1])
        sc[label] = {"s_per_iteration": stl["total_ms"] / 1e3, "mu": [r["mu"] for r in recs],
                     "e_corr": [r["e_corr"] for r in recs], "mu_evals": [r["mu_evals"] for r in recs],
                     "n_final": recs[-1]["n_electrons"], "leakage_final": recs[-1]["leakage"]}
    s.single_prec_run(False)
    sc["final_sigma_max_abs_diff"] = float(np.abs(finals["fp64"][0] - finals["tf32x3_final_fp64"][0]).max())
    sc["final_e_corr_diff"] = abs(finals["fp64"][1]["e_corr"] - finals["tf32x3_final_fp64"][1]["e_corr"])
    sc["speedup"] = sc["fp64"]["s_per_iteration"] / sc["tf32x3_final_fp64"]["s_per_iteration"]

    line = {
        "metric": METRIC, "value": reps.seconds_per_iteration(ms), "unit": "s", "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "c128", "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "precision": "fp64", "l2": "flushed (256 MiB write) before each step",
                   "parallelism": "replicas" if world > 1 else "1 GPU"},
        "e2e": {"value": e2e_s, "unit": "s", "h2d_bytes_per_step": gbytes, "d2h_bytes_per_step": 2 * gbytes},
        "gpu_launches": launches,
        "stages_ms": stages,
        "contraction_tflops": {"p0": st["p0_flops"] / (stages["p0_ms"] * 1e-3) / 1e12,
                               "sigma": st["sigma_flops"] / (stages["sigma_ms"] * 1e-3) / 1e12},
        "roofline": roofline,
        # the four tau <-> omega transforms of an iteration (HBM-bound) and the block solves
        # (FP64 latency-bound, no roofline claim), from events inside the iteration's graph
        # (bound: FP64 FMA, about 25 flop per byte at n ~ 100; the HBM figure is given too)
        "transforms": {"ms": stages["transform_ms"], "bytes_alg": st["transform_bytes"],
                       "achieved_gbs": st["transform_bytes"] / (stages["transform_ms"] * 1e-3) / 1e9,
                       "peak_gbs": peaks.get("hbm_gbs"),
                       "frac_hbm": (st["transform_bytes"] / (stages["transform_ms"] * 1e-3) / 1e9 / peaks["hbm_gbs"])
                                   if peaks.get("hbm_gbs") else None,
                       "flops_alg": st["transform_flops"], "bound": "fp64",
                       "achieved_tflops": st["transform_flops"] / (stages["transform_ms"] * 1e-3) / 1e12,
                       "frac_fp64": st["transform_flops"] / (stages["transform_ms"] * 1e-3) / 1e12 / fp64_peak
                                    if fp64_peak > 0 else None},
        "solves": {"ms": stages["solve_ms"], "flops": st["solve_flops"],
                   "gflops": st["solve_flops"] / (stages["solve_ms"] * 1e-3) / 1e9},
        "clocks": clocks.summary(),
        "mixed": mixed,
        "mixed_bf16x3": mixed_bf16,
        "reference_gpu_proxy": proxy,
        "autotune": {"best": tune["best"], "default": _autotune.DEFAULT_CANDIDATES[0],
                     "trials": tune["trials"]},
        "sc_loop": sc,
        "peaks": {"hbm_gbs": peaks.get("hbm_gbs"), "bf16_tflops": peaks.get("bf16_tflops"),
                  "fp64_tflops_measured": fp64_peak},
    }
    s.close()
    if reps.reports and world == 1 and not args.no_cpu_baseline:  # rank 0 at N = 1 only
        ref = _cpu_reference(cr, tr, 1, with_numpy=True)
        line["cpu_baseline"] = {"value": ref["value"], "unit": "s", "cores": ref["cores"], "kind": "port",
                                "sample": ref["sample"], "numpy_contractions_s": ref["numpy_contractions_s"],
                                "numpy_note": ref["numpy_note"]}
    if reps.reports:
        print(json.dumps(line))
    reps.close()


def run_profile(args):
    """One FP64 and one TF32x3 iteration of the workload, then (C2) two FP64
    self-consistent iterations: the command that ncu captures (a plain run of
    it must exit 0 first)."""
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
    s.iteration(cr.mu)
    s.single_prec_run(True, "tf32x3")
    s.set_G(G0)
    s.iteration(cr.mu)
    st = s.stats()
    if CONFIG == "C2":  # the SC loop only on the benchmark workload
        s.single_prec_run(False)
        s.set_G(G0)
        s.set_Selfenergy(np.zeros(s.g_size, np.complex128))
        s.sc_loop(2, 0.5, float(cr.layout.nao), cr.mu, step=0.05, tol=1e-10, max_evals=24)
    s.close()
    print(f"profile run: {CONFIG}, one FP64 and one TF32x3 iteration (last {st['total_ms']:.2f} ms), "
          "then two FP64 self-consistent iterations")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--config", default="C2", choices=sorted(WORKLOADS),
                    help="workload (C2 is the benchmark; C3 is for profiling and manual runs)")
    ap.add_argument("--profile", action="store_true",
                    help="one FP64 and one TF32x3 iteration and two self-consistent iterations only "
                         "(the command for ncu captures)")
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
