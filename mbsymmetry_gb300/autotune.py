"""Empirical tuning of the contraction kernels for one workload.

Sliced path (precision "ozaki"): every P0 / Sigma stage is a list of block
GEMMs whose output width N is set by an irrep block size (AO block for the
G products and the final Sigma GEMM, aux block for the final P0 GEMM).  A
tcgen05 round stages 128 rows x 16 complex K whatever N is, so narrow blocks
run faster on the CUDA-core float-float kernel.  gwgb_params.oz_simt_cols is
the width class boundary: blocks with N <= oz_simt_cols go to the CUDA cores.
OZAKI_CANDIDATES spans the classes (none, N <= 4, 8, 16, 32), scored on the
whole iteration (the boundary moves work in both contractions).

Split FP32-class paths (tf32x3 / bf16x3):

The engine picks tile shapes per irrep-block size class by rule (tau per
U/Sigma tile from 128 / k1_b and the shared-memory budget, aux rows per chunk
from what fits, W-GEMM pack width from the aux block size, slices from the
per-tau cost).  Three global settings of those rules trade occupancy against
chunk length and load balance, and the best values depend on the block-size
distribution: gwgb_params.uvt_smem_kb (shared memory per U/Sigma CTA),
sw_npk_max (widest W-GEMM pack) and uv_waves (contribution slices per tau).
``autotune`` times a small candidate set on the caller's own layout and data
(one handle per candidate, CUDA-event timing of the Sigma stage of full
iterations) and returns the fastest; ``cache`` stores results keyed by a
fingerprint of the layout's block sizes, nts, precision, the library version
and the GPU model.
"""
import hashlib
import json
import os

import numpy as np

from .solver import GWSolver

DEFAULT_CANDIDATES = (
    {"uvt_smem_kb": 0, "sw_npk_max": 0, "uv_waves": 0},      # the built-in choice (0: engine rules)
    {"uvt_smem_kb": 110, "sw_npk_max": 64, "uv_waves": 8},
    {"uvt_smem_kb": 110, "sw_npk_max": 64, "uv_waves": 4},
    {"uvt_smem_kb": 110, "sw_npk_max": 64, "uv_waves": 16},
    {"uvt_smem_kb": 72, "sw_npk_max": 64, "uv_waves": 8},
    {"uvt_smem_kb": 150, "sw_npk_max": 64, "uv_waves": 8},
    {"uvt_smem_kb": 200, "sw_npk_max": 64, "uv_waves": 8},
    {"uvt_smem_kb": 110, "sw_npk_max": 32, "uv_waves": 8},
)

OZAKI_CANDIDATES = (
    {"oz_simt_cols": 0},    # the built-in boundary (8)
    {"oz_simt_cols": -1},   # every block GEMM on tcgen05
    {"oz_simt_cols": 4},
    {"oz_simt_cols": 16},
    {"oz_simt_cols": 32},
)


def _device_key(device: int) -> str:
    """Library version plus the GPU's name, SM count and shared memory per block:
    a cached setting is reused only with the same kernels on the same kind of GPU."""
    from . import _abi
    key = _abi.load().gwgb_version().decode()
    try:
        import torch
        if torch.cuda.is_available():
            p = torch.cuda.get_device_properties(device)
            key += f"|{p.name}|{p.multi_processor_count}|{getattr(p, 'shared_memory_per_block_optin', 0)}"
    except Exception:  # noqa: BLE001 - no device information: the key holds the library version only
        pass
    return key


def fingerprint(layout, nts: int, precision: str, device: int = 0) -> str:
    """Hash of what the tile rules see (block sizes per k / q, the V block list,
    nts, precision) and of the kernels and GPU that were timed."""
    h = hashlib.sha256()
    h.update(_device_key(device).encode())
    for arrs in (layout.ao_sizes, layout.aux_sizes, layout.tensor_irreps):
        for a in arrs:
            h.update(np.ascontiguousarray(a, dtype=np.int64).tobytes())
            h.update(b"|")
    h.update(np.asarray(layout.irre_list, dtype=np.int64).tobytes())
    h.update(f"{nts}:{precision}".encode())
    return h.hexdigest()[:16]


def autotune(layout, ns, transforms, V, F, S, mu, G=None, precision="tf32x3", candidates=None,
             warmup=1, reps=2, cache=None, device=0):
    """Time each candidate on this workload; return {"best": settings, "trials": [...]}.

    G: the Green's function to iterate from (default: Dyson of Sigma = 0 at mu).
    candidates: default OZAKI_CANDIDATES for "ozaki", else DEFAULT_CANDIDATES.
    The metric is the whole iteration for "ozaki" and the Sigma stage (the
    stage the settings shape) otherwise, median of `reps` iterations after
    `warmup`; each trial records both.
    With ``cache`` (a JSON file path) an earlier result for the same
    fingerprint is returned without timing, and new results are added.
    Each candidate is a full handle with V in device memory, built and closed
    in turn: the device needs room for one such handle besides any the caller
    holds (at C5 scale, 180 GB, tune before creating the working handle)."""
    if candidates is None:
        candidates = OZAKI_CANDIDATES if precision == "ozaki" else DEFAULT_CANDIDATES
    metric = "iteration_ms" if precision == "ozaki" else "sigma_ms"
    key = fingerprint(layout, transforms.nts, precision, device)
    store = {}
    if cache and os.path.exists(cache):
        with open(cache) as f:
            store = json.load(f)
        if key in store:
            return store[key]
    trials = []
    for cand in candidates:
        s = GWSolver(layout, ns, transforms, precision=precision, device=device, tune=cand)
        try:
            s.set_shared_Coulomb(V)
            s.set_fock(F, S)
            if G is None:
                s.set_Selfenergy(np.zeros(s.g_size, np.complex128))
                s.dyson(mu)
                G0 = s.G_tau()
            else:
                G0 = G
            sig, tot = [], []
            for r in range(warmup + reps):
                s.set_G(G0)
                s.iteration(mu)
                st = s.stats()
                if r >= warmup:
                    sig.append(st["sigma_ms"])
                    tot.append(st["total_ms"])
            trials.append({"settings": dict(cand), "sigma_ms": float(np.median(sig)),
                           "iteration_ms": float(np.median(tot))})
        finally:
            s.close()
    best = min(trials, key=lambda t: t[metric])
    out = {"fingerprint": key, "precision": precision, "metric": metric, "best": best["settings"], "trials": trials}
    if cache:
        store[key] = out
        with open(cache, "w") as f:
            json.dump(store, f, indent=1)
    return out
