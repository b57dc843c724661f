"""Host-side mirror of the reference's GW solver interface over the C ABI.

``GWSolver`` exposes the methods of SymmetryMBPT's ``solver_block_t`` /
``cugw_solver_block_t`` (``SymmetryMBPT/include/solver/solver_block_t.h:37-65``,
``SymmetryMBPT/include/solver/cugw_solver_block.h:117-180``) with the same
names and meaning -- ``solve()``, ``solve_P0()``, ``solve_sigma()``,
``compute_Pq_from_P0q()``, ``P0_q_t_QP()``, ``single_prec_run()`` -- plus the
Dyson step of ``dyson_sc_block_t::compute_G``
(``SymmetryMBPT/src/scmbpt/sc_type_block.cpp:6-87``).  G(tau) and Sigma(tau)
live in caller-owned host arrays (the reference keeps them in MPI shared
windows owned by ``sc_loop_block_t``); every call goes through
``libgwgb.so``.  Errors raise :class:`~mbsymmetry_gb300._abi.GwgbError`, a
``RuntimeError`` as the reference's ``std::runtime_error``.
"""
from __future__ import annotations

import ctypes
from typing import Optional

import numpy as np

from . import _abi
from .layout import BlockLayout
from .transformer import IRTransforms, gm_matrix


def _ptr(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


class GWSolver:
    def __init__(self, layout: BlockLayout, ns: int, transforms: IRTransforms,
                 precision: str = "fp64", device: int = 0, tune: dict = None):
        """tune: optional gwgb_params settings chosen by autotune.autotune()
        (its "best" entry): oz_simt_cols, the width-class boundary of the
        sliced path, or the tile settings of the FP32-class tcgen05 Sigma
        path (uvt_smem_kb, sw_npk_max, uv_waves)."""
        self.lib = _abi.load()
        self.layout = layout
        self.ns = ns
        self.tr = transforms
        self.nts = transforms.nts
        p = _abi.GwgbParams(ns=ns, nts=transforms.nts, nw=transforms.nw, nw_b=transforms.nw_b,
                            beta=transforms.beta, precision=_abi.PREC_NAMES[precision], device=device,
                            nt_batch=0, flags=0, **{k: int(v) for k, v in (tune or {}).items()})
        self._lay_c, self._keep = layout.to_c()
        h = ctypes.c_void_p()
        _abi.check(self.lib.gwgb_create(ctypes.byref(p), ctypes.byref(self._lay_c), ctypes.byref(h)))
        self.h = h
        L = layout
        _abi.check(self.lib.gwgb_set_reps(self.h, _ptr(np.ascontiguousarray(L.orep)), L.orep.size,
                                          _ptr(np.ascontiguousarray(L.auxrep)), L.auxrep.size))
        tf = np.ascontiguousarray(transforms.Tct[0])
        tl = np.ascontiguousarray(transforms.Tct[transforms.ncheb - 1])
        _abi.check(self.lib.gwgb_set_transforms(
            self.h, _ptr(transforms.Tnt), _ptr(transforms.Ttn), _ptr(transforms.Tnt_BF), _ptr(transforms.Ttn_FB),
            _ptr(transforms.wsample_fermi), _ptr(tf), _ptr(tl)))
        M = gm_matrix(transforms)
        _abi.check(self.lib.gwgb_set_energy_matrix(self.h, _ptr(M), M.shape[0]))

    def close(self):
        if getattr(self, "h", None):
            self.lib.gwgb_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    # -- sizes ----------------------------------------------------------------
    @property
    def g_size(self) -> int:
        return self.nts * self.ns * self.layout.flat_ao_size

    @property
    def p_size(self) -> int:
        return self.nts * self.layout.flat_aux_size

    # -- inputs (set_shared_Coulomb, copy_*_host_to_device) --------------------
    def set_shared_Coulomb(self, V: np.ndarray):
        V = np.ascontiguousarray(V, dtype=np.complex128)
        _abi.check(self.lib.gwgb_upload_V(self.h, _ptr(V), V.size))

    def set_fock(self, F: np.ndarray, S: np.ndarray):
        F = np.ascontiguousarray(F, dtype=np.complex128)
        S = np.ascontiguousarray(S, dtype=np.complex128)
        _abi.check(self.lib.gwgb_set_fock(self.h, _ptr(F), _ptr(S)))

    def single_prec_run(self, run_sp: bool, kind: str = "ozaki"):
        """Split-precision contractions on (``kind``: "ozaki", the path with the
        1e-7 Ha bound, or the FP32-class "tf32x3" / "bf16x3") or off (FP64)."""
        _abi.check(self.lib.gwgb_set_precision(self.h, _abi.PREC_NAMES[kind if run_sp else "fp64"]))

    # -- G / Sigma / P host <-> device ----------------------------------------
    def set_G(self, G: np.ndarray):
        G = np.ascontiguousarray(G, dtype=np.complex128)
        assert G.size == self.g_size
        _abi.check(self.lib.gwgb_set_G(self.h, _ptr(G)))

    def G_tau(self, out: Optional[np.ndarray] = None) -> np.ndarray:
        out = np.empty(self.g_size, np.complex128) if out is None else out
        _abi.check(self.lib.gwgb_get_G(self.h, _ptr(out)))
        return out

    def set_Selfenergy(self, S: np.ndarray):
        S = np.ascontiguousarray(S, dtype=np.complex128)
        assert S.size == self.g_size
        _abi.check(self.lib.gwgb_set_sigma(self.h, _ptr(S)))

    def Selfenergy(self, out: Optional[np.ndarray] = None) -> np.ndarray:
        out = np.empty(self.g_size, np.complex128) if out is None else out
        _abi.check(self.lib.gwgb_get_sigma(self.h, _ptr(out)))
        return out

    def set_P0(self, P: np.ndarray):
        P = np.ascontiguousarray(P, dtype=np.complex128)
        assert P.size == self.p_size
        _abi.check(self.lib.gwgb_set_P0(self.h, _ptr(P)))

    def P0_q_t_QP(self, out: Optional[np.ndarray] = None) -> np.ndarray:
        out = np.empty(self.p_size, np.complex128) if out is None else out
        _abi.check(self.lib.gwgb_get_P0(self.h, _ptr(out)))
        return out

    # -- solver API (cugw_solver_block_t) --------------------------------------
    def solve_P0(self):
        _abi.check(self.lib.gwgb_solve_P0(self.h))

    def compute_Pq_from_P0q(self):
        _abi.check(self.lib.gwgb_solve_Pq(self.h))

    def solve_sigma(self):
        _abi.check(self.lib.gwgb_solve_sigma(self.h))

    def solve(self):
        _abi.check(self.lib.gwgb_solve(self.h))

    def dyson(self, mu: float):
        _abi.check(self.lib.gwgb_dyson(self.h, float(mu)))

    def iteration(self, mu: float):
        _abi.check(self.lib.gwgb_iteration(self.h, float(mu)))

    # -- self-consistent loop (not in the reference; see include/gwgb.h) -------
    def set_hcore(self, H: np.ndarray):
        H = np.ascontiguousarray(H, dtype=np.complex128)
        _abi.check(self.lib.gwgb_set_hcore(self.h, _ptr(H)))

    @staticmethod
    def _mu_search(n_electrons, mu0, step, tol, max_evals):
        return _abi.GwgbMuSearch(n_electrons=float(n_electrons), mu0=float(mu0), step=float(step),
                                 tol=float(tol), max_evals=int(max_evals), pad=0)

    def find_mu(self, n_electrons: float, mu0: float, step: float = 0.05, tol: float = 1e-10,
                max_evals: int = 32):
        """Dyson with a device-side mu search; returns (mu, N(mu))."""
        ms = self._mu_search(n_electrons, mu0, step, tol, max_evals)
        mu, n = ctypes.c_double(), ctypes.c_double()
        _abi.check(self.lib.gwgb_find_mu(self.h, ctypes.byref(ms), ctypes.byref(mu), ctypes.byref(n)))
        return mu.value, n.value

    def energy(self, with_one_body: bool = False):
        """(E_corr, E_one) of the resident Sigma and G (E_one needs set_hcore)."""
        ec, eo = ctypes.c_double(), ctypes.c_double()
        _abi.check(self.lib.gwgb_energy(self.h, ctypes.byref(ec), ctypes.byref(eo) if with_one_body else None))
        return ec.value, (eo.value if with_one_body else None)

    def sc_loop(self, niter: int, alpha: float, n_electrons: float, mu0: float, step: float = 0.05,
                tol: float = 1e-10, max_evals: int = 32, final_fp64: bool = False, log=None) -> list:
        """niter self-consistent GW iterations (one CUDA graph launch each);
        one dict per iteration: mu, n_electrons, e_corr, e_one, leakage, mu_evals, precision.
        With ``log`` (a writable text file) one JSON line per iteration is
        written, with the mean device time per iteration."""
        ms = self._mu_search(n_electrons, mu0, step, tol, max_evals)
        recs = (_abi.GwgbScRecord * niter)()
        _abi.check(self.lib.gwgb_sc_loop(self.h, int(niter), float(alpha), ctypes.byref(ms),
                                         1 if final_fp64 else 0, recs))
        out = [{name: getattr(r, name) for name, _ in _abi.GwgbScRecord._fields_} for r in recs]
        if log is not None:
            import json
            ms_it = self.stats()["total_ms"]
            for i, r in enumerate(out):
                log.write(json.dumps({"iteration": i, "ms_per_iteration_mean": ms_it, **r}) + "\n")
        return out

    # -- checkpoint / resume (the reference writes none) ----------------------
    def save_state(self, path: str, mu: float, iteration: int = 0, **extra) -> None:
        """Write G(tau), Sigma(tau) and mu: ``<path>.npz`` (the arrays, host
        layout [nts][ns][flat_ao]) and ``<path>.json`` (a header), so that a
        self-consistent run can resume with :meth:`load_state` + :meth:`sc_loop`."""
        import json
        np.savez(path + ".npz", G=self.G_tau(), Sigma=self.Selfenergy())
        hdr = {"format": "gwgb-state-1", "nts": self.nts, "ns": self.ns,
               "flat_ao": int(self.layout.flat_ao_size), "nk": int(self.layout.nk),
               "ink": int(self.layout.ink), "beta": float(self.tr.beta), "mu": float(mu),
               "iteration": int(iteration), "engine": self.lib.gwgb_version().decode()}
        hdr.update(extra)
        with open(path + ".json", "w") as f:
            json.dump(hdr, f, indent=1)

    def load_state(self, path: str) -> dict:
        """Read a state written by :meth:`save_state` into the engine; returns
        its header (``mu``, ``iteration``, ...).  Shapes are checked."""
        import json
        with open(path + ".json") as f:
            hdr = json.load(f)
        if hdr.get("format") != "gwgb-state-1":
            raise ValueError(f"{path}.json: not a gwgb state file")
        for key, val in (("nts", self.nts), ("ns", self.ns), ("flat_ao", self.layout.flat_ao_size),
                         ("nk", self.layout.nk), ("ink", self.layout.ink)):
            if int(hdr[key]) != int(val):
                raise ValueError(f"{path}: {key} = {hdr[key]} does not match this solver ({val})")
        z = np.load(path + ".npz")
        self.set_G(z["G"])
        self.set_Selfenergy(z["Sigma"])
        return hdr

    def synchronize(self):
        _abi.check(self.lib.gwgb_synchronize(self.h))

    def solve_sigma_from_P(self):
        """The Sigma contraction from the current G and P buffers (P0 is not recomputed)."""
        _abi.check(self.lib.gwgb_solve_sigma_from_P(self.h))

    def hf_exchange(self, rho: np.ndarray) -> np.ndarray:
        """Hartree-Fock exchange on the block engine,
            K(k) = -(1/nk) sum_k2 sum_Q V^Q(k, k2) rho(k2) V^Q(k, k2)^H,
        as the Sigma contraction with P = identity and G = rho at tau = 0 (the
        reference's HF solver is a stub, cuhf_solver_block.h:36-39).  rho and the
        result: [s][flat_ao] over the stored k.  Overwrites the handle's G, P and Sigma."""
        L = self.layout
        fa = L.flat_ao_size
        rho = np.ascontiguousarray(rho, dtype=np.complex128).reshape(self.ns, fa)
        G = np.zeros(self.g_size, np.complex128)
        G[:self.ns * fa] = rho.ravel()
        P = np.zeros(self.p_size, np.complex128)
        for r, q in enumerate(L.irre_list):
            base = self.nts * L.qaux_slice_offsets_irre[r]
            for iq, qb in enumerate(L.aux_sizes[q]):
                o = base + L.aux_offsets[q][iq]
                P[o:o + qb * qb] = np.eye(qb).ravel()
        self.set_G(G)
        self.set_P0(P)
        self.solve_sigma_from_P()
        return self.Selfenergy()[:self.ns * fa].reshape(self.ns, fa).copy()

    def hf_hartree(self, rho: np.ndarray) -> np.ndarray:
        """Hartree (direct) term J(k) = sum_Q V^Q(k, k) c_Q, c_Q = (f/nk) sum_{k', s}
        Tr[V^Q(k', k') rho_s(k')] (f = 2 for ns = 1), on the diagonal AO blocks of the
        stored k (gwgb_hf_hartree).  rho: [s][flat_ao]; returns [s][flat_ao] (the same J
        for every spin).  Overwrites the handle's G."""
        fa = self.layout.flat_ao_size
        rho = np.ascontiguousarray(rho, dtype=np.complex128).reshape(self.ns, fa)
        G = np.zeros(self.g_size, np.complex128)
        G[:self.ns * fa] = rho.ravel()
        self.set_G(G)
        J = np.zeros(fa, np.complex128)
        _abi.check(self.lib.gwgb_hf_hartree(self.h, J.ctypes.data))
        return np.tile(J, (self.ns, 1))

    def refproxy(self, nt_batch: int = 4, nstreams: int = 16) -> dict:
        """Run the reference's cuBLAS call sequence for P0 and Sigma on this
        GPU (measurement only; gwgb_refproxy_run).  P0 comes from the current G,
        Sigma from G and the P~ of the last solve()."""
        st = _abi.GwgbProxyStats()
        _abi.check(self.lib.gwgb_refproxy_run(self.h, nt_batch, nstreams, ctypes.byref(st)))
        return {name: getattr(st, name) for name, _ in _abi.GwgbProxyStats._fields_}

    def refproxy_results(self):
        """(P0 [q_irr][t][qslice], Sigma [t][s][flat_ao]) of the last refproxy()."""
        P = np.zeros(self.p_size, np.complex128)
        S = np.zeros(self.g_size, np.complex128)
        _abi.check(self.lib.gwgb_refproxy_get(self.h, P.ctypes.data, S.ctypes.data))
        return P, S

    def stats(self) -> dict:
        s = _abi.GwgbStats()
        _abi.check(self.lib.gwgb_get_stats(self.h, ctypes.byref(s)))
        return {name: getattr(s, name) for name, _ in _abi.GwgbStats._fields_}

    def launch_timing(self, on: bool = True):
        """Bracket every sliced-path GEMM / reduction launch with CUDA events
        (gwgb_set_launch_timing); read them with launch_stats()."""
        _abi.check(self.lib.gwgb_set_launch_timing(self.h, 1 if on else 0))

    def launch_stats(self) -> list:
        """One dict per sliced-path launch of the last solve / iteration:
        stage, kernel, tasks, ran, ms, flops, mma_flops, bytes."""
        n = ctypes.c_int32()
        _abi.check(self.lib.gwgb_get_launch_stats(self.h, None, 0, ctypes.byref(n)))
        arr = (_abi.GwgbLaunchStat * max(1, n.value))()
        _abi.check(self.lib.gwgb_get_launch_stats(self.h, arr, n.value, ctypes.byref(n)))
        out = []
        for x in arr[:n.value]:
            d = {name: getattr(x, name) for name, _ in _abi.GwgbLaunchStat._fields_}
            d["stage"] = _abi.LAUNCH_STAGES[x.stage]
            d["kernel"] = _abi.LAUNCH_KERNELS[x.kernel]
            out.append(d)
        return out

    def name(self) -> str:
        return "GB300 GW solver"
