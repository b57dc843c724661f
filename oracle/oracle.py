"""Python binding of the FP64 CPU oracle (``oracle/libgworacle.so``).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and
bench.py's CPU-baseline / reference arm as the checker or the timed CPU
baseline.  The product package never imports it.

The oracle restates SymmetryMBPT's CPU algorithm (see ``gw_oracle.c``) on the
reference's host layouts; :class:`Oracle` runs a whole GW iteration or single
stages.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from ctypes import c_double, c_int, c_int64, c_void_p

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libgworacle.so")

_lib = None


def build(quiet: bool = True):
    """Compile the oracle with its Makefile (gcc, OpenMP)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True,
                   stdout=subprocess.DEVNULL if quiet else None)


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB):
        build()
    lib = ctypes.CDLL(LIB)
    lib.gwo_layout_create.restype = c_void_p
    lib.gwo_layout_create.argtypes = [c_void_p]
    lib.gwo_layout_destroy.argtypes = [c_void_p]
    for n in ("gwo_flat_ao", "gwo_flat_aux", "gwo_flat_ao_full", "gwo_flat_aux_full", "gwo_flat_V",
              "gwo_flat_orep", "gwo_flat_auxrep"):
        getattr(lib, n).restype = c_int64
        getattr(lib, n).argtypes = [c_void_p]
    lib.gwo_rotate_G.argtypes = [c_void_p, c_int, c_int, c_void_p, c_void_p, c_void_p]
    lib.gwo_p0.argtypes = [c_void_p, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p]
    lib.gwo_mirror_P0.argtypes = [c_void_p, c_int, c_void_p]
    lib.gwo_p_tilde.restype = c_int
    lib.gwo_p_tilde.argtypes = [c_void_p, c_int, c_int, c_void_p, c_void_p, c_void_p]
    lib.gwo_rotate_P.argtypes = [c_void_p, c_int, c_void_p, c_void_p, c_void_p]
    lib.gwo_sigma.argtypes = [c_void_p, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p]
    lib.gwo_dyson.restype = c_int
    lib.gwo_dyson.argtypes = [c_void_p, c_int, c_int, c_int, c_double, c_double, c_void_p, c_void_p,
                              c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                              ctypes.POINTER(c_double)]
    lib.gwo_set_threads.argtypes = [c_int]
    lib.gwo_get_threads.restype = c_int
    _lib = lib
    return lib


def _p(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


class Oracle:
    """FP64 CPU GW iteration over one :class:`~mbsymmetry_gb300.layout.BlockLayout`."""

    def __init__(self, layout, ns: int, nts: int, threads: int = 0):
        self.lib = load()
        self.layout = layout
        self.ns = ns
        self.nts = nts
        self._c, self._keep = layout.to_c()
        self.h = self.lib.gwo_layout_create(ctypes.byref(self._c))
        self.lib.gwo_set_threads(threads)
        assert self.lib.gwo_flat_ao(self.h) == layout.flat_ao_size
        assert self.lib.gwo_flat_aux(self.h) == layout.flat_aux_size
        assert self.lib.gwo_flat_V(self.h) == layout.flat_V_size

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.gwo_layout_destroy(self.h)
            self.h = None

    def threads(self) -> int:
        return self.lib.gwo_get_threads()

    # -- stages ------------------------------------------------------------ #
    def rotate_G(self, G_irr, orep=None):
        L = self.layout
        orep = L.orep if orep is None else orep
        out = np.zeros(L.flat_ao_size_full * self.ns * self.nts, dtype=np.complex128)
        G_irr = np.ascontiguousarray(G_irr, dtype=np.complex128)
        orep = np.ascontiguousarray(orep, dtype=np.complex128)
        self.lib.gwo_rotate_G(self.h, self.ns, self.nts, _p(G_irr), _p(orep), _p(out))
        return out

    def p0(self, G_full, V, nt_max=None):
        L = self.layout
        nt_max = self.nts // 2 if nt_max is None else nt_max
        out = np.zeros(self.nts * L.flat_aux_size, dtype=np.complex128)
        self.lib.gwo_p0(self.h, self.ns, self.nts, nt_max, _p(G_full), _p(V), _p(out))
        return out

    def mirror_P0(self, P0):
        P0 = np.ascontiguousarray(P0, dtype=np.complex128).copy()
        self.lib.gwo_mirror_P0(self.h, self.nts, _p(P0))
        return P0

    def p_tilde(self, P0, tr):
        P = np.ascontiguousarray(P0, dtype=np.complex128).copy()
        rc = self.lib.gwo_p_tilde(self.h, self.nts, tr.nw_b, _p(tr.Tnt_BF), _p(tr.Ttn_FB), _p(P))
        if rc:
            raise RuntimeError("oracle: singular block in the W~ solve")
        return P

    def rotate_P(self, P_irr, auxrep=None):
        L = self.layout
        auxrep = L.auxrep if auxrep is None else auxrep
        out = np.zeros(self.nts * L.flat_aux_size_full, dtype=np.complex128)
        P_irr = np.ascontiguousarray(P_irr, dtype=np.complex128)
        auxrep = np.ascontiguousarray(auxrep, dtype=np.complex128)
        self.lib.gwo_rotate_P(self.h, self.nts, _p(P_irr), _p(auxrep), _p(out))
        return out

    def sigma(self, G_full, P_full, V, nt_max=None):
        L = self.layout
        nt_max = self.nts if nt_max is None else nt_max
        out = np.zeros(self.nts * self.ns * L.flat_ao_size, dtype=np.complex128)
        self.lib.gwo_sigma(self.h, self.ns, self.nts, nt_max, _p(G_full), _p(P_full), _p(V), _p(out))
        return out

    def dyson(self, Sigma, F, S, tr, mu):
        L = self.layout
        out = np.zeros(self.nts * self.ns * L.flat_ao_size, dtype=np.complex128)
        Sigma = np.ascontiguousarray(Sigma, dtype=np.complex128)
        F = np.ascontiguousarray(F, dtype=np.complex128)
        S = np.ascontiguousarray(S, dtype=np.complex128)
        leak = c_double(0.0)
        tf = np.ascontiguousarray(tr.Tct[0])
        tl = np.ascontiguousarray(tr.Tct[tr.ncheb - 1])
        rc = self.lib.gwo_dyson(self.h, self.ns, self.nts, tr.nw, tr.beta, mu, _p(tr.wsample_fermi),
                                _p(tr.Tnt), _p(tr.Ttn), _p(F), _p(S), _p(Sigma), _p(out), _p(tf),
                                _p(tl), ctypes.byref(leak))
        if rc:
            raise RuntimeError("oracle: singular block in Dyson")
        return out, leak.value

    # -- whole iteration (cugw_solver_block.cpp:254-315 + sc_type_block.cpp) -- #
    def gw_sigma(self, G_irr, V, tr):
        """Sigma from G: rotate G, P0, P~, rotate P, Sigma."""
        Gf = self.rotate_G(G_irr)
        P0 = self.p0(Gf, V)
        P = self.p_tilde(P0, tr)
        Pf = self.rotate_P(P)
        return self.sigma(Gf, Pf, V), P0, P

    def iteration(self, G_irr, V, F, S, tr, mu):
        Sigma, P0, P = self.gw_sigma(G_irr, V, tr)
        G, leak = self.dyson(Sigma, F, S, tr, mu)
        return G, Sigma, P0, P, leak

    # -- self-consistent loop: electron count, energies, mu search, mixing -- #
    # Not in the reference (sc_loop_block_t keeps mu fixed, never assigns its
    # energy and does not iterate); these restate the formulas of the engine's
    # loop with dense numpy traces, independently of its block-wise kernels.
    def k_weights(self):
        """Mesh k points mapped to each stored k."""
        L = self.layout
        return np.bincount(L.irre_index, minlength=L.ink).astype(np.float64)

    def _trace(self, A, B):
        """sum_{s,k} w_k Re Tr[A_k,s B_k,s] for two [ns][flat_ao] arrays."""
        L = self.layout
        fa = L.flat_ao_size
        Ab = L.G_flat_to_block(np.asarray(A).reshape(self.ns, fa))
        Bb = L.G_flat_to_block(np.asarray(B).reshape(self.ns, fa))
        t = np.einsum("skab,skba->sk", Ab, Bb).real
        return float((t * self.k_weights()[None, :]).sum())

    def n_electrons(self, G, S):
        """N = -(2/ns)/nk sum_{s,k} Re Tr[G(beta) S]."""
        L = self.layout
        Gb = np.asarray(G).reshape(self.nts, self.ns * L.flat_ao_size)[-1]
        return -(2.0 / self.ns) / L.nk * self._trace(Gb, S)

    def energy(self, Sigma, G, F, S, M, H=None):
        """(E_corr, E_one, N): Galitskii-Migdal energy with the interior-tau
        weights M, the one-body energy (with H) and the electron count."""
        L = self.layout
        nf = self.ns * L.flat_ao_size
        Sg = np.asarray(Sigma).reshape(self.nts, nf)
        Gt = np.asarray(G).reshape(self.nts, nf)
        MG = np.asarray(M) @ Gt[1:-1]
        ec = sum(self._trace(Sg[1 + i], MG[i]) for i in range(self.nts - 2))
        ec *= -(1.0 / self.ns) / L.nk
        eo = 0.0
        if H is not None:
            eo = -(1.0 / self.ns) / L.nk * (self._trace(Gt[-1], H) + self._trace(Gt[-1], F))
        return ec, eo, self.n_electrons(G, S)

    def find_mu(self, Sigma, F, S, tr, n_target, mu0, step=0.05, tol=1e-12, maxit=400):
        """Bracket, then bisect N(mu) = n_target.  Returns (mu, G, leakage)."""
        def f(mu):
            G, leak = self.dyson(Sigma, F, S, tr, mu)
            return self.n_electrons(G, S) - n_target, G, leak

        f0, G0, l0 = f(mu0)
        if abs(f0) <= tol:
            return mu0, G0, l0
        lo = hi = mu0
        flo = fhi = f0
        d = step
        while flo > 0:
            hi, fhi = lo, flo
            lo -= d
            d *= 2
            flo = f(lo)[0]
        while fhi < 0:
            lo, flo = hi, fhi
            hi += d
            d *= 2
            fhi = f(hi)[0]
        best = (abs(f0), mu0, G0, l0)
        for _ in range(maxit):
            mid = 0.5 * (lo + hi)
            fm, Gm, lm = f(mid)
            if abs(fm) < best[0]:
                best = (abs(fm), mid, Gm, lm)
            if abs(fm) <= tol or hi - lo < 1e-15 * max(1.0, abs(mid)):
                break
            if fm < 0:
                lo = mid
            else:
                hi = mid
        return best[1], best[2], best[3]

    def sc_loop(self, G, Sigma, V, F, S, tr, M, niter, alpha, n_target, mu0, H=None, mus=None):
        """niter iterations: Sigma_new = GW(G); Sigma = alpha Sigma_new +
        (1 - alpha) Sigma_old; mu from N(mu) = n_target (or mus[it] when
        given); G = Dyson(Sigma, mu); energies.  Returns (G, Sigma, records)."""
        Sold = np.asarray(Sigma, dtype=np.complex128).copy()
        mu = mu0
        recs = []
        for it in range(niter):
            Snew, _, _ = self.gw_sigma(G, V, tr)
            Sig = alpha * Snew + (1.0 - alpha) * Sold
            Sold = Sig
            if mus is not None:
                mu = mus[it]
                G, leak = self.dyson(Sig, F, S, tr, mu)
            else:
                mu, G, leak = self.find_mu(Sig, F, S, tr, n_target, mu)
            ec, eo, n = self.energy(Sig, G, F, S, M, H)
            recs.append({"mu": mu, "n_electrons": n, "e_corr": ec, "e_one": eo, "leakage": leak})
        return G, Sold, recs
