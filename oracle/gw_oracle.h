/*
 * gw_oracle.h — FP64 CPU restatement of SymmetryMBPT's GW iteration.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle: the parity tests, the
 * smoke check and bench.py's cpu_baseline / reference arm call it as the
 * checker or the timed CPU baseline.  The product path (libgwgb) never links,
 * loads or calls it.
 *
 * Parity status: pinned on the reference's LiH nk=2x2x2 fixture through the
 * reference's own cross-relations (block vs dense P0, P~, Dyson), see
 * tests/golden/make_golden.py.
 *
 * Every routine works on the reference's host layouts (include/gwgb.h) and
 * cites the reference file:line it restates.  Complex numbers are
 * interleaved (re, im) doubles.
 */
#ifndef GW_ORACLE_H
#define GW_ORACLE_H

#include <stdint.h>
#include "../include/gwgb.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gwo_layout gwo_layout;

/* Derive all offsets from a gwgb_layout (symmetry_utils.cpp:96-307). */
gwo_layout *gwo_layout_create(const gwgb_layout *L);
void gwo_layout_destroy(gwo_layout *l);
int64_t gwo_flat_ao(const gwo_layout *l);      /* irreducible k */
int64_t gwo_flat_aux(const gwo_layout *l);     /* irreducible q */
int64_t gwo_flat_ao_full(const gwo_layout *l); /* all k */
int64_t gwo_flat_aux_full(const gwo_layout *l);/* all q */
int64_t gwo_flat_V(const gwo_layout *l);
int64_t gwo_flat_orep(const gwo_layout *l);
int64_t gwo_flat_auxrep(const gwo_layout *l);

/* iBZ -> full-BZ rotation of G: out layout [k][t][s][kslice(k)] at
 * ns*nts*kao_slice_offsets(k) (cugw_routines_block.cu:100-186). */
void gwo_rotate_G(const gwo_layout *l, int ns, int nts, const double *G_irr,
                  const double *orep, double *G_full);

/* P0 for t < nt_max (gw_block.cpp:6-84 loop nest, q over the irreducible
 * list as cugw_routines_block.cu:276-294 runs it); out [ink][nts][qslice]
 * zeroed first, prefactor (-2 if ns==1 else -1)/nk applied. */
void gwo_p0(const gwo_layout *l, int ns, int nts, int nt_max, const double *G_full,
            const double *V, double *P0);

/* P0(beta - t) = P0(t) mirror (cugw_solver_block.cpp:441-456). */
void gwo_mirror_P0(const gwo_layout *l, int nts, double *P0);

/* P~ = (1 - P~0)^-1 P~0 per (q, Omega, block), in place on [ink][nts][qslice]
 * (cugw_solver_block.cpp:385-439).  Tnt_BF [nw_b][nts-2], Ttn_FB [nts][nw_b]. */
int gwo_p_tilde(const gwo_layout *l, int nts, int nw_b, const double *Tnt_BF,
                const double *Ttn_FB, double *P);

/* P~(q_irr) -> P~(q) for all q: out [q][t][qslice(q)] at nts*qaux_slice_offsets(q)
 * (cugw_qkpt_block.cu:288-340). */
void gwo_rotate_P(const gwo_layout *l, int nts, const double *P_irr,
                  const double *auxrep, double *P_full);

/* Sigma for t < nt_max over irreducible k, all q (gw_block.cpp:86-158 loop
 * nest; k over the irreducible list as cugw_routines_block.cu:296-318);
 * out [nts][ns][flat_ao], zeroed first, scaled by -1/nk. */
void gwo_sigma(const gwo_layout *l, int ns, int nts, int nt_max, const double *G_full,
               const double *P_full, const double *V, double *Sigma);

/* Dyson (sc_type_block.cpp:6-87): G(tau) from Sigma(tau), F, S.
 * Tnt [nw][nts-2], Ttn [nts][nw]; wsample [nw] Matsubara indices.
 * Writes the leakage ratio when tct_first/tct_last are given. */
int gwo_dyson(const gwo_layout *l, int ns, int nts, int nw, double beta, double mu,
              const int64_t *wsample, const double *Tnt, const double *Ttn,
              const double *F, const double *S, const double *Sigma, double *G,
              const double *tct_first, const double *tct_last, double *leakage);

/* Threads used by the OpenMP loops (0 = runtime default). */
void gwo_set_threads(int n);
int gwo_get_threads(void);

#ifdef __cplusplus
}
#endif

#endif
