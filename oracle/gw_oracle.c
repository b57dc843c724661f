/*
 * gw_oracle.c — FP64 CPU restatement of SymmetryMBPT's symmetry-adapted GW
 * iteration (the oracle).
 *
 * TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and
 * bench.py (cpu_baseline and the --impl reference arm) as the checker or the
 * timed CPU baseline.  Nothing in the product library calls it.
 *
 * Loop nests follow the reference's CPU implementation
 * (SymmetryMBPT/src/cpu_ref/gw_block.cpp) with the k/q loops restricted to
 * the irreducible lists exactly as the reference's GPU driver runs them
 * (SymmetryMBPT/src/cuda/cugw_routines_block.cu:276-318); small complex
 * GEMMs are written as plain loops.  The OpenMP parallelisation gives each
 * thread whole output slices (P0[q][t], Sigma[k][t]) so results do not
 * depend on the thread count.
 */
#define _GNU_SOURCE
#include "gw_oracle.h"

#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double _Complex cplx;

struct gwo_layout {
  int nk, ink;
  int *irre_list, *index, *irre_index, *conj_index, *q_ind, *q_ind2;
  /* per k: block lists */
  int *ao_ptr, *ao_sz; int64_t *ao_off;
  int *aux_ptr, *aux_sz; int64_t *aux_off;
  int64_t *kao_off, *kao_sz, *qaux_off, *qaux_sz;           /* full BZ */
  int64_t *kao_off_irre, *qaux_off_irre;                    /* iBZ */
  int64_t flat_ao, flat_aux, flat_ao_full, flat_aux_full;
  /* V */
  int *kp_ptr, *ti; int64_t *t_off, *kp_off, *kp_sz; int64_t flat_V;
  /* reps */
  int *or_ptr, *or_ir; int64_t *or_off, *kor_off; int64_t flat_orep;
  int *ar_ptr, *ar_ir; int64_t *ar_off, *kar_off; int64_t flat_auxrep;
};

static int g_threads = 0;
void gwo_set_threads(int n) { g_threads = n; }
int gwo_get_threads(void) {
#ifdef _OPENMP
  return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
  return 1;
#endif
}

static int *dup_i(const int32_t *s, size_t n) {
  int *d = (int *)malloc((n ? n : 1) * sizeof(int));
  for (size_t i = 0; i < n; ++i) d[i] = s[i];
  return d;
}

/* k_i - k_j + k_k (symmetry_utils.cpp:337-341). */
static int mom_cons(const gwo_layout *l, int i, int j, int k) {
  int q = l->q_ind2[i * l->nk + j];
  return l->q_ind[k * l->nk + q];
}

gwo_layout *gwo_layout_create(const gwgb_layout *L) {
  gwo_layout *l = (gwo_layout *)calloc(1, sizeof(gwo_layout));
  int nk = L->nk, ink = L->ink, np = nk * nk;
  l->nk = nk; l->ink = ink;
  l->irre_list = dup_i(L->irre_list, ink);
  l->index = dup_i(L->index, nk);
  l->irre_index = dup_i(L->irre_index, nk);
  l->conj_index = dup_i(L->conj_index, nk);
  l->q_ind = dup_i(L->q_ind, (size_t)np);
  l->q_ind2 = dup_i(L->q_ind2, (size_t)np);
  l->ao_ptr = dup_i(L->ao_block_ptr, nk + 1);
  l->ao_sz = dup_i(L->ao_sizes, L->ao_block_ptr[nk]);
  l->aux_ptr = dup_i(L->aux_block_ptr, nk + 1);
  l->aux_sz = dup_i(L->aux_sizes, L->aux_block_ptr[nk]);
  l->ao_off = (int64_t *)malloc(sizeof(int64_t) * (L->ao_block_ptr[nk] + 1));
  l->aux_off = (int64_t *)malloc(sizeof(int64_t) * (L->aux_block_ptr[nk] + 1));
  l->kao_off = (int64_t *)malloc(sizeof(int64_t) * nk);
  l->kao_sz = (int64_t *)malloc(sizeof(int64_t) * nk);
  l->qaux_off = (int64_t *)malloc(sizeof(int64_t) * nk);
  l->qaux_sz = (int64_t *)malloc(sizeof(int64_t) * nk);
  int64_t ka = 0, qa = 0;
  for (int k = 0; k < nk; ++k) {
    int64_t acc = 0;
    for (int b = l->ao_ptr[k]; b < l->ao_ptr[k + 1]; ++b) {
      l->ao_off[b] = acc; acc += (int64_t)l->ao_sz[b] * l->ao_sz[b];
    }
    l->kao_sz[k] = acc; l->kao_off[k] = ka; ka += acc;
    acc = 0;
    for (int b = l->aux_ptr[k]; b < l->aux_ptr[k + 1]; ++b) {
      l->aux_off[b] = acc; acc += (int64_t)l->aux_sz[b] * l->aux_sz[b];
    }
    l->qaux_sz[k] = acc; l->qaux_off[k] = qa; qa += acc;
  }
  l->flat_ao_full = ka; l->flat_aux_full = qa;
  /* iBZ re-packing (symmetry_utils.cpp:174-191) */
  l->kao_off_irre = (int64_t *)malloc(sizeof(int64_t) * ink);
  l->qaux_off_irre = (int64_t *)malloc(sizeof(int64_t) * ink);
  ka = 0; qa = 0;
  for (int ik = 0; ik < ink; ++ik) {
    int k = l->irre_list[ik];
    l->kao_off_irre[ik] = ka; ka += l->kao_sz[k];
    l->qaux_off_irre[ik] = qa; qa += l->qaux_sz[k];
  }
  l->flat_ao = ka; l->flat_aux = qa;
  /* V pair slices: block (iq, ik1, ik2) of pair (k1, k2) is [q_b][k1_b][k2_b]
   * with q = k2 - k1 (the q of gw_block.cpp:23-24). */
  l->kp_ptr = dup_i(L->kpair_block_ptr, np + 1);
  int nvb = l->kp_ptr[np];
  l->ti = dup_i(L->tensor_irreps, 3 * (size_t)nvb);
  l->t_off = (int64_t *)malloc(sizeof(int64_t) * (nvb + 1));
  l->kp_off = (int64_t *)malloc(sizeof(int64_t) * np);
  l->kp_sz = (int64_t *)malloc(sizeof(int64_t) * np);
  int64_t va = 0;
  for (int p = 0; p < np; ++p) {
    int k1 = p / nk, k2 = p % nk;
    int q = mom_cons(l, k2, k1, 0);
    int64_t acc = 0;
    for (int b = l->kp_ptr[p]; b < l->kp_ptr[p + 1]; ++b) {
      int iq = l->ti[3 * b], i1 = l->ti[3 * b + 1], i2 = l->ti[3 * b + 2];
      l->t_off[b] = acc;
      acc += (int64_t)l->aux_sz[l->aux_ptr[q] + iq] * l->ao_sz[l->ao_ptr[k1] + i1] *
             l->ao_sz[l->ao_ptr[k2] + i2];
    }
    l->kp_sz[p] = acc; l->kp_off[p] = va; va += acc;
  }
  l->flat_V = va;
  /* rotation blocks: (block at conj(k), block at its irreducible k) */
  l->or_ptr = dup_i(L->orep_block_ptr, nk + 1);
  l->or_ir = dup_i(L->orep_irreps, 2 * (size_t)l->or_ptr[nk]);
  l->or_off = (int64_t *)malloc(sizeof(int64_t) * (l->or_ptr[nk] + 1));
  l->kor_off = (int64_t *)malloc(sizeof(int64_t) * nk);
  l->ar_ptr = dup_i(L->auxrep_block_ptr, nk + 1);
  l->ar_ir = dup_i(L->auxrep_irreps, 2 * (size_t)l->ar_ptr[nk]);
  l->ar_off = (int64_t *)malloc(sizeof(int64_t) * (l->ar_ptr[nk] + 1));
  l->kar_off = (int64_t *)malloc(sizeof(int64_t) * nk);
  int64_t oa = 0, aa = 0;
  for (int k = 0; k < nk; ++k) {
    int ck = l->conj_index[k];
    int kk = l->irre_list[l->irre_index[ck]];
    l->kor_off[k] = oa;
    int64_t acc = 0;
    for (int b = l->or_ptr[k]; b < l->or_ptr[k + 1]; ++b) {
      l->or_off[b] = acc;
      acc += (int64_t)l->ao_sz[l->ao_ptr[ck] + l->or_ir[2 * b]] *
             l->ao_sz[l->ao_ptr[kk] + l->or_ir[2 * b + 1]];
    }
    oa += acc;
    l->kar_off[k] = aa;
    acc = 0;
    for (int b = l->ar_ptr[k]; b < l->ar_ptr[k + 1]; ++b) {
      l->ar_off[b] = acc;
      acc += (int64_t)l->aux_sz[l->aux_ptr[ck] + l->ar_ir[2 * b]] *
             l->aux_sz[l->aux_ptr[kk] + l->ar_ir[2 * b + 1]];
    }
    aa += acc;
  }
  l->flat_orep = oa; l->flat_auxrep = aa;
  return l;
}

void gwo_layout_destroy(gwo_layout *l) {
  if (!l) return;
  void *ptrs[] = {l->irre_list, l->index, l->irre_index, l->conj_index, l->q_ind, l->q_ind2,
                  l->ao_ptr, l->ao_sz, l->ao_off, l->aux_ptr, l->aux_sz, l->aux_off,
                  l->kao_off, l->kao_sz, l->qaux_off, l->qaux_sz, l->kao_off_irre, l->qaux_off_irre,
                  l->kp_ptr, l->ti, l->t_off, l->kp_off, l->kp_sz, l->or_ptr, l->or_ir, l->or_off,
                  l->kor_off, l->ar_ptr, l->ar_ir, l->ar_off, l->kar_off};
  for (size_t i = 0; i < sizeof(ptrs) / sizeof(ptrs[0]); ++i) free(ptrs[i]);
  free(l);
}

int64_t gwo_flat_ao(const gwo_layout *l) { return l->flat_ao; }
int64_t gwo_flat_aux(const gwo_layout *l) { return l->flat_aux; }
int64_t gwo_flat_ao_full(const gwo_layout *l) { return l->flat_ao_full; }
int64_t gwo_flat_aux_full(const gwo_layout *l) { return l->flat_aux_full; }
int64_t gwo_flat_V(const gwo_layout *l) { return l->flat_V; }
int64_t gwo_flat_orep(const gwo_layout *l) { return l->flat_orep; }
int64_t gwo_flat_auxrep(const gwo_layout *l) { return l->flat_auxrep; }

/* y[0:n] += a * x[0:n] on interleaved (re, im) doubles: the inner loop of the
 * GEMMs below, written on real arithmetic so that it vectorises. */
static inline void zaxpy(int n, cplx a, const cplx *x, cplx *y) {
  const double ar = creal(a), ai = cimag(a);
  const double *xd = (const double *)x;
  double *yd = (double *)y;
  for (int j = 0; j < n; ++j) {
    const double xr = xd[2 * j], xi = xd[2 * j + 1];
    yd[2 * j] += ar * xr - ai * xi;
    yd[2 * j + 1] += ar * xi + ai * xr;
  }
}

/* C(m x n) += A(m x k) * B(k x n), all row-major (i-p-j order: contiguous rows). */
static void zgemm_nn_acc(int m, int n, int k, const cplx *A, int lda, const cplx *B, int ldb,
                         cplx *C, int ldc) {
  for (int i = 0; i < m; ++i) {
    cplx *c = C + (size_t)i * ldc;
    for (int p = 0; p < k; ++p) zaxpy(n, A[(size_t)i * lda + p], B + (size_t)p * ldb, c);
  }
}

/* C(m x n) = A(m x k) * B(k x n), all row-major, overwrite. */
static void zgemm_nn(int m, int n, int k, const cplx *A, int lda, const cplx *B, int ldb,
                     cplx *C, int ldc) {
  for (int i = 0; i < m; ++i) {
    cplx *c = C + (size_t)i * ldc;
    for (int j = 0; j < n; ++j) c[j] = 0;
  }
  zgemm_nn_acc(m, n, k, A, lda, B, ldb, C, ldc);
}

/* out = O * X * O^H for one (m x n) block O and (n x n) X, row-major. */
static void rotate_block(int m, int n, const cplx *O, const cplx *X, int ldx, cplx *out, int ldo,
                         cplx *tmp) {
  zgemm_nn(m, n, n, O, n, X, ldx, tmp, n);  /* tmp = O X  (m x n) */
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < m; ++j) {
      cplx acc = 0;
      for (int p = 0; p < n; ++p) acc += tmp[(size_t)i * n + p] * conj(O[(size_t)j * n + p]);
      out[(size_t)i * ldo + j] = acc;
    }
}

void gwo_rotate_G(const gwo_layout *l, int ns, int nts, const double *G_irr_d, const double *orep_d,
                  double *G_full_d) {
  const cplx *G_irr = (const cplx *)G_irr_d;
  const cplx *orep = (const cplx *)orep_d;
  cplx *G_full = (cplx *)G_full_d;
  int nk = l->nk;
#pragma omp parallel for schedule(dynamic) num_threads(gwo_get_threads())
  for (int k = 0; k < nk; ++k) {
    int ck = l->conj_index[k];
    int ick = l->irre_index[ck];
    int kk = l->irre_list[ick];
    int64_t ksz = l->kao_sz[k], iksz = l->kao_sz[kk];
    cplx *dst = G_full + l->kao_off[k] * ns * nts;
    cplx *tmp = (cplx *)malloc(sizeof(cplx) * 64 * 64 + sizeof(cplx) * ksz * 4 + 16);
    for (int t = 0; t < nts; ++t)
      for (int s = 0; s < ns; ++s) {
        /* source: host layout [t][s][flat_ao] (the reorder of cugw_routines_block.cu:106-118) */
        const cplx *src = G_irr + ((size_t)t * ns + s) * l->flat_ao + l->kao_off_irre[ick];
        cplx *d = dst + ((size_t)t * ns + s) * ksz;
        if (l->index[ck] == ck) {
          memcpy(d, src, sizeof(cplx) * iksz);
        } else {
          for (int b = l->or_ptr[ck]; b < l->or_ptr[ck + 1]; ++b) {
            int ia1 = l->or_ir[2 * b], ia2 = l->or_ir[2 * b + 1];
            int m = l->ao_sz[l->ao_ptr[ck] + ia1], n = l->ao_sz[l->ao_ptr[kk] + ia2];
            const cplx *O = orep + l->kor_off[ck] + l->or_off[b];
            rotate_block(m, n, O, src + l->ao_off[l->ao_ptr[kk] + ia2], n,
                         d + l->ao_off[l->ao_ptr[ck] + ia1], m, tmp);
          }
        }
        if (k != ck)
          for (int64_t i = 0; i < ksz; ++i) d[i] = conj(d[i]);
      }
    free(tmp);
  }
}

/* G_full slice of k at (t, s). */
static inline const cplx *gfull(const gwo_layout *l, const cplx *G, int ns, int nts, int k, int t, int s) {
  return G + l->kao_off[k] * ns * nts + ((size_t)t * ns + s) * l->kao_sz[k];
}

void gwo_p0(const gwo_layout *l, int ns, int nts, int nt_max, const double *G_full_d, const double *V_d,
            double *P0_d) {
  const cplx *G = (const cplx *)G_full_d;
  const cplx *V = (const cplx *)V_d;
  cplx *P0 = (cplx *)P0_d;
  int nk = l->nk, ink = l->ink;
  memset(P0, 0, sizeof(cplx) * (size_t)nts * l->flat_aux);
  double pref = -1.0 / nk * (ns == 1 ? 2.0 : 1.0);
  /* each (q, t) owns P0[q][t]: loops k1, s, V block inside (gw_block.cpp:19-79) */
#pragma omp parallel num_threads(gwo_get_threads())
  {
    size_t cap = 0;
    cplx *X1 = NULL, *X2 = NULL, *VT = NULL;
#pragma omp for collapse(2) schedule(dynamic)
    for (int iq_irr = 0; iq_irr < ink; ++iq_irr)
      for (int t = 0; t < nt_max; ++t) {
        int q = l->irre_list[iq_irr];
        int64_t qsz = l->qaux_sz[q];
        cplx *P = P0 + (size_t)nts * l->qaux_off_irre[iq_irr] + (size_t)t * qsz;
        for (int k1 = 0; k1 < nk; ++k1) {
          int k2 = mom_cons(l, k1, 0, q); /* k2 = k1 + q */
          int p = k1 * nk + k2;
          const cplx *Vp = V + l->kp_off[p];
          for (int s = 0; s < ns; ++s) {
            const cplx *Gm = gfull(l, G, ns, nts, k1, nts - 1 - t, s); /* G^{k1}(beta - t) */
            const cplx *G2 = gfull(l, G, ns, nts, k2, t, s);           /* G^{k2}(t) */
            for (int b = l->kp_ptr[p]; b < l->kp_ptr[p + 1]; ++b) {
              int iq = l->ti[3 * b], i1 = l->ti[3 * b + 1], i2 = l->ti[3 * b + 2];
              int qb = l->aux_sz[l->aux_ptr[q] + iq];
              int b1 = l->ao_sz[l->ao_ptr[k1] + i1], b2 = l->ao_sz[l->ao_ptr[k2] + i2];
              const cplx *Vb = Vp + l->t_off[b];
              const cplx *Gtp = Gm + l->ao_off[l->ao_ptr[k1] + i1];
              const cplx *Gmn = G2 + l->ao_off[l->ao_ptr[k2] + i2];
              size_t need = (size_t)qb * b1 * b2;
              if (need > cap) {
                free(X1); free(X2); free(VT);
                cap = need;
                X1 = (cplx *)malloc(sizeof(cplx) * cap);
                X2 = (cplx *)malloc(sizeof(cplx) * cap);
                VT = (cplx *)malloc(sizeof(cplx) * cap);
              }
              /* X1[t'][Q][m] = sum_p G^{k1}(beta-t)[t'][p] V[Q][p][m]   (gw_block.cpp:57-62) */
              for (int Q = 0; Q < qb; ++Q)
                zgemm_nn(b1, b2, b1, Gtp, b1, Vb + (size_t)Q * b1 * b2, b2, X1 + (size_t)Q * b2, qb * b2);
              /* X2[t'][m][P] = sum_n G^{k2}(t)[m][n] conj(V[P][t'][n])   (gw_block.cpp:67-69) */
              for (int P_ = 0; P_ < qb; ++P_)
                for (int tp = 0; tp < b1; ++tp)
                  for (int n = 0; n < b2; ++n)
                    VT[((size_t)tp * b2 + n) * qb + P_] = conj(Vb[((size_t)P_ * b1 + tp) * b2 + n]);
              for (int tp = 0; tp < b1; ++tp)
                zgemm_nn(b2, qb, b2, Gmn, b2, VT + (size_t)tp * b2 * qb, qb, X2 + (size_t)tp * b2 * qb, qb);
              /* P0[Q][P] += sum_{t',m} X1[t'][Q][m] X2[t'][m][P]   (gw_block.cpp:72-74) */
              cplx *Pb = P + l->aux_off[l->aux_ptr[q] + iq];
              for (int tp = 0; tp < b1; ++tp)
                zgemm_nn_acc(qb, qb, b2, X1 + (size_t)tp * qb * b2, b2, X2 + (size_t)tp * b2 * qb, qb, Pb, qb);
            }
          }
        }
        for (int64_t i = 0; i < qsz; ++i) P[i] *= pref;
      }
    free(X1); free(X2); free(VT);
  }
}

void gwo_mirror_P0(const gwo_layout *l, int nts, double *P0_d) {
  cplx *P0 = (cplx *)P0_d;
  for (int iq = 0; iq < l->ink; ++iq) {
    int64_t qsz = l->qaux_sz[l->irre_list[iq]];
    cplx *base = P0 + (size_t)nts * l->qaux_off_irre[iq];
    for (int t = 0; t < nts / 2; ++t)
      memcpy(base + (size_t)(nts - t - 1) * qsz, base + (size_t)t * qsz, sizeof(cplx) * qsz);
  }
}

/* Inverse of a Hermitian matrix by LDL^H with symmetric diagonal pivoting
 * (the factorisation Eigen::LDLT computes, used at cugw_solver_block.cpp:411-420),
 * then solve with the identity.  A is overwritten by A^-1. Returns 0 or -1. */
static int ldlt_inverse(int n, cplx *A, cplx *W, int *perm) {
  /* W holds the factor (L below the diagonal, D on it) */
  memcpy(W, A, sizeof(cplx) * n * n);
  for (int i = 0; i < n; ++i) perm[i] = i;
  for (int k = 0; k < n; ++k) {
    int p = k;
    double best = fabs(creal(W[k * n + k]));
    for (int i = k + 1; i < n; ++i) {
      double v = fabs(creal(W[i * n + i]));
      if (v > best) { best = v; p = i; }
    }
    if (p != k) {
      for (int j = 0; j < n; ++j) { cplx t = W[k * n + j]; W[k * n + j] = W[p * n + j]; W[p * n + j] = t; }
      for (int i = 0; i < n; ++i) { cplx t = W[i * n + k]; W[i * n + k] = W[i * n + p]; W[i * n + p] = t; }
      int t = perm[k]; perm[k] = perm[p]; perm[p] = t;
    }
    double d = creal(W[k * n + k]);
    if (d == 0.0) return -1;
    for (int i = k + 1; i < n; ++i) W[i * n + k] /= d;          /* L(i,k) */
    for (int i = k + 1; i < n; ++i)
      for (int j = k + 1; j <= i; ++j) {
        W[i * n + j] -= W[i * n + k] * d * conj(W[j * n + k]);
        W[j * n + i] = conj(W[i * n + j]);
      }
  }
  /* solve (P^T L D L^H P) X = I column by column */
  cplx *y = W + n * n;
  for (int c = 0; c < n; ++c) {
    for (int i = 0; i < n; ++i) y[i] = (perm[i] == c) ? 1.0 : 0.0;
    for (int i = 0; i < n; ++i)            /* L y = b */
      for (int j = 0; j < i; ++j) y[i] -= W[i * n + j] * y[j];
    for (int i = 0; i < n; ++i) y[i] /= creal(W[i * n + i]);
    for (int i = n - 1; i >= 0; --i)       /* L^H x = y */
      for (int j = i + 1; j < n; ++j) y[i] -= conj(W[j * n + i]) * y[j];
    for (int i = 0; i < n; ++i) A[perm[i] * n + c] = y[i];
  }
  return 0;
}

int gwo_p_tilde(const gwo_layout *l, int nts, int nw_b, const double *Tnt_BF_d, const double *Ttn_FB_d,
                double *P_d) {
  const cplx *Tnt = (const cplx *)Tnt_BF_d;
  const cplx *Ttn = (const cplx *)Ttn_FB_d;
  cplx *P = (cplx *)P_d;
  int ncheb = nts - 2;
  int fail = 0;
#pragma omp parallel for schedule(dynamic) num_threads(gwo_get_threads()) reduction(| : fail)
  for (int iq = 0; iq < l->ink; ++iq) {
    int q = l->irre_list[iq];
    int64_t qsz = l->qaux_sz[q];
    cplx *base = P + (size_t)nts * l->qaux_off_irre[iq];
    cplx *Pt = (cplx *)malloc(sizeof(cplx) * nts * qsz);
    cplx *Pw = (cplx *)calloc((size_t)nw_b * qsz, sizeof(cplx));
    for (int t = 0; t < nts / 2; ++t) { /* mirror (cugw_solver_block.cpp:395-398) */
      memcpy(Pt + (size_t)t * qsz, base + (size_t)t * qsz, sizeof(cplx) * qsz);
      memcpy(Pt + (size_t)(nts - t - 1) * qsz, base + (size_t)t * qsz, sizeof(cplx) * qsz);
    }
    /* P0(iOmega) = Tnt_BF * P0(tau_1..tau_ncheb)   (transformer_t.h:66-78) */
    zgemm_nn(nw_b, (int)qsz, ncheb, Tnt, ncheb, Pt + qsz, (int)qsz, Pw, (int)qsz);
    int maxb = 0;
    for (int b = l->aux_ptr[q]; b < l->aux_ptr[q + 1]; ++b) if (l->aux_sz[b] > maxb) maxb = l->aux_sz[b];
    cplx *A = (cplx *)malloc(sizeof(cplx) * maxb * maxb);
    cplx *W = (cplx *)malloc(sizeof(cplx) * (maxb * maxb + maxb));
    cplx *R = (cplx *)malloc(sizeof(cplx) * maxb * maxb);
    int *perm = (int *)malloc(sizeof(int) * maxb);
    for (int n = 0; n < nw_b; ++n)
      for (int b = l->aux_ptr[q]; b < l->aux_ptr[q + 1]; ++b) {
        int m = l->aux_sz[b];
        cplx *Pb = Pw + (size_t)n * qsz + l->aux_off[b];
        /* A = I - (P + P^H)/2 ; A^-1 ; (A^-1 + A^-H)/2 ; P <- A^-1 P  (cugw_solver_block.cpp:412-424) */
        for (int i = 0; i < m; ++i)
          for (int j = 0; j < m; ++j)
            A[i * m + j] = (i == j ? 1.0 : 0.0) - 0.5 * (Pb[i * m + j] + conj(Pb[j * m + i]));
        if (ldlt_inverse(m, A, W, perm)) fail = 1;
        for (int i = 0; i < m; ++i)
          for (int j = 0; j < m; ++j) R[i * m + j] = 0.5 * (A[i * m + j] + conj(A[j * m + i]));
        zgemm_nn(m, m, m, R, m, Pb, m, A, m);
        memcpy(Pb, A, sizeof(cplx) * m * m);
      }
    /* P(tau) = Ttn_FB * P(iOmega)   (transformer_t.h:87-99), all nts rows */
    zgemm_nn(nts, (int)qsz, nw_b, Ttn, nw_b, Pw, (int)qsz, Pt, (int)qsz);
    memcpy(base, Pt, sizeof(cplx) * nts * qsz);
    free(A); free(W); free(R); free(perm); free(Pt); free(Pw);
  }
  return fail ? -1 : 0;
}

void gwo_rotate_P(const gwo_layout *l, int nts, const double *P_irr_d, const double *auxrep_d,
                  double *P_full_d) {
  const cplx *P_irr = (const cplx *)P_irr_d;
  const cplx *A = (const cplx *)auxrep_d;
  cplx *P_full = (cplx *)P_full_d;
#pragma omp parallel for schedule(dynamic) num_threads(gwo_get_threads())
  for (int q = 0; q < l->nk; ++q) {
    int cq = l->conj_index[q];
    int q_ir = l->irre_index[q];               /* cugw_qkpt_block.cu:147 */
    int qq = l->irre_list[q_ir];
    int64_t qsz = l->qaux_sz[q], iqsz = l->qaux_sz[qq];
    cplx *tmp = (cplx *)malloc(sizeof(cplx) * (iqsz + 64) * 2);
    for (int t = 0; t < nts; ++t) {
      const cplx *src = P_irr + (size_t)nts * l->qaux_off_irre[q_ir] + (size_t)t * iqsz;
      cplx *d = P_full + (size_t)nts * l->qaux_off[q] + (size_t)t * qsz;
      if (l->index[cq] == cq) {
        memcpy(d, src, sizeof(cplx) * iqsz);
      } else {
        for (int b = l->ar_ptr[cq]; b < l->ar_ptr[cq + 1]; ++b) {
          int ia1 = l->ar_ir[2 * b], ia2 = l->ar_ir[2 * b + 1];
          int m = l->aux_sz[l->aux_ptr[cq] + ia1], n = l->aux_sz[l->aux_ptr[qq] + ia2];
          const cplx *O = A + l->kar_off[cq] + l->ar_off[b];
          rotate_block(m, n, O, src + l->aux_off[l->aux_ptr[qq] + ia2], n,
                       d + l->aux_off[l->aux_ptr[cq] + ia1], m, tmp);
        }
      }
      if (q != cq)
        for (int64_t i = 0; i < qsz; ++i) d[i] = conj(d[i]);
    }
    free(tmp);
  }
}

void gwo_sigma(const gwo_layout *l, int ns, int nts, int nt_max, const double *G_full_d,
               const double *P_full_d, const double *V_d, double *Sigma_d) {
  const cplx *G = (const cplx *)G_full_d;
  const cplx *Pf = (const cplx *)P_full_d;
  const cplx *V = (const cplx *)V_d;
  cplx *Sig = (cplx *)Sigma_d;
  int nk = l->nk, ink = l->ink;
  memset(Sig, 0, sizeof(cplx) * (size_t)nts * ns * l->flat_ao);
  /* each (k, t) owns Sigma[t][:][k]: loops q, s, V block inside (gw_block.cpp:97-155) */
#pragma omp parallel num_threads(gwo_get_threads())
  {
    size_t cap = 0;
    cplx *Y1 = NULL, *Y2 = NULL, *VT = NULL;
#pragma omp for collapse(2) schedule(dynamic)
    for (int ik = 0; ik < ink; ++ik)
      for (int t = 0; t < nt_max; ++t) {
        int k1 = l->irre_list[ik];
        for (int q = 0; q < nk; ++q) {
          int k2 = mom_cons(l, k1, q, 0); /* k2 = k1 - q */
          int p = k1 * nk + k2;
          const cplx *Vp = V + l->kp_off[p];
          const cplx *Pq = Pf + (size_t)nts * l->qaux_off[q] + (size_t)t * l->qaux_sz[q];
          for (int s = 0; s < ns; ++s) {
            const cplx *G2 = gfull(l, G, ns, nts, k2, t, s);
            cplx *S = Sig + ((size_t)t * ns + s) * l->flat_ao + l->kao_off_irre[ik];
            for (int b = l->kp_ptr[p]; b < l->kp_ptr[p + 1]; ++b) {
              int iq = l->ti[3 * b], i1 = l->ti[3 * b + 1], i2 = l->ti[3 * b + 2];
              int qb = l->aux_sz[l->aux_ptr[q] + iq];
              int b1 = l->ao_sz[l->ao_ptr[k1] + i1], b2 = l->ao_sz[l->ao_ptr[k2] + i2];
              const cplx *Vb = Vp + l->t_off[b];
              const cplx *Gmn = G2 + l->ao_off[l->ao_ptr[k2] + i2];
              const cplx *PQP = Pq + l->aux_off[l->aux_ptr[q] + iq];
              size_t need = (size_t)qb * b1 * b2;
              if (need > cap) {
                free(Y1); free(Y2); free(VT);
                cap = need;
                Y1 = (cplx *)malloc(sizeof(cplx) * cap);
                Y2 = (cplx *)malloc(sizeof(cplx) * cap);
                VT = (cplx *)malloc(sizeof(cplx) * cap);
              }
              /* Y1[Q,i][n] = sum_m V[Q,i][m] G^{k2}(t)[m][n]   (gw_block.cpp:134-136) */
              zgemm_nn(qb * b1, b2, b2, Vb, b2, Gmn, b2, Y1, b2);
              /* Y2[i,n][P] = sum_Q Y1[Q][i,n] P[Q][P]   (gw_block.cpp:139-141) */
              int K = b1 * b2;
              memset(Y2, 0, sizeof(cplx) * (size_t)K * qb);
              for (int Q = 0; Q < qb; ++Q)
                for (int in = 0; in < K; ++in) zaxpy(qb, Y1[(size_t)Q * K + in], PQP + (size_t)Q * qb, Y2 + (size_t)in * qb);
              /* Sigma[i][j] += sum_{n,P} Y2[i][n,P] conj(V[P][j][n])   (gw_block.cpp:146-150) */
              for (int P_ = 0; P_ < qb; ++P_)
                for (int j = 0; j < b1; ++j)
                  for (int n = 0; n < b2; ++n)
                    VT[((size_t)n * qb + P_) * b1 + j] = conj(Vb[((size_t)P_ * b1 + j) * b2 + n]);
              cplx *Sb = S + l->ao_off[l->ao_ptr[k1] + i1];
              zgemm_nn_acc(b1, b1, b2 * qb, Y2, b2 * qb, VT, b1, Sb, b1);
            }
          }
        }
        for (int s = 0; s < ns; ++s) {
          cplx *S = Sig + ((size_t)t * ns + s) * l->flat_ao + l->kao_off_irre[ik];
          for (int64_t i = 0; i < l->kao_sz[k1]; ++i) S[i] *= -1.0 / nk;
        }
      }
    free(Y1); free(Y2); free(VT);
  }
}

/* Inverse by Gauss-Jordan elimination with full pivoting (the pivoting
 * strategy of Eigen::FullPivLU used at sc_type_block.cpp:55).  Returns -1 on
 * an exactly singular matrix. */
static int fullpiv_inverse(int n, cplx *A, int *ipiv, int *indxr, int *indxc) {
  for (int j = 0; j < n; ++j) ipiv[j] = 0;
  for (int i = 0; i < n; ++i) {
    double big = -1.0;
    int irow = 0, icol = 0;
    for (int j = 0; j < n; ++j)
      if (ipiv[j] != 1)
        for (int k = 0; k < n; ++k)
          if (ipiv[k] == 0) {
            double v = cabs(A[j * n + k]);
            if (v > big) { big = v; irow = j; icol = k; }
          }
    ipiv[icol]++;
    if (irow != icol)
      for (int l = 0; l < n; ++l) { cplx t = A[irow * n + l]; A[irow * n + l] = A[icol * n + l]; A[icol * n + l] = t; }
    indxr[i] = irow; indxc[i] = icol;
    if (A[icol * n + icol] == 0) return -1;
    cplx pivinv = 1.0 / A[icol * n + icol];
    A[icol * n + icol] = 1.0;
    for (int l = 0; l < n; ++l) A[icol * n + l] *= pivinv;
    for (int ll = 0; ll < n; ++ll)
      if (ll != icol) {
        cplx dum = A[ll * n + icol];
        A[ll * n + icol] = 0;
        for (int l = 0; l < n; ++l) A[ll * n + l] -= A[icol * n + l] * dum;
      }
  }
  for (int l = n - 1; l >= 0; --l)
    if (indxr[l] != indxc[l])
      for (int k = 0; k < n; ++k) {
        cplx t = A[k * n + indxr[l]]; A[k * n + indxr[l]] = A[k * n + indxc[l]]; A[k * n + indxc[l]] = t;
      }
  return 0;
}

int gwo_dyson(const gwo_layout *l, int ns, int nts, int nw, double beta, double mu, const int64_t *wsample,
              const double *Tnt_d, const double *Ttn_d, const double *F_d, const double *S_d,
              const double *Sigma_d, double *G_d, const double *tct_first, const double *tct_last,
              double *leakage) {
  const cplx *Tnt = (const cplx *)Tnt_d, *Ttn = (const cplx *)Ttn_d;
  const cplx *F = (const cplx *)F_d, *Sv = (const cplx *)S_d, *Sig = (const cplx *)Sigma_d;
  cplx *G = (cplx *)G_d;
  int ncheb = nts - 2, ink = l->ink;
  int64_t fa = l->flat_ao;
  memset(G, 0, sizeof(cplx) * (size_t)nts * ns * fa);
  double c_last = 0.0, c_first = 0.0;
  int fail = 0;
#pragma omp parallel for schedule(dynamic) num_threads(gwo_get_threads()) reduction(max : c_last, c_first) reduction(| : fail)
  for (int isk = 0; isk < ns * ink; ++isk) {
    int s = isk / ink, ik = isk % ink; /* sc_type_block.cpp:25-27 */
    int k = l->irre_list[ik];
    int64_t ksz = l->kao_sz[k], koff = l->kao_off_irre[ik];
    cplx *St = (cplx *)malloc(sizeof(cplx) * nts * ksz);
    cplx *Sw = (cplx *)malloc(sizeof(cplx) * nw * ksz);
    cplx *Gt = (cplx *)malloc(sizeof(cplx) * nts * ksz);
    for (int t = 0; t < nts; ++t)
      memcpy(St + t * ksz, Sig + ((size_t)t * ns + s) * fa + koff, sizeof(cplx) * ksz);
    zgemm_nn(nw, (int)ksz, ncheb, Tnt, ncheb, St + ksz, (int)ksz, Sw, (int)ksz); /* tau_to_omega */
    int maxb = 0;
    for (int b = l->ao_ptr[k]; b < l->ao_ptr[k + 1]; ++b) if (l->ao_sz[b] > maxb) maxb = l->ao_sz[b];
    int *piv = (int *)malloc(sizeof(int) * 3 * (maxb + 1));
    for (int ic = 0; ic < nw; ++ic) {
      cplx muomega = I * ((2.0 * (double)wsample[ic] + 1.0) * M_PI / beta) + mu; /* transformer_t.h:51-53 */
      for (int b = l->ao_ptr[k]; b < l->ao_ptr[k + 1]; ++b) {
        int m = l->ao_sz[b];
        int64_t o = l->ao_off[b];
        cplx *Gb = Sw + (size_t)ic * ksz + o;
        const cplx *Sb = Sv + (size_t)s * fa + koff + o;
        const cplx *Fb = F + (size_t)s * fa + koff + o;
        for (int i = 0; i < m * m; ++i) Gb[i] = muomega * Sb[i] - Fb[i] - Gb[i];
        if (fullpiv_inverse(m, Gb, piv, piv + maxb + 1, piv + 2 * (maxb + 1))) fail = 1;
      }
    }
    free(piv);
    zgemm_nn(nts, (int)ksz, nw, Ttn, nw, Sw, (int)ksz, Gt, (int)ksz); /* omega_to_tau */
    for (int t = 0; t < nts; ++t)
      memcpy(G + ((size_t)t * ns + s) * fa + koff, Gt + t * ksz, sizeof(cplx) * ksz);
    if (tct_first && tct_last) { /* tau_to_chebyshev_c leakage check (sc_type_block.cpp:66-71) */
      for (int64_t i = 0; i < ksz; ++i) {
        cplx a = 0, b = 0;
        for (int t = 0; t < ncheb; ++t) {
          a += tct_last[t] * Gt[(size_t)(t + 1) * ksz + i];
          b += tct_first[t] * Gt[(size_t)(t + 1) * ksz + i];
        }
        if (cabs(a) > c_last) c_last = cabs(a);
        if (cabs(b) > c_first) c_first = cabs(b);
      }
    }
    free(St); free(Sw); free(Gt);
  }
  if (leakage) *leakage = (c_first > 0) ? c_last / c_first : 0.0;
  return fail ? -1 : 0;
}
