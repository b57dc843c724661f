// FP64 kernels of the GW engine: block rotations, the P0 and Sigma
// contractions, the tau <-> omega transforms and the batched block inverses.
//
// GB300's FP64 rate is a small fraction of its tensor rate, so these kernels
// are FP64-pipe bound: they keep the reference's three-GEMM contraction
// order (no redundant flops), keep every SM busy with owner-computes tiles
// (one CTA owns an output block for a tau range and sums all its (k, q, s)
// contributions, so no atomics and bitwise run-to-run reproducibility), and
// stage the per-contribution intermediates in shared memory.
#include "common.h"
#include "kernels.h"

namespace gwgb {

__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// c + a * b
__device__ __forceinline__ double2 cfma(double2 a, double2 b, double2 c) {
  c.x = fma(a.x, b.x, c.x);
  c.x = fma(-a.y, b.y, c.x);
  c.y = fma(a.x, b.y, c.y);
  c.y = fma(a.y, b.x, c.y);
  return c;
}
// c + conj(a) * b
__device__ __forceinline__ double2 cfma_conja(double2 a, double2 b, double2 c) {
  c.x = fma(a.x, b.x, c.x);
  c.x = fma(a.y, b.y, c.x);
  c.y = fma(a.x, b.y, c.y);
  c.y = fma(-a.y, b.x, c.y);
  return c;
}
__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }

// ---------------------------------------------------------------------------
// P0 contraction (restates gw_block.cpp:52-75 / cugw_qkpt_block.cu:195-267):
//   X1[t,m][Q] = sum_p G^{k1}(beta - tau)[t][p] V[Q][p][m]
//   X2[P][t,m] = sum_n conj(V[P][t][n]) G^{k2}(tau)[m][n]
//   P0(tau)[Q][P] += sum_{t,m} X1[t,m][Q] X2[P][t,m]
// The t (row of the k1 block) range is processed in chunks so the
// intermediates of any block size fit in shared memory.  A tile sums one
// slice of the block's contributions into its own partial block; the slices
// are added in a fixed order by reduce_slices_kernel.
// ---------------------------------------------------------------------------
template <int MAXO>
__global__ void __launch_bounds__(256, 2) p0_fp64_kernel(const P0Tile *__restrict__ tiles,
                                                         const P0Contrib *__restrict__ contribs,
                                                         const double2 *__restrict__ V,
                                                         const double2 *__restrict__ G,
                                                         double2 *__restrict__ Part, int ns, int nts,
                                                         int smem_cap) {
  extern __shared__ double2 sm[];
  const P0Tile tile = tiles[blockIdx.x];
  const int qb = tile.qb, nt = tile.nt;
  const int nout = nt * qb * qb;
  double2 acc[MAXO];
#pragma unroll
  for (int i = 0; i < MAXO; ++i) acc[i] = make_double2(0.0, 0.0);

  for (int c = tile.c0; c < tile.c1; ++c) {
    const P0Contrib cb = contribs[c];
    const int b1 = cb.b1, b2 = cb.b2;
    const double2 *Vb = V + cb.v;
    int TT = smem_cap / (2 * qb * b2 * nt);
    TT = TT < b1 ? TT : b1;
    for (int s = 0; s < ns; ++s) {
      for (int r0 = 0; r0 < b1; r0 += TT) {
        const int tn = (b1 - r0) < TT ? (b1 - r0) : TT;
        const int K = tn * b2;
        double2 *X1 = sm;
        double2 *X2 = sm + (size_t)nt * qb * K;
        __syncthreads();
        for (int e = threadIdx.x; e < nt * qb * K; e += blockDim.x) {
          const int it = e / (qb * K);
          const int rem = e - it * qb * K;
          const int Q = rem / K, k = rem - Q * K;
          const int tt = k / b2, m = k - tt * b2;
          const int tau = tile.t0 + it;
          const double2 *Gm = G + cb.ga + ((size_t)(nts - 1 - tau) * ns + s) * cb.sa + (size_t)(r0 + tt) * b1;
          const double2 *Vq = Vb + (size_t)Q * b1 * b2 + m;
          double2 a = make_double2(0.0, 0.0);
          for (int p = 0; p < b1; ++p) a = cfma(Gm[p], Vq[(size_t)p * b2], a);
          X1[(size_t)(it * qb + Q) * K + k] = a;
        }
        for (int e = threadIdx.x; e < nt * qb * K; e += blockDim.x) {
          const int it = e / (qb * K);
          const int rem = e - it * qb * K;
          const int P = rem / K, k = rem - P * K;
          const int tt = k / b2, m = k - tt * b2;
          const int tau = tile.t0 + it;
          const double2 *G2 = G + cb.gb + ((size_t)tau * ns + s) * cb.sb + (size_t)m * b2;
          const double2 *Vr = Vb + ((size_t)P * b1 + r0 + tt) * b2;
          double2 a = make_double2(0.0, 0.0);
          for (int n = 0; n < b2; ++n) a = cfma_conja(Vr[n], G2[n], a);
          X2[(size_t)(it * qb + P) * K + k] = a;
        }
        __syncthreads();
#pragma unroll
        for (int i = 0; i < MAXO; ++i) {
          const int o = threadIdx.x + i * blockDim.x;
          if (o < nout) {
            const int it = o / (qb * qb);
            const int rem = o - it * qb * qb;
            const int Q = rem / qb, P = rem - Q * qb;
            const double2 *x1 = X1 + (size_t)(it * qb + Q) * K;
            const double2 *x2 = X2 + (size_t)(it * qb + P) * K;
            double2 a = acc[i];
            for (int k = 0; k < K; ++k) a = cfma(x1[k], x2[k], a);
            acc[i] = a;
          }
        }
      }
    }
  }
#pragma unroll
  for (int i = 0; i < MAXO; ++i) {
    const int o = threadIdx.x + i * blockDim.x;
    if (o < nout) Part[tile.part + o] = acc[i];
  }
}

// ---------------------------------------------------------------------------
// Sigma contraction (restates gw_block.cpp:128-151 / cugw_qkpt_block.cu:343-412):
//   Y1[Q][i][n] = sum_m V[Q][i][m] G^{k2}(tau)[m][n]
//   Y2[i][n][P] = sum_Q Y1[Q][i][n] P(tau)[Q][P]
//   Sigma(tau)[i][j] += sum_{n,P} Y2[i][n][P] conj(V[P][j][n])
// The n range is processed in chunks so the intermediates fit in shared memory.
// Like P0, a tile writes the partial sum of one slice of the contributions.
// ---------------------------------------------------------------------------
template <int MAXO>
__global__ void __launch_bounds__(256, 2) sigma_fp64_kernel(const SigTile *__restrict__ tiles,
                                                            const SigContrib *__restrict__ contribs,
                                                            const double2 *__restrict__ V,
                                                            const double2 *__restrict__ G,
                                                            const double2 *__restrict__ P,
                                                            double2 *__restrict__ Part, int ns, int smem_cap) {
  extern __shared__ double2 sm[];
  const SigTile tile = tiles[blockIdx.x];
  const int b1 = tile.b1, nt = tile.nt, s = tile.s;
  const int nout = nt * b1 * b1;
  double2 acc[MAXO];
#pragma unroll
  for (int i = 0; i < MAXO; ++i) acc[i] = make_double2(0.0, 0.0);

  for (int c = tile.c0; c < tile.c1; ++c) {
    const SigContrib cb = contribs[c];
    const int qb = cb.qb, b2 = cb.b2;
    const double2 *Vb = V + cb.v;
    int NT = smem_cap / (2 * qb * b1 * nt);
    NT = NT < b2 ? NT : b2;
    for (int n0 = 0; n0 < b2; n0 += NT) {
      const int nn_n = (b2 - n0) < NT ? (b2 - n0) : NT;
      double2 *Y1 = sm;                                  // [nt][qb][b1][nn]
      double2 *Y2 = sm + (size_t)nt * qb * b1 * nn_n;    // [nt][b1][nn][qb]
      __syncthreads();
      for (int e = threadIdx.x; e < nt * qb * b1 * nn_n; e += blockDim.x) {
        const int it = e / (qb * b1 * nn_n);
        int rem = e - it * qb * b1 * nn_n;
        const int Q = rem / (b1 * nn_n);
        rem -= Q * b1 * nn_n;
        const int i = rem / nn_n, nn = rem - i * nn_n;
        const int tau = tile.t0 + it;
        const double2 *G2 = G + cb.gb + ((size_t)tau * ns + s) * cb.sb + n0 + nn;
        const double2 *Vr = Vb + ((size_t)Q * b1 + i) * b2;
        double2 a = make_double2(0.0, 0.0);
        for (int m = 0; m < b2; ++m) a = cfma(Vr[m], G2[(size_t)m * b2], a);
        Y1[e] = a;
      }
      __syncthreads();
      for (int e = threadIdx.x; e < nt * b1 * nn_n * qb; e += blockDim.x) {
        const int it = e / (b1 * nn_n * qb);
        int rem = e - it * b1 * nn_n * qb;
        const int i = rem / (nn_n * qb);
        rem -= i * nn_n * qb;
        const int nn = rem / qb, Pi = rem - nn * qb;
        const int tau = tile.t0 + it;
        const double2 *Pt = P + cb.pq + (size_t)tau * cb.pstride + Pi;
        const double2 *y1 = Y1 + ((size_t)it * qb * b1 + i) * nn_n + nn;
        double2 a = make_double2(0.0, 0.0);
        if (cb.pconj)  // P~(q) of a time-reversal partner: conj(P~(q'))
          for (int Q = 0; Q < qb; ++Q) a = cfma(y1[(size_t)Q * b1 * nn_n], cconj(Pt[(size_t)Q * qb]), a);
        else
          for (int Q = 0; Q < qb; ++Q) a = cfma(y1[(size_t)Q * b1 * nn_n], Pt[(size_t)Q * qb], a);
        Y2[e] = a;
      }
      __syncthreads();
#pragma unroll
      for (int ii = 0; ii < MAXO; ++ii) {
        const int o = threadIdx.x + ii * blockDim.x;
        if (o < nout) {
          const int it = o / (b1 * b1);
          const int rem = o - it * b1 * b1;
          const int i = rem / b1, j = rem - i * b1;
          const double2 *y2 = Y2 + ((size_t)it * b1 + i) * nn_n * qb;
          double2 a = acc[ii];
          for (int nn = 0; nn < nn_n; ++nn) {
            const double2 *vc = Vb + (size_t)j * b2 + n0 + nn;
            for (int Pi = 0; Pi < qb; ++Pi)
              a = cfma(y2[nn * qb + Pi], cconj(vc[(size_t)Pi * b1 * b2]), a);
          }
          acc[ii] = a;
        }
      }
    }
  }
#pragma unroll
  for (int ii = 0; ii < MAXO; ++ii) {
    const int o = threadIdx.x + ii * blockDim.x;
    if (o < nout) Part[tile.part + o] = acc[ii];
  }
}

// Fixed-order sum of the slices (deterministic), scaled, into P0 or Sigma.
__global__ void reduce_slices_kernel(const RedTask *__restrict__ tasks, const double2 *__restrict__ part,
                                     double2 *__restrict__ out, int nts, double scale, int mirror) {
  const RedTask tk = tasks[blockIdx.x];
  const int n = tk.nt * tk.elems;
  for (int o = blockIdx.y * blockDim.x + threadIdx.x; o < n; o += gridDim.y * blockDim.x) {
    double2 a = part[tk.part + o];
    for (int sl = 1; sl < tk.nslice; ++sl) a = cadd(a, part[tk.part + (int64_t)sl * n + o]);
    const int it = o / tk.elems, e = o - it * tk.elems;
    const int tau = tk.t0 + it;
    const double2 v = cscale(a, scale);
    out[tk.out + (int64_t)tau * tk.ostride + e] = v;
    if (mirror) out[tk.out + (int64_t)(nts - 1 - tau) * tk.ostride + e] = v;
  }
}

// ---------------------------------------------------------------------------
// Pre-rotated V of the Sigma contributions: Vt[Q'][x] = sum_Q op(O[Q][Q']) V[Q][x]
// (op = conj for a time-reversal partner; o < 0: a copy), once per V / rep
// upload.  One CTA per contribution block.
// ---------------------------------------------------------------------------
__global__ void vrot_kernel(const VrTask *__restrict__ tasks, const double2 *__restrict__ V,
                            const double2 *__restrict__ O, double2 *__restrict__ Vt) {
  const VrTask t = tasks[blockIdx.x];
  const int qb = t.qb, n = t.b1b2;
  const double2 *v = V + t.v;
  double2 *out = Vt + t.vt;
  if (t.o < 0) {
    for (int e = threadIdx.x; e < qb * n; e += blockDim.x) out[e] = v[e];
    return;
  }
  const double2 *o = O + t.o;
  for (int e = threadIdx.x; e < qb * n; e += blockDim.x) {
    const int Qp = e / n, x = e - Qp * n;
    double2 a = make_double2(0.0, 0.0);
    if (t.conj)
      for (int Q = 0; Q < qb; ++Q) a = cfma(cconj(o[Q * qb + Qp]), v[(size_t)Q * n + x], a);
    else
      for (int Q = 0; Q < qb; ++Q) a = cfma(o[Q * qb + Qp], v[(size_t)Q * n + x], a);
    out[e] = a;
  }
}

// ---------------------------------------------------------------------------
// Block rotation dst = O src O^H (+conj), or slice copy (+conj); restates
// cugw_routines_block.cu:134-186 (G) and cugw_qkpt_block.cu:288-340 (P).
// grid = (tasks, batch)
// ---------------------------------------------------------------------------
__global__ void rotate_kernel(const RotTask *__restrict__ tasks, const double2 *__restrict__ src,
                              const double2 *__restrict__ O, double2 *__restrict__ dst) {
  extern __shared__ double2 sm[];
  const RotTask t = tasks[blockIdx.x];
  const double2 *s = src + t.src + (size_t)blockIdx.y * t.sstride;
  double2 *d = dst + t.dst + (size_t)blockIdx.y * t.dstride;
  if (!t.rotate) {
    for (int i = threadIdx.x; i < t.m; i += blockDim.x) d[i] = t.conj ? cconj(s[i]) : s[i];
    return;
  }
  const int m = t.m, n = t.n;
  double2 *Os = sm;               // m x n
  double2 *X = sm + m * n;        // n x n
  double2 *T = X + n * n;         // m x n
  const double2 *Og = O + t.o;
  for (int i = threadIdx.x; i < m * n; i += blockDim.x) Os[i] = Og[i];
  for (int i = threadIdx.x; i < n * n; i += blockDim.x) X[i] = s[i];
  __syncthreads();
  for (int e = threadIdx.x; e < m * n; e += blockDim.x) {
    const int i = e / n, j = e - i * n;
    double2 a = make_double2(0.0, 0.0);
    for (int p = 0; p < n; ++p) a = cfma(Os[i * n + p], X[p * n + j], a);
    T[e] = a;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
    const int i = e / m, j = e - i * m;
    double2 a = make_double2(0.0, 0.0);
    for (int p = 0; p < n; ++p) a = cfma(T[i * n + p], cconj(Os[j * n + p]), a);
    d[e] = t.conj ? cconj(a) : a;
  }
}

// P0(beta - t) = P0(t) (cugw_solver_block.cpp:441-456); grid over q, threads over elements.
__global__ void mirror_kernel(double2 *__restrict__ P, const int64_t *__restrict__ qoff,
                              const int32_t *__restrict__ qsz, int nts) {
  const int q = blockIdx.x;
  const int64_t base = (int64_t)nts * qoff[q];
  const int sz = qsz[q];
  const int half = nts / 2;
  for (int64_t e = (int64_t)blockIdx.y * blockDim.x + threadIdx.x; e < (int64_t)half * sz;
       e += (int64_t)gridDim.y * blockDim.x) {
    const int t = (int)(e / sz);
    const int i = (int)(e - (int64_t)t * sz);
    P[base + (int64_t)(nts - 1 - t) * sz + i] = P[base + (int64_t)t * sz + i];
  }
}

// Zero rows t >= nts/2 of every P0 slice (state left by solve_P0).
__global__ void zero_upper_kernel(double2 *__restrict__ P, const int64_t *__restrict__ qoff,
                                  const int32_t *__restrict__ qsz, int nts) {
  const int q = blockIdx.x;
  const int64_t base = (int64_t)nts * qoff[q];
  const int sz = qsz[q];
  const int half = nts / 2;
  for (int64_t e = (int64_t)blockIdx.y * blockDim.x + threadIdx.x; e < (int64_t)(nts - half) * sz;
       e += (int64_t)gridDim.y * blockDim.x)
    P[base + (int64_t)half * sz + e] = make_double2(0.0, 0.0);
}

// ---------------------------------------------------------------------------
// tau <-> omega transform (transformer_t.h:66-99, 226-308):
//   Y[slab][r][c] = sum_i T[r][i] X[slab][row0 + i][c],  r < nout, i < nin.
// One CTA = 32 columns x 8R output rows (R per warp, rows r0 + warp*R + j),
// grid = (slab, column tile, row tile).  The T rows of the tile are staged
// through shared memory in 32-wide chunks of i.  Warps whose rows all lie
// beyond nout skip the arithmetic (the FP64 pipe is the bound).
// ---------------------------------------------------------------------------
constexpr int TR_MAXOUT = 160;  // nout limit of the engine's grids
template <int R>
__global__ void __launch_bounds__(256) transform_kernel(const TSlab *__restrict__ slabs,
                                                        const double2 *__restrict__ T, int nout,
                                                        int nin, int row0,
                                                        const double2 *__restrict__ X,
                                                        double2 *__restrict__ Y) {
  __shared__ double2 Ts[8 * R][33];
  const TSlab sl = slabs[blockIdx.x];
  const int cl = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int c = blockIdx.y * 32 + cl;
  const int r0 = blockIdx.z * 8 * R;
  const int nr = min(8 * R, nout - r0);
  const bool active = c < sl.ncols && w * R < nr;
  double2 acc[R];
#pragma unroll
  for (int j = 0; j < R; ++j) acc[j] = make_double2(0.0, 0.0);
  const double2 *x = X + sl.x + (int64_t)row0 * sl.ldx + c;
  for (int i0 = 0; i0 < nin; i0 += 32) {
    const int ni = (nin - i0) < 32 ? (nin - i0) : 32;
    __syncthreads();
    for (int e = threadIdx.x; e < nr * 32; e += 256) {
      const int r = e >> 5, ii = e & 31;
      Ts[r][ii] = (ii < ni) ? T[(int64_t)(r0 + r) * nin + i0 + ii] : make_double2(0.0, 0.0);
    }
    __syncthreads();
    if (active) {
      for (int ii = 0; ii < ni; ++ii) {
        const double2 xv = x[(int64_t)(i0 + ii) * sl.ldx];
#pragma unroll
        for (int j = 0; j < R; ++j) acc[j] = cfma(Ts[w * R + j][ii], xv, acc[j]);
      }
    }
  }
  if (active) {
#pragma unroll
    for (int j = 0; j < R; ++j) {
      const int rl = w * R + j;
      if (rl < nr) Y[sl.y + (int64_t)(r0 + rl) * sl.ldy + c] = acc[j];
    }
  }
}

// ---------------------------------------------------------------------------
// Batched block inverses by Gauss-Jordan elimination with full pivoting (the
// pivoting strategy of Eigen::FullPivLU, sc_type_block.cpp:55), one warp per
// matrix.  An exactly singular block sets *bad and leaves its output
// untouched.
//   mode 0 (W~ solve, cugw_solver_block.cpp:412-424):
//     A = I - (P + P^H)/2 ; A^-1 ; R = (A^-1 + A^-H)/2 ; P <- R P
//   mode 1 (Dyson, sc_type_block.cpp:48-57):
//     A = (i w_n + mu) S - F - Sigma(i w_n) ; G = A^-1   (in place)
// ---------------------------------------------------------------------------
// nm = largest block of the launch; every warp of the CTA owns 2*nm^2 complex
// and 3*nm ints of shared memory.
__global__ void inverse_kernel(const InvTask *__restrict__ tasks, int ntasks, double2 *__restrict__ W,
                               const double2 *__restrict__ S, const double2 *__restrict__ F,
                               const int64_t *__restrict__ wsample, double beta, double mu, int mode,
                               int *__restrict__ bad, int nm, const double *__restrict__ mu_ptr,
                               double2 *__restrict__ Wout, const int *__restrict__ skip) {
  if (skip && *skip) return;  // the mu search has converged (uniform over the grid)
  const int WPB = blockDim.x >> 5;
  extern __shared__ double2 smem_inv[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double2 *A = smem_inv + (size_t)warp * 2 * nm * nm;
  double2 *B = A + nm * nm;
  int *ipiv = reinterpret_cast<int *>(smem_inv + (size_t)WPB * 2 * nm * nm) + warp * 3 * nm;
  int *indxr = ipiv + nm;
  int *indxc = indxr + nm;
  const int ti = blockIdx.x * WPB + warp;
  if (ti >= ntasks) return;
  const InvTask tk = tasks[ti];
  const int n = tk.n;
  double2 *g = W + tk.a;
  if (mode == 0) {
    for (int e = lane; e < n * n; e += 32) B[e] = g[e];
    __syncwarp();
    for (int e = lane; e < n * n; e += 32) {
      const int i = e / n, j = e - i * n;
      const double2 pij = B[e], pji = B[j * n + i];
      A[e] = make_double2((i == j ? 1.0 : 0.0) - 0.5 * (pij.x + pji.x), -0.5 * (pij.y - pji.y));
    }
  } else {
    if (mu_ptr) mu = *mu_ptr;
    const double wn = (2.0 * (double)wsample[tk.w] + 1.0) * 3.14159265358979323846 / beta;
    for (int e = lane; e < n * n; e += 32) {
      const double2 sv = S[tk.s + e], fv = F[tk.f + e], sg = g[e];
      // (mu + i wn) * S - F - Sigma
      A[e] = make_double2(mu * sv.x - wn * sv.y - fv.x - sg.x, mu * sv.y + wn * sv.x - fv.y - sg.y);
    }
  }
  for (int j = lane; j < n; j += 32) ipiv[j] = 0;
  __syncwarp();
  int singular = 0;
  for (int it = 0; it < n; ++it) {
    // pivot: largest |A[j][k]| over unused rows j and columns k, first in row-major order on ties
    double best = -1.0;
    int bidx = 0x7fffffff;
    for (int e = lane; e < n * n; e += 32) {
      const int j = e / n, k = e - j * n;
      if (ipiv[j] == 1 || ipiv[k] != 0) continue;
      const double2 v = A[e];
      const double av = v.x * v.x + v.y * v.y;
      if (av > best || (av == best && e < bidx)) { best = av; bidx = e; }
    }
    for (int off = 16; off > 0; off >>= 1) {
      const double ob = __shfl_down_sync(0xffffffffu, best, off);
      const int oi = __shfl_down_sync(0xffffffffu, bidx, off);
      if (ob > best || (ob == best && oi < bidx)) { best = ob; bidx = oi; }
    }
    best = __shfl_sync(0xffffffffu, best, 0);
    bidx = __shfl_sync(0xffffffffu, bidx, 0);
    if (!(best > 0.0)) { singular = 1; break; }
    const int irow = bidx / n, icol = bidx - irow * n;
    __syncwarp();
    if (lane == 0) { ipiv[icol] += 1; indxr[it] = irow; indxc[it] = icol; }
    if (irow != icol)
      for (int l = lane; l < n; l += 32) {
        const double2 t = A[irow * n + l];
        A[irow * n + l] = A[icol * n + l];
        A[icol * n + l] = t;
      }
    __syncwarp();
    const double2 pv = A[icol * n + icol];
    const double den = pv.x * pv.x + pv.y * pv.y;
    const double2 pinv = make_double2(pv.x / den, -pv.y / den);
    __syncwarp();
    for (int l = lane; l < n; l += 32) {
      const double2 v = (l == icol) ? make_double2(1.0, 0.0) : A[icol * n + l];
      A[icol * n + l] = cmul(v, pinv);
    }
    __syncwarp();
    for (int ll = lane; ll < n; ll += 32) {
      if (ll == icol) continue;
      const double2 f = A[ll * n + icol];
      A[ll * n + icol] = make_double2(0.0, 0.0);
      for (int l = 0; l < n; ++l) {
        const double2 r = A[icol * n + l];
        A[ll * n + l] = make_double2(A[ll * n + l].x - (r.x * f.x - r.y * f.y),
                                     A[ll * n + l].y - (r.x * f.y + r.y * f.x));
      }
    }
    __syncwarp();
  }
  if (singular) {
    if (lane == 0) atomicExch(bad, 1);
    return;
  }
  // undo the column permutation in reverse order
  for (int l = n - 1; l >= 0; --l) {
    const int r = indxr[l], c = indxc[l];
    if (r != c)
      for (int k = lane; k < n; k += 32) {
        const double2 t = A[k * n + r];
        A[k * n + r] = A[k * n + c];
        A[k * n + c] = t;
      }
    __syncwarp();
  }
  if (mode == 1) {
    double2 *o = Wout ? Wout + tk.a : g;
    for (int e = lane; e < n * n; e += 32) o[e] = A[e];
    return;
  }
  // R = (A^-1 + A^-H)/2, each unordered pair by one lane
  for (int e = lane; e < n * n; e += 32) {
    const int i = e / n, j = e - i * n;
    if (j < i) continue;
    const double2 aij = A[e], aji = A[j * n + i];
    const double2 r = make_double2(0.5 * (aij.x + aji.x), 0.5 * (aij.y - aji.y));
    A[e] = r;
    A[j * n + i] = cconj(r);
  }
  __syncwarp();
  for (int e = lane; e < n * n; e += 32) {
    const int i = e / n, j = e - i * n;
    double2 a = make_double2(0.0, 0.0);
    for (int l = 0; l < n; ++l) a = cfma(A[i * n + l], B[l * n + j], a);
    g[e] = a;
  }
}

// Same Gauss-Jordan inverse with one CTA per block (blocks larger than 16):
// the pivot search, the row scaling and the elimination run over all n^2
// elements with the same per-element arithmetic and the same pivot order as
// inverse_kernel.  Shared: A [n^2] | B [n^2] | fcol [n] (complex) | 3n ints.
constexpr int INV_CTA_THREADS = 128;
__host__ __device__ constexpr int inv_cta_smem_bytes(int n) { return (2 * n * n + n) * 16 + 3 * n * 4 + 64; }

__global__ void __launch_bounds__(INV_CTA_THREADS) inverse_cta_kernel(
    const InvTask *__restrict__ tasks, double2 *__restrict__ W, const double2 *__restrict__ S,
    const double2 *__restrict__ F, const int64_t *__restrict__ wsample, double beta, double mu, int mode,
    int *__restrict__ bad, int nm, const double *__restrict__ mu_ptr, double2 *__restrict__ Wout,
    const int *__restrict__ skip) {
  if (skip && *skip) return;
  constexpr int NT = INV_CTA_THREADS, NW = NT / 32;
  extern __shared__ double2 smem_inv[];
  __shared__ double red_best[NW];
  __shared__ int red_idx[NW];
  __shared__ int piv[3];  // irow, icol, singular
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const InvTask tk = tasks[blockIdx.x];
  const int n = tk.n;
  double2 *A = smem_inv;
  double2 *B = A + nm * nm;
  double2 *fcol = B + nm * nm;
  int *ipiv = reinterpret_cast<int *>(fcol + nm);
  int *indxr = ipiv + nm;
  int *indxc = indxr + nm;
  double2 *g = W + tk.a;
  if (mode == 0) {
    for (int e = tid; e < n * n; e += NT) B[e] = g[e];
    __syncthreads();
    for (int e = tid; e < n * n; e += NT) {
      const int i = e / n, j = e - i * n;
      const double2 pij = B[e], pji = B[j * n + i];
      A[e] = make_double2((i == j ? 1.0 : 0.0) - 0.5 * (pij.x + pji.x), -0.5 * (pij.y - pji.y));
    }
  } else {
    if (mu_ptr) mu = *mu_ptr;
    const double wn = (2.0 * (double)wsample[tk.w] + 1.0) * 3.14159265358979323846 / beta;
    for (int e = tid; e < n * n; e += NT) {
      const double2 sv = S[tk.s + e], fv = F[tk.f + e], sg = g[e];
      A[e] = make_double2(mu * sv.x - wn * sv.y - fv.x - sg.x, mu * sv.y + wn * sv.x - fv.y - sg.y);
    }
  }
  for (int j = tid; j < n; j += NT) ipiv[j] = 0;
  __syncthreads();
  for (int it = 0; it < n; ++it) {
    double best = -1.0;
    int bidx = 0x7fffffff;
    for (int e = tid; e < n * n; e += NT) {
      const int j = e / n, k = e - j * n;
      if (ipiv[j] == 1 || ipiv[k] != 0) continue;
      const double2 v = A[e];
      const double av = v.x * v.x + v.y * v.y;
      if (av > best || (av == best && e < bidx)) { best = av; bidx = e; }
    }
    for (int off = 16; off > 0; off >>= 1) {
      const double ob = __shfl_down_sync(0xffffffffu, best, off);
      const int oi = __shfl_down_sync(0xffffffffu, bidx, off);
      if (ob > best || (ob == best && oi < bidx)) { best = ob; bidx = oi; }
    }
    if (lane == 0) { red_best[warp] = best; red_idx[warp] = bidx; }
    __syncthreads();
    if (tid == 0) {
      double b = red_best[0];
      int bi = red_idx[0];
      for (int w = 1; w < NW; ++w)
        if (red_best[w] > b || (red_best[w] == b && red_idx[w] < bi)) { b = red_best[w]; bi = red_idx[w]; }
      if (!(b > 0.0)) {
        piv[2] = 1;
      } else {
        const int irow = bi / n, icol = bi - irow * n;
        piv[0] = irow; piv[1] = icol; piv[2] = 0;
        ipiv[icol] += 1; indxr[it] = irow; indxc[it] = icol;
      }
    }
    __syncthreads();
    if (piv[2]) break;
    const int irow = piv[0], icol = piv[1];
    if (irow != icol) {
      for (int l = tid; l < n; l += NT) {
        const double2 t = A[irow * n + l];
        A[irow * n + l] = A[icol * n + l];
        A[icol * n + l] = t;
      }
      __syncthreads();
    }
    const double2 pv = A[icol * n + icol];
    const double den = pv.x * pv.x + pv.y * pv.y;
    const double2 pinv = make_double2(pv.x / den, -pv.y / den);
    __syncthreads();
    for (int l = tid; l < n; l += NT) {
      const double2 v = (l == icol) ? make_double2(1.0, 0.0) : A[icol * n + l];
      A[icol * n + l] = cmul(v, pinv);
    }
    for (int ll = tid; ll < n; ll += NT) fcol[ll] = A[ll * n + icol];
    __syncthreads();
    for (int e = tid; e < n * n; e += NT) {
      const int ll = e / n, l = e - ll * n;
      if (ll == icol) continue;
      const double2 f = fcol[ll];
      const double2 r = A[icol * n + l];
      const double2 a = (l == icol) ? make_double2(0.0, 0.0) : A[e];
      A[e] = make_double2(a.x - (r.x * f.x - r.y * f.y), a.y - (r.x * f.y + r.y * f.x));
    }
    __syncthreads();
  }
  if (piv[2]) {
    if (tid == 0) atomicExch(bad, 1);
    return;
  }
  for (int l = n - 1; l >= 0; --l) {
    const int r = indxr[l], c = indxc[l];
    if (r != c) {
      for (int k = tid; k < n; k += NT) {
        const double2 t = A[k * n + r];
        A[k * n + r] = A[k * n + c];
        A[k * n + c] = t;
      }
      __syncthreads();
    }
  }
  if (mode == 1) {
    double2 *o = Wout ? Wout + tk.a : g;
    for (int e = tid; e < n * n; e += NT) o[e] = A[e];
    return;
  }
  for (int e = tid; e < n * n; e += NT) {
    const int i = e / n, j = e - i * n;
    if (j < i) continue;
    const double2 aij = A[e], aji = A[j * n + i];
    const double2 r = make_double2(0.5 * (aij.x + aji.x), 0.5 * (aij.y - aji.y));
    A[e] = r;
    A[j * n + i] = cconj(r);
  }
  __syncthreads();
  for (int e = tid; e < n * n; e += NT) {
    const int i = e / n, j = e - i * n;
    double2 a = make_double2(0.0, 0.0);
    for (int l = 0; l < n; ++l) a = cfma(A[i * n + l], B[l * n + j], a);
    g[e] = a;
  }
}

// Leakage check of G (sc_type_block.cpp:66-71): max over elements of
// |sum_t tct[t] G(tau_{t+1})| for the first and last IR coefficient.
__global__ void leakage_kernel(const TSlab *__restrict__ slabs, const double2 *__restrict__ G,
                               const double *__restrict__ tct_first, const double *__restrict__ tct_last,
                               int ncheb, unsigned long long *__restrict__ out) {
  const TSlab sl = slabs[blockIdx.x];
  double mf = 0.0, ml = 0.0;
  for (int c = blockIdx.y * blockDim.x + threadIdx.x; c < sl.ncols; c += gridDim.y * blockDim.x) {
    double2 a = make_double2(0.0, 0.0), b = make_double2(0.0, 0.0);
    for (int t = 0; t < ncheb; ++t) {
      const double2 g = G[sl.y + (int64_t)(t + 1) * sl.ldy + c];
      a.x += tct_first[t] * g.x; a.y += tct_first[t] * g.y;
      b.x += tct_last[t] * g.x;  b.y += tct_last[t] * g.y;
    }
    mf = fmax(mf, sqrt(a.x * a.x + a.y * a.y));
    ml = fmax(ml, sqrt(b.x * b.x + b.y * b.y));
  }
  for (int off = 16; off > 0; off >>= 1) {
    mf = fmax(mf, __shfl_down_sync(0xffffffffu, mf, off));
    ml = fmax(ml, __shfl_down_sync(0xffffffffu, ml, off));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(out, (unsigned long long)__double_as_longlong(mf));
    atomicMax(out + 1, (unsigned long long)__double_as_longlong(ml));
  }
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
void launch_p0_fp64(const P0Tile *tiles, int ntiles, int maxo, const P0Contrib *contribs,
                    const double2 *V, const double2 *G, double2 *Part, int ns, int nts, int smem_bytes,
                    cudaStream_t st) {
  if (ntiles == 0) return;
  const int cap = smem_bytes / (int)sizeof(double2);
  if (maxo <= 8) {
    p0_fp64_kernel<8><<<ntiles, 256, smem_bytes, st>>>(tiles, contribs, V, G, Part, ns, nts, cap);
  } else {
    p0_fp64_kernel<16><<<ntiles, 256, smem_bytes, st>>>(tiles, contribs, V, G, Part, ns, nts, cap);
  }
  GWGB_CUDA(cudaGetLastError());
}

// Hartree term (HF on the block layout; the reference's HF solver is a stub,
// cuhf_solver_block.h:36-39).  One thread per aux index Q (c) or per element of
// an AO block (J); every sum runs over its items in list order (deterministic).
__global__ void hartree_c_kernel(const HcTask *__restrict__ tasks, const HcItem *__restrict__ items,
                                 const double2 *__restrict__ V, const double2 *__restrict__ G, int ns,
                                 double scale, double2 *__restrict__ c) {
  const HcTask t = tasks[blockIdx.x];
  for (int Q = threadIdx.x; Q < t.qb; Q += blockDim.x) {
    double2 acc = make_double2(0.0, 0.0);
    for (int it = t.i0; it < t.i1; ++it) {
      const HcItem x = items[it];
      const double2 *vq = V + x.v + (int64_t)Q * x.b * x.b;
      for (int s = 0; s < ns; ++s) {
        const double2 *r = G + x.g + (int64_t)s * x.gstride;
        for (int a = 0; a < x.b; ++a)
          for (int b = 0; b < x.b; ++b) acc = cfma(vq[a * x.b + b], r[b * x.b + a], acc);
      }
    }
    c[t.cout + Q] = make_double2(acc.x * scale, acc.y * scale);
  }
}

__global__ void hartree_j_kernel(const HjTask *__restrict__ tasks, const HjItem *__restrict__ items,
                                 const double2 *__restrict__ V, const double2 *__restrict__ c,
                                 double2 *__restrict__ J) {
  const HjTask t = tasks[blockIdx.x];
  const int bb = t.b * t.b;
  for (int e = threadIdx.x; e < bb; e += blockDim.x) {
    double2 acc = make_double2(0.0, 0.0);
    for (int it = t.i0; it < t.i1; ++it) {
      const HjItem x = items[it];
      for (int Q = 0; Q < x.qb; ++Q) acc = cfma(V[x.v + (int64_t)Q * bb + e], c[x.c + Q], acc);
    }
    J[t.out + e] = acc;
  }
}

void launch_hartree(const HcTask *ct, int nct, const HcItem *ci, const HjTask *jt, int njt, const HjItem *ji,
                    const double2 *V, const double2 *G, int ns, double scale, double2 *c, double2 *J,
                    cudaStream_t st) {
  if (nct > 0) {
    hartree_c_kernel<<<nct, 128, 0, st>>>(ct, ci, V, G, ns, scale, c);
    GWGB_CUDA(cudaGetLastError());
  }
  if (njt > 0) {
    hartree_j_kernel<<<njt, 128, 0, st>>>(jt, ji, V, c, J);
    GWGB_CUDA(cudaGetLastError());
  }
}

void launch_reduce_slices(const RedTask *tasks, int ntasks, const double2 *part, double2 *out, int nts,
                          double scale, int mirror, cudaStream_t st, int ny) {
  if (ntasks == 0) return;
  reduce_slices_kernel<<<dim3(ntasks, std::max(1, std::min(ny, 65535))), 256, 0, st>>>(tasks, part, out, nts, scale,
                                                                                       mirror);
  GWGB_CUDA(cudaGetLastError());
}

void launch_sigma_fp64(const SigTile *tiles, int ntiles, int maxo, const SigContrib *contribs,
                       const double2 *V, const double2 *G, const double2 *P, double2 *Part, int ns,
                       int smem_bytes, cudaStream_t st) {
  if (ntiles == 0) return;
  const int cap = smem_bytes / (int)sizeof(double2);
  if (maxo <= 8) {
    sigma_fp64_kernel<8><<<ntiles, 256, smem_bytes, st>>>(tiles, contribs, V, G, P, Part, ns, cap);
  } else {
    sigma_fp64_kernel<16><<<ntiles, 256, smem_bytes, st>>>(tiles, contribs, V, G, P, Part, ns, cap);
  }
  GWGB_CUDA(cudaGetLastError());
}

void launch_rotate(const RotTask *tasks, int ntasks, int nbatch, int smem_bytes, const double2 *src,
                   const double2 *O, double2 *dst, cudaStream_t st) {
  if (ntasks == 0 || nbatch == 0) return;
  rotate_kernel<<<dim3(ntasks, nbatch), 128, smem_bytes, st>>>(tasks, src, O, dst);
  GWGB_CUDA(cudaGetLastError());
}

void launch_vrot(const VrTask *tasks, int ntasks, const double2 *V, const double2 *O, double2 *Vt, cudaStream_t st) {
  if (ntasks == 0) return;
  vrot_kernel<<<ntasks, 256, 0, st>>>(tasks, V, O, Vt);
  GWGB_CUDA(cudaGetLastError());
}

void launch_mirror(double2 *P, const int64_t *qoff, const int32_t *qsz, int nq, int nts, cudaStream_t st) {
  mirror_kernel<<<dim3(nq, 8), 256, 0, st>>>(P, qoff, qsz, nts);
  GWGB_CUDA(cudaGetLastError());
}

void launch_zero_upper(double2 *P, const int64_t *qoff, const int32_t *qsz, int nq, int nts, cudaStream_t st) {
  zero_upper_kernel<<<dim3(nq, 8), 256, 0, st>>>(P, qoff, qsz, nts);
  GWGB_CUDA(cudaGetLastError());
}

void launch_transform(const TSlab *slabs, int nslabs, int max_cols, const double2 *T, int nout, int nin,
                      int row0, const double2 *X, double2 *Y, cudaStream_t st) {
  if (nslabs == 0 || nout == 0) return;
  GWGB_REQUIRE(nout <= TR_MAXOUT, GWGB_E_UNSUPPORTED, "transform output longer than 160 rows");
  const int ct = (max_cols + 31) / 32;
  // the largest rows-per-warp that still gives about two CTAs per SM
  auto ctas = [&](int R) { return (int64_t)nslabs * ct * ((nout + 8 * R - 1) / (8 * R)); };
  if (nout > 8 && ctas(4) >= 304) {
    transform_kernel<4><<<dim3(nslabs, ct, (nout + 31) / 32), 256, 0, st>>>(slabs, T, nout, nin, row0, X, Y);
  } else if (nout > 8 && ctas(2) >= 304) {
    transform_kernel<2><<<dim3(nslabs, ct, (nout + 15) / 16), 256, 0, st>>>(slabs, T, nout, nin, row0, X, Y);
  } else {
    transform_kernel<1><<<dim3(nslabs, ct, (nout + 7) / 8), 256, 0, st>>>(slabs, T, nout, nin, row0, X, Y);
  }
  GWGB_CUDA(cudaGetLastError());
}

void launch_inverse(const InvTask *tasks, int ntasks, int nmax, double2 *W, const double2 *S,
                    const double2 *F, const int64_t *wsample, double beta, double mu, int mode, int *bad,
                    cudaStream_t st, const double *mu_ptr, double2 *Wout, const int *skip) {
  if (ntasks == 0) return;
  if (nmax > 16) {  // one CTA per block
    inverse_cta_kernel<<<ntasks, INV_CTA_THREADS, inv_cta_smem_bytes(nmax), st>>>(
        tasks, W, S, F, wsample, beta, mu, mode, bad, nmax, mu_ptr, Wout, skip);
  } else {          // one warp per block
    const int w = inv_warps_per_block(nmax);
    inverse_kernel<<<(ntasks + w - 1) / w, 32 * w, inv_smem_bytes(nmax), st>>>(
        tasks, ntasks, W, S, F, wsample, beta, mu, mode, bad, nmax, mu_ptr, Wout, skip);
  }
  GWGB_CUDA(cudaGetLastError());
}

void launch_leakage(const TSlab *slabs, int nslabs, const double2 *G, const double *tf, const double *tl,
                    int ncheb, unsigned long long *out, cudaStream_t st) {
  if (nslabs == 0) return;
  leakage_kernel<<<dim3(nslabs, 4), 256, 0, st>>>(slabs, G, tf, tl, ncheb, out);
  GWGB_CUDA(cudaGetLastError());
}

void set_fp64_kernel_attributes(int smem_bytes) {
  GWGB_CUDA(cudaFuncSetAttribute(p0_fp64_kernel<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes));
  GWGB_CUDA(cudaFuncSetAttribute(p0_fp64_kernel<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes));
  GWGB_CUDA(cudaFuncSetAttribute(sigma_fp64_kernel<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes));
  GWGB_CUDA(cudaFuncSetAttribute(sigma_fp64_kernel<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes));
  GWGB_CUDA(cudaFuncSetAttribute(rotate_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, rotate_smem_bytes(MAX_BLOCK)));
  set_inverse_kernel_attributes();
}

void set_inverse_kernel_attributes() {
  GWGB_CUDA(cudaFuncSetAttribute(inverse_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, inv_smem_bytes(MAX_BLOCK)));
  GWGB_CUDA(cudaFuncSetAttribute(inverse_cta_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 inv_cta_smem_bytes(MAX_BLOCK)));
}

}  // namespace gwgb
