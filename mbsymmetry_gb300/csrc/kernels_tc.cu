// Mixed-precision Sigma contraction on tcgen05.
//
// The reference evaluates, per (k1, q, block, tau), Y1 = V G, Y2 = Y1^T P,
// Sigma += Y2 V^H (gw_block.cpp:128-151).  Here the same sum is associated as
//   W_c(tau)[Q][(j,n)] = sum_P P(tau)[Q][P] conj(V_c[P][j][n])            (1)
//   U_c(tau)[Q][j][m]  = sum_n W_c(tau)[Q][(j,n)] G^{k2}(tau)[m][n]          (2)
//   Sigma(tau)[i][j]  += sum_{Q,m} V_c[Q][i][m] U_c(tau)[Q][j][m]           (3)
// which has the same flop count; (1) carries the q_b^2 term and, because its
// right operand conj(V_c) does not depend on tau, all tau points and all
// contributions c that share the aux block (q, iq) form ONE GEMM:
//   rows (tau, Q) x columns (c, j, n), K = P.
// (1) runs here as a tcgen05 kind::tf32 GEMM (3-pass split hi*hi + hi*lo +
// lo*hi, FP32 accumulation in TMEM) writing W to HBM in FP32; (2) and (3) run
// in a per-(owner, tau) kernel in FP32 with FP64 accumulation across
// contributions.
#include "common.h"
#include "kernels.h"
#include "kernels_tc.h"
#include "tc_common.cuh"

namespace gwgb {

namespace {

__device__ __forceinline__ void split_store(float *hi, float *lo, uint32_t off, float x) {
  const uint32_t h = tc::to_tf32(x);
  const uint32_t l = tc::to_tf32(x - __uint_as_float(h));
  *reinterpret_cast<uint32_t *>(reinterpret_cast<unsigned char *>(hi) + off) = h;
  *reinterpret_cast<uint32_t *>(reinterpret_cast<unsigned char *>(lo) + off) = l;
}

}  // namespace

// ---------------------------------------------------------------------------
// (1): one CTA = one 128-row tile (tau, Q) x one column pack of contributions.
// Shared memory: A_hi | A_lo (128 x KP) | B_hi | B_lo (NP x KP), KP = pad8(2 qb),
// NP = pad16(2 * ncol).  Accumulator: TMEM, 128 lanes x NP columns.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) sigma_w_tc_kernel(const SwTile *__restrict__ tiles,
                                                         const SwCol *__restrict__ cols,
                                                         const double2 *__restrict__ V,
                                                         const double2 *__restrict__ P, float2 *__restrict__ W,
                                                         int *__restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ uint32_t tmem_slot;
  __shared__ __align__(8) uint64_t mbar;
  const SwTile tl = tiles[blockIdx.x];
  const int qb = tl.qb;
  const int KP = tl.kp, NP = tl.np;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  float *Ahi = reinterpret_cast<float *>(smem_raw);
  float *Alo = Ahi + 128 * KP;
  float *Bhi = Alo + 128 * KP;
  float *Blo = Bhi + NP * KP;
  uint32_t ncols_alloc = 32;
  while ((int)ncols_alloc < NP) ncols_alloc <<= 1;
  if (warp == 0) tc::tmem_alloc(&tmem_slot, ncols_alloc);
  if (tid == 0) tc::mbar_init(&mbar, 1);

  // A: rows (tau, Q) of P(tau), K = (P, re/im)
  const int rows = tl.nt * qb;
  for (int e = tid; e < 128 * KP; e += blockDim.x) {
    const int r = e / KP, k = e - r * KP;
    const int kc = k >> 1;
    float x = 0.f;
    if (r < rows && kc < qb) {
      const int it = r / qb, Q = r - it * qb;
      const double2 v = __ldg(P + tl.pa + (int64_t)(tl.t0 + it) * tl.pstride + (int64_t)Q * qb + kc);
      x = (float)((k & 1) ? v.y : v.x);
    }
    split_store(Ahi, Alo, tc::kmajor_offset(r, k, KP), x);
  }
  // B: rows (col, d) of the real embedding of conj(V_c[P][j][n]), K = (P, c)
  for (int e = tid; e < NP * KP; e += blockDim.x) {
    const int n = e / KP, k = e - n * KP;
    const int col = n >> 1, d = n & 1, kc = k >> 1, cpart = k & 1;
    float x = 0.f;
    if (col < tl.ncol && kc < qb) {
      int ci = tl.c0;
      while (ci + 1 < tl.c1 && cols[ci + 1].col0 <= col) ++ci;
      const SwCol cc = cols[ci];
      const int lc = col - cc.col0 + cc.l0;
      const int jj = lc / cc.b2, nn = lc - jj * cc.b2;
      const double2 v = __ldg(V + cc.v + ((int64_t)kc * cc.b1 + jj) * cc.b2 + nn);
      // [[Br, Bi], [-Bi, Br]] with B = conj(v): Br = v.x, Bi = -v.y
      x = (float)(d == 0 ? (cpart == 0 ? v.x : v.y) : (cpart == 0 ? -v.y : v.x));
    }
    split_store(Bhi, Blo, tc::kmajor_offset(n, k, KP), x);
  }
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_slot;
  if (tid == 0) {
    const uint32_t idesc = tc::idesc_tf32(128, NP);
    const uint32_t sboA = (uint32_t)(KP / 4) * 128, sboB = sboA;
    const uint32_t a_hi = tc::smem_u32(Ahi), a_lo = tc::smem_u32(Alo);
    const uint32_t b_hi = tc::smem_u32(Bhi), b_lo = tc::smem_u32(Blo);
    for (int s = 0; s < KP / 8; ++s) {
      const uint32_t off = (uint32_t)s * 256;
      tc::mma_tf32(tmem, tc::make_desc(a_lo + off, 128, sboA), tc::make_desc(b_hi + off, 128, sboB), idesc, s > 0);
      tc::mma_tf32(tmem, tc::make_desc(a_hi + off, 128, sboA), tc::make_desc(b_lo + off, 128, sboB), idesc, 1);
      tc::mma_tf32(tmem, tc::make_desc(a_hi + off, 128, sboA), tc::make_desc(b_hi + off, 128, sboB), idesc, 1);
    }
    tc::commit(&mbar);
  }
  bool ok = tc::mbar_wait(&mbar, 0);
  if (!ok && lane == 0) atomicExch(err, 1);
  ok = __syncthreads_and(ok);
  tc::fence_after_sync();
  if (ok) {
    // drain: lane r of warp w holds row 32w + lane
    const int r = warp * 32 + lane;
    const bool live = r < rows;
    const int it = live ? r / qb : 0, Q = live ? r - (r / qb) * qb : 0;
    const int tau = tl.t0 + it;
    for (int c0 = 0; c0 < NP; c0 += 8) {
      float v[8];
      tc::tmem_ld8(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
      if (live) {
#pragma unroll
        for (int j = 0; j < 8; j += 2) {
          const int col = (c0 + j) >> 1;
          if (col < tl.ncol) {
            int ci = tl.c0;
            while (ci + 1 < tl.c1 && cols[ci + 1].col0 <= col) ++ci;
            const SwCol cc = cols[ci];
            const int lc = col - cc.col0 + cc.l0;
            const int jj = lc / cc.b2, nn = lc - jj * cc.b2;
            W[cc.w + (((int64_t)tau * qb + Q) * cc.b1 + jj) * cc.b2 + nn] = make_float2(v[j], v[j + 1]);
          }
        }
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, ncols_alloc);
}

// ---------------------------------------------------------------------------
// (2) + (3): one CTA per (k_irr, AO block, spin, tau); FP32 per contribution,
// FP64 across.  Shared: acc64 [b1^2] double2 | acc32 [b1^2] float2 |
// G2 [b2^2] | V [QC][b1][b2] | W [QC][b1][b2] | U [QC][b1][b2] (float2).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) sigma_uv_kernel(const SigTile *__restrict__ tiles,
                                                       const SigContrib *__restrict__ contribs,
                                                       const int64_t *__restrict__ woff,
                                                       const double2 *__restrict__ V,
                                                       const double2 *__restrict__ G, const float2 *__restrict__ W,
                                                       double2 *__restrict__ Sig, int ns, double scale,
                                                       int smem_bytes) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  const SigTile tile = tiles[blockIdx.x];
  const int b1 = tile.b1, s = tile.s, tau = tile.t0;
  double2 *acc64 = reinterpret_cast<double2 *>(smem_raw);
  float2 *acc32 = reinterpret_cast<float2 *>(acc64 + b1 * b1);
  float2 *G2s = acc32 + b1 * b1;
  for (int e = threadIdx.x; e < b1 * b1; e += blockDim.x) acc64[e] = make_double2(0.0, 0.0);
  for (int c = tile.c0; c < tile.c1; ++c) {
    const SigContrib cb = contribs[c];
    const int qb = cb.qb, b2 = cb.b2;
    const int blk = b1 * b2;
    float2 *Vs = G2s + b2 * b2;
    const int per_q = 3 * blk;
    const int avail = (smem_bytes - (int)((char *)Vs - (char *)smem_raw)) / 8;
    int QC = avail / per_q;
    QC = QC < qb ? QC : qb;
    float2 *Ws = Vs + QC * blk;
    float2 *Us = Ws + QC * blk;
    const double2 *Vb = V + cb.v;
    const double2 *G2 = G + cb.gb + ((int64_t)tau * ns + s) * cb.sb;
    const float2 *Wt = W + woff[c] + (int64_t)tau * qb * blk;
    __syncthreads();
    for (int e = threadIdx.x; e < b2 * b2; e += blockDim.x) {
      const double2 g = __ldg(G2 + e);
      G2s[e] = make_float2((float)g.x, (float)g.y);
    }
    for (int e = threadIdx.x; e < b1 * b1; e += blockDim.x) acc32[e] = make_float2(0.f, 0.f);
    for (int q0 = 0; q0 < qb; q0 += QC) {
      const int qn = (qb - q0) < QC ? (qb - q0) : QC;
      __syncthreads();
      for (int e = threadIdx.x; e < qn * blk; e += blockDim.x) {
        const double2 v = __ldg(Vb + (int64_t)q0 * blk + e);
        Vs[e] = make_float2((float)v.x, (float)v.y);
        Ws[e] = Wt[(int64_t)q0 * blk + e];
      }
      __syncthreads();
      // U[Q][j][m] = sum_n W[Q][j][n] G2[m][n]
      for (int e = threadIdx.x; e < qn * blk; e += blockDim.x) {
        const int Qj = e / b2, m = e - Qj * b2;
        const float2 *w = Ws + Qj * b2;
        const float2 *g = G2s + m * b2;
        float ur = 0.f, ui = 0.f;
        for (int n = 0; n < b2; ++n) {
          ur = fmaf(w[n].x, g[n].x, ur);
          ur = fmaf(-w[n].y, g[n].y, ur);
          ui = fmaf(w[n].x, g[n].y, ui);
          ui = fmaf(w[n].y, g[n].x, ui);
        }
        Us[e] = make_float2(ur, ui);
      }
      __syncthreads();
      // acc32[i][j] += sum_{Q,m} V[Q][i][m] U[Q][j][m]
      for (int o = threadIdx.x; o < b1 * b1; o += blockDim.x) {
        const int i = o / b1, j = o - i * b1;
        float ar = 0.f, ai = 0.f;
        for (int Q = 0; Q < qn; ++Q) {
          const float2 *vv = Vs + Q * blk + i * b2;
          const float2 *uu = Us + Q * blk + j * b2;
          for (int m = 0; m < b2; ++m) {
            ar = fmaf(vv[m].x, uu[m].x, ar);
            ar = fmaf(-vv[m].y, uu[m].y, ar);
            ai = fmaf(vv[m].x, uu[m].y, ai);
            ai = fmaf(vv[m].y, uu[m].x, ai);
          }
        }
        acc32[o].x += ar;
        acc32[o].y += ai;
      }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < b1 * b1; e += blockDim.x) {
      acc64[e].x += (double)acc32[e].x;
      acc64[e].y += (double)acc32[e].y;
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < b1 * b1; e += blockDim.x)
    Sig[tile.sig + (int64_t)tau * tile.sstride + e] = make_double2(acc64[e].x * scale, acc64[e].y * scale);
}

void launch_sigma_tc(const SwTile *wtiles, int nwtiles, int wsmem, const SwCol *wcols, const SigTile *tiles1,
                     int ntiles1, const SigContrib *contribs, const int64_t *woff, const double2 *V,
                     const double2 *G, const double2 *P, float2 *W, double2 *Sig, int ns, double scale,
                     int uv_smem, int *err, cudaStream_t st) {
  if (nwtiles > 0) {
    sigma_w_tc_kernel<<<nwtiles, 128, wsmem, st>>>(wtiles, wcols, V, P, W, err);
    GWGB_CUDA(cudaGetLastError());
  }
  if (ntiles1 > 0) {
    sigma_uv_kernel<<<ntiles1, 128, uv_smem, st>>>(tiles1, contribs, woff, V, G, W, Sig, ns, scale, uv_smem);
    GWGB_CUDA(cudaGetLastError());
  }
}

void set_tc_kernel_attributes(int smem_bytes) {
  GWGB_CUDA(cudaFuncSetAttribute(sigma_w_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes));
  GWGB_CUDA(cudaFuncSetAttribute(sigma_uv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes));
}

}  // namespace gwgb

// ===========================================================================
// Mixed-precision P0 on tcgen05.  The reference's chain (gw_block.cpp:52-75)
// is associated as
//   X2_c(tau)[P][t][m]  = sum_n conj(V_c[P][t][n]) G^{k2}(tau)[m][n]
//   Z_c(tau)[P][(p,m)]  = sum_t G^{k1}(beta - tau)[t][p] X2_c(tau)[P][t][m]
//   P0(tau)[Q][P]      += sum_{(p,m)} V_c[Q][p][m] Z_c(tau)[P][(p,m)]
// (same flop count).  The last line carries the q_b^2 term; with rows
// (tau, P) and K running over every (contribution, spin) of the aux block it
// is one GEMM per block whose right operand V_c does not depend on tau.
// ===========================================================================
namespace gwgb {

// Z stage, FP32: one CTA per (contribution, spin), all tau < nts/2.
// Shared: G2 [b2^2] | Gm [b1^2] | V [PC][b1][b2] | X2 [PC][b1][b2]  (float2)
__global__ void __launch_bounds__(128) p0_z_kernel(const PzTask *__restrict__ tasks, const double2 *__restrict__ V,
                                                   const double2 *__restrict__ G, float2 *__restrict__ Z, int ns,
                                                   int nts, int smem_bytes) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  const PzTask tk = tasks[blockIdx.x];
  const int b1 = tk.b1, b2 = tk.b2, qb = tk.qb, blk = b1 * b2;
  float2 *G2s = reinterpret_cast<float2 *>(smem_raw);
  float2 *Gms = G2s + b2 * b2;
  float2 *Vs = Gms + b1 * b1;
  const int avail = smem_bytes / 8 - b2 * b2 - b1 * b1;
  int PC = avail / (2 * blk);
  PC = PC < qb ? PC : qb;
  float2 *X2 = Vs + PC * blk;
  const double2 *Vb = V + tk.v;
  for (int p0 = 0; p0 < qb; p0 += PC) {
    const int pn = (qb - p0) < PC ? (qb - p0) : PC;
    __syncthreads();
    for (int e = threadIdx.x; e < pn * blk; e += blockDim.x) {
      const double2 v = __ldg(Vb + (int64_t)p0 * blk + e);
      Vs[e] = make_float2((float)v.x, (float)v.y);
    }
    for (int tau = 0; tau < nts / 2; ++tau) {
      const double2 *G2 = G + tk.gb + ((int64_t)tau * ns + tk.s) * tk.sb;
      const double2 *Gm = G + tk.ga + ((int64_t)(nts - 1 - tau) * ns + tk.s) * tk.sa;
      __syncthreads();
      for (int e = threadIdx.x; e < b2 * b2; e += blockDim.x) {
        const double2 g = __ldg(G2 + e);
        G2s[e] = make_float2((float)g.x, (float)g.y);
      }
      for (int e = threadIdx.x; e < b1 * b1; e += blockDim.x) {
        const double2 g = __ldg(Gm + e);
        Gms[e] = make_float2((float)g.x, (float)g.y);
      }
      __syncthreads();
      // X2[P][t][m] = sum_n conj(V[P][t][n]) G2[m][n]
      for (int e = threadIdx.x; e < pn * blk; e += blockDim.x) {
        const int Pt = e / b2, m = e - Pt * b2;
        const float2 *vr = Vs + Pt * b2;
        const float2 *g = G2s + m * b2;
        float xr = 0.f, xi = 0.f;
        for (int n = 0; n < b2; ++n) {
          xr = fmaf(vr[n].x, g[n].x, xr);
          xr = fmaf(vr[n].y, g[n].y, xr);
          xi = fmaf(vr[n].x, g[n].y, xi);
          xi = fmaf(-vr[n].y, g[n].x, xi);
        }
        X2[e] = make_float2(xr, xi);
      }
      __syncthreads();
      // Z[P][(p,m)] = sum_t Gm[t][p] X2[P][t][m]
      float2 *Zt = Z + tk.z + ((int64_t)tau * qb + p0) * blk;
      for (int e = threadIdx.x; e < pn * blk; e += blockDim.x) {
        const int P = e / blk, pm = e - P * blk;
        const int p = pm / b2, m = pm - p * b2;
        const float2 *x = X2 + P * blk + m;
        float zr = 0.f, zi = 0.f;
        for (int t = 0; t < b1; ++t) {
          const float2 g = Gms[t * b1 + p], xv = x[t * b2];
          zr = fmaf(g.x, xv.x, zr);
          zr = fmaf(-g.y, xv.y, zr);
          zi = fmaf(g.x, xv.y, zi);
          zi = fmaf(g.y, xv.x, zi);
        }
        Zt[e] = make_float2(zr, zi);
      }
    }
  }
}

// tcgen05 stage: D[(tau,P)][Q] = sum_chunks Z[(tau,P)][k] V[Q][k]; TMEM FP32,
// drained every `drain_every` chunks into the FP64 output (owned by this CTA).
// Shared: A_hi | A_lo (128 x 64) | B_hi | B_lo (NP x 64), 32-bit elements.
__global__ void __launch_bounds__(128) p0_tc_kernel(const PtTile *__restrict__ tiles,
                                                    const PtChunk *__restrict__ chunks,
                                                    const double2 *__restrict__ V, const float2 *__restrict__ Z,
                                                    double2 *__restrict__ P0, int nts, double pref, int mirror,
                                                    int drain_every, int *__restrict__ err) {
  constexpr int KP = 64;  // real K per chunk (32 complex)
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ uint32_t tmem_slot;
  __shared__ __align__(8) uint64_t mbar;
  const PtTile tl = tiles[blockIdx.x];
  const int qb = tl.qb, NP = tl.np;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  float *Ahi = reinterpret_cast<float *>(smem_raw);
  float *Alo = Ahi + 128 * KP;
  float *Bhi = Alo + 128 * KP;
  float *Blo = Bhi + NP * KP;
  uint32_t ncols_alloc = 32;
  while ((int)ncols_alloc < NP) ncols_alloc <<= 1;
  if (warp == 0) tc::tmem_alloc(&tmem_slot, ncols_alloc);
  if (tid == 0) tc::mbar_init(&mbar, 1);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_slot;
  const int rows = tl.nt * qb;
  const int r = warp * 32 + lane;
  const bool live = r < rows;
  const int it = live ? r / qb : 0, Prow = live ? r - (r / qb) * qb : 0;
  const int tau = tl.t0 + it;
  bool ok = true;
  int since_drain = 0, ndrain = 0;
  uint32_t phase = 0;
  for (int ch = tl.k0; ch < tl.k1 && ok; ++ch) {
    const PtChunk cc = chunks[ch];
    // stage A: Z rows (tau, P), K = (pm, re/im)
    for (int e = tid; e < 128 * KP; e += blockDim.x) {
      const int rr = e / KP, k = e - rr * KP;
      const int kc = k >> 1;
      float x = 0.f;
      if (rr < rows && kc < cc.kn) {
        const int i2 = rr / qb, P = rr - i2 * qb;
        const float2 z = Z[cc.z + ((int64_t)(tl.t0 + i2) * qb + P) * cc.b1b2 + cc.kc0 + kc];
        x = (k & 1) ? z.y : z.x;
      }
      split_store(Ahi, Alo, tc::kmajor_offset(rr, k, KP), x);
    }
    // stage B: rows (Q, d) of the real embedding of V^T (B[k][Q] = V[Q][k]): d=0 -> (Vr, -Vi), d=1 -> (Vi, Vr)
    for (int e = tid; e < NP * KP; e += blockDim.x) {
      const int n = e / KP, k = e - n * KP;
      const int Q = n >> 1, d = n & 1, kc = k >> 1, cp = k & 1;
      float x = 0.f;
      if (Q < qb && kc < cc.kn) {
        const double2 v = __ldg(V + cc.v + (int64_t)Q * cc.b1b2 + cc.kc0 + kc);
        x = (float)(d == 0 ? (cp == 0 ? v.x : -v.y) : (cp == 0 ? v.y : v.x));
      }
      split_store(Bhi, Blo, tc::kmajor_offset(n, k, KP), x);
    }
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (tid == 0) {
      const uint32_t idesc = tc::idesc_tf32(128, NP);
      const uint32_t sbo = (uint32_t)(KP / 4) * 128;
      const uint32_t a_hi = tc::smem_u32(Ahi), a_lo = tc::smem_u32(Alo);
      const uint32_t b_hi = tc::smem_u32(Bhi), b_lo = tc::smem_u32(Blo);
      const int ksteps = (2 * cc.kn + 7) / 8;
      for (int s = 0; s < ksteps; ++s) {
        const uint32_t off = (uint32_t)s * 256;
        tc::mma_tf32(tmem, tc::make_desc(a_lo + off, 128, sbo), tc::make_desc(b_hi + off, 128, sbo), idesc,
                     (since_drain > 0 || s > 0) ? 1u : 0u);
        tc::mma_tf32(tmem, tc::make_desc(a_hi + off, 128, sbo), tc::make_desc(b_lo + off, 128, sbo), idesc, 1);
        tc::mma_tf32(tmem, tc::make_desc(a_hi + off, 128, sbo), tc::make_desc(b_hi + off, 128, sbo), idesc, 1);
      }
      tc::commit(&mbar);
    }
    ok = tc::mbar_wait(&mbar, phase);
    phase ^= 1u;
    if (!ok && lane == 0) atomicExch(err, 1);
    ok = __syncthreads_and(ok);
    tc::fence_after_sync();
    ++since_drain;
    const bool last = (ch + 1 == tl.k1);
    if (ok && (since_drain >= drain_every || last)) {
      for (int c0 = 0; c0 < NP; c0 += 8) {
        float v[8];
        tc::tmem_ld8(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
        if (live) {
#pragma unroll
          for (int j = 0; j < 8; j += 2) {
            const int Q = (c0 + j) >> 1;
            if (Q < qb) {
              double2 *o = P0 + tl.pout + (int64_t)tau * tl.pstride + (int64_t)Q * qb + Prow;
              const double2 prev = ndrain ? *o : make_double2(0.0, 0.0);
              *o = make_double2(prev.x + (double)v[j], prev.y + (double)v[j + 1]);
            }
          }
        }
      }
      since_drain = 0;
      ++ndrain;
    }
    tc::fence_before_sync();
    __syncthreads();  // operands and TMEM are free for the next chunk
    tc::fence_after_sync();
  }
  // prefactor, tau mirror; blocks of a tile without contributions are zero
  if (live) {
    for (int Q = 0; Q < qb; ++Q) {
      double2 *o = P0 + tl.pout + (int64_t)tau * tl.pstride + (int64_t)Q * qb + Prow;
      const double2 v = (ndrain && ok) ? make_double2(o->x * pref, o->y * pref) : make_double2(0.0, 0.0);
      *o = v;
      if (mirror) P0[tl.pout + (int64_t)(nts - 1 - tau) * tl.pstride + (int64_t)Q * qb + Prow] = v;
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, ncols_alloc);
}

void launch_p0_tc(const PzTask *ztasks, int nz, int zsmem, const PtTile *ptiles, int npt, int psmem,
                  const PtChunk *chunks, const double2 *V, const double2 *G, float2 *Z, double2 *P0, int ns,
                  int nts, double pref, int mirror, int drain_every, int *err, cudaStream_t st) {
  if (nz > 0) {
    p0_z_kernel<<<nz, 128, zsmem, st>>>(ztasks, V, G, Z, ns, nts, zsmem);
    GWGB_CUDA(cudaGetLastError());
  }
  if (npt > 0) {
    p0_tc_kernel<<<npt, 128, psmem, st>>>(ptiles, chunks, V, Z, P0, nts, pref, mirror, drain_every, err);
    GWGB_CUDA(cudaGetLastError());
  }
}

void set_tc_p0_kernel_attributes(int smem_bytes) {
  GWGB_CUDA(cudaFuncSetAttribute(p0_z_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes));
  GWGB_CUDA(cudaFuncSetAttribute(p0_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes));
}

}  // namespace gwgb
