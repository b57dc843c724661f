// Mixed-precision P0 and Sigma contractions: TF32 tensor-core products with
// a 3-pass split (x = hi + lo, hi*hi + hi*lo + lo*hi; about 2^-21 relative
// error per product), FP32 accumulation inside one (k, q, s) contribution and
// FP64 accumulation across contributions.  V, G and P stay FP64 in HBM and
// are split into TF32 pairs when fragments are loaded; the W~ and Dyson
// solves and the transforms stay FP64.
//
// Complex products use the real embedding
//   [Cr Ci] = [Ar Ai] * [[Br, Bi], [-Bi, Br]]
// so an interleaved (re, im) row of A is an A fragment row as is, and the
// B fragment is built from B and i*B.
//
// One CTA owns one output block at one tau point and sums all contributions
// (owner computes: no atomics, reproducible).  Each contribution is the
// reference's three-GEMM chain (gw_block.cpp:52-75 and :128-151), each GEMM
// a warp-tiled mma.m16n8k8 TF32 loop with intermediates in shared memory.
#include "common.h"
#include "kernels.h"
#include "kernels_mixed.h"

namespace gwgb {

namespace {

__device__ __forceinline__ uint32_t to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ void split(float x, uint32_t &hi, uint32_t &lo) {
  hi = to_tf32(x);
  lo = to_tf32(x - __uint_as_float(hi));
}

__device__ __forceinline__ void mma_tf32(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ float2 ld64(const double2 *p) {
  const double2 v = __ldg(p);
  return make_float2((float)v.x, (float)v.y);
}

// Component c (0 = re, 1 = im) of the real-embedding row pair of B:
// row 2k holds (Br, Bi), row 2k+1 holds (-Bi, Br); d selects the column of the pair.
__device__ __forceinline__ float bcomp(float2 b, int c, int d) {
  return c == 0 ? (d == 0 ? b.x : b.y) : (d == 0 ? -b.y : b.x);
}

// C(M x N) += A(M x K) B(K x N) over complex values, results added into the
// FP32 shared matrix C (row stride ldc).  Each warp takes output tiles of 16
// rows x 4 complex columns, tiles tile = warp, warp + nwarps, ...  A and B
// are functors (r, k) -> float2 that return 0 outside the matrix.
template <bool ACCUM, class LA, class LB>
__device__ __forceinline__ void warp_cgemm(int M, int N, int K, const LA &A, const LB &B, float2 *C, int ldc) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int g = lane >> 2, t = lane & 3;
  const int tm = (M + 15) >> 4, tn = (N + 3) >> 2;
  for (int tile = warp; tile < tm * tn; tile += nwarps) {
    const int r0 = (tile / tn) << 4, n0 = (tile % tn) << 2;
    float c[4] = {0.f, 0.f, 0.f, 0.f};
    const int ra = r0 + g, rb = r0 + g + 8;
    const int nb = n0 + (g >> 1), d = g & 1, ca = t & 1;
    for (int k0 = 0; k0 < K; k0 += 4) {
      const int ka = k0 + (t >> 1), kb = ka + 2;
      const float2 x00 = A(ra, ka), x10 = A(rb, ka), x01 = A(ra, kb), x11 = A(rb, kb);
      const float2 y0 = B(ka, nb), y1 = B(kb, nb);
      uint32_t ah0, al0, ah1, al1, ah2, al2, ah3, al3, bh0, bl0, bh1, bl1;
      split(ca ? x00.y : x00.x, ah0, al0);
      split(ca ? x10.y : x10.x, ah1, al1);
      split(ca ? x01.y : x01.x, ah2, al2);
      split(ca ? x11.y : x11.x, ah3, al3);
      split(bcomp(y0, ca, d), bh0, bl0);
      split(bcomp(y1, ca, d), bh1, bl1);
      mma_tf32(c, al0, al1, al2, al3, bh0, bh1);
      mma_tf32(c, ah0, ah1, ah2, ah3, bl0, bl1);
      mma_tf32(c, ah0, ah1, ah2, ah3, bh0, bh1);
    }
    const int col = n0 + t;
    if (col < N) {
      if (ra < M) {
        float2 *p = C + (size_t)ra * ldc + col;
        *p = ACCUM ? make_float2(p->x + c[0], p->y + c[1]) : make_float2(c[0], c[1]);
      }
      if (rb < M) {
        float2 *p = C + (size_t)rb * ldc + col;
        *p = ACCUM ? make_float2(p->x + c[2], p->y + c[3]) : make_float2(c[2], c[3]);
      }
    }
  }
}

// ---- operand views -------------------------------------------------------
struct GlobalMat {  // element (r, k) of a FP64 complex matrix, optional conj
  const double2 *p;
  int rs, cs, M, K;
  bool conj;
  __device__ float2 operator()(int r, int k) const {
    if (r >= M || k >= K) return make_float2(0.f, 0.f);
    float2 v = ld64(p + (size_t)r * rs + (size_t)k * cs);
    return conj ? make_float2(v.x, -v.y) : v;
  }
};
struct SharedMat {  // element (r, k) of a FP32 complex shared matrix
  const float2 *p;
  int rs, cs, M, K;
  __device__ float2 operator()(int r, int k) const {
    if (r >= M || k >= K) return make_float2(0.f, 0.f);
    return p[(size_t)r * rs + (size_t)k * cs];
  }
};

// P0 stage 1 B operand: B(p, (m, Q)) = V[Q][p][m], column index c = m*qb + Q
struct P0S1B {
  const double2 *V;
  int b1, b2, qb, K, N;
  __device__ float2 operator()(int p, int c) const {
    if (p >= K || c >= N) return make_float2(0.f, 0.f);
    const int m = c / qb, Q = c - m * qb;
    return ld64(V + ((size_t)Q * b1 + p) * b2 + m);
  }
};
// P0 stage 2 A operand: A((P, tt), n) = conj(V[P][r0 + tt][n]), row r = P*TT + tt
struct P0S2A {
  const double2 *V;
  int b1, b2, TT, r0, M, K;
  __device__ float2 operator()(int r, int n) const {
    if (r >= M || n >= K) return make_float2(0.f, 0.f);
    const int P = r / TT, tt = r - P * TT;
    const float2 v = ld64(V + ((size_t)P * b1 + r0 + tt) * b2 + n);
    return make_float2(v.x, -v.y);
  }
};
// P0 stage 3: A(Q, kk) = X1[tt][(m, Q)], kk = tt*b2 + m;  B(kk, P) = X2[(P, tt)][m]
struct P0S3A {
  const float2 *X1;
  int b2, qb, M, K;
  __device__ float2 operator()(int Q, int kk) const {
    if (Q >= M || kk >= K) return make_float2(0.f, 0.f);
    const int tt = kk / b2, m = kk - tt * b2;
    return X1[((size_t)tt * b2 + m) * qb + Q];
  }
};
struct P0S3B {
  const float2 *X2;
  int b2, TT, K, N;
  __device__ float2 operator()(int kk, int P) const {
    if (kk >= K || P >= N) return make_float2(0.f, 0.f);
    const int tt = kk / b2, m = kk - tt * b2;
    return X2[((size_t)P * TT + tt) * b2 + m];
  }
};
// Sigma stage 3 B operand: B((nn, P), j) = conj(V[P][j][n0 + nn]), kk = nn*qb + P
struct SgS3B {
  const double2 *V;
  int b1, b2, qb, n0, K, N;
  __device__ float2 operator()(int kk, int j) const {
    if (kk >= K || j >= N) return make_float2(0.f, 0.f);
    const int nn = kk / qb, P = kk - nn * qb;
    const float2 v = ld64(V + ((size_t)P * b1 + j) * b2 + n0 + nn);
    return make_float2(v.x, -v.y);
  }
};

}  // namespace

// ---------------------------------------------------------------------------
// P0, one CTA per (q_irr, aux block, tau).  Shared memory:
//   acc64 [qb*qb] double2 | acc32 [qb*qb] float2 | X1 [TT*b2*qb] | X2 [qb*TT*b2]
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) p0_mixed_kernel(const P0Tile *__restrict__ tiles,
                                                       const P0Contrib *__restrict__ contribs,
                                                       const double2 *__restrict__ V,
                                                       const double2 *__restrict__ G, double2 *__restrict__ P0,
                                                       int ns, int nts, double pref, int mirror, int smem_bytes) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const P0Tile tile = tiles[blockIdx.x];
  const int qb = tile.qb, tau = tile.t0;
  double2 *acc64 = reinterpret_cast<double2 *>(smem_raw);
  float2 *acc32 = reinterpret_cast<float2 *>(acc64 + qb * qb);
  float2 *work = acc32 + qb * qb;
  const int cap = (smem_bytes - qb * qb * 24) / 8;  // float2 slots for X1 + X2
  for (int e = threadIdx.x; e < qb * qb; e += blockDim.x) acc64[e] = make_double2(0.0, 0.0);
  for (int c = tile.c0; c < tile.c1; ++c) {
    const P0Contrib cb = contribs[c];
    const int b1 = cb.b1, b2 = cb.b2;
    const double2 *Vb = V + cb.v;
    int TT = cap / (2 * b2 * qb);
    TT = TT < b1 ? TT : b1;
    for (int s = 0; s < ns; ++s) {
      const double2 *Gm = G + cb.ga + ((size_t)(nts - 1 - tau) * ns + s) * cb.sa;  // G^{k1}(beta - tau)
      const double2 *G2 = G + cb.gb + ((size_t)tau * ns + s) * cb.sb;             // G^{k2}(tau)
      __syncthreads();
      for (int e = threadIdx.x; e < qb * qb; e += blockDim.x) acc32[e] = make_float2(0.f, 0.f);
      for (int r0 = 0; r0 < b1; r0 += TT) {
        const int tn = (b1 - r0) < TT ? (b1 - r0) : TT;
        float2 *X1 = work;                      // [tn][b2*qb]
        float2 *X2 = work + tn * b2 * qb;       // [qb*tn][b2]
        __syncthreads();
        // X1[tt][(m,Q)] = sum_p Gm[r0+tt][p] V[Q][p][m]
        warp_cgemm<false>(tn, b2 * qb, b1, GlobalMat{Gm + (size_t)r0 * b1, b1, 1, tn, b1, false},
                          P0S1B{Vb, b1, b2, qb, b1, b2 * qb}, X1, b2 * qb);
        // X2[(P,tt)][m] = sum_n conj(V[P][r0+tt][n]) G2[m][n]
        warp_cgemm<false>(qb * tn, b2, b2, P0S2A{Vb, b1, b2, tn, r0, qb * tn, b2},
                          GlobalMat{G2, 1, b2, b2, b2, false}, X2, b2);
        __syncthreads();
        // acc32[Q][P] += sum_{tt,m} X1[tt][(m,Q)] X2[(P,tt)][m]
        warp_cgemm<true>(qb, qb, tn * b2, P0S3A{X1, b2, qb, qb, tn * b2}, P0S3B{X2, b2, tn, tn * b2, qb}, acc32,
                         qb);
      }
      __syncthreads();
      for (int e = threadIdx.x; e < qb * qb; e += blockDim.x) {
        acc64[e].x += (double)acc32[e].x;
        acc64[e].y += (double)acc32[e].y;
      }
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < qb * qb; e += blockDim.x) {
    const double2 v = make_double2(acc64[e].x * pref, acc64[e].y * pref);
    P0[tile.p + (size_t)tau * tile.pstride + e] = v;
    if (mirror) P0[tile.p + (size_t)(nts - 1 - tau) * tile.pstride + e] = v;
  }
}

// ---------------------------------------------------------------------------
// Sigma, one CTA per (k_irr, AO block, spin, tau).  Shared memory:
//   acc64 [b1*b1] double2 | acc32 [b1*b1] float2 | Y1 [qb*b1*NT] | Y2 [b1*NT*qb]
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) sigma_mixed_kernel(const SigTile *__restrict__ tiles,
                                                          const SigContrib *__restrict__ contribs,
                                                          const double2 *__restrict__ V,
                                                          const double2 *__restrict__ G,
                                                          const double2 *__restrict__ P, double2 *__restrict__ Sig,
                                                          int ns, double scale, int smem_bytes) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const SigTile tile = tiles[blockIdx.x];
  const int b1 = tile.b1, s = tile.s, tau = tile.t0;
  double2 *acc64 = reinterpret_cast<double2 *>(smem_raw);
  float2 *acc32 = reinterpret_cast<float2 *>(acc64 + b1 * b1);
  float2 *work = acc32 + b1 * b1;
  const int cap = (smem_bytes - b1 * b1 * 24) / 8;
  for (int e = threadIdx.x; e < b1 * b1; e += blockDim.x) acc64[e] = make_double2(0.0, 0.0);
  for (int c = tile.c0; c < tile.c1; ++c) {
    const SigContrib cb = contribs[c];
    const int qb = cb.qb, b2 = cb.b2;
    const double2 *Vb = V + cb.v;
    const double2 *G2 = G + cb.gb + ((size_t)tau * ns + s) * cb.sb;
    const double2 *Pt = P + cb.pq + (size_t)tau * cb.pstride;
    int NT = cap / (2 * qb * b1);
    NT = NT < b2 ? NT : b2;
    __syncthreads();
    for (int e = threadIdx.x; e < b1 * b1; e += blockDim.x) acc32[e] = make_float2(0.f, 0.f);
    for (int n0 = 0; n0 < b2; n0 += NT) {
      const int nn = (b2 - n0) < NT ? (b2 - n0) : NT;
      float2 *Y1 = work;                    // [(Q,i)][nn]
      float2 *Y2 = work + qb * b1 * nn;     // [(i,nn)][P]
      __syncthreads();
      // Y1[(Q,i)][nn] = sum_m V[(Q,i)][m] G2[m][n0+nn]
      warp_cgemm<false>(qb * b1, nn, b2, GlobalMat{Vb, b2, 1, qb * b1, b2, false},
                        GlobalMat{G2 + n0, b2, 1, b2, nn, false}, Y1, nn);
      __syncthreads();
      // Y2[(i,nn)][P] = sum_Q Y1[(Q,i)][nn] P[Q][P]     (row r = i*nn + nn', A(r,Q) = Y1[Q*b1*nn + r])
      warp_cgemm<false>(b1 * nn, qb, qb, SharedMat{Y1, 1, b1 * nn, b1 * nn, qb},
                        GlobalMat{Pt, qb, 1, qb, qb, false}, Y2, qb);
      __syncthreads();
      // acc32[i][j] += sum_{nn,P} Y2[(i,nn)][P] conj(V[P][j][n0+nn])
      warp_cgemm<true>(b1, b1, nn * qb, SharedMat{Y2, nn * qb, 1, b1, nn * qb},
                       SgS3B{Vb, b1, b2, qb, n0, nn * qb, b1}, acc32, b1);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < b1 * b1; e += blockDim.x) {
      acc64[e].x += (double)acc32[e].x;
      acc64[e].y += (double)acc32[e].y;
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < b1 * b1; e += blockDim.x)
    Sig[tile.sig + (size_t)tau * tile.sstride + e] = make_double2(acc64[e].x * scale, acc64[e].y * scale);
}

void launch_p0_mixed(const P0Tile *tiles, int ntiles, const P0Contrib *contribs, const double2 *V,
                     const double2 *G, double2 *P0, int ns, int nts, double pref, int mirror, int smem_bytes,
                     cudaStream_t st) {
  if (ntiles == 0) return;
  p0_mixed_kernel<<<ntiles, 128, smem_bytes, st>>>(tiles, contribs, V, G, P0, ns, nts, pref, mirror, smem_bytes);
  GWGB_CUDA(cudaGetLastError());
}

void launch_sigma_mixed(const SigTile *tiles, int ntiles, const SigContrib *contribs, const double2 *V,
                        const double2 *G, const double2 *P, double2 *Sig, int ns, double scale, int smem_bytes,
                        cudaStream_t st) {
  if (ntiles == 0) return;
  sigma_mixed_kernel<<<ntiles, 128, smem_bytes, st>>>(tiles, contribs, V, G, P, Sig, ns, scale, smem_bytes);
  GWGB_CUDA(cudaGetLastError());
}

void set_mixed_kernel_attributes(int smem_bytes) {
  GWGB_CUDA(cudaFuncSetAttribute(p0_mixed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes));
  GWGB_CUDA(cudaFuncSetAttribute(sigma_mixed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes));
}

}  // namespace gwgb
