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
// (1) runs here as a tcgen05 GEMM on split operands (TF32x3: kind::tf32, two
// planes, three products; BF16x3: kind::f16, three BF16 planes, six products;
// FP32 accumulation in TMEM) writing W to HBM in FP32, one tau chunk at a time;
// (2) and (3) run per (owner, tau range, slice of contributions): (2) on CUDA
// cores in FP32, written split into the operand planes of (3), which runs as a
// tcgen05 GEMM with rows (tau, j) and K = (Q, m) (sigma_uvt_kernel; the FP32
// SIMT kernels sigma_uv_{blocked,small} take AO blocks above 64).  FP32
// accumulates within an aux-row chunk, FP64 above; every tile writes an FP64
// partial block that reduce_slices_kernel sums in order.
#include "common.h"
#include "kernels.h"
#include "kernels_tc.h"
#include <cuda_bf16.h>

#include "tc_common.cuh"

namespace gwgb {

namespace {

// Operand planes of the split products.  TF32x3: x = hi + lo (two TF32
// planes), products lo*hi + hi*lo + hi*hi.  BF16x3: x = b0 + b1 + b2 (three
// BF16 planes), products b2*b0 + b1*b1 + b0*b2 + b1*b0 + b0*b1 + b0*b0 (the
// terms below 2^-24 relative are dropped; smallest first).  Each plane is a
// K-major no-swizzle tile; plane i of an operand starts i * plane_bytes in.
template <bool BF>
struct Planes {
  static constexpr int N = BF ? 3 : 2;      // planes per operand
  static constexpr int EB = BF ? 2 : 4;     // bytes per element
  static constexpr int KSTEP = BF ? 16 : 8; // K of one MMA
  __device__ static uint32_t off(int r, int k, int K) {
    return BF ? tc::kmajor_offset16(r, k, K) : tc::kmajor_offset(r, k, K);
  }
  __device__ static uint32_t sbo(int K) { return (uint32_t)(K * EB / 16) * 128; }
  __device__ static void store(unsigned char *base, uint32_t plane_bytes, uint32_t off, float x) {
    if constexpr (BF) {
      const __nv_bfloat16 b0 = __float2bfloat16_rn(x);
      const float r1 = x - __bfloat162float(b0);
      const __nv_bfloat16 b1 = __float2bfloat16_rn(r1);
      const __nv_bfloat16 b2 = __float2bfloat16_rn(r1 - __bfloat162float(b1));
      *reinterpret_cast<unsigned short *>(base + off) = __bfloat16_as_ushort(b0);
      *reinterpret_cast<unsigned short *>(base + plane_bytes + off) = __bfloat16_as_ushort(b1);
      *reinterpret_cast<unsigned short *>(base + 2 * plane_bytes + off) = __bfloat16_as_ushort(b2);
    } else {
      const uint32_t h = tc::to_tf32(x);
      const uint32_t l = tc::to_tf32(x - __uint_as_float(h));
      *reinterpret_cast<uint32_t *>(base + off) = h;
      *reinterpret_cast<uint32_t *>(base + plane_bytes + off) = l;
    }
  }
  // four consecutive K elements of one row (a 16-byte TF32 / 8-byte BF16 segment
  // of a core-matrix row): one vector store per plane
  __device__ static void store4(unsigned char *base, uint32_t plane_bytes, uint32_t off, float4 x) {
    if constexpr (BF) {
      const float v[4] = {x.x, x.y, x.z, x.w};
      uint32_t w[3][2];
#pragma unroll
      for (int j = 0; j < 4; j += 2) {
        unsigned short b[3][2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const __nv_bfloat16 b0 = __float2bfloat16_rn(v[j + h]);
          const float r1 = v[j + h] - __bfloat162float(b0);
          const __nv_bfloat16 b1 = __float2bfloat16_rn(r1);
          const __nv_bfloat16 b2 = __float2bfloat16_rn(r1 - __bfloat162float(b1));
          b[0][h] = __bfloat16_as_ushort(b0);
          b[1][h] = __bfloat16_as_ushort(b1);
          b[2][h] = __bfloat16_as_ushort(b2);
        }
#pragma unroll
        for (int pl = 0; pl < 3; ++pl) w[pl][j / 2] = (uint32_t)b[pl][0] | ((uint32_t)b[pl][1] << 16);
      }
#pragma unroll
      for (int pl = 0; pl < 3; ++pl)
        *reinterpret_cast<uint2 *>(base + pl * plane_bytes + off) = make_uint2(w[pl][0], w[pl][1]);
    } else {
      uint4 h, l;
      h.x = tc::to_tf32(x.x); l.x = tc::to_tf32(x.x - __uint_as_float(h.x));
      h.y = tc::to_tf32(x.y); l.y = tc::to_tf32(x.y - __uint_as_float(h.y));
      h.z = tc::to_tf32(x.z); l.z = tc::to_tf32(x.z - __uint_as_float(h.z));
      h.w = tc::to_tf32(x.w); l.w = tc::to_tf32(x.w - __uint_as_float(h.w));
      *reinterpret_cast<uint4 *>(base + off) = h;
      *reinterpret_cast<uint4 *>(base + plane_bytes + off) = l;
    }
  }
  __device__ static uint32_t idesc(int M, int Nn) { return BF ? tc::idesc_bf16(M, Nn) : tc::idesc_tf32(M, Nn); }
  // all split products of one K step (byte offset koff inside every plane)
  __device__ static void mma_step(uint32_t d, uint32_t a, uint32_t apl, uint32_t b, uint32_t bpl, uint32_t koff,
                                  uint32_t sbo_a, uint32_t sbo_b, uint32_t idesc, uint32_t acc_first) {
    auto da = [&](int i) { return tc::make_desc(a + i * apl + koff, 128, sbo_a); };
    auto db = [&](int i) { return tc::make_desc(b + i * bpl + koff, 128, sbo_b); };
    if constexpr (BF) {
      tc::mma_bf16(d, da(2), db(0), idesc, acc_first);
      tc::mma_bf16(d, da(1), db(1), idesc, 1);
      tc::mma_bf16(d, da(0), db(2), idesc, 1);
      tc::mma_bf16(d, da(1), db(0), idesc, 1);
      tc::mma_bf16(d, da(0), db(1), idesc, 1);
      tc::mma_bf16(d, da(0), db(0), idesc, 1);
    } else {
      tc::mma_tf32(d, da(1), db(0), idesc, acc_first);
      tc::mma_tf32(d, da(0), db(1), idesc, 1);
      tc::mma_tf32(d, da(0), db(0), idesc, 1);
    }
  }
};

}  // namespace

// ---------------------------------------------------------------------------
// (1): one CTA = 128 rows (tau, Q) of one aux block x a range of its columns
// in packs of npk complex columns.  A is staged once by all threads; then the
// warps specialise into a pipeline over the packs:
//   warps 5-7  stage B packs into a ring of two buffers   (full[b] / empty[b])
//   warp 4     one lane issues the MMAs of a pack into one of two TMEM
//              accumulators                               (done[a] / afree[a])
//   warps 0-3  drain an accumulator (TMEM lanes = rows) through a per-warp
//              shared tile of 32 rows x 16 complex, written out as whole
//              128-byte row segments (coalesced)
// so staging, MMAs and the W stores of consecutive packs overlap.  Every wait
// is bounded; a wait that runs out sets the error word and an abort flag that
// ends the other roles' loops, and the TMEM is released only after the MMAs
// issued so far have completed (bounded wait).
// Shared: A planes (128 x K) | B buffer 0 planes (2 npk x K) | buffer 1 planes |
// drain tiles [4][32][36] floats; K = 2 q_b padded to the MMA K step.
// ---------------------------------------------------------------------------
constexpr int SW_DRAIN_LD = 36;  // floats per row of a drain tile (32 + 4: spreads the banks)
static_assert(4 * 32 * SW_DRAIN_LD * 4 == 18432, "the host sizes the drain tiles as 18432 bytes");
template <bool BF>
__global__ void __launch_bounds__(256) sigma_w_tc_kernel(const SwTile *__restrict__ tiles,
                                                         const float2 *__restrict__ Bcat,
                                                         const double2 *__restrict__ P, float2 *__restrict__ W,
                                                         int tau0, int *__restrict__ err) {
  using PL = Planes<BF>;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ uint32_t tmem_slot;
  __shared__ __align__(8) uint64_t bar[9];  // full[2] | empty[2] | done[2] | afree[2] | last
  __shared__ int abort_flag, issued;
  const SwTile tl = tiles[blockIdx.x];
  const int qb = tl.qb;
  const int KP = BF ? ((tl.kp + 15) & ~15) : tl.kp;
  const int SW_PACK = tl.npk, BR = 2 * tl.npk;  // complex columns per pack, B rows per pack
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t apl = 128u * KP * PL::EB, bpl = (uint32_t)BR * KP * PL::EB;  // plane bytes
  unsigned char *A = smem_raw;
  unsigned char *Bb = A + PL::N * apl;  // 2 buffers x N planes
  uint64_t *full = bar, *empty = bar + 2, *done = bar + 4, *afree = bar + 6, *last = bar + 8;
  constexpr int NPROD = 96;  // producer threads (warps 5-7)
  if (warp == 0) tc::tmem_alloc(&tmem_slot, 256);
  if (tid == 0) {
    for (int b = 0; b < 2; ++b) {
      tc::mbar_init(&full[b], NPROD);
      tc::mbar_init(&empty[b], 1);
      tc::mbar_init(&done[b], 1);
      tc::mbar_init(&afree[b], 128);
    }
    tc::mbar_init(last, 1);
    abort_flag = 0;
    issued = 0;
  }
  const int rows = tl.nt * qb;
  // A: rows (tau, Q) of P(tau), K = (P, re/im); every row is qb contiguous complex.
  // A lane writes one K quad (two complex) of one row; a warp covers 8 rows x 4 quads
  // (contiguous core-matrix bytes: conflict-free vector stores).
  const int nq = KP / 4;
  for (int e = tid; e < 128 * nq; e += 256) {
    const int rl = e & 7, rest = e >> 3;
    const int q = rest % nq, r = (rest / nq) * 8 + rl;
    double2 v0 = make_double2(0.0, 0.0), v1 = v0;
    if (r < rows) {
      const int it = r / qb, Q = r - it * qb;
      const double2 *row = P + tl.pa + (int64_t)(tl.t0 + it) * tl.pstride + (int64_t)Q * qb;
      if (2 * q < qb) v0 = __ldg(row + 2 * q);
      if (2 * q + 1 < qb) v1 = __ldg(row + 2 * q + 1);
      if (tl.pconj) { v0.y = -v0.y; v1.y = -v1.y; }
    }
    PL::store4(A, apl, PL::off(r, 4 * q, KP), make_float4((float)v0.x, (float)v0.y, (float)v1.x, (float)v1.y));
  }
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_slot;
  const int npacks = (tl.c1 - tl.c0 + SW_PACK - 1) / SW_PACK;
  // bounded wait; false when it ran out (error word and abort flag set) or another role aborted
  auto bwait = [&](uint64_t *b, uint32_t par) -> bool {
    for (int rep = 0; rep < 64; ++rep) {
      if (tc::mbar_wait(b, par, 65536)) return true;
      if (*(volatile int *)&abort_flag) return false;
    }
    atomicExch(err, 1);
    *(volatile int *)&abort_flag = 1;
    return false;
  };
  if (warp >= 5) {
    // producers: rows (col, d) of the real embedding of B = conj(V): d=0 -> (Br, -Bi),
    // d=1 -> (Bi, Br), Br = Vr, Bi = -Vi; a thread writes one K quad (two complex) of
    // both rows of one column
    const int ptid = tid - (256 - NPROD);
    for (int pk = 0; pk < npacks; ++pk) {
      const int b = pk & 1;
      if (pk >= 2 && !bwait(&empty[b], ((pk >> 1) - 1) & 1)) break;
      unsigned char *B = Bb + b * PL::N * bpl;
      const int c0 = tl.c0 + pk * SW_PACK;
      // batches of 8 items: their 16 loads are in flight together (the pack comes
      // from HBM; one load at a time per thread left the producers latency-bound)
      constexpr int BU = 8;
      for (int e0 = ptid; e0 < SW_PACK * nq; e0 += BU * NPROD) {
        float2 b0[BU], b1[BU];  // conj(V) as stored
#pragma unroll
        for (int u = 0; u < BU; ++u) {
          const int e = e0 + u * NPROD;
          const int cll = e & 3, rest = e >> 2;
          const int q = rest % nq, col = c0 + (rest / nq) * 4 + cll;
          b0[u] = b1[u] = make_float2(0.f, 0.f);
          if (e < SW_PACK * nq && col < tl.c1) {
            const float2 *bc = Bcat + tl.bcat + (int64_t)col * qb;
            if (2 * q < qb) b0[u] = __ldg(bc + 2 * q);
            if (2 * q + 1 < qb) b1[u] = __ldg(bc + 2 * q + 1);
          }
        }
#pragma unroll
        for (int u = 0; u < BU; ++u) {
          const int e = e0 + u * NPROD;
          if (e < SW_PACK * nq) {
            const int cll = e & 3, rest = e >> 2;
            const int q = rest % nq, cl = (rest / nq) * 4 + cll;
            PL::store4(B, bpl, PL::off(2 * cl, 4 * q, KP), make_float4(b0[u].x, -b0[u].y, b1[u].x, -b1[u].y));
            PL::store4(B, bpl, PL::off(2 * cl + 1, 4 * q, KP), make_float4(b0[u].y, b0[u].x, b1[u].y, b1[u].x));
          }
        }
      }
      tc::fence_async_smem();
      tc::mbar_arrive(&full[b]);
    }
  } else if (warp == 4) {
    if (lane == 0) {  // MMA issuer
      const uint32_t idesc = PL::idesc(128, 2 * SW_PACK);
      const uint32_t sbo = PL::sbo(KP);
      int n = 0;
      for (int pk = 0; pk < npacks; ++pk) {
        const int b = pk & 1;
        if (!bwait(&full[b], (pk >> 1) & 1)) break;
        if (pk >= 2 && !bwait(&afree[b], ((pk >> 1) - 1) & 1)) break;
        tc::fence_after_sync();
        const uint32_t a = tc::smem_u32(A), bb = tc::smem_u32(Bb + b * PL::N * bpl);
        const uint32_t d = tmem + (uint32_t)(b * 2 * SW_PACK);
        for (int st = 0; st < KP / PL::KSTEP; ++st)
          PL::mma_step(d, a, apl, bb, bpl, (uint32_t)st * 256, sbo, sbo, idesc, st > 0);
        tc::commit(&empty[b]);
        tc::commit(&done[b]);
        ++n;
      }
      if (n > 0) tc::commit(last);  // arrives when every MMA issued above has completed
      issued = n;
    }
    __syncwarp();
  } else {
    // drain: warp w owns TMEM lanes (rows) 32 w .. 32 w + 31; a lane reads its row's
    // 16 complex columns into the warp's tile, then 8 lanes write one row's 128 bytes
    float *tile = reinterpret_cast<float *>(Bb + 2 * PL::N * bpl) + warp * 32 * SW_DRAIN_LD;
    const int seg = lane & 7, rsub = lane >> 3;
    for (int pk = 0; pk < npacks; ++pk) {
      const int a = pk & 1;
      const bool okw = __all_sync(0xffffffffu, bwait(&done[a], (pk >> 1) & 1));
      if (!okw) break;
      tc::fence_after_sync();
      const uint32_t acc = tmem + (uint32_t)(a * 2 * SW_PACK) + ((uint32_t)(warp * 32) << 16);
      const int c0 = tl.c0 + pk * SW_PACK;
      for (int j0 = 0; j0 < 2 * SW_PACK; j0 += 32) {
#pragma unroll
        for (int h = 0; h < 4; ++h) {
          float v[8];
          tc::tmem_ld8(acc + (uint32_t)(j0 + 8 * h), v);
          float4 *t = reinterpret_cast<float4 *>(tile + lane * SW_DRAIN_LD + 8 * h);
          t[0] = make_float4(v[0], v[1], v[2], v[3]);
          t[1] = make_float4(v[4], v[5], v[6], v[7]);
        }
        __syncwarp();
        const int col = c0 + (j0 >> 1) + 2 * seg;  // even: packs start at even columns, ld is even
#pragma unroll
        for (int rr = 0; rr < 32; rr += 4) {
          const int rl = rr + rsub, r = warp * 32 + rl;
          if (r < rows) {
            const int it = r / qb, Q = r - it * qb;
            float2 *wrow = W + tl.wcat + ((int64_t)(tl.t0 - tau0 + it) * qb + Q) * tl.ld;  // one tau chunk
            const float4 x = *reinterpret_cast<const float4 *>(tile + rl * SW_DRAIN_LD + 4 * seg);
            if (col + 1 < tl.c1) *reinterpret_cast<float4 *>(wrow + col) = x;
            else if (col < tl.c1) wrow[col] = make_float2(x.x, x.y);
          }
        }
        __syncwarp();
      }
      tc::fence_before_sync();
      tc::mbar_arrive(&afree[a]);
    }
  }
  __syncthreads();
  if (tid == 0) {  // every commit's arrive has landed (and every MMA completed) before the CTA ends
    const int n = issued;
    for (int b = 0; b < 2 && b < n; ++b) {
      const int pl = ((n - 1 - b) >> 1) * 2 + b;  // the last pack that used buffer / accumulator b
      tc::mbar_wait(&empty[b], (uint32_t)(pl >> 1) & 1u, 4000000);
      tc::mbar_wait(&done[b], (uint32_t)(pl >> 1) & 1u, 4000000);
    }
    if (n > 0) tc::mbar_wait(last, 0u, 4000000);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 256);
}

// Bcat[col0 + (j*b2 + n)][P] = conj(V_c[P][j][n]) (FP32), once per V upload.
__global__ void bcat_kernel(const BcTask *__restrict__ tasks, const double2 *__restrict__ V, float2 *__restrict__ Bcat) {
  const BcTask tk = tasks[blockIdx.x];
  for (int e = threadIdx.x; e < tk.qb * tk.b1b2; e += blockDim.x) {
    const int P = e / tk.b1b2, jn = e - P * tk.b1b2;
    const double2 v = __ldg(V + tk.v + e);
    Bcat[tk.bcat + (int64_t)(tk.col0 + jn) * tk.qb + P] = make_float2((float)v.x, -(float)v.y);
  }
}

void launch_bcat(const BcTask *tasks, int ntasks, const double2 *V, float2 *Bcat, cudaStream_t st) {
  if (ntasks == 0) return;
  bcat_kernel<<<ntasks, 256, 0, st>>>(tasks, V, Bcat);
  GWGB_CUDA(cudaGetLastError());
}

// ---------------------------------------------------------------------------
// (2) + (3) for owners with small contributions (fewer than 200 (Q, m) terms
// on average): the same stages with one output per thread in U and KS lanes
// (shuffle-reduced) per (i, j) in the Sigma stage; at these sizes the
// per-contribution barriers dominate and the tile reduction of
// sigma_uv_blocked costs more than its register blocking saves.
// Shared: acc64 [nt][b1^2] double2 | acc32 [nt][b1^2] | G2 [b2^2] |
//         V [QC][b1][b2] | W [QC][b1][b2] | U [QC][b1][b2] (float2).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void sigma_uv_small(const SigTile &tile, const SigContrib *__restrict__ contribs,
                                               const WRef *__restrict__ wref, const double2 *__restrict__ V,
                                               const double2 *__restrict__ G, const float2 *__restrict__ W,
                                               double2 *__restrict__ Part, int ns, int smem_bytes,
    int tau0) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  const int b1 = tile.b1, s = tile.s, nt = tile.nt, bb = b1 * b1;
  const int tid = threadIdx.x;
  double2 *acc64 = reinterpret_cast<double2 *>(smem_raw);
  float2 *acc32 = reinterpret_cast<float2 *>(acc64 + nt * bb);
  float2 *G2s = acc32 + nt * bb;
  // lanes per (i, j) output in the S stage: a power of two with bb * KS <= 256
  int KS = 1;
  while (KS < 32 && bb * KS * 2 <= 256) KS *= 2;
  for (int e = tid; e < nt * bb; e += 256) acc64[e] = make_double2(0.0, 0.0);
  for (int c = tile.c0; c < tile.c1; ++c) {
    const SigContrib cb = contribs[c];
    const int qb = cb.qb, b2 = cb.b2;
    const int blk = b1 * b2;
    float2 *Vs = G2s + b2 * b2;
    const int avail = (smem_bytes - (int)((char *)Vs - (char *)smem_raw)) / 8;
    int QC = avail / (3 * blk);
    QC = QC < qb ? QC : qb;
    if (QC < 1) return;  // the host sizes shared memory for QC >= 1; never loop without progress
    float2 *Ws = Vs + QC * blk;
    float2 *Us = Ws + QC * blk;
    const double2 *Vb = V + cb.v;
    const WRef wr = wref[c];
    __syncthreads();
    for (int e = tid; e < nt * bb; e += 256) acc32[e] = make_float2(0.f, 0.f);
    for (int q0 = 0; q0 < qb; q0 += QC) {
      const int qn = (qb - q0) < QC ? (qb - q0) : QC;
      __syncthreads();
      for (int e = tid; e < qn * blk; e += 256) {
        const double2 v = __ldg(Vb + (int64_t)q0 * blk + e);
        Vs[e] = make_float2((float)v.x, (float)v.y);
      }
      for (int it = 0; it < nt; ++it) {
        const int tau = tile.t0 + it;
        const double2 *G2 = G + cb.gb + ((int64_t)tau * ns + s) * cb.sb;
        const float2 *Wt = W + wr.base + ((int64_t)(tau - tau0) * qb + q0) * wr.ld;  // W holds one tau chunk
        __syncthreads();
        for (int e = tid; e < b2 * b2; e += 256) {
          const double2 g = __ldg(G2 + e);
          G2s[e] = make_float2((float)g.x, (float)g.y);
        }
        for (int e = tid; e < qn * blk; e += 256) {
          const int Qr = e / blk, jn = e - Qr * blk;
          Ws[e] = Wt[(int64_t)Qr * wr.ld + jn];
        }
        __syncthreads();
        for (int e = tid; e < qn * blk; e += 256) {
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
        const int K = qn * b2;
        float2 *acc = acc32 + it * bb;
        if (KS == 1) {
          for (int o = tid; o < bb; o += 256) {
            const int i = o / b1, j = o - i * b1;
            float ar = 0.f, ai = 0.f;
            for (int k = 0; k < K; ++k) {
              const int Q = k / b2, m = k - Q * b2;
              const float2 vv = Vs[Q * blk + i * b2 + m], uu = Us[Q * blk + j * b2 + m];
              ar = fmaf(vv.x, uu.x, ar);
              ar = fmaf(-vv.y, uu.y, ar);
              ai = fmaf(vv.x, uu.y, ai);
              ai = fmaf(vv.y, uu.x, ai);
            }
            acc[o].x += ar;
            acc[o].y += ai;
          }
        } else {
          const int o = tid / KS, ks = tid - (tid / KS) * KS;
          float ar = 0.f, ai = 0.f;
          if (o < bb) {
            const int i = o / b1, j = o - i * b1;
            for (int k = ks; k < K; k += KS) {
              const int Q = k / b2, m = k - Q * b2;
              const float2 vv = Vs[Q * blk + i * b2 + m], uu = Us[Q * blk + j * b2 + m];
              ar = fmaf(vv.x, uu.x, ar);
              ar = fmaf(-vv.y, uu.y, ar);
              ai = fmaf(vv.x, uu.y, ai);
              ai = fmaf(vv.y, uu.x, ai);
            }
          }
          for (int off = KS / 2; off > 0; off >>= 1) {
            ar += __shfl_xor_sync(0xffffffffu, ar, off);
            ai += __shfl_xor_sync(0xffffffffu, ai, off);
          }
          if (ks == 0 && o < bb) {
            acc[o].x += ar;
            acc[o].y += ai;
          }
        }
      }
    }
    __syncthreads();
    for (int e = tid; e < nt * bb; e += 256) {
      acc64[e].x += (double)acc32[e].x;
      acc64[e].y += (double)acc32[e].y;
    }
  }
  __syncthreads();
  for (int e = tid; e < nt * bb; e += 256) Part[tile.part + e] = acc64[e];  // [nt][b1][b1], summed by slices
}

// ---------------------------------------------------------------------------
// (2) + (3): one CTA per (k_irr, AO block, spin, range of nt tau); FP32 per
// contribution, FP64 across.  Per contribution and chunk of QC aux rows the
// V rows are staged once and reused for every tau of the range:
//   U[Q][j][m]   = sum_n W(tau)[Q][j][n] G2(tau)[m][n]   (a thread: one (Q, j), up to 8 m)
//   S[i][j]     += sum_{Q,m} V[Q][i][m] U[Q][j][m]        (a thread: a 4x4 (i, j) tile over
//                                                          every NG-th (Q, m); the NG
//                                                          partial tiles are summed in order)
// Shared: acc64 [nt][b1^2] double2 | acc32 [nt][b1^2] | red [256][16] | G2 [b2^2] |
//         V [QC][b1][b2] | W [QC][b1][b2] | U [QC][b1][b2] (float2).
// ---------------------------------------------------------------------------
constexpr int UV_TB = 4;   // Sigma-stage tile edge
constexpr int UV_MB = 8;   // U-stage outputs per thread
__device__ __forceinline__ void sigma_uv_blocked(const SigTile &tile, const SigContrib *__restrict__ contribs,
                                                 const WRef *__restrict__ wref, const double2 *__restrict__ V,
                                                 const double2 *__restrict__ G, const float2 *__restrict__ W,
                                                 double2 *__restrict__ Part, int ns, int smem_bytes,
    int tau0) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  const int b1 = tile.b1, s = tile.s, nt = tile.nt, bb = b1 * b1;
  const int tid = threadIdx.x;
  double2 *acc64 = reinterpret_cast<double2 *>(smem_raw);
  float2 *acc32 = reinterpret_cast<float2 *>(acc64 + nt * bb);
  float2 *red = acc32 + nt * bb;
  float2 *G2s = red + 256 * UV_TB * UV_TB;
  const int nT = (b1 + UV_TB - 1) / UV_TB, ntile = nT * nT;
  const int NGmax = ntile >= 256 ? 1 : 256 / ntile;  // groups splitting the (Q, m) sum
  const int mytile = tid % ntile, g = tid / ntile;
  const int i0 = (mytile / nT) * UV_TB, j0 = (mytile % nT) * UV_TB;
  for (int e = tid; e < nt * bb; e += 256) acc64[e] = make_double2(0.0, 0.0);
  for (int c = tile.c0; c < tile.c1; ++c) {
    const SigContrib cb = contribs[c];
    const int qb = cb.qb, b2 = cb.b2;
    const int blk = b1 * b2;
    const int mch = (b2 + UV_MB - 1) / UV_MB;
    float2 *Vs = G2s + b2 * b2;
    const int avail = (smem_bytes - (int)((char *)Vs - (char *)smem_raw)) / 8;
    int QC = avail / (3 * blk);
    QC = QC < qb ? QC : qb;
    if (QC < 1) return;  // the host sizes shared memory for QC >= 1; never loop without progress
    float2 *Ws = Vs + QC * blk;
    float2 *Us = Ws + QC * blk;
    const double2 *Vb = V + cb.v;
    const WRef wr = wref[c];
    __syncthreads();
    for (int e = tid; e < nt * bb; e += 256) acc32[e] = make_float2(0.f, 0.f);
    for (int q0 = 0; q0 < qb; q0 += QC) {
      const int qn = (qb - q0) < QC ? (qb - q0) : QC;
      __syncthreads();
      for (int e = tid; e < qn * blk; e += 256) {
        const double2 v = __ldg(Vb + (int64_t)q0 * blk + e);
        Vs[e] = make_float2((float)v.x, (float)v.y);
      }
      for (int it = 0; it < nt; ++it) {
        const int tau = tile.t0 + it;
        const double2 *G2 = G + cb.gb + ((int64_t)tau * ns + s) * cb.sb;
        const float2 *Wt = W + wr.base + ((int64_t)(tau - tau0) * qb + q0) * wr.ld;  // W holds one tau chunk
        __syncthreads();
        for (int e = tid; e < b2 * b2; e += 256) {
          const double2 gg = __ldg(G2 + e);
          G2s[e] = make_float2((float)gg.x, (float)gg.y);
        }
        for (int e = tid; e < qn * blk; e += 256) {
          const int Qr = e / blk, jn = e - Qr * blk;
          Ws[e] = Wt[(int64_t)Qr * wr.ld + jn];
        }
        __syncthreads();
        for (int item = tid; item < qn * b1 * mch; item += 256) {
          const int r = item / mch, m0 = (item - r * mch) * UV_MB;
          const float2 *w = Ws + r * b2;
          float ur[UV_MB], ui[UV_MB];
#pragma unroll
          for (int j = 0; j < UV_MB; ++j) ur[j] = ui[j] = 0.f;
          for (int n = 0; n < b2; ++n) {
            const float2 wv = w[n];
#pragma unroll
            for (int j = 0; j < UV_MB; ++j) {
              if (m0 + j < b2) {
                const float2 gv = G2s[(m0 + j) * b2 + n];
                ur[j] = fmaf(wv.x, gv.x, ur[j]);
                ur[j] = fmaf(-wv.y, gv.y, ur[j]);
                ui[j] = fmaf(wv.x, gv.y, ui[j]);
                ui[j] = fmaf(wv.y, gv.x, ui[j]);
              }
            }
          }
#pragma unroll
          for (int j = 0; j < UV_MB; ++j)
            if (m0 + j < b2) Us[r * b2 + m0 + j] = make_float2(ur[j], ui[j]);
        }
        __syncthreads();
        const int K = qn * b2;
        // at least 16 (Q, m) terms per group: the group sums below are serial
        const int NG = max(1, min(NGmax, K / 16));
        if (g < NG) {
          float ar[UV_TB][UV_TB], ai[UV_TB][UV_TB];
#pragma unroll
          for (int x = 0; x < UV_TB; ++x)
#pragma unroll
            for (int y = 0; y < UV_TB; ++y) ar[x][y] = ai[x][y] = 0.f;
          for (int k = g; k < K; k += NG) {
            const int Q = k / b2, m = k - Q * b2;
            float2 va[UV_TB], ua[UV_TB];
#pragma unroll
            for (int x = 0; x < UV_TB; ++x) {
              va[x] = (i0 + x < b1) ? Vs[Q * blk + (i0 + x) * b2 + m] : make_float2(0.f, 0.f);
              ua[x] = (j0 + x < b1) ? Us[Q * blk + (j0 + x) * b2 + m] : make_float2(0.f, 0.f);
            }
#pragma unroll
            for (int x = 0; x < UV_TB; ++x)
#pragma unroll
              for (int y = 0; y < UV_TB; ++y) {
                ar[x][y] = fmaf(va[x].x, ua[y].x, ar[x][y]);
                ar[x][y] = fmaf(-va[x].y, ua[y].y, ar[x][y]);
                ai[x][y] = fmaf(va[x].x, ua[y].y, ai[x][y]);
                ai[x][y] = fmaf(va[x].y, ua[y].x, ai[x][y]);
              }
          }
          float2 *rp = red + (g * ntile + mytile) * (UV_TB * UV_TB);
#pragma unroll
          for (int x = 0; x < UV_TB; ++x)
#pragma unroll
            for (int y = 0; y < UV_TB; ++y) rp[x * UV_TB + y] = make_float2(ar[x][y], ai[x][y]);
        }
        __syncthreads();
        float2 *acc = acc32 + it * bb;
        for (int o = tid; o < bb; o += 256) {
          const int i = o / b1, j = o - i * b1;
          const int tl = (i / UV_TB) * nT + j / UV_TB, e = (i % UV_TB) * UV_TB + (j % UV_TB);
          float sr = 0.f, si = 0.f;
          for (int gg = 0; gg < NG; ++gg) {
            const float2 v = red[(gg * ntile + tl) * (UV_TB * UV_TB) + e];
            sr += v.x;
            si += v.y;
          }
          acc[o].x += sr;
          acc[o].y += si;
        }
      }
    }
    __syncthreads();
    for (int e = tid; e < nt * bb; e += 256) {
      acc64[e].x += (double)acc32[e].x;
      acc64[e].y += (double)acc32[e].y;
    }
  }
  __syncthreads();
  for (int e = tid; e < nt * bb; e += 256) Part[tile.part + e] = acc64[e];  // [nt][b1][b1], summed by slices
}

// The two variants as separate kernels (each launch gets its own shared
// memory size and register count): tiles [0, nblocked) take sigma_uv_blocked,
// the rest (owners whose contributions average fewer than 200 (Q, m) terms)
// sigma_uv_small.
__global__ void __launch_bounds__(256) sigma_uv_blocked_kernel(const SigTile *__restrict__ tiles,
                                                               const SigContrib *__restrict__ contribs,
                                                               const WRef *__restrict__ wref,
                                                               const double2 *__restrict__ V,
                                                               const double2 *__restrict__ G,
                                                               const float2 *__restrict__ W,
                                                               double2 *__restrict__ Part, int ns,
                                                               int smem_bytes, int tau0) {
  const SigTile tile = tiles[blockIdx.x];
  sigma_uv_blocked(tile, contribs, wref, V, G, W, Part, ns, smem_bytes, tau0);
}

__global__ void __launch_bounds__(256) sigma_uv_small_kernel(const SigTile *__restrict__ tiles,
                                                             const SigContrib *__restrict__ contribs,
                                                             const WRef *__restrict__ wref,
                                                             const double2 *__restrict__ V,
                                                             const double2 *__restrict__ G,
                                                             const float2 *__restrict__ W,
                                                             double2 *__restrict__ Part, int ns,
                                                             int smem_bytes, int tau0) {
  const SigTile tile = tiles[blockIdx.x];
  sigma_uv_small(tile, contribs, wref, V, G, W, Part, ns, smem_bytes, tau0);
}

// ---------------------------------------------------------------------------
// (2) on CUDA cores feeding (3) on tcgen05: one CTA per (owner, range of nt tau
// with nt * b1 <= 128, slice of contributions).  Per contribution and chunk of
// qn aux rows Q:
//   U[(tau, Q, j)][m] = sum_n W(tau)[Q][j][n] G2(tau)[m][n]   FP32 SIMT: a thread owns
//       8 m of one row and stores them, split, straight into the operand planes of
//   S[(tau, j)][(i, re/im)] += sum_K A[(tau, j)][K] Bv[(i, re/im)][K]   tcgen05, M = 128,
//       N = 2 b1 padded to 16, K = (Q, m, re/im), FP32 accumulation in TMEM over
//       the whole contribution,
// with Bv the real embedding of Vt[Q][i][m] (row 2i: (Vr, -Vi), row 2i+1: (Vi, Vr)).
// After every chunk the TMEM accumulator (a short K) is added to an FP64
// accumulator in shared memory, written to the tile's partial block
// Part[tile.part + (it * b1 + i) * b1 + j] at the end; FP32 holds partial sums
// over one chunk of aux rows, FP64 everything above.
// Shared: FP64 acc [(tau, j)][b1|1] | A planes (128 x ks) | Bv planes (nsp x ks) |
// W [nt][qn][b1][b2|1] | G2^T [nt][b2][m8] (float2), ks = qn * kq padded to the
// MMA K step, kq = 2 b2 padded to 4, m8 = b2 padded to 8.
// ---------------------------------------------------------------------------
// U stage of sigma_uvt_kernel: U[(tau, Q, j)][m] = sum_n W[(tau, Q, j)][n] G2^T[tau][n][m]
// for MB consecutive m per thread, written split into the A planes at
// row tau*b1 + j, K = Q*kq + 2m (+1 for the imaginary part).
template <bool BF, int MB>
__device__ __forceinline__ void uvt_u_phase(int tid, int nrow, int qn, int b1, int b2, int m8, int kq, int ks,
                                            const float2 *Ws, int wld, const float2 *G2t, unsigned char *A,
                                            uint32_t apl) {
  using PL = Planes<BF>;
  const int mc_n = (MB == 8) ? (m8 >> 3) : (((b2 + 3) & ~3) >> 2);
  for (int item = tid; item < mc_n * nrow; item += 256) {
    const int mc = item / nrow, row = item - mc * nrow;
    const int it = row / (qn * b1), Q = (row / b1) % qn, j = row % b1;
    const float2 *w = Ws + row * wld;
    const float4 *g = reinterpret_cast<const float4 *>(G2t + it * b2 * m8 + MB * mc);
    float ur[MB], ui[MB];
#pragma unroll
    for (int x = 0; x < MB; ++x) ur[x] = ui[x] = 0.f;
    for (int n = 0; n < b2; ++n) {
      const float2 wv = w[n];
      const float4 *gn = g + n * (m8 >> 1);
#pragma unroll
      for (int h = 0; h < MB / 2; ++h) {
        const float4 gg = gn[h];
        ur[2 * h] = fmaf(wv.x, gg.x, ur[2 * h]);
        ur[2 * h] = fmaf(-wv.y, gg.y, ur[2 * h]);
        ui[2 * h] = fmaf(wv.x, gg.y, ui[2 * h]);
        ui[2 * h] = fmaf(wv.y, gg.x, ui[2 * h]);
        ur[2 * h + 1] = fmaf(wv.x, gg.z, ur[2 * h + 1]);
        ur[2 * h + 1] = fmaf(-wv.y, gg.w, ur[2 * h + 1]);
        ui[2 * h + 1] = fmaf(wv.x, gg.w, ui[2 * h + 1]);
        ui[2 * h + 1] = fmaf(wv.y, gg.z, ui[2 * h + 1]);
      }
    }
    const int ra = it * b1 + j, kend = (Q + 1) * kq;
#pragma unroll
    for (int h = 0; h < MB / 2; ++h) {
      const int k = Q * kq + 2 * MB * mc + 4 * h;
      if (k < kend) PL::store4(A, apl, PL::off(ra, k, ks), make_float4(ur[2 * h], ui[2 * h], ur[2 * h + 1], ui[2 * h + 1]));
    }
  }
}

template <bool BF>
__global__ void __launch_bounds__(256) sigma_uvt_kernel(const SigTile *__restrict__ tiles,
                                                        const SigContrib *__restrict__ contribs,
                                                        const WRef *__restrict__ wref, const double2 *__restrict__ V,
                                                        const double2 *__restrict__ G, const float2 *__restrict__ W,
                                                        double2 *__restrict__ Part, int ns, int smem_bytes, int tau0,
                                                        int *__restrict__ err) {
  using PL = Planes<BF>;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ uint32_t tmem_slot;
  __shared__ __align__(8) uint64_t mbar;
  const SigTile tile = tiles[blockIdx.x];
  const int b1 = tile.b1, nt = tile.nt, s = tile.s;
  const int rows = nt * b1;             // <= 128 (host-checked)
  const int nsp = uvt_nsp(b1);          // <= 128
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tile.c0 == tile.c1) {  // an owner without contributions: a zero block
    for (int e = tid; e < nt * b1 * b1; e += 256) Part[tile.part + e] = make_double2(0.0, 0.0);
    return;
  }
  if (warp == 0) tc::tmem_alloc(&tmem_slot, 128);
  if (tid == 0) tc::mbar_init(&mbar, 1);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_slot;
  uint32_t phase = 0;
  bool ok = true, pending = false;
  const int ald = b1 | 1;
  double2 *acc = reinterpret_cast<double2 *>(smem_raw);
  unsigned char *const opnd = smem_raw + uvt_acc_bytes(nt, b1);
  for (int e = tid; e < rows * ald; e += 256) acc[e] = make_double2(0.0, 0.0);
  const uint32_t idesc = PL::idesc(128, nsp);
  // Wait for the MMA group in flight and add its accumulator (one chunk of aux
  // rows: a short K, so FP32 holds only a short sum) to the FP64 partial block;
  // warps w and w+4 share TMEM lanes 32 (w % 4) .. +31 and split the columns.
  auto flush = [&]() {
    const bool done = tc::mbar_wait(&mbar, phase);
    if (done) phase ^= 1u;
    if (!done && tid == 0) atomicExch(err, 1);
    ok = __syncthreads_and(done) != 0;
    tc::fence_after_sync();
    pending = !done;
    if (!ok) return;
    const int r = (warp & 3) * 32 + lane;
    const int cbeg = (warp < 4) ? 0 : (nsp >> 1), cend = (warp < 4) ? (nsp >> 1) : nsp;
    for (int c8 = cbeg; c8 < cend; c8 += 8) {
      float v[8];
      tc::tmem_ld8(tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)c8, v);
      if (r < rows) {
#pragma unroll
        for (int h = 0; h < 8; h += 2) {
          const int i = (c8 + h) >> 1;
          if (i < b1) {
            double2 &a = acc[r * ald + i];
            a.x += (double)v[h];
            a.y += (double)v[h + 1];
          }
        }
      }
    }
    tc::fence_before_sync();
    __syncthreads();  // accumulator drained before the next group overwrites it
    tc::fence_after_sync();
  };
  for (int c = tile.c0; c < tile.c1 && ok; ++c) {
    if (pending) flush();  // the previous group reads shared memory laid out for its contribution
    if (!ok) break;
    const SigContrib cb = contribs[c];
    const int qb = cb.qb, b2 = cb.b2;
    const int kq = uvt_kq(b2), wld = uvt_wld(b2), m8 = uvt_m8(b2);
    // aux rows per chunk: sized for the owner's tau count, not this tile's, so that
    // the K steps (the rounding) are the same for every tau chunking
    int qc = qb;
    while (qc > 1 && uvt_smem(qc, tile.ntq, b1, b2, BF) > smem_bytes) --qc;
    const int ksm = uvt_ks(qc, kq, BF);
    unsigned char *A = opnd;
    unsigned char *Bv = A + PL::N * 128u * ksm * PL::EB;
    float2 *Ws = reinterpret_cast<float2 *>(Bv + PL::N * (uint32_t)nsp * ksm * PL::EB);
    float2 *G2t = Ws + uvt_ws_elems(qc, nt, b1, b2);  // 16-byte aligned (float4 reads)
    const double2 *Vb = V + cb.v;
    const WRef wr = wref[c];
    // G2^T for every tau of the range (no MMA of this CTA is in flight here)
    for (int e0 = tid; e0 < nt * b2 * m8; e0 += 4 * 256) {  // 4 loads in flight per thread
      double2 v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int e = e0 + u * 256;
        const int it = e / (b2 * m8), r = e - it * (b2 * m8), n = r / m8, m = r - n * m8;
        v[u] = make_double2(0.0, 0.0);
        if (e < nt * b2 * m8 && m < b2) v[u] = __ldg(G + cb.gb + ((int64_t)(tile.t0 + it) * ns + s) * cb.sb + m * b2 + n);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (e0 + u * 256 < nt * b2 * m8) G2t[e0 + u * 256] = make_float2((float)v[u].x, (float)v[u].y);
    }
    for (int q0 = 0; q0 < qb; q0 += qc) {
      const int qn = min(qc, qb - q0);
      const int ks = uvt_ks(qn, kq, BF);
      const uint32_t apl = 128u * ks * PL::EB, bpl = (uint32_t)nsp * ks * PL::EB;
      // W rows (tau, Q) of the chunk (b1*b2 contiguous complex each); within a
      // contribution they are loaded while the previous chunk's MMAs run (the MMAs
      // read only A and Bv)
      const int wrow = b1 * b2;
      auto stage_w = [&]() {  // batches of 8 loads in flight per thread
        constexpr int BU = 8;
        const int total = nt * qn * wrow;
        for (int e0 = tid; e0 < total; e0 += BU * 256) {
          float2 w[BU];
#pragma unroll
          for (int u = 0; u < BU; ++u) {
            const int e = e0 + u * 256;
            if (e < total) {
              const int r = e / wrow, x = e - r * wrow, it = r / qn, Q = r - it * qn;
              w[u] = W[wr.base + ((int64_t)(tile.t0 + it - tau0) * qb + q0 + Q) * wr.ld + x];
            }
          }
#pragma unroll
          for (int u = 0; u < BU; ++u) {
            const int e = e0 + u * 256;
            if (e < total) {
              const int r = e / wrow, x = e - r * wrow, j = x / b2, n = x - j * b2;
              Ws[(r * b1 + j) * wld + n] = w[u];
            }
          }
        }
      };
      const bool early = pending;
      if (early) stage_w();
      if (pending) flush();
      if (!ok) break;
      if (!early) stage_w();
      // Bv: m pairs of Vt rows; zero rows >= 2 b1 and K columns >= qn * kq
      const int mp = kq >> 2;
      for (int e = tid; e < qn * b1 * mp; e += 256) {
        const int p = e % mp, r = e / mp, i = r % b1, Q = r / b1, m = 2 * p;
        const double2 *vr = Vb + ((int64_t)(q0 + Q) * b1 + i) * b2;
        double2 v0 = make_double2(0.0, 0.0), v1 = v0;
        if (m < b2) v0 = __ldg(vr + m);
        if (m + 1 < b2) v1 = __ldg(vr + m + 1);
        const int k = Q * kq + 4 * p;
        PL::store4(Bv, bpl, PL::off(2 * i, k, ks),
                   make_float4((float)v0.x, (float)-v0.y, (float)v1.x, (float)-v1.y));
        PL::store4(Bv, bpl, PL::off(2 * i + 1, k, ks),
                   make_float4((float)v0.y, (float)v0.x, (float)v1.y, (float)v1.x));
      }
      const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
      for (int e = tid; e < (nsp - 2 * b1) * (ks >> 2); e += 256) {
        const int r = 2 * b1 + e / (ks >> 2), k = 4 * (e % (ks >> 2));
        PL::store4(Bv, bpl, PL::off(r, k, ks), z4);
      }
      const int kpad = (ks - qn * kq) >> 2;
      for (int e = tid; e < 2 * b1 * kpad; e += 256) {
        const int r = e / kpad, k = qn * kq + 4 * (e % kpad);
        PL::store4(Bv, bpl, PL::off(r, k, ks), z4);
      }
      for (int e = tid; e < rows * kpad; e += 256) {
        const int r = e / kpad, k = qn * kq + 4 * (e % kpad);
        PL::store4(A, apl, PL::off(r, k, ks), z4);
      }
      __syncthreads();
      // U, MB m per thread (4 when b2 padded to 4 is shorter than padded to 8);
      // lanes of a warp share m (G2 reads are broadcasts)
      if (((b2 + 3) & ~3) < m8)
        uvt_u_phase<BF, 4>(tid, nt * qn * b1, qn, b1, b2, m8, kq, ks, Ws, wld, G2t, A, apl);
      else
        uvt_u_phase<BF, 8>(tid, nt * qn * b1, qn, b1, b2, m8, kq, ks, Ws, wld, G2t, A, apl);
      tc::fence_async_smem();
      tc::fence_before_sync();
      __syncthreads();
      tc::fence_after_sync();
      if (tid == 0) {
        const uint32_t a = tc::smem_u32(A), b = tc::smem_u32(Bv), sbo = PL::sbo(ks);
        for (int st = 0; st < ks / PL::KSTEP; ++st)
          PL::mma_step(tmem, a, apl, b, bpl, (uint32_t)st * 256, sbo, sbo, idesc, st > 0 ? 1u : 0u);
        tc::commit(&mbar);
      }
      pending = true;
    }
  }
  if (pending && ok) flush();  // the last group
  if (pending) tc::mbar_wait(&mbar, phase, 100000);  // MMAs still in flight after a timeout (bounded)
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 128);
  if (ok)
    for (int e = tid; e < nt * b1 * b1; e += 256) {
      const int it = e / (b1 * b1), x = e - it * (b1 * b1), i = x / b1, j = x - i * b1;
      Part[tile.part + e] = acc[(it * b1 + j) * ald + i];
    }
}

void launch_sigma_tc(bool bf16, const SwTile *wtiles, int nwtiles, int wsmem, const float2 *Bcat, const SigTile *uvt,
                     int nuvt, int uvt_smem, const SigTile *tiles1, int ntiles1, const SigContrib *contribs,
                     const WRef *wref, const double2 *V, const double2 *G, const double2 *P, float2 *W, double2 *Part,
                     int ns, int uv_smem, int nblocked, int uv_smem_small, int tau0, int *err, cudaStream_t st) {
  if (nwtiles > 0) {
    if (bf16)
      sigma_w_tc_kernel<true><<<nwtiles, 256, wsmem, st>>>(wtiles, Bcat, P, W, tau0, err);
    else
      sigma_w_tc_kernel<false><<<nwtiles, 256, wsmem, st>>>(wtiles, Bcat, P, W, tau0, err);
    GWGB_CUDA(cudaGetLastError());
  }
  if (nuvt > 0) {
    if (bf16)
      sigma_uvt_kernel<true><<<nuvt, 256, uvt_smem, st>>>(uvt, contribs, wref, V, G, W, Part, ns, uvt_smem, tau0, err);
    else
      sigma_uvt_kernel<false><<<nuvt, 256, uvt_smem, st>>>(uvt, contribs, wref, V, G, W, Part, ns, uvt_smem, tau0, err);
    GWGB_CUDA(cudaGetLastError());
  }
  // tiles1 = [blocked tiles (nblocked) | small tiles]: owners with AO blocks above 64
  if (nblocked > 0) {
    sigma_uv_blocked_kernel<<<nblocked, 256, uv_smem, st>>>(tiles1, contribs, wref, V, G, W, Part, ns, uv_smem,
                                                             tau0);
    GWGB_CUDA(cudaGetLastError());
  }
  if (ntiles1 > nblocked) {
    sigma_uv_small_kernel<<<ntiles1 - nblocked, 256, uv_smem_small, st>>>(tiles1 + nblocked, contribs, wref, V, G, W,
                                                                          Part, ns, uv_smem_small, tau0);
    GWGB_CUDA(cudaGetLastError());
  }
}

void set_tc_kernel_attributes(int smem_bytes, int sw_smem_bytes) {
  GWGB_CUDA(cudaFuncSetAttribute(sigma_w_tc_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, sw_smem_bytes));
  GWGB_CUDA(cudaFuncSetAttribute(sigma_w_tc_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sw_smem_bytes));
  GWGB_CUDA(cudaFuncSetAttribute(sigma_uv_blocked_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes));
  GWGB_CUDA(cudaFuncSetAttribute(sigma_uv_small_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes));
  GWGB_CUDA(cudaFuncSetAttribute(sigma_uvt_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes));
  GWGB_CUDA(cudaFuncSetAttribute(sigma_uvt_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes));
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

// Z stage, FP32: one CTA per (contribution, spin), all tau < nts/2.  Both
// small products are register-blocked: a thread owns up to 8 outputs of one
// row and reads each staged operand once per inner step (the other operand
// is a shared-memory broadcast).
// Shared: G2 [b2^2] | Gm [b1^2] | V [PC][b1][b2] | X2 [PC][b1][b2]  (float2)
constexpr int ZB = 8;  // outputs per thread in the Z stage products
__global__ void __launch_bounds__(256) p0_z_kernel(const PzTask *__restrict__ tasks, const double2 *__restrict__ V,
                                                   const double2 *__restrict__ G, float2 *__restrict__ Z, int ns,
                                                   int nts, int smem_bytes, int tau0, int tau1) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  const PzTask tk = tasks[blockIdx.x];
  const int b1 = tk.b1, b2 = tk.b2, qb = tk.qb, blk = b1 * b2;
  const int tid = threadIdx.x;
  float2 *G2s = reinterpret_cast<float2 *>(smem_raw);
  float2 *Gms = G2s + b2 * b2;
  float2 *Vs = Gms + b1 * b1;
  const int avail = smem_bytes / 8 - b2 * b2 - b1 * b1;
  int PC = avail / (2 * blk);
  PC = PC < qb ? PC : qb;
  if (PC < 1) return;  // the host sizes shared memory for PC >= 1; never loop without progress
  float2 *X2 = Vs + PC * blk;
  const double2 *Vb = V + tk.v;
  const int mch = (b2 + ZB - 1) / ZB, pch = (b1 + ZB - 1) / ZB;
  for (int p0 = 0; p0 < qb; p0 += PC) {
    const int pn = (qb - p0) < PC ? (qb - p0) : PC;
    __syncthreads();
    for (int e = tid; e < pn * blk; e += 256) {
      const double2 v = __ldg(Vb + (int64_t)p0 * blk + e);
      Vs[e] = make_float2((float)v.x, (float)v.y);
    }
    for (int tau = tau0; tau < tau1; ++tau) {  // one tau chunk of Zcat
      const double2 *G2 = G + tk.gb + ((int64_t)tau * ns + tk.s) * tk.sb;
      const double2 *Gm = G + tk.ga + ((int64_t)(nts - 1 - tau) * ns + tk.s) * tk.sa;
      __syncthreads();
      for (int e = tid; e < b2 * b2; e += 256) {
        const double2 g = __ldg(G2 + e);
        G2s[e] = make_float2((float)g.x, (float)g.y);
      }
      for (int e = tid; e < b1 * b1; e += 256) {
        const double2 g = __ldg(Gm + e);
        Gms[e] = make_float2((float)g.x, (float)g.y);
      }
      __syncthreads();
      // X2[P][t][m] = sum_n conj(V[P][t][n]) G2[m][n]: row (P, t), up to ZB values of m
      for (int item = tid; item < pn * b1 * mch; item += 256) {
        const int r = item / mch, m0 = (item - r * mch) * ZB;
        const float2 *vr = Vs + r * b2;
        float xr[ZB], xi[ZB];
#pragma unroll
        for (int j = 0; j < ZB; ++j) xr[j] = xi[j] = 0.f;
        for (int n = 0; n < b2; ++n) {
          const float2 v = vr[n];
#pragma unroll
          for (int j = 0; j < ZB; ++j) {
            if (m0 + j < b2) {
              const float2 g = G2s[(m0 + j) * b2 + n];
              xr[j] = fmaf(v.x, g.x, xr[j]);
              xr[j] = fmaf(v.y, g.y, xr[j]);
              xi[j] = fmaf(v.x, g.y, xi[j]);
              xi[j] = fmaf(-v.y, g.x, xi[j]);
            }
          }
        }
#pragma unroll
        for (int j = 0; j < ZB; ++j)
          if (m0 + j < b2) X2[r * b2 + m0 + j] = make_float2(xr[j], xi[j]);
      }
      __syncthreads();
      // Z[P][(p,m)] = sum_t Gm[t][p] X2[P][t][m]: (P, m), up to ZB values of p
      //   -> Zcat row (tau, p0 + P), columns zcol + p*b2 + m
      float2 *Zt = Z + tk.z + ((int64_t)(tau - tau0) * qb + p0) * tk.zld + tk.zcol;
      for (int item = tid; item < pn * b2 * pch; item += 256) {
        const int P = item / (b2 * pch);
        const int rem = item - P * b2 * pch;
        const int m = rem / pch, pb = (rem - (rem / pch) * pch) * ZB;
        const float2 *x = X2 + P * blk + m;
        float zr[ZB], zi[ZB];
#pragma unroll
        for (int j = 0; j < ZB; ++j) zr[j] = zi[j] = 0.f;
        for (int t = 0; t < b1; ++t) {
          const float2 xv = x[t * b2];
#pragma unroll
          for (int j = 0; j < ZB; ++j) {
            if (pb + j < b1) {
              const float2 g = Gms[t * b1 + pb + j];
              zr[j] = fmaf(g.x, xv.x, zr[j]);
              zr[j] = fmaf(-g.y, xv.y, zr[j]);
              zi[j] = fmaf(g.x, xv.y, zi[j]);
              zi[j] = fmaf(g.y, xv.x, zi[j]);
            }
          }
        }
#pragma unroll
        for (int j = 0; j < ZB; ++j)
          if (pb + j < b1) Zt[(int64_t)P * tk.zld + (pb + j) * b2 + m] = make_float2(zr[j], zi[j]);
      }
    }
  }
}

// tcgen05 stage, split-K: D[(tau,P)][Q] = sum_k Zcat[(tau,P)][k] Vcat[Q][k] over
// this CTA's K slice (chunks of 16 complex = 32 real columns), FP32 in TMEM,
// then FP64 partial sums to Ppart.  256 threads stage the operands (8 loads in
// flight per thread); warps 0-3 drain TMEM lanes 0-127.
// Shared: A planes (128 x 32) | B planes (NP x 32): 64 KB (TF32) / 48 KB (BF16) at NP = 128.
template <bool BF>
__global__ void __launch_bounds__(256) p0_tc_kernel(const PkTile *__restrict__ tiles,
                                                    const float2 *__restrict__ Z, const float2 *__restrict__ Vcat,
                                                    double2 *__restrict__ Ppart, int tau0, int *__restrict__ err) {
  using PL = Planes<BF>;
  constexpr int KP = 32;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ uint32_t tmem_slot;
  __shared__ __align__(8) uint64_t mbar;
  const PkTile tl = tiles[blockIdx.x];
  const int qb = tl.qb, NP = tl.np;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t apl = 128u * KP * PL::EB, bpl = (uint32_t)NP * KP * PL::EB;
  unsigned char *A = smem_raw;
  unsigned char *B = A + PL::N * apl;
  uint32_t ncols_alloc = 32;
  while ((int)ncols_alloc < NP) ncols_alloc <<= 1;
  if (warp == 0) tc::tmem_alloc(&tmem_slot, ncols_alloc);
  if (tid == 0) tc::mbar_init(&mbar, 1);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_slot;
  const int rows = tl.nt * qb;
  const float2 *Zb = Z + tl.z + (int64_t)(tl.t0 - tau0) * qb * tl.zld;  // Zcat holds one tau chunk
  const float2 *Vb = Vcat + tl.vc;
  bool ok = true;
  uint32_t phase = 0;
  for (int ch = 0; ch < tl.kcn && ok; ++ch) {
    const int kbase = (tl.kc0 + ch) * 16;
    // A: 128 rows x 16 complex, row r = (tau, P); zero rows beyond `rows`.  A lane
    // loads two complex (16 B) and writes one K quad; a warp covers 8 rows x 4 quads.
#pragma unroll 4
    for (int e = tid; e < 128 * 8; e += 256) {
      const int r = (e >> 6) * 8 + (e & 7), q = (e >> 3) & 7;
      float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
      if (r < rows) z = *reinterpret_cast<const float4 *>(Zb + (int64_t)r * tl.zld + kbase + 2 * q);
      PL::store4(A, apl, PL::off(r, 4 * q, KP), z);
    }
    // B: rows (Q, d) of the real embedding of V^T: d=0 -> (Vr, -Vi), d=1 -> (Vi, Vr);
    // a lane writes one K quad of both rows of one Q
#pragma unroll 2
    for (int e = tid; e < (NP / 2) * 8; e += 256) {
      const int Q = (e >> 5) * 4 + (e & 3), q = (e >> 2) & 7;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (Q < qb) v = *reinterpret_cast<const float4 *>(Vb + (int64_t)Q * tl.zld + kbase + 2 * q);
      if (Q < NP / 2) {
        PL::store4(B, bpl, PL::off(2 * Q, 4 * q, KP), make_float4(v.x, -v.y, v.z, -v.w));
        PL::store4(B, bpl, PL::off(2 * Q + 1, 4 * q, KP), make_float4(v.y, v.x, v.w, v.z));
      }
    }
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (tid == 0) {
      const uint32_t idesc = PL::idesc(128, NP);
      const uint32_t sbo = PL::sbo(KP);
      const uint32_t a = tc::smem_u32(A), b = tc::smem_u32(B);
#pragma unroll
      for (int st = 0; st < KP / PL::KSTEP; ++st)
        PL::mma_step(tmem, a, apl, b, bpl, (uint32_t)st * 256, sbo, sbo, idesc, (ch > 0 || st > 0) ? 1u : 0u);
      tc::commit(&mbar);
    }
    ok = tc::mbar_wait(&mbar, phase);
    phase ^= 1u;
    if (!ok && lane == 0) atomicExch(err, 1);
    ok = __syncthreads_and(ok);
    tc::fence_after_sync();
  }
  if (warp < 4) {
    const int r = warp * 32 + lane;
    for (int c0 = 0; c0 < NP; c0 += 8) {
      float v[8];
      tc::tmem_ld8(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
      if (r < rows) {
#pragma unroll
        for (int j = 0; j < 8; j += 2) {
          const int Q = (c0 + j) >> 1;
          if (Q < qb)
            Ppart[tl.part + (int64_t)r * qb + Q] =
                (ok && tl.kcn > 0) ? make_double2((double)v[j], (double)v[j + 1]) : make_double2(0.0, 0.0);
        }
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, ncols_alloc);
}

// Sum the K slices in order, apply the prefactor and write P0 (and its mirror).
__global__ void p0_reduce_kernel(const PrTile *__restrict__ tiles, const double2 *__restrict__ Ppart,
                                 double2 *__restrict__ P0, int nts, double pref, int mirror) {
  const PrTile tl = tiles[blockIdx.x];
  const int qb = tl.qb, rows = tl.nt * qb;
  const int64_t slice = (int64_t)rows * qb;
  // gridDim.y CTAs share a tile (one tau chunk has few tiles); each element sums its
  // slices in order
  for (int e = blockIdx.y * blockDim.x + threadIdx.x; e < rows * qb; e += gridDim.y * blockDim.x) {
    const int r = e / qb, Q = e - r * qb;
    double2 acc = make_double2(0.0, 0.0);
    for (int sl = 0; sl < tl.nslice; ++sl) {
      const double2 v = Ppart[tl.part + sl * slice + e];
      acc.x += v.x;
      acc.y += v.y;
    }
    const int it = r / qb, P = r - it * qb;
    const int tau = tl.t0 + it;
    const double2 o = make_double2(acc.x * pref, acc.y * pref);
    P0[tl.pout + (int64_t)tau * tl.pstride + (int64_t)Q * qb + P] = o;
    if (mirror) P0[tl.pout + (int64_t)(nts - 1 - tau) * tl.pstride + (int64_t)Q * qb + P] = o;
  }
}

// Vcat[Q][zcol + pm] = V_c[Q][pm] (FP32), once per V upload.
__global__ void vcat_kernel(const VcTask *__restrict__ tasks, const double2 *__restrict__ V, float2 *__restrict__ Vcat) {
  const VcTask tk = tasks[blockIdx.x];
  for (int e = threadIdx.x; e < tk.qb * tk.b1b2; e += blockDim.x) {
    const int Q = e / tk.b1b2, pm = e - Q * tk.b1b2;
    const double2 v = __ldg(V + tk.v + e);
    Vcat[tk.vc + (int64_t)Q * tk.zld + tk.zcol + pm] = make_float2((float)v.x, (float)v.y);
  }
}

void launch_vcat(const VcTask *tasks, int ntasks, const double2 *V, float2 *Vcat, cudaStream_t st) {
  if (ntasks == 0) return;
  vcat_kernel<<<ntasks, 256, 0, st>>>(tasks, V, Vcat);
  GWGB_CUDA(cudaGetLastError());
}

void launch_p0_tc(bool bf16, const PzTask *ztasks, int nz, int zsmem, const PkTile *ktiles, int nk, const PrTile *rtiles,
                  int nr, const double2 *V, const double2 *G, float2 *Z, const float2 *Vcat, double2 *Ppart,
                  double2 *P0, int ns, int nts, int tau0, int tau1, double pref, int mirror, int *err,
                  cudaStream_t st) {
  if (nz > 0) {
    p0_z_kernel<<<nz, 256, zsmem, st>>>(ztasks, V, G, Z, ns, nts, zsmem, tau0, tau1);
    GWGB_CUDA(cudaGetLastError());
  }
  if (nk > 0) {
    if (bf16)
      p0_tc_kernel<true><<<nk, 256, 64 * 1024, st>>>(ktiles, Z, Vcat, Ppart, tau0, err);
    else
      p0_tc_kernel<false><<<nk, 256, 64 * 1024, st>>>(ktiles, Z, Vcat, Ppart, tau0, err);
    GWGB_CUDA(cudaGetLastError());
  }
  if (nr > 0) {
    p0_reduce_kernel<<<dim3(nr, 4), 256, 0, st>>>(rtiles, Ppart, P0, nts, pref, mirror);
    GWGB_CUDA(cudaGetLastError());
  }
}

void set_tc_p0_kernel_attributes(int smem_bytes) {
  GWGB_CUDA(cudaFuncSetAttribute(p0_z_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes));
  GWGB_CUDA(cudaFuncSetAttribute(p0_tc_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024));
  GWGB_CUDA(cudaFuncSetAttribute(p0_tc_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024));
}

}  // namespace gwgb

// ===========================================================================
// Test hook: a bounded mbarrier wait that runs out (nothing arrives on the
// barrier); the kernel records it in a status word and returns.
// ===========================================================================
namespace gwgb {

__device__ int g_wait_test_status;

__global__ void wait_timeout_kernel(int polls) {
  __shared__ __align__(8) uint64_t mbar;
  if (threadIdx.x != 0) return;
  tc::mbar_init(&mbar, 1);
  asm volatile("fence.mbarrier_init.release.cluster;");
  const bool done = tc::mbar_wait(&mbar, 0u, polls);
  g_wait_test_status = done ? 0 : 1;
}

int run_wait_timeout_test(int polls) {
  int zero = 0, status = 0;
  GWGB_CUDA(cudaMemcpyToSymbol(g_wait_test_status, &zero, sizeof(int)));
  wait_timeout_kernel<<<1, 32>>>(polls);
  GWGB_CUDA(cudaGetLastError());
  GWGB_CUDA(cudaDeviceSynchronize());
  GWGB_CUDA(cudaMemcpyFromSymbol(&status, g_wait_test_status, sizeof(int)));
  return status;
}

}  // namespace gwgb
