// tcgen05 (TMEM) mixed-precision contraction kernels: work descriptors and launchers.
#pragma once

#include "common.h"

namespace gwgb {

// One CTA of the Sigma W-GEMM: rows (tau, Q) of one aux block (q, iq), all
// columns (c, j, n) of the block in packs of npk complex columns.
//   A = P(tau)[Q][P] (FP64, staged once), B = Bcat[col][P] = conj(V_c[P][j][n])
//   (FP32, built once per V upload), W = Wcat[((tau - t_chunk)*qb + Q)*ncol + col]
//   (FP32; the W buffer holds one tau chunk starting at t_chunk).
struct SwTile {
  int64_t pa;       // P(q) block base at tau = 0
  int64_t bcat;     // Bcat base of the block: Bcat[col*qb + P]
  int64_t wcat;     // Wcat base of the block
  int32_t pstride;  // per-tau stride of P(q)
  int32_t qb;
  int32_t t0, nt;   // tau range; nt * qb <= 128
  int32_t ncol;     // complex columns of the block (the row length of W)
  int32_t kp;       // K = 2 qb padded to 8 (the BF16 kernel pads it to 16)
  int32_t npk;      // complex columns per pack (16, 32 or 64)
  int32_t pconj;    // A = conj(P~(q')) (time-reversal partner)
  int32_t c0, c1;   // the columns [c0, c1) this CTA computes
  int32_t ld;       // W row stride (ncol rounded up to even: 16-byte stores)
  int32_t pad;
};

// Bcat entries: one per Sigma contribution.
struct BcTask {
  int64_t v;        // V block [qb][b1][b2]
  int64_t bcat;     // Bcat base of the block
  int32_t qb, b1b2, col0, pad;
};

// sw_smem_bytes: the W GEMM kernel (up to the device's opt-in limit)
void set_tc_kernel_attributes(int smem_bytes, int sw_smem_bytes);
void set_tc_p0_kernel_attributes(int smem_bytes);

// W reference of one Sigma contribution:
//   W_c(tau)[Q][(j,n)] = W[base + ((tau - t_chunk)*qb + Q)*ld + j*b2 + n]
struct WRef {
  int64_t base;
  int64_t ld;
};

// Geometry of sigma_uvt_kernel (U on CUDA cores feeding the Sigma GEMM on
// tcgen05), shared by the kernel and the host's tile planning: K elements per
// aux row (2 b2 padded to 4), the W row stride in shared memory (odd: no bank
// conflicts), m padded to 8, N = 2 b1 padded to 16, K of a chunk of qn aux rows
// padded to the MMA K step, and the shared memory of such a chunk.
__host__ __device__ inline int uvt_kq(int b2) { return (2 * b2 + 3) & ~3; }
__host__ __device__ inline int uvt_wld(int b2) { return b2 | 1; }
__host__ __device__ inline int uvt_m8(int b2) { return (b2 + 7) & ~7; }
__host__ __device__ inline int uvt_nsp(int b1) { return (2 * b1 + 15) & ~15; }
__host__ __device__ inline int uvt_ks(int qn, int kq, bool bf) {
  const int st = bf ? 16 : 8;
  return (qn * kq + st - 1) / st * st;
}
__host__ __device__ inline int uvt_ws_elems(int qn, int nt, int b1, int b2) {
  return (nt * qn * b1 * uvt_wld(b2) + 1) & ~1;
}
// FP64 accumulator rows (tau, j) x b1 with an odd row stride
__host__ __device__ inline int uvt_acc_bytes(int nt, int b1) { return 16 * nt * b1 * (b1 | 1); }
__host__ __device__ inline int64_t uvt_smem(int qn, int nt, int b1, int b2, bool bf) {
  const int ks = uvt_ks(qn, uvt_kq(b2), bf);
  return (int64_t)uvt_acc_bytes(nt, b1) + (int64_t)(bf ? 6 : 8) * (128 + uvt_nsp(b1)) * ks +
         8ll * uvt_ws_elems(qn, nt, b1, b2) + 8ll * nt * b2 * uvt_m8(b2);
}

// One tau chunk (starting at tau0) of the Sigma stages: the W GEMM tiles, the
// U/Sigma tiles of owners with AO blocks up to 64 (uvt: U on CUDA cores, Sigma
// on tcgen05), then the FP32 U/Sigma tiles of larger owners (tiles1 =
// [nblocked register-blocked | the rest]); all write FP64 partial blocks to Part.
void launch_sigma_tc(bool bf16, const SwTile *wtiles, int nwtiles, int wsmem, const float2 *Bcat, const SigTile *uvt,
                     int nuvt, int uvt_smem, const SigTile *tiles1, int ntiles1, const SigContrib *contribs,
                     const WRef *wref, const double2 *V, const double2 *G, const double2 *P, float2 *W, double2 *Part,
                     int ns, int uv_smem, int nblocked, int uv_smem_small, int tau0, int *err, cudaStream_t st);

void launch_bcat(const BcTask *tasks, int ntasks, const double2 *V, float2 *Bcat, cudaStream_t st);

}  // namespace gwgb

namespace gwgb {

// P0, stage Z: one CTA per (contribution, spin) over one tau chunk of
// [0, nts/2).  Z of the aux block is one matrix Zcat[(tau - t_chunk, P)][K] with
// K concatenating the (p, m) columns of every (contribution, spin); this task
// writes columns [zcol, zcol + b1*b2).
struct PzTask {
  int64_t v;       // V block [qb][b1][b2]
  int64_t ga, gb;  // G^{k1}, G^{k2} block bases
  int64_t z;       // Zcat base of the aux block: Zcat[((tau - t_chunk)*qb + P)*zld + zcol + p*b2 + m]
  int32_t sa, sb;  // (t, s) strides of the G slices
  int32_t b1, b2, qb, s;
  int32_t zld, zcol;
};

// Vcat[Q][K] = V_c[Q][(p, m)] at the same K columns as Zcat (one entry per (contribution, spin)).
struct VcTask {
  int64_t v;        // V block
  int64_t vc;       // Vcat base of the aux block: Vcat[Q*zld + zcol + pm]
  int32_t qb, b1b2, zld, zcol;
};

// Split-K tcgen05 GEMM tile: rows (tau, P) of one aux block, a K slice; FP64
// partial sums go to Ppart[part + r*qb + Q] and are summed in slice order.
struct PkTile {
  int64_t z;        // Zcat base of the block
  int64_t vc;       // Vcat base of the block
  int64_t part;     // partial-sum base of this (tile, slice)
  int32_t zld;      // K row length (complex, multiple of 16)
  int32_t qb;
  int32_t t0, nt;   // tau range, nt * qb <= 128
  int32_t kc0, kcn; // K slice in 16-complex chunks
  int32_t np;       // pad16(2 qb)
  int32_t pad;
};

// Reduction of the slices of one (aux block, tau range) into P0.
struct PrTile {
  int64_t part;     // first slice of the tile
  int64_t pout;     // P0 block base at tau = 0
  int32_t pstride, qb;
  int32_t t0, nt;
  int32_t nslice;
  int32_t pad;
};

// One tau chunk [tau0, tau1) of the P0 stages: Z tasks, the GEMM tiles of the
// chunk, then the ordered sums of the chunk's slices (rtiles).
void launch_p0_tc(bool bf16, const PzTask *ztasks, int nz, int zsmem, const PkTile *ktiles, int nk, const PrTile *rtiles,
                  int nr, const double2 *V, const double2 *G, float2 *Z, const float2 *Vcat, double2 *Ppart,
                  double2 *P0, int ns, int nts, int tau0, int tau1, double pref, int mirror, int *err,
                  cudaStream_t st);

void launch_vcat(const VcTask *tasks, int ntasks, const double2 *V, float2 *Vcat, cudaStream_t st);

// Runs the bounded-wait test kernel; returns 1 when the wait ran out.
int run_wait_timeout_test(int polls);

}  // namespace gwgb
