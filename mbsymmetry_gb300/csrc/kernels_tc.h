// tcgen05 (TMEM) mixed-precision contraction kernels: work descriptors and launchers.
#pragma once

#include "common.h"

namespace gwgb {

// One CTA of the Sigma W-GEMM: 128 rows (tau, Q) of one aux block (q, iq)
// times a pack of contribution columns (c, j, n).
struct SwTile {
  int64_t pa;       // P(q) block base at tau = 0
  int32_t pstride;  // per-tau stride of P(q)
  int32_t qb;
  int32_t t0, nt;   // tau range; nt * qb <= 128
  int32_t c0, c1;   // SwCol range
  int32_t ncol;     // complex columns of the pack
  int32_t kp, np;   // padded real K (pad8(2 qb)) and real N (pad16(2 ncol))
  int32_t pad;
};

// A contiguous range of the flattened (j, n) columns of one contribution.
struct SwCol {
  int64_t v;        // V block [qb][b1][b2]
  int64_t w;        // W_c base: W[((tau*qb + Q)*b1 + j)*b2 + n]
  int32_t b1, b2;
  int32_t l0;       // first flattened column (j*b2 + n) of the range
  int32_t col0;     // first pack column of the range
};

void set_tc_kernel_attributes(int smem_bytes);
void set_tc_p0_kernel_attributes(int smem_bytes);

void launch_sigma_tc(const SwTile *wtiles, int nwtiles, int wsmem, const SwCol *wcols, const SigTile *tiles1,
                     int ntiles1, const SigContrib *contribs, const int64_t *woff, const double2 *V,
                     const double2 *G, const double2 *P, float2 *W, double2 *Sig, int ns, double scale,
                     int uv_smem, int *err, cudaStream_t st);

}  // namespace gwgb

namespace gwgb {

// P0, stage Z: one CTA per (contribution, spin) over all tau < nts/2.
struct PzTask {
  int64_t v;       // V block [qb][b1][b2]
  int64_t ga, gb;  // G^{k1}, G^{k2} block bases
  int64_t z;       // Z base: Z[((tau*qb + P)*b1 + p)*b2 + m]
  int32_t sa, sb;  // (t, s) strides of the G slices
  int32_t b1, b2, qb, s;
};

// P0, tcgen05 stage: one CTA per (q_irr, aux block, tau range of nt*qb <= 128 rows).
struct PtTile {
  int64_t pout;     // P0 block base at tau = 0
  int32_t pstride;
  int32_t qb;
  int32_t t0, nt;
  int32_t k0, k1;   // PtChunk range (all contributions of the block, split in K chunks)
  int32_t np;       // pad16(2 qb)
  int32_t pad;
};

// A K chunk: columns [kc0, kc0 + kn) of the flattened (p, m) index of one (contribution, spin).
struct PtChunk {
  int64_t z;        // Z base of the (contribution, spin)
  int64_t v;        // V block base
  int32_t b1b2;     // row length of Z and of V[Q]
  int32_t kc0, kn;
  int32_t pad;
};

void launch_p0_tc(const PzTask *ztasks, int nz, int zsmem, const PtTile *ptiles, int npt, int psmem,
                  const PtChunk *chunks, const double2 *V, const double2 *G, float2 *Z, double2 *P0, int ns,
                  int nts, double pref, int mirror, int drain_every, int *err, cudaStream_t st);

}  // namespace gwgb
