// Error-free sliced contractions on tcgen05 ("BF16 x4 fixed-point slices"):
// work descriptors and launchers.
//
// Every contraction stage of the GW iteration (P0: Z1, Z, P0; Sigma: W, U,
// Sigma) is a batch of complex GEMMs C = A B^T over the irrep blocks.  Here
// they all run through one grouped persistent kernel (oz_gemm_kernel) whose
// tasks are (descriptor, repetition, row tile, column tile).  Operands are
// "float-float" complex numbers: float4 {re_hi, im_hi, re_lo, im_lo}, value
// (re_hi + re_lo) + i (im_hi + im_lo), about 48 significant bits.
#pragma once

#include "common.h"

namespace gwgb {

// Row map of an operand or of the output: local row r (of the whole descriptor,
// not of a tile) -> base + (r / d) * s1 + (r % d) * s0 (complex elements), or,
// with d == 0, -> rowtab[base + r] (a table of row offsets).
struct OzRows {
  int64_t base;
  int64_t s1;
  int32_t s0;
  int32_t d;
};

constexpr int OZ_CONJ_A = 1;  // A read conjugated
constexpr int OZ_CONJ_B = 2;  // B read conjugated
constexpr int OZ_OUT_F64 = 4; // C written as complex FP64, alpha * value (else float-float)

// C[r][n] = sum_k A[r][k] B[n][k] for r < M, n < N, k < K (complex).
//   A[r][k] at A + a(r) + k * aks + rep * ra, B[n][k] at B + b(n) + k * bks + rep * rb,
//   C[r][n] at C + c(r) + (n / cnd) * cn1 + (n % cnd) * cn0 + rep * rc.
// Every output element is written by exactly one task (no accumulation across
// tasks), so the result is independent of the launch order.
struct OzDesc {
  OzRows a, b, c;
  int64_t cn1;
  int64_t ra, rb, rc;
  double alpha;      // OZ_OUT_F64 only
  int32_t cn0, cnd;
  int32_t aks, bks;
  int32_t M, N, K;
  int32_t flags;
};

// One CTA work item: rows [128 mt, 128 mt + 128) and complex columns
// [32 nt, 32 nt + 32) of descriptor `desc` at repetitions [rep0, rep0 + nrep)
// (independent GEMMs done one after the other); mtnt = mt << 16 | nt.
struct OzTask {
  int32_t desc, rep0, nrep, mtnt;
};

// Element copy of a [X][Y][Z] block into float-float form at
//   dst + x * dx + y * dy + z * dz (optionally conjugated): builds the
// tau-independent operands (concatenated V blocks, their transposes) once per
// V / rotation upload.
struct OzPerm {
  int64_t src, dst;
  int64_t dx, dy, dz;
  int32_t X, Y, Z;
  int32_t conj;
};

// Tile geometry (shared with the host's work-list checks).
constexpr int OZ_M = 128;   // rows per tile (TMEM lanes)
constexpr int OZ_NC = 32;   // complex columns per tile
constexpr int OZ_KR = 16;   // complex K per round (one slicing exponent per row and round)

void set_oz_kernel_attributes();

// All tasks of one stage in one persistent launch (two CTAs per SM, tasks
// taken in list order with a stride of the grid size).  err: set to 1 when a
// bounded tensor-core completion wait ran out.
void launch_oz_gemm(const OzDesc *descs, const OzTask *tasks, int ntasks, const float4 *A, const float4 *B, void *C,
                    const int64_t *rowtab, int nsm, int *err, cudaStream_t st);

// The same tasks on the CUDA cores in float-float arithmetic (one CTA per task):
// for block GEMMs with few output columns.
void launch_oz_simt(const OzDesc *descs, const OzTask *tasks, int ntasks, const float4 *A, const float4 *B, void *C,
                    const int64_t *rowtab, cudaStream_t st);

// y[i] = float-float(x[i]) for n complex elements.
void launch_to_ffc(const double2 *x, float4 *y, int64_t n, cudaStream_t st);

void launch_oz_perm(const OzPerm *tasks, int ntasks, const double2 *src, float4 *dst, cudaStream_t st);

}  // namespace gwgb
