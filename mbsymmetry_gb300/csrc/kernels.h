// Launchers of the GW engine kernels (host side).
#pragma once

#include "common.h"

namespace gwgb {

// Largest irrep block (AO or aux) the FP64 kernels accept.
constexpr int MAX_BLOCK = 64;

// Block inverses: one warp per block; as many warps per CTA as fit in ~48 KB
// of shared memory (2 n^2 complex + 3 n ints per warp), 1 to 8.
__host__ __device__ constexpr int inv_bytes_per_warp(int nmax) { return 2 * nmax * nmax * 16 + 3 * nmax * 4; }
__host__ __device__ constexpr int inv_warps_per_block(int nmax) {
  return (48 * 1024) / inv_bytes_per_warp(nmax) < 1 ? 1
         : ((48 * 1024) / inv_bytes_per_warp(nmax) > 8 ? 8 : (48 * 1024) / inv_bytes_per_warp(nmax));
}
__host__ __device__ constexpr int inv_smem_bytes(int nmax) {
  return inv_warps_per_block(nmax) * inv_bytes_per_warp(nmax);
}
__host__ __device__ constexpr int rotate_smem_bytes(int nmax) { return 3 * nmax * nmax * 16; }

void set_fp64_kernel_attributes(int smem_bytes);
// The shared-memory limits of the two block-inverse kernels only (sizes fixed by MAX_BLOCK).
void set_inverse_kernel_attributes();

// FP64 contractions: each tile writes its partial block to Part[tile.part];
// launch_reduce_slices then sums the slices in order into P0 / Sigma.
void launch_p0_fp64(const P0Tile *tiles, int ntiles, int maxo, const P0Contrib *contribs,
                    const double2 *V, const double2 *G, double2 *Part, int ns, int nts, int smem_bytes,
                    cudaStream_t st);

void launch_sigma_fp64(const SigTile *tiles, int ntiles, int maxo, const SigContrib *contribs,
                       const double2 *V, const double2 *G, const double2 *P, double2 *Part, int ns,
                       int smem_bytes, cudaStream_t st);

// ny: CTAs per task (each takes every ny-th 256-element stretch of the block)
void launch_reduce_slices(const RedTask *tasks, int ntasks, const double2 *part, double2 *out, int nts,
                          double scale, int mirror, cudaStream_t st, int ny = 1);

void launch_rotate(const RotTask *tasks, int ntasks, int nbatch, int smem_bytes, const double2 *src,
                   const double2 *O, double2 *dst, cudaStream_t st);

// Vt = op(O)^T V for every Sigma contribution (VrTask).
void launch_vrot(const VrTask *tasks, int ntasks, const double2 *V, const double2 *O, double2 *Vt, cudaStream_t st);

void launch_mirror(double2 *P, const int64_t *qoff, const int32_t *qsz, int nq, int nts, cudaStream_t st);
void launch_zero_upper(double2 *P, const int64_t *qoff, const int32_t *qsz, int nq, int nts, cudaStream_t st);

void launch_transform(const TSlab *slabs, int nslabs, int max_cols, const double2 *T, int nout, int nin,
                      int row0, const double2 *X, double2 *Y, cudaStream_t st);

// Batched block inverses.  mode 0: W~ (R = sym((1 - sym(P))^-1), R P); mode 1:
// Dyson ((mu + i w_n) S - F - Sigma)^-1.  Optional: mu read from *mu_ptr,
// output to Wout instead of in place, nothing done while *skip != 0.
void launch_inverse(const InvTask *tasks, int ntasks, int nmax, double2 *W, const double2 *S,
                    const double2 *F, const int64_t *wsample, double beta, double mu, int mode, int *bad,
                    cudaStream_t st, const double *mu_ptr = nullptr, double2 *Wout = nullptr,
                    const int *skip = nullptr);

void launch_leakage(const TSlab *slabs, int nslabs, const double2 *G, const double *tf, const double *tl,
                    int ncheb, unsigned long long *out, cudaStream_t st);

// Hartree term: c over the aux blocks of q = 0, then J over the AO blocks of the stored k.
void launch_hartree(const HcTask *ct, int nct, const HcItem *ci, const HjTask *jt, int njt, const HjItem *ji,
                    const double2 *V, const double2 *G, int ns, double scale, double2 *c, double2 *J,
                    cudaStream_t st);

}  // namespace gwgb
