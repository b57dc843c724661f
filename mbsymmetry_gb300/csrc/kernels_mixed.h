// Launchers of the mixed-precision (TF32 3-pass) contraction kernels.
#pragma once

#include "common.h"

namespace gwgb {

void set_mixed_kernel_attributes(int smem_bytes);

void launch_p0_mixed(const P0Tile *tiles, int ntiles, const P0Contrib *contribs, const double2 *V,
                     const double2 *G, double2 *P0, int ns, int nts, double pref, int mirror, int smem_bytes,
                     cudaStream_t st);

void launch_sigma_mixed(const SigTile *tiles, int ntiles, const SigContrib *contribs, const double2 *V,
                        const double2 *G, const double2 *P, double2 *Sig, int ns, double scale, int smem_bytes,
                        cudaStream_t st);

}  // namespace gwgb
