// Shared host/device definitions of the GB300 GW engine.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <stdexcept>
#include <string>

#include "../../include/gwgb.h"

namespace gwgb {

// Sets the thread-local message returned by gwgb_last_error().
void set_last_error(const std::string &msg);

// Error carrying a gwgb status code; the C ABI turns it into a return value.
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

#define GWGB_CUDA(call)                                                                     \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess)                                                                  \
      throw ::gwgb::Error(e_ == cudaErrorMemoryAllocation ? GWGB_E_NOMEM : GWGB_E_CUDA,     \
                          std::string(#call) + ": " + cudaGetErrorString(e_));              \
  } while (0)

#define GWGB_REQUIRE(cond, code, msg)                                                       \
  do {                                                                                      \
    if (!(cond)) throw ::gwgb::Error((code), (msg));                                        \
  } while (0)

// ---------------------------------------------------------------------------
// Work descriptors of the contraction kernels.  Offsets are in complex
// elements.  A G block of k is addressed as  base + (t*ns + s)*stride.
// ---------------------------------------------------------------------------

// One V block of one (k1, k2 = k1 + q) pair feeding a P0 output block.
struct P0Contrib {
  int64_t v;       // V block [qb][b1][b2]
  int64_t ga;      // G^{k1} block base
  int64_t gb;      // G^{k2} block base
  int32_t sa, sb;  // (t,s) strides of the two G slices
  int32_t b1, b2;  // block sizes at k1 and k2
};

// One P0 output block P0[q_irr][t][block iq] for a tau range.
struct P0Tile {
  int64_t p;        // offset of the block at t = 0 in the P0 buffer
  int64_t part;     // FP64 path: this tile's partial-sum slice [nt][qb][qb]
  int32_t pstride;  // per-t stride (qslice size)
  int32_t qb;       // aux block size
  int32_t c0, c1;   // contribution range
  int32_t t0, nt;   // tau range [t0, t0 + nt)
  int32_t cost;     // relative cost (for ordering only)
  int32_t pad;
};

// One V block of one (k1, k2 = k1 - q) pair feeding a Sigma output block.
struct SigContrib {
  int64_t v;        // pre-rotated V block Vt [qb][b1][b2] (in the Vt buffer)
  int64_t gb;       // G^{k2} block base
  int64_t pq;       // block of P~ of the irreducible q' at t = 0
  int32_t sb;       // (t,s) stride of the G^{k2} slice
  int32_t pstride;  // per-t stride of P~(q')
  int32_t b2, qb;
  int32_t pconj;    // read conj(P~(q')) (q is a time-reversal partner)
  int32_t pad;
};

// Vt = op(O)^T V over the aux index of one Sigma contribution: Vt[Q'][x] =
// sum_Q op(O[Q][Q']) V[Q][x], op = conj for a time-reversal partner; o < 0:
// Vt = V.  With it, V P~(q) V^H = Vt P~(q') Vt^H for P~(q) = O P~(q') O^H.
struct VrTask {
  int64_t v, vt;    // source V block, target Vt block
  int64_t o;        // auxrep block (qb x qb) or -1
  int32_t qb, b1b2;
  int32_t conj, pad;
};

// One Sigma output block Sigma[t][s][k_irr block ik1] for a tau range.
struct SigTile {
  int64_t sig;        // offset of the block at t = 0, spin s
  int64_t part;       // FP64 path: this tile's partial-sum slice [nt][b1][b1]
  int32_t sstride;    // per-t stride (ns * flat_ao)
  int32_t b1;
  int32_t c0, c1;
  int32_t t0, nt;
  int32_t s, cost;
  int32_t ntq;        // tcgen05 U/Sigma tiles: the tau count the aux-row chunks are sized
                      // for (the owner's, so the K steps never depend on the tau chunking)
  int32_t pad;
};

// Rotation task: dst = O * src * O^H per (batch index), optionally conjugated;
// or a plain copy (+conj) of a slice when rotate == 0.
struct RotTask {
  int64_t dst;       // destination base at batch 0
  int64_t src;       // source base at batch 0
  int64_t o;         // rotation block offset (rotate == 1)
  int32_t dstride;   // per-batch strides
  int32_t sstride;
  int32_t m, n;      // O is m x n; src block n x n; dst block m x m (copy: m = element count)
  int32_t rotate, conj;
};

// Slab of a tau <-> omega transform: Y[r][c] = sum_i T[r][i] X[x_row0 + i][c].
struct TSlab {
  int64_t x;     // offset of X row 0 (before x_row0 is applied)
  int64_t y;     // offset of Y row 0
  int32_t ldx;   // row strides
  int32_t ldy;
  int32_t ncols;
  int32_t pad;
};

// One small dense block for a batched inverse.
// Ordered sum of the contribution slices of one output block over a tau range:
//   out[(t0 + it) * ostride + e] = scale * sum_sl part[(sl * nt + it) * elems + e]
// and, when mirroring (P0), the same value at tau' = nts - 1 - tau.
struct RedTask {
  int64_t part;     // first slice
  int64_t out;      // output block at tau = 0
  int32_t ostride;  // per-tau stride of the output
  int32_t elems;    // elements of the block
  int32_t t0, nt;
  int32_t nslice;
  int32_t pad;
};

struct InvTask {
  int64_t a;       // matrix offset (row-major n x n) in the work buffer
  int64_t s, f;    // Dyson: S and F block offsets (in the [ns][flat_ao] buffers)
  int32_t n;
  int32_t w;       // frequency index (Dyson) or -1
};

// Hartree (direct) term of HF on the block layout, from q = 0 V blocks:
//   c[Q] = scale sum_{k', s} sum_{a,b} V^Q_ab(k', k') rho_s(k')_ba,
//   J(k)_ij = sum_Q V^Q_ij(k, k) c[Q]   (diagonal AO blocks, i1 = i2).
struct HcItem {    // one V block of pair (k', k') and rho(k') of its AO block
  int64_t v;       // V block [qb][b][b]
  int64_t g;       // rho block at spin 0 (G at tau = 0)
  int32_t gstride; // spin stride of G
  int32_t b;
};
struct HcTask {    // c over one aux block of q = 0: items [i0, i1) summed in order
  int64_t cout;
  int32_t qb, i0, i1, pad;
};
struct HjItem {    // one V block of pair (k, k) and its aux block's c
  int64_t v;
  int64_t c;
  int32_t qb, pad;
};
struct HjTask {    // J over one AO block of a stored k: items [i0, i1) summed in order
  int64_t out;
  int32_t b, i0, i1, pad;
};

}  // namespace gwgb
