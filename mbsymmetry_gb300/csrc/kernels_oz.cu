// Error-free sliced complex GEMMs on tcgen05 for the P0 and Sigma stages.
//
// Why: a TF32/BF16 split with FP32 accumulation carries about 24 bits, and the
// GW contractions sum many terms of both signs, so their error stays near
// 1e-6 relative -- far from 1e-7 Ha absolute on Sigma.  Here each operand row
// is cut, per round of OZ_KR complex K, into four BF16 slices of a fixed-point
// representation (the Ozaki scheme: Ozaki, Ogita, Oishi, Rump, Numer. Algor.
// 59 (2012) 95-118; Ootomo, Ozaki, Yokota, IJHPCA 2024):
//   x = 2^(E-7) (s0 + s1 2^-8 + s2 2^-16 + s3 2^-24) + O(2^(E-32)),
//   E: the row's exponent (|x| < 2^E), s_i integers with |s_i| <= 129,
// stored as BF16 values s_i 2^(-8 i) (exact: 8 significant bits).  The
// product of two such rows is a sum of slice products whose class c = i + j
// carries weight 2^(-8 c); the classes 0 to 3 are computed (10 MMAs per K
// step) into three TMEM accumulators:
//   D0 = class 0 (s0 t0: integers <= 2^14 per term, a round's sum < 2^20),
//   D1 = class 1 (integer multiples of 2^-8 below 2^13 per term),
//   D2 = classes 2 and 3 (below 2^-2 per term),
// so D0 and D1 are exact in FP32 and D2's rounding lies near 2^-40 of the
// row-by-column scale.  Dropped terms (classes 4 to 6) and the slice
// remainder are below 2^-30 of that scale.  After every round the three
// accumulators are combined, scaled by 2^(Ea + Eb - 14) (exact) and added to
// a float-float accumulator (two FP32 numbers, about 48 bits) in registers.
// No FP64 arithmetic runs in the GEMM except the final conversion of
// FP64-valued outputs.  Complex products use the real embedding
//   A = [Ar Ai] (K interleaved), B rows (n, 0) = [Br -Bi], (n, 1) = [Bi Br],
// so C[r][(n,0)] = Re, C[r][(n,1)] = Im of sum_k A[r][k] B[n][k].
//
// Kernel structure: persistent, two CTAs per SM (80 KB shared memory and 256
// TMEM columns each), 128 threads; tasks in list order with a grid stride.
// Per round every thread stages one A row (max, exponent, slices: K-major
// no-swizzle core-matrix layout), four threads stage one complex B row (two
// real rows), one thread issues the 20 MMAs and commits to an mbarrier, all
// threads wait (bounded) and drain their TMEM lane.  The other CTA on the SM
// overlaps its staging and drain with these MMAs.
#include "common.h"
#include "kernels_oz.h"
#include <cuda_bf16.h>

#include "tc_common.cuh"

namespace gwgb {

namespace {

constexpr int OZ_NR = 2 * OZ_NC;            // real columns (rows of the real-embedded B)
constexpr int OZ_KP = 2 * OZ_KR;            // real K per round (BF16 elements per operand row)
constexpr int OZ_SBO = (OZ_KP / 8) * 128;   // bytes between 8-row groups of core matrices
constexpr int OZ_PA = OZ_M * OZ_KP * 2;     // bytes of one A slice plane
constexpr int OZ_PB = OZ_NR * OZ_KP * 2;    // bytes of one B slice plane
constexpr int OZ_EMIN = -100, OZ_EMAX = 100;
static_assert(OZ_KP % 16 == 0, "a round is a whole number of BF16 MMA K steps");

// E with |x| < 2^E for every |x| <= m (m >= 0), clamped to [OZ_EMIN, OZ_EMAX].
__device__ __forceinline__ int oz_exponent(float m) {
  const int e = (int)((__float_as_uint(m) >> 23) & 0xff) - 126;  // m = f 2^e, f in [0.5, 1)
  if (!(m > 0.f) || e < OZ_EMIN) return OZ_EMIN;
  return e > OZ_EMAX ? OZ_EMAX : e;
}

// 2^e as a float for e in [-126, 127]; 0 below (the term underflows).
__device__ __forceinline__ float oz_pow2(int e) {
  if (e < -126) return 0.f;
  return __uint_as_float((uint32_t)(e > 127 ? 254 : e + 127) << 23);
}

// Four fixed-point slices of x = hi + lo in units of 2^(E-7) (f = 2^(7-E)),
// returned with their weights: s0, s1 2^-8, s2 2^-16, s3 2^-24.
__device__ __forceinline__ void oz_slice(float hi, float lo, float f, float (&s)[4]) {
  const float h = hi * f, l = lo * f;  // exact scalings
  const float s0 = rintf(h);
  const float r = h - s0;              // exact, |r| <= 1/2
  const float rh = r + l;              // two-sum of r and l
  const float bb = rh - r;
  const float rl = (r - (rh - bb)) + (l - bb);
  const float t1 = rh * 256.f;
  const float s1 = rintf(t1);
  const float t2 = ((t1 - s1) + rl * 256.f) * 256.f;
  const float s2 = rintf(t2);
  const float s3 = rintf((t2 - s2) * 256.f);
  s[0] = s0;
  s[1] = s1 * 0x1p-8f;
  s[2] = s2 * 0x1p-16f;
  s[3] = s3 * 0x1p-24f;
}

__device__ __forceinline__ uint32_t bf2(float lo_elem, float hi_elem) {
  return (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(lo_elem)) |
         ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(hi_elem)) << 16);
}

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// (h, l) += (vh, vl), float-float addition.
__device__ __forceinline__ void ff_add(float &h, float &l, float vh, float vl) {
  float s, e;
  two_sum(h, vh, s, e);
  e += l + vl;
  h = s + e;
  l = e - (h - s);
}

// Byte offset of the 16-byte row segment (8 BF16 elements from real column k8,
// a multiple of 8) of row r in a K-major no-swizzle tile.
__device__ __forceinline__ uint32_t seg_off(int r, int k8) {
  return (uint32_t)((r >> 3) * OZ_SBO + (k8 >> 3) * 128 + (r & 7) * 16);
}

// Offset of local row r of a row map (d == 0: from the row table).
__device__ __forceinline__ int64_t row_off(const OzRows &m, int r, const int64_t *__restrict__ rowtab) {
  if (m.d == 0) return __ldg(rowtab + m.base + r);
  if (m.d == 1) return m.base + (int64_t)r * m.s1;
  return m.base + (int64_t)(r / m.d) * m.s1 + (int64_t)(r % m.d) * m.s0;
}

// 32 lanes x 8 consecutive 32-bit columns from registers into TMEM (this warp's lane quarter).
__device__ __forceinline__ void tmem_st8(uint32_t taddr, const float (&v)[8]) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(taddr),
               "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])),
               "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])),
               "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7]))
               : "memory");
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

constexpr int OZ_THREADS = 512;         // warps 0-7 drain (TMEM lanes), 8-15 stage; lane 0 of warp 8 issues MMAs
constexpr int OZ_ACC = 3 * OZ_NR;       // TMEM columns of one accumulator set D0 | D1 | D2
constexpr int OZ_TMEM_WS = 512;         // two accumulator sets, then the float-float sums (hi | lo)
constexpr int OZ_SUM = 2 * OZ_ACC;      // TMEM column of the running sums of multi-round GEMMs
constexpr int OZ_BUF = 4 * OZ_PA + 4 * OZ_PB;
constexpr int OZ_SMEM_WS = 120 * 1024;  // two tile buffers (96 KB); more than half an SM: one CTA per SM
static_assert(2 * OZ_BUF + 1024 <= OZ_SMEM_WS, "two tile buffers must fit the requested shared memory");
static_assert(2 * OZ_ACC + 2 * OZ_NR <= OZ_TMEM_WS, "two accumulator sets and the sums must fit the TMEM allocation");

// Combined, scaled value of one accumulator column: (D0 + D1 + D2) * sc as a
// float-float pair (D0, D1 exact; D2 small).
__device__ __forceinline__ void oz_combine(float x0, float x1, float x2, float sc, float &h, float &l) {
  float vh, vl;
  two_sum(x0, x1, vh, vl);
  vl += x2;
  h = vh + vl;
  l = (vl - (h - vh)) * sc;
  h *= sc;
}

__device__ __forceinline__ void oz_store(void *Cg, int64_t o, bool f64, double alpha, float rh, float ih, float rl,
                                         float il) {
  if (f64)
    reinterpret_cast<double2 *>(Cg)[o] =
        make_double2(alpha * ((double)rh + (double)rl), alpha * ((double)ih + (double)il));
  else
    reinterpret_cast<float4 *>(Cg)[o] = make_float4(rh, ih, rl, il);
}

// Persistent warp-specialised sliced GEMM.  Every role walks the same work
// sequence (tasks of this CTA with a grid stride, repetitions, rounds of
// OZ_KR complex K), counting rounds i.  Rings: 2 shared tile buffers
// (full / empty), 2 TMEM accumulator sets (done / afree), 4 exponent slots
// (eready / efree).  Every wait is bounded; a wait that runs out sets the error
// word and an abort flag that ends every role's loop, and TMEM is released only
// after the MMAs issued so far have completed (bounded wait on `last`).
__global__ void __launch_bounds__(OZ_THREADS, 1)
    oz_gemm_kernel(const OzDesc *__restrict__ descs, const OzTask *__restrict__ tasks, int ntasks,
                   const float4 *__restrict__ Ag, const float4 *__restrict__ Bg, void *__restrict__ Cg,
                   const int64_t *__restrict__ rowtab, int *__restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint32_t tslot;
  __shared__ __align__(8) uint64_t full[2], empty[2], done[2], afree[2], eready[4], efree[4], last;
  __shared__ int ea_s[4][OZ_M], eb_s[4][OZ_NC];
  __shared__ float amax[2][2][OZ_M];  // per tile buffer: partial row maxima of the two A halves
  __shared__ __align__(8) uint64_t mx[2];
  __shared__ int abort_flag, issued;
  const int tid = threadIdx.x, warp = tid >> 5;
  if (warp == 0) tc::tmem_alloc(&tslot, OZ_TMEM_WS);
  if (tid == 0) {
    for (int j = 0; j < 2; ++j) {
      tc::mbar_init(&full[j], 256);
      tc::mbar_init(&empty[j], 1);
      tc::mbar_init(&done[j], 1);
      tc::mbar_init(&afree[j], 256);
    }
    for (int j = 0; j < 4; ++j) {
      tc::mbar_init(&eready[j], 256);
      tc::mbar_init(&efree[j], 256);
    }
    tc::mbar_init(&last, 1);
    tc::mbar_init(&mx[0], 256);
    tc::mbar_init(&mx[1], 256);
    abort_flag = 0;
    issued = 0;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tm = tslot;
  // bounded wait; false when it ran out (error word and abort flag set) or another role aborted.
  // Each poll may suspend the thread for up to 20 us (hint) until the phase completes, so
  // waiting roles do not take issue slots from the working ones; 2^16 polls bound the wait.
  auto bwait = [&](uint64_t *b, uint32_t par) -> bool {
    for (int rep = 0; rep < 256; ++rep) {
      for (int it = 0; it < 256; ++it) {
        uint32_t ok;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\nselp.b32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(tc::smem_u32(b)), "r"(par), "r"(20000u)
            : "memory");
        if (ok) return true;
      }
      if (*(volatile int *)&abort_flag) return false;
    }
    atomicExch(err, 1);
    *(volatile int *)&abort_flag = 1;
    return false;
  };
  auto aborted = [&]() { return *(volatile int *)&abort_flag != 0; };
  // Every stop decision is taken by the whole warp (the tcgen05 loads, the
  // shuffles and the warp barrier of the staging loop need all 32 lanes): a
  // warp stops when any lane saw the abort flag or a wait that ran out.  Each
  // lane's wait is bounded, so the votes end, and a timed-out wait can never
  // leave part of a warp waiting for lanes that left the loop.
  auto warp_aborted = [&]() { return __any_sync(0xffffffffu, aborted()); };
  auto warp_ok = [&](bool ok) { return __all_sync(0xffffffffu, ok); };

  if (warp >= 8) {
    // ------------------------------ producers (and the MMA issuer) ------------------------------
    // A: two threads per row (h = K half); B: eight threads per complex row (two complex K each).
    const int pt = tid - 256;
    const int ar = pt & 127, ah = pt >> 7;
    const int bn = pt >> 3, bq = pt & 7;
    int i = 0, nissued = 0;
    bool stop = false;
    for (int ti = blockIdx.x; ti < ntasks && !stop; ti += gridDim.x) {
      const OzTask tk = tasks[ti];
      const OzDesc dg = descs[tk.desc];
      const int mt = tk.mtnt >> 16, nt = tk.mtnt & 0xffff;
      const int Mt = min(OZ_M, dg.M - mt * OZ_M), Nt = min(OZ_NC, dg.N - nt * OZ_NC);
      const int ngrp = (Nt + 7) >> 3;
      const bool rv = ar < Mt, bv = bn < Nt, bw = bn < 8 * ngrp;
      const int64_t arow0 = rv ? row_off(dg.a, mt * OZ_M + ar, rowtab) : 0;
      const int64_t brow0 = bv ? row_off(dg.b, nt * OZ_NC + bn, rowtab) : 0;
      const bool ca = dg.flags & OZ_CONJ_A, cb = dg.flags & OZ_CONJ_B;
      for (int rr = 0; rr < tk.nrep && !stop; ++rr) {
        const int rep = tk.rep0 + rr;
        const float4 *arow = Ag + arow0 + (int64_t)rep * dg.ra;
        const float4 *brow = Bg + brow0 + (int64_t)rep * dg.rb;
        for (int k0 = 0; k0 < dg.K; k0 += OZ_KR, ++i) {
          if (warp_aborted()) { stop = true; break; }
          const int b = i & 1, e = i & 3;
          if (i >= 2 && !warp_ok(bwait(&empty[b], ((i >> 1) - 1) & 1))) { stop = true; break; }
          if (i >= 4 && !warp_ok(bwait(&efree[e], ((i >> 2) - 1) & 1))) { stop = true; break; }
          const int kn = min(OZ_KR, dg.K - k0);
          const int nks = (kn + 7) >> 3;  // MMA K steps this round (8 complex each)
          const int kw = 4 * nks;         // complex K per thread of an A row (4 or 8)
          unsigned char *As = smem + b * OZ_BUF, *Bs = As + 4 * OZ_PA;
          {  // A: this thread's half [kw h, kw h + kw) of row ar; exponent from both halves
            float4 v[8];
            float m = 0.f;
#pragma unroll
            for (int k = 0; k < 8; ++k) {
              const int kk = kw * ah + k;
              v[k] = make_float4(0.f, 0.f, 0.f, 0.f);
              if (rv && k < kw && kk < kn) v[k] = __ldg(arow + (int64_t)(k0 + kk) * dg.aks);
              m = fmaxf(m, fmaxf(fabsf(v[k].x), fabsf(v[k].y)));
            }
            amax[b][ah][ar] = m;
            tc::mbar_arrive(&mx[b]);  // both halves' maxima posted (bounded wait, no named barrier)
            if (!warp_ok(bwait(&mx[b], (i >> 1) & 1))) { stop = true; break; }
            const int ea = oz_exponent(fmaxf(amax[b][0][ar], amax[b][1][ar]));
            const float f = oz_pow2(7 - ea);
#pragma unroll
            for (int g = 0; g < 2; ++g) {  // segments of 4 complex (8 reals per plane)
              if (4 * g < kw) {
                uint32_t w[4][4];
                if (rv) {
#pragma unroll
                  for (int j = 0; j < 4; ++j) {
                    float4 x = v[g * 4 + j];
                    if (ca) { x.y = -x.y; x.w = -x.w; }
                    float sr[4], si[4];
                    oz_slice(x.x, x.z, f, sr);
                    oz_slice(x.y, x.w, f, si);
#pragma unroll
                    for (int p = 0; p < 4; ++p) w[p][j] = bf2(sr[p], si[p]);
                  }
                } else {
#pragma unroll
                  for (int p = 0; p < 4; ++p) w[p][0] = w[p][1] = w[p][2] = w[p][3] = 0u;
                }
                const uint32_t o = seg_off(ar, 8 * (kw * ah / 4 + g));
#pragma unroll
                for (int p = 0; p < 4; ++p)
                  *reinterpret_cast<uint4 *>(As + p * OZ_PA + o) = make_uint4(w[p][0], w[p][1], w[p][2], w[p][3]);
              }
            }
            if (ah == 0) ea_s[e][ar] = ea;
          }
          {  // B: rows (n,0) = [Br -Bi], (n,1) = [Bi Br]; complex K [2 bq, 2 bq + 2) of row bn
            float4 v[2];
            float mb = 0.f;
#pragma unroll
            for (int j = 0; j < 2; ++j) {
              const int k = 2 * bq + j;
              v[j] = make_float4(0.f, 0.f, 0.f, 0.f);
              if (bv && k < kn) v[j] = __ldg(brow + (int64_t)(k0 + k) * dg.bks);
              if (cb) { v[j].y = -v[j].y; v[j].w = -v[j].w; }
              mb = fmaxf(mb, fmaxf(fabsf(v[j].x), fabsf(v[j].y)));
            }
            mb = fmaxf(mb, __shfl_xor_sync(0xffffffffu, mb, 1));
            mb = fmaxf(mb, __shfl_xor_sync(0xffffffffu, mb, 2));
            mb = fmaxf(mb, __shfl_xor_sync(0xffffffffu, mb, 4));
            const int eb = oz_exponent(mb);
            if (bq == 0) eb_s[e][bn] = eb;
            if (bw && 2 * bq < 8 * nks) {
              uint32_t w0[4][2], w1[4][2];
              if (bv) {
                const float f = oz_pow2(7 - eb);
#pragma unroll
                for (int j = 0; j < 2; ++j) {
                  float sr[4], si[4];
                  oz_slice(v[j].x, v[j].z, f, sr);
                  oz_slice(v[j].y, v[j].w, f, si);
#pragma unroll
                  for (int p = 0; p < 4; ++p) {
                    w0[p][j] = bf2(sr[p], -si[p]);
                    w1[p][j] = bf2(si[p], sr[p]);
                  }
                }
              } else {
#pragma unroll
                for (int p = 0; p < 4; ++p) w0[p][0] = w0[p][1] = w1[p][0] = w1[p][1] = 0u;
              }
              // 8-byte halves of the 16-byte core-matrix row segments of complex K [4 (bq/2), +4)
              const uint32_t o0 = seg_off(2 * bn, 8 * (bq >> 1)) + 8 * (bq & 1);
              const uint32_t o1 = seg_off(2 * bn + 1, 8 * (bq >> 1)) + 8 * (bq & 1);
#pragma unroll
              for (int p = 0; p < 4; ++p) {
                *reinterpret_cast<uint2 *>(Bs + p * OZ_PB + o0) = make_uint2(w0[p][0], w0[p][1]);
                *reinterpret_cast<uint2 *>(Bs + p * OZ_PB + o1) = make_uint2(w1[p][0], w1[p][1]);
              }
            }
          }
          tc::fence_async_smem();
          tc::mbar_arrive(&eready[e]);
          tc::mbar_arrive(&full[b]);
          if (pt == 0) {  // MMA issue for this round once all producers have staged it
            const int a = i & 1;
            bool ok = bwait(&full[b], (i >> 1) & 1);
            if (ok && i >= 2) ok = bwait(&afree[a], ((i >> 1) - 1) & 1);
            if (ok) {
              tc::fence_after_sync();
              const uint32_t id = tc::idesc_bf16(OZ_M, 16 * ngrp);
              const uint32_t a0 = tc::smem_u32(As), b0 = a0 + 4 * OZ_PA;
              const uint32_t d0 = tm + (uint32_t)(a * OZ_ACC), d1 = d0 + OZ_NR, d2 = d0 + 2 * OZ_NR;
              for (int ks = 0; ks < nks; ++ks) {
                auto da = [&](int p) { return tc::make_desc(a0 + p * OZ_PA + ks * 256, 128, OZ_SBO); };
                auto db = [&](int p) { return tc::make_desc(b0 + p * OZ_PB + ks * 256, 128, OZ_SBO); };
                const uint32_t acc = ks > 0 ? 1u : 0u;
                tc::mma_bf16(d0, da(0), db(0), id, acc);
                tc::mma_bf16(d1, da(0), db(1), id, acc);
                tc::mma_bf16(d1, da(1), db(0), id, 1u);
                tc::mma_bf16(d2, da(0), db(2), id, acc);
                tc::mma_bf16(d2, da(1), db(1), id, 1u);
                tc::mma_bf16(d2, da(2), db(0), id, 1u);
                tc::mma_bf16(d2, da(0), db(3), id, 1u);
                tc::mma_bf16(d2, da(1), db(2), id, 1u);
                tc::mma_bf16(d2, da(2), db(1), id, 1u);
                tc::mma_bf16(d2, da(3), db(0), id, 1u);
              }
              tc::commit(&empty[b]);
              tc::commit(&done[a]);
              ++nissued;
            }
          }
          __syncwarp();
        }
      }
    }
    if (pt == 0) {
      if (nissued > 0) tc::commit(&last);  // arrives when every MMA issued above has completed
      issued = nissued;
    }
  } else {
    // ------------------------------ drain ------------------------------
    // warp w: TMEM lanes (rows) 32 (w & 3) .. + 31, complex columns [16 (w >> 2), + 16)
    const int r = 32 * (warp & 3) + (tid & 31), ch = warp >> 2;
    const uint32_t tlane = tm + ((uint32_t)(32 * (warp & 3)) << 16);
    const uint32_t sum_h = tlane + OZ_SUM, sum_l = sum_h + OZ_NR;
    int i = 0;
    bool stop = false;
    for (int ti = blockIdx.x; ti < ntasks && !stop; ti += gridDim.x) {
      const OzTask tk = tasks[ti];
      const OzDesc dg = descs[tk.desc];
      const int mt = tk.mtnt >> 16, nt = tk.mtnt & 0xffff;
      const int Mt = min(OZ_M, dg.M - mt * OZ_M), Nt = min(OZ_NC, dg.N - nt * OZ_NC);
      const int ngrp = (Nt + 7) >> 3;
      const bool rv = r < Mt, f64 = dg.flags & OZ_OUT_F64;
      const int64_t crow0 = rv ? row_off(dg.c, mt * OZ_M + r, rowtab) : 0;
      const int ng0 = nt * OZ_NC + 16 * ch;
      const int nq0 = ng0 / dg.cnd, nr0 = ng0 - nq0 * dg.cnd;  // column ng0 = nq0 * cnd + nr0
      for (int rr = 0; rr < tk.nrep && !stop; ++rr) {
        const int64_t co = crow0 + (int64_t)(tk.rep0 + rr) * dg.rc;
        for (int k0 = 0; k0 < dg.K; k0 += OZ_KR, ++i) {
          if (warp_aborted()) { stop = true; break; }
          const int a = i & 1, e = i & 3;
          if (!warp_ok(bwait(&done[a], (i >> 1) & 1) && bwait(&eready[e], (i >> 2) & 1))) { stop = true; break; }
          tc::fence_after_sync();
          const bool first = k0 == 0, lastr = k0 + OZ_KR >= dg.K;
          const int ea = ea_s[e][r];
          const uint32_t base = tlane + (uint32_t)(a * OZ_ACC);
          int nq = nq0, nrr = nr0;  // output column cursor
#pragma unroll
          for (int gl = 0; gl < 4; ++gl) {  // this warp's groups of 8 real columns (4 complex)
            const int g = 4 * ch + gl;
            if (g < 2 * ngrp) {
              float x0[8], x1[8], x2[8], sh[8], sl[8];
              tc::tmem_ld8(base + (uint32_t)(8 * g), x0);
              tc::tmem_ld8(base + (uint32_t)(OZ_NR + 8 * g), x1);
              tc::tmem_ld8(base + (uint32_t)(2 * OZ_NR + 8 * g), x2);
              if (!first) {
                tc::tmem_ld8(sum_h + (uint32_t)(8 * g), sh);
                tc::tmem_ld8(sum_l + (uint32_t)(8 * g), sl);
              }
#pragma unroll
              for (int j = 0; j < 8; ++j) {
                const float sc = oz_pow2(ea + eb_s[e][4 * g + (j >> 1)] - 14);
                float vh, vl;
                oz_combine(x0[j], x1[j], x2[j], sc, vh, vl);
                if (first) {
                  sh[j] = vh;
                  sl[j] = vl;
                } else {
                  ff_add(sh[j], sl[j], vh, vl);
                }
              }
              if (lastr) {
#pragma unroll
                for (int j = 0; j < 8; j += 2) {
                  const int n = 4 * g + (j >> 1);
                  if (rv && n < Nt) {
                    oz_store(Cg, co + nq * dg.cn1 + nrr * dg.cn0, f64, dg.alpha, sh[j], sh[j + 1], sl[j], sl[j + 1]);
                    if (++nrr == dg.cnd) {
                      nrr = 0;
                      ++nq;
                    }
                  }
                }
              } else {
                tmem_st8(sum_h + (uint32_t)(8 * g), sh);
                tmem_st8(sum_l + (uint32_t)(8 * g), sl);
              }
            }
          }
          if (!lastr) tmem_wait_st();
          tc::fence_before_sync();
          tc::mbar_arrive(&afree[a]);
          tc::mbar_arrive(&efree[e]);
        }
      }
    }
  }
  __syncthreads();
  if (tid == 0 && issued > 0) tc::mbar_wait(&last, 0u, 4000000);  // every issued MMA has completed
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tm, OZ_TMEM_WS);
}

// (h, l) += (a + al)(b + bl) without renormalising (the a_l b_l term, below
// 2^-48 of the product, is dropped): the product's rounding error comes from an
// FMA (exact), the sum's from a two-sum; both go to the low word.
__device__ __forceinline__ void ff_mac(float &h, float &l, float a, float al, float b, float bl) {
  const float p = a * b;
  float e = fmaf(a, b, -p);
  e = fmaf(a, bl, e);
  e = fmaf(al, b, e);
  const float s = h + p;
  const float bb = s - h;
  l += ((h - (s - bb)) + (p - bb)) + e;
  h = s;
}

// Narrow block GEMMs (few output columns) on the CUDA cores in float-float:
// the same descriptors and tasks as oz_gemm_kernel (one CTA per task, one
// thread per row of the 128-row tile, four output columns at a time), for
// shapes where a tensor-core round would stage 128 x 16 slices for a handful
// of columns.  Every operand keeps its float-float value (no slicing), so the
// result carries about 46 bits.  B is read with addresses uniform across the
// warp (broadcast loads).
__global__ void __launch_bounds__(OZ_M) oz_simt_kernel(const OzDesc *__restrict__ descs,
                                                       const OzTask *__restrict__ tasks, const float4 *__restrict__ Ag,
                                                       const float4 *__restrict__ Bg, void *__restrict__ Cg,
                                                       const int64_t *__restrict__ rowtab) {
  const OzTask tk = tasks[blockIdx.x];
  const OzDesc dg = descs[tk.desc];
  const int mt = tk.mtnt >> 16, nt = tk.mtnt & 0xffff;
  const int Mt = min(OZ_M, dg.M - mt * OZ_M), Nt = min(OZ_NC, dg.N - nt * OZ_NC);
  const int r = threadIdx.x;
  if (r >= Mt) return;
  const int64_t arow0 = row_off(dg.a, mt * OZ_M + r, rowtab), crow0 = row_off(dg.c, mt * OZ_M + r, rowtab);
  const float sa = (dg.flags & OZ_CONJ_A) ? -1.f : 1.f, sb = (dg.flags & OZ_CONJ_B) ? -1.f : 1.f;
  const bool f64 = dg.flags & OZ_OUT_F64;
  for (int rr = 0; rr < tk.nrep; ++rr) {
    const int rep = tk.rep0 + rr;
    const float4 *arow = Ag + arow0 + (int64_t)rep * dg.ra;
    const int64_t co = crow0 + (int64_t)rep * dg.rc;
    for (int n0 = 0; n0 < Nt; n0 += 4) {
      const int nc = min(4, Nt - n0);
      const float4 *bp[4];
#pragma unroll
      for (int c = 0; c < 4; ++c)  // columns past the tile re-read column n0 (results unused)
        bp[c] = Bg + row_off(dg.b, nt * OZ_NC + n0 + (c < nc ? c : 0), rowtab) + (int64_t)rep * dg.rb;
      float acc[4][4];  // per column: re (h, l), im (h, l)
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[c][0] = acc[c][1] = acc[c][2] = acc[c][3] = 0.f;
      for (int k = 0; k < dg.K; ++k) {
        const float4 a = __ldg(arow + (int64_t)k * dg.aks);
        const float ai = sa * a.y, ail = sa * a.w;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          const float4 b = __ldg(bp[c] + (int64_t)k * dg.bks);
          const float bi = sb * b.y, bil = sb * b.w;
          ff_mac(acc[c][0], acc[c][1], a.x, a.z, b.x, b.z);    // re += ar br
          ff_mac(acc[c][0], acc[c][1], -ai, -ail, bi, bil);    //     - ai bi
          ff_mac(acc[c][2], acc[c][3], a.x, a.z, bi, bil);     // im += ar bi
          ff_mac(acc[c][2], acc[c][3], ai, ail, b.x, b.z);     //     + ai br
        }
      }
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        if (c < nc) {
          const int n = nt * OZ_NC + n0 + c;
          const int nq = n / dg.cnd, nr = n - nq * dg.cnd;
          const float rh = acc[c][0] + acc[c][1], ih = acc[c][2] + acc[c][3];
          const float rl = acc[c][1] - (rh - acc[c][0]), il = acc[c][3] - (ih - acc[c][2]);
          oz_store(Cg, co + nq * dg.cn1 + (int64_t)nr * dg.cn0, f64, dg.alpha, rh, ih, rl, il);
        }
      }
    }
  }
}

__global__ void to_ffc_kernel(const double2 *__restrict__ x, float4 *__restrict__ y, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double2 v = x[i];
    const float hr = __double2float_rn(v.x), hi = __double2float_rn(v.y);
    y[i] = make_float4(hr, hi, __double2float_rn(v.x - (double)hr), __double2float_rn(v.y - (double)hi));
  }
}

__global__ void oz_perm_kernel(const OzPerm *__restrict__ tasks, const double2 *__restrict__ src,
                               float4 *__restrict__ dst) {
  const OzPerm t = tasks[blockIdx.x];
  const int yz = t.Y * t.Z, n = t.X * yz;
  for (int e = threadIdx.x; e < n; e += blockDim.x) {
    const int x = e / yz, y = (e / t.Z) % t.Y, z = e % t.Z;
    double2 v = src[t.src + e];
    if (t.conj) v.y = -v.y;
    const float hr = __double2float_rn(v.x), hi = __double2float_rn(v.y);
    dst[t.dst + x * t.dx + y * t.dy + z * t.dz] =
        make_float4(hr, hi, __double2float_rn(v.x - (double)hr), __double2float_rn(v.y - (double)hi));
  }
}

}  // namespace

void set_oz_kernel_attributes() {
  GWGB_CUDA(cudaFuncSetAttribute(oz_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, OZ_SMEM_WS));
}

void launch_oz_gemm(const OzDesc *descs, const OzTask *tasks, int ntasks, const float4 *A, const float4 *B, void *C,
                    const int64_t *rowtab, int nsm, int *err, cudaStream_t st) {
  if (ntasks == 0) return;
  const int grid = std::min(ntasks, std::max(1, nsm));
  oz_gemm_kernel<<<grid, OZ_THREADS, OZ_SMEM_WS, st>>>(descs, tasks, ntasks, A, B, C, rowtab, err);
  GWGB_CUDA(cudaGetLastError());
}

void launch_oz_simt(const OzDesc *descs, const OzTask *tasks, int ntasks, const float4 *A, const float4 *B, void *C,
                    const int64_t *rowtab, cudaStream_t st) {
  if (ntasks == 0) return;
  oz_simt_kernel<<<ntasks, OZ_M, 0, st>>>(descs, tasks, A, B, C, rowtab);
  GWGB_CUDA(cudaGetLastError());
}

void launch_to_ffc(const double2 *x, float4 *y, int64_t n, cudaStream_t st) {
  if (n == 0) return;
  const int64_t blocks = std::min<int64_t>((n + 255) / 256, 8 * 1024);
  to_ffc_kernel<<<(int)blocks, 256, 0, st>>>(x, y, n);
  GWGB_CUDA(cudaGetLastError());
}

void launch_oz_perm(const OzPerm *tasks, int ntasks, const double2 *src, float4 *dst, cudaStream_t st) {
  if (ntasks == 0) return;
  oz_perm_kernel<<<ntasks, 256, 0, st>>>(tasks, src, dst);
  GWGB_CUDA(cudaGetLastError());
}

}  // namespace gwgb
