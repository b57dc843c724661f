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
constexpr int OZ_TILES = 4 * OZ_PA + 4 * OZ_PB;
constexpr int OZ_SMEM = 80 * 1024;          // requested per CTA: at most two CTAs per SM
constexpr int OZ_TMEM = 256;                // D0 | D1 | D2, OZ_NR columns each
constexpr int OZ_EMIN = -100, OZ_EMAX = 100;
static_assert(OZ_TILES + 1024 <= OZ_SMEM, "slice planes must fit the requested shared memory");
static_assert(3 * OZ_NR <= OZ_TMEM, "three accumulators must fit the TMEM allocation");
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

__device__ __forceinline__ int64_t row_off(const OzRows &m, int r) {
  return m.base + (int64_t)(r / m.d) * m.s1 + (int64_t)(r % m.d) * m.s0;
}

__global__ void __launch_bounds__(128, 2)
    oz_gemm_kernel(const OzDesc *__restrict__ descs, const OzTask *__restrict__ tasks, int ntasks,
                   const float4 *__restrict__ Ag, const float4 *__restrict__ Bg, void *__restrict__ Cg,
                   int *__restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint32_t tslot;
  __shared__ __align__(8) uint64_t bar;
  __shared__ int ebs[OZ_NC];
  __shared__ int abort_flag;
  unsigned char *As = smem, *Bs = smem + 4 * OZ_PA;
  const int tid = threadIdx.x, warp = tid >> 5;
  if (warp == 0) tc::tmem_alloc(&tslot, OZ_TMEM);
  if (tid == 0) {
    tc::mbar_init(&bar, 1);
    abort_flag = 0;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tm = tslot;
  const uint32_t tlane = tm + ((uint32_t)(warp * 32) << 16);
  uint32_t phase = 0;
  bool pending = false;  // a commit whose completion nobody observed (abort path)

  for (int ti = blockIdx.x; ti < ntasks && !abort_flag; ti += gridDim.x) {
   const OzTask tk = tasks[ti];
   for (int rr = 0; rr < tk.nrep && !abort_flag; ++rr) {
    const int rep = tk.rep0 + rr, mt = tk.mtnt >> 16, nt = tk.mtnt & 0xffff;
    const OzDesc &dg = descs[tk.desc];
    const int M = dg.M, N = dg.N, K = dg.K, flags = dg.flags;
    const int Mt = min(OZ_M, M - mt * OZ_M), Nt = min(OZ_NC, N - nt * OZ_NC);
    const int aks = dg.aks, bks = dg.bks;
    // this thread's A row and (with qd) B row
    const int r = tid;
    const bool rv = r < Mt;
    const float4 *arow = Ag + (rv ? row_off(dg.a, mt * OZ_M + r) + (int64_t)rep * dg.ra : 0);
    const int bn = tid >> 2, qd = tid & 3;
    const bool bv = bn < Nt;
    const float4 *brow = Bg + (bv ? row_off(dg.b, nt * OZ_NC + bn) + (int64_t)rep * dg.rb : 0);
    const bool ca = flags & OZ_CONJ_A, cb = flags & OZ_CONJ_B;
    float acc_h[OZ_NR], acc_l[OZ_NR];
#pragma unroll
    for (int j = 0; j < OZ_NR; ++j) acc_h[j] = acc_l[j] = 0.f;

    for (int k0 = 0; k0 < K; k0 += OZ_KR) {
      const int kn = min(OZ_KR, K - k0);
      // ---- A: one row per thread; exponent from the row's largest hi part ----
      float m = 0.f;
      if (rv)
        for (int k = 0; k < kn; ++k) {
          const float4 v = __ldg(arow + (int64_t)(k0 + k) * aks);
          m = fmaxf(m, fmaxf(fabsf(v.x), fabsf(v.y)));
        }
      const int ea = oz_exponent(m);
      {
        const float f = oz_pow2(7 - ea);
#pragma unroll
        for (int g = 0; g < OZ_KR / 4; ++g) {
          uint32_t w[4][4];
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const int k = g * 4 + j;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (rv && k < kn) v = __ldg(arow + (int64_t)(k0 + k) * aks);
            if (ca) { v.y = -v.y; v.w = -v.w; }
            float sr[4], si[4];
            oz_slice(v.x, v.z, f, sr);
            oz_slice(v.y, v.w, f, si);
#pragma unroll
            for (int p = 0; p < 4; ++p) w[p][j] = bf2(sr[p], si[p]);
          }
          const uint32_t o = seg_off(r, 8 * g);
#pragma unroll
          for (int p = 0; p < 4; ++p)
            *reinterpret_cast<uint4 *>(As + p * OZ_PA + o) = make_uint4(w[p][0], w[p][1], w[p][2], w[p][3]);
        }
      }
      // ---- B: four threads per complex row (4 complex K each); rows (n,0) = [Br -Bi], (n,1) = [Bi Br] ----
      {
        float4 v[4];
        float mb = 0.f;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int k = 4 * qd + j;
          v[j] = make_float4(0.f, 0.f, 0.f, 0.f);
          if (bv && k < kn) v[j] = __ldg(brow + (int64_t)(k0 + k) * bks);
          if (cb) { v[j].y = -v[j].y; v[j].w = -v[j].w; }
          mb = fmaxf(mb, fmaxf(fabsf(v[j].x), fabsf(v[j].y)));
        }
        mb = fmaxf(mb, __shfl_xor_sync(0xffffffffu, mb, 1));
        mb = fmaxf(mb, __shfl_xor_sync(0xffffffffu, mb, 2));
        const int eb = oz_exponent(mb);
        if (qd == 0) ebs[bn] = eb;
        const float f = oz_pow2(7 - eb);
        uint32_t w0[4][4], w1[4][4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          float sr[4], si[4];
          oz_slice(v[j].x, v[j].z, f, sr);
          oz_slice(v[j].y, v[j].w, f, si);
#pragma unroll
          for (int p = 0; p < 4; ++p) {
            w0[p][j] = bf2(sr[p], -si[p]);
            w1[p][j] = bf2(si[p], sr[p]);
          }
        }
        const uint32_t o0 = seg_off(2 * bn, 8 * qd), o1 = seg_off(2 * bn + 1, 8 * qd);
#pragma unroll
        for (int p = 0; p < 4; ++p) {
          *reinterpret_cast<uint4 *>(Bs + p * OZ_PB + o0) = make_uint4(w0[p][0], w0[p][1], w0[p][2], w0[p][3]);
          *reinterpret_cast<uint4 *>(Bs + p * OZ_PB + o1) = make_uint4(w1[p][0], w1[p][1], w1[p][2], w1[p][3]);
        }
      }
      tc::fence_async_smem();
      tc::fence_before_sync();
      __syncthreads();
      tc::fence_after_sync();
      // ---- MMAs: classes 0 | 1 | 2-3 into D0 | D1 | D2 ----
      if (tid == 0) {
        const uint32_t a0 = tc::smem_u32(As), b0 = tc::smem_u32(Bs);
        const uint32_t id = tc::idesc_bf16(OZ_M, OZ_NR);
        const uint32_t d0 = tm, d1 = tm + OZ_NR, d2 = tm + 2 * OZ_NR;
#pragma unroll
        for (int ks = 0; ks < OZ_KP / 16; ++ks) {
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
        tc::commit(&bar);
      }
      const bool ok = tc::mbar_wait(&bar, phase);
      phase ^= 1u;
      if (__syncthreads_or(!ok)) {
        if (tid == 0) {
          atomicExch(err, 1);
          abort_flag = 1;
        }
        pending = true;
        break;
      }
      tc::fence_after_sync();
      // ---- drain: combine the classes, scale, add to the float-float accumulator ----
#pragma unroll
      for (int j0 = 0; j0 < OZ_NR; j0 += 8) {
        float x0[8], x1[8], x2[8];
        tc::tmem_ld8(tlane + (uint32_t)j0, x0);
        tc::tmem_ld8(tlane + (uint32_t)(OZ_NR + j0), x1);
        tc::tmem_ld8(tlane + (uint32_t)(2 * OZ_NR + j0), x2);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const float sc = oz_pow2(ea + ebs[(j0 + j) >> 1] - 14);
          float vh, vl;
          two_sum(x0[j], x1[j], vh, vl);
          vl += x2[j];
          const float s = vh + vl;
          vl -= s - vh;
          ff_add(acc_h[j0 + j], acc_l[j0 + j], s * sc, vl * sc);
        }
      }
      tc::fence_before_sync();
      __syncthreads();  // shared tiles, ebs and TMEM free for the next round
    }
    __syncthreads();
    if (abort_flag) break;
    // ---- output ----
    if (rv) {
      const int64_t co = row_off(dg.c, mt * OZ_M + r) + (int64_t)rep * dg.rc;
#pragma unroll
      for (int n = 0; n < OZ_NC; ++n) {
        if (n < Nt) {
          const int ng = nt * OZ_NC + n;
          const int64_t o = co + (int64_t)(ng / dg.cnd) * dg.cn1 + (int64_t)(ng % dg.cnd) * dg.cn0;
          if (flags & OZ_OUT_F64) {
            const double al = dg.alpha;
            reinterpret_cast<double2 *>(Cg)[o] =
                make_double2(al * ((double)acc_h[2 * n] + (double)acc_l[2 * n]),
                             al * ((double)acc_h[2 * n + 1] + (double)acc_l[2 * n + 1]));
          } else {
            reinterpret_cast<float4 *>(Cg)[o] =
                make_float4(acc_h[2 * n], acc_h[2 * n + 1], acc_l[2 * n], acc_l[2 * n + 1]);
          }
        }
      }
    }
   }
  }
  __syncthreads();
  if (tid == 0 && pending) tc::mbar_wait(&bar, phase ^ 1u, 4000000);  // the MMAs of the aborted round
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tm, OZ_TMEM);
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
  GWGB_CUDA(cudaFuncSetAttribute(oz_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, OZ_SMEM));
}

void launch_oz_gemm(const OzDesc *descs, const OzTask *tasks, int ntasks, const float4 *A, const float4 *B, void *C,
                    int nsm, int *err, cudaStream_t st) {
  if (ntasks == 0) return;
  const int grid = std::min(ntasks, 2 * std::max(1, nsm));
  oz_gemm_kernel<<<grid, 128, OZ_SMEM, st>>>(descs, tasks, ntasks, A, B, C, err);
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
