// Throughput probes for the roofline denominators that MEASURED_PEAKS.json
// does not hold: the FP64 and FP32 FMA rates (CUDA cores), the FP64 tensor rate
// (mma.sync f64, "DMMA"), and the tcgen05 rates of kind::tf32 and kind::f16
// with BF16 operands.  Measurement code for bench.py; not part of the engine
// or its C ABI.  Every wait on the tensor core is bounded.
#include <cuda_runtime.h>
#include <cstdint>

#include "../mbsymmetry_gb300/csrc/tc_common.cuh"

using namespace gwgb;

__global__ void dfma_loop(double *out, int iters, double b, double c) {
  double a0 = threadIdx.x * 1e-3, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3;
  double a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
  for (int i = 0; i < iters; ++i) {
    a0 = fma(a0, b, c); a1 = fma(a1, b, c); a2 = fma(a2, b, c); a3 = fma(a3, b, c);
    a4 = fma(a4, b, c); a5 = fma(a5, b, c); a6 = fma(a6, b, c); a7 = fma(a7, b, c);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

__global__ void ffma_loop(float *out, int iters, float b, float c) {
  float a[16];
#pragma unroll
  for (int j = 0; j < 16; ++j) a[j] = threadIdx.x * 1e-3f + j;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 16; ++j) a[j] = fmaf(a[j], b, c);
  }
  float s = 0.f;
#pragma unroll
  for (int j = 0; j < 16; ++j) s += a[j];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// Warp-level FP64 tensor MMA (m8n8k4, 512 flop per instruction), four
// independent accumulators per warp.
__global__ void dmma_loop(double *out, int iters, double av, double bv) {
  double d[4][2];
#pragma unroll
  for (int j = 0; j < 4; ++j) d[j][0] = d[j][1] = 0.0;
  const double a = av + threadIdx.x * 1e-9, b = bv;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 4; ++j)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                   : "+d"(d[j][0]), "+d"(d[j][1])
                   : "d"(a), "d"(b));
  }
  double s = 0;
#pragma unroll
  for (int j = 0; j < 4; ++j) s += d[j][0] + d[j][1];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// One CTA per SM: M = 128, N = 256 MMAs from fixed shared-memory tiles into two
// TMEM accumulators, issued back to back by one thread in batches of 64; at
// most two batches are in flight (each batch commits to its own mbarrier and
// is waited for, with a bounded wait, before that barrier is reused).
template <bool BF>
__global__ void __launch_bounds__(128) tc_loop(int batches, int *err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint32_t tslot;
  __shared__ __align__(8) uint64_t bar[2];
  constexpr int ROWB = 32;  // bytes of one operand row of one MMA (K = 8 TF32 / 16 BF16)
  unsigned char *A = smem, *B = smem + 128 * ROWB;
  for (int e = threadIdx.x; e < (128 + 256) * ROWB / 4; e += blockDim.x)
    reinterpret_cast<uint32_t *>(smem)[e] = BF ? 0x3c003c00u : 0x3a800000u;  // small exact values
  if ((threadIdx.x >> 5) == 0) tc::tmem_alloc(&tslot, 512);
  if (threadIdx.x == 0) {
    tc::mbar_init(&bar[0], 1);
    tc::mbar_init(&bar[1], 1);
  }
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tslot;
  if (threadIdx.x == 0) {
    const uint32_t sbo = (ROWB / 16) * 128;
    const uint64_t ad = tc::make_desc(tc::smem_u32(A), 128, sbo), bd = tc::make_desc(tc::smem_u32(B), 128, sbo);
    const uint32_t id = BF ? tc::idesc_bf16(128, 256) : tc::idesc_tf32(128, 256);
    bool ok = true;
    int b = 0;
    for (; b < batches && ok; ++b) {
      for (int i = 0; i < 64; ++i) {
        const uint32_t d = tmem + (uint32_t)((i & 1) * 256);
        if (BF) tc::mma_bf16(d, ad, bd, id, 1u);
        else tc::mma_tf32(d, ad, bd, id, 1u);
      }
      tc::commit(&bar[b & 1]);
      if (b >= 1) ok = tc::mbar_wait(&bar[(b - 1) & 1], ((b - 1) >> 1) & 1);
    }
    // the last committed batch (and, after an early stop, the one before it)
    if (b >= 1 && !tc::mbar_wait(&bar[(b - 1) & 1], ((b - 1) >> 1) & 1)) ok = false;
    if (!ok) atomicExch(err, 1);
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if ((threadIdx.x >> 5) == 0) tc::tmem_dealloc(tmem, 512);
}

namespace {

template <typename L>
float best_ms(L launch, int reps) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int r = 0; r < reps; ++r) {
    cudaEventRecord(e0);
    launch();
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return best;
}

}  // namespace

// Best-of-5 FP64 FMA throughput of device `dev` in TFLOP/s (2 flops per FMA);
// negative on a CUDA error.
extern "C" double gwgb_probe_fp64_tflops(int dev) {
  if (cudaSetDevice(dev) != cudaSuccess) return -1.0;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * 8, threads = 256, iters = 1 << 14;
  double *out = nullptr;
  if (cudaMalloc(&out, sizeof(double) * blocks * threads) != cudaSuccess) return -1.0;
  dfma_loop<<<blocks, threads>>>(out, 64, 1.0000001, 1e-9);
  const float ms = best_ms([&] { dfma_loop<<<blocks, threads>>>(out, iters, 1.0000001, 1e-9); }, 5);
  cudaError_t err = cudaGetLastError();
  cudaFree(out);
  if (err != cudaSuccess) return -1.0;
  return 2.0 * 8.0 * (double)iters * blocks * threads / (ms * 1e-3) / 1e12;
}

// Best-of-5 FP32 FMA throughput (CUDA cores) in TFLOP/s (2 flops per FMA);
// negative on a CUDA error.
extern "C" double gwgb_probe_fp32_tflops(int dev) {
  if (cudaSetDevice(dev) != cudaSuccess) return -1.0;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * 8, threads = 256, iters = 1 << 14;
  float *out = nullptr;
  if (cudaMalloc(&out, sizeof(float) * blocks * threads) != cudaSuccess) return -1.0;
  ffma_loop<<<blocks, threads>>>(out, 64, 0.9999999f, 1e-6f);
  const float ms = best_ms([&] { ffma_loop<<<blocks, threads>>>(out, iters, 0.9999999f, 1e-6f); }, 5);
  cudaError_t err = cudaGetLastError();
  cudaFree(out);
  if (err != cudaSuccess) return -1.0;
  return 2.0 * 16.0 * (double)iters * blocks * threads / (ms * 1e-3) / 1e12;
}

// Best-of-5 FP64 tensor-core (mma.sync f64) throughput in TFLOP/s.
extern "C" double gwgb_probe_dmma_tflops(int dev) {
  if (cudaSetDevice(dev) != cudaSuccess) return -1.0;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * 4, threads = 256, iters = 1 << 12;
  double *out = nullptr;
  if (cudaMalloc(&out, sizeof(double) * blocks * threads) != cudaSuccess) return -1.0;
  dmma_loop<<<blocks, threads>>>(out, 16, 1.0, 1e-3);
  const float ms = best_ms([&] { dmma_loop<<<blocks, threads>>>(out, iters, 1.0, 1e-3); }, 5);
  cudaError_t err = cudaGetLastError();
  cudaFree(out);
  if (err != cudaSuccess) return -1.0;
  const double warps = (double)blocks * threads / 32;
  return 512.0 * 4.0 * iters * warps / (ms * 1e-3) / 1e12;
}

// Best-of-5 tcgen05 dense throughput in TFLOP/s: kind 0 = kind::tf32,
// kind 1 = kind::f16 with BF16 A and B (FP32 accumulate).  Negative on a CUDA
// error or when a bounded completion wait ran out.
extern "C" double gwgb_probe_tc_tflops(int dev, int kind) {
  if (cudaSetDevice(dev) != cudaSuccess) return -1.0;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int *err = nullptr;
  if (cudaMalloc(&err, sizeof(int)) != cudaSuccess) return -1.0;
  cudaMemset(err, 0, sizeof(int));
  // 120 KB of shared memory per CTA: one CTA per SM, so no CTA waits for
  // another's 512 TMEM columns
  const int smem = 120 * 1024;
  const int batches = 128;
  if (cudaFuncSetAttribute(tc_loop<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess ||
      cudaFuncSetAttribute(tc_loop<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess) {
    cudaFree(err);
    return -1.0;
  }
  auto launch = [&](int nb) {
    if (kind == 1) tc_loop<true><<<sms, 128, smem>>>(nb, err);
    else tc_loop<false><<<sms, 128, smem>>>(nb, err);
  };
  launch(8);
  const float ms = best_ms([&] { launch(batches); }, 5);
  int h = 0;
  cudaError_t e = cudaMemcpy(&h, err, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(err);
  if (e != cudaSuccess || cudaGetLastError() != cudaSuccess || h) return -1.0;
  const double k = kind == 1 ? 16.0 : 8.0;
  return 2.0 * 128.0 * 256.0 * k * 64.0 * batches * sms / (ms * 1e-3) / 1e12;
}
