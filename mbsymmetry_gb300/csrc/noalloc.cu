// gwgb_wsolve_noalloc: the W~ solve of one irreducible q on caller-owned
// device buffers, with no device allocation at all.
//
// Some callers cannot allocate device memory while they run: a host code that
// hands out all of HBM from its own pool (the memory a cudaMalloc would need
// is already owned by that pool), a plugin called inside a region where the
// host framework forbids new allocations, or code that must not trigger the
// implicit synchronisation of cudaMalloc/cudaFree.  For them this entry point
// takes only the inputs and outputs from the caller and keeps its work space
// -- the P(i Omega) buffer, the transform slab descriptors, the block-inverse
// task list and a status word -- in one file-scope device array of
// GWGB_NOALLOC_SCRATCH_BYTES bytes.  That array exists on every GPU that
// loads the library, for the life of the process.
//
// Set-up: the first call on a device looks up the array's device address
// with cudaGetSymbolAddress (with that device current) and sets the
// shared-memory limits of the two block-inverse kernels it launches.
// Every call shares the one array and finds the previous call's contents in
// it; the status word is cleared at the start of each call and the rest is
// fully overwritten before it is read.  Calls that overlap on the GPU (two
// streams, two host threads) race on the array: serialise them.  Every call
// copies the status word to the host and synchronises `stream`, so no call
// can be recorded into a CUDA graph.  The caller's current device is the
// same after the call as before it.
#include <mutex>

#include "common.h"
#include "kernels.h"

namespace gwgb {

static __device__ __align__(256) unsigned char g_wsolve_scratch[GWGB_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
void *g_scratch_ptr[kMaxDevices] = {nullptr};

// Descriptors of one q slice, passed by value to the set-up kernel.
struct WsolveDesc {
  int32_t nblocks;
  int32_t nw_b;
  int32_t qslice;
  int32_t sizes[GWGB_NOALLOC_MAX_BLOCKS];
  int32_t offs[GWGB_NOALLOC_MAX_BLOCKS];
};

// Writes the two transform slabs and the (Omega, block) inverse tasks into
// the scratch array and clears the status word.
__global__ void wsolve_setup_kernel(WsolveDesc d, TSlab *slabs, InvTask *tasks, int *status) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid == 0) {
    slabs[0] = {0, 0, d.qslice, d.qslice, d.qslice, 0};  // P0(tau) -> P(i Omega)
    slabs[1] = {0, 0, d.qslice, d.qslice, d.qslice, 0};  // P(i Omega) -> P(tau)
    status[0] = 0;
  }
  for (int e = tid; e < d.nw_b * d.nblocks; e += gridDim.x * blockDim.x) {
    const int w = e / d.nblocks, b = e - w * d.nblocks;
    tasks[e] = {(int64_t)w * d.qslice + d.offs[b], 0, 0, d.sizes[b], -1};
  }
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Makes `device` current for the life of the guard and then restores the
// device that was current before (the caller's host thread state).
struct DeviceGuard {
  int saved = -1;
  explicit DeviceGuard(int device) {
    GWGB_CUDA(cudaGetDevice(&saved));
    if (saved != device) GWGB_CUDA(cudaSetDevice(device));
  }
  ~DeviceGuard() {
    int now = -1;
    if (saved >= 0 && cudaGetDevice(&now) == cudaSuccess && now != saved) cudaSetDevice(saved);
  }
};

}  // namespace
}  // namespace gwgb

extern "C" int gwgb_wsolve_noalloc(int32_t device, const double *P0_t, double *P_t, const double *Tnt_BF,
                                   const double *Ttn_FB, int32_t nts, int32_t nw_b,
                                   const int32_t *block_sizes, int32_t nblocks, void *stream) {
  using namespace gwgb;
  try {
    GWGB_REQUIRE(P0_t && P_t && Tnt_BF && Ttn_FB && block_sizes, GWGB_E_INVALID,
                 "gwgb_wsolve_noalloc: NULL pointer argument");
    GWGB_REQUIRE(device >= 0 && device < kMaxDevices, GWGB_E_INVALID, "gwgb_wsolve_noalloc: bad device ordinal");
    GWGB_REQUIRE(nts >= 4 && nts % 2 == 0, GWGB_E_INVALID, "Number of tau points should be even number");
    GWGB_REQUIRE(nts <= 160 && nw_b >= 1 && nw_b <= 160, GWGB_E_UNSUPPORTED,
                 "gwgb_wsolve_noalloc: tau/frequency grids are limited to 160 points");
    GWGB_REQUIRE(nblocks >= 1 && nblocks <= GWGB_NOALLOC_MAX_BLOCKS, GWGB_E_UNSUPPORTED,
                 "gwgb_wsolve_noalloc: 1 to 64 aux blocks per q are supported");
    WsolveDesc d{};
    d.nblocks = nblocks;
    d.nw_b = nw_b;
    int64_t qslice = 0;
    int nmax = 0;
    for (int b = 0; b < nblocks; ++b) {
      const int s = block_sizes[b];
      GWGB_REQUIRE(s >= 1 && s <= MAX_BLOCK, GWGB_E_UNSUPPORTED, "gwgb_wsolve_noalloc: aux block size outside 1..64");
      d.sizes[b] = s;
      d.offs[b] = (int32_t)qslice;
      qslice += (int64_t)s * s;
      nmax = s > nmax ? s : nmax;
    }
    d.qslice = (int32_t)qslice;
    // scratch layout: [status | 2 slabs][tasks][P(i Omega)]
    const size_t head = align256(sizeof(int) * 8 + 2 * sizeof(TSlab));
    const size_t task_bytes = align256((size_t)nw_b * nblocks * sizeof(InvTask));
    const size_t pw_bytes = (size_t)nw_b * qslice * sizeof(double2);
    GWGB_REQUIRE(head + task_bytes + pw_bytes <= GWGB_NOALLOC_SCRATCH_BYTES, GWGB_E_UNSUPPORTED,
                 "gwgb_wsolve_noalloc: nw_b * qslice needs " + std::to_string(head + task_bytes + pw_bytes) +
                     " bytes of scratch; the limit is " + std::to_string((size_t)GWGB_NOALLOC_SCRATCH_BYTES));

    DeviceGuard guard(device);
    void *base = nullptr;
    {
      std::lock_guard<std::mutex> lk(g_setup_mu);
      if (!g_scratch_ptr[device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_wsolve_scratch);
        if (e != cudaSuccess)
          throw Error(GWGB_E_CUDA, std::string("cudaGetSymbolAddress(g_wsolve_scratch): ") + cudaGetErrorString(e));
        set_inverse_kernel_attributes();
        g_scratch_ptr[device] = p;
      }
      base = g_scratch_ptr[device];
    }
    unsigned char *sc = static_cast<unsigned char *>(base);
    int *status = reinterpret_cast<int *>(sc);
    TSlab *slabs = reinterpret_cast<TSlab *>(sc + 32);
    InvTask *tasks = reinterpret_cast<InvTask *>(sc + head);
    double2 *Pw = reinterpret_cast<double2 *>(sc + head + task_bytes);
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    wsolve_setup_kernel<<<8, 256, 0, st>>>(d, slabs, tasks, status);
    GWGB_CUDA(cudaGetLastError());
    const int ncheb = nts - 2;
    launch_transform(slabs, 1, (int)qslice, reinterpret_cast<const double2 *>(Tnt_BF), nw_b, ncheb, 1,
                     reinterpret_cast<const double2 *>(P0_t), Pw, st);
    launch_inverse(tasks, nw_b * nblocks, nmax, Pw, nullptr, nullptr, nullptr, 1.0, 0.0, 0, status, st);
    launch_transform(slabs + 1, 1, (int)qslice, reinterpret_cast<const double2 *>(Ttn_FB), nts, nw_b, 0, Pw,
                     reinterpret_cast<double2 *>(P_t), st);
    int host_status = 0;
    GWGB_CUDA(cudaMemcpyAsync(&host_status, status, sizeof(int), cudaMemcpyDeviceToHost, st));
    GWGB_CUDA(cudaStreamSynchronize(st));
    GWGB_REQUIRE(host_status == 0, GWGB_E_NUMERIC, "singular block in the W~ solve (1 - P~0)");
    return GWGB_OK;
  } catch (const Error &e) {
    set_last_error(e.what());
    return e.code;
  } catch (const std::exception &e) {
    set_last_error(e.what());
    return GWGB_E_INVALID;
  }
}
