// gw_noalloc.cu -- the likelihood reduction for callers that cannot allocate
// device memory.
//
// gw_llh_noalloc computes, for K parameter points, the summed per-bin
// likelihood from bin sums the caller already holds on the device: the same
// per-bin terms and the same fixed-order block / last-block reduction as the
// engine's k_bins_llh.  That reduction needs scratch memory (one partial per
// block and one arrival counter per point).  The engine allocates it with
// cudaMalloc; here it is a fixed-size array in device global memory that the
// library defines at file scope, so the call itself allocates nothing.
//
// Who needs this: code that evaluates the likelihood from inside a framework
// that owns the device memory (a caching allocator or a fitter's memory pool
// that has claimed the GPU), or from a per-evaluation callback that must not
// call cudaMalloc/cudaFree because those calls can synchronise the device and
// stall the caller's other streams.
//
// Limits and sharing:
//  * K <= kNoAllocMaxPoints and K * ceil(n_bins / 256) <= kNoAllocMaxBlocks;
//    larger requests are rejected with GW_ERR_LIMIT before anything launches.
//    The array holds 65536 FP64 block partials and 4096 counters (about
//    528 KiB) on every GPU that loads the library, until the process exits.
//  * Every call shares the one array per device, and the array keeps the last
//    call's contents: each call clears the counters it uses before its
//    kernel.  Calls whose work overlaps on the GPU (different streams, or a
//    second host thread) race on the array; serialise them.
//  * The first call on a device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current and caches it for the
//    rest of the process; make that first call before any stream capture.
//    The address belongs to the device's primary context: cudaDeviceReset
//    destroys that context (the module is loaded again, possibly elsewhere),
//    so the cached address is stale after a reset and the entry point must
//    not be called on that device again in the same process.
#include <mutex>

#include "gw.h"
#include "gw_device.cuh"

namespace {
constexpr int kNoAllocMaxBlocks = 65536;
constexpr int kNoAllocMaxPoints = 4096;
constexpr size_t kNoAllocBytes =
    (size_t)kNoAllocMaxBlocks * sizeof(double) + (size_t)kNoAllocMaxPoints * sizeof(unsigned int);
constexpr int kMaxDevices = 64;
}  // namespace

// The scratch array.  In host code this name is only a stand-in for the
// device object: its device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char gw_noalloc_scratch[kNoAllocBytes];

namespace gw {
namespace {

// Variant of k_bins_llh: per-bin terms from caller-provided sums, reduced per
// point in the same fixed order; scratch = the file-scope array.
__global__ void __launch_bounds__(256) k_llh_noalloc(const double* __restrict__ sums,
                                                     const double* __restrict__ sums2,
                                                     const double* __restrict__ data, int n_bins, int llh_type,
                                                     double* blocks, unsigned int* counters, double* llh) {
  const int k = blockIdx.y;
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  double term = 0.0;
  if (b < n_bins) {
    const double s = sums[(size_t)k * n_bins + b];
    const double s2 = sums2[(size_t)k * n_bins + b];
    if (llh_type == GW_LLH_POISSON) {
      term = llh_poisson(data[b], s);
    } else {
      term = llh_bb_bin(data[b], s, sqrt(s2));
    }
  }
  __shared__ double red[32];
  __shared__ bool last;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int o = 16; o; o >>= 1) term += __shfl_xor_sync(0xffffffffu, term, o);
  if (lane == 0) red[warp] = term;
  __syncthreads();
  if (warp == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    double t = lane < nw ? red[lane] : 0.0;
    for (int o = 16; o; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) {
      blocks[(size_t)k * gridDim.x + blockIdx.x] = t;
      __threadfence();
      const unsigned prev = atomicAdd(&counters[k], 1u);
      last = (prev == gridDim.x - 1);
    }
  }
  __syncthreads();
  if (!last) return;
  if (warp == 0) {
    __threadfence();
    double t = 0.0;
    for (int i = lane; i < (int)gridDim.x; i += 32) t += __ldcg(&blocks[(size_t)k * gridDim.x + i]);
    for (int o = 16; o; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) {
      llh[k] = t;
      counters[k] = 0u;
    }
  }
}

std::mutex g_mu;
void* g_scratch[kMaxDevices] = {};

}  // namespace
}  // namespace gw

void gw_internal_set_error(const char* msg);  // gw_engine.cpp

extern "C" int gw_llh_noalloc(const double* d_sums, const double* d_sums2, const double* d_data, int32_t n_bins,
                              int32_t K, int32_t llh_type, double* d_llh, void* stream) {
  if (!d_sums || !d_sums2 || !d_data || !d_llh || n_bins < 1 || K < 1 ||
      (llh_type != GW_LLH_POISSON && llh_type != GW_LLH_BARLOW_BEESTON_OA2021)) {
    gw_internal_set_error("gw_llh_noalloc: null pointer, empty size or unknown likelihood type");
    return GW_ERR_ARG;
  }
  const int64_t nblk = ((int64_t)n_bins + 255) / 256;
  if (K > kNoAllocMaxPoints || (int64_t)K * nblk > kNoAllocMaxBlocks) {
    gw_internal_set_error("gw_llh_noalloc: K * ceil(n_bins/256) must be <= 65536 and K <= 4096");
    return GW_ERR_LIMIT;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    gw_internal_set_error("gw_llh_noalloc: no usable current CUDA device");
    return GW_ERR_CUDA;
  }
  void* base = nullptr;
  {
    std::lock_guard<std::mutex> lk(gw::g_mu);
    if (!gw::g_scratch[dev]) {
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, gw_noalloc_scratch);
      if (e != cudaSuccess || !p) {
        cudaGetLastError();
        gw_internal_set_error("gw_llh_noalloc: cudaGetSymbolAddress of the scratch array failed");
        return GW_ERR_CUDA;
      }
      gw::g_scratch[dev] = p;
    }
    base = gw::g_scratch[dev];
  }
  double* blocks = (double*)base;
  unsigned int* counters = (unsigned int*)((unsigned char*)base + (size_t)kNoAllocMaxBlocks * sizeof(double));
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(counters, 0, sizeof(unsigned int) * (size_t)K, s);
  if (e == cudaSuccess) {
    gw::k_llh_noalloc<<<dim3((unsigned)nblk, (unsigned)K), 256, 0, s>>>(d_sums, d_sums2, d_data, n_bins, llh_type,
                                                                        blocks, counters, d_llh);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) {
    gw_internal_set_error(cudaGetErrorString(e));
    return GW_ERR_CUDA;
  }
  return GW_OK;
}
