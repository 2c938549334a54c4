// gw_mlp.cu -- the learned surrogate: a BF16 MLP trained and evaluated with
// hand-written tcgen05 kernels (libgw.so, C ABI gwm_* in include/gw.h).
//
// Every GEMM is C[M x N] = A[M x K] * B[N x K]^T with both operands K-major
// (contiguous along K) in BF16 and FP32 accumulation in tensor memory (TMEM):
//   * one CTA (4 warps) owns a 128 x BN output tile;
//   * the K loop stages 128 x 64 and BN x 64 BF16 tiles in shared memory in
//     the canonical no-swizzle core-matrix layout (8 rows x 16 bytes per core
//     matrix), double-buffered;
//   * one elected thread issues tcgen05.mma (M = 128, N = BN, K = 16 each) and
//     tcgen05.commit to an mbarrier per stage; every wait on it is bounded;
//   * the epilogue reads the accumulator with tcgen05.ld (each warp its 32 TMEM
//     lanes = rows) and fuses bias, SiLU, the SiLU derivative of the backward
//     pass, and row-major / transposed BF16 or FP32 stores;
//   * TMEM is allocated once per CTA and freed on every exit path.
// Forward: z = W x + b, h = silu(z); backward: dX = dY W (with the SiLU
// derivative fused), dW = dY^T X; Adam on FP32 master weights refreshes the
// BF16 weights and their transposes.
#include <cuda_bf16.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "gw.h"

namespace gwm {
namespace {

typedef __nv_bfloat16 bf16;

constexpr int kBM = 128;
constexpr int kBK = 64;
constexpr int kThreads = 128;
constexpr uint64_t kWaitNs = 1000000000ull;  // 1 s per MMA commit

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  for (;;) {
    if (mbar_try_wait(bar, parity)) return true;
    if (global_ns() - t0 > kWaitNs) return false;
  }
}

// ---- tcgen05 primitives ----
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor, no swizzle: start address, byte offset
// between core matrices adjacent along K (LBO) and along M/N (SBO).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version
  return d;
}

// Instruction descriptor, kind::f16: D = F32, A = B = BF16, both K-major.
__host__ __device__ constexpr uint32_t instr_desc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.u32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ float sigmoidf_(float z) { return 1.f / (1.f + __expf(-z)); }

struct Epilogue {
  const float* bias;    // [N] or null
  int act;              // 1: SiLU
  const float* gate;    // [M x N] pre-activations: multiply by silu'(gate) (backward) or null
  float* out_f32;       // [M x N] value before the activation, or null
  bf16* out_bf16;       // [M x N] after the activation, or null
  bf16* out_bf16_t;     // [N x M] after the activation, or null
  int ld_t;             // leading dimension of out_bf16_t (>= M)
};

// Copies a rows x 64 BF16 tile (row-major source, K contiguous) into the
// core-matrix layout: (r, k) -> (r/8)*1024 + (k/8)*128 + (r%8)*16 + (k%8)*2.
__device__ __forceinline__ void load_tile(unsigned char* dst, const bf16* __restrict__ src, int rows, int row0,
                                          int nrows_total, int K, int k0) {
  const int chunks = rows * 8;  // 16-byte chunks
  for (int c = threadIdx.x; c < chunks; c += kThreads) {
    const int r = c >> 3, j = c & 7;
    const int gr = row0 + r, gk = k0 + 8 * j;
    uint4 val = make_uint4(0, 0, 0, 0);
    if (gr < nrows_total) {
      const bf16* p = src + (size_t)gr * K + gk;
      if (gk + 8 <= K) {
        val = *reinterpret_cast<const uint4*>(p);
      } else if (gk < K) {
        bf16 tmp[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) tmp[q] = (gk + q < K) ? p[q] : __float2bfloat16(0.f);
        memcpy(&val, tmp, 16);
      }
    }
    *reinterpret_cast<uint4*>(dst + (r >> 3) * 1024 + j * 128 + (r & 7) * 16) = val;
  }
}

template <int BN>
__global__ void __launch_bounds__(kThreads) k_gemm(const bf16* __restrict__ A, const bf16* __restrict__ B, int M,
                                                   int N, int K, Epilogue ep, uint32_t* status) {
  extern __shared__ __align__(1024) unsigned char smem[];
  constexpr int kATile = kBM * kBK * 2;  // 16 KB
  constexpr int kBTile = BN * kBK * 2;
  unsigned char* sa[2] = {smem, smem + kATile + kBTile};
  unsigned char* sb[2] = {smem + kATile, smem + 2 * kATile + kBTile};
  __shared__ uint64_t bar[2];
  __shared__ uint32_t tmem_base;
  __shared__ int failed;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.y * kBM, n0 = blockIdx.x * BN;
  if (warp == 0) tmem_alloc(&tmem_base, BN);
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    failed = 0;
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base;
  constexpr uint32_t idesc = instr_desc(kBM, BN);
  const int nk = (K + kBK - 1) / kBK;

  int issued = -1;  // last tile whose MMAs were issued
  for (int kt = 0; kt < nk; ++kt) {
    const int st = kt & 1;
    if (kt >= 2) {
      // the MMAs that read this stage two tiles ago must be done
      const bool ok = mbar_wait_bounded(&bar[st], (uint32_t)(((kt - 2) >> 1) & 1));
      if (!ok) failed = 1;
    }
    __syncthreads();
    if (failed) break;
    issued = kt;
    load_tile(sa[st], A, kBM, m0, M, K, kt * kBK);
    load_tile(sb[st], B, BN, n0, N, K, kt * kBK);
    fence_proxy_async();
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
      const uint32_t a0 = smem_u32(sa[st]), b0 = smem_u32(sb[st]);
#pragma unroll
      for (int s = 0; s < kBK / 16; ++s) {
        const uint64_t ad = smem_desc(a0 + s * 256, 128, 1024);
        const uint64_t bd = smem_desc(b0 + s * 256, 128, 1024);
        mma_bf16(tmem, ad, bd, idesc, (kt > 0 || s > 0) ? 1u : 0u);
      }
      mma_commit(&bar[st]);
    }
  }
  // wait for the last commit (it covers every earlier MMA of this thread)
  if (!failed && issued >= 0) {
    if (!mbar_wait_bounded(&bar[issued & 1], (uint32_t)((issued >> 1) & 1))) failed = 1;
  }
  __syncthreads();
  if (failed) {
    if (tid == 0) {
      atomicOr(status, 1u);
      // wait once more (bounded) for MMAs still in flight before freeing TMEM
      if (issued >= 0) mbar_wait_bounded(&bar[issued & 1], (uint32_t)((issued >> 1) & 1));
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, BN);
    return;
  }
  tc_fence_after();

  // epilogue: warp w reads TMEM lanes 32w..32w+31 = tile rows
  const int r = m0 + warp * 32 + lane;
  const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
  for (int c0 = 0; c0 < BN; c0 += 8) {
    float v[8];
    tmem_ld8(lane_addr + (uint32_t)c0, v);
    if (r >= M) continue;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int n = n0 + c0 + q;
      if (n >= N) continue;
      float z = v[q];
      if (ep.bias) z += ep.bias[n];
      if (ep.gate) {
        const float g = ep.gate[(size_t)r * N + n];
        const float sg = sigmoidf_(g);
        z *= sg * (1.f + g * (1.f - sg));
      }
      if (ep.out_f32) ep.out_f32[(size_t)r * N + n] = z;
      const float a = (ep.act == 1) ? z * sigmoidf_(z) : z;
      if (ep.out_bf16) ep.out_bf16[(size_t)r * N + n] = __float2bfloat16(a);
      if (ep.out_bf16_t) ep.out_bf16_t[(size_t)n * ep.ld_t + r] = __float2bfloat16(a);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, BN);
}

// ---- small kernels ----
__global__ void k_to_bf16(const float* __restrict__ x, int rows, int cols, bf16* y, bf16* yt, int ld_t) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)rows * cols) return;
  const int r = (int)(i / cols), c = (int)(i % cols);
  const bf16 v = __float2bfloat16(x[i]);
  if (y) y[i] = v;
  if (yt) yt[(size_t)c * ld_t + r] = v;
}

// Mean squared error and its gradient: dy = 2 (y - t) / (rows * cols).
__global__ void k_mse(const float* __restrict__ y, const float* __restrict__ t, int rows, int cols, bf16* dy,
                      bf16* dyt, int ld_t, float* loss) {
  const int64_t n = (int64_t)rows * cols;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  float e2 = 0.f;
  if (i < n) {
    const float e = y[i] - t[i];
    e2 = e * e;
    const bf16 g = __float2bfloat16(2.f * e / (float)n);
    const int r = (int)(i / cols), c = (int)(i % cols);
    dy[i] = g;
    dyt[(size_t)c * ld_t + r] = g;
  }
  for (int o = 16; o; o >>= 1) e2 += __shfl_xor_sync(0xffffffffu, e2, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, e2 / (float)n);
}

// Column sums of a row-major BF16 matrix (bias gradients), one thread per column.
__global__ void k_colsum(const bf16* __restrict__ g, int rows, int cols, float* out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  float s = 0.f;
  for (int r = 0; r < rows; ++r) s += __bfloat162float(g[(size_t)r * cols + c]);
  out[c] = s;
}

// Adam on FP32 master weights; refreshes the BF16 copy and its transpose.
__global__ void k_adam(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       int n, int rows, int cols, float lr, float b1, float b2, float eps, float c1, float c2,
                       bf16* wb, bf16* wt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  w[i] = wi;
  if (wb) {
    const bf16 b = __float2bfloat16(wi);
    wb[i] = b;
    if (wt && rows > 0) {
      const int r = i / cols, c = i % cols;
      wt[(size_t)c * rows + r] = b;
    }
  }
}

// Standardised inputs: x = (theta - mean) / scale, FP32.
__global__ void k_standardize(const double* __restrict__ theta, int rows, int cols, const float* __restrict__ mean,
                              const float* __restrict__ scale, float* x) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)rows * cols) return;
  const int c = (int)(i % cols);
  x[i] = (float)((theta[i] - (double)mean[c]) / (double)scale[c]);
}

// Head of the surrogate, one thread per (point, bin):
//   log rate = b + sum_k x_k Wt[k][bin] + mu + sd * mlp  (FP32 affine base)
//   sums = exp(log rate), sums2 = ratio * sums             (FP64 for the LLH)
__global__ void k_head(const float* __restrict__ x, int din, const float* __restrict__ wt,
                       const float* __restrict__ b0, const float* __restrict__ mu, const float* __restrict__ sd,
                       const float* __restrict__ ratio, const float* __restrict__ mlp, int nb, double* sums,
                       double* sums2, double* logr) {
  const int bin = blockIdx.x * blockDim.x + threadIdx.x;
  const int m = blockIdx.y;
  if (bin >= nb) return;
  const float* xm = x + (size_t)m * din;
  float acc = b0[bin];
  for (int k = 0; k < din; ++k) acc = fmaf(xm[k], wt[(size_t)k * nb + bin], acc);
  const double lr = (double)acc + (double)mu[bin] + (double)sd[bin] * (double)mlp[(size_t)m * nb + bin];
  const double sv = exp(lr);
  sums[(size_t)m * nb + bin] = sv;
  sums2[(size_t)m * nb + bin] = (double)ratio[bin] * sv;
  if (logr) logr[(size_t)m * nb + bin] = lr;
}

}  // namespace
}  // namespace gwm

// ---------------------------------------------------------------------------
// Host side: the network object and the C ABI.
// ---------------------------------------------------------------------------
using gwm::bf16;

struct gwm_net {
  int n_layers = 0;
  std::vector<int> dims;  // dims[0] = inputs, dims[L] = outputs
  int batch_max = 0;
  int device = 0;
  cudaStream_t stream = nullptr;
  std::vector<void*> allocs;
  // per layer l (0..L-1): weights [dims[l+1] x dims[l]]
  std::vector<float*> w, b, gw_, gb, mw, vw, mb, vb;
  std::vector<bf16*> wb, wt;
  // activations: x0 (input), then per layer z (f32), h (bf16) and h^T (bf16)
  std::vector<bf16*> h, ht;   // h[0] = input
  std::vector<float*> z;      // z[l] = pre-activation of layer l
  std::vector<bf16*> dz, dzt; // gradients of pre-activations
  float* xin = nullptr;       // staging of the FP32 input
  float* target = nullptr;
  float* loss = nullptr;
  uint32_t* status = nullptr;
  int64_t step = 0;
  std::string err;
  // surrogate head (gwm_set_head / gwm_predict)
  bool has_head = false;
  float *h_mean = nullptr, *h_scale = nullptr, *h_wt = nullptr, *h_b0 = nullptr, *h_mu = nullptr, *h_sd = nullptr,
        *h_ratio = nullptr;
  double *h_data = nullptr, *h_theta = nullptr, *h_sums = nullptr, *h_sums2 = nullptr, *h_llh = nullptr,
         *h_logr = nullptr;
};

static thread_local std::string g_gwm_err;

static int gwm_fail(gwm_net* n, int code, const char* msg) {
  if (n) n->err = msg;
  else g_gwm_err = msg;
  return code;
}

#define GWM_CUDA(n, call)                                             \
  do {                                                                \
    cudaError_t _e = (call);                                          \
    if (_e != cudaSuccess) return gwm_fail((n), GW_ERR_CUDA, cudaGetErrorString(_e)); \
  } while (0)

template <typename T>
static int gwm_alloc(gwm_net* n, T** p, size_t count) {
  void* q = nullptr;
  if (cudaMalloc(&q, sizeof(T) * (count ? count : 1)) != cudaSuccess) {
    cudaGetLastError();
    return gwm_fail(n, GW_ERR_NOMEM, "cudaMalloc failed");
  }
  cudaMemset(q, 0, sizeof(T) * (count ? count : 1));
  n->allocs.push_back(q);
  *p = (T*)q;
  return GW_OK;
}

static size_t gemm_smem(int bn) { return 2 * (size_t)(gwm::kBM * gwm::kBK * 2 + bn * gwm::kBK * 2) + 1024; }

// C[M x N] = A[M x K] * B[N x K]^T with the given epilogue.
static int gemm(gwm_net* n, const bf16* A, const bf16* B, int M, int N, int K, const gwm::Epilogue& ep) {
  if (K % 8 != 0) return gwm_fail(n, GW_ERR_ARG, "GEMM K must be a multiple of 8");
  const int bn = N >= 256 ? 256 : (N > 64 ? 128 : 64);
  dim3 grid((N + bn - 1) / bn, (M + gwm::kBM - 1) / gwm::kBM);
  const size_t smem = gemm_smem(bn);
  if (bn == 256) {
    GWM_CUDA(n, cudaFuncSetAttribute(gwm::k_gemm<256>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    gwm::k_gemm<256><<<grid, gwm::kThreads, smem, n->stream>>>(A, B, M, N, K, ep, n->status);
  } else if (bn == 128) {
    GWM_CUDA(n, cudaFuncSetAttribute(gwm::k_gemm<128>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    gwm::k_gemm<128><<<grid, gwm::kThreads, smem, n->stream>>>(A, B, M, N, K, ep, n->status);
  } else {
    GWM_CUDA(n, cudaFuncSetAttribute(gwm::k_gemm<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    gwm::k_gemm<64><<<grid, gwm::kThreads, smem, n->stream>>>(A, B, M, N, K, ep, n->status);
  }
  GWM_CUDA(n, cudaGetLastError());
  return GW_OK;
}

static int check_status(gwm_net* n) {
  uint32_t h = 0;
  GWM_CUDA(n, cudaMemcpyAsync(&h, n->status, sizeof(uint32_t), cudaMemcpyDeviceToHost, n->stream));
  GWM_CUDA(n, cudaStreamSynchronize(n->stream));
  if (h) {
    cudaMemsetAsync(n->status, 0, sizeof(uint32_t), n->stream);
    return gwm_fail(n, GW_ERR_DEVICE_TIMEOUT, "a bounded wait on a tensor-core commit gave up");
  }
  return GW_OK;
}

extern "C" int gwm_create(const int32_t* dims, int32_t n_layers, int32_t batch_max, int32_t device, gwm_net** out) {
  if (!dims || !out || n_layers < 1 || n_layers > 16 || batch_max < 1 || batch_max % 8)
    return gwm_fail(nullptr, GW_ERR_ARG, "gwm_create: bad arguments (batch_max must be a multiple of 8)");
  for (int l = 0; l <= n_layers; ++l)
    if (dims[l] < 8 || dims[l] % 8) return gwm_fail(nullptr, GW_ERR_ARG, "gwm_create: widths must be multiples of 8");
  gwm_net* n = new gwm_net();
  n->n_layers = n_layers;
  n->dims.assign(dims, dims + n_layers + 1);
  n->batch_max = batch_max;
  n->device = device;
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&n->stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    delete n;
    return gwm_fail(nullptr, GW_ERR_CUDA, "gwm_create: no usable CUDA device");
  }
  const int L = n_layers, Bm = batch_max;
  n->w.resize(L); n->b.resize(L); n->gw_.resize(L); n->gb.resize(L); n->mw.resize(L); n->vw.resize(L);
  n->mb.resize(L); n->vb.resize(L); n->wb.resize(L); n->wt.resize(L);
  n->h.resize(L); n->ht.resize(L); n->z.resize(L); n->dz.resize(L); n->dzt.resize(L);
  int rc = GW_OK;
  for (int l = 0; l < L && rc == GW_OK; ++l) {
    const size_t nw = (size_t)dims[l + 1] * dims[l];
    rc |= gwm_alloc(n, &n->w[l], nw) | gwm_alloc(n, &n->gw_[l], nw) | gwm_alloc(n, &n->mw[l], nw) |
          gwm_alloc(n, &n->vw[l], nw) | gwm_alloc(n, &n->wb[l], nw) | gwm_alloc(n, &n->wt[l], nw);
    rc |= gwm_alloc(n, &n->b[l], dims[l + 1]) | gwm_alloc(n, &n->gb[l], dims[l + 1]) |
          gwm_alloc(n, &n->mb[l], dims[l + 1]) | gwm_alloc(n, &n->vb[l], dims[l + 1]);
    rc |= gwm_alloc(n, &n->h[l], (size_t)Bm * dims[l]) | gwm_alloc(n, &n->ht[l], (size_t)Bm * dims[l]);
    rc |= gwm_alloc(n, &n->z[l], (size_t)Bm * dims[l + 1]);
    rc |= gwm_alloc(n, &n->dz[l], (size_t)Bm * dims[l + 1]) | gwm_alloc(n, &n->dzt[l], (size_t)Bm * dims[l + 1]);
  }
  rc |= gwm_alloc(n, &n->xin, (size_t)Bm * dims[0]) | gwm_alloc(n, &n->target, (size_t)Bm * dims[L]) |
        gwm_alloc(n, &n->loss, 1) | gwm_alloc(n, &n->status, 1);
  if (rc != GW_OK) {
    g_gwm_err = n->err;
    for (void* p : n->allocs) cudaFree(p);
    delete n;
    return GW_ERR_NOMEM;
  }
  *out = n;
  return GW_OK;
}

extern "C" int gwm_destroy(gwm_net* n) {
  if (!n) return GW_ERR_ARG;
  cudaSetDevice(n->device);
  cudaStreamSynchronize(n->stream);
  for (void* p : n->allocs) cudaFree(p);
  cudaStreamDestroy(n->stream);
  delete n;
  return GW_OK;
}

extern "C" int gwm_last_error(const gwm_net* n, char* buf, size_t len) {
  if (!buf || !len) return GW_ERR_ARG;
  snprintf(buf, len, "%s", n ? n->err.c_str() : g_gwm_err.c_str());
  return GW_OK;
}

// Weights of layer l: w [dims[l+1] x dims[l]] row-major, b [dims[l+1]] (host, FP32).
extern "C" int gwm_set_layer(gwm_net* n, int32_t l, const float* w, const float* b) {
  if (!n || !w || !b || l < 0 || l >= n->n_layers) return GW_ERR_ARG;
  GWM_CUDA(n, cudaSetDevice(n->device));
  const int rows = n->dims[l + 1], cols = n->dims[l];
  const size_t nw = (size_t)rows * cols;
  GWM_CUDA(n, cudaMemcpy(n->w[l], w, sizeof(float) * nw, cudaMemcpyHostToDevice));
  GWM_CUDA(n, cudaMemcpy(n->b[l], b, sizeof(float) * rows, cudaMemcpyHostToDevice));
  // BF16 copies through a zero-learning-rate Adam pass (also clears the moments)
  GWM_CUDA(n, cudaMemset(n->gw_[l], 0, sizeof(float) * nw));
  GWM_CUDA(n, cudaMemset(n->mw[l], 0, sizeof(float) * nw));
  GWM_CUDA(n, cudaMemset(n->vw[l], 0, sizeof(float) * nw));
  GWM_CUDA(n, cudaMemset(n->mb[l], 0, sizeof(float) * rows));
  GWM_CUDA(n, cudaMemset(n->vb[l], 0, sizeof(float) * rows));
  gwm::k_adam<<<(unsigned)((nw + 255) / 256), 256, 0, n->stream>>>(n->w[l], n->gw_[l], n->mw[l], n->vw[l], (int)nw,
                                                                   rows, cols, 0.f, 0.9f, 0.999f, 1e-8f, 1.f, 1.f,
                                                                   n->wb[l], n->wt[l]);
  GWM_CUDA(n, cudaGetLastError());
  GWM_CUDA(n, cudaStreamSynchronize(n->stream));
  n->step = 0;
  return GW_OK;
}

extern "C" int gwm_get_layer(gwm_net* n, int32_t l, float* w, float* b) {
  if (!n || !w || !b || l < 0 || l >= n->n_layers) return GW_ERR_ARG;
  GWM_CUDA(n, cudaSetDevice(n->device));
  GWM_CUDA(n, cudaStreamSynchronize(n->stream));
  const size_t nw = (size_t)n->dims[l + 1] * n->dims[l];
  GWM_CUDA(n, cudaMemcpy(w, n->w[l], sizeof(float) * nw, cudaMemcpyDeviceToHost));
  GWM_CUDA(n, cudaMemcpy(b, n->b[l], sizeof(float) * n->dims[l + 1], cudaMemcpyDeviceToHost));
  return GW_OK;
}

static int forward(gwm_net* n, int B) {
  const int L = n->n_layers;
  for (int l = 0; l < L; ++l) {
    gwm::Epilogue ep{};
    ep.bias = n->b[l];
    ep.act = (l + 1 < L) ? 1 : 0;
    ep.out_f32 = n->z[l];
    if (l + 1 < L) {
      ep.out_bf16 = n->h[l + 1];
      ep.out_bf16_t = n->ht[l + 1];
      ep.ld_t = B;
    }
    int rc = gemm(n, n->h[l], n->wb[l], B, n->dims[l + 1], n->dims[l], ep);
    if (rc) return rc;
  }
  return GW_OK;
}

static int load_input(gwm_net* n, const float* x, int B, bool device_ptr) {
  const size_t cnt = (size_t)B * n->dims[0];
  GWM_CUDA(n, cudaMemcpyAsync(n->xin, x, sizeof(float) * cnt,
                              device_ptr ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, n->stream));
  gwm::k_to_bf16<<<(unsigned)((cnt + 255) / 256), 256, 0, n->stream>>>(n->xin, B, n->dims[0], n->h[0], n->ht[0], B);
  GWM_CUDA(n, cudaGetLastError());
  return GW_OK;
}

// Forward pass of B inputs x [B x dims[0]] (FP32, host or device) into
// y [B x dims[L]] (FP32, same side as x).
extern "C" int gwm_forward(gwm_net* n, const float* x, int32_t B, float* y, int32_t device_ptrs) {
  if (!n || !x || !y || B < 1 || B > n->batch_max || B % 8) return gwm_fail(n, GW_ERR_ARG, "gwm_forward: bad batch");
  GWM_CUDA(n, cudaSetDevice(n->device));
  int rc = load_input(n, x, B, device_ptrs != 0);
  if (!rc) rc = forward(n, B);
  if (rc) return rc;
  const int L = n->n_layers;
  GWM_CUDA(n, cudaMemcpyAsync(y, n->z[L - 1], sizeof(float) * (size_t)B * n->dims[L],
                              device_ptrs ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, n->stream));
  return check_status(n);
}

static int backward(gwm_net* n, int B) {
  const int L = n->n_layers;
  // dz[L-1] (and its transpose) was written by the loss kernel
  for (int l = L - 1; l >= 0; --l) {
    // dW_l = dz_l^T h_l : [dims[l+1] x dims[l]], K = B
    gwm::Epilogue e1{};
    e1.out_f32 = n->gw_[l];
    int rc = gemm(n, n->dzt[l], n->ht[l], n->dims[l + 1], n->dims[l], B, e1);
    if (rc) return rc;
    gwm::k_colsum<<<(n->dims[l + 1] + 255) / 256, 256, 0, n->stream>>>(n->dz[l], B, n->dims[l + 1], n->gb[l]);
    GWM_CUDA(n, cudaGetLastError());
    if (l > 0) {
      // dz_{l-1} = (dz_l W_l) * silu'(z_{l-1}) : [B x dims[l]], K = dims[l+1]
      gwm::Epilogue e2{};
      e2.gate = n->z[l - 1];
      e2.out_bf16 = n->dz[l - 1];
      e2.out_bf16_t = n->dzt[l - 1];
      e2.ld_t = B;
      rc = gemm(n, n->dz[l], n->wt[l], B, n->dims[l], n->dims[l + 1], e2);
      if (rc) return rc;
    }
  }
  return GW_OK;
}

static int loss_and_grad(gwm_net* n, const float* t, int B, bool device_ptr) {
  const int L = n->n_layers, C = n->dims[L];
  const size_t cnt = (size_t)B * C;
  GWM_CUDA(n, cudaMemcpyAsync(n->target, t, sizeof(float) * cnt,
                              device_ptr ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, n->stream));
  GWM_CUDA(n, cudaMemsetAsync(n->loss, 0, sizeof(float), n->stream));
  gwm::k_mse<<<(unsigned)((cnt + 255) / 256), 256, 0, n->stream>>>(n->z[L - 1], n->target, B, C, n->dz[L - 1],
                                                                    n->dzt[L - 1], B, n->loss);
  GWM_CUDA(n, cudaGetLastError());
  return GW_OK;
}

// Gradients of the mean squared error for a batch (no update): copied to
// the host, layer by layer, gw[l] [dims[l+1] x dims[l]], gb[l] [dims[l+1]].
extern "C" int gwm_gradients(gwm_net* n, const float* x, const float* t, int32_t B, float* const* gw,
                             float* const* gb, float* loss) {
  if (!n || !x || !t || !gw || !gb || B < 8 || B > n->batch_max || B % 8)
    return gwm_fail(n, GW_ERR_ARG, "gwm_gradients: bad batch");
  GWM_CUDA(n, cudaSetDevice(n->device));
  int rc = load_input(n, x, B, false);
  if (!rc) rc = forward(n, B);
  if (!rc) rc = loss_and_grad(n, t, B, false);
  if (!rc) rc = backward(n, B);
  if (rc) return rc;
  rc = check_status(n);
  if (rc) return rc;
  for (int l = 0; l < n->n_layers; ++l) {
    GWM_CUDA(n, cudaMemcpy(gw[l], n->gw_[l], sizeof(float) * (size_t)n->dims[l + 1] * n->dims[l],
                           cudaMemcpyDeviceToHost));
    GWM_CUDA(n, cudaMemcpy(gb[l], n->gb[l], sizeof(float) * n->dims[l + 1], cudaMemcpyDeviceToHost));
  }
  if (loss) GWM_CUDA(n, cudaMemcpy(loss, n->loss, sizeof(float), cudaMemcpyDeviceToHost));
  return GW_OK;
}

// One Adam step on a batch (x, t on the device when device_ptrs != 0).
extern "C" int gwm_train_step(gwm_net* n, const float* x, const float* t, int32_t B, float lr, int32_t device_ptrs,
                              float* loss) {
  if (!n || !x || !t || B < 8 || B > n->batch_max || B % 8) return gwm_fail(n, GW_ERR_ARG, "gwm_train_step: bad batch");
  GWM_CUDA(n, cudaSetDevice(n->device));
  int rc = load_input(n, x, B, device_ptrs != 0);
  if (!rc) rc = forward(n, B);
  if (!rc) rc = loss_and_grad(n, t, B, device_ptrs != 0);
  if (!rc) rc = backward(n, B);
  if (rc) return rc;
  n->step += 1;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - powf(b1, (float)n->step), c2 = 1.f - powf(b2, (float)n->step);
  for (int l = 0; l < n->n_layers; ++l) {
    const int rows = n->dims[l + 1], cols = n->dims[l];
    const int nw = rows * cols;
    gwm::k_adam<<<(nw + 255) / 256, 256, 0, n->stream>>>(n->w[l], n->gw_[l], n->mw[l], n->vw[l], nw, rows, cols, lr,
                                                         b1, b2, 1e-8f, c1, c2, n->wb[l], n->wt[l]);
    gwm::k_adam<<<(rows + 255) / 256, 256, 0, n->stream>>>(n->b[l], n->gb[l], n->mb[l], n->vb[l], rows, 0, 1, lr,
                                                           b1, b2, 1e-8f, c1, c2, nullptr, nullptr);
    GWM_CUDA(n, cudaGetLastError());
  }
  if (loss) {
    GWM_CUDA(n, cudaMemcpyAsync(loss, n->loss, sizeof(float), cudaMemcpyDeviceToHost, n->stream));
  }
  return check_status(n);
}

// Plain GEMM through the same kernel (tests): C[M x N] = A[M x K] B[N x K]^T,
// BF16 inputs, FP32 output, all host arrays.
extern "C" int gwm_gemm_test(const uint16_t* A, const uint16_t* B, int32_t M, int32_t N, int32_t K, float* C) {
  if (!A || !B || !C || M < 1 || N < 1 || K < 8 || K % 8) return gwm_fail(nullptr, GW_ERR_ARG, "gwm_gemm_test: bad sizes");
  gwm_net tmp;
  if (cudaStreamCreate(&tmp.stream) != cudaSuccess) return gwm_fail(nullptr, GW_ERR_CUDA, "no stream");
  bf16 *dA = nullptr, *dB = nullptr;
  float* dC = nullptr;
  int rc = gwm_alloc(&tmp, &dA, (size_t)M * K) | gwm_alloc(&tmp, &dB, (size_t)N * K) |
           gwm_alloc(&tmp, &dC, (size_t)M * N) | gwm_alloc(&tmp, &tmp.status, 1);
  if (rc == GW_OK) {
    cudaMemcpy(dA, A, sizeof(uint16_t) * (size_t)M * K, cudaMemcpyHostToDevice);
    cudaMemcpy(dB, B, sizeof(uint16_t) * (size_t)N * K, cudaMemcpyHostToDevice);
    gwm::Epilogue ep{};
    ep.out_f32 = dC;
    rc = gemm(&tmp, dA, dB, M, N, K, ep);
    if (rc == GW_OK) rc = check_status(&tmp);
    if (rc == GW_OK && cudaMemcpy(C, dC, sizeof(float) * (size_t)M * N, cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = GW_ERR_CUDA;
  }
  if (rc != GW_OK) g_gwm_err = tmp.err;
  for (void* p : tmp.allocs) cudaFree(p);
  cudaStreamDestroy(tmp.stream);
  return rc;
}

// ---------------------------------------------------------------------------
// Surrogate head: standardisation, affine base, output scaling, rate -> LLH.
// ---------------------------------------------------------------------------
extern "C" int gwm_set_head(gwm_net* n, const float* in_mean, const float* in_scale, const float* base_w,
                            const float* base_b, const float* out_mu, const float* out_sd, const float* ratio,
                            const double* data) {
  if (!n || !in_mean || !in_scale || !base_w || !base_b || !out_mu || !out_sd || !ratio || !data) return GW_ERR_ARG;
  GWM_CUDA(n, cudaSetDevice(n->device));
  const int din = n->dims[0], nb = n->dims[n->n_layers], Bm = n->batch_max;
  if (!n->has_head) {
    int rc = gwm_alloc(n, &n->h_mean, din) | gwm_alloc(n, &n->h_scale, din) |
             gwm_alloc(n, &n->h_wt, (size_t)din * nb) | gwm_alloc(n, &n->h_b0, nb) | gwm_alloc(n, &n->h_mu, nb) |
             gwm_alloc(n, &n->h_sd, nb) | gwm_alloc(n, &n->h_ratio, nb) | gwm_alloc(n, &n->h_data, nb) |
             gwm_alloc(n, &n->h_theta, (size_t)Bm * din) | gwm_alloc(n, &n->h_sums, (size_t)Bm * nb) |
             gwm_alloc(n, &n->h_sums2, (size_t)Bm * nb) | gwm_alloc(n, &n->h_llh, Bm) |
             gwm_alloc(n, &n->h_logr, (size_t)Bm * nb);
    if (rc) return rc;
    n->has_head = true;
  }
  // base_w arrives as [nb x din]; stored transposed [din x nb] for the head kernel
  std::vector<float> wt((size_t)din * nb);
  for (int b = 0; b < nb; ++b)
    for (int k = 0; k < din; ++k) wt[(size_t)k * nb + b] = base_w[(size_t)b * din + k];
  GWM_CUDA(n, cudaMemcpy(n->h_mean, in_mean, sizeof(float) * din, cudaMemcpyHostToDevice));
  GWM_CUDA(n, cudaMemcpy(n->h_scale, in_scale, sizeof(float) * din, cudaMemcpyHostToDevice));
  GWM_CUDA(n, cudaMemcpy(n->h_wt, wt.data(), sizeof(float) * wt.size(), cudaMemcpyHostToDevice));
  GWM_CUDA(n, cudaMemcpy(n->h_b0, base_b, sizeof(float) * nb, cudaMemcpyHostToDevice));
  GWM_CUDA(n, cudaMemcpy(n->h_mu, out_mu, sizeof(float) * nb, cudaMemcpyHostToDevice));
  GWM_CUDA(n, cudaMemcpy(n->h_sd, out_sd, sizeof(float) * nb, cudaMemcpyHostToDevice));
  GWM_CUDA(n, cudaMemcpy(n->h_ratio, ratio, sizeof(float) * nb, cudaMemcpyHostToDevice));
  GWM_CUDA(n, cudaMemcpy(n->h_data, data, sizeof(double) * nb, cudaMemcpyHostToDevice));
  return GW_OK;
}

// Surrogate statistical likelihood of B parameter points theta [B x din]
// (host FP64): llh [B]; log_rates [B x nb] optional.  llh_type as gw_eval.
extern "C" int gwm_predict(gwm_net* n, const double* theta, int32_t B, int32_t llh_type, double* llh,
                           double* log_rates) {
  if (!n || !theta || !llh || B < 1 || B > n->batch_max) return gwm_fail(n, GW_ERR_ARG, "gwm_predict: bad batch");
  if (!n->has_head) return gwm_fail(n, GW_ERR_STATE, "gwm_predict: gwm_set_head has not been called");
  GWM_CUDA(n, cudaSetDevice(n->device));
  const int din = n->dims[0], nb = n->dims[n->n_layers], L = n->n_layers;
  const int Bp = ((B + 7) / 8) * 8;  // GEMM rows in multiples of 8; the extra rows are zeros
  if (Bp > n->batch_max) return gwm_fail(n, GW_ERR_ARG, "gwm_predict: batch above batch_max after padding");
  if (Bp > B) GWM_CUDA(n, cudaMemsetAsync(n->h_theta, 0, sizeof(double) * (size_t)Bp * din, n->stream));
  GWM_CUDA(n, cudaMemcpyAsync(n->h_theta, theta, sizeof(double) * (size_t)B * din, cudaMemcpyHostToDevice, n->stream));
  gwm::k_standardize<<<(unsigned)(((size_t)Bp * din + 255) / 256), 256, 0, n->stream>>>(n->h_theta, Bp, din,
                                                                                     n->h_mean, n->h_scale, n->xin);
  gwm::k_to_bf16<<<(unsigned)(((size_t)Bp * din + 255) / 256), 256, 0, n->stream>>>(n->xin, Bp, din, n->h[0],
                                                                                    n->ht[0], Bp);
  GWM_CUDA(n, cudaGetLastError());
  int rc = forward(n, Bp);
  if (rc) return rc;
  gwm::k_head<<<dim3((nb + 255) / 256, B), 256, 0, n->stream>>>(n->xin, din, n->h_wt, n->h_b0, n->h_mu, n->h_sd,
                                                                 n->h_ratio, n->z[L - 1], nb, n->h_sums, n->h_sums2,
                                                                 log_rates ? n->h_logr : nullptr);
  GWM_CUDA(n, cudaGetLastError());
  rc = gw_llh_noalloc(n->h_sums, n->h_sums2, n->h_data, nb, B, llh_type, n->h_llh, n->stream);
  if (rc) return gwm_fail(n, rc, "gwm_predict: likelihood reduction failed");
  GWM_CUDA(n, cudaMemcpyAsync(llh, n->h_llh, sizeof(double) * B, cudaMemcpyDeviceToHost, n->stream));
  if (log_rates)
    GWM_CUDA(n, cudaMemcpyAsync(log_rates, n->h_logr, sizeof(double) * (size_t)B * nb, cudaMemcpyDeviceToHost,
                                n->stream));
  return check_status(n);
}
