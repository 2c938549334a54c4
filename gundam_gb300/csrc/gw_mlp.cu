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
#include <cuda.h>
#include <cuda_bf16.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cfloat>
#include <cstring>
#include <mutex>
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

__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor, K-major with the 128-byte swizzle: rows of
// 64 BF16 (128 bytes), 8-row atoms of 1024 bytes (SBO) whose 16-byte chunks
// are XOR-permuted by the row within the atom (the pattern the TMA unit
// writes with CU_TENSOR_MAP_SWIZZLE_128B into 1024-byte-aligned buffers);
// LBO is unused for this layout.  A K step of 16 elements adds 32 bytes.
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t addr) {
  uint64_t d = (uint64_t)((addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;             // LBO (unused)
  d |= (uint64_t)(1024 >> 4) << 32;   // SBO
  d |= (uint64_t)1 << 46;             // descriptor version
  d |= (uint64_t)2 << 61;             // layout: 128-byte swizzle
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

// 2-D tiled TMA load of box {8 elements, R rows} at (k, row) into shared
// memory, completing on an mbarrier (transaction bytes).
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int k, int row, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(k), "r"(row), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// Pipelined GEMM tile, C[128 x BN] = A[128 x K] * B[BN x K]^T.
//   * thread 0 (warp 0) issues the TMA loads of each 64-wide K tile into one
//     of S shared-memory stages (one box of 64 K-elements x rows per operand,
//     128-byte swizzle, 1024-byte-aligned stages); rows beyond M / N and
//     columns beyond K arrive as zeros;
//   * thread 32 (warp 1) waits for a stage, issues its four K = 16 MMAs and
//     commits them to the stage's "empty" barrier, which lets the producer
//     refill it; a final commit signals the epilogue;
//   * all four warps read the accumulator from TMEM (warp w: rows 32w..32w+31)
//     and store through a per-warp shared-memory transpose, so that row-major
//     stores and gate loads are coalesced.
// Every wait is bounded; on a timeout the tile records the failure in
// *status, drains its own copies (bounded) and frees TMEM.
template <int BN, int S>
__global__ void __launch_bounds__(kThreads) k_gemm(const __grid_constant__ CUtensorMap tmA,
                                                   const __grid_constant__ CUtensorMap tmB, int M, int N, int K,
                                                   Epilogue ep, uint32_t* status) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  constexpr int kA = kBM * kBK * 2;  // 16 KB
  constexpr int kB = BN * kBK * 2;
  constexpr int kStage = kA + kB;
  __shared__ __align__(8) uint64_t full[S], empty[S], done;
  __shared__ float sbias[BN];  // the tile's bias columns, read by every row of the epilogue
  __shared__ uint32_t tmem_base;
  __shared__ volatile int failed;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.y * kBM, n0 = blockIdx.x * BN;
  if (warp == 0) tmem_alloc(&tmem_base, BN);
  if (ep.bias) {
    // one coalesced load per column instead of one load per element in the
    // epilogue, where the dependent loads stalled the tile's four warps
    for (int c = tid; c < BN; c += kThreads) sbias[c] = (n0 + c < N) ? ep.bias[n0 + c] : 0.f;
  }
  if (tid == 0) {
    for (int i = 0; i < S; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], 1);
    }
    mbar_init(&done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    failed = 0;
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base;
  const int nk = (K + kBK - 1) / kBK;
  int produced = 0;

  if (tid == 0) {
    // producer
    for (int kt = 0; kt < nk; ++kt) {
      const int st = kt % S;
      if (kt >= S && !mbar_wait_bounded(&empty[st], (uint32_t)(((kt / S) - 1) & 1))) {
        failed = 1;
        break;
      }
      if (failed) break;
      unsigned char* a = smem + st * kStage;
      unsigned char* b = a + kA;
      mbar_arrive_expect(&full[st], (uint32_t)kStage);
      tma_load_2d(a, &tmA, kt * kBK, m0, &full[st]);
      tma_load_2d(b, &tmB, kt * kBK, n0, &full[st]);
      produced = kt + 1;
    }
  } else if (tid == 32) {
    // MMA issuer
    constexpr uint32_t idesc = instr_desc(kBM, BN);
    int kt = 0;
    for (; kt < nk; ++kt) {
      const int st = kt % S;
      if (!mbar_wait_bounded(&full[st], (uint32_t)((kt / S) & 1))) {
        failed = 1;
        break;
      }
      if (failed) break;
      tc_fence_after();
      const uint32_t a0 = smem_u32(smem + st * kStage), b0 = a0 + kA;
#pragma unroll
      for (int s16 = 0; s16 < kBK / 16; ++s16) {
        const uint64_t ad = smem_desc_sw128(a0 + s16 * 32);
        const uint64_t bd = smem_desc_sw128(b0 + s16 * 32);
        mma_bf16(tmem, ad, bd, idesc, (kt > 0 || s16 > 0) ? 1u : 0u);
      }
      mma_commit(&empty[st]);
    }
    // covers every MMA issued above (or none)
    mma_commit(&done);
  }
  __syncwarp();
  const bool ok = mbar_wait_bounded(&done, 0);
  if (!ok) failed = 1;
  __syncthreads();
  if (failed) {
    if (tid == 0) {
      atomicOr(status, 1u);
      // drain the copies this tile issued (bounded) before the block exits
      for (int kt = produced > S ? produced - S : 0; kt < produced; ++kt)
        mbar_wait_bounded(&full[kt % S], (uint32_t)((kt / S) & 1));
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, BN);
    return;
  }
  tc_fence_after();

  // epilogue: the pipeline's shared memory is free now
  float* tr = reinterpret_cast<float*>(smem) + warp * (32 * 33);
  const int rbase = m0 + warp * 32;
  const int r = rbase + lane;
  const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
  for (int c0 = 0; c0 < BN; c0 += 32) {
    if (n0 + c0 >= N) break;
    float v[32];
    tmem_ld32(lane_addr + (uint32_t)c0, v);
    const int ncol = min(32, N - (n0 + c0));
    if (ep.gate) {
      // coalesced load of the gate tile [32 rows x 32 cols] -> transpose
      __syncwarp();
      for (int i = 0; i < 32; ++i) {
        const int rr = rbase + i;
        tr[i * 33 + lane] = (rr < M && lane < ncol) ? ep.gate[(size_t)rr * N + n0 + c0 + lane] : 0.f;
      }
      __syncwarp();
#pragma unroll
      for (int q = 0; q < 32; ++q) {
        const float g = tr[lane * 33 + q];
        const float sg = sigmoidf_(g);
        v[q] *= sg * (1.f + g * (1.f - sg));
      }
    }
#pragma unroll
    for (int q = 0; q < 32; ++q)
      if (ep.bias && q < ncol) v[q] += sbias[c0 + q];
    if (ep.out_f32) {
      __syncwarp();
#pragma unroll
      for (int q = 0; q < 32; ++q) tr[lane * 33 + q] = v[q];
      __syncwarp();
      for (int i = 0; i < 32; ++i) {
        const int rr = rbase + i;
        if (rr < M && lane < ncol) ep.out_f32[(size_t)rr * N + n0 + c0 + lane] = tr[i * 33 + lane];
      }
    }
    if (ep.out_bf16 || ep.out_bf16_t) {
#pragma unroll
      for (int q = 0; q < 32; ++q) v[q] = (ep.act == 1) ? v[q] * sigmoidf_(v[q]) : v[q];
      if (ep.out_bf16_t && r < M) {
#pragma unroll
        for (int q = 0; q < 32; ++q)
          if (q < ncol) ep.out_bf16_t[(size_t)(n0 + c0 + q) * ep.ld_t + r] = __float2bfloat16(v[q]);
      }
      if (ep.out_bf16) {
        __syncwarp();
#pragma unroll
        for (int q = 0; q < 32; ++q) tr[lane * 33 + q] = v[q];
        __syncwarp();
        for (int i = 0; i < 32; ++i) {
          const int rr = rbase + i;
          if (rr < M && lane < ncol) ep.out_bf16[(size_t)rr * N + n0 + c0 + lane] = __float2bfloat16(tr[i * 33 + lane]);
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, BN);
}

// ---- small kernels ----
// Rows of a row-major FP32 matrix to BF16, row-major and transposed.  Row r
// of the output is row perm[r] of x (perm null: row r).  32 x 32 tiles go
// through shared memory so both stores are coalesced; block (32, 8).
__global__ void k_rows_to_bf16(const float* __restrict__ x, const int32_t* __restrict__ perm, int rows, int cols,
                               bf16* y, bf16* yt, int ld_t) {
  __shared__ bf16 tile[32][34];
  const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;
  for (int i = ty; i < 32; i += 8) {
    const int r = r0 + i, c = c0 + tx;
    bf16 v = __float2bfloat16(0.f);
    if (r < rows && c < cols) {
      const size_t src = perm ? (size_t)perm[r] : (size_t)r;
      v = __float2bfloat16(x[src * cols + c]);
      if (y) y[(size_t)r * cols + c] = v;
    }
    tile[i][tx] = v;
  }
  if (!yt) return;
  __syncthreads();
  for (int i = ty; i < 32; i += 8) {
    const int c = c0 + i, r = r0 + tx;
    if (c < cols && r < rows) yt[(size_t)c * ld_t + r] = tile[tx][i];
  }
}

// Mean squared error against target rows perm[r] of t (perm null: row r) and
// its gradient dy = 2 (y - t) / (rows * cols), row-major and transposed
// (tiled as k_rows_to_bf16).  loss += scale * sum e^2 / (rows * cols), one
// atomic per block.
__global__ void k_mse(const float* __restrict__ y, const float* __restrict__ t, const int32_t* __restrict__ perm,
                      int rows, int cols, bf16* dy, bf16* dyt, int ld_t, float* loss, float scale) {
  __shared__ bf16 tile[32][34];
  __shared__ float red[8];
  const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const float inv = 1.f / ((float)rows * (float)cols);
  float e2 = 0.f;
  for (int i = ty; i < 32; i += 8) {
    const int r = r0 + i, c = c0 + tx;
    bf16 g = __float2bfloat16(0.f);
    if (r < rows && c < cols) {
      const size_t tr = perm ? (size_t)perm[r] : (size_t)r;
      const float e = y[(size_t)r * cols + c] - t[tr * cols + c];
      e2 += e * e;
      g = __float2bfloat16(2.f * e * inv);
      dy[(size_t)r * cols + c] = g;
    }
    tile[i][tx] = g;
  }
  __syncthreads();
  for (int i = ty; i < 32; i += 8) {
    const int c = c0 + i, r = r0 + tx;
    if (c < cols && r < rows) dyt[(size_t)c * ld_t + r] = tile[tx][i];
  }
  for (int o = 16; o; o >>= 1) e2 += __shfl_xor_sync(0xffffffffu, e2, o);
  if (tx == 0) red[ty] = e2;
  __syncthreads();
  if (ty == 0 && tx == 0) {
    float b = 0.f;
    for (int i = 0; i < 8; ++i) b += red[i];
    atomicAdd(loss, b * inv * scale);
  }
}

// Column sums of a row-major BF16 matrix (bias gradients): block (32, 16),
// 32 columns per block, a fixed-order reduction over the 16 row strides.
__global__ void k_colsum(const bf16* __restrict__ g, int rows, int cols, float* out) {
  __shared__ float part[16][33];
  const int c = blockIdx.x * 32 + threadIdx.x;
  float s = 0.f;
  if (c < cols)
    for (int r = threadIdx.y; r < rows; r += 16) s += __bfloat162float(g[(size_t)r * cols + c]);
  part[threadIdx.y][threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.y == 0 && c < cols) {
    float t = 0.f;
    for (int i = 0; i < 16; ++i) t += part[i][threadIdx.x];
    out[c] = t;
  }
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

// Surrogate head (device pointers).  The predicted log rate of a bin is
//   base(x) + mu + sd * mlp(x)
// with x the standardised parameters and base either affine (nodes == 0:
// b0 + sum_k x_k tab[k][bin]) or additive piecewise-linear (nodes >= 2:
// b0 + sum_k interp_k(x_k), interp_k linear between `nodes` equally spaced
// values tab[k][0..nodes-1][bin] over x_k in [-lim, lim], constant outside).
// Sum w^2 is modelled as exp(r_b + sum_k x_k r_w[k][bin]) * rate (r_w optional).
struct Head {
  int din, nb, nodes;
  float lim;
  const float* tab;
  const float* b0;
  const float* mu;
  const float* sd;
  const float* r_w;
  const float* r_b;
};

__device__ __forceinline__ float head_base(const Head& h, const float* __restrict__ x, int bin) {
  float acc = h.b0[bin];
  if (h.nodes >= 2) {
    const float inv_w = (float)(h.nodes - 1) / (2.f * h.lim);
    for (int k = 0; k < h.din; ++k) {
      const float xc = fminf(fmaxf(x[k], -h.lim), h.lim);
      const float u = (xc + h.lim) * inv_w;
      const int i = min((int)u, h.nodes - 2);
      const float t = u - (float)i;
      const float* T = h.tab + ((size_t)k * h.nodes + i) * h.nb + bin;
      acc += fmaf(t, T[h.nb] - T[0], T[0]);
    }
  } else {
    for (int k = 0; k < h.din; ++k) acc = fmaf(x[k], h.tab[(size_t)k * h.nb + bin], acc);
  }
  return acc;
}


// log(data / mc) for data, mc > 0: log1p((data - mc) / mc) near 1, where
// log(data) - log(mc) would cancel in FP32, and the difference of logs away
// from it, where the ratio itself can underflow or overflow.
__device__ __forceinline__ float log_ratio_f(float data, float mc) {
  const float r = (data - mc) / mc;
  return fabsf(r) < 0.5f ? log1pf(r) : logf(data) - logf(mc);
}

// Per-bin likelihood term of the surrogate in FP32 (stage 1 only; the exact
// engine keeps its FP64 path).  Same formulas as the engine's FP64 ones:
// Poisson (PoissonLogLikelihood.h:19-53) and Barlow-Beeston OA2021
// (BarlowBeestonBanff2022.h:150-294), with log(data / mc) from log_ratio_f.
__device__ __forceinline__ float llh_term_f(int type, float data, float pred, float sumw2) {
  if (type == GW_LLH_POISSON) {
    if (pred <= 0.f) return INFINITY;
    if (data <= 0.f) return 2.f * pred;
    return 2.f * ((pred - data) + data * log_ratio_f(data, pred));
  }
  if (type != GW_LLH_BARLOW_BEESTON_OA2021) return 0.f;
  if (pred <= -1.f) return (pred <= 0.f && data > 0.f) ? INFINITY : 0.f;
  float newmc = pred, penalty = 0.f;
  if (sumw2 > 0.f) {
    const float f2 = sumw2 / (pred * pred);
    const float temp = sumw2 / pred - 1.f;
    const float temp2 = temp * temp + 4.f * data * f2;
    if (temp2 < 0.f) return INFINITY;
    const float beta = 0.5f * (sqrtf(temp2) - temp);
    newmc = fmaxf(pred * beta, FLT_MIN);
    penalty = (beta - 1.f) * (beta - 1.f) / (2.f * f2);
  }
  newmc = fmaxf(newmc, FLT_MIN);
  float stat;
  if (data <= FLT_EPSILON) stat = newmc;
  else stat = (newmc - data) + data * log_ratio_f(data, newmc);
  return 2.f * stat + 2.f * penalty;
}

// Derivatives of the FP32 per-bin term with respect to log(rate) and to
// log(sum w^2):
//   Poisson: dL/dlog mu = 2 (mu - n), dL/dlog s2 = 0;
//   Barlow-Beeston OA2021: beta minimises the bin's joint likelihood (its
//   quadratic is the stationarity condition), so by the envelope theorem the
//   derivatives are the partials at fixed beta of
//   L = 2 (beta mu - n + n log(n / (beta mu))) + (beta - 1)^2 mu^2 / s2:
//     dL/dlog mu = 2 (beta mu - n) + 2 (beta - 1)^2 / f2,
//     dL/dlog s2 = -(beta - 1)^2 / f2,  f2 = s2 / mu^2.
__device__ __forceinline__ void llh_term_grad_f(int type, float data, float pred, float sumw2, float& gmu,
                                                float& gs2) {
  gmu = 0.f;
  gs2 = 0.f;
  if (type == GW_LLH_POISSON) {
    if (pred > 0.f) gmu = 2.f * (pred - data);
    return;
  }
  if (type != GW_LLH_BARLOW_BEESTON_OA2021 || !(pred > 0.f)) return;
  if (sumw2 > 0.f) {
    const float f2 = sumw2 / (pred * pred);
    const float temp = sumw2 / pred - 1.f;
    const float temp2 = temp * temp + 4.f * data * f2;
    if (temp2 < 0.f) return;
    const float beta = 0.5f * (sqrtf(temp2) - temp);
    const float pen = (beta - 1.f) * (beta - 1.f) / f2;
    gmu = 2.f * (beta * pred - data) + 2.f * pen;
    gs2 = -pen;
  } else {
    gmu = 2.f * (pred - data);
  }
}

// Head and likelihood terms, fused.  Block (32 bins, 8 point rows); thread
// (x, y) of block (bx, by) handles bin 32 bx + x and the PPT points
// by * 8 PPT + y + 8 j.  The block first stages, for each of its points and
// parameters, the input x and (additive base) the table offset of the
// interpolation interval and its weight in shared memory; the inner loop is
// then two coalesced table loads and two FMAs per point and parameter, with
// the table lines of a bin shared through L1 across the block's points.
// Per point and block, the 32 bins' terms are summed by a fixed shuffle tree
// into part[point][bx] (FP64); optional outputs: sums, sums2 (FP64), log rates.
// GRAD: also, per (point, bin), G = dL/dlog mu + dL/dlog s2 (the derivative
// with respect to the log rate, the modelled sum of w^2 moving with it) and
// S = dL/dlog s2 into gbuf / sbuf, and dY = G * sd (the derivative with
// respect to the network output) as BF16 into dy.
template <int PPT, bool GRAD = false>
__global__ void __launch_bounds__(256) k_head_llh(Head h, const float* __restrict__ x, const float* __restrict__ mlp,
                                                  int C, const double* __restrict__ data, int llh_type,
                                                  double* __restrict__ part, double* sums, double* sums2,
                                                  double* logr, float* gbuf = nullptr, float* sbuf = nullptr,
                                                  bf16* dy = nullptr) {
  extern __shared__ unsigned char sh_raw[];
  constexpr int NP = 8 * PPT;  // points per block
  const int din = h.din;
  float* s_z = reinterpret_cast<float*>(sh_raw);          // [NP][din]
  float* s_t = s_z + NP * din;                            // [NP][din]
  int* s_off = reinterpret_cast<int*>(s_t + NP * din);    // [NP][din]
  const int mb = blockIdx.y * NP;
  const int tid = threadIdx.y * 32 + threadIdx.x;
  const bool additive = h.nodes >= 2;
  const float inv_w = additive ? (float)(h.nodes - 1) / (2.f * h.lim) : 0.f;
  for (int e = tid; e < NP * din; e += 256) {
    const int ml = e / din, k = e - ml * din, m = mb + ml;
    const float z = m < C ? x[(size_t)m * din + k] : 0.f;
    s_z[e] = z;
    if (additive) {
      const float xc = fminf(fmaxf(z, -h.lim), h.lim);
      const float u = (xc + h.lim) * inv_w;
      const int i = min((int)u, h.nodes - 2);
      s_t[e] = u - (float)i;
      s_off[e] = (k * h.nodes + i) * h.nb;
    } else {
      s_t[e] = z;
      s_off[e] = k * h.nb;
    }
  }
  __syncthreads();
  const int bin = blockIdx.x * 32 + threadIdx.x;
  const bool bin_ok = bin < h.nb;
  float acc[PPT], racc[PPT];
#pragma unroll
  for (int j = 0; j < PPT; ++j) {
    acc[j] = bin_ok ? h.b0[bin] : 0.f;
    racc[j] = bin_ok ? h.r_b[bin] : 0.f;
  }
  if (bin_ok) {
    const float* __restrict__ tab = h.tab + bin;
    const float* __restrict__ rw = h.r_w ? h.r_w + bin : nullptr;
    const int nb = h.nb;
#pragma unroll 4
    for (int k = 0; k < din; ++k) {
      const float w = rw ? __ldg(rw + (size_t)k * nb) : 0.f;
#pragma unroll
      for (int j = 0; j < PPT; ++j) {
        const int e = (threadIdx.y + 8 * j) * din + k;
        const int off = s_off[e];
        const float t = s_t[e];
        if (additive) {
          const float lo = __ldg(tab + off), hi = __ldg(tab + off + nb);
          acc[j] += fmaf(t, hi - lo, lo);
        } else {
          acc[j] = fmaf(t, __ldg(tab + off), acc[j]);
        }
        racc[j] = fmaf(s_z[e], w, racc[j]);
      }
    }
  }
#pragma unroll
  for (int j = 0; j < PPT; ++j) {
    const int m = mb + threadIdx.y + 8 * j;
    float term = 0.f;
    if (bin_ok && m < C) {
      const size_t o = (size_t)m * h.nb + bin;
      const float lr = acc[j] + h.mu[bin] + h.sd[bin] * mlp[o];
      const float mu = expf(lr), s2 = expf(lr + racc[j]);
      term = llh_term_f(llh_type, (float)data[bin], mu, s2);
      if (sums) sums[o] = (double)mu;
      if (sums2) sums2[o] = (double)s2;
      if (logr) logr[o] = (double)lr;
      if constexpr (GRAD) {
        float gmu, gs2;
        llh_term_grad_f(llh_type, (float)data[bin], mu, s2, gmu, gs2);
        const float G = gmu + gs2;
        gbuf[o] = G;
        sbuf[o] = gs2;
        dy[o] = __float2bfloat16(G * h.sd[bin]);
      }
    }
    double t = (double)term;
    for (int off = 16; off; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
    if (threadIdx.x == 0 && m < C) part[(size_t)m * gridDim.x + blockIdx.x] = t;
  }
}

// llh[m] = sum over blocks of part[m][*], one warp per point, fixed order.
__global__ void k_llh_finish(const double* __restrict__ part, int nblk, int C, double* __restrict__ llh) {
  const int m = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (m >= C) return;
  double s = 0.0;
  for (int b = lane; b < nblk; b += 32) s += part[(size_t)m * nblk + b];
  for (int off = 16; off; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  if (lane == 0) llh[m] = s;
}

// Gradient of the likelihood through the base and the sum-of-w^2 model, for
// point m = blockIdx.x and parameters k = blockIdx.y * 8 + (0..7):
//   gz[m][k] = sum_b G[m][b] * d base_b / d x_k + S[m][b] * r_w[k][b]
// (d base / d x_k: the slope of the interpolation interval of x_k, zero
// outside [-lim, lim]; affine base: tab[k][b]).  The point's G and S rows are
// staged in shared memory; fixed-order block reduction.
__global__ void __launch_bounds__(256) k_base_grad(Head h, const float* __restrict__ x, const float* __restrict__ G,
                                                   const float* __restrict__ S, float* __restrict__ gz) {
  extern __shared__ float shg[];
  float* g = shg;            // [nb]
  float* sg = shg + h.nb;    // [nb]
  __shared__ float red[8][8];
  const int m = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int b = tid; b < h.nb; b += 256) {
    g[b] = G[(size_t)m * h.nb + b];
    sg[b] = S[(size_t)m * h.nb + b];
  }
  __syncthreads();
  const bool additive = h.nodes >= 2;
  const float inv_w = additive ? (float)(h.nodes - 1) / (2.f * h.lim) : 0.f;
  for (int q = 0; q < 8; ++q) {
    const int k = blockIdx.y * 8 + q;
    if (k >= h.din) break;
    const float z = x[(size_t)m * h.din + k];
    const float* lo;
    float scale_ = 1.f;
    if (additive) {
      const float xc = fminf(fmaxf(z, -h.lim), h.lim);
      const float u = (xc + h.lim) * inv_w;
      const int i = min((int)u, h.nodes - 2);
      lo = h.tab + ((size_t)k * h.nodes + i) * h.nb;
      scale_ = (z > -h.lim && z < h.lim) ? inv_w : 0.f;
    } else {
      lo = h.tab + (size_t)k * h.nb;
    }
    const float* rw = h.r_w ? h.r_w + (size_t)k * h.nb : nullptr;
    float acc = 0.f;
    for (int b = tid; b < h.nb; b += 256) {
      const float slope = additive ? (lo[b + h.nb] - lo[b]) * scale_ : lo[b];
      acc = fmaf(g[b], slope, acc);
      if (rw) acc = fmaf(sg[b], rw[b], acc);
    }
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) red[q][warp] = acc;
  }
  __syncthreads();
  if (tid < 8) {
    const int k = blockIdx.y * 8 + tid;
    if (k < h.din) {
      float t = 0.f;
      for (int w = 0; w < 8; ++w) t += red[tid][w];
      gz[(size_t)m * h.din + k] = t;
    }
  }
}

// Per point (block), G groups of P32 threads as k_finish_accept: the value
// f = llh + penalty and the gradient with respect to the parameters,
// (gz + dx) / scale + 2 C^-1 (theta - mean) (prior optional).
__global__ void k_grad_finish(const double* __restrict__ part, int nblk, const double* __restrict__ theta, int P,
                              const float* __restrict__ scale, const float* __restrict__ gz,
                              const float* __restrict__ dx, const double* __restrict__ m,
                              const float* __restrict__ icov, double* __restrict__ f, double* __restrict__ grad) {
  extern __shared__ float shf2[];
  const int P32 = (P + 31) & ~31, Gn = blockDim.x / P32;
  float* d = shf2;              // [P32]
  float* up = shf2 + P32;       // [Gn][P32]
  float* red = up + Gn * P32;   // [P32]
  __shared__ double s_llh;
  const int c = blockIdx.x, lane = threadIdx.x & 31;
  if (threadIdx.x < 32) {
    double t = 0.0;
    for (int b = lane; b < nblk; b += 32) t += part[(size_t)c * nblk + b];
    for (int off = 16; off; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
    if (lane == 0) s_llh = t;
  }
  const int g = threadIdx.x / P32, p = threadIdx.x - g * P32;
  if (m) {
    if (g == 0) d[p] = p < P ? (float)(theta[(size_t)c * P + p] - m[p]) : 0.f;
    __syncthreads();
    const int ks = (P + Gn - 1) / Gn;
    if (p < P) {
      const int k0 = g * ks, k1 = min(P, (g + 1) * ks);
      float u0 = 0.f, u1 = 0.f;
      int k = k0;
      for (; k + 2 <= k1; k += 2) {
        u0 = fmaf(icov[(size_t)k * P + p], d[k], u0);
        u1 = fmaf(icov[(size_t)(k + 1) * P + p], d[k + 1], u1);
      }
      for (; k < k1; ++k) u0 = fmaf(icov[(size_t)k * P + p], d[k], u0);
      up[g * P32 + p] = u0 + u1;
    }
    __syncthreads();
  }
  if (g == 0) {
    float u = 0.f;
    if (m)
      for (int q = 0; q < Gn; ++q) u += (p < P) ? up[q * P32 + p] : 0.f;
    red[p] = m ? d[p] * u : 0.f;
    if (p < P) {
      const size_t o = (size_t)c * P + p;
      grad[o] = (double)((gz[o] + dx[o]) / scale[p]) + (m ? 2.0 * (double)u : 0.0);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double pen = 0.0;
    if (m)
      for (int i = 0; i < P32; ++i) pen += (double)red[i];
    f[c] = s_llh + pen;
  }
}

// Training target of a reweighted point, one thread per (point, bin):
//   t = (log(sum of weights) - base(x) - mu) / sd
// with the same FP32 base as k_head, so that k_head inverts it.
__global__ void k_target(Head h, const float* __restrict__ x, const double* __restrict__ sums,
                         float* __restrict__ t) {
  const int bin = blockIdx.x * blockDim.x + threadIdx.x;
  const int m = blockIdx.y;
  if (bin >= h.nb) return;
  const float* xm = x + (size_t)m * h.din;
  const double sv = sums[(size_t)m * h.nb + bin];
  const double lr = log(sv > 1e-300 ? sv : 1e-300);
  t[(size_t)m * h.nb + bin] = (float)((lr - (double)head_base(h, xm, bin) - (double)h.mu[bin]) / (double)h.sd[bin]);
}

}  // namespace
}  // namespace gwm

// ---------------------------------------------------------------------------
// Host side: the network object and the C ABI.
// ---------------------------------------------------------------------------
using gwm::bf16;

struct gwm_chain_state;
static void chain_free(gwm_chain_state* s);

struct gwm_net {
  gwm_chain_state* chain = nullptr;  // device state of the surrogate sub-chains (gwm_set_chain)
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
  int h_nodes = 0;
  float h_lim = 0.f;
  size_t h_tab_elems = 0;
  bool h_has_rw = false;
  float *h_mean = nullptr, *h_scale = nullptr, *h_tab = nullptr, *h_b0 = nullptr, *h_mu = nullptr, *h_sd = nullptr,
        *h_rb = nullptr, *h_rw = nullptr;
  double *h_data = nullptr, *h_theta = nullptr, *h_sums = nullptr, *h_sums2 = nullptr, *h_llh = nullptr,
         *h_logr = nullptr, *h_part = nullptr;
  // gradient buffers (gwm_value_grad), allocated on first use
  float *g_G = nullptr, *g_S = nullptr, *g_gz = nullptr, *g_dx = nullptr;
  double *g_f = nullptr, *g_grad = nullptr;
  // training set on the device (gwm_train_reserve / gwm_train_append*):
  // standardised inputs [train_max x dims[0]] and targets [train_max x dims[L]]
  float *train_x = nullptr, *train_t = nullptr;
  int64_t train_n = 0, train_max = 0;
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

static size_t gemm_smem(int bn, int stages) {
  return (size_t)stages * (gwm::kBM * gwm::kBK * 2 + bn * gwm::kBK * 2) + 1024;
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, []() {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
    else
      cudaGetLastError();
  });
  return fn;
}

// Tensor map of a row-major BF16 matrix [rows x K] (K % 8 == 0, 16-byte
// aligned rows) read in boxes of 64 K-elements (128 bytes) x box_rows rows
// with the 128-byte swizzle, zero fill.
static int make_map(gwm_net* n, CUtensorMap* map, const bf16* p, int rows, int K, int box_rows) {
  EncodeTiledFn enc = encode_tiled();
  if (!enc) return gwm_fail(n, GW_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
  if (((uintptr_t)p & 15) != 0) return gwm_fail(n, GW_ERR_ARG, "GEMM operand not 16-byte aligned");
  const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)K * 2};
  const cuuint32_t box[2] = {(cuuint32_t)gwm::kBK, (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void*)p, dims, strides, box, estr,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return gwm_fail(n, GW_ERR_CUDA, "cuTensorMapEncodeTiled failed");
  return GW_OK;
}

template <int BN, int S>
static int launch_gemm(gwm_net* n, const bf16* A, const bf16* B, int M, int N, int K, const gwm::Epilogue& ep) {
  CUtensorMap ma, mb;
  int rc = make_map(n, &ma, A, M, K, gwm::kBM);
  if (!rc) rc = make_map(n, &mb, B, N, K, BN);
  if (rc) return rc;
  const size_t smem = gemm_smem(BN, S);
  static std::once_flag once;
  std::call_once(once, [smem]() {
    cudaFuncSetAttribute(gwm::k_gemm<BN, S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  });
  dim3 grid((N + BN - 1) / BN, (M + gwm::kBM - 1) / gwm::kBM);
  gwm::k_gemm<BN, S><<<grid, gwm::kThreads, smem, n->stream>>>(ma, mb, M, N, K, ep, n->status);
  GWM_CUDA(n, cudaGetLastError());
  return GW_OK;
}

// C[M x N] = A[M x K] * B[N x K]^T with the given epilogue.  The widest tile
// that still gives one CTA per SM or more (148 of GB300's 152), else the
// narrowest (64 columns): at the network's sizes a launch is one wave, and
// a tile runs few K steps, so more CTAs, not wider tiles, keep the tensor
// pipe busy (hidden layers, M = 2048, N = 512: 64 CTAs of 128 columns left
// 88 SMs idle).  Ring depth: 128 x 256 tiles take two stages, so that two CTAs
// (and their accumulators, 256 TMEM columns each) share an SM and one's
// epilogue overlaps the other's MMAs; 64- and 128-column tiles take four.
// The tile shape does not change the order of any accumulation.
static int gemm(gwm_net* n, const bf16* A, const bf16* B, int M, int N, int K, const gwm::Epilogue& ep) {
  if (K % 8 != 0) return gwm_fail(n, GW_ERR_ARG, "GEMM K must be a multiple of 8");
  const int tiles_m = (M + gwm::kBM - 1) / gwm::kBM;
  constexpr int kWave = 148;
  if (N > 128 && tiles_m * ((N + 255) / 256) >= kWave) return launch_gemm<256, 2>(n, A, B, M, N, K, ep);
  if (N > 64 && tiles_m * ((N + 127) / 128) >= kWave) return launch_gemm<128, 4>(n, A, B, M, N, K, ep);
  return launch_gemm<64, 4>(n, A, B, M, N, K, ep);
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
  cudaFree(n->train_x);
  cudaFree(n->train_t);
  cudaFree(n->h_tab);
  chain_free(n->chain);
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

static dim3 tiles32(int rows, int cols) { return dim3((unsigned)((cols + 31) / 32), (unsigned)((rows + 31) / 32)); }

// Input rows to BF16 (and transposed) for the first GEMM; row r is perm[r] of x (perm null: r).
// The transposed copy feeds the weight gradient of the first layer only.
static int stage_input(gwm_net* n, const float* x, const int32_t* perm, int B, bool transposed = true) {
  gwm::k_rows_to_bf16<<<tiles32(B, n->dims[0]), dim3(32, 8), 0, n->stream>>>(
      x, perm, B, n->dims[0], n->h[0], transposed ? n->ht[0] : nullptr, B);
  GWM_CUDA(n, cudaGetLastError());
  return GW_OK;
}

static int load_input(gwm_net* n, const float* x, int B, bool device_ptr) {
  const size_t cnt = (size_t)B * n->dims[0];
  GWM_CUDA(n, cudaMemcpyAsync(n->xin, x, sizeof(float) * cnt,
                              device_ptr ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, n->stream));
  return stage_input(n, n->xin, nullptr, B);
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
    gwm::k_colsum<<<(n->dims[l + 1] + 31) / 32, dim3(32, 16), 0, n->stream>>>(n->dz[l], B, n->dims[l + 1], n->gb[l]);
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

// Loss and output gradient against targets t (rows perm[r] when perm is set);
// adds scale * loss into *loss.
static int mse(gwm_net* n, const float* t, const int32_t* perm, int B, float* loss, float scale) {
  const int L = n->n_layers, C = n->dims[L];
  gwm::k_mse<<<tiles32(B, C), dim3(32, 8), 0, n->stream>>>(n->z[L - 1], t, perm, B, C, n->dz[L - 1], n->dzt[L - 1],
                                                            B, loss, scale);
  GWM_CUDA(n, cudaGetLastError());
  return GW_OK;
}

static int loss_and_grad(gwm_net* n, const float* t, int B, bool device_ptr) {
  const int L = n->n_layers, C = n->dims[L];
  const size_t cnt = (size_t)B * C;
  GWM_CUDA(n, cudaMemcpyAsync(n->target, t, sizeof(float) * cnt,
                              device_ptr ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, n->stream));
  GWM_CUDA(n, cudaMemsetAsync(n->loss, 0, sizeof(float), n->stream));
  return mse(n, n->target, nullptr, B, n->loss, 1.f);
}

// One Adam update of every layer with learning rate lr.
static int adam_all(gwm_net* n, float lr) {
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
  if (!rc) rc = adam_all(n, lr);
  if (rc) return rc;
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
static gwm::Head head_view(const gwm_net* n) {
  gwm::Head h{};
  h.din = n->dims[0];
  h.nb = n->dims[n->n_layers];
  h.nodes = n->h_nodes;
  h.lim = n->h_lim;
  h.tab = n->h_tab;
  h.b0 = n->h_b0;
  h.mu = n->h_mu;
  h.sd = n->h_sd;
  h.r_w = n->h_has_rw ? n->h_rw : nullptr;
  h.r_b = n->h_rb;
  return h;
}

// Buffers of the head and of gwm_predict; the base table is (re)sized to tab_elems.
static int head_alloc(gwm_net* n, size_t tab_elems) {
  const int din = n->dims[0], nb = n->dims[n->n_layers], Bm = n->batch_max;
  if (!n->has_head) {
    int rc = gwm_alloc(n, &n->h_mean, din) | gwm_alloc(n, &n->h_scale, din) | gwm_alloc(n, &n->h_b0, nb) |
             gwm_alloc(n, &n->h_mu, nb) | gwm_alloc(n, &n->h_sd, nb) | gwm_alloc(n, &n->h_rb, nb) |
             gwm_alloc(n, &n->h_rw, (size_t)din * nb) | gwm_alloc(n, &n->h_data, nb) |
             gwm_alloc(n, &n->h_theta, (size_t)Bm * din) | gwm_alloc(n, &n->h_sums, (size_t)Bm * nb) |
             gwm_alloc(n, &n->h_sums2, (size_t)Bm * nb) | gwm_alloc(n, &n->h_llh, Bm) |
             gwm_alloc(n, &n->h_logr, (size_t)Bm * nb) | gwm_alloc(n, &n->h_part, (size_t)Bm * ((nb + 31) / 32));
    if (rc) return rc;
    n->has_head = true;
  }
  if (n->h_tab_elems != tab_elems) {
    GWM_CUDA(n, cudaStreamSynchronize(n->stream));
    cudaFree(n->h_tab);
    n->h_tab = nullptr;
    n->h_tab_elems = 0;
    if (cudaMalloc(&n->h_tab, sizeof(float) * tab_elems) != cudaSuccess) {
      cudaGetLastError();
      n->h_tab = nullptr;
      return gwm_fail(n, GW_ERR_NOMEM, "cudaMalloc failed (head table)");
    }
    n->h_tab_elems = tab_elems;
  }
  return GW_OK;
}

// Uploads the parts shared by both head forms.
static int head_common(gwm_net* n, const float* in_mean, const float* in_scale, const float* base_b,
                       const float* out_mu, const float* out_sd, const float* ratio_w, const double* data) {
  const int din = n->dims[0], nb = n->dims[n->n_layers];
  GWM_CUDA(n, cudaMemcpy(n->h_mean, in_mean, sizeof(float) * din, cudaMemcpyHostToDevice));
  GWM_CUDA(n, cudaMemcpy(n->h_scale, in_scale, sizeof(float) * din, cudaMemcpyHostToDevice));
  GWM_CUDA(n, cudaMemcpy(n->h_b0, base_b, sizeof(float) * nb, cudaMemcpyHostToDevice));
  GWM_CUDA(n, cudaMemcpy(n->h_mu, out_mu, sizeof(float) * nb, cudaMemcpyHostToDevice));
  GWM_CUDA(n, cudaMemcpy(n->h_sd, out_sd, sizeof(float) * nb, cudaMemcpyHostToDevice));
  GWM_CUDA(n, cudaMemcpy(n->h_data, data, sizeof(double) * nb, cudaMemcpyHostToDevice));
  n->h_has_rw = ratio_w != nullptr;
  if (ratio_w) {
    // [nb x din] -> [din x nb]
    std::vector<float> rt((size_t)din * nb);
    for (int b = 0; b < nb; ++b)
      for (int k = 0; k < din; ++k) rt[(size_t)k * nb + b] = ratio_w[(size_t)b * din + k];
    GWM_CUDA(n, cudaMemcpy(n->h_rw, rt.data(), sizeof(float) * rt.size(), cudaMemcpyHostToDevice));
  }
  return GW_OK;
}

extern "C" int gwm_set_head(gwm_net* n, const float* in_mean, const float* in_scale, const float* base_w,
                            const float* base_b, const float* out_mu, const float* out_sd, const float* ratio,
                            const double* data) {
  if (!n || !in_mean || !in_scale || !base_w || !base_b || !out_mu || !out_sd || !ratio || !data) return GW_ERR_ARG;
  GWM_CUDA(n, cudaSetDevice(n->device));
  const int din = n->dims[0], nb = n->dims[n->n_layers];
  int rc = head_alloc(n, (size_t)din * nb);
  if (rc) return rc;
  // base_w arrives as [nb x din]; stored transposed [din x nb] for the head kernel
  std::vector<float> wt((size_t)din * nb), lr(nb);
  for (int b = 0; b < nb; ++b)
    for (int k = 0; k < din; ++k) wt[(size_t)k * nb + b] = base_w[(size_t)b * din + k];
  for (int b = 0; b < nb; ++b) lr[b] = ratio[b] > 0.f ? logf(ratio[b]) : -1e30f;
  GWM_CUDA(n, cudaMemcpy(n->h_tab, wt.data(), sizeof(float) * wt.size(), cudaMemcpyHostToDevice));
  GWM_CUDA(n, cudaMemcpy(n->h_rb, lr.data(), sizeof(float) * nb, cudaMemcpyHostToDevice));
  n->h_nodes = 0;
  n->h_lim = 0.f;
  return head_common(n, in_mean, in_scale, base_b, out_mu, out_sd, nullptr, data);
}

extern "C" int gwm_set_head_additive(gwm_net* n, const float* in_mean, const float* in_scale, int32_t nodes,
                                     float lim, const float* base_tab, const float* base_b, const float* out_mu,
                                     const float* out_sd, const float* ratio_w, const float* ratio_b,
                                     const double* data) {
  if (!n || !in_mean || !in_scale || !base_tab || !base_b || !out_mu || !out_sd || !ratio_b || !data || nodes < 2 ||
      nodes > 4096 || !(lim > 0.f))
    return gwm_fail(n, GW_ERR_ARG, "gwm_set_head_additive: bad arguments");
  GWM_CUDA(n, cudaSetDevice(n->device));
  const int din = n->dims[0], nb = n->dims[n->n_layers];
  const size_t te = (size_t)din * nodes * nb;
  int rc = head_alloc(n, te);
  if (rc) return rc;
  GWM_CUDA(n, cudaMemcpy(n->h_tab, base_tab, sizeof(float) * te, cudaMemcpyHostToDevice));
  GWM_CUDA(n, cudaMemcpy(n->h_rb, ratio_b, sizeof(float) * nb, cudaMemcpyHostToDevice));
  n->h_nodes = nodes;
  n->h_lim = lim;
  return head_common(n, in_mean, in_scale, base_b, out_mu, out_sd, ratio_w, data);
}

// Fused head + likelihood of the first C rows of the network's output (xin
// holds their standardised inputs): h_llh [C]; with `outputs`, h_sums,
// h_sums2 and h_logr too.
static int head_llh(gwm_net* n, int C, int llh_type, bool outputs, bool finish = true) {
  const int nb = n->dims[n->n_layers], L = n->n_layers;
  constexpr int kPPT = 2;
  const int nbx = (nb + 31) / 32;
  dim3 grid(nbx, (C + 8 * kPPT - 1) / (8 * kPPT));
  const size_t shm = (size_t)8 * kPPT * n->dims[0] * 12;
  if (shm > 48 * 1024) {
    static std::once_flag once;
    std::call_once(once, []() {
      cudaFuncSetAttribute(gwm::k_head_llh<kPPT>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    });
    if (shm > 200 * 1024) return gwm_fail(n, GW_ERR_LIMIT, "surrogate head: too many inputs");
  }
  gwm::k_head_llh<kPPT><<<grid, dim3(32, 8), shm, n->stream>>>(
      head_view(n), n->xin, n->z[L - 1], C, n->h_data, llh_type, n->h_part, outputs ? n->h_sums : nullptr,
      outputs ? n->h_sums2 : nullptr, outputs ? n->h_logr : nullptr);
  if (finish) gwm::k_llh_finish<<<(C + 7) / 8, 256, 0, n->stream>>>(n->h_part, nbx, C, n->h_llh);
  GWM_CUDA(n, cudaGetLastError());
  return GW_OK;
}

// Surrogate statistical likelihood of B parameter points theta [B x din]
// (host FP64): llh [B]; log_rates [B x nb] optional.  llh_type as gw_eval.
extern "C" int gwm_predict(gwm_net* n, const double* theta, int32_t B, int32_t llh_type, double* llh,
                           double* log_rates) {
  if (!n || !theta || !llh || B < 1 || B > n->batch_max) return gwm_fail(n, GW_ERR_ARG, "gwm_predict: bad batch");
  if (!n->has_head) return gwm_fail(n, GW_ERR_STATE, "gwm_predict: gwm_set_head has not been called");
  GWM_CUDA(n, cudaSetDevice(n->device));
  const int din = n->dims[0], nb = n->dims[n->n_layers];
  const int Bp = ((B + 7) / 8) * 8;  // GEMM rows in multiples of 8; the extra rows are zeros
  if (Bp > n->batch_max) return gwm_fail(n, GW_ERR_ARG, "gwm_predict: batch above batch_max after padding");
  if (Bp > B) GWM_CUDA(n, cudaMemsetAsync(n->h_theta, 0, sizeof(double) * (size_t)Bp * din, n->stream));
  GWM_CUDA(n, cudaMemcpyAsync(n->h_theta, theta, sizeof(double) * (size_t)B * din, cudaMemcpyHostToDevice, n->stream));
  gwm::k_standardize<<<(unsigned)(((size_t)Bp * din + 255) / 256), 256, 0, n->stream>>>(n->h_theta, Bp, din,
                                                                                     n->h_mean, n->h_scale, n->xin);
  int rc = stage_input(n, n->xin, nullptr, Bp, false);
  if (rc) return rc;
  GWM_CUDA(n, cudaGetLastError());
  rc = forward(n, Bp);
  if (rc) return rc;
  rc = head_llh(n, B, llh_type, log_rates != nullptr);
  if (rc) return rc;
  GWM_CUDA(n, cudaMemcpyAsync(llh, n->h_llh, sizeof(double) * B, cudaMemcpyDeviceToHost, n->stream));
  if (log_rates)
    GWM_CUDA(n, cudaMemcpyAsync(log_rates, n->h_logr, sizeof(double) * (size_t)B * nb, cudaMemcpyDeviceToHost,
                                n->stream));
  return check_status(n);
}

// ---------------------------------------------------------------------------
// Training set on the device and the training loop.
// ---------------------------------------------------------------------------
extern "C" int gwm_train_reserve(gwm_net* n, int64_t n_max) {
  if (!n || n_max < 8) return gwm_fail(n, GW_ERR_ARG, "gwm_train_reserve: n_max must be >= 8");
  GWM_CUDA(n, cudaSetDevice(n->device));
  GWM_CUDA(n, cudaStreamSynchronize(n->stream));
  cudaFree(n->train_x);
  cudaFree(n->train_t);
  n->train_x = n->train_t = nullptr;
  n->train_n = n->train_max = 0;
  const int din = n->dims[0], nb = n->dims[n->n_layers];
  if (cudaMalloc(&n->train_x, sizeof(float) * (size_t)n_max * din) != cudaSuccess ||
      cudaMalloc(&n->train_t, sizeof(float) * (size_t)n_max * nb) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(n->train_x);
    cudaFree(n->train_t);
    n->train_x = n->train_t = nullptr;
    return gwm_fail(n, GW_ERR_NOMEM, "gwm_train_reserve: cudaMalloc failed");
  }
  n->train_max = n_max;
  return GW_OK;
}

extern "C" int gwm_train_size(gwm_net* n, int64_t* count) {
  if (!n || !count) return GW_ERR_ARG;
  *count = n->train_n;
  return GW_OK;
}

// Standardises h_theta rows and turns h_sums rows into targets at the end of
// the training set (the head must be set).
static int append_rows(gwm_net* n, int K) {
  const int din = n->dims[0], nb = n->dims[n->n_layers];
  float* x = n->train_x + (size_t)n->train_n * din;
  gwm::k_standardize<<<(unsigned)(((size_t)K * din + 255) / 256), 256, 0, n->stream>>>(n->h_theta, K, din, n->h_mean,
                                                                                    n->h_scale, x);
  gwm::k_target<<<dim3((nb + 255) / 256, K), 256, 0, n->stream>>>(head_view(n), x, n->h_sums,
                                                                  n->train_t + (size_t)n->train_n * nb);
  GWM_CUDA(n, cudaGetLastError());
  n->train_n += K;
  return GW_OK;
}

static int append_check(gwm_net* n, const double* theta, int K, const char* who) {
  if (!n || !theta || K < 1 || K > n->batch_max) return gwm_fail(n, GW_ERR_ARG, who);
  if (!n->has_head) return gwm_fail(n, GW_ERR_STATE, "training targets need the head (gwm_set_head) first");
  if (n->train_n + K > n->train_max) return gwm_fail(n, GW_ERR_LIMIT, "training set full (gwm_train_reserve)");
  return GW_OK;
}

// Appends K points theta [K x dims[0]] (host FP64) with their bin sums
// [K x dims[L]] (FP64, host, or device memory when sums_on_device != 0).
extern "C" int gwm_train_append(gwm_net* n, const double* theta, const double* sums, int32_t K,
                                int32_t sums_on_device) {
  int rc = append_check(n, theta, K, "gwm_train_append: bad arguments");
  if (rc) return rc;
  if (!sums) return gwm_fail(n, GW_ERR_ARG, "gwm_train_append: sums missing");
  GWM_CUDA(n, cudaSetDevice(n->device));
  const int din = n->dims[0], nb = n->dims[n->n_layers];
  GWM_CUDA(n, cudaMemcpyAsync(n->h_theta, theta, sizeof(double) * (size_t)K * din, cudaMemcpyHostToDevice, n->stream));
  GWM_CUDA(n, cudaMemcpyAsync(n->h_sums, sums, sizeof(double) * (size_t)K * nb,
                              sums_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, n->stream));
  rc = append_rows(n, K);
  if (rc) return rc;
  GWM_CUDA(n, cudaStreamSynchronize(n->stream));
  return GW_OK;
}

// Appends K points theta [K x dims[0]] (host FP64) reweighted exactly by the
// engine e on the network's stream; nothing leaves the device.  The engine's
// parameter count must equal dims[0], its bin count dims[L], and K <= its k_max.
extern "C" int gwm_train_append_eval(gwm_net* n, gw_engine* e, const double* theta, int32_t K) {
  int rc = append_check(n, theta, K, "gwm_train_append_eval: bad arguments");
  if (rc) return rc;
  if (!e) return gwm_fail(n, GW_ERR_ARG, "gwm_train_append_eval: no engine");
  GWM_CUDA(n, cudaSetDevice(n->device));
  const int din = n->dims[0];
  GWM_CUDA(n, cudaMemcpyAsync(n->h_theta, theta, sizeof(double) * (size_t)K * din, cudaMemcpyHostToDevice, n->stream));
  rc = gw_eval_device(e, n->h_theta, K, n->h_sums, n->h_sums2, nullptr, nullptr, (void*)n->stream);
  if (rc) {
    char buf[256];
    gw_last_error(e, buf, sizeof(buf));
    n->err = std::string("gwm_train_append_eval: engine: ") + buf;
    return rc;
  }
  return append_rows(n, K);
}

// Trains on the device-resident set: `epochs` passes of floor(count / batch)
// Adam steps over a seeded permutation per epoch, learning rate cosine-decayed
// from lr0 to lr_min over all steps.  No host synchronisation between steps;
// losses[e] = mean training loss of epoch e (optional).
extern "C" int gwm_train_epochs(gwm_net* n, int32_t epochs, int32_t batch, float lr0, float lr_min, uint64_t seed,
                                float* losses) {
  if (!n || epochs < 1 || batch < 8 || batch % 8 || batch > n->batch_max)
    return gwm_fail(n, GW_ERR_ARG, "gwm_train_epochs: bad epochs or batch");
  if (n->train_n < batch) return gwm_fail(n, GW_ERR_STATE, "gwm_train_epochs: fewer training points than one batch");
  GWM_CUDA(n, cudaSetDevice(n->device));
  const int64_t N = n->train_n;
  const int64_t spe = N / batch, total = (int64_t)epochs * spe;
  const int din = n->dims[0], nb = n->dims[n->n_layers];
  // permutations of all epochs, drawn on the host (splitmix64 + Fisher-Yates)
  std::vector<int32_t> perm((size_t)epochs * N);
  uint64_t st = seed;
  auto next = [&st]() {
    uint64_t z = (st += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  };
  for (int e = 0; e < epochs; ++e) {
    int32_t* p = perm.data() + (size_t)e * N;
    for (int64_t i = 0; i < N; ++i) p[i] = (int32_t)i;
    for (int64_t i = N - 1; i > 0; --i) {
      const int64_t j = (int64_t)(next() % (uint64_t)(i + 1));
      std::swap(p[i], p[j]);
    }
  }
  int32_t* d_perm = nullptr;
  float* d_loss = nullptr;
  if (cudaMalloc(&d_perm, sizeof(int32_t) * perm.size()) != cudaSuccess ||
      cudaMalloc(&d_loss, sizeof(float) * epochs) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(d_perm);
    return gwm_fail(n, GW_ERR_NOMEM, "gwm_train_epochs: cudaMalloc failed");
  }
  int rc = GW_OK;
  if (cudaMemcpyAsync(d_perm, perm.data(), sizeof(int32_t) * perm.size(), cudaMemcpyHostToDevice, n->stream) !=
          cudaSuccess ||
      cudaMemsetAsync(d_loss, 0, sizeof(float) * epochs, n->stream) != cudaSuccess)
    rc = gwm_fail(n, GW_ERR_CUDA, "gwm_train_epochs: copy failed");
  const float inv_spe = 1.f / (float)spe;
  for (int64_t s = 0; s < total && rc == GW_OK; ++s) {
    const int64_t e = s / spe, j = s % spe;
    const int32_t* p = d_perm + e * N + j * batch;
    const double c = std::cos(M_PI * (double)s / (double)total);
    const float lr = (float)(lr_min + 0.5 * (lr0 - lr_min) * (1.0 + c));
    rc = stage_input(n, n->train_x, p, batch);
    if (!rc) rc = forward(n, batch);
    if (!rc) rc = mse(n, n->train_t, p, batch, d_loss + e, inv_spe);
    if (!rc) rc = backward(n, batch);
    if (!rc) rc = adam_all(n, lr);
  }
  (void)din;
  (void)nb;
  if (rc == GW_OK) rc = check_status(n);
  if (rc == GW_OK && losses &&
      cudaMemcpy(losses, d_loss, sizeof(float) * epochs, cudaMemcpyDeviceToHost) != cudaSuccess)
    rc = gwm_fail(n, GW_ERR_CUDA, "gwm_train_epochs: loss copy failed");
  cudaStreamSynchronize(n->stream);
  cudaFree(d_perm);
  cudaFree(d_loss);
  return rc;
}

// Copies rows [first, first + count) of the training set to the host:
// x [count x dims[0]] standardised inputs, t [count x dims[L]] targets.
extern "C" int gwm_train_read(gwm_net* n, int64_t first, int32_t count, float* x, float* t) {
  if (!n || first < 0 || count < 0 || first + count > n->train_n) return gwm_fail(n, GW_ERR_ARG, "gwm_train_read: range");
  GWM_CUDA(n, cudaSetDevice(n->device));
  GWM_CUDA(n, cudaStreamSynchronize(n->stream));
  const int din = n->dims[0], nb = n->dims[n->n_layers];
  if (x && count)
    GWM_CUDA(n, cudaMemcpy(x, n->train_x + (size_t)first * din, sizeof(float) * (size_t)count * din,
                           cudaMemcpyDeviceToHost));
  if (t && count)
    GWM_CUDA(n, cudaMemcpy(t, n->train_t + (size_t)first * nb, sizeof(float) * (size_t)count * nb,
                           cudaMemcpyDeviceToHost));
  return GW_OK;
}

// ---------------------------------------------------------------------------
// Surrogate random-walk Metropolis sub-chains on the device: stage 1 of the
// delayed-acceptance sampler.  Per chain c and sub-step s:
//   prop = phi + L n,  n ~ N(0, I) (counter-based hash of (seed, s, c, k));
//   f(prop) = surrogate statistical LLH + (prop - m)^T C^-1 (prop - m);
//   accept when log u < -(f(prop) - f(phi)) / 2, u from the same hash.
// The surrogate of a point depends on that point alone (row-independent GEMM
// tiles, fixed-order reductions), so f is a fixed function of the point.
// ---------------------------------------------------------------------------
namespace gwm {
namespace {

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ uint64_t hash4(uint64_t seed, uint64_t step, uint64_t chain, uint64_t k) {
  uint64_t h = mix64(seed + 0x9E3779B97F4A7C15ull);
  h = mix64(h ^ (step * 0xD1B54A32D192ED03ull));
  h = mix64(h ^ (chain * 0xABC98388FB8FAC03ull));
  return mix64(h ^ (k * 0x8CB92BA72F3D8DD7ull));
}

// uniform in (0, 1), 53 bits
__device__ __forceinline__ double u01(uint64_t h) { return ((double)(h >> 11) + 0.5) * (1.0 / 9007199254740992.0); }

// First step of a sub-step, block per chain: standard normals n[k]
// (Box-Muller on hash pairs, FP32), the proposal prop = phi + L n with the
// increment in FP32 (Lt = L transposed, so that thread p reads column p
// coalesced; the increment depends on n alone, so the proposal is
// symmetric), written in FP64, and its standardised inputs
// x = (prop - mean) / scale (FP32, as k_standardize) with the BF16 row of the
// first GEMM (as k_rows_to_bf16).
__global__ void k_propose_stage(const double* __restrict__ phi, int P, const float* __restrict__ Lt, uint64_t seed,
                                uint64_t step, double* __restrict__ prop, const float* __restrict__ mean,
                                const float* __restrict__ scale, float* __restrict__ x, bf16* __restrict__ h0) {
  // blockDim.x = G * P32: group g of the column's partial sums covers the
  // k-range [g*ks, (g+1)*ks); the groups are combined in a fixed order
  extern __shared__ float shp[];
  const int P32 = (P + 31) & ~31, G = blockDim.x / P32;
  float* nrm = shp;            // [P + 1]
  float* part = shp + P + 1;   // [G][P32]
  const int c = blockIdx.x;
  for (int k2 = threadIdx.x; 2 * k2 < P; k2 += blockDim.x) {
    const float u1 = (float)u01(hash4(seed, step, c, 2 * k2));
    const float u2 = (float)u01(hash4(seed, step, c, 2 * k2 + 1));
    const float r = sqrtf(-2.f * logf(u1));
    float sn, cs;
    sincospif(2.f * u2, &sn, &cs);
    nrm[2 * k2] = r * cs;
    if (2 * k2 + 1 < P) nrm[2 * k2 + 1] = r * sn;
  }
  __syncthreads();
  const int g = threadIdx.x / P32, p = threadIdx.x - g * P32;
  const int ks = (P + G - 1) / G;
  if (p < P) {
    const int k0 = g * ks, k1 = min(min(P, (g + 1) * ks), p + 1);
    float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
    int k = k0;
    for (; k + 4 <= k1; k += 4) {
      a0 = fmaf(Lt[(size_t)k * P + p], nrm[k], a0);
      a1 = fmaf(Lt[(size_t)(k + 1) * P + p], nrm[k + 1], a1);
      a2 = fmaf(Lt[(size_t)(k + 2) * P + p], nrm[k + 2], a2);
      a3 = fmaf(Lt[(size_t)(k + 3) * P + p], nrm[k + 3], a3);
    }
    for (; k < k1; ++k) a0 = fmaf(Lt[(size_t)k * P + p], nrm[k], a0);
    part[g * P32 + p] = (a0 + a1) + (a2 + a3);
  }
  __syncthreads();
  if (g == 0 && p < P) {
    float inc = 0.f;
    for (int q = 0; q < G; ++q) inc += part[q * P32 + p];
    const size_t o = (size_t)c * P + p;
    const double v = phi[o] + (double)inc;
    prop[o] = v;
    const float z = (float)((v - (double)mean[p]) / (double)scale[p]);
    x[o] = z;
    h0[o] = __float2bfloat16(z);
  }
}

// Last step of a sub-step, block per chain: the surrogate LLH of the proposal
// from the per-block partials (the order of k_llh_finish), its prior penalty
// d^T C^-1 d, d = prop - m (FP32, C^-1 read by columns, fixed-order
// reduction; skipped when m is null), and the Metropolis decision on
// f = llh + penalty: accept when log u < -(f - f_current) / 2 with u from the
// hash of (seed, step, chain); NaN proposals are rejected.  first != 0 takes
// the value unconditionally (the initial evaluation).
__global__ void k_finish_accept(const double* __restrict__ part, int nblk, const double* __restrict__ prop, int P,
                                const double* __restrict__ m, const float* __restrict__ icov, uint64_t seed,
                                uint64_t step, int first, double* __restrict__ phi, double* __restrict__ f,
                                int32_t* __restrict__ n_acc) {
  // blockDim.x = G * P32 as k_propose_stage
  extern __shared__ float shf[];
  const int P32 = (P + 31) & ~31, G = blockDim.x / P32;
  float* d = shf;              // [P32]
  float* up = shf + P32;       // [G][P32]
  float* red = up + G * P32;   // [P32]
  __shared__ double s_llh;
  __shared__ int s_take;
  const int c = blockIdx.x, lane = threadIdx.x & 31;
  if (threadIdx.x < 32) {
    double t = 0.0;
    for (int b = lane; b < nblk; b += 32) t += part[(size_t)c * nblk + b];
    for (int off = 16; off; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
    if (lane == 0) s_llh = t;
  }
  const int g = threadIdx.x / P32, p = threadIdx.x - g * P32;
  if (m) {
    if (g == 0) d[p] = p < P ? (float)(prop[(size_t)c * P + p] - m[p]) : 0.f;
    __syncthreads();
    const int ks = (P + G - 1) / G;
    if (p < P) {
      const int k0 = g * ks, k1 = min(P, (g + 1) * ks);
      float u0 = 0.f, u1 = 0.f, u2 = 0.f, u3 = 0.f;
      int k = k0;
      for (; k + 4 <= k1; k += 4) {
        u0 = fmaf(icov[(size_t)k * P + p], d[k], u0);
        u1 = fmaf(icov[(size_t)(k + 1) * P + p], d[k + 1], u1);
        u2 = fmaf(icov[(size_t)(k + 2) * P + p], d[k + 2], u2);
        u3 = fmaf(icov[(size_t)(k + 3) * P + p], d[k + 3], u3);
      }
      for (; k < k1; ++k) u0 = fmaf(icov[(size_t)k * P + p], d[k], u0);
      up[g * P32 + p] = (u0 + u1) + (u2 + u3);
    }
    __syncthreads();
    if (g == 0) {
      float u = 0.f;
      for (int q = 0; q < G; ++q) u += (p < P) ? up[q * P32 + p] : 0.f;
      red[p] = d[p] * u;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double pen = 0.0;
    if (m)
      for (int i = 0; i < P32; ++i) pen += (double)red[i];
    const double fn = s_llh + pen;
    int take;
    if (first) {
      f[c] = fn;
      take = 0;
    } else {
      const double u = u01(hash4(seed, step, c, 0xFFFFFFFFull));
      take = log(u) < -(fn - f[c]) * 0.5;  // NaN proposals are rejected
      if (take) {
        f[c] = fn;
        n_acc[c] += 1;
      }
    }
    s_take = take;
  }
  __syncthreads();
  if (s_take)
    for (int q = threadIdx.x; q < P; q += blockDim.x) phi[(size_t)c * P + q] = prop[(size_t)c * P + q];
}

}  // namespace
}  // namespace gwm

// Chain state on the device (sized at gwm_set_chain).
struct gwm_chain_state {
  int P = 0;
  bool prior = false;
  float *Lt = nullptr, *icov = nullptr;
  double *m = nullptr, *phi = nullptr, *f = nullptr, *pen = nullptr;
  int32_t* nacc = nullptr;
};

static void chain_free(gwm_chain_state* s) {
  if (!s) return;
  cudaFree(s->Lt);
  cudaFree(s->m);
  cudaFree(s->icov);
  cudaFree(s->phi);
  cudaFree(s->f);
  cudaFree(s->pen);
  cudaFree(s->nacc);
  delete s;
}

// Evaluates the surrogate of the first C rows of h_theta (device) up to the
// per-block likelihood partials h_part.  Rows C..roundup(C, 8) of h_theta must
// be finite.
static int surrogate_llh_device(gwm_net* n, int C, int llh_type) {
  const int din = n->dims[0];
  const int Bp = ((C + 7) / 8) * 8;
  gwm::k_standardize<<<(unsigned)(((size_t)Bp * din + 255) / 256), 256, 0, n->stream>>>(n->h_theta, Bp, din,
                                                                                     n->h_mean, n->h_scale, n->xin);
  int rc = stage_input(n, n->xin, nullptr, Bp, false);
  if (!rc) rc = forward(n, Bp);
  if (rc) return rc;
  return head_llh(n, C, llh_type, false, false);
}

// Proposal Cholesky factor L [P x P] (lower, row-major, host FP64) and the
// Gaussian prior (mean [P], inverse covariance [P x P]; both null for none)
// of the sub-chains; P == dims[0].  Room for up to batch_max chains.
extern "C" int gwm_set_chain(gwm_net* n, const double* prop_chol, const double* prior_mean,
                             const double* prior_icov) {
  if (!n || !prop_chol || ((prior_mean == nullptr) != (prior_icov == nullptr)))
    return gwm_fail(n, GW_ERR_ARG, "gwm_set_chain: bad arguments");
  if (!n->has_head) return gwm_fail(n, GW_ERR_STATE, "gwm_set_chain: gwm_set_head first");
  if (n->dims[0] > 1024) return gwm_fail(n, GW_ERR_LIMIT, "gwm_set_chain: at most 1024 parameters");
  GWM_CUDA(n, cudaSetDevice(n->device));
  GWM_CUDA(n, cudaStreamSynchronize(n->stream));
  const int P = n->dims[0], Cm = n->batch_max;
  gwm_chain_state* s = n->chain;
  if (!s) {
    s = new gwm_chain_state();
    s->P = P;
    bool ok = cudaMalloc(&s->Lt, sizeof(float) * P * P) == cudaSuccess &&
              cudaMalloc(&s->m, sizeof(double) * P) == cudaSuccess &&
              cudaMalloc(&s->icov, sizeof(float) * P * P) == cudaSuccess &&
              cudaMalloc(&s->phi, sizeof(double) * (size_t)Cm * P) == cudaSuccess &&
              cudaMalloc(&s->f, sizeof(double) * Cm) == cudaSuccess &&
              cudaMalloc(&s->pen, sizeof(double) * Cm) == cudaSuccess &&
              cudaMalloc(&s->nacc, sizeof(int32_t) * Cm) == cudaSuccess;
    if (!ok) {
      cudaGetLastError();
      chain_free(s);
      return gwm_fail(n, GW_ERR_NOMEM, "gwm_set_chain: cudaMalloc failed");
    }
    n->chain = s;
  }
  std::vector<float> f32((size_t)P * P);
  for (int p = 0; p < P; ++p)
    for (int k = 0; k < P; ++k) f32[(size_t)k * P + p] = (float)prop_chol[(size_t)p * P + k];
  GWM_CUDA(n, cudaMemcpy(s->Lt, f32.data(), sizeof(float) * f32.size(), cudaMemcpyHostToDevice));
  s->prior = prior_mean != nullptr;
  if (s->prior) {
    // symmetric: C^-1 [k][p] read as column p; symmetrised in FP64 first
    for (int p = 0; p < P; ++p)
      for (int k = 0; k < P; ++k)
        f32[(size_t)k * P + p] = (float)(0.5 * (prior_icov[(size_t)k * P + p] + prior_icov[(size_t)p * P + k]));
    GWM_CUDA(n, cudaMemcpy(s->m, prior_mean, sizeof(double) * P, cudaMemcpyHostToDevice));
    GWM_CUDA(n, cudaMemcpy(s->icov, f32.data(), sizeof(float) * f32.size(), cudaMemcpyHostToDevice));
  }
  return GW_OK;
}

// Runs n_sub surrogate Metropolis steps for C chains from theta0 [C x P]
// (host FP64) with surrogate values f0 [C] (stat LLH + prior penalty, host;
// null: computed first, on the device).  Writes the end points phi [C x P],
// their surrogate values fphi [C] and the accepted sub-steps n_acc [C].
// n_sub == 0 with f0 == null evaluates the surrogate at theta0.
extern "C" int gwm_substeps(gwm_net* n, const double* theta0, const double* f0, int32_t C, int32_t n_sub,
                            int32_t llh_type, uint64_t seed, double* phi, double* fphi, int32_t* n_acc) {
  if (!n || !theta0 || !phi || !fphi || C < 1 || C > n->batch_max || n_sub < 0)
    return gwm_fail(n, GW_ERR_ARG, "gwm_substeps: bad arguments");
  gwm_chain_state* s = n->chain;
  if (!s || !n->has_head) return gwm_fail(n, GW_ERR_STATE, "gwm_substeps: gwm_set_chain first");
  GWM_CUDA(n, cudaSetDevice(n->device));
  const int P = s->P;
  const int Bp = ((C + 7) / 8) * 8;
  // G thread groups of P32 threads per chain split the k-range of the
  // proposal and penalty mat-vecs
  const int P32 = (P + 31) & ~31;
  const int G = std::max(1, std::min(4, 1024 / P32));
  const unsigned thr = (unsigned)(G * P32);
  const bool prior = s->prior;
  const size_t sh_prop = sizeof(float) * ((size_t)P + 1 + (size_t)G * P32);
  GWM_CUDA(n, cudaMemcpyAsync(s->phi, theta0, sizeof(double) * (size_t)C * P, cudaMemcpyHostToDevice, n->stream));
  GWM_CUDA(n, cudaMemsetAsync(s->nacc, 0, sizeof(int32_t) * C, n->stream));
  // rows C..Bp of the staging buffer stay finite (zeros)
  if (Bp > C)
    GWM_CUDA(n, cudaMemsetAsync(n->h_theta + (size_t)C * P, 0, sizeof(double) * (size_t)(Bp - C) * P, n->stream));
  int rc = GW_OK;
  const int nbx = (n->dims[n->n_layers] + 31) / 32;
  const size_t sh_fin = sizeof(float) * ((size_t)P32 * (G + 2));
  if (f0) {
    GWM_CUDA(n, cudaMemcpyAsync(s->f, f0, sizeof(double) * C, cudaMemcpyHostToDevice, n->stream));
  } else {
    GWM_CUDA(n, cudaMemcpyAsync(n->h_theta, s->phi, sizeof(double) * (size_t)C * P, cudaMemcpyDeviceToDevice,
                                n->stream));
    rc = surrogate_llh_device(n, C, llh_type);
    if (rc) return rc;
    gwm::k_finish_accept<<<C, thr, sh_fin, n->stream>>>(n->h_part, nbx, s->phi, P, prior ? s->m : nullptr, s->icov,
                                                       seed, 0, 1, s->phi, s->f, s->nacc);
    GWM_CUDA(n, cudaGetLastError());
  }
  // rows C..Bp of the first GEMM's input stay zero through the sub-steps
  if (Bp > C) GWM_CUDA(n, cudaMemsetAsync(n->h[0] + (size_t)C * P, 0, sizeof(bf16) * (size_t)(Bp - C) * P, n->stream));
  for (int st = 0; st < n_sub && rc == GW_OK; ++st) {
    gwm::k_propose_stage<<<C, thr, sh_prop, n->stream>>>(s->phi, P, s->Lt, seed, (uint64_t)st + 1, n->h_theta,
                                                        n->h_mean, n->h_scale, n->xin, n->h[0]);
    GWM_CUDA(n, cudaGetLastError());
    rc = forward(n, Bp);
    if (!rc) rc = head_llh(n, C, llh_type, false, false);
    if (rc) break;
    gwm::k_finish_accept<<<C, thr, sh_fin, n->stream>>>(n->h_part, nbx, n->h_theta, P, prior ? s->m : nullptr,
                                                       s->icov, seed, (uint64_t)st + 1, 0, s->phi, s->f, s->nacc);
    GWM_CUDA(n, cudaGetLastError());
  }
  if (rc) return rc;
  GWM_CUDA(n, cudaMemcpyAsync(phi, s->phi, sizeof(double) * (size_t)C * P, cudaMemcpyDeviceToHost, n->stream));
  GWM_CUDA(n, cudaMemcpyAsync(fphi, s->f, sizeof(double) * C, cudaMemcpyDeviceToHost, n->stream));
  if (n_acc) GWM_CUDA(n, cudaMemcpyAsync(n_acc, s->nacc, sizeof(int32_t) * C, cudaMemcpyDeviceToHost, n->stream));
  return check_status(n);
}

// ---------------------------------------------------------------------------
// Gradient of the surrogate -2 log L (plus the chain's prior penalty, when
// gwm_set_chain gave one) with respect to the parameters.
// ---------------------------------------------------------------------------
// dX of the network for dY in dz[L-1]: the backward GEMMs without the weight
// gradients; the input gradient lands in g_dx (FP32).
static int backward_dx(gwm_net* n, int B) {
  const int L = n->n_layers;
  for (int l = L - 1; l >= 1; --l) {
    gwm::Epilogue e{};
    e.gate = n->z[l - 1];
    e.out_bf16 = n->dz[l - 1];
    int rc = gemm(n, n->dz[l], n->wt[l], B, n->dims[l], n->dims[l + 1], e);
    if (rc) return rc;
  }
  gwm::Epilogue e0{};
  e0.out_f32 = n->g_dx;
  return gemm(n, n->dz[0], n->wt[0], B, n->dims[0], n->dims[1], e0);
}

extern "C" int gwm_value_grad(gwm_net* n, const double* theta, int32_t C, int32_t llh_type, double* f, double* grad) {
  if (!n || !theta || !f || !grad || C < 1 || C > n->batch_max) return gwm_fail(n, GW_ERR_ARG, "gwm_value_grad: bad batch");
  if (!n->has_head) return gwm_fail(n, GW_ERR_STATE, "gwm_value_grad: gwm_set_head first");
  if (n->dims[0] > 1024) return gwm_fail(n, GW_ERR_LIMIT, "gwm_value_grad: at most 1024 parameters");
  GWM_CUDA(n, cudaSetDevice(n->device));
  const int din = n->dims[0], nb = n->dims[n->n_layers], L = n->n_layers, Bm = n->batch_max;
  const int Bp = ((C + 7) / 8) * 8;
  if (Bp > Bm) return gwm_fail(n, GW_ERR_ARG, "gwm_value_grad: batch above batch_max after padding");
  if (!n->g_G) {
    int rc = gwm_alloc(n, &n->g_G, (size_t)Bm * nb) | gwm_alloc(n, &n->g_S, (size_t)Bm * nb) |
             gwm_alloc(n, &n->g_gz, (size_t)Bm * din) | gwm_alloc(n, &n->g_dx, (size_t)Bm * din) |
             gwm_alloc(n, &n->g_f, Bm) | gwm_alloc(n, &n->g_grad, (size_t)Bm * din);
    if (rc) return rc;
  }
  if (Bp > C) GWM_CUDA(n, cudaMemsetAsync(n->h_theta, 0, sizeof(double) * (size_t)Bp * din, n->stream));
  GWM_CUDA(n, cudaMemcpyAsync(n->h_theta, theta, sizeof(double) * (size_t)C * din, cudaMemcpyHostToDevice, n->stream));
  gwm::k_standardize<<<(unsigned)(((size_t)Bp * din + 255) / 256), 256, 0, n->stream>>>(n->h_theta, Bp, din,
                                                                                     n->h_mean, n->h_scale, n->xin);
  int rc = stage_input(n, n->xin, nullptr, Bp, false);
  if (!rc) rc = forward(n, Bp);
  if (rc) return rc;
  // the head: likelihood partials, G, S and dY (rows C..Bp of dY stay zero)
  GWM_CUDA(n, cudaMemsetAsync(n->dz[L - 1], 0, sizeof(bf16) * (size_t)Bp * nb, n->stream));
  constexpr int kPPT = 2;
  const int nbx = (nb + 31) / 32;
  const size_t shm = (size_t)8 * kPPT * din * 12;
  if (shm > 48 * 1024) {
    static std::once_flag once;
    std::call_once(once, []() {
      cudaFuncSetAttribute(gwm::k_head_llh<kPPT, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    });
    if (shm > 200 * 1024) return gwm_fail(n, GW_ERR_LIMIT, "surrogate head: too many inputs");
  }
  gwm::k_head_llh<kPPT, true><<<dim3(nbx, (C + 8 * kPPT - 1) / (8 * kPPT)), dim3(32, 8), shm, n->stream>>>(
      head_view(n), n->xin, n->z[L - 1], C, n->h_data, llh_type, n->h_part, nullptr, nullptr, nullptr, n->g_G,
      n->g_S, n->dz[L - 1]);
  GWM_CUDA(n, cudaGetLastError());
  rc = backward_dx(n, Bp);
  if (rc) return rc;
  const size_t shb = sizeof(float) * 2 * (size_t)nb;
  if (shb > 48 * 1024) {
    if (shb > 200 * 1024) return gwm_fail(n, GW_ERR_LIMIT, "gwm_value_grad: too many bins");
    static std::once_flag once2;
    std::call_once(once2, []() {
      cudaFuncSetAttribute(gwm::k_base_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    });
  }
  gwm::k_base_grad<<<dim3(C, (din + 7) / 8), 256, shb, n->stream>>>(head_view(n), n->xin, n->g_G, n->g_S, n->g_gz);
  GWM_CUDA(n, cudaGetLastError());
  const int P32 = (din + 31) & ~31;
  const int Gn = std::max(1, std::min(4, 1024 / P32));
  const bool prior = n->chain && n->chain->prior;
  gwm::k_grad_finish<<<C, (unsigned)(Gn * P32), sizeof(float) * (size_t)P32 * (Gn + 2), n->stream>>>(
      n->h_part, nbx, n->h_theta, din, n->h_scale, n->g_gz, n->g_dx, prior ? n->chain->m : nullptr,
      prior ? n->chain->icov : nullptr, n->g_f, n->g_grad);
  GWM_CUDA(n, cudaGetLastError());
  GWM_CUDA(n, cudaMemcpyAsync(f, n->g_f, sizeof(double) * C, cudaMemcpyDeviceToHost, n->stream));
  GWM_CUDA(n, cudaMemcpyAsync(grad, n->g_grad, sizeof(double) * (size_t)C * din, cudaMemcpyDeviceToHost, n->stream));
  return check_status(n);
}
