// gw_ws.cu -- small-K reweighting kernel: the warp-specialised K = 1 kernel
// (k_plain_ws, gw_kernels.cu) with each evaluator thread taking its dial at
// KP parameter points instead of one.
//
// Six evaluator warps walk a tile's type-ordered dials, one thread per dial,
// and write the dial's KP values into its event-major slot of a [slot][KP]
// buffer; two reducer warps form each event's ordered product
// (EventDialCache.cpp:156-171) for the KP points and reduce w and w^2 per
// (tile, bin, point) in FP64, one warp per (local bin, point), lanes over the
// bin's events in a fixed order.  Two value buffers alternate between the two
// sides (named barriers FULL_b / EMPTY_b), so the next chunk of points (or the
// next tile) is evaluated while the reducers empty the previous one.  A tile's
// payload and headers arrive by one bulk copy and stay in shared memory for
// all ceil(K / KP) chunks, so HBM sees each dial once per K points; at small
// K the kernel stays bound by HBM bandwidth, as the K = 1 kernel is, while
// the header decode, parameter and clamp loads of a dial are shared by its KP
// points and pairs of points go through the packed FP32 (f32x2) arithmetic.
//
// Every CTA runs the same number of hand-overs on both sides (each named
// barrier phase gets its full thread count), so the protocol cannot
// deadlock.  A bulk-copy wait that gives up marks the block failed: no
// further copy is issued, no header is decoded, and thread 0 waits (bounded)
// for the copies still in flight before the CTA exits.
#include "gw_device.cuh"

namespace gw {
namespace {

constexpr int kSEval = 192, kSRed = 64, kSThreads = kSEval + kSRed;
constexpr int kSBarEval = 1, kSBarFull = 2, kSBarEmpty = 4, kSBarRed = 6;

// The KP values of one slot: stores, loads and the elementwise product.
template <typename T, int KP>
__device__ __forceinline__ void slot_store(T* dst, const T (&v)[KP]) {
  if constexpr (kIsDf<T>) {
#pragma unroll
    for (int j = 0; j < KP; j += 2)
      *(float4*)(dst + j) = make_float4(v[j].hi, v[j].lo, v[j + 1].hi, v[j + 1].lo);
  } else if constexpr (sizeof(T) == 4 && KP == 2) {
    *(float2*)dst = make_float2(v[0], v[1]);
  } else if constexpr (sizeof(T) == 4 && KP % 4 == 0) {
#pragma unroll
    for (int j = 0; j < KP; j += 4) *(float4*)(dst + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
  } else {
#pragma unroll
    for (int j = 0; j < KP; j += 2) *(double2*)(dst + j) = make_double2(v[j], v[j + 1]);
  }
}

template <typename T, int KP>
__device__ __forceinline__ void slot_mul(T (&w)[KP], const T* src) {
  if constexpr (kIsDf<T>) {
#pragma unroll
    for (int j = 0; j < KP; j += 2) {
      const float4 a = *(const float4*)(src + j);
      w[j] *= dfloat(a.x, a.y);
      w[j + 1] *= dfloat(a.z, a.w);
    }
  } else if constexpr (sizeof(T) == 4) {
#pragma unroll
    for (int j = 0; j < KP; j += 2) {
      const float2 a = *(const float2*)(src + j);
      upk2(mul2(pk2(w[j], w[j + 1]), pk2(a.x, a.y)), w[j], w[j + 1]);
    }
  } else {
#pragma unroll
    for (int j = 0; j < KP; j += 2) {
      const double2 a = *(const double2*)(src + j);
      w[j] *= a.x;
      w[j + 1] *= a.y;
    }
  }
}

// Shared memory (all sizes multiples of 16 bytes):
//   [2][TB] payload stages | [2][HB] tile headers (tile order) |
//   [2][NS][KP] dial values (NS = HB / 8 slots) | [KP][256] FP64 event
//   weights | [256] base weights | [264] event words
template <typename T, int KP>
size_t ws_bytes(const DevView& v) {
  return 2 * (size_t)v.tile_payload_bytes + 2 * (size_t)v.tile_hdr_bytes +
         2 * (size_t)(v.tile_hdr_bytes / 8) * KP * sizeof(T) + (size_t)kMaxTileEvents * KP * sizeof(double) +
         kMaxTileEvents * sizeof(T) + (kMaxTileEvents + 8) * sizeof(uint16_t);
}

template <typename T, int KP, int MB>
__global__ void __launch_bounds__(kSThreads, MB) k_ws(const DevView v, int K) {
  static_assert(KP % 2 == 0 && (KP * sizeof(T)) % 8 == 0, "whole point pairs per slot");
  extern __shared__ __align__(128) unsigned char smem[];
  const int TB = v.tile_payload_bytes;
  const int HB = v.tile_hdr_bytes;
  const int NS = HB / 8;
  uint64_t* shdr = (uint64_t*)(smem + 2 * TB);                     // [2][NS]
  T* dval = (T*)(smem + 2 * TB + 2 * HB);                          // [2][NS][KP]
  double* wsh = (double*)(dval + 2 * (size_t)NS * KP);             // [KP][256]
  T* sw0 = (T*)(wsh + kMaxTileEvents * KP);                        // [256]
  uint16_t* sev = (uint16_t*)(sw0 + kMaxTileEvents);               // [264]
  __shared__ uint64_t bar[2];
  __shared__ int s_bstart[kMaxLocalBins], s_bend[kMaxLocalBins];
  __shared__ volatile int s_fail;

  const int tid = threadIdx.x;
  const int ntile = (int)blockIdx.x < v.n_tiles
                        ? (v.n_tiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x
                        : 0;
  const int nch = (K + KP - 1) / KP;
  const int Q = ntile * nch;
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
    s_fail = 0;
    if (ntile > 0) issue_tile_hdr(v, blockIdx.x, smem, shdr, &bar[0]);
    if (ntile > 1) issue_tile_hdr(v, blockIdx.x + gridDim.x, smem + TB, shdr + NS, &bar[1]);
  }
  __syncthreads();

  if (tid < kSEval) {
    // ---------------- evaluators ----------------
    int nd = 0, nd_next = 0;
    if (ntile > 0) nd = v.tiles[blockIdx.x].ndials;
    if (ntile > 1) nd_next = v.tiles[blockIdx.x + gridDim.x].ndials;
    int pend0 = ntile > 0 ? 0 : -1, pend1 = ntile > 1 ? 1 : -1;  // thread 0: copy in flight per stage
    for (int it = 0; it < ntile; ++it) {
      const int tile = blockIdx.x + it * gridDim.x;
      const int st = it & 1;
      const bool ok = mbar_wait_bounded(&bar[st], (uint32_t)((it >> 1) & 1), kWaitLimitNs);
      if (!ok) s_fail = 1;
      if (tid == 0 && ok) {
        if (st) pend1 = -1;
        else pend0 = -1;
      }
      const T* pl = (const T*)(smem + st * TB);
      const uint64_t* hs = shdr + st * NS;
      for (int c = 0; c < nch; ++c) {
        const int q = it * nch + c;
        const int b = q & 1;
        if (q >= 2) named_sync(kSBarEmpty + b, kSThreads);  // the reducers are done with buffer b
        if (ok && !s_fail) {
          T* dv = dval + (size_t)b * NS * KP;
          for (int i = tid; i < nd; i += kSEval) {
            const uint64_t h = hs[i];
            T val[KP];
            dial_values<T, KP, true>(v, h, pl, c * KP, 1, val);
            slot_store<T, KP>(dv + (size_t)hdr_slot(h) * KP, val);
          }
        }
        named_arrive(kSBarFull + b, kSThreads);
      }
      if (it + 1 < ntile) {
        nd = nd_next;
        if (it + 2 < ntile) nd_next = v.tiles[tile + 2 * gridDim.x].ndials;
      }
      named_sync(kSBarEval, kSEval);  // stage st fully read; s_fail visible
      if (tid == 0 && it + 2 < ntile && !s_fail) {
        issue_tile_hdr(v, tile + 2 * gridDim.x, smem + st * TB, shdr + st * NS, &bar[st]);
        if (st) pend1 = it + 2;
        else pend0 = it + 2;
      }
    }
    // the reducers' last two EMPTY arrivals
    for (int q = Q >= 2 ? Q - 2 : 0; q < Q; ++q) named_sync(kSBarEmpty + (q & 1), kSThreads);
    if (tid == 0 && s_fail) {
      if (pend0 >= 0) mbar_wait_bounded(&bar[0], (uint32_t)((pend0 >> 1) & 1), kWaitLimitNs);
      if (pend1 >= 0) mbar_wait_bounded(&bar[1], (uint32_t)((pend1 >> 1) & 1), kWaitLimitNs);
    }
  } else {
    // ---------------- reducers ----------------
    const int r = tid - kSEval;
    const int rwarp = r >> 5, lane = r & 31;
    // the next tile's descriptor, event words and base weights, loaded one
    // tile ahead (reducer thread r stores events r, r + 64, ...)
    constexpr int kEvPer = kMaxTileEvents / kSRed;
    TileDesc tdn;
    uint16_t pev[kEvPer];
    T pw0[kEvPer];
    auto prefetch = [&](int t) {
      tdn = v.tiles[t];
#pragma unroll
      for (int j = 0; j < kEvPer; ++j) {
        const int e = r + j * kSRed;
        if (e < (int)tdn.nevents) {
          pev[j] = v.evinfo[tdn.event0 + e];
          pw0[j] = ((const T*)v.w0)[tdn.event0 + e];
        }
      }
    };
    if (ntile > 0) prefetch(blockIdx.x);
    for (int it = 0; it < ntile; ++it) {
      const int tile = blockIdx.x + it * gridDim.x;
      const TileDesc td = tdn;
      const int ne = td.nevents;
#pragma unroll
      for (int j = 0; j < kEvPer; ++j) {
        const int e = r + j * kSRed;
        if (e < ne) {
          sev[e] = pev[j];
          sw0[e] = pw0[j];
        }
      }
      if (it + 1 < ntile) prefetch(tile + gridDim.x);
      if (r == 0) sev[ne] = make_evinfo(td.ndials, 0);
      if (r < kMaxLocalBins) {
        s_bstart[r] = 0;
        s_bend[r] = 0;
      }
      named_sync(kSBarRed, kSRed);
      // the event range of each local bin (events are bin-sorted)
      for (int e = r; e < ne; e += kSRed) {
        const int lb = ev_lbin(sev[e]);
        if (e == 0 || ev_lbin(sev[e - 1]) != lb) s_bstart[lb] = e;
        if (e + 1 == ne || ev_lbin(sev[e + 1]) != lb) s_bend[lb] = e + 1;
      }
      for (int c = 0; c < nch; ++c) {
        const int q = it * nch + c;
        const int b = q & 1;
        named_sync(kSBarFull + b, kSThreads);  // buffer b holds this chunk's values
        const T* dv = dval + (size_t)b * NS * KP;
        for (int e = r; e < ne; e += kSRed) {
          const int s0 = ev_slot(sev[e]), s1 = ev_slot(sev[e + 1]);
          T w[KP];
#pragma unroll
          for (int j = 0; j < KP; ++j) w[j] = T(1);
          for (int sl = s0; sl < s1; ++sl) slot_mul<T, KP>(w, dv + (size_t)sl * KP);
          const T w0 = sw0[e];
#pragma unroll
          for (int j = 0; j < KP; ++j) {
            T wj = w[j];
            if (v.has_cap && wj > (T)v.cap) wj = (T)v.cap;
            wsh[j * kMaxTileEvents + e] = (double)(w0 * wj);
          }
        }
        named_arrive(kSBarEmpty + b, kSThreads);  // buffer b consumed
        named_sync(kSBarRed, kSRed);              // wsh and the bin markers complete
        // one warp per (local bin, point): fixed-order FP64 sums of w and w^2
        for (int task = rwarp; task < (int)td.nbins * KP; task += kSRed / 32) {
          const int lb = task / KP, j = task - lb * KP;
          const int kg = c * KP + j;
          const int b0 = s_bstart[lb], b1 = s_bend[lb];
          if (b1 > b0 && kg < K) {
            double sw = 0.0, sw2 = 0.0;
            for (int e = b0 + lane; e < b1; e += 32) {
              const double w = wsh[j * kMaxTileEvents + e];
              sw += w;
              sw2 += w * w;
            }
            for (int o = 16; o; o >>= 1) {
              sw += __shfl_xor_sync(0xffffffffu, sw, o);
              sw2 += __shfl_xor_sync(0xffffffffu, sw2, o);
            }
            if (lane == 0) {
              const int slot = (lb == 0) ? (int)td.slot0 : v.bin_slot[td.bin0 + lb];
              v.partials[(size_t)slot * v.kpad + kg] = make_double2(sw, sw2);
            }
          }
        }
        named_sync(kSBarRed, kSRed);  // wsh (and, after the last chunk, sev and the markers) are reused
      }
    }
  }
  __syncthreads();
  if (tid == 0 && s_fail) atomicOr(v.status, kStatusCopyTimeout);
}

template <typename T, int KP, int MB>
void launch_s(const DevView& v, int K, int grid, size_t smem, cudaStream_t s) {
  k_ws<T, KP, MB><<<grid, kSThreads, smem, s>>>(v, K);
}

// kind 3: points per pass KP (= points per evaluator thread), 256 threads, 2 stages
// GW_WS: FP64, FP32 and double-float; GW_WS2: FP64 and FP32 only.
#define GW_WS(KP, MB)                                                                                 \
  {3, KP, KP, kSThreads, 2, MB,                                                                       \
   {(const void*)k_ws<double, KP, MB>, (const void*)k_ws<float, KP, MB>, (const void*)k_ws<dfloat, KP, MB>}, \
   {launch_s<double, KP, MB>, launch_s<float, KP, MB>, launch_s<dfloat, KP, MB>}}
#define GW_WS2(KP, MB)                                                                                \
  {3, KP, KP, kSThreads, 2, MB, {(const void*)k_ws<double, KP, MB>, (const void*)k_ws<float, KP, MB>, nullptr}, \
   {launch_s<double, KP, MB>, launch_s<float, KP, MB>, nullptr}}

const ShapeEntry kWsShapes[] = {
    GW_WS2(2, 3), GW_WS(2, 2), GW_WS2(4, 3), GW_WS(4, 2), GW_WS2(8, 2),
};
#undef GW_WS
#undef GW_WS2

}  // namespace

int ws_shapes(const ShapeEntry** out) {
  *out = kWsShapes;
  return (int)(sizeof(kWsShapes) / sizeof(kWsShapes[0]));
}

size_t ws_smem_bytes(const DevView& v, int kc) {
  const bool f = v.precision == 1;  // FP32; FP64 and double-float values are 8 bytes
  switch (kc) {
    case 2: return f ? ws_bytes<float, 2>(v) : ws_bytes<double, 2>(v);
    case 4: return f ? ws_bytes<float, 4>(v) : ws_bytes<double, 4>(v);
    case 8: return f ? ws_bytes<float, 8>(v) : ws_bytes<double, 8>(v);
    default: return 0;
  }
}

}  // namespace gw
