// gw_multi.cu -- K > 1 reweighting kernel with threads over dials (each
// thread evaluates its dial for a chunk of points).
#include "gw_device.cuh"

namespace gw {
namespace {

// ---------------------------------------------------------------------------
// K > 1, dial-parallel: the plain kernel's mapping (threads over the tile's
// type-ordered dials, so a warp runs one dial type at a time) with each thread
// evaluating its dial for KR consecutive points, a chunk of KCH = KR*KS points
// per pass over the tile.  Per chunk: dial values -> dval[KCH][slot]; ordered
// per-event products -> wsh[KCH][event] (FP64); one warp per (bin, point)
// reduces the tile's events of that bin.  The payload stays in shared memory
// for all K points.
// ---------------------------------------------------------------------------
template <typename T, int KCH, int KR, int ST>
__global__ void __launch_bounds__(256) k_multi(const DevView v, int K) {
  constexpr int NT = 256, NW = NT / 32, KS = KCH / KR;
  extern __shared__ __align__(128) unsigned char smem[];
  const int TB = v.tile_payload_bytes;
  unsigned char* stage0 = smem;
  unsigned char* stage1 = smem + (ST == 2 ? TB : 0);
  uint64_t* shdr = (uint64_t*)(smem + ST * TB);        // [1024], tile order
  double* wsh = (double*)(shdr + 1024);                 // [KCH][256]
  T* dval = (T*)(wsh + kMaxTileEvents * KCH);           // [KCH][1024]
  T* sw0 = dval + 1024 * KCH;                           // [256]
  uint16_t* sev = (uint16_t*)(sw0 + kMaxTileEvents);   // [257]
  __shared__ uint64_t bar[2];
  __shared__ int s_bstart[kMaxLocalBins], s_bend[kMaxLocalBins];

  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();

  int tile = blockIdx.x;
  if (tid == 0 && tile < v.n_tiles) issue_tile(v, tile, stage0, &bar[0]);
  for (int it = 0; tile < v.n_tiles; ++it, tile += gridDim.x) {
    const int st = (ST == 2) ? (it & 1) : 0;
    const uint32_t parity = (ST == 2) ? (uint32_t)((it >> 1) & 1) : (uint32_t)(it & 1);
    const int next = tile + gridDim.x;
    if (ST == 2 && tid == 0 && next < v.n_tiles) issue_tile(v, next, st ? stage0 : stage1, &bar[st ^ 1]);

    const TileDesc td = v.tiles[tile];
    const int nd = td.ndials, ne = td.nevents;
    for (int i = tid; i < nd; i += NT) shdr[i] = v.hdr[td.dial0 + i];
    for (int e = tid; e < ne; e += NT) {
      sev[e] = v.evinfo[td.event0 + e];
      sw0[e] = ((const T*)v.w0)[td.event0 + e];
    }
    if (tid == 0) sev[ne] = make_evinfo(nd, 0);
    if (tid < kMaxLocalBins) {
      s_bstart[tid] = 0;
      s_bend[tid] = 0;
    }
    const bool ok = mbar_wait_bounded(&bar[st], parity, kWaitLimitNs);
    if (__syncthreads_or(!ok)) {
      if (tid == 0) {
        atomicOr(v.status, kStatusCopyTimeout);
        if (ST == 2 && next < v.n_tiles)
          mbar_wait_bounded(&bar[st ^ 1], (uint32_t)(((it + 1) >> 1) & 1), kWaitLimitNs);
      }
      return;
    }
    for (int e = tid; e < ne; e += NT) {
      const int lb = ev_lbin(sev[e]);
      if (e == 0 || ev_lbin(sev[e - 1]) != lb) s_bstart[lb] = e;
      if (e + 1 == ne || ev_lbin(sev[e + 1]) != lb) s_bend[lb] = e + 1;
    }
    const T* pl = (const T*)(st ? stage1 : stage0);

    for (int kb = 0; kb < K; kb += KCH) {
      // dial values for points kb .. kb+KCH-1
      for (int item = tid; item < nd * KS; item += NT) {
        const int i = item / KS, ks = item - i * KS;
        const uint64_t h = shdr[i];
        T val[KR];
        dial_values<T, KR>(v, h, pl, kb + ks * KR, 1, val);
        T* dst = dval + (ks * KR) * 1024 + hdr_slot(h);
#pragma unroll
        for (int j = 0; j < KR; ++j) dst[j * 1024] = val[j];
      }
      __syncthreads();
      // ordered per-event products (EventDialCache.cpp:156-171)
      for (int t = tid; t < ne * KCH; t += NT) {
        const int j = t / ne, e = t - j * ne;
        const int s0 = ev_slot(sev[e]), s1 = ev_slot(sev[e + 1]);
        const T* dv = dval + j * 1024;
        T w = T(1);
        for (int s = s0; s < s1; ++s) w *= dv[s];
        if (v.has_cap && w > (T)v.cap) w = (T)v.cap;
        w = sw0[e] * w;
        wsh[j * kMaxTileEvents + e] = (double)w;
      }
      __syncthreads();
      // one warp per (local bin, point): fixed-order FP64 sums of w and w^2
      for (int task = warp; task < (int)td.nbins * KCH; task += NW) {
        const int lb = task / KCH, j = task - lb * KCH;
        const int b0 = s_bstart[lb], b1 = s_bend[lb];
        if (b1 > b0 && kb + j < K) {
          double s = 0.0, s2 = 0.0;
          for (int e = b0 + lane; e < b1; e += 32) {
            const double w = wsh[j * kMaxTileEvents + e];
            s += w;
            s2 += w * w;
          }
          for (int o = 16; o; o >>= 1) {
            s += __shfl_xor_sync(0xffffffffu, s, o);
            s2 += __shfl_xor_sync(0xffffffffu, s2, o);
          }
          if (lane == 0) {
            const int slot = (lb == 0) ? (int)td.slot0 : v.bin_slot[td.bin0 + lb];
            v.partials[(size_t)slot * v.kpad + kb + j] = make_double2(s, s2);
          }
        }
      }
      __syncthreads();
    }
    if (ST == 1 && tid == 0 && next < v.n_tiles) issue_tile(v, next, stage0, &bar[0]);
  }
}

template <typename T, int KCH, int KR, int ST>
void launch_m(const DevView& v, int K, int grid, size_t smem, cudaStream_t s) {
  k_multi<T, KCH, KR, ST><<<grid, 256, smem, s>>>(v, K);
}

// FP64 and FP32 only: in double-float the small-K warp-specialised kernels
// (gw_ws.cu) take this family's range of K.
#define GW_MULTI(KCH, KR, ST)                                                                  \
  {1, KCH, KR, 256, ST, 0,                                                                     \
   {(const void*)k_multi<double, KCH, KR, ST>, (const void*)k_multi<float, KCH, KR, ST>, nullptr}, \
   {launch_m<double, KCH, KR, ST>, launch_m<float, KCH, KR, ST>, nullptr}}

const ShapeEntry kMultiShapes[] = {
    GW_MULTI(2, 2, 2), GW_MULTI(4, 2, 2), GW_MULTI(4, 4, 1), GW_MULTI(4, 4, 2),
    GW_MULTI(8, 4, 1), GW_MULTI(8, 4, 2), GW_MULTI(8, 8, 1), GW_MULTI(16, 8, 1),
};
#undef GW_MULTI

}  // namespace

int multi_shapes(const ShapeEntry** out) {
  *out = kMultiShapes;
  return (int)(sizeof(kMultiShapes) / sizeof(kMultiShapes[0]));
}

}  // namespace gw
