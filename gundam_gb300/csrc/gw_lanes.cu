// gw_lanes.cu -- K > 1 reweighting kernel with lanes over parameter points
// (one warp evaluates one dial for up to 32*KR points at once).
#include "gw_device.cuh"

namespace gw {
namespace {

// ---------------------------------------------------------------------------
// K > 1: events in order, lanes = parameter points.  KC points share one
// warp pass (32/KC events per pass); the tile payload is read from HBM once
// for all K points.  ST = payload stages (2: the next tile's copy overlaps
// this tile's work; 1: less shared memory, more resident CTAs).  MB = CTAs
// per SM the register allocation targets (0: the compiler's choice).
//
// Bin partials: warp w's events are a contiguous, bin-sorted run, so the
// (warp, local bin) pairs it touches are w + lb for lb in [first, last] of
// its run, and these indices never collide between warps: NW + 3 entries
// instead of NW * 4.  The reduction adds a bin's entries in warp order, the
// same fixed order (and so the same FP64 result) for every launch.
// ---------------------------------------------------------------------------
template <typename T, int KC, int KR, int NT, int ST, int MB>
__global__ void __launch_bounds__(NT, MB) k_batched(const DevView v, int K) {
  constexpr int NW = NT / 32;
  constexpr int EPW = 32 / KC;
  constexpr int KP = KC * KR;  // points per pass
  constexpr int NE = NW + kMaxLocalBins - 1;
  extern __shared__ __align__(128) unsigned char smem[];
  const int TB = v.tile_payload_bytes;
  const int HB = v.tile_hdr_bytes;
  // ST stages of [payload | headers in slot order | event words | work
  // prefix | base weights], every part filled by bulk copy (issue_tile_lanes)
  const int SB = TB + HB + (int)lanes_ev_bytes(sizeof(T));
  double2* wpart = (double2*)(smem + ST * SB);               // [NE][KR][32]
  __shared__ uint64_t bar[2];
  __shared__ TileDesc s_td[2];
  __shared__ int s_present[kMaxLocalBins];
  __shared__ int s_run[NW][2];  // first, last local bin of each warp's run (first > last: none)

  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  int tile = blockIdx.x;
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
    if (tile < v.n_tiles) issue_tile_lanes(v, tile, smem, TB, HB, sizeof(T), &bar[0], &s_td[0]);
  }
  __syncthreads();

  for (int it = 0; tile < v.n_tiles; ++it, tile += gridDim.x) {
    const int st = (ST == 2) ? (it & 1) : 0;
    const uint32_t parity = (ST == 2) ? (uint32_t)((it >> 1) & 1) : (uint32_t)(it & 1);
    const int next = tile + gridDim.x;
    const TileDesc td = s_td[st];
    if (ST == 2 && tid == 0 && next < v.n_tiles)
      issue_tile_lanes(v, next, smem + (st ^ 1) * SB, TB, HB, sizeof(T), &bar[st ^ 1], &s_td[st ^ 1]);

    const int nd = td.ndials, ne = td.nevents;
    unsigned char* stage = smem + st * SB;
    const uint64_t* shdr = (const uint64_t*)(stage + TB);  // indexed by slot
    unsigned char* evb = stage + TB + HB;
    // sev[e]: event e's first slot and local bin, sev[ne] the sentinel;
    // secc[e]: estimated work through event e; sw0[e]: its base weight
    uint16_t* sev = (uint16_t*)evb + (td.event0 & 7u);
    const uint16_t* secc = (const uint16_t*)(evb + 2 * kLaneEvWords) + (td.event0 & 7u);
    const T* sw0 = (const T*)(evb + 4 * kLaneEvWords) + (td.event0 & (16u / sizeof(T) - 1u));
    if (tid < kMaxLocalBins) s_present[tid] = 0;
    const bool ok = mbar_wait_bounded(&bar[st], parity, kWaitLimitNs);
    if (tid == 0 && ok) sev[ne] = make_evinfo(nd, 0);
    if (__syncthreads_or(!ok)) {
      if (tid == 0) {
        atomicOr(v.status, kStatusCopyTimeout);
        // the copies still pending: the next stage's, or with one stage the
        // one that timed out; one more bounded wait each before exiting
        if (ST == 2 && next < v.n_tiles)
          mbar_wait_bounded(&bar[st ^ 1], (uint32_t)(((it + 1) >> 1) & 1), kWaitLimitNs);
        if (ST == 1) mbar_wait_bounded(&bar[0], parity, kWaitLimitNs);
      }
      return;
    }
    for (int e = tid; e < ne; e += NT) s_present[ev_lbin(sev[e])] = 1;
    const T* pl = (const T*)stage;

    // Each warp takes a contiguous run of events holding ~1/NW of the tile's
    // estimated work (dial_cost): the first event whose preceding work
    // reaches warp*total/NW (a fixed, deterministic split, so the FP64
    // summation order does not depend on scheduling).
    auto before = [&](int e) { return e == 0 ? 0 : (int)secc[e - 1]; };  // work before event e
    auto first_event_at = [&](int target) {
      int lo = 0, hi = ne;  // before(ne) is the total
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (before(mid) < target) lo = mid + 1;
        else hi = mid;
      }
      return lo;
    };
    const int total = before(ne);
    const int e_lo = (warp == 0) ? 0 : first_event_at((warp * total) / NW);
    const int e_hi = (warp == NW - 1) ? ne : first_event_at(((warp + 1) * total) / NW);
    const int b_first = (e_lo < e_hi) ? ev_lbin(sev[e_lo]) : 1;
    const int b_last = (e_lo < e_hi) ? ev_lbin(sev[e_hi - 1]) : 0;
    if (lane == 0) {
      s_run[warp][0] = b_first;
      s_run[warp][1] = b_last;
    }
    const int sub = lane / KC, kl = lane % KC;

    for (int kb = 0; kb < K; kb += KP) {
      const int k0 = kb + kl;  // this lane's points: k0 + j*KC
      for (int lb = b_first; lb <= b_last; ++lb)
#pragma unroll
        for (int j = 0; j < KR; ++j) wpart[((warp + lb) * KR + j) * 32 + lane] = make_double2(0.0, 0.0);
      // Running (sum w, sum w^2) of the current bin: with up to two points
      // per lane in the lane's own partial entries in shared memory (zeroed
      // above; fewer live registers: 2.62 against 2.72 ms at K = 64), with
      // more in registers, written out when the bin changes (9.03 against
      // 9.20 ms at K = 256).  The same FP64 additions in the same order.
      constexpr bool kSharedSums = KR <= 2;
      int cur = -1;
      double s[kSharedSums ? 1 : KR], s2[kSharedSums ? 1 : KR];
      if constexpr (!kSharedSums) {
#pragma unroll
        for (int j = 0; j < KR; ++j) s[j] = s2[j] = 0.0;
      }
      for (int base = e_lo; base < e_hi; base += EPW) {
        const int e = base + sub;
        if (e < e_hi) {
          const uint16_t ei = sev[e];
          const int s0 = ev_slot(ei), s1 = ev_slot(sev[e + 1]);
          T w[KR];
#pragma unroll
          for (int j = 0; j < KR; ++j) w[j] = T(1);
          if constexpr (KR >= 4) {
            // four or more points per lane: a grid-form dial's table entries
            // are loaded one dial ahead (K = 256 on 2M mixed events: 9.05
            // against 9.79 ms); with two points per lane the extra live
            // registers cost more than the hidden latency (+7 % at K = 64)
            uint64_t hn = 0;
            GridAhead<T, KR> an;
            if (s0 < s1) {
              hn = shdr[s0];
              if (hdr_type(hn) == kGrid) grid_load<T, KR>(v, hn, k0, KC, an);
            }
            for (int sl = s0; sl < s1; ++sl) {
              const uint64_t h = hn;
              const GridAhead<T, KR> a = an;
              if (sl + 1 < s1) {
                hn = shdr[sl + 1];
                if (hdr_type(hn) == kGrid) grid_load<T, KR>(v, hn, k0, KC, an);
              }
              T val[KR];
              if (hdr_type(h) == kGrid)
                grid_eval<T, KR>(pl, h, a, val);
              else
                dial_values<T, KR>(v, h, pl, k0, KC, val);
#pragma unroll
              for (int j = 0; j < KR; ++j) w[j] *= val[j];
            }
          } else {
            for (int sl = s0; sl < s1; ++sl) {
              T val[KR];
              dial_values<T, KR>(v, shdr[sl], pl, k0, KC, val);
#pragma unroll
              for (int j = 0; j < KR; ++j) w[j] *= val[j];
            }
          }
          const T w0 = sw0[e];
          const int lb = ev_lbin(ei);
          if constexpr (kSharedSums) {
            double2* part = wpart + (warp + lb) * KR * 32 + lane;
#pragma unroll
            for (int j = 0; j < KR; ++j) {
              T wj = w[j];
              if (v.has_cap && wj > (T)v.cap) wj = (T)v.cap;
              wj = w0 * wj;
              const double wd = (double)wj;
              double2 q = part[j * 32];
              q.x += wd;
              q.y += wd * wd;
              part[j * 32] = q;
            }
          } else {
            if (lb != cur) {
              if (cur >= 0) {
#pragma unroll
                for (int j = 0; j < KR; ++j)
                  wpart[((warp + cur) * KR + j) * 32 + lane] = make_double2(s[j], s2[j]);
              }
              cur = lb;
#pragma unroll
              for (int j = 0; j < KR; ++j) s[j] = s2[j] = 0.0;
            }
#pragma unroll
            for (int j = 0; j < KR; ++j) {
              T wj = w[j];
              if (v.has_cap && wj > (T)v.cap) wj = (T)v.cap;
              wj = w0 * wj;
              const double wd = (double)wj;
              s[j] += wd;
              s2[j] += wd * wd;
            }
          }
        }
      }
      if constexpr (!kSharedSums) {
        if (cur >= 0) {
#pragma unroll
          for (int j = 0; j < KR; ++j) wpart[((warp + cur) * KR + j) * 32 + lane] = make_double2(s[j], s2[j]);
        }
      }
      __syncthreads();
      // one stage: after the last pass nothing reads the payload any more, so
      // the next tile's copy overlaps this tile's reduction
      if (ST == 1 && kb + KP >= K && tid == 0 && next < v.n_tiles)
        issue_tile_lanes(v, next, smem, TB, HB, sizeof(T), &bar[0], &s_td[0]);
      for (int t = tid; t < kMaxLocalBins * KP; t += NT) {
        const int lb = t / KP, r = t % KP;
        const int j = r / KC, kk = r % KC;
        const int kg = kb + kk + j * KC;
        if (kg < K && lb < (int)td.nbins && s_present[lb]) {
          double a = 0.0, a2 = 0.0;
          for (int w = 0; w < NW; ++w) {
            if (lb < s_run[w][0] || lb > s_run[w][1]) continue;
#pragma unroll
            for (int sb = 0; sb < EPW; ++sb) {
              const double2 p = wpart[((w + lb) * KR + j) * 32 + sb * KC + kk];
              a += p.x;
              a2 += p.y;
            }
          }
          const int slot = (lb == 0) ? (int)td.slot0 : v.bin_slot[td.bin0 + lb];
          v.partials[(size_t)slot * v.kpad + kg] = make_double2(a, a2);
        }
      }
      __syncthreads();
    }
  }
}

template <typename T, int KC, int KR, int NT, int ST, int MB>
void launch_b(const DevView& v, int K, int grid, size_t smem, cudaStream_t s) {
  k_batched<T, KC, KR, NT, ST, MB><<<grid, NT, smem, s>>>(v, K);
}

// GW_SHAPE compiles the shape for FP64, FP32 and double-float; GW_SHAPE2 for
// FP64 and FP32 only (double-float needs more registers than the 3- and
// 4-CTA-per-SM targets give it, and each instantiation costs build time).
#define GW_SHAPE(KC, KR, NT, ST, MB)                                                                   \
  {0, KC, KR, NT, ST, MB,                                                                              \
   {(const void*)k_batched<double, KC, KR, NT, ST, MB>, (const void*)k_batched<float, KC, KR, NT, ST, MB>, \
    (const void*)k_batched<dfloat, KC, KR, NT, ST, MB>},                                               \
   {launch_b<double, KC, KR, NT, ST, MB>, launch_b<float, KC, KR, NT, ST, MB>,                         \
    launch_b<dfloat, KC, KR, NT, ST, MB>}}
#define GW_SHAPE2(KC, KR, NT, ST, MB)                                                                  \
  {0, KC, KR, NT, ST, MB,                                                                              \
   {(const void*)k_batched<double, KC, KR, NT, ST, MB>, (const void*)k_batched<float, KC, KR, NT, ST, MB>, \
    nullptr},                                                                                          \
   {launch_b<double, KC, KR, NT, ST, MB>, launch_b<float, KC, KR, NT, ST, MB>, nullptr}}

// (32, 2, 256, 1) with 3 and 4 CTAs per SM are the fastest at K = 64 on the
// 5M-event mixed workload (9.5 / 9.4 ms against 11.2 ms with the compiler's
// own register choice); the others cover small K and K >= 128.
const ShapeEntry kLaneShapes[] = {
    GW_SHAPE2(8, 1, 256, 2, 0), GW_SHAPE(16, 1, 256, 2, 0),  GW_SHAPE2(32, 1, 256, 2, 0),
    GW_SHAPE(32, 1, 256, 1, 0), GW_SHAPE2(32, 2, 256, 1, 3), GW_SHAPE2(32, 2, 256, 1, 4),
    GW_SHAPE2(32, 2, 256, 2, 3), GW_SHAPE2(32, 2, 128, 1, 6), GW_SHAPE2(32, 4, 128, 1, 0),
    GW_SHAPE(16, 2, 256, 1, 0),  GW_SHAPE2(32, 4, 256, 1, 2),
};
#undef GW_SHAPE2
#undef GW_SHAPE

}  // namespace

int lane_shapes(const ShapeEntry** out) {
  *out = kLaneShapes;
  return (int)(sizeof(kLaneShapes) / sizeof(kLaneShapes[0]));
}

}  // namespace gw
