// gw_device.cuh -- device helpers shared by the kernel translation units:
// bulk-copy (TMA) + mbarrier primitives with bounded waits, and the
// multi-point dial evaluation used by every reweighting kernel.
#pragma once
#include <cfloat>
#include <cmath>
#include <cstdint>

#include "gw_dials.cuh"
#include "gw_internal.h"

namespace gw {
namespace {

template <typename T> struct Vec2;
template <> struct Vec2<double> { using type = double2; };
template <> struct Vec2<float> { using type = float2; };
struct __align__(16) dfloat2 {
  dfloat x, y;
};
template <> struct Vec2<dfloat> { using type = dfloat2; };

// ---------------------------------------------------------------------------
// Bulk-copy (TMA) and mbarrier helpers.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
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

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Waits for the barrier phase; gives up (returns false) after limit_ns.
__device__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint64_t limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  for (;;) {
    if (mbar_try_wait(bar, parity)) return true;
    if (global_ns() - t0 > limit_ns) return false;
  }
}

constexpr uint64_t kWaitLimitNs = 2000000000ull;  // 2 s per tile copy

// Named barriers of warp-specialised kernels: `count` threads (a multiple of
// 32) complete a phase; arrive does not wait, sync does.
__device__ __forceinline__ void named_sync(int id, int count) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}
__device__ __forceinline__ void named_arrive(int id, int count) {
  asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(count) : "memory");
}

// Thread 0: start the bulk copy of a tile's payload into a stage buffer.
__device__ __forceinline__ void issue_tile(const DevView& v, int tile, unsigned char* buf, uint64_t* bar) {
  const TileDesc td = v.tiles[tile];
  const uint32_t bytes = (uint32_t)td.payload_16b * 16u;
  mbar_expect_tx(bar, bytes);
  if (bytes > 0) bulk_load(buf, v.payload + td.payload_off, bytes, bar);
}

// Thread 0: the same, plus the tile's headers into hbuf under the same
// barrier.  A tile's headers start at an even index (16-byte aligned) and the
// array is padded, so the copy is whole 16-byte units: ceil(ndials / 2) * 16
// bytes <= tile_hdr_bytes.
__device__ __forceinline__ void issue_tile_hdr(const DevView& v, int tile, unsigned char* buf, uint64_t* hbuf,
                                               uint64_t* bar) {
  const TileDesc td = v.tiles[tile];
  const uint32_t bytes = (uint32_t)td.payload_16b * 16u;
  const uint32_t hbytes = (((uint32_t)td.ndials + 1u) / 2u) * 16u;
  mbar_expect_tx(bar, bytes + hbytes);
  if (bytes > 0) bulk_load(buf, v.payload + td.payload_off, bytes, bar);
  if (hbytes > 0) bulk_load(hbuf, v.hdr + td.dial0, hbytes, bar);
}

// DialResponseSupervisor::process (DialResponseSupervisor.cpp:10-18): a
// response below lo becomes lo, above hi becomes hi, anything else (NaN
// included) passes.  In FP32 that is the NaN-propagating max then min, two
// instructions instead of two compare-and-select pairs (with lo <= hi, which
// the builder checks).
template <typename T>
__device__ __forceinline__ T clamp_response(T r, T lo, T hi) {
  if (r < lo) r = lo;
  else if (r > hi) r = hi;
  return r;
}
__device__ __forceinline__ float clamp_response(float r, float lo, float hi) {
  float t;
  asm("max.NaN.f32 %0, %1, %2;" : "=f"(t) : "f"(r), "f"(lo));
  asm("min.NaN.f32 %0, %1, %2;" : "=f"(t) : "f"(t), "f"(hi));
  return t;
}

// A lanes-kernel stage: the tile's payload (TB bytes), its headers in slot
// order (HB bytes), then its event words, work prefix and base weights, each
// copied from the 16-byte boundary at or below the tile's first event, so that
// every input of a tile arrives by bulk copy.  Event buffers hold up to 7
// leading words of the previous tile and room for the sentinel after the last.
constexpr int kLaneEvWords = kMaxTileEvents + 8;  // uint16 words per event buffer (528 bytes)
__host__ __device__ constexpr size_t lanes_ev_bytes(size_t tsz) {
  return 2 * (size_t)kLaneEvWords * 2 + (((size_t)kMaxTileEvents + 4) * tsz + 15) / 16 * 16;
}

// Thread 0: every bulk copy of a lanes-kernel tile under one mbarrier.  The
// event arrays carry 8 words (base weights: 4 values) of slack past their
// end, so the rounded copies stay inside them.
// The tile's descriptor goes to *std, where the CTA reads it after its next
// barrier, so no thread waits on a global load when the tile starts.  The
// calling thread writes a sentinel into the stage's event words after each
// copy lands; the proxy fence orders that write before the bulk copies that
// overwrite the stage next.
__device__ __forceinline__ void issue_tile_lanes(const DevView& v, int tile, unsigned char* stage, int TB, int HB,
                                                 uint32_t tsz, uint64_t* bar, TileDesc* std) {
  const TileDesc td = v.tiles[tile];
  *std = td;
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  const uint32_t pb = (uint32_t)td.payload_16b * 16u;
  const uint32_t hb = (((uint32_t)td.ndials + 1u) / 2u) * 16u;
  const uint32_t e0 = td.event0, ne = td.nevents;
  const uint32_t a16 = e0 & ~7u;
  const uint32_t eb = ((e0 - a16 + ne) * 2u + 15u) & ~15u;
  const uint32_t aw = e0 & ~(16u / tsz - 1u);
  const uint32_t wb = ((e0 - aw + ne) * tsz + 15u) & ~15u;
  mbar_expect_tx(bar, pb + hb + 2u * eb + wb);
  unsigned char* ev = stage + TB + HB;
  if (pb > 0) bulk_load(stage, v.payload + td.payload_off, pb, bar);
  if (hb > 0) bulk_load(stage + TB, v.hdr_ev + td.dial0, hb, bar);
  bulk_load(ev, v.evinfo + a16, eb, bar);
  bulk_load(ev + 2 * kLaneEvWords, v.evcost + a16, eb, bar);
  bulk_load(ev + 4 * kLaneEvWords, (const unsigned char*)v.w0 + (size_t)aw * tsz, wb, bar);
}

// ---------------------------------------------------------------------------
// One dial at KR parameter points (k0, k0 + kstep, ...): the header is
// decoded, the type dispatched and the response clamp loaded once; the KR
// evaluations are independent (instruction-level parallelism).
// ---------------------------------------------------------------------------
// Uniform-knot splines with stored slopes at KR points: in FP32 with an even
// KR, pairs of points go through the packed-FP32 evaluator.
// Uniform-knot splines in the coefficient form at KR points: pairs of points
// in packed FP32 when T is float and KR even.
template <typename T, int KR>
__device__ __forceinline__ void coef_values(const T* __restrict__ d, int n, const T (&x)[KR], bool trunc,
                                            T (&val)[KR]) {
  if constexpr (sizeof(T) == 4 && KR % 2 == 0) {
#pragma unroll
    for (int j = 0; j < KR; j += 2) eval_coef2(d, n, x[j], x[j + 1], trunc, val[j], val[j + 1]);
  } else {
#pragma unroll
    for (int j = 0; j < KR; ++j) val[j] = eval_coef<T>(d, n, x[j], trunc);
  }
}

template <typename T, bool catmull, int KR>
__device__ __forceinline__ void prepared_values(const T* __restrict__ d, int n, const T (&x)[KR], bool trunc,
                                                T (&val)[KR]) {
  if constexpr (sizeof(T) == 4 && KR % 2 == 0) {
#pragma unroll
    for (int j = 0; j < KR; j += 2) eval_prepared2<catmull>(d, n, x[j], x[j + 1], trunc, val[j], val[j + 1]);
  } else {
#pragma unroll
    for (int j = 0; j < KR; ++j) val[j] = eval_prepared<T, catmull>(d, n, x[j], trunc);
  }
}

// A grid-form dial's inputs at KR points (k0, k0 + kstep, ...): the grid's
// interval and fraction per point and its response clamp.  The lanes kernel
// loads them one dial ahead of the evaluation, so the (mostly L2) latency of
// the grid table overlaps the previous dial's arithmetic.
template <typename T, int KR>
struct GridAhead {
  GridPoint<T> g[KR];
  typename Vec2<T>::type c;
};

template <typename T, int KR>
__device__ __forceinline__ void grid_load(const DevView& v, uint64_t h, int k0, int kstep, GridAhead<T, KR>& a) {
  const int g = hdr_p0(h);
  const GridPoint<T>* gp = (const GridPoint<T>*)v.grid_pts + (size_t)g * v.kpad + k0;
#pragma unroll
  for (int j = 0; j < KR; ++j) a.g[j] = gp[j * kstep];
  a.c = ((const typename Vec2<T>::type*)v.grid_clamp)[g];
}

template <typename T, int KR>
__device__ __forceinline__ void grid_eval(const T* __restrict__ pl, uint64_t h, const GridAhead<T, KR>& a,
                                          T (&val)[KR]) {
  const T* d = pl + hdr_off(h);
#pragma unroll
  for (int j = 0; j < KR; ++j) val[j] = clamp_response(coef_cubic(d + a.g[j].jb, a.g[j].u), a.c.x, a.c.y);
}

// The KR values of one parameter at points k0, k0 + kstep, ...  With VX the
// points are contiguous (kstep == 1) and k0 * sizeof(T) is a multiple of
// KR * sizeof(T) (at most 16), so whole 8- or 16-byte vectors are loaded.
template <typename T, int KR, bool VX>
__device__ __forceinline__ void load_points(const T* __restrict__ p, int kstep, T (&x)[KR]) {
  if constexpr (VX && KR == 2 && sizeof(T) == 4) {
    const float2 f = *reinterpret_cast<const float2*>(p);  // k0 even: 8-byte aligned
    x[0] = f.x;
    x[1] = f.y;
  } else if constexpr (VX && (KR * sizeof(T)) % 16 == 0) {
    if constexpr (kIsDf<T>) {
      const float4* q = reinterpret_cast<const float4*>(p);
#pragma unroll
      for (int i = 0; i < KR / 2; ++i) {
        const float4 f = q[i];
        x[2 * i] = dfloat(f.x, f.y);
        x[2 * i + 1] = dfloat(f.z, f.w);
      }
    } else if constexpr (sizeof(T) == 4) {
      const float4* q = reinterpret_cast<const float4*>(p);
#pragma unroll
      for (int i = 0; i < KR / 4; ++i) {
        const float4 f = q[i];
        x[4 * i] = f.x;
        x[4 * i + 1] = f.y;
        x[4 * i + 2] = f.z;
        x[4 * i + 3] = f.w;
      }
    } else {
      const double2* q = reinterpret_cast<const double2*>(p);
#pragma unroll
      for (int i = 0; i < KR / 2; ++i) {
        const double2 f = q[i];
        x[2 * i] = f.x;
        x[2 * i + 1] = f.y;
      }
    }
  } else {
#pragma unroll
    for (int j = 0; j < KR; ++j) x[j] = p[j * kstep];
  }
}

template <typename T, int KR, bool VX = false>
__device__ __forceinline__ void dial_values(const DevView& v, uint64_t h, const T* __restrict__ pl, int k0,
                                            int kstep, T (&val)[KR]) {
  const int type = hdr_type(h);
  const int n = hdr_n(h);
  const T* d = pl + hdr_off(h);
  const int p0 = hdr_p0(h);
  T lo, hi;
  if (type == kGrid) {
    // the grid form: interval and fraction per point from k_params, the
    // response clamp per grid (already within [-1e20, 1e20])
    const GridPoint<T>* gp = (const GridPoint<T>*)v.grid_pts + (size_t)p0 * v.kpad + k0;
    const typename Vec2<T>::type c = ((const typename Vec2<T>::type*)v.grid_clamp)[p0];
    if constexpr (VX && sizeof(GridPoint<T>) == 8 && KR % 2 == 0) {
      // contiguous points, k0 even: two 8-byte entries per 16-byte load
      const float4* q = reinterpret_cast<const float4*>(gp);
#pragma unroll
      for (int j = 0; j < KR; j += 2) {
        const float4 f = q[j / 2];
        val[j] = clamp_response(coef_cubic(d + __float_as_int(f.y), (T)f.x), c.x, c.y);
        val[j + 1] = clamp_response(coef_cubic(d + __float_as_int(f.w), (T)f.z), c.x, c.y);
      }
    } else {
#pragma unroll
      for (int j = 0; j < KR; ++j) {
        const GridPoint<T> g = gp[j * kstep];
        val[j] = clamp_response(coef_cubic(d + g.jb, g.u), c.x, c.y);
      }
    }
    return;
  }
  if (type >= kTabulated) {
    // Tabulated.h:27-28 and Kriged.cpp:14-21; clamp of the table's dials.
    const TableDesc td = v.tables[p0];
    lo = (T)td.lower;
    hi = (T)td.upper;
    // per-point tables are laid out [entry][kpad]
    const int64_t st = td.per_k ? v.kpad : 1;
    const T* tab = (const T*)v.table_arena + td.offset;
#pragma unroll
    for (int j = 0; j < KR; ++j) {
      const int64_t kk = td.per_k ? (int64_t)(k0 + j * kstep) : 0;
      if (type == kTabulated) {
        const T f = d[0];
        const int idx = (int)d[1];
        val[j] = f * tab[idx * st + kk] + (T(1) - f) * tab[(idx + 1) * st + kk];
      } else {
        T a = T(0);
        for (int q = 0; q < n; ++q) a += d[n + q] * tab[(int64_t)(int)d[q] * st + kk];
        val[j] = a;
      }
    }
  } else {
    const T* xs = (const T*)v.x + (size_t)p0 * v.kpad + k0;
    const typename Vec2<T>::type c = ((const typename Vec2<T>::type*)v.pclamp)[p0];
    lo = c.x;
    hi = c.y;
    const bool trunc = (v.pflags[p0] & 1) != 0;
    T x[KR];
    load_points<T, KR, VX>(xs, kstep, x);
    if (type == kNorm) {
#pragma unroll
      for (int j = 0; j < KR; ++j) val[j] = x[j];
    } else {
      // Spline, graph and surface responses: Calculate*.h clamps to
      // [-1e20, 1e20] before the response clamp; with lower <= upper the two
      // clamps are one clamp to the intersection.
      if constexpr (sizeof(T) == 4) {  // lo, hi are never NaN
        lo = fmaxf(lo, -1e20f);
        hi = fminf(hi, 1e20f);
      } else {
        if (lo < T(-1e20)) lo = T(-1e20);
        if (hi > T(1e20)) hi = T(1e20);
      }
      // the stored spline form is checked inside each spline type's branch,
      // so the other types pay nothing for it
      if (type == kMonotonic) {
        if (v.spline_coefs) {
          coef_values<T, KR>(d, n, x, trunc, val);
        } else if (v.spline_knots) {
#pragma unroll
          for (int j = 0; j < KR; ++j) val[j] = eval_knots<T, true>(d, n, x[j], trunc);
        } else {
          prepared_values<T, true, KR>(d, n, x, trunc, val);
        }
      } else if (type == kUniform) {
        if (v.spline_coefs)
          coef_values<T, KR>(d, n, x, trunc, val);
        else
          prepared_values<T, false, KR>(d, n, x, trunc, val);
      } else if (type == kGeneral) {
#pragma unroll
        for (int j = 0; j < KR; ++j) val[j] = eval_general<T>(d, n, x[j], trunc);
      } else if (type == kGraph) {
#pragma unroll
        for (int j = 0; j < KR; ++j) val[j] = eval_graph<T>(d, n, x[j], trunc);
      } else if (type == kBilinear) {
        T y[KR];
        load_points<T, KR, VX>((const T*)v.x + (size_t)hdr_p1(h) * v.kpad + k0, kstep, y);
#pragma unroll
        for (int j = 0; j < KR; ++j) val[j] = eval_bilinear<T>(d, x[j], y[j], trunc);
      } else if (type == kCompact) {
        if (v.spline_coefs) {
          coef_values<T, KR>(d, n, x, trunc, val);
        } else if (v.spline_knots) {
#pragma unroll
          for (int j = 0; j < KR; ++j) val[j] = eval_knots<T, false>(d, n, x[j], trunc);
        } else {
          prepared_values<T, true, KR>(d, n, x, trunc, val);
        }
      } else if (type == kBicubic) {
        T y[KR];
        load_points<T, KR, VX>((const T*)v.x + (size_t)hdr_p1(h) * v.kpad + k0, kstep, y);
#pragma unroll
        for (int j = 0; j < KR; ++j) val[j] = eval_bicubic<T>(d, x[j], y[j], trunc);
      } else {
#pragma unroll
        for (int j = 0; j < KR; ++j) val[j] = T(1);
        return;
      }
    }
  }
#pragma unroll
  for (int j = 0; j < KR; ++j) val[j] = clamp_response(val[j], lo, hi);
}

// Per-bin likelihoods.
__device__ __forceinline__ double llh_poisson(double data, double pred) {
  // PoissonLogLikelihood.h:19-53
  if (pred <= 0.0) return HUGE_VAL;
  if (data <= 0.0) return 2.0 * pred;
  return 2.0 * (pred - data + data * log(data / pred));
}

__device__ __forceinline__ double llh_bb_oa2021(double data, double pred, double mcuncert) {
  // BarlowBeestonBanff2022.h:150-294 with its defaults (expectedValueMinimum
  // = -1, fractionalErrorLimit = 1e150, usePoissonLikelihood = false).
  if (pred <= -1.0) {
    if (pred <= 0.0 && data > 0.0) return HUGE_VAL;
    return 0.0;
  }
  double newmc = pred;
  double penalty = 0.0;
  if (mcuncert > 0.0) {
    const double fractional = fmin(sqrt(mcuncert) / pred, 1.0e150);
    const double temp = pred * fractional * fractional - 1;
    const double temp2 = temp * temp + 4 * data * fractional * fractional;
    if (temp2 < 0) return HUGE_VAL;
    const double beta = (-1 * temp + sqrt(temp2)) / 2.;
    newmc = fmax(pred * beta, DBL_MIN);
    penalty = (beta - 1) * (beta - 1) / (2 * fractional * fractional);
  }
  double stat;
  if (data <= DBL_EPSILON) {
    stat = newmc;
  } else if (newmc > DBL_MIN) {
    stat = newmc - data + data * (log(data) - log(newmc));
  } else {
    const double mc = DBL_MIN;
    stat = mc - data + data * (log(data) - log(mc));
  }
  return 2.0 * stat + 2.0 * penalty;
}

// One Barlow-Beeston bin from the histogram's (sum of w, sqrt of sum of w^2),
// as BarlowBeestonBanff2022::eval(const SamplePair&, int) takes it
// (BarlowBeestonBanff2022.h:92-148): the stored sqrt squared again, and +inf
// for a non-finite value (the reference's throwIfInfLlh = false branch).
__device__ __forceinline__ double llh_bb_bin(double data, double pred, double sqrt_sum_w2) {
  double mcuncert = sqrt_sum_w2;
  mcuncert *= mcuncert;
  if (!isfinite(mcuncert) || mcuncert < 0.0) return HUGE_VAL;
  return llh_bb_oa2021(data, pred, mcuncert);
}

}  // namespace
}  // namespace gw
