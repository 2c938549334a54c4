// gw_dials.cuh -- per-dial response functions evaluated on the device.
//
// Each function restates the arithmetic of the reference's shared CPU/GPU
// headers in src/Utils/include/Calculate*.h, in the same operation order, for
// T = double (FP64 mode), T = float (FP32 mode) or T = dfloat (double-float
// mode: the same operations in double-float arithmetic on the FP32 pipe).  Data is read from the tile
// payload in shared memory.  The CPU dial wrappers call these with bounds
// (-1e20, 1e20) and apply the collection's response clamp afterwards
// (MonotonicSpline.cpp:71-84, DialResponseSupervisor.cpp:10-18); the engine
// applies both as one clamp after the call (gw_kernels.cu, dial_values).
#pragma once
#include <type_traits>

#include "gw_dfloat.h"
#include "gw_layout.h"

namespace gw {

// Division: IEEE in FP64 mode (parity with the reference), the fast
// reciprocal-multiply form in FP32 mode (within the FP32 tolerance).
__device__ __forceinline__ double fdiv(double a, double b) { return a / b; }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ dfloat fdiv(dfloat a, dfloat b) { return df_div(a, b); }

template <typename T>
constexpr bool kIsDf = std::is_same<T, dfloat>::value;

// Hermite cubic on [p1, p2] with end slopes m1, m2 (already scaled by the
// interval width), Horner form of CalculateUniformSpline.h:71-74.
template <typename T>
__device__ __forceinline__ T hermite(T p1, T m1, T p2, T m2, T fx) {
  return ((((T(2) * p1 - T(2) * p2 + m2 + m1) * fx + T(3) * p2 - T(3) * p1 - m2 - T(2) * m1) * fx +
           m1) * fx + p1);
}

// The same cubic in double-float arithmetic, written p1 + fx(m1 + fx(B + fx A))
// with A = m1 + m2 - 2 dc, B = 3 dc - 2 m1 - m2, dc = p2 - p1, the doublings
// exact: 9 double-float sums and products instead of the 19 of the form above.
__device__ __forceinline__ dfloat hermite(dfloat p1, dfloat m1, dfloat p2, dfloat m2, dfloat fx) {
  const dfloat dc = p2 - p1;
  const dfloat a = (m1 + m2) - df_scale(dc, 2.0f);
  const dfloat b = (df_mul_f(dc, 3.0f) - df_scale(m1, 2.0f)) - m2;
  return p1 + fx * (m1 + fx * (b + fx * a));
}

// Hermite spline on non-uniform knots: CalculateGeneralSpline.h:51-197, with
// its 5-step branch-free search (:135-159).  Here the payload drops the unused
// [low, step] prefix: d = [(y, dydx, x) x n].
template <typename T>
__device__ __forceinline__ T eval_general(const T* __restrict__ d, int n, T x, bool trunc) {
  if (trunc) {  // GeneralSpline.cpp:33-42
    const T lo = d[2];
    const T hi = d[3 * (n - 1) + 2];
    if (x <= lo) x = lo;
    else if (x >= hi) x = hi;
  }
  const int kc = n - 1;
  int ix = 0;
  // a step of offset >= kc never moves (ix is still 0 there), so it is
  // skipped: a branch on the dial's knot count, uniform across a warp in the
  // lanes-over-points kernels
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    if (off < kc && ix + off < kc && x > d[3 * (ix + off) + 2]) ix += off;
  }
  const T x1 = d[3 * ix + 2];
  const T x2 = d[3 * (ix + 1) + 2];
  const T step = x2 - x1;
  const T fx = fdiv(x - x1, step);
  const T p1 = d[3 * ix];
  const T m1 = d[3 * ix + 1] * step;
  const T p2 = d[3 * (ix + 1)];
  const T m2 = d[3 * (ix + 1) + 1] * step;
  return (hermite(p1, m1, p2, m2, fx));
}

// Piecewise-linear graph: CalculateGraph.h:43-88.  d = [(y, x) x n].
template <typename T>
__device__ __forceinline__ T eval_graph(const T* __restrict__ d, int n, T x, bool trunc) {
  if (n < 2) return d[0];
  if (trunc) {  // Graph.cpp:47-51 returns the end values directly
    if (x <= d[1]) return d[0];
    if (x >= d[2 * n - 1]) return d[2 * n - 2];
  }
  int ix = 0;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    if (off < n && ix + off < n && x > d[2 * (ix + off) + 1]) ix += off;
  }
  if (ix + 1 >= n) ix--;
  const T p1 = d[2 * ix];
  const T x1 = d[2 * ix + 1];
  const T p2 = d[2 * (ix + 1)];
  const T x2 = d[2 * (ix + 1) + 1];
  const T step = x2 - x1;
  const T fx = fdiv(x - x1, step);
  const T m = p2 - p1;
  return (p1 + fx * m);
}

// Catmull-Rom splines on uniform knots (CalculateMonotonicSpline.h:49-148 with
// the Fritsch-Carlson limiter, CalculateCompactSpline.h:48-126 without) and
// Hermite splines on uniform knots with stored slopes
// (CalculateUniformSpline.h:46-80).  The host stores each
// knot's value and its slope in index units (for Catmull-Rom splines the
// slope after the Fritsch-Carlson limiter, for uniform splines dydx*step) and
// 1/step instead of step: d = [low, 1/step, (y, s) x n].  Inside the knot
// range this is exactly the Hermite cubic the reference evaluates; beyond the
// ends the reference's clamped neighbour indices make the outer slope equal
// the end difference (CalculateMonotonicSpline.h:66-103), restored here.
//
// The interval is i = clamp(floor(xx), 0, n - 2) and fx = xx - i; the
// reference's index tests (ix < 0, ix > n - 2) are fx < 0 and fx >= 1.  In
// FP32 the floor is one addition rounded toward minus infinity: for
// |xx| < 2^22, xx + 1.5*2^23 lies where the float spacing is one, so the
// rounded sum is 1.5*2^23 + floor(xx) exactly; larger |xx| still lands on the
// correct side of the clamp.  The integer i is read from the mantissa of
// i + 2^23.  No float<->int conversion instructions are issued.
template <typename T>
__device__ __forceinline__ void knot_interval(T& xx, int n, bool trunc, T& fi, int& i) {
  if constexpr (sizeof(T) == 4) {
    const float nm2 = __int_as_float(0x4B000000 | (n - 2)) - 8388608.0f;  // (float)(n - 2)
    if (trunc) xx = fminf(fmaxf(xx, 0.0f), nm2 + 1.0f);
    const float f = __fadd_rd(xx, 12582912.0f) - 12582912.0f;
    fi = fminf(fmaxf(f, 0.0f), nm2);
    i = __float_as_int(fi + 8388608.0f) - 0x4B000000;
  } else {
    if (trunc) xx = (xx < T(0)) ? T(0) : ((xx > T(n - 1)) ? T(n - 1) : xx);
    i = min(max((int)xx, 0), n - 2);
    fi = (T)i;
  }
}

template <typename T, bool catmull>
__device__ __forceinline__ T eval_prepared(const T* __restrict__ d, int n, T x, bool trunc) {
  T xx = (x - d[0]) * d[1];
  T fi;
  int i;
  knot_interval(xx, n, trunc, fi, i);
  const T fx = xx - fi;
  const T* k = d + 2 + 2 * i;
  const T p1 = k[0];
  T m1 = k[1];
  const T p2 = k[2];
  T m2 = k[3];
  if (catmull) {
    if (fx < T(0)) m2 = p2 - p1;
    if (fx >= T(1)) m1 = p2 - p1;
  }
  return (hermite(p1, m1, p2, m2, fx));
}

__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ dfloat mul_rn(dfloat a, dfloat b) { return a * b; }

// Catmull-Rom knot slope from the differences on either side, with the
// Fritsch-Carlson limiter when `limit` (CalculateMonotonicSpline.h:66-127);
// the same operations as the host's precomputed slopes.  The halving is an
// explicitly rounded multiply, so the compiler cannot fuse it into the
// Hermite sums that follow: the slope is rounded exactly as the host's.
template <typename T, bool limit>
__device__ __forceinline__ T knot_slope(T dl, T dr) {
  T s = mul_rn(T(0.5), dl + dr);
  if (limit) {
    if (dr * dl <= T(0)) s = T(0);
    const T adl = (dl < T(0)) ? -dl : dl;
    const T adr = (dr < T(0)) ? -dr : dr;
    const T delta = T(3) * ((adl < adr) ? adl : adr);
    if (s > delta) s = delta;
    if (s < -delta) s = -delta;
  }
  return s;
}

// The same Catmull-Rom splines stored as knot values only, the reference's
// data d = [low, 1/step, y_0 .. y_{n-1}]: the two slopes of the interval are
// formed here from its neighbours (an end knot's slope is the end
// difference, which knot_slope returns for equal sides).
template <typename T, bool limit>
__device__ __forceinline__ T eval_knots(const T* __restrict__ d, int n, T x, bool trunc) {
  T xx = (x - d[0]) * d[1];
  T fi;
  int i;
  knot_interval(xx, n, trunc, fi, i);
  const T fx = xx - fi;
  const T* y = d + 2;
  const T p1 = y[i];
  const T p2 = y[i + 1];
  const T dc = p2 - p1;
  const T dl = (i > 0) ? p1 - y[i - 1] : dc;
  const T dr = (i + 2 < n) ? y[i + 2] - p2 : dc;
  T m1 = knot_slope<T, limit>(dl, dc);
  T m2 = knot_slope<T, limit>(dc, dr);
  if (fx < T(0)) m2 = dc;
  if (fx >= T(1)) m1 = dc;
  return (hermite(p1, m1, p2, m2, fx));
}

// ---------------------------------------------------------------------------
// Two FP32 evaluations in one instruction stream: sm_100+ packed FP32
// arithmetic (add / sub / mul / fma .f32x2) on pairs held in one 64-bit
// register.  Used where a thread evaluates one dial at two parameter points
// (the batched kernel with two points per lane).
// ---------------------------------------------------------------------------
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 pk2(float a, float b) {
  f32x2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ void upk2(f32x2 r, float& a, float& b) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
}
__device__ __forceinline__ f32x2 add2(f32x2 a, f32x2 b) {
  f32x2 r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f32x2 add2_rm(f32x2 a, f32x2 b) {
  f32x2 r;
  asm("add.rm.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f32x2 sub2(f32x2 a, f32x2 b) {
  f32x2 r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f32x2 mul2(f32x2 a, f32x2 b) {
  f32x2 r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f32x2 fma2(f32x2 a, f32x2 b, f32x2 c) {
  f32x2 r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
  return r;
}

// eval_prepared at two points (FP32): the same interval, fraction and
// end-slope rules; the Hermite cubic in the form p1 + fx(m1 + fx(B + fx A)),
// A = m1 + m2 - 2(p2 - p1), B = 3(p2 - p1) - 2 m1 - m2.
template <bool catmull>
__device__ __forceinline__ void eval_prepared2(const float* __restrict__ d, int n, float xa, float xb, bool trunc,
                                               float& va, float& vb) {
  f32x2 xx = mul2(sub2(pk2(xa, xb), pk2(d[0], d[0])), pk2(d[1], d[1]));
  const float nm2 = __int_as_float(0x4B000000 | (n - 2)) - 8388608.0f;  // (float)(n - 2)
  float xa2, xb2;
  if (trunc) {
    upk2(xx, xa2, xb2);
    xx = pk2(fminf(fmaxf(xa2, 0.0f), nm2 + 1.0f), fminf(fmaxf(xb2, 0.0f), nm2 + 1.0f));
  }
  const f32x2 magic = pk2(12582912.0f, 12582912.0f);
  float fa, fb;
  upk2(sub2(add2_rm(xx, magic), magic), fa, fb);
  fa = fminf(fmaxf(fa, 0.0f), nm2);
  fb = fminf(fmaxf(fb, 0.0f), nm2);
  const f32x2 fi = pk2(fa, fb);
  float ba, bb;
  upk2(add2(fi, pk2(8388608.0f, 8388608.0f)), ba, bb);
  const float* ka = d + 2 + 2 * (__float_as_int(ba) - 0x4B000000);
  const float* kb = d + 2 + 2 * (__float_as_int(bb) - 0x4B000000);
  const f32x2 fx = sub2(xx, fi);
  const f32x2 p1 = pk2(ka[0], kb[0]);
  const f32x2 p2 = pk2(ka[2], kb[2]);
  const f32x2 dc = sub2(p2, p1);
  float m1a = ka[1], m2a = ka[3], m1b = kb[1], m2b = kb[3];
  if (catmull) {
    float fxa, fxb, dca, dcb;
    upk2(fx, fxa, fxb);
    upk2(dc, dca, dcb);
    if (fxa < 0.0f) m2a = dca;
    if (fxa >= 1.0f) m1a = dca;
    if (fxb < 0.0f) m2b = dcb;
    if (fxb >= 1.0f) m1b = dcb;
  }
  const f32x2 m1 = pk2(m1a, m1b), m2 = pk2(m2a, m2b);
  const f32x2 two = pk2(-2.0f, -2.0f);
  const f32x2 a = add2(fma2(two, dc, m2), m1);
  const f32x2 b = fma2(two, m1, sub2(mul2(pk2(3.0f, 3.0f), dc), m2));
  upk2(fma2(fma2(fma2(a, fx, b), fx, m1), fx, p1), va, vb);
}

// Uniform-knot splines in the coefficient form (GW_FLAG_SPLINE_COEFS):
// d = [-low/step, 1/step, 0, 0, (c0, c1, c2, c3) x (n + 1)].  xx = (x - low)
// / step as one multiply-add, j = clamp(floor(xx), -1, n - 1), u = xx - j,
// and the block j + 1 holds the cubic of u on that interval (the blocks of
// j = -1 and j = n - 1 hold the reference's extrapolation beyond the first and
// the last knot, re-expanded about their own origin), so no end rule is
// applied here.  With truncation xx is first clamped to [0, n - 1] (the end
// knots' values).  The coefficient blocks are 16-byte aligned.
// The interval of xx = (x - low) / step in the coefficient form: with
// truncation xx is first clamped to [0, n - 1]; j = clamp(floor(xx), -1,
// n - 1) and u = xx - j.  Returns j + 1, the index of the coefficient block.
template <typename T>
__device__ __forceinline__ int coef_interval(T& xx, int n, bool trunc, T& u) {
  if (trunc) xx = (xx < T(0)) ? T(0) : ((xx > T(n - 1)) ? T(n - 1) : xx);
  int j;
  T fj;
  if constexpr (sizeof(T) == 4) {
    const float f = __fadd_rd(xx, 12582912.0f) - 12582912.0f;  // floor, as knot_interval
    const float nm1 = __int_as_float(0x4B000000 | (n - 1)) - 8388608.0f;
    fj = fminf(fmaxf(f, -1.0f), nm1);
    j = __float_as_int(fj + 8388609.0f) - 0x4B000000;  // j + 1
  } else {
    const T xc = (xx < T(-1)) ? T(-1) : ((xx > T(n - 1)) ? T(n - 1) : xx);
    int i = (int)xc;     // truncation, in [-1, n - 1]
    if (T(i) > xc) --i;  // floor
    fj = T(i);
    j = i + 1;
  }
  u = xx - fj;
  return j;
}

// The cubic of one coefficient block at u.
template <typename T>
__device__ __forceinline__ T coef_cubic(const T* __restrict__ c, T u) {
  return c[0] + u * (c[1] + u * (c[2] + u * c[3]));
}
__device__ __forceinline__ float coef_cubic(const float* __restrict__ c, float u) {
  const float4 q = *(const float4*)c;  // blocks are 16-byte aligned
  return q.x + u * (q.y + u * (q.z + u * q.w));
}

// Uniform-knot splines in the coefficient form (GW_FLAG_SPLINE_COEFS):
// d = [-low/step, 1/step, 0, 0, (c0, c1, c2, c3) x (n + 1)].  xx = (x - low)
// / step as one multiply-add, j = clamp(floor(xx), -1, n - 1), u = xx - j,
// and the block j + 1 holds the cubic of u on that interval (the blocks of
// j = -1 and j = n - 1 hold the reference's extrapolation beyond the first and
// the last knot, re-expanded about their own origin), so no end rule is
// applied here.  With truncation xx is first clamped to [0, n - 1] (the end
// knots' values).  The coefficient blocks are 16-byte aligned.
template <typename T>
__device__ __forceinline__ T eval_coef(const T* __restrict__ d, int n, T x, bool trunc) {
  T xx = x * d[1] + d[0];
  T u;
  const int j = coef_interval(xx, n, trunc, u);
  return coef_cubic(d + 4 + 4 * j, u);
}

// The same at two points (FP32): one 16-byte load per point, the index and
// the cubic in packed FP32.
__device__ __forceinline__ void eval_coef2(const float* __restrict__ d, int n, float xa, float xb, bool trunc,
                                           float& va, float& vb) {
  f32x2 xx = fma2(pk2(xa, xb), pk2(d[1], d[1]), pk2(d[0], d[0]));
  const float nm1 = __int_as_float(0x4B000000 | (n - 1)) - 8388608.0f;  // (float)(n - 1)
  if (trunc) {
    float a, b;
    upk2(xx, a, b);
    xx = pk2(fminf(fmaxf(a, 0.0f), nm1), fminf(fmaxf(b, 0.0f), nm1));
  }
  const f32x2 magic = pk2(12582912.0f, 12582912.0f);
  float fa, fb;
  upk2(sub2(add2_rm(xx, magic), magic), fa, fb);
  fa = fminf(fmaxf(fa, -1.0f), nm1);
  fb = fminf(fmaxf(fb, -1.0f), nm1);
  const f32x2 fj = pk2(fa, fb);
  float ba, bb;
  upk2(add2(fj, pk2(8388609.0f, 8388609.0f)), ba, bb);
  const float4 ca = *(const float4*)(d + 4 + 4 * (__float_as_int(ba) - 0x4B000000));
  const float4 cb = *(const float4*)(d + 4 + 4 * (__float_as_int(bb) - 0x4B000000));
  const f32x2 u = sub2(xx, fj);
  const f32x2 v = fma2(fma2(fma2(pk2(ca.w, cb.w), u, pk2(ca.z, cb.z)), u, pk2(ca.y, cb.y)), u, pk2(ca.x, cb.x));
  upk2(v, va, vb);
}

// Index of the facet for a value: BilinearIndex / BicubicIndex
// (CalculateBilinearInterpolation.h:36-60), restricted to in-range reads.
template <typename T>
__device__ __forceinline__ int surface_index(T v, const T* __restrict__ a, int na) {
  int i = 0;
  if (8 < na && !(v < a[8])) i = 8;
  if ((i + 4) < na && !(v < a[i + 4])) i += 4;
  if ((i + 2) < na && !(v < a[i + 2])) i += 2;
  if ((i + 1) < na && !(v < a[i + 1])) i += 1;
  return i;
}

template <typename T>
__device__ __forceinline__ T lin(T x, T x0, T p0, T x1, T p1) {
  return p0 + fdiv((p1 - p0) * (x - x0), x1 - x0);
}

// Bilinear surface: CalculateBilinearInterpolation.h:103-152.
// d = [nx, ny, xx[nx], yy[ny], z[nx*ny]] (z index = ix*ny + iy).
template <typename T>
__device__ __forceinline__ T eval_bilinear(const T* __restrict__ d, T x, T y, bool trunc) {
  const int nx = (int)d[0];
  const int ny = (int)d[1];
  const T* xx = d + 2;
  const T* yy = xx + nx;
  const T* z = yy + ny;
  if (trunc) {  // Bilinear.cpp:40-64
    if (x < xx[0]) x = xx[0];
    if (x > xx[nx - 1]) x = xx[nx - 1];
    if (y < yy[0]) y = yy[0];
    if (y > yy[ny - 1]) y = yy[ny - 1];
  }
  const int ix = surface_index(x, xx, nx - 1);
  const int iy = surface_index(y, yy, ny - 1);
  const T v0 = lin(x, xx[ix], z[ix * ny + iy], xx[ix + 1], z[(ix + 1) * ny + iy]);
  const T v1 = lin(x, xx[ix], z[ix * ny + iy + 1], xx[ix + 1], z[(ix + 1) * ny + iy + 1]);
  return (lin(y, yy[iy], v0, yy[iy + 1], v1));
}

// One Catmull-Rom segment through (x0,p0)..(x3,p3) evaluated between x1 and
// x2: BicubicCINT (CalculateBicubicSpline.h:62-110, Horner branch).
template <typename T>
__device__ __forceinline__ T cubic_seg(T x, T x0, T p0, T x1, T p1, T x2, T p2, T x3, T p3) {
  const T step = x2 - x1;
  const T fx = fdiv(x - x1, step);
  T m1 = fdiv(step * (p2 - p0), x2 - x0);
  T m2 = fdiv(step * (p3 - p1), x3 - x1);
  if (fx < T(0)) m2 = m1;
  if (fx > T(1)) m1 = m2;
  return ((((-T(2) * p2 + T(2) * p1 + m2 + m1) * fx + T(3) * p2 - T(3) * p1 - m2 - T(2) * m1) * fx +
           m1) * fx + p1);
}

// Value of knot (i, j) of the surface, linearly extended by one knot beyond
// each edge as CalculateBicubicSpline.h:145-331 does.
template <typename T>
__device__ __forceinline__ T surf_knot(const T* __restrict__ z, int nx, int ny, int i, int j) {
  // extend along y first, then along x (same expressions as the reference)
  auto zy = [&](int ii, int jj) -> T {
    if (jj < 0) return T(2) * z[ii * ny + 0] - z[ii * ny + 1];
    if (jj > ny - 1) return T(2) * z[ii * ny + ny - 1] - z[ii * ny + ny - 2];
    return z[ii * ny + jj];
  };
  if (i < 0) return T(2) * zy(0, j) - zy(1, j);
  if (i > nx - 1) return T(2) * zy(nx - 1, j) - zy(nx - 2, j);
  return zy(i, j);
}

template <typename T>
__device__ __forceinline__ T axis_at(const T* __restrict__ a, int n, int i) {
  if (i < 0) return T(2) * a[0] - a[1];
  if (i > n - 1) return T(2) * a[n - 1] - a[n - 2];
  return a[i];
}

// Bicubic surface: four Catmull-Rom rows along x, then one along y
// (CalculateBicubicSpline.h:145-331).
template <typename T>
__device__ __forceinline__ T eval_bicubic(const T* __restrict__ d, T x, T y, bool trunc) {
  const int nx = (int)d[0];
  const int ny = (int)d[1];
  const T* xx = d + 2;
  const T* yy = xx + nx;
  const T* z = yy + ny;
  if (trunc) {
    if (x < xx[0]) x = xx[0];
    if (x > xx[nx - 1]) x = xx[nx - 1];
    if (y < yy[0]) y = yy[0];
    if (y > yy[ny - 1]) y = yy[ny - 1];
  }
  const int ix = surface_index(x, xx, nx - 1);
  const int iy = surface_index(y, yy, ny - 1);
  const T a0 = axis_at(xx, nx, ix - 1), a1 = xx[ix], a2 = xx[ix + 1], a3 = axis_at(xx, nx, ix + 2);
  T v[4];
  T u[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int j = iy - 1 + r;
    u[r] = axis_at(yy, ny, j);
    v[r] = cubic_seg(x, a0, surf_knot(z, nx, ny, ix - 1, j), a1, surf_knot(z, nx, ny, ix, j), a2,
                     surf_knot(z, nx, ny, ix + 1, j), a3, surf_knot(z, nx, ny, ix + 2, j));
  }
  return (cubic_seg(y, u[0], v[0], u[1], v[1], u[2], v[2], u[3], v[3]));
}

}  // namespace gw
