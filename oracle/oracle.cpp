// oracle.cpp -- CPU oracle (test infrastructure; see oracle.h).
//
// Every function below names the reference code it restates.  Paths are
// relative to the GUNDAM source tree.  Compiled with -ffp-contract=off so
// that x86-64 and aarch64 hosts round every operation the same way.
#include "oracle.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>

namespace {

enum { NORM = 1, MONOTONIC, UNIFORM, GENERAL, COMPACT, GRAPH, BILINEAR, BICUBIC, TABULATED, KRIGED };

// --- src/Utils/include/CalculateMonotonicSpline.h:49-148 (limiter = true)
// --- src/Utils/include/CalculateCompactSpline.h:48-126   (limiter = false)
// data = [low, step, y_0..y_{dim-1}]
double catmull_rom(double x, double lowerBound, double upperBound, const double* data, int dim, bool limiter) {
  const double low = data[0];
  const double step = data[1];
  const double xx = (x - low) / step;
  const int ix = (xx < 0) ? (int)(xx - 1) : (int)xx;
  int d21_0 = ix - 1;
  if (d21_0 < 0) d21_0 = 0;
  if (d21_0 > dim - 2) d21_0 = dim - 2;
  const int d21_1 = d21_0 + 1;
  int d32_0 = ix;
  if (d32_0 < 0) d32_0 = 0;
  if (d32_0 > dim - 2) d32_0 = dim - 2;
  const int d32_1 = d32_0 + 1;
  int d43_0 = ix + 1;
  if (d43_0 < 0) d43_0 = 0;
  if (d43_0 > dim - 2) d43_0 = dim - 2;
  const int d43_1 = d43_0 + 1;
  const double p2 = data[2 + d32_0];
  const double p3 = data[2 + d32_1];
  const double fx = xx - d32_0;
  const double d21 = data[2 + d21_1] - data[2 + d21_0];
  const double d32 = p3 - p2;
  const double d43 = data[2 + d43_1] - data[2 + d43_0];
  double m2 = 0.5 * (d21 + d32);
  double m3 = 0.5 * (d32 + d43);
  if (limiter) {
    if (d32 * d21 <= 0.0) m2 = 0.0;
    if (d43 * d32 <= 0.0) m3 = 0.0;
    const double ad21 = std::fabs(d21), ad32 = std::fabs(d32), ad43 = std::fabs(d43);
    const double delta2 = 3.0 * std::min(ad21, ad32);
    const double delta3 = 3.0 * std::min(ad32, ad43);
    if (m2 > delta2) m2 = delta2;
    if (m2 < -delta2) m2 = -delta2;
    if (m3 > delta3) m3 = delta3;
    if (m3 < -delta3) m3 = -delta3;
  }
  double v = ((((2.0 * p2 - 2.0 * p3 + m3 + m2) * fx + 3.0 * p3 - 3.0 * p2 - m3 - 2.0 * m2) * fx + m2) * fx + p2);
  if (v < lowerBound) v = lowerBound;
  if (v > upperBound) v = upperBound;
  return v;
}

// --- src/Utils/include/CalculateUniformSpline.h:46-80; dim = data length
double uniform_spline(double x, double lowerBound, double upperBound, const double* data, int dim) {
  const double step = data[1];
  const double xx = (x - data[0]) / step;
  int ix = (int)xx;
  if (ix < 0) ix = 0;
  if (2 * ix + 7 > dim) ix = (dim - 2) / 2 - 2;
  const double fx = xx - ix;
  const double p1 = data[2 + 2 * ix];
  const double m1 = data[2 + 2 * ix + 1] * step;
  const double p2 = data[2 + 2 * ix + 2];
  const double m2 = data[2 + 2 * ix + 3] * step;
  double v = ((((2.0 * p1 - 2.0 * p2 + m2 + m1) * fx + 3.0 * p2 - 3.0 * p1 - m2 - 2.0 * m1) * fx + m1) * fx + p1);
  if (v < lowerBound) v = lowerBound;
  if (v > upperBound) v = upperBound;
  return v;
}

// --- src/Utils/include/CalculateGeneralSpline.h:51-197 (binary-if search :135-159)
double general_spline(double x, double lowerBound, double upperBound, const double* data, int dim) {
  const int knotCount = (dim - 2) / 3 - 1;
  int ix = 0;
  for (int off = 16; off > 0; off /= 2) {
    if ((ix + off < knotCount) && (x > data[2 + 3 * (ix + off) + 2])) ix += off;
  }
  const double x1 = data[2 + 3 * ix + 2];
  const double x2 = data[2 + 3 * (ix + 1) + 2];
  const double step = x2 - x1;
  const double fx = (x - x1) / step;
  const double p1 = data[2 + 3 * ix];
  const double m1 = data[2 + 3 * ix + 1] * step;
  const double p2 = data[2 + 3 * (ix + 1)];
  const double m2 = data[2 + 3 * (ix + 1) + 1] * step;
  double v = ((((2.0 * p1 - 2.0 * p2 + m2 + m1) * fx + 3.0 * p2 - 3.0 * p1 - m2 - 2.0 * m1) * fx + m1) * fx + p1);
  if (v < lowerBound) v = lowerBound;
  if (v > upperBound) v = upperBound;
  return v;
}

// --- src/Utils/include/CalculateGraph.h:43-88; dim = data length
double graph(double x, double lowerBound, double upperBound, const double* data, int dim) {
  if (dim < 4) return data[0];
  const int knotCount = dim / 2;
  int ix = 0;
  int top = 1;
  while (2 * top <= knotCount) top *= 2;  // largest power of two <= knotCount
  for (int off = top; off > 0; off /= 2) {
    if ((ix + off < knotCount) && (x > data[2 * (ix + off) + 1])) ix += off;
  }
  if (ix + 1 >= knotCount) ix--;
  const double p1 = data[2 * ix];
  const double x1 = data[2 * ix + 1];
  const double p2 = data[2 * (ix + 1)];
  const double x2 = data[2 * (ix + 1) + 1];
  const double step = x2 - x1;
  const double fx = (x - x1) / step;
  const double m = p2 - p1;
  double v = p1 + fx * m;
  if (v < lowerBound) v = lowerBound;
  if (v > upperBound) v = upperBound;
  return v;
}

// --- BilinearIndex, src/Utils/include/CalculateBilinearInterpolation.h:36-60
int surface_index(double v, const double* a, int na) {
  int i = 0;
  if (8 < na && !(v < a[8])) i = 8;
  if ((i + 4) < na && !(v < a[i + 4])) i += 4;
  if ((i + 2) < na && !(v < a[i + 2])) i += 2;
  if ((i + 1) < na && !(v < a[i + 1])) i += 1;
  return i;
}

// --- BilinearCINT, CalculateBilinearInterpolation.h:64-72
double bil_cint(double x, double x0, double p0, double x1, double p1) { return p0 + (p1 - p0) * (x - x0) / (x1 - x0); }

// --- CalculateBilinearInterpolation.h:103-152
double bilinear(double x, double y, double lowerBound, double upperBound, const double* knots, int nx, int ny,
                const double* xx, int nnx, const double* yy, int nny) {
  const int ix = surface_index(x, xx, nnx - 1);
  const int iy = surface_index(y, yy, nny - 1);
  double a0 = xx[ix], b0 = knots[ix * ny + iy], a1 = xx[ix + 1], b1 = knots[(ix + 1) * ny + iy];
  const double u0 = yy[iy];
  const double v0 = bil_cint(x, a0, b0, a1, b1);
  a0 = xx[ix];
  b0 = knots[ix * ny + iy + 1];
  a1 = xx[ix + 1];
  b1 = knots[(ix + 1) * ny + iy + 1];
  const double u1 = yy[iy + 1];
  const double v1 = bil_cint(x, a0, b0, a1, b1);
  double val = bil_cint(y, u0, v0, u1, v1);
  if (val < lowerBound) val = lowerBound;
  if (val > upperBound) val = upperBound;
  return val;
}

// --- BicubicCINT, src/Utils/include/CalculateBicubicSpline.h:62-110 (Horner branch)
double bic_cint(double x, double x0, double p0, double x1, double p1, double x2, double p2, double x3, double p3) {
  const double step = x2 - x1;
  const double fx = (x - x1) / step;
  double m1 = step * (p2 - p0) / (x2 - x0);
  double m2 = step * (p3 - p1) / (x3 - x1);
  if (fx < 0.0) m2 = m1;
  if (fx > 1.0) m1 = m2;
  return ((((-2.0 * p2 + 2.0 * p1 + m2 + m1) * fx + 3 * p2 - 3 * p1 - m2 - 2 * m1) * fx + m1) * fx + p1);
}

// --- CalculateBicubicSpline.h:145-331: rows iy-1..iy+2 along x, with knots
// beyond an edge extended linearly, then one cubic along y.
double bicubic(double x, double y, double lowerBound, double upperBound, const double* knots, int nx, int ny,
               const double* xx, int nnx, const double* yy, int nny) {
  const int ix = surface_index(x, xx, nnx - 1);
  const int iy = surface_index(y, yy, nny - 1);
  auto K = [&](int i, int j) { return knots[i * ny + j]; };
  // Knot (i, j) for j in [iy-1, iy+2]; rows below/above the grid are
  // extended as 2*K(i, edge) - K(i, edge -/+ 1).
  auto ky = [&](int i, int j) -> double {
    if (j < 0) return 2 * K(i, 0) - K(i, 1);
    if (j > nny - 1) return 2 * K(i, nny - 1) - K(i, nny - 2);
    return K(i, j);
  };
  double v[4], u[4];
  for (int r = 0; r < 4; ++r) {
    const int j = iy - 1 + r;
    const double a1 = xx[ix], a2 = xx[ix + 1];
    const double b1 = ky(ix, j), b2 = ky(ix + 1, j);
    double a0, b0, a3, b3;
    if (ix > 0) {
      a0 = xx[ix - 1];
      b0 = ky(ix - 1, j);
    } else {
      a0 = 2 * xx[ix] - xx[ix + 1];
      b0 = 2 * b1 - b2;
    }
    if (ix < nnx - 2) {
      a3 = xx[ix + 2];
      b3 = ky(ix + 2, j);
    } else {
      a3 = 2 * xx[ix + 1] - xx[ix];
      b3 = 2 * b2 - b1;
    }
    if (j < 0) u[r] = 2 * yy[iy] - yy[iy + 1];
    else if (j > nny - 1) u[r] = 2 * yy[iy + 1] - yy[iy];
    else u[r] = yy[j];
    v[r] = bic_cint(x, a0, b0, a1, b1, a2, b2, a3, b3);
  }
  double val = bic_cint(y, u[0], v[0], u[1], v[1], u[2], v[2], u[3], v[3]);
  if (val < lowerBound) val = lowerBound;
  if (val > upperBound) val = upperBound;
  return val;
}

// CPU dial classes: evalResponse with the allowDialExtrapolation handling.
double dial_response(int type, const double* d, int n, double x, double y, bool truncate) {
  switch (type) {
    case NORM:  // Norm.h:21
      return x;
    case MONOTONIC:  // MonotonicSpline.cpp:71-84
    case COMPACT: {  // CompactSpline.cpp (same wrapper)
      const int dim = n - 2;
      if (truncate) {
        const double lo = d[0], hi = d[0] + (dim - 1) * d[1];
        if (x <= lo) x = lo;
        else if (x >= hi) x = hi;
      }
      return catmull_rom(x, -1E20, 1E20, d, dim, type == MONOTONIC);
    }
    case UNIFORM: {  // UniformSpline.cpp:47-60
      if (truncate) {
        const int k = (n - 2) / 2;
        const double lo = d[0], hi = d[0] + (k - 1) * d[1];
        if (x <= lo) x = lo;
        else if (x >= hi) x = hi;
      }
      return uniform_spline(x, -1E20, 1E20, d, n);
    }
    case GENERAL: {  // GeneralSpline.cpp:33-42
      if (truncate) {
        const int k = (n - 2) / 3;
        const double lo = d[2 + 2], hi = d[2 + 3 * (k - 1) + 2];
        if (x <= lo) x = lo;
        else if (x >= hi) x = hi;
      }
      return general_spline(x, -1E20, 1E20, d, n);
    }
    case GRAPH: {  // Graph.cpp:41-54
      if (truncate) {
        if (x <= d[1]) return d[0];
        if (x >= d[n - 1]) return d[n - 2];
      }
      return graph(x, -1E20, 1E20, d, n);
    }
    case BILINEAR:  // Bilinear.cpp:40-64
    case BICUBIC: {  // Bicubic.cpp:25-46
      const int nx = (int)d[0], ny = (int)d[1];
      const double* xx = d + 2;
      const double* yy = xx + nx;
      const double* knots = yy + ny;
      if (truncate) {
        if (x < xx[0]) x = xx[0];
        if (x > xx[nx - 1]) x = xx[nx - 1];
        if (y < yy[0]) y = yy[0];
        if (y > yy[ny - 1]) y = yy[ny - 1];
      }
      if (type == BILINEAR) return bilinear(x, y, -1E20, 1E20, knots, nx, ny, xx, nx, yy, ny);
      return bicubic(x, y, -1E20, 1E20, knots, nx, ny, xx, nx, yy, ny);
    }
    default:
      return 1.0;
  }
}

// DialResponseSupervisor::process (DialResponseSupervisor.cpp:10-18); an
// unset bound is +-DBL_MAX here (NaN in the reference).
inline double supervise(double v, double lo, double hi) {
  if (v < lo) return lo;
  if (v > hi) return hi;
  return v;
}

// DialInputBuffer::update (DialInputBuffer.cpp:44-89): fmod mirroring.
inline double mirror(double x, double lo, double hi) {
  if (!(lo > -DBL_MAX && hi < DBL_MAX)) return x;
  const double range = hi - lo;
  double t = std::fabs(std::fmod(x - lo, 2 * range));
  if (t > range) {
    t -= 2 * range;
    t = -t;
  }
  return t + lo;
}

// PoissonLogLikelihood::eval (PoissonLogLikelihood.h:19-53)
double poisson(double dataVal, double predVal) {
  if (predVal <= 0) return std::numeric_limits<double>::infinity();
  if (dataVal <= 0) return 2.0 * predVal;
  return 2.0 * (predVal - dataVal + dataVal * std::log(dataVal / predVal));
}

// BarlowBeestonBanff2022::eval (BarlowBeestonBanff2022.h:150-294), defaults
// expectedValueMinimum = -1, fractionalErrorLimit = 1e150,
// usePoissonLikelihood = false; an infinite result is returned instead of
// thrown.
double bb_oa2021(double dataVal, double predVal, double mcuncert) {
  const double expectedValueMinimum = -1.0;
  const double fractionalErrorLimit = 1.0E+150;
  if (predVal <= expectedValueMinimum) {
    if (predVal <= 0.0 && dataVal > 0.0) return std::numeric_limits<double>::infinity();
    return 0.0;
  }
  double newmc = predVal;
  double penalty = 0.0;
  if (mcuncert > 0.0) {
    const double fractional = std::min(std::sqrt(mcuncert) / predVal, fractionalErrorLimit);
    const double temp = predVal * fractional * fractional - 1;
    const double temp2 = temp * temp + 4 * dataVal * fractional * fractional;
    if (temp2 < 0) return std::numeric_limits<double>::infinity();
    const double beta = (-1 * temp + std::sqrt(temp2)) / 2.;
    newmc = std::max(predVal * beta, std::numeric_limits<double>::min());
    penalty = (beta - 1) * (beta - 1) / (2 * fractional * fractional);
  }
  double stat = 0;
  if (dataVal <= std::numeric_limits<double>::epsilon()) {
    stat = newmc;
  } else if (newmc > std::numeric_limits<double>::min()) {
    stat = newmc - dataVal + dataVal * (std::log(dataVal) - std::log(newmc));
  } else {
    const double mc = std::numeric_limits<double>::min();
    stat = mc - dataVal + dataVal * (std::log(dataVal) - std::log(mc));
  }
  double chisq = 2.0 * stat;
  chisq += 2.0 * penalty;
  return chisq;
}

double llh_bin(int type, double data, double pred, double sqrt_sum2) {
  if (type == 1) return poisson(data, pred);
  if (type == 2) {
    double mcuncert = sqrt_sum2;  // BarlowBeestonBanff2022.h:126-127: sqrtSumSqWeights squared
    mcuncert *= mcuncert;
    // BarlowBeestonBanff2022.h:130-144: a non-finite or negative value is +inf
    // (throwIfInfLlh = false; the default configuration ends the process)
    if (!std::isfinite(mcuncert) || mcuncert < 0.0) return std::numeric_limits<double>::infinity();
    return bb_oa2021(data, pred, mcuncert);
  }
  return 0.0;
}

// "Oscillation-like" table function of the stress workload.
double osc_table(const double* q, double E) {
  const double s = std::sin(q[1] * 1.267 / E + q[2]);
  return 1.0 - q[0] * s * s * (1.0 + q[3] * (std::log(E) - q[4])) * q[5];
}

// GenericToolbox::ParallelWorker::getThreadBoundIndices: contiguous split.
inline void bounds(int t, int nt, int64_t n, int64_t* b, int64_t* e) {
  const int64_t per = n / nt, rem = n % nt;
  *b = t * per + std::min<int64_t>(t, rem);
  *e = *b + per + (t < rem ? 1 : 0);
}

template <typename F>
void run_threads(int nt, F f) {
  if (nt <= 1) {
    f(0);
    return;
  }
  std::vector<std::thread> th;
  th.reserve(nt);
  for (int t = 0; t < nt; ++t) th.emplace_back(f, t);
  for (auto& x : th) x.join();
}

}  // namespace

struct oracle {
  oracle_input in;
  std::vector<int64_t> bin_start;   // events of each bin, in event order
  std::vector<int32_t> bin_events;
  std::vector<double> weights;      // current point
  std::vector<double> x;            // mirrored parameter values
  std::vector<std::vector<double>> tables;
};

extern "C" int oracle_create(const oracle_input* in, oracle** out) {
  if (!in || !out) return 1;
  oracle* o = new oracle();
  o->in = *in;
  const int N = in->n_events, B = in->n_bins;
  o->bin_start.assign((size_t)B + 1, 0);
  for (int e = 0; e < N; ++e) {
    const int b = in->event_bin[e];
    if (b < 0 || b >= B) {
      delete o;
      return 2;
    }
    o->bin_start[(size_t)b + 1]++;
  }
  for (int b = 0; b < B; ++b) o->bin_start[(size_t)b + 1] += o->bin_start[(size_t)b];
  o->bin_events.resize((size_t)N);
  std::vector<int64_t> fill(o->bin_start.begin(), o->bin_start.end() - 1);
  for (int e = 0; e < N; ++e) o->bin_events[(size_t)fill[in->event_bin[e]]++] = e;
  o->weights.assign((size_t)N, 0.0);
  o->x.assign((size_t)in->n_params, 0.0);
  o->tables.resize((size_t)in->n_tables);
  *out = o;
  return 0;
}

extern "C" int oracle_destroy(oracle* o) {
  delete o;
  return 0;
}

extern "C" int oracle_eval(oracle* o, const double* params, int32_t K, int32_t threads, double* sums,
                           double* sums2, double* llh_stat, double* penalty, double* weights) {
  if (!o || !params || K < 1) return 1;
  const oracle_input& in = o->in;
  const int N = in.n_events, P = in.n_params, B = in.n_bins;
  const int nt = std::max(1, (int)threads);
  std::vector<double> s1((size_t)B), s2((size_t)B);
  for (int k = 0; k < K; ++k) {
    const double* par = params + (size_t)k * P;
    for (int p = 0; p < P; ++p) o->x[(size_t)p] = mirror(par[p], in.mirror_lo[p], in.mirror_hi[p]);
    // tables: host copies, or the device-side function restated
    for (int t = 0; t < in.n_tables; ++t) {
      const int64_t a = in.table_node_start[t], b = in.table_node_start[t + 1];
      std::vector<double>& tab = o->tables[(size_t)t];
      tab.assign(in.table_nodes + a, in.table_nodes + b);
      if (in.table_fn_par[6 * t] >= 0) {
        double q[6];
        for (int i = 0; i < 6; ++i) q[i] = o->x[(size_t)in.table_fn_par[6 * t + i]];
        for (double& v : tab) v = osc_table(q, v);
      }
    }
    // Propagator::reweightEvents: one contiguous event range per thread
    run_threads(nt, [&](int t) {
      int64_t eb, ee;
      bounds(t, nt, N, &eb, &ee);
      for (int64_t e = eb; e < ee; ++e) {
        double tempReweight = 1;
        for (int64_t i = in.event_dial_start[e]; i < in.event_dial_start[e + 1]; ++i) {
          const int type = in.dial_type[i];
          const double* d = in.dial_data + in.dial_data_start[i];
          const int n = (int)(in.dial_data_start[i + 1] - in.dial_data_start[i]);
          double r;
          if (type == TABULATED) {  // Tabulated.h:27-28 (float fraction)
            const std::vector<double>& tb = o->tables[(size_t)d[0]];
            const float f = (float)d[2];
            const int idx = (int)d[1];
            r = f * tb[(size_t)idx] + (1.0 - f) * tb[(size_t)idx + 1];
            r = supervise(r, in.table_clamp[2 * (int)d[0]], in.table_clamp[2 * (int)d[0] + 1]);
          } else if (type == KRIGED) {  // Kriged.cpp:14-21 (float weights)
            const std::vector<double>& tb = o->tables[(size_t)d[0]];
            const int m = (int)d[1];
            double v = 0.0;
            for (int j = 0; j < m; ++j) {
              const float w = (float)d[2 + m + j];
              v += w * tb[(size_t)d[2 + j]];
            }
            r = supervise(v, in.table_clamp[2 * (int)d[0]], in.table_clamp[2 * (int)d[0] + 1]);
          } else {
            const int p0 = in.dial_par0[i];
            const int p1 = in.dial_par1[i];
            const double xv = o->x[(size_t)p0];
            const double yv = p1 >= 0 ? o->x[(size_t)p1] : 0.0;
            r = dial_response(type, d, n, xv, yv, in.truncate[p0] != 0);
            r = supervise(r, in.clamp_lo[p0], in.clamp_hi[p0]);
          }
          tempReweight *= r;
        }
        // GlobalEventReweightCap::process (EventDialCache.h:26-35)
        if (in.max_weight > 0 && tempReweight > in.max_weight) tempReweight = in.max_weight;
        double current = in.event_w0[e];
        current *= tempReweight;
        o->weights[(size_t)e] = current;
      }
    });
    // Histogram::refillHistogram: one contiguous bin range per thread
    run_threads(nt, [&](int t) {
      int64_t bb, be;
      bounds(t, nt, B, &bb, &be);
      for (int64_t b = bb; b < be; ++b) {
        double sw = 0, sw2 = 0;
        for (int64_t i = o->bin_start[(size_t)b]; i < o->bin_start[(size_t)b + 1]; ++i) {
          const double w = o->weights[(size_t)o->bin_events[(size_t)i]];
          sw += w;
          sw2 += w * w;
        }
        s1[(size_t)b] = sw;
        s2[(size_t)b] = sw2;
      }
    });
    if (sums) std::memcpy(sums + (size_t)k * B, s1.data(), sizeof(double) * B);
    if (sums2) std::memcpy(sums2 + (size_t)k * B, s2.data(), sizeof(double) * B);
    if (llh_stat) {
      // LikelihoodInterface::evalStatLikelihood: sum of per-sample sums
      double total = 0.0;
      for (int s = 0; s < in.n_samples; ++s) {
        double out = 0.0;
        for (int b = in.sample_bin_start[s]; b < in.sample_bin_start[s + 1]; ++b)
          out += llh_bin(in.llh_type, in.data[b], s1[(size_t)b], std::sqrt(s2[(size_t)b]));
        total += out;
      }
      llh_stat[k] = total;
    }
    if (penalty) {
      double pen = 0.0;
      if (in.prior_mean && in.prior_icov) {
        std::vector<double> delta((size_t)P), u((size_t)P, 0.0);
        for (int p = 0; p < P; ++p) delta[(size_t)p] = par[p] - in.prior_mean[p];
        for (int i = 0; i < P; ++i) {
          double acc = 0.0;
          for (int j = 0; j < P; ++j) acc += in.prior_icov[(size_t)i * P + j] * delta[(size_t)j];
          u[(size_t)i] = acc;
        }
        for (int i = 0; i < P; ++i) pen += delta[(size_t)i] * u[(size_t)i];
      }
      penalty[k] = pen;
    }
    if (weights && k == 0) std::memcpy(weights, o->weights.data(), sizeof(double) * N);
  }
  return 0;
}

extern "C" double oracle_dial(int32_t type, const double* data, int32_t n_data, double x, double y,
                              int32_t truncate) {
  return dial_response(type, data, n_data, x, y, truncate != 0);
}

extern "C" double oracle_llh_bin(int32_t type, double data, double pred, double sqrt_sum_w2) {
  return llh_bin(type, data, pred, sqrt_sum_w2);
}
