// gw_workload.cpp -- seeded synthetic workloads with the benchmark shapes.
//
// Dial data follow the reference's DialBase::getDialData() layouts:
//   monotonic  [low, step, y...]              (MonotonicSpline.cpp:12-69)
//   uniform    [low, step, (y, dydx)...]      (UniformSpline.cpp:14-45)
//   general    [low, step, (y, dydx, x)...]   (GeneralSpline.cpp:12-31)
//   graph      [(y, x)...]                    (Graph.cpp:32-39)
//   bilinear   [nx, ny, xx, yy, z]            (Bilinear.cpp:8-37)
// Knot slopes of uniform/general splines are Catmull-Rom slopes
// (DialUtils.cpp:95-125).  Each event draws its structure (kinematics,
// sample, dial types, parameters, knot counts) from one counter-seeded stream
// and its knot values from a second one, so two passes (count, then fill) see
// the same numbers and the output does not depend on the thread count.
#include "gw_workload.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>
#include <thread>
#include <vector>

#include "gw.h"

namespace {

thread_local std::string g_err;

inline uint64_t splitmix64(uint64_t& x) {
  uint64_t z = (x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// xoshiro256** seeded from (seed, stream, sub) through splitmix64.
struct Rng {
  uint64_t s[4];
  Rng(uint64_t seed, uint64_t stream, uint64_t sub) {
    uint64_t x = seed ^ (stream * 0xD1B54A32D192ED03ull) ^ (sub * 0x8CB92BA72F3D8DD7ull);
    for (auto& v : s) v = splitmix64(x);
  }
  static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  uint64_t next() {
    const uint64_t r = rotl(s[1] * 5, 7) * 9;
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return r;
  }
  double uniform() { return (double)(next() >> 11) * 0x1.0p-53; }
  double uniform_open() { return ((double)(next() >> 11) + 0.5) * 0x1.0p-53; }
  double normal() {
    const double u1 = uniform_open(), u2 = uniform();
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
  }
  int below(int n) { return std::min(n - 1, (int)(uniform() * n)); }
  int poisson_small(double lambda) {
    const double L = std::exp(-lambda);
    double p = 1.0;
    int k = 0;
    do {
      ++k;
      p *= uniform();
    } while (p > L);
    return k - 1;
  }
  using result_type = uint64_t;
  static constexpr uint64_t min() { return 0; }
  static constexpr uint64_t max() { return ~0ull; }
  uint64_t operator()() { return next(); }
};

struct Config {
  int id = 0;
  int n_events = 0;
  int n_params = 0;
  int n_spline = 0;        // parameters [0, n_spline) drive splines/graphs/surfaces
  int norm_first = 0, n_norm = 0;
  int table_par_first = -1;
  std::vector<std::pair<int, int>> grids;  // per sample (n_p, n_cos)
  double max_weight = 0.0;
};

Config make_config(int id) {
  Config c;
  c.id = id;
  switch (id) {
    case GWW_C1:
      c.n_events = 100000;
      c.n_params = 22;
      c.n_spline = 20;
      c.norm_first = 20;
      c.n_norm = 2;
      c.grids = {{20, 20}};
      break;
    case GWW_C2:
      c.n_events = 5000000;
      c.n_params = 200;
      c.n_spline = 190;
      c.norm_first = 190;
      c.n_norm = 10;
      c.grids.assign(8, {25, 15});
      break;
    case GWW_C5:
      c.n_events = 40000000;
      c.n_params = 400;
      c.n_spline = 394;
      c.table_par_first = 394;
      c.grids.assign(10, {40, 20});
      c.grids.push_back({40, 25});
      c.grids.push_back({40, 25});
      break;
    case GWW_MIXED_SMALL:
      c.n_events = 3000;
      c.n_params = 16;
      c.n_spline = 12;
      c.norm_first = 12;
      c.n_norm = 2;
      c.grids = {{6, 5}, {6, 5}};
      c.max_weight = 3.0;
      break;
    default:
      c.id = 0;
  }
  return c;
}

// (p, cos theta): p ~ LogNormal(ln 0.8 GeV, 0.6), cos = 1 - Exp(4) clipped to [-1, 1].
inline void kinematics(Rng& r, double* p, double* c) {
  *p = std::exp(std::log(0.8) + 0.6 * r.normal());
  double v = 1.0 + std::log(r.uniform_open()) / 4.0;
  *c = std::min(1.0, std::max(-1.0, v));
}

struct DialSpec {
  int type;
  int p0, p1;
  int n;      // knots / points / kriging weights
  double e;   // kriging energy
};

struct Quantiles {
  std::vector<double> p_edges, c_edges;
};

// Equal-probability edges from a fixed-seed pilot of 10^6 events.
Quantiles pilot_edges(int n_p, int n_c) {
  const int n = 1000000;
  std::vector<double> ps(n), cs(n);
  for (int i = 0; i < n; ++i) {
    Rng r(0x5EEDull, (uint64_t)i, 7);
    kinematics(r, &ps[i], &cs[i]);
  }
  std::sort(ps.begin(), ps.end());
  std::sort(cs.begin(), cs.end());
  Quantiles q;
  for (int i = 1; i < n_p; ++i) q.p_edges.push_back(ps[(size_t)((double)i / n_p * n)]);
  for (int i = 1; i < n_c; ++i) q.c_edges.push_back(cs[(size_t)((double)i / n_c * n)]);
  return q;
}

inline int edge_bin(const std::vector<double>& edges, double v) {
  return (int)(std::upper_bound(edges.begin(), edges.end(), v) - edges.begin());
}

constexpr int kKrigedNodes = 4096;
constexpr double kEmin = 0.1, kEmax = 10.0;

struct Gen {
  Config c;
  uint64_t seed;
  std::vector<Quantiles> q;          // per sample
  std::vector<int> sample_offset;
  std::vector<double> prior_mean;
  std::vector<double> host_tables[2];  // MIXED_SMALL tables
  std::vector<double> kriged_nodes;    // C5 node energies
  std::vector<double> kriged_nominal;  // C5 table at the prior mean

  // Structure of event e; returns the bin.
  int structure(int64_t e, std::vector<DialSpec>& dials) {
    Rng S(seed, (uint64_t)e, 0);
    double p, cth;
    kinematics(S, &p, &cth);
    const int ns = (int)c.grids.size();
    const int sample = ns > 1 ? S.below(ns) : 0;
    int ip = edge_bin(q[sample].p_edges, p);
    int ic = edge_bin(q[sample].c_edges, cth);
    if (c.id == GWW_MIXED_SMALL && sample == 1 && (ic % 2) == 1) ic -= 1;  // leaves empty bins
    const int bin = sample_offset[sample] + ip * c.grids[sample].second + ic;
    dials.clear();
    auto spline_par = [&]() { return S.below(c.n_spline); };
    switch (c.id) {
      case GWW_C1: {
        for (int i = 0; i < 3; ++i) dials.push_back({GW_DIAL_MONOTONIC, spline_par(), -1, 7, 0});
        dials.push_back({GW_DIAL_NORM, 20, -1, 0, 0});
        dials.push_back({GW_DIAL_NORM, 21, -1, 0, 0});
        break;
      }
      case GWW_C2: {
        const int nd = S.poisson_small(8.0);
        for (int i = 0; i < nd; ++i) {
          const double u = S.uniform();
          if (u < 0.50) dials.push_back({GW_DIAL_MONOTONIC, spline_par(), -1, 7, 0});
          else if (u < 0.70) dials.push_back({GW_DIAL_UNIFORM, spline_par(), -1, 11, 0});
          else if (u < 0.80) {
            const int p0 = spline_par();
            dials.push_back({GW_DIAL_GENERAL, p0, -1, 5 + S.below(11), 0});
          } else if (u < 0.90) {
            const int p0 = spline_par();
            dials.push_back({GW_DIAL_GRAPH, p0, -1, 3 + S.below(5), 0});
          } else if (u < 0.95) {
            const int p0 = spline_par();
            const int p1 = (p0 + 1 + S.below(c.n_spline - 1)) % c.n_spline;
            dials.push_back({GW_DIAL_BILINEAR, p0, p1, 0, 0});
          } else {
            dials.push_back({GW_DIAL_NORM, c.norm_first + S.below(c.n_norm), -1, 0, 0});
          }
        }
        break;
      }
      case GWW_C5: {
        const int nd = S.poisson_small(10.0);
        for (int i = 0; i < nd; ++i) {
          const double u = S.uniform() * 0.9;
          if (u < 0.50) dials.push_back({GW_DIAL_MONOTONIC, spline_par(), -1, 7, 0});
          else if (u < 0.70) dials.push_back({GW_DIAL_UNIFORM, spline_par(), -1, 11, 0});
          else if (u < 0.80) {
            const int p0 = spline_par();
            dials.push_back({GW_DIAL_GENERAL, p0, -1, 5 + S.below(11), 0});
          } else {
            const int p0 = spline_par();
            dials.push_back({GW_DIAL_GRAPH, p0, -1, 3 + S.below(5), 0});
          }
        }
        const double E = std::exp(std::log(kEmin) + S.uniform() * std::log(kEmax / kEmin));
        dials.push_back({GW_DIAL_KRIGED, -1, -1, 4, E});
        break;
      }
      case GWW_MIXED_SMALL: {
        const int nd = S.poisson_small(4.0);
        for (int i = 0; i < nd; ++i) {
          const int t = S.below(10);
          const int p0 = S.below(c.n_spline);
          switch (t) {
            case 0: dials.push_back({GW_DIAL_MONOTONIC, p0, -1, 3 + S.below(10), 0}); break;
            case 1: dials.push_back({GW_DIAL_UNIFORM, p0, -1, 2 + S.below(12), 0}); break;
            case 2: dials.push_back({GW_DIAL_GENERAL, p0, -1, 2 + S.below(14), 0}); break;
            case 3: dials.push_back({GW_DIAL_COMPACT, p0, -1, 3 + S.below(10), 0}); break;
            case 4: dials.push_back({GW_DIAL_GRAPH, p0, -1, 1 + S.below(15), 0}); break;
            case 5:
            case 6: {
              const int p1 = (p0 + 1 + S.below(c.n_spline - 1)) % c.n_spline;
              dials.push_back({t == 5 ? GW_DIAL_BILINEAR : GW_DIAL_BICUBIC, p0, p1, 0, 0});
              break;
            }
            case 7: dials.push_back({GW_DIAL_NORM, c.norm_first + S.below(c.n_norm), -1, 0, 0}); break;
            case 8: dials.push_back({GW_DIAL_TABULATED, -1, -1, 0, 0}); break;
            default: dials.push_back({GW_DIAL_KRIGED, -1, -1, 1 + S.below(6), 0}); break;
          }
        }
        break;
      }
      default:
        break;
    }
    return bin;
  }

  static int data_len(const DialSpec& d) {
    switch (d.type) {
      case GW_DIAL_NORM: return 0;
      case GW_DIAL_MONOTONIC:
      case GW_DIAL_COMPACT: return 2 + d.n;
      case GW_DIAL_UNIFORM: return 2 + 2 * d.n;
      case GW_DIAL_GENERAL: return 2 + 3 * d.n;
      case GW_DIAL_GRAPH: return 2 * d.n;
      case GW_DIAL_BILINEAR:
      case GW_DIAL_BICUBIC: return 2 + 5 + 5 + 25;
      case GW_DIAL_TABULATED: return 3;
      case GW_DIAL_KRIGED: return 2 + 2 * d.n;
      default: return 0;
    }
  }

  // Knot values y_k = s^{x_k} exp(N(0, 0.1|x_k|)), forced monotone.
  static void knot_values(Rng& V, const double* x, int n, double* y) {
    const double s = std::exp(std::log(0.8) + V.uniform() * std::log(1.25 / 0.8));
    for (int k = 0; k < n; ++k) y[k] = std::pow(s, x[k]) * std::exp(0.1 * std::fabs(x[k]) * V.normal());
    if (s >= 1.0) {
      for (int k = 1; k < n; ++k) y[k] = std::max(y[k], y[k - 1]);
    } else {
      for (int k = 1; k < n; ++k) y[k] = std::min(y[k], y[k - 1]);
    }
  }

  static void cr_slopes(const double* x, const double* y, int n, double* dy) {
    if (n == 1) {
      dy[0] = 0;
      return;
    }
    dy[0] = (y[1] - y[0]) / (x[1] - x[0]);
    dy[n - 1] = (y[n - 1] - y[n - 2]) / (x[n - 1] - x[n - 2]);
    for (int k = 1; k < n - 1; ++k) dy[k] = (y[k + 1] - y[k - 1]) / (x[k + 1] - x[k - 1]);
  }

  static double lin_at(const double* x, const double* y, int n, double x0) {
    if (n == 1) return y[0];
    int i = 0;
    while (i < n - 2 && x0 > x[i + 1]) ++i;
    return y[i] + (y[i + 1] - y[i]) * (x0 - x[i]) / (x[i + 1] - x[i]);
  }

  // Fills the data vector of one dial; returns an approximate nominal response.
  double fill(Rng& V, const DialSpec& d, double* out) {
    double x[32], y[32], dy[32];
    const int n = d.n;
    auto nominal_of = [&](int par) { return par >= 0 ? prior_mean[par] : 0.0; };
    switch (d.type) {
      case GW_DIAL_NORM:
        return nominal_of(d.p0);
      case GW_DIAL_MONOTONIC:
      case GW_DIAL_COMPACT: {
        const double step = 6.0 / (n - 1);
        for (int k = 0; k < n; ++k) x[k] = -3.0 + k * step;
        knot_values(V, x, n, y);
        out[0] = -3.0;
        out[1] = step;
        for (int k = 0; k < n; ++k) out[2 + k] = y[k];
        return lin_at(x, y, n, nominal_of(d.p0));
      }
      case GW_DIAL_UNIFORM: {
        const double step = 6.0 / (n - 1);
        for (int k = 0; k < n; ++k) x[k] = -3.0 + k * step;
        knot_values(V, x, n, y);
        cr_slopes(x, y, n, dy);
        out[0] = -3.0;
        out[1] = step;
        for (int k = 0; k < n; ++k) {
          out[2 + 2 * k] = y[k];
          out[3 + 2 * k] = dy[k];
        }
        return lin_at(x, y, n, nominal_of(d.p0));
      }
      case GW_DIAL_GENERAL:
      case GW_DIAL_GRAPH: {
        const double sp = 6.0 / std::max(1, n - 1);
        for (int k = 0; k < n; ++k) {
          x[k] = -3.0 + k * sp;
          if (k > 0 && k < n - 1) x[k] += (V.uniform() - 0.5) * 0.6 * sp;
        }
        if (n == 1) x[0] = 0.0;
        knot_values(V, x, n, y);
        if (d.type == GW_DIAL_GENERAL) {
          cr_slopes(x, y, n, dy);
          out[0] = x[0];
          out[1] = (x[n - 1] - x[0]) / (n - 1.0);
          for (int k = 0; k < n; ++k) {
            out[2 + 3 * k] = y[k];
            out[3 + 3 * k] = dy[k];
            out[4 + 3 * k] = x[k];
          }
        } else {
          for (int k = 0; k < n; ++k) {
            out[2 * k] = y[k];
            out[2 * k + 1] = x[k];
          }
        }
        return lin_at(x, y, n, nominal_of(d.p0));
      }
      case GW_DIAL_BILINEAR:
      case GW_DIAL_BICUBIC: {
        const double g[5] = {-3.0, -1.5, 0.0, 1.5, 3.0};
        const double s1 = std::exp(std::log(0.8) + V.uniform() * std::log(1.25 / 0.8));
        const double s2 = std::exp(std::log(0.8) + V.uniform() * std::log(1.25 / 0.8));
        out[0] = 5;
        out[1] = 5;
        for (int i = 0; i < 5; ++i) {
          out[2 + i] = g[i];
          out[7 + i] = g[i];
        }
        for (int i = 0; i < 5; ++i)
          for (int j = 0; j < 5; ++j)
            out[12 + i * 5 + j] = std::pow(s1, g[i]) * std::pow(s2, g[j]) *
                                  std::exp(0.05 * (std::fabs(g[i]) + std::fabs(g[j])) * V.normal());
        // nominal: bilinear value at (mean0, mean1)
        const double a = nominal_of(d.p0), b = nominal_of(d.p1);
        int i = 0, j = 0;
        while (i < 3 && a > g[i + 1]) ++i;
        while (j < 3 && b > g[j + 1]) ++j;
        const double fa = (a - g[i]) / 1.5, fb = (b - g[j]) / 1.5;
        const double* z = out + 12;
        const double v0 = z[i * 5 + j] + (z[(i + 1) * 5 + j] - z[i * 5 + j]) * fa;
        const double v1 = z[i * 5 + j + 1] + (z[(i + 1) * 5 + j + 1] - z[i * 5 + j + 1]) * fa;
        return v0 + (v1 - v0) * fb;
      }
      case GW_DIAL_TABULATED: {
        const std::vector<double>& t = host_tables[0];
        const int idx = V.below((int)t.size() - 1);
        const double f = (double)(float)V.uniform();
        out[0] = 0;
        out[1] = idx;
        out[2] = f;
        return f * t[idx] + (1.0 - f) * t[idx + 1];
      }
      case GW_DIAL_KRIGED: {
        if (c.id == GWW_C5) {
          const double tpos = (std::log(d.e) - std::log(kEmin)) / std::log(kEmax / kEmin) * (kKrigedNodes - 1);
          int j0 = (int)std::floor(tpos) - 1;
          j0 = std::max(0, std::min(kKrigedNodes - 4, j0));
          float w[4];
          float sum = 0.f;
          for (int i = 0; i < 4; ++i) {
            w[i] = (float)std::max(0.0, 1.0 - std::fabs(tpos - (j0 + i)) / 2.0);
            sum += w[i];
          }
          out[0] = 0;
          out[1] = 4;
          double nominal = 0.0;
          for (int i = 0; i < 4; ++i) {
            const float wi = w[i] / sum;
            out[2 + i] = j0 + i;
            out[6 + i] = (double)wi;
            nominal += (double)wi * kriged_nominal[(size_t)(j0 + i)];
          }
          return nominal;
        }
        const std::vector<double>& t = host_tables[1];
        out[0] = 1;
        out[1] = n;
        double nominal = 0.0;
        for (int i = 0; i < n; ++i) {
          const int idx = V.below((int)t.size());
          const float w = (float)(0.2 + 0.6 * V.uniform());
          out[2 + i] = idx;
          out[2 + n + i] = (double)w;
          nominal += (double)w * t[(size_t)idx];
        }
        return nominal;
      }
      default:
        return 1.0;
    }
  }
};

double osc_table(const double* q, double E) {
  const double s = std::sin(q[1] * 1.267 / E + q[2]);
  return 1.0 - q[0] * s * s * (1.0 + q[3] * (std::log(E) - q[4])) * q[5];
}

template <typename T>
T* alloc_copy(const std::vector<T>& v) {
  T* p = (T*)std::malloc(std::max<size_t>(1, v.size()) * sizeof(T));
  if (p && !v.empty()) std::memcpy(p, v.data(), v.size() * sizeof(T));
  return p;
}

template <typename F>
void parallel_for(int64_t n, int threads, F f) {
  const int64_t chunk = 4096;
  const int64_t nchunks = (n + chunk - 1) / chunk;
  std::vector<std::thread> th;
  for (int t = 0; t < threads; ++t) {
    th.emplace_back([&, t]() {
      for (int64_t c = t; c < nchunks; c += threads) {
        const int64_t b = c * chunk, e = std::min(n, b + chunk);
        for (int64_t i = b; i < e; ++i) f(i);
      }
    });
  }
  for (auto& x : th) x.join();
}

// Wishart(df, I_n) draw rescaled to unit diagonal.
std::vector<double> wishart_correlation(int n, int df, uint64_t seed) {
  Rng r(seed, 0xFFFFFFF0ull, 3);
  std::vector<double> z((size_t)n * df);
  for (auto& v : z) v = r.normal();
  std::vector<double> w((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j <= i; ++j) {
      double s = 0;
      for (int k = 0; k < df; ++k) s += z[(size_t)i * df + k] * z[(size_t)j * df + k];
      w[(size_t)i * n + j] = w[(size_t)j * n + i] = s;
    }
  std::vector<double> d(n);
  for (int i = 0; i < n; ++i) d[i] = 1.0 / std::sqrt(w[(size_t)i * n + i]);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) w[(size_t)i * n + j] *= d[i] * d[j];
  for (int i = 0; i < n; ++i) w[(size_t)i * n + i] = 1.0;
  return w;
}

}  // namespace

extern "C" const char* gww_last_error(void) { return g_err.c_str(); }

extern "C" int gww_create(int32_t config, int64_t n_events, uint64_t seed, int32_t threads, gww_workload** out) {
  if (!out) return GW_ERR_ARG;
  *out = nullptr;
  Gen g;
  g.c = make_config(config);
  if (g.c.id == 0) {
    g_err = "unknown workload configuration";
    return GW_ERR_ARG;
  }
  if (n_events > 0) {
    if (n_events > INT32_MAX) {
      g_err = "too many events";
      return GW_ERR_ARG;
    }
    g.c.n_events = (int)n_events;
  }
  g.seed = seed;
  if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
  const Config& c = g.c;
  const int N = c.n_events, P = c.n_params;
  try {
    // binning
    const int ns = (int)c.grids.size();
    g.sample_offset.resize(ns + 1, 0);
    for (int s = 0; s < ns; ++s) {
      g.q.push_back(pilot_edges(c.grids[s].first, c.grids[s].second));
      g.sample_offset[s + 1] = g.sample_offset[s] + c.grids[s].first * c.grids[s].second;
    }
    const int B = g.sample_offset[ns];

    // prior, mirrors, clamps, truncation
    std::vector<double> cov((size_t)P * P, 0.0);
    g.prior_mean.assign(P, 0.0);
    std::vector<double> mlo(P, -DBL_MAX), mhi(P, DBL_MAX), clo(P, 0.0), chi(P, DBL_MAX);
    std::vector<uint8_t> trunc(P, 0);
    if (c.id == GWW_C2 || c.id == GWW_C5) {
      const int n = c.n_spline;
      std::vector<double> r = wishart_correlation(n, n + 50, seed);
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) cov[(size_t)i * P + j] = r[(size_t)i * n + j];
    } else {
      for (int i = 0; i < c.n_spline; ++i) cov[(size_t)i * P + i] = 1.0;
    }
    for (int i = 0; i < c.n_norm; ++i) {
      const int p = c.norm_first + i;
      g.prior_mean[p] = 1.0;
      cov[(size_t)p * P + p] = 0.01;
    }
    if (c.table_par_first >= 0) {
      const double mean[6] = {0.5, 2.5, 0.0, 0.1, 0.0, 1.0};
      const double sig[6] = {0.05, 0.1, 0.1, 0.02, 0.1, 0.02};
      for (int i = 0; i < 6; ++i) {
        const int p = c.table_par_first + i;
        g.prior_mean[p] = mean[i];
        cov[(size_t)p * P + p] = sig[i] * sig[i];
      }
    }
    if (c.id == GWW_MIXED_SMALL) {
      mlo[3] = -2.0;
      mhi[3] = 2.5;
      mlo[7] = -1.0;
      mhi[7] = 3.0;
      trunc[4] = trunc[5] = trunc[8] = 1;
      chi[9] = chi[10] = 1.3;
      clo[11] = 0.2;
      // host tables
      g.host_tables[0].resize(50);
      for (int j = 0; j < 50; ++j) g.host_tables[0][j] = 0.7 + 0.3 * std::sin(0.3 * j);
      g.host_tables[1].resize(64);
      for (int j = 0; j < 64; ++j) g.host_tables[1][j] = 0.8 + 0.25 * std::cos(0.2 * j);
    }
    for (int i = 0; i < P; ++i)
      if (cov[(size_t)i * P + i] == 0.0) cov[(size_t)i * P + i] = 1.0;  // parameters no dial uses
    if (c.id == GWW_C5) {
      g.kriged_nodes.resize(kKrigedNodes);
      g.kriged_nominal.resize(kKrigedNodes);
      double q[6];
      for (int i = 0; i < 6; ++i) q[i] = g.prior_mean[c.table_par_first + i];
      for (int j = 0; j < kKrigedNodes; ++j) {
        g.kriged_nodes[j] = std::exp(std::log(kEmin) + (double)j / (kKrigedNodes - 1) * std::log(kEmax / kEmin));
        g.kriged_nominal[j] = osc_table(q, g.kriged_nodes[j]);
      }
    }

    // pass 1: structure and sizes
    std::vector<int32_t> ebin((size_t)N);
    std::vector<int64_t> ecount((size_t)N + 1, 0), edata((size_t)N + 1, 0);
    parallel_for(N, threads, [&](int64_t e) {
      std::vector<DialSpec> ds;
      ds.reserve(32);
      ebin[(size_t)e] = g.structure(e, ds);
      int64_t nd = 0;
      for (const DialSpec& d : ds) nd += Gen::data_len(d);
      ecount[(size_t)e + 1] = (int64_t)ds.size();
      edata[(size_t)e + 1] = nd;
    });
    for (int e = 0; e < N; ++e) {
      ecount[(size_t)e + 1] += ecount[(size_t)e];
      edata[(size_t)e + 1] += edata[(size_t)e];
    }
    const int64_t D = ecount[(size_t)N], ND = edata[(size_t)N];

    gww_workload* w = (gww_workload*)std::calloc(1, sizeof(gww_workload));
    if (!w) throw std::bad_alloc();
    w->config = config;
    w->n_events = N;
    w->n_params = P;
    w->n_bins = B;
    w->n_samples = ns;
    w->n_dials = D;
    w->n_data = ND;
    w->max_weight = c.max_weight;
    w->event_bin = alloc_copy(ebin);
    w->event_w0 = (double*)std::malloc(sizeof(double) * std::max(1, N));
    w->event_dial_start = alloc_copy(ecount);
    w->dial_type = (uint8_t*)std::malloc(std::max<int64_t>(1, D));
    w->dial_par0 = (int32_t*)std::malloc(sizeof(int32_t) * std::max<int64_t>(1, D));
    w->dial_par1 = (int32_t*)std::malloc(sizeof(int32_t) * std::max<int64_t>(1, D));
    w->dial_data_start = (int64_t*)std::malloc(sizeof(int64_t) * (D + 1));
    w->dial_data = (double*)std::malloc(sizeof(double) * std::max<int64_t>(1, ND));
    if (!w->event_w0 || !w->dial_type || !w->dial_par0 || !w->dial_par1 || !w->dial_data_start || !w->dial_data) {
      gww_destroy(w);
      throw std::bad_alloc();
    }
    std::vector<double> nominal((size_t)N);
    // pass 2: fill
    parallel_for(N, threads, [&](int64_t e) {
      std::vector<DialSpec> ds;
      ds.reserve(32);
      g.structure(e, ds);
      Rng V(seed, (uint64_t)e, 1);
      int64_t di = ecount[(size_t)e];
      int64_t off = edata[(size_t)e];
      double w0 = 1.0;
      if (c.id == GWW_MIXED_SMALL) w0 = 0.5 + V.uniform();
      double nom = 1.0;
      for (const DialSpec& d : ds) {
        w->dial_type[di] = (uint8_t)d.type;
        w->dial_par0[di] = d.p0;
        w->dial_par1[di] = d.p1;
        w->dial_data_start[di] = off;
        double r = g.fill(V, d, w->dial_data + off);
        const int pc = d.p0;
        if (pc >= 0) r = std::min(std::max(r, clo[pc]), chi[pc]);
        else r = std::max(r, 0.0);
        nom *= r;
        off += Gen::data_len(d);
        ++di;
      }
      if (c.max_weight > 0 && nom > c.max_weight) nom = c.max_weight;
      w->event_w0[e] = w0;
      nominal[(size_t)e] = w0 * nom;
    });
    w->dial_data_start[D] = ND;

    // data histogram: Poisson draw of the (approximate) nominal prediction
    std::vector<double> pred((size_t)B, 0.0), data((size_t)B, 0.0);
    for (int e = 0; e < N; ++e) pred[(size_t)ebin[(size_t)e]] += nominal[(size_t)e];
    for (int b = 0; b < B; ++b) {
      Rng r(seed, 0xDA7A0000ull + (uint64_t)b, 2);
      std::poisson_distribution<long> pd(std::max(pred[(size_t)b], 1e-12));
      data[(size_t)b] = (double)pd(r);
    }
    w->mirror_lo = alloc_copy(mlo);
    w->mirror_hi = alloc_copy(mhi);
    w->clamp_lo = alloc_copy(clo);
    w->clamp_hi = alloc_copy(chi);
    w->truncate = alloc_copy(trunc);
    w->prior_mean = alloc_copy(g.prior_mean);
    w->prior_cov = alloc_copy(cov);
    w->sample_bin_start = alloc_copy(g.sample_offset);
    w->data = alloc_copy(data);
    // tables
    std::vector<int32_t> tsize, tpar;
    std::vector<int64_t> tstart{0};
    std::vector<double> tnodes, tclamp;
    if (c.id == GWW_MIXED_SMALL) {
      for (int t = 0; t < 2; ++t) {
        tsize.push_back((int32_t)g.host_tables[t].size());
        for (int i = 0; i < 6; ++i) tpar.push_back(-1);
        tnodes.insert(tnodes.end(), g.host_tables[t].begin(), g.host_tables[t].end());
        tstart.push_back((int64_t)tnodes.size());
        tclamp.push_back(t == 0 ? 0.0 : 0.75);
        tclamp.push_back(t == 0 ? DBL_MAX : 1.2);
      }
    } else if (c.id == GWW_C5) {
      tsize.push_back(kKrigedNodes);
      for (int i = 0; i < 6; ++i) tpar.push_back(c.table_par_first + i);
      tnodes = g.kriged_nodes;
      tstart.push_back((int64_t)tnodes.size());
      tclamp.push_back(0.0);
      tclamp.push_back(DBL_MAX);
    }
    w->n_tables = (int32_t)tsize.size();
    w->table_size = alloc_copy(tsize);
    w->table_fn_par = alloc_copy(tpar);
    w->table_node_start = alloc_copy(tstart);
    w->table_nodes = alloc_copy(tnodes);
    w->table_clamp = alloc_copy(tclamp);
    *out = w;
  } catch (const std::bad_alloc&) {
    g_err = "host allocation failed";
    return GW_ERR_NOMEM;
  }
  return GW_OK;
}

extern "C" int gww_destroy(gww_workload* w) {
  if (!w) return GW_ERR_ARG;
  void* ptrs[] = {w->event_bin,     w->event_w0,       w->event_dial_start, w->dial_type,   w->dial_par0,
                  w->dial_par1,     w->dial_data_start, w->dial_data,       w->mirror_lo,   w->mirror_hi,
                  w->clamp_lo,      w->clamp_hi,       w->truncate,         w->prior_mean,  w->prior_cov,
                  w->sample_bin_start, w->data,        w->table_size,       w->table_fn_par, w->table_node_start,
                  w->table_nodes,   w->table_clamp};
  for (void* p : ptrs) std::free(p);
  std::free(w);
  return GW_OK;
}
