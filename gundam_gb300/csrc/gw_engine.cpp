// gw_engine.cpp -- host side of libgw: the cache builder and the C ABI.
//
// The builder takes the same per-dial calls that Cache::Manager::Update makes
// on the reference's calculators (CacheManager.cpp:477-740), keeps them in
// insertion order, and at gw_initialize():
//   1. groups dials by event in insertion order (the order EventDialCache
//      multiplies them in, EventDialCache.cpp:156-171);
//   2. sorts events by global bin (RecursiveSums::Initialize,
//      CacheRecursiveSums.cpp:92-153), stable, so each bin keeps event order;
//   3. cuts the sorted events into tiles (gw_layout.h) and packs each tile's
//      headers and payload in the engine precision;
//   4. builds the (tile, bin) partial-sum slots and uploads everything.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "gw.h"
#include "gw_dfloat.h"
#include "gw_internal.h"

using namespace gw;

namespace {

thread_local std::string g_create_error;

struct HostTable {
  int32_t size = 0;
  std::vector<double> values;
  double lower = 0.0;   // minDialResponse default (DialCollection.cpp:453)
  double upper = DBL_MAX;
  bool dirty = true;
  bool has_fn = false;
  int32_t fn_kind = 0;
  int32_t fn_par[6] = {0, 0, 0, 0, 0, 0};
  std::vector<double> nodes;
};

struct DialRec {
  int32_t result;
  int32_t p0;
  int32_t p1;
  int32_t n_data;
  int64_t data_off;
  uint8_t type;
};

struct PinnedBuf {
  void* p = nullptr;
  size_t bytes = 0;
  ~PinnedBuf() {
    if (p) cudaFreeHost(p);
  }
};

}  // namespace

struct gw_engine {
  gw_config cfg{};
  std::string err;
  bool initialized = false;

  // ---- builder state (host) ----
  std::vector<double> mirror_lo, mirror_hi, clamp_lo, clamp_hi;
  std::vector<uint8_t> pflags;
  std::vector<double> initial;
  std::vector<int32_t> bin;
  std::vector<DialRec> dials;
  std::vector<double> dial_data;
  std::vector<HostTable> tables;
  bool has_cap = false;
  double cap = DBL_MAX;
  std::vector<double> data;
  int32_t llh_type = GW_LLH_NONE;
  std::vector<double> prior_mean, prior_icov;
  bool has_prior = false;
  struct EigenBlock {
    int first, n;
    std::vector<double> V;
  };
  std::vector<EigenBlock> eigen;

  // ---- device state ----
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  DevView view{};
  int kpad = 32;
  int n_slots = 0;
  int plain_grid = 1;
  BatchedShape shape{0, 32, 2, 256, 1, 4};
  int batched_grid = 1;
  bool tuned = false;
  int max_fn_table = 0;
  std::vector<void*> dev_allocs;  // owned device allocations
  void* d_params = nullptr;
  void* d_sums = nullptr;
  void* d_sums2 = nullptr;
  void* d_llh = nullptr;
  void* d_llh_stat = nullptr;
  void* d_evw = nullptr;
  PinnedBuf h_params, h_sums, h_sums2, h_llh, h_llh_stat, h_status;
  bool copy_weights = false;
  bool weights_valid = false;
  bool use_graph = false;
  std::map<int, cudaGraphExec_t> graphs;
  // gw_eval_device graphs, per (K, parameter / output pointers, stream)
  std::map<std::vector<uintptr_t>, cudaGraphExec_t> dev_graphs;
  void clear_graphs() {
    for (auto& g : graphs) cudaGraphExecDestroy(g.second);
    graphs.clear();
    for (auto& g : dev_graphs) cudaGraphExecDestroy(g.second);
    dev_graphs.clear();
  }
  std::vector<int32_t> sorted_to_result;
  gw_layout_info layout{};
  int64_t resident = 0;
  // Every launch chain uses the engine's one set of scratch arrays (mirrored
  // parameters, penalty, partial sums, likelihood counters, status word), so
  // chains on different streams are ordered by an event recorded at the end
  // of each chain (chain_begin / chain_end).
  cudaEvent_t chain_done = nullptr;
  cudaStream_t chain_stream = nullptr;  // stream of the last chain; nullptr: none yet
  bool chain_any = false;
  // profiling
  bool profiling = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> prof_events;
  size_t prof_used = 0;
  int64_t kernel_launches = 0;

  ~gw_engine() {
    clear_graphs();
    for (auto& pe : prof_events) {
      cudaEventDestroy(pe.first);
      cudaEventDestroy(pe.second);
    }
    if (chain_done) cudaEventDestroy(chain_done);
    for (void* p : dev_allocs) cudaFree(p);
    if (stream) cudaStreamDestroy(stream);
  }
};

// ---------------------------------------------------------------------------
// error helpers
// ---------------------------------------------------------------------------
static int fail(gw_engine* e, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (e) e->err = buf;
  else g_create_error = buf;
  return code;
}

#define GW_CUDA(e, call)                                                                      \
  do {                                                                                        \
    cudaError_t _st = (call);                                                                 \
    if (_st != cudaSuccess)                                                                   \
      return fail((e), GW_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(_st));         \
  } while (0)

#define GW_REQUIRE_BUILDER(e)                                                   \
  do {                                                                          \
    if (!(e)) return GW_ERR_ARG;                                                \
    if ((e)->initialized) return fail((e), GW_ERR_STATE, "engine already initialized"); \
  } while (0)

// Cross-stream ordering of the engine's launch chains.  Every chain reads and
// writes the engine's one set of scratch arrays, so a chain (or a copy into
// the engine's tables or data) on stream s first waits for the last chain,
// whichever stream that ran on, and each chain records chain_done on its
// stream when its launches are queued.  Nothing is waited on or recorded
// while s is being captured into a caller's graph: a captured wait on an
// event recorded outside the capture is not allowed, so a caller that
// captures engine calls orders its streams itself.
static int chain_begin(gw_engine* e, cudaStream_t s) {
  if (!e->chain_any || e->chain_stream == s) return GW_OK;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  GW_CUDA(e, cudaStreamIsCapturing(s, &cs));
  if (cs != cudaStreamCaptureStatusNone) return GW_OK;
  GW_CUDA(e, cudaStreamWaitEvent(s, e->chain_done, 0));
  return GW_OK;
}

static int chain_end(gw_engine* e, cudaStream_t s) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  GW_CUDA(e, cudaStreamIsCapturing(s, &cs));
  if (cs != cudaStreamCaptureStatusNone) return GW_OK;
  GW_CUDA(e, cudaEventRecord(e->chain_done, s));
  e->chain_stream = s;
  e->chain_any = true;
  return GW_OK;
}

static bool par_ok(const gw_engine* e, int32_t p) { return p >= 0 && p < e->cfg.n_params; }
static bool res_ok(const gw_engine* e, int32_t r) { return r >= 0 && r < e->cfg.n_results; }

// ---------------------------------------------------------------------------
// lifetime
// ---------------------------------------------------------------------------
extern "C" int gw_has_gpu(int32_t* has_gpu) {
  if (!has_gpu) return GW_ERR_ARG;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) n = 0;
  *has_gpu = n > 0 ? 1 : 0;
  return GW_OK;
}

extern "C" int gw_create(const gw_config* c, gw_engine** out) {
  if (!c || !out) return fail(nullptr, GW_ERR_ARG, "null argument");
  *out = nullptr;
  if (c->n_results < 0 || c->n_params < 1 || c->n_params > 8192 || c->n_bins < 1 || c->k_max < 1 ||
      c->k_max > 4096 || (c->precision != GW_FP64 && c->precision != GW_FP32 && c->precision != GW_DF64) ||
      (c->flags != 0 && c->flags != GW_FLAG_SPLINE_KNOTS && c->flags != GW_FLAG_SPLINE_SLOPES &&
       c->flags != GW_FLAG_SPLINE_COEFS && c->flags != GW_FLAG_SPLINE_GRID))
    return fail(nullptr, GW_ERR_ARG,
                "bad gw_config (n_results=%d n_params=%d n_bins=%d k_max=%d precision=%d flags=%d)",
                c->n_results, c->n_params, c->n_bins, c->k_max, c->precision, c->flags);
  std::unique_ptr<gw_engine> e(new (std::nothrow) gw_engine());
  if (!e) return fail(nullptr, GW_ERR_NOMEM, "host allocation failed");
  e->cfg = *c;
  const int P = c->n_params;
  // Cache::Parameters::Reset (CacheParameters.cpp:126-133): no mirror, open clamps.
  e->mirror_lo.assign(P, -DBL_MAX);
  e->mirror_hi.assign(P, DBL_MAX);
  e->clamp_lo.assign(P, -DBL_MAX);
  e->clamp_hi.assign(P, DBL_MAX);
  e->pflags.assign(P, 0);
  e->initial.assign(c->n_results, 1.0);
  e->bin.assign(c->n_results, -1);
  e->data.assign(c->n_bins, 0.0);
  if (c->device < 0) return fail(nullptr, GW_ERR_ARG, "bad device %d", c->device);
  e->device = c->device;
  *out = e.release();
  return GW_OK;
}

extern "C" int gw_destroy(gw_engine* e) {
  if (!e) return GW_ERR_ARG;
  cudaSetDevice(e->device);
  if (e->stream) cudaStreamSynchronize(e->stream);
  delete e;
  return GW_OK;
}

extern "C" int gw_last_error(const gw_engine* e, char* buf, size_t len) {
  if (!buf || len == 0) return GW_ERR_ARG;
  const std::string& s = e ? e->err : g_create_error;
  snprintf(buf, len, "%s", s.c_str());
  return GW_OK;
}

// ---------------------------------------------------------------------------
// Cache::Parameters
// ---------------------------------------------------------------------------
extern "C" int gw_set_lower_mirror(gw_engine* e, int32_t p, double v) {
  GW_REQUIRE_BUILDER(e);
  if (!par_ok(e, p)) return fail(e, GW_ERR_ARG, "Parameter index out of range: %d", p);
  e->mirror_lo[p] = v;
  return GW_OK;
}
extern "C" int gw_set_upper_mirror(gw_engine* e, int32_t p, double v) {
  GW_REQUIRE_BUILDER(e);
  if (!par_ok(e, p)) return fail(e, GW_ERR_ARG, "Parameter index out of range: %d", p);
  e->mirror_hi[p] = v;
  return GW_OK;
}
extern "C" int gw_set_lower_clamp(gw_engine* e, int32_t p, double v) {
  GW_REQUIRE_BUILDER(e);
  if (!par_ok(e, p)) return fail(e, GW_ERR_ARG, "Parameter index out of range: %d", p);
  e->clamp_lo[p] = v;
  return GW_OK;
}
extern "C" int gw_set_upper_clamp(gw_engine* e, int32_t p, double v) {
  GW_REQUIRE_BUILDER(e);
  if (!par_ok(e, p)) return fail(e, GW_ERR_ARG, "Parameter index out of range: %d", p);
  e->clamp_hi[p] = v;
  return GW_OK;
}
extern "C" int gw_set_extrapolation(gw_engine* e, int32_t p, int32_t allow) {
  GW_REQUIRE_BUILDER(e);
  if (!par_ok(e, p)) return fail(e, GW_ERR_ARG, "Parameter index out of range: %d", p);
  e->pflags[p] = allow ? (uint8_t)(e->pflags[p] & ~1u) : (uint8_t)(e->pflags[p] | 1u);
  return GW_OK;
}

// ---------------------------------------------------------------------------
// Cache::Weights, histogram indices
// ---------------------------------------------------------------------------
extern "C" int gw_set_initial_value(gw_engine* e, int32_t r, double v) {
  GW_REQUIRE_BUILDER(e);
  if (!res_ok(e, r)) return fail(e, GW_ERR_ARG, "Result index out of range: %d", r);
  e->initial[r] = v;
  return GW_OK;
}
extern "C" int gw_set_initial_values(gw_engine* e, int32_t first, int32_t n, const double* v) {
  GW_REQUIRE_BUILDER(e);
  if (n < 0 || !v || first < 0 || (int64_t)first + n > e->cfg.n_results)
    return fail(e, GW_ERR_ARG, "bad result range [%d, %d)", first, first + n);
  std::memcpy(e->initial.data() + first, v, sizeof(double) * (size_t)n);
  return GW_OK;
}
extern "C" int gw_set_event_index(gw_engine* e, int32_t r, int32_t b) {
  GW_REQUIRE_BUILDER(e);
  if (!res_ok(e, r)) return fail(e, GW_ERR_ARG, "Result index out of range: %d", r);
  if (b < 0 || b >= e->cfg.n_bins) return fail(e, GW_ERR_ARG, "Bin index out of range: %d", b);
  e->bin[r] = b;
  return GW_OK;
}
extern "C" int gw_set_event_indices(gw_engine* e, int32_t first, int32_t n, const int32_t* bins) {
  GW_REQUIRE_BUILDER(e);
  if (n < 0 || !bins || first < 0 || (int64_t)first + n > e->cfg.n_results)
    return fail(e, GW_ERR_ARG, "bad result range [%d, %d)", first, first + n);
  for (int32_t i = 0; i < n; ++i) {
    if (bins[i] < 0 || bins[i] >= e->cfg.n_bins)
      return fail(e, GW_ERR_ARG, "Bin index out of range: %d (result %d)", bins[i], first + i);
  }
  std::memcpy(e->bin.data() + first, bins, sizeof(int32_t) * (size_t)n);
  return GW_OK;
}
extern "C" int gw_set_maximum_event_weight(gw_engine* e, double m) {
  GW_REQUIRE_BUILDER(e);
  if (std::isnan(m)) return fail(e, GW_ERR_ARG, "maximum event weight is NaN");
  e->has_cap = std::isfinite(m);
  e->cap = m;
  return GW_OK;
}

// ---------------------------------------------------------------------------
// dials
// ---------------------------------------------------------------------------
static int add_dial(gw_engine* e, int type, int32_t r, int32_t p0, int32_t p1, const double* d, int32_t n) {
  if (!res_ok(e, r)) return fail(e, GW_ERR_ARG, "Result index out of range: %d", r);
  if (n < 0 || (n > 0 && !d)) return fail(e, GW_ERR_ARG, "bad dial data");
  DialRec rec;
  rec.result = r;
  rec.p0 = p0;
  rec.p1 = p1;
  rec.n_data = n;
  rec.data_off = (int64_t)e->dial_data.size();
  rec.type = (uint8_t)type;
  e->dials.push_back(rec);
  e->dial_data.insert(e->dial_data.end(), d, d + n);
  return GW_OK;
}

extern "C" int gw_reserve_norm(gw_engine* e, int32_t r, int32_t p) {
  GW_REQUIRE_BUILDER(e);
  if (!par_ok(e, p)) return fail(e, GW_ERR_ARG, "Parameter index out of range: %d", p);
  return add_dial(e, kNorm, r, p, -1, nullptr, 0);
}

extern "C" int gw_add_spline(gw_engine* e, int32_t type, int32_t r, int32_t p, const double* d, int32_t n) {
  GW_REQUIRE_BUILDER(e);
  if (type != kMonotonic && type != kUniform && type != kGeneral && type != kCompact)
    return fail(e, GW_ERR_ARG, "not a spline type: %d", type);
  if (!par_ok(e, p)) return fail(e, GW_ERR_ARG, "Parameter index out of range: %d", p);
  return add_dial(e, type, r, p, -1, d, n);
}

extern "C" int gw_add_graph(gw_engine* e, int32_t r, int32_t p, const double* d, int32_t n) {
  GW_REQUIRE_BUILDER(e);
  if (!par_ok(e, p)) return fail(e, GW_ERR_ARG, "Parameter index out of range: %d", p);
  return add_dial(e, kGraph, r, p, -1, d, n);
}

extern "C" int gw_add_surface(gw_engine* e, int32_t type, int32_t r, int32_t p1, int32_t p2, const double* d,
                              int32_t n) {
  GW_REQUIRE_BUILDER(e);
  if (type != kBilinear && type != kBicubic) return fail(e, GW_ERR_ARG, "not a surface type: %d", type);
  if (!par_ok(e, p1) || !par_ok(e, p2)) return fail(e, GW_ERR_ARG, "Parameter index out of range");
  return add_dial(e, type, r, p1, p2, d, n);
}

extern "C" int gw_add_tabulated(gw_engine* e, int32_t r, int32_t table, int32_t index, double fraction) {
  GW_REQUIRE_BUILDER(e);
  const double d[3] = {(double)table, (double)index, fraction};
  return add_dial(e, kTabulated, r, -1, -1, d, 3);
}

extern "C" int gw_add_kriged(gw_engine* e, int32_t r, int32_t table, int32_t n, const int32_t* index,
                             const float* weight) {
  GW_REQUIRE_BUILDER(e);
  if (n < 0 || n > kMaxKnots || (n > 0 && (!index || !weight)))
    return fail(e, GW_ERR_ARG, "bad kriged dial (n=%d)", n);
  std::vector<double> d(2 + 2 * (size_t)n);
  d[0] = table;
  d[1] = n;
  for (int i = 0; i < n; ++i) {
    d[2 + i] = index[i];
    d[2 + n + i] = (double)weight[i];
  }
  return add_dial(e, kKriged, r, -1, -1, d.data(), (int32_t)d.size());
}

extern "C" int gw_add_dials(gw_engine* e, int64_t n, const uint8_t* type, const int32_t* result,
                            const int32_t* par0, const int32_t* par1, const int64_t* start, const double* d) {
  GW_REQUIRE_BUILDER(e);
  if (n < 0 || (n > 0 && (!type || !result || !par0 || !start))) return fail(e, GW_ERR_ARG, "null array");
  const int64_t base = (int64_t)e->dial_data.size();
  const int64_t total = n > 0 ? start[n] - start[0] : 0;
  if (total < 0) return fail(e, GW_ERR_ARG, "bad data_start");
  e->dials.reserve(e->dials.size() + (size_t)n);
  for (int64_t i = 0; i < n; ++i) {
    const int t = type[i];
    if (t < kNorm || t > kKriged) return fail(e, GW_ERR_ARG, "dial %lld: bad type %d", (long long)i, t);
    if (!res_ok(e, result[i])) return fail(e, GW_ERR_ARG, "dial %lld: result out of range", (long long)i);
    if (t < kTabulated && !par_ok(e, par0[i]))
      return fail(e, GW_ERR_ARG, "dial %lld: parameter index out of range: %d", (long long)i, par0[i]);
    if ((t == kBilinear || t == kBicubic) && (!par1 || !par_ok(e, par1[i])))
      return fail(e, GW_ERR_ARG, "dial %lld: second parameter out of range", (long long)i);
    const int64_t len = start[i + 1] - start[i];
    if (len < 0 || len > (1 << 20)) return fail(e, GW_ERR_ARG, "dial %lld: bad data length", (long long)i);
    DialRec rec;
    rec.result = result[i];
    rec.p0 = t < kTabulated ? par0[i] : -1;
    rec.p1 = (t == kBilinear || t == kBicubic) ? par1[i] : -1;
    rec.n_data = (int32_t)len;
    rec.data_off = base + (start[i] - start[0]);
    rec.type = (uint8_t)t;
    e->dials.push_back(rec);
  }
  if (total > 0) e->dial_data.insert(e->dial_data.end(), d + start[0], d + start[0] + total);
  return GW_OK;
}

// ---------------------------------------------------------------------------
// tables
// ---------------------------------------------------------------------------
extern "C" int gw_create_table(gw_engine* e, int32_t size, int32_t* table) {
  GW_REQUIRE_BUILDER(e);
  if (size < 2 || !table) return fail(e, GW_ERR_ARG, "bad table size %d", size);
  if (e->tables.size() >= 65535) return fail(e, GW_ERR_LIMIT, "too many tables");
  HostTable t;
  t.size = size;
  t.values.assign(size, 0.0);
  e->tables.push_back(std::move(t));
  *table = (int32_t)e->tables.size() - 1;
  return GW_OK;
}

extern "C" int gw_set_table(gw_engine* e, int32_t table, const double* values, int32_t size) {
  if (!e) return GW_ERR_ARG;
  if (table < 0 || table >= (int32_t)e->tables.size()) return fail(e, GW_ERR_ARG, "bad table %d", table);
  HostTable& t = e->tables[table];
  if (size != t.size || !values) return fail(e, GW_ERR_ARG, "table %d: size %d != %d", table, size, t.size);
  if (t.has_fn) return fail(e, GW_ERR_STATE, "table %d is filled on the device", table);
  for (int32_t i = 0; i < size; ++i) {
    // WeightTabulated.cpp:165-168 rejects non-finite entries.
    if (!std::isfinite(values[i])) return fail(e, GW_ERR_NOT_FINITE, "Table entry is not finite (%d)", i);
  }
  std::memcpy(t.values.data(), values, sizeof(double) * (size_t)size);
  t.dirty = true;
  return GW_OK;
}

extern "C" int gw_set_table_clamp(gw_engine* e, int32_t table, double lower, double upper) {
  GW_REQUIRE_BUILDER(e);
  if (table < 0 || table >= (int32_t)e->tables.size()) return fail(e, GW_ERR_ARG, "bad table %d", table);
  e->tables[table].lower = lower;
  e->tables[table].upper = upper;
  return GW_OK;
}

extern "C" int gw_set_table_function(gw_engine* e, int32_t table, int32_t fn, const int32_t* params,
                                     int32_t n_params, const double* nodes, int32_t size) {
  GW_REQUIRE_BUILDER(e);
  if (table < 0 || table >= (int32_t)e->tables.size()) return fail(e, GW_ERR_ARG, "bad table %d", table);
  HostTable& t = e->tables[table];
  if (fn != GW_TABLE_FN_OSCILLATION || n_params != 6 || !params || !nodes || size != t.size)
    return fail(e, GW_ERR_ARG, "bad table function for table %d", table);
  for (int i = 0; i < 6; ++i)
    if (!par_ok(e, params[i])) return fail(e, GW_ERR_ARG, "table function parameter out of range");
  for (int i = 0; i < size; ++i)
    if (!(nodes[i] > 0.0) || !std::isfinite(nodes[i])) return fail(e, GW_ERR_ARG, "table node %d not > 0", i);
  t.has_fn = true;
  t.fn_kind = fn;
  std::memcpy(t.fn_par, params, sizeof(t.fn_par));
  t.nodes.assign(nodes, nodes + size);
  return GW_OK;
}

// ---------------------------------------------------------------------------
// likelihood
// ---------------------------------------------------------------------------
extern "C" int gw_set_data(gw_engine* e, const double* data, int32_t n_bins) {
  if (!e || !data) return GW_ERR_ARG;
  if (n_bins != e->cfg.n_bins) return fail(e, GW_ERR_ARG, "data has %d bins, engine %d", n_bins, e->cfg.n_bins);
  std::memcpy(e->data.data(), data, sizeof(double) * (size_t)n_bins);
  if (e->initialized) {
    GW_CUDA(e, cudaSetDevice(e->device));
    const int rc = chain_begin(e, e->stream);  // a chain on another stream may still read the data
    if (rc) return rc;
    GW_CUDA(e, cudaMemcpyAsync((void*)e->view.data, data, sizeof(double) * (size_t)n_bins, cudaMemcpyHostToDevice,
                               e->stream));
    GW_CUDA(e, cudaStreamSynchronize(e->stream));
  }
  return GW_OK;
}

extern "C" int gw_set_likelihood(gw_engine* e, int32_t t) {
  if (!e) return GW_ERR_ARG;
  if (t != GW_LLH_NONE && t != GW_LLH_POISSON && t != GW_LLH_BARLOW_BEESTON_OA2021)
    return fail(e, GW_ERR_ARG, "bad likelihood type %d", t);
  e->llh_type = t;
  e->view.llh_type = t;
  e->clear_graphs();
  return GW_OK;
}

extern "C" int gw_set_prior(gw_engine* e, const double* mean, const double* icov) {
  GW_REQUIRE_BUILDER(e);
  if (!mean || !icov) {
    e->has_prior = false;
    return GW_OK;
  }
  const size_t P = (size_t)e->cfg.n_params;
  e->prior_mean.assign(mean, mean + P);
  e->prior_icov.assign(icov, icov + P * P);
  e->has_prior = true;
  return GW_OK;
}

// ParameterSet eigen decomposition (ParameterSet.cpp:766-780,
// ParametersManager::convertEigenToOrig, ParametersManager.cpp:329-334):
// parameters [first, first + n) are given in the eigen basis and the engine
// forms original = V * given on the device before mirroring and the dials.
extern "C" int gw_add_eigen_block(gw_engine* e, int32_t first, int32_t n, const double* V) {
  GW_REQUIRE_BUILDER(e);
  if (!V || n < 1 || first < 0 || first + n > e->cfg.n_params)
    return fail(e, GW_ERR_ARG, "eigen block [%d, %d) outside the %d parameters", first, first + n, e->cfg.n_params);
  for (const auto& b : e->eigen)
    if (first < b.first + b.n && b.first < first + n)
      return fail(e, GW_ERR_ARG, "eigen block [%d, %d) overlaps [%d, %d)", first, first + n, b.first, b.first + b.n);
  for (int64_t i = 0; i < (int64_t)n * n; ++i)
    if (!std::isfinite(V[i])) return fail(e, GW_ERR_NOT_FINITE, "eigen block matrix is not finite");
  e->eigen.push_back({first, n, std::vector<double>(V, V + (size_t)n * n)});
  return GW_OK;
}

// ---------------------------------------------------------------------------
// initialize: validate, sort, tile, pack, upload
// ---------------------------------------------------------------------------
namespace {

// Payload elements a dial occupies, or -1 (with a message) when invalid.
int64_t payload_elems(gw_engine* e, const DialRec& r, const double* d, int* n_out) {
  const int n = r.n_data;
  switch (r.type) {
    case kNorm:
      *n_out = 0;
      return 0;
    case kMonotonic:
    case kCompact: {
      const int k = n - 2;
      if (k < 2 || k > kMaxKnots || !(d[1] > 0.0)) return -1;
      *n_out = k;
      return k + 2;
    }
    case kUniform: {
      if (n < 2 || (n - 2) % 2) return -1;
      const int k = (n - 2) / 2;
      if (k < 2 || k > kMaxKnots || !(d[1] > 0.0)) return -1;
      *n_out = k;
      return 2 + 2 * k;
    }
    case kGeneral: {
      if (n < 2 || (n - 2) % 3) return -1;
      const int k = (n - 2) / 3;
      if (k < 2 || k > kMaxKnots) return -1;
      for (int i = 1; i < k; ++i)
        if (!(d[2 + 3 * i + 2] > d[2 + 3 * (i - 1) + 2])) return -1;
      *n_out = k;
      return 3 * k;
    }
    case kGraph: {
      if (n < 2 || n % 2) return -1;
      const int k = n / 2;
      if (k > kMaxKnots) return -1;
      for (int i = 1; i < k; ++i)
        if (!(d[2 * i + 1] > d[2 * (i - 1) + 1])) return -1;
      *n_out = k;
      return 2 * k;
    }
    case kBilinear:
    case kBicubic: {
      if (n < 2) return -1;
      const double fx = d[0], fy = d[1];
      if (fx != std::floor(fx) || fy != std::floor(fy) || fx < 2 || fy < 2 || fx > 17 || fy > 17) return -1;
      const int nx = (int)fx, ny = (int)fy;
      if (n != 2 + nx + ny + nx * ny) return -1;
      for (int i = 1; i < nx; ++i)
        if (!(d[2 + i] > d[2 + i - 1])) return -1;
      for (int i = 1; i < ny; ++i)
        if (!(d[2 + nx + i] > d[2 + nx + i - 1])) return -1;
      *n_out = 0;
      return n;
    }
    case kTabulated: {
      if (n != 3) return -1;
      const int t = (int)d[0];
      if ((double)t != d[0] || t < 0 || t >= (int)e->tables.size()) return -1;
      const int idx = (int)d[1];
      if ((double)idx != d[1] || idx < 0 || idx + 1 >= e->tables[t].size || idx >= (1 << 24)) return -1;
      *n_out = 0;
      return 2;
    }
    case kKriged: {
      if (n < 2) return -1;
      const int t = (int)d[0];
      if ((double)t != d[0] || t < 0 || t >= (int)e->tables.size()) return -1;
      const int m = (int)d[1];
      if ((double)m != d[1] || m < 0 || m > kMaxKnots || n != 2 + 2 * m) return -1;
      for (int i = 0; i < m; ++i) {
        const int idx = (int)d[2 + i];
        if ((double)idx != d[2 + i] || idx < 0 || idx >= e->tables[t].size || idx >= (1 << 24)) return -1;
      }
      *n_out = m;
      return 2 * m;
    }
    default:
      return -1;
  }
}

// Writes the engine payload of one dial (reference data vector -> payload).
template <typename T>
void write_payload(const DialRec& r, const double* d, T* out) {
  switch (r.type) {
    case kNorm:
      break;
    case kGeneral: {  // drop the unused [low, step] prefix
      for (int i = 0; i < r.n_data - 2; ++i) out[i] = (T)d[2 + i];
      break;
    }
    case kTabulated:
      out[0] = (T)d[2];  // fraction
      out[1] = (T)d[1];  // index
      break;
    case kKriged: {
      const int m = (int)d[1];
      for (int i = 0; i < 2 * m; ++i) out[i] = (T)d[2 + i];
      break;
    }
    default:
      for (int i = 0; i < r.n_data; ++i) out[i] = (T)d[i];
  }
}

// Knot values and slopes in index units of a uniform-knot spline: for
// uniform splines the stored dydx times the step; for Catmull-Rom splines the
// slope CalculateMonotonicSpline.h:66-127 forms from the neighbours (with the
// Fritsch-Carlson limiter for monotonic splines), the end knots the end
// difference.  In FP64.
static void knot_slopes(const DialRec& r, const double* d, int n, double* y, double* s) {
  const double step = d[1];
  if (r.type == kUniform) {
    for (int k = 0; k < n; ++k) {
      y[k] = d[2 + 2 * k];
      s[k] = d[3 + 2 * k] * step;
    }
    return;
  }
  const bool limit = r.type == kMonotonic;
  for (int k = 0; k < n; ++k) y[k] = d[2 + k];
  for (int k = 0; k < n; ++k) {
    if (k == 0) {
      s[k] = y[1] - y[0];
    } else if (k == n - 1) {
      s[k] = y[n - 1] - y[n - 2];
    } else {
      const double dl = y[k] - y[k - 1], dr = y[k + 1] - y[k];
      double v = 0.5 * (dl + dr);
      if (limit) {
        if (dr * dl <= 0.0) v = 0.0;
        const double delta = 3.0 * std::min(std::fabs(dl), std::fabs(dr));
        if (v > delta) v = delta;
        if (v < -delta) v = -delta;
      }
      s[k] = v;
    }
  }
}

// Stored form of a spline's Catmull-Rom or Hermite data (SplineForm).
enum SplineForm { kFormSlopes = 0, kFormKnots = 1, kFormCoefs = 2, kFormGrid = 3 };

// Engine layout of Catmull-Rom (monotonic, compact) and uniform splines.
// Slopes form: [low, 1/step, (y, s) x n], s the knot slope in index units
// (knot_slopes); knots form (Catmull-Rom only): [low, 1/step, y x n], the
// slopes formed in the kernel; coefficients form: below.
template <typename T>
void write_prepared(const DialRec& r, const double* d, int n, T* out, int form) {
  const double low = d[0], step = d[1];
  if (form == kFormCoefs || form == kFormGrid) {
    // the grid form keeps the blocks alone: [(c0, c1, c2, c3) x (n + 1)]
    const int b0 = form == kFormGrid ? 0 : 4;
    // [-low/step, 1/step, 0, 0, (c0, c1, c2, c3) x (n + 1)]: interval j + 1
    // holds the cubic v(u) = c0 + u (c1 + u (c2 + u c3)) of u = xx - j, xx =
    // (x - low) / step, for j = -1 .. n - 1.  j = 0 .. n - 2 are the Hermite
    // cubics on the knot intervals (CalculateUniformSpline.h:71-74 expanded);
    // j = -1 and j = n - 1 re-expand the end intervals' cubics, which the
    // reference evaluates beyond the knots (for Catmull-Rom splines with the
    // end difference as the outer slope, CalculateMonotonicSpline.h:66-103),
    // about u = xx + 1 and u = xx - (n - 1).
    std::vector<double> y((size_t)n), sl((size_t)n);
    knot_slopes(r, d, n, y.data(), sl.data());
    const bool catmull = r.type != kUniform;
    auto cubic = [&](int i, double m1, double m2, double* c) {
      const double dc = y[(size_t)i + 1] - y[(size_t)i];
      c[0] = y[(size_t)i];
      c[1] = m1;
      c[2] = 3.0 * dc - 2.0 * m1 - m2;
      c[3] = m1 + m2 - 2.0 * dc;
    };
    if (form == kFormCoefs) {
      out[0] = (T)(-low / step);
      out[1] = (T)(1.0 / step);
      out[2] = (T)0.0;
      out[3] = (T)0.0;
    }
    double c[4];
    for (int j = 0; j + 1 < n; ++j) {
      cubic(j, sl[(size_t)j], sl[(size_t)j + 1], c);
      for (int q = 0; q < 4; ++q) out[b0 + 4 * (j + 1) + q] = (T)c[q];
    }
    // before the first knot: P(t), t = xx, as P(u - 1)
    cubic(0, sl[0], catmull ? y[1] - y[0] : sl[1], c);
    const double left[4] = {c[0] - c[1] + c[2] - c[3], c[1] - 2.0 * c[2] + 3.0 * c[3], c[2] - 3.0 * c[3], c[3]};
    // after the last knot: P(t), t = xx - (n - 2), as P(u + 1)
    cubic(n - 2, catmull ? y[(size_t)n - 1] - y[(size_t)n - 2] : sl[(size_t)n - 2], sl[(size_t)n - 1], c);
    const double right[4] = {c[0] + c[1] + c[2] + c[3], c[1] + 2.0 * c[2] + 3.0 * c[3], c[2] + 3.0 * c[3], c[3]};
    for (int q = 0; q < 4; ++q) {
      out[b0 + q] = (T)left[q];
      out[b0 + 4 * n + q] = (T)right[q];
    }
    return;
  }
  out[0] = (T)low;
  out[1] = (T)(1.0 / step);
  if (form == kFormKnots && r.type != kUniform) {  // [low, 1/step, y x n]: slopes formed in the kernel
    for (int k = 0; k < n; ++k) out[2 + k] = (T)d[2 + k];
    return;
  }
  std::vector<double> y((size_t)n), sl((size_t)n);
  knot_slopes(r, d, n, y.data(), sl.data());
  for (int k = 0; k < n; ++k) {
    out[2 + 2 * k] = (T)y[(size_t)k];
    out[3 + 2 * k] = (T)sl[(size_t)k];
  }
}

// Stored elements of a dial in the engine precision.  Non-empty payloads are
// padded to an odd element count: threads that read consecutive same-type
// dials then hit distinct shared-memory banks.
int32_t stored_elems(const DialRec& r, int n, int32_t raw, int form) {
  const bool uniform_knots = r.type == kMonotonic || r.type == kCompact || r.type == kUniform;
  if (form == kFormCoefs && uniform_knots) return 4 + 4 * (n + 1);  // 16-byte multiple, packed first
  if (form == kFormGrid && uniform_knots) return 4 * (n + 1);
  int32_t el = (r.type == kMonotonic || r.type == kCompact) ? (form == kFormKnots ? 2 + n : 2 + 2 * n) : raw;
  if (el > 0 && (el & 1) == 0) ++el;
  return el;
}

struct TilePlan {
  int64_t ev_begin, ev_end;  // into the sorted event list
  int32_t ndials;
  int32_t payload_elems;
  int64_t dial0;
  uint64_t payload_off;
  int32_t bin0;
  int32_t nbins;
};

template <typename T>
int build_and_upload(gw_engine* e) {
  const int N = e->cfg.n_results;
  const int B = e->cfg.n_bins;
  const int64_t D = (int64_t)e->dials.size();
  const size_t tsz = sizeof(T);
  // stored form of the uniform-knot splines (gw_config.flags).  Default:
  // knot values for FP32 K = 1 engines (bandwidth-bound); the grid form for
  // engines evaluating 32 or more points, where the lanes-over-points kernel
  // runs (64 points of a 2M-event mixed workload: FP32 2.74 ms against
  // 3.27 ms with stored slopes, FP64 12.3 ms against 18.8 ms with the
  // coefficient form).  At 16-31 points the threads-over-dials kernels win,
  // and their scattered per-dial reads of the grid table pay only while the
  // table stays in L1 (FP32, 16 points: a 100k-event workload with 20 grids
  // 0.054 ms against 0.072 ms with stored slopes; the 2M-event workload with
  // 400 grids 2.48 ms against 1.84 ms), so there the grid form is kept when
  // the table holds at most 32 KB, else FP64 engines take the coefficient
  // form (their evaluation is bound by the FP64 pipe) and the others stored
  // slopes; precomputed slopes otherwise
  const int form_small = (e->cfg.precision == GW_FP64) ? kFormCoefs : kFormSlopes;
  const bool grid_if_small = e->cfg.flags == 0 && e->cfg.k_max >= 16 && e->cfg.k_max < 32;
  int form = e->cfg.flags == GW_FLAG_SPLINE_KNOTS           ? kFormKnots
             : e->cfg.flags == GW_FLAG_SPLINE_COEFS         ? kFormCoefs
             : e->cfg.flags == GW_FLAG_SPLINE_GRID          ? kFormGrid
             : e->cfg.flags == GW_FLAG_SPLINE_SLOPES        ? kFormSlopes
             : (e->cfg.k_max == 1 && tsz == 4)              ? kFormKnots
             : (e->cfg.k_max >= 32 || grid_if_small)        ? kFormGrid
                                                            : kFormSlopes;

  // 1. every result needs a bin (CacheManager.cpp:727-729 "Histogram cells are missing")
  for (int r = 0; r < N; ++r)
    if (e->bin[r] < 0) return fail(e, GW_ERR_STATE, "result %d has no histogram bin", r);
  // response clamps must be ordered (the kernels apply them as one interval)
  for (int p = 0; p < e->cfg.n_params; ++p)
    if (!(e->clamp_lo[p] <= e->clamp_hi[p]))
      return fail(e, GW_ERR_ARG, "parameter %d: lower clamp %g above upper clamp %g", p, e->clamp_lo[p],
                  e->clamp_hi[p]);
  for (size_t t = 0; t < e->tables.size(); ++t)
    if (!(e->tables[t].lower <= e->tables[t].upper))
      return fail(e, GW_ERR_ARG, "table %zu: lower clamp above upper clamp", t);

  // 2. dials grouped by result, insertion order kept (counting sort)
  std::vector<int64_t> rstart((size_t)N + 1, 0);
  for (const DialRec& r : e->dials) rstart[(size_t)r.result + 1]++;
  for (int r = 0; r < N; ++r) rstart[r + 1] += rstart[r];
  std::vector<int64_t> byres((size_t)D);
  {
    std::vector<int64_t> fillp(rstart.begin(), rstart.end() - 1);
    for (int64_t i = 0; i < D; ++i) byres[(size_t)fillp[e->dials[(size_t)i].result]++] = i;
  }
  // the grid form: uniform-knot splines that share (parameter, first knot,
  // step, knot count) share one knot grid, whose interval and fraction
  // k_params forms once per point; up to kMaxGrids grids in first-seen
  // order, the splines of any further grid keep the coefficient form
  std::vector<int32_t> grid_of;
  std::vector<GridDesc> grids;
  if (form == kFormGrid) {
    grid_of.assign((size_t)D, -1);
    struct Key {
      int32_t p0, n;
      double low, step;
      bool operator<(const Key& o) const {
        if (p0 != o.p0) return p0 < o.p0;
        if (n != o.n) return n < o.n;
        if (low != o.low) return low < o.low;
        return step < o.step;
      }
    };
    auto key_of = [&](const DialRec& r, Key* k) {
      if (r.type != kMonotonic && r.type != kCompact && r.type != kUniform) return false;
      const double* d = e->dial_data.data() + r.data_off;
      const int n = r.type == kUniform ? (r.n_data - 2) / 2 : r.n_data - 2;
      if (n < 2 || n > kMaxKnots || !(d[1] > 0.0) || !std::isfinite(d[0]) || !std::isfinite(d[1])) return false;
      *k = Key{r.p0, n, d[0], d[1]};
      return true;
    };
    // each thread names the grids of its dials locally; the local names are
    // then merged in first-seen order of the dials
    const int nth = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    const int64_t chunk = (D + nth - 1) / std::max(nth, 1);
    std::vector<std::map<Key, int32_t>> local((size_t)nth);
    std::vector<std::vector<std::pair<int64_t, Key>>> first((size_t)nth);
    std::vector<std::thread> th;
    for (int t = 0; t < nth; ++t) {
      th.emplace_back([&, t]() {
        for (int64_t i = t * chunk; i < std::min<int64_t>(D, (t + 1) * chunk); ++i) {
          Key k;
          if (!key_of(e->dials[(size_t)i], &k)) continue;
          auto it = local[(size_t)t].find(k);
          if (it == local[(size_t)t].end()) {
            it = local[(size_t)t].emplace(k, (int32_t)first[(size_t)t].size()).first;
            first[(size_t)t].emplace_back(i, k);
          }
          grid_of[(size_t)i] = it->second;
        }
      });
    }
    for (auto& x : th) x.join();
    th.clear();
    std::map<Key, int32_t> global;
    std::vector<std::vector<int32_t>> to_global((size_t)nth);
    for (int t = 0; t < nth; ++t) {
      for (const auto& f : first[(size_t)t]) {
        auto it = global.find(f.second);
        int32_t g = -1;
        if (it != global.end()) {
          g = it->second;
        } else if ((int)grids.size() < kMaxGrids) {
          g = (int32_t)grids.size();
          global.emplace(f.second, g);
          GridDesc gd{};
          gd.a = -f.second.low / f.second.step;
          gd.b = 1.0 / f.second.step;
          gd.p0 = f.second.p0;
          gd.n = f.second.n;
          gd.trunc = (e->pflags[(size_t)f.second.p0] & 1) ? 1 : 0;
          grids.push_back(gd);
        }
        to_global[(size_t)t].push_back(g);
      }
    }
    for (int t = 0; t < nth; ++t) {
      th.emplace_back([&, t]() {
        for (int64_t i = t * chunk; i < std::min<int64_t>(D, (t + 1) * chunk); ++i)
          if (grid_of[(size_t)i] >= 0) grid_of[(size_t)i] = to_global[(size_t)t][(size_t)grid_of[(size_t)i]];
      });
    }
    for (auto& x : th) x.join();
    const int64_t kpad_of = ((e->cfg.k_max + 63) / 64) * 64;
    if (grid_if_small && (int64_t)grids.size() * kpad_of * (int64_t)sizeof(GridPoint<T>) > 32768) {
      form = form_small;
      grids.clear();
      grid_of.clear();
    }
  }
  // the stored form of the uniform-knot splines outside the grids
  const int dial_form = form == kFormGrid ? kFormCoefs : form;

  // per-dial payload sizes and knot counts
  std::vector<int32_t> pel((size_t)D), pn((size_t)D);
  {
    std::atomic<int64_t> bad{-1};
    const int nth = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    std::vector<std::thread> th;
    for (int t = 0; t < nth; ++t) {
      th.emplace_back([&, t]() {
        for (int64_t i = t; i < D; i += nth) {
          int n = 0;
          const DialRec& r = e->dials[(size_t)i];
          const int64_t el = payload_elems(e, r, e->dial_data.data() + r.data_off, &n);
          if (el < 0) {
            int64_t exp = -1;
            bad.compare_exchange_strong(exp, i);
          }
          const int f = (!grid_of.empty() && grid_of[(size_t)i] >= 0) ? kFormGrid : dial_form;
          pel[(size_t)i] = el < 0 ? -1 : stored_elems(r, n, (int32_t)el, f);
          pn[(size_t)i] = n;
        }
      });
    }
    for (auto& x : th) x.join();
    if (bad.load() >= 0) {
      const DialRec& r = e->dials[(size_t)bad.load()];
      return fail(e, GW_ERR_ARG, "dial %lld (type %d, result %d, %d values) has invalid data",
                  (long long)bad.load(), (int)r.type, r.result, r.n_data);
    }
  }

  // 3. stable sort of results by bin
  std::vector<int64_t> bstart((size_t)B + 1, 0);
  for (int r = 0; r < N; ++r) bstart[(size_t)e->bin[r] + 1]++;
  for (int b = 0; b < B; ++b) bstart[b + 1] += bstart[b];
  std::vector<int32_t> sorted((size_t)N);
  {
    std::vector<int64_t> fillp(bstart.begin(), bstart.end() - 1);
    for (int r = 0; r < N; ++r) sorted[(size_t)fillp[e->bin[r]]++] = r;
  }

  // 4. tiles
  // default tile payload: 28 KB in FP32 (fastest of a 12-32 KB sweep on the
  // 5M-event mixed workload at K = 1; larger FP32 tiles cost the K = 1 kernel
  // its third CTA per SM), 32 KB for FP32 engines evaluating 16 or more points
  // (K = 64: 8.55 ms against 8.68 ms at 28 KB; beyond 32 KB the tiles' event
  // and dial limits bind first), 40 KB for the 8-byte precisions (FP64
  // and double-float: fastest of 16-48 KB at K = 1 and K = 64; at 48 KB one
  // CTA per SM is left)
  const int64_t tile_default = tsz == 4 ? (e->cfg.k_max >= 16 ? 32768 : 28672) : 40960;
  int64_t cap_elems = (e->cfg.tile_bytes > 0 ? e->cfg.tile_bytes : tile_default) / (int64_t)tsz;
  cap_elems = std::min<int64_t>(cap_elems, kMaxPayloadElems);
  cap_elems = std::max<int64_t>(cap_elems, 64);
  std::vector<TilePlan> tiles;
  {
    TilePlan cur{0, 0, 0, 0, 0, 0, -1, 0};
    for (int64_t i = 0; i < N; ++i) {
      const int r = sorted[(size_t)i];
      const int nd = (int)(rstart[r + 1] - rstart[r]);
      int64_t pe = 0;
      for (int64_t j = rstart[r]; j < rstart[r + 1]; ++j) pe += pel[(size_t)byres[(size_t)j]];
      if (nd > kMaxTileDials || pe > cap_elems)
        return fail(e, GW_ERR_LIMIT, "result %d alone exceeds a tile (%d dials, %lld payload values, limit %lld)",
                    r, nd, (long long)pe, (long long)cap_elems);
      const int b = e->bin[r];
      const bool fits = cur.ev_end > cur.ev_begin && cur.ndials + nd <= kMaxTileDials &&
                        cur.payload_elems + pe <= cap_elems && (cur.ev_end - cur.ev_begin) < kMaxTileEvents &&
                        b - cur.bin0 < kMaxLocalBins;
      if (!fits && cur.ev_end > cur.ev_begin) {
        tiles.push_back(cur);
        cur = TilePlan{i, i, 0, 0, 0, 0, -1, 0};
      }
      if (cur.ev_end == cur.ev_begin) {
        cur.ev_begin = i;
        cur.bin0 = b;
      }
      cur.ev_end = i + 1;
      cur.ndials += nd;
      cur.payload_elems += (int32_t)pe;
      cur.nbins = b - cur.bin0 + 1;
    }
    if (cur.ev_end > cur.ev_begin) tiles.push_back(cur);
  }
  const int64_t T_ = (int64_t)tiles.size();
  if (T_ > INT32_MAX) return fail(e, GW_ERR_LIMIT, "too many tiles");
  // every tile's headers start on a 16-byte boundary (an even header index),
  // so one bulk copy moves them with the payload
  int64_t hdr_total = 0;
  int32_t max_tile_dials = 0;
  {
    int64_t d0 = 0;
    uint64_t off = 0;
    for (TilePlan& t : tiles) {
      t.dial0 = d0;
      d0 += t.ndials;
      d0 = (d0 + 1) & ~(int64_t)1;
      max_tile_dials = std::max(max_tile_dials, t.ndials);
      t.payload_off = off;
      const uint64_t bytes = ((uint64_t)t.payload_elems * tsz + 15) & ~(uint64_t)15;
      off += bytes;
    }
    hdr_total = d0;
  }
  const uint64_t payload_total = T_ ? tiles.back().payload_off +
                                          (((uint64_t)tiles.back().payload_elems * tsz + 15) & ~(uint64_t)15)
                                    : 0;

  // 5. partial-sum slots: bin b receives one slot per tile that holds events of b
  std::vector<int32_t> bin_slot((size_t)B + 1, 0);
  std::vector<int32_t> tile_slot0((size_t)T_, 0);
  {
    std::vector<int32_t> cover((size_t)B, 0);
    std::vector<int32_t> first_rank((size_t)T_, 0);
    for (int64_t t = 0; t < T_; ++t) {
      const TilePlan& tp = tiles[(size_t)t];
      int last_b = -1;
      for (int64_t i = tp.ev_begin; i < tp.ev_end; ++i) {
        const int b = e->bin[sorted[(size_t)i]];
        if (b != last_b) {
          if (b == tp.bin0) first_rank[(size_t)t] = cover[b];
          cover[b]++;
          last_b = b;
        }
      }
    }
    for (int b = 0; b < B; ++b) bin_slot[b + 1] = bin_slot[b] + cover[b];
    for (int64_t t = 0; t < T_; ++t) tile_slot0[(size_t)t] = bin_slot[tiles[(size_t)t].bin0] + first_rank[(size_t)t];
    if ((int64_t)bin_slot[B] != bin_slot[B]) return fail(e, GW_ERR_LIMIT, "too many slots");
  }
  e->n_slots = bin_slot[B];

  // 6. pack tiles (parallel over tiles)
  std::vector<TileDesc> tdesc((size_t)T_);
  std::vector<uint64_t> hdr((size_t)hdr_total, 0);
  // the lanes kernel walks a tile's dials event by event: it bulk-copies the
  // headers in slot order (engines of more than one point)
  std::vector<uint64_t> hdr_ev(e->cfg.k_max > 1 ? (size_t)hdr_total : 0, 0);
  std::vector<unsigned char> payload((size_t)payload_total, 0);
  std::vector<uint16_t> evinfo((size_t)N);
  std::vector<uint16_t> evcost((size_t)N);
  std::vector<T> w0((size_t)N);
  {
    const int nth = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    std::vector<std::thread> th;
    for (int t = 0; t < nth; ++t) {
      th.emplace_back([&, t]() {
        std::vector<int64_t> ev_major;  // dial ids in event-major order
        std::vector<int32_t> order;
        for (int64_t ti = t; ti < T_; ti += nth) {
          const TilePlan& tp = tiles[(size_t)ti];
          auto htype = [&](int64_t di) {
            return (!grid_of.empty() && grid_of[(size_t)di] >= 0) ? (int)kGrid : (int)e->dials[(size_t)di].type;
          };
          ev_major.clear();
          int cost = 0;
          for (int64_t i = tp.ev_begin; i < tp.ev_end; ++i) {
            const int r = sorted[(size_t)i];
            evinfo[(size_t)i] = make_evinfo((int)ev_major.size(), e->bin[r] - tp.bin0);
            w0[(size_t)i] = (T)e->initial[r];
            cost += kEventCost;
            for (int64_t j = rstart[r]; j < rstart[r + 1]; ++j) {
              const int64_t di = byres[(size_t)j];
              ev_major.push_back(di);
              cost += dial_cost(htype(di), pn[(size_t)di]);
            }
            evcost[(size_t)i] = (uint16_t)cost;
          }
          const int nd = (int)ev_major.size();
          order.resize(nd);
          for (int s = 0; s < nd; ++s) order[s] = s;
          // type order; in the coefficient form the three uniform-knot spline
          // types first, so their 16-byte-multiple payloads start 16-byte aligned
          auto key = [&](int a) {
            const int ty = htype(ev_major[a]);
            const bool first = dial_form == kFormCoefs &&
                               (ty == kMonotonic || ty == kCompact || ty == kUniform || ty == kGrid);
            return (first ? 0 : 16) + ty;
          };
          std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return key(a) < key(b); });
          T* pl = (T*)(payload.data() + tp.payload_off);
          int off = 0;
          for (int j = 0; j < nd; ++j) {
            const int slot = order[j];
            const int64_t di = ev_major[slot];
            const DialRec& r = e->dials[(size_t)di];
            const int g = grid_of.empty() ? -1 : grid_of[(size_t)di];
            const int p0 = g >= 0 ? g : r.type >= kTabulated ? (int)e->dial_data[(size_t)r.data_off] : r.p0;
            const int p1 = r.p1 >= 0 ? r.p1 : 0;
            hdr[(size_t)(tp.dial0 + j)] = make_header(g >= 0 ? (int)kGrid : (int)r.type, pn[(size_t)di], slot, off,
                                                      p0, p1);
            if (!hdr_ev.empty()) hdr_ev[(size_t)(tp.dial0 + slot)] = hdr[(size_t)(tp.dial0 + j)];
            if (r.type == kMonotonic || r.type == kCompact || r.type == kUniform)
              write_prepared<T>(r, e->dial_data.data() + r.data_off, pn[(size_t)di], pl + off,
                                g >= 0 ? kFormGrid : dial_form);
            else
              write_payload<T>(r, e->dial_data.data() + r.data_off, pl + off);
            off += pel[(size_t)di];
          }
          TileDesc& d = tdesc[(size_t)ti];
          d.payload_off = tp.payload_off;
          d.dial0 = (uint32_t)tp.dial0;
          d.event0 = (uint32_t)tp.ev_begin;
          d.bin0 = (uint32_t)tp.bin0;
          d.slot0 = (uint32_t)tile_slot0[(size_t)ti];
          d.ndials = (uint16_t)nd;
          d.nevents = (uint16_t)(tp.ev_end - tp.ev_begin);
          d.payload_16b = (uint16_t)((tp.payload_elems * tsz + 15) / 16);
          d.nbins = (uint16_t)tp.nbins;
        }
      });
    }
    for (auto& x : th) x.join();
  }

  // 7. device upload
  {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
      cudaGetLastError();
      return fail(e, GW_ERR_CUDA, "no CUDA device available");
    }
    if (e->device >= ndev) return fail(e, GW_ERR_ARG, "bad device %d (%d present)", e->device, ndev);
  }
  GW_CUDA(e, cudaSetDevice(e->device));
  GW_CUDA(e, cudaDeviceGetAttribute(&e->num_sms, cudaDevAttrMultiProcessorCount, e->device));
  GW_CUDA(e, cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking));
  GW_CUDA(e, cudaEventCreateWithFlags(&e->chain_done, cudaEventDisableTiming));
  e->kpad = ((e->cfg.k_max + 63) / 64) * 64;  // a batched pass covers up to 64 points
  const int P = e->cfg.n_params;
  const int kpad = e->kpad;

  auto alloc = [&](size_t bytes, void** p) -> int {
    const size_t n = bytes ? bytes : 16;
    void* q = nullptr;
    if (cudaMalloc(&q, n) != cudaSuccess) {
      cudaGetLastError();
      return fail(e, GW_ERR_NOMEM, "cudaMalloc of %zu bytes failed", n);
    }
    e->dev_allocs.push_back(q);
    e->resident += (int64_t)n;
    *p = q;
    return GW_OK;
  };
  auto upload = [&](const void* src, size_t bytes, void** dst) -> int {
    int rc = alloc(bytes, dst);
    if (rc) return rc;
    if (bytes) GW_CUDA(e, cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice));
    return GW_OK;
  };
  int rc;
  void* p;
  DevView& v = e->view;
  v = DevView{};
  v.precision = e->cfg.precision;
  v.n_params = P;
  v.n_bins = B;
  v.n_events = N;
  v.n_tiles = (int)T_;
  v.kpad = kpad;
  v.llh_type = e->llh_type;
  v.has_prior = e->has_prior ? 1 : 0;
  v.has_cap = e->has_cap ? 1 : 0;
  v.cap = e->cap;
  v.tile_payload_bytes = (int)(((cap_elems * tsz) + 127) & ~(int64_t)127);
  v.tile_hdr_bytes = std::max(16, ((max_tile_dials + 1) / 2) * 16);
  v.spline_knots = dial_form == kFormKnots ? 1 : 0;
  v.spline_coefs = dial_form == kFormCoefs ? 1 : 0;

  // slack after the per-dial and per-event arrays (reads rounded out to
  // 16-byte boundaries stay inside the allocation)
  hdr.resize(hdr.size() + 2, 0);
  evinfo.resize(evinfo.size() + 8, 0);
  w0.resize(w0.size() + 4, T(0));
  if ((rc = upload(tdesc.data(), tdesc.size() * sizeof(TileDesc), &p))) return rc;
  v.tiles = (const TileDesc*)p;
  if ((rc = upload(hdr.data(), hdr.size() * sizeof(uint64_t), &p))) return rc;
  v.hdr = (const uint64_t*)p;
  if (!hdr_ev.empty()) {
    hdr_ev.resize(hdr_ev.size() + 2, 0);
    if ((rc = upload(hdr_ev.data(), hdr_ev.size() * sizeof(uint64_t), &p))) return rc;
    v.hdr_ev = (const uint64_t*)p;
  }
  if ((rc = upload(payload.data(), payload.size(), &p))) return rc;
  v.payload = (const unsigned char*)p;
  if ((rc = upload(evinfo.data(), evinfo.size() * sizeof(uint16_t), &p))) return rc;
  v.evinfo = (const uint16_t*)p;
  evcost.resize(evcost.size() + 8, 0);
  if ((rc = upload(evcost.data(), evcost.size() * sizeof(uint16_t), &p))) return rc;
  v.evcost = (const uint16_t*)p;
  if ((rc = upload(w0.data(), w0.size() * sizeof(T), &p))) return rc;
  v.w0 = p;
  if ((rc = upload(bin_slot.data(), bin_slot.size() * sizeof(int32_t), &p))) return rc;
  v.bin_slot = (const int32_t*)p;
  {
    std::vector<T> pc(2 * (size_t)P);
    for (int i = 0; i < P; ++i) {
      // FP32 mode: +-DBL_MAX defaults become +-FLT_MAX
      double lo = e->clamp_lo[i], hi = e->clamp_hi[i];
      if (tsz == 4) {
        lo = std::max(lo, -(double)FLT_MAX);
        hi = std::min(hi, (double)FLT_MAX);
      }
      pc[2 * i] = (T)lo;
      pc[2 * i + 1] = (T)hi;
    }
    if ((rc = upload(pc.data(), pc.size() * sizeof(T), &p))) return rc;
    v.pclamp = p;
  }
  if ((rc = upload(e->pflags.data(), e->pflags.size(), &p))) return rc;
  v.pflags = (const uint8_t*)p;
  if ((rc = upload(e->mirror_lo.data(), sizeof(double) * P, &p))) return rc;
  v.mirror_lo = (const double*)p;
  if ((rc = upload(e->mirror_hi.data(), sizeof(double) * P, &p))) return rc;
  v.mirror_hi = (const double*)p;
  if (e->has_prior) {
    if ((rc = upload(e->prior_mean.data(), sizeof(double) * P, &p))) return rc;
    v.prior_mean = (const double*)p;
    if ((rc = upload(e->prior_icov.data(), sizeof(double) * (size_t)P * P, &p))) return rc;
    v.prior_icov = (const double*)p;
  }
  if (!e->eigen.empty()) {
    std::vector<int32_t> f, n;
    std::vector<int64_t> off;
    std::vector<double> Vs;
    for (const auto& b : e->eigen) {
      f.push_back(b.first);
      n.push_back(b.n);
      off.push_back((int64_t)Vs.size());
      Vs.insert(Vs.end(), b.V.begin(), b.V.end());
    }
    v.n_eigen = (int)e->eigen.size();
    if ((rc = upload(f.data(), sizeof(int32_t) * f.size(), &p))) return rc;
    v.eig_first = (const int32_t*)p;
    if ((rc = upload(n.data(), sizeof(int32_t) * n.size(), &p))) return rc;
    v.eig_n = (const int32_t*)p;
    if ((rc = upload(off.data(), sizeof(int64_t) * off.size(), &p))) return rc;
    v.eig_off = (const int64_t*)p;
    if ((rc = upload(Vs.data(), sizeof(double) * Vs.size(), &p))) return rc;
    v.eig_V = (const double*)p;
  }
  if ((rc = upload(e->data.data(), sizeof(double) * B, &p))) return rc;
  v.data = (const double*)p;
  // tables
  {
    std::vector<TableDesc> td(e->tables.size());
    std::vector<TableFn> fns;
    std::vector<double> nodes;
    int64_t arena = 0;
    for (size_t i = 0; i < e->tables.size(); ++i) {
      const HostTable& h = e->tables[i];
      td[i].offset = arena;
      td[i].size = h.size;
      td[i].per_k = h.has_fn ? 1 : 0;
      td[i].lower = h.lower;
      td[i].upper = h.upper;
      if (tsz == 4) {
        td[i].lower = std::max(td[i].lower, -(double)FLT_MAX);
        td[i].upper = std::min(td[i].upper, (double)FLT_MAX);
      }
      arena += h.has_fn ? (int64_t)h.size * kpad : h.size;
      if (h.has_fn) {
        TableFn f{};
        f.table = (int32_t)i;
        f.kind = h.fn_kind;
        std::memcpy(f.par, h.fn_par, sizeof(f.par));
        f.nodes = (int64_t)nodes.size();
        nodes.insert(nodes.end(), h.nodes.begin(), h.nodes.end());
        fns.push_back(f);
        e->max_fn_table = std::max(e->max_fn_table, h.size);
      }
    }
    if ((rc = upload(td.data(), td.size() * sizeof(TableDesc), &p))) return rc;
    v.tables = (const TableDesc*)p;
    if ((rc = upload(fns.data(), fns.size() * sizeof(TableFn), &p))) return rc;
    v.table_fns = (const TableFn*)p;
    if ((rc = upload(nodes.data(), nodes.size() * sizeof(double), &p))) return rc;
    v.table_nodes = (const double*)p;
    if ((rc = alloc((size_t)arena * tsz, &p))) return rc;
    v.table_arena = p;
    v.n_tables = (int)td.size();
    v.n_table_fns = (int)fns.size();
    for (HostTable& h : e->tables) h.dirty = !h.has_fn;
  }
  // knot grids of the grid form, their response clamps (the parameter's,
  // intersected with [-1e20, 1e20] in the engine precision, as the kernels do
  // for the other dials) and the per-point intervals k_params forms
  v.n_grids = (int)grids.size();
  if (!grids.empty()) {
    if ((rc = upload(grids.data(), grids.size() * sizeof(GridDesc), &p))) return rc;
    v.grids = (const GridDesc*)p;
    std::vector<T> gc(2 * grids.size());
    for (size_t g = 0; g < grids.size(); ++g) {
      const int q = grids[g].p0;
      double lo = e->clamp_lo[(size_t)q], hi = e->clamp_hi[(size_t)q];
      if (tsz == 4) {
        lo = std::max(lo, -(double)FLT_MAX);
        hi = std::min(hi, (double)FLT_MAX);
      }
      // the conversion to T is monotone, so clamping before it equals
      // clamping after it
      gc[2 * g] = (T)std::max(lo, -1e20);
      gc[2 * g + 1] = (T)std::min(hi, 1e20);
    }
    if ((rc = upload(gc.data(), gc.size() * sizeof(T), &p))) return rc;
    v.grid_clamp = p;
    if ((rc = alloc(grids.size() * (size_t)kpad * sizeof(GridPoint<T>), &p))) return rc;
    GW_CUDA(e, cudaMemset(p, 0, grids.size() * (size_t)kpad * sizeof(GridPoint<T>)));
    v.grid_pts = p;
  }
  e->sorted_to_result = sorted;
  if ((rc = upload(sorted.data(), sorted.size() * sizeof(int32_t), &p))) return rc;
  v.sorted_to_result = (const int32_t*)p;
  if ((rc = alloc((size_t)P * kpad * tsz, &p))) return rc;
  GW_CUDA(e, cudaMemset(p, 0, (size_t)P * kpad * tsz));
  v.x = p;
  if ((rc = alloc(sizeof(double) * kpad, &p))) return rc;
  GW_CUDA(e, cudaMemset(p, 0, sizeof(double) * kpad));
  v.penalty = (double*)p;
  if ((rc = alloc(sizeof(double2) * (size_t)std::max(e->n_slots, 1) * kpad, &p))) return rc;
  v.partials = (double2*)p;
  v.llh_nblk = (B + 255) / 256;
  if ((rc = alloc(sizeof(double) * (size_t)kpad * v.llh_nblk, &p))) return rc;
  v.llh_blocks = (double*)p;
  if ((rc = alloc(sizeof(unsigned int) * kpad, &p))) return rc;
  GW_CUDA(e, cudaMemset(p, 0, sizeof(unsigned int) * kpad));
  v.llh_counter = (unsigned int*)p;
  if ((rc = alloc(sizeof(uint32_t), &p))) return rc;
  GW_CUDA(e, cudaMemset(p, 0, sizeof(uint32_t)));
  v.status = (uint32_t*)p;
  // evaluation I/O buffers
  if ((rc = alloc(sizeof(double) * (size_t)kpad * P, &e->d_params))) return rc;
  if ((rc = alloc(sizeof(double) * (size_t)kpad * B, &e->d_sums))) return rc;
  if ((rc = alloc(sizeof(double) * (size_t)kpad * B, &e->d_sums2))) return rc;
  if ((rc = alloc(sizeof(double) * (size_t)kpad, &e->d_llh))) return rc;
  if ((rc = alloc(sizeof(double) * (size_t)kpad, &e->d_llh_stat))) return rc;
  GW_CUDA(e, cudaMallocHost(&e->h_params.p, sizeof(double) * (size_t)kpad * P));
  GW_CUDA(e, cudaMallocHost(&e->h_sums.p, sizeof(double) * (size_t)kpad * B));
  GW_CUDA(e, cudaMallocHost(&e->h_sums2.p, sizeof(double) * (size_t)kpad * B));
  GW_CUDA(e, cudaMallocHost(&e->h_llh.p, sizeof(double) * (size_t)kpad));
  GW_CUDA(e, cudaMallocHost(&e->h_llh_stat.p, sizeof(double) * (size_t)kpad));
  GW_CUDA(e, cudaMallocHost(&e->h_status.p, sizeof(uint32_t)));

  // layout facts
  gw_layout_info& L = e->layout;
  L = gw_layout_info{};
  L.n_tiles = T_;
  L.n_dials = D;
  L.payload_bytes = (int64_t)payload_total;
  L.header_bytes = D * 8;
  L.event_bytes = (int64_t)N * (2 + (int64_t)tsz);
  L.partial_slots = e->n_slots;
  for (const DialRec& r : e->dials) L.dials_by_type[r.type]++;

  GW_CUDA(e, prepare_params(v));
  // grids; the warp-specialised K = 1 kernel is the default (measured faster
  // on every configuration; gw_autotune(e, 1) re-checks)
  v.plain_kind = 1;
  int bps = plain_blocks_per_sm(v);
  if (bps < 1) {
    v.plain_kind = 0;
    bps = plain_blocks_per_sm(v);
  }
  if (bps < 1) return fail(e, GW_ERR_CUDA, "plain kernel does not fit on an SM");
  e->plain_grid = (int)std::max<int64_t>(1, std::min<int64_t>(T_, (int64_t)bps * e->num_sms));
  const int K0 = e->cfg.k_max;
  if (e->cfg.precision == GW_DF64)  // compiled for a subset of the shapes (gw_lanes.cu, gw_ws.cu)
    e->shape = K0 >= 8 ? BatchedShape{0, 32, 1, 256, 1, 0} : BatchedShape{3, 2, 2, 256, 2, 2};
  else if (K0 >= 8)
    e->shape = BatchedShape{1, 8, 4, 256, 1, 0};
  else
    e->shape = BatchedShape{1, 4, 2, 256, 2, 0};
  const int bb = batched_blocks_per_sm(v, e->shape);
  if (bb < 1) return fail(e, GW_ERR_CUDA, "batched kernel does not fit on an SM");
  e->batched_grid = (int)std::max<int64_t>(1, std::min<int64_t>(T_, (int64_t)bb * e->num_sms));
  GW_CUDA(e, cudaDeviceSynchronize());
  return GW_OK;
}

}  // namespace

extern "C" int gw_initialize(gw_engine* e) {
  GW_REQUIRE_BUILDER(e);
  int rc;
  try {
    rc = e->cfg.precision == GW_FP32   ? build_and_upload<float>(e)
         : e->cfg.precision == GW_DF64 ? build_and_upload<dfloat>(e)
                                       : build_and_upload<double>(e);
  } catch (const std::bad_alloc&) {
    rc = fail(e, GW_ERR_NOMEM, "host allocation failed while packing");
  }
  if (rc == GW_OK) {
    e->initialized = true;
    // the builder's host copies are no longer needed
    std::vector<DialRec>().swap(e->dials);
    std::vector<double>().swap(e->dial_data);
  }
  return rc;
}

// ---------------------------------------------------------------------------
// evaluation
// ---------------------------------------------------------------------------
static int refresh_tables(gw_engine* e) {
  const size_t tsz = e->cfg.precision == GW_FP32 ? 4 : 8;
  // table offsets are recomputed in creation order (same as the upload)
  int64_t off = 0;
  bool copied = false;
  for (HostTable& h : e->tables) {
    if (!h.has_fn && h.dirty) {
      if (!copied) {
        const int rc = chain_begin(e, e->stream);  // a chain on another stream may still read the table
        if (rc) return rc;
      }
      unsigned char* dst = (unsigned char*)e->view.table_arena + off * tsz;
      if (e->cfg.precision == GW_FP64) {
        GW_CUDA(e, cudaMemcpyAsync(dst, h.values.data(), sizeof(double) * h.size, cudaMemcpyHostToDevice,
                                   e->stream));
      } else if (e->cfg.precision == GW_DF64) {
        std::vector<dfloat> f(h.size);
        for (int64_t i = 0; i < (int64_t)h.size; ++i) f[i] = dfloat(h.values[i]);
        GW_CUDA(e, cudaMemcpyAsync(dst, f.data(), sizeof(dfloat) * h.size, cudaMemcpyHostToDevice, e->stream));
        GW_CUDA(e, cudaStreamSynchronize(e->stream));
      } else {
        std::vector<float> f(h.values.begin(), h.values.end());
        GW_CUDA(e, cudaMemcpyAsync(dst, f.data(), sizeof(float) * h.size, cudaMemcpyHostToDevice, e->stream));
        GW_CUDA(e, cudaStreamSynchronize(e->stream));
      }
      h.dirty = false;
      copied = true;
    }
    off += h.has_fn ? (int64_t)h.size * e->kpad : h.size;
  }
  // a launch on another stream must see the new tables
  if (copied) GW_CUDA(e, cudaStreamSynchronize(e->stream));
  return GW_OK;
}

static int launch_chain(gw_engine* e, const double* d_params, int K, double* d_sums, double* d_sums2, double* d_llh,
                        double* d_llh_stat, cudaStream_t s) {
  DevView v = e->view;
  v.event_weights = (e->copy_weights && K == 1) ? (double*)e->d_evw : nullptr;
  GW_CUDA(e, launch_params(v, d_params, K, s));
  if (v.n_table_fns) GW_CUDA(e, launch_table_fns(v, K, e->max_fn_table, s));
  cudaEvent_t ev_end = nullptr;
  if (e->profiling) {
    if (e->prof_used == e->prof_events.size()) {
      cudaEvent_t a, b;
      GW_CUDA(e, cudaEventCreate(&a));
      GW_CUDA(e, cudaEventCreate(&b));
      e->prof_events.emplace_back(a, b);
    }
    GW_CUDA(e, cudaEventRecord(e->prof_events[e->prof_used].first, s));
    ev_end = e->prof_events[e->prof_used].second;
    e->prof_used++;
  }
  if (K == 1) {
    GW_CUDA(e, launch_plain(v, e->plain_grid, s));
  } else {
    if (!batched_shape_covers(v, e->shape, K))
      return fail(e, GW_ERR_ARG, "the selected batched shape (%d points per pass) does not cover K = %d within "
                  "the engine's %d padded point columns; select another shape or autotune for this K",
                  e->shape.kind == 0 ? e->shape.kc * e->shape.kr : e->shape.kc, K, v.kpad);
    GW_CUDA(e, launch_batched(v, K, e->shape, e->batched_grid, s));
  }
  if (ev_end) GW_CUDA(e, cudaEventRecord(ev_end, s));
  GW_CUDA(e, launch_bins_llh(v, K, d_sums, d_sums2, d_llh, d_llh_stat, s));
  e->kernel_launches += 3 + (v.n_table_fns ? 1 : 0);
  return GW_OK;
}

static int check_status(gw_engine* e) {
  GW_CUDA(e, cudaMemcpyAsync(e->h_status.p, e->view.status, sizeof(uint32_t), cudaMemcpyDeviceToHost, e->stream));
  GW_CUDA(e, cudaStreamSynchronize(e->stream));
  const uint32_t st = *(uint32_t*)e->h_status.p;
  if (st) {
    GW_CUDA(e, cudaMemsetAsync(e->view.status, 0, sizeof(uint32_t), e->stream));
    GW_CUDA(e, cudaStreamSynchronize(e->stream));
    return fail(e, GW_ERR_DEVICE_TIMEOUT, "device status 0x%x: a bounded wait for a tile copy gave up", st);
  }
  return GW_OK;
}

extern "C" int gw_eval(gw_engine* e, const double* params, int32_t K, double* sums, double* sums2, double* llh,
                       double* llh_stat) {
  if (!e || !params) return GW_ERR_ARG;
  if (!e->initialized) return fail(e, GW_ERR_STATE, "gw_initialize has not been called");
  if (K < 1 || K > e->cfg.k_max) return fail(e, GW_ERR_ARG, "K=%d outside [1, %d]", K, e->cfg.k_max);
  const int P = e->cfg.n_params, B = e->cfg.n_bins;
  GW_CUDA(e, cudaSetDevice(e->device));
  int rc = refresh_tables(e);
  if (rc) return rc;
  std::memcpy(e->h_params.p, params, sizeof(double) * (size_t)K * P);
  cudaStream_t s = e->stream;
  auto run = [&]() -> int {
    GW_CUDA(e, cudaMemcpyAsync(e->d_params, e->h_params.p, sizeof(double) * (size_t)K * P,
                               cudaMemcpyHostToDevice, s));
    int r = launch_chain(e, (const double*)e->d_params, K, (double*)e->d_sums, (double*)e->d_sums2,
                         (double*)e->d_llh, (double*)e->d_llh_stat, s);
    if (r) return r;
    GW_CUDA(e, cudaMemcpyAsync(e->h_sums.p, e->d_sums, sizeof(double) * (size_t)K * B, cudaMemcpyDeviceToHost, s));
    GW_CUDA(e, cudaMemcpyAsync(e->h_sums2.p, e->d_sums2, sizeof(double) * (size_t)K * B, cudaMemcpyDeviceToHost,
                               s));
    GW_CUDA(e, cudaMemcpyAsync(e->h_llh.p, e->d_llh, sizeof(double) * (size_t)K, cudaMemcpyDeviceToHost, s));
    GW_CUDA(e, cudaMemcpyAsync(e->h_llh_stat.p, e->d_llh_stat, sizeof(double) * (size_t)K, cudaMemcpyDeviceToHost,
                               s));
    return GW_OK;
  };
  rc = chain_begin(e, s);
  if (rc) return rc;
  if (e->use_graph) {
    auto it = e->graphs.find(K);
    if (it == e->graphs.end()) {
      GW_CUDA(e, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
      int r = run();
      cudaGraph_t g = nullptr;
      cudaError_t ce = cudaStreamEndCapture(s, &g);
      if (r) {
        if (g) cudaGraphDestroy(g);
        return r;
      }
      if (ce != cudaSuccess) return fail(e, GW_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(ce));
      cudaGraphExec_t ex = nullptr;
      ce = cudaGraphInstantiate(&ex, g, 0);
      cudaGraphDestroy(g);
      if (ce != cudaSuccess) return fail(e, GW_ERR_CUDA, "graph instantiate failed: %s", cudaGetErrorString(ce));
      it = e->graphs.emplace(K, ex).first;
    }
    GW_CUDA(e, cudaGraphLaunch(it->second, s));
  } else {
    rc = run();
    if (rc) return rc;
  }
  rc = chain_end(e, s);
  if (rc) return rc;
  rc = check_status(e);  // synchronizes the stream
  if (rc) return rc;
  if (sums) std::memcpy(sums, e->h_sums.p, sizeof(double) * (size_t)K * B);
  if (sums2) std::memcpy(sums2, e->h_sums2.p, sizeof(double) * (size_t)K * B);
  if (llh) std::memcpy(llh, e->h_llh.p, sizeof(double) * (size_t)K);
  if (llh_stat) std::memcpy(llh_stat, e->h_llh_stat.p, sizeof(double) * (size_t)K);
  e->weights_valid = e->copy_weights && K == 1;
  return GW_OK;
}

extern "C" int gw_eval_device(gw_engine* e, const double* d_params, int32_t K, double* d_sums, double* d_sums2,
                              double* d_llh, double* d_llh_stat, void* stream) {
  if (!e || !d_params) return GW_ERR_ARG;
  if (!e->initialized) return fail(e, GW_ERR_STATE, "gw_initialize has not been called");
  if (K < 1 || K > e->cfg.k_max) return fail(e, GW_ERR_ARG, "K=%d outside [1, %d]", K, e->cfg.k_max);
  GW_CUDA(e, cudaSetDevice(e->device));
  int rc = refresh_tables(e);
  if (rc) return rc;
  cudaStream_t s = stream ? (cudaStream_t)stream : e->stream;
  rc = chain_begin(e, s);
  if (rc) return rc;
  if (e->use_graph) {
    // the launch chain captured once per (K, pointers, stream) and replayed
    const std::vector<uintptr_t> key = {(uintptr_t)K,       (uintptr_t)d_params, (uintptr_t)d_sums,
                                        (uintptr_t)d_sums2, (uintptr_t)d_llh,    (uintptr_t)d_llh_stat,
                                        (uintptr_t)s};
    auto it = e->dev_graphs.find(key);
    if (it == e->dev_graphs.end()) {
      GW_CUDA(e, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
      const int r = launch_chain(e, d_params, K, d_sums, d_sums2, d_llh, d_llh_stat, s);
      cudaGraph_t g = nullptr;
      const cudaError_t ce = cudaStreamEndCapture(s, &g);
      if (r) {
        if (g) cudaGraphDestroy(g);
        return r;
      }
      if (ce != cudaSuccess) return fail(e, GW_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(ce));
      cudaGraphExec_t ex = nullptr;
      const cudaError_t ie = cudaGraphInstantiate(&ex, g, 0);
      cudaGraphDestroy(g);
      if (ie != cudaSuccess) return fail(e, GW_ERR_CUDA, "graph instantiate failed: %s", cudaGetErrorString(ie));
      it = e->dev_graphs.emplace(key, ex).first;
    }
    GW_CUDA(e, cudaGraphLaunch(it->second, s));
  } else {
    rc = launch_chain(e, d_params, K, d_sums, d_sums2, d_llh, d_llh_stat, s);
  }
  if (rc == GW_OK) rc = chain_end(e, s);
  if (rc == GW_OK) e->weights_valid = e->copy_weights && K == 1;
  return rc;
}

extern "C" int gw_sync(gw_engine* e) {
  if (!e) return GW_ERR_ARG;
  if (!e->initialized) return GW_OK;
  GW_CUDA(e, cudaSetDevice(e->device));
  GW_CUDA(e, cudaDeviceSynchronize());
  return check_status(e);
}

extern "C" int gw_use_graph(gw_engine* e, int32_t on) {
  if (!e) return GW_ERR_ARG;
  e->use_graph = on != 0;
  return GW_OK;
}

// K = 1: times both K = 1 kernels and keeps the faster.
static int autotune_plain(gw_engine* e) {
  GW_CUDA(e, cudaDeviceSynchronize());  // every earlier chain, whichever stream
  std::vector<double> pts((size_t)e->cfg.n_params);
  for (size_t i = 0; i < pts.size(); ++i) pts[i] = 0.001 * (double)((i * 7919) % 17) - 0.008;
  GW_CUDA(e, cudaMemcpy(e->d_params, pts.data(), sizeof(double) * pts.size(), cudaMemcpyHostToDevice));
  cudaEvent_t a, b;
  GW_CUDA(e, cudaEventCreate(&a));
  GW_CUDA(e, cudaEventCreate(&b));
  float best = 1e30f;
  int best_kind = e->view.plain_kind;
  for (int kind = 0; kind < 3; ++kind) {
    if (gw_set_plain_kernel(e, kind) != GW_OK) continue;
    int rc = launch_chain(e, (const double*)e->d_params, 1, (double*)e->d_sums, (double*)e->d_sums2,
                          (double*)e->d_llh, (double*)e->d_llh_stat, e->stream);
    if (rc) return rc;
    GW_CUDA(e, cudaEventRecord(a, e->stream));
    for (int rep = 0; rep < 5; ++rep) {
      rc = launch_chain(e, (const double*)e->d_params, 1, (double*)e->d_sums, (double*)e->d_sums2,
                        (double*)e->d_llh, (double*)e->d_llh_stat, e->stream);
      if (rc) return rc;
    }
    GW_CUDA(e, cudaEventRecord(b, e->stream));
    GW_CUDA(e, cudaEventSynchronize(b));
    float ms = 0;
    GW_CUDA(e, cudaEventElapsedTime(&ms, a, b));
    if (ms < best) {
      best = ms;
      best_kind = kind;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  int rc = gw_set_plain_kernel(e, best_kind);
  if (rc) return rc;
  return check_status(e);
}

extern "C" int gw_autotune(gw_engine* e, int32_t K) {
  if (!e) return GW_ERR_ARG;
  if (!e->initialized) return fail(e, GW_ERR_STATE, "gw_initialize has not been called");
  if (K == 1) {
    GW_CUDA(e, cudaSetDevice(e->device));
    return autotune_plain(e);
  }
  if (K < 1 || K > e->cfg.k_max) return fail(e, GW_ERR_ARG, "autotune needs 1 <= K <= k_max");
  GW_CUDA(e, cudaSetDevice(e->device));
  GW_CUDA(e, cudaDeviceSynchronize());  // every earlier chain, whichever stream
  // deterministic synthetic points: all parameters at 0 except tiny offsets
  std::vector<double> pts((size_t)K * e->cfg.n_params);
  for (size_t i = 0; i < pts.size(); ++i) pts[i] = 0.001 * (double)((i * 7919) % 17) - 0.008;
  GW_CUDA(e, cudaMemcpy(e->d_params, pts.data(), sizeof(double) * pts.size(), cudaMemcpyHostToDevice));
  cudaEvent_t a, b_ev;
  GW_CUDA(e, cudaEventCreate(&a));
  GW_CUDA(e, cudaEventCreate(&b_ev));
  float best = 1e30f;
  BatchedShape best_shape = e->shape;
  int best_grid = e->batched_grid;
  for (int i = 0; i < batched_shape_count(); ++i) {
    const BatchedShape b = batched_shape(i);
    if (b.kind == 0) {
      if (b.kc > 8 && b.kc / 2 >= K) continue;  // lanes beyond K would idle
      if (b.kc * b.kr > 2 * ((K + 31) / 32) * 32) continue;
    } else if (b.kc > 2 * K) {
      continue;
    }
    if (!batched_shape_covers(e->view, b, K)) continue;
    const int bps = batched_blocks_per_sm(e->view, b);
    if (bps < 1) continue;
    e->shape = b;
    e->batched_grid = (int)std::max<int64_t>(1, std::min<int64_t>(e->view.n_tiles, (int64_t)bps * e->num_sms));
    int rc = launch_chain(e, (const double*)e->d_params, K, (double*)e->d_sums, (double*)e->d_sums2,
                          (double*)e->d_llh, (double*)e->d_llh_stat, e->stream);
    if (rc) return rc;
    GW_CUDA(e, cudaEventRecord(a, e->stream));
    for (int rep = 0; rep < 3; ++rep) {
      rc = launch_chain(e, (const double*)e->d_params, K, (double*)e->d_sums, (double*)e->d_sums2,
                        (double*)e->d_llh, (double*)e->d_llh_stat, e->stream);
      if (rc) return rc;
    }
    GW_CUDA(e, cudaEventRecord(b_ev, e->stream));
    GW_CUDA(e, cudaEventSynchronize(b_ev));
    float ms = 0;
    GW_CUDA(e, cudaEventElapsedTime(&ms, a, b_ev));
    if (ms < best) {
      best = ms;
      best_shape = b;
      best_grid = e->batched_grid;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b_ev);
  e->shape = best_shape;
  e->batched_grid = best_grid;
  e->tuned = true;
  e->clear_graphs();
  return check_status(e);
}

extern "C" int gw_set_shape(gw_engine* e, int32_t kind, int32_t kc, int32_t threads, int32_t stages) {
  if (!e) return GW_ERR_ARG;
  if (!e->initialized) return fail(e, GW_ERR_STATE, "gw_initialize has not been called");
  for (int i = 0; i < batched_shape_count(); ++i) {
    const BatchedShape b = batched_shape(i);
    const int per_pass = b.kind == 0 ? b.kc * b.kr : b.kc;
    if (b.kind == kind && per_pass == kc && b.threads == threads && b.stages == stages)
      return gw_set_shape_index(e, i);
  }
  return fail(e, GW_ERR_ARG, "no compiled shape (%d, %d, %d, %d)", kind, kc, threads, stages);
}

extern "C" int gw_set_shape_index(gw_engine* e, int32_t i) {
  if (!e) return GW_ERR_ARG;
  if (!e->initialized) return fail(e, GW_ERR_STATE, "gw_initialize has not been called");
  if (i < 0 || i >= batched_shape_count()) return fail(e, GW_ERR_ARG, "shape index %d out of range", i);
  GW_CUDA(e, cudaSetDevice(e->device));
  const BatchedShape b = batched_shape(i);
  const int bps = batched_blocks_per_sm(e->view, b);
  if (bps < 1) return fail(e, GW_ERR_ARG, "shape %d does not fit on an SM", i);
  e->shape = b;
  e->batched_grid = (int)std::max<int64_t>(1, std::min<int64_t>(e->view.n_tiles, (int64_t)bps * e->num_sms));
  e->clear_graphs();
  return GW_OK;
}

extern "C" int gw_get_shape_index(const gw_engine* e, int32_t* i) {
  if (!e || !i) return GW_ERR_ARG;
  *i = -1;
  for (int j = 0; j < batched_shape_count(); ++j) {
    const BatchedShape b = batched_shape(j);
    if (b.kind == e->shape.kind && b.kc == e->shape.kc && b.kr == e->shape.kr && b.threads == e->shape.threads &&
        b.stages == e->shape.stages && b.minb == e->shape.minb) {
      *i = j;
      break;
    }
  }
  return GW_OK;
}

extern "C" int gw_shape_count(void) { return batched_shape_count(); }

extern "C" int gw_shape_at(int32_t i, int32_t* kind, int32_t* kc, int32_t* kr, int32_t* threads, int32_t* stages,
                           int32_t* min_blocks) {
  if (i < 0 || i >= batched_shape_count() || !kind || !kc || !kr || !threads || !stages || !min_blocks)
    return GW_ERR_ARG;
  const BatchedShape b = batched_shape(i);
  *kind = b.kind;
  *kc = b.kind == 0 ? b.kc * b.kr : b.kc;
  *kr = b.kr;
  *threads = b.threads;
  *stages = b.stages;
  *min_blocks = b.minb;
  return GW_OK;
}

extern "C" int gw_set_plain_kernel(gw_engine* e, int32_t kind) {
  if (!e || kind < 0 || kind > 2) return GW_ERR_ARG;
  if (!e->initialized) return fail(e, GW_ERR_STATE, "gw_initialize has not been called");
  GW_CUDA(e, cudaSetDevice(e->device));
  const int old = e->view.plain_kind;
  e->view.plain_kind = kind;
  const int bps = plain_blocks_per_sm(e->view);
  if (bps < 1) {
    e->view.plain_kind = old;
    return fail(e, GW_ERR_ARG, "K = 1 kernel %d does not fit on an SM", kind);
  }
  e->plain_grid = (int)std::max<int64_t>(1, std::min<int64_t>(e->view.n_tiles, (int64_t)bps * e->num_sms));
  e->clear_graphs();
  return GW_OK;
}

extern "C" int gw_get_plain_kernel(const gw_engine* e, int32_t* kind) {
  if (!e || !kind) return GW_ERR_ARG;
  *kind = e->view.plain_kind;
  return GW_OK;
}

extern "C" int gw_get_shape(const gw_engine* e, int32_t* kind, int32_t* kc, int32_t* threads, int32_t* stages) {
  if (!e || !kind || !kc || !threads || !stages) return GW_ERR_ARG;
  *kind = e->shape.kind;
  *kc = e->shape.kind == 0 ? e->shape.kc * e->shape.kr : e->shape.kc;
  *threads = e->shape.threads;
  *stages = e->shape.stages;
  return GW_OK;
}

extern "C" int gw_set_event_weight_copy(gw_engine* e, int32_t enable) {
  if (!e) return GW_ERR_ARG;
  if (!e->initialized) return fail(e, GW_ERR_STATE, "gw_initialize has not been called");
  GW_CUDA(e, cudaSetDevice(e->device));
  if (enable && !e->d_evw) {
    const size_t bytes = sizeof(double) * (size_t)std::max(1, e->cfg.n_results);
    GW_CUDA(e, cudaMalloc(&e->d_evw, bytes));
    e->dev_allocs.push_back(e->d_evw);
    e->resident += (int64_t)bytes;
  }
  e->copy_weights = enable != 0;
  e->clear_graphs();
  return GW_OK;
}

extern "C" int gw_get_event_weights(gw_engine* e, double* w) {
  if (!e || !w) return GW_ERR_ARG;
  if (!e->weights_valid) return fail(e, GW_ERR_STATE, "no event weights: enable the copy and evaluate with K=1");
  GW_CUDA(e, cudaSetDevice(e->device));
  GW_CUDA(e, cudaStreamSynchronize(e->stream));
  if (e->chain_any) GW_CUDA(e, cudaEventSynchronize(e->chain_done));  // the chain that wrote them, any stream
  GW_CUDA(e, cudaMemcpy(w, e->d_evw, sizeof(double) * (size_t)e->cfg.n_results, cudaMemcpyDeviceToHost));
  return GW_OK;
}

extern "C" int gw_resident_memory(const gw_engine* e, int64_t* bytes) {
  if (!e || !bytes) return GW_ERR_ARG;
  *bytes = e->resident;
  return GW_OK;
}

extern "C" int gw_get_layout(const gw_engine* e, gw_layout_info* info) {
  if (!e || !info) return GW_ERR_ARG;
  if (!e->initialized) return GW_ERR_STATE;
  *info = e->layout;
  return GW_OK;
}

extern "C" int gw_set_profiling(gw_engine* e, int32_t on) {
  if (!e) return GW_ERR_ARG;
  if (on && e->use_graph) return fail(e, GW_ERR_STATE, "profiling records events per launch; turn graphs off");
  e->profiling = on != 0;
  e->prof_used = 0;
  return GW_OK;
}

extern "C" int gw_read_profile(gw_engine* e, double* weights_ms, int64_t* weights_launches,
                               int64_t* kernel_launches) {
  if (!e || !weights_ms || !weights_launches || !kernel_launches) return GW_ERR_ARG;
  double total = 0.0;
  if (e->prof_used) {
    GW_CUDA(e, cudaSetDevice(e->device));
    GW_CUDA(e, cudaEventSynchronize(e->prof_events[e->prof_used - 1].second));
    for (size_t i = 0; i < e->prof_used; ++i) {
      float ms = 0.f;
      GW_CUDA(e, cudaEventElapsedTime(&ms, e->prof_events[i].first, e->prof_events[i].second));
      total += ms;
    }
  }
  *weights_ms = total;
  *weights_launches = (int64_t)e->prof_used;
  *kernel_launches = e->kernel_launches;
  e->prof_used = 0;
  e->kernel_launches = 0;
  return GW_OK;
}

// Error text of calls that have no engine (read with gw_last_error(NULL, ...)).
void gw_internal_set_error(const char* msg) { g_create_error = msg ? msg : ""; }
