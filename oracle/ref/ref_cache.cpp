// ref_cache.cpp -- a C-ABI driver of GUNDAM's own Cache::Manager calculators
// compiled for the host (HEMI_CUDA_DISABLE): test infrastructure, built by
// oracle/ref/build_ref.py into oracle/_ref/libref_cache.so, never shipped.
//
// It fills the reference's operator API the way Cache::Manager::Update does
// (src/CacheManager/src/CacheManager.cpp:477-740): Cache::Parameters (clamps,
// mirrors), Cache::Weights (initial values) and one Cache::Weight::* calculator
// per dial type (ReserveNorm / AddSpline / AddGraph / AddData), then
// Cache::RecursiveSums (SetEventIndex, Initialize); an evaluation is
// SetParameter for every parameter, Weights::Apply and RecursiveSums::Apply
// (Cache::Manager::Fill, CacheManager.cpp:750-810).  Table dials are not
// driven here.
#include <cstdint>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "CacheParameters.h"
#include "CacheRecursiveSums.h"
#include "CacheWeights.h"
#include "WeightBilinear.h"
#include "WeightCompactSpline.h"
#include "WeightGeneralSpline.h"
#include "WeightGraph.h"
#include "WeightMonotonicSpline.h"
#include "WeightNormalization.h"
#include "WeightUniformSpline.h"

namespace {
// dial type codes of include/gw.h
enum { kNorm = 1, kMono = 2, kUni = 3, kGen = 4, kCompact = 5, kGraph = 6, kBilin = 7 };
}  // namespace

struct ref_cache {
  int P = 0, B = 0;
  std::unique_ptr<Cache::Parameters> params;
  std::unique_ptr<Cache::Weights> weights;
  std::unique_ptr<Cache::Weight::Normalization> norm;
  std::unique_ptr<Cache::Weight::MonotonicSpline> mono;
  std::unique_ptr<Cache::Weight::UniformSpline> uni;
  std::unique_ptr<Cache::Weight::GeneralSpline> gen;
  std::unique_ptr<Cache::Weight::CompactSpline> compact;
  std::unique_ptr<Cache::Weight::Graph> graph;
  std::unique_ptr<Cache::Weight::Bilinear> bilin;
  std::unique_ptr<Cache::RecursiveSums> sums;
  std::string err;
};

static thread_local std::string g_err;

extern "C" {

int ref_cache_create(int32_t n_events, int32_t n_params, int32_t n_bins, int64_t n_dials, const uint8_t* type,
                     const int32_t* result, const int32_t* par0, const int32_t* par1, const int64_t* data_start,
                     const double* data, const double* w0, const int32_t* bin, const double* clamp_lo,
                     const double* clamp_hi, const double* mirror_lo, const double* mirror_hi, ref_cache** out) {
  try {
    auto c = std::make_unique<ref_cache>();
    c->P = n_params;
    c->B = n_bins;
    int64_t cnt[8] = {0}, space[8] = {0};
    for (int64_t i = 0; i < n_dials; ++i) {
      if (type[i] < 1 || type[i] > 7) {
        g_err = "unsupported dial type for the reference driver";
        return 1;
      }
      cnt[type[i]]++;
      space[type[i]] += data_start[i + 1] - data_start[i];
    }
    c->params = std::make_unique<Cache::Parameters>((std::size_t)n_params);
    for (int p = 0; p < n_params; ++p) {
      c->params->SetLowerClamp(p, clamp_lo[p]);
      c->params->SetUpperClamp(p, clamp_hi[p]);
      if (mirror_lo && mirror_hi && mirror_lo[p] > -1e300 && mirror_hi[p] < 1e300) {
        c->params->SetLowerMirror(p, mirror_lo[p]);
        c->params->SetUpperMirror(p, mirror_hi[p]);
      }
    }
    c->weights = std::make_unique<Cache::Weights>((std::size_t)n_events);
    for (int e = 0; e < n_events; ++e) c->weights->SetInitialValue(e, w0[e]);
    auto& res = c->weights->GetWeights();
    auto& vals = c->params->GetParameters();
    auto& lo = c->params->GetLowerClamps();
    auto& hi = c->params->GetUpperClamps();
    if (cnt[kNorm]) {
      c->norm = std::make_unique<Cache::Weight::Normalization>(res, vals, (std::size_t)cnt[kNorm]);
      c->weights->AddWeightCalculator(c->norm.get());
    }
    if (cnt[kCompact]) {
      c->compact = std::make_unique<Cache::Weight::CompactSpline>(res, vals, lo, hi, (std::size_t)cnt[kCompact],
                                                                  (std::size_t)space[kCompact], "space");
      c->weights->AddWeightCalculator(c->compact.get());
    }
    if (cnt[kMono]) {
      c->mono = std::make_unique<Cache::Weight::MonotonicSpline>(res, vals, lo, hi, (std::size_t)cnt[kMono],
                                                                 (std::size_t)space[kMono], "space");
      c->weights->AddWeightCalculator(c->mono.get());
    }
    if (cnt[kUni]) {
      c->uni = std::make_unique<Cache::Weight::UniformSpline>(res, vals, lo, hi, (std::size_t)cnt[kUni],
                                                              (std::size_t)space[kUni], "space");
      c->weights->AddWeightCalculator(c->uni.get());
    }
    if (cnt[kGen]) {
      c->gen = std::make_unique<Cache::Weight::GeneralSpline>(res, vals, lo, hi, (std::size_t)cnt[kGen],
                                                              (std::size_t)space[kGen], "space");
      c->weights->AddWeightCalculator(c->gen.get());
    }
    if (cnt[kGraph]) {
      c->graph = std::make_unique<Cache::Weight::Graph>(res, vals, lo, hi, (std::size_t)cnt[kGraph],
                                                        (std::size_t)space[kGraph]);
      c->weights->AddWeightCalculator(c->graph.get());
    }
    if (cnt[kBilin]) {
      c->bilin = std::make_unique<Cache::Weight::Bilinear>(res, vals, lo, hi, (std::size_t)cnt[kBilin],
                                                           (std::size_t)space[kBilin]);
      c->weights->AddWeightCalculator(c->bilin.get());
    }
    std::vector<double> d;
    for (int64_t i = 0; i < n_dials; ++i) {
      d.assign(data + data_start[i], data + data_start[i + 1]);
      switch (type[i]) {
        case kNorm: c->norm->ReserveNorm(result[i], par0[i]); break;
        case kMono: c->mono->AddSpline(result[i], par0[i], d); break;
        case kUni: c->uni->AddSpline(result[i], par0[i], d); break;
        case kGen: c->gen->AddSpline(result[i], par0[i], d); break;
        case kCompact: c->compact->AddSpline(result[i], par0[i], d); break;
        case kGraph: c->graph->AddGraph(result[i], par0[i], d); break;
        case kBilin: c->bilin->AddData(result[i], par0[i], par1[i], d); break;
      }
    }
    c->sums = std::make_unique<Cache::RecursiveSums>(res, (std::size_t)n_bins);
    for (int e = 0; e < n_events; ++e) c->sums->SetEventIndex(e, bin[e]);
    c->sums->Initialize();
    *out = c.release();
    return 0;
  } catch (const std::exception& ex) {
    g_err = ex.what();
    return 1;
  }
}

// One evaluation at `params` [n_params]: bin sums and sums of squares [n_bins]
// and (optional) per-event weights [n_events].
int ref_cache_eval(ref_cache* c, const double* params, double* sums, double* sums2, double* weights) {
  try {
    for (int p = 0; p < c->P; ++p) c->params->SetParameter(p, params[p]);
    c->weights->Apply();
    c->sums->Invalidate();
    c->sums->Apply();
    const double* s = c->sums->GetSumsPointer();
    const double* s2 = c->sums->GetSums2Pointer();
    std::memcpy(sums, s, sizeof(double) * (size_t)c->B);
    std::memcpy(sums2, s2, sizeof(double) * (size_t)c->B);
    if (weights) {
      const std::size_t n = c->weights->GetResultCount();
      for (std::size_t i = 0; i < n; ++i) weights[i] = c->weights->GetResult((int)i);
    }
    return 0;
  } catch (const std::exception& ex) {
    c->err = ex.what();
    return 1;
  }
}

const char* ref_cache_error(ref_cache* c) { return c ? c->err.c_str() : g_err.c_str(); }

void ref_cache_destroy(ref_cache* c) { delete c; }
}
