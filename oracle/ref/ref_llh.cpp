// ref_llh.cpp -- a C-ABI driver of GUNDAM's own per-bin likelihood classes
// compiled for the host: test infrastructure, built by oracle/ref/build_ref.py
// into oracle/_ref/libref_llh.so, never shipped.
//
// Each bin goes through JointProbability::<class>::eval(const SamplePair&,
// int) (PoissonLogLikelihood.h:19-53 via JointProbabilityBase.h:37-43;
// BarlowBeestonBanff2022.h:92-294) on a one-bin model and data histogram
// holding (sum of weights, sqrt of the sum of squared weights), so the
// reference squares the stored sqrt itself, as in a fit.  Options keep their
// class defaults; for Barlow-Beeston the value is taken with throwIfInfLlh =
// false (the reference then returns +inf where the default throws) and
// `threw` records what the default configuration does instead: 1 = throws,
// 2 = ends the process (a non-finite sum of squared weights,
// BarlowBeestonBanff2022.h:126-144; the driver does not call it then).
#include <cstdint>
#include <stdexcept>

#include "BarlowBeestonBanff2022.h"
#include "PoissonLogLikelihood.h"

namespace {
struct OneBin {
  Sample model, data;
  SamplePair pair;
  OneBin(double data_v, double pred, double sqrt_sum_w2) {
    model.histogram.content = {GwRefBinContent{pred, sqrt_sum_w2}};
    model.histogram.context = {GwRefBinContext{}};
    data.histogram.content = {GwRefBinContent{data_v, std::sqrt(data_v)}};
    data.histogram.context = {GwRefBinContext{}};
    pair.model = &model;
    pair.data = &data;
  }
};
}  // namespace

extern "C" int ref_llh_bins(int32_t type, const double* data, const double* pred, const double* sqrt_sum_w2,
                            int32_t n, double* out, int32_t* threw) {
  if (!data || !pred || !sqrt_sum_w2 || !out || !threw || n < 0) return 1;
  // called through the base class, as the likelihood interface holds them
  // (a derived class's eval(double, double, double, int) hides the others)
  JointProbability::PoissonLogLikelihood poisson_obj;
  JointProbability::BarlowBeestonBanff2022 bb_quiet_obj;
  bb_quiet_obj.throwIfInfLlh = false;
  JointProbability::BarlowBeestonBanff2022 bb_default_obj;
  const JointProbability::JointProbabilityBase& poisson = poisson_obj;
  const JointProbability::JointProbabilityBase& bb_quiet = bb_quiet_obj;
  const JointProbability::JointProbabilityBase& bb_default = bb_default_obj;
  for (int32_t i = 0; i < n; ++i) {
    OneBin b(data[i], pred[i], sqrt_sum_w2[i]);
    threw[i] = 0;
    if (type == 1) {
      out[i] = poisson.eval(b.pair, 0);
    } else if (type == 2) {
      out[i] = bb_quiet.eval(b.pair, 0);
      const double mc = sqrt_sum_w2[i] * sqrt_sum_w2[i];
      if (!std::isfinite(mc) || mc < 0.0) {
        threw[i] = 2;  // the default configuration ends the process here (std::exit)
        continue;
      }
      try {
        (void)bb_default.eval(b.pair, 0);
      } catch (const std::exception&) {
        threw[i] = 1;
      }
    } else {
      return 1;
    }
  }
  return 0;
}
