// Stand-in for GUNDAM's Sample / Histogram / JsonBaseClass / TMath, enough to
// compile the likelihood classes of
// src/StatisticalInference/JointProbability/include/ on the host outside the
// GUNDAM build (test infrastructure, oracle/ref/ref_llh.cpp): a sample is a
// histogram of (sum of weights, sqrt of sum of squared weights) per bin, as
// Histogram::refillHistogram leaves it (src/SamplesManager/src/Histogram.cpp).
#ifndef GW_REF_STUB_SAMPLE_H
#define GW_REF_STUB_SAMPLE_H
#include <cmath>
#include <initializer_list>
#include <limits>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

namespace TMath {
inline double Log(double x) { return std::log(x); }
}  // namespace TMath

// Configuration reader of JsonBaseClass: the stand-in reads nothing, so every
// option keeps the default its class gives it.
struct GwRefConfigStub {
  struct Field {
    Field(const char*) {}
    Field(const char*, std::initializer_list<const char*>) {}
  };
  void defineFields(std::initializer_list<Field>) {}
  void checkConfiguration() {}
  template <typename T>
  void fillValue(T&, const char*) {}
};

class JsonBaseClass {
 public:
  virtual ~JsonBaseClass() = default;

 protected:
  virtual void configureImpl() {}
  GwRefConfigStub _config_;
};

struct GwRefBinContent {
  double sumWeights{0};
  double sqrtSumSqWeights{0};
};
struct GwRefBin {
  int index{0};
  std::string getSummary() const { return "bin"; }
  int getIndex() const { return index; }
};
struct GwRefBinContext {
  GwRefBin bin;
};

class GwRefHistogram {
 public:
  std::vector<GwRefBinContent> content;
  std::vector<GwRefBinContext> context;
  const std::vector<GwRefBinContent>& getBinContentList() const { return content; }
  const std::vector<GwRefBinContext>& getBinContextList() const { return context; }
  int getNbBins() const { return (int)content.size(); }
  std::vector<std::tuple<const GwRefBinContent&, const GwRefBinContext&>> loop() const {
    std::vector<std::tuple<const GwRefBinContent&, const GwRefBinContext&>> out;
    for (size_t i = 0; i < content.size(); ++i) out.emplace_back(content[i], context[i]);
    return out;
  }
};

class Sample {
 public:
  GwRefHistogram histogram;
  const GwRefHistogram& getHistogram() const { return histogram; }
  const std::string& getName() const { return name; }
  int getIndex() const { return 0; }
  std::string name{"sample"};
};
#endif
