// ref_dials.cpp -- exports the reference's own per-dial functions
// (src/Utils/include/Calculate*.h of the GUNDAM source tree) through a C ABI
// so the oracle can be pinned against them.  This file only includes those
// headers from the reference tree (given with -I at build time) and wraps
// them; it is built by build_ref.py into oracle/_ref/, never shipped.
#include <cstring>
#include <vector>

#include "CalculateBicubicSpline.h"
#include "CalculateBilinearInterpolation.h"
#include "CalculateCompactSpline.h"
#include "CalculateGeneralSpline.h"
#include "CalculateGraph.h"
#include "CalculateMonotonicSpline.h"
#include "CalculateUniformSpline.h"

namespace {
// The surface index search reads a[8] even for small grids; give every call
// a zero-padded copy so those reads stay inside the buffer.
std::vector<double> padded(const double* d, int n) {
  std::vector<double> v((size_t)n + 64, 0.0);
  std::memcpy(v.data(), d, sizeof(double) * (size_t)n);
  return v;
}
}  // namespace

extern "C" {
double ref_monotonic(double x, double lo, double hi, const double* d, int n_data) {
  std::vector<double> v = padded(d, n_data);
  return CalculateMonotonicSpline(x, lo, hi, v.data(), n_data - 2);
}
double ref_compact(double x, double lo, double hi, const double* d, int n_data) {
  std::vector<double> v = padded(d, n_data);
  return CalculateCompactSpline(x, lo, hi, v.data(), n_data - 2);
}
double ref_uniform(double x, double lo, double hi, const double* d, int n_data) {
  std::vector<double> v = padded(d, n_data);
  return CalculateUniformSpline(x, lo, hi, v.data(), n_data);
}
double ref_general(double x, double lo, double hi, const double* d, int n_data) {
  std::vector<double> v = padded(d, n_data);
  return CalculateGeneralSpline(x, lo, hi, v.data(), n_data);
}
double ref_graph(double x, double lo, double hi, const double* d, int n_data) {
  std::vector<double> v = padded(d, n_data);
  return CalculateGraph(x, lo, hi, v.data(), n_data);
}
// d = [nx, ny, xx[nx], yy[ny], knots[nx*ny]] as the Bilinear/Bicubic dials keep it.
double ref_bilinear(double x, double y, double lo, double hi, const double* d, int n_data) {
  std::vector<double> v = padded(d, n_data);
  const int nx = (int)v[0], ny = (int)v[1];
  const double* xx = v.data() + 2;
  const double* yy = xx + nx;
  const double* knots = yy + ny;
  return CalculateBilinearInterpolation(x, y, lo, hi, knots, nx, ny, xx, nx, yy, ny);
}
double ref_bicubic(double x, double y, double lo, double hi, const double* d, int n_data) {
  std::vector<double> v = padded(d, n_data);
  const int nx = (int)v[0], ny = (int)v[1];
  const double* xx = v.data() + 2;
  const double* yy = xx + nx;
  const double* knots = yy + ny;
  return CalculateBicubicSpline(x, y, lo, hi, knots, nx, ny, xx, nx, yy, ny);
}
}
