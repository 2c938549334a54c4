// Stand-in for ROOT's TSpline3 declaration: the Cache::Manager calculators only
// name it in FindPoints(const TSpline3*), which the driver never calls.
#ifndef GW_REF_STUB_TSPLINE_H
#define GW_REF_STUB_TSPLINE_H
class TSpline3 {
 public:
  int GetNp() const { return 0; }
};
#endif
