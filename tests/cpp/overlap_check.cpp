// Host build of the overlap corrections of the grand mobility (overlap.cuh,
// the device code of correction_method 1 and 2) for tests/test_overlap.py,
// which compares it with the oracle's restatement of GRPY_YZD.f90 and
// Regularization.f90.
#include <cmath>
#define __device__
#define __host__
#define __forceinline__ inline
using std::erf;
using std::exp;
using std::fabs;
using std::fma;
using std::sqrt;
#include "overlap.cuh"

extern "C" void ovl_correction60(int method, const double R[3], double ai, double aj, double out[60]) {
  rsd_overlap_correction60(method, R, ai, aj, out);
}

extern "C" void ovl_regular60(const double R[3], double ai, double aj, double out[60]) {
  rsd_overlap::regular60(R, ai, aj, out);
}

extern "C" void ovl_yamakawa60(const double R[3], double ai, double aj, double out[60]) {
  double Y[45];
  rsd_overlap::y2_basis(Y);
  rsd_overlap::yamakawa60(R, ai, aj, Y, out);
}

extern "C" void ovl_free_space60(const double R[3], double ai, double aj, double out[60]) {
  double Y[45];
  rsd_overlap::y2_basis(Y);
  rsd_overlap::free_space60(R, ai, aj, Y, out);
}
