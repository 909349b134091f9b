// Host build of the double-single arithmetic (dsf.cuh) for its accuracy
// test, tests/test_dsf.py.  Built without floating-point contraction, so the
// host evaluates the same operation sequence as the device.
#include <cstdio>

#include "dsf.cuh"

static dsf_tables g_tab;
static bool g_ready = false;

static void ready() {
  if (!g_ready) {
    dsf_tables_fill(g_tab, 0, 1);
    g_ready = true;
  }
}

extern "C" void dsf_check_erfc_gauss(double x, double out[2]) {
  ready();
  dsf e, g;
  dsf_erfc_gauss(dsf_from(x), g_tab, &e, &g);
  out[0] = dsf_to(e);
  out[1] = dsf_to(g);
}

extern "C" double dsf_check_exp_neg(double y) {
  ready();
  return dsf_to(dsf_exp_neg(dsf_from(y), g_tab));
}

extern "C" void dsf_check_sqrt_rcp(double a, double out[2]) {
  out[0] = dsf_to(dsf_sqrt(dsf_from(a)));
  out[1] = dsf_to(dsf_rcp(dsf_from(a)));
}

// a*b + c and a - b in double-single
extern "C" void dsf_check_ops(double a, double b, double c, double out[2]) {
  out[0] = dsf_to(fma(dsf_from(a), dsf_from(b), dsf_from(c)));
  out[1] = dsf_to(dsf_from(a) - dsf_from(b));
}

// sum_i a_i b_i + sum_i c_i, n terms each, through the unnormalised
// accumulator (the products first, then the plain additions), renormalised
// every `every` steps
extern "C" double dsf_check_accumulate(int n, const double* a, const double* b, const double* c, int every) {
  dsacc s(0);
  int k = 0;
  for (int i = 0; i < n; i++) {
    s = fma(dsf_from(a[i]), dsf_from(b[i]), s);
    if (++k == every) dsacc_norm(s), k = 0;
  }
  for (int i = 0; i < n; i++) {
    s += dsf_from(c[i]);
    if (++k == every) dsacc_norm(s), k = 0;
  }
  return dsacc_to(s);
}
