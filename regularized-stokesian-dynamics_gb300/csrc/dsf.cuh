// Double-single ("float-float") arithmetic for the FP32 pipe.
//
// A value is the unevaluated sum hi + lo of two floats with |lo| <= ulp(hi)/2,
// about 48 significant bits (relative rounding ~4e-15), with float's exponent
// range.  Sums use Knuth's two-sum and products Dekker's exact product
// through a fused multiply-add, renormalised by a quick two-sum: the
// "sloppy" double-single operations of D. H. Bailey's DSFUN package.  Every
// step is an explicitly rounded operation, so the compiler neither contracts
// nor reassociates them.  On GB300 a double-single multiply-add costs about
// ten FP32 instructions, several times cheaper than an FP64 one.
//
// Elementary functions (for the Ewald near-image sums):
//   dsf_sqrt, dsf_rcp   one Newton correction of the float result;
//   dsf_exp_neg         exp(y), y <= 0: Tang's table-driven method, y =
//                       (64 m + j) ln2/64 + r with a Cody-Waite split of
//                       ln2/64, 2^(j/64) from a table, exp(r) by its degree-6
//                       Taylor polynomial (|r| <= ln2/128);
//   dsf_erfc            erfc(x) = exp(-x^2) erfcx(x) for 0 <= x < 6, erfcx
//                       from piecewise degree-11 Chebyshev interpolants
//                       (tables generated by gen_dsf_tables.py).
// The tables live in shared memory (dsf_tables_fill) and are passed in.
// The header also compiles as host C++ (for the accuracy tests); build the
// host side without floating-point contraction.
#pragma once
#include <cmath>

#include "dsf_tables.cuh"

#if defined(__CUDACC__)
#define DSF_FN __host__ __device__ __forceinline__
#else
#define DSF_FN inline
#endif

#if defined(__CUDA_ARCH__)
#define DSF_ADD(a, b) __fadd_rn(a, b)
#define DSF_SUB(a, b) __fsub_rn(a, b)
#define DSF_MUL(a, b) __fmul_rn(a, b)
#define DSF_FMA(a, b, c) __fmaf_rn(a, b, c)
#define DSF_D2F(d) __double2float_rn(d)
#define DSF_SQRT(a) __fsqrt_rn(a)
#define DSF_RCP(a) __frcp_rn(a)
#define DSF_DIV(a, b) __fdiv_rn(a, b)
#else
#define DSF_ADD(a, b) ((a) + (b))
#define DSF_SUB(a, b) ((a) - (b))
#define DSF_MUL(a, b) ((a) * (b))
#define DSF_FMA(a, b, c) std::fma((float)(a), (float)(b), (float)(c))
#define DSF_D2F(d) ((float)(d))
#define DSF_SQRT(a) std::sqrt((float)(a))
#define DSF_RCP(a) (1.0f / (a))
#define DSF_DIV(a, b) ((a) / (b))
#endif

struct dsf {
  float hi, lo;
  DSF_FN dsf() {}
  DSF_FN dsf(float h, float l) : hi(h), lo(l) {}
  DSF_FN dsf(int v) : hi((float)v), lo(0.f) {}
};

DSF_FN dsf dsf_from(double d) {
  const float h = DSF_D2F(d);
  return dsf(h, DSF_D2F(d - (double)h));
}

DSF_FN double dsf_to(dsf a) { return (double)a.hi + (double)a.lo; }

DSF_FN dsf dsf_quick_two_sum(float a, float b) {
  const float s = DSF_ADD(a, b);
  return dsf(s, DSF_SUB(b, DSF_SUB(s, a)));
}

DSF_FN dsf operator+(dsf a, dsf b) {
  const float s = DSF_ADD(a.hi, b.hi);
  const float bb = DSF_SUB(s, a.hi);
  float e = DSF_ADD(DSF_SUB(a.hi, DSF_SUB(s, bb)), DSF_SUB(b.hi, bb));
  e = DSF_ADD(e, DSF_ADD(a.lo, b.lo));
  return dsf_quick_two_sum(s, e);
}

DSF_FN dsf operator-(dsf a) { return dsf(-a.hi, -a.lo); }
DSF_FN dsf operator-(dsf a, dsf b) { return a + (-b); }

DSF_FN dsf operator*(dsf a, dsf b) {
  const float p = DSF_MUL(a.hi, b.hi);
  float e = DSF_FMA(a.hi, b.hi, -p);
  e = DSF_FMA(a.hi, b.lo, DSF_FMA(a.lo, b.hi, e));
  return dsf_quick_two_sum(p, e);
}

// small integer constants (exact in float)
DSF_FN dsf operator*(int k, dsf b) {
  const float kf = (float)k;
  const float p = DSF_MUL(kf, b.hi);
  const float e = DSF_FMA(kf, b.lo, DSF_FMA(kf, b.hi, -p));
  return dsf_quick_two_sum(p, e);
}
DSF_FN dsf operator*(dsf b, int k) { return k * b; }

DSF_FN dsf& operator+=(dsf& a, dsf b) {
  a = a + b;
  return a;
}

DSF_FN dsf fma(dsf a, dsf b, dsf c) { return a * b + c; }

// Unnormalised double-single accumulator: hi is the FP32 running sum and lo
// collects the exact rounding error of every addition into hi (Knuth's
// two-sum) and the error of every product (Dekker's product through FMAs),
// so an accumulate costs 12 FP32 operations instead of 18.  lo is a plain
// FP32 sum, so it grows by about ulp(hi) per step and its own rounding with
// it: renormalise (dsacc_norm, 3 operations) every few steps (at most 16)
// to keep hi + lo within ~2^-47 of the exact sum of the magnitudes added.
struct dsacc {
  float hi, lo;
  DSF_FN dsacc() {}
  DSF_FN dsacc(float h, float l) : hi(h), lo(l) {}
  DSF_FN dsacc(int v) : hi((float)v), lo(0.f) {}
};

// c + a b
DSF_FN dsacc fma(dsf a, dsf b, dsacc c) {
  const float p = DSF_MUL(a.hi, b.hi);
  float pe = DSF_FMA(a.hi, b.hi, -p);
  pe = DSF_FMA(a.hi, b.lo, DSF_FMA(a.lo, b.hi, pe));
  const float s = DSF_ADD(c.hi, p);
  const float bb = DSF_SUB(s, c.hi);
  const float e = DSF_ADD(DSF_SUB(c.hi, DSF_SUB(s, bb)), DSF_SUB(p, bb));
  return dsacc(s, DSF_ADD(c.lo, DSF_ADD(e, pe)));
}

DSF_FN dsacc& operator+=(dsacc& c, dsf v) {
  const float s = DSF_ADD(c.hi, v.hi);
  const float bb = DSF_SUB(s, c.hi);
  const float e = DSF_ADD(DSF_SUB(c.hi, DSF_SUB(s, bb)), DSF_SUB(v.hi, bb));
  c.lo = DSF_ADD(c.lo, DSF_ADD(e, v.lo));
  c.hi = s;
  return c;
}

DSF_FN void dsacc_norm(dsacc& c) {
  const float s = DSF_ADD(c.hi, c.lo);
  c.lo = DSF_SUB(c.lo, DSF_SUB(s, c.hi));
  c.hi = s;
}

DSF_FN double dsacc_to(dsacc a) { return (double)a.hi + (double)a.lo; }

// sqrt(a), a > 0
DSF_FN dsf dsf_sqrt(dsf a) {
  const float s = DSF_SQRT(a.hi);
  const float p = DSF_MUL(s, s);
  const float e = DSF_FMA(s, s, -p);
  const float d = DSF_ADD(DSF_SUB(DSF_SUB(a.hi, p), e), a.lo);  // a - s^2 (a.hi - p is exact)
  return dsf_quick_two_sum(s, DSF_MUL(d, DSF_DIV(0.5f, s)));
}

// 1 / a, a != 0
DSF_FN dsf dsf_rcp(dsf a) {
  const float q = DSF_RCP(a.hi);
  const float p = DSF_MUL(a.hi, q);
  const float pe = DSF_FMA(a.hi, q, -p);
  const float e = DSF_SUB(DSF_SUB(DSF_SUB(1.0f, p), pe), DSF_MUL(a.lo, q));  // 1 - a q (1 - p is exact)
  return dsf_quick_two_sum(q, DSF_MUL(q, e));
}

// Tables in shared memory: 2^(j/64) (64 entries) and the erfcx pieces.
struct dsf_tables {
  dsf exp2[64];
  dsf erfcx[RSD_ERFCX_NPIECE][RSD_ERFCX_DEG + 1];
};

// exp(y) for -88 < y <= 0
DSF_FN dsf dsf_exp_neg(dsf y, const dsf_tables& T) {
  // ln2/64 = C1 + C2: C1 = 2839 / 2^18 has 12 significant bits, so k C1 is
  // exact for |k| < 2^12 (y >= -38); C2 = ln2/64 - C1 as a float pair
  const float C1 = 2839.0f / 262144.0f;
  const dsf C2(4.991591140424134e-07f, 2.572804640231345e-14f);
  const float kf = rintf(DSF_MUL(y.hi, 92.33248261689366f));
  const int k = (int)kf;
  const dsf r = dsf(DSF_SUB(y.hi, DSF_MUL(kf, C1)), y.lo) - k * C2;
  // degree-6 Taylor polynomial of exp(r), |r| <= ln2/128
  dsf p(0.0013888889225199819f, -3.3631094437103215e-11f);  // 1/720
  p = p * r + dsf(0.008333333767950535f, -4.34617203337595e-10f);  // 1/120
  p = p * r + dsf(0.0416666679084301f, -1.2417634698280722e-09f);  // 1/24
  p = p * r + dsf(0.1666666716337204f, -4.967053879312289e-09f);  // 1/6
  p = p * r + dsf(0.5f, 0.0f);
  p = p * r + dsf(1.0f, 0.0f);
  p = p * r + dsf(1.0f, 0.0f);
  const dsf v = p * T.exp2[k & 63];
  const int m = k >> 6;  // floor(k / 64)
  return dsf(ldexpf(v.hi, m), ldexpf(v.lo, m));
}

// erfc(x) and exp(-x^2) for 0 <= x < 6
DSF_FN void dsf_erfc_gauss(dsf x, const dsf_tables& T, dsf* erfc_x, dsf* gauss) {
  const dsf g = dsf_exp_neg(-(x * x), T);
  int piece = (int)DSF_MUL(x.hi, 4.0f);
  piece = piece < 0 ? 0 : (piece > RSD_ERFCX_NPIECE - 1 ? RSD_ERFCX_NPIECE - 1 : piece);
  const dsf t = x - dsf(DSF_MUL((float)piece + 0.5f, 0.25f), 0.0f);
  const dsf* c = T.erfcx[piece];
  dsf e = c[RSD_ERFCX_DEG];
  for (int n = RSD_ERFCX_DEG - 1; n >= 0; n--) e = e * t + c[n];
  *erfc_x = g * e;
  *gauss = g;
}

// Fills T from the generated double tables (hi/lo splits); on the device
// the tables sit in constant memory.
#if defined(__CUDACC__)
__device__ __forceinline__
#else
inline
#endif
void dsf_tables_fill(dsf_tables& T, int tid, int nthr) {
  for (int i = tid; i < 64; i += nthr) T.exp2[i] = dsf_from(rsd_exp2_table[i]);
  for (int i = tid; i < RSD_ERFCX_NPIECE * (RSD_ERFCX_DEG + 1); i += nthr)
    T.erfcx[i / (RSD_ERFCX_DEG + 1)][i % (RSD_ERFCX_DEG + 1)] =
        dsf_from(rsd_erfcx_coef[i / (RSD_ERFCX_DEG + 1)][i % (RSD_ERFCX_DEG + 1)]);
}
