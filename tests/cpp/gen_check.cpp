// Host build of the generated Ewald closed forms (ewald_gen.cuh) for a unit
// test of the generator: one pair block summed exactly like the CUDA kernel
// sums it, compared by tests/test_generated_forms.py with the oracle.
#include <cmath>
#include <cstdio>
#include <cstring>
#define __device__
#define __host__
#define __forceinline__ inline
using std::fma;
#include "ewald_gen.cuh"

static const double PAI = 3.141592653589793238462643383279502884;
static const double PIP5 = 0.564189583547756286948079451560772585844;

extern "C" void gen_pair_block(const double R[3], const double LR[9], const double LI[9], double LV, double lam,
                               int NR, int NI, double ai, double aj, double phix, int include_k, double out[60]) {
  double acc[RSD_NMOM_REAL] = {0};
  for (int nx = -NR; nx <= NR; nx++)
    for (int ny = -NR; ny <= NR; ny++)
      for (int nz = -NR; nz <= NR; nz++) {
        double x[3];
        for (int i = 0; i < 3; i++) x[i] = R[i] + LR[i] * nx + LR[i + 3] * ny + LR[i + 6] * nz;
        double r = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
        double E0 = std::erfc(lam * r), Ed = 2.0 * PIP5 * lam * std::exp(-r * r * lam * lam);
        rsd_real_image<double>(x[0], x[1], x[2], r, 1.0 / r, E0, Ed, lam, acc);
      }
  double o_r[60];
  rsd_real_epilogue<double>(acc, ai, aj, phix, o_r);
  double o_c[60] = {0}, o_s[60] = {0};
  if (include_k) {
    double ac[RSD_NMOM_KCOS] = {0}, as[RSD_NMOM_KSIN] = {0}, wc[RSD_NMOM_KCOS], ws[RSD_NMOM_KSIN];
    for (int nx = -NI; nx <= NI; nx++)
      for (int ny = -NI; ny <= NI; ny++)
        for (int nz = -NI; nz <= NI; nz++) {
          if (!nx && !ny && !nz) continue;
          double k[3];
          for (int j = 0; j < 3; j++) k[j] = 2 * PAI * (nx * LI[0 + 3 * j] + ny * LI[1 + 3 * j] + nz * LI[2 + 3 * j]);
          double k2 = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
          double S = 8.0 * PAI * (1 + k2 / (4 * lam * lam) + k2 * k2 / (8 * lam * lam * lam * lam)) *
                     std::exp(-k2 / (4 * lam * lam)) / (k2 * k2);
          rsd_kcos_weights<double>(k[0], k[1], k[2], S, lam, wc);
          rsd_ksin_weights<double>(k[0], k[1], k[2], S, lam, ws);
          double kr = k[0] * R[0] + k[1] * R[1] + k[2] * R[2], c = std::cos(kr), s = std::sin(kr);
          for (int m = 0; m < RSD_NMOM_KCOS; m++) ac[m] += wc[m] * c;
          for (int m = 0; m < RSD_NMOM_KSIN; m++) as[m] += ws[m] * s;
        }
    rsd_kcos_epilogue<double>(ac, ai, aj, phix, o_c);
    rsd_ksin_epilogue<double>(as, ai, aj, phix, o_s);
  }
  const double na = 1.0 / (6.0 * ai), na3 = 1.0 / (6.0 * ai * ai * ai);
  for (int q = 0; q < 60; q++) {
    double v = o_r[q] + (o_c[q] + o_s[q]) / LV;
    bool a3 = (q >= 6 && q < 12) || (q >= 15 && q < 30) || q >= 45;
    out[q] = v * (a3 ? na3 : na);
  }
}

// The mixed split of the CUDA kernels: images in the central shell and the
// first reciprocal shell in double, the rest accumulated in float; `epi64`
// selects a double epilogue for the float moments.
static double g_rcut = 1e300;  // real images with lam*r < g_rcut stay in double
static int g_kshell = 1;       // reciprocal vectors with max|n| <= g_kshell stay in double
extern "C" void gen_set_split(double rcut, int kshell) {
  g_rcut = rcut;
  g_kshell = kshell;
}
extern "C" void gen_pair_block_mixed(const double R[3], const double LR[9], const double LI[9], double LV, double lam,
                                     int NR, int NI, double ai, double aj, double phix, int epi64, double out[60]) {
  double acc[RSD_NMOM_REAL] = {0};
  float accf[RSD_NMOM_REAL] = {0};
  const float lamf = (float)lam, cdf = (float)(2.0 * PIP5) * lamf;
  for (int nx = -NR; nx <= NR; nx++)
    for (int ny = -NR; ny <= NR; ny++)
      for (int nz = -NR; nz <= NR; nz++) {
        double x[3];
        for (int i = 0; i < 3; i++) x[i] = R[i] + LR[i] * nx + LR[i + 3] * ny + LR[i + 6] * nz;
        const bool central = lam * std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]) < g_rcut;
        if (central) {
          double r = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
          rsd_real_image<double>(x[0], x[1], x[2], r, 1.0 / r, std::erfc(lam * r),
                                 2.0 * PIP5 * lam * std::exp(-r * r * lam * lam), lam, acc);
        } else {
          const float x0 = (float)x[0], x1 = (float)x[1], x2 = (float)x[2];
          const float r2 = x0 * x0 + x1 * x1 + x2 * x2, r = std::sqrt(r2);
          rsd_real_image<float>(x0, x1, x2, r, 1.0f / r, std::erfc(lamf * r), cdf * std::exp(-r2 * lamf * lamf), lamf,
                                accf);
        }
      }
  double o_r[60], o_f[60];
  rsd_real_epilogue<double>(acc, ai, aj, phix, o_r);
  if (epi64) {
    double a2[RSD_NMOM_REAL];
    for (int m = 0; m < RSD_NMOM_REAL; m++) a2[m] = accf[m];
    rsd_real_epilogue<double>(a2, ai, aj, phix, o_f);
  } else {
    float of[60];
    rsd_real_epilogue<float>(accf, (float)ai, (float)aj, (float)phix, of);
    for (int q = 0; q < 60; q++) o_f[q] = of[q];
  }
  double ac[RSD_NMOM_KCOS] = {0}, as[RSD_NMOM_KSIN] = {0};
  float acf[RSD_NMOM_KCOS] = {0}, asf[RSD_NMOM_KSIN] = {0};
  const int w = 2 * NI + 1;
  for (int q = (w * w * w - 1) / 2 + 1; q < w * w * w; q++) {
    const int nx = q / (w * w) - NI, ny = (q / w) % w - NI, nz = q % w - NI;
    double k[3];
    for (int j = 0; j < 3; j++) k[j] = 2 * PAI * (nx * LI[0 + 3 * j] + ny * LI[1 + 3 * j] + nz * LI[2 + 3 * j]);
    double k2 = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
    double S = 8.0 * PAI * (1 + k2 / (4 * lam * lam) + k2 * k2 / (8 * lam * lam * lam * lam)) *
               std::exp(-k2 / (4 * lam * lam)) / (k2 * k2);
    double wc[RSD_NMOM_KCOS], ws[RSD_NMOM_KSIN];
    rsd_kcos_weights<double>(k[0], k[1], k[2], S, lam, wc);
    rsd_ksin_weights<double>(k[0], k[1], k[2], S, lam, ws);
    double kr = k[0] * R[0] + k[1] * R[1] + k[2] * R[2], c = std::cos(kr), s = std::sin(kr);
    if (std::abs(nx) <= g_kshell && std::abs(ny) <= g_kshell && std::abs(nz) <= g_kshell) {
      for (int m = 0; m < RSD_NMOM_KCOS; m++) ac[m] += wc[m] * c;
      for (int m = 0; m < RSD_NMOM_KSIN; m++) as[m] += ws[m] * s;
    } else {
      for (int m = 0; m < RSD_NMOM_KCOS; m++) acf[m] = std::fma((float)wc[m], (float)c, acf[m]);
      for (int m = 0; m < RSD_NMOM_KSIN; m++) asf[m] = std::fma((float)ws[m], (float)s, asf[m]);
    }
  }
  double o_c[60], o_s[60], o_cf[60], o_sf[60];
  rsd_kcos_epilogue<double>(ac, ai, aj, phix, o_c);
  rsd_ksin_epilogue<double>(as, ai, aj, phix, o_s);
  {
    double a2[RSD_NMOM_KCOS], b2[RSD_NMOM_KSIN];
    for (int m = 0; m < RSD_NMOM_KCOS; m++) a2[m] = acf[m];
    for (int m = 0; m < RSD_NMOM_KSIN; m++) b2[m] = asf[m];
    rsd_kcos_epilogue<double>(a2, ai, aj, phix, o_cf);
    rsd_ksin_epilogue<double>(b2, ai, aj, phix, o_sf);
  }
  const double na = 1.0 / (6.0 * ai), na3 = 1.0 / (6.0 * ai * ai * ai);
  for (int q = 0; q < 60; q++) {
    double v = o_r[q] + o_f[q] + 2.0 * (o_c[q] + o_s[q] + o_cf[q] + o_sf[q]) / LV;
    bool a3 = (q >= 6 && q < 12) || (q >= 15 && q < 30) || q >= 45;
    out[q] = v * (a3 ? na3 : na);
  }
}

// The real-space epilogue as a coefficient table (rsd_real_epi_coef +
// rsd_real_epi_apply) against the generated epilogue, for given moments.
extern "C" void gen_real_epilogue_both(const double acc[RSD_NMOM_REAL], double ai, double aj, double phix,
                                       double direct[60], double table[60]) {
  rsd_real_epilogue<double>(acc, ai, aj, phix, direct);
  double c[RSD_REAL_EPI_NC];
  rsd_real_epi_coef<double>(ai, aj, phix, c);
  rsd_real_epi_apply<double, double, double>(acc, c, table);
}
