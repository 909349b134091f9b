// Overlap corrections of the grand mobility, per_GRPY_YZD.f90:98-116: for a
// pair whose minimum image overlaps or touches (r <= a_i + a_j), method 1
// adds Yamakawa's overlapping-sphere pair blocks (GRPY_YZD.f90:326-786) and
// method 2 the regularized pair blocks (Regularization.f90:18-162, generated
// in overlap_gen.cuh), each minus the free-space pair (stokesian_Green.f90:
// 11-109) (overlap_Yamakawa_CORRECTION_IJ and overlap_Regular_CORRECTION_IJ,
// GRPY_YZD.f90:789-836).
//
// rsd_overlap_correction60 returns the correction as the 60 values of a
// pair in the order of the pair kernels (TT 0-5 and RR 6-11 as the upper
// triangles (00,01,02,11,12,22), TR 12-14 as (01,02,12), QQ 15-29 as the
// upper triangle of the 5 x 5 block by rows, G 30-44 and H 45-59 as 3 x 5
// by rows), in their units before the factor 1/(pi mu_f).
//
// The free-space pair is the generated real-space image at lambda = 0 (the
// unscreened chain of Ewald_summation.f90) plus the one term by which
// stokesian_Green.f90's chain differs from it: its Init_DDD2_Jg (295-312)
// writes the delta_ij x_k x_l / r^7 term with the opposite sign, which
// after the block formulas and the non-dimensionalisation adds
//   dQQ_ijkl = 3/8 (a_i^2 + a_j^2) (d_ik x_j x_l + d_jk x_i x_l) / r^7,
//   dH_ijk   = -3/8 a_j^2 (eps_ijl x_l) x_k / r^7
// before the Y2 projections.
//
// Device code (one thread per overlapping pair, which are few); the header
// also compiles for the host, where the unit test defines __device__ away.
#pragma once
#include "ewald_gen.cuh"
#include "overlap_gen.cuh"

namespace rsd_overlap {

// Y2(m, i, j) at m + 5 (i + 3 j), tensors.f90:43-67
__device__ inline void y2_basis(double Y[45]) {
  const double s2 = 0.70710678118654752440, s6 = 0.40824829046386301637, s23 = 0.81649658092772603273;
  for (int q = 0; q < 45; q++) Y[q] = 0.0;
  Y[0 + 5 * (0 + 3 * 1)] = s2;
  Y[0 + 5 * (1 + 3 * 0)] = s2;
  Y[1 + 5 * (1 + 3 * 2)] = -s2;
  Y[1 + 5 * (2 + 3 * 1)] = -s2;
  Y[2 + 5 * (0 + 3 * 0)] = -s6;
  Y[2 + 5 * (1 + 3 * 1)] = -s6;
  Y[2 + 5 * (2 + 3 * 2)] = s23;
  Y[3 + 5 * (0 + 3 * 2)] = -s2;
  Y[3 + 5 * (2 + 3 * 0)] = -s2;
  Y[4 + 5 * (0 + 3 * 0)] = s2;
  Y[4 + 5 * (1 + 3 * 1)] = -s2;
}

__device__ inline double kd(int i, int j) { return i == j ? 1.0 : 0.0; }

// eps_ijk x_k
__device__ inline double eps_x(int i, int j, const double* x) {
  const int k = 3 - i - j;
  if (i == j) return 0.0;
  const double s = ((j - i + 3) % 3 == 1) ? 1.0 : -1.0;  // (i, j, k) cyclic
  return s * x[k];
}

// Y2 projections of the rank-3 (c, I, J) and rank-4 tensors into the 60
// value slots (GH_TR, QQ_TR, tensors.f90:993-1023), added with weight w.
template <typename F3>
__device__ inline void add_gh(const double* Y, F3 t3, double w, double* out15) {
  for (int c = 0; c < 3; c++)
    for (int m = 0; m < 5; m++) {
      double s = 0.0;
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) s += t3(c, i, j) * Y[m + 5 * (i + 3 * j)];
      out15[5 * c + m] += w * s;
    }
}

template <typename F4>
__device__ inline void add_qq(const double* Y, F4 t4, double w, double* out15) {
  int q = 0;
  for (int x = 0; x < 5; x++)
    for (int y = x; y < 5; y++) {
      double s = 0.0;
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
          const double yx = Y[x + 5 * (i + 3 * j)];
          if (yx == 0.0) continue;
          for (int k = 0; k < 3; k++)
            for (int l = 0; l < 3; l++) s += yx * t4(i, j, k, l) * Y[y + 5 * (k + 3 * l)];
        }
      out15[q++] += w * s;
    }
}

// Yamakawa's overlapping-sphere pair blocks (YAMAKAWA_IJ, GRPY_YZD.f90:
// 768-786) as 60 values, valid for r <= a_i + a_j (r > 0).
__device__ inline void yamakawa60(const double R[3], double ai, double aj, const double* Y, double* v) {
  const double dist = sqrt(R[0] * R[0] + R[1] * R[1] + R[2] * R[2]);
  const double rw[3] = {R[0] / dist, R[1] / dist, R[2] / dist};
  const double abig = ai <= aj ? aj : ai, adiff = ai <= aj ? aj - ai : ai - aj;
  const bool inside = dist <= adiff;
  const double d = ai - aj, dist2 = dist * dist, dist3 = dist2 * dist;
  const double ai2 = ai * ai, aj2 = aj * aj, ai3 = ai2 * ai, aj3 = aj2 * aj;
  const int sym[6][2] = {{0, 0}, {0, 1}, {0, 2}, {1, 1}, {1, 2}, {2, 2}};
  // TT (YAMAKAWA_TT_IJ, 326-368) and RR (373-439): p_u delta + p_rr r r
  double tu, trr, ru, rrr;
  if (inside) {
    tu = 1.0 / 6.0 / abig;
    ru = 1.0 / 8.0 / (abig * abig * abig);
    trr = rrr = 0.0;
  } else {
    const double pre = 1.0 / (6 * 32 * ai * aj);
    tu = pre * (16 * (ai + aj) - (d * d + 3 * dist2) * (d * d + 3 * dist2) / dist3);
    trr = pre * 3 * (d * d - dist2) * (d * d - dist2) / dist3;
    const double prer = 1.0 / (8 * 64 * ai3 * aj3);
    ru = prer * (5 * dist3 - 27 * dist * (ai2 + aj2) + 32 * (ai3 + aj3) - 9 * (ai2 - aj2) * (ai2 - aj2) / dist -
                 d * d * d * d * (ai2 + 4 * ai * aj + aj2) / dist3);
    rrr = prer * 3 * (d * d - dist2) * (d * d - dist2) * ((ai2 + 4 * ai * aj + aj2) - dist2) / dist3;
  }
  for (int q = 0; q < 6; q++) {
    const int i = sym[q][0], j = sym[q][1];
    v[q] = tu * kd(i, j) + trr * rw[i] * rw[j];
    v[6 + q] = ru * kd(i, j) + rrr * rw[i] * rw[j];
  }
  // TR: YAMAKAWA_RT_IJ(-R, a_j, a_i) (467-500) transposed; with EPSR
  // antisymmetric that is f EPSR(r) for the swapped radii
  {
    const double I = aj, J = ai;  // the RT call's (aaI, aaJ)
    double f;
    if (I <= J && dist <= J - I) {
      f = 0.0;
    } else if (I > J && dist <= I - J) {
      f = dist / (8 * I * I * I);
    } else {
      const double s = (I - J) + dist;
      f = s * s * (J * J + 2 * J * (I + dist) - 3 * (I - dist) * (I - dist)) / (dist2 * 16 * 8 * I * I * I * J);
    }
    v[12] = f * rw[2];   // EPSR(0,1)
    v[13] = -f * rw[1];  // EPSR(0,2)
    v[14] = f * rw[0];   // EPSR(1,2)
  }
  for (int q = 15; q < 60; q++) v[q] = 0.0;
  // G: YAMAKAWA_TD_IJ (582-640), p_ur delta_ij r_k + p_rrr r_i r_j r_k
  {
    double pur = 0.0, prrr = 0.0;
    if (inside) {
      if (ai <= aj) pur = -3.0 * dist / (20.0 * aj3);
    } else {
      const double dist4 = dist2 * dist2, pre = 1.0 / (ai * aj3);
      pur = pre * (10.0 * dist2 - 24.0 * ai * dist + 15.0 * (ai2 - aj2) - d * d * d * d * d * (ai + 5.0 * aj) / dist4) /
            320.0;
      prrr = pre * (d * d - dist2) * (d * d - dist2) * (d * (ai + 5 * aj) - dist2) / (128.0 * dist4);
    }
    add_gh(Y, [&](int c, int i, int j) { return pur * kd(c, i) * rw[j] + prrr * rw[c] * rw[i] * rw[j]; }, 1.0, v + 30);
  }
  // H: YAMAKAWA_RD_IJ (512-553), f EPSR_ci r_j
  if (!inside) {
    const double f = -3.0 / (256.0 * ai3 * aj3 * dist3) * (d * d - dist2) * (d * d - dist2) *
                     ((ai2 + 4 * ai * aj + aj2) - dist2);
    add_gh(Y, [&](int c, int i, int j) { return eps_x(c, i, rw) * rw[j]; }, f, v + 45);
  }
  // QQ: YAMAKAWA_DD_IJ (665-766) over t4D0, t4D1 and t4D2 - t4D1
  {
    double c0, c1, c2;
    if (inside) {
      c0 = c1 = c2 = 3.0 / (abig * abig * abig * 20.0);
    } else {
      const double dist5 = dist3 * dist2, d4 = d * d * d * d, d6 = d4 * d * d;
      const double p6 = d6 * (ai2 + 6.0 * ai * aj + aj2) / dist5, p4 = d4 * (ai2 + 4.0 * ai * aj + aj2) / dist3;
      const double s1 = (ai2 - aj2) * (ai2 - aj2) / dist;
      c0 = 3.0 / (1280.0 * ai3 * aj3) * (3.0 * p6 - 10.0 * p4 + 32.0 * (ai3 + aj3) - 30.0 * (ai2 + aj2) * dist + 5.0 * dist3);
      c1 = 3.0 / (1280.0 * ai3 * aj3) *
           (-2.0 * p6 + 5.0 * p4 - 15.0 * s1 + 32.0 * (ai3 + aj3) - 25.0 * (ai2 + aj2) * dist + 5.0 * dist3);
      c2 = 3.0 / (2560.0 * ai3 * aj3) * (p6 - 30.0 * s1 + 64.0 * (ai3 + aj3) - 40.0 * (ai2 + aj2) * dist + 5.0 * dist3);
    }
    auto t4 = [&](int i, int j, int k, int l) {
      const double rrrr = rw[i] * rw[j] * rw[k] * rw[l];
      const double D0 = 1.5 * (rw[i] * rw[j] - kd(i, j) / 3.0) * (rw[k] * rw[l] - kd(k, l) / 3.0);
      const double D1 = 0.5 * (kd(j, l) * rw[i] * rw[k] + kd(i, k) * rw[j] * rw[l] + kd(j, k) * rw[i] * rw[l] +
                               kd(i, l) * rw[j] * rw[k] - 4.0 * rrrr);
      const double D2 = 0.5 * (kd(i, k) * kd(j, l) + kd(j, k) * kd(i, l) - kd(i, j) * kd(k, l) +
                               kd(k, l) * rw[i] * rw[j] + kd(i, j) * rw[k] * rw[l] - 3.0 * rrrr);
      return c0 * D0 + c1 * D1 + c2 * (D2 - D1);
    };
    add_qq(Y, t4, 1.0, v + 15);
  }
}

// The free-space pair of stokesian_Green.f90:11-109 as 60 values (see the
// file comment).
__device__ inline void free_space60(const double R[3], double ai, double aj, const double* Y, double* v) {
  const double r = sqrt(R[0] * R[0] + R[1] * R[1] + R[2] * R[2]), ir = 1.0 / r;
  double acc[RSD_NMOM_REAL];
  for (int m = 0; m < RSD_NMOM_REAL; m++) acc[m] = 0.0;
  rsd_real_image<double>(R[0], R[1], R[2], r, ir, 1.0, 0.0, 0.0, acc);
  rsd_real_epilogue<double>(acc, ai, aj, 1.0, v);
  const double na = 1.0 / (6.0 * ai), na3 = 1.0 / (6.0 * ai * ai * ai);
  for (int q = 0; q < 60; q++) {
    const bool a3 = (q >= 6 && q < 12) || (q >= 15 && q < 30) || q >= 45;
    v[q] *= a3 ? na3 : na;
  }
  const double ir7 = ir * ir * ir * ir * ir * ir * ir;
  const double wq = 3.0 / 8.0 * (ai * ai + aj * aj) * ir7, wh = -3.0 / 8.0 * aj * aj * ir7;
  add_qq(Y, [&](int i, int j, int k, int l) { return kd(i, k) * R[j] * R[l] + kd(j, k) * R[i] * R[l]; }, wq, v + 15);
  add_gh(Y, [&](int c, int i, int j) { return eps_x(c, i, R) * R[j]; }, wh, v + 45);
}

// The regularized pair blocks of Regular_ROTNE_PRAGER_IJ as 60 values, with
// kap = sqrt(pi) / 3 / |a_i + a_j - r| (Regularization.f90:78); at exact
// contact kap is infinite and the blocks are NaN, as in the reference.
__device__ inline void regular60(const double R[3], double ai, double aj, double* v) {
  const double r = sqrt(R[0] * R[0] + R[1] * R[1] + R[2] * R[2]), ir = 1.0 / r;
  const double kap = 1.77245385090551602730 / 3.0 / fabs((ai + aj) - r);
  const double Ed = 2.0 * 0.56418958354775628695 * kap * exp(-kap * kap * r * r);
  double acc[RSD_NMOM_REG];
  rsd_reg_image<double>(R[0], R[1], R[2], r, ir, erf(kap * r), Ed, kap, acc);
  rsd_reg_epilogue<double>(acc, ai, aj, v);
  const double na = 1.0 / (6.0 * ai), na3 = 1.0 / (6.0 * ai * ai * ai);
  for (int q = 0; q < 60; q++) {
    const bool a3 = (q >= 6 && q < 12) || (q >= 15 && q < 30) || q >= 45;
    v[q] *= a3 ? na3 : na;
  }
}

}  // namespace rsd_overlap

// The correction of overlap_Yamakawa_CORRECTION_IJ (method 1) or
// overlap_Regular_CORRECTION_IJ (method 2) as 60 values; R is the
// minimum-image separation x_i - x_j with 0 < |R| <= a_i + a_j.
__device__ inline void rsd_overlap_correction60(int method, const double R[3], double ai, double aj, double v[60]) {
  double Y[45], f[60];
  rsd_overlap::y2_basis(Y);
  if (method == 1)
    rsd_overlap::yamakawa60(R, ai, aj, Y, v);
  else
    rsd_overlap::regular60(R, ai, aj, v);
  rsd_overlap::free_space60(R, ai, aj, Y, f);
  for (int q = 0; q < 60; q++) v[q] -= f[q];
}
