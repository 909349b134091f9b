/*
 * rsd_oracle.c -- CPU oracle for the hydrodynamic step of regularized
 * Stokesian dynamics.  TEST INFRASTRUCTURE ONLY: it is the checker that the
 * CUDA path is compared against (tests/, __graft_entry__.smoke(), and the
 * cpu_baseline / reference arm of bench.py).  The product never links it.
 *
 * It restates, routine by routine and in the reference's operation order,
 * the Fortran of sherlockyzd/Regularized-Stokesian-Dynamics:
 *   src/tensors.f90         INIT_Y2 43-67, INIT_II 132-172, mulT* 357-431,
 *                           MAT_INV3 704-726, RTD_*_transY2 952-978,
 *                           DD_transY2 936-950, QQ_TR/GH_TR 993-1023
 *   src/csd_post.f90        PER_SKEW_CORRECTION 24-63, PERIOD_CORRECTION
 *                           65-102, SET_LATTICE_SKEW 105-136,
 *                           CALC_LATTICE_INVERSE 158-183
 *   src/Ewald_summation.f90 PER_ROTNE_PRAGER_SELF 19-191,
 *                           PER_ROTNE_PRAGER_IJ 196-423, helpers 427-1257
 *   src/per_GRPY_YZD.f90    PER_GRPERY_INV_FRI 13-200
 *   src/GRPY_YZD.f90        YAMAKAWA_*_IJ 326-786, overlap_*_CORRECTION_IJ
 *                           789-836 (correction methods 1 and 2)
 *   src/Regularization.f90  Regular_ROTNE_PRAGER_IJ 18-162, helpers 169-778
 *   src/stokesian_Green.f90 ROTNE_PRAGER_IJ_FTS 11-109
 *   src/tensors.f90         CALC_RR ... CALC_t4D2 182-440 (Yamakawa tensors)
 *   src/hydro_lub.f90       lubmxcalc 22-308, lubcalc 310-398,
 *                           lubtabcalc 400-525
 * Arrays are column-major like Fortran; indices are 0-based here.
 *
 * Parity status: the reference ships no tests.  The free-space pair tensor
 * chain, the Y2 projection and the SPD inversion are pinned against the
 * reference's own output table src/lubrication tabel/FarfieldForce/
 * tablefar.txt (equal-sphere rows) by tests/test_oracle_pins.py.  The
 * periodic Ewald sum, the lubrication assembly and the solve chain have no
 * reference outputs to pin against (parity unpinned for those parts); they
 * are restated from the source and checked by invariances.
 */
#include <math.h>
#include <stdio.h>
#include <string.h>
#include <stdlib.h>

#define PAI 3.141592653589793238462643383279502884
#define PIP5 0.564189583547756286948079451560772585844

#define I2(i, j) ((i) + 3 * (j))
#define I3(i, j, k) ((i) + 3 * (j) + 9 * (k))
#define I4(i, j, k, l) ((i) + 3 * (j) + 9 * (k) + 27 * (l))
#define IY(m, i, j) ((m) + 5 * ((i) + 3 * (j)))

/* ---------------------------------------------------------------- tensors */
static double KD[9], EPS[27], Y2[45], II[81], IIISO[81];
static int tensors_ready = 0;

/* INIT_KDirac, INIT_EPS, INIT_Y2 (Y21 = Y22 = Y2), INIT_II:
 * src/tensors.f90:1-67,132-172 */
static void init_tensors(void) {
  if (tensors_ready) return;
  memset(KD, 0, sizeof KD);
  KD[I2(0, 0)] = KD[I2(1, 1)] = KD[I2(2, 2)] = 1.0;
  memset(EPS, 0, sizeof EPS);
  EPS[I3(0, 1, 2)] = 1.0;
  EPS[I3(0, 2, 1)] = -1.0;
  EPS[I3(1, 0, 2)] = -1.0;
  EPS[I3(1, 2, 0)] = 1.0;
  EPS[I3(2, 0, 1)] = 1.0;
  EPS[I3(2, 1, 0)] = -1.0;
  memset(Y2, 0, sizeof Y2);
  Y2[IY(0, 0, 1)] = 1.0 / sqrt(2.0);
  Y2[IY(0, 1, 0)] = 1.0 / sqrt(2.0);
  Y2[IY(1, 1, 2)] = -1.0 / sqrt(2.0);
  Y2[IY(1, 2, 1)] = -1.0 / sqrt(2.0);
  Y2[IY(2, 0, 0)] = -1.0 / sqrt(6.0);
  Y2[IY(2, 1, 1)] = -1.0 / sqrt(6.0);
  Y2[IY(2, 2, 2)] = sqrt(2.0 / 3.0);
  Y2[IY(3, 0, 2)] = -1.0 / sqrt(2.0);
  Y2[IY(3, 2, 0)] = -1.0 / sqrt(2.0);
  Y2[IY(4, 0, 0)] = 1.0 / sqrt(2.0);
  Y2[IY(4, 1, 1)] = -1.0 / sqrt(2.0);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      for (int l = 0; l < 3; l++)
        for (int m = 0; m < 3; m++) {
          II[I4(i, j, l, m)] = (3.0 * KD[I2(i, m)] * KD[I2(j, l)] + 3.0 * KD[I2(i, l)] * KD[I2(j, m)] -
                                2.0 * KD[I2(i, j)] * KD[I2(l, m)]) / 6.0;
          IIISO[I4(i, j, l, m)] = (KD[I2(i, m)] * KD[I2(j, l)] + KD[I2(i, l)] * KD[I2(j, m)] +
                                   KD[I2(i, j)] * KD[I2(l, m)]);
        }
  tensors_ready = 1;
}

/* mulT2aT4T2b: src/tensors.f90:357-376 */
static double mul_t2a_t4_t2b(const double *t2a_m, const double *t4, const double *t2b_m) {
  /* t2a_m / t2b_m point at Y2 rows: element (i,j) is at [5*(i+3j)] */
  double a = 0.0;
  /* Fortran loop order: I outer ... L inner */
  for (int I = 0; I < 3; I++)
    for (int J = 0; J < 3; J++)
      for (int K = 0; K < 3; K++)
        for (int L = 0; L < 3; L++)
          a = a + t4[I4(I, J, K, L)] * t2a_m[5 * (I + 3 * J)] * t2b_m[5 * (K + 3 * L)];
  return a;
}

/* QQ_TR / DD_transY2: src/tensors.f90:936-950,993-1006 */
static void qq_tr(double B1[25], const double T4[81]) {
  for (int I = 0; I < 5; I++)
    for (int J = 0; J < 5; J++) B1[I + 5 * J] = mul_t2a_t4_t2b(&Y2[I], T4, &Y2[J]);
}

/* RTD_back_transY2 via mulT3T2_back: src/tensors.f90:402-417,952-964 */
static void gh_tr(double C1[15], const double T3[27]) {
  for (int m = 0; m < 5; m++) {
    double v[3] = {0, 0, 0};
    for (int I = 0; I < 3; I++)
      for (int J = 0; J < 3; J++)
        for (int c = 0; c < 3; c++) v[c] = v[c] + T3[I3(c, I, J)] * Y2[IY(m, I, J)];
    for (int c = 0; c < 3; c++) C1[c + 3 * m] = v[c];
  }
}

/* RTD_front_transY2 via mulT3T2_front: src/tensors.f90:419-431,966-978;
 * C1 is (5,3) */
static void rtd_front(double C1[15], const double T3[27]) {
  for (int m = 0; m < 5; m++) {
    double v[3] = {0, 0, 0};
    for (int I = 0; I < 3; I++)
      for (int J = 0; J < 3; J++)
        for (int c = 0; c < 3; c++) v[c] = v[c] + T3[I3(I, J, c)] * Y2[IY(m, I, J)];
    for (int c = 0; c < 3; c++) C1[m + 5 * c] = v[c];
  }
}

/* MAT_INV3: src/tensors.f90:704-726 */
void rsdo_mat_inv3(double LI[9], const double LR[9], double *det) {
#define A(i, j) LR[(i - 1) + 3 * (j - 1)]
  double d = A(1, 1) * A(2, 2) * A(3, 3) + A(1, 2) * A(2, 3) * A(3, 1) + A(1, 3) * A(2, 1) * A(3, 2) -
             A(1, 3) * A(2, 2) * A(3, 1) - A(2, 3) * A(3, 2) * A(1, 1) - A(3, 3) * A(1, 2) * A(2, 1);
#define L(i, j) LI[(i - 1) + 3 * (j - 1)]
  L(1, 1) = (1.0 / d) * (A(2, 2) * A(3, 3) - A(2, 3) * A(3, 2));
  L(1, 2) = (1.0 / d) * (A(1, 3) * A(3, 2) - A(1, 2) * A(3, 3));
  L(1, 3) = (1.0 / d) * (A(1, 2) * A(2, 3) - A(1, 3) * A(2, 2));
  L(2, 1) = (1.0 / d) * (A(2, 3) * A(3, 1) - A(2, 1) * A(3, 3));
  L(2, 2) = (1.0 / d) * (A(1, 1) * A(3, 3) - A(1, 3) * A(3, 1));
  L(2, 3) = (1.0 / d) * (A(1, 3) * A(2, 1) - A(1, 1) * A(2, 3));
  L(3, 1) = (1.0 / d) * (A(2, 1) * A(3, 2) - A(2, 2) * A(3, 1));
  L(3, 2) = (1.0 / d) * (A(1, 2) * A(3, 1) - A(1, 1) * A(3, 2));
  L(3, 3) = (1.0 / d) * (A(1, 1) * A(2, 2) - A(1, 2) * A(2, 1));
#undef A
#undef L
  *det = d;
}

/* ----------------------------------------------------------------- lattice */
typedef struct {
  double LR[9], LI[9], LV;
  double lammda, sig, logerr, phi;
  int NR, NI;
} rsdo_lattice;

/* Symmetric 3x3 eigenvalues by cyclic Jacobi rotations (the reference calls
 * LAPACK DSYTRD/DORGTR/DSTEQR through EIGEN, src/tensors.f90:679-698; only
 * the eigenvalues are used). */
static void eig3_sym(const double Ain[9], double ev[3]) {
  double a[3][3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) a[i][j] = Ain[i + 3 * j];
  for (int sweep = 0; sweep < 60; sweep++) {
    double off = fabs(a[0][1]) + fabs(a[0][2]) + fabs(a[1][2]);
    if (off == 0.0) break;
    for (int p = 0; p < 2; p++)
      for (int q = p + 1; q < 3; q++) {
        if (a[p][q] == 0.0) continue;
        double theta = (a[q][q] - a[p][p]) / (2.0 * a[p][q]);
        double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < 3; k++) {
          double akp = a[k][p], akq = a[k][q];
          a[k][p] = c * akp - s * akq;
          a[k][q] = s * akp + c * akq;
        }
        for (int k = 0; k < 3; k++) {
          double apk = a[p][k], aqk = a[q][k];
          a[p][k] = c * apk - s * aqk;
          a[q][k] = s * apk + c * aqk;
        }
      }
  }
  ev[0] = a[0][0];
  ev[1] = a[1][1];
  ev[2] = a[2][2];
}

/* SET_LATTICE_SKEW (steady shear branch): src/csd_post.f90:105-136 */
void rsdo_set_lattice_skew(double T, const double LB[3], double gamma, int oscillation, double gamma_alpha,
                           double frequency, double LR[9], double LI[9], double *LV) {
  memset(LR, 0, 9 * sizeof(double));
  LR[I2(0, 0)] = LB[0];
  LR[I2(1, 1)] = LB[1];
  LR[I2(2, 2)] = LB[2];
  if (oscillation) {
    double angle = gamma_alpha * sin(frequency * T);
    double lsh = angle * LB[2];
    LR[I2(0, 2)] = fmod(lsh, LB[0]);
  } else if (gamma != 0.0) {
    double tshear = LB[0] / (LB[2] * gamma);
    double tmod = fmod(T, tshear);
    LR[I2(0, 2)] = LB[2] * tmod * gamma;
  } else {
    LR[I2(0, 2)] = 0.0;
  }
  double det;
  rsdo_mat_inv3(LI, LR, &det);
  *LV = fabs(det);
}

/* CALC_LATTICE_INVERSE: src/csd_post.f90:158-183 */
void rsdo_calc_lattice_inverse(rsdo_lattice *lat, double ews_err, int nn, const double *radii) {
  lat->sig = pow(lat->LV, 1.0 / 3.0) / sqrt(2.0 * PAI);
  lat->lammda = sqrt(PAI) / pow(lat->LV, 1.0 / 3.0);
  lat->logerr = -log(ews_err);
  double MM[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      double s = 0.0;
      for (int k = 0; k < 3; k++) s += lat->LR[I2(k, i)] * lat->LR[I2(k, j)];
      MM[I2(i, j)] = s;
    }
  double le[3];
  eig3_sym(MM, le);
  double lmin = fmin(le[0], fmin(le[1], le[2]));
  double lmax = fmax(le[0], fmax(le[1], le[2]));
  double rnr = 2.0 * lat->logerr * (lat->sig * lat->sig) / lmin;
  lat->NR = (int)(sqrt(rnr) + 1);
  lmin = 1.0 / lmax;
  double rni = lat->logerr / (2.0 * (PAI * PAI) * (lat->sig * lat->sig) * lmin);
  lat->NI = (int)(sqrt(rni) + 1);
  double s3 = 0.0;
  for (int i = 0; i < nn; i++) s3 += radii[i] * radii[i] * radii[i];
  lat->phi = s3 * 4.0 / 3.0 * PAI / lat->LV;
}

/* PER_SKEW_CORRECTION: src/csd_post.f90:24-63 */
void rsdo_per_skew_correction(const double LR[9], const double LI[9], double R[3], double *dmin) {
  double X[3], RC[3], RMIN[3];
  for (int i = 0; i < 3; i++) X[i] = LI[I2(i, 0)] * R[0] + LI[I2(i, 1)] * R[1] + LI[I2(i, 2)] * R[2];
  for (int i = 0; i < 3; i++) {
    X[i] = fmod(X[i], 1.0);
    if (X[i] < 0.0) X[i] = X[i] + 1.0;
  }
  for (int i = 0; i < 3; i++) RC[i] = LR[I2(i, 0)] * X[0] + LR[I2(i, 1)] * X[1] + LR[I2(i, 2)] * X[2];
  double D0 = RC[0] * RC[0] + RC[1] * RC[1] + RC[2] * RC[2];
  for (int i = 0; i < 3; i++) RMIN[i] = RC[i];
  for (int m1 = 0; m1 <= 1; m1++)
    for (int m2 = 0; m2 <= 1; m2++)
      for (int m3 = 0; m3 <= 1; m3++) {
        if (m1 == 0 && m2 == 0 && m3 == 0) continue;
        double M[3] = {m1, m2, m3}, RL[3], d = 0.0;
        for (int i = 0; i < 3; i++) RL[i] = LR[I2(i, 0)] * M[0] + LR[I2(i, 1)] * M[1] + LR[I2(i, 2)] * M[2];
        for (int i = 0; i < 3; i++) d += (RC[i] - RL[i]) * (RC[i] - RL[i]);
        if (d < D0) {
          D0 = d;
          for (int i = 0; i < 3; i++) RMIN[i] = RC[i] - RL[i];
        }
      }
  for (int i = 0; i < 3; i++) R[i] = RMIN[i];
  *dmin = sqrt(D0);
}

/* PERIOD_CORRECTION (steady shear branch): src/csd_post.f90:65-102 */
void rsdo_period_correction(double R[3], const double LB[3], double T, double gamma, int oscillation,
                            double gamma_alpha, double frequency) {
  double lsh = oscillation ? gamma_alpha * sin(frequency * T) * LB[2] : LB[2] * gamma * T;
  if (R[2] > LB[2]) {
    R[2] = R[2] - LB[2];
    R[0] = fmod(R[0] - lsh, LB[0]);
  }
  if (R[2] < 0) {
    R[2] = R[2] + LB[2];
    R[0] = fmod(R[0] + lsh, LB[0]);
  }
  if (R[0] > LB[0])
    R[0] = R[0] - LB[0];
  else if (R[0] < 0)
    R[0] = R[0] + LB[0];
  if (R[1] > LB[1])
    R[1] = R[1] - LB[1];
  else if (R[1] < 0)
    R[1] = R[1] + LB[1];
}

/* ------------------------------------------------- Ewald helper chain */
/* src/Ewald_summation.f90:658-743 */
typedef struct {
  double lam;
} ewctx;

static void erfc_chain(double lam, double r, double e[7]) {
  double rlam2 = r * r * lam * lam;
  double E_def = 2.0 * PIP5 * lam * exp(-rlam2);
  double rlam4 = rlam2 * rlam2;
  e[0] = E_def;
  e[1] = -E_def;
  e[2] = 2.0 * lam * lam * r * E_def;
  e[3] = -2.0 * lam * lam * E_def * (2.0 * rlam2 - 1.0);
  e[4] = 4.0 * lam * lam * lam * lam * r * E_def * (2.0 * rlam2 - 3.0);
  e[5] = -4.0 * lam * lam * lam * lam * E_def * (4.0 * rlam4 - 12.0 * rlam2 + 3.0);
  e[6] = 8.0 * lam * lam * lam * lam * lam * lam * r * E_def * (4.0 * rlam4 - 20.0 * rlam2 + 15.0);
}

/* Init_kijl, Init_kijlm, Init_rijl, Init_rijlm: 748-804 */
static void init_kijl(const double *rn, double *k) {
  for (int l = 0; l < 3; l++)
    for (int j = 0; j < 3; j++)
      for (int i = 0; i < 3; i++)
        k[I3(i, j, l)] = KD[I2(i, j)] * rn[l] + KD[I2(i, l)] * rn[j] + KD[I2(j, l)] * rn[i];
}
static void init_kijlm(const double *rn, double *k) {
  for (int m = 0; m < 3; m++)
    for (int l = 0; l < 3; l++)
      for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++)
          k[I4(i, j, l, m)] = KD[I2(i, j)] * rn[l] * rn[m] + KD[I2(i, l)] * rn[j] * rn[m] +
                              KD[I2(j, l)] * rn[i] * rn[m] + KD[I2(i, m)] * rn[j] * rn[l] +
                              KD[I2(j, m)] * rn[i] * rn[l] + KD[I2(l, m)] * rn[i] * rn[j];
}
static void init_rijl(const double *rn, double *r) {
  for (int l = 0; l < 3; l++)
    for (int j = 0; j < 3; j++)
      for (int i = 0; i < 3; i++) r[I3(i, j, l)] = rn[l] * rn[j] * rn[i];
}
static void init_rijlm(const double *rn, double *r) {
  for (int m = 0; m < 3; m++)
    for (int l = 0; l < 3; l++)
      for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) r[I4(i, j, l, m)] = rn[l] * rn[j] * rn[i] * rn[m];
}

/* The erfc(lambda r)-derivative tensors: 808-1053 */
typedef struct {
  double DD[9], DDD[27], DDDD[81], D2, DD2[3], DDD2[9], DDDD2[27], DDDDD2[81], D4, DD4[3], DDD4[9];
} rerfc_t;

static void rerfc_tensors(double lam, const double *rn, double r, const double e[7], int want_odd, rerfc_t *o) {
  double erfcl = erfc(lam * r);
  double e1 = e[1], e2 = e[2], e3 = e[3], e4 = e[4], e5 = e[5], e6 = e[6];
  double r2 = r * r, r3 = r * r * r, r4 = r2 * r2, r5 = r3 * r2, r6 = r5 * r, r7 = r6 * r, r8 = r7 * r,
         r9 = r8 * r;
  double kl[27], rl[27], klm[81], rlm[81];
  init_kijlm(rn, klm);
  init_rijlm(rn, rlm);
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < 3; i++)
      o->DD[I2(i, j)] = (KD[I2(i, j)] / r - rn[i] * rn[j] / r3) * erfcl + (KD[I2(i, j)] + rn[i] * rn[j] / r2) * e1 +
                        rn[i] * rn[j] / r * e2;
  o->D2 = 2.0 / r * erfcl + 4.0 * e1 + r * e2;
  o->D4 = 12.0 / r * e2 + 8.0 * e3 + r * e4;
  for (int m = 0; m < 3; m++)
    for (int l = 0; l < 3; l++) {
      double kd = KD[I2(l, m)], rr = rn[l] * rn[m];
      o->DDD2[I2(l, m)] = (-2.0 * kd / r3 + 6.0 * rr / r5) * erfcl - (-2.0 * kd / r2 + 6.0 * rr / r4) * e1 +
                          (5.0 * kd / r - 3.0 * rr / r3) * e2 + (kd + 5.0 * rr / r2) * e3 + rr / r * e4;
      o->DDD4[I2(l, m)] = (-12.0 * kd / r3 + 36.0 * rr / r5) * e2 - (-12.0 * kd / r2 + 36.0 * rr / r4) * e3 +
                          (9.0 * kd / r + 3.0 * rr / r3) * e4 + (kd + 9.0 * rr / r2) * e5 + rr / r * e6;
    }
  for (int q = 0; q < 81; q++) {
    double ii = IIISO[q], k = klm[q], rr = rlm[q];
    o->DDDD[q] = (-ii / r3 + 3.0 * k / r5 - 15.0 * rr / r7) * erfcl - (-ii / r2 + 3.0 * k / r4 - 15.0 * rr / r6) * e1 +
                 (ii / r - 3.0 * rr / r5) * e2 + (k / r2 - 2.0 * rr / r4) * e3 + rr / r3 * e4;
    o->DDDDD2[q] = (6.0 * ii / r5 - 30.0 * k / r7 + 210.0 * rr / r9) * erfcl -
                   (6.0 * ii / r4 - 30.0 * k / r6 + 210.0 * rr / r8) * e1 +
                   (-3.0 * ii / r3 + 3.0 * k / r5 + 15.0 * rr / r7) * e2 +
                   (5.0 * ii / r2 - 13.0 * k / r4 + 55.0 * rr / r6) * e3 +
                   (ii / r + 4.0 * k / r3 - 25.0 * rr / r5) * e4 + (k / r2 + 2.0 * rr / r4) * e5 + rr / r3 * e6;
  }
  if (want_odd) {
    init_kijl(rn, kl);
    init_rijl(rn, rl);
    for (int q = 0; q < 27; q++) {
      double k = kl[q], rr = rl[q];
      o->DDD[q] = (-k / r3 + 3.0 * rr / r5) * erfcl - (-k / r2 + 3.0 * rr / r4) * e1 + k / r * e2 + rr / r2 * e3;
      o->DDDD2[q] = (6.0 * k / r5 - 30.0 * rr / r7) * erfcl - (6.0 * k / r4 - 30.0 * rr / r6) * e1 +
                    (-3.0 * k / r3 + 3.0 * rr / r5) * e2 + (5.0 * k / r2 - 13.0 * rr / r4) * e3 +
                    (k / r + 4.0 * rr / r3) * e4 + rr / r2 * e5;
    }
    for (int l = 0; l < 3; l++) {
      o->DD2[l] = -2.0 * rn[l] / r3 * erfcl + 2.0 * rn[l] / r2 * e1 + 5.0 * rn[l] / r * e2 + rn[l] * e3;
      o->DD4[l] = -12.0 * rn[l] / r3 * e2 + 12.0 * rn[l] / r2 * e3 + 9.0 * rn[l] / r * e4 + rn[l] * e5;
    }
  }
}

/* The J / Ror / Kr chain: 427-650 */
typedef struct {
  double Jr[9], D_Jr[27], DD_Jr[81], D2_Jr[9], DD2_Jr[27], DDD2_Jr[81];
  double Ror[9], D_Ror[27], D2_Ror[9], Kr[27], D_Kr[81], D2_Kr[27], DD2_Kr[81];
} jchain_t;

static void j_chain(const rerfc_t *t, int want_odd, jchain_t *c) {
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < 3; i++) {
      c->Jr[I2(i, j)] = KD[I2(i, j)] * t->D2 - t->DD[I2(i, j)];
      c->D2_Jr[I2(i, j)] = KD[I2(i, j)] * t->D4 - t->DDD2[I2(i, j)];
    }
  for (int l = 0; l < 3; l++)
    for (int m = 0; m < 3; m++)
      for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) {
          c->DD_Jr[I4(i, j, m, l)] = KD[I2(i, j)] * t->DDD2[I2(m, l)] - t->DDDD[I4(m, l, i, j)];
          c->DDD2_Jr[I4(i, j, m, l)] = KD[I2(i, j)] * t->DDD4[I2(m, l)] - t->DDDDD2[I4(m, l, i, j)];
        }
  /* Init_D_Ror */
  memset(c->D_Ror, 0, sizeof c->D_Ror);
  for (int m = 0; m < 3; m++)
    for (int n = 0; n < 3; n++)
      for (int l = 0; l < 3; l++)
        for (int j = 0; j < 3; j++)
          for (int i = 0; i < 3; i++)
            c->D_Ror[I3(i, j, l)] = c->D_Ror[I3(i, j, l)] - 0.5 * EPS[I3(j, m, n)] * c->DD_Jr[I4(i, n, l, m)];
  /* Init_D_Kr, Init_DD2_Kr */
  for (int l = 0; l < 3; l++)
    for (int k = 0; k < 3; k++)
      for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) {
          c->D_Kr[I4(i, j, k, l)] = 0.5 * (c->DD_Jr[I4(i, j, l, k)] + c->DD_Jr[I4(i, k, l, j)]);
          c->DD2_Kr[I4(i, j, k, l)] = 0.5 * (c->DDD2_Jr[I4(i, j, l, k)] + c->DDD2_Jr[I4(i, k, l, j)]);
        }
  if (!want_odd) return;
  for (int l = 0; l < 3; l++)
    for (int j = 0; j < 3; j++)
      for (int i = 0; i < 3; i++) {
        c->D_Jr[I3(i, j, l)] = KD[I2(i, j)] * t->DD2[l] - t->DDD[I3(l, i, j)];
        c->DD2_Jr[I3(i, j, l)] = KD[I2(i, j)] * t->DD4[l] - t->DDDD2[I3(l, i, j)];
      }
  memset(c->Ror, 0, sizeof c->Ror);
  memset(c->D2_Ror, 0, sizeof c->D2_Ror);
  for (int k = 0; k < 3; k++)
    for (int l = 0; l < 3; l++)
      for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) {
          c->Ror[I2(i, j)] = c->Ror[I2(i, j)] - 0.5 * EPS[I3(j, k, l)] * c->D_Jr[I3(i, l, k)];
          c->D2_Ror[I2(i, j)] = c->D2_Ror[I2(i, j)] - 0.5 * EPS[I3(j, k, l)] * c->DD2_Jr[I3(i, l, k)];
        }
  for (int k = 0; k < 3; k++)
    for (int j = 0; j < 3; j++)
      for (int i = 0; i < 3; i++) {
        c->Kr[I3(i, j, k)] = 0.5 * (c->D_Jr[I3(i, j, k)] + c->D_Jr[I3(i, k, j)]);
        c->D2_Kr[I3(i, j, k)] = 0.5 * (c->DD2_Jr[I3(i, j, k)] + c->DD2_Jr[I3(i, k, j)]);
      }
}

/* Fourier tensors: 1057-1257 */
typedef struct {
  double F_Jk[9], F_DJk[27], F_DDJk[81], F_D2Jk[9], F_DD2Jk[27];
  double F_Rk[9], F_DRk[27], F_D2Rk[9], F_Kk[27], F_DKk[81], F_D2Kk[27], F_DD2Kk[81];
} fchain_t;

static void f_chain(double lam, const double *kn, double dist, int want_odd, fchain_t *f) {
  double k2 = dist * dist, k4 = k2 * k2;
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < 3; i++)
      f->F_Jk[I2(i, j)] = (KD[I2(i, j)] * k2 - kn[i] * kn[j]) / k4 * 8.0 * PAI *
                          (1 + k2 / (4.0 * lam * lam) + k4 / (8.0 * lam * lam * lam * lam)) *
                          exp(-k2 / (4.0 * lam * lam));
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < 3; i++) f->F_D2Jk[I2(i, j)] = -dist * dist * f->F_Jk[I2(i, j)];
  for (int l = 0; l < 3; l++)
    for (int m = 0; m < 3; m++)
      for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) f->F_DDJk[I4(i, j, m, l)] = -kn[m] * kn[l] * f->F_Jk[I2(i, j)];
  memset(f->F_DRk, 0, sizeof f->F_DRk);
  for (int m = 0; m < 3; m++)
    for (int n = 0; n < 3; n++)
      for (int l = 0; l < 3; l++)
        for (int j = 0; j < 3; j++)
          for (int i = 0; i < 3; i++)
            f->F_DRk[I3(i, j, l)] = f->F_DRk[I3(i, j, l)] - 0.5 * EPS[I3(j, m, n)] * f->F_DDJk[I4(i, n, l, m)];
  for (int l = 0; l < 3; l++)
    for (int k = 0; k < 3; k++)
      for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) {
          f->F_DKk[I4(i, j, k, l)] = 0.5 * (f->F_DDJk[I4(i, j, l, k)] + f->F_DDJk[I4(i, k, l, j)]);
          f->F_DD2Kk[I4(i, j, k, l)] = kn[k] * kn[l] * dist * dist * f->F_Jk[I2(i, j)];
        }
  if (!want_odd) return;
  for (int l = 0; l < 3; l++)
    for (int j = 0; j < 3; j++)
      for (int i = 0; i < 3; i++) {
        f->F_DJk[I3(i, j, l)] = kn[l] * f->F_Jk[I2(i, j)];
        f->F_DD2Jk[I3(i, j, l)] = kn[l] * f->F_D2Jk[I2(i, j)];
      }
  memset(f->F_Rk, 0, sizeof f->F_Rk);
  memset(f->F_D2Rk, 0, sizeof f->F_D2Rk);
  for (int m = 0; m < 3; m++)
    for (int n = 0; n < 3; n++)
      for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) {
          f->F_Rk[I2(i, j)] = f->F_Rk[I2(i, j)] - 0.5 * EPS[I3(j, m, n)] * f->F_DJk[I3(i, n, m)];
          f->F_D2Rk[I2(i, j)] = f->F_D2Rk[I2(i, j)] - 0.5 * EPS[I3(j, m, n)] * f->F_DD2Jk[I3(i, n, m)];
        }
  for (int k = 0; k < 3; k++)
    for (int j = 0; j < 3; j++)
      for (int i = 0; i < 3; i++) {
        f->F_Kk[I3(i, j, k)] = 0.5 * (f->F_DJk[I3(i, j, k)] + f->F_DJk[I3(i, k, j)]);
        f->F_D2Kk[I3(i, j, k)] = f->F_DD2Jk[I3(i, j, k)];
      }
}

/* ------------------------------------------------ PER_ROTNE_PRAGER_SELF */
/* src/Ewald_summation.f90:19-191.  Outputs TTS(3,3), RRS(3,3), QQS_TR(5,5). */
void rsdo_per_rotne_prager_self(const rsdo_lattice *lat, double aaI, double TTS[9], double RRS[9],
                                double QQS_TR[25]) {
  init_tensors();
  const double lam = lat->lammda, phix = 1 - 0.2 * lat->phi, aaJ = aaI;
  const double nondim_a = 1.0 / (6.0 * aaI), nondim_a3 = 1.0 / (6.0 * aaI * aaI * aaI);
  double TTSA[9] = {0}, TTSB[9] = {0}, RRSA[9] = {0}, RRSB[9] = {0}, QQSA[81] = {0}, QQSB[81] = {0};
  rerfc_t t;
  jchain_t c;
  fchain_t f;
  const int NR = lat->NR, NI = lat->NI;
  for (int nx = -NR; nx <= NR; nx++)
    for (int ny = -NR; ny <= NR; ny++)
      for (int nz = -NR; nz <= NR; nz++) {
        if (nx == 0 && ny == 0 && nz == 0) continue;
        double NL[3] = {nx, ny, nz}, RN[3];
        for (int i = 0; i < 3; i++)
          RN[i] = lat->LR[I2(i, 0)] * NL[0] + lat->LR[I2(i, 1)] * NL[1] + lat->LR[I2(i, 2)] * NL[2];
        double dist = sqrt(RN[0] * RN[0] + RN[1] * RN[1] + RN[2] * RN[2]);
        double e[7];
        erfc_chain(lam, dist, e);
        rerfc_tensors(lam, RN, dist, e, 0, &t);
        j_chain(&t, 0, &c);
        for (int q = 0; q < 9; q++) {
          double TTSAA = 0.75 * aaI * c.Jr[q];
          double TTSAB = 0.75 * aaI * (aaI * aaI + aaJ * aaJ) / 6.0 * c.D2_Jr[q] * phix;
          TTSA[q] = TTSA[q] + (TTSAA + TTSAB);
        }
        double RRSAA[9] = {0};
        for (int k = 0; k < 3; k++)
          for (int l = 0; l < 3; l++)
            for (int j = 0; j < 3; j++)
              for (int i = 0; i < 3; i++)
                RRSAA[I2(i, j)] = RRSAA[I2(i, j)] + EPS[I3(i, k, l)] * c.D_Ror[I3(l, j, k)];
        for (int q = 0; q < 9; q++) RRSA[q] = RRSA[q] + 3.0 * aaI * aaI * aaI / 8.0 * RRSAA[q];
        for (int l = 0; l < 3; l++)
          for (int k = 0; k < 3; k++)
            for (int j = 0; j < 3; j++)
              for (int i = 0; i < 3; i++) {
                double QQSAA = 0.5 * (c.D_Kr[I4(i, k, l, j)] + c.D_Kr[I4(j, k, l, i)]);
                double QQSAB = 0.5 * (c.DD2_Kr[I4(i, k, l, j)] + c.DD2_Kr[I4(j, k, l, i)]);
                int q = I4(i, j, k, l);
                QQSA[q] = QQSA[q] - 3.0 / 4.0 * aaI * aaI * aaI * QQSAA -
                          3.0 / 40.0 * aaI * aaI * aaI * (aaI * aaI + aaJ * aaJ) * QQSAB;
              }
      }
  for (int nx = -NI; nx <= NI; nx++)
    for (int ny = -NI; ny <= NI; ny++)
      for (int nz = -NI; nz <= NI; nz++) {
        if (nx == 0 && ny == 0 && nz == 0) continue;
        double NL[3] = {nx, ny, nz}, KN[3];
        for (int j = 0; j < 3; j++)
          KN[j] = 2 * PAI * (NL[0] * lat->LI[I2(0, j)] + NL[1] * lat->LI[I2(1, j)] + NL[2] * lat->LI[I2(2, j)]);
        double dist = sqrt(KN[0] * KN[0] + KN[1] * KN[1] + KN[2] * KN[2]);
        f_chain(lam, KN, dist, 0, &f);
        for (int q = 0; q < 9; q++)
          TTSB[q] = TTSB[q] + 0.75 * aaI * f.F_Jk[q] + 1.0 / 8.0 * aaI * (aaI * aaI + aaJ * aaJ) * phix * f.F_D2Jk[q];
        double RRSBA[9] = {0};
        for (int k = 0; k < 3; k++)
          for (int l = 0; l < 3; l++)
            for (int j = 0; j < 3; j++)
              for (int i = 0; i < 3; i++)
                RRSBA[I2(i, j)] = RRSBA[I2(i, j)] + EPS[I3(i, k, l)] * f.F_DRk[I3(l, j, k)];
        for (int q = 0; q < 9; q++) RRSB[q] = RRSB[q] + 3.0 / 8.0 * aaI * aaI * aaI * RRSBA[q];
        for (int l = 0; l < 3; l++)
          for (int k = 0; k < 3; k++)
            for (int j = 0; j < 3; j++)
              for (int i = 0; i < 3; i++) {
                double QQSBA = 0.5 * (f.F_DKk[I4(i, k, l, j)] + f.F_DKk[I4(j, k, l, i)]);
                double QQSBB = 0.5 * (f.F_DD2Kk[I4(i, k, l, j)] + f.F_DD2Kk[I4(j, k, l, i)]);
                int q = I4(i, j, k, l);
                QQSB[q] = QQSB[q] - 3.0 / 4.0 * aaI * aaI * aaI * QQSBA -
                          3.0 / 40.0 * aaI * aaI * aaI * (aaI * aaI + aaJ * aaJ) * QQSBB;
              }
      }
  const double LV = lat->LV;
  double ttsr = (1.0 - 6.0 * lam / sqrt(PAI) * aaI + 40.0 / 3.0 / sqrt(PAI) * lam * lam * lam * aaI * aaI * aaI * phix);
  for (int q = 0; q < 9; q++) TTS[q] = (TTSA[q] + TTSB[q] / LV + ttsr * KD[q]) * nondim_a;
  double rrsr = (0.75 * (1.0 - 0.0 * lat->phi) - 10.0 / sqrt(PAI) * aaI * aaI * aaI * lam * lam * lam);
  for (int q = 0; q < 9; q++) RRS[q] = (rrsr * KD[q] + RRSA[q] + RRSB[q] / LV) * nondim_a3;
  double qqsr =
      (0.9 - lam * lam * lam * aaI * aaI * aaI / 25.0 / sqrt(PAI) * (50.0 - 126.0 * lam * lam * aaI * aaI) * 6.0);
  double QQS[81];
  for (int q = 0; q < 81; q++) QQS[q] = (QQSA[q] + QQSB[q] / LV + qqsr * II[q]) * nondim_a3;
  qq_tr(QQS_TR, QQS);
}

/* Test hook: see the comment at its use in rsdo_per_rotne_prager_ij. */
int rsdo_farfield_table_variant = 0;

/* -------------------------------------------------- PER_ROTNE_PRAGER_IJ */
/* src/Ewald_summation.f90:196-423.  Outputs TTP, RRP, TRP (3,3),
 * QQP_TR (5,5), GPQ_TR, HPQ_TR (3,5).  R is the minimum-image separation.
 * With include_k = 0 and NR = 0 and lam = 0 this is the free-space pair
 * (the n = 0 image of the unscreened sum). */
static void per_rotne_prager_ij_v(const rsdo_lattice *lat, const double R[3], double aaI, double aaJ,
                                  int include_k, int table_variant, double TTP[9], double RRP[9], double TRP[9],
                                  double QQP_TR[25], double GPQ_TR[15], double HPQ_TR[15]);
void rsdo_per_rotne_prager_ij(const rsdo_lattice *lat, const double R[3], double aaI, double aaJ, int include_k,
                              double TTP[9], double RRP[9], double TRP[9], double QQP_TR[25], double GPQ_TR[15],
                              double HPQ_TR[15]) {
  per_rotne_prager_ij_v(lat, R, aaI, aaJ, include_k, rsdo_farfield_table_variant, TTP, RRP, TRP, QQP_TR, GPQ_TR,
                        HPQ_TR);
}

static void per_rotne_prager_ij_v(const rsdo_lattice *lat, const double R[3], double aaI, double aaJ,
                                  int include_k, int table_variant, double TTP[9], double RRP[9], double TRP[9],
                                  double QQP_TR[25], double GPQ_TR[15], double HPQ_TR[15]) {
  init_tensors();
  const double lam = lat->lammda, phix = 1 - 0.2 * lat->phi;
  const double nondim_a = 1.0 / (6.0 * aaI), nondim_a3 = 1.0 / (6.0 * aaI * aaI * aaI);
  double TTPA[9] = {0}, TTPB[9] = {0}, RRPA[9] = {0}, RRPB[9] = {0}, QQPA[81] = {0}, QQPB[81] = {0};
  double GPQA[27] = {0}, HPQA[27] = {0}, GPQB[27] = {0}, HPQB[27] = {0}, TRPA[9] = {0}, TRPB[9] = {0};
  rerfc_t t;
  jchain_t c;
  fchain_t f;
  const int NR = lat->NR, NI = lat->NI;
  for (int nx = -NR; nx <= NR; nx++)
    for (int ny = -NR; ny <= NR; ny++)
      for (int nz = -NR; nz <= NR; nz++) {
        double NL[3] = {nx, ny, nz}, RN[3];
        for (int i = 0; i < 3; i++)
          RN[i] = R[i] + (lat->LR[I2(i, 0)] * NL[0] + lat->LR[I2(i, 1)] * NL[1] + lat->LR[I2(i, 2)] * NL[2]);
        double dist = sqrt(RN[0] * RN[0] + RN[1] * RN[1] + RN[2] * RN[2]);
        double e[7];
        erfc_chain(lam, dist, e);
        rerfc_tensors(lam, RN, dist, e, 1, &t);
        j_chain(&t, 1, &c);
        if (table_variant) {
          /* The generator of the reference's tablefar.txt (FarfieldForce/
           * tools.f90 Init_DDD2_Jg) writes the delta_ij x_k x_l / r^7 term
           * of the free-space fourth derivative with the opposite sign
           * from Ewald_summation.f90's chain; reproduce it to pin the rest
           * of the machinery against that table. */
          double r7 = dist * dist * dist * dist * dist * dist * dist;
          for (int l = 0; l < 3; l++)
            for (int k = 0; k < 3; k++)
              for (int i = 0; i < 3; i++) c.DD2_Kr[I4(i, i, k, l)] += -60.0 * RN[k] * RN[l] / r7;
        }
        for (int q = 0; q < 9; q++) {
          double TTPAA = 0.75 * aaI * c.Jr[q];
          double TTPAB = 0.75 * aaI * (aaI * aaI + aaJ * aaJ) / 6.0 * c.D2_Jr[q] * phix;
          TTPA[q] = TTPA[q] + (TTPAA + TTPAB);
        }
        double RRPAA[9] = {0};
        for (int k = 0; k < 3; k++)
          for (int l = 0; l < 3; l++)
            for (int j = 0; j < 3; j++)
              for (int i = 0; i < 3; i++)
                RRPAA[I2(i, j)] = RRPAA[I2(i, j)] + EPS[I3(i, k, l)] * c.D_Ror[I3(l, j, k)];
        for (int q = 0; q < 9; q++) RRPA[q] = RRPA[q] + 3.0 * aaI * aaI * aaI / 8.0 * RRPAA[q];
        for (int l = 0; l < 3; l++)
          for (int k = 0; k < 3; k++)
            for (int j = 0; j < 3; j++)
              for (int i = 0; i < 3; i++) {
                double QQPAA = 0.5 * (c.D_Kr[I4(i, k, l, j)] + c.D_Kr[I4(j, k, l, i)]);
                double QQPAB = 0.5 * (c.DD2_Kr[I4(i, k, l, j)] + c.DD2_Kr[I4(j, k, l, i)]);
                int q = I4(i, j, k, l);
                QQPA[q] = QQPA[q] - 3.0 / 4.0 * aaI * aaI * aaI * QQPAA -
                          3.0 / 40.0 * aaI * aaI * aaI * (aaI * aaI + aaJ * aaJ) * QQPAB;
              }
        for (int q = 0; q < 27; q++) {
          double GPQAA = c.Kr[q] + (aaI * aaI / 6.0 + 0.1 * aaJ * aaJ) * c.D2_Kr[q];
          GPQA[q] = GPQA[q] - 0.75 * aaI * GPQAA;
        }
        double HPQAA[27] = {0};
        for (int l = 0; l < 3; l++)
          for (int m = 0; m < 3; m++)
            for (int k = 0; k < 3; k++)
              for (int j = 0; j < 3; j++)
                for (int i = 0; i < 3; i++)
                  HPQAA[I3(i, j, k)] = HPQAA[I3(i, j, k)] + EPS[I3(i, l, m)] * (c.D_Kr[I4(m, j, k, l)] +
                                                                              0.1 * aaJ * aaJ * c.DD2_Kr[I4(m, j, k, l)]);
        for (int q = 0; q < 27; q++) HPQA[q] = HPQA[q] - 3.0 / 8.0 * aaI * aaI * aaI * HPQAA[q];
        for (int q = 0; q < 9; q++) {
          double TRPAA = aaI * (3.0 / 4.0) * c.Ror[q] + aaI * aaI * aaI / 8.0 * c.D2_Ror[q];
          TRPA[q] = TRPA[q] + TRPAA;
        }
      }
  if (include_k) {
    for (int nx = -NI; nx <= NI; nx++)
      for (int ny = -NI; ny <= NI; ny++)
        for (int nz = -NI; nz <= NI; nz++) {
          if (nx == 0 && ny == 0 && nz == 0) continue;
          double NL[3] = {nx, ny, nz}, KN[3];
          for (int j = 0; j < 3; j++)
            KN[j] = 2 * PAI * (NL[0] * lat->LI[I2(0, j)] + NL[1] * lat->LI[I2(1, j)] + NL[2] * lat->LI[I2(2, j)]);
          double dist = sqrt(KN[0] * KN[0] + KN[1] * KN[1] + KN[2] * KN[2]);
          f_chain(lam, KN, dist, 1, &f);
          double kr = KN[0] * R[0] + KN[1] * R[1] + KN[2] * R[2];
          double ck = cos(kr), sk = sin(kr);
          for (int q = 0; q < 9; q++) {
            double TTPBA = 0.75 * aaI * f.F_Jk[q];
            double TTPBB = 0.75 * aaI * (aaI * aaI + aaJ * aaJ) / 6.0 * f.F_D2Jk[q] * phix;
            TTPB[q] = TTPB[q] + (TTPBA + TTPBB) * ck;
          }
          double RRPBA[9] = {0};
          for (int k = 0; k < 3; k++)
            for (int l = 0; l < 3; l++)
              for (int j = 0; j < 3; j++)
                for (int i = 0; i < 3; i++)
                  RRPBA[I2(i, j)] = RRPBA[I2(i, j)] + EPS[I3(i, k, l)] * f.F_DRk[I3(l, j, k)];
          for (int q = 0; q < 9; q++) RRPB[q] = RRPB[q] + 3.0 / 8.0 * aaI * aaI * aaI * RRPBA[q] * ck;
          for (int l = 0; l < 3; l++)
            for (int k = 0; k < 3; k++)
              for (int j = 0; j < 3; j++)
                for (int i = 0; i < 3; i++) {
                  double QQPBA = 0.5 * (f.F_DKk[I4(i, k, l, j)] + f.F_DKk[I4(j, k, l, i)]);
                  double QQPBB = 0.5 * (f.F_DD2Kk[I4(i, k, l, j)] + f.F_DD2Kk[I4(j, k, l, i)]);
                  int q = I4(i, j, k, l);
                  QQPB[q] = QQPB[q] + (-3.0 / 4.0 * aaI * aaI * aaI * QQPBA -
                                       3.0 / 40.0 * aaI * aaI * aaI * (aaI * aaI + aaJ * aaJ) * QQPBB) * ck;
                }
          for (int q = 0; q < 27; q++) {
            double GPQBA = f.F_Kk[q] + (aaI * aaI / 6.0 + 0.1 * aaJ * aaJ) * f.F_D2Kk[q];
            GPQB[q] = GPQB[q] + 0.75 * aaI * GPQBA * sk;
          }
          double HPQBA[27] = {0};
          for (int l = 0; l < 3; l++)
            for (int m = 0; m < 3; m++)
              for (int k = 0; k < 3; k++)
                for (int j = 0; j < 3; j++)
                  for (int i = 0; i < 3; i++)
                    HPQBA[I3(i, j, k)] = HPQBA[I3(i, j, k)] +
                                         EPS[I3(i, l, m)] * (f.F_DKk[I4(m, j, k, l)] + 0.1 * aaJ * aaJ * f.F_DD2Kk[I4(m, j, k, l)]);
          for (int q = 0; q < 27; q++) HPQB[q] = HPQB[q] - 3.0 / 8.0 * aaI * aaI * aaI * HPQBA[q] * ck;
          for (int q = 0; q < 9; q++) {
            double TRPBA = aaI * (3.0 / 4.0) * f.F_Rk[q] + aaI * aaI * aaI / 8.0 * f.F_D2Rk[q];
            TRPB[q] = TRPB[q] - TRPBA * sk;
          }
        }
  }
  const double LV = include_k ? lat->LV : 1.0;
  double QQP[81], GPQ[27], HPQ[27];
  for (int q = 0; q < 9; q++) {
    TTP[q] = (TTPA[q] + TTPB[q] / LV) * nondim_a;
    RRP[q] = (RRPA[q] + RRPB[q] / LV) * nondim_a3;
    TRP[q] = (TRPA[q] + TRPB[q] / LV) * nondim_a;
  }
  for (int q = 0; q < 81; q++) QQP[q] = (QQPA[q] + QQPB[q] / LV) * nondim_a3;
  for (int q = 0; q < 27; q++) {
    GPQ[q] = (GPQA[q] + GPQB[q] / LV) * nondim_a;
    HPQ[q] = (HPQA[q] + HPQB[q] / LV) * nondim_a3;
  }
  gh_tr(GPQ_TR, GPQ);
  gh_tr(HPQ_TR, HPQ);
  qq_tr(QQP_TR, QQP);
}

/* ------------------------------------------------ overlap corrections */
/* Unit-vector tensors of the Yamakawa forms, src/tensors.f90:182-440:
 * CALC_RR (RR_ij = r_i r_j), CALC_EPSR (EPSR_ij = eps_ijk r_k), CALC_UR
 * (UR_ijk = delta_ij r_k), CALC_RRR, CALC_EPSRR (EPSR_ij r_k), and the
 * rank-4 CALC_t4D0 = 3/2 (RR - I/3)(RR - I/3),
 * CALC_t4D1 = 1/2 (d_jl r_i r_k + d_ik r_j r_l + d_jk r_i r_l + d_il r_j r_k
 *                  - 4 r_i r_j r_k r_l),
 * CALC_t4D2 = 1/2 (d_ik d_jl + d_jk d_il - d_ij d_kl + d_kl r_i r_j
 *                  + d_ij r_k r_l - 3 r_i r_j r_k r_l)
 * (the index pairs as t2at2b_t4 + t4trans build them, 443-560). */
typedef struct {
  double RR[9], EPSR[9], UR[27], RRR[27], EPSRR[27], D0[81], D1[81], D2[81];
} yk_tensors_t;

static void yk_tensors(const double R[3], double *dist, yk_tensors_t *t) {
  init_tensors();
  const double d = sqrt(R[0] * R[0] + R[1] * R[1] + R[2] * R[2]);
  const double rw[3] = {R[0] / d, R[1] / d, R[2] / d};
  *dist = d;
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < 3; i++) t->RR[I2(i, j)] = rw[i] * rw[j];
  memset(t->EPSR, 0, sizeof t->EPSR);
  t->EPSR[I2(0, 1)] = rw[2];
  t->EPSR[I2(1, 2)] = rw[0];
  t->EPSR[I2(2, 0)] = rw[1];
  t->EPSR[I2(1, 0)] = -rw[2];
  t->EPSR[I2(2, 1)] = -rw[0];
  t->EPSR[I2(0, 2)] = -rw[1];
  for (int k = 0; k < 3; k++)
    for (int j = 0; j < 3; j++)
      for (int i = 0; i < 3; i++) {
        t->UR[I3(i, j, k)] = KD[I2(i, j)] * rw[k];
        t->RRR[I3(i, j, k)] = rw[i] * rw[j] * rw[k];
        t->EPSRR[I3(i, j, k)] = t->EPSR[I2(i, j)] * rw[k];
      }
  for (int l = 0; l < 3; l++)
    for (int k = 0; k < 3; k++)
      for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) {
          const double rrrr = rw[i] * rw[j] * rw[k] * rw[l];
          const int q = I4(i, j, k, l);
          t->D0[q] = 1.5 * (t->RR[I2(i, j)] - KD[I2(i, j)] / 3.0) * (t->RR[I2(k, l)] - KD[I2(k, l)] / 3.0);
          t->D1[q] = 0.5 * (KD[I2(j, l)] * rw[i] * rw[k] + KD[I2(i, k)] * rw[j] * rw[l] +
                            KD[I2(j, k)] * rw[i] * rw[l] + KD[I2(i, l)] * rw[j] * rw[k] - 4.0 * rrrr);
          t->D2[q] = 0.5 * (KD[I2(i, k)] * KD[I2(j, l)] + KD[I2(j, k)] * KD[I2(i, l)] -
                            KD[I2(i, j)] * KD[I2(k, l)] + KD[I2(k, l)] * rw[i] * rw[j] +
                            KD[I2(i, j)] * rw[k] * rw[l] - 3.0 * rrrr);
        }
}

/* YAMAKAWA_TT_IJ, src/GRPY_YZD.f90:326-368: both radius orders use the same
 * form outside; inside the larger sphere the larger sphere's mobility. */
static void yamakawa_tt(const double R[3], double aaI, double aaJ, double A1[9]) {
  yk_tensors_t t;
  double dist;
  yk_tensors(R, &dist, &t);
  const double abig = aaI <= aaJ ? aaJ : aaI, adiff = aaI <= aaJ ? aaJ - aaI : aaI - aaJ;
  if (dist <= adiff) {
    for (int q = 0; q < 9; q++) A1[q] = 1.0 / 6.0 / abig * KD[q];
    return;
  }
  const double dist2 = dist * dist, dist3 = dist2 * dist, d = aaI - aaJ;
  const double pre = 1.0 / (6 * 32 * aaI * aaJ);
  const double pu = 16 * (aaI + aaJ) - (d * d + 3 * dist2) * (d * d + 3 * dist2) / dist3;
  const double prr = 3 * (d * d - dist2) * (d * d - dist2) / dist3;
  for (int q = 0; q < 9; q++) A1[q] = pre * (pu * KD[q] + prr * t.RR[q]);
}

/* YAMAKAWA_RR_IJ, src/GRPY_YZD.f90:373-439 */
static void yamakawa_rr(const double R[3], double aaI, double aaJ, double A1[9]) {
  yk_tensors_t t;
  double dist;
  yk_tensors(R, &dist, &t);
  const double abig = aaI <= aaJ ? aaJ : aaI, adiff = aaI <= aaJ ? aaJ - aaI : aaI - aaJ;
  if (dist <= adiff) {
    for (int q = 0; q < 9; q++) A1[q] = 1.0 / 8.0 / (abig * abig * abig) * KD[q];
    return;
  }
  const double dist2 = dist * dist, dist3 = dist2 * dist, d = aaI - aaJ;
  const double aI2 = aaI * aaI, aJ2 = aaJ * aaJ, aI3 = aI2 * aaI, aJ3 = aJ2 * aaJ;
  const double pre = 1.0 / (8 * 64 * aI3 * aJ3);
  const double pu = 5 * dist3 - 27 * dist * (aI2 + aJ2) + 32 * (aI3 + aJ3) - 9 * (aI2 - aJ2) * (aI2 - aJ2) / dist -
                    d * d * d * d * (aI2 + 4 * aaI * aaJ + aJ2) / dist3;
  const double prr = 3 * (d * d - dist2) * (d * d - dist2) * ((aI2 + 4 * aaI * aaJ + aJ2) - dist2) / dist3;
  for (int q = 0; q < 9; q++) A1[q] = pre * (pu * KD[q] + prr * t.RR[q]);
}

/* YAMAKAWA_RT_IJ, src/GRPY_YZD.f90:467-500 */
static void yamakawa_rt(const double R[3], double aaI, double aaJ, double A1[9]) {
  yk_tensors_t t;
  double dist;
  yk_tensors(R, &dist, &t);
  double f;
  if (aaI <= aaJ && dist <= aaJ - aaI) {
    f = 0.0;
  } else if (aaI > aaJ && dist <= aaI - aaJ) {
    f = dist / (8 * aaI * aaI * aaI);
  } else {
    const double pre = 1.0 / (16 * 8 * aaI * aaI * aaI * aaJ);
    const double s = (aaI - aaJ) + dist;
    f = pre * s * s * (aaJ * aaJ + 2 * aaJ * (aaI + dist) - 3 * (aaI - dist) * (aaI - dist)) / (dist * dist);
  }
  for (int q = 0; q < 9; q++) A1[q] = f * t.EPSR[q];
}

/* YAMAKAWA_RD_IJ, src/GRPY_YZD.f90:512-553 */
static void yamakawa_rd(const double R[3], double aaI, double aaJ, double C1[27]) {
  yk_tensors_t t;
  double dist;
  yk_tensors(R, &dist, &t);
  const double adiff = aaI <= aaJ ? aaJ - aaI : aaI - aaJ;
  if (dist <= adiff) {
    memset(C1, 0, sizeof(double) * 27);
    return;
  }
  const double dist2 = dist * dist, d = aaI - aaJ;
  const double f = -3.0 / (256.0 * aaI * aaI * aaI * aaJ * aaJ * aaJ * dist2 * dist) * (d * d - dist2) *
                   (d * d - dist2) * ((aaI * aaI + 4 * aaI * aaJ + aaJ * aaJ) - dist2);
  for (int q = 0; q < 27; q++) C1[q] = f * t.EPSRR[q];
}

/* YAMAKAWA_TD_IJ, src/GRPY_YZD.f90:582-640 */
static void yamakawa_td(const double R[3], double aaI, double aaJ, double C1[27]) {
  yk_tensors_t t;
  double dist;
  yk_tensors(R, &dist, &t);
  if (aaI <= aaJ && dist <= aaJ - aaI) {
    for (int q = 0; q < 27; q++) C1[q] = -3.0 * dist / (20.0 * aaJ * aaJ * aaJ) * t.UR[q];
    return;
  }
  if (aaI > aaJ && dist <= aaI - aaJ) {
    memset(C1, 0, sizeof(double) * 27);
    return;
  }
  const double dist2 = dist * dist, dist4 = dist2 * dist2, d = aaI - aaJ;
  const double pre = 1.0 / (aaI * aaJ * aaJ * aaJ);
  const double pur = (10.0 * dist2 - 24.0 * aaI * dist + 15.0 * (aaI * aaI - aaJ * aaJ) -
                      d * d * d * d * d * (aaI + 5.0 * aaJ) / dist4) / 320.0;
  const double prrr = (d * d - dist2) * (d * d - dist2) * (d * (aaI + 5 * aaJ) - dist2) / (128.0 * dist4);
  for (int q = 0; q < 27; q++) C1[q] = pre * (pur * t.UR[q] + prrr * t.RRR[q]);
}

/* YAMAKAWA_DD_IJ, src/GRPY_YZD.f90:665-766 (t4D2 is replaced by
 * t4D2 - t4D1 before either branch, 693) */
static void yamakawa_dd(const double R[3], double aaI, double aaJ, double B1[81]) {
  yk_tensors_t t;
  double dist;
  yk_tensors(R, &dist, &t);
  for (int q = 0; q < 81; q++) t.D2[q] = t.D2[q] - t.D1[q];
  const double abig = aaI <= aaJ ? aaJ : aaI, adiff = aaI <= aaJ ? aaJ - aaI : aaI - aaJ;
  if (dist <= adiff) {
    for (int q = 0; q < 81; q++) B1[q] = 3.0 / (abig * abig * abig * 20.0) * (t.D0[q] + t.D1[q] + t.D2[q]);
    return;
  }
  const double dist3 = dist * dist * dist, dist5 = dist3 * dist * dist, d = aaI - aaJ;
  const double aI2 = aaI * aaI, aJ2 = aaJ * aaJ, aI3 = aI2 * aaI, aJ3 = aJ2 * aaJ;
  const double d4 = d * d * d * d, d6 = d4 * d * d;
  const double c0 = 3.0 / (1280.0 * aI3 * aJ3) *
                    (+3.0 * d6 * (aI2 + 6.0 * aaI * aaJ + aJ2) / dist5 - 10.0 * d4 * (aI2 + 4.0 * aaI * aaJ + aJ2) / dist3 +
                     32.0 * (aI3 + aJ3) - 30.0 * (aI2 + aJ2) * dist + 5.0 * dist3);
  const double c1 = 3.0 / (1280.0 * aI3 * aJ3) *
                    (-2.0 * d6 * (aI2 + 6.0 * aaI * aaJ + aJ2) / dist5 + 5.0 * d4 * (aI2 + 4.0 * aaI * aaJ + aJ2) / dist3 -
                     15.0 * (aI2 - aJ2) * (aI2 - aJ2) / dist + 32.0 * (aI3 + aJ3) - 25.0 * (aI2 + aJ2) * dist +
                     5.0 * dist3);
  const double c2 = 3.0 / (2560.0 * aI3 * aJ3) *
                    (+d6 * (aI2 + 6.0 * aaI * aaJ + aJ2) / dist5 - 30.0 * (aI2 - aJ2) * (aI2 - aJ2) / dist +
                     64.0 * (aI3 + aJ3) - 40.0 * (aI2 + aJ2) * dist + 5.0 * dist3);
  for (int q = 0; q < 81; q++) B1[q] = c0 * t.D0[q] + c1 * t.D1[q] + c2 * t.D2[q];
}

/* YAMAKAWA_IJ, src/GRPY_YZD.f90:768-786: the overlapping-sphere pair
 * blocks (TR from the RT block of the swapped pair, transposed). */
void rsdo_yamakawa_ij(const double R[3], double aaI, double aaJ, double TTPY[9], double RRPY[9], double TRPY[9],
                      double QQPY_TR[25], double GPQY_TR[15], double HPQY_TR[15]) {
  init_tensors();
  yamakawa_tt(R, aaI, aaJ, TTPY);
  yamakawa_rr(R, aaI, aaJ, RRPY);
  const double mR[3] = {-R[0], -R[1], -R[2]};
  double RT0[9], G[27], H[27], Q[81];
  yamakawa_rt(mR, aaJ, aaI, RT0);
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < 3; i++) TRPY[I2(i, j)] = RT0[I2(j, i)];
  yamakawa_td(R, aaI, aaJ, G);
  yamakawa_rd(R, aaI, aaJ, H);
  yamakawa_dd(R, aaI, aaJ, Q);
  gh_tr(GPQY_TR, G);
  gh_tr(HPQY_TR, H);
  qq_tr(QQPY_TR, Q);
}

/* ROTNE_PRAGER_IJ_FTS, src/stokesian_Green.f90:11-109: the free-space
 * pair.  Its chain (Init_*_Jg, 215-433) is the unscreened one of
 * PER_ROTNE_PRAGER_IJ, except that Init_DDD2_Jg (295-312) writes the
 * delta_ij x_k x_l / r^7 term with the sign of the tablefar.txt generator:
 * the n = 0 image at lammda = 0 with that variant. */
void rsdo_rotne_prager_ij_fts(const double R[3], double aaI, double aaJ, double TTP[9], double RRP[9], double TRP[9],
                              double QQP_TR[25], double GPQ_TR[15], double HPQ_TR[15]) {
  rsdo_lattice fl;
  memset(&fl, 0, sizeof fl);
  fl.LV = 1.0;
  per_rotne_prager_ij_v(&fl, R, aaI, aaJ, 0, 1, TTP, RRP, TRP, QQP_TR, GPQ_TR, HPQ_TR);
}

/* The regularized potential of src/Regularization.f90, Phi'(r) = erf(kapa r):
 * Init_E_def / Init_erf1..5 (400-472, erf1..erf5 the derivatives of
 * erf(kapa r)), Init_DD_phir ... Init_DDD4_phir (552-778), into the
 * derivative tensors that the J chain (Init_Jr ... Init_DD2_Kr, 169-392,
 * the same steps as Ewald_summation.f90's) takes. */
static void rphi_tensors(double kapa, const double *rn, double r, rerfc_t *o) {
  const double rlam2 = r * r * kapa * kapa, rlam4 = rlam2 * rlam2;
  const double E_def = 2.0 * PIP5 * kapa * exp(-rlam2);
  const double f0 = erf(kapa * r), erf1 = E_def, erf2 = -2.0 * kapa * kapa * r * E_def;
  const double erf3 = 2.0 * kapa * kapa * E_def * (2.0 * rlam2 - 1.0);
  const double erf4 = -4.0 * kapa * kapa * kapa * kapa * r * E_def * (2.0 * rlam2 - 3.0);
  const double erf5 = 4.0 * kapa * kapa * kapa * kapa * E_def * (4.0 * rlam4 - 12.0 * rlam2 + 3.0);
  const double r2 = r * r, r3 = r2 * r, r4 = r2 * r2, r5 = r3 * r2, r6 = r5 * r, r7 = r6 * r, r8 = r7 * r,
               r9 = r8 * r;
  double kl[27], rl[27], klm[81], rlm[81];
  init_kijl(rn, kl);
  init_rijl(rn, rl);
  init_kijlm(rn, klm);
  init_rijlm(rn, rlm);
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < 3; i++)
      o->DD[I2(i, j)] = (KD[I2(i, j)] / r - rn[i] * rn[j] / r3) * f0 + rn[i] * rn[j] / r2 * erf1;
  o->D2 = 2.0 / r * f0 + erf1;
  o->D4 = 4.0 / r * erf2 + erf3;
  for (int l = 0; l < 3; l++) {
    o->DD2[l] = -2.0 * rn[l] / r3 * f0 + 2.0 * rn[l] / r2 * erf1 + rn[l] / r * erf2;
    o->DD4[l] = -4.0 * rn[l] / r3 * erf2 + 4.0 * rn[l] / r2 * erf3 + rn[l] / r * erf4;
  }
  for (int m = 0; m < 3; m++)
    for (int l = 0; l < 3; l++) {
      const double kd = KD[I2(l, m)], rr = rn[l] * rn[m];
      o->DDD2[I2(l, m)] = (-2.0 * kd / r3 + 6.0 * rr / r5) * f0 + (2.0 * kd / r2 - 6.0 * rr / r4) * erf1 +
                          (kd / r + rr / r3) * erf2 + rr / r2 * erf3;
      o->DDD4[I2(l, m)] = (-4.0 * kd / r3 + 12.0 * rr / r5) * erf2 + (4.0 * kd / r2 - 12.0 * rr / r4) * erf3 +
                          (kd / r + 3.0 * rr / r3) * erf4 + rr / r2 * erf5;
    }
  for (int q = 0; q < 27; q++) {
    const double k = kl[q], rr = rl[q];
    o->DDD[q] = (-k / r3 + 3.0 * rr / r5) * f0 + (k / r2 - 3.0 * rr / r4) * erf1 + rr / r3 * erf2;
    o->DDDD2[q] = (6.0 * k / r5 - 30.0 * rr / r7) * f0 + (-6.0 * k / r4 + 30.0 * rr / r6) * erf1 +
                  (k / r3 - 9.0 * rr / r5) * erf2 + (k / r2 - rr / r4) * erf3 + rr / r3 * erf4;
  }
  for (int q = 0; q < 81; q++) {
    const double ii = IIISO[q], k = klm[q], rr = rlm[q];
    o->DDDD[q] = (-ii / r3 + 3.0 * k / r5 - 15.0 * rr / r7) * f0 + (ii / r2 - 3.0 * k / r4 + 15.0 * rr / r6) * erf1 +
                 (k / r3 - 6.0 * rr / r5) * erf2 + rr / r4 * erf3;
    o->DDDDD2[q] = (6.0 * ii / r5 - 30.0 * k / r7 + 210.0 * rr / r9) * f0 +
                   (-6.0 * ii / r4 + 30.0 * k / r6 - 210.0 * rr / r8) * erf1 +
                   (ii / r3 - 9.0 * k / r5 + 75.0 * rr / r7) * erf2 + (ii / r2 - k / r4 - 5.0 * rr / r6) * erf3 +
                   (k / r3 - 4.0 * rr / r5) * erf4 + rr / r4 * erf5;
  }
}

/* Regular_ROTNE_PRAGER_IJ, src/Regularization.f90:18-162: the pair blocks
 * of the regularized Green's function with kapa = sqrt(pi)/3/|a_I + a_J -
 * r| (78), one image, the block formulas of PER_ROTNE_PRAGER_IJ's real sum
 * without the volume-fraction factor. */
void rsdo_regular_rotne_prager_ij(const double R[3], double aaI, double aaJ, double TTP[9], double RRP[9],
                                  double TRP[9], double QQP_TR[25], double GPQ_TR[15], double HPQ_TR[15]) {
  init_tensors();
  const double nondim_a = 1.0 / (6.0 * aaI), nondim_a3 = 1.0 / (6.0 * aaI * aaI * aaI);
  const double dist = sqrt(R[0] * R[0] + R[1] * R[1] + R[2] * R[2]);
  const double kapa = sqrt(PAI) / 3.0 / fabs((aaI + aaJ) - dist);
  rerfc_t t;
  jchain_t c;
  rphi_tensors(kapa, R, dist, &t);
  j_chain(&t, 1, &c);
  double QQP[81], GPQ[27], HPQ[27], RRPAA[9] = {0}, HPQAA[27] = {0};
  for (int q = 0; q < 9; q++)
    TTP[q] = (0.75 * aaI * c.Jr[q] + 0.75 * aaI * (aaI * aaI + aaJ * aaJ) / 6.0 * c.D2_Jr[q]) * nondim_a;
  for (int k = 0; k < 3; k++)
    for (int l = 0; l < 3; l++)
      for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) RRPAA[I2(i, j)] = RRPAA[I2(i, j)] + EPS[I3(i, k, l)] * c.D_Ror[I3(l, j, k)];
  for (int q = 0; q < 9; q++) RRP[q] = 3.0 * aaI * aaI * aaI / 8.0 * RRPAA[q] * nondim_a3;
  for (int l = 0; l < 3; l++)
    for (int k = 0; k < 3; k++)
      for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) {
          const double QQPAA = 0.5 * (c.D_Kr[I4(i, k, l, j)] + c.D_Kr[I4(j, k, l, i)]);
          const double QQPAB = 0.5 * (c.DD2_Kr[I4(i, k, l, j)] + c.DD2_Kr[I4(j, k, l, i)]);
          QQP[I4(i, j, k, l)] = (-3.0 / 4.0 * aaI * aaI * aaI * QQPAA -
                                 3.0 / 40.0 * aaI * aaI * aaI * (aaI * aaI + aaJ * aaJ) * QQPAB) * nondim_a3;
        }
  for (int q = 0; q < 27; q++)
    GPQ[q] = -0.75 * aaI * (c.Kr[q] + (aaI * aaI / 6.0 + 0.1 * aaJ * aaJ) * c.D2_Kr[q]) * nondim_a;
  for (int l = 0; l < 3; l++)
    for (int m = 0; m < 3; m++)
      for (int k = 0; k < 3; k++)
        for (int j = 0; j < 3; j++)
          for (int i = 0; i < 3; i++)
            HPQAA[I3(i, j, k)] = HPQAA[I3(i, j, k)] +
                                 EPS[I3(i, l, m)] * (c.D_Kr[I4(m, j, k, l)] + 0.1 * aaJ * aaJ * c.DD2_Kr[I4(m, j, k, l)]);
  for (int q = 0; q < 27; q++) HPQ[q] = -3.0 / 8.0 * aaI * aaI * aaI * HPQAA[q] * nondim_a3;
  for (int q = 0; q < 9; q++) TRP[q] = (aaI * (3.0 / 4.0) * c.Ror[q] + aaI * aaI * aaI / 8.0 * c.D2_Ror[q]) * nondim_a;
  gh_tr(GPQ_TR, GPQ);
  gh_tr(HPQ_TR, HPQ);
  qq_tr(QQP_TR, QQP);
}

/* overlap_Yamakawa_CORRECTION_IJ (method 1), src/GRPY_YZD.f90:789-811,
 * and overlap_Regular_CORRECTION_IJ (method 2), 813-836: Yamakawa's
 * overlapping-sphere blocks, or the regularized ones, minus the free-space
 * pair.  Returns -1 for another method, 0 otherwise. */
int rsdo_overlap_correction_ij(int method, const double R[3], double aaI, double aaJ, double TTPC[9],
                               double RRPC[9], double TRPC[9], double QQPC_TR[25], double GPQC_TR[15],
                               double HPQC_TR[15]) {
  if (method != 1 && method != 2) return -1;
  double TTY[9], RRY[9], TRY[9], QQY[25], GY[15], HY[15];
  double TT[9], RR[9], TR[9], QQ[25], G[15], H[15];
  if (method == 1)
    rsdo_yamakawa_ij(R, aaI, aaJ, TTY, RRY, TRY, QQY, GY, HY);
  else
    rsdo_regular_rotne_prager_ij(R, aaI, aaJ, TTY, RRY, TRY, QQY, GY, HY);
  rsdo_rotne_prager_ij_fts(R, aaI, aaJ, TT, RR, TR, QQ, G, H);
  for (int q = 0; q < 9; q++) {
    TTPC[q] = TTY[q] - TT[q];
    RRPC[q] = RRY[q] - RR[q];
    TRPC[q] = TRY[q] - TR[q];
  }
  for (int q = 0; q < 25; q++) QQPC_TR[q] = QQY[q] - QQ[q];
  for (int q = 0; q < 15; q++) {
    GPQC_TR[q] = GY[q] - G[q];
    HPQC_TR[q] = HY[q] - H[q];
  }
  return 0;
}

/* Scatter of one (alpha,beta) block and its mirror into grmobmx(11N,11N),
 * src/per_GRPY_YZD.f90:123-151,160-188 */
static void scatter_pair(double *G, long n11, int NN, int al, int be, const double *a, const double *b,
                         const double *c, const double *g, const double *h, const double *m) {
#define GM(r, q) G[(long)(r) + (long)(q) * n11]
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < 3; i++) {
      GM(3 * al + i, 3 * be + j) = a[I2(i, j)];
      GM(3 * al + i, 3 * NN + 3 * be + j) = b[I2(i, j)];
      GM(3 * NN + 3 * al + i, 3 * NN + 3 * be + j) = c[I2(i, j)];
      GM(3 * NN + 3 * be + j, 3 * al + i) = b[I2(i, j)];
    }
  for (int j = 0; j < 5; j++)
    for (int i = 0; i < 3; i++) {
      GM(3 * al + i, 6 * NN + 5 * be + j) = g[i + 3 * j];
      GM(3 * NN + 3 * al + i, 6 * NN + 5 * be + j) = h[i + 3 * j];
      GM(6 * NN + 5 * be + j, 3 * al + i) = g[i + 3 * j];
      GM(6 * NN + 5 * be + j, 3 * NN + 3 * al + i) = h[i + 3 * j];
    }
  for (int j = 0; j < 5; j++)
    for (int i = 0; i < 5; i++) GM(6 * NN + 5 * al + i, 6 * NN + 5 * be + j) = m[i + 5 * j];
#undef GM
}

/* PER_GRPERY_INV_FRI: src/per_GRPY_YZD.f90:13-200.  Writes the full
 * grand mobility grmobmx (11N x 11N, column-major) already divided by
 * (pi mu_f); APP/APQ/AQQ are its blocks.  lat must hold LR, LI, LV; the
 * routine fills lammda, NR, NI, phi exactly as CALC_LATTICE_INVERSE does.
 * correction_method 1 (Yamakawa) or 2 (regularized) adds its correction to
 * overlapping pairs; another nonzero method with an overlapping pair
 * returns the count of such pairs (positive) without applying one. */
int rsdo_per_grpery_inv_fri(int NN, const double *p_pos, const double *radii, rsdo_lattice *lat, double ews_err,
                            double mu_f, int correction_method, double *grmobmx) {
  init_tensors();
  rsdo_calc_lattice_inverse(lat, ews_err, NN, radii);
  const long n11 = 11L * NN;
  memset(grmobmx, 0, sizeof(double) * n11 * n11);
  int overl = 0;
#pragma omp parallel for schedule(static)
  for (int al = 0; al < NN; al++) {
    double TTS[9], RRS[9], QQS[25], zero9[9] = {0}, zero15[15] = {0};
    rsdo_per_rotne_prager_self(lat, radii[al], TTS, RRS, QQS);
    scatter_pair(grmobmx, n11, NN, al, al, TTS, zero9, RRS, zero15, zero15, QQS);
  }
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : overl)
  for (int al = 0; al < NN; al++) {
    for (int be = al + 1; be < NN; be++) {
      double R[3], dmin;
      for (int i = 0; i < 3; i++) R[i] = p_pos[3 * al + i] - p_pos[3 * be + i];
      rsdo_per_skew_correction(lat->LR, lat->LI, R, &dmin);
      double TTP[9], RRP[9], TRP[9], QQP[25], GPQ[15], HPQ[15];
      rsdo_per_rotne_prager_ij(lat, R, radii[al], radii[be], 1, TTP, RRP, TRP, QQP, GPQ, HPQ);
      /* per_GRPY_YZD.f90:98-116: the correction for pairs whose minimum
       * image overlaps (or touches), evaluated at the minimum image */
      if (correction_method != 0 && dmin <= radii[al] + radii[be]) {
        double TTC[9], RRC[9], TRC[9], QQC[25], GC[15], HC[15];
        if (rsdo_overlap_correction_ij(correction_method, R, radii[al], radii[be], TTC, RRC, TRC, QQC, GC, HC) == 0) {
          for (int q = 0; q < 9; q++) {
            TTP[q] += TTC[q];
            RRP[q] += RRC[q];
            TRP[q] += TRC[q];
          }
          for (int q = 0; q < 25; q++) QQP[q] += QQC[q];
          for (int q = 0; q < 15; q++) {
            GPQ[q] += GC[q];
            HPQ[q] += HC[q];
          }
        } else {
          overl++;
        }
      }
      double TRPm[9], GPQm[15];
      for (int q = 0; q < 9; q++) TRPm[q] = -TRP[q];
      for (int q = 0; q < 15; q++) GPQm[q] = -GPQ[q];
      scatter_pair(grmobmx, n11, NN, al, be, TTP, TRP, RRP, GPQ, HPQ, QQP);
      scatter_pair(grmobmx, n11, NN, be, al, TTP, TRPm, RRP, GPQm, HPQ, QQP);
    }
  }
  const double s = PAI * mu_f;
  for (long q = 0; q < n11 * n11; q++) grmobmx[q] = grmobmx[q] / s;
  return overl;
}

/* --------------------------------------------------------- lubrication */
typedef struct {
  int nabc, ngh, nm;
  double abc[64][11];
  double gh[64][7];
  double m[64][4];
} rsdo_lubtab;

/* readlubabc / readlubgh / readlubm: src/hydro_lub.f90:529-596 (one
 * header line, then whitespace-separated rows) */
static int read_table(const char *path, int ncol, int nrow, double *dst, int stride) {
  FILE *fp = fopen(path, "r");
  if (!fp) return -1;
  char line[1024];
  if (!fgets(line, sizeof line, fp)) {
    fclose(fp);
    return -1;
  }
  for (int r = 0; r < nrow; r++)
    for (int c = 0; c < ncol; c++)
      if (fscanf(fp, "%lf", &dst[r * stride + c]) != 1) {
        fclose(fp);
        return -1;
      }
  fclose(fp);
  return 0;
}

int rsdo_lubtab_load(rsdo_lubtab *t, const char *dir) {
  char p[2048];
  t->nabc = 39;
  t->ngh = 47;
  t->nm = 47;
  snprintf(p, sizeof p, "%s/r2babc.dat", dir);
  if (read_table(p, 11, t->nabc, &t->abc[0][0], 11)) return -1;
  snprintf(p, sizeof p, "%s/r2bgh.dat", dir);
  if (read_table(p, 7, t->ngh, &t->gh[0][0], 7)) return -1;
  snprintf(p, sizeof p, "%s/r2bm.dat", dir);
  if (read_table(p, 4, t->nm, &t->m[0][0], 4)) return -1;
  return 0;
}

int rsdo_lubtab_sizeof(void) { return (int)sizeof(rsdo_lubtab); }

/* lubcalc + lubtabcalc: src/hydro_lub.f90:310-525.  out[19] =
 * x11a x12a y11a y12a y11b y12b x11c x12c y11c y12c x11g x12g y11g y12g
 * y11h y12h xm ym zm */
void rsdo_lubcalc(const rsdo_lubtab *t, double r, double o[19]) {
  if (r < 2.1) {
    double xi = r - 2.0, invxi = 1.0 / xi, loginvxi = log(invxi), xiloginvxi = xi * loginvxi;
    o[0] = -1.23041 + 0.25 * invxi + 1.8918 * xi + 9.0 * loginvxi / 40.0 + 3.0 * xiloginvxi / 112.0;
    o[1] = -o[0] + 0.00312 - 0.0011 * xi;
    o[2] = -0.39394 + 0.95665 * xi + loginvxi / 6.0;
    o[3] = -o[2] + 0.004636 - 0.007049 * xi;
    o[4] = 0.408286 - 0.84055 * xi - loginvxi / 6.0 - xiloginvxi / 12.0;
    o[6] = 0.0479 + 0.12494 * xi - xiloginvxi / 6.0;
    o[7] = -o[6] + 0.016869 + 0.049536 * xi;
    o[8] = -0.605434 + 0.939139 * xi + 4.0 * loginvxi / 15.0 + 94.0 * xiloginvxi / 375.0;
    o[9] = loginvxi / 15.0 + 62.0 * xiloginvxi / 375.0 - 0.219032 + 0.332843 * xi;
    o[5] = -0.405978 + 0.833042 * xi + loginvxi / 6.0 + xiloginvxi / 12.0;
    o[10] = -1.16897 + 1.47882 * xi + invxi / 4.0 + 9.0 * loginvxi / 40.0 + 39.0 * xiloginvxi / 280.0;
    o[11] = -o[10] + 0.01 - 0.00167 * xi;
    o[12] = -0.2041 + 0.44226 * xi + loginvxi / 12.0 + xiloginvxi / 24.0;
    o[13] = -o[12] + 0.012265 - 0.02757 * xi;
    o[14] = -0.143777 + 0.264207 * xi + loginvxi / 30.0 + 137.0 * xiloginvxi / 1500.0;
    o[15] = -0.298166 + 0.534123 * xi + 2.0 * loginvxi / 15.0 + 113.0 * xiloginvxi / 1500.0;
    o[16] = invxi / 6.0 + 3.0 * loginvxi / 20.0 + 47.0 * xiloginvxi / 280.0 - 0.740815 + 0.706802 * xi;
    o[17] = -0.193518 + 0.553883 * xi + loginvxi / 12.0 - 29.0 * xiloginvxi / 500.0;
    o[18] = 0.00645755 - 0.021142 * xi;
    return;
  }
  for (int q = 0; q < 19; q++) o[q] = 0;
  for (int i = 0; i < t->nabc - 1; i++) {
    const double *a = t->abc[i], *b = t->abc[i + 1];
    if (a[0] <= r && b[0] > r) {
      for (int q = 0; q < 10; q++) o[q] = a[q + 1] + (r - a[0]) * (b[q + 1] - a[q + 1]) / (b[0] - a[0]);
      break;
    }
  }
  for (int i = 0; i < t->ngh - 1; i++) {
    const double *a = t->gh[i], *b = t->gh[i + 1];
    if (a[0] <= r && b[0] > r) {
      for (int q = 0; q < 6; q++) o[10 + q] = a[q + 1] + (r - a[0]) * (b[q + 1] - a[q + 1]) / (b[0] - a[0]);
      break;
    }
  }
  for (int i = 0; i < t->nm - 1; i++) {
    const double *a = t->m[i], *b = t->m[i + 1];
    if (a[0] <= r && b[0] > r) {
      for (int q = 0; q < 3; q++) o[16 + q] = (a[q + 1] + (r - a[0]) * (b[q + 1] - a[q + 1]) / (b[0] - a[0])) / 2.0;
      break;
    }
  }
}

/* lubmxcalc: src/hydro_lub.f90:22-308.  rfu (6N,6N), rfe (6N,5N),
 * rse (5N,5N), column-major, fully overwritten.  Returns the number of
 * pairs with s <= 2 (the reference prints "lubrication Contact Error" and
 * mirrors s to 4.00001 - s). */
int rsdo_lubmxcalc(int NN, int Nb, int is_period, const double *p_pos, const double *radii, const double LR[9],
                   const double LI[9], double mu_f, const rsdo_lubtab *tab, double *rfu, double *rfe, double *rse) {
  init_tensors();
  const long n6 = 6L * NN, n5 = 5L * NN;
  double *APPl = calloc(n6 * n6, sizeof(double));
  double *AQPl = calloc(n5 * n6, sizeof(double));
  double *AQQl = calloc(n5 * n5, sizeof(double));
#define P(r, c) APPl[(long)(r) + (long)(c) * n6]
#define QP(r, c) AQPl[(long)(r) + (long)(c) * n5]
#define QQ(r, c) AQQl[(long)(r) + (long)(c) * n5]
  int contacts = 0;
  for (int al = 0; al < NN; al++)
    for (int be = al + 1; be < NN; be++) {
      if (al + 1 > NN - Nb) continue;
      double rx[3], r;
      for (int i = 0; i < 3; i++) rx[i] = p_pos[3 * al + i] - p_pos[3 * be + i];
      r = sqrt(rx[0] * rx[0] + rx[1] * rx[1] + rx[2] * rx[2]);
      if (is_period) rsdo_per_skew_correction(LR, LI, rx, &r);
      double r_ave = 0.5 * (radii[al] + radii[be]), s = r / r_ave, o[19];
      if (s <= 2.0) {
        contacts++;
        s = 4.00001 - s;
        rsdo_lubcalc(tab, s, o);
      } else if (s > 4.0) {
        continue;
      } else {
        rsdo_lubcalc(tab, s, o);
      }
      const double x11a = o[0], x12a = o[1], y11a = o[2], y12a = o[3], y11b = o[4], y12b = o[5], x11c = o[6],
                   x12c = o[7], y11c = o[8], y12c = o[9], x11g = o[10], x12g = o[11], y11g = o[12],
                   y12g = o[13], y11h = o[14], y12h = o[15], xm = o[16], ym = o[17], zm = o[18];
      double e[3] = {rx[0] / r, rx[1] / r, rx[2] / r};
      double alub[2][2][9], blub[2][2][9], club[2][2][9], glub[2][2][27], hlub[2][2][27], mlub[81];
      for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) {
          double ee = e[i] * e[j], kd = KD[I2(i, j)];
          double pe = EPS[I3(i, j, 0)] * e[0] + EPS[I3(i, j, 1)] * e[1] + EPS[I3(i, j, 2)] * e[2];
          alub[0][0][I2(i, j)] = x11a * e[i] * e[j] + y11a * (kd - ee);
          alub[0][1][I2(i, j)] = x12a * e[i] * e[j] + y12a * (kd - ee);
          blub[0][0][I2(i, j)] = y11b * pe;
          blub[0][1][I2(i, j)] = y12b * pe;
          club[0][0][I2(i, j)] = x11c * e[i] * e[j] + y11c * (kd - ee);
          club[0][1][I2(i, j)] = x12c * e[i] * e[j] + y12c * (kd - ee);
        }
      for (int k = 0; k < 3; k++)
        for (int j = 0; j < 3; j++)
          for (int i = 0; i < 3; i++) {
            double t1 = (e[i] * e[j] - KD[I2(i, j)] / 3.0) * e[k];
            double t2 = (e[i] * KD[I2(j, k)] + e[j] * KD[I2(i, k)] - 2 * e[i] * e[j] * e[k]);
            glub[0][0][I3(i, j, k)] = x11g * t1 + y11g * t2;
            glub[0][1][I3(i, j, k)] = x12g * t1 + y12g * t2;
            double pik = EPS[I3(i, k, 0)] * e[0] + EPS[I3(i, k, 1)] * e[1] + EPS[I3(i, k, 2)] * e[2];
            double pjk = EPS[I3(j, k, 0)] * e[0] + EPS[I3(j, k, 1)] * e[1] + EPS[I3(j, k, 2)] * e[2];
            hlub[0][0][I3(i, j, k)] = y11h * (pik * e[j] + pjk * e[i]);
            hlub[0][1][I3(i, j, k)] = y12h * (pik * e[j] + pjk * e[i]);
          }
      for (int l = 0; l < 3; l++)
        for (int k = 0; k < 3; k++)
          for (int j = 0; j < 3; j++)
            for (int i = 0; i < 3; i++) {
#define kd(a, b) KD[I2(a, b)]
              mlub[I4(i, j, k, l)] =
                  xm * (3.0 * (e[i] * e[j] - kd(i, j) / 3.0) * (e[k] * e[l] - kd(k, l) / 3.0) / 2.0) +
                  ym * (e[i] * kd(j, l) * e[k] + e[j] * kd(i, l) * e[k] + e[i] * kd(j, k) * e[l] +
                        e[j] * kd(i, k) * e[l] - 4.0 * e[i] * e[j] * e[k] * e[l]) / 2.0 +
                  zm * (kd(i, k) * kd(j, l) + kd(j, k) * kd(i, l) - kd(i, j) * kd(k, l) + e[i] * e[j] * kd(k, l) +
                        kd(i, j) * e[k] * e[l] - e[i] * kd(j, l) * e[k] - e[j] * kd(i, l) * e[k] -
                        e[i] * kd(j, k) * e[l] - e[j] * kd(i, k) * e[l] + e[i] * e[j] * e[k] * e[l]) / 2.0;
#undef kd
            }
      for (int q = 0; q < 9; q++) {
        alub[1][1][q] = alub[0][0][q];
        alub[1][0][q] = alub[0][1][q];
        blub[1][1][q] = -blub[0][0][q];
        blub[1][0][q] = -blub[0][1][q];
        club[1][1][q] = club[0][0][q];
        club[1][0][q] = club[0][1][q];
      }
      for (int q = 0; q < 27; q++) {
        glub[1][1][q] = -glub[0][0][q];
        glub[1][0][q] = -glub[0][1][q];
        hlub[1][1][q] = hlub[0][0][q];
        hlub[1][0][q] = hlub[0][1][q];
      }
      double mmx[25];
      qq_tr(mmx, mlub);
      double gY[2][2][15], hY[2][2][15];
      for (int m = 0; m < 2; m++)
        for (int n = 0; n < 2; n++) {
          rtd_front(gY[m][n], glub[m][n]);
          rtd_front(hY[m][n], hlub[m][n]);
        }
      const int A = al, B = be, N3 = 3 * NN;
      for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) {
          P(3 * A + i, 3 * A + j) += alub[0][0][I2(i, j)];
          P(3 * B + i, 3 * B + j) += alub[1][1][I2(i, j)];
          P(N3 + 3 * A + i, N3 + 3 * A + j) += club[0][0][I2(i, j)];
          P(N3 + 3 * B + i, N3 + 3 * B + j) += club[1][1][I2(i, j)];
          P(N3 + 3 * A + i, 3 * A + j) += blub[0][0][I2(i, j)];
          P(N3 + 3 * B + i, 3 * B + j) += blub[1][1][I2(i, j)];
        }
      for (int j = 0; j < 3; j++)
        for (int i = 0; i < 5; i++) {
          QP(5 * A + i, 3 * A + j) += gY[0][0][i + 5 * j];
          QP(5 * B + i, 3 * B + j) += gY[1][1][i + 5 * j];
          QP(5 * A + i, N3 + 3 * A + j) += hY[0][0][i + 5 * j];
          QP(5 * B + i, N3 + 3 * B + j) += hY[1][1][i + 5 * j];
        }
      for (int j = 0; j < 5; j++)
        for (int i = 0; i < 5; i++) {
          QQ(5 * A + i, 5 * A + j) += mmx[i + 5 * j];
          QQ(5 * B + i, 5 * B + j) += mmx[i + 5 * j];
        }
      for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) {
          P(3 * A + i, 3 * B + j) += alub[0][1][I2(i, j)];
          P(N3 + 3 * A + i, N3 + 3 * B + j) += club[0][1][I2(i, j)];
          P(N3 + 3 * A + i, 3 * B + j) += blub[0][1][I2(i, j)];
          P(N3 + 3 * B + i, 3 * A + j) += blub[1][0][I2(i, j)];
        }
      for (int j = 0; j < 3; j++)
        for (int i = 0; i < 5; i++) {
          QP(5 * A + i, 3 * B + j) += gY[0][1][i + 5 * j];
          QP(5 * B + i, 3 * A + j) += gY[1][0][i + 5 * j];
          QP(5 * A + i, N3 + 3 * B + j) += hY[0][1][i + 5 * j];
          QP(5 * B + i, N3 + 3 * A + j) += hY[1][0][i + 5 * j];
        }
      for (int j = 0; j < 5; j++)
        for (int i = 0; i < 5; i++) {
          QQ(5 * A + i, 5 * B + j) += mmx[i + 5 * j];
          QQ(5 * B + i, 5 * A + j) += mmx[i + 5 * j];
        }
    }
  /* APPl(1:3N,3N+1:6N) = transpose(APPl(3N+1:6N,1:3N)); mirror upper */
  for (long c = 0; c < 3L * NN; c++)
    for (long r = 0; r < 3L * NN; r++) P(r, 3L * NN + c) = P(3L * NN + c, r);
  for (long i = 0; i < n6 - 1; i++)
    for (long j = i + 1; j < n6; j++) P(j, i) = P(i, j);
  const double s6 = 6.0, pm = PAI * mu_f;
  for (long q = 0; q < n6 * n6; q++) rfu[q] = APPl[q] * s6 * pm;
  for (long c = 0; c < n5; c++)
    for (long r = 0; r < n6; r++) rfe[r + c * n6] = QP(c, r) * s6 * pm;
  for (long q = 0; q < n5 * n5; q++) rse[q] = AQQl[q] * s6 * pm;
#undef P
#undef QP
#undef QQ
  free(APPl);
  free(AQPl);
  free(AQQl);
  return contacts;
}

/* Exported helpers for the tests: the Y2 projections and the isotropic
 * fourth-order tensor II (src/tensors.f90:132-172). */
void rsdo_qq_tr(double B1[25], const double T4[81]) {
  init_tensors();
  qq_tr(B1, T4);
}
void rsdo_gh_tr(double C1[15], const double T3[27]) {
  init_tensors();
  gh_tr(C1, T3);
}
void rsdo_rtd_front(double C1[15], const double T3[27]) {
  init_tensors();
  rtd_front(C1, T3);
}
void rsdo_tensor_II(double out[81]) {
  init_tensors();
  memcpy(out, II, sizeof II);
}
void rsdo_tensor_Y2(double out[45]) {
  init_tensors();
  memcpy(out, Y2, sizeof Y2);
}
int rsdo_lattice_sizeof(void) { return (int)sizeof(rsdo_lattice); }
