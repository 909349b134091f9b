// The fused step (STEPPER_Stokesian, src/stepper.f90:33-156) on the device:
// lattice -> grand mobility -> R_inf = M^-1 -> R = R_inf + R_lub -> RPP
// factorisation and solves -> velocities, stresslets -> explicit Euler step
// with the Lees-Edwards wrap -> relative viscosity.  Everything stays in HBM;
// the host sees only the lattice (a few scalars) and the outputs it asks for.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "rsd_internal.cuh"

namespace {

__global__ void axpy_block_k(int64_t rows, int64_t cols, const double* __restrict__ B, int64_t ldb,
                             double* __restrict__ A, int64_t lda) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= rows * cols) return;
  const int64_t i = t % rows, j = t / rows;
  A[i + j * lda] += B[i + j * ldb];
}

__global__ void fill_ein(int nn, const double* __restrict__ ei5, double* __restrict__ ein) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < 5 * nn) ein[t] = ei5[t % 5];
}

// averageU (src/matrices.f90:230-253): U_ave = sum_i (APP F)(3i) / N with
// F(3j) = 6 pi mu_f radii_test; out[0] accumulates sum_ij APP(3i,3j)
// Mh, Ml: the mixed form's M as FP32 planes (hi + lo, the half with row
// particle <= column particle stored); null for FP64 M
__global__ void sum_app_xx(int nn, const double* __restrict__ M, const float* __restrict__ Mh,
                           const float* __restrict__ Ml, int64_t ld, double* __restrict__ out) {
  __shared__ double red[256];
  double s = 0.0;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < (int64_t)nn * nn;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t % nn), j = (int)(t / nn);
    const int64_t o = 3 * i + (int64_t)(3 * j) * ld;
    const int64_t os = 3 * min(i, j) + (int64_t)(3 * max(i, j)) * ld;  // the stored half of the planes
    s += Mh ? (double)Mh[os] + (double)Ml[os] : M[o];
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int d = 128; d > 0; d >>= 1) {
    if (threadIdx.x < d) red[threadIdx.x] += red[threadIdx.x + d];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = red[0];
}

struct bg_flow {
  double UOE[9];  // omegaT + Eij (calc_uo_bg, csd_post.f90:507)
  double omega[3];
  double LB[3];
  double T, dt, gamma;
};

__device__ inline void period_correction(double R[3], const bg_flow& f) {
  // PERIOD_CORRECTION (csd_post.f90:65-102), steady shear
  const double lsh = f.LB[2] * f.gamma * f.T;
  if (R[2] > f.LB[2]) {
    R[2] = R[2] - f.LB[2];
    R[0] = fmod(R[0] - lsh, f.LB[0]);
  }
  if (R[2] < 0) {
    R[2] = R[2] + f.LB[2];
    R[0] = fmod(R[0] + lsh, f.LB[0]);
  }
  if (R[0] > f.LB[0])
    R[0] = R[0] - f.LB[0];
  else if (R[0] < 0)
    R[0] = R[0] + f.LB[0];
  if (R[1] > f.LB[1])
    R[1] = R[1] - f.LB[1];
  else if (R[1] < 0)
    R[1] = R[1] + f.LB[1];
}

// STEPPER_conf (stepper.f90:160-227) for the plain-particle case: U_pos =
// U_par + uo_bg(x); x += dt U_pos for i < nn - nb; LE wrap; U_pos recomputed
// with the wrapped positions.
__global__ void euler_update(int nn, int nb, bg_flow f, const double* __restrict__ U_par, double* __restrict__ conf,
                             double* __restrict__ U_pos) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nn) return;
  double x[3] = {conf[3 * i], conf[3 * i + 1], conf[3 * i + 2]};
  double up[3];
  for (int r = 0; r < 3; r++)
    up[r] = U_par[3 * i + r] + (f.UOE[r] * x[0] + f.UOE[r + 3] * x[1] + f.UOE[r + 6] * x[2]);
  if (i < nn - nb)
    for (int r = 0; r < 3; r++) x[r] = x[r] + f.dt * up[r];
  period_correction(x, f);
  for (int r = 0; r < 3; r++) {
    conf[3 * i + r] = x[r];
    U_pos[3 * i + r] = U_par[3 * i + r] + (f.UOE[r] * x[0] + f.UOE[r + 3] * x[1] + f.UOE[r + 6] * x[2]);
    U_pos[3 * nn + 3 * i + r] = U_par[3 * nn + 3 * i + r] + f.omega[r];
  }
}

// yetamu_solve (csd_post.f90:313-367): the three stresslet sums over
// S(5i+3) / (-2 EIN(5i+3))
__global__ void yeta_sums(int nn, const double* __restrict__ Sh, const double* __restrict__ Sfp,
                          const double* __restrict__ Sb, const double* __restrict__ ein, double* __restrict__ out) {
  __shared__ double r0[256], r1[256], r2[256];
  double a = 0, b = 0, c = 0;
  for (int i = threadIdx.x; i < nn; i += blockDim.x) {
    const double d = -2.0 * ein[5 * i + 3];
    const double fp = Sfp ? Sfp[5 * i + 3] : 0.0, bb = Sb ? Sb[5 * i + 3] : 0.0;
    a += (fp + Sh[5 * i + 3] + bb) / d;
    b += bb / d;
    c += fp / d;
  }
  r0[threadIdx.x] = a;
  r1[threadIdx.x] = b;
  r2[threadIdx.x] = c;
  __syncthreads();
  for (int d = 128; d > 0; d >>= 1) {
    if (threadIdx.x < d) {
      r0[threadIdx.x] += r0[threadIdx.x + d];
      r1[threadIdx.x] += r1[threadIdx.x + d];
      r2[threadIdx.x] += r2[threadIdx.x + d];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = r0[0];
    out[1] = r1[0];
    out[2] = r2[0];
  }
}

__global__ void nan_check(int64_t n, const double* __restrict__ v, int* __restrict__ flag) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n && !isfinite(v[t])) atomicExch(flag, 1);
}

}  // namespace

int rsd_axpy_block(rsd_ctx* ctx, int64_t rows, int64_t cols, const double* B, int64_t ldb, double* A, int64_t lda) {
  const int64_t tot = rows * cols;
  if (tot <= 0) return RSD_OK;
  axpy_block_k<<<(unsigned)((tot + 255) / 256), 256, 0, ctx->stream>>>(rows, cols, B, ldb, A, lda); RSD_LAUNCH_NOTE();
  RSD_CUDA(ctx, cudaGetLastError());
  return RSD_OK;
}

// INIT_u_bg (csd_post.f90:442-479) with EI_bg = 0 on input and steady shear:
// Eij(1,3) = Eij(3,1) = gamma/2, omega_bg = (0, gamma/2, 0).
static void background(double gamma, double Eij[9], double omega[3], double UOE[9]) {
  memset(Eij, 0, 9 * sizeof(double));
  Eij[0 + 3 * 2] = Eij[2 + 3 * 0] = gamma * 0.5;
  omega[0] = 0.0;
  omega[1] = gamma * 0.5;
  omega[2] = 0.0;
  auto eps = [](int i, int j, int k) { return (double)((i - j) * (j - k) * (k - i)) / 2.0; };
  for (int I = 0; I < 3; I++)
    for (int J = 0; J < 3; J++) {
      const double om = eps(J, I, 0) * omega[0] + eps(J, I, 1) * omega[1] + eps(J, I, 2) * omega[2];
      UOE[I + 3 * J] = om + Eij[I + 3 * J];
    }
}

static void ei5_of(const double E[9], double out[5]) {
  const double s2 = 1.0 / sqrt(2.0), s6 = 1.0 / sqrt(6.0), s23 = sqrt(2.0 / 3.0);
  double Y[5][9] = {{0}};
  Y[0][0 + 3 * 1] = Y[0][1 + 3 * 0] = s2;
  Y[1][1 + 3 * 2] = Y[1][2 + 3 * 1] = -s2;
  Y[2][0] = Y[2][4] = -s6;
  Y[2][8] = s23;
  Y[3][0 + 3 * 2] = Y[3][2 + 3 * 0] = -s2;
  Y[4][0] = s2;
  Y[4][4] = -s2;
  for (int m = 0; m < 5; m++) {
    double a = 0.0;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) a = a + E[i + 3 * j] * Y[m][i + 3 * j];
    out[m] = a;
  }
}

int rsd_mixed_solve(rsd_ctx* ctx, int nn, double* M, int64_t ld, const double* d_pos, const double* d_radii,
                    const rsd_lattice* lat, const rsd_lubtab* tab, const rsd_step_params* p, const double* ein,
                    const double* Fe, double* U_par, double* S_hyd, rsd_step_info* info, float* rpp_out = nullptr,
                    int64_t rpp_ld = 0);
int rsd_lp_pcg_internal(rsd_ctx* ctx, rsd_lp* net, int mode, int nn, const double* d_pos, const double* d_radii,
                        const rsd_lattice* lat, const double* d_rpp, int64_t ld, int nrhs, const double* d_b,
                        double* d_x, double tol, int maxit, int* iters, double* resid);

// The step; with rpp_out it stops once RPP = (M^-1)_PP + rfu is formed and
// copies it there (FP64 for the FP64 form, FP32 for the mixed form).
static int step_impl(rsd_ctx* ctx, const rsd_lubtab* tab, const rsd_step_params* p, double* d_conf,
                     const double* d_radii, const double* d_Fe, double* d_U_pos, double* d_SijN, double yeta_mu[5],
                     rsd_step_info* info, void* rpp_out, int64_t rpp_ld, rsd_lattice* lat_out) {
  if (!ctx || !p || !d_conf || !d_radii || (!rpp_out && (!d_U_pos || !d_SijN)) || p->nn < 1 || p->nb < 0 ||
      p->nb > p->nn || !(p->mu_f > 0) || !(p->ews_err > 0) || (p->use_lub && !tab))
    return rsd_fail(ctx, RSD_EARG, "rsd_stepper_stokesian_dev: bad arguments");
  if (p->precision != RSD_PREC_FP64 && p->precision != RSD_PREC_MIXED)
    return rsd_fail(ctx, RSD_EARG, "unknown precision %d", p->precision);
  RSD_TRY(rsd_set_device(ctx));
  cudaStream_t s = ctx->stream;
  const int nn = p->nn;
  const int64_t n = 11LL * nn, P = 6LL * nn, Q = 5LL * nn;
  rsd_step_info loc{};
  // lattice at the start of the step (STEPPER_Stokesian 54-56)
  rsd_lattice lat{};
  RSD_TRY(rsd_set_lattice_skew(p->T, p->LB, p->gamma, 0, 0.0, 0.0, &lat));
  std::vector<double> radii(nn);
  RSD_CUDA(ctx, cudaMemcpyAsync(radii.data(), d_radii, nn * sizeof(double), cudaMemcpyDeviceToHost, s));
  RSD_CUDA(ctx, cudaStreamSynchronize(s));
  RSD_TRY(rsd_calc_lattice_inverse(&lat, p->ews_err, nn, radii.data()));
  loc.NR = lat.NR;
  loc.NI = lat.NI;
  loc.phi = lat.phi;
  loc.LV = lat.LV;
  if (lat_out) *lat_out = lat;
  double* M = (double*)rsd_scratch(ctx, "step_M", sizeof(double) * n * n);
  double* V = (double*)rsd_scratch(ctx, "step_vec", sizeof(double) * (4 * P + 4 * Q + 1024));
  if (!M || !V) return RSD_ENOMEM;
  double* X = V;               // P x 2
  double* Upar = V;            // = X(:,0)
  double* ein = V + 2 * P;     // Q
  double* S = ein + Q;         // Q
  double* red = S + Q;         // 1024 scratch
  double* Fe = red + 1024;     // P
  double Eij[9], omega[3], UOE[9], ei5[5];
  background(p->gamma, Eij, omega, UOE);
  ei5_of(Eij, ei5);
  double* d_ei5 = red + 512;
  RSD_CUDA(ctx, cudaMemcpyAsync(d_ei5, ei5, sizeof ei5, cudaMemcpyHostToDevice, s));
  fill_ein<<<(unsigned)((Q + 255) / 256), 256, 0, s>>>(nn, d_ei5, ein); RSD_LAUNCH_NOTE();
  if (d_Fe)
    RSD_CUDA(ctx, cudaMemcpyAsync(Fe, d_Fe, sizeof(double) * P, cudaMemcpyDeviceToDevice, s));
  else
    RSD_CUDA(ctx, cudaMemsetAsync(Fe, 0, sizeof(double) * P, s));
  cudaEventRecord(ctx->ev[0], s);
  {
    // grand mobility
    rsd_range r("rsd_assembly");
    RSD_TRY(rsd_ewald_assemble(ctx, nn, d_conf, d_radii, &lat, p->mu_f, p->precision, M, n));
    if (ctx->correction_method) {  // overlap corrections (per_GRPY_YZD.f90:98-116)
      int nov = 0;
      RSD_TRY(rsd_count_overlaps(ctx, nn, d_conf, d_radii, &lat, &nov));
      RSD_TRY(rsd_overlap_correct(ctx, ctx->correction_method, p->precision, nn, d_conf, d_radii, &lat, p->mu_f, nov,
                                  M, n));
    }
  }
  cudaEventRecord(ctx->ev[1], s);
  // averageU on APP before it is overwritten
  const bool planes = p->precision == RSD_PREC_MIXED;
  const float* Mh = planes ? reinterpret_cast<const float*>(M) : nullptr;
  sum_app_xx<<<256, 256, 0, s>>>(nn, M, Mh, planes ? Mh + (size_t)n * n : nullptr, n, red); RSD_LAUNCH_NOTE();
  std::vector<double> hred(256);
  RSD_CUDA(ctx, cudaMemcpyAsync(hred.data(), red, 256 * sizeof(double), cudaMemcpyDeviceToHost, s));
  int info_m = 0;
  if (p->precision == RSD_PREC_FP64) {
    // MobToResist_FTS: R_inf = M^-1
    RSD_TRY(rsd_potrf_upper_tag(ctx, (int)n, M, n, &info_m, "mob"));
    if (info_m) {
      loc.info = info_m;
      if (info) *info = loc;
      return info_m;
    }
    RSD_TRY(rsd_potri_upper_tag(ctx, (int)n, M, n, "mob"));
    RSD_TRY(rsd_mirror_upper(ctx, (int)n, M, n));
    cudaEventRecord(ctx->ev[2], s);
    // arrangResist: R = R_inf + R_lub
    int nc = 0;
    if (p->use_lub) RSD_TRY(rsd_lub_assemble(ctx, tab, nn, p->nb, 1, d_conf, d_radii, &lat, p->mu_f, M, n, 1, &nc));
    loc.n_contact = nc;
    if (rpp_out) {
      RSD_CUDA(ctx, cudaMemcpy2DAsync(rpp_out, sizeof(double) * rpp_ld, M, sizeof(double) * n, sizeof(double) * P, P,
                                      cudaMemcpyDeviceToDevice, s));
      RSD_CUDA(ctx, cudaStreamSynchronize(s));
      if (info) *info = loc;
      return RSD_OK;
    }
    cudaEventRecord(ctx->ev[3], s);
    // RHS [Fe + RPQ EIN, RPQ EIN]; RPP factored in place (RPQ, RQQ untouched)
    const double* RPQ = M + P * n;
    RSD_CUDA(ctx, cudaMemcpyAsync(X, Fe, sizeof(double) * P, cudaMemcpyDeviceToDevice, s));
    rsd_gemm_f64(s, (int)P, 1, (int)Q, 1.0, RPQ, n, 0, ein, Q, 0, 1.0, X, P);
    rsd_gemm_f64(s, (int)P, 1, (int)Q, 1.0, RPQ, n, 0, ein, Q, 0, 0.0, X + P, P);
    bool solved = false;
    if (ctx->rpp_mode != RSD_PC_NONE) {
      // PCG on RPP with the chosen preconditioner; the factorisation stays
      // the fallback when it does not reach the tolerance
      double* B = (double*)rsd_scratch(ctx, "step_rhs", sizeof(double) * 2 * P);
      if (!B) return RSD_ENOMEM;
      RSD_CUDA(ctx, cudaMemcpyAsync(B, X, sizeof(double) * 2 * P, cudaMemcpyDeviceToDevice, s));
      const double tol = ctx->rpp_tol > 0 ? ctx->rpp_tol : 1e-12;
      int it = 0;
      double res = 0.0;
      RSD_TRY(rsd_lp_pcg_internal(ctx, (rsd_lp*)ctx->rpp_net, ctx->rpp_mode, nn, d_conf, d_radii, &lat, M, n, 2, B, X,
                                  tol, ctx->rpp_maxit > 0 ? ctx->rpp_maxit : 1000, &it, &res));
      loc.rpp_iterations = it;
      if (res <= tol) {
        solved = true;
      } else {
        loc.rpp_iterations = -it;  // did not converge: factorisation below
        RSD_CUDA(ctx, cudaMemcpyAsync(X, B, sizeof(double) * 2 * P, cudaMemcpyDeviceToDevice, s));
      }
    }
    if (!solved) {
      int info_r = 0;
      RSD_TRY(rsd_potrf_upper_tag(ctx, (int)P, M, n, &info_r, "rpp"));
      if (info_r) {
        loc.info = info_r;
        if (info) *info = loc;
        return info_r;
      }
      RSD_TRY(rsd_potrs_upper_tag(ctx, (int)P, M, n, X, P, 2, "rpp"));
    }
    // SijN_hyd = RPQ^T RPP^-1 RPQ EIN - RQQ EIN
    rsd_gemm_f64(s, (int)Q, 1, (int)P, 1.0, RPQ, n, 1, X + P, P, 0, 0.0, S, Q);
    rsd_gemm_f64(s, (int)Q, 1, (int)Q, -1.0, M + P + P * n, n, 0, ein, Q, 0, 1.0, S, Q);
    RSD_CUDA(ctx, cudaGetLastError());
  } else {
    cudaEventRecord(ctx->ev[2], s);
    {
      rsd_range r("rsd_solve");
      RSD_TRY(rsd_mixed_solve(ctx, nn, M, n, d_conf, d_radii, &lat, tab, p, ein, d_Fe ? Fe : nullptr, Upar, S, &loc,
                              (float*)rpp_out, rpp_ld));
    }
    if (rpp_out) {
      RSD_CUDA(ctx, cudaStreamSynchronize(s));
      if (info) *info = loc;
      return RSD_OK;
    }
    cudaEventRecord(ctx->ev[3], s);
  }
  cudaEventRecord(ctx->ev[4], s);
  // velocities, Euler step, LE wrap
  bg_flow f{};
  memcpy(f.UOE, UOE, sizeof UOE);
  memcpy(f.omega, omega, sizeof omega);
  memcpy(f.LB, p->LB, sizeof f.LB);
  f.T = p->T;
  f.dt = p->dt;
  f.gamma = p->gamma;
  euler_update<<<(nn + 127) / 128, 128, 0, s>>>(nn, p->nb, f, Upar, d_conf, d_U_pos); RSD_LAUNCH_NOTE();
  RSD_CUDA(ctx, cudaMemcpyAsync(d_SijN, S, sizeof(double) * Q, cudaMemcpyDeviceToDevice, s));
  yeta_sums<<<1, 256, 0, s>>>(nn, S, nullptr, nullptr, ein, red + 256); RSD_LAUNCH_NOTE();
  int* flag = ctx->d_info + 8;
  RSD_CUDA(ctx, cudaMemsetAsync(flag, 0, sizeof(int), s));
  nan_check<<<(unsigned)((6 * nn + 255) / 256), 256, 0, s>>>(6LL * nn, d_U_pos, flag); RSD_LAUNCH_NOTE();
  cudaEventRecord(ctx->ev[5], s);
  double ys[3];
  RSD_CUDA(ctx, cudaMemcpyAsync(ys, red + 256, sizeof ys, cudaMemcpyDeviceToHost, s));
  RSD_CUDA(ctx, cudaMemcpyAsync(ctx->h_info + 8, flag, sizeof(int), cudaMemcpyDeviceToHost, s));
  RSD_CUDA(ctx, cudaStreamSynchronize(s));
  float t01, t12, t23, t45;
  cudaEventElapsedTime(&t01, ctx->ev[0], ctx->ev[1]);
  cudaEventElapsedTime(&t12, ctx->ev[1], ctx->ev[2]);
  cudaEventElapsedTime(&t23, ctx->ev[2], ctx->ev[3]);
  cudaEventElapsedTime(&t45, ctx->ev[3], ctx->ev[5]);
  ctx->phase_ms[0] = t01;
  if (p->precision == RSD_PREC_MIXED) {
    // the lubrication assembly sits inside the mixed solve (event 6)
    float t26, t63;
    cudaEventElapsedTime(&t26, ctx->ev[2], ctx->ev[6]);
    cudaEventElapsedTime(&t63, ctx->ev[6], ctx->ev[3]);
    ctx->phase_ms[1] = t26;
    ctx->phase_ms[2] = t12 + t63 + t45;
    float t73;  // refinement part of the solve (event 7 = factors done)
    cudaEventElapsedTime(&t73, ctx->ev[7], ctx->ev[3]);
    ctx->phase_ms[3] = t73;
  } else {
    ctx->phase_ms[1] = t23;
    ctx->phase_ms[2] = t12 + t45;
  }
  if (p->precision != RSD_PREC_MIXED) ctx->phase_ms[3] = 0;
  double sxx = 0.0;
  for (int b = 0; b < 256; b++) sxx += hred[b];
  const double f6 = 6.0 * RSD_PI * p->mu_f * 1.0;  // radii_test = 1 after non-dimensionalisation
  const double U_ave = sxx * f6 / nn;
  if (yeta_mu) {
    yeta_mu[0] = ys[0] / lat.LV / p->mu_f;
    yeta_mu[1] = lat.phi;
    yeta_mu[2] = 1.0 / U_ave;
    yeta_mu[3] = ys[1] / lat.LV / p->mu_f;
    yeta_mu[4] = ys[2] / lat.LV / p->mu_f;
  }
  if (info) *info = loc;
  if (ctx->h_info[8]) return rsd_fail(ctx, RSD_ENAN, "non-finite velocity (main.f90:223 NaN check)");
  return RSD_OK;
}

extern "C" int rsd_stepper_stokesian_dev(rsd_ctx* ctx, const rsd_lubtab* tab, const rsd_step_params* p,
                                         double* d_conf, const double* d_radii, const double* d_Fe, double* d_U_pos,
                                         double* d_SijN, double yeta_mu[5], rsd_step_info* info) {
  return step_impl(ctx, tab, p, d_conf, d_radii, d_Fe, d_U_pos, d_SijN, yeta_mu, info, nullptr, 0, nullptr);
}

extern "C" int rsd_resistance_pp_dev(rsd_ctx* ctx, const rsd_lubtab* tab, const rsd_step_params* p,
                                     const double* d_conf, const double* d_radii, void* d_rpp, int64_t ld,
                                     rsd_lattice* lat) {
  if (!ctx || !p || !d_rpp || ld < 6LL * p->nn) return rsd_fail(ctx, RSD_EARG, "rsd_resistance_pp_dev: bad arguments");
  rsd_step_info info{};
  return step_impl(ctx, tab, p, const_cast<double*>(d_conf), d_radii, nullptr, nullptr, nullptr, nullptr, &info, d_rpp,
                   ld, lat);
}

extern "C" int rsd_stepper_stokesian(rsd_ctx* ctx, const rsd_lubtab* tab, const rsd_step_params* p, double* conf,
                                     const double* radii, const double* Fe, double* U_pos, double* SijN,
                                     double yeta_mu[5], rsd_step_info* info) {
  if (!ctx || !p || !conf || !radii || !U_pos || !SijN || p->nn < 1)
    return rsd_fail(ctx, RSD_EARG, "rsd_stepper_stokesian: bad arguments");
  RSD_TRY(rsd_set_device(ctx));
  const int nn = p->nn;
  for (int i = 0; i < 3 * nn; i++)
    if (!std::isfinite(conf[i])) return rsd_fail(ctx, RSD_ENAN, "non-finite position");
  cudaStream_t s = ctx->stream;
  double* dc = (double*)rsd_scratch(ctx, "io_conf", sizeof(double) * 3 * nn);
  double* dr = (double*)rsd_scratch(ctx, "io_radii", sizeof(double) * nn);
  double* du = (double*)rsd_scratch(ctx, "io_upos", sizeof(double) * 6 * nn);
  double* ds = (double*)rsd_scratch(ctx, "io_sijn", sizeof(double) * 5 * nn);
  double* df = Fe ? (double*)rsd_scratch(ctx, "io_fe", sizeof(double) * 6 * nn) : nullptr;
  if (!dc || !dr || !du || !ds || (Fe && !df)) return RSD_ENOMEM;
  RSD_CUDA(ctx, cudaMemcpyAsync(dc, conf, sizeof(double) * 3 * nn, cudaMemcpyHostToDevice, s));
  RSD_CUDA(ctx, cudaMemcpyAsync(dr, radii, sizeof(double) * nn, cudaMemcpyHostToDevice, s));
  if (Fe) RSD_CUDA(ctx, cudaMemcpyAsync(df, Fe, sizeof(double) * 6 * nn, cudaMemcpyHostToDevice, s));
  int rc = rsd_stepper_stokesian_dev(ctx, tab, p, dc, dr, df, du, ds, yeta_mu, info);
  if (rc != RSD_OK) return rc;
  RSD_CUDA(ctx, cudaMemcpyAsync(conf, dc, sizeof(double) * 3 * nn, cudaMemcpyDeviceToHost, s));
  RSD_CUDA(ctx, cudaMemcpyAsync(U_pos, du, sizeof(double) * 6 * nn, cudaMemcpyDeviceToHost, s));
  RSD_CUDA(ctx, cudaMemcpyAsync(SijN, ds, sizeof(double) * 5 * nn, cudaMemcpyDeviceToHost, s));
  RSD_CUDA(ctx, cudaStreamSynchronize(s));
  return RSD_OK;
}

