// C-ABI entry points (include/rsd_capi.h): context and buffers, the lattice
// routines, the lubrication tables, the drop-in replacements of the
// reference's subroutines, and the fused device-resident step.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

#include "rsd_internal.cuh"

std::atomic<long long> rsd_launches{0};
extern "C" long long rsd_launch_count(void) { return rsd_launches.load(); }

// ------------------------------------------------------------ errors
int rsd_fail(rsd_ctx* ctx, int code, const char* fmt, ...) {
  if (ctx) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    ctx->err = buf;
  }
  return code;
}

int rsd_cuda_check(rsd_ctx* ctx, cudaError_t e, const char* what) {
  if (e == cudaErrorMemoryAllocation) return rsd_fail(ctx, RSD_ENOMEM, "%s: %s", what, cudaGetErrorString(e));
  return rsd_fail(ctx, RSD_ECUDA, "%s: %s", what, cudaGetErrorString(e));
}

void* rsd_scratch(rsd_ctx* ctx, const char* name, size_t bytes) {
  if (bytes == 0) bytes = 1;
  rsd_buf& b = ctx->bufs[name];
  if (b.bytes >= bytes) return b.p;
  if (b.p) {
    cudaStreamSynchronize(ctx->stream);
    cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
  }
  if (cudaMalloc(&b.p, bytes) != cudaSuccess) {
    cudaGetLastError();
    rsd_fail(ctx, RSD_ENOMEM, "cannot allocate %zu bytes for %s", bytes, name);
    b.p = nullptr;
    return nullptr;
  }
  b.bytes = bytes;
  return b.p;
}

int rsd_set_device(rsd_ctx* ctx) {
  RSD_CUDA(ctx, cudaSetDevice(ctx->device));
  return RSD_OK;
}

rsd_lat_dev rsd_lat_pack(const rsd_lattice* lat) {
  rsd_lat_dev L{};
  for (int i = 0; i < 9; i++) {
    L.LR[i] = lat->LR[i];
    L.LI[i] = lat->LI[i];
  }
  L.LV = lat->LV;
  L.lam = lat->lammda;
  L.phix = 1 - 0.2 * lat->phi;  // Ewald_summation.f90:55,222
  L.NR = lat->NR;
  L.NI = lat->NI;
  return L;
}

// ------------------------------------------------------------ context
extern "C" int rsd_ctx_create(rsd_ctx** out, int device) {
  if (!out) return RSD_EARG;
  *out = nullptr;
  rsd_ctx* c = new rsd_ctx();
  c->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&c->d_info, 64 * sizeof(int));
  if (e == cudaSuccess) e = cudaMallocHost(&c->h_info, 64 * sizeof(int));
  for (int i = 0; i < 8 && e == cudaSuccess; i++) e = cudaEventCreate(&c->ev[i]);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) {
    cudaGetLastError();
    delete c;
    return RSD_ECUDA;
  }
  *out = c;
  return RSD_OK;
}

int rsd_side_stream(rsd_ctx* c) {
  if (c->side) return RSD_OK;
  int lo = 0, hi = 0;
  RSD_CUDA(c, cudaDeviceGetStreamPriorityRange(&lo, &hi));
  RSD_CUDA(c, cudaStreamCreateWithPriority(&c->side, cudaStreamNonBlocking, hi));
  RSD_CUDA(c, cudaStreamCreateWithPriority(&c->side2, cudaStreamNonBlocking, hi));
  RSD_CUDA(c, cudaEventCreateWithFlags(&c->ev_panel, cudaEventDisableTiming));
  RSD_CUDA(c, cudaEventCreateWithFlags(&c->ev_next, cudaEventDisableTiming));
  for (int i = 0; i < 4; i++) RSD_CUDA(c, cudaEventCreateWithFlags(&c->ev_la[i], cudaEventDisableTiming));
  return RSD_OK;
}

extern "C" int rsd_ctx_destroy(rsd_ctx* c) {
  if (!c) return RSD_OK;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->side) {
    cudaStreamSynchronize(c->side);
    cudaStreamDestroy(c->side);
  }
  if (c->side2) {
    cudaStreamSynchronize(c->side2);
    cudaStreamDestroy(c->side2);
  }
  for (int i = 0; i < 4; i++)
    if (c->ev_la[i]) cudaEventDestroy(c->ev_la[i]);
  if (c->ev_panel) cudaEventDestroy(c->ev_panel);
  if (c->ev_next) cudaEventDestroy(c->ev_next);
  for (auto& kv : c->bufs)
    if (kv.second.p) cudaFree(kv.second.p);
  for (int i = 0; i < 8; i++)
    if (c->ev[i]) cudaEventDestroy(c->ev[i]);
  if (c->d_info) cudaFree(c->d_info);
  if (c->h_info) cudaFreeHost(c->h_info);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return RSD_OK;
}

extern "C" const char* rsd_ctx_last_error(const rsd_ctx* c) { return c ? c->err.c_str() : "no context"; }
extern "C" void* rsd_ctx_stream(rsd_ctx* c) { return c ? (void*)c->stream : nullptr; }

extern "C" int rsd_ctx_set_mixed_split(rsd_ctx* c, double lam_r_cut, int32_t kshell) {
  if (!c) return RSD_EARG;
  if (!(lam_r_cut >= 0.0 && lam_r_cut <= 6.0) || kshell < 0)
    return rsd_fail(c, RSD_EARG, "mixed split: 0 <= lam_r_cut <= 6, kshell >= 0");
  c->mixed_rcut = lam_r_cut;
  c->mixed_kshell = kshell;
  return RSD_OK;
}

extern "C" int rsd_ctx_set_mixed_truncation(rsd_ctx* c, double lam_r_max, double k2_over_4lam2_max) {
  if (!c) return RSD_EARG;
  if (!(lam_r_max > 0.0) || !(k2_over_4lam2_max > 0.0))
    return rsd_fail(c, RSD_EARG, "mixed truncation: both limits must be positive");
  c->mixed_rmax = lam_r_max;
  c->mixed_kexp = k2_over_4lam2_max;
  return RSD_OK;
}

extern "C" int rsd_ctx_set_mixed_lambda_scale(rsd_ctx* c, double scale) {
  if (!c) return RSD_EARG;
  if (!(scale >= 0.5 && scale <= 4.0)) return rsd_fail(c, RSD_EARG, "mixed lambda scale must be in [0.5, 4]");
  c->mixed_lambda_scale = scale;
  return RSD_OK;
}

extern "C" int rsd_ctx_set_correction_method(rsd_ctx* c, int method) {
  if (!c) return RSD_EARG;
  if (method < 0 || method > 2) return rsd_fail(c, RSD_EARG, "correction_method must be 0, 1 or 2");
  c->correction_method = method;
  return RSD_OK;
}

extern "C" int rsd_ctx_set_wait_limits(rsd_ctx* c, int64_t tc_wait_ns, int64_t tri_spin_polls) {
  if (!c) return RSD_EARG;
  if (tc_wait_ns < 0 || tri_spin_polls < 0) return rsd_fail(c, RSD_EARG, "wait limits must be >= 0");
  c->tc_wait_ns = tc_wait_ns;
  c->tri_spin_polls = tri_spin_polls;
  return RSD_OK;
}

extern "C" int rsd_ctx_set_factor_schedule(rsd_ctx* c, int32_t schedule) {
  if (!c) return RSD_EARG;
  if (schedule != 0 && schedule != 1) return rsd_fail(c, RSD_EARG, "factor schedule: 0 or 1");
  c->factor_schedule = schedule;
  return RSD_OK;
}

extern "C" int rsd_ctx_set_refinement(rsd_ctx* c, int32_t mode, int32_t restart) {
  if (!c) return RSD_EARG;
  if ((mode != 0 && mode != 1) || restart < 0 || restart > 30)
    return rsd_fail(c, RSD_EARG, "refinement: mode 0 or 1, restart 0..30");
  c->refine_gmres = mode;
  c->gmres_restart = restart > 0 ? restart : 30;
  return RSD_OK;
}

extern "C" int rsd_ctx_set_rpp_solver(rsd_ctx* c, int32_t mode, rsd_lp* net, double tol, int32_t maxit) {
  if (!c) return RSD_EARG;
  if (mode < RSD_PC_NONE || mode > RSD_PC_LEARNED || (mode == RSD_PC_LEARNED && !net) || tol < 0 || maxit < 0)
    return rsd_fail(c, RSD_EARG, "rpp solver: mode 0-4 (4 needs a network), tol >= 0, maxit >= 0");
  c->rpp_mode = mode;
  c->rpp_net = net;
  c->rpp_tol = tol;
  c->rpp_maxit = maxit;
  return RSD_OK;
}

extern "C" int rsd_ctx_set_mixed_real_passes(rsd_ctx* c, int passes) {
  if (!c) return RSD_EARG;
  if (passes < 1 || passes > 4) return rsd_fail(c, RSD_EARG, "mixed real-space passes must be 1 to 4");
  c->mixed_real_passes = passes;
  return RSD_OK;
}

extern "C" int rsd_ctx_set_tensor_cores(rsd_ctx* c, int mode) {
  if (!c) return RSD_EARG;
  if (mode != 0 && mode != 1 && mode != 3) return rsd_fail(c, RSD_EARG, "tensor-core mode must be 0, 1 or 3");
  c->use_tc = mode;
  return RSD_OK;
}
extern "C" int rsd_ctx_phase_ms(const rsd_ctx* c, double ms[4]) {
  if (!c || !ms) return RSD_EARG;
  for (int i = 0; i < 4; i++) ms[i] = c->phase_ms[i];
  return RSD_OK;
}

// ------------------------------------------------------------ lattice
static void mat_inv3(double LI[9], const double LR[9], double* det) {
#define A(i, j) LR[(i - 1) + 3 * (j - 1)]
#define L(i, j) LI[(i - 1) + 3 * (j - 1)]
  const double d = A(1, 1) * A(2, 2) * A(3, 3) + A(1, 2) * A(2, 3) * A(3, 1) + A(1, 3) * A(2, 1) * A(3, 2) -
                   A(1, 3) * A(2, 2) * A(3, 1) - A(2, 3) * A(3, 2) * A(1, 1) - A(3, 3) * A(1, 2) * A(2, 1);
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

extern "C" int rsd_set_lattice_skew(double T, const double LB[3], double gamma, int32_t oscillation,
                                    double gamma_alpha, double frequency, rsd_lattice* lat) {
  if (!LB || !lat) return RSD_EARG;
  memset(lat->LR, 0, sizeof lat->LR);
  lat->LR[0] = LB[0];
  lat->LR[4] = LB[1];
  lat->LR[8] = LB[2];
  if (oscillation) {
    lat->LR[6] = fmod(gamma_alpha * sin(frequency * T) * LB[2], LB[0]);
  } else if (gamma != 0.0) {
    const double tshear = LB[0] / (LB[2] * gamma);
    lat->LR[6] = LB[2] * fmod(T, tshear) * gamma;
  }
  double det;
  mat_inv3(lat->LI, lat->LR, &det);
  lat->LV = fabs(det);
  return RSD_OK;
}

// eigenvalues of a symmetric 3x3 matrix (cyclic Jacobi)
static void eig3(const double Ain[9], double ev[3]) {
  double a[3][3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) a[i][j] = Ain[i + 3 * j];
  for (int sweep = 0; sweep < 60; sweep++) {
    if (a[0][1] == 0.0 && a[0][2] == 0.0 && a[1][2] == 0.0) break;
    for (int p = 0; p < 2; p++)
      for (int q = p + 1; q < 3; q++) {
        if (a[p][q] == 0.0) continue;
        const double th = (a[q][q] - a[p][p]) / (2.0 * a[p][q]);
        const double t = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < 3; k++) {
          const double x = a[k][p], y = a[k][q];
          a[k][p] = c * x - s * y;
          a[k][q] = s * x + c * y;
        }
        for (int k = 0; k < 3; k++) {
          const double x = a[p][k], y = a[q][k];
          a[p][k] = c * x - s * y;
          a[q][k] = s * x + c * y;
        }
      }
  }
  for (int i = 0; i < 3; i++) ev[i] = a[i][i];
}

// CALC_LATTICE_INVERSE (src/csd_post.f90:158-183) for a given cube sum of
// the radii: the one place that derives lammda, NR, NI and phi, shared by
// rsd_calc_lattice_inverse and the allocation-free assembly (which reduces
// the cube sum on the device).
int rsd_lattice_params(rsd_lattice* lat, double ews_err, double sum_a3) {
  if (!lat || !(ews_err > 0.0) || !(lat->LV > 0.0)) return RSD_EARG;
  lat->sig = pow(lat->LV, 1.0 / 3.0) / sqrt(2.0 * RSD_PI);
  lat->lammda = sqrt(RSD_PI) / pow(lat->LV, 1.0 / 3.0);
  lat->logerr = -log(ews_err);
  double MM[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      double s = 0.0;
      for (int k = 0; k < 3; k++) s += lat->LR[k + 3 * i] * lat->LR[k + 3 * j];
      MM[i + 3 * j] = s;
    }
  double le[3];
  eig3(MM, le);
  const double lmin = fmin(le[0], fmin(le[1], le[2])), lmax = fmax(le[0], fmax(le[1], le[2]));
  lat->NR = (int)(sqrt(2.0 * lat->logerr * (lat->sig * lat->sig) / lmin) + 1);
  lat->NI = (int)(sqrt(lat->logerr / (2.0 * (RSD_PI * RSD_PI) * (lat->sig * lat->sig) * (1.0 / lmax))) + 1);
  lat->phi = sum_a3 * 4.0 / 3.0 * RSD_PI / lat->LV;
  if (lat->NR > 40 || lat->NI > 40) return RSD_EARG;  // absurd lattice
  return RSD_OK;
}

extern "C" int rsd_calc_lattice_inverse(rsd_lattice* lat, double ews_err, int32_t nn, const double* radii) {
  if (!lat || !radii || nn < 1) return RSD_EARG;
  double s3 = 0.0;
  for (int i = 0; i < nn; i++) s3 += radii[i] * radii[i] * radii[i];
  return rsd_lattice_params(lat, ews_err, s3);
}

// ------------------------------------------------------------ lub tables
static int read_table(const char* path, int ncol, int nrow, double* dst) {
  FILE* fp = fopen(path, "r");
  if (!fp) return -1;
  char line[1024];
  if (!fgets(line, sizeof line, fp)) {
    fclose(fp);
    return -1;
  }
  for (int r = 0; r < nrow; r++)
    for (int c = 0; c < ncol; c++)
      if (fscanf(fp, "%lf", &dst[r * ncol + c]) != 1) {
        fclose(fp);
        return -1;
      }
  fclose(fp);
  return 0;
}

extern "C" int rsd_lubtab_load(rsd_lubtab** out, const char* dir) {
  if (!out || !dir) return RSD_EARG;
  rsd_lubtab* t = new rsd_lubtab();
  t->nabc = 39;
  t->ngh = 47;
  t->nm = 47;
  std::string d(dir);
  if (read_table((d + "/r2babc.dat").c_str(), 11, t->nabc, t->abc) ||
      read_table((d + "/r2bgh.dat").c_str(), 7, t->ngh, t->gh) || read_table((d + "/r2bm.dat").c_str(), 4, t->nm, t->m)) {
    delete t;
    *out = nullptr;
    return RSD_EIO;
  }
  *out = t;
  return RSD_OK;
}

extern "C" int rsd_lubtab_create(rsd_lubtab** out, int32_t nabc, const double* abc, int32_t ngh, const double* gh,
                                 int32_t nm, const double* m) {
  if (!out || !abc || !gh || !m || nabc < 2 || ngh < 2 || nm < 2 || nabc > 64 || ngh > 64 || nm > 64) return RSD_EARG;
  rsd_lubtab* t = new rsd_lubtab();
  t->nabc = nabc;
  t->ngh = ngh;
  t->nm = nm;
  memcpy(t->abc, abc, sizeof(double) * 11 * nabc);
  memcpy(t->gh, gh, sizeof(double) * 7 * ngh);
  memcpy(t->m, m, sizeof(double) * 4 * nm);
  *out = t;
  return RSD_OK;
}

extern "C" int rsd_lubtab_destroy(rsd_lubtab* t) {
  if (!t) return RSD_OK;
  for (auto& kv : t->dev) {
    cudaSetDevice(kv.first);
    cudaFree(kv.second);
  }
  delete t;
  return RSD_OK;
}

// ------------------------------------------------------------ helpers
static int upload(rsd_ctx* ctx, const char* name, const double* h, size_t n, double** d) {
  *d = (double*)rsd_scratch(ctx, name, n * sizeof(double));
  if (!*d) return RSD_ENOMEM;
  RSD_CUDA(ctx, cudaMemcpyAsync(*d, h, n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  return RSD_OK;
}

// host (rows x cols, ld rows) <-> device sub-block at d (ld ldd)
static int get_block(rsd_ctx* ctx, double* h, int64_t rows, int64_t cols, const double* d, int64_t ldd) {
  RSD_CUDA(ctx, cudaMemcpy2DAsync(h, rows * sizeof(double), d, ldd * sizeof(double), rows * sizeof(double), cols,
                                  cudaMemcpyDeviceToHost, ctx->stream));
  return RSD_OK;
}
static int put_block(rsd_ctx* ctx, double* d, int64_t ldd, const double* h, int64_t rows, int64_t cols) {
  RSD_CUDA(ctx, cudaMemcpy2DAsync(d, ldd * sizeof(double), h, rows * sizeof(double), rows * sizeof(double), cols,
                                  cudaMemcpyHostToDevice, ctx->stream));
  return RSD_OK;
}
static int sync(rsd_ctx* ctx) {
  RSD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return RSD_OK;
}

static bool finite_all(const double* p, size_t n) {
  for (size_t i = 0; i < n; i++)
    if (!std::isfinite(p[i])) return false;
  return true;
}

// ------------------------------------------------------------ kernel 1
extern "C" int rsd_per_grpery_inv_fri_dev(rsd_ctx* ctx, int32_t nn, const double* d_pos, const double* d_radii,
                                          rsd_lattice* lat, double ews_err, double mu_f, int32_t correction_method,
                                          double* d_M, int64_t ldm) {
  if (!ctx || !lat || !d_pos || !d_radii || !d_M || nn < 1 || ldm < 11LL * nn || !(mu_f > 0))
    return rsd_fail(ctx, RSD_EARG, "rsd_per_grpery_inv_fri_dev: bad arguments");
  RSD_TRY(rsd_set_device(ctx));
  std::vector<double> radii(nn);
  RSD_CUDA(ctx, cudaMemcpy(radii.data(), d_radii, nn * sizeof(double), cudaMemcpyDeviceToHost));
  if (correction_method < 0 || correction_method > 2)
    return rsd_fail(ctx, RSD_EARG, "correction_method=%d: 0 (none), 1 (Yamakawa) or 2 (regularized)", correction_method);
  RSD_TRY(rsd_calc_lattice_inverse(lat, ews_err, nn, radii.data()));
  // overlap corrections, per_GRPY_YZD.f90:98-116: method 1 (Yamakawa) or 2
  // (regularized Green's function), added after the Ewald sums
  int nov = 0;
  if (correction_method != 0) RSD_TRY(rsd_count_overlaps(ctx, nn, d_pos, d_radii, lat, &nov));
  RSD_TRY(rsd_ewald_assemble(ctx, nn, d_pos, d_radii, lat, mu_f, RSD_PREC_FP64, d_M, ldm));
  return rsd_overlap_correct(ctx, correction_method, RSD_PREC_FP64, nn, d_pos, d_radii, lat, mu_f, nov, d_M, ldm);
}

extern "C" int rsd_per_grpery_inv_fri(rsd_ctx* ctx, int32_t nn, const double* p_pos, const double* radii,
                                      rsd_lattice* lat, double ews_err, double mu_f, int32_t correction_method,
                                      double* APP, double* APQ, double* AQQ) {
  if (!ctx || !p_pos || !radii || !lat || !APP || !APQ || !AQQ || nn < 1)
    return rsd_fail(ctx, RSD_EARG, "rsd_per_grpery_inv_fri: bad arguments");
  if (!finite_all(p_pos, 3 * (size_t)nn) || !finite_all(radii, nn))
    return rsd_fail(ctx, RSD_ENAN, "non-finite positions or radii");
  RSD_TRY(rsd_set_device(ctx));
  double *dp, *dr;
  RSD_TRY(upload(ctx, "in_pos", p_pos, 3 * (size_t)nn, &dp));
  RSD_TRY(upload(ctx, "in_radii", radii, nn, &dr));
  const int64_t n = 11LL * nn;
  double* M = (double*)rsd_scratch(ctx, "M", sizeof(double) * n * n);
  if (!M) return RSD_ENOMEM;
  RSD_TRY(rsd_per_grpery_inv_fri_dev(ctx, nn, dp, dr, lat, ews_err, mu_f, correction_method, M, n));
  RSD_TRY(get_block(ctx, APP, 6LL * nn, 6LL * nn, M, n));
  RSD_TRY(get_block(ctx, APQ, 6LL * nn, 5LL * nn, M + 6LL * nn * n, n));
  RSD_TRY(get_block(ctx, AQQ, 5LL * nn, 5LL * nn, M + 6LL * nn + 6LL * nn * n, n));
  return sync(ctx);
}

// ------------------------------------------------------------ kernel 2
extern "C" int rsd_lubmxcalc_dev(rsd_ctx* ctx, const rsd_lubtab* tab, int32_t nn, int32_t nb, int32_t is_period,
                                 const double* d_pos, const double* d_radii, const rsd_lattice* lat, double mu_f,
                                 double* d_L, int64_t ldl, int32_t accumulate, int32_t* n_contact) {
  if (!ctx || !tab || !d_pos || !d_radii || !d_L || nn < 1 || nb < 0 || nb > nn || (is_period && !lat))
    return rsd_fail(ctx, RSD_EARG, "rsd_lubmxcalc_dev: bad arguments");
  RSD_TRY(rsd_set_device(ctx));
  rsd_lattice none{};
  int nc = 0;
  RSD_TRY(rsd_lub_assemble(ctx, tab, nn, nb, is_period, d_pos, d_radii, lat ? lat : &none, mu_f, d_L, ldl, accumulate,
                           &nc));
  if (n_contact) *n_contact = nc;
  return RSD_OK;
}

extern "C" int rsd_lubmxcalc(rsd_ctx* ctx, const rsd_lubtab* tab, int32_t nn, int32_t nb, int32_t is_period,
                             const double* p_pos, const double* radii, const rsd_lattice* lat, double mu_f, double* rfu,
                             double* rfe, double* rse, int32_t* n_contact) {
  if (!ctx || !p_pos || !radii || !rfu || !rfe || !rse || nn < 1)
    return rsd_fail(ctx, RSD_EARG, "rsd_lubmxcalc: bad arguments");
  if (!finite_all(p_pos, 3 * (size_t)nn)) return rsd_fail(ctx, RSD_ENAN, "non-finite positions");
  RSD_TRY(rsd_set_device(ctx));
  double *dp, *dr;
  RSD_TRY(upload(ctx, "in_pos", p_pos, 3 * (size_t)nn, &dp));
  RSD_TRY(upload(ctx, "in_radii", radii, nn, &dr));
  const int64_t n = 11LL * nn;
  double* L = (double*)rsd_scratch(ctx, "L", sizeof(double) * n * n);
  if (!L) return RSD_ENOMEM;
  RSD_TRY(rsd_lubmxcalc_dev(ctx, tab, nn, nb, is_period, dp, dr, lat, mu_f, L, n, 0, n_contact));
  RSD_TRY(get_block(ctx, rfu, 6LL * nn, 6LL * nn, L, n));
  RSD_TRY(get_block(ctx, rfe, 6LL * nn, 5LL * nn, L + 6LL * nn * n, n));
  RSD_TRY(get_block(ctx, rse, 5LL * nn, 5LL * nn, L + 6LL * nn + 6LL * nn * n, n));
  return sync(ctx);
}

// ------------------------------------------------------------ kernel 3
extern "C" int rsd_matrev_dev(rsd_ctx* ctx, int32_t n, double* d_A, int64_t lda, int32_t* info) {
  if (!ctx || !d_A || n < 1 || lda < n || !info) return rsd_fail(ctx, RSD_EARG, "rsd_matrev_dev: bad arguments");
  RSD_TRY(rsd_set_device(ctx));
  int inf = 0;
  RSD_TRY(rsd_potrf_upper_tag(ctx, n, d_A, lda, &inf, "matrev"));
  *info = inf;
  if (inf == 0) {
    RSD_TRY(rsd_potri_upper_tag(ctx, n, d_A, lda, "matrev"));
    RSD_TRY(rsd_mirror_upper(ctx, n, d_A, lda));
  }
  return RSD_OK;
}

extern "C" int rsd_matrev(rsd_ctx* ctx, int32_t n, double* A, int32_t* info) {
  if (!ctx || !A || n < 1 || !info) return rsd_fail(ctx, RSD_EARG, "rsd_matrev: bad arguments");
  RSD_TRY(rsd_set_device(ctx));
  double* d;
  RSD_TRY(upload(ctx, "matrev_A", A, (size_t)n * n, &d));
  RSD_TRY(rsd_matrev_dev(ctx, n, d, n, info));
  RSD_CUDA(ctx, cudaMemcpyAsync(A, d, sizeof(double) * (size_t)n * n, cudaMemcpyDeviceToHost, ctx->stream));
  return sync(ctx);
}

extern "C" int rsd_cholesky(rsd_ctx* ctx, int32_t n, double* B, int32_t* info) {
  if (!ctx || !B || n < 1 || !info) return rsd_fail(ctx, RSD_EARG, "rsd_cholesky: bad arguments");
  RSD_TRY(rsd_set_device(ctx));
  // the lower triangle of B is the input (DPOTRF 'L'); U = L^T from the
  // upper factorisation of the same symmetric matrix
  std::vector<double> Bs((size_t)n * n);
  for (int j = 0; j < n; j++)
    for (int i = 0; i < n; i++) Bs[i + (size_t)j * n] = (i <= j) ? B[j + (size_t)i * n] : 0.0;
  double* d;
  RSD_TRY(upload(ctx, "chol_B", Bs.data(), (size_t)n * n, &d));
  int inf = 0;
  RSD_TRY(rsd_potrf_upper_tag(ctx, n, d, n, &inf, "chol"));
  *info = inf;
  RSD_CUDA(ctx, cudaMemcpyAsync(Bs.data(), d, sizeof(double) * (size_t)n * n, cudaMemcpyDeviceToHost, ctx->stream));
  RSD_TRY(sync(ctx));
  for (int j = 0; j < n; j++)
    for (int i = 0; i < n; i++) B[i + (size_t)j * n] = (i >= j) ? Bs[j + (size_t)i * n] : 0.0;
  return inf > 0 ? inf : RSD_OK;
}

// ------------------------------------------------------------- Brownian
namespace {
// columns j = blockIdx.y, blockIdx.y + gridDim.y, ...
__global__ void zero_strict_lower(int n, double* __restrict__ A, int64_t lda) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  for (int j = blockIdx.y; j < n; j += gridDim.y)
    if (i < n && i > j) A[i + (int64_t)j * lda] = 0.0;
}

// deta of DMDX_CAL: PARAMETER(deta=0.001) gives a REAL*8 the value of the
// default-real (single precision) literal
constexpr double DMDX_DETA = (double)0.001f;

// d_out = (A1 - A2) Z / deta with A1, A2 the translational blocks of the
// grand mobility at conf +- deta Z / 2 (DMDX_CAL, stepper.f90:664-688).
int dmdx_dev(rsd_ctx* ctx, int32_t nn, const double* conf, const double* radii, rsd_lattice* lat, double ews_err,
             double mu_f, int32_t correction_method, const double* Z, double* d_out) {
  const int64_t n = 11LL * nn, t = 3LL * nn;
  std::vector<double> c1(3 * (size_t)nn), c2(3 * (size_t)nn);
  for (size_t k = 0; k < c1.size(); k++) {
    c1[k] = conf[k] + 0.5 * DMDX_DETA * Z[k];
    c2[k] = conf[k] - 0.5 * DMDX_DETA * Z[k];
  }
  double *d1, *d2, *dr, *dz;
  RSD_TRY(upload(ctx, "dmdx_conf1", c1.data(), c1.size(), &d1));
  RSD_TRY(upload(ctx, "dmdx_conf2", c2.data(), c2.size(), &d2));
  RSD_TRY(upload(ctx, "dmdx_radii", radii, nn, &dr));
  RSD_TRY(upload(ctx, "dmdx_z", Z, (size_t)t, &dz));
  double* M1 = (double*)rsd_scratch(ctx, "dmdx_M1", sizeof(double) * n * n);
  double* M2 = (double*)rsd_scratch(ctx, "dmdx_M2", sizeof(double) * n * n);
  if (!M1 || !M2) return RSD_ENOMEM;
  RSD_TRY(rsd_per_grpery_inv_fri_dev(ctx, nn, d1, dr, lat, ews_err, mu_f, correction_method, M1, n));
  RSD_TRY(rsd_per_grpery_inv_fri_dev(ctx, nn, d2, dr, lat, ews_err, mu_f, correction_method, M2, n));
  rsd_gemm_f64(ctx->stream, (int)t, 1, (int)t, 1.0 / DMDX_DETA, M1, n, 0, dz, t, 0, 0.0, d_out, t);
  rsd_gemm_f64(ctx->stream, (int)t, 1, (int)t, -1.0 / DMDX_DETA, M2, n, 0, dz, t, 0, 1.0, d_out, t);
  RSD_CUDA(ctx, cudaGetLastError());
  return RSD_OK;
}
}  // namespace

extern "C" int rsd_dmdx_cal(rsd_ctx* ctx, int32_t nn, const double* conf, const double* radii, rsd_lattice* lat,
                            double ews_err, double mu_f, int32_t correction_method, const double* Z, double* DMDX) {
  if (!ctx || nn < 1 || !conf || !radii || !lat || !Z || !DMDX)
    return rsd_fail(ctx, RSD_EARG, "rsd_dmdx_cal: bad arguments");
  if (!finite_all(conf, 3 * (size_t)nn) || !finite_all(radii, nn) || !finite_all(Z, 3 * (size_t)nn))
    return rsd_fail(ctx, RSD_ENAN, "non-finite positions, radii or Z");
  RSD_TRY(rsd_set_device(ctx));
  double* d = (double*)rsd_scratch(ctx, "dmdx_out", sizeof(double) * 3 * (size_t)nn);
  if (!d) return RSD_ENOMEM;
  RSD_TRY(dmdx_dev(ctx, nn, conf, radii, lat, ews_err, mu_f, correction_method, Z, d));
  RSD_CUDA(ctx, cudaMemcpyAsync(DMDX, d, sizeof(double) * 3 * (size_t)nn, cudaMemcpyDeviceToHost, ctx->stream));
  return sync(ctx);
}

extern "C" int rsd_brownian_velocity(rsd_ctx* ctx, int32_t nn, const double* APP, const double* conf,
                                     const double* radii, rsd_lattice* lat, double ews_err, double mu_f,
                                     int32_t correction_method, const double* Z, double kBT, double dt,
                                     double* u_brown, int32_t* info) {
  if (!ctx || nn < 1 || !APP || !conf || !radii || !lat || !Z || !u_brown || !info || !(dt != 0.0))
    return rsd_fail(ctx, RSD_EARG, "rsd_brownian_velocity: bad arguments");
  if (!finite_all(Z, 3 * (size_t)nn)) return rsd_fail(ctx, RSD_ENAN, "non-finite Z");
  RSD_TRY(rsd_set_device(ctx));
  const int64_t t = 3LL * nn, p = 6LL * nn;
  // CHOLESKY of the translational block A = APP(1:3N, 1:3N): U = L^T from
  // the upper factorisation, the strict lower part cleared
  std::vector<double> As((size_t)(t * t));
  for (int64_t j = 0; j < t; j++)
    for (int64_t i = 0; i < t; i++) As[i + j * t] = (i <= j) ? APP[j + i * p] : 0.0;
  double *dA, *dz;
  RSD_TRY(upload(ctx, "brown_A", As.data(), As.size(), &dA));
  RSD_TRY(upload(ctx, "brown_z", Z, (size_t)t, &dz));
  int inf = 0;
  RSD_TRY(rsd_potrf_upper_tag(ctx, (int)t, dA, t, &inf, "brown"));
  *info = inf;
  if (inf) return inf;
  zero_strict_lower<<<dim3((unsigned)((t + 255) / 256), (unsigned)(t < 65535 ? t : 65535)), 256, 0, ctx->stream>>>(
      (int)t, dA, t);
  double* vb = (double*)rsd_scratch(ctx, "brown_vb", sizeof(double) * 2 * (size_t)t);
  if (!vb) return RSD_ENOMEM;
  // VB = sqrt(2 kBT) L Z / DT (stepper.f90:79)
  rsd_gemm_f64(ctx->stream, (int)t, 1, (int)t, std::sqrt(2.0 * kBT) / dt, dA, t, 1, dz, t, 0, 0.0, vb, t);
  RSD_CUDA(ctx, cudaGetLastError());
  RSD_TRY(dmdx_dev(ctx, nn, conf, radii, lat, ews_err, mu_f, correction_method, Z, vb + t));
  std::vector<double> h(2 * (size_t)t);
  RSD_CUDA(ctx, cudaMemcpyAsync(h.data(), vb, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, ctx->stream));
  RSD_TRY(sync(ctx));
  // u_brown = VB + kBT DMDX (stepper.f90:81-83)
  for (int64_t k = 0; k < t; k++) u_brown[k] = h[k] + kBT * h[t + k];
  return RSD_OK;
}

extern "C" int rsd_mob_to_resist_fts(rsd_ctx* ctx, int32_t nn, const double* APP, const double* APQ,
                                     const double* AQQ, double* RPP, double* RPQ, double* RQQ, int32_t* info) {
  if (!ctx || nn < 1 || !APP || !APQ || !AQQ || !RPP || !RPQ || !RQQ || !info)
    return rsd_fail(ctx, RSD_EARG, "rsd_mob_to_resist_fts: bad arguments");
  RSD_TRY(rsd_set_device(ctx));
  const int64_t n = 11LL * nn, p = 6LL * nn, q = 5LL * nn;
  double* M = (double*)rsd_scratch(ctx, "M", sizeof(double) * n * n);
  if (!M) return RSD_ENOMEM;
  RSD_TRY(put_block(ctx, M, n, APP, p, p));
  RSD_TRY(put_block(ctx, M + p * n, n, APQ, p, q));
  RSD_TRY(put_block(ctx, M + p + p * n, n, AQQ, q, q));
  RSD_TRY(rsd_matrev_dev(ctx, (int)n, M, n, info));
  RSD_TRY(get_block(ctx, RPP, p, p, M, n));
  RSD_TRY(get_block(ctx, RPQ, p, q, M + p * n, n));
  RSD_TRY(get_block(ctx, RQQ, q, q, M + p + p * n, n));
  return sync(ctx);
}

extern "C" int rsd_arrangement(rsd_ctx* ctx, int32_t nn, const double* RPP, const double* RPQ, const double* RQQ,
                               double* mu, int32_t* info) {
  if (!ctx || nn < 1 || !RPP || !RPQ || !RQQ || !mu || !info)
    return rsd_fail(ctx, RSD_EARG, "rsd_arrangement: bad arguments");
  RSD_TRY(rsd_set_device(ctx));
  const int64_t p = 6LL * nn, q = 5LL * nn;
  double *dP, *dQ, *dX, *dmu;
  RSD_TRY(upload(ctx, "arr_RPP", RPP, p * p, &dP));
  RSD_TRY(upload(ctx, "arr_RPQ", RPQ, p * q, &dQ));
  RSD_TRY(upload(ctx, "arr_X", RPQ, p * q, &dX));
  RSD_TRY(upload(ctx, "arr_mu", RQQ, q * q, &dmu));
  int inf = 0;
  RSD_TRY(rsd_potrf_upper_tag(ctx, (int)p, dP, p, &inf, "arr"));
  *info = inf;
  if (inf) return RSD_OK;
  RSD_TRY(rsd_potrs_upper_tag(ctx, (int)p, dP, p, dX, p, (int)q, "arr"));
  rsd_gemm_f64(ctx->stream, (int)q, (int)q, (int)p, 1.0, dQ, p, 1, dX, p, 0, -1.0, dmu, q);
  RSD_CUDA(ctx, cudaGetLastError());
  RSD_CUDA(ctx, cudaMemcpyAsync(mu, dmu, sizeof(double) * q * q, cudaMemcpyDeviceToHost, ctx->stream));
  return sync(ctx);
}

// EI_transY2 (src/tensors.f90:890-903) for one symmetric 3x3 tensor
static void ei_trans_y2(const double E[9], double out[5]) {
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

// The resistance solve of STEPPER_NOGmres; RPP (the inverse left by
// Rheology) is written only when non-null, and the stresslet dipole of the
// interparticle forces is added only when conf is non-null.
static int nogmres_impl(rsd_ctx* ctx, int32_t nn, const double* APP, const double* APQ, const double* AQQ,
                        const double* rfu, const double* rfe, const double* rse, const double* Fe, const double* EIN,
                        const double* Fe_inter, const double* conf, const double* u_brown, double* U_par,
                        double* SijN_hyd, double* SijN_FP, double* SijN_B, double* RPP, int32_t* info) {
  RSD_TRY(rsd_set_device(ctx));
  cudaStream_t s = ctx->stream;
  const int64_t n = 11LL * nn, p = 6LL * nn, q = 5LL * nn;
  double* M = (double*)rsd_scratch(ctx, "M", sizeof(double) * n * n);
  double* Lb = (double*)rsd_scratch(ctx, "L", sizeof(double) * n * n);
  double* V = (double*)rsd_scratch(ctx, "nog_vec", sizeof(double) * (3 * p + 2 * q + 8 * p));
  if (!M || !Lb || !V) return RSD_ENOMEM;
  // MobToResist_FTS
  RSD_TRY(put_block(ctx, M, n, APP, p, p));
  RSD_TRY(put_block(ctx, M + p * n, n, APQ, p, q));
  RSD_TRY(put_block(ctx, M + p + p * n, n, AQQ, q, q));
  int inf_m = 0;
  RSD_TRY(rsd_potrf_upper_tag(ctx, (int)n, M, n, &inf_m, "mob"));
  if (inf_m) {
    *info = inf_m;
    return RSD_OK;
  }
  RSD_TRY(rsd_potri_upper_tag(ctx, (int)n, M, n, "mob"));
  RSD_TRY(rsd_mirror_upper(ctx, (int)n, M, n));
  // arrangResist: R = R0 + [rfu rfe; . rse] on the blocks used below
  RSD_TRY(put_block(ctx, Lb, n, rfu, p, p));
  RSD_TRY(put_block(ctx, Lb + p * n, n, rfe, p, q));
  RSD_TRY(put_block(ctx, Lb + p + p * n, n, rse, q, q));
  // R += L on the P-P, P-Q and Q-Q blocks
  {
    RSD_TRY(rsd_axpy_block(ctx, p, p, Lb, n, M, n));
    RSD_TRY(rsd_axpy_block(ctx, p, q, Lb + p * n, n, M + p * n, n));
    RSD_TRY(rsd_axpy_block(ctx, q, q, Lb + p + p * n, n, M + p + p * n, n));
  }
  // RHS: [Fe + RPQ EIN, RPQ EIN, Fe_inter]
  double* X = V;                  // p x 3
  double* ein = V + 3 * p;        // q
  double* UB = V + 3 * p + q;     // p
  double* tmp = V + 4 * p + q;    // 3 q
  RSD_CUDA(ctx, cudaMemcpyAsync(ein, EIN, sizeof(double) * q, cudaMemcpyHostToDevice, s));
  RSD_CUDA(ctx, cudaMemcpyAsync(X, Fe, sizeof(double) * p, cudaMemcpyHostToDevice, s));
  RSD_CUDA(ctx, cudaMemsetAsync(X + p, 0, sizeof(double) * p, s));
  RSD_CUDA(ctx, cudaMemcpyAsync(X + 2 * p, Fe_inter, sizeof(double) * p, cudaMemcpyHostToDevice, s));
  RSD_CUDA(ctx, cudaMemsetAsync(UB, 0, sizeof(double) * p, s));
  if (u_brown) RSD_CUDA(ctx, cudaMemcpyAsync(UB, u_brown, sizeof(double) * 3 * nn, cudaMemcpyHostToDevice, s));
  const double* RPQd = M + p * n;
  rsd_gemm_f64(s, (int)p, 1, (int)q, 1.0, RPQd, n, 0, ein, q, 0, 1.0, X, p);
  rsd_gemm_f64(s, (int)p, 1, (int)q, 1.0, RPQd, n, 0, ein, q, 0, 0.0, X + p, p);
  // RPP (factor and inverse on a copy so RPQ/RQQ stay intact)
  double* P = (double*)rsd_scratch(ctx, "nog_RPP", sizeof(double) * p * p);
  if (!P) return RSD_ENOMEM;
  RSD_CUDA(ctx, cudaMemcpy2DAsync(P, p * sizeof(double), M, n * sizeof(double), p * sizeof(double), p,
                                  cudaMemcpyDeviceToDevice, s));
  int inf_r = 0;
  RSD_TRY(rsd_potrf_upper_tag(ctx, (int)p, P, p, &inf_r, "rpp"));
  if (inf_r) {
    *info = inf_r;
    return RSD_OK;
  }
  RSD_TRY(rsd_potrs_upper_tag(ctx, (int)p, P, p, X, p, 3, "rpp"));
  // S_hyd = RPQ^T X1 - RQQ EIN ; S_FP(part) = RPQ^T X2 ; S_B = RPQ^T UB
  double* S = tmp;  // 3 q
  rsd_gemm_f64(s, (int)q, 1, (int)p, 1.0, RPQd, n, 1, X + p, p, 0, 0.0, S, q);
  rsd_gemm_f64(s, (int)q, 1, (int)q, -1.0, M + p + p * n, n, 0, ein, q, 0, 1.0, S, q);
  rsd_gemm_f64(s, (int)q, 1, (int)p, 1.0, RPQd, n, 1, X + 2 * p, p, 0, 0.0, S + q, q);
  rsd_gemm_f64(s, (int)q, 1, (int)p, 1.0, RPQd, n, 1, UB, p, 0, 0.0, S + 2 * q, q);
  RSD_CUDA(ctx, cudaGetLastError());
  RSD_CUDA(ctx, cudaMemcpyAsync(U_par, X, sizeof(double) * p, cudaMemcpyDeviceToHost, s));
  RSD_CUDA(ctx, cudaMemcpyAsync(SijN_hyd, S, sizeof(double) * q, cudaMemcpyDeviceToHost, s));
  RSD_CUDA(ctx, cudaMemcpyAsync(SijN_FP, S + q, sizeof(double) * q, cudaMemcpyDeviceToHost, s));
  RSD_CUDA(ctx, cudaMemcpyAsync(SijN_B, S + 2 * q, sizeof(double) * q, cudaMemcpyDeviceToHost, s));
  // Rheology leaves RPP inverted
  if (RPP) {
    RSD_TRY(rsd_potri_upper_tag(ctx, (int)p, P, p, "rpp"));
    RSD_TRY(rsd_mirror_upper(ctx, (int)p, P, p));
    RSD_CUDA(ctx, cudaMemcpyAsync(RPP, P, sizeof(double) * p * p, cudaMemcpyDeviceToHost, s));
  }
  RSD_TRY(sync(ctx));
  // stresslet dipole of the interparticle forces (Rheology 425-444)
  for (int kk = 0; conf && kk < nn; kk++) {
    double Sij[9];
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++)
        Sij[i + 3 * j] = 0.5 * (conf[3 * kk + i] * Fe_inter[3 * kk + j] + conf[3 * kk + j] * Fe_inter[3 * kk + i]);
    double part[5];
    ei_trans_y2(Sij, part);
    for (int m = 0; m < 5; m++) SijN_FP[5 * kk + m] += part[m];
  }
  *info = 0;
  return RSD_OK;
}

extern "C" int rsd_stepper_nogmres(rsd_ctx* ctx, int32_t nn, const double* APP, const double* APQ, const double* AQQ,
                                   const double* rfu, const double* rfe, const double* rse, const double* Fe,
                                   const double* EIN, const double* Fe_inter, const double* conf,
                                   const double* u_brown, double* U_par, double* SijN_hyd, double* SijN_FP,
                                   double* SijN_B, double* RPP, int32_t* info) {
  if (!ctx || nn < 1 || !APP || !APQ || !AQQ || !rfu || !rfe || !rse || !Fe || !EIN || !Fe_inter || !conf ||
      !U_par || !SijN_hyd || !SijN_FP || !SijN_B || !RPP || !info)
    return rsd_fail(ctx, RSD_EARG, "rsd_stepper_nogmres: bad arguments");
  return nogmres_impl(ctx, nn, APP, APQ, AQQ, rfu, rfe, rse, Fe, EIN, Fe_inter, conf, u_brown, U_par, SijN_hyd,
                      SijN_FP, SijN_B, RPP, info);
}

// hydro_SD_FTS: the solution of the FTS resistance problem that the
// reference's splitting iteration approaches, U = RPP^-1 (Fe + RPQ EIN) and
// S = RPQ^T U - RQQ EIN (= mu EIN + RPQ^T RPP^-1 Fe), solved directly.
extern "C" int rsd_hydro_sd_fts(rsd_ctx* ctx, int32_t nn, const double* APP, const double* APQ, const double* AQQ,
                                const double* rfu, const double* rfe, const double* rse, const double* Fe,
                                const double* EIN, double* U_par, double* SijN, int32_t* info) {
  if (!ctx || nn < 1 || !APP || !APQ || !AQQ || !rfu || !rfe || !rse || !Fe || !EIN || !U_par || !SijN || !info)
    return rsd_fail(ctx, RSD_EARG, "rsd_hydro_sd_fts: bad arguments");
  std::vector<double> s_fe(5 * (size_t)nn), s_b(5 * (size_t)nn);
  RSD_TRY(nogmres_impl(ctx, nn, APP, APQ, AQQ, rfu, rfe, rse, Fe, EIN, Fe, nullptr, nullptr, U_par, SijN,
                       s_fe.data(), s_b.data(), nullptr, info));
  if (*info == 0)
    for (size_t k = 0; k < s_fe.size(); k++) SijN[k] += s_fe[k];
  return RSD_OK;
}
