// Internal declarations shared by the CUDA translation units.
#pragma once
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <cstdint>
#include <cstdio>
#include <atomic>
#include <map>
#include <string>

#include "../../include/rsd_capi.h"

#define RSD_PI 3.141592653589793238462643383279502884
#define RSD_PIP5 0.564189583547756286948079451560772585844

// Count of kernel launches issued by this library (a diagnostic the
// benchmark reports for its timed region).
extern std::atomic<long long> rsd_launches;
#define RSD_LAUNCH_NOTE() rsd_launches.fetch_add(1, std::memory_order_relaxed)

struct rsd_buf {
  void* p = nullptr;
  size_t bytes = 0;
};

struct rsd_ctx {
  int device = 0;
  int sm_count = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  std::map<std::string, rsd_buf> bufs;  // grow-only device buffers by name
  cudaEvent_t ev[8] = {};
  double phase_ms[4] = {0, 0, 0, 0};
  int use_tc = 1;         // FP32 factorisations: 0 SIMT, 1 per-factor TF32/3xTF32, 3 all 3xTF32
  double mixed_rcut = 4.5;  // mixed assembly: FP64 real images below this lambda r
  int mixed_kshell = 1;     // mixed assembly: FP64 reciprocal shells max|n_i| <= this
  double mixed_rmax = 6.0;  // mixed assembly: real images with lambda r beyond this dropped
  double mixed_kexp = 10.0 * 3.141592653589793;  // and reciprocal vectors with k^2/(4 lambda^2) beyond this
  int mixed_real_passes = 1;  // mixed assembly, equal radii: passes over the near images (moment parts)
  double mixed_lambda_scale = 1.75;  // mixed assembly: Ewald splitting parameter relative to the reference's
  int correction_method = 0;  // fused step: overlap corrections of the grand mobility (0, 1 or 2)
  long long tc_wait_ns = 0;      // bound of the tensor-core kernels' mbarrier waits (0: 0.5 s)
  long long tri_spin_polls = 0;  // bound of the dataflow sweeps' waits in polls (0: 2^21)
  int factor_schedule = 1;   // two-level FP32 Cholesky: 1 look-ahead on the diagonal chain, 0 in-order panels
  int refine_gmres = 0;      // mixed form: flexible GMRES (1) or the stationary iteration (0) as refinement
  int gmres_restart = 30;    // GMRES restart length
  int rpp_mode = 0;          // plain FP64 step: RPP by Cholesky (0) or PCG with this preconditioner
  void* rpp_net = nullptr;   // the network of the learned preconditioner
  double rpp_tol = 0.0;      // PCG relative residual (0: 1e-12)
  int rpp_maxit = 0;         // PCG iteration cap (0: 1000)
  cudaStream_t side = nullptr;   // higher-priority stream for look-ahead panels
  cudaStream_t side2 = nullptr;  // second high-priority stream: the wide panel work beside the diagonal chain
  cudaEvent_t ev_panel = nullptr, ev_next = nullptr;
  cudaEvent_t ev_la[4] = {};     // look-ahead events of the two-level Cholesky
  int* d_info = nullptr;  // device-side status words
  int* h_info = nullptr;  // pinned mirror
};

struct rsd_lubtab {
  int nabc = 0, ngh = 0, nm = 0;
  double abc[64 * 11];
  double gh[64 * 7];
  double m[64 * 4];
  // device copy, per device ordinal (small; uploaded on first use)
  std::map<int, double*> dev;
};

// Error helpers: record a message in the context and return a status.
int rsd_fail(rsd_ctx* ctx, int code, const char* fmt, ...);
int rsd_cuda_check(rsd_ctx* ctx, cudaError_t e, const char* what);
#define RSD_CUDA(ctx, call)                                   \
  do {                                                        \
    cudaError_t _e = (call);                                  \
    if (_e != cudaSuccess) return rsd_cuda_check(ctx, _e, #call); \
  } while (0)
#define RSD_TRY(call)        \
  do {                       \
    int _rc = (call);        \
    if (_rc != 0) return _rc; \
  } while (0)

// Grow-only named device buffer; returns nullptr (and sets ctx->err) on
// allocation failure.
void* rsd_scratch(rsd_ctx* ctx, const char* name, size_t bytes);
int rsd_set_device(rsd_ctx* ctx);
// Scoped NVTX range around a phase of the step (a no-op unless a profiler
// is attached), so that a profiler can select one phase's launches.
struct rsd_range {
  explicit rsd_range(const char* name) { nvtxRangePushA(name); }
  ~rsd_range() { nvtxRangePop(); }
  rsd_range(const rsd_range&) = delete;
  rsd_range& operator=(const rsd_range&) = delete;
};

// creates ctx->side, side2, ev_panel, ev_next and ev_la on first use
int rsd_side_stream(rsd_ctx* ctx);

// ------------------------------------------------------------ lattice
struct rsd_lat_dev {
  double LR[9], LI[9], LV, lam, phix;
  int NR, NI;
};
rsd_lat_dev rsd_lat_pack(const rsd_lattice* lat);
// CALC_LATTICE_INVERSE's derived values (lammda, sig, logerr, NR, NI, phi)
// from lat->LR, lat->LV, EWS_ERR and the cube sum of the radii (capi.cu)
int rsd_lattice_params(rsd_lattice* lat, double ews_err, double sum_a3);

// PER_SKEW_CORRECTION (src/csd_post.f90:24-63): minimum image in the
// skewed lattice, testing the 8 corner shifts like the reference.
__host__ __device__ inline void rsd_skew_correction(const double* LR, const double* LI, double R[3], double* dmin) {
  double X[3], RC[3], RMIN[3];
  for (int i = 0; i < 3; i++) X[i] = LI[i] * R[0] + LI[i + 3] * R[1] + LI[i + 6] * R[2];
  for (int i = 0; i < 3; i++) {
    X[i] = fmod(X[i], 1.0);
    if (X[i] < 0.0) X[i] = X[i] + 1.0;
  }
  for (int i = 0; i < 3; i++) RC[i] = LR[i] * X[0] + LR[i + 3] * X[1] + LR[i + 6] * X[2];
  double D0 = RC[0] * RC[0] + RC[1] * RC[1] + RC[2] * RC[2];
  for (int i = 0; i < 3; i++) RMIN[i] = RC[i];
  for (int m = 1; m < 8; m++) {
    const double M0 = (m >> 2) & 1, M1 = (m >> 1) & 1, M2 = m & 1;
    double d = 0.0, RL[3];
    for (int i = 0; i < 3; i++) RL[i] = LR[i] * M0 + LR[i + 3] * M1 + LR[i + 6] * M2;
    for (int i = 0; i < 3; i++) d += (RC[i] - RL[i]) * (RC[i] - RL[i]);
    if (d < D0) {
      D0 = d;
      for (int i = 0; i < 3; i++) RMIN[i] = RC[i] - RL[i];
    }
  }
  for (int i = 0; i < 3; i++) R[i] = RMIN[i];
  *dmin = sqrt(D0);
}

// The lattice shift of rsd_skew_correction, found in FP32: the integer
// multiples k of the lattice vectors (columns of LR) with R - LR k the
// minimum image among the 8 corner shifts of the cell R falls in.  Where two
// images are within FP32 rounding of each other either may be chosen; both
// are minimum images to that accuracy.  For screening and for kernels that
// apply the shift in their own precision (no FP64 operations).
__host__ __device__ inline void rsd_skew_shift_f32(const float* LR, const float* LI, const float R[3], int k[3]) {
  float X[3], RC[3];
  for (int i = 0; i < 3; i++) {
    X[i] = floorf(LI[i] * R[0] + LI[i + 3] * R[1] + LI[i + 6] * R[2]);
    k[i] = (int)X[i];
  }
  for (int i = 0; i < 3; i++) RC[i] = R[i] - (LR[i] * X[0] + LR[i + 3] * X[1] + LR[i + 6] * X[2]);
  float D0 = RC[0] * RC[0] + RC[1] * RC[1] + RC[2] * RC[2];
  int best = 0;
  for (int m = 1; m < 8; m++) {
    const float M0 = (float)((m >> 2) & 1), M1 = (float)((m >> 1) & 1), M2 = (float)(m & 1);
    float d = 0.f;
    for (int i = 0; i < 3; i++) {
      const float e = RC[i] - (LR[i] * M0 + LR[i + 3] * M1 + LR[i + 6] * M2);
      d += e * e;
    }
    if (d < D0) {
      D0 = d;
      best = m;
    }
  }
  k[0] += (best >> 2) & 1;
  k[1] += (best >> 1) & 1;
  k[2] += best & 1;
}

// ------------------------------------------------------------ kernels
// Ewald (ewald.cu).  RSD_PREC_FP64: d_M is the FP64 grand mobility (ld
// ldm).  RSD_PREC_MIXED: the same buffer holds it as two FP32 planes, hi at
// (float*)d_M and lo at (float*)d_M + ldm * 11 nn, both with ld ldm, and
// only the entries whose row's particle is at most the column's are written
// (M is symmetric); rsd_mirror_planes fills the others.
int rsd_ewald_assemble(rsd_ctx* ctx, int nn, const double* d_pos, const double* d_radii, const rsd_lattice* lat,
                       double mu_f, int precision, double* d_M, int64_t ldm);
int rsd_mirror_planes(rsd_ctx* ctx, int nn, double* d_M, int64_t ldm);
int rsd_count_overlaps(rsd_ctx* ctx, int nn, const double* d_pos, const double* d_radii, const rsd_lattice* lat,
                       int* count);
// Adds the overlap correction of correction_method 1 or 2 (GRPY_YZD.f90:
// 789-836) for the npair overlapping pairs that rsd_count_overlaps counted,
// to the grand mobility in the layout of `precision` (FP64, or the mixed
// form's FP32 planes over the stored half).
int rsd_overlap_correct(rsd_ctx* ctx, int method, int precision, int nn, const double* d_pos, const double* d_radii,
                        const rsd_lattice* lat, double mu_f, int npair, double* d_M, int64_t ldm);
// Lubrication (lub.cu)
int rsd_lub_assemble(rsd_ctx* ctx, const rsd_lubtab* tab, int nn, int nb, int is_period, const double* d_pos,
                     const double* d_radii, const rsd_lattice* lat, double mu_f, double* d_L, int64_t ldl,
                     int accumulate, int* n_contact);
// Sparse lubrication operator of the mixed-precision refinement (lub.cu):
// the near-pair blocks (139 unscaled values each) and the per-particle self
// blocks (121 scaled values each, entry (r, c) at r + 11 c).
struct rsd_lub_sparse {
  int nn = 0, npair = 0;
  const int2* pairs = nullptr;
  const double* blk = nullptr;
  const int *off = nullptr, *off2 = nullptr, *list2 = nullptr;
  const double* self = nullptr;
  double scale = 0.0;
};
int rsd_lub_build_sparse(rsd_ctx* ctx, const rsd_lubtab* tab, int nn, int nb, int is_period, const double* d_pos,
                         const double* d_radii, const rsd_lattice* lat, double mu_f, rsd_lub_sparse* sp,
                         int* n_contact);
int rsd_lub_spmv(rsd_ctx* ctx, const rsd_lub_sparse* sp, int nr, const double* w, int64_t ldw, double* y,
                 int64_t ldy);
int rsd_lub_add_pp_f32(rsd_ctx* ctx, const rsd_lub_sparse* sp, float* A, int64_t lda);
// Dense linear algebra (dense.cu)
int rsd_potrf_upper(rsd_ctx* ctx, int n, double* d_A, int64_t lda, int* info);
int rsd_potri_upper(rsd_ctx* ctx, int n, double* d_A, int64_t lda);  // after potrf; result upper
int rsd_mirror_upper(rsd_ctx* ctx, int n, double* d_A, int64_t lda);
int rsd_trsv_upper(rsd_ctx* ctx, int n, const double* d_U, int64_t ldu, double* d_X, int64_t ldx, int nrhs,
                   int transpose);
// Tagged variants: the diagonal-block inverses of a factorisation are kept
// in a scratch buffer named by `tag`, so two factorisations can coexist.
int rsd_potrf_upper_tag(rsd_ctx* ctx, int n, double* d_A, int64_t lda, int* info, const char* tag);
int rsd_potri_upper_tag(rsd_ctx* ctx, int n, double* d_A, int64_t lda, const char* tag);
int rsd_potrs_upper_tag(rsd_ctx* ctx, int n, const double* d_U, int64_t ldu, double* d_X, int64_t ldx, int nrhs,
                        const char* tag);
void rsd_gemm_f64(cudaStream_t s, int m, int n, int k, double alpha, const double* A, int64_t lda, int ta,
                  const double* B, int64_t ldb, int tb, double beta, double* C, int64_t ldc);
int rsd_zero_lower(rsd_ctx* ctx, int n, double* d_A, int64_t lda);
// A(rows x cols) += B, both column-major sub-blocks (step.cu)
int rsd_axpy_block(rsd_ctx* ctx, int64_t rows, int64_t cols, const double* B, int64_t ldb, double* A, int64_t lda);

// Tensor-core (tcgen05) GEMM on K-major FP32 operands (tc_gemm.cu):
// C = alpha A^T B (store) or C += alpha A^T B (reduce) on 128-tiles, prec 1
// (TF32) or 3 (3xTF32); and the blocked-Cholesky trailing update on top of it.
int rsd_tc_gemm_ok(const float* A, int64_t lda, const float* B, int64_t ldb, const float* C, int64_t ldc);
int rsd_tc_gemm(rsd_ctx* ctx, int prec, int m, int n, int K, float alpha, const float* A, int64_t lda,
                const float* B, int64_t ldb, float* C, int64_t ldc, int reduce, int tri, int klo_col, int* d_err,
                cudaStream_t stream = 0, int ksplit = 0);
int rsd_tc_gemm_zbatch(rsd_ctx* ctx, int prec, int m, int n, int K, float alpha, const float* A, int64_t lda,
                       int64_t a_rows, int64_t a_cols, const float* B, int64_t ldb, int64_t b_rows, int64_t b_cols,
                       float* C, int64_t ldc, int64_t c_rows, int64_t c_cols, int nbatch, int zak, int zam, int zbk,
                       int zbn, int zcm, int zcn, int ndec, int* d_err);
int rsd_tc_syrk_ok(const float* panel, int64_t lda, const float* C, int64_t ldc, int kb);
int rsd_tc_syrk(rsd_ctx* ctx, int prec, const float* panel, int64_t lda, int kb, int rest, float* C, int64_t ldc,
                int* d_err);

// Block-scaled FP32 factor for the refinement solves (dense.cu): U = D Uh with
// D = blockdiag(U_bb) over 512-blocks; Uh's strict upper block strips and the
// blocks G_b = (U_bb^T U_bb)^-1.
struct rsd_uhat {
  int n = 0;
  const float* Uh = nullptr;
  int64_t ld = 0;
  const float* G = nullptr;
};
int rsd_uhat_build(rsd_ctx* ctx, int n, const float* U, int64_t ldu, const float* W2, const char* tag, rsd_uhat* out);
// zero_lead: the number of leading entries of X known to be zero (the
// forward sweep skips the whole zero blocks)
int rsd_uhat_solve(rsd_ctx* ctx, const rsd_uhat* h, float* X, int64_t ldx, int nrhs, float* Y, int zero_lead = 0);
// device word that turns nonzero when a wait of the solves' dataflow sweeps
// timed out (zero it before the solves, read it after synchronising)
int* rsd_uhat_error_flag(rsd_ctx* ctx);
