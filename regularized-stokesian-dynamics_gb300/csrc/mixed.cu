// Mixed-precision grand-resistance solve: FP32 factorisations, FP64
// refinement.  Same outputs as STEPPER_NOGmres (src/stepper.f90:348-410):
// U_par = RPP^-1 (Fe + RPQ EIN) and SijN_hyd = (RPQ^T RPP^-1 RPQ - RQQ) EIN
// with R = M^-1 + L, but without forming M^-1.
//
// Augmented system in (f, U), with w = [U; -EIN]:
//     M f = w                    (f = R_inf w, the far-field forces)
//     f_P + (L w)_P = Fe          (force balance with lubrication)
// and then SijN_hyd = f_Q + (L w)_Q.  Its residual needs only the products
// M f (an HBM-bound dense GEMV in double-single arithmetic over M's two
// FP32 planes, ~FP64 accuracy for the sums) and L w (an FP64 block-sparse
// product over the near pairs, L is never formed densely here).  The correction is
// solved with FP32 factors:
//   M' = [M_QQ M_QP; M_PQ M_PP] = U'^T U'  (stresslets ordered first), so the
//   trailing block U'_PP is the Cholesky factor of the Schur complement
//   A = M_PP - M_PQ M_QQ^-1 M_QP and (M^-1)_PP = A^-1 = U'_PP^-1 U'_PP^-T;
//   RPP32 = A^-1 + rfu = V^T V.
//   correction: y = M^-1 r1; dU = RPP^-1 (r2 - y_P); df = y + M^-1 [dU; 0].
// Iterates until ||r|| <= tol ||b|| per right-hand side.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "dsf.cuh"
#include "rsd_internal.cuh"

template <typename T>
int rsd_gemv(rsd_ctx* ctx, int trans, int m, int k, T alpha, const T* A, int64_t lda, const T* X, int64_t ldx,
             int nrhs, T beta, T* y, int64_t ldy);
template <typename T>
int rsd_potrf_upper_t(rsd_ctx* ctx, int n, T* d_A, int64_t lda, int* info, const char* tag, int tc);
template <typename T>
int rsd_potri_upper_t(rsd_ctx* ctx, int n, T* d_A, int64_t lda, const char* tag, int tc);
template <typename T>
int rsd_potrs_upper_t(rsd_ctx* ctx, int n, const T* d_U, int64_t ldu, T* d_X, int64_t ldx, int nrhs, const char* tag,
                      const T* W);
template <typename T>
int rsd_mirror_upper_t(rsd_ctx* ctx, int n, T* d_A, int64_t lda);
template <typename T>
int rsd_diag_inverses_t(rsd_ctx* ctx, int n, const T* U, int64_t ldu, const char* tag, T** Wout);
int rsd_wide_inverses_s(rsd_ctx* ctx, int n, const float* U, int64_t ldu, const char* tag, const float* W128,
                        float** W2out);
const float* rsd_potrf_inverses_s(rsd_ctx* ctx, int n, const char* tag);
int rsd_potrs_wide_s(rsd_ctx* ctx, int n, const float* U, int64_t ldu, const float* W2, float* X, int64_t ldx,
                     int nrhs, float* Y);

namespace {

// particle of grand-matrix index x
__device__ __forceinline__ int grand_pid(int N, int x) {
  return x < 3 * N ? x / 3 : (x < 6 * N ? (x - 3 * N) / 3 : (x - 6 * N) / 5);
}

// M32 = M in [Q, P] order from the hi plane holding only the stored half
// (entries whose row's particle is at most the column's; the rest is read
// at the transposed position): 32 x 32 output tiles, the direct and the
// transposed source tiles staged in shared memory so that reads and writes
// stay coalesced; a tile loads only the kinds it needs.
__device__ __forceinline__ int64_t perm_src(int N, int64_t i) {
  const int64_t Q = 5LL * N;
  return i < Q ? 6LL * N + i : i - Q;
}

__global__ void convert_perm_half(int N, int64_t n, const float* __restrict__ Mh, int64_t ld,
                                  float* __restrict__ M32) {
  __shared__ float D[32][33], T[32][33];
  __shared__ int64_t si[32], sj[32];
  __shared__ int pi[32], pj[32], need;
  const int64_t I0 = (int64_t)blockIdx.x * 32, J0 = (int64_t)blockIdx.y * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;
  if (ty == 0) {
    const int64_t i = min(I0 + tx, n - 1), j = min(J0 + tx, n - 1);
    si[tx] = perm_src(N, i);
    sj[tx] = perm_src(N, j);
    pi[tx] = grand_pid(N, (int)si[tx]);
    pj[tx] = grand_pid(N, (int)sj[tx]);
    // need: bit 0 = some entry stored directly, bit 1 = some entry transposed
    const int imin = __reduce_min_sync(0xffffffffu, pi[tx]), imax = __reduce_max_sync(0xffffffffu, pi[tx]);
    const int jmin = __reduce_min_sync(0xffffffffu, pj[tx]), jmax = __reduce_max_sync(0xffffffffu, pj[tx]);
    if (tx == 0) need = (imin <= jmax ? 1 : 0) | (imax > jmin ? 2 : 0);
  }
  __syncthreads();
  const int t = ty * 32 + tx;
  const bool full = I0 + 32 <= n && J0 + 32 <= n && si[31] - si[0] == 31;  // rows contiguous in the source
  if (need == 1 && full && (ld & 3) == 0 && (n & 3) == 0 && (si[0] & 3) == 0) {
    // all in place: one 16-byte move per thread (4 rows of one column)
    const int r4 = 4 * (t & 7), k = t >> 3;
    *reinterpret_cast<float4*>(M32 + I0 + r4 + (J0 + k) * n) =
        *reinterpret_cast<const float4*>(Mh + si[0] + r4 + sj[k] * ld);
    return;
  }
  for (int k = ty; k < 32; k += blockDim.y) {
    if (need & 1) D[k][tx] = Mh[si[tx] + sj[k] * ld];  // (I0 + tx, J0 + k) in place
    if (need & 2) T[k][tx] = Mh[sj[tx] + si[k] * ld];  // (I0 + k, J0 + tx) at the mirrored position
  }
  __syncthreads();
  for (int k = ty; k < 32; k += blockDim.y) {
    const int64_t i = I0 + tx, j = J0 + k;
    if (i < n && j < n) M32[i + j * n] = pi[tx] <= pj[k] ? D[k][tx] : T[tx][k];
  }
}

// x (FP64) as float pairs
__global__ void to_dsf_vec(int64_t n, const double* __restrict__ x, float2* __restrict__ xs) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const dsf d = dsf_from(x[t]);
  xs[t] = make_float2(d.hi, d.lo);
}

// part[c][r][i] = sum over the chunk c of columns p of M(i, p) x(p, r), with
// M = hi + lo and x as float pairs, in double-single arithmetic on the FP32
// pipe (the FP64 pipe of GB300 would bound an FP64 product at ~1/60 of the
// FP32 rate; this one is bound by HBM).  Chunks of GEMV_PL_CHUNK columns
// keep the double-single rounding of each partial near 2^-48 sqrt(chunk).
constexpr int GEMV_PL_CHUNK = 512;
template <int R>
__global__ void gemv_planes_part(int m, int k, const float* __restrict__ Mh, const float* __restrict__ Ml, int64_t ld,
                                 const float2* __restrict__ xs, double* __restrict__ part) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  const int p0 = c * GEMV_PL_CHUNK, p1 = min(k, p0 + GEMV_PL_CHUNK);
  if (i >= m) return;
  dsf acc[R];
#pragma unroll
  for (int r = 0; r < R; r++) acc[r] = dsf(0);
#pragma unroll 4
  for (int p = p0; p < p1; p++) {
    const int64_t o = i + (int64_t)p * ld;
    const dsf a(Mh[o], Ml[o]);
#pragma unroll
    for (int r = 0; r < R; r++) {
      const float2 x = xs[p + (int64_t)r * k];
      acc[r] = fma(a, dsf(x.x, x.y), acc[r]);
    }
  }
#pragma unroll
  for (int r = 0; r < R; r++) part[((size_t)c * R + r) * m + i] = dsf_to(acc[r]);
}

// Symmetric M f over the stored half of M's planes: the entries whose row's
// particle is at most the column's (pair blocks in the rows of their first
// particle, and the whole diagonal particle blocks).  A CTA takes a 128 x 128
// tile: row products of its stored entries (-> prow[R][C]) and column
// products of its entries strictly above the particle diagonal
// (-> pcol[C][R]), in double-single; tiles with no stored entry write zero
// partials.  About half of M is read.  Needs n % 4 == 0.
constexpr int SYMV_T = 128;
constexpr int symv_smem(int nr) { return (int)(sizeof(dsf) * 8 * nr * SYMV_T + sizeof(float2) * nr * SYMV_T * 33); }
template <int NR>
__global__ void __launch_bounds__(256) symv_planes_part(int N, int n, const float* __restrict__ Mh,
                                                        const float* __restrict__ Ml, int64_t ld,
                                                        const float2* __restrict__ xs, int nbt,
                                                        double* __restrict__ prow, double* __restrict__ pcol) {
  // dynamic shared memory (symv_smem(NR) bytes): the row partials of the 8
  // warps, then the per-lane column partials, reduced after the tile
  extern __shared__ __align__(16) unsigned char symv_raw[];
  auto red = reinterpret_cast<dsf(*)[NR][SYMV_T]>(symv_raw);
  auto colp = reinterpret_cast<float2(*)[SYMV_T][33]>(symv_raw + sizeof(dsf) * 8 * NR * SYMV_T);
  __shared__ int skip;
  const int R = blockIdx.x, C = blockIdx.y, r0 = R * SYMV_T, c0 = C * SYMV_T;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  double* pr = prow + ((size_t)R * nbt + C) * NR * SYMV_T;
  double* pc = pcol + ((size_t)C * nbt + R) * NR * SYMV_T;
  if (warp == 0) {  // stored entries exist iff min over rows of pid <= max over columns
    int rmin = 1 << 30, cmax = -1;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const int r = r0 + 4 * lane + k, c = c0 + 4 * lane + k;
      if (r < n) rmin = min(rmin, grand_pid(N, r));
      if (c < n) cmax = max(cmax, grand_pid(N, c));
    }
    rmin = __reduce_min_sync(0xffffffffu, rmin);
    cmax = __reduce_max_sync(0xffffffffu, cmax);
    if (lane == 0) skip = rmin > cmax;
  }
  __syncthreads();
  if (skip) {
    for (int e = t; e < NR * SYMV_T; e += 256) pr[e] = pc[e] = 0.0;
    return;
  }
  const int rb = r0 + 4 * lane;  // this lane's four rows (one section: boundaries are multiples of 4)
  int prr[4];
  dsf xr[NR][4];
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const bool ok = rb + k < n;
    prr[k] = ok ? grand_pid(N, rb + k) : (1 << 30);
#pragma unroll
    for (int r = 0; r < NR; r++) {
      const float2 v = ok ? xs[rb + k + (int64_t)r * n] : make_float2(0.f, 0.f);
      xr[r][k] = dsf(v.x, v.y);
    }
  }
  dsacc racc[NR][4];
#pragma unroll
  for (int r = 0; r < NR; r++)
#pragma unroll
    for (int k = 0; k < 4; k++) racc[r][k] = dsacc(0);
#pragma unroll 8
  for (int cc = 0; cc < SYMV_T / 8; cc++) {
    const int cl = warp * (SYMV_T / 8) + cc, c = c0 + cl;
    dsacc cacc[NR];
#pragma unroll
    for (int r = 0; r < NR; r++) cacc[r] = dsacc(0);
    if (c < n) {
      const int pcn = grand_pid(N, c);
      if (rb < n && prr[0] <= pcn) {  // the lane's rows hold stored entries of this column
        const int64_t o = rb + (int64_t)c * ld;
        const float4 h = *reinterpret_cast<const float4*>(Mh + o), l = *reinterpret_cast<const float4*>(Ml + o);
        const dsf m[4] = {dsf(h.x, l.x), dsf(h.y, l.y), dsf(h.z, l.z), dsf(h.w, l.w)};
#pragma unroll
        for (int r = 0; r < NR; r++) {
          const float2 xv = xs[c + (int64_t)r * n];
          const dsf xc(xv.x, xv.y);
#pragma unroll
          for (int k = 0; k < 4; k++) {
            if (prr[k] <= pcn) racc[r][k] = fma(m[k], xc, racc[r][k]);
            if (prr[k] < pcn) cacc[r] = fma(m[k], xr[r][k], cacc[r]);
          }
        }
      }
    }
#pragma unroll
    for (int r = 0; r < NR; r++) {
      dsacc_norm(cacc[r]);
      colp[r][cl][lane] = make_float2(cacc[r].hi, cacc[r].lo);
    }
  }
#pragma unroll
  for (int r = 0; r < NR; r++)
#pragma unroll
    for (int k = 0; k < 4; k++) {
      dsacc_norm(racc[r][k]);
      red[warp][r][4 * lane + k] = dsf(racc[r][k].hi, racc[r][k].lo);
    }
  __syncthreads();
  for (int e = t; e < NR * SYMV_T; e += 256) {
    const int r = e / SYMV_T, il = e % SYMV_T;
    dsf v = red[0][r][il];
#pragma unroll
    for (int w = 1; w < 8; w++) v = v + red[w][r][il];
    pr[e] = dsf_to(v);
    dsf u(colp[r][il][0].x, colp[r][il][0].y);
#pragma unroll 8
    for (int q = 1; q < 32; q++) u = u + dsf(colp[r][il][q].x, colp[r][il][q].y);
    pc[e] = dsf_to(u);
  }
}

// y(:, r) += alpha * (sum_C prow[K][C] + sum_R pcol[K][R]) for row block K, fixed order
__global__ void symv_planes_reduce(int n, int nr, int nbt, const double* __restrict__ prow,
                                   const double* __restrict__ pcol, double alpha, double* __restrict__ y,
                                   int64_t ldy) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int K = i / SYMV_T, e = i % SYMV_T;
  for (int r = 0; r < nr; r++) {
    double s0 = 0.0, s1 = 0.0;
    for (int J = 0; J < nbt; J++) {
      s0 += prow[(((size_t)K * nbt + J) * nr + r) * SYMV_T + e];
      s1 += pcol[(((size_t)K * nbt + J) * nr + r) * SYMV_T + e];
    }
    y[i + (int64_t)r * ldy] += alpha * (s0 + s1);
  }
}

// y(:, r) += alpha * sum_c part[c][r]
__global__ void gemv_planes_reduce(int m, int nr, int nchunk, const double* __restrict__ part, double alpha,
                                   double* __restrict__ y, int64_t ldy) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  for (int r = 0; r < nr; r++) {
    double s = 0.0;
    for (int c = 0; c < nchunk; c++) s += part[((size_t)c * nr + r) * m + i];
    y[i + (int64_t)r * ldy] += alpha * s;
  }
}

__global__ void copy_block_f(int64_t rows, int64_t cols, const float* __restrict__ S, int64_t lds,
                             float* __restrict__ D, int64_t ldd) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= rows * cols) return;
  const int64_t i = t % rows, j = t / rows;
  D[i + j * ldd] = S[i + j * lds];
}

// w = [U; -EIN] per column
__global__ void build_w(int64_t P, int64_t Q, int nr, const double* __restrict__ U, const double* __restrict__ ein,
                        double* __restrict__ w) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t n = P + Q;
  if (t >= n * nr) return;
  const int64_t i = t % n, c = t / n;
  w[t] = i < P ? U[i + c * P] : -ein[i - P];
}

// r2 = Fe_c - f_P - (Lw)_P  (Fe only in column 0 when have_fe)
__global__ void build_r2(int64_t P, int64_t n, int nr, const double* __restrict__ Fe, int have_fe,
                         const double* __restrict__ f, const double* __restrict__ Lw, double* __restrict__ r2) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= P * nr) return;
  const int64_t i = t % P, c = t / P;
  const double fe = (have_fe && c == 0) ? Fe[i] : 0.0;
  r2[t] = fe - f[i + c * n] - Lw[i + c * n];
}

// per-column sums of squares of r1 (n), r2 (P) and of b = ([0; -EIN], Fe)
__global__ void norms(int64_t P, int64_t n, int nr, const double* __restrict__ r1, const double* __restrict__ r2,
                      const double* __restrict__ ein, const double* __restrict__ Fe, int have_fe,
                      double* __restrict__ out) {
  __shared__ double sr[256], sb[256];
  const int c = blockIdx.x;
  double a = 0, b = 0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    const double v = r1[i + c * n];
    a += v * v;
    if (i >= P) {
      const double e = ein[i - P];
      b += e * e;
    }
  }
  for (int64_t i = threadIdx.x; i < P; i += blockDim.x) {
    const double v = r2[i + c * P];
    a += v * v;
    if (have_fe && c == 0) b += Fe[i] * Fe[i];
  }
  sr[threadIdx.x] = a;
  sb[threadIdx.x] = b;
  __syncthreads();
  for (int d = 128; d > 0; d >>= 1) {
    if (threadIdx.x < d) {
      sr[threadIdx.x] += sr[threadIdx.x + d];
      sb[threadIdx.x] += sb[threadIdx.x + d];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[2 * c] = sr[0];
    out[2 * c + 1] = sb[0];
  }
}

// x32' = perm(x) (FP32, [Q, P] order); x may have a zero Q part (zq)
__global__ void to32_perm(int64_t P, int64_t Q, int nr, const double* __restrict__ x, int64_t ldx, int zq,
                          float* __restrict__ y) {
  const int64_t n = P + Q;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * nr) return;
  const int64_t i = t % n, c = t / n;
  double v;
  if (i < Q)
    v = zq ? 0.0 : x[P + i + c * ldx];
  else
    v = x[i - Q + c * ldx];
  y[t] = (float)v;
}

// y (FP64, [P, Q] order) (+)= unperm(x32')
__global__ void from32_perm(int64_t P, int64_t Q, int nr, const float* __restrict__ x, double* __restrict__ y,
                            int add) {
  const int64_t n = P + Q;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * nr) return;
  const int64_t i = t % n, c = t / n;
  const double v = (double)(i < P ? x[Q + i + c * n] : x[i - P + c * n]);
  y[i + c * n] = add ? y[i + c * n] + v : v;
}

// u32 = r2 - y_P
__global__ void rhs_u(int64_t P, int64_t n, int nr, const double* __restrict__ r2, const double* __restrict__ y,
                      float* __restrict__ u) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= P * nr) return;
  const int64_t i = t % P, c = t / P;
  u[t] = (float)(r2[t] - y[i + c * n]);
}

__global__ void update_fu(int64_t P, int64_t n, int nr, const double* __restrict__ df, const float* __restrict__ du,
                          double* __restrict__ f, double* __restrict__ U) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n * nr) f[t] += df[t];
  if (t < P * nr) U[t] += (double)du[t];
}

// dU as an FP64 [dU; 0] vector block for the second M^-1 application
__global__ void du_vec(int64_t P, int64_t n, int nr, const float* __restrict__ du, double* __restrict__ v) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * nr) return;
  const int64_t i = t % n, c = t / n;
  v[t] = i < P ? (double)du[i + c * P] : 0.0;
}

// S = f_Q + (Lw)_Q of column c; U_par = U column 0
__global__ void outputs(int64_t P, int64_t Q, int c, const double* __restrict__ f, const double* __restrict__ Lw,
                        const double* __restrict__ U, double* __restrict__ Upar, double* __restrict__ S) {
  const int64_t n = P + Q;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < Q) S[t] = f[P + t + c * n] + Lw[P + t + c * n];
  if (t < P) Upar[t] = U[t];
}

inline unsigned nblk(int64_t n) { return (unsigned)((n + 255) / 256); }

// ---- flexible GMRES on the augmented system (one right-hand side at a time)
// x = (f [n], U [P]); A x = (M f - [U; 0], f_P + (L [U; 0])_P); the
// preconditioner is the correction of the stationary iteration above.
// Krylov vectors are FP64 of length n + P.

// out[k] = V_k . w for k < nk (one block per k)
__global__ void gm_dots(int64_t len, int nk, const double* __restrict__ V, int64_t ldv, const double* __restrict__ w,
                        double* __restrict__ out) {
  __shared__ double red[256];
  const int k = blockIdx.x;
  double a = 0.0;
  for (int64_t i = threadIdx.x; i < len; i += 256) a += V[i + k * ldv] * w[i];
  red[threadIdx.x] = a;
  __syncthreads();
  for (int d = 128; d > 0; d >>= 1) {
    if (threadIdx.x < d) red[threadIdx.x] += red[threadIdx.x + d];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[k] = red[0];
}

// w -= sum_k h[k] V_k; hacc[k] += h[k] (thread 0 of block 0)
__global__ void gm_orth(int64_t len, int nk, const double* __restrict__ V, int64_t ldv, const double* __restrict__ h,
                        double* __restrict__ w, double* __restrict__ hacc) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0)
    for (int k = 0; k < nk; k++) hacc[k] += h[k];
  if (i >= len) return;
  double s = w[i];
  for (int k = 0; k < nk; k++) s -= h[k] * V[i + k * ldv];
  w[i] = s;
}

// v = w / sqrt(nrm2[0])
__global__ void gm_scale(int64_t len, const double* __restrict__ w, const double* __restrict__ nrm2,
                         double* __restrict__ v) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < len) v[i] = w[i] / sqrt(nrm2[0]);
}

// x += sum_k y[k] Z_k
__global__ void gm_update(int64_t len, int nk, const double* __restrict__ Z, int64_t ldz, const double* __restrict__ y,
                          double* __restrict__ x) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= len) return;
  double s = 0.0;
  for (int k = 0; k < nk; k++) s += y[k] * Z[i + k * ldz];
  x[i] += s;
}

// w = [u; 0] (length n) from u (length P)
__global__ void gm_u0(int64_t P, int64_t n, const double* __restrict__ u, double* __restrict__ w) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) w[i] = i < P ? u[i] : 0.0;
}

// a1 = -w (then + M f by the symmetric product); a2 = f_P + Lw_P
__global__ void gm_neg(int64_t n, const double* __restrict__ w, double* __restrict__ a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = -w[i];
}
__global__ void gm_a2(int64_t P, const double* __restrict__ f, const double* __restrict__ Lw, double* __restrict__ a2) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < P) a2[i] = f[i] + Lw[i];
}

// FP32 vector to FP64
__global__ void gm_f2d(int64_t n, const float* __restrict__ x, double* __restrict__ y) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = (double)x[i];
}

// sum of squares of v[0:len] into out[0] (one block)
__global__ void gm_nrm2(int64_t len, const double* __restrict__ v, double* __restrict__ out) {
  __shared__ double red[256];
  double a = 0.0;
  for (int64_t i = threadIdx.x; i < len; i += 256) a += v[i] * v[i];
  red[threadIdx.x] = a;
  __syncthreads();
  for (int d = 128; d > 0; d >>= 1) {
    if (threadIdx.x < d) red[threadIdx.x] += red[threadIdx.x + d];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = red[0];
}

}  // namespace

// rpp_out (optional): stop once RPP32 = A^-1 + rfu is formed and copy it
// there (6nn x 6nn, ld rpp_ld, full symmetric storage, FP32).
int rsd_mixed_solve(rsd_ctx* ctx, int nn, double* M, int64_t ld, const double* d_pos, const double* d_radii,
                    const rsd_lattice* lat, const rsd_lubtab* tab, const rsd_step_params* p, const double* ein,
                    const double* Fe, double* U_par, double* S_hyd, rsd_step_info* info, float* rpp_out,
                    int64_t rpp_ld) {
  cudaStream_t s = ctx->stream;
  const int64_t N = nn, n = 11 * N, P = 6 * N, Q = 5 * N;
  const int have_fe = Fe != nullptr;
  const int nr = have_fe ? 2 : 1;
  const double tol = p->tol > 0 ? p->tol : 1e-12;
  const int maxit = p->max_iter > 0 ? p->max_iter : 50;
  // M as FP32 planes hi + lo in the buffer of the FP64 matrix (rsd_ewald_assemble)
  const float* Mh = reinterpret_cast<const float*>(M);
  const float* Ml = Mh + (size_t)ld * n;
  const unsigned gchunks = (unsigned)((n + GEMV_PL_CHUNK - 1) / GEMV_PL_CHUNK);
  const bool symv = n % 4 == 0 && ld % 4 == 0;
  bool mirrored = false;
  const int nbt = (int)((n + SYMV_T - 1) / SYMV_T);
  if (symv)
    RSD_CUDA(ctx, cudaFuncSetAttribute(symv_planes_part<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, symv_smem(2)));
  float2* fs = (float2*)rsd_scratch(ctx, "mixed_fs", sizeof(float2) * (size_t)nr * n);
  double* gpart = symv ? (double*)rsd_scratch(ctx, "mixed_symv_part", sizeof(double) * 2 * 2 * (size_t)nbt * nbt * SYMV_T)
                       : (double*)rsd_scratch(ctx, "mixed_gemv_part", sizeof(double) * (size_t)gchunks * nr * n);
  if (!fs || !gpart) return RSD_ENOMEM;
  float* M32 = (float*)rsd_scratch(ctx, "mixed_M32", sizeof(float) * n * n);
  float* A32 = (float*)rsd_scratch(ctx, "mixed_A32", sizeof(float) * P * P);
  double* V = (double*)rsd_scratch(ctx, "mixed_vec", sizeof(double) * (size_t)nr * (7 * n + 2 * P) + 64 * 8);
  float* V32 = (float*)rsd_scratch(ctx, "mixed_vec32", sizeof(float) * (size_t)nr * (2 * n + 2 * P));
  if (!M32 || !A32 || !V || !V32) return RSD_ENOMEM;
  double *f = V, *U = f + nr * n, *w = U + nr * P, *r1 = w + nr * n, *Lw = r1 + nr * n, *r2 = Lw + nr * n,
         *y = r2 + nr * P, *y2 = y + nr * n, *dv = y2 + nr * n, *nrm = dv + nr * n;
  float *t32 = V32, *u32 = V32 + nr * n, *ywork = u32 + nr * P;
  // sparse FP64 lubrication operator (R_lub - R_2B in the grand layout)
  int nc = 0;
  rsd_lub_sparse lub;
  if (p->use_lub) RSD_TRY(rsd_lub_build_sparse(ctx, tab, nn, p->nb, 1, d_pos, d_radii, lat, p->mu_f, &lub, &nc));
  info->n_contact = nc;
  cudaEventRecord(ctx->ev[6], s);
  // FP32 factor of M' (stresslets first)
  {
    const dim3 tg((unsigned)((n + 31) / 32), (unsigned)((n + 31) / 32));
    convert_perm_half<<<tg, dim3(32, 8), 0, s>>>(nn, n, Mh, ld, M32); RSD_LAUNCH_NOTE();
  }
  int inf = 0;
  // Tensor-core precision per factor.  The refinement contracts by about the
  // preconditioner's relative error times the condition number it meets:
  // cond(M') is moderate, so TF32 (2^-11) suffices for the factor of M' and
  // for the inverse A^-1 (at N = 2048, phi = 0.5: 7 iterations instead of 6
  // with 3xTF32 there, for half the inverse's time); the factor of RPP meets
  // cond(RPP), which grows like the inverse lubrication gap, and uses 3xTF32
  // (about 2^-21, close to FP32; TF32 there takes ~17 iterations).
  RSD_TRY(rsd_potrf_upper_t<float>(ctx, (int)n, M32, n, &inf, "m32", ctx->use_tc == 3 ? 3 : 1));
  if (inf) {
    info->info = inf;
    return rsd_fail(ctx, inf, "FP32 factor of the grand mobility: leading minor %d not positive", inf);
  }
  float* W_m = nullptr;
  RSD_TRY(rsd_wide_inverses_s(ctx, (int)n, M32, n, "m32", rsd_potrf_inverses_s(ctx, (int)n, "m32"), &W_m));
  // block-scaled factors for one-launch-per-block refinement solves (the
  // tensor-core GEMMs that form them need leading dimensions divisible by 4)
  rsd_uhat uh_m, uh_r;
  const bool use_uh = ctx->use_tc && n % 4 == 0 && P % 4 == 0 && !rpp_out;
  if (use_uh) RSD_TRY(rsd_uhat_build(ctx, (int)n, M32, n, W_m, "m32", &uh_m));
  // A^-1 from the trailing factor block, then RPP32 = A^-1 + rfu and its factor
  copy_block_f<<<nblk(P * P), 256, 0, s>>>(P, P, M32 + Q + Q * n, n, A32, P); RSD_LAUNCH_NOTE();
  RSD_TRY(rsd_potri_upper_t<float>(ctx, (int)P, A32, P, "a32", ctx->use_tc == 3 ? 3 : 1));
  RSD_TRY(rsd_mirror_upper_t<float>(ctx, (int)P, A32, P));
  if (p->use_lub) RSD_TRY(rsd_lub_add_pp_f32(ctx, &lub, A32, P));
  if (rpp_out) {
    RSD_CUDA(ctx, cudaMemcpy2DAsync(rpp_out, sizeof(float) * rpp_ld, A32, sizeof(float) * P, sizeof(float) * P, P,
                                    cudaMemcpyDeviceToDevice, s));
    return RSD_OK;
  }
  RSD_TRY(rsd_potrf_upper_t<float>(ctx, (int)P, A32, P, &inf, "rpp32", 3));
  if (inf) {
    info->info = inf;
    return rsd_fail(ctx, inf, "FP32 factor of RPP: leading minor %d not positive", inf);
  }
  float* W_r = nullptr;
  RSD_TRY(rsd_wide_inverses_s(ctx, (int)P, A32, P, "rpp32", rsd_potrf_inverses_s(ctx, (int)P, "rpp32"), &W_r));
  if (use_uh) RSD_TRY(rsd_uhat_build(ctx, (int)P, A32, P, W_r, "rpp32", &uh_r));
  // refinement
  int* tri_err = rsd_uhat_error_flag(ctx);
  if (!tri_err) return RSD_ENOMEM;
  RSD_CUDA(ctx, cudaMemsetAsync(tri_err, 0, sizeof(int), s));
  // Right-preconditioned flexible GMRES(m) per right-hand side, FP64
  // residuals; the preconditioner is the stationary iteration's correction.
  // Starts from zero; gm_maxit bounds the iterations over all right-hand
  // sides; returns the iterations and the worst relative residual.
  auto run_gmres = [&](int gm_maxit, int* its_out, double* res_out) -> int {
    const int m = ctx->gmres_restart > 0 ? ctx->gmres_restart : 30;
    const int64_t len = n + P;
    double* KV = (double*)rsd_scratch(ctx, "gm_basis", sizeof(double) * (size_t)(2 * m + 1) * len + 8 * 64);
    if (!KV) return RSD_ENOMEM;
    double *Vb = KV, *Zb = Vb + (size_t)(m + 1) * len, *dn = Zb + (size_t)m * len;
    double* hacc = (double*)rsd_scratch(ctx, "gm_hacc", sizeof(double) * 64);
    double* hbuf = (double*)rsd_scratch(ctx, "gm_hbuf", sizeof(double) * 64);
    double* Lz = (double*)rsd_scratch(ctx, "gm_lz", sizeof(double) * (size_t)n);
    if (!hacc || !hbuf || !Lz) return RSD_ENOMEM;
    RSD_CUDA(ctx, cudaMemsetAsync(f, 0, sizeof(double) * nr * n, s));
    RSD_CUDA(ctx, cudaMemsetAsync(U, 0, sizeof(double) * nr * P, s));
    // the product M v (FP64 v of length n, planes in double-single) into out (added)
    auto symv_add = [&](const double* v, double* out) -> int {
      to_dsf_vec<<<nblk(n), 256, 0, s>>>(n, v, fs); RSD_LAUNCH_NOTE();
      if (symv) {
        double* pcol = gpart + (size_t)nbt * nbt * SYMV_T;
        symv_planes_part<1><<<dim3(nbt, nbt), 256, symv_smem(1), s>>>(nn, (int)n, Mh, Ml, ld, fs, nbt, gpart, pcol); RSD_LAUNCH_NOTE();
        symv_planes_reduce<<<(unsigned)((n + 255) / 256), 256, 0, s>>>((int)n, 1, nbt, gpart, pcol, 1.0, out, n); RSD_LAUNCH_NOTE();
      } else {
        if (!mirrored) {
          RSD_TRY(rsd_mirror_planes(ctx, nn, M, ld));
          mirrored = true;
        }
        gemv_planes_part<1><<<dim3((unsigned)((n + 255) / 256), gchunks), 256, 0, s>>>((int)n, (int)n, Mh, Ml, ld, fs, gpart); RSD_LAUNCH_NOTE();
        gemv_planes_reduce<<<(unsigned)((n + 255) / 256), 256, 0, s>>>((int)n, 1, gchunks, gpart, 1.0, out, n); RSD_LAUNCH_NOTE();
      }
      return RSD_OK;
    };
    // residual of column c: (r1, r2) = b - A x into out (length n + P);
    // Lw (column c) keeps L [U; -EIN] for the stresslet output
    auto residual = [&](int c, double* out) -> int {
      double *fc = f + (size_t)c * n, *Uc = U + (size_t)c * P, *wc = w + (size_t)c * n, *Lc = Lw + (size_t)c * n;
      build_w<<<nblk(n), 256, 0, s>>>(P, Q, 1, Uc, ein, wc); RSD_LAUNCH_NOTE();
      gm_neg<<<nblk(n), 256, 0, s>>>(n, wc, out); RSD_LAUNCH_NOTE();
      RSD_TRY(symv_add(fc, out));  // out = M f - w
      gm_neg<<<nblk(n), 256, 0, s>>>(n, out, out); RSD_LAUNCH_NOTE();  // r1 = w - M f
      if (p->use_lub) {
        RSD_TRY(rsd_lub_spmv(ctx, &lub, 1, wc, n, Lc, n));
      } else {
        RSD_CUDA(ctx, cudaMemsetAsync(Lc, 0, sizeof(double) * n, s));
      }
      build_r2<<<nblk(P), 256, 0, s>>>(P, n, 1, Fe, have_fe && c == 0, fc, Lc, out + n); RSD_LAUNCH_NOTE();
      return RSD_OK;
    };
    // z = P v (v, z of length n + P)
    auto precond = [&](const double* v, double* z) -> int {
      to32_perm<<<nblk(n), 256, 0, s>>>(P, Q, 1, v, n, 0, t32); RSD_LAUNCH_NOTE();
      if (use_uh)
        RSD_TRY(rsd_uhat_solve(ctx, &uh_m, t32, n, 1, ywork));
      else
        RSD_TRY(rsd_potrs_wide_s(ctx, (int)n, M32, n, W_m, t32, n, 1, ywork));
      from32_perm<<<nblk(n), 256, 0, s>>>(P, Q, 1, t32, z, 0); RSD_LAUNCH_NOTE();  // y = M^-1 v1
      rhs_u<<<nblk(P), 256, 0, s>>>(P, n, 1, v + n, z, u32); RSD_LAUNCH_NOTE();
      if (use_uh)
        RSD_TRY(rsd_uhat_solve(ctx, &uh_r, u32, P, 1, ywork));
      else
        RSD_TRY(rsd_potrs_wide_s(ctx, (int)P, A32, P, W_r, u32, P, 1, ywork));
      du_vec<<<nblk(n), 256, 0, s>>>(P, n, 1, u32, dv); RSD_LAUNCH_NOTE();
      to32_perm<<<nblk(n), 256, 0, s>>>(P, Q, 1, dv, n, 1, t32); RSD_LAUNCH_NOTE();
      if (use_uh)
        RSD_TRY(rsd_uhat_solve(ctx, &uh_m, t32, n, 1, ywork, (int)Q));
      else
        RSD_TRY(rsd_potrs_wide_s(ctx, (int)n, M32, n, W_m, t32, n, 1, ywork));
      from32_perm<<<nblk(n), 256, 0, s>>>(P, Q, 1, t32, z, 1); RSD_LAUNCH_NOTE();  // df
      gm_f2d<<<nblk(P), 256, 0, s>>>(P, u32, z + n); RSD_LAUNCH_NOTE();           // dU
      return RSD_OK;
    };
    // a = A z
    auto apply_a = [&](const double* z, double* a) -> int {
      gm_u0<<<nblk(n), 256, 0, s>>>(P, n, z + n, dv); RSD_LAUNCH_NOTE();  // [zU; 0]
      gm_neg<<<nblk(n), 256, 0, s>>>(n, dv, a); RSD_LAUNCH_NOTE();
      RSD_TRY(symv_add(z, a));  // M zf - [zU; 0]
      if (p->use_lub) {
        RSD_TRY(rsd_lub_spmv(ctx, &lub, 1, dv, n, Lz, n));
        gm_a2<<<nblk(P), 256, 0, s>>>(P, z, Lz, a + n); RSD_LAUNCH_NOTE();
      } else {
        RSD_CUDA(ctx, cudaMemcpyAsync(a + n, z, sizeof(double) * P, cudaMemcpyDeviceToDevice, s));
      }
      return RSD_OK;
    };
    // |b_c|: b = ([0; -EIN], Fe_c)
    std::vector<double> bnorm(nr);
    {
      norms<<<nr, 256, 0, s>>>(P, n, nr, r1, r2, ein, Fe, have_fe, nrm); RSD_LAUNCH_NOTE();  // b part only is used
      std::vector<double> hb(2 * nr);
      RSD_CUDA(ctx, cudaMemcpyAsync(hb.data(), nrm, sizeof(double) * 2 * nr, cudaMemcpyDeviceToHost, s));
      RSD_CUDA(ctx, cudaStreamSynchronize(s));
      for (int c = 0; c < nr; c++) bnorm[c] = sqrt(hb[2 * c + 1]) > 0 ? sqrt(hb[2 * c + 1]) : 1.0;
    }
    int total_it = 0;
    double worst = 0.0;
    std::vector<double> H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1), yv(m), hh(m + 2);
    for (int c = 0; c < nr; c++) {
      double rel = 0.0;
      for (int cycle = 0;; cycle++) {
        RSD_TRY(residual(c, Vb));
        gm_nrm2<<<1, 256, 0, s>>>(len, Vb, dn); RSD_LAUNCH_NOTE();
        double beta2 = 0.0;
        int herr = 0;
        RSD_CUDA(ctx, cudaMemcpyAsync(&beta2, dn, sizeof(double), cudaMemcpyDeviceToHost, s));
        RSD_CUDA(ctx, cudaMemcpyAsync(&herr, tri_err, sizeof(int), cudaMemcpyDeviceToHost, s));
        RSD_CUDA(ctx, cudaStreamSynchronize(s));
        if (herr) return rsd_fail(ctx, RSD_ETIMEOUT, "refinement: a triangular sweep's wait timed out");
        const double beta = sqrt(beta2);
        rel = beta / bnorm[c];
        if (!std::isfinite(rel)) return rsd_fail(ctx, RSD_ENAN, "refinement residual is not finite");
        if (rel <= tol || total_it >= gm_maxit) break;
        gm_scale<<<nblk(len), 256, 0, s>>>(len, Vb, dn, Vb); RSD_LAUNCH_NOTE();
        std::fill(g.begin(), g.end(), 0.0);
        g[0] = beta;
        int j = 0;
        for (; j < m && total_it < gm_maxit; j++) {
          double* vj = Vb + (size_t)j * len;
          double* zj = Zb + (size_t)j * len;
          double* vn = Vb + (size_t)(j + 1) * len;
          RSD_TRY(precond(vj, zj));
          RSD_TRY(apply_a(zj, vn));
          total_it++;
          // classical Gram-Schmidt, twice
          RSD_CUDA(ctx, cudaMemsetAsync(hacc, 0, sizeof(double) * (j + 1), s));
          for (int pass = 0; pass < 2; pass++) {
            gm_dots<<<j + 1, 256, 0, s>>>(len, j + 1, Vb, len, vn, hbuf); RSD_LAUNCH_NOTE();
            gm_orth<<<nblk(len), 256, 0, s>>>(len, j + 1, Vb, len, hbuf, vn, hacc); RSD_LAUNCH_NOTE();
          }
          gm_nrm2<<<1, 256, 0, s>>>(len, vn, dn); RSD_LAUNCH_NOTE();
          RSD_CUDA(ctx, cudaMemcpyAsync(hh.data(), hacc, sizeof(double) * (j + 1), cudaMemcpyDeviceToHost, s));
          RSD_CUDA(ctx, cudaMemcpyAsync(hh.data() + j + 1, dn, sizeof(double), cudaMemcpyDeviceToHost, s));
          RSD_CUDA(ctx, cudaStreamSynchronize(s));
          const double hn = sqrt(hh[j + 1]);
          if (hn > 0.0) {
            gm_scale<<<nblk(len), 256, 0, s>>>(len, vn, dn, vn); RSD_LAUNCH_NOTE();
          }
          // Givens rotations on column j of H
          double* Hj = H.data() + (size_t)j * (m + 1);
          for (int i = 0; i <= j; i++) Hj[i] = hh[i];
          Hj[j + 1] = hn;
          for (int i = 0; i < j; i++) {
            const double t = cs[i] * Hj[i] + sn[i] * Hj[i + 1];
            Hj[i + 1] = -sn[i] * Hj[i] + cs[i] * Hj[i + 1];
            Hj[i] = t;
          }
          const double den = std::hypot(Hj[j], Hj[j + 1]);
          cs[j] = den > 0 ? Hj[j] / den : 1.0;
          sn[j] = den > 0 ? Hj[j + 1] / den : 0.0;
          Hj[j] = den;
          Hj[j + 1] = 0.0;
          g[j + 1] = -sn[j] * g[j];
          g[j] = cs[j] * g[j];
          if (std::fabs(g[j + 1]) <= 0.5 * tol * bnorm[c] || hn == 0.0) {
            j++;
            break;
          }
        }
        // y = H^-1 g (upper triangular, j x j), x += Z y
        for (int i = j - 1; i >= 0; i--) {
          double t = g[i];
          for (int k = i + 1; k < j; k++) t -= H[(size_t)k * (m + 1) + i] * yv[k];
          yv[i] = t / H[(size_t)i * (m + 1) + i];
        }
        RSD_CUDA(ctx, cudaMemcpyAsync(hbuf, yv.data(), sizeof(double) * j, cudaMemcpyHostToDevice, s));
        // x = (f_c, U_c) is not contiguous: update the two parts
        gm_update<<<nblk(n), 256, 0, s>>>(n, j, Zb, len, hbuf, f + (size_t)c * n); RSD_LAUNCH_NOTE();
        gm_update<<<nblk(P), 256, 0, s>>>(P, j, Zb + n, len, hbuf, U + (size_t)c * P); RSD_LAUNCH_NOTE();
      }
      worst = fmax(worst, rel);
    }
    *its_out = total_it;
    *res_out = worst;
    return RSD_OK;
  };
  // A solve is accepted within the stagnation band of the tolerance.
  const double accept = 100.0 * tol;
  cudaEventRecord(ctx->ev[7], s);
  if (ctx->refine_gmres) {
    int its = 0;
    double res = 0.0;
    RSD_TRY(run_gmres(maxit, &its, &res));
    outputs<<<nblk(P), 256, 0, s>>>(P, Q, nr - 1, f, Lw, U, U_par, S_hyd); RSD_LAUNCH_NOTE();
    RSD_CUDA(ctx, cudaGetLastError());
    info->iterations = its;
    info->residual = res;
    if (!(res <= accept))
      return rsd_fail(ctx, RSD_ENOCONV, "refinement did not converge: residual %.3e after %d iterations", res, its);
    return RSD_OK;
  }
  int h_tri_err = 0;
  RSD_CUDA(ctx, cudaMemsetAsync(f, 0, sizeof(double) * nr * n, s));
  RSD_CUDA(ctx, cudaMemsetAsync(U, 0, sizeof(double) * nr * P, s));
  double worst = 0.0, best_res = INFINITY;
  int it = 0;
  std::vector<double> hn(2 * nr), hist;
  for (;; it++) {
    build_w<<<nblk(n * nr), 256, 0, s>>>(P, Q, nr, U, ein, w); RSD_LAUNCH_NOTE();
    RSD_CUDA(ctx, cudaMemcpyAsync(r1, w, sizeof(double) * nr * n, cudaMemcpyDeviceToDevice, s));
    // r1 -= M f, double-single products of the two planes
    to_dsf_vec<<<nblk(n * nr), 256, 0, s>>>(n * nr, f, fs); RSD_LAUNCH_NOTE();
    if (symv) {  // both right-hand sides in one pass over the stored half of M
      double* pcol = gpart + (size_t)nbt * nbt * SYMV_T * nr;
      if (nr == 2) {
        symv_planes_part<2><<<dim3(nbt, nbt), 256, symv_smem(2), s>>>(nn, (int)n, Mh, Ml, ld, fs, nbt, gpart, pcol); RSD_LAUNCH_NOTE();
      } else {
        symv_planes_part<1><<<dim3(nbt, nbt), 256, symv_smem(1), s>>>(nn, (int)n, Mh, Ml, ld, fs, nbt, gpart, pcol); RSD_LAUNCH_NOTE();
      }
      symv_planes_reduce<<<(unsigned)((n + 255) / 256), 256, 0, s>>>((int)n, nr, nbt, gpart, pcol, -1.0, r1, n); RSD_LAUNCH_NOTE();
    } else {
      // full product: the mirrored entries are filled in first
      if (!mirrored) {
        RSD_TRY(rsd_mirror_planes(ctx, nn, M, ld));
        mirrored = true;
      }
      if (nr == 1) {
        gemv_planes_part<1><<<dim3((unsigned)((n + 255) / 256), gchunks), 256, 0, s>>>((int)n, (int)n, Mh, Ml, ld, fs, gpart); RSD_LAUNCH_NOTE();
      } else {
        gemv_planes_part<2><<<dim3((unsigned)((n + 255) / 256), gchunks), 256, 0, s>>>((int)n, (int)n, Mh, Ml, ld, fs, gpart); RSD_LAUNCH_NOTE();
      }
      gemv_planes_reduce<<<(unsigned)((n + 255) / 256), 256, 0, s>>>((int)n, nr, gchunks, gpart, -1.0, r1, n); RSD_LAUNCH_NOTE();
    }
    if (p->use_lub) {
      RSD_TRY(rsd_lub_spmv(ctx, &lub, nr, w, n, Lw, n));
    } else {
      RSD_CUDA(ctx, cudaMemsetAsync(Lw, 0, sizeof(double) * nr * n, s));
    }
    build_r2<<<nblk(P * nr), 256, 0, s>>>(P, n, nr, Fe, have_fe, f, Lw, r2); RSD_LAUNCH_NOTE();
    norms<<<nr, 256, 0, s>>>(P, n, nr, r1, r2, ein, Fe, have_fe, nrm); RSD_LAUNCH_NOTE();
    RSD_CUDA(ctx, cudaMemcpyAsync(hn.data(), nrm, sizeof(double) * 2 * nr, cudaMemcpyDeviceToHost, s));
    RSD_CUDA(ctx, cudaMemcpyAsync(&h_tri_err, tri_err, sizeof(int), cudaMemcpyDeviceToHost, s));
    RSD_CUDA(ctx, cudaStreamSynchronize(s));
    if (h_tri_err) return rsd_fail(ctx, RSD_ETIMEOUT, "refinement: a triangular sweep's wait timed out");
    worst = 0.0;
    for (int c = 0; c < nr; c++) {
      const double rr = sqrt(hn[2 * c]) / (sqrt(hn[2 * c + 1]) > 0 ? sqrt(hn[2 * c + 1]) : 1.0);
      worst = std::isfinite(rr) ? fmax(worst, rr) : INFINITY;
    }
    if (worst <= tol || it >= maxit) break;
    // Divergence: FP32 factors too far from the FP64 system (a pair so close
    // that cond(RPP) times the factors' precision exceeds one) make the
    // stationary iteration grow; the flexible GMRES below takes over.
    if (!std::isfinite(worst) || (it >= 2 && worst > 1e3 * best_res)) break;
    best_res = fmin(best_res, worst);
    // Stagnation: the FP64 residual of a stiff system (many near-contact
    // pairs: forces ~1/gap times the velocities) has a floor of about the
    // residual arithmetic's rounding times |M||f| / |b|, which can sit just
    // above tol.  Within 100 tol, an iteration that does not halve the best
    // of the previous two ends the refinement (the solution does not improve
    // further); the reported residual is the one reached.
    hist.push_back(worst);
    if (it >= 2 && worst <= 100.0 * tol && worst > 0.5 * fmin(hist[it - 1], hist[it - 2])) break;
    // y = M^-1 r1
    to32_perm<<<nblk(n * nr), 256, 0, s>>>(P, Q, nr, r1, n, 0, t32); RSD_LAUNCH_NOTE();
    if (use_uh)
      RSD_TRY(rsd_uhat_solve(ctx, &uh_m, t32, n, nr, ywork));
    else
      RSD_TRY(rsd_potrs_wide_s(ctx, (int)n, M32, n, W_m, t32, n, nr, ywork));
    from32_perm<<<nblk(n * nr), 256, 0, s>>>(P, Q, nr, t32, y, 0); RSD_LAUNCH_NOTE();
    // dU = RPP^-1 (r2 - y_P)
    rhs_u<<<nblk(P * nr), 256, 0, s>>>(P, n, nr, r2, y, u32); RSD_LAUNCH_NOTE();
    if (use_uh)
      RSD_TRY(rsd_uhat_solve(ctx, &uh_r, u32, P, nr, ywork));
    else
      RSD_TRY(rsd_potrs_wide_s(ctx, (int)P, A32, P, W_r, u32, P, nr, ywork));
    // df = y + M^-1 [dU; 0]
    du_vec<<<nblk(n * nr), 256, 0, s>>>(P, n, nr, u32, dv); RSD_LAUNCH_NOTE();
    to32_perm<<<nblk(n * nr), 256, 0, s>>>(P, Q, nr, dv, n, 1, t32); RSD_LAUNCH_NOTE();
    if (use_uh)
      RSD_TRY(rsd_uhat_solve(ctx, &uh_m, t32, n, nr, ywork, (int)Q));
    else
      RSD_TRY(rsd_potrs_wide_s(ctx, (int)n, M32, n, W_m, t32, n, nr, ywork));
    from32_perm<<<nblk(n * nr), 256, 0, s>>>(P, Q, nr, t32, y, 1); RSD_LAUNCH_NOTE();
    update_fu<<<nblk(n * nr), 256, 0, s>>>(P, n, nr, y, u32, f, U); RSD_LAUNCH_NOTE();
  }
  if (!(worst <= accept)) {
    // diverged or stalled above the band: flexible GMRES from zero over the
    // same corrections, which converges where a few modes of the FP32
    // factors are poor
    int its = 0;
    double res = 0.0;
    RSD_TRY(run_gmres(std::max(3 * maxit, 100), &its, &res));
    it += its;
    worst = res;
    info->fallback = 1;
  }
  outputs<<<nblk(P), 256, 0, s>>>(P, Q, nr - 1, f, Lw, U, U_par, S_hyd); RSD_LAUNCH_NOTE();
  RSD_CUDA(ctx, cudaGetLastError());
  info->iterations = it;
  info->residual = worst;
  if (!(worst <= accept))
    return rsd_fail(ctx, RSD_ENOCONV, "refinement did not converge: residual %.3e after %d iterations", worst, it);
  return RSD_OK;
}
