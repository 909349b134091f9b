// Kernel 3: dense SPD factorisation and inverse for the grand resistance
// (MATREV, src/matrices.f90:4-34, which calls LAPACK DPOTRF('U') and
// DPOTRI('U') and mirrors the upper triangle).  Column-major throughout.
//
//   rsd_potrf_upper   blocked right-looking Cholesky A = U^T U: per block
//                     column one CTA factors the nb x nb diagonal block in
//                     shared memory and inverts it (W = U_jj^-1); the panel
//                     solve is W^T * panel and the trailing update a
//                     symmetric rank-nb GEMM on the upper tiles only.
//   rsd_potri_upper   A^-1 = U^-1 U^-T: blocked triangular inverse (each
//                     step two GEMMs, the first skipping the zero triangle)
//                     then the in-place product U^-1 U^-T by column blocks.
//   rsd_trsv_upper    U^T y = b and U x = y for a few right-hand sides,
//                     using the stored diagonal-block inverses.
// The GEMM is one templated SIMT kernel (FP64 here; the FP32 instance
// serves the mixed-precision path).
#include <cuda_runtime.h>

#include "rsd_internal.cuh"

namespace {

struct GemmP {
  int m, n, k;
  const void* A;
  int64_t lda;
  int ta;
  const void* B;
  int64_t ldb;
  int tb;
  void* C;
  int64_t ldc;
  double alpha, beta;
  int uplo;    // 1: skip tiles strictly below the diagonal
  int kA_row;  // op(A)(i,p) = 0 for p < i + offA: start k at row0 + offA
  int offA;
  int kB_col;  // op(B)(p,c) = 0 for p < c + offB: start k at col0 + offB
  int offB;
};

template <typename T, int BM, int BN, int BK>
__global__ void __launch_bounds__(256) gemm_kernel(GemmP g) {
  constexpr int TM = BM / 16, TN = BN / 16;
  const int row0 = blockIdx.x * BM, col0 = blockIdx.y * BN;
  if (g.uplo && row0 >= col0 + BN) return;
  int kbeg = 0;
  if (g.kA_row) kbeg = max(kbeg, row0 + g.offA);
  if (g.kB_col) kbeg = max(kbeg, col0 + g.offB);
  const int kend = g.k;
  __shared__ T As[BK][BM + 1];
  __shared__ T Bs[BK][BN + 1];
  const int t = threadIdx.x, tx = t % 16, ty = t / 16;
  const T* A = (const T*)g.A;
  const T* B = (const T*)g.B;
  T acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; i++)
#pragma unroll
    for (int j = 0; j < TN; j++) acc[i][j] = T(0);
  for (int k0 = kbeg; k0 < kend; k0 += BK) {
    // A tile: op(A)(row0+i, k0+p)
    if (!g.ta) {
      for (int e = t; e < BM * BK; e += 256) {
        const int i = e % BM, p = e / BM, gr = row0 + i, gk = k0 + p;
        As[p][i] = (gr < g.m && gk < kend) ? A[gr + (int64_t)gk * g.lda] : T(0);
      }
    } else {
      for (int e = t; e < BM * BK; e += 256) {
        const int p = e % BK, i = e / BK, gr = row0 + i, gk = k0 + p;
        As[p][i] = (gr < g.m && gk < kend) ? A[gk + (int64_t)gr * g.lda] : T(0);
      }
    }
    // B tile: op(B)(k0+p, col0+c)
    if (!g.tb) {
      for (int e = t; e < BN * BK; e += 256) {
        const int p = e % BK, c = e / BK, gc = col0 + c, gk = k0 + p;
        Bs[p][c] = (gc < g.n && gk < kend) ? B[gk + (int64_t)gc * g.ldb] : T(0);
      }
    } else {
      for (int e = t; e < BN * BK; e += 256) {
        const int c = e % BN, p = e / BN, gc = col0 + c, gk = k0 + p;
        Bs[p][c] = (gc < g.n && gk < kend) ? B[gc + (int64_t)gk * g.ldb] : T(0);
      }
    }
    __syncthreads();
#pragma unroll
    for (int p = 0; p < BK; p++) {
      T a[TM], b[TN];
#pragma unroll
      for (int i = 0; i < TM; i++) a[i] = As[p][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < TN; j++) b[j] = Bs[p][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < TM; i++)
#pragma unroll
        for (int j = 0; j < TN; j++) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
  T* C = (T*)g.C;
  const T alpha = (T)g.alpha, beta = (T)g.beta;
#pragma unroll
  for (int i = 0; i < TM; i++)
#pragma unroll
    for (int j = 0; j < TN; j++) {
      const int r = row0 + ty + 16 * i, c = col0 + tx + 16 * j;
      if (r < g.m && c < g.n) {
        T* p = C + r + (int64_t)c * g.ldc;
        *p = (g.beta == 0.0) ? alpha * acc[i][j] : alpha * acc[i][j] + beta * *p;
      }
    }
}

template <typename T, int BM, int BN, int BK>
void launch_gemm(cudaStream_t s, const GemmP& g) {
  if (g.m <= 0 || g.n <= 0) return;
  dim3 grd((g.m + BM - 1) / BM, (g.n + BN - 1) / BN);
  gemm_kernel<T, BM, BN, BK><<<grd, 256, 0, s>>>(g);
}

GemmP gp(int m, int n, int k, double alpha, const void* A, int64_t lda, int ta, const void* B, int64_t ldb, int tb,
         double beta, void* C, int64_t ldc) {
  GemmP g{};
  g.m = m;
  g.n = n;
  g.k = k;
  g.alpha = alpha;
  g.A = A;
  g.lda = lda;
  g.ta = ta;
  g.B = B;
  g.ldb = ldb;
  g.tb = tb;
  g.beta = beta;
  g.C = C;
  g.ldc = ldc;
  return g;
}

// One CTA: Cholesky (upper) of the jb x jb diagonal block in shared memory,
// then W = U^-1 (upper, zero below).  info: first failing global index + 1.
__global__ void __launch_bounds__(256) potf2_upper_inv(double* __restrict__ A, int64_t lda, int jb,
                                                       double* __restrict__ W, int ldw, int* __restrict__ info,
                                                       int j0) {
  extern __shared__ double sm[];
  double* S = sm;             // jb x jb, column-major, ld = jb
  double* col = sm + jb * jb;  // scratch column
  __shared__ int failed;
  const int t = threadIdx.x;
  for (int e = t; e < jb * jb; e += blockDim.x) {
    const int i = e % jb, j = e / jb;
    S[e] = (i <= j) ? A[i + (int64_t)j * lda] : 0.0;
  }
  if (t == 0) failed = 0;
  __syncthreads();
  for (int k = 0; k < jb; k++) {
    if (t == 0) {
      const double d = S[k + k * jb];
      if (!(d > 0.0) || !isfinite(d)) {
        failed = 1;
        if (atomicCAS(info, 0, j0 + k + 1) == 0) {
        }
      } else {
        S[k + k * jb] = sqrt(d);
      }
    }
    __syncthreads();
    if (failed) break;
    const double dk = S[k + k * jb];
    for (int j = k + 1 + t; j < jb; j += blockDim.x) S[k + j * jb] /= dk;
    __syncthreads();
    for (int j = k + 1 + t; j < jb; j += blockDim.x) {
      const double skj = S[k + j * jb];
      for (int i = k + 1; i <= j; i++) S[i + j * jb] -= S[k + i * jb] * skj;
    }
    __syncthreads();
  }
  for (int e = t; e < jb * jb; e += blockDim.x) {
    const int i = e % jb, j = e / jb;
    if (i <= j) A[i + (int64_t)j * lda] = S[e];
  }
  __syncthreads();
  if (failed) {
    for (int e = t; e < jb * jb; e += blockDim.x) W[(e % jb) + (int64_t)(e / jb) * ldw] = 0.0;
    return;
  }
  // in-place upper triangular inverse, column by column
  for (int j = 0; j < jb; j++) {
    const double wjj = 1.0 / S[j + j * jb];
    for (int i = t; i < j; i += blockDim.x) {
      double s = 0.0;
      for (int p = i; p < j; p++) s += S[i + p * jb] * S[p + j * jb];
      col[i] = -s * wjj;
    }
    __syncthreads();
    for (int i = t; i < j; i += blockDim.x) S[i + j * jb] = col[i];
    if (t == 0) S[j + j * jb] = wjj;
    __syncthreads();
  }
  for (int e = t; e < jb * jb; e += blockDim.x) {
    const int i = e % jb, j = e / jb;
    W[i + (int64_t)j * ldw] = (i <= j) ? S[e] : 0.0;
  }
}

__global__ void zero_lower_k(int n, double* __restrict__ A, int64_t lda) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n * n) return;
  const int i = (int)(t % n), j = (int)(t / n);
  if (i > j) A[i + (int64_t)j * lda] = 0.0;
}

// A(i,j) = A(j,i) for i > j, in 32x32 tiles through shared memory
__global__ void mirror_upper_k(int n, double* __restrict__ A, int64_t lda) {
  __shared__ double tile[32][33];
  const int bi = blockIdx.x, bj = blockIdx.y;  // target tile rows bi, cols bj, bi >= bj
  if (bi < bj) return;
  const int tx = threadIdx.x, ty = threadIdx.y;
  // load source tile (rows bj, cols bi) = upper part
  for (int r = ty; r < 32; r += 8) {
    const int i = bj * 32 + tx, j = bi * 32 + r;
    tile[r][tx] = (i < n && j < n) ? A[i + (int64_t)j * lda] : 0.0;
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    const int i = bi * 32 + tx, j = bj * 32 + r;  // target (i, j) = source (j, i)
    if (i < n && j < n && i > j) A[i + (int64_t)j * lda] = tile[tx][r];
  }
}

constexpr int NB64 = 128;

int potf2_smem(int jb) { return (jb * jb + jb) * (int)sizeof(double); }

}  // namespace

void rsd_gemm_f64(cudaStream_t s, int m, int n, int k, double alpha, const double* A, int64_t lda, int ta,
                  const double* B, int64_t ldb, int tb, double beta, double* C, int64_t ldc) {
  launch_gemm<double, 64, 64, 16>(s, gp(m, n, k, alpha, A, lda, ta, B, ldb, tb, beta, C, ldc));
}

int rsd_zero_lower(rsd_ctx* ctx, int n, double* d_A, int64_t lda) {
  const int64_t tot = (int64_t)n * n;
  zero_lower_k<<<(unsigned)((tot + 255) / 256), 256, 0, ctx->stream>>>(n, d_A, lda);
  RSD_CUDA(ctx, cudaGetLastError());
  return RSD_OK;
}

int rsd_mirror_upper(rsd_ctx* ctx, int n, double* d_A, int64_t lda) {
  const int nt = (n + 31) / 32;
  mirror_upper_k<<<dim3(nt, nt), dim3(32, 8), 0, ctx->stream>>>(n, d_A, lda);
  RSD_CUDA(ctx, cudaGetLastError());
  return RSD_OK;
}

static double* diag_inverses(rsd_ctx* ctx, int n, const char* tag) {
  const int nblk = (n + NB64 - 1) / NB64;
  std::string name = std::string("potrf_W_") + tag;
  return (double*)rsd_scratch(ctx, name.c_str(), sizeof(double) * (size_t)nblk * NB64 * NB64);
}

// Blocked upper Cholesky in place; the diagonal-block inverses are kept in
// the scratch buffer named by `tag` for rsd_potri_upper / rsd_trsv_upper.
int rsd_potrf_upper_tag(rsd_ctx* ctx, int n, double* d_A, int64_t lda, int* info, const char* tag) {
  if (n < 1 || lda < n) return rsd_fail(ctx, RSD_EARG, "potrf: n=%d lda=%lld", n, (long long)lda);
  cudaStream_t s = ctx->stream;
  double* W = diag_inverses(ctx, n, tag);
  double* P = (double*)rsd_scratch(ctx, "potrf_panel", sizeof(double) * (size_t)NB64 * n);
  if (!W || !P) return RSD_ENOMEM;
  static bool attr = false;
  if (!attr) {
    RSD_CUDA(ctx, cudaFuncSetAttribute(potf2_upper_inv, cudaFuncAttributeMaxDynamicSharedMemorySize, potf2_smem(NB64)));
    attr = true;
  }
  RSD_CUDA(ctx, cudaMemsetAsync(ctx->d_info, 0, sizeof(int), s));
  for (int j0 = 0, b = 0; j0 < n; j0 += NB64, b++) {
    const int jb = n - j0 < NB64 ? n - j0 : NB64;
    double* Ajj = d_A + j0 + (int64_t)j0 * lda;
    double* Wb = W + (size_t)b * NB64 * NB64;
    potf2_upper_inv<<<1, 256, potf2_smem(jb), s>>>(Ajj, lda, jb, Wb, NB64, ctx->d_info, j0);
    const int rest = n - j0 - jb;
    if (rest > 0) {
      double* Apan = d_A + j0 + (int64_t)(j0 + jb) * lda;
      // panel: W^T * A(j0:j0+jb, j0+jb:n)
      launch_gemm<double, 64, 64, 16>(s, gp(jb, rest, jb, 1.0, Wb, NB64, 1, Apan, lda, 0, 0.0, P, NB64));
      RSD_CUDA(ctx, cudaMemcpy2DAsync(Apan, lda * sizeof(double), P, NB64 * sizeof(double), jb * sizeof(double),
                                      rest, cudaMemcpyDeviceToDevice, s));
      // trailing: A22 -= P^T P (upper tiles)
      GemmP g = gp(rest, rest, jb, -1.0, P, NB64, 1, P, NB64, 0, 1.0, d_A + (j0 + jb) + (int64_t)(j0 + jb) * lda, lda);
      g.uplo = 1;
      launch_gemm<double, 64, 64, 16>(s, g);
    }
  }
  RSD_CUDA(ctx, cudaGetLastError());
  RSD_CUDA(ctx, cudaMemcpyAsync(ctx->h_info, ctx->d_info, sizeof(int), cudaMemcpyDeviceToHost, s));
  RSD_CUDA(ctx, cudaStreamSynchronize(s));
  *info = *ctx->h_info;
  return RSD_OK;
}

int rsd_potrf_upper(rsd_ctx* ctx, int n, double* d_A, int64_t lda, int* info) {
  return rsd_potrf_upper_tag(ctx, n, d_A, lda, info, "A");
}

// After rsd_potrf_upper_tag(.., tag): A <- A^-1 in the upper triangle.
int rsd_potri_upper_tag(rsd_ctx* ctx, int n, double* d_A, int64_t lda, const char* tag) {
  cudaStream_t s = ctx->stream;
  double* W = diag_inverses(ctx, n, tag);
  double* T1 = (double*)rsd_scratch(ctx, "potri_T1", sizeof(double) * (size_t)NB64 * n);
  if (!W || !T1) return RSD_ENOMEM;
  RSD_TRY(rsd_zero_lower(ctx, n, d_A, lda));
  // triangular inverse X = U^-1, left to right
  for (int j0 = 0, b = 0; j0 < n; j0 += NB64, b++) {
    const int jb = n - j0 < NB64 ? n - j0 : NB64;
    double* Wb = W + (size_t)b * NB64 * NB64;
    if (j0 > 0) {
      GemmP g = gp(j0, jb, j0, 1.0, d_A, lda, 0, d_A + (int64_t)j0 * lda, lda, 0, 0.0, T1, n);
      g.kA_row = 1;
      g.offA = 0;
      launch_gemm<double, 64, 64, 16>(s, g);
      launch_gemm<double, 64, 64, 16>(s, gp(j0, jb, jb, -1.0, T1, n, 0, Wb, NB64, 0, 0.0, d_A + (int64_t)j0 * lda, lda));
    }
    RSD_CUDA(ctx, cudaMemcpy2DAsync(d_A + j0 + (int64_t)j0 * lda, lda * sizeof(double), Wb, NB64 * sizeof(double),
                                    jb * sizeof(double), jb, cudaMemcpyDeviceToDevice, s));
  }
  // A^-1 = X X^T, column blocks left to right (in place)
  for (int i0 = 0; i0 < n; i0 += NB64) {
    const int ib = n - i0 < NB64 ? n - i0 : NB64;
    const int m = i0 + ib, k = n - i0;
    GemmP g = gp(m, ib, k, 1.0, d_A + (int64_t)i0 * lda, lda, 0, d_A + i0 + (int64_t)i0 * lda, lda, 1, 0.0, T1, n);
    g.kA_row = 1;
    g.offA = -i0;
    g.kB_col = 1;
    g.offB = 0;
    launch_gemm<double, 64, 64, 16>(s, g);
    RSD_CUDA(ctx, cudaMemcpy2DAsync(d_A + (int64_t)i0 * lda, lda * sizeof(double), T1, n * sizeof(double),
                                    m * sizeof(double), ib, cudaMemcpyDeviceToDevice, s));
  }
  RSD_CUDA(ctx, cudaGetLastError());
  return RSD_OK;
}

int rsd_potri_upper(rsd_ctx* ctx, int n, double* d_A, int64_t lda) { return rsd_potri_upper_tag(ctx, n, d_A, lda, "A"); }

// Solve A X = B with A = U^T U factored by rsd_potrf_upper_tag(.., tag);
// X (n x nrhs, leading dimension ldx) holds B on entry.
int rsd_potrs_upper_tag(rsd_ctx* ctx, int n, const double* d_U, int64_t ldu, double* d_X, int64_t ldx, int nrhs,
                        const char* tag) {
  cudaStream_t s = ctx->stream;
  double* W = diag_inverses(ctx, n, tag);
  double* T = (double*)rsd_scratch(ctx, "potrs_tmp", sizeof(double) * (size_t)NB64 * nrhs);
  if (!W || !T) return RSD_ENOMEM;
  const int nblk = (n + NB64 - 1) / NB64;
  // forward: U^T y = b
  for (int b = 0; b < nblk; b++) {
    const int j0 = b * NB64, jb = n - j0 < NB64 ? n - j0 : NB64;
    if (j0 > 0)
      launch_gemm<double, 64, 64, 16>(s, gp(jb, nrhs, j0, -1.0, d_U + (int64_t)j0 * ldu, ldu, 1, d_X, ldx, 0, 1.0,
                                            d_X + j0, ldx));
    launch_gemm<double, 64, 64, 16>(s, gp(jb, nrhs, jb, 1.0, W + (size_t)b * NB64 * NB64, NB64, 1, d_X + j0, ldx, 0,
                                          0.0, T, NB64));
    RSD_CUDA(ctx, cudaMemcpy2DAsync(d_X + j0, ldx * sizeof(double), T, NB64 * sizeof(double), jb * sizeof(double),
                                    nrhs, cudaMemcpyDeviceToDevice, s));
  }
  // backward: U x = y
  for (int b = nblk - 1; b >= 0; b--) {
    const int j0 = b * NB64, jb = n - j0 < NB64 ? n - j0 : NB64;
    const int rest = n - j0 - jb;
    if (rest > 0)
      launch_gemm<double, 64, 64, 16>(s, gp(jb, nrhs, rest, -1.0, d_U + j0 + (int64_t)(j0 + jb) * ldu, ldu, 0,
                                            d_X + j0 + jb, ldx, 0, 1.0, d_X + j0, ldx));
    launch_gemm<double, 64, 64, 16>(s, gp(jb, nrhs, jb, 1.0, W + (size_t)b * NB64 * NB64, NB64, 0, d_X + j0, ldx, 0,
                                          0.0, T, NB64));
    RSD_CUDA(ctx, cudaMemcpy2DAsync(d_X + j0, ldx * sizeof(double), T, NB64 * sizeof(double), jb * sizeof(double),
                                    nrhs, cudaMemcpyDeviceToDevice, s));
  }
  RSD_CUDA(ctx, cudaGetLastError());
  return RSD_OK;
}

int rsd_trsv_upper(rsd_ctx* ctx, int n, const double* d_U, int64_t ldu, double* d_X, int64_t ldx, int nrhs,
                   int transpose) {
  (void)transpose;
  return rsd_potrs_upper_tag(ctx, n, d_U, ldu, d_X, ldx, nrhs, "A");
}
