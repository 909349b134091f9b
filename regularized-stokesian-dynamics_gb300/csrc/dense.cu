// Kernel 3: dense SPD factorisation, inverse and solves for the grand
// resistance (MATREV, src/matrices.f90:4-34, which calls LAPACK DPOTRF('U')
// and DPOTRI('U') and mirrors the upper triangle).  Column-major throughout,
// templated on the element type: FP64 for the plain form, FP32 for the
// factorisations of the mixed form.
//
//   potrf_upper   blocked right-looking Cholesky A = U^T U: per block column
//                 one CTA factors the nb x nb diagonal block in shared memory
//                 and inverts it (W = U_jj^-1); the panel solve is W^T * panel
//                 and the trailing update a symmetric rank-nb GEMM on the
//                 upper tiles only.
//   potri_upper   A^-1 = U^-1 U^-T: blocked triangular inverse (two GEMMs per
//                 step, the first skipping the zero triangle), then the
//                 in-place product U^-1 U^-T by column blocks.
//   potrs_upper   U^T y = b, U x = y for a few right-hand sides: right-looking
//                 block substitution (diagonal blocks by their inverses, the
//                 updates as wide GEMVs).
//   gemv          y = alpha op(A) X + beta y for 1..4 columns, split over k
//                 with a fixed-order second pass (deterministic).
#include <cuda_runtime.h>

#include <string>

#include <type_traits>

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
  int batch;              // > 1: blockIdx.z = b runs the same product on A + b sA, B + b sB, C + b sC
  int64_t sA, sB, sC;     // batch strides in elements
};

// C = alpha op(A) op(B) + beta C, one BM x BN tile per CTA of 256 threads
// (each TM x TN outputs), k in steps of BK through double-buffered shared
// memory with the next tile prefetched into registers during the FMAs.
template <typename T, int BM, int BN, int BK>
__global__ void __launch_bounds__(256) gemm_kernel(GemmP g) {
  constexpr int TM = BM / 16, TN = BN / 16;
  constexpr int LA = BM * BK / 256, LB = BN * BK / 256;
  const int row0 = blockIdx.x * BM, col0 = blockIdx.y * BN;
  if (g.uplo && row0 >= col0 + BN) return;
  int kbeg = 0;
  if (g.kA_row) kbeg = max(kbeg, row0 + g.offA);
  if (g.kB_col) kbeg = max(kbeg, col0 + g.offB);
  const int kend = g.k;
  __shared__ T As[2][BK][BM + 1];
  __shared__ T Bs[2][BK][BN + 1];
  const int t = threadIdx.x, tx = t % 16, ty = t / 16;
  const T* A = (const T*)g.A + blockIdx.z * g.sA;
  const T* B = (const T*)g.B + blockIdx.z * g.sB;
  T ra[LA], rb[LB];
  auto load = [&](int k0) {
#pragma unroll
    for (int q = 0; q < LA; q++) {
      const int e = t + 256 * q;
      int i, p;
      if (!g.ta) {
        i = e % BM;
        p = e / BM;
      } else {
        p = e % BK;
        i = e / BK;
      }
      const int gr = row0 + i, gk = k0 + p;
      ra[q] = (gr < g.m && gk < kend) ? (g.ta ? A[gk + (int64_t)gr * g.lda] : A[gr + (int64_t)gk * g.lda]) : T(0);
    }
#pragma unroll
    for (int q = 0; q < LB; q++) {
      const int e = t + 256 * q;
      int c, p;
      if (!g.tb) {
        p = e % BK;
        c = e / BK;
      } else {
        c = e % BN;
        p = e / BN;
      }
      const int gc = col0 + c, gk = k0 + p;
      rb[q] = (gc < g.n && gk < kend) ? (g.tb ? B[gc + (int64_t)gk * g.ldb] : B[gk + (int64_t)gc * g.ldb]) : T(0);
    }
  };
  auto store = [&](int buf) {
#pragma unroll
    for (int q = 0; q < LA; q++) {
      const int e = t + 256 * q;
      if (!g.ta)
        As[buf][e / BM][e % BM] = ra[q];
      else
        As[buf][e % BK][e / BK] = ra[q];
    }
#pragma unroll
    for (int q = 0; q < LB; q++) {
      const int e = t + 256 * q;
      if (!g.tb)
        Bs[buf][e % BK][e / BK] = rb[q];
      else
        Bs[buf][e / BN][e % BN] = rb[q];
    }
  };
  T acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; i++)
#pragma unroll
    for (int j = 0; j < TN; j++) acc[i][j] = T(0);
  int buf = 0;
  if (kbeg < kend) {
    load(kbeg);
    store(0);
  }
  __syncthreads();
  for (int k0 = kbeg; k0 < kend; k0 += BK) {
    const bool more = k0 + BK < kend;
    if (more) load(k0 + BK);
#pragma unroll
    for (int p = 0; p < BK; p++) {
      T a[TM], b[TN];
#pragma unroll
      for (int i = 0; i < TM; i++) a[i] = As[buf][p][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < TN; j++) b[j] = Bs[buf][p][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < TM; i++)
#pragma unroll
        for (int j = 0; j < TN; j++) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    if (more) store(buf ^ 1);
    __syncthreads();
    buf ^= 1;
  }
  T* C = (T*)g.C + blockIdx.z * g.sC;
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

// FP32 GEMM with 16-byte vector accesses (aligned operands only): 128 x 128
// tile per CTA of 256 threads, each thread an 8 x 8 block made of two 4-row
// and two 4-column strips, so the shared-memory fragments and the C
// epilogue are float4 accesses; k in steps of 8, double-buffered with the
// next tile prefetched into registers.
__global__ void __launch_bounds__(256) sgemm_vec(GemmP g) {
  constexpr int BM = 128, BN = 128, BK = 8;
  const int row0 = blockIdx.x * BM, col0 = blockIdx.y * BN;
  if (g.uplo && row0 >= col0 + BN) return;
  int kbeg = 0;
  if (g.kA_row) kbeg = max(kbeg, row0 + g.offA);
  if (g.kB_col) kbeg = max(kbeg, col0 + g.offB);
  kbeg &= ~3;  // stays 16-byte aligned; the extra k columns are zeros in op(A)/op(B)
  const int kend = g.k;
  __shared__ __align__(16) float As[2][BK][BM];
  __shared__ __align__(16) float Bs[2][BK][BN];
  const int t = threadIdx.x, tx = t % 16, ty = t / 16;
  const float* A = (const float*)g.A + blockIdx.z * g.sA;
  const float* B = (const float*)g.B + blockIdx.z * g.sB;
  float4 ra, rb;
  // op(A) tile element coordinates of this thread's float4
  int ai, ap, bc, bp;
  if (!g.ta) {
    ai = (t % 32) * 4;  // 4 consecutive rows
    ap = t / 32;
  } else {
    ai = t / 2;  // one row, 4 consecutive k
    ap = (t % 2) * 4;
  }
  if (!g.tb) {
    bc = t / 2;  // one column, 4 consecutive k
    bp = (t % 2) * 4;
  } else {
    bc = (t % 32) * 4;  // 4 consecutive columns
    bp = t / 32;
  }
  auto ldA = [&](int k0) {
    float v[4];
    if (!g.ta) {
      const int gr = row0 + ai, gk = k0 + ap;
      if (gk < kend && gr + 3 < g.m) {
        ra = *reinterpret_cast<const float4*>(A + gr + (int64_t)gk * g.lda);
        return;
      }
      for (int q = 0; q < 4; q++) v[q] = (gk < kend && gr + q < g.m) ? A[gr + q + (int64_t)gk * g.lda] : 0.f;
    } else {
      const int gr = row0 + ai, gk = k0 + ap;
      if (gr < g.m && gk + 3 < kend) {
        ra = *reinterpret_cast<const float4*>(A + gk + (int64_t)gr * g.lda);
        return;
      }
      for (int q = 0; q < 4; q++) v[q] = (gr < g.m && gk + q < kend) ? A[gk + q + (int64_t)gr * g.lda] : 0.f;
    }
    ra = make_float4(v[0], v[1], v[2], v[3]);
  };
  auto ldB = [&](int k0) {
    float v[4];
    if (!g.tb) {
      const int gc = col0 + bc, gk = k0 + bp;
      if (gc < g.n && gk + 3 < kend) {
        rb = *reinterpret_cast<const float4*>(B + gk + (int64_t)gc * g.ldb);
        return;
      }
      for (int q = 0; q < 4; q++) v[q] = (gc < g.n && gk + q < kend) ? B[gk + q + (int64_t)gc * g.ldb] : 0.f;
    } else {
      const int gc = col0 + bc, gk = k0 + bp;
      if (gk < kend && gc + 3 < g.n) {
        rb = *reinterpret_cast<const float4*>(B + gc + (int64_t)gk * g.ldb);
        return;
      }
      for (int q = 0; q < 4; q++) v[q] = (gk < kend && gc + q < g.n) ? B[gc + q + (int64_t)gk * g.ldb] : 0.f;
    }
    rb = make_float4(v[0], v[1], v[2], v[3]);
  };
  auto stA = [&](int buf) {
    if (!g.ta) {
      *reinterpret_cast<float4*>(&As[buf][ap][ai]) = ra;
    } else {
      As[buf][ap + 0][ai] = ra.x;
      As[buf][ap + 1][ai] = ra.y;
      As[buf][ap + 2][ai] = ra.z;
      As[buf][ap + 3][ai] = ra.w;
    }
  };
  auto stB = [&](int buf) {
    if (!g.tb) {
      Bs[buf][bp + 0][bc] = rb.x;
      Bs[buf][bp + 1][bc] = rb.y;
      Bs[buf][bp + 2][bc] = rb.z;
      Bs[buf][bp + 3][bc] = rb.w;
    } else {
      *reinterpret_cast<float4*>(&Bs[buf][bp][bc]) = rb;
    }
  };
  float acc[8][8];
#pragma unroll
  for (int i = 0; i < 8; i++)
#pragma unroll
    for (int j = 0; j < 8; j++) acc[i][j] = 0.f;
  int buf = 0;
  if (kbeg < kend) {
    ldA(kbeg);
    ldB(kbeg);
    stA(0);
    stB(0);
  }
  __syncthreads();
  for (int k0 = kbeg; k0 < kend; k0 += BK) {
    const bool more = k0 + BK < kend;
    if (more) {
      ldA(k0 + BK);
      ldB(k0 + BK);
    }
#pragma unroll
    for (int p = 0; p < BK; p++) {
      const float4 a0 = *reinterpret_cast<const float4*>(&As[buf][p][tx * 4]);
      const float4 a1 = *reinterpret_cast<const float4*>(&As[buf][p][64 + tx * 4]);
      const float4 b0 = *reinterpret_cast<const float4*>(&Bs[buf][p][ty * 4]);
      const float4 b1 = *reinterpret_cast<const float4*>(&Bs[buf][p][64 + ty * 4]);
      const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
      const float b[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
      for (int i = 0; i < 8; i++)
#pragma unroll
        for (int j = 0; j < 8; j++) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    if (more) {
      stA(buf ^ 1);
      stB(buf ^ 1);
    }
    __syncthreads();
    buf ^= 1;
  }
  float* C = (float*)g.C + blockIdx.z * g.sC;
  const float alpha = (float)g.alpha, beta = (float)g.beta;
#pragma unroll
  for (int j = 0; j < 8; j++) {
    const int c = col0 + (j < 4 ? ty * 4 + j : 64 + ty * 4 + j - 4);
    if (c >= g.n) continue;
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int r = row0 + h * 64 + tx * 4;
      float* pc = C + r + (int64_t)c * g.ldc;
      const float* av = &acc[h * 4][j];
      if (r + 3 < g.m) {
        float4 o;
        if (g.beta == 0.0) {
          o = make_float4(alpha * av[0], alpha * av[8], alpha * av[16], alpha * av[24]);
        } else {
          const float4 old = *reinterpret_cast<const float4*>(pc);
          o = make_float4(alpha * av[0] + beta * old.x, alpha * av[8] + beta * old.y, alpha * av[16] + beta * old.z,
                          alpha * av[24] + beta * old.w);
        }
        *reinterpret_cast<float4*>(pc) = o;
      } else {
        for (int q = 0; q < 4; q++)
          if (r + q < g.m) pc[q] = (g.beta == 0.0) ? alpha * av[8 * q] : alpha * av[8 * q] + beta * pc[q];
      }
    }
  }
}

inline bool aligned16(const void* p, int64_t ld) { return ((uintptr_t)p % 16 == 0) && (ld % 4 == 0); }

template <typename T>
struct Tile;
template <>
struct Tile<double> {
  static constexpr int BM = 64, BN = 64, BK = 16;
};
template <>
struct Tile<float> {
  static constexpr int BM = 128, BN = 128, BK = 16;
};

template <typename T>
void launch_gemm(cudaStream_t s, const GemmP& g) {
  if (g.m <= 0 || g.n <= 0) return;
  const unsigned nb = g.batch > 1 ? (unsigned)g.batch : 1u;
  const bool strides16 = (g.sA % 4 == 0) && (g.sB % 4 == 0) && (g.sC % 4 == 0);
  if (sizeof(T) == 4 && strides16 && aligned16(g.A, g.lda) && aligned16(g.B, g.ldb) && aligned16(g.C, g.ldc)) {
    dim3 grd((g.m + 127) / 128, (g.n + 127) / 128, nb);
    sgemm_vec<<<grd, 256, 0, s>>>(g); RSD_LAUNCH_NOTE();
    return;
  }
  constexpr int BM = Tile<T>::BM, BN = Tile<T>::BN, BK = Tile<T>::BK;
  dim3 grd((g.m + BM - 1) / BM, (g.n + BN - 1) / BN, nb);
  gemm_kernel<T, BM, BN, BK><<<grd, 256, 0, s>>>(g); RSD_LAUNCH_NOTE();
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

constexpr int NB = 128;  // block size of the blocked factorisations

// One CTA: Cholesky (upper) of the jb x jb diagonal block in shared memory.
// The trailing update of each column step is spread over a 16 x 16 thread
// grid.  info: first failing global index + 1 (DPOTRF's INFO).
template <typename T>
__global__ void __launch_bounds__(256) potf2_upper(T* __restrict__ A, int64_t lda, int jb, int* __restrict__ info,
                                                   int j0) {
  extern __shared__ unsigned char smraw[];
  T* S = (T*)smraw;  // jb x jb, column-major, ld = jb
  T* rowk = S + jb * jb;  // scaled pivot row, read without bank conflicts
  __shared__ int failed;
  const int t = threadIdx.x, tx = t % 16, ty = t / 16;
  for (int e = t; e < jb * jb; e += blockDim.x) {
    const int i = e % jb, j = e / jb;
    S[e] = (i <= j) ? A[i + (int64_t)j * lda] : T(0);
  }
  if (t == 0) failed = 0;
  __syncthreads();
  for (int k = 0; k < jb; k++) {
    if (t == 0) {
      const T d = S[k + k * jb];
      if (!(d > T(0)) || !isfinite(d)) {
        failed = 1;
        atomicCAS(info, 0, j0 + k + 1);
      } else {
        S[k + k * jb] = sqrt(d);
      }
    }
    __syncthreads();
    if (failed) break;
    const T rk = T(1) / S[k + k * jb];
    for (int j = k + 1 + t; j < jb; j += blockDim.x) {
      const T v = S[k + j * jb] * rk;
      S[k + j * jb] = v;
      rowk[j] = v;
    }
    __syncthreads();
    for (int j = k + 1 + ty; j < jb; j += 16) {
      const T skj = rowk[j];
      for (int i = k + 1 + tx; i <= j; i += 16) S[i + j * jb] -= rowk[i] * skj;
    }
    __syncthreads();
  }
  for (int e = t; e < jb * jb; e += blockDim.x) {
    const int i = e % jb, j = e / jb;
    if (i <= j) A[i + (int64_t)j * lda] = S[e];
  }
}

// FP32 diagonal block (jb <= 128): upper Cholesky factor U and its inverse
// W = U^-1 in one CTA of 8 warps.  Right-looking over 32-wide sub-blocks D:
//   - warp 0 factors D in registers (lane = column) and inverts the factor
//     by back substitution, also in registers; D^-1 is the sub-block's
//     diagonal block of W, kept row- and column-major for the steps below;
//   - the row panel R next to D becomes D^-T R: lane = row, column `lane` of
//     D^-1 in registers, each column of R read as 16-byte broadcasts;
//   - the trailing block loses R^T R: lane = row i, column i of R in
//     registers, each other column read as 16-byte broadcasts (from the
//     transposed copy RT that the panel step writes).
// W's off-diagonal blocks come one column block at a time,
// W(0:c, c) = -W(0:c, 0:c) (U(0:c, c) D_c^-1): warps 1-7 form column block
// c while warp 0 factors sub-block c + 1, and all warps form the last one.
// Every shared load is a 16-byte broadcast or a walk with lanes on distinct
// banks (columns PV = 132 floats apart, so 16-byte column reads of 8 lanes
// fall on distinct bank groups).  U goes back to A; W goes to Wout (NB x NB,
// lower part and rows/columns past jb zero).  info as DPOTRF.
constexpr int PV = NB + 4;      // ld of U and W (16-byte aligned columns)
constexpr int DV = 36;          // ld of the D^-1 copies and of RT
constexpr int TV = 3 * 32 + 4;  // ld of T = U(0:c, c) D_c^-1, c <= 3
// Loads of an FP32 tile into shared memory with many loads in flight: a
// loop of one load per iteration serialises the DRAM round trips of a
// single CTA (~0.7 us each), so each thread first issues a batch of 16
// (16-byte vectors where the column starts are 16-byte aligned), then
// writes them.  Tile: rows x cols of a column-major matrix (ld lda) into
// S(i, j) = S[i + j * lds]; with upper = 1 only i <= j is kept (the rest 0).
// Entries outside rows x cols up to NB x cmax are written as 0.
__device__ __forceinline__ void load_tile_f32(const float* __restrict__ A, int64_t lda, int rows, int cols, int cmax,
                                              float* __restrict__ S, int lds, int upper) {
  const int t = threadIdx.x, nt = blockDim.x;
  const bool vec = ((lda & 3) == 0) && (((uintptr_t)A & 15) == 0) && ((rows & 3) == 0);
  if (vec) {
    const int per_col = NB / 4, total = per_col * cmax;
    for (int f0 = 0; f0 < total; f0 += 16 * nt) {
      float4 v[16];
#pragma unroll
      for (int q = 0; q < 16; q++) {
        const int f = f0 + t + q * nt, j = f / per_col, i = (f % per_col) * 4;
        v[q] = (f < total && j < cols && i < rows) ? *reinterpret_cast<const float4*>(A + i + (int64_t)j * lda)
                                                   : make_float4(0.f, 0.f, 0.f, 0.f);
      }
#pragma unroll
      for (int q = 0; q < 16; q++) {
        const int f = f0 + t + q * nt, j = f / per_col, i = (f % per_col) * 4;
        if (f < total) {
          S[i + j * lds] = (!upper || i <= j) ? v[q].x : 0.f;
          S[i + 1 + j * lds] = (!upper || i + 1 <= j) ? v[q].y : 0.f;
          S[i + 2 + j * lds] = (!upper || i + 2 <= j) ? v[q].z : 0.f;
          S[i + 3 + j * lds] = (!upper || i + 3 <= j) ? v[q].w : 0.f;
        }
      }
    }
  } else {
    const int total = NB * cmax;
    for (int e0 = 0; e0 < total; e0 += 16 * nt) {
      float v[16];
#pragma unroll
      for (int q = 0; q < 16; q++) {
        const int e = e0 + t + q * nt, i = e % NB, j = e / NB;
        v[q] = (e < total && i < rows && j < cols && (!upper || i <= j)) ? A[i + (int64_t)j * lda] : 0.f;
      }
#pragma unroll
      for (int q = 0; q < 16; q++) {
        const int e = e0 + t + q * nt;
        if (e < total) S[(e % NB) + (e / NB) * lds] = v[q];
      }
    }
  }
}

// Step K of the 32 x 32 register factor of diag32_factor_inv (lane =
// column), then steps K+1..31.  Template recursion keeps every index of r
// and dinv a compile-time constant, so both stay in registers.
template <int K>
__device__ __forceinline__ void chol32_step(float (&r)[32], float (&dinv)[32], int lane, int& bad) {
  if constexpr (K < 32) {
    const float pv = __shfl_sync(0xffffffffu, r[K], K);
    bad = (bad == 0 && !(pv > 0.f && pv <= 3.402823466e38f)) ? K + 1 : bad;
    const float inv = rsqrtf(pv);  // every lane forms the pivot's 1/sqrt itself
    dinv[K] = inv;
    r[K] = lane >= K ? r[K] * inv : r[K];
#pragma unroll
    for (int i = K + 1; i < 32; i++) {
      const float u = __shfl_sync(0xffffffffu, r[K], i);
      r[i] = lane >= i ? fmaf(-u, r[K], r[i]) : r[i];
    }
    chol32_step<K + 1>(r, dinv, lane, bad);
  }
}

// A full 32 x 32 diagonal sub-block (warp-wide, no branches): the factor in
// registers (written to S), then D^-1 column `lane` by back substitution in
// axpy form, U's columns read from shared memory as 16-byte broadcasts.
// D^-1 goes to Wm, to Dn (row-major) and to Dt (column-major), ld DV.
// Returns the 1-based index of the first pivot that is not positive and
// finite, 0 if none (the same for every lane).
__device__ __forceinline__ int diag32_factor_inv(float* S, float* Wm, float* Dn, float* Dt, int k0, int lane) {
  float r[32], dinv[32];
  float4* sc = reinterpret_cast<float4*>(S + k0 + (k0 + lane) * PV);
#pragma unroll
  for (int g = 0; g < 8; g++) {
    const float4 v = sc[g];
    r[4 * g] = v.x;
    r[4 * g + 1] = v.y;
    r[4 * g + 2] = v.z;
    r[4 * g + 3] = v.w;
  }
  int bad = 0;
  chol32_step<0>(r, dinv, lane, bad);
  if (bad) return bad;
  // entries below the diagonal stay as loaded (zero)
#pragma unroll
  for (int g = 0; g < 8; g++) sc[g] = make_float4(r[4 * g], r[4 * g + 1], r[4 * g + 2], r[4 * g + 3]);
  __syncwarp();
  float x[32], acc[32];
#pragma unroll
  for (int i = 0; i < 32; i++) acc[i] = 0.f;
#pragma unroll
  for (int q = 0; q < 32; q++) {
    const int p = 31 - q;
    const float v = ((p == lane ? 1.f : 0.f) - acc[p]) * dinv[p];
    x[p] = p <= lane ? v : 0.f;
    // acc(i) += U(i, p) x(p); the terms added to acc(i >= p) are never read
    const float4* up = reinterpret_cast<const float4*>(S + k0 + (k0 + p) * PV);
#pragma unroll
    for (int g = 0; g < (p + 3) / 4; g++) {
      const float4 u = up[g];
      acc[4 * g] = fmaf(u.x, x[p], acc[4 * g]);
      acc[4 * g + 1] = fmaf(u.y, x[p], acc[4 * g + 1]);
      acc[4 * g + 2] = fmaf(u.z, x[p], acc[4 * g + 2]);
      acc[4 * g + 3] = fmaf(u.w, x[p], acc[4 * g + 3]);
    }
  }
  float4* wc = reinterpret_cast<float4*>(Wm + k0 + (k0 + lane) * PV);
  float4* dt = reinterpret_cast<float4*>(Dt + lane * DV);
#pragma unroll
  for (int g = 0; g < 8; g++) {
    const float4 v = make_float4(x[4 * g], x[4 * g + 1], x[4 * g + 2], x[4 * g + 3]);
    wc[g] = v;
    dt[g] = v;
  }
#pragma unroll
  for (int i = 0; i < 32; i++) Dn[i * DV + lane] = x[i];
  return 0;
}

// The trailing sub-block of kw < 32 columns (zero-padded to 32), as
// diag32_factor_inv with IEEE square roots and divisions.
__device__ __forceinline__ int diag_partial_factor_inv(float* S, float* Wm, float* Dn, float* Dt, int k0, int kw,
                                                       int lane) {
  float r[32];
#pragma unroll
  for (int i = 0; i < 32; i++) r[i] = S[(k0 + i) + (k0 + lane) * PV];
  int bad = 0;
#pragma unroll
  for (int k = 0; k < 32; k++) {
    if (k < kw && !bad) {
      const float piv = __shfl_sync(0xffffffffu, r[k], k);
      if (!(piv > 0.f) || !isfinite(piv)) {
        bad = k + 1;
      } else {
        const float d = sqrtf(piv);
        if (lane > k) r[k] = r[k] / d;
        else if (lane == k) r[k] = d;
#pragma unroll
        for (int i = k + 1; i < 32; i++) {
          const float uki = __shfl_sync(0xffffffffu, r[k], i);
          if (lane >= i) r[i] -= uki * r[k];
        }
      }
    }
  }
  if (bad) return bad;
  // column `lane` of D^-1: back substitution against the rows of U_D, whose
  // entry (ii, p) lane p holds in r[ii]
  float x[32];
#pragma unroll
  for (int ii = 31; ii >= 0; ii--) {
    float v = (ii == lane) ? 1.f : 0.f;
#pragma unroll
    for (int p = ii + 1; p < 32; p++) v -= __shfl_sync(0xffffffffu, r[ii], p) * x[p];
    const float dii = __shfl_sync(0xffffffffu, r[ii], ii);
    x[ii] = (ii < kw && lane < kw && ii <= lane) ? v / dii : 0.f;
  }
  if (lane < kw) {
#pragma unroll
    for (int i = 0; i < 32; i++) {
      if (i <= lane) S[(k0 + i) + (k0 + lane) * PV] = r[i];
      Wm[(k0 + i) + (k0 + lane) * PV] = x[i];
    }
  }
#pragma unroll
  for (int i = 0; i < 32; i++) {
    Dn[i * DV + lane] = x[i];
    Dt[lane * DV + i] = x[i];
  }
  return 0;
}

// 32-term dot product of a register column with a 16-byte aligned shared
// column read as broadcasts, in four partial sums.
__device__ __forceinline__ float dot32_bcast(const float (&a)[32], const float* __restrict__ col) {
  const float4* c4 = reinterpret_cast<const float4*>(col);
  float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
#pragma unroll
  for (int g = 0; g < 8; g++) {
    const float4 v = c4[g];
    s0 = fmaf(a[4 * g], v.x, s0);
    s1 = fmaf(a[4 * g + 1], v.y, s1);
    s2 = fmaf(a[4 * g + 2], v.z, s2);
    s3 = fmaf(a[4 * g + 3], v.w, s3);
  }
  return (s0 + s1) + (s2 + s3);
}

// Column block c >= 1 of W = U^-1 (rows 0..32c-1) by warps tw = 0..nw-1 of
// a team: T = U(0:c, c) D_c^-1 into Tt, then W(0:c, c) = -W(0:c, 0:c) T
// (W upper triangular).  Tasks are (32-row block, 8 columns), lane = row;
// `sync` (a barrier of the team) separates the two products.
template <typename Sync>
__device__ __forceinline__ void w_column_block(const float* __restrict__ S, float* __restrict__ Wm,
                                               const float* __restrict__ Dt, float* __restrict__ Tt, int c, int tw,
                                               int nw, int lane, Sync sync) {
  const int ntask = 4 * c;
  for (int task = tw; task < ntask; task += nw) {
    const int rb = task >> 2, j0 = (task & 3) * 8, p = 32 * rb + lane;
    float u[32];
#pragma unroll
    for (int q = 0; q < 32; q++) u[q] = S[p + (32 * c + q) * PV];
#pragma unroll 4  // a full unroll hoists all 64 broadcasts and spills
    for (int jj = 0; jj < 8; jj++) Tt[(j0 + jj) * TV + p] = dot32_bcast(u, Dt + (j0 + jj) * DV);
  }
  sync();
  for (int task = tw; task < ntask; task += nw) {
    const int rb = task >> 2, j0 = (task & 3) * 8, p = 32 * rb + lane;
    float acc[8];
#pragma unroll
    for (int jj = 0; jj < 8; jj++) acc[jj] = 0.f;
    for (int pb = rb; pb < c; pb++) {
      float w[32];
#pragma unroll
      for (int q = 0; q < 32; q++) w[q] = Wm[p + (32 * pb + q) * PV];
#pragma unroll
      for (int jj = 0; jj < 8; jj++) acc[jj] += dot32_bcast(w, Tt + (j0 + jj) * TV + 32 * pb);
    }
#pragma unroll
    for (int jj = 0; jj < 8; jj++) Wm[p + (32 * c + j0 + jj) * PV] = -acc[jj];
  }
}

constexpr int SMEM_POTF2_INV = (2 * NB * PV + NB * DV + 4 * 32 * DV + 32 * TV) * (int)sizeof(float);
__global__ void __launch_bounds__(256) potf2_inv_f32(float* __restrict__ A, int64_t lda, int jb,
                                                     int* __restrict__ info, int j0, float* __restrict__ Wout) {
  extern __shared__ __align__(16) unsigned char smraw[];
  float* S = (float*)smraw;      // U, NB x NB, ld PV
  float* Wm = S + NB * PV;       // W, NB x NB, ld PV
  float* RT = Wm + NB * PV;      // R = D^-T (row panel) transposed: column c of R at RT[c * DV]
  float* Dd = RT + NB * DV;      // two buffers of D^-1: row-major (Dn), then column-major (Dt), ld DV
  float* Tt = Dd + 4 * 32 * DV;  // T = U(0:c, c) D_c^-1: column j at Tt[j * TV]
  __shared__ int failed;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  load_tile_f32(A, lda, jb, jb, NB, S, PV, 1);
  {
    float4* w4 = reinterpret_cast<float4*>(Wm);
    for (int e = t; e < NB * PV / 4; e += 256) w4[e] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  if (t == 0) failed = 0;
  __syncthreads();
  const int nsub = (jb + 31) / 32;
  for (int kb = 0; kb < nsub; kb++) {
    const int k0 = kb * 32, kw = min(32, jb - k0);
    float* Dn = Dd + (kb & 1) * 2 * 32 * DV;
    float* Dt = Dn + 32 * DV;
    if (warp == 0) {
      const int bad = kw == 32 ? diag32_factor_inv(S, Wm, Dn, Dt, k0, lane)
                               : diag_partial_factor_inv(S, Wm, Dn, Dt, k0, kw, lane);
      if (bad && lane == 0) {
        failed = 1;
        atomicCAS(info, 0, j0 + k0 + bad);
      }
    } else if (kb >= 2) {
      // column block kb - 1 of W, beside the factor of sub-block kb
      w_column_block(S, Wm, Dd + ((kb - 1) & 1) * 2 * 32 * DV + 32 * DV, Tt, kb - 1, warp - 1, 7, lane,
                     [] { asm volatile("bar.sync 1, 224;" ::: "memory"); });
    }
    __syncthreads();
    if (failed) return;
    const int m0 = k0 + kw, mw = jb - m0;
    if (mw <= 0) continue;
    // row panel: R <- D^-T R, lane = row, four columns per warp
    {
      float dl[32];
#pragma unroll
      for (int q = 0; q < 32; q++) dl[q] = Dn[q * DV + lane];  // D^-1(q, lane)
      for (int c0 = 4 * warp; c0 < mw; c0 += 32) {
        float v[4];
#pragma unroll
        for (int cc = 0; cc < 4; cc++) v[cc] = dot32_bcast(dl, S + k0 + (m0 + min(c0 + cc, mw - 1)) * PV);
        __syncwarp();
#pragma unroll
        for (int cc = 0; cc < 4; cc++)
          if (c0 + cc < mw) {
            if (lane < kw) S[(k0 + lane) + (m0 + c0 + cc) * PV] = v[cc];
            RT[(c0 + cc) * DV + lane] = lane < kw ? v[cc] : 0.f;
          }
      }
    }
    __syncthreads();
    // trailing update of the upper part: lane = row i of a 32-row block,
    // column i of R in registers, 8 columns per task (columns >= the block)
    {
      const int nrb = (mw + 31) / 32;
      int ntask = 0;
      for (int rb = 0; rb < nrb; rb++) ntask += (mw - 32 * rb + 7) / 8;
      for (int task = warp; task < ntask; task += 8) {
        int rb = 0, rem = task;
        while (rem >= (mw - 32 * rb + 7) / 8) {
          rem -= (mw - 32 * rb + 7) / 8;
          rb++;
        }
        const int c0 = 32 * rb + 8 * rem, i = 32 * rb + lane;
        float a[32];
        const float4* ri = reinterpret_cast<const float4*>(RT + i * DV);
#pragma unroll
        for (int g = 0; g < 8; g++) {
          const float4 v = ri[g];
          a[4 * g] = v.x;
          a[4 * g + 1] = v.y;
          a[4 * g + 2] = v.z;
          a[4 * g + 3] = v.w;
        }
        float o[8];
#pragma unroll
        for (int jj = 0; jj < 8; jj++) o[jj] = dot32_bcast(a, RT + min(c0 + jj, mw - 1) * DV);
#pragma unroll
        for (int jj = 0; jj < 8; jj++) {
          const int c = c0 + jj;
          if (c < mw && i <= c) S[(m0 + i) + (m0 + c) * PV] -= o[jj];
        }
      }
    }
    __syncthreads();
  }
  if (nsub >= 2) {
    w_column_block(S, Wm, Dd + ((nsub - 1) & 1) * 2 * 32 * DV + 32 * DV, Tt, nsub - 1, warp, 8, lane,
                   [] { __syncthreads(); });
    __syncthreads();
  }
  const bool avec = ((lda & 3) == 0) && (((uintptr_t)A & 15) == 0);
  for (int e = t; e < NB * NB / 4; e += 256) {
    const int j = e / (NB / 4), i = (e % (NB / 4)) * 4;
    const float4 w = *reinterpret_cast<const float4*>(Wm + i + j * PV);
    const float4 u = *reinterpret_cast<const float4*>(S + i + j * PV);
    const bool cj = j < jb;
    const float wv[4] = {w.x, w.y, w.z, w.w}, uv[4] = {u.x, u.y, u.z, u.w};
    float wo[4];
#pragma unroll
    for (int q = 0; q < 4; q++) wo[q] = (cj && i + q <= j && i + q < jb) ? wv[q] : 0.f;
    *reinterpret_cast<float4*>(Wout + i + j * NB) = make_float4(wo[0], wo[1], wo[2], wo[3]);
    if (!cj) continue;
    if (avec && i + 3 <= j && i + 3 < jb) {
      *reinterpret_cast<float4*>(A + i + (int64_t)j * lda) = u;
    } else {
#pragma unroll
      for (int q = 0; q < 4; q++)
        if (i + q <= j && i + q < jb) A[i + q + (int64_t)j * lda] = uv[q];
    }
  }
}

// Panel solve U_jj^T X = B in place (B = A(j0:j0+jb, j0+jb:n)): the factor
// block and 64 columns of B in shared memory, one thread per column
// (forward substitution), coalesced loads and stores of the columns.
constexpr int TRSM_COLS = 64;
template <typename T>
__global__ void __launch_bounds__(TRSM_COLS) trsm_panel(const T* __restrict__ Ujj, int64_t lda, int jb, int rest,
                                                        T* __restrict__ B) {
  extern __shared__ unsigned char smraw[];
  T* S = (T*)smraw;        // jb x jb
  T* Xs = S + jb * jb;     // row i, column c at Xs[i * TRSM_COLS + c]
  const int t = threadIdx.x, c0 = blockIdx.x * TRSM_COLS;
  for (int e = t; e < jb * jb; e += TRSM_COLS) {
    const int i = e % jb, j = e / jb;
    S[e] = (i <= j) ? Ujj[i + (int64_t)j * lda] : T(0);
  }
  for (int e = t; e < jb * TRSM_COLS; e += TRSM_COLS) {
    const int i = e % jb, c = e / jb;
    Xs[i * TRSM_COLS + c] = (c0 + c < rest) ? B[i + (int64_t)(c0 + c) * lda] : T(0);
  }
  __syncthreads();
  for (int i = 0; i < jb; i++) {
    T s = Xs[i * TRSM_COLS + t];
    for (int p = 0; p < i; p++) s -= S[p + i * jb] * Xs[p * TRSM_COLS + t];
    Xs[i * TRSM_COLS + t] = s / S[i + i * jb];
  }
  __syncthreads();
  for (int e = t; e < jb * TRSM_COLS; e += TRSM_COLS) {
    const int i = e % jb, c = e / jb;
    if (c0 + c < rest) B[i + (int64_t)(c0 + c) * lda] = Xs[i * TRSM_COLS + c];
  }
}

// Inverses of all diagonal blocks of an upper triangular U (one CTA each).
template <typename T>
__global__ void __launch_bounds__(256) trtri_diag(int n, const T* __restrict__ U, int64_t ldu, T* __restrict__ W) {
  extern __shared__ unsigned char smraw[];
  T* S = (T*)smraw;
  T* col = S + NB * NB;
  const int b = blockIdx.x, j0 = b * NB, jb = min(NB, n - j0), t = threadIdx.x;
  const T* Ub = U + j0 + (int64_t)j0 * ldu;
  for (int e = t; e < jb * jb; e += blockDim.x) {
    const int i = e % jb, j = e / jb;
    S[e] = (i <= j) ? Ub[i + (int64_t)j * ldu] : T(0);
  }
  __syncthreads();
  for (int j = 0; j < jb; j++) {
    const T wjj = T(1) / S[j + j * jb];
    for (int i = t; i < j; i += blockDim.x) {
      T s = T(0);
      for (int p = i; p < j; p++) s += S[i + p * jb] * S[p + j * jb];
      col[i] = -s * wjj;
    }
    __syncthreads();
    for (int i = t; i < j; i += blockDim.x) S[i + j * jb] = col[i];
    if (t == 0) S[j + j * jb] = wjj;
    __syncthreads();
  }
  T* Wb = W + (size_t)b * NB * NB;
  for (int e = t; e < NB * NB; e += blockDim.x) {
    const int i = e % NB, j = e / NB;
    Wb[e] = (i < jb && j < jb && i <= j) ? S[i + j * jb] : T(0);
  }
}

template <typename T>
__global__ void zero_lower_k(int n, T* __restrict__ A, int64_t lda) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n * n) return;
  const int i = (int)(t % n), j = (int)(t / n);
  if (i > j) A[i + (int64_t)j * lda] = T(0);
}

template <typename T>
__global__ void mirror_upper_k(int n, T* __restrict__ A, int64_t lda) {
  __shared__ T tile[32][33];
  const int bi = blockIdx.x, bj = blockIdx.y;
  if (bi < bj) return;
  const int tx = threadIdx.x, ty = threadIdx.y;
  for (int r = ty; r < 32; r += 8) {
    const int i = bj * 32 + tx, j = bi * 32 + r;
    tile[r][tx] = (i < n && j < n) ? A[i + (int64_t)j * lda] : T(0);
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    const int i = bi * 32 + tx, j = bj * 32 + r;
    if (i < n && j < n && i > j) A[i + (int64_t)j * lda] = tile[tx][r];
  }
}

// y(m x r) = alpha A(m x k) X(k x r) + beta y, A column-major, split over k
// into gridDim.y chunks; partials[chunk][col][row]
template <typename T, int R>
__global__ void gemv_n_part(int m, int k, const T* __restrict__ A, int64_t lda, const T* __restrict__ X, int64_t ldx,
                            int kchunk, T* __restrict__ part) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  const int p0 = c * kchunk, p1 = min(k, p0 + kchunk);
  if (i >= m) return;
  T acc[R];
#pragma unroll
  for (int r = 0; r < R; r++) acc[r] = T(0);
  for (int p = p0; p < p1; p++) {
    const T a = A[i + (int64_t)p * lda];
#pragma unroll
    for (int r = 0; r < R; r++) acc[r] = fma(a, X[p + (int64_t)r * ldx], acc[r]);
  }
#pragma unroll
  for (int r = 0; r < R; r++) part[((size_t)c * R + r) * m + i] = acc[r];
}

template <typename T, int R>
__global__ void gemv_reduce(int m, int nchunk, const T* __restrict__ part, T alpha, T beta, T* __restrict__ y,
                            int64_t ldy) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
#pragma unroll
  for (int r = 0; r < R; r++) {
    T s = T(0);
    for (int c = 0; c < nchunk; c++) s += part[((size_t)c * R + r) * m + i];
    T* py = y + i + (int64_t)r * ldy;
    *py = (beta == T(0)) ? alpha * s : alpha * s + beta * *py;
  }
}

// y(m x r) = alpha A^T X + beta y with A (k x m) column-major: one warp per
// output row (a column of A), lanes stride over k, shuffle reduction
template <typename T, int R>
__global__ void gemv_t_k(int m, int k, const T* __restrict__ A, int64_t lda, const T* __restrict__ X, int64_t ldx,
                         T alpha, T beta, T* __restrict__ y, int64_t ldy) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= m) return;
  const T* a = A + (int64_t)w * lda;
  T acc[R];
#pragma unroll
  for (int r = 0; r < R; r++) acc[r] = T(0);
  for (int p = lane; p < k; p += 32) {
    const T av = a[p];
#pragma unroll
    for (int r = 0; r < R; r++) acc[r] = fma(av, X[p + (int64_t)r * ldx], acc[r]);
  }
#pragma unroll
  for (int r = 0; r < R; r++) {
    T v = acc[r];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) {
      T* py = y + w + (int64_t)r * ldy;
      *py = (beta == T(0)) ? alpha * v : alpha * v + beta * *py;
    }
  }
}

// x_j <- W_jj x_j (trans = 0) or W_jj^T x_j (trans = 1) in place, one CTA;
// the block W_jj is staged in shared memory first
template <typename T>
__global__ void __launch_bounds__(256) trsv_diag(int jb, const T* __restrict__ W, int ldw, int trans,
                                                 T* __restrict__ X, int64_t ldx, int nrhs) {
  extern __shared__ unsigned char smraw[];
  T* Ws = (T*)smraw;           // jb x jb
  T* b = Ws + NB * NB;         // jb x nrhs
  const int t = threadIdx.x;
  for (int e = t; e < jb * jb; e += blockDim.x) Ws[e] = W[(e % jb) + (int64_t)(e / jb) * ldw];
  for (int e = t; e < jb * nrhs; e += blockDim.x) b[e] = X[(e % jb) + (int64_t)(e / jb) * ldx];
  __syncthreads();
  for (int e = t; e < jb * nrhs; e += blockDim.x) {
    const int i = e % jb, r = e / jb;
    T s = T(0);
    if (!trans)
      for (int p = i; p < jb; p++) s += Ws[i + p * jb] * b[p + r * jb];
    else
      for (int p = 0; p <= i; p++) s += Ws[p + i * jb] * b[p + r * jb];
    X[i + (int64_t)r * ldx] = s;
  }
}

template <typename T>
int smem_potf2(int jb) {
  return (jb * jb + jb) * (int)sizeof(T);
}
template <typename T>
int smem_trsm() {
  return (NB * NB + NB * TRSM_COLS) * (int)sizeof(T);
}
template <typename T>
int smem_trsv() {
  return (NB * NB + NB * 4) * (int)sizeof(T);
}

template <typename T>
const char* tname();
template <>
const char* tname<double>() {
  return "d";
}
template <>
const char* tname<float>() {
  return "s";
}

template <typename T>
T* diag_inverses(rsd_ctx* ctx, int n, const char* tag) {
  const int nblk = (n + NB - 1) / NB;
  std::string name = std::string("potrf_W_") + tname<T>() + tag;
  return (T*)rsd_scratch(ctx, name.c_str(), sizeof(T) * (size_t)nblk * NB * NB);
}

template <typename T>
int ensure_attrs(rsd_ctx* ctx) {
  static bool done = false;
  if (done) return RSD_OK;
  RSD_CUDA(ctx, cudaFuncSetAttribute(potf2_upper<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_potf2<T>(NB)));
  RSD_CUDA(ctx, cudaFuncSetAttribute(trsm_panel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_trsm<T>()));
  RSD_CUDA(ctx, cudaFuncSetAttribute(trsv_diag<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_trsv<T>()));
  RSD_CUDA(ctx, cudaFuncSetAttribute(trtri_diag<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_potf2<T>(NB)));
  RSD_CUDA(ctx, cudaFuncSetAttribute(potf2_inv_f32, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_POTF2_INV));
  done = true;
  return RSD_OK;
}

}  // namespace

// ------------------------------------------------------------ templates
template <typename T>
void rsd_gemm(cudaStream_t s, int m, int n, int k, double alpha, const T* A, int64_t lda, int ta, const T* B,
              int64_t ldb, int tb, double beta, T* C, int64_t ldc) {
  launch_gemm<T>(s, gp(m, n, k, alpha, A, lda, ta, B, ldb, tb, beta, C, ldc));
}

template <typename T>
int rsd_gemv(rsd_ctx* ctx, int trans, int m, int k, T alpha, const T* A, int64_t lda, const T* X, int64_t ldx,
             int nrhs, T beta, T* y, int64_t ldy) {
  if (m <= 0) return RSD_OK;
  if (nrhs < 1 || nrhs > 4) return rsd_fail(ctx, RSD_EARG, "gemv: nrhs %d", nrhs);
  cudaStream_t s = ctx->stream;
  if (trans) {
    const int warps = 8;
#define GT(R) gemv_t_k<T, R><<<(m + warps - 1) / warps, 32 * warps, 0, s>>>(m, k, A, lda, X, ldx, alpha, beta, y, ldy)
    switch (nrhs) {
      case 1: GT(1); break;
      case 2: GT(2); break;
      case 3: GT(3); break;
      default: GT(4); break;
    }
#undef GT
    RSD_LAUNCH_NOTE();
  } else {
    // enough chunks of k to fill the GPU when m is small
    const int rowblocks = (m + 255) / 256;
    int nchunk = (4 * ctx->sm_count + rowblocks - 1) / rowblocks;
    nchunk = max(1, min(nchunk, (k + 63) / 64));
    const int kchunk = (k + nchunk - 1) / nchunk;
    nchunk = (k + kchunk - 1) / kchunk;
    if (nchunk < 1) nchunk = 1;
    T* part = (T*)rsd_scratch(ctx, trans ? "gemv_part_t" : (sizeof(T) == 8 ? "gemv_part_d" : "gemv_part_s"),
                              sizeof(T) * (size_t)nchunk * nrhs * m);
    if (!part) return RSD_ENOMEM;
#define GN(R)                                                                                      \
  gemv_n_part<T, R><<<dim3(rowblocks, nchunk), 256, 0, s>>>(m, k, A, lda, X, ldx, kchunk, part); \
  gemv_reduce<T, R><<<rowblocks, 256, 0, s>>>(m, nchunk, part, alpha, beta, y, ldy)
    switch (nrhs) {
      case 1: GN(1); break;
      case 2: GN(2); break;
      case 3: GN(3); break;
      default: GN(4); break;
    }
#undef GN
    RSD_LAUNCH_NOTE();
    RSD_LAUNCH_NOTE();
  }
  RSD_CUDA(ctx, cudaGetLastError());
  return RSD_OK;
}

template <typename T>
int rsd_zero_lower_t(rsd_ctx* ctx, int n, T* d_A, int64_t lda) {
  const int64_t tot = (int64_t)n * n;
  zero_lower_k<T><<<(unsigned)((tot + 255) / 256), 256, 0, ctx->stream>>>(n, d_A, lda); RSD_LAUNCH_NOTE();
  RSD_CUDA(ctx, cudaGetLastError());
  return RSD_OK;
}

template <typename T>
int rsd_mirror_upper_t(rsd_ctx* ctx, int n, T* d_A, int64_t lda) {
  const int nt = (n + 31) / 32;
  mirror_upper_k<T><<<dim3(nt, nt), dim3(32, 8), 0, ctx->stream>>>(n, d_A, lda); RSD_LAUNCH_NOTE();
  RSD_CUDA(ctx, cudaGetLastError());
  return RSD_OK;
}

// C (m x nc, ld ldc) -= P(:, 0:m)^T P(:, 0:nc) for a kb-row panel P (ld ldp);
// uplo: only the tiles on and above the diagonal.  Tensor cores (prec tc)
// where the layout allows, else the SIMT GEMM.
template <typename T>
int trailing_update(rsd_ctx* ctx, int tc, const T* P, int64_t ldp, int kb, int m, int nc, T* C, int64_t ldc,
                    int uplo) {
  if constexpr (std::is_same<T, float>::value) {
    if (tc && ctx->use_tc && rsd_tc_syrk_ok(P, ldp, C, ldc, kb))
      return rsd_tc_gemm(ctx, tc, m, nc, kb, -1.0f, P, ldp, P, ldp, C, ldc, 1, uplo, 0, ctx->d_info + 1);
  }
  GemmP g = gp(m, nc, kb, -1.0, P, ldp, 1, P, ldp, 0, 1.0, C, ldc);
  g.uplo = uplo;
  launch_gemm<T>(ctx->stream, g);
  return RSD_OK;
}

// Two-level FP32 Cholesky on tensor cores: outer panels of NBO = 512 rows
// are factored in NB = 128 steps (diagonal block, row panel by
// substitution, and an update of the outer panel's remaining rows only),
// then the trailing matrix takes one K = 512 update per outer panel, so it
// is read and written a quarter as often as with 128-wide steps.
//
// Schedule 0: the inner steps run in order on the side stream; the next
// outer panel starts once the first 512 rows of the trailing update have
// landed (one outer step of look-ahead).
//
// Schedule 1 (default): the chain of diagonal blocks carries only what the
// next diagonal block needs.  On stream a (side): the factor and inverse of
// block k, then block k+1's column tile of row panel k and the update of the
// diagonal tile (k+1, k+1); block k+1's factor can start at once.  On stream
// b (side2), beside that factor: the rest of row panel k and of the
// in-panel update.  Between outer panels likewise: a updates the next
// diagonal tile with the K = 512 product, the main stream the rest of the
// next outer panel's rows and then the remainder of the trailing matrix.
// Events: A (a's near work done), B (the work the next near step reads),
// M (the previous remainder, which the next diagonal tile reads).
constexpr int NBO = 512;
static int potrf_two_level_sched0(rsd_ctx* ctx, int n, float* d_A, int64_t lda, int tc, float* W) {
  cudaStream_t s = ctx->stream, s2 = ctx->side;
  RSD_CUDA(ctx, cudaEventRecord(ctx->ev_next, s));
  for (int J0 = 0; J0 < n; J0 += NBO) {
    const int JB = n - J0 < NBO ? n - J0 : NBO;
    RSD_CUDA(ctx, cudaStreamWaitEvent(s2, ctx->ev_next, 0));
    for (int j0 = J0; j0 < J0 + JB; j0 += NB) {
      const int jb = J0 + JB - j0 < NB ? J0 + JB - j0 : NB;
      float* Ajj = d_A + j0 + (int64_t)j0 * lda;
      const int rest = n - j0 - jb;
      float* Apan = d_A + j0 + (int64_t)(j0 + jb) * lda;
      float* Wb = W + (size_t)(j0 / NB) * NB * NB;
      potf2_inv_f32<<<1, 256, SMEM_POTF2_INV, s2>>>(Ajj, lda, jb, ctx->d_info, j0, Wb); RSD_LAUNCH_NOTE();
      if (rest <= 0) continue;
      // row panel U_jj^-T B = W_jj^T B in place on tensor cores (each output
      // tile reads only its own columns of B)
      RSD_TRY(rsd_tc_gemm(ctx, tc, jb, rest, jb, 1.0f, Wb, NB, Apan, lda, Apan, lda, 0, 0, 0, ctx->d_info + 1, s2));
      const int m_in = J0 + JB - (j0 + jb);  // rows of this outer panel still to update
      if (m_in > 0)
        RSD_TRY(rsd_tc_gemm(ctx, tc, m_in, rest, jb, -1.0f, Apan, lda, Apan, lda, Apan + jb, lda, 1, 1, 0,
                            ctx->d_info + 1, s2));
    }
    RSD_CUDA(ctx, cudaEventRecord(ctx->ev_panel, s2));
    RSD_CUDA(ctx, cudaStreamWaitEvent(s, ctx->ev_panel, 0));
    const int restO = n - J0 - JB;
    if (restO > 0) {
      const float* PO = d_A + J0 + (int64_t)(J0 + JB) * lda;
      float* C = d_A + (J0 + JB) + (int64_t)(J0 + JB) * lda;
      const int m1 = restO < NBO ? restO : NBO;
      RSD_TRY(rsd_tc_gemm(ctx, tc, m1, restO, JB, -1.0f, PO, lda, PO, lda, C, lda, 1, 1, 0, ctx->d_info + 1, s));
      RSD_CUDA(ctx, cudaEventRecord(ctx->ev_next, s));
      if (restO > NBO)
        RSD_TRY(rsd_tc_gemm(ctx, tc, restO - NBO, restO - NBO, JB, -1.0f, PO + (int64_t)NBO * lda, lda,
                            PO + (int64_t)NBO * lda, lda, C + NBO + (int64_t)NBO * lda, lda, 1, 1, 0,
                            ctx->d_info + 1, s));
    }
  }
  return RSD_OK;
}

static int potrf_two_level_sched1(rsd_ctx* ctx, int n, float* d_A, int64_t lda, int tc, float* W) {
  cudaStream_t s = ctx->stream, sa = ctx->side, sb = ctx->side2;
  cudaEvent_t evA = ctx->ev_la[0], evB = ctx->ev_la[1], evM = ctx->ev_la[2], evS = ctx->ev_la[3];
  int* err = ctx->d_info + 1;
  // the matrix is ready on the main stream; B and M start out satisfied
  RSD_CUDA(ctx, cudaEventRecord(evS, s));
  RSD_CUDA(ctx, cudaStreamWaitEvent(sa, evS, 0));
  RSD_CUDA(ctx, cudaStreamWaitEvent(sb, evS, 0));
  RSD_CUDA(ctx, cudaEventRecord(evB, s));
  RSD_CUDA(ctx, cudaEventRecord(evM, s));
  for (int J0 = 0; J0 < n; J0 += NBO) {
    const int JB = n - J0 < NBO ? n - J0 : NBO;
    for (int j0 = J0; j0 < J0 + JB; j0 += NB) {
      const int jb = J0 + JB - j0 < NB ? J0 + JB - j0 : NB;
      float* Ajj = d_A + j0 + (int64_t)j0 * lda;
      const int rest = n - j0 - jb;
      float* Apan = d_A + j0 + (int64_t)(j0 + jb) * lda;
      float* Wb = W + (size_t)(j0 / NB) * NB * NB;
      potf2_inv_f32<<<1, 256, SMEM_POTF2_INV, sa>>>(Ajj, lda, jb, ctx->d_info, j0, Wb); RSD_LAUNCH_NOTE();
      if (rest <= 0) continue;
      RSD_CUDA(ctx, cudaStreamWaitEvent(sa, evB, 0));
      const int m_in = J0 + JB - (j0 + jb);  // rows of this outer panel below block k
      if (m_in <= 0) {
        // last block of the outer panel: its whole row panel on the chain
        RSD_TRY(rsd_tc_gemm(ctx, tc, jb, rest, jb, 1.0f, Wb, NB, Apan, lda, Apan, lda, 0, 0, 0, err, sa));
        continue;
      }
      const int jn = m_in < NB ? m_in : NB;  // width of block k+1
      // near: row panel k on block k+1's columns, then the diagonal tile (k+1, k+1)
      RSD_TRY(rsd_tc_gemm(ctx, tc, jb, jn, jb, 1.0f, Wb, NB, Apan, lda, Apan, lda, 0, 0, 0, err, sa));
      RSD_TRY(rsd_tc_gemm(ctx, tc, jn, jn, jb, -1.0f, Apan, lda, Apan, lda, Apan + jb, lda, 1, 1, 0, err, sa));
      RSD_CUDA(ctx, cudaEventRecord(evA, sa));
      // far, beside block k+1's factor
      RSD_CUDA(ctx, cudaStreamWaitEvent(sb, evA, 0));
      if (rest > jn) {
        float* Afar = Apan + (int64_t)jn * lda;
        RSD_TRY(rsd_tc_gemm(ctx, tc, jb, rest - jn, jb, 1.0f, Wb, NB, Afar, lda, Afar, lda, 0, 0, 0, err, sb));
        RSD_TRY(rsd_tc_gemm(ctx, tc, jn, rest - jn, jb, -1.0f, Apan, lda, Afar, lda, Afar + jb, lda, 1, 0, 0, err, sb));
        if (m_in > jn)
          RSD_TRY(rsd_tc_gemm(ctx, tc, m_in - jn, rest - jn, jb, -1.0f, Afar, lda, Afar, lda, Afar + jb + jn, lda, 1,
                              1, 0, err, sb));
      }
      RSD_CUDA(ctx, cudaEventRecord(evB, sb));
    }
    const int restO = n - J0 - JB;
    if (restO <= 0) continue;
    const float* PO = d_A + J0 + (int64_t)(J0 + JB) * lda;
    float* C = d_A + (J0 + JB) + (int64_t)(J0 + JB) * lda;
    const int jn = restO < NB ? restO : NB;
    const int m1 = restO < NBO ? restO : NBO;
    // near: the next diagonal tile, after the previous remainder reached it
    RSD_CUDA(ctx, cudaStreamWaitEvent(sa, evM, 0));
    RSD_TRY(rsd_tc_gemm(ctx, tc, jn, jn, JB, -1.0f, PO, lda, PO, lda, C, lda, 1, 1, 0, err, sa));
    RSD_CUDA(ctx, cudaEventRecord(evA, sa));
    // the rest of the next outer panel's rows, then the remainder
    RSD_CUDA(ctx, cudaStreamWaitEvent(s, evA, 0));
    if (restO > jn) {
      const float* POf = PO + (int64_t)jn * lda;
      float* Cf = C + (int64_t)jn * lda;
      RSD_TRY(rsd_tc_gemm(ctx, tc, jn, restO - jn, JB, -1.0f, PO, lda, POf, lda, Cf, lda, 1, 0, 0, err, s));
      if (m1 > jn)
        RSD_TRY(rsd_tc_gemm(ctx, tc, m1 - jn, restO - jn, JB, -1.0f, POf, lda, POf, lda, Cf + jn, lda, 1, 1, 0, err,
                            s));
    }
    RSD_CUDA(ctx, cudaEventRecord(evB, s));
    if (restO > NBO)
      RSD_TRY(rsd_tc_gemm(ctx, tc, restO - NBO, restO - NBO, JB, -1.0f, PO + (int64_t)NBO * lda, lda,
                          PO + (int64_t)NBO * lda, lda, C + NBO + (int64_t)NBO * lda, lda, 1, 1, 0, err, s));
    RSD_CUDA(ctx, cudaEventRecord(evM, s));
  }
  // join both side streams into the main stream
  RSD_CUDA(ctx, cudaEventRecord(evA, sa));
  RSD_CUDA(ctx, cudaStreamWaitEvent(s, evA, 0));
  RSD_CUDA(ctx, cudaEventRecord(evB, sb));
  RSD_CUDA(ctx, cudaStreamWaitEvent(s, evB, 0));
  return RSD_OK;
}

int potrf_two_level_f32(rsd_ctx* ctx, int n, float* d_A, int64_t lda, int tc, float* W) {
  return ctx->factor_schedule == 0 ? potrf_two_level_sched0(ctx, n, d_A, lda, tc, W)
                                   : potrf_two_level_sched1(ctx, n, d_A, lda, tc, W);
}

// Blocked right-looking upper Cholesky with one step of look-ahead: the
// diagonal block and row panel of step j+1 are factored on a second,
// higher-priority stream as soon as the first tile row of step j's trailing
// update has landed, while the rest of that update runs on the main stream.
template <typename T>
int rsd_potrf_upper_t(rsd_ctx* ctx, int n, T* d_A, int64_t lda, int* info, const char* tag, int tc) {
  if (n < 1 || lda < n) return rsd_fail(ctx, RSD_EARG, "potrf: n=%d lda=%lld", n, (long long)lda);
  RSD_TRY(ensure_attrs<T>(ctx));
  RSD_TRY(rsd_side_stream(ctx));
  cudaStream_t s = ctx->stream, s2 = ctx->side;
  T* W = diag_inverses<T>(ctx, n, tag);
  if (!W) return RSD_ENOMEM;
  constexpr bool F32 = std::is_same<T, float>::value;
  T* T1 = nullptr;
  if (F32) {
    T1 = (T*)rsd_scratch(ctx, "potrf_panel_s", sizeof(T) * (size_t)NB * n);
    if (!T1) return RSD_ENOMEM;
  }
  RSD_CUDA(ctx, cudaMemsetAsync(ctx->d_info, 0, 2 * sizeof(int), s));
  bool two_level = false;
  if constexpr (F32) two_level = tc && ctx->use_tc && rsd_tc_syrk_ok(d_A, lda, d_A, lda, NB);
  if constexpr (F32) {
    if (two_level) RSD_TRY(potrf_two_level_f32(ctx, n, d_A, lda, tc, W));
  }
  if (!two_level) {
    RSD_CUDA(ctx, cudaEventRecord(ctx->ev_next, s));
    for (int j0 = 0, b = 0; j0 < n; j0 += NB, b++) {
      const int jb = n - j0 < NB ? n - j0 : NB;
      T* Ajj = d_A + j0 + (int64_t)j0 * lda;
      const int rest = n - j0 - jb;
      T* Apan = d_A + j0 + (int64_t)(j0 + jb) * lda;
      // panel j on the side stream, after the first tile row of step j-1's update
      RSD_CUDA(ctx, cudaStreamWaitEvent(s2, ctx->ev_next, 0));
      if constexpr (F32) {
        // factor + inverse of the diagonal block, then the panel as W_jj^T B
        T* Wb = W + (size_t)b * NB * NB;
        potf2_inv_f32<<<1, 256, SMEM_POTF2_INV, s2>>>(Ajj, lda, jb, ctx->d_info, j0, Wb); RSD_LAUNCH_NOTE();
        if (rest > 0) {
          launch_gemm<T>(s2, gp(jb, rest, jb, 1.0, Wb, NB, 1, Apan, lda, 0, 0.0, T1, NB));
          RSD_CUDA(ctx, cudaMemcpy2DAsync(Apan, lda * sizeof(T), T1, NB * sizeof(T), jb * sizeof(T), rest,
                                          cudaMemcpyDeviceToDevice, s2));
        }
      } else {
        potf2_upper<T><<<1, 256, smem_potf2<T>(jb), s2>>>(Ajj, lda, jb, ctx->d_info, j0); RSD_LAUNCH_NOTE();
        if (rest > 0) {
          trsm_panel<T><<<(rest + TRSM_COLS - 1) / TRSM_COLS, TRSM_COLS, smem_trsm<T>(), s2>>>(Ajj, lda, jb, rest, Apan); RSD_LAUNCH_NOTE();
        }
      }
      RSD_CUDA(ctx, cudaEventRecord(ctx->ev_panel, s2));
      RSD_CUDA(ctx, cudaStreamWaitEvent(s, ctx->ev_panel, 0));
      if (rest > 0) {
        // trailing A22 -= Apan^T Apan: first tile row (the next panel's input), then the rest
        T* A22 = d_A + (j0 + jb) + (int64_t)(j0 + jb) * lda;
        const int m1 = rest < NB ? rest : NB;
        RSD_TRY(trailing_update<T>(ctx, tc, Apan, lda, jb, m1, rest, A22, lda, 0));
        RSD_CUDA(ctx, cudaEventRecord(ctx->ev_next, s));
        if (rest > NB)
          RSD_TRY(trailing_update<T>(ctx, tc, Apan + (int64_t)NB * lda, lda, jb, rest - NB, rest - NB,
                                     A22 + NB + (int64_t)NB * lda, lda, 1));
      }
    }
  }
  // diagonal-block inverses for the solves; the FP32 paths made them with
  // their diagonal blocks, the FP64 one takes them here
  if (!F32) {
    const int nblk = (n + NB - 1) / NB;
    trtri_diag<T><<<nblk, 256, smem_potf2<T>(NB), s>>>(n, d_A, lda, W); RSD_LAUNCH_NOTE();
  }
  RSD_CUDA(ctx, cudaGetLastError());
  RSD_CUDA(ctx, cudaMemcpyAsync(ctx->h_info, ctx->d_info, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
  RSD_CUDA(ctx, cudaStreamSynchronize(s));
  *info = ctx->h_info[0];
  if (ctx->h_info[1]) return rsd_fail(ctx, RSD_ETIMEOUT, "potrf: tensor-core update timed out (code %d)", ctx->h_info[1]);
  return RSD_OK;
}

// the diagonal-block inverses that the FP32 potrf with this tag left
const float* rsd_potrf_inverses_s(rsd_ctx* ctx, int n, const char* tag) { return diag_inverses<float>(ctx, n, tag); }

// inverses of the diagonal blocks of an upper factor U (n x n, ld ldu)
template <typename T>
int rsd_diag_inverses_t(rsd_ctx* ctx, int n, const T* U, int64_t ldu, const char* tag, T** Wout) {
  RSD_TRY(ensure_attrs<T>(ctx));
  T* W = diag_inverses<T>(ctx, n, tag);
  if (!W) return RSD_ENOMEM;
  const int nblk = (n + NB - 1) / NB;
  trtri_diag<T><<<nblk, 256, smem_potf2<T>(NB), ctx->stream>>>(n, U, ldu, W); RSD_LAUNCH_NOTE();
  RSD_CUDA(ctx, cudaGetLastError());
  *Wout = W;
  return RSD_OK;
}

// In-place inverse of an upper triangular matrix A (n x n, lower part zero):
// blocked, left to right; W holds the inverses of A's NB diagonal blocks.
template <typename T>
int trtri_inplace_t(rsd_ctx* ctx, int n, T* d_A, int64_t lda, const T* W, T* T1, int64_t ldt) {
  cudaStream_t s = ctx->stream;
  for (int j0 = 0, b = 0; j0 < n; j0 += NB, b++) {
    const int jb = n - j0 < NB ? n - j0 : NB;
    const T* Wb = W + (size_t)b * NB * NB;
    if (j0 > 0) {
      GemmP g = gp(j0, jb, j0, 1.0, d_A, lda, 0, d_A + (int64_t)j0 * lda, lda, 0, 0.0, T1, ldt);
      g.kA_row = 1;
      g.offA = 0;
      launch_gemm<T>(s, g);
      launch_gemm<T>(s, gp(j0, jb, jb, -1.0, T1, ldt, 0, Wb, NB, 0, 0.0, d_A + (int64_t)j0 * lda, lda));
    }
    RSD_CUDA(ctx, cudaMemcpy2DAsync(d_A + j0 + (int64_t)j0 * lda, lda * sizeof(T), Wb, NB * sizeof(T),
                                    jb * sizeof(T), jb, cudaMemcpyDeviceToDevice, s));
  }
  return RSD_OK;
}

// WT(j0:j0+jb, j0:j0+jb) = W_jj^T for the diagonal blocks
__global__ void put_diag_transposed(int jb, const float* __restrict__ Wb, float* __restrict__ WT, int64_t ldw) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= jb * jb) return;
  const int i = t % jb, j = t / jb;  // WT(i, j) = W(j, i)
  WT[i + (int64_t)j * ldw] = Wb[j + (int64_t)i * NB];
}

// A <- A^-1 (upper triangle) from its upper factor U in A, on tensor cores:
// WT = (U^-1)^T is built one block row at a time (K-major operands
// throughout: T1^T = U(0:j0, jblk)^T WT(0:j0, 0:j0) over k >= m, then
// WT(jblk, 0:j0) = -W_jj^T T1^T), and A^-1 = W W^T = WT^T WT over k >= the
// tile's column.  prec 1 (TF32) or 3 (3xTF32).
constexpr int POTRI_KSPLIT = 1024;
int potri_tc_s(rsd_ctx* ctx, int prec, int n, float* d_A, int64_t lda, const char* tag) {
  cudaStream_t s = ctx->stream;
  float* W = nullptr;
  RSD_TRY(rsd_diag_inverses_t<float>(ctx, n, d_A, lda, tag, &W));
  const int64_t ldw = (n + 3) / 4 * 4;
  float* WT = (float*)rsd_scratch(ctx, "potri_WT_s", sizeof(float) * (size_t)ldw * n);
  float* T1 = (float*)rsd_scratch(ctx, "potri_T1t_s", sizeof(float) * (size_t)NB * n);
  if (!WT || !T1) return RSD_ENOMEM;
  RSD_CUDA(ctx, cudaMemsetAsync(ctx->d_info + 1, 0, sizeof(int), s));
  RSD_CUDA(ctx, cudaMemsetAsync(WT, 0, sizeof(float) * (size_t)ldw * n, s));
  int* err = ctx->d_info + 1;
  for (int j0 = 0, b = 0; j0 < n; j0 += NB, b++) {
    const int jb = n - j0 < NB ? n - j0 : NB;
    const float* Wb = W + (size_t)b * NB * NB;
    put_diag_transposed<<<(jb * jb + 255) / 256, 256, 0, s>>>(jb, Wb, WT + j0 + (int64_t)j0 * ldw, ldw); RSD_LAUNCH_NOTE();
    if (j0 == 0) continue;
    // long K ranges are split across CTAs (their partial products added
    // into the zeroed T1), so that a step does not wait on its longest tile
    if (j0 > POTRI_KSPLIT) {
      RSD_CUDA(ctx, cudaMemsetAsync(T1, 0, sizeof(float) * (size_t)NB * j0, s));
      RSD_TRY(rsd_tc_gemm(ctx, prec, jb, j0, j0, 1.0f, d_A + (int64_t)j0 * lda, lda, WT, ldw, T1, NB, 1, 0, 1, err, s,
                          POTRI_KSPLIT));
    } else {
      RSD_TRY(rsd_tc_gemm(ctx, prec, jb, j0, j0, 1.0f, d_A + (int64_t)j0 * lda, lda, WT, ldw, T1, NB, 0, 0, 1, err));
    }
    RSD_TRY(rsd_tc_gemm(ctx, prec, jb, j0, jb, -1.0f, Wb, NB, T1, NB, WT + j0, ldw, 0, 0, 0, err));
  }
  RSD_TRY(rsd_tc_gemm(ctx, prec, n, n, n, 1.0f, WT, ldw, WT, ldw, d_A, lda, 0, 1, 1, err));
  RSD_CUDA(ctx, cudaMemcpyAsync(ctx->h_info + 1, err, sizeof(int), cudaMemcpyDeviceToHost, s));
  RSD_CUDA(ctx, cudaStreamSynchronize(s));
  if (ctx->h_info[1]) return rsd_fail(ctx, RSD_ETIMEOUT, "potri: tensor-core GEMM timed out (code %d)", ctx->h_info[1]);
  return RSD_OK;
}

// A <- A^-1 (upper triangle) from its upper Cholesky factor in A
template <typename T>
int rsd_potri_upper_t(rsd_ctx* ctx, int n, T* d_A, int64_t lda, const char* tag, int tc) {
  if constexpr (std::is_same<T, float>::value) {
    if (tc && ctx->use_tc && rsd_tc_gemm_ok(d_A, lda, d_A, lda, d_A, lda)) return potri_tc_s(ctx, tc, n, d_A, lda, tag);
  }
  cudaStream_t s = ctx->stream;
  T* W = nullptr;
  RSD_TRY(rsd_diag_inverses_t<T>(ctx, n, d_A, lda, tag, &W));
  T* T1 = (T*)rsd_scratch(ctx, sizeof(T) == 8 ? "potri_T1_d" : "potri_T1_s", sizeof(T) * (size_t)NB * n);
  if (!T1) return RSD_ENOMEM;
  RSD_TRY(rsd_zero_lower_t<T>(ctx, n, d_A, lda));
  RSD_TRY(trtri_inplace_t<T>(ctx, n, d_A, lda, W, T1, n));
  for (int i0 = 0; i0 < n; i0 += NB) {
    const int ib = n - i0 < NB ? n - i0 : NB;
    const int m = i0 + ib, k = n - i0;
    GemmP g = gp(m, ib, k, 1.0, d_A + (int64_t)i0 * lda, lda, 0, d_A + i0 + (int64_t)i0 * lda, lda, 1, 0.0, T1, n);
    g.kA_row = 1;
    g.offA = -i0;
    g.kB_col = 1;
    g.offB = 0;
    launch_gemm<T>(s, g);
    RSD_CUDA(ctx, cudaMemcpy2DAsync(d_A + (int64_t)i0 * lda, lda * sizeof(T), T1, n * sizeof(T), m * sizeof(T), ib,
                                    cudaMemcpyDeviceToDevice, s));
  }
  RSD_CUDA(ctx, cudaGetLastError());
  return RSD_OK;
}

// Inverses of the NB2 x NB2 diagonal blocks of an upper factor U, for the
// wide-block solves: each block copied out (lower part zero) and inverted in
// place by the blocked triangular inverse.  W2: nblk2 blocks of NB2 x NB2.
constexpr int NB2 = 512;
__global__ void copy_upper_block(int jb, const float* __restrict__ U, int64_t ldu, float* __restrict__ D) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= NB2 * NB2) return;
  const int i = t % NB2, j = t / NB2;
  D[t] = (i < jb && j < jb && i <= j) ? U[i + (int64_t)j * ldu] : (i == j ? 1.0f : 0.0f);
}

// The full NB2 diagonal blocks of U (blockIdx.z = block) into D (one
// NB2 x NB2 block each, lower part zero).
__global__ void copy_upper_blocks(const float* __restrict__ U, int64_t ldu, float* __restrict__ D) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.z;
  if (t >= NB2 * NB2) return;
  const int i = t % NB2, j = t / NB2;
  const int64_t o = (int64_t)b * NB2;
  D[(size_t)b * NB2 * NB2 + t] = i <= j ? U[(o + i) + (o + j) * ldu] : 0.0f;
}

// D_b(j0:j0+NB, j0:j0+NB) = W_{b NB2/NB + j0/NB} for every block b = blockIdx.z
__global__ void put_diag_blocks(int j0, const float* __restrict__ W, float* __restrict__ D) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.z;
  if (t >= NB * NB) return;
  const int i = t % NB, j = t / NB;
  D[(size_t)b * NB2 * NB2 + (j0 + i) + (int64_t)(j0 + j) * NB2] = W[((size_t)b * (NB2 / NB) + j0 / NB) * NB * NB + t];
}

// In-place inverses of nblk upper triangular NB2 x NB2 blocks D_b (ld NB2,
// stride NB2^2) from their NB diagonal-block inverses: trtri_inplace_t on
// all blocks at once, one batched GEMM pair per NB column block.
int trtri_wide_batched_s(rsd_ctx* ctx, int nblk, float* D, const float* W, float* T1) {
  cudaStream_t s = ctx->stream;
  for (int j0 = 0; j0 < NB2; j0 += NB) {
    if (j0 > 0) {
      GemmP g = gp(j0, NB, j0, 1.0, D, NB2, 0, D + (int64_t)j0 * NB2, NB2, 0, 0.0, T1, NB2);
      g.kA_row = 1;
      g.offA = 0;
      g.batch = nblk;
      g.sA = g.sB = (int64_t)NB2 * NB2;
      g.sC = (int64_t)NB2 * NB;
      launch_gemm<float>(s, g);
      GemmP g2 = gp(j0, NB, NB, -1.0, T1, NB2, 0, W + (size_t)(j0 / NB) * NB * NB, NB, 0, 0.0,
                    D + (int64_t)j0 * NB2, NB2);
      g2.batch = nblk;
      g2.sA = (int64_t)NB2 * NB;
      g2.sB = (int64_t)(NB2 / NB) * NB * NB;
      g2.sC = (int64_t)NB2 * NB2;
      launch_gemm<float>(s, g2);
    }
    put_diag_blocks<<<dim3(NB * NB / 256, 1, nblk), 256, 0, s>>>(j0, W, D); RSD_LAUNCH_NOTE();
  }
  return RSD_OK;
}

// W128 (optional): the NB x NB diagonal-block inverses that the FP32 potrf
// of U left (NB-block b at W128 + b NB^2); the full NB2 blocks then start
// from them (all blocks in one batched pass) instead of inverting their NB
// blocks again.
int rsd_wide_inverses_s(rsd_ctx* ctx, int n, const float* U, int64_t ldu, const char* tag, const float* W128,
                        float** W2out) {
  const int nblk2 = (n + NB2 - 1) / NB2;
  std::string name = std::string("wide_W_") + tag;
  float* W2 = (float*)rsd_scratch(ctx, name.c_str(), sizeof(float) * (size_t)nblk2 * NB2 * NB2);
  float* Wt = (float*)rsd_scratch(ctx, "wide_Wsmall", sizeof(float) * (size_t)(NB2 / NB) * NB * NB);
  float* T1 = (float*)rsd_scratch(ctx, "wide_T1", sizeof(float) * (size_t)NB * NB2);
  if (!W2 || !Wt || !T1) return RSD_ENOMEM;
  RSD_TRY(ensure_attrs<float>(ctx));
  int b0 = 0;
  if (W128 && n >= NB2) {
    const int full = n / NB2;
    float* Tb = (float*)rsd_scratch(ctx, "wide_T1b", sizeof(float) * (size_t)full * NB * NB2);
    if (!Tb) return RSD_ENOMEM;
    copy_upper_blocks<<<dim3(NB2 * NB2 / 256, 1, full), 256, 0, ctx->stream>>>(U, ldu, W2); RSD_LAUNCH_NOTE();
    RSD_TRY(trtri_wide_batched_s(ctx, full, W2, W128, Tb));
    b0 = full;
  }
  for (int b = b0; b < nblk2; b++) {
    const int j0 = b * NB2, jb = n - j0 < NB2 ? n - j0 : NB2;
    float* D = W2 + (size_t)b * NB2 * NB2;
    copy_upper_block<<<(NB2 * NB2 + 255) / 256, 256, 0, ctx->stream>>>(jb, U + j0 + (int64_t)j0 * ldu, ldu, D); RSD_LAUNCH_NOTE();
    const float* Wb = Wt;
    if (W128 && jb == NB2) {
      Wb = W128 + (size_t)(j0 / NB) * NB * NB;
    } else {
      trtri_diag<float><<<NB2 / NB, 256, smem_potf2<float>(NB), ctx->stream>>>(NB2, D, NB2, Wt); RSD_LAUNCH_NOTE();
    }
    RSD_TRY(trtri_inplace_t<float>(ctx, NB2, D, NB2, Wb, T1, NB2));
  }
  RSD_CUDA(ctx, cudaGetLastError());
  *W2out = W2;
  return RSD_OK;
}

// (U^T U) X = B with the NB2 block inverses: per block two wide GEMVs
// (diagonal block by its inverse, then the update of the remaining rows).
// X holds B on entry; Y is a work vector of the same shape.
// ------------------------------------------- block-scaled factor solves
// U = D Uh with D = blockdiag(U_bb) over NB2 blocks, so Uh_bb = I and
// Uh_bc = W_b U_bc (W_b = U_bb^-1).  Then U^T U x = r is solved as
//   forward   z_b = r_b - sum_{c<b} Uh_cb^T z_c        (unit diagonal blocks)
//   middle    w_b = G_b z_b,  G_b = W_b W_b^T = (U_bb^T U_bb)^-1
//   backward  x_b = w_b - sum_{c>b} Uh_bc x_c
// Each direction is one dataflow launch over all blocks (tri_forward,
// tri_backward), the middle one block-diagonal product (blockdiag_gemv).
// Uh and G are formed once per factor on tensor cores (3xTF32).
namespace {

__global__ void transpose_block(int nb2, const float* __restrict__ W, float* __restrict__ WT) {
  __shared__ float t[32][33];
  const int b = blockIdx.z;
  const float* Wb = W + (size_t)b * nb2 * nb2;
  float* Tb = WT + (size_t)b * nb2 * nb2;
  const int i0 = blockIdx.x * 32, j0 = blockIdx.y * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) t[k][threadIdx.x] = Wb[(i0 + threadIdx.x) + (size_t)(j0 + k) * nb2];
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) Tb[(j0 + threadIdx.x) + (size_t)(i0 + k) * nb2] = t[threadIdx.x][k];
}

// ------------------------------------------- dataflow block sweeps
// One persistent launch per direction of the block-scaled solve instead of
// one launch per 512-block.  A task is one 32-wide part (of TRI_Q) of a
// target block: its CTA walks the source blocks in order,
// waits until each source block is published, and accumulates that tile's
// product in registers, so every sum has a fixed order (deterministic) and
// nothing is reduced across CTAs.  Tasks are taken from a ticket counter in
// target order (block 1, 2, ... forward; nb-2, ..., 0 backward), so every
// task a CTA waits for was taken earlier by a running CTA (no deadlock).  A
// finished part is published by data, fence and a per-block counter; a
// block is usable once all TRI_Q of its parts are in.  Waits are bounded
// (the context's poll limit, TRI_SPIN_LIMIT by default); a timeout sets *err
// and every CTA leaves its loop.
constexpr int TRI_Q = 16, TRI_QS = NB2 / TRI_Q;  // parts per block, columns/rows per part
constexpr int TRI_THREADS = 256;
constexpr long long TRI_SPIN_LIMIT = 1LL << 21;  // polls of >= 64 ns: a fraction of a second
constexpr int TRI_MAX_BLOCKS = 256;              // order up to 131072

struct TriArgs {
  const float* Uh;  // strict upper block strips, ld
  int64_t ld;
  int n, nb;        // order, 512-blocks
  float* V;         // in/out vector(s), ld ldv
  int64_t ldv;
  int* ready;       // per block: parts published
  int* ticket;
  int* err;
  int b0;           // forward: blocks before b0 are zero on entry (and stay zero)
  long long spin;   // polls before a wait gives up
};

// waits until all parts of block blk are published (thread 0 of the CTA)
__device__ __forceinline__ void tri_wait(const TriArgs& A, int blk, volatile int* abort_s) {
  long long it = 0;
  while (*((volatile int*)(A.ready + blk)) < TRI_Q) {
    if (*((volatile int*)A.err) != 0) {
      *abort_s = 1;
      return;
    }
    if (++it > A.spin) {
      atomicExch(A.err, 1);
      *abort_s = 1;
      return;
    }
    __nanosleep(64);
  }
  __threadfence();
}

// forward: z_j = V_j - sum_{c<j} Uh_cj^T z_c, in place on V (z_0 = V_0)
template <int NR>
__global__ void __launch_bounds__(TRI_THREADS) tri_forward(TriArgs A) {
  __shared__ __align__(16) float zs[NR][NB2];
  __shared__ int task_s;
  __shared__ volatile int abort_s;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const int nb = A.nb, b0 = A.b0, total = TRI_Q * (nb - 1 - b0);
  if (t == 0) abort_s = 0;
  for (;;) {
    __syncthreads();
    if (t == 0) task_s = atomicAdd(A.ticket, 1);
    __syncthreads();
    const int task = task_s;
    if (task >= total || abort_s) break;
    const int j = b0 + 1 + task / TRI_Q, q = task % TRI_Q;
    // columns col0 + cc of block j (TRI_QS / 8 per warp); each lane sums 16
    // rows of each source tile per column.  A tile is loaded into registers
    // before its source block is awaited (it does not depend on it).
    constexpr int CPW = TRI_QS / 8;
    const int col0 = j * NB2 + q * TRI_QS + warp * CPW;
    float acc[CPW][NR];
#pragma unroll
    for (int cc = 0; cc < CPW; cc++)
#pragma unroll
      for (int r = 0; r < NR; r++) acc[cc][r] = 0.f;
    for (int c = b0; c < j; c++) {  // the zero blocks before b0 add nothing
      const int c0 = c * NB2;  // a full block: c < nb - 1
      float4 v[CPW][NB2 / 128];
#pragma unroll
      for (int cc = 0; cc < CPW; cc++) {
        const int col = min(col0 + cc, A.n - 1);
        const float* u = A.Uh + c0 + (int64_t)col * A.ld;
#pragma unroll
        for (int i = 0; i < NB2 / 128; i++) v[cc][i] = __ldcs(reinterpret_cast<const float4*>(u + 4 * lane + 128 * i));
      }
      if (t == 0 && c > b0) tri_wait(A, c, &abort_s);
      __syncthreads();
      if (abort_s) break;
      for (int e = t; e < NB2; e += TRI_THREADS)
        for (int r = 0; r < NR; r++) zs[r][e] = __ldcg(A.V + c0 + e + r * A.ldv);
      __syncthreads();
#pragma unroll
      for (int cc = 0; cc < CPW; cc++)
#pragma unroll
        for (int i = 0; i < NB2 / 128; i++) {
          const int k = 4 * lane + 128 * i;
#pragma unroll
          for (int r = 0; r < NR; r++)
            acc[cc][r] += v[cc][i].x * zs[r][k] + v[cc][i].y * zs[r][k + 1] + v[cc][i].z * zs[r][k + 2] +
                          v[cc][i].w * zs[r][k + 3];
        }
      __syncthreads();  // zs is reloaded for the next source block
    }
    if (abort_s) break;
#pragma unroll
    for (int cc = 0; cc < CPW; cc++)
#pragma unroll
      for (int r = 0; r < NR; r++) {
        float a = acc[cc][r];
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        const int col = col0 + cc;
        if (lane == 0 && col < A.n) {
          float* v = A.V + col + r * A.ldv;
          *v = __ldcg(v) - a;
        }
      }
    __threadfence();
    __syncthreads();
    if (t == 0) atomicAdd(A.ready + j, 1);
  }
}

// backward: x_b = V_b - sum_{c>b} Uh_bc x_c, in place on V (x_{nb-1} = V_{nb-1})
template <int NR>
__global__ void __launch_bounds__(TRI_THREADS) tri_backward(TriArgs A) {
  __shared__ __align__(16) float xs[NR][NB2];
  __shared__ float red[32][NR][TRI_QS];
  __shared__ int task_s;
  __shared__ volatile int abort_s;
  const int t = threadIdx.x;
  const int nb = A.nb, total = TRI_Q * (nb - 1);
  if (t == 0) abort_s = 0;
  for (;;) {
    __syncthreads();
    if (t == 0) task_s = atomicAdd(A.ticket, 1);
    __syncthreads();
    const int task = task_s;
    if (task >= total || abort_s) break;
    const int b = nb - 2 - task / TRI_Q, q = task % TRI_Q;
    // rows r0 + rl .. + 3 of block b (a full block): 8 threads x 4 rows;
    // 32 k streams of 16 columns.  A tile is loaded into registers before its
    // source block is awaited.
    constexpr int KPS = NB2 / 32;
    const int r0 = b * NB2 + q * TRI_QS, rl = 4 * (t & 7), ks = t >> 3;
    float acc[NR][4];
#pragma unroll
    for (int r = 0; r < NR; r++)
#pragma unroll
      for (int i = 0; i < 4; i++) acc[r][i] = 0.f;
    for (int c = nb - 1; c > b; c--) {
      const int cst = c * NB2, kc = min(NB2, A.n - cst);
      const float* u = A.Uh + r0 + rl + (int64_t)cst * A.ld;
      float4 v[KPS];
#pragma unroll
      for (int kk = 0; kk < KPS; kk++) {
        const int k = min(ks * KPS + kk, kc - 1);
        v[kk] = __ldcs(reinterpret_cast<const float4*>(u + (int64_t)k * A.ld));
      }
      if (t == 0 && c < nb - 1) tri_wait(A, c, &abort_s);
      __syncthreads();
      if (abort_s) break;
      for (int e = t; e < NB2; e += TRI_THREADS)
        for (int r = 0; r < NR; r++) xs[r][e] = e < kc ? __ldcg(A.V + cst + e + r * A.ldv) : 0.f;
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < KPS; kk++) {
        const int k = ks * KPS + kk;  // x is zero past kc
#pragma unroll
        for (int r = 0; r < NR; r++) {
          const float x = xs[r][k];
          acc[r][0] += v[kk].x * x;
          acc[r][1] += v[kk].y * x;
          acc[r][2] += v[kk].z * x;
          acc[r][3] += v[kk].w * x;
        }
      }
      __syncthreads();  // xs is reloaded for the next source block
    }
    if (abort_s) break;
#pragma unroll
    for (int r = 0; r < NR; r++)
#pragma unroll
      for (int i = 0; i < 4; i++) red[ks][r][rl + i] = acc[r][i];
    __syncthreads();
    for (int e = t; e < NR * TRI_QS; e += TRI_THREADS) {
      const int r = e / TRI_QS, il = e % TRI_QS;
      float v = 0.f;
#pragma unroll
      for (int w = 0; w < 32; w++) v += red[w][r][il];
      float* p = A.V + r0 + il + r * A.ldv;
      *p = __ldcg(p) - v;
    }
    __threadfence();
    __syncthreads();
    if (t == 0) atomicAdd(A.ready + b, 1);
  }
}

// w_b = G_b z_b for every block: a CTA takes 128 rows of one block (32
// lanes x 4 rows, float4 loads) and splits the block's columns over its 8
// warps, reduced in shared memory
template <int NR>
__global__ void __launch_bounds__(256) blockdiag_gemv(int n, const float* __restrict__ G, const float* __restrict__ z,
                                                      float* __restrict__ w, int64_t ldx) {
  __shared__ __align__(16) float zsh[NR][NB2];
  __shared__ float red[8][NR][128];
  const int b = blockIdx.x / (NB2 / 128), rq = blockIdx.x % (NB2 / 128);
  const int j0 = b * NB2, jb = min(NB2, n - j0);
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  for (int e = t; e < NB2; e += 256)
    for (int r = 0; r < NR; r++) zsh[r][e] = e < jb ? z[j0 + e + r * ldx] : 0.f;
  __syncthreads();
  const float* Gb = G + (size_t)b * NB2 * NB2 + rq * 128 + 4 * lane;  // G_b is NB2 x NB2, zero-padded
  float acc[NR][4];
#pragma unroll
  for (int r = 0; r < NR; r++)
#pragma unroll
    for (int i = 0; i < 4; i++) acc[r][i] = 0.f;
  const int kbeg = warp * (NB2 / 8);
#pragma unroll 8
  for (int kk = 0; kk < NB2 / 8; kk++) {
    const int k = kbeg + kk;
    const float4 g = *reinterpret_cast<const float4*>(Gb + (size_t)k * NB2);
#pragma unroll
    for (int r = 0; r < NR; r++) {
      const float x = zsh[r][k];
      acc[r][0] += g.x * x;
      acc[r][1] += g.y * x;
      acc[r][2] += g.z * x;
      acc[r][3] += g.w * x;
    }
  }
#pragma unroll
  for (int r = 0; r < NR; r++)
#pragma unroll
    for (int i = 0; i < 4; i++) red[warp][r][4 * lane + i] = acc[r][i];
  __syncthreads();
  for (int e = t; e < NR * 128; e += 256) {
    const int r = e / 128, il = e % 128, row = rq * 128 + il;
    float v = 0.f;
#pragma unroll
    for (int q = 0; q < 8; q++) v += red[q][r][il];
    if (row < jb) w[j0 + row + r * ldx] = v;
  }
}

}  // namespace

// Builds Uh (strict upper block strips, ld ldu, in a buffer of its own) and
// the G_b blocks from the factor U and its NB2 block inverses W2.
int rsd_uhat_build(rsd_ctx* ctx, int n, const float* U, int64_t ldu, const float* W2, const char* tag,
                   rsd_uhat* out) {
  if (ldu % 4 != 0 || ((uintptr_t)U & 15)) return rsd_fail(ctx, RSD_EARG, "uhat: unsupported layout");
  const int nblk2 = (n + NB2 - 1) / NB2;
  std::string nu = std::string("uhat_U_") + tag, ng = std::string("uhat_G_") + tag;
  float* Uh = (float*)rsd_scratch(ctx, nu.c_str(), sizeof(float) * (size_t)ldu * n);
  float* G = (float*)rsd_scratch(ctx, ng.c_str(), sizeof(float) * (size_t)nblk2 * NB2 * NB2);
  float* WT = (float*)rsd_scratch(ctx, "uhat_WT", sizeof(float) * (size_t)nblk2 * NB2 * NB2);
  if (!Uh || !G || !WT) return RSD_ENOMEM;
  cudaStream_t s = ctx->stream;
  transpose_block<<<dim3(NB2 / 32, NB2 / 32, nblk2), dim3(32, 8), 0, s>>>(NB2, W2, WT); RSD_LAUNCH_NOTE();
  RSD_CUDA(ctx, cudaMemsetAsync(ctx->d_info + 1, 0, sizeof(int), s));
  int* err = ctx->d_info + 1;
  // all blocks in two batched launches: G_b = W_b W_b^T, and the strips
  // Uh_b = W_b^T U(block b rows, columns after block b), whose width drops
  // by NB2 from one block to the next
  const int64_t nw = (int64_t)nblk2 * NB2;
  RSD_TRY(rsd_tc_gemm_zbatch(ctx, 3, NB2, NB2, NB2, 1.0f, WT, NB2, NB2, nw, WT, NB2, NB2, nw, G, NB2, NB2, nw, nblk2,
                             0, NB2, 0, NB2, 0, NB2, 0, err));
  if (nblk2 > 1) {
    const float* U1 = U + (int64_t)NB2 * ldu;  // columns from NB2 on
    float* Uh1 = Uh + (int64_t)NB2 * ldu;
    RSD_TRY(rsd_tc_gemm_zbatch(ctx, 3, NB2, n - NB2, NB2, 1.0f, WT, NB2, NB2, nw, U1, ldu, n, n - NB2, Uh1, ldu, n,
                               n - NB2, nblk2 - 1, 0, NB2, NB2, NB2, NB2, NB2, NB2, err));
  }
  RSD_CUDA(ctx, cudaMemcpyAsync(ctx->h_info + 1, err, sizeof(int), cudaMemcpyDeviceToHost, s));
  RSD_CUDA(ctx, cudaStreamSynchronize(s));
  if (ctx->h_info[1]) return rsd_fail(ctx, RSD_ETIMEOUT, "uhat: tensor-core GEMM timed out");
  out->n = n;
  out->Uh = Uh;
  out->ld = ldu;
  out->G = G;
  return RSD_OK;
}

// X (n x nrhs, ld ldx) <- (U^T U)^-1 X with the block-scaled factor; Y is
// n x nrhs scratch (ld ldx).
int rsd_uhat_solve(rsd_ctx* ctx, const rsd_uhat* h, float* X, int64_t ldx, int nrhs, float* Y, int zero_lead) {
  if (nrhs < 1 || nrhs > 2) return rsd_fail(ctx, RSD_EARG, "uhat solve: 1 or 2 right-hand sides");
  const int n = h->n, nblk2 = (n + NB2 - 1) / NB2;
  cudaStream_t s = ctx->stream;
  const int gsm = ctx->sm_count > 0 ? ctx->sm_count : 148;
  if (nblk2 > TRI_MAX_BLOCKS) return rsd_fail(ctx, RSD_EUNSUP, "uhat solve: order %d above %d", n, TRI_MAX_BLOCKS * NB2);
  int* sync = rsd_uhat_error_flag(ctx);  // [0] error (cumulative), [1] ticket, ready counts
  if (!sync) return RSD_ENOMEM;
  // leading zero blocks of the right-hand side: the forward sweep starts at
  // the first block that can be nonzero (z is zero before it)
  const int b0 = zero_lead > 0 ? min(zero_lead / NB2, nblk2 - 1) : 0;
  TriArgs A{h->Uh, h->ld, n, nblk2, X, ldx, sync + 2, sync + 1, sync, b0,
            ctx->tri_spin_polls > 0 ? ctx->tri_spin_polls : TRI_SPIN_LIMIT};
  const int tasks = TRI_Q * (nblk2 - 1);
  const int grid = max(1, min(tasks, 4 * gsm));
  const int ftasks = TRI_Q * (nblk2 - 1 - b0);
  if (ftasks > 0) {  // forward, in place on X
    RSD_CUDA(ctx, cudaMemsetAsync(sync + 1, 0, sizeof(int) * (size_t)(1 + nblk2), s));
    const int fgrid = max(1, min(ftasks, 4 * gsm));
    if (nrhs == 1)
      tri_forward<1><<<fgrid, TRI_THREADS, 0, s>>>(A);
    else
      tri_forward<2><<<fgrid, TRI_THREADS, 0, s>>>(A);
    RSD_LAUNCH_NOTE();
  }
  if (nrhs == 1)
    blockdiag_gemv<1><<<nblk2 * (NB2 / 128), 256, 0, s>>>(n, h->G, X, Y, ldx);
  else
    blockdiag_gemv<2><<<nblk2 * (NB2 / 128), 256, 0, s>>>(n, h->G, X, Y, ldx);
  RSD_LAUNCH_NOTE();
  if (tasks > 0) {  // backward, in place on Y
    A.V = Y;
    A.b0 = 0;
    RSD_CUDA(ctx, cudaMemsetAsync(sync + 1, 0, sizeof(int) * (size_t)(1 + nblk2), s));
    if (nrhs == 1)
      tri_backward<1><<<grid, TRI_THREADS, 0, s>>>(A);
    else
      tri_backward<2><<<grid, TRI_THREADS, 0, s>>>(A);
    RSD_LAUNCH_NOTE();
  }
  for (int r = 0; r < nrhs; r++)
    RSD_CUDA(ctx, cudaMemcpyAsync(X + r * ldx, Y + r * ldx, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
  RSD_CUDA(ctx, cudaGetLastError());
  return RSD_OK;
}

// The dataflow sweeps' synchronisation words; element 0 is a cumulative
// error flag, nonzero once a sweep's wait timed out (the caller zeroes it
// and reads it after synchronising the stream).
int* rsd_uhat_error_flag(rsd_ctx* ctx) {
  return (int*)rsd_scratch(ctx, "tri_sync", sizeof(int) * (size_t)(2 * TRI_MAX_BLOCKS + 2));
}

int rsd_potrs_wide_s(rsd_ctx* ctx, int n, const float* U, int64_t ldu, const float* W2, float* X, int64_t ldx,
                     int nrhs, float* Y) {
  const int nblk2 = (n + NB2 - 1) / NB2;
  // forward: U^T y = b, y_b = W_b^T (b_b - sum) ; X keeps the running rhs
  for (int b = 0; b < nblk2; b++) {
    const int j0 = b * NB2, jb = n - j0 < NB2 ? n - j0 : NB2, rest = n - j0 - jb;
    RSD_TRY(rsd_gemv<float>(ctx, 1, jb, jb, 1.0f, W2 + (size_t)b * NB2 * NB2, NB2, X + j0, ldx, nrhs, 0.0f, Y + j0,
                            ldx));
    if (rest > 0)
      RSD_TRY(rsd_gemv<float>(ctx, 1, rest, jb, -1.0f, U + j0 + (int64_t)(j0 + jb) * ldu, ldu, Y + j0, ldx, nrhs, 1.0f,
                              X + j0 + jb, ldx));
  }
  // backward: U x = y ; Y keeps the running rhs, X receives x
  for (int b = nblk2 - 1; b >= 0; b--) {
    const int j0 = b * NB2, jb = n - j0 < NB2 ? n - j0 : NB2;
    RSD_TRY(rsd_gemv<float>(ctx, 0, jb, jb, 1.0f, W2 + (size_t)b * NB2 * NB2, NB2, Y + j0, ldx, nrhs, 0.0f, X + j0,
                            ldx));
    if (j0 > 0)
      RSD_TRY(rsd_gemv<float>(ctx, 0, j0, jb, -1.0f, U + (int64_t)j0 * ldu, ldu, X + j0, ldx, nrhs, 1.0f, Y, ldx));
  }
  RSD_CUDA(ctx, cudaGetLastError());
  return RSD_OK;
}

// Solve (U^T U) X = B in place (X holds B), nrhs <= 4; W from the factor's
// diagonal blocks (computed here when W == nullptr)
template <typename T>
int rsd_potrs_upper_t(rsd_ctx* ctx, int n, const T* d_U, int64_t ldu, T* d_X, int64_t ldx, int nrhs, const char* tag,
                      const T* W) {
  cudaStream_t s = ctx->stream;
  if (!W) {
    T* Wn = nullptr;
    RSD_TRY(rsd_diag_inverses_t<T>(ctx, n, d_U, ldu, tag, &Wn));
    W = Wn;
  }
  const int nblk = (n + NB - 1) / NB;
  if (nrhs > 4) {
    // many right-hand sides: left-looking block substitution with GEMMs
    T* Tb = (T*)rsd_scratch(ctx, sizeof(T) == 8 ? "potrs_tmp_d" : "potrs_tmp_s", sizeof(T) * (size_t)NB * nrhs);
    if (!Tb) return RSD_ENOMEM;
    for (int b = 0; b < nblk; b++) {
      const int j0 = b * NB, jb = n - j0 < NB ? n - j0 : NB;
      if (j0 > 0) launch_gemm<T>(s, gp(jb, nrhs, j0, -1.0, d_U + (int64_t)j0 * ldu, ldu, 1, d_X, ldx, 0, 1.0, d_X + j0, ldx));
      launch_gemm<T>(s, gp(jb, nrhs, jb, 1.0, W + (size_t)b * NB * NB, NB, 1, d_X + j0, ldx, 0, 0.0, Tb, NB));
      RSD_CUDA(ctx, cudaMemcpy2DAsync(d_X + j0, ldx * sizeof(T), Tb, NB * sizeof(T), jb * sizeof(T), nrhs,
                                      cudaMemcpyDeviceToDevice, s));
    }
    for (int b = nblk - 1; b >= 0; b--) {
      const int j0 = b * NB, jb = n - j0 < NB ? n - j0 : NB, rest = n - j0 - jb;
      if (rest > 0)
        launch_gemm<T>(s, gp(jb, nrhs, rest, -1.0, d_U + j0 + (int64_t)(j0 + jb) * ldu, ldu, 0, d_X + j0 + jb, ldx, 0,
                             1.0, d_X + j0, ldx));
      launch_gemm<T>(s, gp(jb, nrhs, jb, 1.0, W + (size_t)b * NB * NB, NB, 0, d_X + j0, ldx, 0, 0.0, Tb, NB));
      RSD_CUDA(ctx, cudaMemcpy2DAsync(d_X + j0, ldx * sizeof(T), Tb, NB * sizeof(T), jb * sizeof(T), nrhs,
                                      cudaMemcpyDeviceToDevice, s));
    }
    RSD_CUDA(ctx, cudaGetLastError());
    return RSD_OK;
  }
  // forward: U^T y = b
  for (int b = 0; b < nblk; b++) {
    const int j0 = b * NB, jb = n - j0 < NB ? n - j0 : NB, rest = n - j0 - jb;
    trsv_diag<T><<<1, 256, smem_trsv<T>(), s>>>(jb, W + (size_t)b * NB * NB, NB, 1, d_X + j0, ldx, nrhs); RSD_LAUNCH_NOTE();
    if (rest > 0)
      RSD_TRY(rsd_gemv<T>(ctx, 1, rest, jb, T(-1), d_U + j0 + (int64_t)(j0 + jb) * ldu, ldu, d_X + j0, ldx, nrhs,
                          T(1), d_X + j0 + jb, ldx));
  }
  // backward: U x = y
  for (int b = nblk - 1; b >= 0; b--) {
    const int j0 = b * NB, jb = n - j0 < NB ? n - j0 : NB;
    trsv_diag<T><<<1, 256, smem_trsv<T>(), s>>>(jb, W + (size_t)b * NB * NB, NB, 0, d_X + j0, ldx, nrhs); RSD_LAUNCH_NOTE();
    if (j0 > 0)
      RSD_TRY(rsd_gemv<T>(ctx, 0, j0, jb, T(-1), d_U + (int64_t)j0 * ldu, ldu, d_X + j0, ldx, nrhs, T(1), d_X, ldx));
  }
  RSD_CUDA(ctx, cudaGetLastError());
  return RSD_OK;
}

template void rsd_gemm<float>(cudaStream_t, int, int, int, double, const float*, int64_t, int, const float*, int64_t,
                              int, double, float*, int64_t);
template int rsd_gemv<float>(rsd_ctx*, int, int, int, float, const float*, int64_t, const float*, int64_t, int, float,
                             float*, int64_t);
template int rsd_gemv<double>(rsd_ctx*, int, int, int, double, const double*, int64_t, const double*, int64_t, int,
                              double, double*, int64_t);
template int rsd_potrf_upper_t<float>(rsd_ctx*, int, float*, int64_t, int*, const char*, int);
template int rsd_potri_upper_t<float>(rsd_ctx*, int, float*, int64_t, const char*, int);
template int rsd_potrs_upper_t<float>(rsd_ctx*, int, const float*, int64_t, float*, int64_t, int, const char*,
                                      const float*);
template int rsd_mirror_upper_t<float>(rsd_ctx*, int, float*, int64_t);
template int rsd_diag_inverses_t<float>(rsd_ctx*, int, const float*, int64_t, const char*, float**);

// ------------------------------------------------------------ FP64 names
void rsd_gemm_f64(cudaStream_t s, int m, int n, int k, double alpha, const double* A, int64_t lda, int ta,
                  const double* B, int64_t ldb, int tb, double beta, double* C, int64_t ldc) {
  launch_gemm<double>(s, gp(m, n, k, alpha, A, lda, ta, B, ldb, tb, beta, C, ldc));
}
int rsd_zero_lower(rsd_ctx* ctx, int n, double* d_A, int64_t lda) { return rsd_zero_lower_t<double>(ctx, n, d_A, lda); }
int rsd_mirror_upper(rsd_ctx* ctx, int n, double* d_A, int64_t lda) {
  return rsd_mirror_upper_t<double>(ctx, n, d_A, lda);
}
int rsd_potrf_upper_tag(rsd_ctx* ctx, int n, double* d_A, int64_t lda, int* info, const char* tag) {
  return rsd_potrf_upper_t<double>(ctx, n, d_A, lda, info, tag, 0);
}
int rsd_potrf_upper(rsd_ctx* ctx, int n, double* d_A, int64_t lda, int* info) {
  return rsd_potrf_upper_t<double>(ctx, n, d_A, lda, info, "A", 0);
}
int rsd_potri_upper_tag(rsd_ctx* ctx, int n, double* d_A, int64_t lda, const char* tag) {
  return rsd_potri_upper_t<double>(ctx, n, d_A, lda, tag, 0);
}
int rsd_potri_upper(rsd_ctx* ctx, int n, double* d_A, int64_t lda) {
  return rsd_potri_upper_t<double>(ctx, n, d_A, lda, "A", 0);
}
int rsd_potrs_upper_tag(rsd_ctx* ctx, int n, const double* d_U, int64_t ldu, double* d_X, int64_t ldx, int nrhs,
                        const char* tag) {
  // the factor's diagonal-block inverses are still in the tag's buffer
  const double* W = diag_inverses<double>(ctx, n, tag);
  return rsd_potrs_upper_t<double>(ctx, n, d_U, ldu, d_X, ldx, nrhs, tag, W);
}
int rsd_trsv_upper(rsd_ctx* ctx, int n, const double* d_U, int64_t ldu, double* d_X, int64_t ldx, int nrhs,
                   int transpose) {
  (void)transpose;
  return rsd_potrs_upper_tag(ctx, n, d_U, ldu, d_X, ldx, nrhs, "A");
}

// ------------------------------------------------ FP32 exported blocks
static int check_prec(rsd_ctx* ctx, int prec) {
  if (prec != 0 && prec != 1 && prec != 3) return rsd_fail(ctx, RSD_EARG, "prec must be 0, 1 or 3 (got %d)", prec);
  return RSD_OK;
}

extern "C" int rsd_syrk_f32_dev(rsd_ctx* ctx, int32_t n, int32_t k, const float* d_P, int64_t ldp, float* d_C,
                                int64_t ldc, int32_t prec) {
  if (!ctx) return RSD_EARG;
  if (n < 1 || k < 1 || ldp < k || ldc < n || !d_P || !d_C)
    return rsd_fail(ctx, RSD_EARG, "rsd_syrk_f32_dev: bad arguments");
  RSD_TRY(check_prec(ctx, prec));
  RSD_TRY(rsd_set_device(ctx));
  if (prec && ctx->use_tc && k <= NB && rsd_tc_syrk_ok(d_P, ldp, d_C, ldc, k)) {
    RSD_CUDA(ctx, cudaMemsetAsync(ctx->d_info + 1, 0, sizeof(int), ctx->stream));
    RSD_TRY(rsd_tc_syrk(ctx, prec, d_P, ldp, k, n, d_C, ldc, ctx->d_info + 1));
    RSD_CUDA(ctx, cudaMemcpyAsync(ctx->h_info + 1, ctx->d_info + 1, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    RSD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (ctx->h_info[1]) return rsd_fail(ctx, RSD_ETIMEOUT, "syrk: tensor-core update timed out");
    return RSD_OK;
  }
  GemmP g = gp(n, n, k, -1.0, d_P, ldp, 1, d_P, ldp, 0, 1.0, d_C, ldc);
  g.uplo = 1;
  launch_gemm<float>(ctx->stream, g);
  RSD_CUDA(ctx, cudaGetLastError());
  RSD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return RSD_OK;
}

extern "C" int rsd_potrf_f32_dev(rsd_ctx* ctx, int32_t n, float* d_A, int64_t lda, int32_t prec, int32_t* info) {
  if (!ctx) return RSD_EARG;
  if (n < 1 || lda < n || !d_A || !info) return rsd_fail(ctx, RSD_EARG, "rsd_potrf_f32_dev: bad arguments");
  RSD_TRY(check_prec(ctx, prec));
  RSD_TRY(rsd_set_device(ctx));
  int inf = 0;
  RSD_TRY(rsd_potrf_upper_t<float>(ctx, n, d_A, lda, &inf, "f32dev", prec));
  *info = inf;
  return RSD_OK;
}

extern "C" int rsd_potri_f32_dev(rsd_ctx* ctx, int32_t n, float* d_A, int64_t lda, int32_t prec) {
  if (!ctx) return RSD_EARG;
  if (n < 1 || lda < n || !d_A) return rsd_fail(ctx, RSD_EARG, "rsd_potri_f32_dev: bad arguments");
  RSD_TRY(check_prec(ctx, prec));
  RSD_TRY(rsd_set_device(ctx));
  RSD_TRY(rsd_potri_upper_t<float>(ctx, n, d_A, lda, "f32dev", prec));
  RSD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return RSD_OK;
}
