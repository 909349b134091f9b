// Learned preconditioner of the resistance solve.  The FTS step solves
// RPP U = F' (STEPPER_NOGmres, src/stepper.f90:370-393: MATREV(RPP)), RPP
// the 6N x 6N translational/rotational block of R = M^-1 + R_lub.  This file
// holds:
//   - the graph of near-neighbour pairs (minimum-image centre distance
//     below 3 a_avg on the Lees-Edwards lattice), CSR by destination;
//   - a block-sparse approximate inverse of RPP in factorised form
//     G = D^-1/2 Z^T Z D^-1/2 (D = diag RPP, Z block lower triangular with
//     6 x 6 blocks on the particle diagonal and on the pairs (a, b), b < a):
//     SPD whenever the diagonal blocks of Z are non-singular, so it can
//     precondition conjugate gradients;
//   - Z either exact (the factorised sparse approximate inverse, FSAI, of
//     Kolotilina and Yeremin, 1993: row block a minimises the Kaporin
//     condition number over the pattern, from one local dense solve on the
//     lower neighbours of a) or learned: a 3-layer message-passing network,
//     hidden width 64, BF16 weights and activations with FP32 accumulation,
//     whose inputs are the Jacobi-scaled blocks of RPP on the graph and the
//     pair gaps, emits for every lower edge (a <- b) the direction
//     W_ab = Z_aa^-1 Z_ab; the row block is then Z_a = C [W_a.., I] with C
//     fixed by (Z A Z^T)_aa = I from the local matrix (lp_normalize), which
//     keeps G SPD and its diagonal blocks exact whatever the network emits;
//   - the network's forward pass, its backward pass against a supervised
//     loss (the exact FSAI directions of the training matrices), and an Adam
//     step, all as kernels here;
//   - preconditioned conjugate gradients in FP64 on RPP (dense symmetric
//     products), with the preconditioner none, Jacobi, block-Jacobi (FSAI
//     on the diagonal pattern), exact FSAI or learned.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "rsd_internal.cuh"

template <typename T>
int rsd_gemv(rsd_ctx* ctx, int trans, int m, int k, T alpha, const T* A, int64_t lda, const T* X, int64_t ldx,
             int nrhs, T beta, T* y, int64_t ldy);

namespace {

constexpr int H = 64;          // hidden width
constexpr int NF_NODE = 36;    // node input: the scaled 6 x 6 self block
constexpr int NF_EDGE = 40;    // edge input: the scaled 6 x 6 pair block, gap, log gap, lower flag, zero pad
constexpr int NLAYER = 3;
constexpr int NOUT = 36;       // a 6 x 6 block of Z
constexpr int LP_KMAX = 16;    // lower neighbours per particle kept in a row block of Z
constexpr float LP_CUT = 3.0f; // graph: centre distance below LP_CUT a_avg

// parameter layout (FP32 master copy; weight matrices row-major [out][in])
struct Layout {
  int64_t enc_n_w, enc_n_b, enc_e_w, enc_e_b;
  int64_t msg_w[NLAYER], msg_b[NLAYER], upd_w[NLAYER], upd_b[NLAYER];
  int64_t head_n_w, head_n_b, head_e_w, head_e_b;
  int64_t total;
};

constexpr Layout make_layout() {
  Layout L{};
  int64_t o = 0;
  L.enc_n_w = o; o += H * NF_NODE;
  L.enc_n_b = o; o += H;
  L.enc_e_w = o; o += H * NF_EDGE;
  L.enc_e_b = o; o += H;
  for (int l = 0; l < NLAYER; l++) {
    L.msg_w[l] = o; o += H * 3 * H;
    L.msg_b[l] = o; o += H;
    L.upd_w[l] = o; o += H * 2 * H;
    L.upd_b[l] = o; o += H;
  }
  L.head_n_w = o; o += NOUT * H;
  L.head_n_b = o; o += NOUT;
  L.head_e_w = o; o += NOUT * 3 * H;
  L.head_e_b = o; o += NOUT;
  L.total = o;
  return L;
}
constexpr Layout LAY = make_layout();

}  // namespace

struct rsd_lp {
  int device = 0;
  float* w = nullptr;            // FP32 master parameters
  __nv_bfloat16* wb = nullptr;   // BF16 copies read by the kernels
  float* g = nullptr;            // gradient
  float* m = nullptr;            // Adam moments
  float* v = nullptr;
  double* gn2 = nullptr;         // squared norm of the last gradient (device)
  float clip = 0.f;              // global gradient-norm clip (0: off)
  double max_loss = 0.0;         // a train step with a larger loss makes no update (0: off)
  double last_gnorm = 0.0;       // norm of the last gradient
  int64_t skipped = 0;           // train steps that made no update
  int64_t step = 0;
};

namespace {

// ------------------------------------------------------------------ graph
// CSR by destination: edges e in [off[a], off[a+1]) are (a <- src[e]) with
// src[e] != a, sorted by src; rev[e] is the edge (src[e] <- a); gap[e] the
// surface gap r - (a_a + a_b).
// (evaluated with the lower index first, so that the relation is symmetric
// bit for bit)
__device__ inline bool lp_pair(const rsd_lat_dev& L, const double* pos, const double* radii, int a0, int b0,
                               double* gap) {
  const int a = min(a0, b0), b = max(a0, b0);
  double R[3] = {pos[3 * a] - pos[3 * b], pos[3 * a + 1] - pos[3 * b + 1], pos[3 * a + 2] - pos[3 * b + 2]};
  double dmin;
  rsd_skew_correction(L.LR, L.LI, R, &dmin);
  const double ab = 0.5 * (radii[a] + radii[b]);
  *gap = dmin - 2.0 * ab;
  return dmin < (double)LP_CUT * ab;
}

__global__ void lp_count(int nn, rsd_lat_dev L, const double* __restrict__ pos, const double* __restrict__ radii,
                         int* __restrict__ cnt) {
  const int a = blockIdx.x;
  int c = 0;
  for (int b = threadIdx.x; b < nn; b += blockDim.x) {
    double g;
    if (b != a && lp_pair(L, pos, radii, a, b, &g)) c++;
  }
  __shared__ int red[256];
  red[threadIdx.x] = c;
  __syncthreads();
  for (int d = blockDim.x / 2; d > 0; d >>= 1) {
    if (threadIdx.x < d) red[threadIdx.x] += red[threadIdx.x + d];
    __syncthreads();
  }
  if (threadIdx.x == 0) cnt[a] = red[0];
}

// one warp per destination: the sources in ascending order (ballot + prefix)
__global__ void lp_fill(int nn, rsd_lat_dev L, const double* __restrict__ pos, const double* __restrict__ radii,
                        const int* __restrict__ off, int* __restrict__ src, int* __restrict__ dst,
                        float* __restrict__ gap) {
  const int a = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32, lane = threadIdx.x & 31;
  if (a >= nn) return;
  int o = off[a];
  for (int b0 = 0; b0 < nn; b0 += 32) {
    const int b = b0 + lane;
    double g = 0.0;
    const bool in = b < nn && b != a && lp_pair(L, pos, radii, a, b, &g);
    const unsigned m = __ballot_sync(0xffffffffu, in);
    if (in) {
      const int k = o + __popc(m & ((1u << lane) - 1u));
      src[k] = b;
      dst[k] = a;
      gap[k] = (float)g;
    }
    o += __popc(m);
  }
}

// rev[e]: the edge (src <- dst) in src's list (binary search, lists sorted)
__global__ void lp_rev(int ne, const int* __restrict__ off, const int* __restrict__ src, const int* __restrict__ dst,
                       int* __restrict__ rev) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const int b = src[e], a = dst[e];
  int lo = off[b], hi = off[b + 1] - 1, r = -1;
  while (lo <= hi) {
    const int mid = (lo + hi) >> 1;
    if (src[mid] == a) {
      r = mid;
      break;
    }
    if (src[mid] < a)
      lo = mid + 1;
    else
      hi = mid - 1;
  }
  rev[e] = r;
}

// ------------------------------------------------------------ RPP access
// entry (i, j) of RPP in the particle-block layout (6a + k: k < 3
// translation 3a + k of the grand layout, k >= 3 rotation 3N + 3a + k - 3)
__device__ __forceinline__ int64_t grand_row(int nn, int i) {
  const int a = i / 6, k = i % 6;
  return k < 3 ? 3 * a + k : 3 * nn + 3 * a + (k - 3);
}

template <typename T>
__device__ __forceinline__ double rpp_at(const T* A, int64_t ld, int nn, int i, int j) {
  return (double)A[grand_row(nn, i) + grand_row(nn, j) * ld];
}

// dinv[i] = 1 / sqrt(RPP(i, i)) in the particle-block layout
template <typename T>
__global__ void lp_dinv(int nn, const T* __restrict__ A, int64_t ld, double* __restrict__ dinv, int* __restrict__ bad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 6 * nn) return;
  const double d = rpp_at(A, ld, nn, i, i);
  if (!(d > 0.0)) atomicExch(bad, 1);
  dinv[i] = d > 0.0 ? 1.0 / sqrt(d) : 1.0;
}

// network inputs: node a -> the scaled self block (36); edge e = (a <- b) ->
// the scaled block (a, b) (36), gap, log(gap + 1e-4) / 4, [b < a], 0
// Entries of a Jacobi-scaled symmetric positive definite matrix lie in
// [-1, 1]; an FP32 resistance matrix that has lost definiteness (overlapping
// spheres) can leave that range, and is clamped back so that the network's
// inputs stay bounded.
__device__ __forceinline__ float clamp1(float v) { return fminf(fmaxf(v, -1.f), 1.f); }

template <typename T>
__global__ void lp_features(int nn, int ne, const T* __restrict__ A, int64_t ld, const double* __restrict__ dinv,
                            const int* __restrict__ src, const int* __restrict__ dst, const float* __restrict__ gap,
                            __nv_bfloat16* __restrict__ xn, __nv_bfloat16* __restrict__ xe) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < nn * 36) {
    const int a = t / 36, q = t % 36, r = q / 6, c = q % 6;
    const int i = 6 * a + r, j = 6 * a + c;
    xn[t] = __float2bfloat16(clamp1((float)(rpp_at(A, ld, nn, i, j) * dinv[i] * dinv[j])));
  }
  const int u = t - nn * 36;
  if (u >= 0 && u < ne * NF_EDGE) {
    const int e = u / NF_EDGE, q = u % NF_EDGE;
    const int a = dst[e], b = src[e];
    float v;
    if (q < 36) {
      const int i = 6 * a + q / 6, j = 6 * b + q % 6;
      v = clamp1((float)(rpp_at(A, ld, nn, i, j) * dinv[i] * dinv[j]));
    } else if (q == 36) {
      v = gap[e];
    } else if (q == 37) {
      v = logf(fmaxf(gap[e], 0.f) + 1e-4f) * 0.25f;
    } else if (q == 38) {
      v = b < a ? 1.f : 0.f;
    } else {
      v = 0.f;
    }
    xe[u] = __float2bfloat16(v);
  }
}

// ------------------------------------------------------------ exact FSAI
// One CTA per particle a: J = (up to LP_KMAX nearest lower neighbours, a),
// the scaled local matrix B = A^[J, J] in shared memory (FP64), its
// Cholesky factor, Y = B^-1 E_a (6 right-hand sides), S = L^-1 for the
// Cholesky factor L of Y_aa (so that S Y_aa S^T = I), and the row block
// Z_a = S Y^T, written
// as the diagonal block zd[a] and the blocks ze[e] of the kept lower edges
// (other lower edges of a get zero blocks).
constexpr int FS_THREADS = 128;

// S = L^-1 for Y = L L^T (Cholesky of a symmetric positive definite 6 x 6
// matrix, row-major in and out).  Any factor C with C Y C^T = I gives the same
// G = Z^T Z; the Cholesky one is the cheapest and needs no iteration.
__device__ void sym6_chol_inv(const double* Y, double* S) {
  double L[6][6];
  for (int i = 0; i < 6; i++)
    for (int j = 0; j < 6; j++) L[i][j] = 0.0;
  for (int j = 0; j < 6; j++) {
    double d = 0.5 * (Y[j * 6 + j] + Y[j * 6 + j]);
    for (int k = 0; k < j; k++) d -= L[j][k] * L[j][k];
    L[j][j] = sqrt(fmax(d, 1e-300));
    for (int i = j + 1; i < 6; i++) {
      double x = 0.5 * (Y[i * 6 + j] + Y[j * 6 + i]);
      for (int k = 0; k < j; k++) x -= L[i][k] * L[j][k];
      L[i][j] = x / L[j][j];
    }
  }
  // S = L^-1 (lower triangular), column by column
  for (int c = 0; c < 6; c++)
    for (int i = 0; i < 6; i++) {
      double x = i == c ? 1.0 : 0.0;
      for (int k = c; k < i; k++) x -= L[i][k] * S[k * 6 + c];
      S[i * 6 + c] = i < c ? 0.0 : x / L[i][i];
    }
}

template <typename T>
__global__ void __launch_bounds__(FS_THREADS) lp_fsai(int nn, int lower_only_self, const T* __restrict__ A, int64_t ld,
                                                      const double* __restrict__ dinv, const int* __restrict__ off,
                                                      const int* __restrict__ src, const float* __restrict__ gap,
                                                      float* __restrict__ zd, float* __restrict__ ze,
                                                      float* __restrict__ wt, int* __restrict__ bad) {
  extern __shared__ double fs_smem[];
  __shared__ int nb_s[LP_KMAX + 1];
  __shared__ int eidx_s[LP_KMAX];
  __shared__ int k_s;
  __shared__ double S_s[36], P_s[36];
  const int a = blockIdx.x, t = threadIdx.x;
  const int e0 = off[a], e1 = off[a + 1];
  if (t == 0) {
    // the nearest lower neighbours, up to LP_KMAX (selection by gap)
    int k = 0;
    if (!lower_only_self) {
      for (int e = e0; e < e1; e++) {
        if (src[e] >= a) continue;
        if (k < LP_KMAX) {
          eidx_s[k++] = e;
        } else {
          int worst = 0;
          for (int q = 1; q < k; q++)
            if (gap[eidx_s[q]] > gap[eidx_s[worst]]) worst = q;
          if (gap[e] < gap[eidx_s[worst]]) eidx_s[worst] = e;
        }
      }
    }
    for (int q = 0; q < k; q++) nb_s[q] = src[eidx_s[q]];
    nb_s[k] = a;
    k_s = k;
  }
  __syncthreads();
  const int k = k_s, m = 6 * (k + 1);
  double* B = fs_smem;            // m x m, column-major
  double* Y = B + m * m;          // m x 6
  for (int q = t; q < m * m; q += FS_THREADS) {
    const int r = q % m, c = q / m;
    const int i = 6 * nb_s[r / 6] + r % 6, j = 6 * nb_s[c / 6] + c % 6;
    B[q] = rpp_at(A, ld, nn, i, j) * dinv[i] * dinv[j];
  }
  __syncthreads();
  // Cholesky B = L L^T (lower, in place), column by column
  for (int j = 0; j < m; j++) {
    if (t == 0) {
      const double d = B[j + j * m];
      if (!(d > 0.0)) atomicExch(bad, 2);
      B[j + j * m] = sqrt(fmax(d, 1e-300));
    }
    __syncthreads();
    const double piv = B[j + j * m];
    for (int i = j + 1 + t; i < m; i += FS_THREADS) B[i + j * m] /= piv;
    __syncthreads();
    for (int q = t; q < (m - j - 1) * (m - j - 1); q += FS_THREADS) {
      const int i = j + 1 + q % (m - j - 1), c = j + 1 + q / (m - j - 1);
      if (i >= c) B[i + c * m] -= B[i + j * m] * B[c + j * m];
    }
    __syncthreads();
  }
  // Y = B^-1 E_a, E_a the last 6 unit columns: forward then backward
  // substitution, one thread per right-hand side
  if (t < 6) {
    double* y = Y + t * m;
    for (int i = 0; i < m; i++) y[i] = (i == m - 6 + t) ? 1.0 : 0.0;
    for (int i = 0; i < m; i++) {
      double s = y[i];
      for (int c = 0; c < i; c++) s -= B[i + c * m] * y[c];
      y[i] = s / B[i + i * m];
    }
    for (int i = m - 1; i >= 0; i--) {
      double s = y[i];
      for (int r = i + 1; r < m; r++) s -= B[r + i * m] * y[r];
      y[i] = s / B[i + i * m];
    }
  }
  __syncthreads();
  if (t == 0) {
    double Yaa[36];
    for (int r = 0; r < 6; r++)
      for (int c = 0; c < 6; c++) Yaa[r * 6 + c] = Y[c * m + (m - 6 + r)];
    sym6_chol_inv(Yaa, S_s);
    for (int r = 0; r < 6; r++)  // P = S^T S = Y_aa^-1
      for (int c = 0; c < 6; c++) {
        double x = 0.0;
        for (int q = 0; q < 6; q++) x += S_s[q * 6 + r] * S_s[q * 6 + c];
        P_s[r * 6 + c] = x;
      }
  }
  __syncthreads();
  // the directions W_ab = Z_aa^-1 Z_ab = Y_aa^-1 Y_b^T of the kept edges
  // (NaN for lower edges not kept): the learned network's targets
  if (wt) {
    for (int q = t; q < 36 * k; q += FS_THREADS) {
      const int grp = q / 36, r = (q % 36) / 6, c = q % 6;
      double x = 0.0;
      for (int y = 0; y < 6; y++) x += P_s[r * 6 + y] * Y[y * m + 6 * grp + c];
      wt[(size_t)eidx_s[grp] * 36 + r * 6 + c] = (float)x;
    }
    for (int e = e0 + t; e < e1; e += FS_THREADS) {
      if (src[e] >= a) continue;
      bool kept = false;
      for (int q = 0; q < k; q++) kept |= eidx_s[q] == e;
      if (!kept)
        for (int x = 0; x < 36; x++) wt[(size_t)e * 36 + x] = __int_as_float(0x7fc00000);
    }
  }
  // Z_a = S Y^T: block of column group g is S (Y[g rows])^T
  for (int q = t; q < 36 * (k + 1); q += FS_THREADS) {
    const int grp = q / 36, r = (q % 36) / 6, c = q % 6;
    double s = 0.0;
    for (int x = 0; x < 6; x++) s += S_s[r * 6 + x] * Y[x * m + 6 * grp + c];
    if (grp == k)
      zd[(size_t)a * 36 + r * 6 + c] = (float)s;
    else
      ze[(size_t)eidx_s[grp] * 36 + r * 6 + c] = (float)s;
  }
  // the lower edges not kept get zero blocks
  for (int e = e0 + t; e < e1; e += FS_THREADS) {
    if (src[e] >= a) continue;
    bool kept = false;
    for (int q = 0; q < k; q++) kept |= eidx_s[q] == e;
    if (!kept)
      for (int x = 0; x < 36; x++) ze[(size_t)e * 36 + x] = 0.f;
  }
}

// From directions W_ab (edge blocks of w, the network's output for the kept
// lower edges) to the factor Z: the row block Z_a = C [W_a.., I] with C the
// inverse Cholesky factor of M_a = [W_a.., I] A^_JJ [W_a.., I]^T (6 x 6, SPD
// for any W since the last block is I), so that (Z A^ Z^T)_aa = I and
// G = Z^T Z is SPD whatever the network emits.  One CTA per particle, the
// same neighbour selection as lp_fsai.
template <typename T>
__global__ void __launch_bounds__(FS_THREADS) lp_normalize(int nn, const T* __restrict__ A, int64_t ld,
                                                           const double* __restrict__ dinv,
                                                           const int* __restrict__ off, const int* __restrict__ src,
                                                           const float* __restrict__ gap,
                                                           const float* __restrict__ w, float* __restrict__ zd,
                                                           float* __restrict__ ze) {
  extern __shared__ double fs_smem[];
  __shared__ int nb_s[LP_KMAX + 1];
  __shared__ int eidx_s[LP_KMAX];
  __shared__ int k_s;
  __shared__ double M_s[36], S_s[36];
  const int a = blockIdx.x, t = threadIdx.x;
  const int e0 = off[a], e1 = off[a + 1];
  if (t == 0) {
    int k = 0;
    for (int e = e0; e < e1; e++) {
      if (src[e] >= a) continue;
      if (k < LP_KMAX) {
        eidx_s[k++] = e;
      } else {
        int worst = 0;
        for (int q = 1; q < k; q++)
          if (gap[eidx_s[q]] > gap[eidx_s[worst]]) worst = q;
        if (gap[e] < gap[eidx_s[worst]]) eidx_s[worst] = e;
      }
    }
    for (int q = 0; q < k; q++) nb_s[q] = src[eidx_s[q]];
    nb_s[k] = a;
    k_s = k;
  }
  __syncthreads();
  const int k = k_s, m = 6 * (k + 1);
  double* B = fs_smem;      // m x m, column-major
  double* Wf = B + m * m;   // 6 x m, row-major: [W_a.., I]
  double* Tm = Wf + 6 * m;  // m x 6: B Wf^T
  for (int q = t; q < m * m; q += FS_THREADS) {
    const int r = q % m, c = q / m;
    const int i = 6 * nb_s[r / 6] + r % 6, j = 6 * nb_s[c / 6] + c % 6;
    B[q] = rpp_at(A, ld, nn, i, j) * dinv[i] * dinv[j];
  }
  for (int q = t; q < 6 * m; q += FS_THREADS) {
    const int r = q / m, j = q % m, grp = j / 6, c = j % 6;
    Wf[q] = grp == k ? (r == c ? 1.0 : 0.0) : (double)w[(size_t)eidx_s[grp] * 36 + r * 6 + c];
  }
  __syncthreads();
  for (int q = t; q < 6 * m; q += FS_THREADS) {
    const int i = q / 6, r = q % 6;
    double x = 0.0;
    for (int j = 0; j < m; j++) x += B[i + (size_t)j * m] * Wf[r * m + j];
    Tm[i * 6 + r] = x;
  }
  __syncthreads();
  if (t < 36) {
    const int r = t / 6, c = t % 6;
    double x = 0.0;
    for (int i = 0; i < m; i++) x += Wf[r * m + i] * Tm[i * 6 + c];
    M_s[t] = x;
  }
  __syncthreads();
  if (t == 0) sym6_chol_inv(M_s, S_s);
  __syncthreads();
  for (int q = t; q < 36 * (k + 1); q += FS_THREADS) {
    const int grp = q / 36, r = (q % 36) / 6, c = q % 6;
    double x = 0.0;
    for (int y = 0; y < 6; y++) x += S_s[r * 6 + y] * Wf[y * m + 6 * grp + c];
    if (grp == k)
      zd[(size_t)a * 36 + r * 6 + c] = (float)x;
    else
      ze[(size_t)eidx_s[grp] * 36 + r * 6 + c] = (float)x;
  }
  for (int e = e0 + t; e < e1; e += FS_THREADS) {
    if (src[e] >= a) continue;
    bool kept = false;
    for (int q = 0; q < k; q++) kept |= eidx_s[q] == e;
    if (!kept)
      for (int x = 0; x < 36; x++) ze[(size_t)e * 36 + x] = 0.f;
  }
}

// ------------------------------------------------------------ the network
// Dense layer on rows: y[r] = act(W [seg0(r); seg1(r); seg2(r)] + b), the
// segments gathered from BF16 arrays (width w_s, row index idx_s[r] or r),
// FP32 accumulation; optionally sum[r] = res[r] + y[r].  One warp per row,
// lane o computes outputs o and o + 32 from the transposed weights staged in
// shared memory as FP32.
struct Seg {
  const __nv_bfloat16* p;
  const int* idx;
  int w;
};

struct LayerArgs {
  int rows, kin, kout, act;
  Seg s[3];
  int nseg;
  const __nv_bfloat16* W;  // [kout][kin]
  const float* b;
  __nv_bfloat16* y;        // [rows][kout] (post-activation), may be null
  float* y32;              // FP32 output instead (the heads), may be null
  const __nv_bfloat16* res;
  __nv_bfloat16* sum;      // res + y
  const float* add_eye;    // heads: + identity on 6 x 6 (non-null flag)
};

constexpr int LW = 8;  // warps per CTA

__global__ void __launch_bounds__(32 * LW) lp_layer_fwd(LayerArgs A) {
  extern __shared__ float ls[];
  float* Wt = ls;                       // [kin][kout]
  float* xs = ls + A.kin * A.kout;      // [LW][kin]
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  for (int q = t; q < A.kin * A.kout; q += 32 * LW) {
    const int o = q / A.kin, k = q % A.kin;
    Wt[k * A.kout + o] = __bfloat162float(A.W[q]);
  }
  __syncthreads();
  float* x = xs + warp * A.kin;
  for (int r = blockIdx.x * LW + warp; r < A.rows; r += gridDim.x * LW) {
    int k0 = 0;
    for (int s = 0; s < A.nseg; s++) {
      const int row = A.s[s].idx ? A.s[s].idx[r] : r;
      const __nv_bfloat16* p = A.s[s].p + (size_t)row * A.s[s].w;
      for (int k = lane; k < A.s[s].w; k += 32) x[k0 + k] = __bfloat162float(p[k]);
      k0 += A.s[s].w;
    }
    __syncwarp();
    for (int o = lane; o < A.kout; o += 32) {
      float acc = A.b[o];
      for (int k = 0; k < A.kin; k++) acc = fmaf(Wt[k * A.kout + o], x[k], acc);
      if (A.act) acc = fmaxf(acc, 0.f);
      if (A.add_eye && (o / 6 == o % 6)) acc += 1.f;
      const size_t yo = (size_t)r * A.kout + o;
      const __nv_bfloat16 yb = __float2bfloat16(acc);
      if (A.y) A.y[yo] = yb;
      if (A.y32) A.y32[yo] = acc;
      if (A.sum) A.sum[yo] = __float2bfloat16(__bfloat162float(A.res[yo]) + __bfloat162float(yb));
    }
    __syncwarp();
  }
}

// agg[a] = sum of msg over the edges into a (CSR, fixed order)
__global__ void lp_aggregate(int nn, const int* __restrict__ off, const __nv_bfloat16* __restrict__ msg,
                             __nv_bfloat16* __restrict__ agg) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nn * H) return;
  const int a = t / H, c = t % H;
  float s = 0.f;
  for (int e = off[a]; e < off[a + 1]; e++) s += __bfloat162float(msg[(size_t)e * H + c]);
  agg[t] = __float2bfloat16(s);
}

// Backward of a dense layer over a chunk of LB_ROWS rows per CTA:
//   dz = dy * act'(y) (FP32; y the saved post-activation),
//   dx_s[idx_s(r)] += (W^T dz)[segment s] (FP32 atomics, null to skip),
//   per-CTA partial dW = sum_r dz x^T and db = sum_r dz into part[cta].
constexpr int LB_ROWS = 32;

struct LayerBwdArgs {
  int rows, kin, kout, act;
  Seg s[3];
  int nseg;
  float* dx[3];
  const __nv_bfloat16* W;
  const __nv_bfloat16* y;   // saved activation (relu mask), null for linear
  const float* dy;          // [rows][kout]
  const int* row_mask;      // rows with mask[r] == 0 carry no gradient (null: all)
  float* part;              // [gridDim.x][kout * kin + kout]
};

__global__ void __launch_bounds__(256) lp_layer_bwd(LayerBwdArgs A) {
  extern __shared__ float bs[];
  float* Ws = bs;                          // [kout][kin]
  float* xs = Ws + A.kout * A.kin;         // [LB_ROWS][kin]
  float* dz = xs + LB_ROWS * A.kin;        // [LB_ROWS][kout]
  const int t = threadIdx.x;
  const int r0 = blockIdx.x * LB_ROWS;
  for (int q = t; q < A.kout * A.kin; q += 256) Ws[q] = __bfloat162float(A.W[q]);
  for (int q = t; q < LB_ROWS * A.kout; q += 256) {
    const int rl = q / A.kout, o = q % A.kout, r = r0 + rl;
    float g = 0.f;
    if (r < A.rows && (!A.row_mask || A.row_mask[r])) {
      g = A.dy[(size_t)r * A.kout + o];
      if (A.act && __bfloat162float(A.y[(size_t)r * A.kout + o]) <= 0.f) g = 0.f;
    }
    dz[q] = g;
  }
  for (int q = t; q < LB_ROWS * A.kin; q += 256) {
    const int rl = q / A.kin, k = q % A.kin, r = r0 + rl;
    float v = 0.f;
    if (r < A.rows) {
      int k0 = 0;
      for (int s = 0; s < A.nseg; s++) {
        if (k < k0 + A.s[s].w) {
          const int row = A.s[s].idx ? A.s[s].idx[r] : r;
          v = __bfloat162float(A.s[s].p[(size_t)row * A.s[s].w + (k - k0)]);
          break;
        }
        k0 += A.s[s].w;
      }
    }
    xs[q] = v;
  }
  __syncthreads();
  // input gradients
  for (int q = t; q < LB_ROWS * A.kin; q += 256) {
    const int rl = q / A.kin, k = q % A.kin, r = r0 + rl;
    if (r >= A.rows) continue;
    float s = 0.f;
    for (int o = 0; o < A.kout; o++) s = fmaf(Ws[o * A.kin + k], dz[rl * A.kout + o], s);
    int k0 = 0;
    for (int sg = 0; sg < A.nseg; sg++) {
      if (k < k0 + A.s[sg].w) {
        if (A.dx[sg]) {
          const int row = A.s[sg].idx ? A.s[sg].idx[r] : r;
          atomicAdd(A.dx[sg] + (size_t)row * A.s[sg].w + (k - k0), s);
        }
        break;
      }
      k0 += A.s[sg].w;
    }
  }
  // weight and bias partials of this chunk
  float* p = A.part + (size_t)blockIdx.x * (A.kout * A.kin + A.kout);
  for (int q = t; q < A.kout * A.kin + A.kout; q += 256) {
    float s = 0.f;
    if (q < A.kout * A.kin) {
      const int o = q / A.kin, k = q % A.kin;
      for (int rl = 0; rl < LB_ROWS; rl++) s = fmaf(dz[rl * A.kout + o], xs[rl * A.kin + k], s);
    } else {
      const int o = q - A.kout * A.kin;
      for (int rl = 0; rl < LB_ROWS; rl++) s += dz[rl * A.kout + o];
    }
    p[q] = s;
  }
}

// grad[w_off + q] += sum over CTAs of part (fixed order); bias after weights
__global__ void lp_reduce_parts(int nparts, int nw, int nb, const float* __restrict__ part, float* __restrict__ gw,
                                float* __restrict__ gb) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nw + nb) return;
  float s = 0.f;
  for (int c = 0; c < nparts; c++) s += part[(size_t)c * (nw + nb) + q];
  if (q < nw)
    gw[q] += s;
  else
    gb[q - nw] += s;
}

// dmsg[e] += dagg[dst[e]] (the aggregation's backward)
__global__ void lp_agg_bwd(int ne, const int* __restrict__ dst, const float* __restrict__ dagg,
                           float* __restrict__ dmsg) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ne * H) return;
  dmsg[t] += dagg[(size_t)dst[t / H] * H + t % H];
}

// supervised loss on the directions W of the lower edges kept by the FSAI
// pattern (targets NaN elsewhere; targets beyond 20 in magnitude, from
// nearly singular FP32 local blocks, are left out): L = mean squared error
// over the kept entries; dze its gradient (zero elsewhere)
__global__ void lp_loss(int ne, const float* __restrict__ ze, const float* __restrict__ te,
                        const int* __restrict__ lower, float inv_cnt, float* __restrict__ dze,
                        double* __restrict__ loss) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  double l = 0.0;
  if (u < ne * 36) {
    const float tv = te[u];
    if (lower[u / 36] && isfinite(tv) && fabsf(tv) <= 20.f) {
      const float d = ze[u] - tv;
      dze[u] = 2.f * d * inv_cnt;
      l = (double)d * d * inv_cnt;
    } else {
      dze[u] = 0.f;
    }
  }
  for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
  if ((threadIdx.x & 31) == 0 && l != 0.0) atomicAdd(loss, l);
}

// entries of the targets that enter the loss
__global__ void lp_count_targets(int ne, const float* __restrict__ te, const int* __restrict__ lower,
                                 int* __restrict__ cnt) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  int c = 0;
  if (u < ne * 36) {
    const float tv = te[u];
    c = lower[u / 36] && isfinite(tv) && fabsf(tv) <= 20.f;
  }
  c = __reduce_add_sync(0xffffffffu, c);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(cnt, c);
}

__global__ void lp_lower_flags(int ne, const int* __restrict__ src, const int* __restrict__ dst, int* __restrict__ f) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < ne) f[e] = src[e] < dst[e];
}

// squared Euclidean norm of the gradient, accumulated in FP64
__global__ void lp_gnorm2(int64_t n, const float* __restrict__ g, double* __restrict__ out) {
  double l = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    l += (double)g[i] * g[i];
  for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
  if ((threadIdx.x & 31) == 0 && l != 0.0) atomicAdd(out, l);
}

// Adam (Kingma and Ba, 2015), FP32 master weights; BF16 copies refreshed.
// The gradient is scaled by min(1, clip / |g|) when clip > 0 (global norm
// clipping, Pascanu et al., 2013); a gradient whose norm is not finite makes
// no update.
__global__ void lp_adam(int64_t n, float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                        float* __restrict__ v, __nv_bfloat16* __restrict__ wb, float lr, float b1, float b2, float eps,
                        float c1, float c2, const double* __restrict__ gn2, float clip) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double gn = sqrt(*gn2);
  if (!isfinite(gn)) return;
  const float sc = (clip > 0.f && gn > clip) ? (float)(clip / gn) : 1.f;
  const float gi = g[i] * sc;
  const float mi = b1 * m[i] + (1.f - b1) * gi, vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  w[i] = wi;
  wb[i] = __float2bfloat16(wi);
}

__global__ void lp_to_bf16(int64_t n, const float* __restrict__ w, __nv_bfloat16* __restrict__ wb) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) wb[i] = __float2bfloat16(w[i]);
}

// ------------------------------------------------------------ preconditioner
// y = G v, G = D^-1/2 Z^T Z D^-1/2 (mode FSAI / learned), D^-1 (Jacobi) or I
// t = Z (dinv v): row block a = zd[a] v^_a + sum over lower edges (a <- b) ze[e] v^_b
__global__ void lp_apply_z(int nn, const int* __restrict__ off, const int* __restrict__ src,
                           const float* __restrict__ zd, const float* __restrict__ ze, const double* __restrict__ dinv,
                           const double* __restrict__ v, double* __restrict__ tmp) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 6 * nn) return;
  const int a = t / 6, r = t % 6;
  double s = 0.0;
  for (int c = 0; c < 6; c++) s += (double)zd[(size_t)a * 36 + r * 6 + c] * dinv[6 * a + c] * v[6 * a + c];
  for (int e = off[a]; e < off[a + 1]; e++) {
    const int b = src[e];
    if (b >= a) continue;
    for (int c = 0; c < 6; c++) s += (double)ze[(size_t)e * 36 + r * 6 + c] * dinv[6 * b + c] * v[6 * b + c];
  }
  tmp[t] = s;
}

// y = dinv Z^T t: row block b = zd[b]^T t_b + sum over edges (a <- b), a > b,
// ze[(a <- b)]^T t_a; the edges into b give (b <- a) and rev gives (a <- b)
__global__ void lp_apply_zt(int nn, const int* __restrict__ off, const int* __restrict__ src,
                            const int* __restrict__ rev, const float* __restrict__ zd, const float* __restrict__ ze,
                            const double* __restrict__ dinv, const double* __restrict__ tmp, double* __restrict__ y) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 6 * nn) return;
  const int b = t / 6, c = t % 6;
  double s = 0.0;
  for (int r = 0; r < 6; r++) s += (double)zd[(size_t)b * 36 + r * 6 + c] * tmp[6 * b + r];
  for (int e = off[b]; e < off[b + 1]; e++) {
    const int a = src[e];
    if (a <= b) continue;
    const int f = rev[e];  // (a <- b)
    if (f < 0) continue;
    for (int r = 0; r < 6; r++) s += (double)ze[(size_t)f * 36 + r * 6 + c] * tmp[6 * a + r];
  }
  y[t] = dinv[t] * s;
}

// particle-block layout <-> grand layout of a 6N vector
__global__ void lp_to_blk(int nn, const double* __restrict__ g, double* __restrict__ b) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < 6 * nn) b[t] = g[grand_row(nn, t)];
}
__global__ void lp_from_blk(int nn, const double* __restrict__ b, double* __restrict__ g) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < 6 * nn) g[grand_row(nn, t)] = b[t];
}

__global__ void lp_scale(int n, const double* __restrict__ d, const double* __restrict__ v, double* __restrict__ y) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) y[t] = d[t] * d[t] * v[t];
}

// dot products (one block): out[q] = x_q . y_q for q < nq
__global__ void lp_dots(int n, int nq, const double* __restrict__ x0, const double* __restrict__ y0,
                        const double* __restrict__ x1, const double* __restrict__ y1, double* __restrict__ out) {
  __shared__ double r0[256], r1[256];
  double a = 0.0, b = 0.0;
  for (int i = threadIdx.x; i < n; i += 256) {
    a += x0[i] * y0[i];
    if (nq > 1) b += x1[i] * y1[i];
  }
  r0[threadIdx.x] = a;
  r1[threadIdx.x] = b;
  __syncthreads();
  for (int d = 128; d > 0; d >>= 1) {
    if (threadIdx.x < d) {
      r0[threadIdx.x] += r0[threadIdx.x + d];
      r1[threadIdx.x] += r1[threadIdx.x + d];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = r0[0];
    if (nq > 1) out[1] = r1[0];
  }
}

// CG updates with the scalars on the device: alpha = rz / pq;
// x += alpha p; r -= alpha q
__global__ void lp_cg_xr(int n, const double* __restrict__ sc, const double* __restrict__ p,
                         const double* __restrict__ q, double* __restrict__ x, double* __restrict__ r) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double alpha = sc[0] / sc[1];
  x[i] += alpha * p[i];
  r[i] -= alpha * q[i];
}
// beta = rz_new / rz; p = z + beta p; rz = rz_new
__global__ void lp_cg_p(int n, double* __restrict__ sc, const double* __restrict__ z, double* __restrict__ p) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = z[i] + (sc[2] / sc[0]) * p[i];
}
__global__ void lp_cg_roll(double* sc) { sc[0] = sc[2]; }

inline unsigned nb256(int64_t n) { return (unsigned)((n + 255) / 256); }

// every launch is checked at once: a refused launch leaves its outputs unwritten
#define RSD_LP_CHECK()                                                                  \
  do {                                                                                  \
    cudaError_t _le = cudaGetLastError();                                               \
    if (_le != cudaSuccess) return rsd_cuda_check(ctx, _le, "learned-preconditioner launch"); \
  } while (0)

}  // namespace

// ------------------------------------------------------------------ host
struct lp_graph {
  int nn = 0, ne = 0;
  int *off = nullptr, *src = nullptr, *dst = nullptr, *rev = nullptr, *lower = nullptr;
  float* gap = nullptr;
};

static int lp_build_graph(rsd_ctx* ctx, int nn, const double* d_pos, const double* d_radii, const rsd_lattice* lat,
                          lp_graph* g) {
  cudaStream_t s = ctx->stream;
  rsd_lat_dev L = rsd_lat_pack(lat);
  int* cnt = (int*)rsd_scratch(ctx, "lp_cnt", sizeof(int) * (nn + 1));
  if (!cnt) return RSD_ENOMEM;
  lp_count<<<nn, 256, 0, s>>>(nn, L, d_pos, d_radii, cnt); RSD_LAUNCH_NOTE(); RSD_LP_CHECK();
  std::vector<int> h(nn + 1);
  RSD_CUDA(ctx, cudaMemcpyAsync(h.data(), cnt, sizeof(int) * nn, cudaMemcpyDeviceToHost, s));
  RSD_CUDA(ctx, cudaStreamSynchronize(s));
  std::vector<int> off(nn + 1, 0);
  for (int a = 0; a < nn; a++) off[a + 1] = off[a] + h[a];
  const int ne = off[nn];
  g->nn = nn;
  g->ne = ne;
  g->off = (int*)rsd_scratch(ctx, "lp_off", sizeof(int) * (nn + 1));
  g->src = (int*)rsd_scratch(ctx, "lp_src", sizeof(int) * (ne + 1));
  g->dst = (int*)rsd_scratch(ctx, "lp_dst", sizeof(int) * (ne + 1));
  g->rev = (int*)rsd_scratch(ctx, "lp_rev", sizeof(int) * (ne + 1));
  g->lower = (int*)rsd_scratch(ctx, "lp_lower", sizeof(int) * (ne + 1));
  g->gap = (float*)rsd_scratch(ctx, "lp_gap", sizeof(float) * (ne + 1));
  if (!g->off || !g->src || !g->dst || !g->rev || !g->lower || !g->gap) return RSD_ENOMEM;
  RSD_CUDA(ctx, cudaMemcpyAsync(g->off, off.data(), sizeof(int) * (nn + 1), cudaMemcpyHostToDevice, s));
  if (ne > 0) {
    lp_fill<<<(nn + 7) / 8, 256, 0, s>>>(nn, L, d_pos, d_radii, g->off, g->src, g->dst, g->gap); RSD_LAUNCH_NOTE(); RSD_LP_CHECK();
    lp_rev<<<nb256(ne), 256, 0, s>>>(ne, g->off, g->src, g->dst, g->rev); RSD_LAUNCH_NOTE(); RSD_LP_CHECK();
    lp_lower_flags<<<nb256(ne), 256, 0, s>>>(ne, g->src, g->dst, g->lower); RSD_LAUNCH_NOTE(); RSD_LP_CHECK();
  }
  RSD_CUDA(ctx, cudaStreamSynchronize(s));  // off must outlive the host vector's copy
  RSD_CUDA(ctx, cudaGetLastError());
  return RSD_OK;
}

// Jacobi scaling and (optionally) the network inputs of RPP on the graph
template <typename T>
static int lp_scale_features(rsd_ctx* ctx, const lp_graph& g, const T* A, int64_t ld, double** dinv,
                             __nv_bfloat16** xn, __nv_bfloat16** xe) {
  cudaStream_t s = ctx->stream;
  const int nn = g.nn, ne = g.ne;
  *dinv = (double*)rsd_scratch(ctx, "lp_dinv", sizeof(double) * 6 * nn);
  if (!*dinv) return RSD_ENOMEM;
  int* bad = ctx->d_info + 9;
  RSD_CUDA(ctx, cudaMemsetAsync(bad, 0, sizeof(int), s));
  lp_dinv<T><<<nb256(6 * nn), 256, 0, s>>>(nn, A, ld, *dinv, bad); RSD_LAUNCH_NOTE(); RSD_LP_CHECK();
  if (xn) {
    *xn = (__nv_bfloat16*)rsd_scratch(ctx, "lp_xn", sizeof(__nv_bfloat16) * (size_t)nn * NF_NODE);
    *xe = (__nv_bfloat16*)rsd_scratch(ctx, "lp_xe", sizeof(__nv_bfloat16) * ((size_t)ne * NF_EDGE + 1));
    if (!*xn || !*xe) return RSD_ENOMEM;
    lp_features<T><<<nb256((int64_t)nn * 36 + (int64_t)ne * NF_EDGE), 256, 0, s>>>(nn, ne, A, ld, *dinv, g.src, g.dst,
                                                                                   g.gap, *xn, *xe); RSD_LAUNCH_NOTE(); RSD_LP_CHECK();
  }
  RSD_CUDA(ctx, cudaMemcpyAsync(ctx->h_info + 9, bad, sizeof(int), cudaMemcpyDeviceToHost, s));
  RSD_CUDA(ctx, cudaStreamSynchronize(s));
  if (ctx->h_info[9]) return rsd_fail(ctx, RSD_ENAN, "RPP has a non-positive diagonal entry");
  return RSD_OK;
}

// shared memory of lp_fsai and lp_normalize: the local matrix (m x m) and
// two m x 6 panels, m at most 6 (LP_KMAX + 1)
constexpr size_t LP_LOCAL_SMEM = sizeof(double) * ((size_t)(6 * (LP_KMAX + 1)) * (6 * (LP_KMAX + 1)) +
                                                   2 * (size_t)(6 * (LP_KMAX + 1)) * 6);

template <typename T>
static int lp_exact_fsai(rsd_ctx* ctx, const lp_graph& g, const T* A, int64_t ld, const double* dinv, int self_only,
                         float* zd, float* ze, float* wt = nullptr) {
  cudaStream_t s = ctx->stream;
  static bool attr[2] = {false, false};
  const int which = sizeof(T) == 8;
  if (!attr[which]) {
    RSD_CUDA(ctx, cudaFuncSetAttribute(lp_fsai<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)LP_LOCAL_SMEM));
    attr[which] = true;
  }
  int* bad = ctx->d_info + 10;
  RSD_CUDA(ctx, cudaMemsetAsync(bad, 0, sizeof(int), s));
  lp_fsai<T><<<g.nn, FS_THREADS, LP_LOCAL_SMEM, s>>>(g.nn, self_only, A, ld, dinv, g.off, g.src, g.gap, zd, ze, wt, bad); RSD_LAUNCH_NOTE(); RSD_LP_CHECK();
  RSD_CUDA(ctx, cudaMemcpyAsync(ctx->h_info + 10, bad, sizeof(int), cudaMemcpyDeviceToHost, s));
  RSD_CUDA(ctx, cudaStreamSynchronize(s));
  if (ctx->h_info[10]) return rsd_fail(ctx, RSD_ENAN, "FSAI: a local block of RPP is not positive definite");
  return RSD_OK;
}

// forward pass; activations kept in the context for the backward pass
struct lp_acts {
  __nv_bfloat16 *h[NLAYER + 1], *m[NLAYER + 1], *msg[NLAYER], *agg[NLAYER], *u[NLAYER];
};

static int lp_layer(rsd_ctx* ctx, const LayerArgs& a) {
  if (a.rows <= 0) return RSD_OK;
  const size_t smem = sizeof(float) * ((size_t)a.kin * a.kout + (size_t)LW * a.kin);
  static bool attr = false;
  if (!attr) {
    RSD_CUDA(ctx, cudaFuncSetAttribute(lp_layer_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024));
    attr = true;
  }
  const int grid = (int)std::min<int64_t>((a.rows + LW - 1) / LW, 8LL * (ctx->sm_count > 0 ? ctx->sm_count : 148));
  lp_layer_fwd<<<grid, 32 * LW, smem, ctx->stream>>>(a); RSD_LAUNCH_NOTE(); RSD_LP_CHECK();
  return RSD_OK;
}

static Seg seg(const __nv_bfloat16* p, const int* idx, int w) { return Seg{p, idx, w}; }

static int lp_forward(rsd_ctx* ctx, rsd_lp* net, const lp_graph& g, const __nv_bfloat16* xn,
                      const __nv_bfloat16* xe, lp_acts* A, float* zd, float* ze) {
  const int nn = g.nn, ne = g.ne;
  auto buf = [&](const char* nm, int l, size_t rows) {
    char name[48];
    snprintf(name, sizeof name, "lp_%s%d", nm, l);
    return (__nv_bfloat16*)rsd_scratch(ctx, name, sizeof(__nv_bfloat16) * (rows * H + 1));
  };
  for (int l = 0; l <= NLAYER; l++) {
    A->h[l] = buf("h", l, nn);
    A->m[l] = buf("m", l, ne);
    if (!A->h[l] || !A->m[l]) return RSD_ENOMEM;
  }
  for (int l = 0; l < NLAYER; l++) {
    A->msg[l] = buf("msg", l, ne);
    A->agg[l] = buf("agg", l, nn);
    A->u[l] = buf("u", l, nn);
    if (!A->msg[l] || !A->agg[l] || !A->u[l]) return RSD_ENOMEM;
  }
  const __nv_bfloat16* W = net->wb;
  const float* B = net->w;
  LayerArgs a{};
  // encoders
  a = LayerArgs{nn, NF_NODE, H, 1, {seg(xn, nullptr, NF_NODE)}, 1, W + LAY.enc_n_w, B + LAY.enc_n_b, A->h[0]};
  RSD_TRY(lp_layer(ctx, a));
  a = LayerArgs{ne, NF_EDGE, H, 1, {seg(xe, nullptr, NF_EDGE)}, 1, W + LAY.enc_e_w, B + LAY.enc_e_b, A->m[0]};
  RSD_TRY(lp_layer(ctx, a));
  for (int l = 0; l < NLAYER; l++) {
    a = LayerArgs{ne, 3 * H, H, 1, {seg(A->h[l], g.dst, H), seg(A->h[l], g.src, H), seg(A->m[l], nullptr, H)}, 3,
                  W + LAY.msg_w[l], B + LAY.msg_b[l], A->msg[l]};
    a.res = A->m[l];
    a.sum = A->m[l + 1];
    RSD_TRY(lp_layer(ctx, a));
    lp_aggregate<<<nb256((int64_t)nn * H), 256, 0, ctx->stream>>>(nn, g.off, A->msg[l], A->agg[l]); RSD_LAUNCH_NOTE(); RSD_LP_CHECK();
    a = LayerArgs{nn, 2 * H, H, 1, {seg(A->h[l], nullptr, H), seg(A->agg[l], nullptr, H)}, 2, W + LAY.upd_w[l],
                  B + LAY.upd_b[l], A->u[l]};
    a.res = A->h[l];
    a.sum = A->h[l + 1];
    RSD_TRY(lp_layer(ctx, a));
  }
  // heads: Z_aa = I + W h_a + b; Z_ab from [m_ab; h_a; h_b]
  static const float one = 1.f;
  a = LayerArgs{nn, H, NOUT, 0, {seg(A->h[NLAYER], nullptr, H)}, 1, W + LAY.head_n_w, B + LAY.head_n_b, nullptr, zd};
  a.add_eye = &one;
  RSD_TRY(lp_layer(ctx, a));
  a = LayerArgs{ne, 3 * H, NOUT, 0,
                {seg(A->m[NLAYER], nullptr, H), seg(A->h[NLAYER], g.dst, H), seg(A->h[NLAYER], g.src, H)}, 3,
                W + LAY.head_e_w, B + LAY.head_e_b, nullptr, ze};
  RSD_TRY(lp_layer(ctx, a));
  RSD_CUDA(ctx, cudaGetLastError());
  return RSD_OK;
}

static int lp_layer_back(rsd_ctx* ctx, rsd_lp* net, LayerBwdArgs b, int64_t w_off, int64_t b_off) {
  if (b.rows <= 0) return RSD_OK;
  const int nparts = (b.rows + LB_ROWS - 1) / LB_ROWS;
  const int nw = b.kout * b.kin;
  float* part = (float*)rsd_scratch(ctx, "lp_part", sizeof(float) * (size_t)nparts * (nw + b.kout));
  if (!part) return RSD_ENOMEM;
  b.part = part;
  const size_t smem = sizeof(float) * ((size_t)b.kout * b.kin + (size_t)LB_ROWS * b.kin + (size_t)LB_ROWS * b.kout);
  static bool attr = false;
  if (!attr) {
    RSD_CUDA(ctx, cudaFuncSetAttribute(lp_layer_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024));
    attr = true;
  }
  lp_layer_bwd<<<nparts, 256, smem, ctx->stream>>>(b); RSD_LAUNCH_NOTE(); RSD_LP_CHECK();
  lp_reduce_parts<<<nb256(nw + b.kout), 256, 0, ctx->stream>>>(nparts, nw, b.kout, part, net->g + w_off,
                                                                net->g + b_off); RSD_LAUNCH_NOTE(); RSD_LP_CHECK();
  return RSD_OK;
}

// gradient of the parameters (added into net->g, zeroed here first) from
// dzd (nn x 36) and dze (ne x 36), through the saved activations
static int lp_backward(rsd_ctx* ctx, rsd_lp* net, const lp_graph& g, const __nv_bfloat16* xn,
                       const __nv_bfloat16* xe, const lp_acts& A, const float* dzd, const float* dze) {
  cudaStream_t s = ctx->stream;
  const int nn = g.nn, ne = g.ne;
  RSD_CUDA(ctx, cudaMemsetAsync(net->g, 0, sizeof(float) * LAY.total, s));
  float* dh = (float*)rsd_scratch(ctx, "lp_dh", sizeof(float) * ((size_t)nn * H + 1));
  float* dh2 = (float*)rsd_scratch(ctx, "lp_dh2", sizeof(float) * ((size_t)nn * H + 1));
  float* dm = (float*)rsd_scratch(ctx, "lp_dm", sizeof(float) * ((size_t)ne * H + 1));
  float* dm2 = (float*)rsd_scratch(ctx, "lp_dm2", sizeof(float) * ((size_t)ne * H + 1));
  float* dagg = (float*)rsd_scratch(ctx, "lp_dagg", sizeof(float) * ((size_t)nn * H + 1));
  float* dmsg = (float*)rsd_scratch(ctx, "lp_dmsg", sizeof(float) * ((size_t)ne * H + 1));
  if (!dh || !dh2 || !dm || !dm2 || !dagg || !dmsg) return RSD_ENOMEM;
  const __nv_bfloat16* W = net->wb;
  RSD_CUDA(ctx, cudaMemsetAsync(dh, 0, sizeof(float) * (size_t)nn * H, s));
  RSD_CUDA(ctx, cudaMemsetAsync(dm, 0, sizeof(float) * (size_t)ne * H, s));
  LayerBwdArgs b{};
  // heads (linear)
  b = LayerBwdArgs{nn, H, NOUT, 0, {seg(A.h[NLAYER], nullptr, H)}, 1, {dh}, W + LAY.head_n_w, nullptr, dzd};
  RSD_TRY(lp_layer_back(ctx, net, b, LAY.head_n_w, LAY.head_n_b));
  b = LayerBwdArgs{ne, 3 * H, NOUT, 0,
                   {seg(A.m[NLAYER], nullptr, H), seg(A.h[NLAYER], g.dst, H), seg(A.h[NLAYER], g.src, H)}, 3,
                   {dm, dh, dh}, W + LAY.head_e_w, nullptr, dze, g.lower};
  RSD_TRY(lp_layer_back(ctx, net, b, LAY.head_e_w, LAY.head_e_b));
  for (int l = NLAYER - 1; l >= 0; l--) {
    // h[l+1] = h[l] + u[l]: dh flows to h[l] unchanged (dh2 = dh) and into u[l]
    RSD_CUDA(ctx, cudaMemcpyAsync(dh2, dh, sizeof(float) * (size_t)nn * H, cudaMemcpyDeviceToDevice, s));
    RSD_CUDA(ctx, cudaMemsetAsync(dagg, 0, sizeof(float) * (size_t)nn * H, s));
    b = LayerBwdArgs{nn, 2 * H, H, 1, {seg(A.h[l], nullptr, H), seg(A.agg[l], nullptr, H)}, 2, {dh2, dagg},
                     W + LAY.upd_w[l], A.u[l], dh};
    RSD_TRY(lp_layer_back(ctx, net, b, LAY.upd_w[l], LAY.upd_b[l]));
    // m[l+1] = m[l] + msg[l]: dmsg = dm + dagg[dst]; dm flows to m[l]
    RSD_CUDA(ctx, cudaMemcpyAsync(dmsg, dm, sizeof(float) * (size_t)ne * H, cudaMemcpyDeviceToDevice, s));
    if (ne > 0) {
      lp_agg_bwd<<<nb256((int64_t)ne * H), 256, 0, s>>>(ne, g.dst, dagg, dmsg); RSD_LAUNCH_NOTE(); RSD_LP_CHECK();
    }
    RSD_CUDA(ctx, cudaMemcpyAsync(dm2, dm, sizeof(float) * (size_t)ne * H, cudaMemcpyDeviceToDevice, s));
    b = LayerBwdArgs{ne, 3 * H, H, 1, {seg(A.h[l], g.dst, H), seg(A.h[l], g.src, H), seg(A.m[l], nullptr, H)}, 3,
                     {dh2, dh2, dm2}, W + LAY.msg_w[l], A.msg[l], dmsg};
    RSD_TRY(lp_layer_back(ctx, net, b, LAY.msg_w[l], LAY.msg_b[l]));
    std::swap(dh, dh2);
    std::swap(dm, dm2);
  }
  // encoders: weight gradients only
  b = LayerBwdArgs{nn, NF_NODE, H, 1, {seg(xn, nullptr, NF_NODE)}, 1, {nullptr}, W + LAY.enc_n_w, A.h[0], dh};
  RSD_TRY(lp_layer_back(ctx, net, b, LAY.enc_n_w, LAY.enc_n_b));
  b = LayerBwdArgs{ne, NF_EDGE, H, 1, {seg(xe, nullptr, NF_EDGE)}, 1, {nullptr}, W + LAY.enc_e_w, A.m[0], dm};
  RSD_TRY(lp_layer_back(ctx, net, b, LAY.enc_e_w, LAY.enc_e_b));
  RSD_CUDA(ctx, cudaGetLastError());
  return RSD_OK;
}

// the blocks of Z for `mode` on the graph: FSAI (exact), block-Jacobi (FSAI
// on the diagonal pattern) or learned
template <typename T>
static int lp_make_z(rsd_ctx* ctx, rsd_lp* net, int mode, const lp_graph& g, const T* A, int64_t ld, double** dinv,
                     float** zd, float** ze) {
  *zd = (float*)rsd_scratch(ctx, "lp_zd", sizeof(float) * (size_t)g.nn * 36);
  *ze = (float*)rsd_scratch(ctx, "lp_ze", sizeof(float) * ((size_t)g.ne * 36 + 1));
  if (!*zd || !*ze) return RSD_ENOMEM;
  if (mode == RSD_PC_LEARNED) {
    // the network emits the directions W of the lower edges; lp_normalize
    // turns them into the factor Z (SPD G whatever W is)
    if (!net) return rsd_fail(ctx, RSD_EARG, "learned preconditioner: no network");
    __nv_bfloat16 *xn, *xe;
    RSD_TRY(lp_scale_features<T>(ctx, g, A, ld, dinv, &xn, &xe));
    float* hd = (float*)rsd_scratch(ctx, "lp_head_d", sizeof(float) * (size_t)g.nn * 36);
    float* wp = (float*)rsd_scratch(ctx, "lp_wpred", sizeof(float) * ((size_t)g.ne * 36 + 1));
    if (!hd || !wp) return RSD_ENOMEM;
    lp_acts acts;
    RSD_TRY(lp_forward(ctx, net, g, xn, xe, &acts, hd, wp));
    static bool attr[2] = {false, false};
    const int which = sizeof(T) == 8;
    if (!attr[which]) {
      RSD_CUDA(ctx, cudaFuncSetAttribute(lp_normalize<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)LP_LOCAL_SMEM));
      attr[which] = true;
    }
    lp_normalize<T><<<g.nn, FS_THREADS, LP_LOCAL_SMEM, ctx->stream>>>(g.nn, A, ld, *dinv, g.off, g.src, g.gap, wp,
                                                                      *zd, *ze); RSD_LAUNCH_NOTE(); RSD_LP_CHECK();
    return RSD_OK;
  }
  RSD_TRY(lp_scale_features<T>(ctx, g, A, ld, dinv, nullptr, nullptr));
  if (mode == RSD_PC_FSAI || mode == RSD_PC_BLOCK_JACOBI)
    return lp_exact_fsai<T>(ctx, g, A, ld, *dinv, mode == RSD_PC_BLOCK_JACOBI, *zd, *ze);
  return RSD_OK;
}

// PCG on RPP (FP64, full symmetric storage in the grand layout, ld ld) for
// nrhs right-hand sides (columns of b and x, length 6N in the grand layout);
// the worst relative residual and the largest iteration count are returned.
static int lp_pcg(rsd_ctx* ctx, int mode, const lp_graph& g, const double* A, int64_t ld, const double* dinv,
                  const float* zd, const float* ze, int nrhs, const double* b, double* x, double tol, int maxit,
                  int* iters, double* resid) {
  cudaStream_t s = ctx->stream;
  const int nn = g.nn, P = 6 * nn;
  double* V = (double*)rsd_scratch(ctx, "lp_pcg", sizeof(double) * (6 * (size_t)P + 16));
  if (!V) return RSD_ENOMEM;
  double *r = V, *z = r + P, *p = z + P, *q = p + P, *tmp = q + P, *rb = tmp + P, *sc = rb + P;
  int worst_it = 0;
  double worst_res = 0.0;
  auto precond = [&](const double* in, double* out) -> int {
    if (mode == RSD_PC_NONE) {
      RSD_CUDA(ctx, cudaMemcpyAsync(out, in, sizeof(double) * P, cudaMemcpyDeviceToDevice, s));
    } else if (mode == RSD_PC_JACOBI) {
      lp_scale<<<nb256(P), 256, 0, s>>>(P, dinv, in, out); RSD_LAUNCH_NOTE(); RSD_LP_CHECK();
    } else {
      lp_apply_z<<<nb256(P), 256, 0, s>>>(nn, g.off, g.src, zd, ze, dinv, in, tmp); RSD_LAUNCH_NOTE(); RSD_LP_CHECK();
      lp_apply_zt<<<nb256(P), 256, 0, s>>>(nn, g.off, g.src, g.rev, zd, ze, dinv, tmp, out); RSD_LAUNCH_NOTE(); RSD_LP_CHECK();
    }
    return RSD_OK;
  };
  // the operator in the particle-block layout: q = P A P^T p
  auto matvec = [&](const double* in, double* out) -> int {
    lp_from_blk<<<nb256(P), 256, 0, s>>>(nn, in, tmp); RSD_LAUNCH_NOTE(); RSD_LP_CHECK();
    RSD_TRY(rsd_gemv<double>(ctx, 0, P, P, 1.0, A, ld, tmp, P, 1, 0.0, rb, P));
    lp_to_blk<<<nb256(P), 256, 0, s>>>(nn, rb, out); RSD_LAUNCH_NOTE(); RSD_LP_CHECK();
    return RSD_OK;
  };
  double h[4];
  for (int c = 0; c < nrhs; c++) {
    double* xc = x + (size_t)c * P;
    // r = b (block layout), x = 0
    lp_to_blk<<<nb256(P), 256, 0, s>>>(nn, b + (size_t)c * P, r); RSD_LAUNCH_NOTE(); RSD_LP_CHECK();
    RSD_CUDA(ctx, cudaMemsetAsync(xc, 0, sizeof(double) * P, s));
    RSD_TRY(precond(r, z));
    RSD_CUDA(ctx, cudaMemcpyAsync(p, z, sizeof(double) * P, cudaMemcpyDeviceToDevice, s));
    lp_dots<<<1, 256, 0, s>>>(P, 2, r, z, r, r, sc); RSD_LAUNCH_NOTE(); RSD_LP_CHECK();  // sc[0] = rz, sc[1] = rr
    RSD_CUDA(ctx, cudaMemcpyAsync(h, sc, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
    RSD_CUDA(ctx, cudaStreamSynchronize(s));
    const double bn = sqrt(h[1]) > 0 ? sqrt(h[1]) : 1.0;
    double rn = sqrt(h[1]);
    int it = 0;
    while (rn > tol * bn && it < maxit) {
      RSD_TRY(matvec(p, q));
      lp_dots<<<1, 256, 0, s>>>(P, 1, p, q, p, q, sc + 1); RSD_LAUNCH_NOTE(); RSD_LP_CHECK();  // sc[1] = pq
      lp_cg_xr<<<nb256(P), 256, 0, s>>>(P, sc, p, q, xc, r); RSD_LAUNCH_NOTE(); RSD_LP_CHECK();
      RSD_TRY(precond(r, z));
      lp_dots<<<1, 256, 0, s>>>(P, 2, r, z, r, r, sc + 2); RSD_LAUNCH_NOTE(); RSD_LP_CHECK();  // sc[2] = rz', sc[3] = rr
      lp_cg_p<<<nb256(P), 256, 0, s>>>(P, sc, z, p); RSD_LAUNCH_NOTE(); RSD_LP_CHECK();
      lp_cg_roll<<<1, 1, 0, s>>>(sc); RSD_LAUNCH_NOTE(); RSD_LP_CHECK();
      RSD_CUDA(ctx, cudaMemcpyAsync(h, sc + 3, sizeof(double), cudaMemcpyDeviceToHost, s));
      RSD_CUDA(ctx, cudaStreamSynchronize(s));
      rn = sqrt(h[0]);
      it++;
      if (!std::isfinite(rn)) return rsd_fail(ctx, RSD_ENAN, "PCG residual is not finite");
    }
    // x back to the grand layout, in place through tmp
    lp_from_blk<<<nb256(P), 256, 0, s>>>(nn, xc, tmp); RSD_LAUNCH_NOTE(); RSD_LP_CHECK();
    RSD_CUDA(ctx, cudaMemcpyAsync(xc, tmp, sizeof(double) * P, cudaMemcpyDeviceToDevice, s));
    worst_it = std::max(worst_it, it);
    worst_res = std::max(worst_res, rn / bn);
  }
  if (iters) *iters = worst_it;
  if (resid) *resid = worst_res;
  RSD_CUDA(ctx, cudaGetLastError());
  return RSD_OK;
}

// ------------------------------------------------------------------ C-ABI
extern "C" int64_t rsd_lp_param_count(void) { return LAY.total; }

extern "C" int rsd_lp_create(rsd_lp** out, int device, const float* params, uint64_t seed) {
  if (!out) return RSD_EARG;
  *out = nullptr;
  if (cudaSetDevice(device) != cudaSuccess) return RSD_ECUDA;
  rsd_lp* n = new rsd_lp();
  n->device = device;
  const size_t bytes = sizeof(float) * LAY.total;
  cudaError_t e = cudaMalloc(&n->w, bytes);
  if (e == cudaSuccess) e = cudaMalloc(&n->g, bytes);
  if (e == cudaSuccess) e = cudaMalloc(&n->m, bytes);
  if (e == cudaSuccess) e = cudaMalloc(&n->v, bytes);
  if (e == cudaSuccess) e = cudaMalloc(&n->wb, sizeof(__nv_bfloat16) * LAY.total);
  if (e == cudaSuccess) e = cudaMalloc(&n->gn2, sizeof(double));
  std::vector<float> h(LAY.total, 0.f);
  if (params) {
    memcpy(h.data(), params, bytes);
  } else {
    // He-style uniform initialisation of the weight matrices (splitmix64
    // stream from the seed), zero biases, zero heads (Z starts at I)
    uint64_t st = seed;
    auto next = [&]() {
      st += 0x9E3779B97F4A7C15ull;
      uint64_t z = st;
      z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
      z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
      return (double)((z ^ (z >> 31)) >> 11) * (1.0 / 9007199254740992.0);
    };
    auto fill = [&](int64_t off, int fan_out, int fan_in) {
      const double lim = sqrt(6.0 / fan_in);
      for (int64_t i = 0; i < (int64_t)fan_out * fan_in; i++) h[off + i] = (float)((2.0 * next() - 1.0) * lim);
    };
    fill(LAY.enc_n_w, H, NF_NODE);
    fill(LAY.enc_e_w, H, NF_EDGE);
    for (int l = 0; l < NLAYER; l++) {
      fill(LAY.msg_w[l], H, 3 * H);
      fill(LAY.upd_w[l], H, 2 * H);
    }
  }
  if (e == cudaSuccess) e = cudaMemcpy(n->w, h.data(), bytes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(n->m, 0, bytes);
  if (e == cudaSuccess) e = cudaMemset(n->v, 0, bytes);
  if (e == cudaSuccess) e = cudaMemset(n->g, 0, bytes);
  if (e == cudaSuccess) {
    lp_to_bf16<<<nb256(LAY.total), 256>>>(LAY.total, n->w, n->wb);
    RSD_LAUNCH_NOTE();
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    cudaFree(n->w);
    cudaFree(n->g);
    cudaFree(n->m);
    cudaFree(n->v);
    cudaFree(n->wb);
    cudaFree(n->gn2);
    delete n;
    return RSD_ECUDA;
  }
  *out = n;
  return RSD_OK;
}

extern "C" int rsd_lp_destroy(rsd_lp* n) {
  if (!n) return RSD_OK;
  cudaSetDevice(n->device);
  cudaFree(n->w);
  cudaFree(n->g);
  cudaFree(n->m);
  cudaFree(n->v);
  cudaFree(n->wb);
  cudaFree(n->gn2);
  delete n;
  return RSD_OK;
}

extern "C" int rsd_lp_set_training(rsd_lp* n, float clip_norm, double max_loss) {
  if (!n || !(clip_norm >= 0.f) || !(max_loss >= 0.0)) return RSD_EARG;
  n->clip = clip_norm;
  n->max_loss = max_loss;
  return RSD_OK;
}

extern "C" int rsd_lp_training_stats(rsd_lp* n, double* last_grad_norm, int64_t* skipped, int64_t* steps) {
  if (!n) return RSD_EARG;
  if (last_grad_norm) *last_grad_norm = n->last_gnorm;
  if (skipped) *skipped = n->skipped;
  if (steps) *steps = n->step;
  return RSD_OK;
}

extern "C" int rsd_lp_get_params(rsd_lp* n, float* params, float* grad) {
  if (!n || (!params && !grad)) return RSD_EARG;
  if (cudaSetDevice(n->device) != cudaSuccess) return RSD_ECUDA;
  if (params && cudaMemcpy(params, n->w, sizeof(float) * LAY.total, cudaMemcpyDeviceToHost) != cudaSuccess)
    return RSD_ECUDA;
  if (grad && cudaMemcpy(grad, n->g, sizeof(float) * LAY.total, cudaMemcpyDeviceToHost) != cudaSuccess)
    return RSD_ECUDA;
  return RSD_OK;
}

extern "C" int rsd_lp_graph_dev(rsd_ctx* ctx, int32_t nn, const double* d_pos, const double* d_radii,
                                const rsd_lattice* lat, int32_t* n_edges, int32_t* h_off, int32_t* h_src,
                                float* h_gap) {
  if (!ctx || nn < 1 || !d_pos || !d_radii || !lat || !n_edges) return rsd_fail(ctx, RSD_EARG, "lp graph: bad arguments");
  RSD_TRY(rsd_set_device(ctx));
  lp_graph g;
  RSD_TRY(lp_build_graph(ctx, nn, d_pos, d_radii, lat, &g));
  *n_edges = g.ne;
  cudaStream_t s = ctx->stream;
  if (h_off) RSD_CUDA(ctx, cudaMemcpyAsync(h_off, g.off, sizeof(int) * (nn + 1), cudaMemcpyDeviceToHost, s));
  if (h_src && g.ne) RSD_CUDA(ctx, cudaMemcpyAsync(h_src, g.src, sizeof(int) * g.ne, cudaMemcpyDeviceToHost, s));
  if (h_gap && g.ne) RSD_CUDA(ctx, cudaMemcpyAsync(h_gap, g.gap, sizeof(float) * g.ne, cudaMemcpyDeviceToHost, s));
  RSD_CUDA(ctx, cudaStreamSynchronize(s));
  return RSD_OK;
}

// network forward/backward on a given graph and inputs (device pointers):
// the BF16 kernels on their own, for tests against a reference
extern "C" int rsd_lp_forward_dev(rsd_ctx* ctx, rsd_lp* net, int32_t nn, int32_t ne, const int32_t* d_off,
                                  const int32_t* d_src, const int32_t* d_dst, const float* d_xn, const float* d_xe,
                                  const float* d_dzd, const float* d_dze, float* d_zd, float* d_ze) {
  if (!ctx || !net || nn < 1 || ne < 0 || !d_off || !d_xn || !d_zd || !d_ze || (ne > 0 && (!d_src || !d_dst || !d_xe)))
    return rsd_fail(ctx, RSD_EARG, "lp forward: bad arguments");
  RSD_TRY(rsd_set_device(ctx));
  cudaStream_t s = ctx->stream;
  lp_graph g;
  g.nn = nn;
  g.ne = ne;
  g.off = const_cast<int*>(d_off);
  g.src = const_cast<int*>(d_src);
  g.dst = const_cast<int*>(d_dst);
  g.lower = (int*)rsd_scratch(ctx, "lp_lower_t", sizeof(int) * (ne + 1));
  __nv_bfloat16* xn = (__nv_bfloat16*)rsd_scratch(ctx, "lp_xn_t", sizeof(__nv_bfloat16) * (size_t)nn * NF_NODE);
  __nv_bfloat16* xe = (__nv_bfloat16*)rsd_scratch(ctx, "lp_xe_t", sizeof(__nv_bfloat16) * ((size_t)ne * NF_EDGE + 1));
  if (!g.lower || !xn || !xe) return RSD_ENOMEM;
  if (ne) {
    lp_lower_flags<<<nb256(ne), 256, 0, s>>>(ne, g.src, g.dst, g.lower); RSD_LAUNCH_NOTE(); RSD_LP_CHECK();
  }
  lp_to_bf16<<<nb256((int64_t)nn * NF_NODE), 256, 0, s>>>((int64_t)nn * NF_NODE, d_xn, xn); RSD_LAUNCH_NOTE(); RSD_LP_CHECK();
  if (ne) {
    lp_to_bf16<<<nb256((int64_t)ne * NF_EDGE), 256, 0, s>>>((int64_t)ne * NF_EDGE, d_xe, xe); RSD_LAUNCH_NOTE(); RSD_LP_CHECK();
  }
  lp_acts acts;
  RSD_TRY(lp_forward(ctx, net, g, xn, xe, &acts, d_zd, d_ze));
  if (d_dzd && d_dze) RSD_TRY(lp_backward(ctx, net, g, xn, xe, acts, d_dzd, d_dze));
  RSD_CUDA(ctx, cudaStreamSynchronize(s));
  return RSD_OK;
}

extern "C" int rsd_lp_adam_step(rsd_lp* net, float lr) {
  if (!net || !(lr > 0)) return RSD_EARG;
  if (cudaSetDevice(net->device) != cudaSuccess) return RSD_ECUDA;
  if (cudaMemset(net->gn2, 0, sizeof(double)) != cudaSuccess) return RSD_ECUDA;
  lp_gnorm2<<<4 * 152, 256>>>(LAY.total, net->g, net->gn2);
  RSD_LAUNCH_NOTE();
  double gn2 = 0.0;
  if (cudaGetLastError() != cudaSuccess ||
      cudaMemcpy(&gn2, net->gn2, sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
    return RSD_ECUDA;
  net->last_gnorm = sqrt(gn2);
  if (!std::isfinite(net->last_gnorm)) {
    net->skipped++;
    return RSD_OK;
  }
  net->step++;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - powf(b1, (float)net->step), c2 = 1.f - powf(b2, (float)net->step);
  lp_adam<<<nb256(LAY.total), 256>>>(LAY.total, net->w, net->g, net->m, net->v, net->wb, lr, b1, b2, 1e-8f, c1, c2,
                                     net->gn2, net->clip);
  RSD_LAUNCH_NOTE();
  if (cudaGetLastError() != cudaSuccess) return RSD_ECUDA;
  return cudaDeviceSynchronize() == cudaSuccess ? RSD_OK : RSD_ECUDA;
}

template <typename T>
static int lp_train_t(rsd_ctx* ctx, rsd_lp* net, int nn, const double* d_pos, const double* d_radii,
                      const rsd_lattice* lat, const T* A, int64_t ld, float lr, double* loss) {
  cudaStream_t s = ctx->stream;
  lp_graph g;
  RSD_TRY(lp_build_graph(ctx, nn, d_pos, d_radii, lat, &g));
  double* dinv;
  __nv_bfloat16 *xn, *xe;
  RSD_TRY(lp_scale_features<T>(ctx, g, A, ld, &dinv, &xn, &xe));
  // targets: the directions W of this matrix's exact FSAI (its Z blocks go
  // to td / tz, unused here)
  float* td = (float*)rsd_scratch(ctx, "lp_td", sizeof(float) * (size_t)nn * 36);
  float* tz = (float*)rsd_scratch(ctx, "lp_tz", sizeof(float) * ((size_t)g.ne * 36 + 1));
  float* te = (float*)rsd_scratch(ctx, "lp_te", sizeof(float) * ((size_t)g.ne * 36 + 1));
  int* cnt = (int*)rsd_scratch(ctx, "lp_tcount", sizeof(int));
  float* zd = (float*)rsd_scratch(ctx, "lp_zd", sizeof(float) * (size_t)nn * 36);
  float* ze = (float*)rsd_scratch(ctx, "lp_ze", sizeof(float) * ((size_t)g.ne * 36 + 1));
  float* dzd = (float*)rsd_scratch(ctx, "lp_dzd", sizeof(float) * (size_t)nn * 36);
  float* dze = (float*)rsd_scratch(ctx, "lp_dze", sizeof(float) * ((size_t)g.ne * 36 + 1));
  double* dl = (double*)rsd_scratch(ctx, "lp_loss", sizeof(double));
  if (!td || !tz || !te || !cnt || !zd || !ze || !dzd || !dze || !dl) return RSD_ENOMEM;
  if (g.ne == 0) {
    *loss = 0.0;
    return RSD_OK;
  }
  RSD_TRY(lp_exact_fsai<T>(ctx, g, A, ld, dinv, 0, td, tz, te));
  lp_acts acts;
  RSD_TRY(lp_forward(ctx, net, g, xn, xe, &acts, zd, ze));
  int hcnt = 0;
  RSD_CUDA(ctx, cudaMemsetAsync(cnt, 0, sizeof(int), s));
  lp_count_targets<<<nb256((int64_t)g.ne * 36), 256, 0, s>>>(g.ne, te, g.lower, cnt); RSD_LAUNCH_NOTE(); RSD_LP_CHECK();
  RSD_CUDA(ctx, cudaMemcpyAsync(&hcnt, cnt, sizeof(int), cudaMemcpyDeviceToHost, s));
  RSD_CUDA(ctx, cudaStreamSynchronize(s));
  RSD_CUDA(ctx, cudaMemsetAsync(dl, 0, sizeof(double), s));
  RSD_CUDA(ctx, cudaMemsetAsync(dzd, 0, sizeof(float) * (size_t)nn * 36, s));  // the node head is not trained
  lp_loss<<<nb256((int64_t)g.ne * 36), 256, 0, s>>>(g.ne, ze, te, g.lower, hcnt ? 1.f / hcnt : 0.f, dze, dl); RSD_LAUNCH_NOTE(); RSD_LP_CHECK();
  RSD_TRY(lp_backward(ctx, net, g, xn, xe, acts, dzd, dze));
  RSD_CUDA(ctx, cudaMemcpyAsync(loss, dl, sizeof(double), cudaMemcpyDeviceToHost, s));
  RSD_CUDA(ctx, cudaStreamSynchronize(s));
  if (!std::isfinite(*loss) || (net->max_loss > 0.0 && *loss > net->max_loss)) {  // an outlier: no update
    net->skipped++;
    return RSD_OK;
  }
  return rsd_lp_adam_step(net, lr);
}

extern "C" int rsd_lp_train_step(rsd_ctx* ctx, rsd_lp* net, int32_t nn, const double* d_pos, const double* d_radii,
                                 const rsd_lattice* lat, int32_t fp32, const void* d_rpp, int64_t ld, float lr,
                                 double* loss) {
  if (!ctx || !net || nn < 1 || !d_pos || !d_radii || !lat || !d_rpp || ld < 6LL * nn || !loss)
    return rsd_fail(ctx, RSD_EARG, "lp train: bad arguments");
  RSD_TRY(rsd_set_device(ctx));
  if (fp32) return lp_train_t<float>(ctx, net, nn, d_pos, d_radii, lat, (const float*)d_rpp, ld, lr, loss);
  return lp_train_t<double>(ctx, net, nn, d_pos, d_radii, lat, (const double*)d_rpp, ld, lr, loss);
}

// the blocks of Z (nn x 36 diagonal, ne x 36 edge) for `mode`, copied to the host
extern "C" int rsd_lp_blocks_dev(rsd_ctx* ctx, rsd_lp* net, int32_t mode, int32_t nn, const double* d_pos,
                                 const double* d_radii, const rsd_lattice* lat, int32_t fp32, const void* d_rpp,
                                 int64_t ld, float* h_zd, float* h_ze, int32_t* n_edges) {
  if (!ctx || nn < 1 || !d_pos || !d_radii || !lat || !d_rpp || !h_zd || !n_edges ||
      (mode != RSD_PC_BLOCK_JACOBI && mode != RSD_PC_FSAI && mode != RSD_PC_LEARNED))
    return rsd_fail(ctx, RSD_EARG, "lp blocks: bad arguments");
  RSD_TRY(rsd_set_device(ctx));
  lp_graph g;
  RSD_TRY(lp_build_graph(ctx, nn, d_pos, d_radii, lat, &g));
  double* dinv;
  float *zd, *ze;
  if (fp32)
    RSD_TRY(lp_make_z<float>(ctx, net, mode, g, (const float*)d_rpp, ld, &dinv, &zd, &ze));
  else
    RSD_TRY(lp_make_z<double>(ctx, net, mode, g, (const double*)d_rpp, ld, &dinv, &zd, &ze));
  *n_edges = g.ne;
  cudaStream_t s = ctx->stream;
  RSD_CUDA(ctx, cudaMemcpyAsync(h_zd, zd, sizeof(float) * (size_t)nn * 36, cudaMemcpyDeviceToHost, s));
  if (h_ze && g.ne) RSD_CUDA(ctx, cudaMemcpyAsync(h_ze, ze, sizeof(float) * (size_t)g.ne * 36, cudaMemcpyDeviceToHost, s));
  RSD_CUDA(ctx, cudaStreamSynchronize(s));
  return RSD_OK;
}

int rsd_lp_pcg_internal(rsd_ctx* ctx, rsd_lp* net, int mode, int nn, const double* d_pos, const double* d_radii,
                        const rsd_lattice* lat, const double* d_rpp, int64_t ld, int nrhs, const double* d_b,
                        double* d_x, double tol, int maxit, int* iters, double* resid) {
  lp_graph g;
  RSD_TRY(lp_build_graph(ctx, nn, d_pos, d_radii, lat, &g));
  double* dinv;
  float *zd = nullptr, *ze = nullptr;
  RSD_TRY(lp_make_z<double>(ctx, net, mode, g, d_rpp, ld, &dinv, &zd, &ze));
  return lp_pcg(ctx, mode, g, d_rpp, ld, dinv, zd, ze, nrhs, d_b, d_x, tol, maxit, iters, resid);
}

extern "C" int rsd_lp_pcg_dev(rsd_ctx* ctx, rsd_lp* net, int32_t mode, int32_t nn, const double* d_pos,
                              const double* d_radii, const rsd_lattice* lat, const double* d_rpp, int64_t ld,
                              int32_t nrhs, const double* d_b, double* d_x, double tol, int32_t maxit, int32_t* iters,
                              double* resid) {
  if (!ctx || nn < 1 || !d_pos || !d_radii || !lat || !d_rpp || ld < 6LL * nn || nrhs < 1 || !d_b || !d_x ||
      !(tol > 0) || maxit < 1 || mode < RSD_PC_NONE || mode > RSD_PC_LEARNED)
    return rsd_fail(ctx, RSD_EARG, "lp pcg: bad arguments");
  RSD_TRY(rsd_set_device(ctx));
  int it = 0;
  double res = 0.0;
  RSD_TRY(rsd_lp_pcg_internal(ctx, net, mode, nn, d_pos, d_radii, lat, d_rpp, ld, nrhs, d_b, d_x, tol, maxit, &it,
                              &res));
  if (iters) *iters = it;
  if (resid) *resid = res;
  return RSD_OK;
}
