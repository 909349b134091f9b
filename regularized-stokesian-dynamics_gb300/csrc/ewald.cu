// Kernel 1: Ewald-summed periodic grand mobility (PER_GRPERY_INV_FRI,
// src/per_GRPY_YZD.f90:13-200, with PER_ROTNE_PRAGER_SELF/IJ of
// src/Ewald_summation.f90:19-423).
//
// Layout: the grand mobility M (11N x 11N, column-major, leading dimension
// ldm) in the reference's order: rows/cols 3a..3a+2 translation of particle
// a, 3N+3a.. rotation, 6N+5a.. stresslet (Y2 basis).
//
// Work split (thread per unordered pair a < b):
//   ewald_ktable      per reciprocal vector k (half space k > 0): the
//                     radius-independent weights S(k) k^alpha of the cos and
//                     sin moments (pair independent, computed once per call)
//   ewald_trig        per (k, particle): cos(k.x_a), sin(k.x_a), so that
//                     cos(k.R_ab) = c_a c_b + s_a s_b needs no sincos per pair
//   ewald_pair_k      per pair: reciprocal moments over the half space (x2),
//                     epilogue, writes both 11x11 blocks of the pair
//   ewald_pair_real   per pair: real-space moments over the image cube,
//                     epilogue, adds into both blocks
//   ewald_self        per particle: self block (images n != 0, k != 0, and
//                     the analytic terms of PER_ROTNE_PRAGER_SELF 179-188)
// The closed forms come from ewald_gen.cuh (generated by gen_ewald.py).
#include <cuda_runtime.h>

#include <vector>

#include "ewald_gen.cuh"
#include "overlap.cuh"
#include "dsf.cuh"
#include "rsd_internal.cuh"

namespace {

constexpr int KW = 3 + RSD_NMOM_KCOS + RSD_NMOM_KSIN;  // doubles per k entry

__host__ __device__ inline void half_space_index(int h, int NI, int* nx, int* ny, int* nz) {
  const int w = 2 * NI + 1;
  const int q = (w * w * w - 1) / 2 + 1 + h;  // entries after the origin
  *nx = q / (w * w) - NI;
  *ny = (q / w) % w - NI;
  *nz = q % w - NI;
}

// S(k) of F_Jk (Ewald_summation.f90:1067-1071): F_Jk = S (delta k^2 - k k)
template <typename T>
__device__ inline T kernel_S(T k2, T lam) {
  const T l2 = lam * lam;
  return T(8.0 * RSD_PI) * (T(1) + k2 / (T(4) * l2) + k2 * k2 / (T(8) * l2 * l2)) * exp(-k2 / (T(4) * l2)) / (k2 * k2);
}

__global__ void ewald_ktable(rsd_lat_dev L, int Kh, double* __restrict__ tab) {
  const int h = blockIdx.x * blockDim.x + threadIdx.x;
  if (h >= Kh) return;
  int nx, ny, nz;
  half_space_index(h, L.NI, &nx, &ny, &nz);
  double k[3];
  for (int j = 0; j < 3; j++)
    k[j] = 2.0 * RSD_PI * (nx * L.LI[0 + 3 * j] + ny * L.LI[1 + 3 * j] + nz * L.LI[2 + 3 * j]);
  const double k2 = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
  const double S = kernel_S<double>(k2, L.lam);
  double* e = tab + (size_t)h * KW;
  e[0] = k[0];
  e[1] = k[1];
  e[2] = k[2];
  rsd_kcos_weights<double>(k[0], k[1], k[2], S, L.lam, e + 3);
  rsd_ksin_weights<double>(k[0], k[1], k[2], S, L.lam, e + 3 + RSD_NMOM_KCOS);
}

__global__ void ewald_trig(int nn, int Kh, const double* __restrict__ tab, const double* __restrict__ pos,
                           double2* __restrict__ cs) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  const int h = blockIdx.y;
  if (a >= nn) return;
  const double* e = tab + (size_t)h * KW;
  const double kr = e[0] * pos[3 * a] + e[1] * pos[3 * a + 1] + e[2] * pos[3 * a + 2];
  double s, c;
  sincos(kr, &s, &c);
  cs[(size_t)h * nn + a] = make_double2(c, s);
}

// Weights and trig tables restricted to a list of half-space indices, in
// precision T (the mixed form splits the reciprocal sum by shell).
template <typename T>
__global__ void ewald_ktable_list(rsd_lat_dev L, int count, const int* __restrict__ hlist, T* __restrict__ tab) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= count) return;
  int nx, ny, nz;
  half_space_index(hlist[q], L.NI, &nx, &ny, &nz);
  double k[3];
  for (int j = 0; j < 3; j++)
    k[j] = 2.0 * RSD_PI * (nx * L.LI[0 + 3 * j] + ny * L.LI[1 + 3 * j] + nz * L.LI[2 + 3 * j]);
  const double k2 = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
  const double S = kernel_S<double>(k2, L.lam);
  double wc[RSD_NMOM_KCOS], ws[RSD_NMOM_KSIN];
  rsd_kcos_weights<double>(k[0], k[1], k[2], S, L.lam, wc);
  rsd_ksin_weights<double>(k[0], k[1], k[2], S, L.lam, ws);
  T* e = tab + (size_t)q * KW;
  e[0] = (T)k[0];
  e[1] = (T)k[1];
  e[2] = (T)k[2];
  for (int m = 0; m < RSD_NMOM_KCOS; m++) e[3 + m] = (T)wc[m];
  for (int m = 0; m < RSD_NMOM_KSIN; m++) e[3 + RSD_NMOM_KCOS + m] = (T)ws[m];
}

__device__ __forceinline__ void put_trig(float2* p, double c, double sn) { *p = make_float2((float)c, (float)sn); }
__device__ __forceinline__ void put_trig(float4* p, double c, double sn) {
  const dsf dc = dsf_from(c), ds = dsf_from(sn);
  *p = make_float4(dc.hi, dc.lo, ds.hi, ds.lo);
}

template <typename T2>
__global__ void ewald_trig_list(int nn, rsd_lat_dev L, const int* __restrict__ hlist, const double* __restrict__ pos,
                                T2* __restrict__ cs) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  const int q = blockIdx.y;
  if (a >= nn) return;
  int nx, ny, nz;
  half_space_index(hlist[q], L.NI, &nx, &ny, &nz);
  double k[3];
  for (int j = 0; j < 3; j++)
    k[j] = 2.0 * RSD_PI * (nx * L.LI[0 + 3 * j] + ny * L.LI[1 + 3 * j] + nz * L.LI[2 + 3 * j]);
  const double kr = k[0] * pos[3 * a] + k[1] * pos[3 * a + 1] + k[2] * pos[3 * a + 2];
  double sn, c;
  sincos(kr, &sn, &c);
  put_trig(cs + (size_t)q * nn + a, c, sn);
}

// Scatter of the pair block (a,b), a < b, and its mirror (b,a) with
// b -> -b, g -> -g (per_GRPY_YZD.f90:123-151,160-188).  v holds the 60
// unique values (order of gen_ewald.py) already scaled; add != 0 adds.
// Destinations of the pair blocks.  DenseSink: the FP64 grand mobility
// (column-major, ld).  PlaneSink: the mixed form's grand mobility as two
// FP32 planes, M = hi + lo with |lo| <= ulp(hi)/2 (~48 bits, the precision
// the mixed assembly computes in), read by the FP32 factorisation (hi) and
// by the double-single residual products of the refinement (both).
// put<K> stores (add = 0) or read-modify-writes (add = 1) K entries; all K
// loads are issued before the first store, so a thread waits for one memory
// round trip per group rather than one per entry (the offsets of a group are
// distinct).
struct DenseSink {
  double* M;
  int64_t ld;
  template <int K>
  __device__ __forceinline__ void put(const int64_t* o, const double* x, int add) const {
    if (add) {
      double v[K];
#pragma unroll
      for (int i = 0; i < K; i++) v[i] = M[o[i]];
#pragma unroll
      for (int i = 0; i < K; i++) M[o[i]] = v[i] + x[i];
    } else {
#pragma unroll
      for (int i = 0; i < K; i++) M[o[i]] = x[i];
    }
  }
};

struct PlaneSink {
  float* hi;
  float* lo;
  int64_t ld;
  template <int K>
  __device__ __forceinline__ void put(const int64_t* o, const dsf* x, int add) const {
    if (add) {
      float h[K], l[K];
#pragma unroll
      for (int i = 0; i < K; i++) {
        h[i] = hi[o[i]];
        l[i] = lo[o[i]];
      }
#pragma unroll
      for (int i = 0; i < K; i++) {
        const dsf v = dsf(h[i], l[i]) + x[i];
        hi[o[i]] = v.hi;
        lo[o[i]] = v.lo;
      }
    } else {
#pragma unroll
      for (int i = 0; i < K; i++) {
        hi[o[i]] = x[i].hi;
        lo[o[i]] = x[i].lo;
      }
    }
  }
};

// Writes the pair blocks (a, b) and (b, a), a != b, of the grand mobility
// from the 60 values of a pair (TT 0-5, RR 6-11, TR 12-14, QQ 15-29, G
// 30-44, H 45-59), in 14 groups of at most 25 entries.  V: double
// (DenseSink) or dsf (PlaneSink).
template <typename V, typename S>
__device__ inline void store_pair_t(const S& sk, int N, int a, int b, const V* v, int add) {
  auto at = [&](int r, int c) { return (int64_t)r + (int64_t)c * sk.ld; };
  constexpr int sym[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
  // TT and RR, both orders
#pragma unroll
  for (int blk = 0; blk < 2; blk++) {
    const int o = blk ? 3 * N : 0;
    int64_t p[18];
    V x[18];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        const V t = v[6 * blk + sym[i][j]];
        p[6 * i + 2 * j] = at(o + 3 * a + i, o + 3 * b + j);
        p[6 * i + 2 * j + 1] = at(o + 3 * b + i, o + 3 * a + j);
        x[6 * i + 2 * j] = x[6 * i + 2 * j + 1] = t;
      }
    sk.template put<18>(p, x, add);
  }
  // TR: translation of one particle against rotation of the other, both
  // placements (upper and lower triangle) of each
#pragma unroll
  for (int side = 0; side < 2; side++) {
    const int t = side ? b : a, r = side ? a : b;
    int64_t p[18];
    V x[18];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        V tr = V(0);
        if (i < j) tr = v[12 + (i == 0 ? j - 1 : 2)];
        if (i > j) tr = -v[12 + (j == 0 ? i - 1 : 2)];
        if (side) tr = -tr;
        p[6 * i + 2 * j] = at(3 * t + i, 3 * N + 3 * r + j);
        p[6 * i + 2 * j + 1] = at(3 * N + 3 * r + j, 3 * t + i);
        x[6 * i + 2 * j] = x[6 * i + 2 * j + 1] = tr;
      }
    sk.template put<18>(p, x, add);
  }
  // G (translation-stresslet, odd under a <-> b) and H (rotation-stresslet)
#pragma unroll
  for (int grp = 0; grp < 8; grp++) {
    const int side = grp >> 2, h = (grp >> 1) & 1, lower = grp & 1;
    const int u = side ? b : a, sp = side ? a : b;  // velocity row particle, stresslet column particle
    const int ro = h ? 3 * N : 0;
    int64_t p[15];
    V x[15];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int m = 0; m < 5; m++) {
        V g = v[(h ? 45 : 30) + 5 * i + m];
        if (side && !h) g = -g;
        p[5 * i + m] = lower ? at(6 * N + 5 * sp + m, ro + 3 * u + i) : at(ro + 3 * u + i, 6 * N + 5 * sp + m);
        x[5 * i + m] = g;
      }
    sk.template put<15>(p, x, add);
  }
  // QQ, both orders
#pragma unroll
  for (int side = 0; side < 2; side++) {
    const int r = side ? b : a, c = side ? a : b;
    int64_t p[25];
    V x[25];
#pragma unroll
    for (int xi = 0; xi < 5; xi++)
#pragma unroll
      for (int y = 0; y < 5; y++) {
        const int lo = xi < y ? xi : y, hi = xi < y ? y : xi;
        p[5 * xi + y] = at(6 * N + 5 * r + xi, 6 * N + 5 * c + y);
        x[5 * xi + y] = v[15 + lo * 5 - lo * (lo - 1) / 2 + (hi - lo)];
      }
    sk.template put<25>(p, x, add);
  }
}

// Mixed form: only the entries whose row belongs to particle a (a < b) of
// each pair block are written (121 of 242: the pair's rows of the grand
// matrix, all coalesced along a); the consumers read the other half at the
// mirrored position, or mirror_planes fills it by symmetry.  Values as in
// store_pair_t.
__device__ inline void store_pair_rows_a(const PlaneSink& sk, int N, int a, int b, const dsf* v, int add) {
  auto at = [&](int r, int c) { return (int64_t)r + (int64_t)c * sk.ld; };
  constexpr int sym[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
  {  // TT and RR
    int64_t p[18];
    dsf x[18];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        p[3 * i + j] = at(3 * a + i, 3 * b + j);
        x[3 * i + j] = v[sym[i][j]];
        p[9 + 3 * i + j] = at(3 * N + 3 * a + i, 3 * N + 3 * b + j);
        x[9 + 3 * i + j] = v[6 + sym[i][j]];
      }
    sk.template put<18>(p, x, add);
  }
  {  // TR: a's translation rows against b's rotation, a's rotation rows against b's translation
    int64_t p[18];
    dsf x[18];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int j = 0; j < 3; j++) {
        dsf tr = dsf(0);
        if (i < j) tr = v[12 + (i == 0 ? j - 1 : 2)];
        if (i > j) tr = -v[12 + (j == 0 ? i - 1 : 2)];
        p[3 * i + j] = at(3 * a + i, 3 * N + 3 * b + j);
        x[3 * i + j] = tr;
        p[9 + 3 * i + j] = at(3 * N + 3 * a + j, 3 * b + i);
        x[9 + 3 * i + j] = -tr;
      }
    sk.template put<18>(p, x, add);
  }
#pragma unroll
  for (int grp = 0; grp < 4; grp++) {  // G and H: a's velocity rows, then a's stresslet rows
    const int h = grp & 1, srow = grp >> 1;
    const int ro = h ? 3 * N : 0;
    int64_t p[15];
    dsf x[15];
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int m = 0; m < 5; m++) {
        dsf g = v[(h ? 45 : 30) + 5 * i + m];
        if (srow && !h) g = -g;
        p[5 * i + m] = srow ? at(6 * N + 5 * a + m, ro + 3 * b + i) : at(ro + 3 * a + i, 6 * N + 5 * b + m);
        x[5 * i + m] = g;
      }
    sk.template put<15>(p, x, add);
  }
  {  // QQ
    int64_t p[25];
    dsf x[25];
#pragma unroll
    for (int xi = 0; xi < 5; xi++)
#pragma unroll
      for (int y = 0; y < 5; y++) {
        const int lo = xi < y ? xi : y, hi = xi < y ? y : xi;
        p[5 * xi + y] = at(6 * N + 5 * a + xi, 6 * N + 5 * b + y);
        x[5 * xi + y] = v[15 + lo * 5 - lo * (lo - 1) / 2 + (hi - lo)];
      }
    sk.template put<25>(p, x, add);
  }
}

// particle of grand-matrix index x
__device__ __forceinline__ int grand_particle(int N, int x) {
  return x < 3 * N ? x / 3 : (x < 6 * N ? (x - 3 * N) / 3 : (x - 6 * N) / 5);
}

// M(r, c) = M(c, r) for every entry whose row's particle is above its
// column's (the entries store_pair_rows_a leaves out), on both planes:
// 32 x 32 tiles through shared memory, both the read and the write
// coalesced; tiles with nothing to fill return at once.
__global__ void mirror_planes(int N, int64_t n, float* __restrict__ hi, float* __restrict__ lo, int64_t ld) {
  __shared__ float th[32][33], tl[32][33];
  __shared__ int skip;
  const int r0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;
  if (ty == 0) {  // the particle index is monotonic only within each of the three row sections
    const int rmax = __reduce_max_sync(0xffffffffu, grand_particle(N, (int)min((int64_t)r0 + tx, n - 1)));
    const int cmin = __reduce_min_sync(0xffffffffu, grand_particle(N, (int)min((int64_t)c0 + tx, n - 1)));
    if (tx == 0) skip = rmax <= cmin;
  }
  __syncthreads();
  if (skip) return;
  for (int k = ty; k < 32; k += blockDim.y) {  // source M(c0 + tx, r0 + k)
    const int64_t c = c0 + tx, r = r0 + k;
    if (c < n && r < n) {
      th[k][tx] = hi[c + r * ld];
      tl[k][tx] = lo[c + r * ld];
    }
  }
  __syncthreads();
  for (int k = ty; k < 32; k += blockDim.y) {  // destination M(r0 + tx, c0 + k)
    const int64_t r = r0 + tx, c = c0 + k;
    if (r < n && c < n && grand_particle(N, (int)r) > grand_particle(N, (int)c)) {
      hi[r + c * ld] = th[tx][k];
      lo[r + c * ld] = tl[tx][k];
    }
  }
}

// A pair block computed in FP64 into either destination.
__device__ __forceinline__ void store_pair_d(const DenseSink& sk, int N, int a, int b, const double* o, int add) {
  store_pair_t<double>(sk, N, a, b, o, add);
}
__device__ __forceinline__ void store_pair_d(const PlaneSink& sk, int N, int a, int b, const double* o, int add) {
  dsf v[60];
#pragma unroll
  for (int q = 0; q < 60; q++) v[q] = dsf_from(o[q]);
  store_pair_rows_a(sk, N, a, b, v, add);
}

// scale by nondim (1/(6 a_i) for TT, TR, G; 1/(6 a_i^3) for RR, QQ, H) and
// by 1/(pi mu_f)
__device__ inline void scale_block(double* v, double ai, double inv_pimu) {
  const double na = inv_pimu / (6.0 * ai), na3 = inv_pimu / (6.0 * ai * ai * ai);
  for (int q = 0; q < 60; q++) {
    const bool a3 = (q >= 6 && q < 12) || (q >= 15 && q < 30) || q >= 45;
    v[q] *= a3 ? na3 : na;
  }
}

__device__ inline bool pair_of(int nn, int* a, int* b) {
  *a = blockIdx.x * blockDim.x + threadIdx.x;
  *b = blockIdx.y * blockDim.y + threadIdx.y;
  return *a < nn && *b < nn && *a < *b;
}

template <typename T>
struct Vec2;
template <>
struct Vec2<float> {
  using type = float4;  // four weights per shared-memory load
  static constexpr int W = 4;
};
template <>
struct Vec2<double> {
  using type = double2;
  static constexpr int W = 2;
};

// Reciprocal-space pair sums: per half-space vector, cos and sin of k.(x_a -
// x_b) from the per-particle trig table, times the vector's 80 moment
// weights.  The weights are staged in shared memory 16 vectors at a time and
// read as 16-byte vectors (the same address for every thread of a warp).
template <typename T, typename T2, typename S>
__global__ void __launch_bounds__(128) ewald_pair_k(int nn, rsd_lat_dev L, int Kh, const T* __restrict__ tab,
                                                    const T2* __restrict__ cs, const double* __restrict__ radii,
                                                    double inv_pimu, S sk, int add) {
  constexpr int KWT = 3 + RSD_NMOM_KCOS + RSD_NMOM_KSIN;
  constexpr int NW = RSD_NMOM_KCOS + RSD_NMOM_KSIN;  // 80
  constexpr int KC = 16;
  using V = typename Vec2<T>::type;
  constexpr int VW = Vec2<T>::W;
  static_assert(NW % VW == 0, "weights per vector");
  __shared__ __align__(16) T sw[KC * NW];
  __shared__ T2 sca[KC][32], scb[KC][4];  // trig values of the CTA's 32 + 4 particles (block 32 x 4)
  // blocks entirely on or below the diagonal (a >= b everywhere) have no work
  if ((int)(blockIdx.x * blockDim.x) >= (int)(blockIdx.y * blockDim.y + blockDim.y - 1)) return;
  int a, b;
  const bool valid = pair_of(nn, &a, &b);
  const int tid = threadIdx.y * blockDim.x + threadIdx.x, nthr = blockDim.x * blockDim.y;
  const int a0 = blockIdx.x * blockDim.x, b0 = blockIdx.y * blockDim.y;
  T ac[RSD_NMOM_KCOS], as[RSD_NMOM_KSIN];
#pragma unroll
  for (int m = 0; m < RSD_NMOM_KCOS; m++) ac[m] = T(0);
#pragma unroll
  for (int m = 0; m < RSD_NMOM_KSIN; m++) as[m] = T(0);
  for (int h0 = 0; h0 < Kh; h0 += KC) {
    const int kc = min(KC, Kh - h0);
    __syncthreads();
    for (int e = tid; e < kc * NW; e += nthr) sw[e] = tab[(size_t)(h0 + e / NW) * KWT + 3 + e % NW];
    for (int e = tid; e < kc * 36; e += nthr) {
      const int hh = e / 36, q = e % 36, part = q < 32 ? a0 + q : b0 + q - 32;
      if (part < nn) {
        const T2 v = cs[(size_t)(h0 + hh) * nn + part];
        if (q < 32)
          sca[hh][q] = v;
        else
          scb[hh][q - 32] = v;
      }
    }
    __syncthreads();
    if (!valid) continue;
    for (int hh = 0; hh < kc; hh++) {
      const T2 ua = sca[hh][threadIdx.x], ub = scb[hh][threadIdx.y];
      const T c = ua.x * ub.x + ua.y * ub.y;  // cos(k.(x_a - x_b))
      const T sn = ua.y * ub.x - ua.x * ub.y;  // sin(k.(x_a - x_b))
      const V* e = reinterpret_cast<const V*>(sw + hh * NW);
#pragma unroll
      for (int m4 = 0; m4 < NW / VW; m4++) {
        const V w = e[m4];
        const T* wq = reinterpret_cast<const T*>(&w);
#pragma unroll
        for (int q = 0; q < VW; q++) {
          const int m = m4 * VW + q;
          if (m < RSD_NMOM_KCOS)
            ac[m] = fma(wq[q], c, ac[m]);
          else
            as[m - RSD_NMOM_KCOS] = fma(wq[q], sn, as[m - RSD_NMOM_KCOS]);
        }
      }
    }
  }
  if (!valid) return;
  const T ai = (T)radii[a], aj = (T)radii[b], phix = (T)L.phix;
  T v[60], w[60];
  rsd_kcos_epilogue<T>(ac, ai, aj, phix, v);
  rsd_ksin_epilogue<T>(as, ai, aj, phix, w);
  double o[60];
  const double f = 2.0 / L.LV;  // half space counted twice
#pragma unroll
  for (int q = 0; q < 60; q++) o[q] = ((double)v[q] + (double)w[q]) * f;
  scale_block(o, radii[a], inv_pimu);
  store_pair_d(sk, nn, a, b, o, add);
}

// Reciprocal-space pair sums of the FP64 shells of the mixed form in
// double-single: the trig table holds (cos, sin) as float pairs (float4 per
// vector and particle), the weights are converted to float pairs as they are
// staged in shared memory, and the epilogue runs in FP64.
template <typename S>
__global__ void __launch_bounds__(128) ewald_pair_k_ds(int nn, rsd_lat_dev L, int Kh, const double* __restrict__ tab,
                                                       const float4* __restrict__ cs, const double* __restrict__ radii,
                                                       double inv_pimu, S sk, int add) {
  constexpr int KWT = 3 + RSD_NMOM_KCOS + RSD_NMOM_KSIN;
  constexpr int NW = RSD_NMOM_KCOS + RSD_NMOM_KSIN;
  constexpr int KC = 16;
  __shared__ __align__(16) dsf sw[KC * NW];
  __shared__ float4 sca[KC][32], scb[KC][4];  // trig values of the CTA's 32 + 4 particles (block 32 x 4)
  if ((int)(blockIdx.x * blockDim.x) >= (int)(blockIdx.y * blockDim.y + blockDim.y - 1)) return;
  int a, b;
  const bool valid = pair_of(nn, &a, &b);
  const int tid = threadIdx.y * blockDim.x + threadIdx.x, nthr = blockDim.x * blockDim.y;
  const int a0 = blockIdx.x * blockDim.x, b0 = blockIdx.y * blockDim.y;
  dsf ac[RSD_NMOM_KCOS], as[RSD_NMOM_KSIN];
#pragma unroll
  for (int m = 0; m < RSD_NMOM_KCOS; m++) ac[m] = dsf(0);
#pragma unroll
  for (int m = 0; m < RSD_NMOM_KSIN; m++) as[m] = dsf(0);
  for (int h0 = 0; h0 < Kh; h0 += KC) {
    const int kc = min(KC, Kh - h0);
    __syncthreads();
    for (int e = tid; e < kc * NW; e += nthr) sw[e] = dsf_from(tab[(size_t)(h0 + e / NW) * KWT + 3 + e % NW]);
    for (int e = tid; e < kc * 36; e += nthr) {
      const int hh = e / 36, q = e % 36, part = q < 32 ? a0 + q : b0 + q - 32;
      if (part < nn) {
        const float4 v = cs[(size_t)(h0 + hh) * nn + part];
        if (q < 32)
          sca[hh][q] = v;
        else
          scb[hh][q - 32] = v;
      }
    }
    __syncthreads();
    if (!valid) continue;
    for (int hh = 0; hh < kc; hh++) {
      const float4 ua = sca[hh][threadIdx.x], ub = scb[hh][threadIdx.y];
      const dsf ca(ua.x, ua.y), sa(ua.z, ua.w), cb(ub.x, ub.y), sb(ub.z, ub.w);
      const dsf c = ca * cb + sa * sb;   // cos(k.(x_a - x_b))
      const dsf sn = sa * cb - ca * sb;  // sin(k.(x_a - x_b))
      const dsf* e = sw + hh * NW;
#pragma unroll
      for (int m = 0; m < RSD_NMOM_KCOS; m++) ac[m] = fma(e[m], c, ac[m]);
#pragma unroll
      for (int m = 0; m < RSD_NMOM_KSIN; m++) as[m] = fma(e[RSD_NMOM_KCOS + m], sn, as[m]);
    }
  }
  if (!valid) return;
  double acd[RSD_NMOM_KCOS], asd[RSD_NMOM_KSIN];
#pragma unroll
  for (int m = 0; m < RSD_NMOM_KCOS; m++) acd[m] = dsf_to(ac[m]);
#pragma unroll
  for (int m = 0; m < RSD_NMOM_KSIN; m++) asd[m] = dsf_to(as[m]);
  double v[60], w[60];
  rsd_kcos_epilogue<double>(acd, radii[a], radii[b], L.phix, v);
  rsd_ksin_epilogue<double>(asd, radii[a], radii[b], L.phix, w);
  double o[60];
  const double f = 2.0 / L.LV;  // half space counted twice
#pragma unroll
  for (int q = 0; q < 60; q++) o[q] = (v[q] + w[q]) * f;
  scale_block(o, radii[a], inv_pimu);
  store_pair_d(sk, nn, a, b, o, add);
}

// ---------------------------------------------------- equal radii, k space
// With one radius for every particle, the reciprocal-space epilogue (linear
// in the moments) can be applied per vector instead of per pair: each of
// the 60 block entries is then sum_k W_q(k) cos(k.R) (41 entries: TT, RR,
// QQ, H) or sum_k W_q(k) sin(k.R) (the 18 TR and G entries), with the block
// weights W_q(k) = epilogue(moment weights of k) formed once per vector in
// FP64.  A pair then costs 60 multiply-adds per vector instead of 80, and
// its FP32 rounding is no longer amplified by the epilogue's cancellation
// between moments.
__host__ __device__ constexpr bool kblock_is_sin(int q) { return (q >= 12 && q < 15) || (q >= 30 && q < 45); }
constexpr int KBW = 64;  // weights per vector (60 used, padded for 16-byte rows)

template <typename T>
__device__ __forceinline__ void put_weight(T* p, double v) { *p = (T)v; }
template <>
__device__ __forceinline__ void put_weight<dsf>(dsf* p, double v) { *p = dsf_from(v); }

template <typename T>
__global__ void ewald_kblock_list(rsd_lat_dev L, int count, const int* __restrict__ hlist, double a,
                                  double inv_pimu, T* __restrict__ W) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= count) return;
  int nx, ny, nz;
  half_space_index(hlist[q], L.NI, &nx, &ny, &nz);
  double k[3];
  for (int j = 0; j < 3; j++)
    k[j] = 2.0 * RSD_PI * (nx * L.LI[0 + 3 * j] + ny * L.LI[1 + 3 * j] + nz * L.LI[2 + 3 * j]);
  const double k2 = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
  const double S = kernel_S<double>(k2, L.lam);
  double wc[RSD_NMOM_KCOS], ws[RSD_NMOM_KSIN], v[60], w[60];
  rsd_kcos_weights<double>(k[0], k[1], k[2], S, L.lam, wc);
  rsd_ksin_weights<double>(k[0], k[1], k[2], S, L.lam, ws);
  rsd_kcos_epilogue<double>(wc, a, a, L.phix, v);
  rsd_ksin_epilogue<double>(ws, a, a, L.phix, w);
  // half space counted twice, and the non-dimensionalisation of scale_block
  const double f = 2.0 / L.LV, na = f * inv_pimu / (6.0 * a), na3 = na / (a * a);
  T* e = W + (size_t)q * KBW;
  for (int i = 0; i < 60; i++) {
    const bool a3 = (i >= 6 && i < 12) || (i >= 15 && i < 30) || i >= 45;
    put_weight<T>(e + i, (kblock_is_sin(i) ? w[i] : v[i]) * (a3 ? na3 : na));
  }
  for (int i = 60; i < KBW; i++) put_weight<T>(e + i, 0.0);
}

__device__ __forceinline__ void acc_norm(dsacc& a) { dsacc_norm(a); }

// FP32 sum of the vectors of one chunk (f), folded at the end of every chunk
// into a double-single total (hi + lo, Knuth's two-sum).  A plain FP32 sum
// over all K32 vectors has a rounding error ~ sqrt(K32) times that of its
// terms, which grows with the number of FP32 vectors (with lambda^3).
struct fchunk {
  float f, hi, lo;
};
__device__ __forceinline__ fchunk fma(float e, float c, fchunk a) {
  a.f = __fmaf_rn(e, c, a.f);
  return a;
}
__device__ __forceinline__ void acc_norm(fchunk& a) {
  const float s = __fadd_rn(a.hi, a.f);
  const float bb = __fsub_rn(s, a.hi);
  a.lo = __fadd_rn(a.lo, __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(a.f, bb)));
  a.hi = s;
  a.f = 0.f;
}

__device__ __forceinline__ float trig_c(float2 v) { return v.x; }
__device__ __forceinline__ float trig_s(float2 v) { return v.y; }
__device__ __forceinline__ dsf trig_c(float4 v) { return dsf(v.x, v.y); }
__device__ __forceinline__ dsf trig_s(float4 v) { return dsf(v.z, v.w); }

// Accumulates sum_k W_q(k) {cos, sin}(k.(x_a - x_b)) over Kh vectors into
// acc, for the pair (a, b) of the calling thread (block 32 x 4).  The
// weights of 16 vectors and the trig values of the CTA's 32 + 4 particles
// are staged in shared memory (sw: 16 x KBW, sca: 16 x 32, scb: 16 x 4).
template <typename T, typename TT, typename A>
__device__ __forceinline__ void kblock_accumulate(int nn, int Kh, const T* __restrict__ W, const TT* __restrict__ cs,
                                                  T* sw, TT* sca, TT* scb, bool valid, A (&acc)[60]) {
  constexpr int KC = 16;
  const int tid = threadIdx.y * blockDim.x + threadIdx.x, nthr = blockDim.x * blockDim.y;
  const int a0 = blockIdx.x * blockDim.x, b0 = blockIdx.y * blockDim.y;
  for (int h0 = 0; h0 < Kh; h0 += KC) {
    const int kc = min(KC, Kh - h0);
    __syncthreads();
    for (int e = tid; e < kc * KBW; e += nthr) sw[e] = W[(size_t)h0 * KBW + e];
    for (int e = tid; e < kc * 36; e += nthr) {
      const int hh = e / 36, q = e % 36, part = q < 32 ? a0 + q : b0 + q - 32;
      if (part < nn) {
        const TT v = cs[(size_t)(h0 + hh) * nn + part];
        if (q < 32)
          sca[hh * 32 + q] = v;
        else
          scb[hh * 4 + q - 32] = v;
      }
    }
    __syncthreads();
    if (!valid) continue;
    for (int hh = 0; hh < kc; hh++) {
      const TT ua = sca[hh * 32 + threadIdx.x], ub = scb[hh * 4 + threadIdx.y];
      const T ca = trig_c(ua), sa = trig_s(ua), cb = trig_c(ub), sb = trig_s(ub);
      const T c = ca * cb + sa * sb;   // cos(k.(x_a - x_b))
      const T sn = sa * cb - ca * sb;  // sin(k.(x_a - x_b))
      const T* e = sw + hh * KBW;
#pragma unroll
      for (int q = 0; q < 60; q++) acc[q] = fma(e[q], kblock_is_sin(q) ? sn : c, acc[q]);
    }
#pragma unroll
    for (int q = 0; q < 60; q++) acc_norm(acc[q]);  // at most 16 steps between renormalisations
  }
}

// Reciprocal-space pair blocks with per-vector block weights (equal radii):
// the K32 FP32 vectors first, then the K64 double-single ones on top of the
// FP32 sums; the blocks are written (add = 0) or added (add = 1) once.
__global__ void __launch_bounds__(128) ewald_pair_kblock(int nn, int K32, const float* __restrict__ W32,
                                                         const float2* __restrict__ c32, int K64,
                                                         const dsf* __restrict__ W64, const float4* __restrict__ c64,
                                                         PlaneSink sk, int add) {
  constexpr int KC = 16;
  __shared__ __align__(16) dsf sw[KC * KBW];  // the FP32 phase uses the first half as floats
  __shared__ __align__(16) float4 sca[KC * 32], scb[KC * 4];
  if ((int)(blockIdx.x * blockDim.x) >= (int)(blockIdx.y * blockDim.y + blockDim.y - 1)) return;
  int a, b;
  const bool valid = pair_of(nn, &a, &b);
  dsacc acc[60];
  {
    fchunk f[60];
#pragma unroll
    for (int q = 0; q < 60; q++) f[q] = fchunk{0.f, 0.f, 0.f};
    kblock_accumulate<float, float2>(nn, K32, W32, c32, reinterpret_cast<float*>(sw),
                                     reinterpret_cast<float2*>(sca), reinterpret_cast<float2*>(scb), valid, f);
#pragma unroll
    for (int q = 0; q < 60; q++) acc[q] = dsacc(f[q].hi, f[q].lo);
  }
  kblock_accumulate<dsf, float4>(nn, K64, W64, c64, sw, sca, scb, valid, acc);
  if (!valid) return;
  dsf o[60];
#pragma unroll
  for (int q = 0; q < 60; q++) {
    dsacc_norm(acc[q]);
    o[q] = dsf(acc[q].hi, acc[q].lo);
  }
  store_pair_rows_a(sk, nn, a, b, o, add);
}

// Near/far split of the real-space images for the mixed form.  Image nz of
// lattice column (nx, ny) has FP32 coordinates p + a3 nz, where p = R + nx a1
// + ny a2 is formed in FP64 and rounded once; it is "near" when its FP32
// squared distance, computed by exactly the sequence below, is below rc^2.
// The near (double-single) and far (FP32) kernels evaluate the same sequence
// on the same inputs, so every image is summed by exactly one of them.  An
// image within a rounding of the boundary may fall on either side; both
// sides are accurate there.
__device__ __forceinline__ void column_base(const double R[3], const double* LR, int nx, int ny, double p[3]) {
  for (int k = 0; k < 3; k++) p[k] = __fma_rn(LR[3 + k], (double)ny, __fma_rn(LR[k], (double)nx, R[k]));
}

__device__ __forceinline__ float image_r2f(float p0, float p1, float p2, float a0, float a1, float a2, int nz,
                                           float* x0, float* x1, float* x2) {
  const float z = (float)nz;
  *x0 = __fmaf_rn(a0, z, p0);
  *x1 = __fmaf_rn(a1, z, p1);
  *x2 = __fmaf_rn(a2, z, p2);
  return __fmaf_rn(*x2, *x2, __fmaf_rn(*x1, *x1, __fmul_rn(*x0, *x0)));
}

// Far real-space images of the mixed form in FP32: lambda r from the
// context's mixed_rcut up to mixed_rmax (beyond which the terms change a
// block by less than ~1e-12 of its largest entry), with FP32 coordinates
// p + a3 nz from each column's FP64 base point.  The radial functions of
// erfc(lambda r) feed moments that the epilogue combines with 2-3 orders of
// cancellation, so FP32 is kept for images whose terms are below ~1e-6 of a
// block (a few 1e-11 of a block after the epilogue).
template <typename S>
__global__ void __launch_bounds__(128) ewald_pair_real_far(int nn, rsd_lat_dev L, const double* __restrict__ pos,
                                                           const double* __restrict__ radii, double inv_pimu,
                                                           double rc2, double rmax2, S sk) {
  int a, b;
  if (!pair_of(nn, &a, &b)) return;
  double R[3] = {pos[3 * a] - pos[3 * b], pos[3 * a + 1] - pos[3 * b + 1], pos[3 * a + 2] - pos[3 * b + 2]};
  double dmin;
  rsd_skew_correction(L.LR, L.LI, R, &dmin);
  float acc[RSD_NMOM_REAL];
#pragma unroll
  for (int m = 0; m < RSD_NMOM_REAL; m++) acc[m] = 0.f;
  const float lam = (float)L.lam, lam2 = lam * lam, cd = (float)(2.0 * RSD_PIP5) * lam;
  const float a0 = __double2float_rn(L.LR[6]), a1 = __double2float_rn(L.LR[7]), a2 = __double2float_rn(L.LR[8]);
  const float rc2f = __double2float_rn(rc2), rmax2f = __double2float_rn(rmax2);
  const int NR = L.NR;
  for (int nx = -NR; nx <= NR; nx++)
    for (int ny = -NR; ny <= NR; ny++) {
      double p[3];
      column_base(R, L.LR, nx, ny, p);
      const float p0 = __double2float_rn(p[0]), p1 = __double2float_rn(p[1]), p2 = __double2float_rn(p[2]);
      for (int nz = -NR; nz <= NR; nz++) {
        float x0, x1, x2;
        const float r2 = image_r2f(p0, p1, p2, a0, a1, a2, nz, &x0, &x1, &x2);
        if (r2 < rc2f || r2 >= rmax2f) continue;  // near (the other kernel) or truncated
        const float r = sqrtf(r2), ir = 1.f / r;
        rsd_real_image<float>(x0, x1, x2, r, ir, erfcf(lam * r), cd * expf(-r2 * lam2), lam, acc);
      }
    }
  float v[60];
  rsd_real_epilogue<float>(acc, (float)radii[a], (float)radii[b], (float)L.phix, v);
  double o[60];
#pragma unroll
  for (int q = 0; q < 60; q++) o[q] = (double)v[q];
  scale_block(o, radii[a], inv_pimu);
  store_pair_d(sk, nn, a, b, o, 1);
}

// Near images of the mixed form (lambda r below the context's mixed_rcut) in
// double-single arithmetic on the FP32 pipe: coordinates p + a3 nz, r, 1/r,
// erfc(lambda r) and the Gaussian (dsf.cuh), the moments and their sums all
// carry ~48 bits (so even after the epilogue's 2-3 orders of cancellation a
// block stays within ~1e-12 of FP64); FP64 is left for the per-column set-up
// and the FP64 epilogue.  Same image set as the FP32 far kernel's complement.
template <typename S>
__global__ void __launch_bounds__(128) ewald_pair_real_near_ds(int nn, rsd_lat_dev L, const double* __restrict__ pos,
                                                               const double* __restrict__ radii, double inv_pimu,
                                                               double rc2, S sk) {
  __shared__ dsf_tables T;
  // blocks entirely on or below the diagonal (a >= b everywhere) have no work
  if ((int)(blockIdx.x * blockDim.x) >= (int)(blockIdx.y * blockDim.y + blockDim.y - 1)) return;
  dsf_tables_fill(T, threadIdx.y * blockDim.x + threadIdx.x, blockDim.x * blockDim.y);
  __syncthreads();
  int a, b;
  if (!pair_of(nn, &a, &b)) return;
  double R[3] = {pos[3 * a] - pos[3 * b], pos[3 * a + 1] - pos[3 * b + 1], pos[3 * a + 2] - pos[3 * b + 2]};
  double dmin;
  rsd_skew_correction(L.LR, L.LI, R, &dmin);
  dsacc acc[RSD_NMOM_REAL];
#pragma unroll
  for (int m = 0; m < RSD_NMOM_REAL; m++) acc[m] = dsacc(0);
  int since_norm = 0;
  const dsf lam_s = dsf_from(L.lam), cd_s = dsf_from(2.0 * RSD_PIP5 * L.lam);
  const dsf a30 = dsf_from(L.LR[6]), a31 = dsf_from(L.LR[7]), a32 = dsf_from(L.LR[8]);
  const float a0 = __double2float_rn(L.LR[6]), a1 = __double2float_rn(L.LR[7]), a2 = __double2float_rn(L.LR[8]);
  const float rc2f = __double2float_rn(rc2);
  const int NR = L.NR;
  for (int nx = -NR; nx <= NR; nx++)
    for (int ny = -NR; ny <= NR; ny++) {
      double p[3];
      column_base(R, L.LR, nx, ny, p);
      const float f0 = __double2float_rn(p[0]), f1 = __double2float_rn(p[1]), f2 = __double2float_rn(p[2]);
      const dsf p0 = dsf_from(p[0]), p1 = dsf_from(p[1]), p2 = dsf_from(p[2]);
      for (int nz = -NR; nz <= NR; nz++) {
        float y0, y1, y2;
        if (!(image_r2f(f0, f1, f2, a0, a1, a2, nz, &y0, &y1, &y2) < rc2f)) continue;
        const dsf x0 = p0 + nz * a30, x1 = p1 + nz * a31, x2 = p2 + nz * a32;
        const dsf r = dsf_sqrt(x0 * x0 + x1 * x1 + x2 * x2);
        const dsf ir = dsf_rcp(r);
        dsf E0, G;
        dsf_erfc_gauss(lam_s * r, T, &E0, &G);
        rsd_real_image<dsf, dsacc>(x0, x1, x2, r, ir, E0, cd_s * G, lam_s, acc);
        if (++since_norm == 4) {  // keep the accumulators' lo parts small
#pragma unroll
          for (int m = 0; m < RSD_NMOM_REAL; m++) dsacc_norm(acc[m]);
          since_norm = 0;
        }
      }
    }
  double accd[RSD_NMOM_REAL];
#pragma unroll
  for (int m = 0; m < RSD_NMOM_REAL; m++) accd[m] = dsacc_to(acc[m]);
  double v[60];
  rsd_real_epilogue<double>(accd, radii[a], radii[b], L.phix, v);
  scale_block(v, radii[a], inv_pimu);
  store_pair_d(sk, nn, a, b, v, 1);
}

// ------------------------------------------ equal radii, real space, mixed
// One kernel for both real-space image sets of a pair, all in FP32 and
// double-single arithmetic (the FP64 pipe of GB300 runs at ~1/60 of the
// FP32 rate, so no FP64 is left in the image loops or the epilogue):
//   - images are classified in FP32: column base p = R + nx a1 + ny a2 and
//     image p + nz a3 (fused multiply-adds in a fixed order), near when its
//     squared distance is below rc^2, far up to rmax^2, so every image lands
//     in exactly one set;
//   - each set is processed from a per-thread list of image indices in
//     shared memory (REAL_CAP at a time), so the lanes of a warp run their
//     own images together instead of idling through each other's;
//   - far images: FP32 moments; near images: double-single coordinates
//     R + nx a1 + ny a2 + nz a3, r, erfc, exp and moments (dsacc);
//   - the epilogues apply the coefficient table of the common radius
//     (rsd_real_epi_coef_scaled, formed once in FP64), output by output, and
//     the pair blocks are added to M's planes once.
constexpr int REAL_CAP = 32;
constexpr int REAL_THREADS = 128;
struct RealEqShared {
  dsf_tables T;
  dsf cr[RSD_REAL_EPI_NC];
  float cf[RSD_REAL_EPI_NC];
  int list[REAL_CAP][REAL_THREADS];
  float oh[60][REAL_THREADS];  // the pair block: far part, then hi of the sum
  float ol[60][REAL_THREADS];  // lo of the sum
};
constexpr int SMEM_REAL_EQ = (int)sizeof(RealEqShared);

// The coefficient tables for radius a (double-single and FP32).
__global__ void ewald_real_epi_table(double a, double phix, double inv_pimu, dsf* __restrict__ cr,
                                     float* __restrict__ cf) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double c[RSD_REAL_EPI_NC];
  const double s1 = inv_pimu / (6.0 * a), s3 = s1 / (a * a);
  rsd_real_epi_coef_scaled<double>(a, a, phix, s1, s3, c);
  for (int k = 0; k < RSD_REAL_EPI_NC; k++) {
    cr[k] = dsf_from(c[k]);
    cf[k] = (float)c[k];
  }
}

__device__ __forceinline__ int pack_image(int nx, int ny, int nz, int NR) {
  return (nx + NR) | ((ny + NR) << 8) | ((nz + NR) << 16);
}

// FP32 column base of the classification (the same sequence for both sets)
__device__ __forceinline__ void column_base_f(const float* Rf, const float* A, int nx, int ny, float* p) {
  for (int k = 0; k < 3; k++) p[k] = __fmaf_rn(A[3 + k], (float)ny, __fmaf_rn(A[k], (float)nx, Rf[k]));
}

// Lists the next images of the set (near: r2 < rc2; far: rc2 <= r2 < rmax2)
// from the resumable position (col, nz) into list[.][t], at most REAL_CAP;
// returns the count.
template <bool NEAR>
__device__ __forceinline__ int list_images(RealEqShared& sh, int t, const float* Rf, const float* A, int NR, int& col,
                                           int& nz, float rc2, float rmax2) {
  const int w = 2 * NR + 1, ncol = w * w;
  int cnt = 0, nx = 0, ny = 0;
  float p[3];
  bool base = false;
  while (col < ncol && cnt < REAL_CAP) {
    if (!base) {
      nx = col / w - NR;
      ny = col % w - NR;
      column_base_f(Rf, A, nx, ny, p);
      base = true;
    }
    float y0, y1, y2;
    const float r2 = image_r2f(p[0], p[1], p[2], A[6], A[7], A[8], nz, &y0, &y1, &y2);
    if (NEAR ? (r2 < rc2) : (r2 >= rc2 && r2 < rmax2)) sh.list[cnt++][t] = pack_image(nx, ny, nz, NR);
    if (++nz > NR) {
      nz = -NR;
      col++;
      base = false;
    }
  }
  return cnt;
}

// The near images' moments of part P (of NP, rsd_mom_part): one pass over
// the near set, then that part's share of every output added into the pair
// block held in shared memory (oh + ol).
template <int NP, int P>
__device__ __forceinline__ void near_part(RealEqShared& sh, int t, const float* Rf, const float* A, const dsf* Rs,
                                          const dsf* As, int NR, float rc2, dsf lam_s, dsf cd_s) {
  dsacc acc[RSD_NMOM_REAL];
#pragma unroll
  for (int m = 0; m < RSD_NMOM_REAL; m++) acc[m] = dsacc(0);
  int col = 0, nz = -NR;
  do {
    const int cnt = list_images<true>(sh, t, Rf, A, NR, col, nz, rc2, 0.f);
    for (int q = 0; q < cnt; q++) {
      const int e = sh.list[q][t];
      const int ix = (e & 255) - NR, iy = ((e >> 8) & 255) - NR, iz = (e >> 16) - NR;
      const dsf x0 = Rs[0] + ix * As[0] + iy * As[3] + iz * As[6];
      const dsf x1 = Rs[1] + ix * As[1] + iy * As[4] + iz * As[7];
      const dsf x2 = Rs[2] + ix * As[2] + iy * As[5] + iz * As[8];
      const dsf r = dsf_sqrt(x0 * x0 + x1 * x1 + x2 * x2);
      const dsf ir = dsf_rcp(r);
      dsf E0, G;
      dsf_erfc_gauss(lam_s * r, sh.T, &E0, &G);
      rsd_real_image<dsf, dsacc, NP, P>(x0, x1, x2, r, ir, E0, cd_s * G, lam_s, acc);
      if ((q & 3) == 3) {  // keep the accumulators' lo parts small
#pragma unroll
        for (int m = 0; m < RSD_NMOM_REAL; m++) dsacc_norm(acc[m]);
      }
    }
#pragma unroll
    for (int m = 0; m < RSD_NMOM_REAL; m++) dsacc_norm(acc[m]);
  } while (col < (2 * NR + 1) * (2 * NR + 1));
  dsf accn[RSD_NMOM_REAL];
#pragma unroll
  for (int m = 0; m < RSD_NMOM_REAL; m++) accn[m] = dsf(acc[m].hi, acc[m].lo);
#pragma unroll
  for (int q = 0; q < 60; q++) {
    dsacc o = rsd_real_epi_row<dsf, dsf, dsacc, NP, P>(q, accn, sh.cr);
    o += dsf(sh.oh[q][t], sh.ol[q][t]);
    dsacc_norm(o);
    sh.oh[q][t] = o.hi;
    sh.ol[q][t] = o.lo;
  }
}

template <int NP, int P>
__device__ __forceinline__ void near_parts(RealEqShared& sh, int t, const float* Rf, const float* A, const dsf* Rs,
                                           const dsf* As, int NR, float rc2, dsf lam_s, dsf cd_s) {
  if constexpr (P < NP) {
    near_part<NP, P>(sh, t, Rf, A, Rs, As, NR, rc2, lam_s, cd_s);
    near_parts<NP, P + 1>(sh, t, Rf, A, Rs, As, NR, rc2, lam_s, cd_s);
  }
}

// NP: passes over the near images, each summing one part of the moments
// (fewer live accumulators and a shorter loop body per pass, at the cost of
// evaluating r, erfc and exp once per pass); MINB: CTAs per SM to fit.
template <int NP, int MINB>
__global__ void __launch_bounds__(REAL_THREADS, MINB) ewald_pair_real_eq(int nn, rsd_lat_dev L,
                                                                        const double* __restrict__ pos,
                                                                        const dsf* __restrict__ cr_g,
                                                                        const float* __restrict__ cf_g, float rc2,
                                                                        float rmax2, PlaneSink sk) {
  extern __shared__ __align__(16) unsigned char smraw_real[];
  RealEqShared& sh = *reinterpret_cast<RealEqShared*>(smraw_real);
  // blocks entirely on or below the diagonal (a >= b everywhere) have no work
  if ((int)(blockIdx.x * blockDim.x) >= (int)(blockIdx.y * blockDim.y + blockDim.y - 1)) return;
  const int t = threadIdx.y * blockDim.x + threadIdx.x;
  dsf_tables_fill(sh.T, t, REAL_THREADS);
  for (int k = t; k < RSD_REAL_EPI_NC; k += REAL_THREADS) {
    sh.cr[k] = cr_g[k];
    sh.cf[k] = cf_g[k];
  }
  __syncthreads();
  int a, b;
  if (!pair_of(nn, &a, &b)) return;
  float A[9], LIf[9];
  dsf As[9];
#pragma unroll
  for (int k = 0; k < 9; k++) {
    As[k] = dsf_from(L.LR[k]);
    A[k] = As[k].hi;
    LIf[k] = (float)L.LI[k];
  }
  // minimum image: the lattice shift found in FP32, applied in double-single
  const double R[3] = {pos[3 * a] - pos[3 * b], pos[3 * a + 1] - pos[3 * b + 1], pos[3 * a + 2] - pos[3 * b + 2]};
  dsf Rs[3];
  {
    const float R0[3] = {(float)R[0], (float)R[1], (float)R[2]};
    int k[3];
    rsd_skew_shift_f32(A, LIf, R0, k);
#pragma unroll
    for (int i = 0; i < 3; i++) Rs[i] = dsf_from(R[i]) - (k[0] * As[i] + k[1] * As[3 + i] + k[2] * As[6 + i]);
  }
  const float Rf[3] = {Rs[0].hi, Rs[1].hi, Rs[2].hi};
  const int NR = L.NR;
  const float lamf = (float)L.lam, lam2f = lamf * lamf, cdf = (float)(2.0 * RSD_PIP5 * L.lam);
  // far images, FP32
  {
    float acc[RSD_NMOM_REAL];
#pragma unroll
    for (int m = 0; m < RSD_NMOM_REAL; m++) acc[m] = 0.f;
    int col = 0, nz = -NR;
    do {
      const int cnt = list_images<false>(sh, t, Rf, A, NR, col, nz, rc2, rmax2);
      for (int q = 0; q < cnt; q++) {
        const int e = sh.list[q][t];
        const int ix = (e & 255) - NR, iy = ((e >> 8) & 255) - NR, iz = (e >> 16) - NR;
        float p[3], x0, x1, x2;
        column_base_f(Rf, A, ix, iy, p);
        const float r2 = image_r2f(p[0], p[1], p[2], A[6], A[7], A[8], iz, &x0, &x1, &x2);
        const float r = sqrtf(r2), ir = 1.f / r;
        rsd_real_image<float>(x0, x1, x2, r, ir, erfcf(lamf * r), cdf * expf(-r2 * lam2f), lamf, acc);
      }
    } while (col < (2 * NR + 1) * (2 * NR + 1));
#pragma unroll
    for (int q = 0; q < 60; q++) {
      sh.oh[q][t] = rsd_real_epi_row<float, float, float>(q, acc, sh.cf);
      sh.ol[q][t] = 0.f;
    }
  }
  // near images, double-single, in NP passes
  near_parts<NP, 0>(sh, t, Rf, A, Rs, As, NR, rc2, dsf_from(L.lam), dsf_from(2.0 * RSD_PIP5 * L.lam));
  dsf v[60];
#pragma unroll
  for (int q = 0; q < 60; q++) v[q] = dsf(sh.oh[q][t], sh.ol[q][t]);
  store_pair_rows_a(sk, nn, a, b, v, 1);
}


__global__ void __launch_bounds__(128) ewald_pair_real(int nn, rsd_lat_dev L, const double* __restrict__ pos,
                                                       const double* __restrict__ radii, double inv_pimu,
                                                       DenseSink sk) {
  int a, b;
  if (!pair_of(nn, &a, &b)) return;
  double R[3] = {pos[3 * a] - pos[3 * b], pos[3 * a + 1] - pos[3 * b + 1], pos[3 * a + 2] - pos[3 * b + 2]};
  double dmin;
  rsd_skew_correction(L.LR, L.LI, R, &dmin);
  double acc[RSD_NMOM_REAL];
#pragma unroll
  for (int m = 0; m < RSD_NMOM_REAL; m++) acc[m] = 0.0;
  const double lam = L.lam, lam2 = lam * lam, cd = 2.0 * RSD_PIP5 * lam;
  const int NR = L.NR;
  for (int nx = -NR; nx <= NR; nx++)
    for (int ny = -NR; ny <= NR; ny++) {
      double x0 = R[0] + L.LR[0] * nx + L.LR[3] * ny - L.LR[6] * NR;
      double x1 = R[1] + L.LR[1] * nx + L.LR[4] * ny - L.LR[7] * NR;
      double x2 = R[2] + L.LR[2] * nx + L.LR[5] * ny - L.LR[8] * NR;
      for (int nz = -NR; nz <= NR; nz++) {
        const double r2 = x0 * x0 + x1 * x1 + x2 * x2;
        const double r = sqrt(r2), ir = 1.0 / r;
        const double E0 = erfc(lam * r), Ed = cd * exp(-r2 * lam2);
        rsd_real_image<double>(x0, x1, x2, r, ir, E0, Ed, lam, acc);
        x0 += L.LR[6];
        x1 += L.LR[7];
        x2 += L.LR[8];
      }
    }
  double v[60];
  rsd_real_epilogue<double>(acc, radii[a], radii[b], L.phix, v);
  scale_block(v, radii[a], inv_pimu);
  store_pair_d(sk, nn, a, b, v, 1);
}

// Self-image moments.  The real-space images n != 0 of a particle and the
// cos weights of the half space do not depend on the particle (only the
// epilogue does, through its radius), so one CTA sums them once in FP64:
// out[0..96] = real moments, out[97..145] = kcos weights.
constexpr int SELF_NMOM = RSD_NMOM_REAL + RSD_NMOM_KCOS;
constexpr int SELF_THREADS = 128;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__global__ void __launch_bounds__(SELF_THREADS) ewald_self_moments(rsd_lat_dev L, int Kh,
                                                                   const double* __restrict__ tab,
                                                                   double* __restrict__ out) {
  __shared__ double part[SELF_THREADS / 32][SELF_NMOM];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const double lam = L.lam, lam2 = lam * lam, cd = 2.0 * RSD_PIP5 * lam;
  {
    double acc[RSD_NMOM_REAL];
#pragma unroll
    for (int m = 0; m < RSD_NMOM_REAL; m++) acc[m] = 0.0;
    const int NR = L.NR, w = 2 * NR + 1, nimg = w * w * w;
    for (int i = tid; i < nimg; i += SELF_THREADS) {
      const int nx = i / (w * w) - NR, ny = (i / w) % w - NR, nz = i % w - NR;
      if (!nx && !ny && !nz) continue;  // PER_ROTNE_PRAGER_SELF 61
      const double x0 = L.LR[0] * nx + L.LR[3] * ny + L.LR[6] * nz;
      const double x1 = L.LR[1] * nx + L.LR[4] * ny + L.LR[7] * nz;
      const double x2 = L.LR[2] * nx + L.LR[5] * ny + L.LR[8] * nz;
      const double r2 = x0 * x0 + x1 * x1 + x2 * x2, r = sqrt(r2);
      rsd_real_image<double>(x0, x1, x2, r, 1.0 / r, erfc(lam * r), cd * exp(-r2 * lam2), lam, acc);
    }
#pragma unroll
    for (int m = 0; m < RSD_NMOM_REAL; m++) {
      const double v = warp_sum(acc[m]);
      if (lane == 0) part[warp][m] = v;
    }
  }
  {
    double ac[RSD_NMOM_KCOS];
#pragma unroll
    for (int m = 0; m < RSD_NMOM_KCOS; m++) ac[m] = 0.0;
    for (int h = tid; h < Kh; h += SELF_THREADS) {
      const double* e = tab + (size_t)h * KW + 3;
#pragma unroll
      for (int m = 0; m < RSD_NMOM_KCOS; m++) ac[m] += e[m];
    }
#pragma unroll
    for (int m = 0; m < RSD_NMOM_KCOS; m++) {
      const double v = warp_sum(ac[m]);
      if (lane == 0) part[warp][RSD_NMOM_REAL + m] = v;
    }
  }
  __syncthreads();
  for (int m = tid; m < SELF_NMOM; m += SELF_THREADS) {
    double t = 0.0;
    for (int q = 0; q < SELF_THREADS / 32; q++) t += part[q][m];
    out[m] = t;
  }
}

// Diagonal blocks from the self moments (ewald_self_moments) and the
// particle's radius.
__device__ __forceinline__ void sink_put(const DenseSink& sk, int64_t o, double x) { sk.M[o] = x; }
__device__ __forceinline__ void sink_put(const PlaneSink& sk, int64_t o, double x) {
  const dsf d = dsf_from(x);
  sk.hi[o] = d.hi;
  sk.lo[o] = d.lo;
}

template <typename S>
__global__ void __launch_bounds__(64) ewald_self(int nn, rsd_lat_dev L, const double* __restrict__ mom,
                                                 const double* __restrict__ radii, double inv_pimu, S sk) {
  const int64_t ldm = sk.ld;
  auto M = [&](int64_t o, double x) { sink_put(sk, o, x); };
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= nn) return;
  const double ai = radii[a], lam = L.lam;
  double v[60], w[60];
  {
    double acc[RSD_NMOM_REAL];
    for (int m = 0; m < RSD_NMOM_REAL; m++) acc[m] = mom[m];
    rsd_real_epilogue<double>(acc, ai, ai, L.phix, v);
  }
  {
    double ac[RSD_NMOM_KCOS];
    for (int m = 0; m < RSD_NMOM_KCOS; m++) ac[m] = mom[RSD_NMOM_REAL + m];
    rsd_kcos_epilogue<double>(ac, ai, ai, L.phix, w);
  }
  // analytic self terms (Ewald_summation.f90:179-188)
  const double sp = sqrt(RSD_PI), a3 = ai * ai * ai, l3 = lam * lam * lam;
  const double ttsr = 1.0 - 6.0 * lam / sp * ai + 40.0 / 3.0 / sp * l3 * a3 * L.phix;
  const double rrsr = 0.75 - 10.0 / sp * a3 * l3;
  const double qqsr = 0.9 - l3 * a3 / 25.0 / sp * (50.0 - 126.0 * lam * lam * ai * ai) * 6.0;
  for (int q = 0; q < 60; q++) v[q] += w[q] * (2.0 / L.LV);
  v[0] += ttsr;
  v[3] += ttsr;
  v[5] += ttsr;
  v[6] += rrsr;
  v[9] += rrsr;
  v[11] += rrsr;
  const int dq[5] = {15, 20, 24, 27, 29};  // QQ diagonal in the upper-triangle order
  for (int x = 0; x < 5; x++) v[dq[x]] += qqsr;
  scale_block(v, ai, inv_pimu);
  // diagonal block: TT, RR, QQ; TR, G, H are zero (per_GRPY_YZD.f90:63-66)
  const int N = nn;
  const int sym[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      M((3 * a + i) + (int64_t)(3 * a + j) * ldm, v[sym[i][j]]);
      M((3 * N + 3 * a + i) + (int64_t)(3 * N + 3 * a + j) * ldm, v[6 + sym[i][j]]);
      M((3 * a + i) + (int64_t)(3 * N + 3 * a + j) * ldm, 0.0);
      M((3 * N + 3 * a + j) + (int64_t)(3 * a + i) * ldm, 0.0);
    }
  for (int i = 0; i < 3; i++)
    for (int m = 0; m < 5; m++) {
      M((3 * a + i) + (int64_t)(6 * N + 5 * a + m) * ldm, 0.0);
      M((3 * N + 3 * a + i) + (int64_t)(6 * N + 5 * a + m) * ldm, 0.0);
      M((6 * N + 5 * a + m) + (int64_t)(3 * a + i) * ldm, 0.0);
      M((6 * N + 5 * a + m) + (int64_t)(3 * N + 3 * a + i) * ldm, 0.0);
    }
  int q = 15;
  double qq[5][5];
  for (int x = 0; x < 5; x++)
    for (int y = x; y < 5; y++) qq[x][y] = qq[y][x] = v[q++];
  for (int x = 0; x < 5; x++)
    for (int y = 0; y < 5; y++) M((6 * N + 5 * a + x) + (int64_t)(6 * N + 5 * a + y) * ldm, qq[x][y]);
}

__global__ void overlap_count(int nn, rsd_lat_dev L, const double* __restrict__ pos, const double* __restrict__ radii,
                              int* __restrict__ count) {
  int a, b;
  if (!pair_of(nn, &a, &b)) return;
  double R[3] = {pos[3 * a] - pos[3 * b], pos[3 * a + 1] - pos[3 * b + 1], pos[3 * a + 2] - pos[3 * b + 2]};
  double d;
  rsd_skew_correction(L.LR, L.LI, R, &d);
  if (d <= radii[a] + radii[b]) atomicAdd(count, 1);
}

// Overlapping pairs (minimum image with r <= a_i + a_j, the test of
// per_GRPY_YZD.f90:98) into a list of at most cap pairs; count ends at the
// number found.
__global__ void overlap_list(int nn, rsd_lat_dev L, const double* __restrict__ pos, const double* __restrict__ radii,
                             int cap, int2* __restrict__ list, int* __restrict__ count) {
  int a, b;
  if (!pair_of(nn, &a, &b)) return;
  double R[3] = {pos[3 * a] - pos[3 * b], pos[3 * a + 1] - pos[3 * b + 1], pos[3 * a + 2] - pos[3 * b + 2]};
  double d;
  rsd_skew_correction(L.LR, L.LI, R, &d);
  if (d <= radii[a] + radii[b]) {
    const int k = atomicAdd(count, 1);
    if (k < cap) list[k] = make_int2(a, b);
  }
}

// Overlap correction (correction_method 1 or 2) of the listed pairs, one thread
// per pair, added to the assembled blocks at the minimum image: the blocks
// of different pairs are disjoint, so the sum does not depend on the order
// of the list.
template <typename S>
__global__ void __launch_bounds__(64) overlap_correct(int method, int npair, const int2* __restrict__ list, int nn,
                                                       rsd_lat_dev L, const double* __restrict__ pos,
                                                       const double* __restrict__ radii, double inv_pimu, S sk) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= npair) return;
  const int a = list[q].x, b = list[q].y;
  double R[3] = {pos[3 * a] - pos[3 * b], pos[3 * a + 1] - pos[3 * b + 1], pos[3 * a + 2] - pos[3 * b + 2]};
  double d;
  rsd_skew_correction(L.LR, L.LI, R, &d);
  double v[60];
  rsd_overlap_correction60(method, R, radii[a], radii[b], v);
  for (int k = 0; k < 60; k++) v[k] *= inv_pimu;
  store_pair_d(sk, nn, a, b, v, 1);
}

}  // namespace

int rsd_overlap_correct(rsd_ctx* ctx, int method, int precision, int nn, const double* d_pos, const double* d_radii,
                        const rsd_lattice* lat, double mu_f, int npair, double* d_M, int64_t ldm) {
  if (npair <= 0) return RSD_OK;
  const rsd_lat_dev L = rsd_lat_pack(lat);
  int* cnt = (int*)rsd_scratch(ctx, "overlap_count", sizeof(int));
  int2* list = (int2*)rsd_scratch(ctx, "overlap_list", sizeof(int2) * (size_t)npair);
  if (!cnt || !list) return RSD_ENOMEM;
  RSD_CUDA(ctx, cudaMemsetAsync(cnt, 0, sizeof(int), ctx->stream));
  dim3 blk(32, 4), grd((nn + 31) / 32, (nn + 3) / 4);
  overlap_list<<<grd, blk, 0, ctx->stream>>>(nn, L, d_pos, d_radii, npair, list, cnt); RSD_LAUNCH_NOTE();
  const double inv_pimu = 1.0 / (RSD_PI * mu_f);
  const unsigned nblk = (unsigned)((npair + 63) / 64);
  if (precision == RSD_PREC_MIXED) {
    float* hi = reinterpret_cast<float*>(d_M);
    const PlaneSink psk{hi, hi + (size_t)ldm * (11LL * nn), ldm};
    overlap_correct<PlaneSink><<<nblk, 64, 0, ctx->stream>>>(method, npair, list, nn, L, d_pos, d_radii, inv_pimu,
                                                             psk); RSD_LAUNCH_NOTE();
  } else {
    const DenseSink dsk{d_M, ldm};
    overlap_correct<DenseSink><<<nblk, 64, 0, ctx->stream>>>(method, npair, list, nn, L, d_pos, d_radii, inv_pimu,
                                                             dsk); RSD_LAUNCH_NOTE();
  }
  RSD_CUDA(ctx, cudaGetLastError());
  return RSD_OK;
}

int rsd_count_overlaps(rsd_ctx* ctx, int nn, const double* d_pos, const double* d_radii, const rsd_lattice* lat,
                       int* count) {
  rsd_lat_dev L = rsd_lat_pack(lat);
  int* d = (int*)rsd_scratch(ctx, "overlap_count", sizeof(int));
  if (!d) return RSD_ENOMEM;
  RSD_CUDA(ctx, cudaMemsetAsync(d, 0, sizeof(int), ctx->stream));
  dim3 blk(32, 4), grd((nn + 31) / 32, (nn + 3) / 4);
  overlap_count<<<grd, blk, 0, ctx->stream>>>(nn, L, d_pos, d_radii, d); RSD_LAUNCH_NOTE();
  RSD_CUDA(ctx, cudaGetLastError());
  RSD_CUDA(ctx, cudaMemcpyAsync(count, d, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  RSD_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return RSD_OK;
}

// The Ewald sum does not depend on its splitting parameter lambda (checked
// with the oracle: moving lambda by 1.25-2x changes pair blocks by ~3e-15
// when the image cubes hold the sums).  The mixed form moves it by the
// context's mixed_lambda_scale, which trades double-single real-space
// images for cheaper reciprocal vectors, and sizes the cubes to hold its
// truncation spheres: lambda |x| < mixed_rmax, k^2 / (4 lambda^2) <
// mixed_kexp.  With fractional coordinates of the minimum image within
// [-1/2, 1/2], |n_i| <= r_max |b_i| + 1/2 in real space and |n_i| <= k_max
// |a_i| / (2 pi) in reciprocal space (a_i the lattice vectors, b_i their
// reciprocal vectors).  Scale 1 keeps the reference's lambda and cubes.
static rsd_lat_dev mixed_lattice(const rsd_ctx* ctx, rsd_lat_dev L) {
  const double f = ctx->mixed_lambda_scale;
  if (f == 1.0) return L;
  L.lam *= f;
  double amax = 0.0, bmax = 0.0;
  for (int i = 0; i < 3; i++) {
    double a2 = 0.0, b2 = 0.0;
    for (int j = 0; j < 3; j++) {
      a2 += L.LR[j + 3 * i] * L.LR[j + 3 * i];  // column i of LR
      b2 += L.LI[i + 3 * j] * L.LI[i + 3 * j];  // row i of LI
    }
    amax = fmax(amax, sqrt(a2));
    bmax = fmax(bmax, sqrt(b2));
  }
  const double rmax = ctx->mixed_rmax / L.lam, kmax = 2.0 * L.lam * sqrt(ctx->mixed_kexp);
  L.NR = max(L.NR, (int)ceil(rmax * bmax + 0.5));
  L.NI = max(L.NI, (int)ceil(kmax * amax / (2.0 * RSD_PI)));
  return L;
}

namespace {
template <int NP, int MINB>
int launch_real_eq_t(rsd_ctx* ctx, dim3 grd, dim3 blk, int nn, const rsd_lat_dev& L, const double* d_pos,
                     const dsf* cr, const float* cf, float rc2, float rmax2, const PlaneSink& psk) {
  static bool attr = false;
  if (!attr) {
    RSD_CUDA(ctx, cudaFuncSetAttribute(ewald_pair_real_eq<NP, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       SMEM_REAL_EQ));
    attr = true;
  }
  ewald_pair_real_eq<NP, MINB><<<grd, blk, SMEM_REAL_EQ, ctx->stream>>>(nn, L, d_pos, cr, cf, rc2, rmax2, psk); RSD_LAUNCH_NOTE();
  return RSD_OK;
}

int launch_real_eq(rsd_ctx* ctx, int passes, dim3 grd, dim3 blk, int nn, const rsd_lat_dev& L, const double* d_pos,
                   const dsf* cr, const float* cf, float rc2, float rmax2, const PlaneSink& psk) {
  switch (passes) {
    case 1: return launch_real_eq_t<1, 2>(ctx, grd, blk, nn, L, d_pos, cr, cf, rc2, rmax2, psk);
    case 2: return launch_real_eq_t<2, 2>(ctx, grd, blk, nn, L, d_pos, cr, cf, rc2, rmax2, psk);
    case 3: return launch_real_eq_t<3, 2>(ctx, grd, blk, nn, L, d_pos, cr, cf, rc2, rmax2, psk);
    default: return launch_real_eq_t<4, 2>(ctx, grd, blk, nn, L, d_pos, cr, cf, rc2, rmax2, psk);
  }
}
}  // namespace

int rsd_mirror_planes(rsd_ctx* ctx, int nn, double* d_M, int64_t ldm) {
  const int64_t n11 = 11LL * nn;
  float* hi = reinterpret_cast<float*>(d_M);
  const dim3 mt((unsigned)((n11 + 31) / 32), (unsigned)((n11 + 31) / 32));
  mirror_planes<<<mt, dim3(32, 8), 0, ctx->stream>>>(nn, n11, hi, hi + (size_t)ldm * n11, ldm); RSD_LAUNCH_NOTE();
  RSD_CUDA(ctx, cudaGetLastError());
  return RSD_OK;
}

int rsd_ewald_assemble(rsd_ctx* ctx, int nn, const double* d_pos, const double* d_radii, const rsd_lattice* lat,
                       double mu_f, int precision, double* d_M, int64_t ldm) {
  if (nn < 1 || ldm < 11LL * nn) return rsd_fail(ctx, RSD_EARG, "bad size nn=%d ldm=%lld", nn, (long long)ldm);
  rsd_lat_dev L = rsd_lat_pack(lat);
  if (precision == RSD_PREC_MIXED) L = mixed_lattice(ctx, L);
  if (L.NR > 40 || L.NI > 40) return rsd_fail(ctx, RSD_EARG, "image cubes too large (NR=%d NI=%d)", L.NR, L.NI);
  const int w = 2 * L.NI + 1;
  const int Kh = (w * w * w - 1) / 2;
  double* tab = (double*)rsd_scratch(ctx, "ewald_ktab", sizeof(double) * (size_t)Kh * KW);
  if (!tab) return RSD_ENOMEM;
  // FP64 cos/sin per (vector, particle): the FP64 form only (the mixed form
  // keeps its own FP32 and float-pair lists)
  double2* cs = nullptr;
  if (precision != RSD_PREC_MIXED) {
    cs = (double2*)rsd_scratch(ctx, "ewald_trig", sizeof(double2) * (size_t)Kh * nn);
    if (!cs) return RSD_ENOMEM;
  }
  const double inv_pimu = 1.0 / (RSD_PI * mu_f);
  cudaStream_t s = ctx->stream;
  ewald_ktable<<<(Kh + 127) / 128, 128, 0, s>>>(L, Kh, tab); RSD_LAUNCH_NOTE();
  if (precision != RSD_PREC_MIXED) {
    ewald_trig<<<dim3((nn + 127) / 128, Kh), 128, 0, s>>>(nn, Kh, tab, d_pos, cs); RSD_LAUNCH_NOTE();
  }
  double* mom = (double*)rsd_scratch(ctx, "ewald_self_mom", sizeof(double) * SELF_NMOM);
  if (!mom) return RSD_ENOMEM;
  ewald_self_moments<<<1, SELF_THREADS, 0, s>>>(L, Kh, tab, mom); RSD_LAUNCH_NOTE();
  // mixed form: M as FP32 planes hi + lo (PlaneSink), in the buffer of the FP64 matrix
  const DenseSink dsk{d_M, ldm};
  const PlaneSink psk{reinterpret_cast<float*>(d_M), reinterpret_cast<float*>(d_M) + (size_t)ldm * (11LL * nn), ldm};
  if (precision == RSD_PREC_MIXED) {
    ewald_self<<<(nn + 63) / 64, 64, 0, s>>>(nn, L, mom, d_radii, inv_pimu, psk); RSD_LAUNCH_NOTE();
  } else {
    ewald_self<<<(nn + 63) / 64, 64, 0, s>>>(nn, L, mom, d_radii, inv_pimu, dsk); RSD_LAUNCH_NOTE();
  }
  if (nn > 1) {
    dim3 blk(32, 4), grd((nn + 31) / 32, (nn + 3) / 4);
    if (precision == RSD_PREC_MIXED) {
      // Double-single: real images with lambda r < mixed_rcut (default 4.5)
      // and reciprocal vectors with k^2/(4 lambda^2) <= 3 pi mixed_kshell^2
      // (default 1); FP32 for the rest.  The FP32 error of a block follows
      // the largest FP32 term: at the defaults (with lambda x 1.75) a step's
      // velocities move by ~3e-11 and its stresslets by ~2e-10 relative.
      // Truncation: real images with lambda r >= mixed_rmax and reciprocal
      // vectors with k^2 / (4 lambda^2) >= mixed_kexp are dropped (each
      // changes a block by less than ~1e-12 of its largest entry at the
      // defaults 6.0 and 10 pi; the FP64 form keeps the whole cube).
      const double rc = ctx->mixed_rcut / L.lam, rc2 = rc * rc;
      const double rm = ctx->mixed_rmax / L.lam, rmax2 = rm * rm;
      const int ks = ctx->mixed_kshell;
      // double-single reciprocal vectors: k^2 / (4 lambda^2) <= 3 pi ks^2
      // (at the reference's lambda on a cubic cell, ks = 1 is the shell
      // max|n_i| <= 1); FP32 for the others below the truncation
      const double k2ds = 4.0 * L.lam * L.lam * 3.0 * RSD_PI * ks * ks;
      const double k2max = 4.0 * L.lam * L.lam * ctx->mixed_kexp;
      std::vector<int> h64, h32;
      for (int h = 0; h < Kh; h++) {
        int nx, ny, nz;
        half_space_index(h, L.NI, &nx, &ny, &nz);
        double k2 = 0.0;
        for (int j = 0; j < 3; j++) {
          const double kj = 2.0 * RSD_PI * (nx * L.LI[3 * j] + ny * L.LI[1 + 3 * j] + nz * L.LI[2 + 3 * j]);
          k2 += kj * kj;
        }
        if (k2 <= k2ds * (1.0 + 1e-12))
          h64.push_back(h);
        else if (k2 < k2max)
          h32.push_back(h);
      }
      const int K64 = (int)h64.size(), K32 = (int)h32.size();
      int* dh = (int*)rsd_scratch(ctx, "ewald_hlist", sizeof(int) * (size_t)Kh);
      double* t64 = (double*)rsd_scratch(ctx, "ewald_ktab64", sizeof(double) * (size_t)(K64 > 0 ? K64 : 1) * KW);
      float* t32 = (float*)rsd_scratch(ctx, "ewald_ktab32", sizeof(float) * (size_t)(K32 > 0 ? K32 : 1) * KW);
      float4* c64 = (float4*)rsd_scratch(ctx, "ewald_trig64", sizeof(float4) * (size_t)(K64 > 0 ? K64 : 1) * nn);
      float2* c32 = (float2*)rsd_scratch(ctx, "ewald_trig32", sizeof(float2) * (size_t)(K32 > 0 ? K32 : 1) * nn);
      if (!dh || !t64 || !t32 || !c64 || !c32) return RSD_ENOMEM;
      std::vector<int> all(h64);
      all.insert(all.end(), h32.begin(), h32.end());
      RSD_CUDA(ctx, cudaMemcpyAsync(dh, all.data(), sizeof(int) * all.size(), cudaMemcpyHostToDevice, s));
      RSD_CUDA(ctx, cudaStreamSynchronize(s));
      // equal radii: per-vector block weights (ewald_pair_kblock)
      std::vector<double> hr((size_t)nn);
      RSD_CUDA(ctx, cudaMemcpy(hr.data(), d_radii, sizeof(double) * nn, cudaMemcpyDeviceToHost));
      bool equal = true;
      for (int i = 1; i < nn && equal; i++) equal = hr[i] == hr[0];
      if (K64) {
        ewald_trig_list<float4><<<dim3((nn + 127) / 128, K64), 128, 0, s>>>(nn, L, dh, d_pos, c64); RSD_LAUNCH_NOTE();
      }
      if (K32) {
        ewald_trig_list<float2><<<dim3((nn + 127) / 128, K32), 128, 0, s>>>(nn, L, dh + K64, d_pos, c32); RSD_LAUNCH_NOTE();
      }
      if (equal) {
        dsf* w64 = (dsf*)rsd_scratch(ctx, "ewald_kblock64", sizeof(dsf) * (size_t)(K64 > 0 ? K64 : 1) * KBW);
        float* w32 = (float*)rsd_scratch(ctx, "ewald_kblock32", sizeof(float) * (size_t)(K32 > 0 ? K32 : 1) * KBW);
        if (!w64 || !w32) return RSD_ENOMEM;
        if (K64) {
          ewald_kblock_list<dsf><<<(K64 + 127) / 128, 128, 0, s>>>(L, K64, dh, hr[0], inv_pimu, w64); RSD_LAUNCH_NOTE();
        }
        if (K32) {
          ewald_kblock_list<float><<<(K32 + 127) / 128, 128, 0, s>>>(L, K32, dh + K64, hr[0], inv_pimu, w32); RSD_LAUNCH_NOTE();
        }
        ewald_pair_kblock<<<grd, blk, 0, s>>>(nn, K32, w32, c32, K64, w64, c64, psk, 0); RSD_LAUNCH_NOTE();
      } else {
        if (K64) {
          ewald_ktable_list<double><<<(K64 + 127) / 128, 128, 0, s>>>(L, K64, dh, t64); RSD_LAUNCH_NOTE();
        }
        if (K32) {
          ewald_ktable_list<float><<<(K32 + 127) / 128, 128, 0, s>>>(L, K32, dh + K64, t32); RSD_LAUNCH_NOTE();
        }
        ewald_pair_k_ds<<<grd, blk, 0, s>>>(nn, L, K64, t64, c64, d_radii, inv_pimu, psk, 0); RSD_LAUNCH_NOTE();
        ewald_pair_k<float, float2><<<grd, blk, 0, s>>>(nn, L, K32, t32, c32, d_radii, inv_pimu, psk, 1); RSD_LAUNCH_NOTE();
      }
      if (equal) {
        dsf* cr = (dsf*)rsd_scratch(ctx, "ewald_real_cr", sizeof(dsf) * RSD_REAL_EPI_NC);
        float* cf = (float*)rsd_scratch(ctx, "ewald_real_cf", sizeof(float) * RSD_REAL_EPI_NC);
        if (!cr || !cf) return RSD_ENOMEM;
        ewald_real_epi_table<<<1, 32, 0, s>>>(hr[0], L.phix, inv_pimu, cr, cf); RSD_LAUNCH_NOTE();
        RSD_TRY(launch_real_eq(ctx, ctx->mixed_real_passes, grd, blk, nn, L, d_pos, cr, cf, (float)rc2, (float)rmax2, psk));
      } else {
        ewald_pair_real_near_ds<<<grd, blk, 0, s>>>(nn, L, d_pos, d_radii, inv_pimu, rc2, psk); RSD_LAUNCH_NOTE();
        ewald_pair_real_far<<<grd, blk, 0, s>>>(nn, L, d_pos, d_radii, inv_pimu, rc2, rmax2, psk); RSD_LAUNCH_NOTE();
      }
    } else {
      ewald_pair_k<double, double2><<<grd, blk, 0, s>>>(nn, L, Kh, tab, cs, d_radii, inv_pimu, dsk, 0); RSD_LAUNCH_NOTE();
      ewald_pair_real<<<grd, blk, 0, s>>>(nn, L, d_pos, d_radii, inv_pimu, dsk); RSD_LAUNCH_NOTE();
    }
  }
  RSD_CUDA(ctx, cudaGetLastError());
  return RSD_OK;
}
