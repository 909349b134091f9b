// Kernel 2: two-body lubrication resistance R_lub - R_2B (lubmxcalc,
// src/hydro_lub.f90:22-308, with lubcalc 310-398 and lubtabcalc 400-525).
//
// Pipeline (all FP64, deterministic order):
//   lub_count     one warp per particle a: near partners b > a (s <= 4 in
//                 the minimum image), ballot-compacted -> count[a]
//   lub_scan      exclusive scan of the counts (one block)
//   lub_list      the same sweep writes the pair list, sorted by (a, b)
//   lub_pairs     one thread per near pair: the 19 resistance scalars and
//                 the projected two-body blocks (139 values per pair)
//   lub_cross     one thread per (pair, entry): the (a,b) and (b,a) blocks
//   lub_self      one thread per (particle, entry): the sum of the particle's
//                 own blocks over its pairs, in pair order
// The output is the grand layout L = [rfu rfe; rfe^T rse] (11N x 11N),
// scaled by 6 pi mu_f like hydro_lub.f90:304-306, either written over a
// zeroed matrix or added into one (arrangResist, src/matrices.f90:218-228).
#include <cuda_runtime.h>

#include "rsd_internal.cuh"

namespace {

constexpr int PB = 139;  // doubles per pair block
// offsets inside a pair block
constexpr int O_A11 = 0, O_A12 = 9, O_B11 = 18, O_B12 = 27, O_C11 = 36, O_C12 = 45;
constexpr int O_G11 = 54, O_G12 = 69, O_H11 = 84, O_H12 = 99, O_M = 114;

__constant__ double c_Y2[45];  // Y2(m,i,j) at m + 5*(i + 3*j), tensors.f90:43-67

struct lub_dev_tab {
  const double *abc, *gh, *m;
  int nabc, ngh, nm;
};

__device__ void lubcalc_dev(const lub_dev_tab& t, double r, double* o) {
  if (r < 2.1) {
    const double xi = r - 2.0, invxi = 1.0 / xi, loginvxi = log(invxi), xiloginvxi = xi * loginvxi;
    o[0] = -1.23041 + 0.25 * invxi + 1.8918 * xi + 9.0 * loginvxi / 40.0 + 3.0 * xiloginvxi / 112.0;
    o[1] = -o[0] + 0.00312 - 0.0011 * xi;
    o[2] = -0.39394 + 0.95665 * xi + loginvxi / 6.0;
    o[3] = -o[2] + 0.004636 - 0.007049 * xi;
    o[4] = 0.408286 - 0.84055 * xi - loginvxi / 6.0 - xiloginvxi / 12.0;
    o[5] = -0.405978 + 0.833042 * xi + loginvxi / 6.0 + xiloginvxi / 12.0;
    o[6] = 0.0479 + 0.12494 * xi - xiloginvxi / 6.0;
    o[7] = -o[6] + 0.016869 + 0.049536 * xi;
    o[8] = -0.605434 + 0.939139 * xi + 4.0 * loginvxi / 15.0 + 94.0 * xiloginvxi / 375.0;
    o[9] = loginvxi / 15.0 + 62.0 * xiloginvxi / 375.0 - 0.219032 + 0.332843 * xi;
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
  for (int q = 0; q < 19; q++) o[q] = 0.0;
  for (int i = 0; i < t.nabc - 1; i++) {
    const double* a = t.abc + 11 * i;
    const double* b = a + 11;
    if (a[0] <= r && b[0] > r) {
      for (int q = 0; q < 10; q++) o[q] = a[q + 1] + (r - a[0]) * (b[q + 1] - a[q + 1]) / (b[0] - a[0]);
      break;
    }
  }
  for (int i = 0; i < t.ngh - 1; i++) {
    const double* a = t.gh + 7 * i;
    const double* b = a + 7;
    if (a[0] <= r && b[0] > r) {
      for (int q = 0; q < 6; q++) o[10 + q] = a[q + 1] + (r - a[0]) * (b[q + 1] - a[q + 1]) / (b[0] - a[0]);
      break;
    }
  }
  for (int i = 0; i < t.nm - 1; i++) {
    const double* a = t.m + 4 * i;
    const double* b = a + 4;
    if (a[0] <= r && b[0] > r) {
      for (int q = 0; q < 3; q++) o[16 + q] = (a[q + 1] + (r - a[0]) * (b[q + 1] - a[q + 1]) / (b[0] - a[0])) / 2.0;
      break;
    }
  }
}

__device__ inline double eps3(int i, int j, int k) {
  return (double)((i - j) * (j - k) * (k - i)) / 2.0;  // Levi-Civita for 0..2
}

__device__ inline bool near_pair(const rsd_lat_dev& L, int is_period, const double* pos, const double* radii, int a,
                                 int b) {
  double R[3] = {pos[3 * a] - pos[3 * b], pos[3 * a + 1] - pos[3 * b + 1], pos[3 * a + 2] - pos[3 * b + 2]};
  {  // FP32 screen: pairs clearly beyond the cut-off need no FP64 test
    float LRf[9], LIf[9], Rf[3] = {(float)R[0], (float)R[1], (float)R[2]};
    for (int k = 0; k < 9; k++) {
      LRf[k] = (float)L.LR[k];
      LIf[k] = (float)L.LI[k];
    }
    float d2;
    if (is_period) {
      int k[3];
      rsd_skew_shift_f32(LRf, LIf, Rf, k);
      d2 = 0.f;
      for (int i = 0; i < 3; i++) {
        const float e = Rf[i] - (LRf[i] * k[0] + LRf[i + 3] * k[1] + LRf[i + 6] * k[2]);
        d2 += e * e;
      }
    } else {
      d2 = Rf[0] * Rf[0] + Rf[1] * Rf[1] + Rf[2] * Rf[2];
    }
    const float lim = 2.0f * (float)(radii[a] + radii[b]) * 1.001f + 1e-3f;  // s = 4 with a margin
    if (d2 > lim * lim) return false;
  }
  double r = sqrt(R[0] * R[0] + R[1] * R[1] + R[2] * R[2]);
  if (is_period) rsd_skew_correction(L.LR, L.LI, R, &r);
  const double s = r / (0.5 * (radii[a] + radii[b]));
  return !(s > 4.0);
}

__global__ void lub_count(int nn, int nb, int is_period, rsd_lat_dev L, const double* __restrict__ pos,
                          const double* __restrict__ radii, int* __restrict__ count) {
  const int a = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32, lane = threadIdx.x & 31;
  if (a >= nn) return;
  int c = 0;
  if (a < nn - nb) {
    for (int b0 = a + 1; b0 < nn; b0 += 32) {
      const int b = b0 + lane;
      const bool nr = b < nn && near_pair(L, is_period, pos, radii, a, b);
      c += __popc(__ballot_sync(0xffffffffu, nr));
    }
  }
  if (lane == 0) count[a] = c;
}

// exclusive scan of count[0..n) into off[0..n], one block of 1024 threads
__global__ void lub_scan(int n, const int* __restrict__ count, int* __restrict__ off) {
  __shared__ int part[1024];
  const int t = threadIdx.x;
  const int per = (n + 1023) / 1024;
  const int lo = t * per, hi = min(n, lo + per);
  int s = 0;
  for (int i = lo; i < hi; i++) s += count[i];
  part[t] = s;
  __syncthreads();
  for (int d = 1; d < 1024; d <<= 1) {
    int v = t >= d ? part[t - d] : 0;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  int base = t ? part[t - 1] : 0;
  for (int i = lo; i < hi; i++) {
    off[i] = base;
    base += count[i];
  }
  if (t == 1023) off[n] = part[1023];
}

__global__ void lub_list(int nn, int nb, int is_period, rsd_lat_dev L, const double* __restrict__ pos,
                         const double* __restrict__ radii, const int* __restrict__ off, int2* __restrict__ pairs) {
  const int a = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32, lane = threadIdx.x & 31;
  if (a >= nn || a >= nn - nb) return;
  int w = off[a];
  for (int b0 = a + 1; b0 < nn; b0 += 32) {
    const int b = b0 + lane;
    const bool nr = b < nn && near_pair(L, is_period, pos, radii, a, b);
    const unsigned m = __ballot_sync(0xffffffffu, nr);
    if (nr) pairs[w + __popc(m & ((1u << lane) - 1))] = make_int2(a, b);
    w += __popc(m);
  }
}

// rtd_front: C(m,c) = sum_ij T3(i,j,c) Y2(m,i,j)   (tensors.f90:966-978)
__device__ inline void front_y2(const double T3[27], double* C /*5x3, m + 5c*/) {
  for (int m = 0; m < 5; m++)
    for (int c = 0; c < 3; c++) {
      double v = 0.0;
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) v += T3[i + 3 * j + 9 * c] * c_Y2[m + 5 * (i + 3 * j)];
      C[m + 5 * c] = v;
    }
}

__global__ void lub_pairs(int npair, lub_dev_tab tab, int is_period, rsd_lat_dev L, const double* __restrict__ pos,
                          const double* __restrict__ radii, const int2* __restrict__ pairs, double* __restrict__ blk,
                          int* __restrict__ contacts) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npair) return;
  const int a = pairs[p].x, b = pairs[p].y;
  double R[3] = {pos[3 * a] - pos[3 * b], pos[3 * a + 1] - pos[3 * b + 1], pos[3 * a + 2] - pos[3 * b + 2]};
  double r = sqrt(R[0] * R[0] + R[1] * R[1] + R[2] * R[2]);
  if (is_period) rsd_skew_correction(L.LR, L.LI, R, &r);
  double s = r / (0.5 * (radii[a] + radii[b]));
  if (s <= 2.0) {  // hydro_lub.f90:85-92: report and mirror
    atomicAdd(contacts, 1);
    s = 4.00001 - s;
  }
  double o[19];
  lubcalc_dev(tab, s, o);
  const double x11a = o[0], x12a = o[1], y11a = o[2], y12a = o[3], y11b = o[4], y12b = o[5], x11c = o[6],
               x12c = o[7], y11c = o[8], y12c = o[9], x11g = o[10], x12g = o[11], y11g = o[12], y12g = o[13],
               y11h = o[14], y12h = o[15], xm = o[16], ym = o[17], zm = o[18];
  const double e[3] = {R[0] / r, R[1] / r, R[2] / r};
  double* B = blk + (size_t)p * PB;
  auto kd = [](int i, int j) { return i == j ? 1.0 : 0.0; };
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < 3; i++) {
      const double ee = e[i] * e[j], d = kd(i, j);
      const double pe = eps3(i, j, 0) * e[0] + eps3(i, j, 1) * e[1] + eps3(i, j, 2) * e[2];
      B[O_A11 + i + 3 * j] = x11a * ee + y11a * (d - ee);
      B[O_A12 + i + 3 * j] = x12a * ee + y12a * (d - ee);
      B[O_B11 + i + 3 * j] = y11b * pe;
      B[O_B12 + i + 3 * j] = y12b * pe;
      B[O_C11 + i + 3 * j] = x11c * ee + y11c * (d - ee);
      B[O_C12 + i + 3 * j] = x12c * ee + y12c * (d - ee);
    }
  double g11[27], g12[27], h11[27], h12[27];
  for (int k = 0; k < 3; k++)
    for (int j = 0; j < 3; j++)
      for (int i = 0; i < 3; i++) {
        const double t1 = (e[i] * e[j] - kd(i, j) / 3.0) * e[k];
        const double t2 = e[i] * kd(j, k) + e[j] * kd(i, k) - 2 * e[i] * e[j] * e[k];
        const int q = i + 3 * j + 9 * k;
        g11[q] = x11g * t1 + y11g * t2;
        g12[q] = x12g * t1 + y12g * t2;
        const double pik = eps3(i, k, 0) * e[0] + eps3(i, k, 1) * e[1] + eps3(i, k, 2) * e[2];
        const double pjk = eps3(j, k, 0) * e[0] + eps3(j, k, 1) * e[1] + eps3(j, k, 2) * e[2];
        h11[q] = y11h * (pik * e[j] + pjk * e[i]);
        h12[q] = y12h * (pik * e[j] + pjk * e[i]);
      }
  front_y2(g11, B + O_G11);
  front_y2(g12, B + O_G12);
  front_y2(h11, B + O_H11);
  front_y2(h12, B + O_H12);
  // mlub (hydro_lub.f90:136-142) projected on Y2 x Y2 (DD_transY2)
  double mm[25];
  for (int x = 0; x < 25; x++) mm[x] = 0.0;
  for (int l = 0; l < 3; l++)
    for (int k = 0; k < 3; k++)
      for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) {
          const double t = xm * (3.0 * (e[i] * e[j] - kd(i, j) / 3.0) * (e[k] * e[l] - kd(k, l) / 3.0) / 2.0) +
                           ym * (e[i] * kd(j, l) * e[k] + e[j] * kd(i, l) * e[k] + e[i] * kd(j, k) * e[l] +
                                 e[j] * kd(i, k) * e[l] - 4.0 * e[i] * e[j] * e[k] * e[l]) / 2.0 +
                           zm * (kd(i, k) * kd(j, l) + kd(j, k) * kd(i, l) - kd(i, j) * kd(k, l) + e[i] * e[j] * kd(k, l) +
                                 kd(i, j) * e[k] * e[l] - e[i] * kd(j, l) * e[k] - e[j] * kd(i, l) * e[k] -
                                 e[i] * kd(j, k) * e[l] - e[j] * kd(i, k) * e[l] + e[i] * e[j] * e[k] * e[l]) / 2.0;
          if (t == 0.0) continue;
          for (int x = 0; x < 5; x++) {
            const double yx = c_Y2[x + 5 * (i + 3 * j)];
            if (yx == 0.0) continue;
            for (int y = 0; y < 5; y++) mm[x + 5 * y] += t * yx * c_Y2[y + 5 * (k + 3 * l)];
          }
        }
  for (int x = 0; x < 25; x++) B[O_M + x] = mm[x];
}

__device__ inline void lput(double* L, int64_t ld, int r, int c, double v, int acc) {
  double* p = L + (int64_t)r + (int64_t)c * ld;
  *p = acc ? *p + v : v;
}

// grand-layout index of component k (0..10) of particle part
__device__ inline int gidx(int N, int part, int k) {
  return k < 3 ? 3 * part + k : (k < 6 ? 3 * N + 3 * part + k - 3 : 6 * N + 5 * part + k - 6);
}

// Entry (r, c) of the (a,b) particle block (ab = true) or of the (b,a)
// block (ab = false) of pair block B, r and c in 0..10.
__device__ inline double pair_entry(const double* B, int r, int c, bool ab) {
  if (r < 3 && c < 3) return ab ? B[O_A12 + r + 3 * c] : B[O_A12 + c + 3 * r];  // TT, (b,a) mirrored
  if (r >= 3 && r < 6 && c >= 3 && c < 6)                                          // RR
    return ab ? B[O_C12 + (r - 3) + 3 * (c - 3)] : B[O_C12 + (c - 3) + 3 * (r - 3)];
  if (r >= 3 && r < 6 && c < 3) return (ab ? 1.0 : -1.0) * B[O_B12 + (r - 3) + 3 * c];   // RT: b12, b21 = -b12
  if (r < 3 && c >= 3 && c < 6) return (ab ? -1.0 : 1.0) * B[O_B12 + (c - 3) + 3 * r];   // TR = RT^T
  if (r >= 6 && c < 3) return (ab ? 1.0 : -1.0) * B[O_G12 + (r - 6) + 5 * c];            // G: g12, -g12
  if (r < 3 && c >= 6) return (ab ? -1.0 : 1.0) * B[O_G12 + (c - 6) + 5 * r];            // rfe = QP^T
  if (r >= 6 && c >= 3 && c < 6) return B[O_H12 + (r - 6) + 5 * (c - 3)];               // H: h12 both ways
  if (r >= 3 && r < 6 && c >= 6) return B[O_H12 + (c - 6) + 5 * (r - 3)];
  return B[O_M + (r - 6) + 5 * (c - 6)];                                                 // QQ: mmx both ways
}

// Entry (r, c) of a particle's own block contributed by pair block B;
// sgn = +1 when the particle is the pair's first, -1 when its second.
__device__ inline double self_entry(const double* B, int r, int c, double sgn) {
  if (r < 3 && c < 3) return B[O_A11 + r + 3 * c];
  if (r >= 3 && r < 6 && c >= 3 && c < 6) return B[O_C11 + (r - 3) + 3 * (c - 3)];
  if (r >= 3 && r < 6 && c < 3) return sgn * B[O_B11 + (r - 3) + 3 * c];
  if (r < 3 && c >= 3 && c < 6) return sgn * B[O_B11 + (c - 3) + 3 * r];
  if (r >= 6 && c < 3) return sgn * B[O_G11 + (r - 6) + 5 * c];
  if (r < 3 && c >= 6) return sgn * B[O_G11 + (c - 6) + 5 * r];
  if (r >= 6 && c >= 3 && c < 6) return B[O_H11 + (r - 6) + 5 * (c - 3)];
  if (r >= 3 && r < 6 && c >= 6) return B[O_H11 + (c - 6) + 5 * (r - 3)];
  return B[O_M + (r - 6) + 5 * (c - 6)];
}

// 121 entries of the (a,b) block and 121 of the (b,a) block per pair
__global__ void lub_cross(int npair, int N, const int2* __restrict__ pairs, const double* __restrict__ blk,
                          double scale, double* __restrict__ L, int64_t ld, int acc) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)npair * 121) return;
  const int p = (int)(t / 121), e = (int)(t % 121);
  const int a = pairs[p].x, b = pairs[p].y;
  const double* B = blk + (size_t)p * PB;
  const int r = e % 11, c = e / 11;  // position inside an 11x11 particle block
  lput(L, ld, gidx(N, a, r), gidx(N, b, c), pair_entry(B, r, c, true) * scale, acc);
  lput(L, ld, gidx(N, b, r), gidx(N, a, c), pair_entry(B, r, c, false) * scale, acc);
}

// Second-particle lists: for each particle u, the pairs (a,u) with a < u,
// in pair order (which is a-ascending, the order lubmxcalc adds them in).
__global__ void lub_second_count(int npair, const int2* __restrict__ pairs, int* __restrict__ cnt2) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < npair) atomicAdd(&cnt2[pairs[p].y], 1);
}

__global__ void lub_second_fill(int npair, const int2* __restrict__ pairs, const int* __restrict__ off2,
                                int* __restrict__ cur, int* __restrict__ list2) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npair) return;
  const int b = pairs[p].y;
  list2[off2[b] + atomicAdd(&cur[b], 1)] = p;
}

__global__ void lub_second_sort(int nn, const int* __restrict__ off2, int* __restrict__ list2) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= nn) return;
  for (int i = off2[u] + 1; i < off2[u + 1]; i++) {
    const int v = list2[i];
    int j = i - 1;
    while (j >= off2[u] && list2[j] > v) {
      list2[j + 1] = list2[j];
      j--;
    }
    list2[j + 1] = v;
  }
}

// self block of particle u: its pairs as second particle, then as first,
// in the order lubmxcalc visits them.  Written into L (grand layout) or,
// when L is null, into self[u * 121 + r + 11 c].
__global__ void lub_self(int N, const int* __restrict__ off, const int* __restrict__ off2,
                         const int* __restrict__ list2, const double* __restrict__ blk, double scale,
                         double* __restrict__ L, int64_t ld, int acc, double* __restrict__ self) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)N * 121) return;
  const int u = (int)(t / 121), e = (int)(t % 121);
  const int r = e % 11, c = e / 11;
  double v = 0.0;
  for (int q = off2[u]; q < off2[u + 1]; q++) v += self_entry(blk + (size_t)list2[q] * PB, r, c, -1.0);
  for (int q = off[u]; q < off[u + 1]; q++) v += self_entry(blk + (size_t)q * PB, r, c, 1.0);
  if (L)
    lput(L, ld, gidx(N, u, r), gidx(N, u, c), v * scale, acc);
  else
    self[t] = v * scale;
}

// y = L w for the sparse operator: the particle's self block, then its pairs
// as first and as second particle.  One warp per (particle, right-hand
// side): lane r + 11 g (r < 11, g < 2) takes row r and every other
// neighbour block starting at g; the two halves are added by a shuffle
// (fixed order)
__global__ void lub_spmv_w(int N, const int* __restrict__ off, const int* __restrict__ off2,
                           const int* __restrict__ list2, const int2* __restrict__ pairs,
                           const double* __restrict__ blk, const double* __restrict__ self, double scale, int nr,
                           const double* __restrict__ w, int64_t ldw, double* __restrict__ y, int64_t ldy) {
  const int64_t wid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (wid >= (int64_t)N * nr) return;
  const int u = (int)(wid % N), col = (int)(wid / N);
  const int r = lane % 11, g = lane / 11;
  const double* wc = w + col * ldw;
  double vs = 0.0, vp = 0.0;
  if (g < 2) {
    if (g == 0) {
      const double* S = self + (size_t)u * 121;
#pragma unroll
      for (int c = 0; c < 11; c++) vs += S[r + 11 * c] * wc[gidx(N, u, c)];
    }
    const int p1 = off[u], n1 = off[u + 1] - p1, q2 = off2[u], n2 = off2[u + 1] - q2;
    for (int k = g; k < n1 + n2; k += 2) {
      const bool first = k < n1;
      const int p = first ? p1 + k : list2[q2 + k - n1];
      const double* B = blk + (size_t)p * PB;
      const int o = first ? pairs[p].y : pairs[p].x;
#pragma unroll
      for (int c = 0; c < 11; c++) vp += pair_entry(B, r, c, first) * wc[gidx(N, o, c)];
    }
  }
  vp += __shfl_down_sync(0xffffffffu, vp, 11);
  if (lane < 11) y[gidx(N, u, r) + col * ldy] = vs + vp * scale;
}

// A (FP32, ld lda) += the force/torque-velocity part L_PP of the sparse
// operator: pair blocks (each entry of A is touched by at most one pair or
// self block, so no two threads add to the same entry)
__global__ void lub_pp_pairs(int npair, int N, const int2* __restrict__ pairs, const double* __restrict__ blk,
                             double scale, float* __restrict__ A, int64_t lda) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)npair * 36) return;
  const int p = (int)(t / 36), e = (int)(t % 36);
  const int r = e % 6, c = e / 6;
  const int a = pairs[p].x, b = pairs[p].y;
  const double* B = blk + (size_t)p * PB;
  A[gidx(N, a, r) + gidx(N, b, c) * lda] += (float)(pair_entry(B, r, c, true) * scale);
  A[gidx(N, b, r) + gidx(N, a, c) * lda] += (float)(pair_entry(B, r, c, false) * scale);
}

__global__ void lub_pp_self(int N, const double* __restrict__ self, float* __restrict__ A, int64_t lda) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)N * 36) return;
  const int u = (int)(t / 36), e = (int)(t % 36);
  const int r = e % 6, c = e / 6;
  A[gidx(N, u, r) + gidx(N, u, c) * lda] += (float)self[(size_t)u * 121 + r + 11 * c];
}

__global__ void zero_matrix(int64_t rows, int64_t cols, double* __restrict__ A, int64_t ld) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= rows * cols) return;
  A[(t % rows) + (t / rows) * ld] = 0.0;
}

}  // namespace

static double* lubtab_device(rsd_ctx* ctx, const rsd_lubtab* tab) {
  rsd_lubtab* t = const_cast<rsd_lubtab*>(tab);
  auto it = t->dev.find(ctx->device);
  if (it != t->dev.end()) return it->second;
  double* d = nullptr;
  const size_t n = 64 * 11 + 64 * 7 + 64 * 4;
  if (cudaMalloc(&d, n * sizeof(double)) != cudaSuccess) return nullptr;
  cudaMemcpy(d, t->abc, 64 * 11 * sizeof(double), cudaMemcpyHostToDevice);
  cudaMemcpy(d + 64 * 11, t->gh, 64 * 7 * sizeof(double), cudaMemcpyHostToDevice);
  cudaMemcpy(d + 64 * 18, t->m, 64 * 4 * sizeof(double), cudaMemcpyHostToDevice);
  t->dev[ctx->device] = d;
  return d;
}

// The pair stage shared by the dense and the sparse assembly: near-pair
// list, pair blocks (unscaled), second-particle lists and contact count.
static int lub_pair_stage(rsd_ctx* ctx, const rsd_lubtab* tab, int nn, int nb, int is_period, const double* d_pos,
                          const double* d_radii, const rsd_lattice* lat, rsd_lub_sparse* sp, int* dcon) {
  static bool y2_ready = false;
  if (!y2_ready) {
    double Y[45] = {0};
    const double s2 = 1.0 / sqrt(2.0), s6 = 1.0 / sqrt(6.0);
    auto at = [&](int m, int i, int j) -> double& { return Y[m + 5 * (i + 3 * j)]; };
    at(0, 0, 1) = at(0, 1, 0) = s2;
    at(1, 1, 2) = at(1, 2, 1) = -s2;
    at(2, 0, 0) = at(2, 1, 1) = -s6;
    at(2, 2, 2) = sqrt(2.0 / 3.0);
    at(3, 0, 2) = at(3, 2, 0) = -s2;
    at(4, 0, 0) = s2;
    at(4, 1, 1) = -s2;
    RSD_CUDA(ctx, cudaMemcpyToSymbol(c_Y2, Y, sizeof Y));
    y2_ready = true;
  }
  double* dt = lubtab_device(ctx, tab);
  if (!dt) return rsd_fail(ctx, RSD_ENOMEM, "lub table upload failed");
  lub_dev_tab T{dt, dt + 64 * 11, dt + 64 * 18, tab->nabc, tab->ngh, tab->nm};
  rsd_lat_dev Ld = rsd_lat_pack(lat);
  cudaStream_t s = ctx->stream;
  int* cnt = (int*)rsd_scratch(ctx, "lub_count", sizeof(int) * (nn + 1));
  int* off = (int*)rsd_scratch(ctx, "lub_off", sizeof(int) * (nn + 1));
  if (!cnt || !off) return RSD_ENOMEM;
  const int wpb = 8;
  lub_count<<<(nn + wpb - 1) / wpb, 32 * wpb, 0, s>>>(nn, nb, is_period, Ld, d_pos, d_radii, cnt); RSD_LAUNCH_NOTE();
  lub_scan<<<1, 1024, 0, s>>>(nn, cnt, off); RSD_LAUNCH_NOTE();
  int npair = 0;
  RSD_CUDA(ctx, cudaMemcpyAsync(&npair, off + nn, sizeof(int), cudaMemcpyDeviceToHost, s));
  RSD_CUDA(ctx, cudaStreamSynchronize(s));
  int2* pairs = (int2*)rsd_scratch(ctx, "lub_pairs", sizeof(int2) * (size_t)(npair > 0 ? npair : 1));
  double* blk = (double*)rsd_scratch(ctx, "lub_blocks", sizeof(double) * PB * (size_t)(npair > 0 ? npair : 1));
  int* cnt2 = (int*)rsd_scratch(ctx, "lub_count2", sizeof(int) * (nn + 1));
  int* off2 = (int*)rsd_scratch(ctx, "lub_off2", sizeof(int) * (nn + 1));
  int* cur = (int*)rsd_scratch(ctx, "lub_cur", sizeof(int) * (nn + 1));
  int* list2 = (int*)rsd_scratch(ctx, "lub_list2", sizeof(int) * (size_t)(npair > 0 ? npair : 1));
  if (!pairs || !blk || !cnt2 || !off2 || !cur || !list2) return RSD_ENOMEM;
  RSD_CUDA(ctx, cudaMemsetAsync(dcon, 0, sizeof(int), s));
  RSD_CUDA(ctx, cudaMemsetAsync(cnt2, 0, sizeof(int) * (nn + 1), s));
  RSD_CUDA(ctx, cudaMemsetAsync(cur, 0, sizeof(int) * (nn + 1), s));
  if (npair > 0) {
    lub_list<<<(nn + wpb - 1) / wpb, 32 * wpb, 0, s>>>(nn, nb, is_period, Ld, d_pos, d_radii, off, pairs); RSD_LAUNCH_NOTE();
    lub_pairs<<<(npair + 127) / 128, 128, 0, s>>>(npair, T, is_period, Ld, d_pos, d_radii, pairs, blk, dcon); RSD_LAUNCH_NOTE();
    lub_second_count<<<(npair + 255) / 256, 256, 0, s>>>(npair, pairs, cnt2); RSD_LAUNCH_NOTE();
    lub_scan<<<1, 1024, 0, s>>>(nn, cnt2, off2); RSD_LAUNCH_NOTE();
    lub_second_fill<<<(npair + 255) / 256, 256, 0, s>>>(npair, pairs, off2, cur, list2); RSD_LAUNCH_NOTE();
    lub_second_sort<<<(nn + 127) / 128, 128, 0, s>>>(nn, off2, list2); RSD_LAUNCH_NOTE();
  } else {
    RSD_CUDA(ctx, cudaMemsetAsync(off2, 0, sizeof(int) * (nn + 1), s));
  }
  sp->nn = nn;
  sp->npair = npair;
  sp->pairs = pairs;
  sp->blk = blk;
  sp->off = off;
  sp->off2 = off2;
  sp->list2 = list2;
  return RSD_OK;
}

int rsd_lub_assemble(rsd_ctx* ctx, const rsd_lubtab* tab, int nn, int nb, int is_period, const double* d_pos,
                     const double* d_radii, const rsd_lattice* lat, double mu_f, double* d_L, int64_t ldl,
                     int accumulate, int* n_contact) {
  if (!tab) return rsd_fail(ctx, RSD_EARG, "no lubrication tables");
  if (nn < 1 || ldl < 11LL * nn) return rsd_fail(ctx, RSD_EARG, "bad size nn=%d ldl=%lld", nn, (long long)ldl);
  int* dcon = (int*)rsd_scratch(ctx, "lub_contacts", sizeof(int) * 2);
  if (!dcon) return RSD_ENOMEM;
  cudaStream_t s = ctx->stream;
  if (!accumulate) {
    const int64_t tot = 121LL * nn * nn;
    zero_matrix<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(11LL * nn, 11LL * nn, d_L, ldl); RSD_LAUNCH_NOTE();
  }
  rsd_lub_sparse sp;
  RSD_TRY(lub_pair_stage(ctx, tab, nn, nb, is_period, d_pos, d_radii, lat, &sp, dcon));
  const double scale = 6.0 * (RSD_PI * mu_f);
  if (sp.npair > 0) {
    const int64_t tc = 121LL * sp.npair;
    lub_cross<<<(unsigned)((tc + 255) / 256), 256, 0, s>>>(sp.npair, nn, sp.pairs, sp.blk, scale, d_L, ldl, 1); RSD_LAUNCH_NOTE();
    const int64_t ts = 121LL * nn;
    lub_self<<<(unsigned)((ts + 255) / 256), 256, 0, s>>>(nn, sp.off, sp.off2, sp.list2, sp.blk, scale, d_L, ldl, 1,
                                                            nullptr); RSD_LAUNCH_NOTE();
  }
  RSD_CUDA(ctx, cudaGetLastError());
  if (n_contact) {
    RSD_CUDA(ctx, cudaMemcpyAsync(n_contact, dcon, sizeof(int), cudaMemcpyDeviceToHost, s));
    RSD_CUDA(ctx, cudaStreamSynchronize(s));
  }
  return RSD_OK;
}

// Sparse form for the mixed-precision refinement: the same pair blocks and
// the per-particle self blocks (scaled), no dense 11N x 11N matrix.
int rsd_lub_build_sparse(rsd_ctx* ctx, const rsd_lubtab* tab, int nn, int nb, int is_period, const double* d_pos,
                         const double* d_radii, const rsd_lattice* lat, double mu_f, rsd_lub_sparse* sp,
                         int* n_contact) {
  if (!tab) return rsd_fail(ctx, RSD_EARG, "no lubrication tables");
  if (nn < 1) return rsd_fail(ctx, RSD_EARG, "bad size nn=%d", nn);
  int* dcon = (int*)rsd_scratch(ctx, "lub_contacts", sizeof(int) * 2);
  double* self = (double*)rsd_scratch(ctx, "lub_self_blocks", sizeof(double) * 121 * (size_t)nn);
  if (!dcon || !self) return RSD_ENOMEM;
  cudaStream_t s = ctx->stream;
  RSD_TRY(lub_pair_stage(ctx, tab, nn, nb, is_period, d_pos, d_radii, lat, sp, dcon));
  sp->scale = 6.0 * (RSD_PI * mu_f);
  sp->self = self;
  const int64_t ts = 121LL * nn;
  lub_self<<<(unsigned)((ts + 255) / 256), 256, 0, s>>>(nn, sp->off, sp->off2, sp->list2, sp->blk, sp->scale,
                                                          nullptr, 0, 0, self); RSD_LAUNCH_NOTE();
  RSD_CUDA(ctx, cudaGetLastError());
  if (n_contact) {
    RSD_CUDA(ctx, cudaMemcpyAsync(n_contact, dcon, sizeof(int), cudaMemcpyDeviceToHost, s));
    RSD_CUDA(ctx, cudaStreamSynchronize(s));
  }
  return RSD_OK;
}

// y (11N x nr, grand layout, ld ldy) = L w
int rsd_lub_spmv(rsd_ctx* ctx, const rsd_lub_sparse* sp, int nr, const double* w, int64_t ldw, double* y,
                 int64_t ldy) {
  const int64_t tot = 32LL * sp->nn * nr;  // one warp per particle and right-hand side
  lub_spmv_w<<<(unsigned)((tot + 255) / 256), 256, 0, ctx->stream>>>(sp->nn, sp->off, sp->off2, sp->list2, sp->pairs,
                                                                      sp->blk, sp->self, sp->scale, nr, w, ldw, y,
                                                                      ldy); RSD_LAUNCH_NOTE();
  RSD_CUDA(ctx, cudaGetLastError());
  return RSD_OK;
}

// A (6N x 6N FP32, ld lda) += L_PP
int rsd_lub_add_pp_f32(rsd_ctx* ctx, const rsd_lub_sparse* sp, float* A, int64_t lda) {
  cudaStream_t s = ctx->stream;
  if (sp->npair > 0) {
    const int64_t tp = 36LL * sp->npair;
    lub_pp_pairs<<<(unsigned)((tp + 255) / 256), 256, 0, s>>>(sp->npair, sp->nn, sp->pairs, sp->blk, sp->scale, A,
                                                              lda); RSD_LAUNCH_NOTE();
  }
  const int64_t ts = 36LL * sp->nn;
  lub_pp_self<<<(unsigned)((ts + 255) / 256), 256, 0, s>>>(sp->nn, sp->self, A, lda); RSD_LAUNCH_NOTE();
  RSD_CUDA(ctx, cudaGetLastError());
  return RSD_OK;
}
