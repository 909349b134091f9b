// Allocation-free variant of the grand-mobility assembly (the kernel of
// rsd_per_grpery_inv_fri_dev), for callers that cannot call cudaMalloc:
// applications that hand all device memory to their own fixed pool at start
// (a Fortran driver with a static memory budget, a framework with a caching
// allocator), and loops that must not pay the device-wide synchronisation
// cudaMalloc and cudaFree imply.  The caller still passes inputs and outputs;
// the only scratch, the table of reciprocal-vector weights, lives in the
// file-scope array below.
//
// Limits and sharing:
//   - at most RSD_NOALLOC_MAX_KVEC reciprocal vectors in the half space, i.e.
//     NI <= 8.  In a cubic box NI = int(sqrt(-ln(EWS_ERR)/pi)) + 1, so that
//     holds for EWS_ERR above about 5e-88; a sheared lattice has a larger NI
//     for the same EWS_ERR, so there EWS_ERR must stay above a larger value.  Larger requests return
//     RSD_ELIMIT before any kernel that writes the output runs;
//   - every GPU that loads the library holds the array (~1.6 MB) until the
//     process exits;
//   - every call on a device uses the same array and it keeps the last
//     call's contents; calls that overlap on the GPU (other streams, other
//     host threads) race on it and must be serialised by the caller;
//   - the first call on a device looks the array's address up with
//     cudaGetSymbolAddress, with that device current;
//   - the call reads the radii's cube sum back to the host (one small
//     synchronous copy on `stream`) to derive NR, NI and phi.
// The pair kernel evaluates sincos(k.R) per pair instead of reading the
// per-particle trig table the allocating path keeps.
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <cstring>

#include "ewald_gen.cuh"
#include "rsd_internal.cuh"

#define RSD_NOALLOC_MAX_KVEC 2456  // ((2*8+1)^3 - 1) / 2
#define RSD_NOALLOC_KW (3 + RSD_NMOM_KCOS + RSD_NMOM_KSIN)
#define RSD_NOALLOC_DOUBLES (RSD_NOALLOC_MAX_KVEC * RSD_NOALLOC_KW + 64)

static __device__ __align__(256) double rsd_noalloc_scratch[RSD_NOALLOC_DOUBLES];

namespace {

constexpr int NA_MAXDEV = 64;
// device address of rsd_noalloc_scratch, per device; host threads making
// their first calls at the same time each look it up and store the same value
std::atomic<double*> g_scratch[NA_MAXDEV] = {};

__device__ inline void na_half_space_index(int h, int NI, int* nx, int* ny, int* nz) {
  const int w = 2 * NI + 1;
  const int q = (w * w * w - 1) / 2 + 1 + h;
  *nx = q / (w * w) - NI;
  *ny = (q / w) % w - NI;
  *nz = q % w - NI;
}

__global__ void na_sum_cubes(int nn, const double* __restrict__ radii, double* __restrict__ out) {
  __shared__ double red[256];
  double s = 0.0;
  for (int i = threadIdx.x; i < nn; i += blockDim.x) s += radii[i] * radii[i] * radii[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int d = 128; d > 0; d >>= 1) {
    if (threadIdx.x < d) red[threadIdx.x] += red[threadIdx.x + d];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

__global__ void na_ktable(rsd_lat_dev L, int Kh, double* __restrict__ tab) {
  const int h = blockIdx.x * blockDim.x + threadIdx.x;
  if (h >= Kh) return;
  int nx, ny, nz;
  na_half_space_index(h, L.NI, &nx, &ny, &nz);
  double k[3];
  for (int j = 0; j < 3; j++)
    k[j] = 2.0 * RSD_PI * (nx * L.LI[0 + 3 * j] + ny * L.LI[1 + 3 * j] + nz * L.LI[2 + 3 * j]);
  const double k2 = k[0] * k[0] + k[1] * k[1] + k[2] * k[2], l2 = L.lam * L.lam;
  const double S = 8.0 * RSD_PI * (1.0 + k2 / (4.0 * l2) + k2 * k2 / (8.0 * l2 * l2)) * exp(-k2 / (4.0 * l2)) / (k2 * k2);
  double* e = tab + (size_t)h * RSD_NOALLOC_KW;
  e[0] = k[0];
  e[1] = k[1];
  e[2] = k[2];
  rsd_kcos_weights<double>(k[0], k[1], k[2], S, L.lam, e + 3);
  rsd_ksin_weights<double>(k[0], k[1], k[2], S, L.lam, e + 3 + RSD_NMOM_KCOS);
}

__device__ inline void na_scale(double* v, double ai, double inv_pimu) {
  const double na = inv_pimu / (6.0 * ai), na3 = inv_pimu / (6.0 * ai * ai * ai);
  for (int q = 0; q < 60; q++) {
    const bool a3 = (q >= 6 && q < 12) || (q >= 15 && q < 30) || q >= 45;
    v[q] *= a3 ? na3 : na;
  }
}

// (a,b) block and its (b,a) mirror in the grand layout (per_GRPY_YZD.f90:123-188)
__device__ inline void na_store(double* __restrict__ M, int64_t ld, int N, int a, int b, const double* v, int add) {
  auto put = [&](int r, int c, double x) {
    double* p = M + (int64_t)r + (int64_t)c * ld;
    *p = add ? *p + x : x;
  };
  const int sym[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      const double tt = v[sym[i][j]], rr = v[6 + sym[i][j]];
      double tr = 0.0;
      if (i < j) tr = v[12 + (i == 0 ? j - 1 : 2)];
      if (i > j) tr = -v[12 + (j == 0 ? i - 1 : 2)];
      put(3 * a + i, 3 * b + j, tt);
      put(3 * b + i, 3 * a + j, tt);
      put(3 * N + 3 * a + i, 3 * N + 3 * b + j, rr);
      put(3 * N + 3 * b + i, 3 * N + 3 * a + j, rr);
      put(3 * a + i, 3 * N + 3 * b + j, tr);
      put(3 * N + 3 * b + j, 3 * a + i, tr);
      put(3 * b + i, 3 * N + 3 * a + j, -tr);
      put(3 * N + 3 * a + j, 3 * b + i, -tr);
    }
  for (int i = 0; i < 3; i++)
    for (int m = 0; m < 5; m++) {
      const double g = v[30 + 5 * i + m], h = v[45 + 5 * i + m];
      put(3 * a + i, 6 * N + 5 * b + m, g);
      put(3 * N + 3 * a + i, 6 * N + 5 * b + m, h);
      put(6 * N + 5 * b + m, 3 * a + i, g);
      put(6 * N + 5 * b + m, 3 * N + 3 * a + i, h);
      put(3 * b + i, 6 * N + 5 * a + m, -g);
      put(3 * N + 3 * b + i, 6 * N + 5 * a + m, h);
      put(6 * N + 5 * a + m, 3 * b + i, -g);
      put(6 * N + 5 * a + m, 3 * N + 3 * b + i, h);
    }
  double qq[5][5];
  int q = 15;
  for (int x = 0; x < 5; x++)
    for (int y = x; y < 5; y++) qq[x][y] = qq[y][x] = v[q++];
  for (int x = 0; x < 5; x++)
    for (int y = 0; y < 5; y++) {
      put(6 * N + 5 * a + x, 6 * N + 5 * b + y, qq[x][y]);
      put(6 * N + 5 * b + x, 6 * N + 5 * a + y, qq[x][y]);
    }
}

// one thread per unordered pair a < b: reciprocal sum (sincos per k) then
// real-space sum over the image cube, written once
__global__ void __launch_bounds__(128) na_pair(int nn, rsd_lat_dev L, int Kh, const double* __restrict__ tab,
                                               const double* __restrict__ pos, const double* __restrict__ radii,
                                               double inv_pimu, double* __restrict__ M, int64_t ldm) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y * blockDim.y + threadIdx.y;
  if (a >= nn || b >= nn || a >= b) return;
  const double ai = radii[a], aj = radii[b];
  double v[60];
  {
    double ac[RSD_NMOM_KCOS], as[RSD_NMOM_KSIN];
    for (int m = 0; m < RSD_NMOM_KCOS; m++) ac[m] = 0.0;
    for (int m = 0; m < RSD_NMOM_KSIN; m++) as[m] = 0.0;
    const double D0 = pos[3 * a] - pos[3 * b], D1 = pos[3 * a + 1] - pos[3 * b + 1], D2 = pos[3 * a + 2] - pos[3 * b + 2];
    for (int h = 0; h < Kh; h++) {
      const double* e = tab + (size_t)h * RSD_NOALLOC_KW;
      double sn, c;
      sincos(e[0] * D0 + e[1] * D1 + e[2] * D2, &sn, &c);
      for (int m = 0; m < RSD_NMOM_KCOS; m++) ac[m] = fma(e[3 + m], c, ac[m]);
      for (int m = 0; m < RSD_NMOM_KSIN; m++) as[m] = fma(e[3 + RSD_NMOM_KCOS + m], sn, as[m]);
    }
    double w[60];
    rsd_kcos_epilogue<double>(ac, ai, aj, L.phix, v);
    rsd_ksin_epilogue<double>(as, ai, aj, L.phix, w);
    for (int q = 0; q < 60; q++) v[q] = (v[q] + w[q]) * (2.0 / L.LV);
  }
  {
    double R[3] = {pos[3 * a] - pos[3 * b], pos[3 * a + 1] - pos[3 * b + 1], pos[3 * a + 2] - pos[3 * b + 2]};
    double dmin;
    rsd_skew_correction(L.LR, L.LI, R, &dmin);
    double acc[RSD_NMOM_REAL];
    for (int m = 0; m < RSD_NMOM_REAL; m++) acc[m] = 0.0;
    const double lam = L.lam, cd = 2.0 * RSD_PIP5 * lam;
    for (int nx = -L.NR; nx <= L.NR; nx++)
      for (int ny = -L.NR; ny <= L.NR; ny++)
        for (int nz = -L.NR; nz <= L.NR; nz++) {
          const double x0 = R[0] + L.LR[0] * nx + L.LR[3] * ny + L.LR[6] * nz;
          const double x1 = R[1] + L.LR[1] * nx + L.LR[4] * ny + L.LR[7] * nz;
          const double x2 = R[2] + L.LR[2] * nx + L.LR[5] * ny + L.LR[8] * nz;
          const double r2 = x0 * x0 + x1 * x1 + x2 * x2, r = sqrt(r2);
          rsd_real_image<double>(x0, x1, x2, r, 1.0 / r, erfc(lam * r), cd * exp(-r2 * lam * lam), lam, acc);
        }
    double w[60];
    rsd_real_epilogue<double>(acc, ai, aj, L.phix, w);
    for (int q = 0; q < 60; q++) v[q] += w[q];
  }
  na_scale(v, ai, inv_pimu);
  na_store(M, ldm, nn, a, b, v, 0);
}

// self blocks (PER_ROTNE_PRAGER_SELF, Ewald_summation.f90:19-191)
__global__ void __launch_bounds__(64) na_self(int nn, rsd_lat_dev L, int Kh, const double* __restrict__ tab,
                                              const double* __restrict__ radii, double inv_pimu,
                                              double* __restrict__ M, int64_t ldm) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= nn) return;
  const double ai = radii[a], lam = L.lam, cd = 2.0 * RSD_PIP5 * lam;
  double v[60], w[60];
  {
    double acc[RSD_NMOM_REAL];
    for (int m = 0; m < RSD_NMOM_REAL; m++) acc[m] = 0.0;
    for (int nx = -L.NR; nx <= L.NR; nx++)
      for (int ny = -L.NR; ny <= L.NR; ny++)
        for (int nz = -L.NR; nz <= L.NR; nz++) {
          if (!nx && !ny && !nz) continue;
          const double x0 = L.LR[0] * nx + L.LR[3] * ny + L.LR[6] * nz;
          const double x1 = L.LR[1] * nx + L.LR[4] * ny + L.LR[7] * nz;
          const double x2 = L.LR[2] * nx + L.LR[5] * ny + L.LR[8] * nz;
          const double r2 = x0 * x0 + x1 * x1 + x2 * x2, r = sqrt(r2);
          rsd_real_image<double>(x0, x1, x2, r, 1.0 / r, erfc(lam * r), cd * exp(-r2 * lam * lam), lam, acc);
        }
    rsd_real_epilogue<double>(acc, ai, ai, L.phix, v);
  }
  {
    double ac[RSD_NMOM_KCOS];
    for (int m = 0; m < RSD_NMOM_KCOS; m++) ac[m] = 0.0;
    for (int h = 0; h < Kh; h++)
      for (int m = 0; m < RSD_NMOM_KCOS; m++) ac[m] += tab[(size_t)h * RSD_NOALLOC_KW + 3 + m];
    rsd_kcos_epilogue<double>(ac, ai, ai, L.phix, w);
  }
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
  const int dq[5] = {15, 20, 24, 27, 29};
  for (int x = 0; x < 5; x++) v[dq[x]] += qqsr;
  na_scale(v, ai, inv_pimu);
  const int N = nn;
  const int sym[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      M[(3 * a + i) + (int64_t)(3 * a + j) * ldm] = v[sym[i][j]];
      M[(3 * N + 3 * a + i) + (int64_t)(3 * N + 3 * a + j) * ldm] = v[6 + sym[i][j]];
      M[(3 * a + i) + (int64_t)(3 * N + 3 * a + j) * ldm] = 0.0;
      M[(3 * N + 3 * a + j) + (int64_t)(3 * a + i) * ldm] = 0.0;
    }
  for (int i = 0; i < 3; i++)
    for (int m = 0; m < 5; m++) {
      M[(3 * a + i) + (int64_t)(6 * N + 5 * a + m) * ldm] = 0.0;
      M[(3 * N + 3 * a + i) + (int64_t)(6 * N + 5 * a + m) * ldm] = 0.0;
      M[(6 * N + 5 * a + m) + (int64_t)(3 * a + i) * ldm] = 0.0;
      M[(6 * N + 5 * a + m) + (int64_t)(3 * N + 3 * a + i) * ldm] = 0.0;
    }
  double qq[5][5];
  int q = 15;
  for (int x = 0; x < 5; x++)
    for (int y = x; y < 5; y++) qq[x][y] = qq[y][x] = v[q++];
  for (int x = 0; x < 5; x++)
    for (int y = 0; y < 5; y++) M[(6 * N + 5 * a + x) + (int64_t)(6 * N + 5 * a + y) * ldm] = qq[x][y];
}

}  // namespace

extern "C" int rsd_per_grpery_inv_fri_static(int32_t nn, const double* d_pos, const double* d_radii,
                                             rsd_lattice* lat, double ews_err, double mu_f, double* d_grmobmx,
                                             int64_t ldm, void* stream) {
  if (nn < 1 || !d_pos || !d_radii || !lat || !d_grmobmx || ldm < 11LL * nn || !(mu_f > 0)) return RSD_EARG;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NA_MAXDEV) return RSD_ECUDA;
  double* scratch = g_scratch[dev].load(std::memory_order_acquire);
  if (!scratch) {
    // set-up, once per device, with that device current
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, rsd_noalloc_scratch) != cudaSuccess || !p) {
      cudaGetLastError();
      return RSD_ECUDA;
    }
    scratch = (double*)p;
    g_scratch[dev].store(scratch, std::memory_order_release);
  }
  cudaStream_t s = (cudaStream_t)stream;
  // the cube sum of the radii is the only value that starts the call at
  // zero; it is written whole by one block, so nothing needs clearing
  double* d_sum = scratch + RSD_NOALLOC_MAX_KVEC * RSD_NOALLOC_KW;
  na_sum_cubes<<<1, 256, 0, s>>>(nn, d_radii, d_sum); RSD_LAUNCH_NOTE();
  double sum_a3 = 0.0;
  if (cudaMemcpyAsync(&sum_a3, d_sum, sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return RSD_ECUDA;
  int rc = rsd_lattice_params(lat, ews_err, sum_a3);
  if (rc != RSD_OK) return rc;
  const int w = 2 * lat->NI + 1;
  const int Kh = (w * w * w - 1) / 2;
  if (Kh > RSD_NOALLOC_MAX_KVEC) return RSD_ELIMIT;  // nothing launched beyond the radii sum
  rsd_lat_dev L{};
  for (int i = 0; i < 9; i++) {
    L.LR[i] = lat->LR[i];
    L.LI[i] = lat->LI[i];
  }
  L.LV = lat->LV;
  L.lam = lat->lammda;
  L.phix = 1 - 0.2 * lat->phi;
  L.NR = lat->NR;
  L.NI = lat->NI;
  const double inv_pimu = 1.0 / (RSD_PI * mu_f);
  na_ktable<<<(Kh + 127) / 128, 128, 0, s>>>(L, Kh, scratch); RSD_LAUNCH_NOTE();
  na_self<<<(nn + 63) / 64, 64, 0, s>>>(nn, L, Kh, scratch, d_radii, inv_pimu, d_grmobmx, ldm); RSD_LAUNCH_NOTE();
  if (nn > 1) {
    dim3 blk(32, 4), grd((nn + 31) / 32, (nn + 3) / 4);
    na_pair<<<grd, blk, 0, s>>>(nn, L, Kh, scratch, d_pos, d_radii, inv_pimu, d_grmobmx, ldm); RSD_LAUNCH_NOTE();
  }
  return cudaGetLastError() == cudaSuccess ? RSD_OK : RSD_ECUDA;
}
