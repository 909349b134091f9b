// Tensor-core (tcgen05) GEMM on K-major FP32 operands for the FP32
// factorisations of the mixed-precision form:
//     C(128-tiles) = alpha * A^T B   (TMA store)     or
//     C(128-tiles) += alpha * A^T B  (TMA reduce-add),
// where A (K x M) and B (K x N) are column-major with K contiguous, i.e. both
// MMA operands are K-major.  Products are TF32 (PREC 1) or 3xTF32 (PREC 3:
// each operand split into a TF32 head and an FP32 tail, hi*hi + hi*lo +
// lo*hi, about 2^-21 relative per product) with FP32 accumulation in tensor
// memory.
//
// One CTA per 128 x 128 output tile, six warps:
//   warp 0      TMEM allocation; lane 0 issues the TMA loads of 32-wide K
//               chunks of A and B into 128B-swizzled stages;
//   warp 1      lane 0 issues tcgen05.mma (K = 8 each) and commits each
//               stage back to the producer, then the whole tile;
//   warps 2-5   (PREC 3) split each landed stage into head and tail in
//               shared memory; then the epilogue: tcgen05.ld of the
//               accumulator (TMEM lane = output row), alpha * D staged
//               column-major in shared memory, one TMA store or reduce-add.
// Options per launch: skip the tiles strictly below the diagonal, and start
// the K range of a tile at its first column (for triangular operands whose
// rows below that are zero).
//
// Every mbarrier wait is bounded by the global timer (the context's wait
// limit, 0.5 s by default); a timeout sets an abort flag that ends every
// role's loop, records a code in *err, waits (bounded by 0.5 s) for the TMA
// copies and the MMAs already issued, frees the tensor memory and skips the
// store.  The host turns the code into RSD_ETIMEOUT.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <cstring>

#include "rsd_internal.cuh"

namespace {

constexpr int TC_TILE = 128, TC_KC = 32;
constexpr int TC_CHUNK = TC_TILE * TC_KC * 4;  // one operand chunk: 16 KB
constexpr int TC_THREADS = 192;
constexpr unsigned long long TC_WAIT_NS = 500ull * 1000 * 1000;  // 0.5 s per wait

// PREC 1: three 32 KB stages, so that two CTAs share an SM and one CTA's
// epilogue (TMEM -> shared -> TMA store) overlaps the other's main loop;
// PREC 3: three 64 KB stages (heads and tails), one CTA per SM.
template <int PREC>
struct TcCfg {
  static constexpr int STAGES = 3;
  static constexpr int MIN_CTAS = PREC == 1 ? 2 : 1;
  static constexpr int STAGE_BYTES = (PREC == 1 ? 2 : 4) * TC_CHUNK;
  static constexpr int BAR_BYTES = (3 * STAGES + 1) * 8 + 16;
  static constexpr int SMEM = STAGES * STAGE_BYTES + BAR_BYTES + 1024;
};
static_assert(TcCfg<1>::STAGES * TcCfg<1>::STAGE_BYTES >= TC_TILE * TC_TILE * 4, "epilogue staging");
static_assert(TcCfg<3>::STAGES * TcCfg<3>::STAGE_BYTES >= TC_TILE * TC_TILE * 4, "epilogue staging");

struct TcArgs {
  int K;         // K extent of the operand maps
  int tri;       // skip tiles with row0 > col0
  int klo_col;   // K range of a tile starts at its first column
  int reduce;    // 1: C += alpha D (reduce-add), 0: C = alpha D (store)
  int ksplit;    // > 0: CTA z sums K in [z ksplit, (z + 1) ksplit) (a multiple of TC_KC; reduce = 1)
  float alpha;
  int* err;
  unsigned long long wait_ns;  // bound of each mbarrier wait
  // batches (ksplit = 0): CTA z adds z times these to the coordinates of A
  // (k, m), B (k, n) and C (m, n); the batch's n extent is n - z * ndec
  int zak, zam, zbk, zbn, zcm, zcn, ncols, ndec;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait; false on a timeout (which raises the abort flag) or when
// another role has aborted.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int* abort_flag, int* err,
                                          int code, unsigned long long limit_ns) {
  const uint64_t t0 = global_ns();
  while (!mbar_try_wait(bar, parity)) {
    if (*abort_flag) return false;
    if (global_ns() - t0 > limit_ns) {
      *abort_flag = 1;
      atomicExch(err, code);
      return false;
    }
  }
  return true;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}

__device__ __forceinline__ void tma_load(uint32_t dst, const CUtensorMap* tm, int x, int y, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

// Shared-memory matrix descriptor of a K-major operand with the 128-byte
// swizzle: rows of 128 B, 8-row groups 1024 B apart (stride byte offset),
// leading byte offset unused inside one swizzle atom, descriptor version
// 0b001 at bits 46-48, swizzle mode 2 (128 B) at bits 61-63.
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFF) >> 4);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(1024 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

// kind::tf32 instruction descriptor: D = F32 (bits 4-5), A = B = TF32
// (bits 7-9, 10-12), both K-major (bits 15, 16 clear), N >> 3 at bits
// 17-22, M >> 4 at bits 24-28.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t taddr, uint32_t a, uint32_t b, uint32_t acc) {
  constexpr uint32_t idesc = idesc_tf32(TC_TILE, TC_TILE);
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(taddr),
      "l"(smem_desc_sw128(a)), "l"(smem_desc_sw128(b)), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

template <int PREC>
__global__ void __launch_bounds__(TC_THREADS, TcCfg<PREC>::MIN_CTAS)
    tc_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                   const __grid_constant__ CUtensorMap tmC, const TcArgs a) {
  using Cfg = TcCfg<PREC>;
  constexpr int ST = Cfg::STAGES, SB = Cfg::STAGE_BYTES;
  const int row0 = blockIdx.x * TC_TILE, col0 = blockIdx.y * TC_TILE;
  if (a.tri && row0 > col0) return;
  const int z = a.ksplit > 0 ? 0 : (int)blockIdx.z;
  if (a.ndec > 0 && col0 >= a.ncols - z * a.ndec) return;  // beyond this batch's columns
  const int ak = z * a.zak, am = row0 + z * a.zam, bk = z * a.zbk, bn = col0 + z * a.zbn;
  const int cm = row0 + z * a.zcm, cn = col0 + z * a.zcn;
  int klo = a.klo_col ? col0 : 0, khi = a.K;
  if (a.ksplit > 0) {
    klo = max(klo, (int)blockIdx.z * a.ksplit);
    khi = min(khi, ((int)blockIdx.z + 1) * a.ksplit);
  }
  const int nch = khi > klo ? (khi - klo + TC_KC - 1) / TC_KC : 0;

  extern __shared__ unsigned char smraw[];
  unsigned char* base = (unsigned char*)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  uint64_t* bars = (uint64_t*)(base + ST * SB);  // full[ST], conv[ST], empty[ST], done
  uint32_t* tslot = (uint32_t*)(bars + 3 * ST + 1);
  __shared__ volatile int abort_flag;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t sbase = smem_u32(base);
  const uint32_t bar0 = smem_u32(bars);
  // barrier addresses: full[s], conv[s], empty[s], done
#define TC_FULL(s) (bar0 + 8u * (uint32_t)(s))
#define TC_CONV(s) (bar0 + 8u * (uint32_t)(ST + (s)))
#define TC_EMPTY(s) (bar0 + 8u * (uint32_t)(2 * ST + (s)))
  const uint32_t done = bar0 + 8u * (uint32_t)(3 * ST);

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "r"(TC_TILE));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (threadIdx.x == 32) {
    for (int s = 0; s < ST; s++) {
      mbar_init(TC_FULL(s), 1);
      mbar_init(TC_CONV(s), 128);
      mbar_init(TC_EMPTY(s), 1);
    }
    mbar_init(done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;");
    abort_flag = 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t taddr = *tslot;

  if (warp == 0) {
    if (lane == 0) {  // TMA producer
      int last[ST];
      for (int s = 0; s < ST; s++) last[s] = -1;
      for (int c = 0; c < nch; c++) {
        const int s = c % ST;
        if (c >= ST && !mbar_wait(TC_EMPTY(s), ((c / ST) - 1) & 1, &abort_flag, a.err, 1, a.wait_ns)) break;
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(TC_FULL(s)), "r"(2 * TC_CHUNK)
                     : "memory");
        const uint32_t st = sbase + s * SB;
        tma_load(st, &tmA, ak + klo + c * TC_KC, am, TC_FULL(s));
        tma_load(st + TC_CHUNK, &tmB, bk + klo + c * TC_KC, bn, TC_FULL(s));
        last[s] = c;
      }
      if (abort_flag) {  // let the copies already issued land before the CTA exits
        for (int s = 0; s < ST; s++)
          if (last[s] >= 0) {
            const uint64_t t0 = global_ns();
            while (!mbar_try_wait(TC_FULL(s), (last[s] / ST) & 1) && global_ns() - t0 < TC_WAIT_NS) {
            }
          }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {  // MMA issuer
      bool ok = true;
      int issued = 0;
      for (int c = 0; c < nch; c++) {
        const int s = c % ST;
        ok = mbar_wait(PREC == 3 ? TC_CONV(s) : TC_FULL(s), (c / ST) & 1, &abort_flag, a.err, 2, a.wait_ns);
        if (!ok) break;
        issued = c + 1;
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t st = sbase + s * SB;
#pragma unroll
        for (int kk = 0; kk < TC_KC / 8; kk++) {
          const uint32_t ah = st + kk * 32, bh = st + TC_CHUNK + kk * 32;
          mma_tf32(taddr, ah, bh, (c | kk) ? 1u : 0u);
          if (PREC == 3) {
            const uint32_t al = st + 2 * TC_CHUNK + kk * 32, bl = st + 3 * TC_CHUNK + kk * 32;
            mma_tf32(taddr, ah, bl, 1u);
            mma_tf32(taddr, al, bh, 1u);
          }
        }
        mma_commit(TC_EMPTY(s));
      }
      // `done` completes once every MMA issued here has finished (after an
      // abort too, so that the tensor memory is not freed under them)
      if (issued > 0) {
        mma_commit(done);
      } else {
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(done) : "memory");
      }
    }
  } else {
    const int t = threadIdx.x - 64;  // 0..127
    if (PREC == 3) {  // split each landed stage into TF32 head and tail
      for (int c = 0; c < nch; c++) {
        const int s = c % ST;
        if (!mbar_wait(TC_FULL(s), (c / ST) & 1, &abort_flag, a.err, 3, a.wait_ns)) break;
        unsigned char* st = base + s * SB;
#pragma unroll
        for (int op = 0; op < 2; op++) {
          float4* hi = reinterpret_cast<float4*>(st + op * TC_CHUNK);
          float4* lo = reinterpret_cast<float4*>(st + (2 + op) * TC_CHUNK);
#pragma unroll
          for (int q = 0; q < TC_CHUNK / 16 / 128; q++) {
            const int idx = t + 128 * q;
            const float4 v = hi[idx];
            float4 h, l;
            h.x = __uint_as_float(__float_as_uint(v.x) & 0xffffe000u);
            h.y = __uint_as_float(__float_as_uint(v.y) & 0xffffe000u);
            h.z = __uint_as_float(__float_as_uint(v.z) & 0xffffe000u);
            h.w = __uint_as_float(__float_as_uint(v.w) & 0xffffe000u);
            l.x = v.x - h.x;
            l.y = v.y - h.y;
            l.z = v.z - h.z;
            l.w = v.w - h.w;
            hi[idx] = h;
            lo[idx] = l;
          }
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(TC_CONV(s)) : "memory");
      }
    }
    // epilogue
    // warp-uniform: tcgen05.ld is a warp-collective instruction
    const bool ok = __all_sync(0xffffffffu, mbar_wait(done, 0, &abort_flag, a.err, 4, a.wait_ns) ? 1 : 0) != 0;
    if (ok) {
      asm volatile("tcgen05.fence::after_thread_sync;");
      float* sOut = reinterpret_cast<float*>(base);
      const int q = warp & 3;  // this warp may read TMEM lanes 32q..32q+31
      const int row = 32 * q + lane;
      const uint32_t lane_addr = taddr + ((uint32_t)(32 * q) << 16);
      const bool has = nch > 0;
#pragma unroll 1
      for (int cc = 0; cc < TC_TILE / 32; cc++) {
        uint32_t v[32];
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
            "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
            : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
              "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
              "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
              "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
            : "r"(lane_addr + (uint32_t)(cc * 32)));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int j = 0; j < 32; j++) sOut[(cc * 32 + j) * TC_TILE + row] = has ? a.alpha * __uint_as_float(v[j]) : 0.f;
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    asm volatile("bar.sync 1, 128;" ::: "memory");
    if (t == 0 && ok && !abort_flag && (nch > 0 || !a.reduce)) {
      const uint64_t tm = reinterpret_cast<uint64_t>(&tmC);
      if (a.reduce) {
        asm volatile(
            "cp.reduce.async.bulk.tensor.2d.global.shared::cta.add.tile.bulk_group [%0, {%1, %2}], [%3];" ::"l"(tm),
            "r"(cm), "r"(cn), "r"(sbase)
            : "memory");
      } else {
        asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];" ::"l"(tm),
                     "r"(cm), "r"(cn), "r"(sbase)
                     : "memory");
      }
      asm volatile("cp.async.bulk.commit_group;" ::: "memory");
      asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    }
  }
#undef TC_FULL
#undef TC_CONV
#undef TC_EMPTY
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) {
    if (abort_flag) {  // MMAs issued before an abort may still run: wait (bounded) for `done`
      if (lane == 0) {
        const uint64_t t0 = global_ns();
        while (!mbar_try_wait(done, 0) && global_ns() - t0 < TC_WAIT_NS) {
        }
      }
      __syncwarp();
      asm volatile("tcgen05.fence::after_thread_sync;");
    }
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(TC_TILE));
  }
}

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

int tc_init(rsd_ctx* ctx) {
  if (g_encode) return RSD_OK;
  cudaDriverEntryPointQueryResult q;
  void* fn = nullptr;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      !fn || q != cudaDriverEntryPointSuccess) {
    cudaGetLastError();
    return rsd_fail(ctx, RSD_EUNSUP, "cuTensorMapEncodeTiled is not available");
  }
  RSD_CUDA(ctx, cudaFuncSetAttribute(tc_gemm_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, TcCfg<1>::SMEM));
  RSD_CUDA(ctx, cudaFuncSetAttribute(tc_gemm_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, TcCfg<3>::SMEM));
  g_encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
  return RSD_OK;
}

int encode_2d(rsd_ctx* ctx, CUtensorMap* tm, const float* ptr, uint64_t inner, uint64_t outer, uint64_t ld,
              uint32_t box_inner, uint32_t box_outer, CUtensorMapSwizzle sw) {
  memset(tm, 0, sizeof *tm);
  const cuuint64_t dims[2] = {(cuuint64_t)inner, (cuuint64_t)outer};
  const cuuint64_t strides[1] = {(cuuint64_t)(ld * sizeof(float))};
  const cuuint32_t box[2] = {box_inner, box_outer};
  const cuuint32_t estr[2] = {1, 1};
  CUresult r = g_encode(tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)ptr, dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return rsd_fail(ctx, RSD_EUNSUP, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return RSD_OK;
}

bool aligned16(const void* p) { return ((uintptr_t)p & 15) == 0; }

unsigned long long wait_limit(const rsd_ctx* ctx) {
  return ctx->tc_wait_ns > 0 ? (unsigned long long)ctx->tc_wait_ns : TC_WAIT_NS;
}

}  // namespace

// Nonzero when the tensor-core trailing update applies: 16-byte aligned
// panel and trailing block, leading dimensions a multiple of 4 floats (the
// TMA stride rule) and 0 < kb <= 128.
int rsd_tc_syrk_ok(const float* panel, int64_t lda, const float* C, int64_t ldc, int kb) {
  return aligned16(panel) && aligned16(C) && (lda % 4 == 0) && (ldc % 4 == 0) && kb > 0 && kb <= TC_TILE;
}

int rsd_tc_gemm_ok(const float* A, int64_t lda, const float* B, int64_t ldb, const float* C, int64_t ldc) {
  return aligned16(A) && aligned16(B) && aligned16(C) && lda % 4 == 0 && ldb % 4 == 0 && ldc % 4 == 0;
}

// C (m x n, ld ldc) = alpha A^T B (reduce = 0) or C += alpha A^T B
// (reduce = 1) on the 128-tiles of C, with A (K x m, ld lda) and B (K x n,
// ld ldb) column-major.  tri: only tiles on and above the diagonal.
// klo_col: the K range of the tile at column col0 is [col0, K).  prec: 1
// (TF32) or 3 (3xTF32).  ksplit > 0 (a multiple of 32, reduce = 1 only):
// the K range is cut into slices of that length, one CTA per tile and
// slice, each adding its partial product into C.  d_err receives a nonzero
// code if a wait timed out.  stream: 0 for the context's stream.
int rsd_tc_gemm(rsd_ctx* ctx, int prec, int m, int n, int K, float alpha, const float* A, int64_t lda,
                const float* B, int64_t ldb, float* C, int64_t ldc, int reduce, int tri, int klo_col, int* d_err,
                cudaStream_t stream, int ksplit) {
  if (m < 1 || n < 1 || K < 1 || (prec != 1 && prec != 3) || !rsd_tc_gemm_ok(A, lda, B, ldb, C, ldc) ||
      ksplit < 0 || ksplit % TC_KC != 0 || (ksplit > 0 && !reduce))
    return rsd_fail(ctx, RSD_EARG, "tc_gemm: unsupported arguments (m=%d n=%d K=%d prec=%d)", m, n, K, prec);
  RSD_TRY(tc_init(ctx));
  CUtensorMap tmA, tmB, tmC;
  RSD_TRY(encode_2d(ctx, &tmA, A, K, m, lda, TC_KC, TC_TILE, CU_TENSOR_MAP_SWIZZLE_128B));
  RSD_TRY(encode_2d(ctx, &tmB, B, K, n, ldb, TC_KC, TC_TILE, CU_TENSOR_MAP_SWIZZLE_128B));
  RSD_TRY(encode_2d(ctx, &tmC, C, m, n, ldc, TC_TILE, TC_TILE, CU_TENSOR_MAP_SWIZZLE_NONE));
  TcArgs a{K, tri, klo_col, reduce, ksplit, alpha, d_err, wait_limit(ctx), 0, 0, 0, 0, 0, 0, 0, 0};
  const dim3 grid((m + TC_TILE - 1) / TC_TILE, (n + TC_TILE - 1) / TC_TILE, ksplit > 0 ? (K + ksplit - 1) / ksplit : 1);
  cudaStream_t st = stream ? stream : ctx->stream;
  if (prec == 1) {
    tc_gemm_kernel<1><<<grid, TC_THREADS, TcCfg<1>::SMEM, st>>>(tmA, tmB, tmC, a);
  } else {
    tc_gemm_kernel<3><<<grid, TC_THREADS, TcCfg<3>::SMEM, st>>>(tmA, tmB, tmC, a);
  }
  RSD_LAUNCH_NOTE();
  RSD_CUDA(ctx, cudaGetLastError());
  return RSD_OK;
}

// nbatch products C_z = alpha A_z^T B_z (store) of m x n x K each, one
// launch: the operands are sub-blocks of three column-major arrays (A: a_rows
// x a_cols, ld lda; likewise B and C) whose coordinates move by the given
// steps per batch z (A: k, m; B: k, n; C: m, n); batch z has n - z * ndec
// columns.  prec 1 or 3.
int rsd_tc_gemm_zbatch(rsd_ctx* ctx, int prec, int m, int n, int K, float alpha, const float* A, int64_t lda,
                       int64_t a_rows, int64_t a_cols, const float* B, int64_t ldb, int64_t b_rows, int64_t b_cols,
                       float* C, int64_t ldc, int64_t c_rows, int64_t c_cols, int nbatch, int zak, int zam, int zbk,
                       int zbn, int zcm, int zcn, int ndec, int* d_err) {
  if (m < 1 || n < 1 || K < 1 || nbatch < 1 || (prec != 1 && prec != 3) || !rsd_tc_gemm_ok(A, lda, B, ldb, C, ldc))
    return rsd_fail(ctx, RSD_EARG, "tc_gemm_zbatch: unsupported arguments (m=%d n=%d K=%d)", m, n, K);
  RSD_TRY(tc_init(ctx));
  CUtensorMap tmA, tmB, tmC;
  RSD_TRY(encode_2d(ctx, &tmA, A, a_rows, a_cols, lda, TC_KC, TC_TILE, CU_TENSOR_MAP_SWIZZLE_128B));
  RSD_TRY(encode_2d(ctx, &tmB, B, b_rows, b_cols, ldb, TC_KC, TC_TILE, CU_TENSOR_MAP_SWIZZLE_128B));
  RSD_TRY(encode_2d(ctx, &tmC, C, c_rows, c_cols, ldc, TC_TILE, TC_TILE, CU_TENSOR_MAP_SWIZZLE_NONE));
  TcArgs a{K, 0, 0, 0, 0, alpha, d_err, wait_limit(ctx), zak, zam, zbk, zbn, zcm, zcn, n, ndec};
  const dim3 grid((m + TC_TILE - 1) / TC_TILE, (n + TC_TILE - 1) / TC_TILE, nbatch);
  if (prec == 1) {
    tc_gemm_kernel<1><<<grid, TC_THREADS, TcCfg<1>::SMEM, ctx->stream>>>(tmA, tmB, tmC, a);
  } else {
    tc_gemm_kernel<3><<<grid, TC_THREADS, TcCfg<3>::SMEM, ctx->stream>>>(tmA, tmB, tmC, a);
  }
  RSD_LAUNCH_NOTE();
  RSD_CUDA(ctx, cudaGetLastError());
  return RSD_OK;
}

// C (rest x rest, tiles on and above the diagonal, ld ldc) -= P^T P with P
// (kb x rest, ld lda): the trailing update of the blocked Cholesky.
int rsd_tc_syrk(rsd_ctx* ctx, int prec, const float* panel, int64_t lda, int kb, int rest, float* C, int64_t ldc,
                int* d_err) {
  if (!rsd_tc_syrk_ok(panel, lda, C, ldc, kb) || rest < 1)
    return rsd_fail(ctx, RSD_EARG, "tc_syrk: unsupported layout (lda=%lld ldc=%lld kb=%d)", (long long)lda,
                    (long long)ldc, kb);
  return rsd_tc_gemm(ctx, prec, rest, rest, kb, -1.0f, panel, lda, panel, lda, C, ldc, 1, 1, 0, d_err);
}
