// Tensor-core (tcgen05, TF32) trailing update of the blocked FP32 Cholesky:
//     C(rest x rest, upper tiles) <- C - P^T P,   P = A(j0:j0+kb, j0+kb:n)
// P is K-major for both MMA operands (the kb panel rows of one column are
// contiguous), so one TMA tensor map over P serves as A (rows = output rows)
// and as B (rows = output columns).
//
// One CTA (4 warps) per 128 x 128 output tile:
//   1. one thread issues TMA loads of the K <= 128 slices of A and B into
//      128B-swizzled shared memory (four 16 KB chunks of 32 K-elements each);
//   2. the same thread issues 16 tcgen05.mma (kind::tf32, K = 8) into a
//      128-column FP32 accumulator in tensor memory and commits them to an
//      mbarrier;
//   3. the four warps read the accumulator back with tcgen05.ld (TMEM lane =
//      output row), stage -D column-major in the (now free) operand buffer,
//      and one thread adds it to C with a TMA reduce-add, which clips the
//      ragged edge tiles.
// Tiles strictly below the diagonal are skipped; the diagonal tiles are
// computed whole, like the SIMT GEMM they replace.
//
// Every mbarrier wait is bounded by the global timer: on a timeout the
// kernel records an error code in *err, waits (bounded) for its own copies,
// frees its tensor memory and returns.  The host turns the code into
// RSD_ETIMEOUT.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <cstring>

#include "rsd_internal.cuh"

namespace {

constexpr int TC_BM = 128, TC_BN = 128, TC_BK = 32, TC_KMAX = 128;
constexpr int TC_CHUNK_BYTES = TC_BM * TC_BK * 4;                      // 16 KB
constexpr int TC_OPERAND_BYTES = (TC_KMAX / TC_BK) * TC_CHUNK_BYTES;    // 64 KB
constexpr int TC_SMEM = 2 * TC_OPERAND_BYTES + 1024 + 64;              // + alignment + barriers
constexpr unsigned long long TC_WAIT_NS = 500ull * 1000 * 1000;        // 0.5 s per wait

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

__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity) {
  const uint64_t t0 = global_ns();
  while (!mbar_try_wait(bar, parity)) {
    if (global_ns() - t0 > TC_WAIT_NS) return false;
  }
  return true;
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

__global__ void __launch_bounds__(128, 1)
    tc_syrk_update(const __grid_constant__ CUtensorMap tmP, const __grid_constant__ CUtensorMap tmC, int kb,
                   int* __restrict__ err) {
  const int row0 = blockIdx.x * TC_BM, col0 = blockIdx.y * TC_BN;
  if (row0 >= col0 + TC_BN) return;  // strictly below the diagonal
  extern __shared__ unsigned char smraw[];
  unsigned char* base = (unsigned char*)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  unsigned char* sA = base;
  unsigned char* sB = base + TC_OPERAND_BYTES;
  uint64_t* bars = (uint64_t*)(base + 2 * TC_OPERAND_BYTES);  // [0] operands landed, [1] MMAs done
  uint32_t* tslot = (uint32_t*)(bars + 2);
  __shared__ int ok_flag, out_flag;  // operands landed; every thread staged its row
  const int tid = threadIdx.x, warp = tid >> 5;
  const uint32_t bar_full = smem_u32(&bars[0]), bar_done = smem_u32(&bars[1]);
  const int nchunk = (kb + TC_BK - 1) / TC_BK;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "r"(TC_BN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    ok_flag = 1;
    out_flag = 1;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_full));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_done));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t taddr = *tslot;

  if (tid == 0) {
    const uint32_t bytes = (uint32_t)(2 * nchunk * TC_CHUNK_BYTES);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar_full), "r"(bytes) : "memory");
    const uint64_t tm = reinterpret_cast<uint64_t>(&tmP);
    for (int c = 0; c < nchunk; c++) {
      asm volatile(
          "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
              "r"(smem_u32(sA + c * TC_CHUNK_BYTES)),
          "l"(tm), "r"(c * TC_BK), "r"(row0), "r"(bar_full)
          : "memory");
      asm volatile(
          "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
              "r"(smem_u32(sB + c * TC_CHUNK_BYTES)),
          "l"(tm), "r"(c * TC_BK), "r"(col0), "r"(bar_full)
          : "memory");
    }
    if (!mbar_wait_bounded(bar_full, 0)) {
      ok_flag = 0;
      atomicExch(err, 1);
      mbar_wait_bounded(bar_full, 0);  // a last bounded wait for the copies in flight
    } else {
      asm volatile("tcgen05.fence::after_thread_sync;");
      constexpr uint32_t idesc = idesc_tf32(TC_BM, TC_BN);
      for (int c = 0; c < nchunk; c++)
        for (int kk = 0; kk < TC_BK / 8; kk++) {
          const uint64_t ad = smem_desc_sw128(smem_u32(sA + c * TC_CHUNK_BYTES + kk * 32));
          const uint64_t bd = smem_desc_sw128(smem_u32(sB + c * TC_CHUNK_BYTES + kk * 32));
          const uint32_t acc = (c | kk) ? 1u : 0u;
          asm volatile(
              "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
              " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(taddr),
              "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
        }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar_done)
                   : "memory");
    }
  }
  __syncthreads();
  if (ok_flag) {
    if (!mbar_wait_bounded(bar_done, 0)) {
      atomicExch(err, 2);
      out_flag = 0;
    } else {
      asm volatile("tcgen05.fence::after_thread_sync;");
      // -D staged column-major (128 rows x 128 columns) over the A buffer
      float* sOut = reinterpret_cast<float*>(sA);
      const uint32_t lane_addr = taddr + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
      for (int cc = 0; cc < TC_BN / 32; cc++) {
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
        for (int j = 0; j < 32; j++) sOut[(cc * 32 + j) * TC_BM + tid] = -__uint_as_float(v[j]);
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(TC_BN));
  if (tid == 0 && ok_flag && out_flag) {
    const uint64_t tm = reinterpret_cast<uint64_t>(&tmC);
    asm volatile(
        "cp.reduce.async.bulk.tensor.2d.global.shared::cta.add.tile.bulk_group [%0, {%1, %2}], [%3];" ::"l"(tm),
        "r"(row0), "r"(col0), "r"(smem_u32(sA))
        : "memory");
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
    asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
  }
}

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

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

}  // namespace

// Nonzero when the tensor-core trailing update applies: 16-byte aligned
// panel and trailing block, leading dimensions a multiple of 4 floats (the
// TMA stride rule) and 0 < kb <= 128.
int rsd_tc_syrk_ok(const float* panel, int64_t lda, const float* C, int64_t ldc, int kb) {
  return ((uintptr_t)panel % 16 == 0) && ((uintptr_t)C % 16 == 0) && (lda % 4 == 0) && (ldc % 4 == 0) && kb > 0 &&
         kb <= TC_KMAX;
}

// C (rest x rest, upper tiles, ld ldc) -= P^T P with P (kb x rest, ld lda),
// TF32 products with FP32 accumulation.  d_err receives a nonzero code if a
// wait timed out.
int rsd_tc_syrk(rsd_ctx* ctx, const float* panel, int64_t lda, int kb, int rest, float* C, int64_t ldc, int* d_err) {
  if (!rsd_tc_syrk_ok(panel, lda, C, ldc, kb) || rest < 1)
    return rsd_fail(ctx, RSD_EARG, "tc_syrk: unsupported layout (lda=%lld ldc=%lld kb=%d)", (long long)lda,
                    (long long)ldc, kb);
  if (!g_encode) {
    cudaDriverEntryPointQueryResult q;
    void* fn = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        !fn || q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      return rsd_fail(ctx, RSD_EUNSUP, "cuTensorMapEncodeTiled is not available");
    }
    RSD_CUDA(ctx, cudaFuncSetAttribute(tc_syrk_update, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM));
    g_encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
  }
  CUtensorMap tmP, tmC;
  RSD_TRY(encode_2d(ctx, &tmP, panel, kb, rest, lda, TC_BK, TC_BM, CU_TENSOR_MAP_SWIZZLE_128B));
  RSD_TRY(encode_2d(ctx, &tmC, C, rest, rest, ldc, TC_BM, TC_BN, CU_TENSOR_MAP_SWIZZLE_NONE));
  const int nt = (rest + TC_BM - 1) / TC_BM;
  tc_syrk_update<<<dim3(nt, nt), 128, TC_SMEM, ctx->stream>>>(tmP, tmC, kb, d_err); RSD_LAUNCH_NOTE();
  RSD_CUDA(ctx, cudaGetLastError());
  return RSD_OK;
}
