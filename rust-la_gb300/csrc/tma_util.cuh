// Shared helpers for the kernels that stage tiles with TMA
// (cp.async.bulk.tensor) and wait on mbarriers: the tcgen05 update of the
// mixed LU (gemm_tc.cu) and the FP64 trailing-update GEMM (gemm_f64.cu).
//
// Every wait is bounded: after LA_TMA_WAIT_NS of %globaltimer time, or as
// soon as another CTA has set the context's error word, it gives up, records
// `code` in the error word and returns false. The caller then waits (also
// bounded) for its own copies still in flight before it exits.
#ifndef LA_TMA_UTIL_CUH
#define LA_TMA_UTIL_CUH

#include <cuda.h>

#include "la_internal.cuh"

namespace la_tma {

constexpr unsigned long long LA_TMA_WAIT_NS = 2000000000ull;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait on an mbarrier phase; false: gave up (timeout or error word set).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err, int code) {
  unsigned long long t0 = 0;
  for (unsigned i = 0;; i++) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 255u) == 255u) {
      if (*reinterpret_cast<volatile int*>(err) != 0) return false;
      const unsigned long long now = gtimer();
      if (t0 == 0) t0 = now;
      else if (now - t0 > LA_TMA_WAIT_NS) {
        atomicCAS(err, 0, code);
        return false;
      }
    }
  }
}
// Bounded wait without touching the error word (draining copies after a failure).
__device__ __forceinline__ void mbar_drain(uint64_t* bar, uint32_t parity) {
  const unsigned long long t0 = gtimer();
  while (!mbar_try_wait(bar, parity))
    if (gtimer() - t0 > LA_TMA_WAIT_NS) break;
}
// 2-D tiled TMA load of box (x, y) into shared memory, completing on `bar`.
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// Driver entry point for tensor-map encoding, fetched once through the runtime
// (no link-time dependency on libcuda).
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

inline EncodeTiledFn get_encoder(la_ctx ctx) {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    cudaError_t e =
        cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !p) {
      if (ctx) ctx->last_error = "cuTensorMapEncodeTiled unavailable";
      return nullptr;
    }
    fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  return fn;
}

// Row-major 2-D map: `rows` rows of `cols` elements, pitch `ld` elements, box
// box_x (columns) x box_y (rows). The base must be 16-byte aligned and
// ld * element size a multiple of 16 (the encoder checks both).
inline bool encode_2d(la_ctx ctx, CUtensorMap* map, CUtensorMapDataType type, size_t esize,
                      const void* base, size_t rows, size_t cols, size_t ld, uint32_t box_x,
                      uint32_t box_y, CUtensorMapSwizzle swz) {
  EncodeTiledFn enc = get_encoder(ctx);
  if (!enc) return false;
  cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)(ld * esize)};
  cuuint32_t box[2] = {box_x, box_y};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = enc(map, type, 2, const_cast<void*>(base), dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, swz, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    if (ctx) ctx->last_error = "cuTensorMapEncodeTiled failed";
    return false;
  }
  return true;
}

}  // namespace la_tma

#endif  // LA_TMA_UTIL_CUH
