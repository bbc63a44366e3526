// Tensor-core trailing update of the mixed-precision LU:
//   C (M x N, f32, row-major) -= alpha * A (M x K) * B^T (B: N x K)
// with A and B both K-major (K contiguous), accumulated in FP32 by
// tcgen05.mma into tensor memory. Operand formats:
//   BF16 or FP16 (kind::f16, K = 16 per instruction);
//   split formats, FP8 e4m3 (kind::f8f6f4, K = 32 per instruction) or FP16
//   (kind::f16): each operand row holds its high parts in columns [0, K) and
//   its low parts in columns [lo, lo + K) (v * scale ~ hi + lo), and the kernel
//   accumulates hi*hi + hi*lo + lo*hi. Three 8-bit products give factors about
//   as accurate as BF16 ones (one e4m3 product alone leaves errors of a few
//   per cent, too much for refinement at kappa >= 1e2); three FP16 products
//   give about 2^-22 per product, close to FP32. Each chunk of the ring is
//   still a 128-byte-wide box of A and one of B: the producer walks three
//   "virtual" chunks per 128 bytes of K, (hi, hi), (hi, lo), (lo, hi).
//
// One CTA per 128 x 128 output tile, 128 threads:
//   warp 0 lane 0 : TMA producer. 128-byte-deep K chunks of A and B (64 16-bit
//                   or 128 8-bit elements, 16 KB each, 128B swizzle) into a
//                   3-stage ring, one mbarrier per stage
//   warp 1 lane 0 : MMA issuer. 4 x tcgen05.mma (M=128, N=128, 32 bytes of K)
//                   per chunk; tcgen05.commit releases the stage
//   all 4 warps   : epilogue. tcgen05.ld of the warp's 32 TMEM lanes (rows),
//                   -alpha * acc into swizzled shared-memory boxes, added to C
//                   by TMA tensor reductions (the SMs never load C)
// Shared memory is 3 x 32 KB per CTA, so two CTAs share an SM and one CTA's
// epilogue overlaps the other's MMAs. Every mbarrier wait is bounded (2 s by
// %globaltimer). On timeout the CTA records an error, waits (bounded) for its
// own copies in flight, frees its tensor memory and returns.
#include <cuda.h>

#include "la_internal.cuh"
#include "tma_util.cuh"

namespace {

constexpr int TM = 128, TN = 128;
constexpr int TKB = 128;  // bytes of K per chunk (one 128-byte swizzle row)
constexpr int STAGES = 3;
constexpr int TC_THREADS = 128;
constexpr uint32_t A_BYTES = TM * TKB;  // 16 KB
constexpr uint32_t B_BYTES = TN * TKB;  // 16 KB
constexpr uint32_t STAGE_BYTES = A_BYTES + B_BYTES;
constexpr size_t TC_SMEM = (size_t)STAGES * STAGE_BYTES + 1024;  // + alignment slack
constexpr uint32_t C_BOX_BYTES = TM * 32 * 4;  // one 128 x 32 FP32 box of the epilogue
static_assert((TN / 32) * C_BOX_BYTES <= STAGES * STAGE_BYTES, "epilogue boxes reuse the stages");
constexpr uint32_t TMEM_COLS = 128;

using la_tma::mbar_expect_tx;
using la_tma::mbar_init;
using la_tma::mbar_try_wait;
using la_tma::smem_u32;
using la_tma::tma_load_2d;

// Bounded wait on an mbarrier phase. false: gave up (timeout or error word set).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err) {
  return la_tma::mbar_wait(bar, parity, err, (int)DERR_TC_TIMEOUT);
}

// Shared-memory matrix descriptor: K-major operand, 128-byte swizzle, 8-row
// core-matrix groups 1024 bytes apart (SBO); LBO unused for this layout.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(1024u >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

// Instruction descriptor of kind::f16 and kind::f8f6f4: D f32 (bits 4-5 = 1),
// A and B formats in bits 7-9 and 10-12 (kind::f16: 0 f16, 1 bf16;
// kind::f8f6f4: 0 e4m3), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_mma(uint32_t ab_fmt) {
  return (1u << 4) | (ab_fmt << 7) | (ab_fmt << 10) | ((uint32_t)(TN >> 3) << 17) |
         ((uint32_t)(TM >> 4) << 24);
}

// F8: 8-bit operands (kind::f8f6f4), else 16-bit (kind::f16). SPLIT: hi/lo
// operands, lo the column of the low parts. K counts elements.
template <bool F8, bool SPLIT>
__global__ void __launch_bounds__(TC_THREADS, 1)
tc_update_kernel(const __grid_constant__ CUtensorMap tmap_a,
                 const __grid_constant__ CUtensorMap tmap_b,
                 const __grid_constant__ CUtensorMap tmap_c, int N, int K, int lo,
                 const float* __restrict__ alpha_ptr, uint32_t idesc, int* err) {
  la_pdl_wait();
  la_pdl_trigger();
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t full[STAGES], empty[STAGES], done;
  __shared__ uint32_t tmem_holder;
  __shared__ int s_fail;

  unsigned char* smem = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.y * TM, n0 = blockIdx.x * TN;
  constexpr int TKE = F8 ? TKB : TKB / 2;  // elements of K per chunk
  const int nk = (SPLIT ? 3 : 1) * ((K + TKE - 1) / TKE);

  if (tid == 0) {
    for (int s = 0; s < STAGES; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(&done, 1);
    s_fail = 0;
    la_tma::mbar_init_fence();
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_holder)),
                 "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_holder;

  int issued = 0;  // chunks whose TMA the producer issued
  if (warp == 0 && lane == 0) {
    for (int kc = 0; kc < nk; kc++) {
      const int s = kc % STAGES;
      if (kc >= STAGES && !mbar_wait(&empty[s], (uint32_t)((kc / STAGES - 1) & 1), err)) {
        s_fail = 1;
        break;
      }
      unsigned char* sa = smem + s * STAGE_BYTES;
      unsigned char* sb = sa + A_BYTES;
      mbar_expect_tx(&full[s], STAGE_BYTES);
      int ax = kc * TKE, bx = ax;
      if (SPLIT) {  // virtual chunk kc: K columns [c, c + TKE) as (hi, hi), (hi, lo), (lo, hi)
        const int c = (kc / 3) * TKE, t = kc % 3;
        ax = c + (t == 2 ? lo : 0);
        bx = c + (t == 1 ? lo : 0);
      }
      tma_load_2d(sa, &tmap_a, ax, m0, &full[s]);
      tma_load_2d(sb, &tmap_b, bx, n0, &full[s]);
      issued = kc + 1;
    }
  } else if (warp == 1 && lane == 0) {
    bool ok = true;
    for (int kc = 0; kc < nk; kc++) {
      const int s = kc % STAGES;
      if (!mbar_wait(&full[s], (uint32_t)((kc / STAGES) & 1), err)) {
        s_fail = 1;
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t sa = smem_u32(smem + s * STAGE_BYTES);
      const uint32_t sb = sa + A_BYTES;
#pragma unroll
      for (int k = 0; k < TKB / 32; k++) {  // 32 bytes of K per instruction
        const uint64_t ad = sdesc(sa + k * 32);
        const uint64_t bd = sdesc(sb + k * 32);
        const uint32_t acc = (kc > 0 || k > 0) ? 1u : 0u;
        if (F8)
          asm volatile(
              "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
              " tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
              "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
        else
          asm volatile(
              "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
              " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
              "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
      }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
              smem_u32(&empty[s]))
          : "memory");
    }
    if (ok)
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
              smem_u32(&done))
          : "memory");
  }
  __syncwarp();

  // Epilogue: every thread owns one accumulator row (TMEM lane). It writes
  // -alpha * acc, 32 columns at a time, into the freed pipeline buffers as
  // four 128 x 32 FP32 boxes in the 128-byte swizzled layout (row r's 16-byte
  // group q at r * 128 + ((q ^ (r & 7)) << 4): a warp's float4 stores are
  // conflict-free), and one thread adds the boxes to C with TMA tensor
  // reductions (cp.reduce.async.bulk.tensor .add): the read-modify-write of C
  // happens in L2, the SMs never load C, and the TMA unit clips the tile at
  // the matrix edges. The decision is block-uniform so the warp-collective
  // tcgen05.ld runs on full warps.
  const bool waited = mbar_wait(&done, 0, err);
  const bool have = __syncthreads_and(waited ? 1 : 0) && !s_fail;
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (have) {
    const float nalpha = -*alpha_ptr;
    const int rl = warp * 32 + lane;
#pragma unroll 1
    for (int cc = 0; cc < TN / 32; cc++) {
      uint32_t r[32];
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(cc * 32);
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
          "%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
            "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
            "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
            "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
            "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
            "=r"(r[31])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      unsigned char* box = smem + (size_t)cc * C_BOX_BYTES;
#pragma unroll
      for (int q = 0; q < 8; q++) {
        const float4 v = make_float4(nalpha * __uint_as_float(r[4 * q]),
                                     nalpha * __uint_as_float(r[4 * q + 1]),
                                     nalpha * __uint_as_float(r[4 * q + 2]),
                                     nalpha * __uint_as_float(r[4 * q + 3]));
        *reinterpret_cast<float4*>(box + rl * 128 + ((q ^ (rl & 7)) << 4)) = v;
      }
    }
    // the boxes, written through the generic proxy, are read by the TMA unit
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();
  if (have && tid == 0) {
    for (int cc = 0; cc < TN / 32; cc++)
      if (n0 + cc * 32 < N)
        asm volatile(
            "cp.reduce.async.bulk.tensor.2d.global.shared::cta.add.tile.bulk_group"
            " [%0, {%1, %2}], [%3];" ::"l"(reinterpret_cast<uint64_t>(&tmap_c)),
            "r"(n0 + cc * 32), "r"(m0), "r"(smem_u32(smem + (size_t)cc * C_BOX_BYTES))
            : "memory");
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
    asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
  }
  // On failure: wait (bounded) for this CTA's copies still in flight.
  if (!have && warp == 0 && lane == 0) {
    for (int kc = 0; kc < issued; kc++)
      la_tma::mbar_drain(&full[kc % STAGES], (uint32_t)((kc / STAGES) & 1));
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(TMEM_COLS));
}

// 2-D K-major operand map: `rows` rows of `cols` elements, pitch `ld`
// elements (ld * element size must be a multiple of 16), box of 128 bytes of
// K x 128 rows. 8-bit operands are mapped as bytes.
bool encode_operand(la_ctx ctx, CUtensorMap* map, const void* base, int fmt, size_t rows,
                    size_t cols, size_t ld) {
  if (fmt == LA_LOWP_F16X3)
    return la_tma::encode_2d(ctx, map, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, base, rows, cols, ld,
                             (uint32_t)(TKB / 2), (uint32_t)TM, CU_TENSOR_MAP_SWIZZLE_128B);
  if (fmt == LA_LOWP_E4M3X3)
    return la_tma::encode_2d(ctx, map, CU_TENSOR_MAP_DATA_TYPE_UINT8, 1, base, rows, cols, ld,
                             (uint32_t)TKB, (uint32_t)TM, CU_TENSOR_MAP_SWIZZLE_128B);
  return la_tma::encode_2d(ctx, map,
                           fmt == LA_LOWP_BF16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16
                                               : CU_TENSOR_MAP_DATA_TYPE_FLOAT16,
                           2, base, rows, cols, ld, (uint32_t)(TKB / 2), (uint32_t)TM,
                           CU_TENSOR_MAP_SWIZZLE_128B);
}

}  // namespace

// C (M x N f32, pitch ldc, 16-byte aligned rows) -= alpha * A * B^T where A is
// M x K and B is N x K, K-major with pitches lda, ldb in elements and
// 16-byte aligned bases. 16-bit formats: pitches multiples of 8 elements.
// Split formats (LA_LOWP_E4M3X3 bytes, LA_LOWP_F16X3 16-bit): the low parts
// at column lo = lda / 2 = ldb / 2, at or beyond K rounded up to a whole
// 128-byte chunk (the high parts' last chunk must not reach them); pitches
// multiples of 32 bytes. alpha is read on the device.
la_status launch_tc_update(la_ctx ctx, cudaStream_t stream, int fmt, int M, int N, int K,
                           const void* A, size_t lda, const void* B, size_t ldb, float* C,
                           size_t ldc, const float* d_alpha) {
  if (M <= 0 || N <= 0 || K <= 0) return LA_OK;
  const bool f8 = fmt == LA_LOWP_E4M3X3;
  const bool split = f8 || fmt == LA_LOWP_F16X3;
  const size_t pq = f8 ? 32 : (split ? 16 : 8);  // pitch quantum in elements
  const int tke = f8 ? TKB : TKB / 2;           // elements per 128-byte chunk
  if ((lda % pq) || (ldb % pq) || (ldc % 4) || (reinterpret_cast<uintptr_t>(A) % 16) ||
      (reinterpret_cast<uintptr_t>(B) % 16) || (reinterpret_cast<uintptr_t>(C) % 16))
    return LA_INVALID;
  if (split && (lda != ldb || (size_t)(K + tke - 1) / tke * tke > lda / 2)) return LA_INVALID;
  const int lo = split ? (int)(lda / 2) : 0;
  // The maps span the columns the kernel reads: [0, K), or for split formats
  // [0, lo + K) (the high parts, padding, the low parts).
  const size_t cols = split ? (size_t)lo + (size_t)K : (size_t)K;
  CUtensorMap ta, tb, tc;
  if (!encode_operand(ctx, &ta, A, fmt, (size_t)M, cols, lda)) return LA_CUDA_ERROR;
  if (!encode_operand(ctx, &tb, B, fmt, (size_t)N, cols, ldb)) return LA_CUDA_ERROR;
  // C (M x N FP32, pitch ldc) in 128 x 32 boxes, 128-byte swizzle: the epilogue's
  // reduction target.
  if (!la_tma::encode_2d(ctx, &tc, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, C, (size_t)M, (size_t)N,
                         ldc, 32u, (uint32_t)TM, CU_TENSOR_MAP_SWIZZLE_128B))
    return LA_CUDA_ERROR;
  static la_device_once configured;
  cudaError_t e = configured.run([](int) {
    const cudaFuncAttribute at = cudaFuncAttributeMaxDynamicSharedMemorySize;
    cudaError_t r = cudaFuncSetAttribute(tc_update_kernel<false, false>, at, (int)TC_SMEM);
    if (r == cudaSuccess) r = cudaFuncSetAttribute(tc_update_kernel<false, true>, at, (int)TC_SMEM);
    if (r == cudaSuccess) r = cudaFuncSetAttribute(tc_update_kernel<true, true>, at, (int)TC_SMEM);
    return r;
  });
  if (e != cudaSuccess) return la_cuda_fail(ctx, e, "cudaFuncSetAttribute(tc_update)");
  dim3 grid((N + TN - 1) / TN, (M + TM - 1) / TM);
  const float* alpha = d_alpha;
  if (f8)
    e = la_launch(ctx, tc_update_kernel<true, true>, grid, dim3(TC_THREADS), TC_SMEM, stream, ta,
                  tb, tc, N, K, lo, alpha, idesc_mma(0u), ctx->d_err);
  else if (split)
    e = la_launch(ctx, tc_update_kernel<false, true>, grid, dim3(TC_THREADS), TC_SMEM, stream, ta,
                  tb, tc, N, K, lo, alpha, idesc_mma(0u), ctx->d_err);
  else
    e = la_launch(ctx, tc_update_kernel<false, false>, grid, dim3(TC_THREADS), TC_SMEM, stream, ta,
                  tb, tc, N, K, 0, alpha, idesc_mma(fmt == LA_LOWP_BF16 ? 1u : 0u), ctx->d_err);
  if (e != cudaSuccess) return la_cuda_fail(ctx, e, "tc_update_kernel launch");
  ctx->launches++;
  return la_check_launch(ctx, "tc_update_kernel");
}

extern "C" la_status la_lowp_update_device(la_ctx ctx, int fmt, size_t m, size_t n, size_t k,
                                           const void* d_a16, size_t lda, const void* d_b16,
                                           size_t ldb, float* d_c, size_t ldc, float alpha) {
  if (!ctx || !d_a16 || !d_b16 || !d_c) return LA_INVALID;
  if (fmt < LA_LOWP_BF16 || fmt > LA_LOWP_F16X3) return LA_INVALID;
  if (m > INT32_MAX || n > INT32_MAX || k > INT32_MAX) return LA_UNSUPPORTED;
  LA_CUDA(ctx, cudaSetDevice(ctx->device));
  float* d_alpha = reinterpret_cast<float*>(ctx->d_small + 4);
  LA_CUDA(ctx, cudaMemcpyAsync(d_alpha, &alpha, sizeof(float), cudaMemcpyHostToDevice,
                               ctx->stream));
  LA_TRY(launch_tc_update(ctx, ctx->stream, fmt, (int)m, (int)n, (int)k, d_a16, lda, d_b16, ldb,
                          d_c, ldc, d_alpha));
  return la_sync_and_check(ctx, "lowp update");
}
