// Context, device memory and error plumbing of liblagpu.
#include <cstdio>
#include <cstring>
#include <new>

#include "la_internal.cuh"

la_status la_cuda_fail(la_ctx ctx, cudaError_t e, const char* what) {
  if (ctx) {
    char buf[512];
    snprintf(buf, sizeof(buf), "%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
    ctx->last_error = buf;
  }
  if (e == cudaErrorMemoryAllocation) return LA_NOMEM;
  return LA_CUDA_ERROR;
}

la_status la_check_launch(la_ctx ctx, const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return la_cuda_fail(ctx, e, what);
  return LA_OK;
}

la_status la_device_alloc(la_ctx ctx, void** p, size_t bytes) {
  *p = nullptr;
  // A failure injected for tests (LA_OPT_INJECT_ALLOC_FAIL): the caller sees
  // exactly what an exhausted device pool gives it.
  if (ctx->inject_alloc_at > 0 && --ctx->inject_alloc_at == 0) {
    ctx->last_error = "la_device_alloc: injected allocation failure";
    return LA_NOMEM;
  }
  if (bytes == 0) bytes = 256;
  cudaError_t e = cudaMallocAsync(p, bytes, ctx->stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    return la_cuda_fail(ctx, e, "cudaMallocAsync");
  }
  return LA_OK;
}

void la_device_free(la_ctx ctx, void* p) {
  if (p) cudaFreeAsync(p, ctx->stream);
}

// Synchronizes the context's stream and turns a device-side error word into a status.
la_status la_sync_and_check(la_ctx ctx, const char* what) {
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return la_cuda_fail(ctx, e, what);
  int err = 0;
  e = cudaMemcpy(&err, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return la_cuda_fail(ctx, e, "read device error word");
  if (err != DERR_NONE) {
    char buf[256];
    snprintf(buf, sizeof(buf), "%s: device wait gave up (code %d)", what, err);
    ctx->last_error = buf;
    int zero = 0;
    cudaMemcpy(ctx->d_err, &zero, sizeof(int), cudaMemcpyHostToDevice);
    return err == DERR_PANEL_CAPACITY ? LA_UNSUPPORTED : LA_TIMEOUT;
  }
  return LA_OK;
}

namespace {

// Register-resident FP64 FMA loop: 8 independent chains per thread.
__global__ void fp64_peak_kernel(double* out, int iters, double a, double b) {
  double r[8];
#pragma unroll
  for (int i = 0; i < 8; i++) r[i] = threadIdx.x * 1e-3 + i;
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int i = 0; i < 8; i++) r[i] = fma(r[i], a, b);
  }
  double s = 0;
  for (int i = 0; i < 8; i++) s += r[i];
  if (s == 123.456) out[0] = s;  // keeps the loop live; practically never taken
}

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

}  // namespace

extern "C" {

int la_abi_version(void) { return LA_ABI_VERSION; }

const char* la_status_string(la_status s) {
  switch (s) {
    case LA_OK: return "ok";
    case LA_SINGULAR: return "singular (reference returns None)";
    case LA_BADSHAPE: return "bad shape (reference panics)";
    case LA_INVALID: return "invalid argument";
    case LA_NOMEM: return "out of memory";
    case LA_CUDA_ERROR: return "CUDA error";
    case LA_TIMEOUT: return "device wait timed out";
    case LA_NOT_CONVERGED: return "iterative refinement did not converge";
    case LA_UNSUPPORTED: return "unsupported size or option";
  }
  return "unknown status";
}

la_status la_ctx_create(int device, la_ctx* out) {
  if (!out) return LA_INVALID;
  *out = nullptr;
  la_ctx ctx = new (std::nothrow) la_context();
  if (!ctx) return LA_NOMEM;
  ctx->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) { la_status s = la_cuda_fail(ctx, e, "cudaSetDevice"); delete ctx; return s; }
  cudaDeviceProp prop;
  e = cudaGetDeviceProperties(&prop, device);
  if (e != cudaSuccess) { la_status s = la_cuda_fail(ctx, e, "props"); delete ctx; return s; }
  ctx->sm_count = prop.multiProcessorCount;
  ctx->smem_optin = prop.sharedMemPerBlockOptin;
  if (!prop.cooperativeLaunch) { delete ctx; return LA_UNSUPPORTED; }
  e = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) { la_status s = la_cuda_fail(ctx, e, "stream"); delete ctx; return s; }
  ctx->stream = ctx->own_stream;
  {
    int lo = 0, hi = 0;
    cudaDeviceGetStreamPriorityRange(&lo, &hi);
    e = cudaStreamCreateWithPriority(&ctx->side_stream, cudaStreamNonBlocking, hi);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming);
    if (e != cudaSuccess) {
      la_status s = la_cuda_fail(ctx, e, "side stream");
      la_ctx_destroy(ctx);
      return s;
    }
  }
  // Keep freed stream-ordered allocations cached in the device pool.
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t thr = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  // Scratch: error word, barrier counter, panel candidate buffers, swap list, small results.
  size_t off = 0;
  const size_t o_err = off; off = align_up(off + 256, 256);
  const size_t o_bar = off; off = align_up(off + 256, 256);
  const size_t o_cabs = off; off = align_up(off + 2 * MAX_PANEL_CTAS * sizeof(double), 256);
  const size_t o_cpos = off; off = align_up(off + 2 * MAX_PANEL_CTAS * sizeof(int), 256);
  const size_t o_crow = off;
  off = align_up(off + (size_t)2 * MAX_PANEL_CTAS * MAX_PANEL_W * sizeof(double), 256);
  const size_t o_da = off; off = align_up(off + 2 * MAX_PANEL_W * sizeof(double), 256);
  const size_t o_ds = off; off = align_up(off + 2 * MAX_PANEL_W * sizeof(double), 256);
  const size_t o_sw = off; off = align_up(off + (1 + 4 * MAX_PANEL_W) * sizeof(int), 256);
  const size_t o_sm = off; off = align_up(off + 8 * sizeof(double), 256);
  const size_t o_sv = off; off = align_up(off + (2 + 2 * SOLVE_WAVE_MAX_GROUPS) * sizeof(int), 256);
  e = cudaMalloc(&ctx->d_scratch, off);
  if (e != cudaSuccess) {
    la_status s = la_cuda_fail(ctx, e, "scratch");
    cudaStreamDestroy(ctx->own_stream);
    delete ctx;
    return s;
  }
  cudaMemset(ctx->d_scratch, 0, off);
  char* base = static_cast<char*>(ctx->d_scratch);
  ctx->scratch_bytes = off;
  ctx->d_err = reinterpret_cast<int*>(base + o_err);
  ctx->d_bar = reinterpret_cast<unsigned*>(base + o_bar);
  ctx->bar_count = 1;
  ctx->d_cand_abs = reinterpret_cast<double*>(base + o_cabs);
  ctx->d_cand_pos = reinterpret_cast<int*>(base + o_cpos);
  ctx->d_cand_row = reinterpret_cast<double*>(base + o_crow);
  ctx->d_diag_a = reinterpret_cast<double*>(base + o_da);
  ctx->d_diag_s = reinterpret_cast<double*>(base + o_ds);
  ctx->d_swaps = reinterpret_cast<int*>(base + o_sw);
  ctx->d_small = reinterpret_cast<double*>(base + o_sm);
  ctx->d_solve_sync = reinterpret_cast<int*>(base + o_sv);
  e = cudaMallocHost(&ctx->h_pinned, 4096);
  if (e != cudaSuccess) {
    la_status s = la_cuda_fail(ctx, e, "pinned");
    cudaFree(ctx->d_scratch);
    cudaStreamDestroy(ctx->own_stream);
    delete ctx;
    return s;
  }
  e = cudaDeviceSynchronize();
  if (e != cudaSuccess) { la_status s = la_cuda_fail(ctx, e, "init sync"); la_ctx_destroy(ctx); return s; }
  *out = ctx;
  return LA_OK;
}

void la_ctx_destroy(la_ctx ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  if (ctx->side_stream) cudaStreamSynchronize(ctx->side_stream);
  for (auto ev : ctx->event_pool) cudaEventDestroy(ev);
  if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
  if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
  if (ctx->side_stream) cudaStreamDestroy(ctx->side_stream);
  if (ctx->h_pinned) cudaFreeHost(ctx->h_pinned);
  if (ctx->d_scratch) cudaFree(ctx->d_scratch);
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  delete ctx;
}

la_status la_ctx_set_stream(la_ctx ctx, void* stream) {
  if (!ctx) return LA_INVALID;
  ctx->stream = stream ? static_cast<cudaStream_t>(stream) : ctx->own_stream;
  return LA_OK;
}

void* la_ctx_get_stream(la_ctx ctx) { return ctx ? static_cast<void*>(ctx->stream) : nullptr; }

la_status la_ctx_synchronize(la_ctx ctx) {
  if (!ctx) return LA_INVALID;
  return la_sync_and_check(ctx, "la_ctx_synchronize");
}

const char* la_ctx_last_error(la_ctx ctx) { return ctx ? ctx->last_error.c_str() : ""; }

uint64_t la_ctx_kernel_launches(la_ctx ctx) { return ctx ? ctx->launches : 0; }

la_status la_ctx_set_option(la_ctx ctx, int option, int64_t value) {
  if (!ctx) return LA_INVALID;
  switch (option) {
    case LA_OPT_ARITH:
      if (value != LA_ARITH_FAST && value != LA_ARITH_EXACT) return LA_INVALID;
      ctx->arith = (int)value;
      return LA_OK;
    case LA_OPT_PANEL_WIDTH:
      if (value != 16 && value != 32 && value != 64) return LA_INVALID;
      ctx->panel_width = (int)value;
      return LA_OK;
    case LA_OPT_PANEL_CTAS:
      if (value < 0 || value > MAX_PANEL_CTAS) return LA_INVALID;
      ctx->panel_ctas = (int)value;
      return LA_OK;
    case LA_OPT_PROFILE:
      ctx->profile = value ? 1 : 0;
      return LA_OK;
    case LA_OPT_LOOKAHEAD:
      ctx->lookahead = value ? 1 : 0;
      return LA_OK;
    case LA_OPT_CLUSTER_PANEL:
      ctx->cluster_panels = value ? 1 : 0;
      return LA_OK;
    case LA_OPT_BATCH_GMRES:
      if (value < 0 || value > 20) return LA_INVALID;
      ctx->batch_gmres = (int)value;
      return LA_OK;
    case LA_OPT_SOLVE_WAVE:
      if (value < 0 || value > 8) return LA_INVALID;
      ctx->solve_wave = (int)value;
      return LA_OK;
    case LA_OPT_INJECT_ALLOC_FAIL:
      if (value < 0 || value > (1 << 20)) return LA_INVALID;
      ctx->inject_alloc_at = (int)value;
      return LA_OK;
    case LA_OPT_INJECT_IR_STALL:
      if (value < 0 || value > (1 << 20)) return LA_INVALID;
      ctx->inject_ir_stall = (int)value;
      return LA_OK;
    case LA_OPT_WAIT_LIMIT_US:
      if (value < 0 || value > 10000000) return LA_INVALID;
      ctx->wait_limit_us = value;
      return LA_OK;
    case LA_OPT_INJECT_PANEL_STALL:
      if (value < 0 || value > (1 << 20)) return LA_INVALID;
      ctx->inject_panel_stall = (int)value;
      return LA_OK;
    case LA_OPT_PDL:
      ctx->pdl = value ? 1 : 0;
      return LA_OK;
  }
  return LA_INVALID;
}

la_status la_ctx_get_option(la_ctx ctx, int option, int64_t* value) {
  if (!ctx || !value) return LA_INVALID;
  switch (option) {
    case LA_OPT_ARITH: *value = ctx->arith; return LA_OK;
    case LA_OPT_PANEL_WIDTH: *value = ctx->panel_width; return LA_OK;
    case LA_OPT_PANEL_CTAS: *value = ctx->panel_ctas; return LA_OK;
    case LA_OPT_PROFILE: *value = ctx->profile; return LA_OK;
    case LA_OPT_LOOKAHEAD: *value = ctx->lookahead; return LA_OK;
    case LA_OPT_CLUSTER_PANEL: *value = ctx->cluster_panels; return LA_OK;
    case LA_OPT_BATCH_GMRES: *value = ctx->batch_gmres; return LA_OK;
    case LA_OPT_SOLVE_WAVE: *value = ctx->solve_wave; return LA_OK;
    case LA_OPT_INJECT_ALLOC_FAIL: *value = ctx->inject_alloc_at; return LA_OK;
    case LA_OPT_INJECT_IR_STALL: *value = ctx->inject_ir_stall; return LA_OK;
    case LA_OPT_WAIT_LIMIT_US: *value = ctx->wait_limit_us; return LA_OK;
    case LA_OPT_INJECT_PANEL_STALL: *value = ctx->inject_panel_stall; return LA_OK;
    case LA_OPT_PDL: *value = ctx->pdl; return LA_OK;
  }
  return LA_INVALID;
}

la_status la_ctx_last_phase_ms(la_ctx ctx, double* ms5) {
  if (!ctx || !ms5) return LA_INVALID;
  for (int i = 0; i < 5; i++) ms5[i] = ctx->phase_ms[i];
  return LA_OK;
}

la_status la_probe_fp64_peak(la_ctx ctx, double* tflops) {
  if (!ctx || !tflops) return LA_INVALID;
  LA_CUDA(ctx, cudaSetDevice(ctx->device));
  const int blocks = ctx->sm_count * 4, threads = 256, iters = 4096;
  cudaEvent_t e0, e1;
  LA_CUDA(ctx, cudaEventCreate(&e0));
  LA_CUDA(ctx, cudaEventCreate(&e1));
  fp64_peak_kernel<<<blocks, threads, 0, ctx->stream>>>(ctx->d_small, iters, 1.0000001, 1e-9);
  ctx->launches++;
  LA_CUDA(ctx, cudaEventRecord(e0, ctx->stream));
  fp64_peak_kernel<<<blocks, threads, 0, ctx->stream>>>(ctx->d_small, iters, 1.0000001, 1e-9);
  ctx->launches++;
  LA_CUDA(ctx, cudaEventRecord(e1, ctx->stream));
  LA_CUDA(ctx, cudaEventSynchronize(e1));
  float ms = 0;
  LA_CUDA(ctx, cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const double flops = 2.0 * 8 * iters * (double)blocks * threads;
  *tflops = flops / (ms * 1e-3) / 1e12;
  return LA_OK;
}

}  // extern "C"
