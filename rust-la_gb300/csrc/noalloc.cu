// LU factorization for callers that cannot allocate device memory.
//
// Some hosts of this library cannot call cudaMalloc at all: code running under
// a memory manager that owns every device allocation (a pool sized at start-up,
// a framework that hands out only pre-registered buffers), or code that must
// keep a fixed device-memory footprint in a hot loop. la_lu_factor_noalloc
// serves them: the caller passes the matrix and the output buffers, and the
// only working memory the factorization needs beyond them, the panel kernel's
// pivot-exchange scratch, lives in the file-scope device array below. That
// array exists once per device that loads the library and stays allocated
// until the process exits.
//
// The call blocks: it waits for the stream to finish the factorization and
// reads the device error word back with a synchronous copy. So it cannot be
// called while any stream is being captured into a CUDA graph (the wait and the
// copy would fail and invalidate the capture).
#include "la_internal.cuh"

namespace {

// Largest supported row count (m). With at most NA_CTAS panel CTAs a panel of
// up to 16384 rows fits in shared memory.
constexpr size_t NA_MAX_ROWS = 16384;
constexpr int NA_CTAS = 64;  // panel CTAs (candidate slots per parity)

// Layout of the scratch array (byte offsets, each 256-aligned).
constexpr size_t NA_OFF_ERR = 0;
constexpr size_t NA_OFF_BAR = 256;
constexpr size_t NA_OFF_CABS = 512;
constexpr size_t NA_OFF_CPOS = NA_OFF_CABS + 2 * NA_CTAS * sizeof(double);
constexpr size_t NA_OFF_CROW = NA_OFF_CPOS + 2 * NA_CTAS * sizeof(int);
constexpr size_t NA_OFF_DIAGA = NA_OFF_CROW + (size_t)2 * NA_CTAS * MAX_PANEL_W * sizeof(double);
constexpr size_t NA_OFF_DIAGS = NA_OFF_DIAGA + 2 * MAX_PANEL_W * sizeof(double);
constexpr size_t NA_OFF_SWAPS = NA_OFF_DIAGS + 2 * MAX_PANEL_W * sizeof(double);
constexpr size_t NA_BYTES = NA_OFF_SWAPS + 4096;  // about 70 KB in total

static __device__ __align__(256) unsigned char g_lu_scratch[NA_BYTES];

// Device address of the scratch array per device, looked up once per device
// (the host-side symbol is only a stand-in and must never be handed to a
// kernel). Atomic, so host threads making their first calls at the same time
// do not race; after cudaDeviceReset the cached address is no longer valid.
std::atomic<unsigned char*> g_scratch_addr[LA_MAX_DEVICES];

// With that device current: the scratch array's device address.
la_status scratch_for_device(int dev, unsigned char** out) {
  if (dev < 0 || dev >= LA_MAX_DEVICES) return LA_UNSUPPORTED;
  unsigned char* a = g_scratch_addr[dev].load(std::memory_order_acquire);
  if (!a) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_lu_scratch);
    if (e != cudaSuccess) return LA_CUDA_ERROR;
    a = static_cast<unsigned char*>(p);
    g_scratch_addr[dev].store(a, std::memory_order_release);  // every thread stores the same value
  }
  *out = a;
  return LA_OK;
}

}  // namespace

extern "C" la_status la_lu_factor_noalloc(void* stream, double* d_a, size_t lda, size_t m,
                                          size_t n, int* d_ipiv, uint64_t* d_piv,
                                          int* d_flags) {
  if (!d_a || !d_ipiv || !d_piv || !d_flags || lda < n) return LA_INVALID;
  if (m == 0 || n == 0) return LA_BADSHAPE;
  if (m > NA_MAX_ROWS || n > (size_t)INT32_MAX / 2) return LA_UNSUPPORTED;
  if (reinterpret_cast<uintptr_t>(d_a) % 16 != 0 || lda % 2 != 0) return LA_INVALID;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return LA_CUDA_ERROR;
  unsigned char* base = nullptr;
  LA_TRY(scratch_for_device(dev, &base));

  // A context that lives on the host stack and points at the static scratch.
  la_context c;
  c.device = dev;
  c.own_stream = static_cast<cudaStream_t>(stream);
  c.stream = c.own_stream;
  c.lookahead = 0;
  c.profile = 0;
  c.arith = LA_ARITH_FAST;
  c.panel_ctas = NA_CTAS;
  c.cand_stride = NA_CTAS;
  if (cudaDeviceGetAttribute(&c.sm_count, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return LA_CUDA_ERROR;
  int optin = 0;
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
    return LA_CUDA_ERROR;
  c.smem_optin = (size_t)optin;
  c.d_err = reinterpret_cast<int*>(base + NA_OFF_ERR);
  c.d_bar = reinterpret_cast<unsigned*>(base + NA_OFF_BAR);
  c.d_cand_abs = reinterpret_cast<double*>(base + NA_OFF_CABS);
  c.d_cand_pos = reinterpret_cast<int*>(base + NA_OFF_CPOS);
  c.d_cand_row = reinterpret_cast<double*>(base + NA_OFF_CROW);
  c.d_diag_a = reinterpret_cast<double*>(base + NA_OFF_DIAGA);
  c.d_diag_s = reinterpret_cast<double*>(base + NA_OFF_DIAGS);
  c.d_swaps = reinterpret_cast<int*>(base + NA_OFF_SWAPS);

  // The array keeps the previous call's contents: clear the error word (the
  // barrier counter is cleared by the factorization itself).
  if (cudaMemsetAsync(c.d_err, 0, sizeof(int), c.stream) != cudaSuccess) return LA_CUDA_ERROR;

  la_lu_handle h;
  h.ctx = &c;
  h.m = m;
  h.n = n;
  h.ld = lda;
  h.d_lu = d_a;
  h.d_ipiv = d_ipiv;
  h.d_piv = d_piv;
  h.arith = LA_ARITH_FAST;
  LA_TRY(lu_factor_enqueue(&c, &h, d_flags));
  if (cudaStreamSynchronize(c.stream) != cudaSuccess) return LA_CUDA_ERROR;
  int err = 0;
  if (cudaMemcpy(&err, c.d_err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
    return LA_CUDA_ERROR;
  // Device error words: a panel that does not fit is LA_UNSUPPORTED; every
  // other code is a bounded device wait that gave up (panel barrier, TMA
  // GEMM), LA_TIMEOUT.
  if (err != DERR_NONE) return err == DERR_PANEL_CAPACITY ? LA_UNSUPPORTED : LA_TIMEOUT;
  return LA_OK;
}
