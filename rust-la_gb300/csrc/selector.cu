// Learned precision selector for batched solves (not in the reference).
//
// Per system, a feature kernel computes 16 cheap features (norms, diagonal
// dominance, row/column scaling spread, a few-step Lanczos estimate of the
// condition number); a small MLP (16 -> 64 -> 64 -> 3, ReLU, softmax, FP32)
// proposes the storage precision of the system's LU factors (FP8, BF16, FP32);
// the FP64 pass of the batched solver stays the fallback and the arbiter of every answer.
//
// The network is trained on the GPU by the kernels below: forward (one thread
// per sample), per-sample deltas, parameter gradients (one thread per
// parameter summing over the samples in a fixed order, so a step is
// deterministic) and Adam. A generator kernel builds the Householder-
// conditioned training and test systems A = H1 diag(s) H2 on the device.
#include <new>
#include <type_traits>

#include "f64conv.h"
#include "la_internal.cuh"

namespace {

constexpr int NF = 16, H1 = 64, H2 = 64, NC = 3;
constexpr int OFF_W1 = 0;                   // [H1][NF]
constexpr int OFF_B1 = OFF_W1 + H1 * NF;    // [H1]
constexpr int OFF_W2 = OFF_B1 + H1;         // [H2][H1]
constexpr int OFF_B2 = OFF_W2 + H2 * H1;    // [H2]
constexpr int OFF_W3 = OFF_B2 + H2;         // [NC][H2]
constexpr int OFF_B3 = OFF_W3 + NC * H2;    // [NC]
constexpr int NPARAM = OFF_B3 + NC;         // 5443
constexpr int ACT = NF + H1 + H2 + NC;      // per-sample activations kept for backprop

struct SysRec {
  long long a, b;
  int n, nrhs;
};

// ---- counter-based random numbers (splitmix64) -----------------------------
__host__ __device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ double u01(unsigned long long key, unsigned long long i) {
  return ((mix64(key ^ mix64(i)) >> 11) + 0.5) * (1.0 / 9007199254740992.0);  // (0, 1)
}
__device__ __forceinline__ double gauss(unsigned long long key, unsigned long long i) {
  const double u1 = u01(key, 2 * i), u2 = u01(key, 2 * i + 1);
  return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

// A_i = H1 diag(s) H2, s_k = kappa_i^(-k/(n-1)), log10 kappa_i uniform in
// [lk0, lk1]; H = product of 4 reflectors I - 2 v v^T / v^T v, v iid N(0,1);
// B_i iid N(0,1). One CTA per system; A_i is built in place in global memory.
__global__ void __launch_bounds__(256)
gen_hh_kernel(const SysRec* __restrict__ sys, int count, double* A, double* B, double lk0,
              double lk1, unsigned long long seed, double* kappa_out) {
  __shared__ double v[512];
  __shared__ double w[512];
  __shared__ double s_vv;
  const int tid = threadIdx.x;
  for (int i = blockIdx.x; i < count; i += gridDim.x) {
    const SysRec d = sys[i];
    const int n = d.n;
    double* a = A + d.a;
    const unsigned long long key = mix64(seed ^ (0xA5A5A5A5ull * (unsigned long long)(i + 1)));
    const double lk = lk0 + (lk1 - lk0) * u01(key, 0x7fffffffull);
    const double kappa = pow(10.0, lk);
    if (tid == 0 && kappa_out) kappa_out[i] = kappa;
    for (int idx = tid; idx < n * n; idx += blockDim.x) {
      const int r = idx / n, c = idx % n;
      a[idx] = (r == c) ? (n > 1 ? pow(kappa, -(double)r / (n - 1)) : 1.0) : 0.0;
    }
    for (int idx = tid; idx < n * d.nrhs; idx += blockDim.x)
      B[d.b + idx] = gauss(key, 0x100000000ull + idx);
    __syncthreads();
    for (int h = 0; h < 8; h++) {
      const bool right = h < 4;
      for (int k = tid; k < n; k += blockDim.x) v[k] = gauss(key, ((unsigned long long)(h + 1) << 40) + k);
      __syncthreads();
      if (tid == 0) {
        double s = 0.0;
        for (int k = 0; k < n; k++) s += v[k] * v[k];
        s_vv = s;
      }
      __syncthreads();
      const double f = 2.0 / s_vv;
      // right: A -= f (A v) v^T ; left: A -= f v (v^T A)
      if (right) {  // w = A v: one warp per row
        const int lane = tid & 31;
        for (int r = tid >> 5; r < n; r += blockDim.x >> 5) {
          double s = 0.0;
          for (int k = lane; k < n; k += 32) s += a[(size_t)r * n + k] * v[k];
          for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
          if (lane == 0) w[r] = s;
        }
      } else {  // w = A^T v: one thread per column
        for (int c = tid; c < n; c += blockDim.x) {
          double s = 0.0;
          for (int k = 0; k < n; k++) s += v[k] * a[(size_t)k * n + c];
          w[c] = s;
        }
      }
      __syncthreads();
      for (int idx = tid; idx < n * n; idx += blockDim.x) {
        const int r = idx / n, c = idx % n;
        a[idx] -= right ? f * w[r] * v[c] : f * v[r] * w[c];
      }
      __syncthreads();
    }
  }
}

// ---- features -----------------------------------------------------------------
// Sum of v over the CTA with one barrier: warp sums go to red[par][warp],
// the slots alternating between calls (par flips on every call, in every
// thread alike), so a slot is rewritten only two calls later, after a barrier
// that every reader of its previous contents has passed.
__device__ double block_sum(double v, double (*red)[8], int& par) {
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  if ((threadIdx.x & 31) == 0) red[par][threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[par][w];
  par ^= 1;
  return t;
}

// log10(max(x, 1e-300)) as a float, from the binary exponent and an FP32 log2
// of the mantissa (x = m 2^e, 1 <= m < 2): the feature is FP32 anyway, and a
// double-precision log10 would occupy GB300's slow FP64 pipe.
__device__ __forceinline__ float lg(double x) {
  x = fmax(x, 1e-300);
  const uint64_t b = la_bits_f64(x);
  const int eb = (int)((b >> 52) & 0x7ff);
  if (eb == 0 || eb == 0x7ff) return (float)log10(x);  // subnormal, infinity, NaN
  const float m = la_f64_to_f32(la_f64_from_bits((b & 0x000fffffffffffffull) |
                                                 0x3ff0000000000000ull));
  return ((float)(eb - 1023) + log2f(m)) * 0.30102999566398120f;
}

constexpr int LK = 4;  // Lanczos steps

struct RowStats {
  float rmax, rmin, dmin, amax, diag_min;
  double fro, dsum, ddom;
};

template <int PF>
__device__ __forceinline__ void load_row_f64(double (&x)[PF], const double* __restrict__ row, int n,
                                             int lane);
__device__ __forceinline__ void load_row_f32(float (&x)[16], const float* row, int n, int lane);

// One Lanczos pass over the rows of warp `warp` (rows warp, warp + NWp, ...):
// t1[r] = a_r . qj and acc += a_r t1[r] (this lane's columns). FIRST: the rows
// come from A in FP64 (converted to FP32 and stored in af), and the row and
// column statistics of pass 0 are taken on the way. The next row's loads are
// issued before the current row is reduced.
template <bool FIRST>
__device__ __forceinline__ void feature_rows(const double* __restrict__ a, float* af, int n,
                                             const float* qj, const float* q0, float* t1,
                                             float (&acc)[16], float (&cs)[16], float (&sq)[16],
                                             RowStats& st, int warp, int lane, int NWp) {
  // Prefetched slots per lane: all 16 from the FP32 copy; 8 (columns < 256)
  // from A in FP64, whose wider raw values would not fit the register budget.
  // The rest of a wider FP64 row is loaded when it is used.
  constexpr int PF = FIRST ? 8 : 16;
  using L = typename std::conditional<FIRST, double, float>::type;
  L xn[PF];
  if (warp < n) {
    if constexpr (FIRST) load_row_f64<PF>(xn, a + (size_t)warp * n, n, lane);
    else load_row_f32(xn, af + (size_t)warp * n, n, lane);
  }
  for (int r = warp; r < n; r += NWp) {
    float x[16];
#pragma unroll
    for (int m = 0; m < 16; m++) {
      if constexpr (FIRST) {
        const int k = lane + 32 * m;
        x[m] = m < PF ? la_f64_to_f32(xn[m < PF ? m : 0])
                      : (k < n ? la_f64_to_f32(__ldg(a + (size_t)r * n + k)) : 0.f);
      } else {
        x[m] = xn[m];
      }
    }
    if (r + NWp < n) {
      if constexpr (FIRST) load_row_f64<PF>(xn, a + (size_t)(r + NWp) * n, n, lane);
      else load_row_f32(xn, af + (size_t)(r + NWp) * n, n, lane);
    }
    float* fr = af + (size_t)r * n;
    float s = 0, rs = 0, f2 = 0, am = 0;
#pragma unroll
    for (int m = 0; m < 16; m++) {
      const int k = lane + 32 * m;
      if (k < n) {
        s = fmaf(x[m], qj[k], s);
        if (FIRST) {
          fr[k] = x[m];
          rs += fabsf(x[m]);
          f2 = fmaf(x[m], x[m], f2);
          am = fmaxf(am, fabsf(x[m]));
        }
      }
    }
    float di = 0.f;
    if (FIRST) {  // the diagonal a_rr: slot r / 32 of lane r % 32
      float xdg = x[0];
#pragma unroll
      for (int m = 1; m < 16; m++) xdg = m == (r >> 5) ? x[m] : xdg;
      di = fabsf(__shfl_sync(0xffffffffu, xdg, r & 31));
    }
    for (int o = 16; o > 0; o >>= 1) {
      s += __shfl_xor_sync(0xffffffffu, s, o);
      if (FIRST) {
        rs += __shfl_xor_sync(0xffffffffu, rs, o);
        f2 += __shfl_xor_sync(0xffffffffu, f2, o);
        am = fmaxf(am, __shfl_xor_sync(0xffffffffu, am, o));
      }
    }
    const float q0r = q0[r];
#pragma unroll
    for (int m = 0; m < 16; m++) {
      acc[m] = fmaf(x[m], s, acc[m]);
      if (FIRST) {
        cs[m] += fabsf(x[m]);
        sq[m] = fmaf(x[m], q0r, sq[m]);
      }
    }
    if (lane == 0) {
      t1[r] = s;
      if (FIRST) {
        const float off = rs - di;
        st.fro += f2;
        st.amax = fmaxf(st.amax, am);
        st.rmax = fmaxf(st.rmax, rs);
        st.rmin = fminf(st.rmin, rs);
        const float ratio = di / fmaxf(off, 1e-30f);
        st.dmin = fminf(st.dmin, ratio);
        st.dsum += log10f(fmaxf(ratio, 1e-30f));
        st.ddom += ratio > 1.f ? 1.0 : 0.0;
        st.diag_min = fminf(st.diag_min, di);
      }
    }
  }
}

// A row's entries k = lane + 32 m (m < PF resp. 16, k < n; zero beyond n)
// into registers, all loads issued before any is used.
template <int PF>
__device__ __forceinline__ void load_row_f64(double (&x)[PF], const double* __restrict__ row, int n,
                                             int lane) {
#pragma unroll
  for (int m = 0; m < PF; m++) {
    const int k = lane + 32 * m;
    x[m] = k < n ? __ldg(row + k) : 0.0;
  }
}
__device__ __forceinline__ void load_row_f32(float (&x)[16], const float* row, int n, int lane) {
#pragma unroll
  for (int m = 0; m < 16; m++) {
    const int k = lane + 32 * m;
    x[m] = k < n ? row[k] : 0.f;
  }
}

// Smallest eigenvalue of the symmetric tridiagonal (alpha, beta) of order
// k <= LK, computed by one full warp (every lane returns it). Multisection on
// the Gershgorin interval: per round, lane l counts the eigenvalues below
// x_l = lo + (hi - lo) (l + 1) / 33 with the division-free Sturm sequence
// p_0 = 1, p_i = (alpha_i - x) p_(i-1) - beta_(i-1)^2 p_(i-2) (the count is
// the number of sign changes; the values stay far inside the FP64 range for
// k <= 4), and a ballot keeps the sub-interval where the count first reaches
// one. Sixteen rounds shrink the interval by 33^16 > 2^80, the resolution of
// 80 bisection steps, with 32 times fewer dependent FP64 operations.
__device__ double tridiag_min_eig_warp(const double* al, const double* be, int k, double sgn) {
  const int lane = threadIdx.x & 31;
  // the tridiagonal sgn * T in registers (compile-time indices, k <= LK)
  double as[LK], bb[LK];
#pragma unroll
  for (int i = 0; i < LK; i++) {
    as[i] = i < k ? sgn * al[i] : 0.0;
    bb[i] = i + 1 < k ? be[i] : 0.0;
  }
  double lo = INFINITY, hi = -INFINITY;
#pragma unroll
  for (int i = 0; i < LK; i++)
    if (i < k) {
      const double r = (i > 0 ? fabs(bb[i - 1]) : 0.0) + fabs(bb[i]);
      lo = fmin(lo, as[i] - r);
      hi = fmax(hi, as[i] + r);
    }
  // Work on T / 2^s with 2^s >= the Gershgorin bound (exact scaling), so the
  // Sturm values stay below 3^k in magnitude whatever the scale of T.
  const double gb = fmax(fabs(lo), fabs(hi));
  int sexp = 0;
  if (gb > 0.0 && gb < INFINITY) frexp(gb, &sexp);
  double bs2[LK];
#pragma unroll
  for (int i = 0; i < LK; i++) {
    as[i] = ldexp(as[i], -sexp);
    const double t = ldexp(bb[i], -sexp);
    bs2[i] = t * t;
  }
  lo = ldexp(lo, -sexp);
  hi = ldexp(hi, -sexp);
  for (int round = 0; round < 16; round++) {
    const double x = lo + (hi - lo) * ((double)(lane + 1) / 33.0);
    double pm2 = 1.0, pm1 = as[0] - x;
    int cnt = pm1 < 0.0 ? 1 : 0;
#pragma unroll
    for (int i = 1; i < LK; i++)
      if (i < k) {
        const double pi = (as[i] - x) * pm1 - bs2[i - 1] * pm2;
        if ((pi < 0.0) != (pm1 < 0.0)) cnt++;
        pm2 = pm1;
        pm1 = pi;
      }
    const unsigned mask = __ballot_sync(0xffffffffu, cnt >= 1);
    const double xl = lo + (hi - lo) * ((double)lane / 33.0);  // lane's left end
    if (mask) {
      const int f = __ffs(mask) - 1;
      const double nlo = __shfl_sync(0xffffffffu, xl, f);
      const double nhi = __shfl_sync(0xffffffffu, x, f);
      lo = nlo;
      hi = nhi;
    } else {
      lo = __shfl_sync(0xffffffffu, x, 31);
    }
  }
  return ldexp(0.5 * (lo + hi), sexp);
}

constexpr int FEAT_CTAS_PER_SM = 4;  // 4 CTAs of 4 warps: four systems in flight per SM

// 16 features per system (one CTA per system). FP64 arithmetic is slow on
// this GPU, so A_i is read in FP64 once and rounded to an FP32 copy in the
// CTA's global scratch slice; every statistic and matrix-vector product works
// in FP32 on that copy (dot products of length n accumulate in FP64). One
// Lanczos step on A^T A is one pass over A: a warp loads a whole row (16
// independent loads per lane), takes t_r = a_r . q, and adds a_r t_r into
// per-lane column accumulators, which are summed across warps in shared
// memory; so both A q and A^T (A q) come from a single read of each element.
// The first pass also reads A in FP64, writes the FP32 copy and takes the row
// and column statistics. LK steps from a fixed start vector q0 with full
// reorthogonalisation; the extreme Ritz values bound sigma_max^2 from below and
// sigma_min^2 from above. The asymmetry feature is the probe
// ||A q0 - A^T q0|| / ||A q0||.
__global__ void __launch_bounds__(128, 4)
features_kernel(const double* __restrict__ A, const SysRec* __restrict__ sys, int count,
                float* __restrict__ F, float* __restrict__ scratch) {
  __shared__ double red[2][8];
  int rpar = 0;
  __shared__ float q[LK + 1][512];
  __shared__ float t1[512];
  __shared__ float t2[512];
  __shared__ float part[8][512];  // per-warp column partial sums
  __shared__ double al[LK], be[LK];
  __shared__ float finf[8][7];   // per-warp extrema
  __shared__ double find[8][5];  // per-warp sums
  __shared__ float totf[7];      // combined extrema
  __shared__ double totd[7];     // combined sums, then the extreme Ritz values
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int NWp = blockDim.x >> 5;
  float* af = scratch + (size_t)blockIdx.x * 512 * 512;
  for (int i = blockIdx.x; i < count; i += gridDim.x) {
    const SysRec d = sys[i];
    const int n = d.n;
    const double* a = A + d.a;
    double nrm = 0;
    for (int k = tid; k < n; k += blockDim.x) {
      const float v = 1.0f + 0.5f * sinf(1.0f + (float)k);
      q[0][k] = v;
      nrm += (double)v * v;
    }
    nrm = sqrt(block_sum(nrm, red, rpar));
    for (int k = tid; k < n; k += blockDim.x) q[0][k] = (float)(q[0][k] / nrm);
    __syncthreads();
    RowStats st = {0.f, INFINITY, INFINITY, 0.f, INFINITY, 0.0, 0.0, 0.0};
    float cmax = 0, cmin = INFINITY;
    double asym = 0, aq = 0;
    int kk = 0;
    for (int j = 0; j < LK && j < n; j++) {
      float acc[16], cs[16], sq[16];
#pragma unroll
      for (int m = 0; m < 16; m++) { acc[m] = 0.f; cs[m] = 0.f; sq[m] = 0.f; }
      // Rows are software-pipelined per warp (feature_rows): the next row's
      // loads are issued before the current row's reduction, so the memory
      // latency overlaps the shuffles.
      if (j == 0)
        feature_rows<true>(a, af, n, q[0], q[0], t1, acc, cs, sq, st, warp, lane, NWp);
      else
        feature_rows<false>(a, af, n, q[j], q[0], t1, acc, cs, sq, st, warp, lane, NWp);
      // t2 = A^T t1: sum the warps' column partials
#pragma unroll
      for (int m = 0; m < 16; m++)
        if (lane + 32 * m < n) part[warp][lane + 32 * m] = acc[m];
      __syncthreads();
      for (int c = tid; c < n; c += blockDim.x) {
        float t = 0.f;
        for (int w = 0; w < NWp; w++) t += part[w][c];
        t2[c] = t;
      }
      __syncthreads();
      if (j == 0) {  // column sums of |A| and A^T q0, the same way
#pragma unroll
        for (int m = 0; m < 16; m++)
          if (lane + 32 * m < n) part[warp][lane + 32 * m] = cs[m];
        __syncthreads();
        for (int c = tid; c < n; c += blockDim.x) {
          float t = 0.f;
          for (int w = 0; w < NWp; w++) t += part[w][c];
          cmax = fmaxf(cmax, t);
          cmin = fminf(cmin, t);
        }
        __syncthreads();
#pragma unroll
        for (int m = 0; m < 16; m++)
          if (lane + 32 * m < n) part[warp][lane + 32 * m] = sq[m];
        __syncthreads();
        for (int c = tid; c < n; c += blockDim.x) {
          float t = 0.f;
          for (int w = 0; w < NWp; w++) t += part[w][c];
          const double dd = la_f32_to_f64(t1[c]) - la_f32_to_f64(t);  // (A q0)_c - (A^T q0)_c
          asym += dd * dd;
          aq = fma(la_f32_to_f64(t1[c]), la_f32_to_f64(t1[c]), aq);
        }
        __syncthreads();
      }
      double aj = 0;
      for (int k = tid; k < n; k += blockDim.x)
        aj = fma(la_f32_to_f64(q[j][k]), la_f32_to_f64(t2[k]), aj);
      aj = block_sum(aj, red, rpar);
      for (int pq = 0; pq <= j; pq++) {  // full reorthogonalisation
        double c = 0;
        for (int k = tid; k < n; k += blockDim.x)
          c = fma(la_f32_to_f64(q[pq][k]), la_f32_to_f64(t2[k]), c);
        c = block_sum(c, red, rpar);
        // each thread updates and later reads only its own entries of t2
        for (int k = tid; k < n; k += blockDim.x)
          t2[k] = la_f64_to_f32(fma(-c, la_f32_to_f64(q[pq][k]), la_f32_to_f64(t2[k])));
      }
      double bj = 0;
      for (int k = tid; k < n; k += blockDim.x)
        bj = fma(la_f32_to_f64(t2[k]), la_f32_to_f64(t2[k]), bj);
      bj = sqrt(block_sum(bj, red, rpar));
      if (tid == 0) { al[j] = aj; be[j] = bj; }
      kk = j + 1;
      if (!(bj > 1e-6 * fabs(aj)) || j + 1 >= LK) break;
      const double ibj = 1.0 / bj;
      for (int k = tid; k < n; k += blockDim.x)
        q[j + 1][k] = la_f64_to_f32(la_f32_to_f64(t2[k]) * ibj);
      __syncthreads();
    }
    // The twelve statistics: a warp reduction each, one barrier, then lane l
    // of warp 0 combines statistic l over the warps.
    {
      // FP32 extrema (max: rmax, amax, cmax; min: rmin, dmin, diag_min, cmin)
      // and FP64 sums (dsum, ddom, fro, asym, aq).
      float v[7] = {st.rmax, st.amax, cmax, st.rmin, st.dmin, st.diag_min, cmin};
      double w[5] = {st.dsum, st.ddom, st.fro, asym, aq};
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
        for (int t = 0; t < 3; t++) v[t] = fmaxf(v[t], __shfl_xor_sync(0xffffffffu, v[t], off));
#pragma unroll
        for (int t = 3; t < 7; t++) v[t] = fminf(v[t], __shfl_xor_sync(0xffffffffu, v[t], off));
#pragma unroll
        for (int t = 0; t < 5; t++) w[t] += __shfl_xor_sync(0xffffffffu, w[t], off);
      }
      if (lane == 0) {
#pragma unroll
        for (int t = 0; t < 7; t++) finf[warp][t] = v[t];
#pragma unroll
        for (int t = 0; t < 5; t++) find[warp][t] = w[t];
      }
      __syncthreads();
      if (warp == 0) {
        if (lane < 7) {
          float acc = finf[0][lane];
          for (int ww = 1; ww < NWp; ww++)
            acc = lane < 3 ? fmaxf(acc, finf[ww][lane]) : fminf(acc, finf[ww][lane]);
          totf[lane] = acc;
        } else if (lane < 12) {
          double acc = find[0][lane - 7];
          for (int ww = 1; ww < NWp; ww++) acc += find[ww][lane - 7];
          totd[lane - 7] = acc;
        }
        // extreme Ritz values of the Lanczos tridiagonal
        const double emax = -tridiag_min_eig_warp(al, be, kk, -1.0);
        const double emin = fmax(tridiag_min_eig_warp(al, be, kk, 1.0), emax * 1e-32);
        if (lane == 0) { totd[5] = emax; totd[6] = emin; }
      }
      __syncthreads();
    }
    const double rmax_b = totf[0], amax_b = totf[1], cmax_b = totf[2];
    const double rmin_b = totf[3], dmin_b = totf[4], diag_b = totf[5], cmin_b = totf[6];
    const double dsum = totd[0], ddom = totd[1], fro = totd[2];
    asym = totd[3];
    aq = totd[4];
    const double emax = totd[5], emin = totd[6];
    if (tid == 0) {
      float* f = F + (size_t)i * NF;
      f[0] = (float)(log2((double)n) / 9.0);
      f[1] = (float)d.nrhs / 4.f;
      f[2] = lg(rmax_b);
      f[3] = lg(cmax_b);
      f[4] = lg(sqrt(fro));
      f[5] = lg(amax_b);
      f[6] = lg(sqrt(fmax(emax, 0.0)));
      f[7] = lg(sqrt(fro) / sqrt(fmax(emax, 1e-300)));
      f[8] = lg(dmin_b);
      f[9] = (float)(dsum / n);
      f[10] = (float)(ddom / n);
      f[11] = lg(rmax_b / fmax(rmin_b, 1e-300));
      f[12] = lg(cmax_b / fmax(cmin_b, 1e-300));
      f[13] = (float)(sqrt(asym) / fmax(sqrt(aq), 1e-300));
      f[14] = lg(diag_b / fmax(amax_b, 1e-300));
      f[15] = lg(sqrt(fmax(emax, 1e-300) / emin));
    }
    __syncthreads();
  }
}

// ---- MLP ------------------------------------------------------------------------
// Forward for one sample: x normalised -> h1 -> h2 -> logits -> softmax.
__device__ void mlp_fwd(const float* __restrict__ P, const float* x, float* h1, float* h2,
                        float* pr) {
  for (int o = 0; o < H1; o++) {
    float s = P[OFF_B1 + o];
    for (int k = 0; k < NF; k++) s = fmaf(P[OFF_W1 + o * NF + k], x[k], s);
    h1[o] = fmaxf(s, 0.f);
  }
  for (int o = 0; o < H2; o++) {
    float s = P[OFF_B2 + o];
    for (int k = 0; k < H1; k++) s = fmaf(P[OFF_W2 + o * H1 + k], h1[k], s);
    h2[o] = fmaxf(s, 0.f);
  }
  float lg3[NC], mx = -INFINITY;
  for (int o = 0; o < NC; o++) {
    float s = P[OFF_B3 + o];
    for (int k = 0; k < H2; k++) s = fmaf(P[OFF_W3 + o * H2 + k], h2[k], s);
    lg3[o] = s;
    mx = fmaxf(mx, s);
  }
  float z = 0.f;
  for (int o = 0; o < NC; o++) { lg3[o] = expf(lg3[o] - mx); z += lg3[o]; }
  for (int o = 0; o < NC; o++) pr[o] = lg3[o] / z;
}

// One thread per sample: normalise, forward, keep activations; with labels,
// also the per-sample output delta and loss: the softmax cross-entropy, or,
// with per-sample class costs (cost, NC per sample), the expected cost
// sum_c p_c cost_c, whose gradient with respect to the logits is
// p_c (cost_c - sum_j p_j cost_j).
// Gate of the class output (inference): a linear score of the raw features
// and the class probabilities, w[0..15] . x + w[16..18] . p + b; a system
// whose score is >= 0 gets class 3 (no mixed attempt, straight to the FP64
// pass). on = 0: no gate.
constexpr int GATE_NCOEF = NF + NC;
struct Gate {
  float w[GATE_NCOEF];
  float b;
  int on;
};

__global__ void mlp_forward_kernel(const float* __restrict__ P, const float* __restrict__ mean,
                                   const float* __restrict__ stdv, const float* __restrict__ X,
                                   int count, float* __restrict__ act, float* __restrict__ probs,
                                   int* __restrict__ cls, const int* __restrict__ y,
                                   const float* __restrict__ cost, float* __restrict__ loss,
                                   Gate gate) {
  __shared__ float Ps[NPARAM];
  for (int i = threadIdx.x; i < NPARAM; i += blockDim.x) Ps[i] = P[i];
  __syncthreads();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= count) return;
  float x[NF], h1[H1], h2[H2], pr[NC];
  for (int k = 0; k < NF; k++) x[k] = (X[(size_t)s * NF + k] - mean[k]) / stdv[k];
  mlp_fwd(Ps, x, h1, h2, pr);
  if (act) {
    float* a = act + (size_t)s * ACT;
    for (int k = 0; k < NF; k++) a[k] = x[k];
    for (int k = 0; k < H1; k++) a[NF + k] = h1[k];
    for (int k = 0; k < H2; k++) a[NF + H1 + k] = h2[k];
    if (cost) {
      float ec = 0.f;
      for (int k = 0; k < NC; k++) ec = fmaf(pr[k], cost[(size_t)s * NC + k], ec);
      for (int k = 0; k < NC; k++) a[NF + H1 + H2 + k] = pr[k] * (cost[(size_t)s * NC + k] - ec);
    } else {
      for (int k = 0; k < NC; k++) a[NF + H1 + H2 + k] = pr[k] - ((y && y[s] == k) ? 1.f : 0.f);
    }
  }
  if (probs)
    for (int k = 0; k < NC; k++) probs[(size_t)s * NC + k] = pr[k];
  if (cls) {
    int best = 0;
    for (int k = 1; k < NC; k++)
      if (pr[k] > pr[best]) best = k;
    if (gate.on) {
      float g = gate.b;
      for (int k = 0; k < NF; k++) g = fmaf(gate.w[k], X[(size_t)s * NF + k], g);
      for (int k = 0; k < NC; k++) g = fmaf(gate.w[NF + k], pr[k], g);
      if (g >= 0.f) best = NC;  // straight to the FP64 pass
    }
    cls[s] = best;
  }
  if (loss && cost) {
    float ec = 0.f;
    for (int k = 0; k < NC; k++) ec = fmaf(pr[k], cost[(size_t)s * NC + k], ec);
    loss[s] = ec;
  } else if (loss && y) {
    loss[s] = -logf(fmaxf(pr[y[s]], 1e-30f));
  }
}

// Hidden-layer deltas per sample: d2 = (W3^T d3) . [h2 > 0], d1 = (W2^T d2) . [h1 > 0].
__global__ void mlp_delta_kernel(const float* __restrict__ P, const float* __restrict__ act,
                                 int count, float* __restrict__ delta) {
  __shared__ float Ps[NPARAM];
  for (int i = threadIdx.x; i < NPARAM; i += blockDim.x) Ps[i] = P[i];
  __syncthreads();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= count) return;
  const float* a = act + (size_t)s * ACT;
  const float* h1 = a + NF;
  const float* h2 = a + NF + H1;
  const float* d3 = a + NF + H1 + H2;
  float d2[H2];
  float* out = delta + (size_t)s * (H1 + H2);
  for (int k = 0; k < H2; k++) {
    float t = 0.f;
    for (int o = 0; o < NC; o++) t = fmaf(Ps[OFF_W3 + o * H2 + k], d3[o], t);
    d2[k] = h2[k] > 0.f ? t : 0.f;
    out[H1 + k] = d2[k];
  }
  for (int k = 0; k < H1; k++) {
    float t = 0.f;
    for (int o = 0; o < H2; o++) t = fmaf(Ps[OFF_W2 + o * H1 + k], d2[o], t);
    out[k] = h1[k] > 0.f ? t : 0.f;
  }
}

// Mean gradient of the loss: one thread per parameter, samples summed in index
// order (deterministic).
__global__ void mlp_grad_kernel(const float* __restrict__ act, const float* __restrict__ delta,
                                int count, float* __restrict__ G) {
  const int pidx = blockIdx.x * blockDim.x + threadIdx.x;
  if (pidx >= NPARAM) return;
  float g = 0.f;
  for (int s = 0; s < count; s++) {
    const float* a = act + (size_t)s * ACT;
    const float* dl = delta + (size_t)s * (H1 + H2);
    float v;
    if (pidx < OFF_B1) { const int o = pidx / NF, k = pidx % NF; v = dl[o] * a[k]; }
    else if (pidx < OFF_W2) { v = dl[pidx - OFF_B1]; }
    else if (pidx < OFF_B2) { const int q = pidx - OFF_W2, o = q / H1, k = q % H1; v = dl[H1 + o] * a[NF + k]; }
    else if (pidx < OFF_W3) { v = dl[H1 + pidx - OFF_B2]; }
    else if (pidx < OFF_B3) { const int q = pidx - OFF_W3, o = q / H2, k = q % H2; v = a[NF + H1 + H2 + o] * a[NF + H1 + k]; }
    else { v = a[NF + H1 + H2 + (pidx - OFF_B3)]; }
    g += v;
  }
  G[pidx] = g / (float)count;
}

// Adam (beta1 0.9, beta2 0.999, eps 1e-8), t = step number from 1.
__global__ void adam_kernel(float* __restrict__ P, const float* __restrict__ G, float* __restrict__ m,
                            float* __restrict__ v, float lr, int t) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= NPARAM) return;
  const float b1 = 0.9f, b2 = 0.999f;
  m[i] = b1 * m[i] + (1.f - b1) * G[i];
  v[i] = b2 * v[i] + (1.f - b2) * G[i] * G[i];
  const float mh = m[i] / (1.f - powf(b1, (float)t));
  const float vh = v[i] / (1.f - powf(b2, (float)t));
  P[i] -= lr * mh / (sqrtf(vh) + 1e-8f);
}

}  // namespace

struct la_mlp_s {
  la_ctx ctx;
  float* d_params = nullptr;  // NPARAM + 2 * NF (mean, std) + 2 * NPARAM (Adam) + NPARAM (grad)
  int step = 0;
  float* P() { return d_params; }
  float* mean() { return d_params + NPARAM; }
  float* stdv() { return d_params + NPARAM + NF; }
  float* am() { return d_params + NPARAM + 2 * NF; }
  float* av() { return am() + NPARAM; }
  float* grad() { return av() + NPARAM; }
  Gate gate{};  // la_mlp_set_gate (off)
};

extern "C" {

int la_mlp_param_count(void) { return NPARAM; }

la_status la_mlp_create(la_ctx ctx, unsigned long long seed, la_mlp* out) {
  if (!ctx || !out) return LA_INVALID;
  LA_CUDA(ctx, cudaSetDevice(ctx->device));
  la_mlp m = new (std::nothrow) la_mlp_s();
  if (!m) return LA_NOMEM;
  m->ctx = ctx;
  const size_t total = NPARAM + 2 * NF + 3 * (size_t)NPARAM;
  la_status s = la_device_alloc(ctx, reinterpret_cast<void**>(&m->d_params), total * sizeof(float));
  if (s != LA_OK) { delete m; return s; }
  // He-style uniform init from a seeded splitmix64 stream; normalisation 0/1.
  std::vector<float> h(total, 0.f);
  unsigned long long st = seed;
  auto uni = [&]() { st = mix64(st); return (float)((st >> 11) * (1.0 / 9007199254740992.0)) * 2.f - 1.f; };
  for (int i = 0; i < H1 * NF; i++) h[OFF_W1 + i] = uni() * sqrtf(6.f / NF);
  for (int i = 0; i < H2 * H1; i++) h[OFF_W2 + i] = uni() * sqrtf(6.f / H1);
  for (int i = 0; i < NC * H2; i++) h[OFF_W3 + i] = uni() * sqrtf(6.f / H2);
  for (int k = 0; k < NF; k++) h[NPARAM + NF + k] = 1.f;
  cudaError_t e = cudaMemcpyAsync(m->d_params, h.data(), total * sizeof(float),
                                  cudaMemcpyHostToDevice, ctx->stream);
  if (e != cudaSuccess) { s = la_cuda_fail(ctx, e, "mlp init"); la_device_free(ctx, m->d_params); delete m; return s; }
  s = la_sync_and_check(ctx, "mlp init");
  if (s != LA_OK) { la_device_free(ctx, m->d_params); delete m; return s; }
  *out = m;
  return LA_OK;
}

void la_mlp_destroy(la_mlp m) {
  if (!m) return;
  cudaSetDevice(m->ctx->device);
  la_device_free(m->ctx, m->d_params);
  cudaStreamSynchronize(m->ctx->stream);
  delete m;
}

// params: NPARAM weights then NF means and NF standard deviations (host).
la_status la_mlp_get_params(la_mlp m, float* params) {
  if (!m || !params) return LA_INVALID;
  LA_CUDA(m->ctx, cudaMemcpyAsync(params, m->d_params, (NPARAM + 2 * NF) * sizeof(float),
                                  cudaMemcpyDeviceToHost, m->ctx->stream));
  return la_sync_and_check(m->ctx, "mlp params");
}

la_status la_mlp_set_params(la_mlp m, const float* params) {
  if (!m || !params) return LA_INVALID;
  LA_CUDA(m->ctx, cudaMemcpyAsync(m->d_params, params, (NPARAM + 2 * NF) * sizeof(float),
                                  cudaMemcpyHostToDevice, m->ctx->stream));
  LA_CUDA(m->ctx, cudaMemsetAsync(m->am(), 0, 3 * (size_t)NPARAM * sizeof(float), m->ctx->stream));
  m->step = 0;
  return la_sync_and_check(m->ctx, "mlp params");
}

// Mean gradient over count samples (device X) of the cross-entropy for labels
// y, or of the expected cost for per-sample class costs (d_cost non-null),
// into m->grad(), without updating.
static la_status mlp_backprop(la_mlp m, const float* d_x, const int* d_y, const float* d_cost,
                              int count, float* loss) {
  la_ctx ctx = m->ctx;
  float *act = nullptr, *delta = nullptr, *dl = nullptr;
  la_status s = la_device_alloc(ctx, reinterpret_cast<void**>(&act), (size_t)count * ACT * 4);
  if (s == LA_OK) s = la_device_alloc(ctx, reinterpret_cast<void**>(&delta), (size_t)count * (H1 + H2) * 4);
  if (s == LA_OK) s = la_device_alloc(ctx, reinterpret_cast<void**>(&dl), (size_t)count * 4);
  if (s == LA_OK) {
    const int g = (count + 127) / 128;
    mlp_forward_kernel<<<g, 128, 0, ctx->stream>>>(m->P(), m->mean(), m->stdv(), d_x, count, act,
                                                   nullptr, nullptr, d_y, d_cost, dl, Gate{});
    mlp_delta_kernel<<<g, 128, 0, ctx->stream>>>(m->P(), act, count, delta);
    mlp_grad_kernel<<<(NPARAM + 127) / 128, 128, 0, ctx->stream>>>(act, delta, count, m->grad());
    ctx->launches += 3;
    s = la_check_launch(ctx, "mlp backprop");
  }
  if (s == LA_OK && loss) {
    std::vector<float> h(count);
    cudaError_t e = cudaMemcpyAsync(h.data(), dl, count * 4, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) s = la_cuda_fail(ctx, e, "loss");
    double t = 0;
    for (float v : h) t += v;
    *loss = (float)(t / count);
  }
  la_device_free(ctx, act);
  la_device_free(ctx, delta);
  la_device_free(ctx, dl);
  return s;
}

la_status la_mlp_gradients(la_mlp m, const float* d_x, const int* d_y, int count, float* grad,
                           float* loss) {
  if (!m || !d_x || !d_y || count <= 0) return LA_INVALID;
  LA_CUDA(m->ctx, cudaSetDevice(m->ctx->device));
  LA_TRY(mlp_backprop(m, d_x, d_y, nullptr, count, loss));
  if (grad) {
    LA_CUDA(m->ctx, cudaMemcpyAsync(grad, m->grad(), NPARAM * sizeof(float),
                                    cudaMemcpyDeviceToHost, m->ctx->stream));
  }
  return la_sync_and_check(m->ctx, "mlp gradients");
}

la_status la_mlp_train_step(la_mlp m, const float* d_x, const int* d_y, int count, float lr,
                            float* loss) {
  if (!m || !d_x || !d_y || count <= 0) return LA_INVALID;
  LA_CUDA(m->ctx, cudaSetDevice(m->ctx->device));
  LA_TRY(mlp_backprop(m, d_x, d_y, nullptr, count, loss));
  m->step++;
  adam_kernel<<<(NPARAM + 127) / 128, 128, 0, m->ctx->stream>>>(m->P(), m->grad(), m->am(),
                                                                 m->av(), lr, m->step);
  m->ctx->launches++;
  return la_check_launch(m->ctx, "adam");
}

la_status la_mlp_gradients_cost(la_mlp m, const float* d_x, const float* d_cost, int count,
                                float* grad, float* loss) {
  if (!m || !d_x || !d_cost || count <= 0) return LA_INVALID;
  LA_CUDA(m->ctx, cudaSetDevice(m->ctx->device));
  LA_TRY(mlp_backprop(m, d_x, nullptr, d_cost, count, loss));
  if (grad) {
    LA_CUDA(m->ctx, cudaMemcpyAsync(grad, m->grad(), NPARAM * sizeof(float),
                                    cudaMemcpyDeviceToHost, m->ctx->stream));
  }
  return la_sync_and_check(m->ctx, "mlp gradients (cost)");
}

la_status la_mlp_train_step_cost(la_mlp m, const float* d_x, const float* d_cost, int count,
                                 float lr, float* loss) {
  if (!m || !d_x || !d_cost || count <= 0) return LA_INVALID;
  LA_CUDA(m->ctx, cudaSetDevice(m->ctx->device));
  LA_TRY(mlp_backprop(m, d_x, nullptr, d_cost, count, loss));
  m->step++;
  adam_kernel<<<(NPARAM + 127) / 128, 128, 0, m->ctx->stream>>>(m->P(), m->grad(), m->am(),
                                                                 m->av(), lr, m->step);
  m->ctx->launches++;
  return la_check_launch(m->ctx, "adam");
}

la_status la_mlp_set_gate(la_mlp m, const float* coef, float bias) {
  if (!m) return LA_INVALID;
  Gate g{};
  if (coef) {
    for (int k = 0; k < GATE_NCOEF; k++) {
      if (!std::isfinite(coef[k])) return LA_INVALID;
      g.w[k] = coef[k];
    }
    if (!std::isfinite(bias)) return LA_INVALID;
    g.b = bias;
    g.on = 1;
  }
  m->gate = g;
  return LA_OK;
}

la_status la_mlp_predict(la_mlp m, const float* d_x, int count, float* d_probs, int* d_class) {
  if (!m || !d_x || count <= 0) return LA_INVALID;
  LA_CUDA(m->ctx, cudaSetDevice(m->ctx->device));
  mlp_forward_kernel<<<(count + 127) / 128, 128, 0, m->ctx->stream>>>(
      m->P(), m->mean(), m->stdv(), d_x, count, nullptr, d_probs, d_class, nullptr, nullptr,
      nullptr, m->gate);
  m->ctx->launches++;
  return la_check_launch(m->ctx, "mlp predict");
}

la_status la_batch_features_device(la_ctx ctx, const double* d_a, const la_batch_system* systems,
                                   int count, float* d_features) {
  if (!ctx || !d_a || !systems || !d_features || count <= 0) return LA_INVALID;
  LA_CUDA(ctx, cudaSetDevice(ctx->device));
  std::vector<SysRec> h(count);
  for (int i = 0; i < count; i++) {
    if (systems[i].n < 1 || systems[i].n > 512) return LA_UNSUPPORTED;
    h[i] = {(long long)systems[i].a_offset, (long long)systems[i].b_offset, systems[i].n,
            systems[i].nrhs};
  }
  SysRec* d = nullptr;
  float* scr = nullptr;
  const int grid = std::min(count, ctx->sm_count * FEAT_CTAS_PER_SM);
  LA_TRY(la_device_alloc(ctx, reinterpret_cast<void**>(&d), count * sizeof(SysRec)));
  la_status s = la_device_alloc(ctx, reinterpret_cast<void**>(&scr),
                                (size_t)grid * 512 * 512 * sizeof(float));
  if (s == LA_OK) {
    cudaError_t e = cudaMemcpyAsync(d, h.data(), count * sizeof(SysRec), cudaMemcpyHostToDevice,
                                    ctx->stream);
    if (e != cudaSuccess) s = la_cuda_fail(ctx, e, "features upload");
  }
  if (s == LA_OK) {
    features_kernel<<<grid, 128, 0, ctx->stream>>>(d_a, d, count, d_features, scr);
    ctx->launches++;
    s = la_check_launch(ctx, "features_kernel");
  }
  la_device_free(ctx, d);
  la_device_free(ctx, scr);
  if (s == LA_OK) s = la_sync_and_check(ctx, "features");
  return s;
}

la_status la_generate_conditioned_batch(la_ctx ctx, const la_batch_system* systems, int count,
                                        double log10_kappa_min, double log10_kappa_max,
                                        unsigned long long seed, double* d_a, double* d_b,
                                        double* d_kappa) {
  if (!ctx || !systems || !d_a || !d_b || count <= 0) return LA_INVALID;
  LA_CUDA(ctx, cudaSetDevice(ctx->device));
  std::vector<SysRec> h(count);
  for (int i = 0; i < count; i++) {
    if (systems[i].n < 1 || systems[i].n > 512) return LA_UNSUPPORTED;
    h[i] = {(long long)systems[i].a_offset, (long long)systems[i].b_offset, systems[i].n,
            systems[i].nrhs};
  }
  SysRec* d = nullptr;
  LA_TRY(la_device_alloc(ctx, reinterpret_cast<void**>(&d), count * sizeof(SysRec)));
  cudaError_t e = cudaMemcpyAsync(d, h.data(), count * sizeof(SysRec), cudaMemcpyHostToDevice,
                                  ctx->stream);
  la_status s = e == cudaSuccess ? LA_OK : la_cuda_fail(ctx, e, "generator upload");
  if (s == LA_OK) {
    gen_hh_kernel<<<std::min(count, ctx->sm_count * 8), 256, 0, ctx->stream>>>(
        d, count, d_a, d_b, log10_kappa_min, log10_kappa_max, seed, d_kappa);
    ctx->launches++;
    s = la_check_launch(ctx, "gen_hh_kernel");
  }
  la_device_free(ctx, d);
  if (s == LA_OK) s = la_sync_and_check(ctx, "generator");
  return s;
}

}  // extern "C"
