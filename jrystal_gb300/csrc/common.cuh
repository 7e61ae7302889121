// Shared helpers for the jrystal_gb300 CUDA library (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>

namespace jrg {

// Complex element type per real precision: float2 for fp32, double2 for fp64.
template <typename R> struct cplx;
template <> struct cplx<float> { using type = float2; };
template <> struct cplx<double> { using type = double2; };
template <typename R> using C_t = typename cplx<R>::type;

template <typename C> __host__ __device__ __forceinline__ C cmk(double x, double y) {
  C r; r.x = (decltype(r.x))x; r.y = (decltype(r.y))y; return r;
}
__host__ __device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__host__ __device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
// a * conj(b)
__host__ __device__ __forceinline__ float2 cmulc(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, a.y * b.y), fmaf(a.y, b.x, -a.x * b.y));
}
__host__ __device__ __forceinline__ double2 cmulc(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, a.y * b.y), fma(a.y, b.x, -a.x * b.y));
}
__host__ __device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__host__ __device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
template <typename C> __host__ __device__ __forceinline__ C czero() { C r; r.x = 0; r.y = 0; return r; }

// FP32 twiddle for the FP64 pair (c, s) = (cos, sin): of the floats next to c
// and next to s (one each side, or the value itself when exact), the pair
// whose squared norm c^2 + s^2 is closest to 1, the nearest pair on ties.
// Nearest rounding alone leaves every |w|^2 - 1 at up to 1e-7 with a sum over
// a table that does not cancel, i.e. a fixed norm loss or gain of every
// transform that uses the table.
__host__ __device__ inline float2 balanced_twiddle(double c, double s) {
  const float c0 = (float)c, s0 = (float)s;
  const float c1 = (double)c0 == c ? c0 : nextafterf(c0, (double)c0 < c ? 2.f : -2.f);
  const float s1 = (double)s0 == s ? s0 : nextafterf(s0, (double)s0 < s ? 2.f : -2.f);
  float2 best = make_float2(c0, s0);
  double be = fabs((double)c0 * c0 + (double)s0 * s0 - 1.0);
  const float cs[2] = {c0, c1}, ss[2] = {s0, s1};
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) {
      const double e = fabs((double)cs[i] * cs[i] + (double)ss[j] * ss[j] - 1.0);
      if (e < be) { be = e; best = make_float2(cs[i], ss[j]); }
    }
  return best;
}

// Weights of a band group for the density partials, formed by warp 0 of the
// block (the FP64 work stays off the other warps): sw[b - b_begin] = w[b] /
// w_ref with w_ref the largest |w| of w[b_begin, b_end) (ratios 0 when all are
// zero), and, in x-block 0, gscale[grp] = w_ref * wscale.  Partials are
// accumulated with the ratios and scaled by gscale in FP64 when reduced.
// The caller synchronises the block before reading sw.
template <typename R>
__device__ __forceinline__ void group_weights(const double* __restrict__ w, int b_begin, int b_end,
                                              double wscale, double* __restrict__ gscale, int grp,
                                              R* sw) {
  if (threadIdx.x >= 32) return;
  const int lane = threadIdx.x;
  double wref = 0.0;
  for (int b = b_begin + lane; b < b_end; b += 32) wref = fmax(wref, fabs(w[b]));
  for (int o = 16; o > 0; o >>= 1) wref = fmax(wref, __shfl_xor_sync(0xffffffffu, wref, o));
  const double winv = wref > 0.0 ? 1.0 / wref : 0.0;
  for (int b = b_begin + lane; b < b_end; b += 32) sw[b - b_begin] = (R)(w[b] * winv);
  if (lane == 0 && blockIdx.x == 0) gscale[grp] = wref * wscale;
}

// bytes of the group-weight array of the density kernels (16-byte aligned start)
__host__ __device__ constexpr size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

// Block-wide sum of a double (all threads get the result).  blockDim.x must
// be a multiple of 32 and at most 1024.
__device__ __forceinline__ double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  const int nw = blockDim.x >> 5;
  double t = 0.0;
  for (int i = 0; i < nw; ++i) t += red[i];
  __syncthreads();
  return t;
}

// optax.adam (scale_by_adam + scale(-lr)) for one element: updates the
// moments in place and returns the parameter increment.
template <typename R>
__device__ __forceinline__ R adam_one(R g, R& m, R& v, R lr, R b1, R b2, R c1, R c2, R eps) {
  m = b1 * m + (1 - b1) * g;
  v = b2 * v + (1 - b2) * g * g;
  return -lr * (m / c1) / (sqrt(v / c2) + eps);
}

// cp.async (sm_80+) copies of 4, 8 or 16 bytes into shared memory
template <int BYTES>
__device__ __forceinline__ void cp_async(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(sa), "l"(gmem), "n"(BYTES) : "memory");
}
// cp.async of BYTES bytes, zero-filled when !pred (no bytes are read then;
// gmem must still be a valid address)
template <int BYTES>
__device__ __forceinline__ void cp_async_zfill(void* smem, const void* gmem, bool pred) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  const int n = pred ? BYTES : 0;
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;" ::"r"(sa), "l"(gmem), "n"(BYTES),
               "r"(n) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

}  // namespace jrg
