// Cholesky factor and inverse of the Gram matrices of the FP32 path, in
// double-float arithmetic on the FP32 pipes.
//
// FP64 arithmetic runs at 1/64 of the FP32 rate on this GPU, and a 160-band
// Cholesky + triangular inverse is ~5.5 million complex multiply-adds per
// (s,k) block, one CTA each; in FP64 through global memory that took 3.1 ms
// for the nine blocks of the 64-atom cell.  Here each block's upper triangle
// lives in shared memory (packed rows, 16 bytes per complex entry: 206 KB at
// 160 bands) as double-float pairs (hi + lo, about 48 significant bits: the
// Dekker/Knuth error-free transformations TwoSum and TwoProd, the latter with
// an FMA), and both the factorisation and the inversion take one barrier per
// pivot (256 threads up to 64 bands, 1024 above; the FP64 element-parallel
// kernel takes more bands than the shared memory holds):
//   factorisation (R^H R = S, R upper): at pivot k every thread reads the
//     unscaled pivot d_k = U[k][k] and updates U[i][j] -= conj(U[k][i])
//     U[k][j] / d_k for k < i <= j (one warp per row, lanes along j); the rows
//     are scaled by 1/sqrt(d_k) once at the end;
//   inversion (X = R^{-1}, in place, bottom-up): location (k, j > k) holds
//     a_kj = -sum_{l > k} R[k][l] X[l][j] when pivot k is reached, so
//     X[k][j] = a_kj / R[k][k] and X[k][k] = 1 / R[k][k]; the rows i < k are
//     updated with X[i][j] -= R[i][k] X[k][j] (j > k) and X[i][k] = -R[i][k] X[k][k],
//     each warp reading R[i][k] before its lane j = k overwrites it; the
//     rows are scaled at the end.
// A pivot d_k <= min_pivot * S_kk, or a non-finite one, sets the breakdown
// bit and is replaced by 1 (as the FP64 kernels do); the condition estimate
// max_k S_kk / d_k goes to the flag word.
#include "plan.h"

namespace jrg {

namespace dfa {

struct df { float hi, lo; };

__device__ __forceinline__ df from_d(double x) {
  const float h = (float)x;
  return {h, (float)(x - (double)h)};
}
__device__ __forceinline__ double to_d(df a) { return (double)a.hi + (double)a.lo; }
// s + e = a + b exactly (Knuth's TwoSum)
__device__ __forceinline__ df two_sum(float a, float b) {
  const float s = a + b, bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
// |a| >= |b| (Dekker's Fast2Sum)
__device__ __forceinline__ df fast_two_sum(float a, float b) {
  const float s = a + b;
  return {s, b - (s - a)};
}
__device__ __forceinline__ df add(df a, df b) {
  df s = two_sum(a.hi, b.hi);
  s.lo += a.lo + b.lo;
  return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df neg(df a) { return {-a.hi, -a.lo}; }
// product, the high part's rounding error recovered with an FMA
__device__ __forceinline__ df mul(df a, df b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}

struct dc { df re, im; };   // complex double-float

__device__ __forceinline__ dc ld(const float4* p) {
  const float4 v = *p;
  return {{v.x, v.y}, {v.z, v.w}};
}
__device__ __forceinline__ void st(float4* p, dc a) { *p = make_float4(a.re.hi, a.re.lo, a.im.hi, a.im.lo); }
__device__ __forceinline__ dc cmul(dc a, dc b) {
  return {add(mul(a.re, b.re), neg(mul(a.im, b.im))), add(mul(a.re, b.im), mul(a.im, b.re))};
}
__device__ __forceinline__ dc csub(dc a, dc b) { return {add(a.re, neg(b.re)), add(a.im, neg(b.im))}; }
__device__ __forceinline__ dc cscale(dc a, df s) { return {mul(a.re, s), mul(a.im, s)}; }
__device__ __forceinline__ dc conj(dc a) { return {a.re, neg(a.im)}; }

// 1 / x for x > 0: FP32 reciprocal refined by one Newton step in double-float
__device__ __forceinline__ df recip(df x) {
  const float r0 = 1.0f / x.hi;
  // e = 1 - x r0, r = r0 + r0 e
  const df xr = mul(x, df{r0, 0.f});
  const df e = add(df{1.0f, 0.f}, neg(xr));
  return add(df{r0, 0.f}, mul(df{r0, 0.f}, e));
}

}  // namespace dfa


__host__ __device__ inline size_t chol_df_smem(int nb) {
  return (size_t)nb * (nb + 1) / 2 * sizeof(float4) + (size_t)nb * (sizeof(double) + 3 * sizeof(float));
}

// the 1/sqrt of the FP64 kernels (FP32 seed, three Newton steps in FP64)
__device__ __forceinline__ double rsqrt_nr(double d) {
  double r = (double)rsqrtf((float)d);
  r = r * (1.5 - 0.5 * d * r * r);
  r = r * (1.5 - 0.5 * d * r * r);
  r = r * (1.5 - 0.5 * d * r * r);
  return r;
}

template <int NT>
__global__ void __launch_bounds__(NT, 1)
k_cholesky_inv_df(const double2* __restrict__ S, double2* __restrict__ Ri, int nb, int* __restrict__ flags,
                  double min_pivot) {
  using namespace dfa;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // FP64 work stays off the per-element paths (1/64 of the FP32 rate): the
  // pivot test compares FP32 values, pivots and their inverse square roots
  // are kept as double-float pairs, and one lane per row forms 1/sqrt(d_k)
  float4* U = reinterpret_cast<float4*>(smem_raw);                         // packed upper rows
  double* sdiag = reinterpret_cast<double*>(U + (size_t)nb * (nb + 1) / 2);  // S_kk
  float* thr = reinterpret_cast<float*>(sdiag + nb);                        // min_pivot S_kk
  df* dpiv = reinterpret_cast<df*>(thr + nb);                               // d_k, then 1/sqrt(d_k)
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarp = NT / 32;
  const size_t off = (size_t)blockIdx.x * nb * nb;
  auto idx = [nb](int i, int j) { return (size_t)i * (2 * nb - i + 1) / 2 + (j - i); };
  // upper triangle of the Hermitian part of S
  for (int i = warp; i < nb; i += nwarp)
    for (int j = i + lane; j < nb; j += 32) {
      const double2 a = S[off + (size_t)i * nb + j], b = S[off + (size_t)j * nb + i];
      const double re = 0.5 * (a.x + b.x), im = i == j ? 0.0 : 0.5 * (a.y - b.y);
      st(U + idx(i, j), dc{from_d(re), from_d(im)});
      if (i == j) { sdiag[i] = a.x; thr[i] = (float)(min_pivot * a.x); }
    }
  __syncthreads();
  // factorisation with unscaled pivot rows
  bool broke = false;
  for (int k = 0; k < nb; ++k) {
    df d = ld(U + idx(k, k)).re;
    if (!(d.hi > thr[k]) || !isfinite(d.hi)) { d = df{1.0f, 0.f}; broke = true; }
    const df invd = recip(d);
    for (int i = k + 1 + warp; i < nb; i += nwarp) {
      const dc a = cscale(conj(ld(U + idx(k, i))), invd);   // conj(U[k][i]) / d_k
      for (int j = i + lane; j < nb; j += 32) {
        float4* p = U + idx(i, j);
        st(p, csub(ld(p), cmul(a, ld(U + idx(k, j)))));
      }
    }
    if (tid == 0) dpiv[k] = d;
    __syncthreads();
  }
  if (broke && tid == 0) atomicOr(flags, 1);
  // row k scaled by 1/sqrt(d_k): R; sdiag keeps S_kk, dpiv becomes 1/sqrt(d_k)
  __syncthreads();
  for (int k = warp; k < nb; k += nwarp) {
    df s{0.f, 0.f}, r{0.f, 0.f};   // 1/sqrt(d_k), sqrt(d_k)
    if (lane == 0) {
      const double dk = to_d(dpiv[k]), rs = rsqrt_nr(dk);
      s = from_d(rs);
      r = from_d(dk * rs);
    }
    s.hi = __shfl_sync(0xffffffffu, s.hi, 0); s.lo = __shfl_sync(0xffffffffu, s.lo, 0);
    r.hi = __shfl_sync(0xffffffffu, r.hi, 0); r.lo = __shfl_sync(0xffffffffu, r.lo, 0);
    for (int j = k + lane; j < nb; j += 32) {
      float4* p = U + idx(k, j);
      if (j == k) st(p, dc{r, df{0.f, 0.f}});
      else st(p, cscale(ld(p), s));
    }
    __syncwarp();
    if (lane == 0) dpiv[k] = s;
  }
  __syncthreads();
  // inversion in place, bottom-up
  for (int k = nb - 1; k >= 0; --k) {
    const df dk = dpiv[k];   // 1 / R[k][k] = X[k][k]
    for (int i = warp; i < k; i += nwarp) {
      const dc r = ld(U + idx(i, k));   // R[i][k]
      __syncwarp();                     // every lane has R[i][k] before lane j = k overwrites it
      for (int j = k + lane; j < nb; j += 32) {
        float4* p = U + idx(i, j);
        if (j == k) {
          st(p, cscale(r, neg(dk)));
        } else {
          const dc xkj = cscale(ld(U + idx(k, j)), dk);   // X[k][j] = a_kj / R[k][k]
          st(p, csub(ld(p), cmul(r, xkj)));
        }
      }
    }
    __syncthreads();
  }
  // X[k][j] = a_kj / R[k][k] (j > k), X[k][k] = 1 / R[k][k]; lower part zero
  for (int i = warp; i < nb; i += nwarp) {
    const df di = dpiv[i];
    for (int j = lane; j < nb; j += 32) {
      double2 v = make_double2(0.0, 0.0);
      if (j == i) v = make_double2(to_d(di), 0.0);
      else if (j > i) {
        const dc x = cscale(ld(U + idx(i, j)), di);
        v = make_double2(to_d(x.re), to_d(x.im));
      }
      Ri[off + (size_t)i * nb + j] = v;
    }
  }
  // condition estimate off the pivot chain: S_kk / d_k = S_kk (1/sqrt(d_k))^2
  if (warp == 0) {
    double c = 0.0;
    for (int k = lane; k < nb; k += 32) {
      const double r = to_d(dpiv[k]);
      c = fmax(c, fabs(sdiag[k]) * r * r);
    }
    for (int o = 16; o > 0; o >>= 1) c = fmax(c, __shfl_xor_sync(0xffffffffu, c, o));
    if (lane == 0) {
      double est = broke ? __longlong_as_double(0x7ff0000000000000LL) : c;
      if (!(est >= 0.0)) est = __longlong_as_double(0x7ff0000000000000LL);
      atomicMax(reinterpret_cast<unsigned long long*>(flags + 2), (unsigned long long)__double_as_longlong(est));
    }
  }
}

// 1: launched; 0: the triangle does not fit in shared memory (use the FP64
// kernel); < 0: -status
int launch_cholesky_inv_df(const double2* S, double2* Ri, int nsk, int nb, int* flags, double min_pivot,
                           cudaStream_t st) {
  const size_t sm = chol_df_smem(nb);
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return 0;
  if (sm > (size_t)optin) return 0;
  // one warp per row of the update: 8 warps up to 64 bands, 32 above
  auto go = [&](auto kern, int nt) -> cudaError_t {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    kern<<<nsk, nt, sm, st>>>(S, Ri, nb, flags, min_pivot);
    return cudaSuccess;
  };
  cudaError_t e = nb <= 64 ? go(k_cholesky_inv_df<256>, 256) : go(k_cholesky_inv_df<1024>, 1024);
  if (e != cudaSuccess) return -cuda_fail(e, "cudaFuncSetAttribute(k_cholesky_inv_df)");
  count_launch();
  e = cudaGetLastError();
  if (e != cudaSuccess) return -cuda_fail(e, "k_cholesky_inv_df");
  return 1;
}

}  // namespace jrg
