// Orthonormalisation of the plane-wave parameters and its adjoint.
//
// C = W R^{-1} with R^H R = W^H W (Cholesky QR).  Per (spin, k) block:
//   gram:     S = X^H Y over the sphere (tiled, split over G, FP64 partials)
//   cholesky: R (upper, positive diagonal), R^{-1}, in FP64
//   rotate:   out = sum_t X_t M_t   (tall [G x B] times small [B x B])
// Adjoint (g_C = dE/dC^*):  A = C^H g_C, K = Hermitian completion of the
// strict upper triangle of A with Re(diag A) on the diagonal,
//   g_W = g_C R^{-H} - C (K R^{-H}),  dE/dw_re = 2 Re g_W, dE/dw_im = 2 Im g_W.
// The internal coefficient layout is band-major: [sk][band][G] complex.
#include <algorithm>
#include <type_traits>
#include "plan.h"

namespace jrg {

// (S,K,G,B) split real/imag (w_im may be NULL: zero) or interleaved complex
// (w_re holds the complex array, w_im NULL, CIN) -> [sk][B][G] complex
template <typename R, bool CIN>
__global__ void k_pack_params(const R* __restrict__ w_re, const R* __restrict__ w_im,
                              C_t<R>* __restrict__ out, int ng, int nb) {
  __shared__ R tre[32][33];
  __shared__ R tim[32][33];
  const int sk = blockIdx.z;
  const int g0 = blockIdx.x * 32, b0 = blockIdx.y * 32;
  const size_t base = (size_t)sk * ng * nb;
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int g = g0 + r, b = b0 + threadIdx.x;
    if (g < ng && b < nb) {
      const size_t o = base + (size_t)g * nb + b;
      if (CIN) {
        tre[r][threadIdx.x] = w_re[2 * o];
        tim[r][threadIdx.x] = w_re[2 * o + 1];
      } else {
        tre[r][threadIdx.x] = w_re[o];
        tim[r][threadIdx.x] = w_im ? w_im[o] : (R)0;
      }
    }
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int b = b0 + r, g = g0 + threadIdx.x;
    if (g < ng && b < nb) {
      C_t<R> v; v.x = tre[threadIdx.x][r]; v.y = tim[threadIdx.x][r];
      out[base + (size_t)b * ng + g] = v;
    }
  }
}

// [sk][B][G] complex -> (S,K,G,B) as split real/imag (times fac) or interleaved complex
template <typename R, bool SPLIT>
__global__ void k_unpack(const C_t<R>* __restrict__ in, R* __restrict__ o_re, R* __restrict__ o_im,
                         C_t<R>* __restrict__ o_c, int ng, int nb, R fac) {
  __shared__ C_t<R> t[32][33];
  const int sk = blockIdx.z;
  const int g0 = blockIdx.x * 32, b0 = blockIdx.y * 32;
  const size_t base = (size_t)sk * ng * nb;
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int b = b0 + r, g = g0 + threadIdx.x;
    if (g < ng && b < nb) t[r][threadIdx.x] = in[base + (size_t)b * ng + g];
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int g = g0 + r, b = b0 + threadIdx.x;
    if (g < ng && b < nb) {
      const C_t<R> v = t[threadIdx.x][r];
      const size_t o = base + (size_t)g * nb + b;
      if (SPLIT) { o_re[o] = fac * v.x; o_im[o] = fac * v.y; }
      else o_c[o] = v;
    }
  }
}

// Input layouts of the tall [G x B] operands:
//   LAYOUT_SPLIT: two real arrays (re, im) indexed [sk][g][b] (the parameter layout)
//   LAYOUT_BAND:  one complex array indexed [sk][b][g] (internal coefficient layout)
enum Layout { LAYOUT_SPLIT = 0, LAYOUT_BAND = 1 };

template <typename R, int LAYOUT>
__device__ __forceinline__ C_t<R> load_tall(const void* __restrict__ p0, const void* __restrict__ p1,
                                            size_t sk, int i, int g, int ng, int nb) {
  if constexpr (LAYOUT == LAYOUT_SPLIT) {
    const size_t o = (sk * ng + g) * nb + i;
    C_t<R> v;
    v.x = reinterpret_cast<const R*>(p0)[o];
    v.y = reinterpret_cast<const R*>(p1)[o];
    return v;
  } else {
    return reinterpret_cast<const C_t<R>*>(p0)[(sk * nb + i) * ng + g];
  }
}

// Partial Gram S[i][j] = sum_g conj(X[i][g]) Y[j][g] over one G split for a
// 32x32 output tile; 16x16 threads, each a 2x2 block (rows ty, ty+16; columns
// tx, tx+16).  Products and chunk-long runs in precision R, runs summed in FP64.
constexpr int kGramTile = 32;
template <typename R> struct GramChunk { static constexpr int value = 64; };
template <> struct GramChunk<double> { static constexpr int value = 32; };  // 48 KB static smem

template <typename R, int LX, int LY>
__global__ void __launch_bounds__(256) k_gram_partial(const void* __restrict__ X0,
                                                      const void* __restrict__ X1,
                                                      const void* __restrict__ Y0,
                                                      const void* __restrict__ Y1,
                                                      double2* __restrict__ part, int ng, int nb,
                                                      int split_len) {
  using C = C_t<R>;
  constexpr int CH = GramChunk<R>::value;
  __shared__ C xs[kGramTile][CH + 1];
  __shared__ C ys[kGramTile][CH + 1];
  const int split = blockIdx.x;
  const int ntile = (nb + kGramTile - 1) / kGramTile;
  const int ti = blockIdx.y / ntile, tj = blockIdx.y % ntile;
  const size_t sk = blockIdx.z;
  const int nsplit = gridDim.x;
  const int g_begin = split * split_len;
  const int g_end = min(ng, g_begin + split_len);
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  double2 acc[2][2];
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int b = 0; b < 2; ++b) acc[a][b] = make_double2(0.0, 0.0);
  const C z0 = czero<C>();
  for (int g0 = g_begin; g0 < g_end; g0 += CH) {
    for (int idx = threadIdx.x; idx < kGramTile * CH; idx += blockDim.x) {
      int r, c;
      if (LX == LAYOUT_SPLIT) { r = idx % kGramTile; c = idx / kGramTile; }
      else { c = idx % CH; r = idx / CH; }
      const int g = g0 + c;
      const int bi = ti * kGramTile + r, bj = tj * kGramTile + r;
      xs[r][c] = (g < g_end && bi < nb) ? load_tall<R, LX>(X0, X1, sk, bi, g, ng, nb) : z0;
      ys[r][c] = (g < g_end && bj < nb) ? load_tall<R, LY>(Y0, Y1, sk, bj, g, ng, nb) : z0;
    }
    __syncthreads();
    C s[2][2];
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
      for (int b = 0; b < 2; ++b) s[a][b] = z0;
#pragma unroll 8
    for (int c = 0; c < CH; ++c) {
      const C x0 = xs[ty][c], x1 = xs[ty + 16][c];
      const C y0 = ys[tx][c], y1 = ys[tx + 16][c];
      // conj(x) * y
      s[0][0].x += x0.x * y0.x + x0.y * y0.y; s[0][0].y += x0.x * y0.y - x0.y * y0.x;
      s[0][1].x += x0.x * y1.x + x0.y * y1.y; s[0][1].y += x0.x * y1.y - x0.y * y1.x;
      s[1][0].x += x1.x * y0.x + x1.y * y0.y; s[1][0].y += x1.x * y0.y - x1.y * y0.x;
      s[1][1].x += x1.x * y1.x + x1.y * y1.y; s[1][1].y += x1.x * y1.y - x1.y * y1.x;
    }
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
      for (int b = 0; b < 2; ++b) { acc[a][b].x += (double)s[a][b].x; acc[a][b].y += (double)s[a][b].y; }
    __syncthreads();
  }
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int b = 0; b < 2; ++b) {
      const int i = ti * kGramTile + ty + 16 * a, j = tj * kGramTile + tx + 16 * b;
      if (i < nb && j < nb) part[((sk * nsplit + split) * nb + i) * nb + j] = acc[a][b];
    }
}

// num_band <= 32: warp-tiled partial Gram.  A block walks its G range in
// chunks of 64 G vectors staged in shared memory as [g][band] (cp.async,
// double-buffered); each of the 8 warps takes 8 G vectors of a chunk and
// every lane accumulates rows li + 4a (a < NBP/4) by columns lj + 8b
// (b < NBP/8) of its warp's partial, lane = 8 li + lj: per G vector NBP/4 +
// NBP/8 shared loads (broadcast within lane groups, conflict-free) feed
// NBP^2/32 complex multiply-adds.  The warps' partials (FP32 sums of at most
// split_len / 8 terms on the FP32 path) are reduced in FP64.
constexpr int kGwCG = 64;   // G vectors per chunk

template <typename R>
size_t gram_w_smem(int NBP, bool same = false) {
  const size_t stage = (same ? 1 : 2) * 2 * (size_t)kGwCG * (NBP + 1) * sizeof(C_t<R>);
  const size_t red = 8 * (size_t)NBP * NBP * sizeof(C_t<R>);
  return stage > red ? stage : red;
}

// SAME: Y is X (W^H W): the chunk is staged once.
template <typename R, int LX, int LY, int NBP, bool SAME = false>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? 2 : 1)
k_gram_w(const void* __restrict__ X0, const void* __restrict__ X1, const void* __restrict__ Y0,
         const void* __restrict__ Y1, double2* __restrict__ part, int ng, int nb, int split_len) {
  using C = C_t<R>;
  constexpr int CG = kGwCG, LD = NBP + 1, TI = NBP / 4, TJ = NBP / 8;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* xs = reinterpret_cast<C*>(smem_raw);   // [2][CG][LD]
  C* ys = SAME ? xs : xs + 2 * CG * LD;     // [2][CG][LD]
  const int split = blockIdx.x;
  const size_t sk = blockIdx.z;
  const int nsplit = gridDim.x;
  const int g_begin = split * split_len;
  const int g_end = min(ng, g_begin + split_len);
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const int li = lane >> 3, lj = lane & 7;
  // zero the padding bands once (rows nb..NBP-1 are never staged)
  for (int e = t; e < 2 * CG * LD; e += 256) {
    if (e % LD >= nb) { xs[e] = czero<C>(); ys[e] = czero<C>(); }
  }
  // parameter layout: the chunk's CG x nb values are contiguous in global
  // memory (element e of the chunk at offset e), and the shared-memory slot
  // of element e (column e / nb, band e % nb) is the same in every chunk: it
  // is computed once per thread instead of per copy
  constexpr int EPT = (CG * NBP + 255) / 256;   // staged elements per thread
  int soff[EPT];
  if constexpr (LX == LAYOUT_SPLIT) {
#pragma unroll
    for (int k = 0; k < EPT; ++k) {
      const int e = t + 256 * k;
      soff[k] = e < CG * nb ? (e / nb) * LD + e % nb : -1;
    }
  }
  auto stage = [&](int buf, int g0) {
    C* xd = xs + buf * CG * LD;
    C* yd = ys + buf * CG * LD;
    if constexpr (LX == LAYOUT_SPLIT && LY == LAYOUT_SPLIT) {
      const size_t base = (sk * ng + g0) * (size_t)nb;
      const int lim = (g_end - g0) * nb;   // elements of the chunk inside the split
#pragma unroll
      for (int k = 0; k < EPT; ++k) {
        if (soff[k] < 0) continue;
        const int e = t + 256 * k;
        C* dx = xd + soff[k];
        C* dy = yd + soff[k];
        if (e >= lim) {
          *dx = czero<C>();
          if (!SAME) *dy = czero<C>();
        } else {
          cp_async<sizeof(R)>(&dx->x, reinterpret_cast<const R*>(X0) + base + e);
          cp_async<sizeof(R)>(&dx->y, reinterpret_cast<const R*>(X1) + base + e);
          if (!SAME) {
            cp_async<sizeof(R)>(&dy->x, reinterpret_cast<const R*>(Y0) + base + e);
            cp_async<sizeof(R)>(&dy->y, reinterpret_cast<const R*>(Y1) + base + e);
          }
        }
      }
      cp_async_commit();
      return;
    }
    for (int e = t; e < CG * nb; e += 256) {
      int r, c;   // band, chunk column
      if (LX == LAYOUT_SPLIT) { r = e % nb; c = e / nb; }
      else { c = e % CG; r = e / CG; }
      const int g = g0 + c;
      C* dx = xd + c * LD + r;
      C* dy = yd + c * LD + r;
      if (g >= g_end) {
        *dx = czero<C>();
        if (!SAME) *dy = czero<C>();
      } else if (LX == LAYOUT_SPLIT) {
        const size_t o = (sk * ng + g) * nb + r;
        cp_async<sizeof(R)>(&dx->x, reinterpret_cast<const R*>(X0) + o);
        cp_async<sizeof(R)>(&dx->y, reinterpret_cast<const R*>(X1) + o);
        if (!SAME) {
          cp_async<sizeof(R)>(&dy->x, reinterpret_cast<const R*>(Y0) + o);
          cp_async<sizeof(R)>(&dy->y, reinterpret_cast<const R*>(Y1) + o);
        }
      } else {
        const size_t o = (sk * nb + r) * ng + g;
        cp_async<sizeof(C)>(dx, reinterpret_cast<const C*>(X0) + o);
        if (!SAME) cp_async<sizeof(C)>(dy, reinterpret_cast<const C*>(Y0) + o);
      }
    }
    cp_async_commit();
  };
  C acc[TI][TJ];
#pragma unroll
  for (int a = 0; a < TI; ++a)
#pragma unroll
    for (int b = 0; b < TJ; ++b) acc[a][b] = czero<C>();
  const int nchunk = (g_end - g_begin + CG - 1) / CG;
  __syncthreads();
  if (nchunk > 0) stage(0, g_begin);
  for (int c = 0; c < nchunk; ++c) {
    if (c + 1 < nchunk) {
      stage((c + 1) & 1, g_begin + (c + 1) * CG);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    const C* xb = xs + (c & 1) * CG * LD + w * (CG / 8) * LD;
    const C* yb = ys + (c & 1) * CG * LD + w * (CG / 8) * LD;
    constexpr int QU = (NBP >= 32 && sizeof(R) == 4) ? 1 : 2;
#pragma unroll QU
    for (int q = 0; q < CG / 8; ++q) {
      C x[TI], y[TJ];
#pragma unroll
      for (int a = 0; a < TI; ++a) x[a] = xb[q * LD + li + 4 * a];
#pragma unroll
      for (int b = 0; b < TJ; ++b) y[b] = yb[q * LD + lj + 8 * b];
#pragma unroll
      for (int a = 0; a < TI; ++a)
#pragma unroll
        for (int b = 0; b < TJ; ++b) {   // conj(x) * y
          acc[a][b].x = fma(x[a].x, y[b].x, fma(x[a].y, y[b].y, acc[a][b].x));
          acc[a][b].y = fma(x[a].x, y[b].y, fma(-x[a].y, y[b].x, acc[a][b].y));
        }
    }
    __syncthreads();
  }
  // the eight warps' FP32 sums are added in FP32 (pairwise, a few roundings
  // against the hundreds of each warp's own runs) and only the block total
  // goes to FP64: FP64 arithmetic runs at 1/64 of the FP32 rate here
  C* red = reinterpret_cast<C*>(smem_raw);   // [8][NBP][NBP]
#pragma unroll
  for (int a = 0; a < TI; ++a)
#pragma unroll
    for (int b = 0; b < TJ; ++b) red[((size_t)w * NBP + li + 4 * a) * NBP + lj + 8 * b] = acc[a][b];
  __syncthreads();
  const int nn = nb * nb;
  for (int e = t; e < nn; e += 256) {
    const int i = e / nb, j = e - i * nb;
    C u[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) u[q] = red[((size_t)q * NBP + i) * NBP + j];
#pragma unroll
    for (int h = 4; h > 0; h >>= 1)
#pragma unroll
      for (int q = 0; q < h; ++q) { u[q].x += u[q + h].x; u[q].y += u[q + h].y; }
    part[(sk * nsplit + split) * nn + e] = make_double2((double)u[0].x, (double)u[0].y);
  }
}

__global__ void k_gram_reduce(const double2* __restrict__ part, double2* __restrict__ out,
                              int nsplit, int nb, int nsk) {
  const size_t n = (size_t)nsk * nb * nb;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x) {
    const size_t sk = e / ((size_t)nb * nb), ij = e % ((size_t)nb * nb);
    double2 s = make_double2(0.0, 0.0);
    for (int p = 0; p < nsplit; ++p) {
      const double2 v = part[((size_t)sk * nsplit + p) * nb * nb + ij];
      s.x += v.x; s.y += v.y;
    }
    out[e] = s;
  }
}

// 1/sqrt(d) for d > 0 without the FP64 square-root/division sequences:
// FP32 seed refined by three Newton steps in FP64 (multiplies and adds only).
__device__ __forceinline__ double rsqrt_fp64(double d) {
  double r = (double)rsqrtf((float)d);
  r = r * (1.5 - 0.5 * d * r * r);
  r = r * (1.5 - 0.5 * d * r * r);
  r = r * (1.5 - 0.5 * d * r * r);
  return r;
}

// Condition estimate of a Gram matrix from its Cholesky pivots: max over k of
// S_kk / d_k (d_k the pivot before the square root; 1 for orthogonal
// columns, ~cond(S) as the columns approach linear dependence; +inf for a
// non-positive or non-finite pivot).  The largest over all (s,k) blocks of a
// call is kept in flags[2..3] as the bit pattern of a non-negative double,
// which orders like the value, so an integer atomicMax of the zeroed word
// gives the maximum.
__device__ __forceinline__ void note_condition(int* flags, double est) {
  if (!(est >= 0.0)) est = __longlong_as_double(0x7ff0000000000000LL);   // NaN -> +inf
  atomicMax(reinterpret_cast<unsigned long long*>(flags + 2), (unsigned long long)__double_as_longlong(est));
}
// A pivot d_k <= min_pivot * S_kk is a breakdown (flags bit 0): below the
// rounding of the Gram (relative ~1e-8 with FP32 products, ~1e-16 in FP64)
// it is noise, and R^-1 would amplify that noise into the coefficients.
__device__ __forceinline__ double pivot_ratio(double s_kk, double d) {
  return (d > 0.0 && isfinite(d)) ? fabs(s_kk) / d : __longlong_as_double(0x7ff0000000000000LL);
}

// nb <= 32: one CTA of nb*nb threads per (s,k), thread (i, j) owns element
// (i, j).  Right-looking Cholesky and a right-looking inverse, so each pivot
// step is two or three dependent FP64 operations per thread (FP64 latency is
// long on this part; the work is spread instead of chained).
__global__ void __launch_bounds__(1024) k_cholesky_inv_elem(const double2* __restrict__ S,
                                                            double2* __restrict__ Rm,
                                                            double2* __restrict__ Ri, int nb,
                                                            int* __restrict__ flags, double min_pivot) {
  __shared__ double2 r[32][33];
  __shared__ double2 x[32][33];
  __shared__ double dinv[32];
  __shared__ double sdiag[32];
  __shared__ double dpiv[32];   // the pivots before the square root
  const int sk = blockIdx.x;
  const int i = threadIdx.x / nb, j = threadIdx.x % nb;
  const bool live = threadIdx.x < nb * nb;
  const size_t off = (size_t)sk * nb * nb;
  if (live) {
    const double2 a = S[off + i * nb + j], b = S[off + j * nb + i];
    r[i][j] = (j >= i) ? make_double2(0.5 * (a.x + b.x), 0.5 * (a.y - b.y)) : make_double2(0.0, 0.0);
    x[i][j] = make_double2(i == j ? 1.0 : 0.0, 0.0);
    if (i == j) sdiag[i] = a.x;
  }
  __syncthreads();
  for (int k = 0; k < nb; ++k) {
    if (live && i == k && j == k) {
      double d = r[k][k].x;
      dpiv[k] = d;
      if (!(d > min_pivot * sdiag[k]) || !isfinite(d)) { atomicOr(flags, 1); d = 1.0; }
      const double rs = rsqrt_fp64(d);
      r[k][k] = make_double2(d * rs, 0.0);
      dinv[k] = rs;
    }
    __syncthreads();
    if (live && i == k && j > k) {
      const double rs = dinv[k];
      const double2 v = r[k][j];
      r[k][j] = make_double2(v.x * rs, v.y * rs);
    }
    __syncthreads();
    if (live && i > k && j >= i) {
      const double2 a = r[k][i], b = r[k][j];
      double2 v = r[i][j];
      v.x -= a.x * b.x + a.y * b.y;
      v.y -= a.x * b.y - a.y * b.x;
      r[i][j] = v;
    }
    __syncthreads();
  }
  // X = R^{-1}: rows finalised bottom-up, each subtracted from the rows above
  for (int k = nb - 1; k >= 0; --k) {
    if (live && i == k && j >= k) {
      const double2 v = x[k][j];
      x[k][j] = make_double2(v.x * dinv[k], v.y * dinv[k]);
    }
    __syncthreads();
    if (live && i < k && j >= k) {
      const double2 a = r[i][k], b = x[k][j];
      double2 v = x[i][j];
      v.x -= a.x * b.x - a.y * b.y;
      v.y -= a.x * b.y + a.y * b.x;
      x[i][j] = v;
    }
    __syncthreads();
  }
  if (live) {
    Rm[off + i * nb + j] = r[i][j];
    Ri[off + i * nb + j] = x[i][j];
  }
  // condition estimate off the pivot chain: one ratio per lane of warp 0
  if (threadIdx.x < 32) {
    double c = threadIdx.x < nb ? pivot_ratio(sdiag[threadIdx.x], dpiv[threadIdx.x]) : 0.0;
    for (int o = 16; o > 0; o >>= 1) c = fmax(c, __shfl_xor_sync(0xffffffffu, c, o));
    if (threadIdx.x == 0) note_condition(flags, c);
  }
}

// nb > 32: the same element-parallel algorithm with the matrices in the
// output buffers (global memory, L1/L2 resident) and 1024 threads looping
// over the elements of each phase.
__global__ void __launch_bounds__(1024) k_cholesky_inv_big(const double2* __restrict__ S,
                                                           double2* __restrict__ Rm,
                                                           double2* __restrict__ Ri, double* dinv_g,
                                                           int nb, int* __restrict__ flags,
                                                           double min_pivot) {
  const int sk = blockIdx.x;
  const size_t off = (size_t)sk * nb * nb;
  double2* r = Rm + off;
  double2* x = Ri + off;
  double* dinv = dinv_g + (size_t)sk * nb;
  const int n2 = nb * nb;
  for (int e = threadIdx.x; e < n2; e += blockDim.x) {
    const int i = e / nb, j = e % nb;
    const double2 a = S[off + e], b = S[off + (size_t)j * nb + i];
    r[e] = (j >= i) ? make_double2(0.5 * (a.x + b.x), 0.5 * (a.y - b.y)) : make_double2(0.0, 0.0);
    x[e] = make_double2(i == j ? 1.0 : 0.0, 0.0);
  }
  __syncthreads();
  bool broke = false;   // thread 0 only
  for (int k = 0; k < nb; ++k) {
    if (threadIdx.x == 0) {
      double d = r[(size_t)k * nb + k].x;
      const double skk = S[off + (size_t)k * nb + k].x;
      if (!(d > min_pivot * skk) || !isfinite(d)) { atomicOr(flags, 1); d = 1.0; broke = true; }
      const double rs = rsqrt_fp64(d);
      r[(size_t)k * nb + k] = make_double2(d * rs, 0.0);
      dinv[k] = rs;
    }
    __syncthreads();
    const double rs = dinv[k];
    for (int j = k + 1 + threadIdx.x; j < nb; j += blockDim.x) {
      const double2 v = r[(size_t)k * nb + j];
      r[(size_t)k * nb + j] = make_double2(v.x * rs, v.y * rs);
    }
    __syncthreads();
    const int m = nb - k - 1;
    for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
      const int i = k + 1 + e / m, j = k + 1 + e % m;
      if (j >= i) {
        const double2 a = r[(size_t)k * nb + i], b = r[(size_t)k * nb + j];
        double2 v = r[(size_t)i * nb + j];
        v.x -= a.x * b.x + a.y * b.y;
        v.y -= a.x * b.y - a.y * b.x;
        r[(size_t)i * nb + j] = v;
      }
    }
    __syncthreads();
  }
  for (int k = nb - 1; k >= 0; --k) {
    const double dk = dinv[k];
    for (int j = k + threadIdx.x; j < nb; j += blockDim.x) {
      const double2 v = x[(size_t)k * nb + j];
      x[(size_t)k * nb + j] = make_double2(v.x * dk, v.y * dk);
    }
    __syncthreads();
    const int w = nb - k;
    for (int e = threadIdx.x; e < k * w; e += blockDim.x) {
      const int i = e / w, j = k + e % w;
      const double2 a = r[(size_t)i * nb + k], b = x[(size_t)k * nb + j];
      double2 v = x[(size_t)i * nb + j];
      v.x -= a.x * b.x - a.y * b.y;
      v.y -= a.x * b.y + a.y * b.x;
      x[(size_t)i * nb + j] = v;
    }
    __syncthreads();
  }
  // condition estimate off the pivot chain: S_kk / d_k = S_kk dinv_k^2 (warp 0)
  if (threadIdx.x < 32) {
    double c = 0.0;
    for (int k = threadIdx.x; k < nb; k += 32)
      c = fmax(c, fabs(S[off + (size_t)k * nb + k].x) * dinv[k] * dinv[k]);
    for (int o = 16; o > 0; o >>= 1) c = fmax(c, __shfl_xor_sync(0xffffffffu, c, o));
    if (threadIdx.x == 0) note_condition(flags, broke ? __longlong_as_double(0x7ff0000000000000LL) : c);
  }
}

// Adjoint small matrices per (s,k):
//   Rh = R^{-H};  K from A;  M2 = K R^{-H}  (stored negated: -M2)
// With occupations f given, A holds C^H (H C) (unweighted): the band energies
// Re A_bb are written to eps and the occupations are folded in as
// A diag(f) (for K) and diag(f) R^{-H} (for Rh).
// Grid (nsk, parts): CTA (sk, p) takes elements p*blockDim .. of the nb x nb
// matrices, so that the FP64 sums of -M2 (1/64 of the FP32 rate) spread over
// all SMs instead of one CTA per (s,k).
constexpr int kAdjSmallThreads = 64;
__global__ void __launch_bounds__(kAdjSmallThreads) k_adjoint_small(const double2* __restrict__ A,
                                                       const double2* __restrict__ Ri,
                                                       double2* __restrict__ Rh,
                                                       double2* __restrict__ negM2, int nb,
                                                       const double* __restrict__ f,
                                                       double* __restrict__ eps, bool with_m2) {
  const int sk = blockIdx.x;
  const size_t off = (size_t)sk * nb * nb;
  const double2* a = A + off;
  const double2* ri = Ri + off;
  const double* fb = f ? f + (size_t)sk * nb : nullptr;
  auto fw = [&](int j) { return fb ? fb[j] : 1.0; };
  const int e0 = blockIdx.y * blockDim.x + threadIdx.x, es = gridDim.y * blockDim.x;
  if (eps)
    for (int b = e0; b < nb; b += es) eps[(size_t)sk * nb + b] = a[b * nb + b].x;
  for (int e = e0; e < nb * nb; e += es) {
    const int i = e / nb, j = e % nb;
    const double2 v = ri[j * nb + i];
    const double s = fw(i);
    Rh[off + e] = make_double2(s * v.x, -s * v.y);
  }
  if (!with_m2) return;   // formed by k_adjoint_m2_tiled
  for (int e = e0; e < nb * nb; e += es) {
    const int i = e / nb, j = e % nb;
    // (K R^{-H})[i][j] = sum_l K[i][l] conj(Ri[j][l]),  Ri upper => l >= j
    double sx = 0.0, sy = 0.0;
    for (int l = j; l < nb; ++l) {
      double2 kil;
      if (l > i) { const double2 t = a[i * nb + l]; const double s = fw(l); kil = make_double2(s * t.x, s * t.y); }
      else if (l < i) { const double2 t = a[l * nb + i]; const double s = fw(i); kil = make_double2(s * t.x, -s * t.y); }
      else kil = make_double2(fw(i) * a[i * nb + i].x, 0.0);
      const double2 r = ri[j * nb + l];   // conj later
      sx += kil.x * r.x + kil.y * r.y;
      sy += kil.y * r.x - kil.x * r.y;
    }
    negM2[off + e] = make_double2(-sx, -sy);
  }
}

// -M2 = -K R^{-H} for larger band counts: a 32 x 32 output tile per CTA
// (256 threads, four elements each), the contraction over l in 32-wide
// tiles of K (the Hermitian completion of A's upper triangle with real
// diagonal, columns weighted by f) and of conj(Ri)^T staged in shared
// memory.  Ri is upper triangular (zero below the diagonal).
__global__ void __launch_bounds__(256) k_adjoint_m2_tiled(const double2* __restrict__ A,
                                                          const double2* __restrict__ Ri,
                                                          double2* __restrict__ negM2, int nb,
                                                          const double* __restrict__ f) {
  __shared__ double2 ks[32][33];   // K[i0 + r][l0 + c]
  __shared__ double2 rs[32][33];   // conj(Ri[j0 + c][l0 + r]) = R^{-H}[l0 + r][j0 + c]
  const size_t off = (size_t)blockIdx.z * nb * nb;
  const double2* a = A + off;
  const double2* ri = Ri + off;
  const double* fb = f ? f + (size_t)blockIdx.z * nb : nullptr;
  const int i0 = blockIdx.y * 32, j0 = blockIdx.x * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;   // ty 0..7
  double2 acc[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) acc[q] = make_double2(0.0, 0.0);
  const int lstart = (j0 / 32) * 32;   // R^{-H}[l][j] = 0 for l < j: tiles below j0 vanish
  for (int l0 = lstart; l0 < nb; l0 += 32) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int r = ty + 8 * q;
      // K[i][l], i = i0 + r, l = l0 + tx
      const int i = i0 + r, l = l0 + tx;
      double2 kv = make_double2(0.0, 0.0);
      if (i < nb && l < nb) {
        const double wl = fb ? fb[l] : 1.0, wi = fb ? fb[i] : 1.0;
        if (l > i) { const double2 t = a[(size_t)i * nb + l]; kv = make_double2(wl * t.x, wl * t.y); }
        else if (l < i) { const double2 t = a[(size_t)l * nb + i]; kv = make_double2(wi * t.x, -wi * t.y); }
        else kv = make_double2(wi * a[(size_t)i * nb + i].x, 0.0);
      }
      ks[r][tx] = kv;
      // R^{-H}[l][j] with l = l0 + r, j = j0 + tx
      const int lr = l0 + r, j = j0 + tx;
      double2 rv = make_double2(0.0, 0.0);
      if (lr < nb && j < nb) { const double2 t = ri[(size_t)j * nb + lr]; rv = make_double2(t.x, -t.y); }
      rs[r][tx] = rv;
    }
    __syncthreads();
#pragma unroll 8
    for (int c = 0; c < 32; ++c) {
      const double2 r = rs[c][tx];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const double2 k = ks[ty + 8 * q][c];
        acc[q].x = fma(k.x, r.x, fma(-k.y, r.y, acc[q].x));
        acc[q].y = fma(k.x, r.y, fma(k.y, r.x, acc[q].y));
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int i = i0 + ty + 8 * q, j = j0 + tx;
    if (i < nb && j < nb) negM2[off + (size_t)i * nb + j] = make_double2(-acc[q].x, -acc[q].y);
  }
}

// out = sum_t X_t M_t with X_t [G x B] tall (layout LX0 / LX1) and M_t
// [B x B] FP64; output band-major complex, (S,K,G,B) complex, or (S,K,G,B)
// split real/imag times fac.  Thread per g, J-wide column tile; the M tile is
// staged in shared memory in precision R.
enum RotOut { ROT_BANDMAJOR = 0, ROT_GMAJOR_C = 1, ROT_GMAJOR_SPLIT = 2, ROT_ADAM = 3 };

template <typename R, int OUT, int J, int LX0, int LX1>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? 2 : 1) k_rotate(const void* __restrict__ X0a, const void* __restrict__ X0b,
                                                const double2* __restrict__ M0,
                                                const void* __restrict__ X1a, const void* __restrict__ X1b,
                                                const double2* __restrict__ M1, void* out0,
                                                void* out1, int ng, int nb, R fac) {
  using C = C_t<R>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* ms = reinterpret_cast<C*>(smem_raw);   // [nterms][nb][J]
  const size_t sk = blockIdx.z;
  const int j0 = blockIdx.y * J;
  const int nj = min(J, nb - j0);
  const int nterms = X1a ? 2 : 1;
  const size_t moff = sk * nb * nb;
  for (int e = threadIdx.x; e < nterms * nb * J; e += blockDim.x) {
    const int t = e / (nb * J), rem = e % (nb * J);
    const int i = rem / J, jj = rem % J;
    const double2* M = t ? M1 : M0;
    double2 v = (jj < nj) ? M[moff + (size_t)i * nb + j0 + jj] : make_double2(0.0, 0.0);
    ms[e] = cmk<C>(v.x, v.y);
  }
  __syncthreads();
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ng) return;
  C acc[J];
#pragma unroll
  for (int jj = 0; jj < J; ++jj) acc[jj] = czero<C>();
  // rows k < nb come from X0, nb <= k < 2 nb from X1; the loads of the next
  // P rows are issued before the current P rows are consumed
  const int K = nterms * nb;
  auto ld = [&](int k) -> C {
    if (k >= K) return czero<C>();
    return k < nb ? load_tall<R, LX0>(X0a, X0b, sk, k, g, ng, nb)
                  : load_tall<R, LX1>(X1a, X1b, sk, k - nb, g, ng, nb);
  };
  constexpr int P = sizeof(R) == 4 ? 8 : 4;
  C cur[P], nxt[P];
#pragma unroll
  for (int q = 0; q < P; ++q) cur[q] = ld(q);
  for (int k0 = 0; k0 < K; k0 += P) {
#pragma unroll
    for (int q = 0; q < P; ++q) nxt[q] = ld(k0 + P + q);
#pragma unroll
    for (int q = 0; q < P; ++q) {
      if (k0 + q < K) {
        const C x = cur[q];
        const C* mt = ms + (size_t)(k0 + q) * J;
#pragma unroll
        for (int jj = 0; jj < J; ++jj) {
          const C m = mt[jj];
          acc[jj].x = fma(x.x, m.x, fma(-x.y, m.y, acc[jj].x));
          acc[jj].y = fma(x.x, m.y, fma(x.y, m.x, acc[jj].y));
        }
      }
    }
#pragma unroll
    for (int q = 0; q < P; ++q) cur[q] = nxt[q];
  }
  const size_t base = sk * nb * ng;
  if (OUT == ROT_BANDMAJOR) {
    C* o = reinterpret_cast<C*>(out0) + base;
#pragma unroll
    for (int jj = 0; jj < J; ++jj)
      if (jj < nj) o[(size_t)(j0 + jj) * ng + g] = acc[jj];
  } else if (OUT == ROT_GMAJOR_C) {
    C* o = reinterpret_cast<C*>(out0) + base + (size_t)g * nb + j0;
#pragma unroll
    for (int jj = 0; jj < J; ++jj)
      if (jj < nj) o[jj] = acc[jj];
  } else {
    R* ore = reinterpret_cast<R*>(out0) + base + (size_t)g * nb + j0;
    R* oim = reinterpret_cast<R*>(out1) + base + (size_t)g * nb + j0;
#pragma unroll
    for (int jj = 0; jj < J; ++jj)
      if (jj < nj) { ore[jj] = fac * acc[jj].x; oim[jj] = fac * acc[jj].y; }
  }
}

// ------------------------------------------------------------------------
// Register-blocked rotation for num_band <= 32 (BANDMAJOR and GMAJOR_SPLIT
// outputs).  A block owns 256 G vectors of one (s, k): the stacked rows of X
// (X0 then X1, K = nterms * nb rows) stream through shared memory in chunks of
// 8 rows with cp.async double buffering, the stacked M (K x NBP, NBP = nb
// rounded up to 8) sits in shared memory, and each thread accumulates a
// 4 (G) x NBP/4 (band) block: per row, two 128-bit x loads and NBP/8 128-bit
// broadcast M loads feed 4 * NBP/4 complex multiply-adds.  G-major outputs
// are transposed through shared memory and written as coalesced runs.
constexpr int kRbKC = 8;     // rows per chunk
constexpr int kRbGT = 256;   // G vectors per block

template <typename R>
size_t rotate_rb_smem(int K, int NBP, bool two_tiles = false) {
  const size_t KP = (size_t)(K + kRbKC - 1) / kRbKC * kRbKC;
  const size_t ms = KP * NBP * sizeof(C_t<R>);
  const size_t xs = 2 * (size_t)kRbKC * kRbGT * sizeof(C_t<R>);
  const size_t tile = (two_tiles ? 2 : 1) * (size_t)kRbGT * (NBP + 1) * sizeof(R);
  return ms + (xs > tile ? xs : tile);
}

template <typename R, int LX0, int OUT, int NBP>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? 2 : 1)
k_rotate_rb(const void* __restrict__ X0a, const void* __restrict__ X0b, const double2* __restrict__ M0,
            const void* __restrict__ X1, const double2* __restrict__ M1, void* out0, void* out1,
            int ng, int nb, R fac, AdamArgs adam, const double* __restrict__ tk, int nk,
            void* __restrict__ kin_part, int sk0) {
  using C = C_t<R>;
  constexpr int KC = kRbKC, GT = kRbGT, TG = 4, TJ = NBP / 4;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nterms = X1 ? 2 : 1;
  const int K = nterms * nb;
  const int KP = (K + KC - 1) / KC * KC;
  C* ms = reinterpret_cast<C*>(smem_raw);        // [KP][NBP]
  C* xs = ms + (size_t)KP * NBP;                  // [2][KC][GT], then the output tile
  const size_t sk = blockIdx.y;
  const int g0 = blockIdx.x * GT;
  const int t = threadIdx.x;
  const size_t moff = sk * nb * nb;
  for (int e = t; e < KP * NBP; e += 256) {
    const int k = e / NBP, j = e % NBP;
    double2 v = make_double2(0.0, 0.0);
    if (k < K && j < nb) v = (k < nb ? M0 : M1)[moff + (size_t)(k < nb ? k : k - nb) * nb + j];
    ms[e] = cmk<C>(v.x, v.y);
  }
  if constexpr (OUT == ROT_ADAM) {
    // pull the block's parameter / moment / scale rows towards L2 while the
    // contraction runs (every line address lies inside the buffers: rows
    // start at or after a 128-byte boundary that is not before the buffer)
    const size_t base = (sk * ng + g0) * nb;
    const size_t len = (size_t)min(GT, ng - g0) * nb;
    const void* rows[8] = {adam.p[0], adam.p[1], adam.m[0], adam.m[1],
                           adam.v[0], adam.v[1], adam.scale[0], adam.scale[1]};
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      if (!rows[q]) continue;
      const size_t esz = q < 6 ? sizeof(R) : sizeof(float);
      const uintptr_t lo = (uintptr_t)rows[q] + base * esz, hi = lo + len * esz;
      for (uintptr_t l = (lo & ~(uintptr_t)127) + (uintptr_t)t * 128; l < hi; l += 256 * 128)
        asm volatile("prefetch.global.L2 [%0];" ::"l"(l));
    }
  }
  const int gs = g0 + t;            // staging column of this thread
  const bool gv = gs < ng;
  auto stage = [&](int buf, int k0) {
    C* dst = xs + (size_t)buf * KC * GT + t;
#pragma unroll
    for (int q = 0; q < KC; ++q) {
      const int k = k0 + q;
      C* d = dst + q * GT;
      if (!gv || k >= K) {
        *d = czero<C>();
      } else if (k < nb && LX0 == LAYOUT_SPLIT) {
        const size_t o = (sk * ng + gs) * nb + k;
        cp_async<sizeof(R)>(&d->x, reinterpret_cast<const R*>(X0a) + o);
        cp_async<sizeof(R)>(&d->y, reinterpret_cast<const R*>(X0b) + o);
      } else {
        const C* src = k < nb ? reinterpret_cast<const C*>(X0a) : reinterpret_cast<const C*>(X1);
        const int i = k < nb ? k : k - nb;
        cp_async<sizeof(C)>(d, src + (sk * nb + i) * ng + gs);
      }
    }
    cp_async_commit();
  };
  const int lane = t & 31, w = t >> 5, wj = w & 3, wg = w >> 2;
  // G columns of this thread: wg * 128 + (a / 2) * 64 + 2 * lane + (a % 2)
  C acc[TG][TJ];
#pragma unroll
  for (int a = 0; a < TG; ++a)
#pragma unroll
    for (int b = 0; b < TJ; ++b) acc[a][b] = czero<C>();
  const int nchunk = KP / KC;
  stage(0, 0);
  for (int c = 0; c < nchunk; ++c) {
    if (c + 1 < nchunk) {
      stage((c + 1) & 1, (c + 1) * KC);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    const C* xb = xs + (size_t)(c & 1) * KC * GT + wg * 128 + 2 * lane;
#pragma unroll
    for (int q = 0; q < KC; ++q) {
      C x[TG], m[TJ];
#pragma unroll
      for (int a = 0; a < TG; a += 2) {
        const C* px = xb + q * GT + (a / 2) * 64;
        x[a] = px[0];
        x[a + 1] = px[1];
      }
      const C* mr = ms + (size_t)(c * KC + q) * NBP + wj * TJ;
      if constexpr (sizeof(R) == 4) {
#pragma unroll
        for (int b = 0; b < TJ; b += 2) {
          const float4 v = *reinterpret_cast<const float4*>(mr + b);
          m[b] = cmk<C>(v.x, v.y);
          m[b + 1] = cmk<C>(v.z, v.w);
        }
      } else {
#pragma unroll
        for (int b = 0; b < TJ; ++b) m[b] = mr[b];
      }
#pragma unroll
      for (int a = 0; a < TG; ++a)
#pragma unroll
        for (int b = 0; b < TJ; ++b) {
          acc[a][b].x = fma(x[a].x, m[b].x, fma(-x[a].y, m[b].y, acc[a][b].x));
          acc[a][b].y = fma(x[a].x, m[b].y, fma(x[a].y, m[b].x, acc[a][b].y));
        }
    }
    __syncthreads();
  }
  if constexpr (OUT == ROT_BANDMAJOR) {
    C* o = reinterpret_cast<C*>(out0) + sk * nb * ng;
#pragma unroll
    for (int a = 0; a < TG; ++a) {
      const int g = g0 + wg * 128 + (a / 2) * 64 + 2 * lane + (a % 2);
#pragma unroll
      for (int b = 0; b < TJ; ++b) {
        const int j = wj * TJ + b;
        if (g < ng && j < nb) o[(size_t)j * ng + g] = acc[a][b];
      }
    }
    if (kin_part) {
      // kinetic partials of this block: sum over its G vectors of
      // |G+k|^2/2 |c_j(G)|^2 per band j, in precision R (the blocks are
      // summed in FP64)
      const double* tkk = tk + ((sk0 + sk) % nk) * (size_t)ng;
      R kp[TJ];
#pragma unroll
      for (int b = 0; b < TJ; ++b) kp[b] = (R)0;
#pragma unroll
      for (int a = 0; a < TG; ++a) {
        const int g = g0 + wg * 128 + (a / 2) * 64 + 2 * lane + (a % 2);
        const R tg = g < ng ? (R)tkk[g] : (R)0;
#pragma unroll
        for (int b = 0; b < TJ; ++b)
          kp[b] += tg * (acc[a][b].x * acc[a][b].x + acc[a][b].y * acc[a][b].y);
      }
#pragma unroll
      for (int b = 0; b < TJ; ++b)
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) kp[b] += __shfl_xor_sync(0xffffffffu, kp[b], off);
      R* red = reinterpret_cast<R*>(xs);   // [2][NBP], the staging ring is free now
      if (lane == 0) {
#pragma unroll
        for (int b = 0; b < TJ; ++b) red[wg * NBP + wj * TJ + b] = kp[b];
      }
      __syncthreads();
      if (t < nb)
        reinterpret_cast<R*>(kin_part)[((size_t)sk * gridDim.x + blockIdx.x) * nb + t] =
            red[t] + red[NBP + t];
    }
  } else if constexpr (OUT == ROT_GMAJOR_SPLIT) {
    // (S,K,G,B) split real/imag times fac, one part at a time through shared
    // memory: tile[g_local][band], row stride NBP + 1
    R* tile = reinterpret_cast<R*>(xs);
    const size_t base = (sk * ng + g0) * nb;
    const int len = min(GT, ng - g0) * nb;
#pragma unroll
    for (int part = 0; part < 2; ++part) {
      if (part) __syncthreads();
#pragma unroll
      for (int a = 0; a < TG; ++a) {
        const int gl = wg * 128 + (a / 2) * 64 + 2 * lane + (a % 2);
#pragma unroll
        for (int b = 0; b < TJ; ++b)
          tile[gl * (NBP + 1) + wj * TJ + b] = fac * (part ? acc[a][b].y : acc[a][b].x);
      }
      __syncthreads();
      R* o = reinterpret_cast<R*>(part ? out1 : out0) + base;
      for (int e = t; e < len; e += 256) {
        const int r = e / nb;
        o[e] = tile[r * (NBP + 1) + (e - r * nb)];
      }
    }
  } else {
    // Adam on the block's contiguous run of parameters (both parts): the
    // gradient tiles go to shared memory first so that the accumulators are
    // dead and 8 elements per thread can be in flight
    R* tile = reinterpret_cast<R*>(xs);   // [2][GT][NBP + 1]
    const size_t base = (sk * ng + g0) * nb;
    const int len = min(GT, ng - g0) * nb;
#pragma unroll
    for (int a = 0; a < TG; ++a) {
      const int gl = wg * 128 + (a / 2) * 64 + 2 * lane + (a % 2);
#pragma unroll
      for (int b = 0; b < TJ; ++b) {
        tile[gl * (NBP + 1) + wj * TJ + b] = fac * acc[a][b].x;
        tile[(GT + gl) * (NBP + 1) + wj * TJ + b] = fac * acc[a][b].y;
      }
    }
    __syncthreads();
    // a Cholesky breakdown of this call leaves parameters and moments as they
    // were (the flag is final: every Cholesky of the call ran before)
    if (adam.guard && *adam.guard) return;
    const R lr = (R)adam.lr, b1 = (R)adam.b1, b2 = (R)adam.b2, c1 = (R)adam.c1, c2 = (R)adam.c2,
            eps = (R)adam.eps;
    constexpr int U = 8;
    for (int e0 = t; e0 < 2 * len; e0 += U * 256) {
      R mi[U], vi[U], pi[U];
      float si[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int e = e0 + u * 256;
        if (e < 2 * len) {
          const int part = e >= len, el = e - part * len;
          mi[u] = reinterpret_cast<const R*>(adam.m[part])[base + el];
          vi[u] = reinterpret_cast<const R*>(adam.v[part])[base + el];
          pi[u] = reinterpret_cast<const R*>(adam.p[part])[base + el];
          si[u] = adam.scale[part] ? adam.scale[part][base + el] : 1.0f;
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int e = e0 + u * 256;
        if (e < 2 * len) {
          const int part = e >= len, el = e - part * len;
          const int r = el / nb;
          const R gr = tile[(part * GT + r) * (NBP + 1) + (el - r * nb)];
          if (adam.grad[part]) reinterpret_cast<R*>(adam.grad[part])[base + el] = gr;
          R d = adam_one<R>(gr, mi[u], vi[u], lr, b1, b2, c1, c2, eps);
          if (adam.scale[part]) d *= (R)si[u];
          reinterpret_cast<R*>(adam.m[part])[base + el] = mi[u];
          reinterpret_cast<R*>(adam.v[part])[base + el] = vi[u];
          reinterpret_cast<R*>(adam.p[part])[base + el] = pi[u] + d;
        }
      }
    }
  }
}

// ------------------------------------------------------------------------
// host launchers
// ------------------------------------------------------------------------
template <typename R>
int launch_pack_params(const void* w_re, const void* w_im, void* out, int nsk, int ng, int nb,
                       bool complex_in, cudaStream_t st) {
  dim3 grid((ng + 31) / 32, (nb + 31) / 32, nsk), block(32, 8);
  if (complex_in)
    k_pack_params<R, true><<<grid, block, 0, st>>>(reinterpret_cast<const R*>(w_re), nullptr,
                                                   reinterpret_cast<C_t<R>*>(out), ng, nb);
  else
    k_pack_params<R, false><<<grid, block, 0, st>>>(reinterpret_cast<const R*>(w_re),
                                                    reinterpret_cast<const R*>(w_im),
                                                    reinterpret_cast<C_t<R>*>(out), ng, nb);
  JRG_LAUNCH_CHECK("k_pack_params");
  return JRG_OK;
}

template <typename R>
int launch_unpack(const void* in, void* o_re, void* o_im, void* o_c, int nsk, int ng, int nb,
                  double fac, cudaStream_t st) {
  dim3 grid((ng + 31) / 32, (nb + 31) / 32, nsk), block(32, 8);
  if (o_c)
    k_unpack<R, false><<<grid, block, 0, st>>>(reinterpret_cast<const C_t<R>*>(in), nullptr,
                                               nullptr, reinterpret_cast<C_t<R>*>(o_c), ng, nb,
                                               (R)fac);
  else
    k_unpack<R, true><<<grid, block, 0, st>>>(reinterpret_cast<const C_t<R>*>(in),
                                              reinterpret_cast<R*>(o_re),
                                              reinterpret_cast<R*>(o_im), nullptr, ng, nb, (R)fac);
  JRG_LAUNCH_CHECK("k_unpack");
  return JRG_OK;
}

int launch_gram_tc(int lx, const void* X0, const void* X1, int ly, const void* Y0, const void* Y1,
                   double* part, double2* out, int nsk, int ng, int nb, int nsplit, cudaStream_t st);
int launch_rotate_tc(int out_kind, int lx0, const void* X0a, const void* X0b, const double2* M0,
                     const void* X1, const double2* M1, void* out0, void* out1, int nsk, int ng,
                     int nb, double fac, uint32_t* bscratch, cudaStream_t st);
// contraction kernels: 0 CUDA cores (default: thread-per-G rotations of
// k_rotate_g.cu), 1 mma.sync TF32 x 3 Gram and rotation (FP32 path), 2
// tcgen05 TF32 x 3 Gram (FP32 path), 3 the register-blocked CUDA-core
// rotations below
static int g_tc_mode = 0;
template <typename R>
int launch_rotate_g(int out_kind, int lx0, const void* X0a, const void* X0b, const double2* M0, const void* X1,
                    const double2* M1, void* out0, void* out1, int nsk, int ng, int nb, double fac,
                    const AdamArgs& adam, const double* tk, int nk, void* kin_part, int sk0, int tri0,
                    cudaStream_t st);
constexpr int kTriUpper = 1, kTriLower = 2;   // zero patterns of M0 for launch_rotate_g
int launch_gram_tc5(int lay, const void* X0, const void* X1, const void* Y0, const void* Y1,
                    double2* part, int nsk, int ng, int nb, int nsplit, int* err, cudaStream_t st);
int launch_gram_big(int lay, const void* X0, const void* X1, const void* Y0, const void* Y1, double2* part,
                    double2* out, int nsk, int ng, int nb, int max_splits, cudaStream_t st);
static bool g_gram_rb = true;       // register-blocked Gram for B <= 32 (else 32x32 tiles)
static bool g_rotate_rb = true;     // register-blocked rotation for B <= 32
void set_gram_rb(bool on) { g_gram_rb = on; g_rotate_rb = on; }

template <typename R>
// full: every element of S is consumed (the band Hamiltonian C^H H C with
// band weights); otherwise the upper triangle suffices (W^H W is Hermitian,
// the energy adjoint reads the upper triangle of C^H g_C) and more than 32
// bands take the upper-tile kernel
int launch_gram(int lx, const void* X0, const void* X1, int ly, const void* Y0, const void* Y1,
                double2* part, double2* out, int nsk, int ng, int nb, int nsplit, cudaStream_t st,
                int* flags, bool full) {
  if (sizeof(R) == 4 && g_tc_mode == 2 && lx == ly) {   // tcgen05 Gram (TF32 x 3)
    const int ns = launch_gram_tc5(lx, X0, X1, Y0, Y1, part, nsk, ng, nb, nsplit, flags, st);
    if (ns < 0) return -ns;
    if (ns > 0) {
      const size_t n = (size_t)nsk * nb * nb;
      k_gram_reduce<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(part, out, ns, nb, nsk);
      JRG_LAUNCH_CHECK("k_gram_reduce");
      return JRG_OK;
    }
  }
  if (sizeof(R) == 4 && g_tc_mode == 1) {   // FP32 path: mma.sync tensor cores (TF32 x3)
    const int t = launch_gram_tc(lx, X0, X1, ly, Y0, Y1, reinterpret_cast<double*>(part), out, nsk,
                                 ng, nb, nsplit, st);
    if (t < 0) return -t;
    if (t > 0) return JRG_OK;
  }
  if (sizeof(R) == 4 && nb > 32 && g_tc_mode == 0 && lx == ly && !full)   // 32 x 32 upper tiles
    return launch_gram_big(lx, X0, X1, Y0, Y1, part, out, nsk, ng, nb, nsplit, st);
  if (nb <= 32 && g_gram_rb) {
    // about four blocks per SM in total: long G ranges per block keep the
    // partial-sum traffic small
    nsplit = std::max(1, std::min(nsplit, (4 * 152 + nsk - 1) / nsk));
    const int split_len = (ng + nsplit - 1) / nsplit;
    const bool same = X0 == Y0 && X1 == Y1 && lx == ly;
    auto go = [&](auto kern, int nbp) -> int {
      const size_t sm = gram_w_smem<R>(nbp, same);
      if (sm > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(gram_w)");
      }
      kern<<<dim3(nsplit, 1, nsk), 256, sm, st>>>(X0, X1, Y0, Y1, part, ng, nb, split_len);
      JRG_LAUNCH_CHECK("k_gram_w");
      return JRG_OK;
    };
    auto pick = [&](auto lxc, auto lyc) -> int {
      constexpr int A = decltype(lxc)::value, B = decltype(lyc)::value;
      if (same) {
        if (nb <= 8) return go(k_gram_w<R, A, B, 8, true>, 8);
        if (nb <= 16) return go(k_gram_w<R, A, B, 16, true>, 16);
        if (nb <= 24) return go(k_gram_w<R, A, B, 24, true>, 24);
        return go(k_gram_w<R, A, B, 32, true>, 32);
      }
      if (nb <= 8) return go(k_gram_w<R, A, B, 8>, 8);
      if (nb <= 16) return go(k_gram_w<R, A, B, 16>, 16);
      if (nb <= 24) return go(k_gram_w<R, A, B, 24>, 24);
      return go(k_gram_w<R, A, B, 32>, 32);
    };
    int rc;
    if (lx == LAYOUT_SPLIT && ly == LAYOUT_SPLIT)
      rc = pick(std::integral_constant<int, LAYOUT_SPLIT>{}, std::integral_constant<int, LAYOUT_SPLIT>{});
    else if (lx == LAYOUT_BAND && ly == LAYOUT_BAND)
      rc = pick(std::integral_constant<int, LAYOUT_BAND>{}, std::integral_constant<int, LAYOUT_BAND>{});
    else
      return fail(JRG_ERR_INVALID, "launch_gram: unsupported layout pair");
    if (rc) return rc;
    const size_t n = (size_t)nsk * nb * nb;
    k_gram_reduce<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(part, out, nsplit, nb, nsk);
    JRG_LAUNCH_CHECK("k_gram_reduce");
    return JRG_OK;
  }
  const int split_len = (ng + nsplit - 1) / nsplit;
  const int ntile = (nb + kGramTile - 1) / kGramTile;
  dim3 grid(nsplit, ntile * ntile, nsk);
  if (lx == LAYOUT_SPLIT && ly == LAYOUT_SPLIT)
    k_gram_partial<R, LAYOUT_SPLIT, LAYOUT_SPLIT><<<grid, 256, 0, st>>>(X0, X1, Y0, Y1, part, ng, nb, split_len);
  else if (lx == LAYOUT_BAND && ly == LAYOUT_BAND)
    k_gram_partial<R, LAYOUT_BAND, LAYOUT_BAND><<<grid, 256, 0, st>>>(X0, X1, Y0, Y1, part, ng, nb, split_len);
  else
    return fail(JRG_ERR_INVALID, "launch_gram: unsupported layout pair");
  JRG_LAUNCH_CHECK("k_gram_partial");
  const size_t n = (size_t)nsk * nb * nb;
  k_gram_reduce<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(part, out, nsplit, nb, nsk);
  JRG_LAUNCH_CHECK("k_gram_reduce");
  return JRG_OK;
}

int launch_cholesky_inv_df(const double2* S, double2* Ri, int nsk, int nb, int* flags, double min_pivot,
                           cudaStream_t st);
// df: the FP32 path uses the double-float kernel (R itself is then not
// written: only R^-1 is consumed)
int launch_cholesky_inv(const double2* S, double2* Rm, double2* Ri, int nsk, int nb, int* flags,
                        double* dinv_scratch, cudaStream_t st, double min_pivot, bool df) {
  if (df && g_tc_mode == 0) {
    const int r = launch_cholesky_inv_df(S, Ri, nsk, nb, flags, min_pivot, st);
    if (r < 0) return -r;
    if (r > 0) return JRG_OK;
  }
  if (nb <= 32) {
    k_cholesky_inv_elem<<<nsk, ((nb * nb + 31) / 32) * 32, 0, st>>>(S, Rm, Ri, nb, flags, min_pivot);
  } else {
    k_cholesky_inv_big<<<nsk, 1024, 0, st>>>(S, Rm, Ri, dinv_scratch, nb, flags, min_pivot);
  }
  JRG_LAUNCH_CHECK("k_cholesky_inv");
  return JRG_OK;
}

int launch_adjoint_small(const double2* A, const double2* Ri, double2* Rh, double2* negM2, int nsk,
                         int nb, cudaStream_t st, const double* f, double* eps) {
  const bool tiled = nb > 32;
  const unsigned parts = (unsigned)((nb * nb + kAdjSmallThreads - 1) / kAdjSmallThreads);
  k_adjoint_small<<<dim3(nsk, parts), kAdjSmallThreads, 0, st>>>(A, Ri, Rh, negM2, nb, f, eps, !tiled);
  JRG_LAUNCH_CHECK("k_adjoint_small");
  if (tiled) {
    const unsigned nt = (unsigned)((nb + 31) / 32);
    k_adjoint_m2_tiled<<<dim3(nt, nt, nsk), 256, 0, st>>>(A, Ri, negM2, nb, f);
    JRG_LAUNCH_CHECK("k_adjoint_m2_tiled");
  }
  return JRG_OK;
}

template <typename R, int OUT, int J>
static int rotate_j(int lx0, const void* X0a, const void* X0b, const double2* M0, int lx1,
                    const void* X1a, const void* X1b, const double2* M1, void* out0, void* out1,
                    int nsk, int ng, int nb, double fac, cudaStream_t st) {
  using C = C_t<R>;
  const int nterms = X1a ? 2 : 1;
  const size_t sm = sizeof(C) * (size_t)nterms * nb * J;
  dim3 grid((ng + 255) / 256, (nb + J - 1) / J, nsk);
  auto go = [&](auto kern) -> int {
    if (sm > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(rotate)");
    }
    kern<<<grid, 256, sm, st>>>(X0a, X0b, M0, X1a, X1b, M1, out0, out1, ng, nb, (R)fac);
    JRG_LAUNCH_CHECK("k_rotate");
    return JRG_OK;
  };
  if (lx0 == LAYOUT_SPLIT) return go(k_rotate<R, OUT, J, LAYOUT_SPLIT, LAYOUT_BAND>);
  return go(k_rotate<R, OUT, J, LAYOUT_BAND, LAYOUT_BAND>);
}

template <typename R, int OUT>
static int rotate_out(int lx0, const void* X0a, const void* X0b, const double2* M0, int lx1,
                      const void* X1a, const void* X1b, const double2* M1, void* out0, void* out1,
                      int nsk, int ng, int nb, double fac, cudaStream_t st) {
  if (nb <= 8) return rotate_j<R, OUT, 8>(lx0, X0a, X0b, M0, lx1, X1a, X1b, M1, out0, out1, nsk, ng, nb, fac, st);
  if (nb <= 16) return rotate_j<R, OUT, 16>(lx0, X0a, X0b, M0, lx1, X1a, X1b, M1, out0, out1, nsk, ng, nb, fac, st);
  if (nb <= 24) return rotate_j<R, OUT, 24>(lx0, X0a, X0b, M0, lx1, X1a, X1b, M1, out0, out1, nsk, ng, nb, fac, st);
  return rotate_j<R, OUT, 32>(lx0, X0a, X0b, M0, lx1, X1a, X1b, M1, out0, out1, nsk, ng, nb, fac, st);
}

// out_kind: ROT_*; lx0: layout of X0 (split: X0a=re, X0b=im; band: X0a); X1 is band-major
// tri0: zero pattern of M0 (0 full, 1 upper triangular, 2 lower triangular)
template <typename R>
int launch_rotate(int out_kind, int lx0, const void* X0a, const void* X0b, const double2* M0,
                  const void* X1, const double2* M1, void* out0, void* out1, int nsk, int ng, int nb,
                  double fac, void* scratch, cudaStream_t st, int tri0) {
  if (X1 && lx0 != LAYOUT_BAND) return fail(JRG_ERR_INVALID, "launch_rotate: two-term form needs band-major inputs");
  if (g_tc_mode == 0)
    return launch_rotate_g<R>(out_kind, lx0, X0a, X0b, M0, X1, M1, out0, out1, nsk, ng, nb, fac, AdamArgs{},
                              nullptr, 1, nullptr, 0, tri0, st);
  if (sizeof(R) == 4 && g_tc_mode == 1) {
    const int t = launch_rotate_tc(out_kind, lx0, X0a, X0b, M0, X1, M1, out0, out1, nsk, ng, nb, fac,
                                   reinterpret_cast<uint32_t*>(scratch), st);
    if (t < 0) return -t;
    if (t > 0) return JRG_OK;
  }
  if (nb <= 32 && g_rotate_rb && out_kind != ROT_GMAJOR_C &&
      (lx0 == LAYOUT_BAND || !X1)) {
    const int K = (X1 ? 2 : 1) * nb;
    auto go = [&](auto kern, int nbp) -> int {
      const size_t sm = rotate_rb_smem<R>(K, nbp);
      if (sm > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(rotate_rb)");
      }
      kern<<<dim3((ng + kRbGT - 1) / kRbGT, nsk), 256, sm, st>>>(X0a, X0b, M0, X1, M1, out0, out1, ng,
                                                                 nb, (R)fac, AdamArgs{}, nullptr, 1,
                                                                 nullptr, 0);
      JRG_LAUNCH_CHECK("k_rotate_rb");
      return JRG_OK;
    };
    auto pick = [&](auto lxc, auto outc) -> int {
      constexpr int L = decltype(lxc)::value, O = decltype(outc)::value;
      if (nb <= 8) return go(k_rotate_rb<R, L, O, 8>, 8);
      if (nb <= 16) return go(k_rotate_rb<R, L, O, 16>, 16);
      if (nb <= 24) return go(k_rotate_rb<R, L, O, 24>, 24);
      return go(k_rotate_rb<R, L, O, 32>, 32);
    };
    using IS = std::integral_constant<int, LAYOUT_SPLIT>;
    using IB = std::integral_constant<int, LAYOUT_BAND>;
    using OB = std::integral_constant<int, ROT_BANDMAJOR>;
    using OS = std::integral_constant<int, ROT_GMAJOR_SPLIT>;
    if (lx0 == LAYOUT_SPLIT)
      return out_kind == ROT_BANDMAJOR ? pick(IS{}, OB{}) : pick(IS{}, OS{});
    return out_kind == ROT_BANDMAJOR ? pick(IB{}, OB{}) : pick(IB{}, OS{});
  }
  if (out_kind == ROT_BANDMAJOR)
    return rotate_out<R, ROT_BANDMAJOR>(lx0, X0a, X0b, M0, LAYOUT_BAND, X1, nullptr, M1, out0, out1, nsk, ng, nb, fac, st);
  if (out_kind == ROT_GMAJOR_C)
    return rotate_out<R, ROT_GMAJOR_C>(lx0, X0a, X0b, M0, LAYOUT_BAND, X1, nullptr, M1, out0, out1, nsk, ng, nb, fac, st);
  return rotate_out<R, ROT_GMAJOR_SPLIT>(lx0, X0a, X0b, M0, LAYOUT_BAND, X1, nullptr, M1, out0, out1, nsk, ng, nb, fac, st);
}

// C = W R^{-1} (parameter layout in, band-major out) with the kinetic
// partials of each block written to kin_part [nsk][nblk][nb] (precision R); returns the
// block count per (s,k) (> 0), 0 when not applicable, or -error.
template <typename R>
int launch_rotate_kinetic(const void* Wre, const void* Wim, const double2* Ri, void* C, int nsk,
                          int ng, int nb, const double* tk, int nk, void* kin_part,
                          cudaStream_t st, int sk0) {
  if (g_tc_mode == 0) {
    const int rc = launch_rotate_g<R>(ROT_BANDMAJOR, LAYOUT_SPLIT, Wre, Wim, Ri, nullptr, nullptr, C, nullptr, nsk,
                                      ng, nb, 1.0, AdamArgs{}, tk, nk, kin_part, sk0, kTriUpper, st);
    return rc ? -rc : (ng + 255) / 256;   // the thread-per-G kernel's 256 G vectors per block
  }
  if (nb > 32 || !g_rotate_rb || (sizeof(R) == 4 && g_tc_mode == 1)) return 0;
  auto go = [&](auto kern, int nbp) -> int {
    const size_t sm = rotate_rb_smem<R>(nb, nbp);
    if (sm > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      if (e != cudaSuccess) return -cuda_fail(e, "cudaFuncSetAttribute(rotate_rb kinetic)");
    }
    const int nblk = (ng + kRbGT - 1) / kRbGT;
    kern<<<dim3(nblk, nsk), 256, sm, st>>>(Wre, Wim, Ri, nullptr, nullptr, C, nullptr, ng, nb,
                                           (R)1.0, AdamArgs{}, tk, nk, kin_part, sk0);
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return -cuda_fail(e, "k_rotate_rb(kinetic)");
    return nblk;
  };
  if (nb <= 8) return go(k_rotate_rb<R, LAYOUT_SPLIT, ROT_BANDMAJOR, 8>, 8);
  if (nb <= 16) return go(k_rotate_rb<R, LAYOUT_SPLIT, ROT_BANDMAJOR, 16>, 16);
  if (nb <= 24) return go(k_rotate_rb<R, LAYOUT_SPLIT, ROT_BANDMAJOR, 24>, 24);
  return go(k_rotate_rb<R, LAYOUT_SPLIT, ROT_BANDMAJOR, 32>, 32);
}

template <typename R>
int launch_rotate_adam(const void* X0, const double2* M0, const void* X1, const double2* M1,
                       const AdamArgs& a, int nsk, int ng, int nb, double fac, cudaStream_t st) {
  if (g_tc_mode == 0)
    return launch_rotate_g<R>(ROT_ADAM, LAYOUT_BAND, X0, nullptr, M0, X1, M1, nullptr, nullptr, nsk, ng, nb, fac,
                              a, nullptr, 1, nullptr, 0, kTriLower, st);
  if (nb > 32) return fail(JRG_ERR_UNSUPPORTED, "k_rotate_rb: num_band > 32");
  auto go = [&](auto kern, int nbp) -> int {
    const size_t sm = rotate_rb_smem<R>(2 * nb, nbp, true);
    if (sm > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(rotate_rb adam)");
    }
    kern<<<dim3((ng + kRbGT - 1) / kRbGT, nsk), 256, sm, st>>>(X0, nullptr, M0, X1, M1, nullptr,
                                                               nullptr, ng, nb, (R)fac, a, nullptr, 1,
                                                               nullptr, 0);
    JRG_LAUNCH_CHECK("k_rotate_rb(adam)");
    return JRG_OK;
  };
  if (nb <= 8) return go(k_rotate_rb<R, LAYOUT_BAND, ROT_ADAM, 8>, 8);
  if (nb <= 16) return go(k_rotate_rb<R, LAYOUT_BAND, ROT_ADAM, 16>, 16);
  if (nb <= 24) return go(k_rotate_rb<R, LAYOUT_BAND, ROT_ADAM, 24>, 24);
  return go(k_rotate_rb<R, LAYOUT_BAND, ROT_ADAM, 32>, 32);
}

// ------------------------------------------------------------------------
// Re-orthonormalisation of the raw parameters (the recovery path after a
// Cholesky breakdown or a growing Gram condition estimate).  Per (s,k) block,
// in place, W = Q diag(n): Q the orthonormal basis of W's columns by
// classical Gram-Schmidt with a second projection pass (CGS2) in FP64, n the
// original column norms.  Cholesky QR of the result returns Q, which for a
// full-rank W is the Cholesky QR factor of W itself (both are the QR factor
// with a positive diagonal R), so the energy is unchanged.  A column with a
// non-finite entry, or whose norm after the projections is below 1e-10 of
// its own (dependent on the previous columns), is replaced by a fixed
// pseudo-random vector projected the same way and given the rms norm of the
// finite columns.  One CTA per (s,k) block; v, the column being projected,
// sits in FP64 scratch (ng complex per block).
// ------------------------------------------------------------------------
constexpr int kReorthThreads = 1024;
constexpr int kReorthChunk = 8;   // projections reduced together

// block sum of kReorthChunk complex values (all threads get the result)
__device__ __forceinline__ void reorth_block_sum(double2 (&h)[kReorthChunk], double* red) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < kReorthChunk; ++q)
    for (int o = 16; o > 0; o >>= 1) {
      h[q].x += __shfl_xor_sync(0xffffffffu, h[q].x, o);
      h[q].y += __shfl_xor_sync(0xffffffffu, h[q].y, o);
    }
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < kReorthChunk; ++q) {
      red[(w * kReorthChunk + q) * 2] = h[q].x;
      red[(w * kReorthChunk + q) * 2 + 1] = h[q].y;
    }
  __syncthreads();
  const int nw = blockDim.x >> 5;
#pragma unroll
  for (int q = 0; q < kReorthChunk; ++q) {
    double x = 0.0, y = 0.0;
    for (int i = 0; i < nw; ++i) { x += red[(i * kReorthChunk + q) * 2]; y += red[(i * kReorthChunk + q) * 2 + 1]; }
    h[q] = make_double2(x, y);
  }
  __syncthreads();
}

template <typename R>
__global__ void __launch_bounds__(kReorthThreads) k_reorthonormalise(R* __restrict__ wr, R* __restrict__ wi,
                                                                     double2* __restrict__ scratch, int ng,
                                                                     int nb) {
  __shared__ double red[32 * kReorthChunk * 2];
  extern __shared__ double colnorm[];   // [nb]: the column's original norm, < 0 for a replaced column
  const size_t sk = blockIdx.x;
  R* xr = wr + sk * (size_t)ng * nb;
  R* xi = wi + sk * (size_t)ng * nb;
  double2* v = scratch + sk * (size_t)ng;
  const int t = threadIdx.x, T = blockDim.x;
  // v -= sum_{j < b} q_j (q_j^H v), twice (the q_j are the finished columns)
  auto project = [&](int b) {
    for (int pass = 0; pass < 2; ++pass)
      for (int j0 = 0; j0 < b; j0 += kReorthChunk) {
        double2 h[kReorthChunk];
#pragma unroll
        for (int q = 0; q < kReorthChunk; ++q) h[q] = make_double2(0.0, 0.0);
        for (int g = t; g < ng; g += T) {
          const double2 x = v[g];
#pragma unroll
          for (int q = 0; q < kReorthChunk; ++q) {
            if (j0 + q < b) {
              const double a = xr[(size_t)g * nb + j0 + q], c = xi[(size_t)g * nb + j0 + q];
              h[q].x += a * x.x + c * x.y;     // conj(q) x
              h[q].y += a * x.y - c * x.x;
            }
          }
        }
        reorth_block_sum(h, red);
        for (int g = t; g < ng; g += T) {
          double2 x = v[g];
#pragma unroll
          for (int q = 0; q < kReorthChunk; ++q) {
            if (j0 + q < b) {
              const double a = xr[(size_t)g * nb + j0 + q], c = xi[(size_t)g * nb + j0 + q];
              x.x -= a * h[q].x - c * h[q].y;
              x.y -= a * h[q].y + c * h[q].x;
            }
          }
          v[g] = x;
        }
        __syncthreads();
      }
  };
  auto norm2 = [&]() {
    double2 h[kReorthChunk];
#pragma unroll
    for (int q = 0; q < kReorthChunk; ++q) h[q] = make_double2(0.0, 0.0);
    for (int g = t; g < ng; g += T) h[0].x += v[g].x * v[g].x + v[g].y * v[g].y;
    reorth_block_sum(h, red);
    return h[0].x;
  };
  for (int b = 0; b < nb; ++b) {
    // the column; a non-finite entry makes its norm non-finite
    for (int g = t; g < ng; g += T) v[g] = make_double2((double)xr[(size_t)g * nb + b], (double)xi[(size_t)g * nb + b]);
    __syncthreads();
    const double n0 = norm2();
    bool good = isfinite(n0) && n0 > 0.0;   // the same value in every thread (block sum)
    double n1 = 0.0;
    if (good) {
      project(b);
      n1 = norm2();
      good = n1 > 1e-20 * n0;
    }
    if (!good) {
      // fixed pseudo-random replacement (hash of g and b), projected the same way
      for (int g = t; g < ng; g += T) {
        const unsigned h1 = (unsigned)g * 2654435761u ^ (unsigned)(b + 1) * 40503u;
        const unsigned h2 = h1 * 2246822519u + 3266489917u;
        v[g] = make_double2((double)(h1 >> 8) / 16777216.0 - 0.5, (double)(h2 >> 8) / 16777216.0 - 0.5);
      }
      __syncthreads();
      project(b);
      n1 = norm2();
    }
    const double s = n1 > 0.0 ? 1.0 / sqrt(n1) : 0.0;
    for (int g = t; g < ng; g += T) {
      xr[(size_t)g * nb + b] = (R)(v[g].x * s);
      xi[(size_t)g * nb + b] = (R)(v[g].y * s);
    }
    if (t == 0) colnorm[b] = good ? sqrt(n0) : -1.0;
    __syncthreads();
  }
  // the columns back to their norms (replaced ones to the rms of the others)
  double rms = 0.0;
  int cnt = 0;
  for (int b = 0; b < nb; ++b)
    if (colnorm[b] > 0.0) { rms += colnorm[b] * colnorm[b]; ++cnt; }
  rms = cnt > 0 ? sqrt(rms / cnt) : 1.0;
  for (size_t e = t; e < (size_t)ng * nb; e += T) {
    const int b = (int)(e % nb);
    const double s = colnorm[b] > 0.0 ? colnorm[b] : rms;
    xr[e] = (R)((double)xr[e] * s);
    xi[e] = (R)((double)xi[e] * s);
  }
}

template <typename R>
int launch_reorthonormalise(void* wr, void* wi, double2* scratch, int nsk, int ng, int nb, cudaStream_t st) {
  const size_t sm = (size_t)nb * sizeof(double);
  if (sm > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k_reorthonormalise<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(k_reorthonormalise)");
  }
  k_reorthonormalise<R><<<nsk, kReorthThreads, sm, st>>>(reinterpret_cast<R*>(wr), reinterpret_cast<R*>(wi),
                                                        scratch, ng, nb);
  JRG_LAUNCH_CHECK("k_reorthonormalise");
  return JRG_OK;
}

#define JRG_INST_ORTH(R)                                                                        \
  template int launch_reorthonormalise<R>(void*, void*, double2*, int, int, int, cudaStream_t);     \
  template int launch_rotate_kinetic<R>(const void*, const void*, const double2*, void*, int, int,  \
                                        int, const double*, int, void*, cudaStream_t, int);     \
  template int launch_rotate_adam<R>(const void*, const double2*, const void*, const double2*,    \
                                     const AdamArgs&, int, int, int, double, cudaStream_t);       \
  template int launch_pack_params<R>(const void*, const void*, void*, int, int, int, bool,         \
                                     cudaStream_t);                                             \
  template int launch_unpack<R>(const void*, void*, void*, void*, int, int, int, double,          \
                                cudaStream_t);                                                  \
  template int launch_gram<R>(int, const void*, const void*, int, const void*, const void*,       \
                              double2*, double2*, int, int, int, int, cudaStream_t, int*, bool); \
  template int launch_rotate<R>(int, int, const void*, const void*, const double2*, const void*,  \
                                const double2*, void*, void*, int, int, int, double, void*,     \
                                cudaStream_t, int);
JRG_INST_ORTH(float)
JRG_INST_ORTH(double)

}  // namespace jrg

extern "C" int jrg_tensor_core_paths(int enable) {
  const int prev = jrg::g_tc_mode;
  if (enable >= 0 && enable <= 3) jrg::g_tc_mode = enable;
  return prev;
}
