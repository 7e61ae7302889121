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

// Partial Gram S[i][j] = sum_g conj(X[i][g]) Y[j][g] over one G split, for a
// 32x32 output tile.  Products and 64-term runs in precision R, runs summed
// in FP64.
constexpr int kGramTile = 32;
template <typename R> struct GramChunk { static constexpr int value = 64; };
template <> struct GramChunk<double> { static constexpr int value = 32; };  // 48 KB static smem

template <typename R>
__global__ void __launch_bounds__(256) k_gram_partial(const C_t<R>* __restrict__ X,
                                                      const C_t<R>* __restrict__ Y,
                                                      double2* __restrict__ part, int ng, int nb,
                                                      int split_len) {
  using C = C_t<R>;
  constexpr int kGramChunk = GramChunk<R>::value;
  __shared__ C xs[kGramTile][kGramChunk + 1];
  __shared__ C ys[kGramTile][kGramChunk + 1];
  const int split = blockIdx.x;
  const int ntile = (nb + kGramTile - 1) / kGramTile;
  const int ti = blockIdx.y / ntile, tj = blockIdx.y % ntile;
  const int sk = blockIdx.z;
  const int nsplit = gridDim.x;
  const C* Xs = X + (size_t)sk * nb * ng;
  const C* Ys = Y + (size_t)sk * nb * ng;
  const int g_begin = split * split_len;
  const int g_end = min(ng, g_begin + split_len);
  // each thread owns 4 outputs: (i, j) = (ty + 8*q, tx) with tx < 32, ty < 8
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  double2 acc[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) acc[q] = make_double2(0.0, 0.0);
  for (int g0 = g_begin; g0 < g_end; g0 += kGramChunk) {
    for (int idx = threadIdx.x; idx < kGramTile * kGramChunk; idx += blockDim.x) {
      const int r = idx / kGramChunk, c = idx % kGramChunk;
      const int g = g0 + c;
      const int bi = ti * kGramTile + r, bj = tj * kGramTile + r;
      xs[r][c] = (g < g_end && bi < nb) ? Xs[(size_t)bi * ng + g] : czero<C>();
      ys[r][c] = (g < g_end && bj < nb) ? Ys[(size_t)bj * ng + g] : czero<C>();
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int i = ty + 8 * q;
      C s = czero<C>();
#pragma unroll 8
      for (int c = 0; c < kGramChunk; ++c) {
        const C a = xs[i][c], b = ys[tx][c];
        // conj(a) * b
        s.x += a.x * b.x + a.y * b.y;
        s.y += a.x * b.y - a.y * b.x;
      }
      acc[q].x += (double)s.x;
      acc[q].y += (double)s.y;
    }
    __syncthreads();
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int i = ti * kGramTile + ty + 8 * q, j = tj * kGramTile + tx;
    if (i < nb && j < nb) part[(((size_t)sk * nsplit + split) * nb + i) * nb + j] = acc[q];
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

// One CTA per (s,k): R = chol(S) (upper, S = R^H R) and Rinv = R^{-1}.
// Works in global memory (B x B double2).  A non-positive or non-finite
// pivot sets flags[0] |= 1 and continues with a unit pivot.
__global__ void __launch_bounds__(256) k_cholesky_inv(const double2* __restrict__ S,
                                                      double2* __restrict__ Rm,
                                                      double2* __restrict__ Ri, int nb,
                                                      int* __restrict__ flags) {
  const int sk = blockIdx.x;
  const size_t off = (size_t)sk * nb * nb;
  const double2* s = S + off;
  double2* r = Rm + off;
  double2* ri = Ri + off;
  for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
    const int i = e / nb, j = e % nb;
    // Hermitian symmetrisation of the accumulated Gram
    const double2 a = s[i * nb + j], b = s[j * nb + i];
    r[e] = (j >= i) ? make_double2(0.5 * (a.x + b.x), 0.5 * (a.y - b.y)) : make_double2(0.0, 0.0);
  }
  __shared__ double piv;
  __syncthreads();
  for (int k = 0; k < nb; ++k) {
    if (threadIdx.x == 0) {
      double d = r[k * nb + k].x;
      if (!(d > 0.0) || !isfinite(d)) { atomicOr(flags, 1); d = 1.0; }
      d = sqrt(d);
      r[k * nb + k] = make_double2(d, 0.0);
      piv = d;
    }
    __syncthreads();
    const double inv = 1.0 / piv;
    for (int j = k + 1 + threadIdx.x; j < nb; j += blockDim.x) {
      double2 v = r[k * nb + j];
      r[k * nb + j] = make_double2(v.x * inv, v.y * inv);
    }
    __syncthreads();
    const int m = nb - k - 1;
    for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
      const int i = k + 1 + e / m, j = k + 1 + e % m;
      if (j >= i) {
        const double2 a = r[k * nb + i], b = r[k * nb + j];
        double2 v = r[i * nb + j];
        // v -= conj(a) * b
        v.x -= a.x * b.x + a.y * b.y;
        v.y -= a.x * b.y - a.y * b.x;
        r[i * nb + j] = v;
      }
    }
    __syncthreads();
  }
  // Rinv: back substitution, one column per thread
  for (int j = threadIdx.x; j < nb; j += blockDim.x) {
    for (int i = 0; i < nb; ++i) ri[i * nb + j] = make_double2(0.0, 0.0);
    const double djj = r[j * nb + j].x;
    ri[j * nb + j] = make_double2(1.0 / djj, 0.0);
    for (int i = j - 1; i >= 0; --i) {
      double sx = 0.0, sy = 0.0;
      for (int l = i + 1; l <= j; ++l) {
        const double2 a = r[i * nb + l], b = ri[l * nb + j];
        sx += a.x * b.x - a.y * b.y;
        sy += a.x * b.y + a.y * b.x;
      }
      const double dii = r[i * nb + i].x;
      ri[i * nb + j] = make_double2(-sx / dii, -sy / dii);
    }
  }
}

// Adjoint small matrices per (s,k), one CTA each:
//   Rh = R^{-H};  K from A;  M2 = K R^{-H}  (stored negated: -M2)
__global__ void __launch_bounds__(256) k_adjoint_small(const double2* __restrict__ A,
                                                       const double2* __restrict__ Ri,
                                                       double2* __restrict__ Rh,
                                                       double2* __restrict__ negM2, int nb) {
  const int sk = blockIdx.x;
  const size_t off = (size_t)sk * nb * nb;
  const double2* a = A + off;
  const double2* ri = Ri + off;
  for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
    const int i = e / nb, j = e % nb;
    const double2 v = ri[j * nb + i];
    Rh[off + e] = make_double2(v.x, -v.y);
  }
  for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
    const int i = e / nb, j = e % nb;
    // (K R^{-H})[i][j] = sum_l K[i][l] conj(Ri[j][l]),  Ri upper => l >= j
    double sx = 0.0, sy = 0.0;
    for (int l = j; l < nb; ++l) {
      double2 kil;
      if (l > i) kil = a[i * nb + l];
      else if (l < i) { const double2 t = a[l * nb + i]; kil = make_double2(t.x, -t.y); }
      else kil = make_double2(a[i * nb + i].x, 0.0);
      const double2 r = ri[j * nb + l];   // conj later
      sx += kil.x * r.x + kil.y * r.y;
      sy += kil.y * r.x - kil.x * r.y;
    }
    negM2[off + e] = make_double2(-sx, -sy);
  }
}

// out[sk][j][g] (band-major) or (S,K,G,B) layouts of sum_t X_t[sk][i][g] M_t[sk][i][j].
// Thread per g, 16-wide j tile; M tile staged in shared memory in precision R.
constexpr int kRotJ = 16;
enum RotOut { ROT_BANDMAJOR = 0, ROT_GMAJOR_C = 1, ROT_GMAJOR_SPLIT = 2 };

template <typename R, int OUT>
__global__ void __launch_bounds__(256) k_rotate(const C_t<R>* __restrict__ X0,
                                                const double2* __restrict__ M0,
                                                const C_t<R>* __restrict__ X1,
                                                const double2* __restrict__ M1, void* out0,
                                                void* out1, int ng, int nb, R fac) {
  using C = C_t<R>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* ms = reinterpret_cast<C*>(smem_raw);   // [nterms][nb][kRotJ]
  const int sk = blockIdx.z;
  const int j0 = blockIdx.y * kRotJ;
  const int nj = min(kRotJ, nb - j0);
  const int nterms = X1 ? 2 : 1;
  const size_t moff = (size_t)sk * nb * nb;
  for (int e = threadIdx.x; e < nterms * nb * kRotJ; e += blockDim.x) {
    const int t = e / (nb * kRotJ), rem = e % (nb * kRotJ);
    const int i = rem / kRotJ, jj = rem % kRotJ;
    const double2* M = t ? M1 : M0;
    double2 v = (jj < nj) ? M[moff + (size_t)i * nb + j0 + jj] : make_double2(0.0, 0.0);
    ms[e] = cmk<C>(v.x, v.y);
  }
  __syncthreads();
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ng) return;
  C acc[kRotJ];
#pragma unroll
  for (int jj = 0; jj < kRotJ; ++jj) acc[jj] = czero<C>();
  for (int t = 0; t < nterms; ++t) {
    const C* X = (t ? X1 : X0) + (size_t)sk * nb * ng;
    const C* mt = ms + (size_t)t * nb * kRotJ;
    for (int i = 0; i < nb; ++i) {
      const C x = X[(size_t)i * ng + g];
#pragma unroll
      for (int jj = 0; jj < kRotJ; ++jj) {
        const C m = mt[i * kRotJ + jj];
        acc[jj].x = fma(x.x, m.x, fma(-x.y, m.y, acc[jj].x));
        acc[jj].y = fma(x.x, m.y, fma(x.y, m.x, acc[jj].y));
      }
    }
  }
  const size_t base = (size_t)sk * nb * ng;
  if (OUT == ROT_BANDMAJOR) {
    C* o = reinterpret_cast<C*>(out0) + base;
#pragma unroll
    for (int jj = 0; jj < kRotJ; ++jj)
      if (jj < nj) o[(size_t)(j0 + jj) * ng + g] = acc[jj];
  } else if (OUT == ROT_GMAJOR_C) {
    C* o = reinterpret_cast<C*>(out0) + base + (size_t)g * nb + j0;
#pragma unroll
    for (int jj = 0; jj < kRotJ; ++jj)
      if (jj < nj) o[jj] = acc[jj];
  } else {
    R* ore = reinterpret_cast<R*>(out0) + base + (size_t)g * nb + j0;
    R* oim = reinterpret_cast<R*>(out1) + base + (size_t)g * nb + j0;
#pragma unroll
    for (int jj = 0; jj < kRotJ; ++jj)
      if (jj < nj) { ore[jj] = fac * acc[jj].x; oim[jj] = fac * acc[jj].y; }
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

template <typename R>
int launch_gram(const void* X, const void* Y, double2* part, double2* out, int nsk, int ng, int nb,
                int nsplit, cudaStream_t st) {
  const int split_len = (ng + nsplit - 1) / nsplit;
  const int ntile = (nb + kGramTile - 1) / kGramTile;
  dim3 grid(nsplit, ntile * ntile, nsk);
  k_gram_partial<R><<<grid, 256, 0, st>>>(reinterpret_cast<const C_t<R>*>(X),
                                          reinterpret_cast<const C_t<R>*>(Y), part, ng, nb,
                                          split_len);
  JRG_LAUNCH_CHECK("k_gram_partial");
  const size_t n = (size_t)nsk * nb * nb;
  k_gram_reduce<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(part, out, nsplit, nb, nsk);
  JRG_LAUNCH_CHECK("k_gram_reduce");
  return JRG_OK;
}

int launch_cholesky_inv(const double2* S, double2* Rm, double2* Ri, int nsk, int nb, int* flags,
                        cudaStream_t st) {
  k_cholesky_inv<<<nsk, 256, 0, st>>>(S, Rm, Ri, nb, flags);
  JRG_LAUNCH_CHECK("k_cholesky_inv");
  return JRG_OK;
}

int launch_adjoint_small(const double2* A, const double2* Ri, double2* Rh, double2* negM2, int nsk,
                         int nb, cudaStream_t st) {
  k_adjoint_small<<<nsk, 256, 0, st>>>(A, Ri, Rh, negM2, nb);
  JRG_LAUNCH_CHECK("k_adjoint_small");
  return JRG_OK;
}

template <typename R>
int launch_rotate(int out_kind, const void* X0, const double2* M0, const void* X1,
                  const double2* M1, void* out0, void* out1, int nsk, int ng, int nb, double fac,
                  cudaStream_t st) {
  using C = C_t<R>;
  const int nterms = X1 ? 2 : 1;
  const size_t sm = sizeof(C) * (size_t)nterms * nb * kRotJ;
  dim3 grid((ng + 255) / 256, (nb + kRotJ - 1) / kRotJ, nsk);
  auto go = [&](auto kern) -> int {
    if (sm > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(rotate)");
    }
    kern<<<grid, 256, sm, st>>>(reinterpret_cast<const C*>(X0), M0, reinterpret_cast<const C*>(X1),
                                M1, out0, out1, ng, nb, (R)fac);
    JRG_LAUNCH_CHECK("k_rotate");
    return JRG_OK;
  };
  if (out_kind == ROT_BANDMAJOR) return go(k_rotate<R, ROT_BANDMAJOR>);
  if (out_kind == ROT_GMAJOR_C) return go(k_rotate<R, ROT_GMAJOR_C>);
  return go(k_rotate<R, ROT_GMAJOR_SPLIT>);
}

#define JRG_INST_ORTH(R)                                                                        \
  template int launch_pack_params<R>(const void*, const void*, void*, int, int, int, bool,         \
                                     cudaStream_t);                                             \
  template int launch_unpack<R>(const void*, void*, void*, void*, int, int, int, double,          \
                                cudaStream_t);                                                  \
  template int launch_gram<R>(const void*, const void*, double2*, double2*, int, int, int, int,   \
                              cudaStream_t);                                                    \
  template int launch_rotate<R>(int, const void*, const double2*, const void*, const double2*,    \
                                void*, void*, int, int, int, double, cudaStream_t);
JRG_INST_ORTH(float)
JRG_INST_ORTH(double)

}  // namespace jrg
