// Rotations out = sum_t X_t M_t of the orthonormalisation (C = W R^{-1}) and
// of its adjoint (g_W = g_C R^{-H} - C K R^{-H}), one thread per G vector.
//
// Each thread holds NJ complex accumulators (a band tile j0 .. j0+NJ-1 of its
// G vector's output row) in registers and streams its own row of X through
// registers four bands at a time (16-byte loads in the parameter layout,
// coalesced loads in the band-major layout), the next four prefetched while
// the current four are used; the tile of M (K rows x NJ columns, FP64 in
// memory, precision R here) sits in shared memory and every thread reads the
// same element (broadcast).  So one 16-byte shared-memory load feeds eight
// FP32 multiply-adds and no staging of X through shared memory is needed.  A
// triangular first term skips its zero rows (R^{-1} is upper triangular,
// R^{-H} lower).  Band tiles of the same G block are adjacent in the grid, so
// the X rows that several tiles read come from L2.
//
// Epilogues: band-major complex output (+ the per-block kinetic partials
// sum_G |G+k|^2/2 |c_j(G)|^2), (S,K,G,B) complex, (S,K,G,B) split real/imag
// times fac, or the Adam update of the parameters in place.
#include "plan.h"

namespace jrg {

enum { RG_BANDMAJOR = 0, RG_GMAJOR_C = 1, RG_GMAJOR_SPLIT = 2, RG_ADAM = 3 };
enum { RG_TRI_FULL = 0, RG_TRI_UPPER = 1, RG_TRI_LOWER = 2 };
enum { RG_SPLIT = 0, RG_BAND = 1 };   // layouts of X0 (X1 is band-major)
constexpr int kRgThreads = 256;

// rows k .. k+RG-1 of X for G vector g (zero past khi or for an invalid g)
template <typename R, int LX, bool VIN, int RG>
__device__ __forceinline__ void rg_load(const void* __restrict__ a, const void* __restrict__ b, size_t sk, int k,
                                        int g, int ng, int nb, int khi, bool valid, C_t<R> (&x)[RG]) {
  using C = C_t<R>;
#pragma unroll
  for (int q = 0; q < RG; ++q) x[q] = czero<C>();
  if (!valid) return;
  if constexpr (LX == RG_SPLIT) {
    const size_t o = (sk * ng + g) * nb + k;
    if constexpr (VIN && sizeof(R) == 4 && RG == 4) {
      if (k < khi) {   // nb % 4 == 0: the four rows lie inside the G vector's row
        const float4 re = __ldg(reinterpret_cast<const float4*>(reinterpret_cast<const float*>(a) + o));
        const float4 im = __ldg(reinterpret_cast<const float4*>(reinterpret_cast<const float*>(b) + o));
        x[0] = make_float2(re.x, im.x); x[1] = make_float2(re.y, im.y);
        x[2] = make_float2(re.z, im.z); x[3] = make_float2(re.w, im.w);
      }
    } else if constexpr (VIN && sizeof(R) == 4 && RG == 2) {
      if (k < khi) {
        const float2 re = __ldg(reinterpret_cast<const float2*>(reinterpret_cast<const float*>(a) + o));
        const float2 im = __ldg(reinterpret_cast<const float2*>(reinterpret_cast<const float*>(b) + o));
        x[0] = make_float2(re.x, im.x); x[1] = make_float2(re.y, im.y);
      }
    } else {
#pragma unroll
      for (int q = 0; q < RG; ++q)
        if (k + q < khi) {
          x[q].x = __ldg(reinterpret_cast<const R*>(a) + o + q);
          x[q].y = __ldg(reinterpret_cast<const R*>(b) + o + q);
        }
    }
  } else {
#pragma unroll
    for (int q = 0; q < RG; ++q)
      if (k + q < khi) x[q] = __ldg(reinterpret_cast<const C*>(a) + (sk * nb + k + q) * ng + g);
  }
}

// acc[q][jj] += x[q] * M[row][jj] for the TG G vectors and NJ columns
template <typename R, int NJ, int TG>
__device__ __forceinline__ void rg_fma_row(C_t<R> (&acc)[TG][NJ], const C_t<R> (&x)[TG],
                                           const C_t<R>* __restrict__ mrow) {
  if constexpr (sizeof(R) == 4) {
#pragma unroll
    for (int jj = 0; jj < NJ; jj += 2) {
      const float4 m = *reinterpret_cast<const float4*>(mrow + jj);
#pragma unroll
      for (int q = 0; q < TG; ++q) {
        acc[q][jj].x = fmaf(x[q].x, m.x, fmaf(-x[q].y, m.y, acc[q][jj].x));
        acc[q][jj].y = fmaf(x[q].x, m.y, fmaf(x[q].y, m.x, acc[q][jj].y));
        acc[q][jj + 1].x = fmaf(x[q].x, m.z, fmaf(-x[q].y, m.w, acc[q][jj + 1].x));
        acc[q][jj + 1].y = fmaf(x[q].x, m.w, fmaf(x[q].y, m.z, acc[q][jj + 1].y));
      }
    }
  } else {
#pragma unroll
    for (int jj = 0; jj < NJ; ++jj) {
      const double2 m = mrow[jj];
#pragma unroll
      for (int q = 0; q < TG; ++q) {
        acc[q][jj].x = fma(x[q].x, m.x, fma(-x[q].y, m.y, acc[q][jj].x));
        acc[q][jj].y = fma(x[q].x, m.y, fma(x[q].y, m.x, acc[q][jj].y));
      }
    }
  }
}

// rows [lo, hi) of one term (lo a multiple of 4): X rows streamed RG at a
// time, the next RG loaded before the current ones are used
template <typename R, int LX, bool VIN, int NJ, int TG, int RG>
__device__ __forceinline__ void rg_term(C_t<R> (&acc)[TG][NJ], const void* __restrict__ a,
                                        const void* __restrict__ b, size_t sk, const int (&g)[TG], int ng, int nb,
                                        int lo, int hi, const C_t<R>* __restrict__ ms) {
  using C = C_t<R>;
  if (lo >= hi) return;
  C cur[TG][RG], nxt[TG][RG];
#pragma unroll
  for (int q = 0; q < TG; ++q) rg_load<R, LX, VIN, RG>(a, b, sk, lo, g[q], ng, nb, hi, g[q] < ng, cur[q]);
  for (int k = lo; k < hi; k += RG) {
    if (k + RG < hi) {
#pragma unroll
      for (int q = 0; q < TG; ++q) rg_load<R, LX, VIN, RG>(a, b, sk, k + RG, g[q], ng, nb, hi, g[q] < ng, nxt[q]);
    }
#pragma unroll
    for (int r = 0; r < RG; ++r) {
      C x[TG];
#pragma unroll
      for (int q = 0; q < TG; ++q) x[q] = cur[q][r];
      rg_fma_row<R, NJ, TG>(acc, x, ms + (size_t)(k + r) * NJ);
    }
#pragma unroll
    for (int q = 0; q < TG; ++q)
#pragma unroll
      for (int r = 0; r < RG; ++r) cur[q][r] = nxt[q][r];
  }
}

// One CTA: TG x 256 G vectors (g = base + t + 256 q) of one (s,k) and one
// band tile.  VIN: 16-byte (RG 4) or 8-byte (RG 2) loads of the parameter
// layout (nb % 4 == 0); VOUT: 16-byte stores of the (S,K,G,B) outputs
// (nb % 4 == 0, NJ % 4 == 0).
template <typename R, int LX0, int OUT, int NJ, int TG, bool VIN, bool VOUT, int MINB>
__global__ void __launch_bounds__(kRgThreads, MINB)
k_rotate_g(const void* __restrict__ X0a, const void* __restrict__ X0b, const double2* __restrict__ M0,
           const void* __restrict__ X1, const double2* __restrict__ M1, void* out0, void* out1, int ng, int nb,
           R fac, AdamArgs adam, const double* __restrict__ tk, int nk, R* __restrict__ kin_part, int sk0,
           int tri0) {
  using C = C_t<R>;
  constexpr int RG = TG == 1 ? 4 : 2;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nterms = X1 ? 2 : 1;
  const int nbp = (nb + 3) & ~3;
  const int KP = nterms * nbp;                 // staged rows, each term padded to a multiple of 4
  C* ms = reinterpret_cast<C*>(smem_raw);      // [KP][NJ]
  const int t = threadIdx.x;
  const int j0 = blockIdx.x * NJ;
  const int nj = min(NJ, nb - j0);
  const size_t sk = blockIdx.z;
  int g[TG];
#pragma unroll
  for (int q = 0; q < TG; ++q) g[q] = (blockIdx.y * TG + q) * kRgThreads + t;
  int lo0 = 0, hi0 = nb;
  if (tri0 == RG_TRI_UPPER) hi0 = min(nb, j0 + NJ);
  if (tri0 == RG_TRI_LOWER) lo0 = j0;
  const size_t moff = sk * nb * nb;
  // M tile in precision R; rows outside a term's range and padding are zero
  for (int e = t; e < KP * NJ; e += kRgThreads) {
    const int r = e / NJ, jj = e - r * NJ;
    const int term = r >= nbp, k = r - term * nbp;
    double2 v = make_double2(0.0, 0.0);
    const bool in = term ? k < nb : (k >= lo0 && k < hi0);
    if (in && jj < nj) v = (term ? M1 : M0)[moff + (size_t)k * nb + j0 + jj];
    ms[e] = cmk<C>(v.x, v.y);
  }
  __syncthreads();
  C acc[TG][NJ];
#pragma unroll
  for (int q = 0; q < TG; ++q)
#pragma unroll
    for (int jj = 0; jj < NJ; ++jj) acc[q][jj] = czero<C>();
  rg_term<R, LX0, VIN, NJ, TG, RG>(acc, X0a, X0b, sk, g, ng, nb, lo0 & ~3, hi0, ms);
  if (X1) rg_term<R, RG_BAND, false, NJ, TG, RG>(acc, X1, nullptr, sk, g, ng, nb, 0, nb, ms + (size_t)nbp * NJ);

  if constexpr (OUT == RG_BANDMAJOR) {
#pragma unroll
    for (int q = 0; q < TG; ++q)
      if (g[q] < ng) {
        C* o = reinterpret_cast<C*>(out0) + (sk * nb + j0) * ng + g[q];
#pragma unroll
        for (int jj = 0; jj < NJ; ++jj)
          if (jj < nj) o[(size_t)jj * ng] = acc[q][jj];
      }
    if (kin_part) {
      // kinetic partials sum_G |G+k|^2/2 |c_j|^2 per 256 G vectors, in
      // precision R (summed over the blocks in FP64 by the kinetic reduction)
      R* red = reinterpret_cast<R*>(ms);   // [8][NJ], after the barrier below
      const int nblk = (ng + kRgThreads - 1) / kRgThreads;
      __syncthreads();   // every thread is done with the M tile
#pragma unroll
      for (int q = 0; q < TG; ++q) {
        const R tg = g[q] < ng ? (R)tk[(size_t)((sk0 + sk) % nk) * ng + g[q]] : (R)0;
        R kp[NJ];
#pragma unroll
        for (int jj = 0; jj < NJ; ++jj) {
          kp[jj] = tg * (acc[q][jj].x * acc[q][jj].x + acc[q][jj].y * acc[q][jj].y);
#pragma unroll
          for (int off = 16; off > 0; off >>= 1) kp[jj] += __shfl_xor_sync(0xffffffffu, kp[jj], off);
        }
        if ((t & 31) == 0) {
#pragma unroll
          for (int jj = 0; jj < NJ; ++jj) red[(t >> 5) * NJ + jj] = kp[jj];
        }
        __syncthreads();
        const int blk = blockIdx.y * TG + q;
        if (t < nj && blk < nblk) {
          R s = 0;
#pragma unroll
          for (int w = 0; w < kRgThreads / 32; ++w) s += red[w * NJ + t];
          kin_part[(sk * nblk + blk) * nb + j0 + t] = s;
        }
        __syncthreads();
      }
    }
  } else if constexpr (OUT == RG_GMAJOR_C) {
#pragma unroll
    for (int q = 0; q < TG; ++q) {
      if (g[q] >= ng) continue;
      C* o = reinterpret_cast<C*>(out0) + (sk * ng + g[q]) * nb + j0;
#pragma unroll
      for (int jj = 0; jj < NJ; ++jj)
        if (jj < nj) o[jj] = acc[q][jj];
    }
  } else if constexpr (OUT == RG_GMAJOR_SPLIT) {
#pragma unroll
    for (int q = 0; q < TG; ++q) {
      if (g[q] >= ng) continue;
      R* ore = reinterpret_cast<R*>(out0) + (sk * ng + g[q]) * nb + j0;
      R* oim = reinterpret_cast<R*>(out1) + (sk * ng + g[q]) * nb + j0;
      if constexpr (VOUT && sizeof(R) == 4) {
#pragma unroll
        for (int jj = 0; jj < NJ; jj += 4)
          if (jj < nj) {
            *reinterpret_cast<float4*>(ore + jj) = make_float4(fac * acc[q][jj].x, fac * acc[q][jj + 1].x,
                                                               fac * acc[q][jj + 2].x, fac * acc[q][jj + 3].x);
            *reinterpret_cast<float4*>(oim + jj) = make_float4(fac * acc[q][jj].y, fac * acc[q][jj + 1].y,
                                                               fac * acc[q][jj + 2].y, fac * acc[q][jj + 3].y);
          }
      } else {
#pragma unroll
        for (int jj = 0; jj < NJ; ++jj)
          if (jj < nj) { ore[jj] = fac * acc[q][jj].x; oim[jj] = fac * acc[q][jj].y; }
      }
    }
  } else {
    // Adam on this thread's elements of the tile (both parts); a Cholesky
    // breakdown of the call (status word non-zero) leaves everything as it was
    if (adam.guard && *adam.guard) return;
    const R lr = (R)adam.lr, b1 = (R)adam.b1, b2 = (R)adam.b2, c1 = (R)adam.c1, c2 = (R)adam.c2,
            eps = (R)adam.eps;
#pragma unroll
    for (int q = 0; q < TG; ++q) {
      if (g[q] >= ng) continue;
      const size_t base = (sk * ng + g[q]) * nb + j0;
      if constexpr (VOUT && sizeof(R) == 4) {
        // 16-byte accesses: nb % 4 == 0 and NJ % 4 == 0
#pragma unroll
        for (int part = 0; part < 2; ++part) {
          float* p = reinterpret_cast<float*>(adam.p[part]) + base;
          float* m = reinterpret_cast<float*>(adam.m[part]) + base;
          float* v = reinterpret_cast<float*>(adam.v[part]) + base;
          float* gout = adam.grad[part] ? reinterpret_cast<float*>(adam.grad[part]) + base : nullptr;
          const float* sc = adam.scale[part] ? adam.scale[part] + base : nullptr;
#pragma unroll
          for (int jj = 0; jj < NJ; jj += 4)
            if (jj < nj) {
              float gv[4], mv[4], vv[4], pv[4], sv[4] = {1.f, 1.f, 1.f, 1.f};
#pragma unroll
              for (int u = 0; u < 4; ++u) gv[u] = fac * (part ? acc[q][jj + u].y : acc[q][jj + u].x);
              *reinterpret_cast<float4*>(mv) = *reinterpret_cast<const float4*>(m + jj);
              *reinterpret_cast<float4*>(vv) = *reinterpret_cast<const float4*>(v + jj);
              *reinterpret_cast<float4*>(pv) = *reinterpret_cast<const float4*>(p + jj);
              if (sc) *reinterpret_cast<float4*>(sv) = *reinterpret_cast<const float4*>(sc + jj);
              if (gout) *reinterpret_cast<float4*>(gout + jj) = *reinterpret_cast<const float4*>(gv);
#pragma unroll
              for (int u = 0; u < 4; ++u) pv[u] += sv[u] * adam_one<float>(gv[u], mv[u], vv[u], lr, b1, b2, c1, c2, eps);
              *reinterpret_cast<float4*>(m + jj) = *reinterpret_cast<const float4*>(mv);
              *reinterpret_cast<float4*>(v + jj) = *reinterpret_cast<const float4*>(vv);
              *reinterpret_cast<float4*>(p + jj) = *reinterpret_cast<const float4*>(pv);
            }
        }
        continue;
      }
#pragma unroll
      for (int part = 0; part < 2; ++part) {
        R* p = reinterpret_cast<R*>(adam.p[part]) + base;
        R* m = reinterpret_cast<R*>(adam.m[part]) + base;
        R* v = reinterpret_cast<R*>(adam.v[part]) + base;
        R* gout = adam.grad[part] ? reinterpret_cast<R*>(adam.grad[part]) + base : nullptr;
        const float* sc = adam.scale[part] ? adam.scale[part] + base : nullptr;
#pragma unroll
        for (int jj = 0; jj < NJ; ++jj)
          if (jj < nj) {
            const R gr = fac * (part ? acc[q][jj].y : acc[q][jj].x);
            if (gout) gout[jj] = gr;
            R mi = m[jj], vi = v[jj];
            R d = adam_one<R>(gr, mi, vi, lr, b1, b2, c1, c2, eps);
            if (sc) d *= (R)sc[jj];
            m[jj] = mi;
            v[jj] = vi;
            p[jj] += d;
          }
      }
    }
  }
}

template <typename R, int NJ>
static size_t rg_smem(int nb, bool two) {
  return (size_t)(two ? 2 : 1) * ((nb + 3) & ~3) * NJ * sizeof(C_t<R>);
}

template <typename R, int LX0, int OUT, int NJ, int TG, int MINB>
static int rg_go(const void* X0a, const void* X0b, const double2* M0, const void* X1, const double2* M1,
                 void* out0, void* out1, int nsk, int ng, int nb, double fac, const AdamArgs& adam,
                 const double* tk, int nk, void* kin_part, int sk0, int tri0, cudaStream_t st) {
  const size_t sm = rg_smem<R, NJ>(nb, X1 != nullptr);
  const bool vin = LX0 == RG_SPLIT && nb % 4 == 0 && sizeof(R) == 4;
  const bool vout = (OUT == RG_GMAJOR_SPLIT || OUT == RG_ADAM) && nb % 4 == 0 && NJ % 4 == 0 && sizeof(R) == 4;
  auto go = [&](auto kern) -> int {
    if (sm > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(k_rotate_g)");
    }
    const dim3 grid((nb + NJ - 1) / NJ, (ng + kRgThreads * TG - 1) / (kRgThreads * TG), nsk);
    kern<<<grid, kRgThreads, sm, st>>>(X0a, X0b, M0, X1, M1, out0, out1, ng, nb, (R)fac, adam, tk, nk,
                                       reinterpret_cast<R*>(kin_part), sk0, tri0);
    JRG_LAUNCH_CHECK("k_rotate_g");
    return JRG_OK;
  };
  if constexpr (LX0 == RG_SPLIT && sizeof(R) == 4) {
    if (vin) return go(k_rotate_g<R, LX0, OUT, NJ, TG, true, false, MINB>);
    return go(k_rotate_g<R, LX0, OUT, NJ, TG, false, false, MINB>);
  } else if constexpr ((OUT == RG_GMAJOR_SPLIT || OUT == RG_ADAM) && sizeof(R) == 4 && NJ % 4 == 0) {
    if (vout) return go(k_rotate_g<R, LX0, OUT, NJ, TG, false, true, MINB>);
    return go(k_rotate_g<R, LX0, OUT, NJ, TG, false, false, MINB>);
  } else {
    return go(k_rotate_g<R, LX0, OUT, NJ, TG, false, false, MINB>);
  }
}

// Tile shapes: the band count rounded up to 8, at most 32 (FP32) or 16
// (FP64) columns per tile, one G vector per thread (two G vectors per thread
// with 8- or 12-column tiles measured within 1 % at 24 bands and slower at
// 160 bands, where more tiles re-read X; 16-column tiles at three CTAs per
// SM slower at 24 bands).
template <typename R, int LX0, int OUT>
static int rg_pick(const void* X0a, const void* X0b, const double2* M0, const void* X1, const double2* M1,
                   void* out0, void* out1, int nsk, int ng, int nb, double fac, const AdamArgs& adam,
                   const double* tk, int nk, void* kin_part, int sk0, int tri0, cudaStream_t st) {
#define RG_ARGS X0a, X0b, M0, X1, M1, out0, out1, nsk, ng, nb, fac, adam, tk, nk, kin_part, sk0, tri0, st
  // the forward rotation (one term, triangular) is latency-bound: 8-column
  // tiles at four CTAs per SM (0.083 -> 0.067 ms at 24 bands); the two-term
  // adjoint keeps one tile
  if (sizeof(R) == 4 && OUT == RG_BANDMAJOR && nb <= 32) return rg_go<R, LX0, OUT, 8, 1, 4>(RG_ARGS);
  if (nb <= 8) return rg_go<R, LX0, OUT, 8, 1, 2>(RG_ARGS);
  if (sizeof(R) == 8 || nb <= 16) return rg_go<R, LX0, OUT, 16, 1, 2>(RG_ARGS);
  if (nb <= 24) return rg_go<R, LX0, OUT, 24, 1, 2>(RG_ARGS);
  return rg_go<R, LX0, OUT, 32, 1, 2>(RG_ARGS);
#undef RG_ARGS
}

// out_kind RG_*; lx0 RG_SPLIT (X0a = re, X0b = im, parameter layout) or
// RG_BAND (X0a complex band-major); X1 band-major or null; tri0 the zero
// pattern of M0.  kin_part (band-major output only): per-block kinetic
// partials [nsk][ceil(ng / 256)][nb] with the kinetic table of k-point
// (sk0 + sk) % nk.
template <typename R>
int launch_rotate_g(int out_kind, int lx0, const void* X0a, const void* X0b, const double2* M0, const void* X1,
                    const double2* M1, void* out0, void* out1, int nsk, int ng, int nb, double fac,
                    const AdamArgs& adam, const double* tk, int nk, void* kin_part, int sk0, int tri0,
                    cudaStream_t st) {
#define RG_ARGS X0a, X0b, M0, X1, M1, out0, out1, nsk, ng, nb, fac, adam, tk, nk, kin_part, sk0, tri0, st
  if (lx0 == RG_SPLIT) {
    switch (out_kind) {
      case RG_BANDMAJOR: return rg_pick<R, RG_SPLIT, RG_BANDMAJOR>(RG_ARGS);
      case RG_GMAJOR_C: return rg_pick<R, RG_SPLIT, RG_GMAJOR_C>(RG_ARGS);
      case RG_GMAJOR_SPLIT: return rg_pick<R, RG_SPLIT, RG_GMAJOR_SPLIT>(RG_ARGS);
      default: return fail(JRG_ERR_INVALID, "launch_rotate_g: Adam output needs band-major inputs");
    }
  }
  switch (out_kind) {
    case RG_BANDMAJOR: return rg_pick<R, RG_BAND, RG_BANDMAJOR>(RG_ARGS);
    case RG_GMAJOR_C: return rg_pick<R, RG_BAND, RG_GMAJOR_C>(RG_ARGS);
    case RG_GMAJOR_SPLIT: return rg_pick<R, RG_BAND, RG_GMAJOR_SPLIT>(RG_ARGS);
    default: return rg_pick<R, RG_BAND, RG_ADAM>(RG_ARGS);
  }
#undef RG_ARGS
}

template int launch_rotate_g<float>(int, int, const void*, const void*, const double2*, const void*,
                                    const double2*, void*, void*, int, int, int, double, const AdamArgs&,
                                    const double*, int, void*, int, int, cudaStream_t);
template int launch_rotate_g<double>(int, int, const void*, const void*, const double2*, const void*,
                                     const double2*, void*, void*, int, int, int, double, const AdamArgs&,
                                     const double*, int, void*, int, int, cudaStream_t);

}  // namespace jrg
