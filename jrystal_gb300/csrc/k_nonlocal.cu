// Nonlocal (beta-projector) term of the norm-conserving pseudopotential
// energy (jrystal/pseudopotential/nloc.py:143-157, 238-248):
//
//   F[s,k,b,j] = sum_G c[s,k,b,G] P[k,j,G]          (c not conjugated)
//   E_nl       = sum_{s,k,b} f[s,k,b] / vol sum_j |F[s,k,b,j]|^2
//   dE_nl / d conj(c[s,k,b,G]) = f[s,k,b] / vol sum_j F[s,k,b,j] conj(P[k,j,G])
//
// P is the projector table on the plane-wave sphere ([K][J][G] complex, the
// rows of potential_nonlocal_psi_reciprocal that are not identically zero).
// Three kernels: G-split partial contractions (FP32 products flushed to FP64
// every 128 G for the FP32 plans), an FP64 reduction over the splits that
// also forms the energy and the weighted F, and the gradient application,
// one thread per G, that adds F conj(P) into the sphere gradient in place.
#include <algorithm>

#include "plan.h"

namespace jrg {

namespace {
constexpr int kBT = 64;    // bands per projection tile
constexpr int kJT = 64;    // projectors per projection tile
constexpr int kFlushG = 128;
template <typename R> __host__ __device__ constexpr int tg_of() { return sizeof(R) == 4 ? 32 : 16; }
template <typename R> __host__ __device__ constexpr int jc_of() { return sizeof(R) == 4 ? 32 : 16; }
}  // namespace

// grid (splits, nsk, btiles * jtiles), 256 threads.  Thread (tb, tj) owns the
// 4 x 4 pairs b = b0 + tb + 16 i, j = j0 + tj + 16 q.
template <typename R>
__global__ void __launch_bounds__(256) k_nl_project(const C_t<R>* __restrict__ c,
                                                    const C_t<R>* __restrict__ proj,
                                                    double2* __restrict__ part, int k_begin, int nk,
                                                    int ng, int nb, int np, int gper, int splits,
                                                    int jtiles) {
  using C = C_t<R>;
  constexpr int TG = tg_of<R>();
  __shared__ C cs[TG][kBT + 1];
  __shared__ C ps[TG][kJT + 1];
  const int split = blockIdx.x, sk = blockIdx.y;
  const int b0 = (blockIdx.z / jtiles) * kBT, j0 = (blockIdx.z % jtiles) * kJT;
  const int k = (k_begin + sk) % nk;
  const int tid = threadIdx.x, tb = tid >> 4, tj = tid & 15;
  const C* cb = c + (size_t)sk * nb * ng;
  const C* pb = proj + (size_t)k * np * ng;
  const int g_lo = split * gper;
  const int g_hi = min(ng, g_lo + gper);
  C acc[4][4];
  double2 dacc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int q = 0; q < 4; ++q) { acc[i][q] = czero<C>(); dacc[i][q] = make_double2(0.0, 0.0); }
  int since_flush = 0;
  for (int gc0 = g_lo; gc0 < g_hi; gc0 += TG) {
    __syncthreads();
    for (int e = tid; e < TG * kBT; e += 256) {
      const int gg = e % TG, bb = e / TG;
      const int g = gc0 + gg, b = b0 + bb;
      cs[gg][bb] = (g < g_hi && b < nb) ? cb[(size_t)b * ng + g] : czero<C>();
    }
    for (int e = tid; e < TG * kJT; e += 256) {
      const int gg = e % TG, jj = e / TG;
      const int g = gc0 + gg, j = j0 + jj;
      ps[gg][jj] = (g < g_hi && j < np) ? pb[(size_t)j * ng + g] : czero<C>();
    }
    __syncthreads();
#pragma unroll 4
    for (int gg = 0; gg < TG; ++gg) {
      C cv[4], pv[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) cv[i] = cs[gg][tb + 16 * i];
#pragma unroll
      for (int q = 0; q < 4; ++q) pv[q] = ps[gg][tj + 16 * q];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          acc[i][q].x = fma(cv[i].x, pv[q].x, fma(-cv[i].y, pv[q].y, acc[i][q].x));
          acc[i][q].y = fma(cv[i].x, pv[q].y, fma(cv[i].y, pv[q].x, acc[i][q].y));
        }
    }
    since_flush += TG;
    if (since_flush >= kFlushG) {
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          dacc[i][q].x += (double)acc[i][q].x;
          dacc[i][q].y += (double)acc[i][q].y;
          acc[i][q] = czero<C>();
        }
      since_flush = 0;
    }
  }
  double2* out = part + ((size_t)sk * splits + split) * nb * np;
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int b = b0 + tb + 16 * i, j = j0 + tj + 16 * q;
      if (b < nb && j < np)
        out[(size_t)b * np + j] = make_double2(dacc[i][q].x + (double)acc[i][q].x,
                                               dacc[i][q].y + (double)acc[i][q].y);
    }
}

// grid nsk, 256 threads: F = sum over splits (FP64), fw = wg / vol * F,
// slot[sk] = sum_b occ_b / vol sum_j |F_bj|^2
__global__ void __launch_bounds__(256) k_nl_reduce(const double2* __restrict__ part,
                                                   double2* __restrict__ fw,
                                                   const double* __restrict__ occ,
                                                   const double* __restrict__ wg,
                                                   double* __restrict__ slot, int nb, int np,
                                                   int splits, double inv_vol) {
  __shared__ double red[32];
  const int sk = blockIdx.x;
  const size_t m = (size_t)nb * np;
  const double2* pp = part + (size_t)sk * splits * m;
  double e = 0.0;
  for (size_t i = threadIdx.x; i < m; i += blockDim.x) {
    double2 f = make_double2(0.0, 0.0);
    for (int s = 0; s < splits; ++s) {
      const double2 v = pp[(size_t)s * m + i];
      f.x += v.x;
      f.y += v.y;
    }
    const int b = (int)(i / np);
    const double a2 = f.x * f.x + f.y * f.y;
    e += occ[(size_t)sk * nb + b] * a2;
    const double w = wg[(size_t)sk * nb + b] * inv_vol;
    fw[(size_t)sk * m + i] = make_double2(w * f.x, w * f.y);
  }
  e = block_sum(e, red);
  if (threadIdx.x == 0) slot[sk] = e * inv_vol;
}

// grid (ceil(ng / 128), nsk), 128 threads, one G each:
// gc[sk][b][G] += sum_j fw[sk][b][j] conj(P[k][j][G])
template <typename R>
__global__ void __launch_bounds__(128) k_nl_apply(C_t<R>* __restrict__ gc,
                                                  const C_t<R>* __restrict__ proj,
                                                  const double2* __restrict__ fw, int k_begin,
                                                  int nk, int ng, int nb, int np) {
  using C = C_t<R>;
  constexpr int JC = jc_of<R>();
  constexpr int BT = 64;
  __shared__ C fs[BT][JC];
  const int sk = blockIdx.y;
  const int k = (k_begin + sk) % nk;
  const int g = blockIdx.x * 128 + threadIdx.x;
  const bool valid = g < ng;
  const C* pb = proj + (size_t)k * np * ng;
  const double2* f = fw + (size_t)sk * nb * np;
  C* out = gc + (size_t)sk * nb * ng;
  for (int j0 = 0; j0 < np; j0 += JC) {
    C pv[JC];
#pragma unroll
    for (int q = 0; q < JC; ++q)
      pv[q] = (valid && j0 + q < np) ? pb[(size_t)(j0 + q) * ng + g] : czero<C>();
    for (int b0 = 0; b0 < nb; b0 += BT) {
      __syncthreads();
      for (int e = threadIdx.x; e < BT * JC; e += 128) {
        const int bb = e / JC, q = e % JC;
        const int b = b0 + bb, j = j0 + q;
        const double2 v = (b < nb && j < np) ? f[(size_t)b * np + j] : make_double2(0.0, 0.0);
        fs[bb][q] = cmk<C>(v.x, v.y);
      }
      __syncthreads();
      const int nbb = min(BT, nb - b0);
      for (int bb = 0; bb < nbb; ++bb) {
        C acc = czero<C>();
#pragma unroll
        for (int q = 0; q < JC; ++q) acc = cadd(acc, cmulc(fs[bb][q], pv[q]));
        if (valid) {
          C* o = out + (size_t)(b0 + bb) * ng + g;
          *o = cadd(*o, acc);
        }
      }
    }
  }
}

int nl_splits(int ng, int nsk, int nb, int np) {
  const int tiles = ((nb + kBT - 1) / kBT) * ((np + kJT - 1) / kJT);
  int sp = (4 * 152 + nsk * tiles - 1) / (nsk * tiles);
  sp = std::max(1, std::min(sp, (ng + kFlushG - 1) / kFlushG));
  // G per split: a multiple of the flush interval
  const int gper = ((ng + sp - 1) / sp + kFlushG - 1) / kFlushG * kFlushG;
  return (ng + gper - 1) / gper;
}

static int nl_gper(int ng, int splits) {
  return ((ng + splits - 1) / splits + kFlushG - 1) / kFlushG * kFlushG;
}

template <typename R>
int launch_nl_project(const void* c, const void* proj, double2* part, int k_begin, int nsk, int nk,
                      int ng, int nb, int np, int splits, cudaStream_t st) {
  if (nsk <= 0 || np <= 0) return JRG_OK;
  const int gper = nl_gper(ng, splits);
  const int jtiles = (np + kJT - 1) / kJT, btiles = (nb + kBT - 1) / kBT;
  dim3 grid(splits, nsk, btiles * jtiles);
  k_nl_project<R><<<grid, 256, 0, st>>>(reinterpret_cast<const C_t<R>*>(c),
                                        reinterpret_cast<const C_t<R>*>(proj), part, k_begin, nk, ng,
                                        nb, np, gper, splits, jtiles);
  JRG_LAUNCH_CHECK("k_nl_project");
  return JRG_OK;
}

int launch_nl_reduce(const double2* part, double2* fw, const double* occ, const double* wg,
                     double* slot, int nsk, int nb, int np, int splits, double inv_vol,
                     cudaStream_t st) {
  if (nsk <= 0 || np <= 0) return JRG_OK;
  k_nl_reduce<<<nsk, 256, 0, st>>>(part, fw, occ, wg, slot, nb, np, splits, inv_vol);
  JRG_LAUNCH_CHECK("k_nl_reduce");
  return JRG_OK;
}

template <typename R>
int launch_nl_apply(void* gc, const void* proj, const double2* fw, int k_begin, int nsk, int nk,
                    int ng, int nb, int np, cudaStream_t st) {
  if (nsk <= 0 || np <= 0) return JRG_OK;
  dim3 grid((ng + 127) / 128, nsk);
  k_nl_apply<R><<<grid, 128, 0, st>>>(reinterpret_cast<C_t<R>*>(gc),
                                      reinterpret_cast<const C_t<R>*>(proj), fw, k_begin, nk, ng,
                                      nb, np);
  JRG_LAUNCH_CHECK("k_nl_apply");
  return JRG_OK;
}

template int launch_nl_project<float>(const void*, const void*, double2*, int, int, int, int, int,
                                      int, int, cudaStream_t);
template int launch_nl_project<double>(const void*, const void*, double2*, int, int, int, int, int,
                                       int, int, cudaStream_t);
template int launch_nl_apply<float>(void*, const void*, const double2*, int, int, int, int, int,
                                    int, cudaStream_t);
template int launch_nl_apply<double>(void*, const void*, const double2*, int, int, int, int, int,
                                     int, cudaStream_t);

}  // namespace jrg
