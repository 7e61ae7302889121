// Nonlocal (beta-projector) term of the norm-conserving pseudopotential
// energy (jrystal/pseudopotential/nloc.py:143-157, 238-248):
//
//   F[s,k,b,j] = sum_G c[s,k,b,G] P[k,j,G]          (c not conjugated)
//   E_nl       = sum_{s,k,b} f[s,k,b] / vol sum_j |F[s,k,b,j]|^2
//   dE_nl / d conj(c[s,k,b,G]) = f[s,k,b] / vol sum_j F[s,k,b,j] conj(P[k,j,G])
//
// P is the projector table on the plane-wave sphere ([K][J][G] complex, the
// rows of potential_nonlocal_psi_reciprocal that are not identically zero).
// Three kernels: G-split partial contractions (cp.async double-buffered
// tiles; two-level sums in the plan's precision, 32-G chunk sums added into a
// running sum, written out in FP64),
// an FP64 reduction over the splits that also forms the energy and the
// weighted F, and the gradient application, one thread per G and four bands
// per pass, that adds F conj(P) into the sphere gradient in place.
#include <algorithm>

#include "plan.h"

namespace jrg {

namespace {
constexpr int kBT = 32;    // largest band tile of the projection
constexpr int kJT = 32;    // largest projector tile of the projection
constexpr int kMinG = 256;   // fewest sphere points per projection split
template <typename R> __host__ __device__ constexpr int tg_of() { return sizeof(R) == 4 ? 32 : 16; }
template <typename R> __host__ __device__ constexpr int jc_of() { return sizeof(R) == 4 ? 32 : 16; }
constexpr int kReduceThreads = 128;   // F entries per reduction CTA
}  // namespace

int nl_chunks(int nb, int np) { return (nb * np + kReduceThreads - 1) / kReduceThreads; }

// grid (splits, nsk, btiles * jtiles), tbn * tjn threads (at most 256): thread
// (tb, tj) owns the 2 x 2 pairs b = b0 + tb + tbn i, j = j0 + tj + tjn q of a
// (2 tbn) x (2 tjn) block tile, so the tile matches nb x np up to rounding to
// even sizes (24 bands x 32 projectors: 12 x 16 threads, no padding).
template <typename R>
__global__ void __launch_bounds__(256) k_nl_project(const C_t<R>* __restrict__ c,
                                                    const C_t<R>* __restrict__ proj,
                                                    double2* __restrict__ part, int k_begin, int nk,
                                                    int ng, int nb, int np, int gper, int splits,
                                                    int jtiles, int tbn, int tjn) {
  using C = C_t<R>;
  constexpr int TG = tg_of<R>();
  __shared__ __align__(16) C cs[2][TG][kBT + 1];
  __shared__ __align__(16) C ps[2][TG][kJT + 1];
  const int split = blockIdx.x, sk = blockIdx.y;
  const int bt = 2 * tbn, jt = 2 * tjn;
  const int b0 = (blockIdx.z / jtiles) * bt, j0 = (blockIdx.z % jtiles) * jt;
  const int k = (k_begin + sk) % nk;
  const int nthr = tbn * tjn;
  const int tid = threadIdx.x, tb = tid / tjn, tj = tid % tjn;
  const bool active = tid < nthr;
  const C* cb = c + (size_t)sk * nb * ng;
  const C* pb = proj + (size_t)k * np * ng;
  const int g_lo = split * gper;
  const int g_hi = min(ng, g_lo + gper);
  C tot[2][2];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int q = 0; q < 2; ++q) tot[i][q] = czero<C>();
  // double-buffered staging: the copies of chunk it+1 run under the math of chunk it
  auto stage = [&](int buf, int gc0) {
    for (int e = tid; e < TG * bt; e += blockDim.x) {
      const int gg = e % TG, bb = e / TG;
      const int g = gc0 + gg, b = b0 + bb;
      const bool ok = g < g_hi && b < nb;
      cp_async_zfill<sizeof(C)>(&cs[buf][gg][bb], ok ? cb + (size_t)b * ng + g : cb, ok);
    }
    for (int e = tid; e < TG * jt; e += blockDim.x) {
      const int gg = e % TG, jj = e / TG;
      const int g = gc0 + gg, j = j0 + jj;
      const bool ok = g < g_hi && j < np;
      cp_async_zfill<sizeof(C)>(&ps[buf][gg][jj], ok ? pb + (size_t)j * ng + g : pb, ok);
    }
    cp_async_commit();
  };
  if (g_lo < g_hi) stage(0, g_lo);
  int it = 0;
  for (int gc0 = g_lo; gc0 < g_hi; gc0 += TG, ++it) {
    const int buf = it & 1;
    if (gc0 + TG < g_hi) {
      stage(buf ^ 1, gc0 + TG);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    if (active) {
      C acc[2][2];
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int q = 0; q < 2; ++q) acc[i][q] = czero<C>();
#pragma unroll 8
      for (int gg = 0; gg < TG; ++gg) {
        const C cv[2] = {cs[buf][gg][tb], cs[buf][gg][tb + tbn]};
        const C pv[2] = {ps[buf][gg][tj], ps[buf][gg][tj + tjn]};
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
          for (int q = 0; q < 2; ++q) {
            acc[i][q].x = fma(cv[i].x, pv[q].x, fma(-cv[i].y, pv[q].y, acc[i][q].x));
            acc[i][q].y = fma(cv[i].x, pv[q].y, fma(cv[i].y, pv[q].x, acc[i][q].y));
          }
      }
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int q = 0; q < 2; ++q) tot[i][q] = cadd(tot[i][q], acc[i][q]);
    }
    __syncthreads();   // buf is restaged two chunks later
  }
  if (!active) return;
  double2* out = part + ((size_t)sk * splits + split) * nb * np;
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int b = b0 + tb + tbn * i, j = j0 + tj + tjn * q;
      if (b < nb && j < np) out[(size_t)b * np + j] = make_double2(tot[i][q].x, tot[i][q].y);
    }
}

// grid (nl_chunks, nsk), 128 threads, one F entry each: F = sum over the
// splits (FP64, in split order), fw = wg / vol * F, and the energy partial
// slot[sk * nl_chunks + chunk] = sum over the CTA's entries of occ_b / vol |F_bj|^2
__global__ void __launch_bounds__(kReduceThreads) k_nl_reduce(const double2* __restrict__ part,
                                                              double2* __restrict__ fw,
                                                              const double* __restrict__ occ,
                                                              const double* __restrict__ wg,
                                                              double* __restrict__ slot, int nb,
                                                              int np, int splits, double inv_vol) {
  __shared__ double red[32];
  const int sk = blockIdx.y;
  const size_t m = (size_t)nb * np;
  const size_t i = (size_t)blockIdx.x * kReduceThreads + threadIdx.x;
  double e = 0.0;
  if (i < m) {
    const double2* pp = part + (size_t)sk * splits * m + i;
    double2 f = make_double2(0.0, 0.0);
    int s = 0;
    for (; s + 8 <= splits; s += 8) {    // eight loads in flight, summed in order
      double2 v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) v[u] = pp[(size_t)(s + u) * m];
#pragma unroll
      for (int u = 0; u < 8; ++u) { f.x += v[u].x; f.y += v[u].y; }
    }
    for (; s < splits; ++s) {
      const double2 v = pp[(size_t)s * m];
      f.x += v.x;
      f.y += v.y;
    }
    const int b = (int)(i / np);
    e = occ[(size_t)sk * nb + b] * (f.x * f.x + f.y * f.y);
    const double w = wg[(size_t)sk * nb + b] * inv_vol;
    fw[(size_t)sk * m + i] = make_double2(w * f.x, w * f.y);
  }
  e = block_sum(e, red);
  if (threadIdx.x == 0) slot[(size_t)sk * gridDim.x + blockIdx.x] = e * inv_vol;
}

// grid (ceil(ng / 128), nsk), 128 threads, one G each, four bands per pass:
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
      for (int bb = 0; bb < nbb; bb += 4) {
        C acc[4];
        C* o[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          acc[i] = czero<C>();
          o[i] = out + (size_t)(b0 + bb + i) * ng + g;
        }
        C old[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) old[i] = (valid && bb + i < nbb) ? *o[i] : czero<C>();
#pragma unroll
        for (int q = 0; q < JC; ++q)
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            // fs (zero past nb) times conj(pv)
            const C a = fs[bb + i][q];
            acc[i].x = fma(a.x, pv[q].x, fma(a.y, pv[q].y, acc[i].x));
            acc[i].y = fma(a.y, pv[q].x, fma(-a.x, pv[q].y, acc[i].y));
          }
#pragma unroll
        for (int i = 0; i < 4; ++i)
          if (valid && bb + i < nbb) *o[i] = cadd(old[i], acc[i]);
      }
    }
  }
}

// thread grid of the projection: 2 x 2 pairs per thread, at most 16 x 16
static void nl_shape(int nb, int np, int* tbn, int* tjn) {
  *tjn = std::min(kJT / 2, (np + 1) / 2);
  *tbn = std::min(std::min(kBT / 2, 256 / *tjn), (nb + 1) / 2);
}

// G splits of the projection: about eight CTAs per SM over all (s,k) blocks
// and tiles, at least kMinG sphere points per split
int nl_splits(int ng, int nsk, int nb, int np) {
  int tbn, tjn;
  nl_shape(nb, np, &tbn, &tjn);
  const int tiles = ((nb + 2 * tbn - 1) / (2 * tbn)) * ((np + 2 * tjn - 1) / (2 * tjn));
  int sp = (8 * 152 + nsk * tiles - 1) / (nsk * tiles);
  sp = std::max(1, std::min(sp, (ng + kMinG - 1) / kMinG));
  const int gper = ((ng + sp - 1) / sp + 31) / 32 * 32;
  return (ng + gper - 1) / gper;
}

static int nl_gper(int ng, int splits) { return ((ng + splits - 1) / splits + 31) / 32 * 32; }

template <typename R>
int launch_nl_project(const void* c, const void* proj, double2* part, int k_begin, int nsk, int nk,
                      int ng, int nb, int np, int splits, cudaStream_t st) {
  if (nsk <= 0 || np <= 0) return JRG_OK;
  const int gper = nl_gper(ng, splits);
  int tbn, tjn;
  nl_shape(nb, np, &tbn, &tjn);
  const int jtiles = (np + 2 * tjn - 1) / (2 * tjn), btiles = (nb + 2 * tbn - 1) / (2 * tbn);
  const int threads = (tbn * tjn + 31) / 32 * 32;
  dim3 grid(splits, nsk, btiles * jtiles);
  k_nl_project<R><<<grid, threads, 0, st>>>(reinterpret_cast<const C_t<R>*>(c),
                                            reinterpret_cast<const C_t<R>*>(proj), part, k_begin,
                                            nk, ng, nb, np, gper, splits, jtiles, tbn, tjn);
  JRG_LAUNCH_CHECK("k_nl_project");
  return JRG_OK;
}

int launch_nl_reduce(const double2* part, double2* fw, const double* occ, const double* wg,
                     double* slot, int nsk, int nb, int np, int splits, double inv_vol,
                     cudaStream_t st) {
  if (nsk <= 0 || np <= 0) return JRG_OK;
  dim3 grid(nl_chunks(nb, np), nsk);
  k_nl_reduce<<<grid, kReduceThreads, 0, st>>>(part, fw, occ, wg, slot, nb, np, splits, inv_vol);
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
