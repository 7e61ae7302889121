// Gram S = X^H Y of the FP32 path for more than 32 bands.
//
// The B x B output is cut into 32 x 32 tiles and only the tiles on or above
// the diagonal are formed: W^H W is Hermitian, and the adjoint's C^H g_C is
// only read on and above its diagonal (the Hermitian completion of its upper
// triangle).  The reduction over the splits fills the lower tiles with the
// conjugate transpose.  One CTA (64 threads) owns one tile of one (s,k) over
// one G range: chunks of 16 G vectors of the tile's 32 X bands and 32 Y bands
// are loaded into registers (16-byte loads of the parameter layout, coalesced
// loads of the band-major layout) while the previous chunk is used from
// shared memory, and each thread accumulates a 4 x 4 block of the tile (rows
// 4ty .. 4ty+3, broadcast to eight lanes; columns tx + 8b, consecutive
// across them: six shared-memory loads per sixteen complex multiply-adds).
// Small tiles keep the padding of the last band tile and the imbalance of
// the last wave small (about ten waves of five CTAs per SM at 160 bands).
// Each chunk's FP32 sums are added into Kahan-compensated FP32 running sums
// (FP64 arithmetic runs at 1/64 of the FP32 rate), and the tile is written
// to its split's FP64 partial.
#include "plan.h"

namespace jrg {

constexpr int kGbT = 32;          // tile edge (bands)
constexpr int kGbQ = kGbT / 4;    // 4 x 4 blocks per tile edge
constexpr int kGbCH = 16;         // G vectors per chunk
constexpr int kGbS = kGbT + 2;    // shared-memory row stride (complex; even: 16-byte aligned pairs)
constexpr int kGbThreads = kGbQ * kGbQ;
// staging: per thread per operand and chunk, kGbSplitPer quads of 4 bands of
// one G vector (parameter layout) or kGbBandPer single elements (band-major)
constexpr int kGbSplitPer = kGbCH * (kGbT / 4) / kGbThreads;
constexpr int kGbBandPer = kGbCH * kGbT / kGbThreads;
static_assert(kGbSplitPer * kGbThreads == kGbCH * (kGbT / 4) && kGbSplitPer >= 1, "split staging map");
static_assert(kGbBandPer * kGbThreads == kGbCH * kGbT && kGbCH == 16, "band staging map");

enum { GB_SPLIT = 0, GB_BAND = 1 };

// tile pair p (row tile <= column tile) of nt tiles
__device__ __forceinline__ void gb_pair(int p, int nt, int& ti, int& tj) {
  ti = 0;
  while (p >= nt - ti) { p -= nt - ti; ++ti; }
  tj = ti + p;
}

// one operand's chunk in registers
template <int LX>
struct GbRegs;
template <>
struct GbRegs<GB_SPLIT> { float4 re[kGbSplitPer], im[kGbSplitPer]; };
template <>
struct GbRegs<GB_BAND> {};   // band-major chunks go straight to shared memory (cp.async)

// parameter layout: the chunk into registers; band-major: cp.async of the
// chunk into the shared-memory buffer s (zero-filled outside the ranges)
template <int LX, bool VEC>
__device__ __forceinline__ void gb_load(GbRegs<LX>& r, const void* __restrict__ p0, const void* __restrict__ p1,
                                        size_t sk, int b0, int g0, int g_end, int ng, int nb,
                                        float2* __restrict__ s) {
  const int t = threadIdx.x;
  if constexpr (LX == GB_SPLIT) {
#pragma unroll
    for (int h = 0; h < kGbSplitPer; ++h) {
      const int e = t + h * kGbThreads;   // (G vector q < kGbCH, band quad c4 < kGbQ)
      const int q = e / kGbQ, c4 = e % kGbQ;
      const int g = g0 + q, b = b0 + 4 * c4;
      float4 re = make_float4(0.f, 0.f, 0.f, 0.f), im = re;
      if (g < g_end) {
        const size_t o = (sk * ng + g) * nb + b;
        const float* a = reinterpret_cast<const float*>(p0) + o;
        const float* c = reinterpret_cast<const float*>(p1) + o;
        if (VEC) {   // nb % 4 == 0: the quad is inside the row or entirely past nb
          if (b < nb) { re = __ldg(reinterpret_cast<const float4*>(a)); im = __ldg(reinterpret_cast<const float4*>(c)); }
        } else {
          if (b + 0 < nb) { re.x = __ldg(a + 0); im.x = __ldg(c + 0); }
          if (b + 1 < nb) { re.y = __ldg(a + 1); im.y = __ldg(c + 1); }
          if (b + 2 < nb) { re.z = __ldg(a + 2); im.z = __ldg(c + 2); }
          if (b + 3 < nb) { re.w = __ldg(a + 3); im.w = __ldg(c + 3); }
        }
      }
      r.re[h] = re;
      r.im[h] = im;
    }
  } else {
#pragma unroll
    for (int h = 0; h < kGbBandPer; ++h) {
      const int e = t + h * kGbThreads;   // (band bl < kGbT, G vector q < kGbCH), q fastest
      const int q = e & (kGbCH - 1), bl = e >> 4;
      const int g = g0 + q, b = b0 + bl;
      const bool in = g < g_end && b < nb;
      const float2* src = reinterpret_cast<const float2*>(p0) + (in ? (sk * nb + b) * ng + g : 0);
      cp_async_zfill<8>(s + q * kGbS + bl, src, in);
    }
    cp_async_commit();
  }
}

template <int LX>
__device__ __forceinline__ void gb_store(const GbRegs<LX>& r, float2* __restrict__ s) {
  const int t = threadIdx.x;
  if constexpr (LX == GB_SPLIT) {
#pragma unroll
    for (int h = 0; h < kGbSplitPer; ++h) {
      const int e = t + h * kGbThreads;
      const int q = e / kGbQ, c4 = e % kGbQ;
      float4* d = reinterpret_cast<float4*>(s + q * kGbS + 4 * c4);
      d[0] = make_float4(r.re[h].x, r.im[h].x, r.re[h].y, r.im[h].y);
      d[1] = make_float4(r.re[h].z, r.im[h].z, r.re[h].w, r.im[h].w);
    }
  } else {
    cp_async_wait<0>();   // this thread's copies; the caller's barrier publishes them
  }
}

// SAME: Y is X (W^H W); a diagonal tile then stages one operand.
template <int LX, bool SAME, bool VEC>
__global__ void __launch_bounds__(kGbThreads, 4)
k_gram_big(const void* __restrict__ X0, const void* __restrict__ X1, const void* __restrict__ Y0,
           const void* __restrict__ Y1, double2* __restrict__ part, int ng, int nb, int split_len) {
  __shared__ __align__(16) float2 xs[2][kGbCH * kGbS];
  __shared__ __align__(16) float2 ys[2][kGbCH * kGbS];
  const int nt = (nb + kGbT - 1) / kGbT;
  int ti, tj;
  gb_pair(blockIdx.y, nt, ti, tj);
  const bool diag = SAME && ti == tj;
  const size_t sk = blockIdx.z;
  const int split = blockIdx.x, nsplit = gridDim.x;
  const int g_begin = split * split_len;
  const int g_end = min(ng, g_begin + split_len);
  const int nchunk = g_end > g_begin ? (g_end - g_begin + kGbCH - 1) / kGbCH : 0;
  const int t = threadIdx.x, tx = t % kGbQ, ty = t / kGbQ;
  float2 acc[4][4], sum[4][4], comp[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      acc[a][b] = make_float2(0.f, 0.f);
      sum[a][b] = acc[a][b];
      comp[a][b] = acc[a][b];
    }
  GbRegs<LX> rx, ry;
  if (nchunk > 0) {
    gb_load<LX, VEC>(rx, X0, X1, sk, ti * kGbT, g_begin, g_end, ng, nb, xs[0]);
    if (!diag) gb_load<LX, VEC>(ry, Y0, Y1, sk, tj * kGbT, g_begin, g_end, ng, nb, ys[0]);
    gb_store<LX>(rx, xs[0]);
    if (!diag) gb_store<LX>(ry, ys[0]);
  }
  __syncthreads();
  for (int c = 0; c < nchunk; ++c) {
    const int cur = c & 1;
    if (c + 1 < nchunk) {   // next chunk into registers while this one is used
      const int g0 = g_begin + (c + 1) * kGbCH;
      gb_load<LX, VEC>(rx, X0, X1, sk, ti * kGbT, g0, g_end, ng, nb, xs[cur ^ 1]);
      if (!diag) gb_load<LX, VEC>(ry, Y0, Y1, sk, tj * kGbT, g0, g_end, ng, nb, ys[cur ^ 1]);
    }
    const float2* xb = xs[cur];
    const float2* yb = diag ? xs[cur] : ys[cur];
#pragma unroll 4
    for (int q = 0; q < kGbCH; ++q) {
      float2 x[4], y[4];
      const float4 x01 = *reinterpret_cast<const float4*>(xb + q * kGbS + 4 * ty);
      const float4 x23 = *reinterpret_cast<const float4*>(xb + q * kGbS + 4 * ty + 2);
      x[0] = make_float2(x01.x, x01.y); x[1] = make_float2(x01.z, x01.w);
      x[2] = make_float2(x23.x, x23.y); x[3] = make_float2(x23.z, x23.w);
#pragma unroll
      for (int b = 0; b < 4; ++b) y[b] = yb[q * kGbS + tx + kGbQ * b];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {   // conj(x) * y
          acc[a][b].x = fmaf(x[a].x, y[b].x, fmaf(x[a].y, y[b].y, acc[a][b].x));
          acc[a][b].y = fmaf(x[a].x, y[b].y, fmaf(-x[a].y, y[b].x, acc[a][b].y));
        }
    }
    // the chunk's sums into the compensated running sums
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) {
        float yv = acc[a][b].x - comp[a][b].x;
        float tv = sum[a][b].x + yv;
        comp[a][b].x = (tv - sum[a][b].x) - yv;
        sum[a][b].x = tv;
        yv = acc[a][b].y - comp[a][b].y;
        tv = sum[a][b].y + yv;
        comp[a][b].y = (tv - sum[a][b].y) - yv;
        sum[a][b].y = tv;
        acc[a][b] = make_float2(0.f, 0.f);
      }
    if (c + 1 < nchunk) {
      gb_store<LX>(rx, xs[cur ^ 1]);
      if (!diag) gb_store<LX>(ry, ys[cur ^ 1]);
    }
    __syncthreads();
  }
  double2* out = part + (sk * nsplit + split) * (size_t)nb * nb;
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const int i = ti * kGbT + 4 * ty + a;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int j = tj * kGbT + tx + kGbQ * b;
      if (i < nb && j < nb)
        out[(size_t)i * nb + j] = make_double2((double)sum[a][b].x - (double)comp[a][b].x,
                                               (double)sum[a][b].y - (double)comp[a][b].y);
    }
  }
}

// out[i][j] = sum over the splits for tiles on or above the diagonal; the
// conjugate of the transposed element below it
__global__ void k_gram_reduce_upper(const double2* __restrict__ part, double2* __restrict__ out, int nsplit,
                                    int nb, int nsk) {
  const size_t nn = (size_t)nb * nb, n = (size_t)nsk * nn;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const size_t sk = e / nn, ij = e % nn;
    const int i = (int)(ij / nb), j = (int)(ij % nb);
    const bool lower = i / kGbT > j / kGbT;
    const size_t src = lower ? (size_t)j * nb + i : ij;
    double sx = 0.0, sy = 0.0;
    for (int p = 0; p < nsplit; ++p) {
      const double2 v = part[(sk * nsplit + p) * nn + src];
      sx += v.x;
      sy += v.y;
    }
    out[e] = make_double2(sx, lower ? -sy : sy);
  }
}

// FP32 path, nb > 32: returns JRG_OK, or an error status.  lx == ly.
int launch_gram_big(int lay, const void* X0, const void* X1, const void* Y0, const void* Y1, double2* part,
                    double2* out, int nsk, int ng, int nb, int max_splits, cudaStream_t st) {
  const int nt = (nb + kGbT - 1) / kGbT;
  const int npair = nt * (nt + 1) / 2;
  // about ten waves of four CTAs per SM, at least 1024 G vectors per CTA
  int nsplit = std::max(1, (40 * 152 + nsk * npair - 1) / (nsk * npair));
  nsplit = std::min(nsplit, std::max(1, ng / 1024));
  nsplit = std::min(nsplit, max_splits);
  const int split_len = (ng + nsplit - 1) / nsplit;
  const bool same = X0 == Y0 && X1 == Y1;
  const bool vec = nb % 4 == 0;
  const dim3 grid(nsplit, npair, nsk);
  if (lay == GB_SPLIT) {
    if (same && vec) k_gram_big<GB_SPLIT, true, true><<<grid, kGbThreads, 0, st>>>(X0, X1, Y0, Y1, part, ng, nb, split_len);
    else if (same) k_gram_big<GB_SPLIT, true, false><<<grid, kGbThreads, 0, st>>>(X0, X1, Y0, Y1, part, ng, nb, split_len);
    else if (vec) k_gram_big<GB_SPLIT, false, true><<<grid, kGbThreads, 0, st>>>(X0, X1, Y0, Y1, part, ng, nb, split_len);
    else k_gram_big<GB_SPLIT, false, false><<<grid, kGbThreads, 0, st>>>(X0, X1, Y0, Y1, part, ng, nb, split_len);
  } else {
    if (same) k_gram_big<GB_BAND, true, false><<<grid, kGbThreads, 0, st>>>(X0, X1, Y0, Y1, part, ng, nb, split_len);
    else k_gram_big<GB_BAND, false, false><<<grid, kGbThreads, 0, st>>>(X0, X1, Y0, Y1, part, ng, nb, split_len);
  }
  JRG_LAUNCH_CHECK("k_gram_big");
  const size_t n = (size_t)nsk * nb * nb;
  k_gram_reduce_upper<<<(unsigned)std::min<size_t>((n + 255) / 256, 4096), 256, 0, st>>>(part, out, nsplit, nb, nsk);
  JRG_LAUNCH_CHECK("k_gram_reduce_upper");
  return JRG_OK;
}

}  // namespace jrg
