// Tensor-core Gram and rotation contractions of the FP32 path (nb <= 32).
//
// Complex products are real GEMMs on the real embedding:
//   Gram:     [Xr Xi]^T [Yr Yi] = [[Xr'Yr, Xr'Yi], [Xi'Yr, Xi'Yi]]  (2nb x 2nb),
//             S = X^H Y:  Re S = B00 + B11,  Im S = B01 - B10
//   rotation: [Xr Xi] [[Mr, Mi], [-Mi, Mr]] = [Re(XM) Im(XM)]  (two-term form
//             stacks a second [X M] block along K)
// on mma.sync.m16n8k8 TF32 with FP32 accumulation.  Each FP32 operand is
// split into a TF32 high part and a TF32 low part (x - hi); the three
// products hi*hi + hi*lo + lo*hi keep the FP32 accuracy of the inputs.  Gram
// accumulators are flushed into FP64 every 32-row chunk (as the CUDA-core
// kernel does); rotation sums have at most 4*nb terms and stay in FP32.
#include "plan.h"

namespace jrg {

__device__ __forceinline__ uint32_t to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ void split_tf32(float x, uint32_t& hi, uint32_t& lo) {
  hi = to_tf32(x);
  lo = to_tf32(x - __uint_as_float(hi));
}
__device__ __forceinline__ void mma_tf32(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2,
                                         uint32_t a3, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}
// hi*hi + hi*lo + lo*hi
__device__ __forceinline__ void mma_tf32x3(float (&d)[4], const float (&a)[4], const float (&b)[2]) {
  uint32_t ah[4], al[4], bh[2], bl[2];
#pragma unroll
  for (int i = 0; i < 4; ++i) split_tf32(a[i], ah[i], al[i]);
#pragma unroll
  for (int i = 0; i < 2; ++i) split_tf32(b[i], bh[i], bl[i]);
  mma_tf32(d, al[0], al[1], al[2], al[3], bh[0], bh[1]);
  mma_tf32(d, ah[0], ah[1], ah[2], ah[3], bl[0], bl[1]);
  mma_tf32(d, ah[0], ah[1], ah[2], ah[3], bh[0], bh[1]);
}

constexpr int kTcChunk = 32;      // G rows per Gram chunk
constexpr int kTcMaxNb = 32;

// loads element (g, m) of the real embedding [Re X | Im X] (m < 2nb)
template <int LAYOUT>
__device__ __forceinline__ float embed(const void* __restrict__ p0, const void* __restrict__ p1,
                                       size_t sk, int g, int m, int ng, int nb) {
  const int i = m < nb ? m : m - nb;
  if constexpr (LAYOUT == 0) {   // split re/im arrays [sk][g][b]
    const float* p = reinterpret_cast<const float*>(m < nb ? p0 : p1);
    return p[(sk * ng + g) * nb + i];
  } else {                       // band-major complex [sk][b][g]
    const float2 v = reinterpret_cast<const float2*>(p0)[(sk * nb + i) * ng + g];
    return m < nb ? v.x : v.y;
  }
}

// Loads rows [g0, g0 + rows) of the real embedding [Re X | Im X] into
// shared memory as TF32 hi and lo parts: hi[k][m], lo[k][m] (pitch P); rows
// past g_end and columns past 2nb are zero.
template <int LAYOUT>
__device__ __forceinline__ void load_split_tile(const void* __restrict__ p0, const void* __restrict__ p1,
                                                size_t sk, int g0, int g_end, int rows, int ng, int nb,
                                                int cols_pad, uint32_t* hi, uint32_t* lo, int P) {
  for (int e = threadIdx.x; e < rows * cols_pad; e += blockDim.x) {
    int k, m;
    if constexpr (LAYOUT == 0) { k = e / cols_pad; m = e - k * cols_pad; }   // row-contiguous source
    else { m = e / rows; k = e - m * rows; }                                 // g-contiguous source
    const int g = g0 + k;
    float v = 0.f;
    if (g < g_end && m < 2 * nb) {
      if constexpr (LAYOUT == 0) {
        v = reinterpret_cast<const float*>(m < nb ? p0 : p1)[(sk * ng + g) * nb + (m < nb ? m : m - nb)];
      } else {
        const float* c = reinterpret_cast<const float*>(p0);
        const int i = m < nb ? m : m - nb;
        v = c[2 * ((sk * nb + i) * ng + g) + (m < nb ? 0 : 1)];
      }
    }
    uint32_t h, l;
    split_tf32(v, h, l);
    hi[k * P + m] = h;
    lo[k * P + m] = l;
  }
}

// partial real-embedded Gram over one G split: part[sk][split][MP][MP] (FP64)
template <int LX, int LY>
__global__ void __launch_bounds__(256) k_gram_tc(const void* __restrict__ X0, const void* __restrict__ X1,
                                                 const void* __restrict__ Y0, const void* __restrict__ Y1,
                                                 double* __restrict__ part, int ng, int nb, int MP,
                                                 int split_len, int same) {
  constexpr int PITCH = 2 * kTcMaxNb + 8;   // 72 words: conflict-free fragment loads
  __shared__ uint32_t Ahi[kTcChunk * PITCH], Alo[kTcChunk * PITCH];
  __shared__ uint32_t Bhi[kTcChunk * PITCH], Blo[kTcChunk * PITCH];
  const size_t sk = blockIdx.z;
  const int split = blockIdx.x, nsplit = gridDim.x;
  const int g_begin = split * split_len, g_end = min(ng, g_begin + split_len);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gq = lane >> 2, tig = lane & 3;
  const int mt_n = MP / 16, nt_n = MP / 8, pairs = mt_n * nt_n;
  float acc[4][4];
  double acc64[4][4];
#pragma unroll
  for (int p = 0; p < 4; ++p)
#pragma unroll
    for (int c = 0; c < 4; ++c) { acc[p][c] = 0.f; acc64[p][c] = 0.0; }
  const uint32_t* bh = same ? Ahi : Bhi;
  const uint32_t* bl = same ? Alo : Blo;
  for (int g0 = g_begin; g0 < g_end; g0 += kTcChunk) {
    load_split_tile<LX>(X0, X1, sk, g0, g_end, kTcChunk, ng, nb, MP, Ahi, Alo, PITCH);
    if (!same) load_split_tile<LY>(Y0, Y1, sk, g0, g_end, kTcChunk, ng, nb, MP, Bhi, Blo, PITCH);
    __syncthreads();
#pragma unroll
    for (int p = 0; p < 4; ++p) {
      const int pair = warp + 8 * p;
      if (pair < pairs) {
        const int mt = pair / nt_n, nt = pair % nt_n;
        const int ma = 16 * mt + gq, nbb = 8 * nt + gq;
#pragma unroll
        for (int k8 = 0; k8 < kTcChunk; k8 += 8) {
          const int r0 = (k8 + tig) * PITCH, r1 = (k8 + tig + 4) * PITCH;
          const uint32_t ah0 = Ahi[r0 + ma], ah1 = Ahi[r0 + ma + 8], ah2 = Ahi[r1 + ma], ah3 = Ahi[r1 + ma + 8];
          const uint32_t al0 = Alo[r0 + ma], al1 = Alo[r0 + ma + 8], al2 = Alo[r1 + ma], al3 = Alo[r1 + ma + 8];
          const uint32_t bh0 = bh[r0 + nbb], bh1 = bh[r1 + nbb], bl0 = bl[r0 + nbb], bl1 = bl[r1 + nbb];
          mma_tf32(acc[p], al0, al1, al2, al3, bh0, bh1);
          mma_tf32(acc[p], ah0, ah1, ah2, ah3, bl0, bl1);
          mma_tf32(acc[p], ah0, ah1, ah2, ah3, bh0, bh1);
        }
      }
    }
#pragma unroll
    for (int p = 0; p < 4; ++p)
#pragma unroll
      for (int c = 0; c < 4; ++c) { acc64[p][c] += (double)acc[p][c]; acc[p][c] = 0.f; }
    __syncthreads();
  }
  double* out = part + (sk * nsplit + split) * (size_t)MP * MP;
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    const int pair = warp + 8 * p;
    if (pair < pairs) {
      const int mt = pair / nt_n, nt = pair % nt_n;
      const int r0 = 16 * mt + gq, c0 = 8 * nt + 2 * tig;
      out[(size_t)r0 * MP + c0] = acc64[p][0];
      out[(size_t)r0 * MP + c0 + 1] = acc64[p][1];
      out[(size_t)(r0 + 8) * MP + c0] = acc64[p][2];
      out[(size_t)(r0 + 8) * MP + c0 + 1] = acc64[p][3];
    }
  }
}

// sum over splits and fold the real embedding into the complex Gram
__global__ void k_gram_tc_reduce(const double* __restrict__ part, double2* __restrict__ out,
                                 int nsplit, int nb, int MP, int nsk) {
  const size_t n = (size_t)nsk * nb * nb;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x) {
    const size_t sk = e / ((size_t)nb * nb);
    const int i = (int)(e % ((size_t)nb * nb)) / nb, j = (int)(e % nb);
    double re = 0.0, im = 0.0;
    for (int p = 0; p < nsplit; ++p) {
      const double* b = part + (sk * nsplit + p) * (size_t)MP * MP;
      re += b[(size_t)i * MP + j] + b[(size_t)(i + nb) * MP + j + nb];
      im += b[(size_t)i * MP + j + nb] - b[(size_t)(i + nb) * MP + j];
    }
    out[e] = make_double2(re, im);
  }
}

// The real-embedded [[Mr, Mi], [-Mi, Mr]] blocks of the (one or two) FP64
// [B x B] matrices, split into TF32 hi/lo once per (s,k): bsplit[sk][2][KP][NP].
__global__ void k_rotate_tc_prep(const double2* __restrict__ M0, const double2* __restrict__ M1,
                                 uint32_t* __restrict__ bsplit, int nb, int KP, int NP) {
  const size_t sk = blockIdx.x;
  const int twonb = 2 * nb, nterms = M1 ? 2 : 1;
  uint32_t* hi = bsplit + sk * 2 * (size_t)KP * NP;
  uint32_t* lo = hi + (size_t)KP * NP;
  for (int e = threadIdx.x; e < KP * NP; e += blockDim.x) {
    const int k = e / NP, n = e % NP;
    const int t = k / twonb, kk = k % twonb;
    double v = 0.0;
    if (t < nterms && n < twonb) {
      const double2 m = (t ? M1 : M0)[sk * nb * nb + (size_t)(kk < nb ? kk : kk - nb) * nb +
                                      (n < nb ? n : n - nb)];
      v = kk < nb ? (n < nb ? m.x : m.y) : (n < nb ? -m.y : m.x);
    }
    const float vh = (float)v;
    const uint32_t h = to_tf32(vh);
    hi[e] = h;
    lo[e] = to_tf32((float)(v - (double)__uint_as_float(h)));
  }
}

// rotation: 128 G rows per CTA (16 per warp), K = 2nb*nterms, N = 2nb
template <int OUT, int LX0>
__global__ void __launch_bounds__(256) k_rotate_tc(const void* __restrict__ X0a, const void* __restrict__ X0b,
                                                   const void* __restrict__ X1,
                                                   const uint32_t* __restrict__ bsplit,
                                                   void* __restrict__ out0, void* __restrict__ out1,
                                                   int ng, int nb, int KP, int NP, float fac) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int AP = KP + 4, BP = NP + 8;
  float* As = reinterpret_cast<float*>(smem_raw);              // [128][AP]
  uint32_t* Bh = reinterpret_cast<uint32_t*>(As + 128 * AP);   // [KP][BP]
  uint32_t* Bl = Bh + KP * BP;
  const size_t sk = blockIdx.y;
  const int g0 = blockIdx.x * 128;
  const int nterms = X1 ? 2 : 1;
  const int twonb = 2 * nb;
  {
    const uint32_t* hi = bsplit + sk * 2 * (size_t)KP * NP;
    const uint32_t* lo = hi + (size_t)KP * NP;
    for (int e = threadIdx.x; e < KP * NP; e += blockDim.x) {
      const int k = e / NP, n = e - k * NP;
      Bh[k * BP + n] = hi[e];
      Bl[k * BP + n] = lo[e];
    }
  }
  // A = [Re X0 | Im X0 | Re X1 | Im X1], rows g0..g0+127
  for (int t = 0; t < nterms; ++t) {
    const int kofs = t * twonb;
    for (int e = threadIdx.x; e < 128 * twonb; e += blockDim.x) {
      int r, m;
      if (t == 0 && LX0 == 0) { r = e / twonb; m = e - r * twonb; }
      else { m = e / 128; r = e - m * 128; }
      const int g = g0 + r;
      float v = 0.f;
      if (g < ng) {
        const int i = m < nb ? m : m - nb;
        if (t == 0 && LX0 == 0) {
          v = reinterpret_cast<const float*>(m < nb ? X0a : X0b)[(sk * ng + g) * nb + i];
        } else {
          const float* c = reinterpret_cast<const float*>(t ? X1 : X0a);
          v = c[2 * ((sk * nb + i) * ng + g) + (m < nb ? 0 : 1)];
        }
      }
      As[r * AP + kofs + m] = v;
    }
  }
  for (int e = threadIdx.x; e < 128 * (KP - nterms * twonb); e += blockDim.x) {
    const int w = KP - nterms * twonb;
    As[(e / w) * AP + nterms * twonb + e % w] = 0.f;
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gq = lane >> 2, tig = lane & 3;
  const int nt_n = NP / 8;
  float acc[8][4];
#pragma unroll
  for (int t = 0; t < 8; ++t)
#pragma unroll
    for (int c = 0; c < 4; ++c) acc[t][c] = 0.f;
  const float* Aw = As + (16 * warp) * AP;
  for (int k8 = 0; k8 < KP; k8 += 8) {
    uint32_t ah[4], al[4];
    split_tf32(Aw[gq * AP + k8 + tig], ah[0], al[0]);
    split_tf32(Aw[(gq + 8) * AP + k8 + tig], ah[1], al[1]);
    split_tf32(Aw[gq * AP + k8 + tig + 4], ah[2], al[2]);
    split_tf32(Aw[(gq + 8) * AP + k8 + tig + 4], ah[3], al[3]);
    const int r0 = (k8 + tig) * BP + gq, r1 = (k8 + tig + 4) * BP + gq;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
      if (nt < nt_n) {
        const uint32_t bh0 = Bh[r0 + 8 * nt], bh1 = Bh[r1 + 8 * nt];
        const uint32_t bl0 = Bl[r0 + 8 * nt], bl1 = Bl[r1 + 8 * nt];
        mma_tf32(acc[nt], al[0], al[1], al[2], al[3], bh0, bh1);
        mma_tf32(acc[nt], ah[0], ah[1], ah[2], ah[3], bl0, bl1);
        mma_tf32(acc[nt], ah[0], ah[1], ah[2], ah[3], bh0, bh1);
      }
    }
  }
  __syncthreads();
  float* Cs = As;   // [128][AP] staging of the [128][NP] result
#pragma unroll
  for (int nt = 0; nt < 8; ++nt) {
    if (nt < nt_n) {
      const int r0 = 16 * warp + gq, c0 = 8 * nt + 2 * tig;
      Cs[r0 * AP + c0] = acc[nt][0];
      Cs[r0 * AP + c0 + 1] = acc[nt][1];
      Cs[(r0 + 8) * AP + c0] = acc[nt][2];
      Cs[(r0 + 8) * AP + c0 + 1] = acc[nt][3];
    }
  }
  __syncthreads();
  const size_t base = sk * nb * ng;
  if (OUT == 0) {            // band-major complex [sk][j][g]
    float2* o = reinterpret_cast<float2*>(out0) + base;
    for (int e = threadIdx.x; e < nb * 128; e += blockDim.x) {
      const int j = e / 128, r = e - j * 128, g = g0 + r;
      if (g < ng) o[(size_t)j * ng + g] = make_float2(Cs[r * AP + j], Cs[r * AP + nb + j]);
    }
  } else if (OUT == 1) {     // (S,K,G,B) complex
    float2* o = reinterpret_cast<float2*>(out0) + base;
    for (int e = threadIdx.x; e < nb * 128; e += blockDim.x) {
      const int r = e / nb, j = e - r * nb, g = g0 + r;
      if (g < ng) o[(size_t)g * nb + j] = make_float2(Cs[r * AP + j], Cs[r * AP + nb + j]);
    }
  } else {                   // (S,K,G,B) split real/imag times fac
    float* ore = reinterpret_cast<float*>(out0) + base;
    float* oim = reinterpret_cast<float*>(out1) + base;
    for (int e = threadIdx.x; e < nb * 128; e += blockDim.x) {
      const int r = e / nb, j = e - r * nb, g = g0 + r;
      if (g < ng) {
        ore[(size_t)g * nb + j] = fac * Cs[r * AP + j];
        oim[(size_t)g * nb + j] = fac * Cs[r * AP + nb + j];
      }
    }
  }
}

static int round_up(int x, int m) { return (x + m - 1) / m * m; }

// Returns 1 when handled on the tensor cores, 0 when nb is too large.
int launch_gram_tc(int lx, const void* X0, const void* X1, int ly, const void* Y0, const void* Y1,
                   double* part, double2* out, int nsk, int ng, int nb, int nsplit,
                   cudaStream_t st) {
  if (nb > kTcMaxNb) return 0;
  const int MP = round_up(2 * nb, 16);
  const int split_len = round_up((ng + nsplit - 1) / nsplit, kTcChunk);
  nsplit = (ng + split_len - 1) / split_len;
  const int same = (X0 == Y0 && X1 == Y1) ? 1 : 0;
  dim3 grid(nsplit, 1, nsk);
  if (lx == 0 && ly == 0)
    k_gram_tc<0, 0><<<grid, 256, 0, st>>>(X0, X1, Y0, Y1, part, ng, nb, MP, split_len, same);
  else if (lx == 1 && ly == 1)
    k_gram_tc<1, 1><<<grid, 256, 0, st>>>(X0, X1, Y0, Y1, part, ng, nb, MP, split_len, same);
  else
    return -fail(JRG_ERR_INVALID, "launch_gram_tc: unsupported layouts");
  {
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return -cuda_fail(e, "k_gram_tc");
  }
  const size_t n = (size_t)nsk * nb * nb;
  k_gram_tc_reduce<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(part, out, nsplit, nb, MP, nsk);
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return -cuda_fail(e, "k_gram_tc_reduce");
  return 1;
}

// out_kind 0/1/2 as k_rotate; lx0 layout of X0 (0 split, 1 band-major); X1
// band-major.  bscratch: nsk*2*KP*NP words for the split B matrices.
int launch_rotate_tc(int out_kind, int lx0, const void* X0a, const void* X0b, const double2* M0,
                     const void* X1, const double2* M1, void* out0, void* out1, int nsk, int ng,
                     int nb, double fac, uint32_t* bscratch, cudaStream_t st) {
  if (nb > kTcMaxNb || !bscratch) return 0;
  const int nterms = X1 ? 2 : 1;
  const int KP = round_up(2 * nb * nterms, 8), NP = round_up(2 * nb, 8);
  k_rotate_tc_prep<<<nsk, 256, 0, st>>>(M0, X1 ? M1 : nullptr, bscratch, nb, KP, NP);
  {
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return -cuda_fail(e, "k_rotate_tc_prep");
  }
  const size_t sm = sizeof(float) * ((size_t)128 * (KP + 4) + 2 * (size_t)KP * (NP + 8));
  dim3 grid((ng + 127) / 128, nsk);
  auto go = [&](auto kern) -> int {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return -cuda_fail(e, "cudaFuncSetAttribute(k_rotate_tc)");
    kern<<<grid, 256, sm, st>>>(X0a, X0b, X1, bscratch, out0, out1, ng, nb, KP, NP, (float)fac);
    count_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess) return -cuda_fail(e, "k_rotate_tc");
    return 1;
  };
  if (lx0 == 0) {
    if (out_kind == 0) return go(k_rotate_tc<0, 0>);
    if (out_kind == 1) return go(k_rotate_tc<1, 0>);
    return go(k_rotate_tc<2, 0>);
  }
  if (out_kind == 0) return go(k_rotate_tc<0, 1>);
  if (out_kind == 1) return go(k_rotate_tc<1, 1>);
  return go(k_rotate_tc<2, 1>);
}

}  // namespace jrg
