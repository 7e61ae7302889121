// Learned diagonal preconditioner: a 3-64-64-64-1 MLP (GELU, softplus
// output) mapping per-coefficient features
//   x1 = |G+k|^2 / E_kin,band   (E_kin,band = sum_G |G+k|^2 |c|^2)
//   x2 = band / num_band
//   x3 = step / total_steps
// to a positive scale of the Adam update of that coefficient.
//
// Parameter layout (FP32 master copy and BF16 working copy, kMlpParams):
//   W1[64][3] b1[64] W2[64][64] b2[64] W3[64][64] b3[64] W4[64] b4
// GELU is the tanh form 0.5 x (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3)))
// (Hendrycks & Gimpel, 2016), evaluated with the tanh.approx.f32 instruction.
//
// Inference over every parameter runs on the tensor cores (mma.sync
// m16n8k16, BF16 operands, FP32 accumulation): a warp takes 16 coefficients,
// computes layer 1 on the CUDA cores, keeps the hidden activations in
// registers (accumulator fragments re-packed as the next layer's A
// fragments) and reduces layer 4 with shuffles.  Training runs layer by
// layer on the CUDA cores with BF16 weights and activations and FP32
// accumulation (a few 1e5-record batches: far from the tensor-core regime).
#include <cuda_bf16.h>
#include "plan.h"

namespace jrg {

constexpr int kH = 64;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + kH * 3, OFF_W2 = OFF_B1 + kH, OFF_B2 = OFF_W2 + kH * kH,
              OFF_W3 = OFF_B2 + kH, OFF_B3 = OFF_W3 + kH * kH, OFF_W4 = OFF_B3 + kH,
              OFF_B4 = OFF_W4 + kH, kMlpParams = OFF_B4 + 1;

__device__ __forceinline__ float tanh_approx(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float gelu(float x) {
  const float u = 0.7978845608028654f * (x + 0.044715f * x * x * x);
  return 0.5f * x * (1.0f + tanh_approx(u));
}
__device__ __forceinline__ float gelu_grad(float x) {
  const float u = 0.7978845608028654f * (x + 0.044715f * x * x * x);
  const float t = tanh_approx(u);
  const float du = 0.7978845608028654f * (1.0f + 3.0f * 0.044715f * x * x);
  return 0.5f * (1.0f + t) + 0.5f * x * (1.0f - t * t) * du;
}
__device__ __forceinline__ float softplus(float x) {
  return x > 20.f ? x : log1pf(__expf(x));
}
__device__ __forceinline__ float sigmoidf_(float x) { return 1.0f / (1.0f + __expf(-x)); }

__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16(x)); }

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}

__device__ __forceinline__ void mma_16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0,
                                          uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

constexpr int kWPitch = kH + 8;   // bf16 row pitch of W2/W3 in shared memory (bank spread)

// acc[j][*] (n8 tile j) -> A fragments of the next layer after GELU
__device__ __forceinline__ void gelu_pack(const float (&acc)[8][4], uint32_t (&a)[4][4]) {
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    a[q][0] = pack_bf16x2(gelu(acc[2 * q][0]), gelu(acc[2 * q][1]));
    a[q][1] = pack_bf16x2(gelu(acc[2 * q][2]), gelu(acc[2 * q][3]));
    a[q][2] = pack_bf16x2(gelu(acc[2 * q + 1][0]), gelu(acc[2 * q + 1][1]));
    a[q][3] = pack_bf16x2(gelu(acc[2 * q + 1][2]), gelu(acc[2 * q + 1][3]));
  }
}

__device__ __forceinline__ void dense_mma(const uint32_t (&a)[4][4], const __nv_bfloat16* W,
                                          const float* bias, float (&acc)[8][4], int g, int tig) {
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const float b0 = bias[8 * j + 2 * tig], b1 = bias[8 * j + 2 * tig + 1];
    acc[j][0] = b0; acc[j][1] = b1; acc[j][2] = b0; acc[j][3] = b1;
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const __nv_bfloat16* row = W + (8 * j + g) * kWPitch + 16 * q + 2 * tig;
      const uint32_t b0 = *reinterpret_cast<const uint32_t*>(row);
      const uint32_t b1 = *reinterpret_cast<const uint32_t*>(row + 8);
      mma_16816(acc[j], a[q], b0, b1);
    }
  }
}

// scale[e] for every parameter element e of (S,K,G,B) (written twice: the
// real and imaginary parameter share the scale of their coefficient).
// LUT: the table of the in-step form instead, element e = b * kLutN + i
// with x1 = i * x1max / (kLutN - 1) (x1max in hdr[0]), x2 = b / nb.
constexpr int kLutN = 4096;
template <bool LUT>
__global__ void __launch_bounds__(128) k_precond_scale(
    const float* __restrict__ wf, const __nv_bfloat16* __restrict__ wb,
    const double* __restrict__ tk, const double* __restrict__ ekin, const double* __restrict__ occ,
    int nk, int ng, int nb, long long total, float t_frac, float smax, float* __restrict__ out,
    const float* __restrict__ hdr = nullptr) {
  __shared__ __align__(16) __nv_bfloat16 w2[kH * kWPitch];
  __shared__ __align__(16) __nv_bfloat16 w3[kH * kWPitch];
  __shared__ float w1[kH * 3], b1[kH], b2[kH], b3[kH], w4[kH];
  __shared__ float b4;
  for (int i = threadIdx.x; i < kH * kH; i += blockDim.x) {
    const int r = i / kH, c = i % kH;
    w2[r * kWPitch + c] = wb[OFF_W2 + i];
    w3[r * kWPitch + c] = wb[OFF_W3 + i];
  }
  for (int i = threadIdx.x; i < kH * 3; i += blockDim.x) w1[i] = __bfloat162float(wb[OFF_W1 + i]);
  for (int i = threadIdx.x; i < kH; i += blockDim.x) {
    b1[i] = wf[OFF_B1 + i]; b2[i] = wf[OFF_B2 + i]; b3[i] = wf[OFF_B3 + i];
    w4[i] = __bfloat162float(wb[OFF_W4 + i]);
  }
  if (threadIdx.x == 0) b4 = wf[OFF_B4];
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane >> 2, tig = lane & 3;
  const long long ntiles = (total + 15) / 16;
  const long long wstride = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long tile = (long long)blockIdx.x * (blockDim.x >> 5) + warp; tile < ntiles; tile += wstride) {
    float x[2][3];
    bool live[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const long long e = tile * 16 + g + 8 * h;
      live[h] = e < total;
      const long long ee = live[h] ? e : 0;
      if constexpr (LUT) {
        const int b = (int)(ee / kLutN), i = (int)(ee % kLutN);
        x[h][0] = hdr[0] * (float)i / (float)(kLutN - 1);
        x[h][1] = (float)b / (float)nb;
        x[h][2] = t_frac;
        continue;
      }
      const int b = (int)(ee % nb);
      const long long rest = ee / nb;
      const int gg = (int)(rest % ng);
      const long long sk = rest / ng;
      const int k = (int)(sk % nk);
      const double ek = ekin[sk * nb + b];
      x[h][0] = (float)(tk[(size_t)k * ng + gg] / (ek > 1e-30 ? ek : 1e-30));
      x[h][1] = (float)b / (float)nb;
      x[h][2] = t_frac;
    }
    // layer 1 (CUDA cores) straight into A fragments
    uint32_t a[4][4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
#pragma unroll
      for (int half = 0; half < 2; ++half) {      // columns 16q + 8*half + 2 tig + {0,1}
        const int c0 = 16 * q + 8 * half + 2 * tig;
        float v[2][2];
#pragma unroll
        for (int h = 0; h < 2; ++h)
#pragma unroll
          for (int d = 0; d < 2; ++d) {
            const int c = c0 + d;
            v[h][d] = gelu(b1[c] + w1[3 * c] * x[h][0] + w1[3 * c + 1] * x[h][1] + w1[3 * c + 2] * x[h][2]);
          }
        a[q][2 * half + 0] = pack_bf16x2(v[0][0], v[0][1]);
        a[q][2 * half + 1] = pack_bf16x2(v[1][0], v[1][1]);
      }
    }
    float acc[8][4];
    dense_mma(a, w2, b2, acc, g, tig);
    gelu_pack(acc, a);
    dense_mma(a, w3, b3, acc, g, tig);
    float p0 = 0.f, p1 = 0.f;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int c = 8 * j + 2 * tig;
      // layer-3 activations rounded to BF16 as the training kernels store them
      p0 += bf16r(gelu(acc[j][0])) * w4[c] + bf16r(gelu(acc[j][1])) * w4[c + 1];
      p1 += bf16r(gelu(acc[j][2])) * w4[c] + bf16r(gelu(acc[j][3])) * w4[c + 1];
    }
    p0 += __shfl_xor_sync(0xffffffffu, p0, 1);
    p0 += __shfl_xor_sync(0xffffffffu, p0, 2);
    p1 += __shfl_xor_sync(0xffffffffu, p1, 1);
    p1 += __shfl_xor_sync(0xffffffffu, p1, 2);
    if (tig == 0) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        if (!live[h]) continue;
        const long long e = tile * 16 + g + 8 * h;
        float s = softplus((h ? p1 : p0) + b4);
        s = fminf(s, smax);
        if constexpr (LUT) {
          out[e] = s;
          continue;
        }
        const long long band = e / ((long long)nb * ng) * nb + e % nb;
        if (occ[band] == 0.0) s = 1.0f;
        out[e] = s;
        out[total + e] = s;
      }
    }
  }
}

// ------------------------------------------------------------------------
// training kernels (CUDA cores, BF16 in, FP32 accumulate)
// ------------------------------------------------------------------------
// Z[n][o] = X[n][:] . W[o][:] + b[o];  H = GELU(Z)   (X: FP32 for layer 1, BF16 after)
template <typename TIN>
__global__ void k_mlp_fwd(const TIN* __restrict__ X, int din, const __nv_bfloat16* __restrict__ W,
                          const float* __restrict__ bias, float* __restrict__ Z,
                          __nv_bfloat16* __restrict__ H, int n) {
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)n * kH) return;
  const int r = (int)(idx / kH), o = (int)(idx % kH);
  float acc = bias[o];
  for (int i = 0; i < din; ++i) acc += (float)X[(size_t)r * din + i] * __bfloat162float(W[o * din + i]);
  Z[idx] = acc;
  H[idx] = __float2bfloat16(gelu(acc));
}

// output layer: z4 = H3 . W4 + b4, s = softplus(z4); loss terms of the
// one-step quadratic model per record  l = w (s a + s^2 c / 2)
// (a = g_t.u: slope of the record's step, c = (g_{t+1} - g_t).u: its secant
// curvature), dl/dz4 = w (a + s c) sigmoid(z4)
__global__ void k_mlp_out_loss(const __nv_bfloat16* __restrict__ H3, const __nv_bfloat16* __restrict__ W4,
                               const float* __restrict__ b4, const float* __restrict__ a,
                               const float* __restrict__ c, const float* __restrict__ w, float* __restrict__ s_out,
                               float* __restrict__ dz4, double* __restrict__ loss_part, int n) {
  __shared__ double red[32];
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  double l = 0.0;
  if (r < n) {
    float z = b4[0];
    for (int i = 0; i < kH; ++i) z += __bfloat162float(H3[(size_t)r * kH + i]) * __bfloat162float(W4[i]);
    const float s = softplus(z);
    if (s_out) s_out[r] = s;
    if (a) {
      const float wr = w ? w[r] : 1.0f;
      l = (double)wr * ((double)s * a[r] + 0.5 * (double)s * s * c[r]);
      dz4[r] = wr * (a[r] + s * c[r]) * sigmoidf_(z);
    }
  }
  if (loss_part) {
    l = block_sum(l, red);
    if (threadIdx.x == 0) loss_part[blockIdx.x] = l;
  }
}

// dH[n][i] = sum_o dZ[n][o] W[o][i] (input-gradient of a dense layer); with
// GELU' of the input layer's pre-activation applied when Zin is given
__global__ void k_mlp_bwd_data(const float* __restrict__ dZ, int dout, const __nv_bfloat16* __restrict__ W,
                               const float* __restrict__ Zin, float* __restrict__ dZin, int n) {
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)n * kH) return;
  const int r = (int)(idx / kH), i = (int)(idx % kH);
  float acc = 0.f;
  for (int o = 0; o < dout; ++o) acc += dZ[(size_t)r * dout + o] * __bfloat162float(W[o * kH + i]);
  dZin[idx] = acc * gelu_grad(Zin[idx]);
}

// partial weight gradient over a chunk of rows: dW[o][i] = sum_r dZ[r][o] X[r][i],
// db[o] = sum_r dZ[r][o]; one block per chunk, thread per (o, i-block)
template <typename TIN>
__global__ void k_mlp_wgrad(const float* __restrict__ dZ, int dout, const TIN* __restrict__ X, int din,
                            float* __restrict__ part, int n, int chunk) {
  const int r0 = blockIdx.x * chunk, r1 = min(n, r0 + chunk);
  const int nw = dout * din + dout;
  float* p = part + (size_t)blockIdx.x * nw;
  for (int e = threadIdx.x; e < nw; e += blockDim.x) {
    float acc = 0.f;
    if (e < dout * din) {
      const int o = e / din, i = e % din;
      for (int r = r0; r < r1; ++r) acc += dZ[(size_t)r * dout + o] * (float)X[(size_t)r * din + i];
    } else {
      const int o = e - dout * din;
      for (int r = r0; r < r1; ++r) acc += dZ[(size_t)r * dout + o];
    }
    p[e] = acc;
  }
}

__global__ void k_sum_parts(const float* __restrict__ part, int nparts, int len, float* __restrict__ out,
                            float scale) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= len) return;
  double acc = 0.0;
  for (int p = 0; p < nparts; ++p) acc += part[(size_t)p * len + e];
  out[e] = (float)(acc * scale);
}

__global__ void k_to_bf16(const float* __restrict__ in, __nv_bfloat16* __restrict__ out, int n) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n) out[e] = __float2bfloat16(in[e]);
}

__global__ void k_sum_double(const double* __restrict__ in, int n, double* __restrict__ out) {
  __shared__ double red[32];
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc += in[i];
  acc = block_sum(acc, red);
  if (threadIdx.x == 0) out[0] = acc;
}

// ------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------
struct MlpWs {
  size_t z1, z2, z3, h1, h2, h3, dz4, dz3, dz2, dz1, part, lpart, total;
  int chunk, nchunks, lblocks;
};
static size_t al(size_t x) { return (x + 255) & ~(size_t)255; }
static MlpWs mlp_layout(int n) {
  MlpWs w;
  w.chunk = 256;
  w.nchunks = (n + w.chunk - 1) / w.chunk;
  w.lblocks = (n + 255) / 256;
  size_t o = 0;
  auto take = [&](size_t b) { size_t r = o; o += al(b); return r; };
  const size_t nh = (size_t)n * kH;
  w.z1 = take(nh * 4); w.z2 = take(nh * 4); w.z3 = take(nh * 4);
  w.h1 = take(nh * 2); w.h2 = take(nh * 2); w.h3 = take(nh * 2);
  w.dz4 = take((size_t)n * 4); w.dz3 = take(nh * 4); w.dz2 = take(nh * 4); w.dz1 = take(nh * 4);
  w.part = take((size_t)w.nchunks * (kH * kH + kH) * 4);
  w.lpart = take((size_t)w.lblocks * 8);
  w.total = o;
  return w;
}

int launch_precond_scale(const float* wf, const void* wb, const double* tk, const double* ekin,
                         const double* occ, int nk, int ng, int nb, long long total, float t_frac,
                         float smax, float* out, cudaStream_t st) {
  const long long ntiles = (total + 15) / 16;
  long long blocks = (ntiles + 3) / 4;
  if (blocks > 152 * 16) blocks = 152 * 16;
  k_precond_scale<false><<<(unsigned)blocks, 128, 0, st>>>(wf, reinterpret_cast<const __nv_bfloat16*>(wb), tk,
                                                           ekin, occ, nk, ng, nb, total, t_frac, smax, out);
  JRG_LAUNCH_CHECK("k_precond_scale");
  return JRG_OK;
}

// ---- in-step form: the network tabulated in x1 ---------------------------
// The features of a coefficient are x1 = |G+k|^2/2 / E_kin(band), x2 = band/B
// and the step fraction x3, so within one call the scale is a function of x1
// for each band b.  The in-step form evaluates the network (the same BF16
// tensor-core inference) on kLutN points x1_i = i x1max / (kLutN - 1) per
// band, x1max the largest x1 of the occupied bands, and every coefficient
// interpolates linearly in its band's table: nb * kLutN network evaluations
// instead of one per coefficient (the inference of 11 M coefficients at the
// 64^3 Si8 cell took ~0.6 ms per step; the table and the interpolation pass,
// a read of the FP32 kinetic table and a write of the scales, take a few
// percent of that).  Workspace: precond_lut_floats(nb, nbt) floats.
size_t precond_lut_floats(int nb, int nbt) { return 4 + (size_t)nb * kLutN + (size_t)nbt; }

// hdr[0] = x1max = tk_max / (smallest occupied-band E_kin); invek[band] =
// 1 / E_kin(band), -1 for an empty band
__global__ void __launch_bounds__(1024) k_precond_prep(float tmax, const double* __restrict__ ekin,
                                                       const double* __restrict__ occ, int nbt,
                                                       float* __restrict__ hdr, float* __restrict__ invek) {
  __shared__ float red[32];
  float emin = 3.0e38f;
  for (int b = threadIdx.x; b < nbt; b += blockDim.x) {
    const double ek = ekin[b];
    const bool on = occ[b] != 0.0;
    const float e = (float)(ek > 1e-30 ? ek : 1e-30);
    invek[b] = on ? 1.0f / e : -1.0f;
    if (on) emin = fminf(emin, e);
  }
  for (int o = 16; o > 0; o >>= 1) emin = fminf(emin, __shfl_xor_sync(0xffffffffu, emin, o));
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) red[w] = emin;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) emin = fminf(emin, red[i]);
    hdr[0] = emin < 3.0e38f ? fmaxf(tmax / emin, 1e-6f) * 1.0001f : 1.0f;
  }
}

// out[e] (and out[total + e]): the band's table at x1 = tkf[k][g] * invek[band]
__global__ void k_precond_apply(const float* __restrict__ hdr, const float* __restrict__ lut,
                                const float* __restrict__ invek, const float* __restrict__ tkf, int nk, int ng,
                                int nb, long long total, float* __restrict__ out) {
  const float pos = (float)(kLutN - 1) / hdr[0];
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int b = (int)(e % nb);
    const long long rest = e / nb;
    const int gg = (int)(rest % ng);
    const long long sk = rest / ng;
    const float ie = invek[sk * nb + b];
    float s = 1.0f;
    if (ie >= 0.f) {
      const float u = fminf(tkf[(size_t)(sk % nk) * ng + gg] * ie * pos, (float)(kLutN - 1));
      const int i0 = min((int)u, kLutN - 2);
      const float f = u - (float)i0;
      const float* tb = lut + (size_t)b * kLutN;
      s = fmaf(f, tb[i0 + 1] - tb[i0], tb[i0]);
    }
    out[e] = s;
    out[total + e] = s;
  }
}

int launch_precond_scale_lut(const float* wf, const void* wb, const double* tk, const float* tkf, float tk_max,
                             const double* ekin, const double* occ, int nk, int ng, int nb, int nbt,
                             long long total, float t_frac, float smax, float* out, float* lutws,
                             cudaStream_t st) {
  float* hdr = lutws;
  float* lut = lutws + 4;
  float* invek = lut + (size_t)nb * kLutN;
  k_precond_prep<<<1, 1024, 0, st>>>(tk_max, ekin, occ, nbt, hdr, invek);
  JRG_LAUNCH_CHECK("k_precond_prep");
  const long long n = (long long)nb * kLutN;
  const long long blocks = ((n + 15) / 16 + 3) / 4;
  k_precond_scale<true><<<(unsigned)blocks, 128, 0, st>>>(wf, reinterpret_cast<const __nv_bfloat16*>(wb), tk,
                                                          ekin, occ, nk, ng, nb, n, t_frac, smax, lut, hdr);
  JRG_LAUNCH_CHECK("k_precond_scale(table)");
  long long ab = (total + 255) / 256;
  if (ab > 152 * 8) ab = 152 * 8;
  k_precond_apply<<<(unsigned)ab, 256, 0, st>>>(hdr, lut, invek, tkf, nk, ng, nb, total, out);
  JRG_LAUNCH_CHECK("k_precond_apply");
  return JRG_OK;
}

}  // namespace jrg

using namespace jrg;

extern "C" {

int jrg_mlp_num_params(void) { return kMlpParams; }

int jrg_mlp_workspace_size(int n, size_t* bytes) {
  if (n < 1 || !bytes) return fail(JRG_ERR_INVALID, "jrg_mlp_workspace_size: bad argument");
  *bytes = mlp_layout(n).total;
  return JRG_OK;
}

int jrg_mlp_to_bf16(const float* w, void* wb, cudaStream_t st) {
  if (!w || !wb) return fail(JRG_ERR_INVALID, "jrg_mlp_to_bf16: null argument");
  k_to_bf16<<<(kMlpParams + 255) / 256, 256, 0, st>>>(w, reinterpret_cast<__nv_bfloat16*>(wb), kMlpParams);
  JRG_LAUNCH_CHECK("k_to_bf16");
  return JRG_OK;
}

// Forward over n records x[n][3] -> s[n]; with a, c (and optional weights w)
// also the summed loss (device double[1]) and, when grad is given, the
// gradient of the mean loss with respect to the FP32 parameters.
int jrg_mlp_train_eval(int n, const float* x, const float* w32, const void* wb, const float* a,
                       const float* c, const float* wt, float* s_out, double* loss, float* grad,
                       void* ws, cudaStream_t st) {
  if (n < 1 || !x || !w32 || !wb || !ws || ((loss || grad) && (!a || !c)))
    return fail(JRG_ERR_INVALID, "jrg_mlp_train_eval: bad argument");
  const MlpWs L = mlp_layout(n);
  char* base = reinterpret_cast<char*>(ws);
  auto F = [&](size_t off) { return reinterpret_cast<float*>(base + off); };
  auto B = [&](size_t off) { return reinterpret_cast<__nv_bfloat16*>(base + off); };
  const __nv_bfloat16* W = reinterpret_cast<const __nv_bfloat16*>(wb);
  const unsigned gh = (unsigned)(((long long)n * kH + 255) / 256);
  k_mlp_fwd<float><<<gh, 256, 0, st>>>(x, 3, W + OFF_W1, w32 + OFF_B1, F(L.z1), B(L.h1), n);
  JRG_LAUNCH_CHECK("k_mlp_fwd");
  k_mlp_fwd<__nv_bfloat16><<<gh, 256, 0, st>>>(B(L.h1), kH, W + OFF_W2, w32 + OFF_B2, F(L.z2), B(L.h2), n);
  JRG_LAUNCH_CHECK("k_mlp_fwd");
  k_mlp_fwd<__nv_bfloat16><<<gh, 256, 0, st>>>(B(L.h2), kH, W + OFF_W3, w32 + OFF_B3, F(L.z3), B(L.h3), n);
  JRG_LAUNCH_CHECK("k_mlp_fwd");
  double* lp = reinterpret_cast<double*>(base + L.lpart);
  k_mlp_out_loss<<<L.lblocks, 256, 0, st>>>(B(L.h3), W + OFF_W4, w32 + OFF_B4, a, c, wt, s_out,
                                            F(L.dz4), (loss ? lp : nullptr), n);
  JRG_LAUNCH_CHECK("k_mlp_out_loss");
  if (loss) {
    k_sum_double<<<1, 256, 0, st>>>(lp, L.lblocks, loss);
    JRG_LAUNCH_CHECK("k_sum_double");
  }
  if (!grad) return JRG_OK;
  const float inv_n = 1.0f / (float)n;
  float* part = F(L.part);
  // layer 4
  k_mlp_wgrad<__nv_bfloat16><<<L.nchunks, 256, 0, st>>>(F(L.dz4), 1, B(L.h3), kH, part, n, L.chunk);
  JRG_LAUNCH_CHECK("k_mlp_wgrad");
  k_sum_parts<<<1, 128, 0, st>>>(part, L.nchunks, kH + 1, grad + OFF_W4, inv_n);
  JRG_LAUNCH_CHECK("k_sum_parts");
  k_mlp_bwd_data<<<gh, 256, 0, st>>>(F(L.dz4), 1, W + OFF_W4, F(L.z3), F(L.dz3), n);
  JRG_LAUNCH_CHECK("k_mlp_bwd_data");
  // layer 3
  k_mlp_wgrad<__nv_bfloat16><<<L.nchunks, 256, 0, st>>>(F(L.dz3), kH, B(L.h2), kH, part, n, L.chunk);
  JRG_LAUNCH_CHECK("k_mlp_wgrad");
  k_sum_parts<<<(kH * kH + kH + 255) / 256, 256, 0, st>>>(part, L.nchunks, kH * kH + kH, grad + OFF_W3, inv_n);
  JRG_LAUNCH_CHECK("k_sum_parts");
  k_mlp_bwd_data<<<gh, 256, 0, st>>>(F(L.dz3), kH, W + OFF_W3, F(L.z2), F(L.dz2), n);
  JRG_LAUNCH_CHECK("k_mlp_bwd_data");
  // layer 2
  k_mlp_wgrad<__nv_bfloat16><<<L.nchunks, 256, 0, st>>>(F(L.dz2), kH, B(L.h1), kH, part, n, L.chunk);
  JRG_LAUNCH_CHECK("k_mlp_wgrad");
  k_sum_parts<<<(kH * kH + kH + 255) / 256, 256, 0, st>>>(part, L.nchunks, kH * kH + kH, grad + OFF_W2, inv_n);
  JRG_LAUNCH_CHECK("k_sum_parts");
  k_mlp_bwd_data<<<gh, 256, 0, st>>>(F(L.dz2), kH, W + OFF_W2, F(L.z1), F(L.dz1), n);
  JRG_LAUNCH_CHECK("k_mlp_bwd_data");
  // layer 1
  k_mlp_wgrad<float><<<L.nchunks, 256, 0, st>>>(F(L.dz1), kH, x, 3, part, n, L.chunk);
  JRG_LAUNCH_CHECK("k_mlp_wgrad");
  k_sum_parts<<<1, 256, 0, st>>>(part, L.nchunks, kH * 3 + kH, grad + OFF_W1, inv_n);
  JRG_LAUNCH_CHECK("k_sum_parts");
  return JRG_OK;
}

}  // extern "C"
