// Single-grid kernels: density reduction, reciprocal-space Hartree and
// external energies, LDA exchange-correlation, potential assembly, kinetic
// energy on the sphere, energy-slot reduction, geometry tables and Ewald.
// Energy sums are accumulated in FP64 per block and reduced deterministically.
#include "plan.h"

namespace jrg {

// rho[s][i] = sum over the groups g of spin s of gscale[g] part[g][i] (FP64
// sum; gscale = the group's reference weight over the cell volume); with
// qpart, block b also stores the FP64 sum of the rho values it wrote
// (kQParts blocks)
// FP32 partials are summed in float-float arithmetic (each gscale as hi + lo,
// exact products by FMA, two-sum accumulation: about 2^-44 relative, with
// FP32 instructions instead of the GPU's slow FP64 pipe); FP64 partials in
// FP64.  Group factors are staged in shared memory (groups_per_spin * ns <=
// kMaxReduceGroups, else read from global memory).
constexpr int kMaxReduceGroups = 1024;
template <typename R>
__global__ void __launch_bounds__(256) k_reduce_density(const R* __restrict__ part, R* __restrict__ rho,
                                                        int groups_per_spin, int ns, long long ngrid,
                                                        const double* __restrict__ gscale,
                                                        double* __restrict__ qpart) {
  __shared__ double red[32];
  __shared__ float2 sg[kMaxReduceGroups];   // gscale as (hi, lo)
  const int ngr = groups_per_spin * ns;
  const bool staged = ngr <= kMaxReduceGroups;
  if (staged)
    for (int g = threadIdx.x; g < ngr; g += blockDim.x) {
      const float h = (float)gscale[g];
      sg[g] = make_float2(h, (float)(gscale[g] - (double)h));
    }
  __syncthreads();
  const long long n = (long long)ns * ngrid;
  double q = 0.0;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x) {
    const long long s = e / ngrid, i = e % ngrid;
    R r;
    if constexpr (sizeof(R) == 4) {
      float sh = 0.f, sl = 0.f;
      for (int g = 0; g < groups_per_spin; ++g) {
        const long long gg = (long long)s * groups_per_spin + g;
        float2 f;
        if (staged) {
          f = sg[gg];
        } else {
          f.x = (float)gscale[gg];
          f.y = (float)(gscale[gg] - (double)f.x);
        }
        const float x = part[gg * ngrid + i];
        const float p = x * f.x;
        const float pe = fmaf(x, f.y, fmaf(x, f.x, -p));   // exact low part of x*hi, plus x*lo
        const float t = sh + p;                            // two-sum of sh and p
        const float bb = t - sh;
        const float te = (sh - (t - bb)) + (p - bb);
        sh = t;
        sl += te + pe;
      }
      r = (R)((double)sh + (double)sl);
    } else {
      double acc = 0.0;
      for (int g = 0; g < groups_per_spin; ++g) {
        const long long gg = (long long)s * groups_per_spin + g;
        acc += gscale[gg] * (double)part[gg * ngrid + i];
      }
      r = (R)acc;
    }
    rho[e] = r;
    q += (double)r;
  }
  if (qpart) {
    q = block_sum(q, red);
    if (threadIdx.x == 0) qpart[blockIdx.x] = q;
  }
}

// k_reduce_density with 16-byte loads and stores (4 FP32 or 2 FP64 points
// per thread) and the group loop unrolled by four with its loads issued
// together, so that each thread keeps several loads in flight: the partials
// are read once from HBM and the kernel sits between the two forks of the
// pipelined step, where nothing else hides its latency.  Same arithmetic
// per point as k_reduce_density.  Needs ngrid % (16 / sizeof(R)) == 0 and
// 16-byte aligned part and rho.
template <typename R> struct Vec16;
template <> struct Vec16<float> { using T = float4; static constexpr int n = 4; };
template <> struct Vec16<double> { using T = double2; static constexpr int n = 2; };

// one float-float accumulation step: (sh, sl) += x * (f.x + f.y)
__device__ __forceinline__ void ff_acc(float& sh, float& sl, float x, float2 f) {
  const float p = x * f.x;
  const float pe = fmaf(x, f.y, fmaf(x, f.x, -p));   // exact low part of x*hi, plus x*lo
  const float t = sh + p;                            // two-sum of sh and p
  const float bb = t - sh;
  const float te = (sh - (t - bb)) + (p - bb);
  sh = t;
  sl += te + pe;
}

template <typename R>
__global__ void __launch_bounds__(256) k_reduce_density_v(const R* __restrict__ part, R* __restrict__ rho,
                                                          int groups_per_spin, int ns, long long ngrid,
                                                          const double* __restrict__ gscale,
                                                          double* __restrict__ qpart) {
  using V = typename Vec16<R>::T;
  constexpr int W = Vec16<R>::n;
  constexpr int U = 4;   // groups per unrolled step
  __shared__ double red[32];
  __shared__ float2 sg[kMaxReduceGroups];
  const int ngr = groups_per_spin * ns;
  const bool staged = ngr <= kMaxReduceGroups;
  if (staged)
    for (int g = threadIdx.x; g < ngr; g += blockDim.x) {
      const float h = (float)gscale[g];
      sg[g] = make_float2(h, (float)(gscale[g] - (double)h));
    }
  __syncthreads();
  const long long ngv = ngrid / W, n = (long long)ns * ngv;
  const V* src = reinterpret_cast<const V*>(part);
  V* dst = reinterpret_cast<V*>(rho);
  double q = 0.0;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x) {
    const long long s = e / ngv, iv = e % ngv;
    const long long g0 = s * groups_per_spin;
    V o;
    if constexpr (sizeof(R) == 4) {
      float h0 = 0.f, h1 = 0.f, h2 = 0.f, h3 = 0.f, l0 = 0.f, l1 = 0.f, l2 = 0.f, l3 = 0.f;
      int g = 0;
      for (; g + U <= groups_per_spin; g += U) {
        V x[U];
        float2 f[U];
#pragma unroll
        for (int u = 0; u < U; ++u) x[u] = src[(g0 + g + u) * ngv + iv];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const long long gg = g0 + g + u;
          if (staged) {
            f[u] = sg[gg];
          } else {
            f[u].x = (float)gscale[gg];
            f[u].y = (float)(gscale[gg] - (double)f[u].x);
          }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
          ff_acc(h0, l0, x[u].x, f[u]);
          ff_acc(h1, l1, x[u].y, f[u]);
          ff_acc(h2, l2, x[u].z, f[u]);
          ff_acc(h3, l3, x[u].w, f[u]);
        }
      }
      for (; g < groups_per_spin; ++g) {
        const long long gg = g0 + g;
        const V x = src[gg * ngv + iv];
        float2 f;
        if (staged) {
          f = sg[gg];
        } else {
          f.x = (float)gscale[gg];
          f.y = (float)(gscale[gg] - (double)f.x);
        }
        ff_acc(h0, l0, x.x, f);
        ff_acc(h1, l1, x.y, f);
        ff_acc(h2, l2, x.z, f);
        ff_acc(h3, l3, x.w, f);
      }
      o.x = (float)((double)h0 + (double)l0);
      o.y = (float)((double)h1 + (double)l1);
      o.z = (float)((double)h2 + (double)l2);
      o.w = (float)((double)h3 + (double)l3);
      q += ((double)o.x + (double)o.y) + ((double)o.z + (double)o.w);
    } else {
      double a0 = 0.0, a1 = 0.0;
      int g = 0;
      for (; g + U <= groups_per_spin; g += U) {
        V x[U];
#pragma unroll
        for (int u = 0; u < U; ++u) x[u] = src[(g0 + g + u) * ngv + iv];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const double f = gscale[g0 + g + u];
          a0 += f * x[u].x;
          a1 += f * x[u].y;
        }
      }
      for (; g < groups_per_spin; ++g) {
        const V x = src[(g0 + g) * ngv + iv];
        const double f = gscale[g0 + g];
        a0 += f * x.x;
        a1 += f * x.y;
      }
      o.x = a0;
      o.y = a1;
      q += o.x + o.y;
    }
    dst[e] = o;
  }
  if (qpart) {
    q = block_sum(q, red);
    if (threadIdx.x == 0) qpart[blockIdx.x] = q;
  }
}

// threads per CTA of the single-grid energy kernels (k_recip_terms,
// k_potential, k_potential_pol; their CTA count is the number of energy
// slots)
constexpr int kGridThreads = 256;   // 512: k_recip_terms 34 vs 19 us, k_potential 28 vs 19 us (64^3)

// the charge factor s of ChargeFix (every thread of the block gets it)
__device__ __forceinline__ double charge_scale(const ChargeFix& cf, double* red) {
  if (!cf.qpart) return 1.0;
  double a = 0.0, t = 0.0;
  for (int i = threadIdx.x; i < kQParts; i += blockDim.x) a += cf.qpart[i];
  for (int i = threadIdx.x; i < cf.nocc; i += blockDim.x) t += cf.occ[i];
  a = block_sum(a, red) * cf.dv;
  t = block_sum(t, red);
  return (a > 0.0 && t > 0.0) ? t / a : 1.0;
}

// Hartree term of a single (spin-summed) density transform rhog, for the
// renormalised density s rho (s from ChargeFix; block 0 stores it):
//   E_H = vol/N^2 * sum 1/2 ginv |s rho_G|^2          (ginv = 4 pi/|G|^2, 0 at G=0)
//   vg  = ginv * s rho_G   (the Hartree potential, before the 1/N of the IFFT)
// The external energy and potential are taken in real space from the FP64
// V_ext(r) table by the potential kernels (Parseval: the same sum).
template <typename R>
__global__ void __launch_bounds__(kGridThreads) k_recip_terms(const C_t<R>* __restrict__ rhog,
                                                     const double* __restrict__ ginv,
                                                     C_t<R>* __restrict__ vg, double* __restrict__ slot_h,
                                                     long long ngrid, double pref, ChargeFix cf) {
  __shared__ double red[32];
  const double s = charge_scale(cf, red);
  if (cf.scale && blockIdx.x == 0 && threadIdx.x == 0) *cf.scale = s;
  double eh = 0.0;
#pragma unroll 4
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ngrid;
       i += (long long)gridDim.x * blockDim.x) {
    const C_t<R> r = rhog[i];
    const double gi = ginv[i];
    const double rx = r.x, ry = r.y;
    eh += 0.5 * gi * (rx * rx + ry * ry);
    C_t<R> o;
    o.x = (R)(s * gi * rx);
    o.y = (R)(s * gi * ry);
    if (vg) vg[i] = o;
  }
  eh = block_sum(eh, red);
  if (threadIdx.x == 0) slot_h[blockIdx.x] = eh * pref * s * s;
}

// LDA: Slater exchange + VWN (1980) paramagnetic correlation fit.
__device__ __forceinline__ void lda_eps_v(double rho, int xc, double* eps, double* v) {
  double e = 0.0, vv = 0.0;
  if (rho > 1e-15) {
    if (xc & JRG_XC_LDA_X) {
      const double cx = 0.7385587663820224;   // (3/4) (3/pi)^(1/3)
      const double ex = -cx * cbrt(rho);
      e += ex;
      vv += 4.0 / 3.0 * ex;
    }
    if (xc & JRG_XC_LDA_C_VWN) {
      const double A = 0.0310907, b = 3.72744, c = 12.9352, x0 = -0.10498;
      const double q = sqrt(4.0 * c - b * b);
      const double xx0 = x0 * x0 + b * x0 + c;
      const double rs = cbrt(3.0 / (4.0 * 3.14159265358979323846 * rho));
      const double x = sqrt(rs);
      const double xx = x * x + b * x + c;
      const double at = atan(q / (2.0 * x + b));
      const double ec = A * (log(x * x / xx) + 2.0 * b / q * at -
                             b * x0 / xx0 * (log((x - x0) * (x - x0) / xx) + 2.0 * (b + 2.0 * x0) / q * at));
      const double den = (2.0 * x + b) * (2.0 * x + b) + q * q;
      const double dec = A * (2.0 / x - (2.0 * x + b) / xx - 4.0 * b / den -
                              b * x0 / xx0 * (2.0 / (x - x0) - (2.0 * x + b) / xx - 4.0 * (b + 2.0 * x0) / den));
      e += ec;
      vv += ec - x / 6.0 * dec;
    }
  }
  *eps = e;
  *v = vv;
}

// rho^(1/3) to about FP64 accuracy from FP32 arithmetic: y = cbrtf(rho)
// and one Newton step y - (y^3 - rho) / (3 y^2), whose residual y^3 - rho is
// formed exactly (y^2 and y^2 * y as float-float products by FMA; p3 - rho
// is exact because p3 and rho agree to a few ulps) and whose correction,
// ~1e-7 of y, needs only FP32 precision.  Two FP64 operations instead of an
// FP64 Newton step with its division (the GPU's FP64 rate is 1/64 of FP32).
__device__ __forceinline__ double cbrt_ff(float rho) {
  const float y = cbrtf(rho);
  const float p2 = y * y, e2 = fmaf(y, y, -p2);
  const float p3 = p2 * y, e3 = fmaf(p2, y, -p3);
  const float res = (p3 - rho) + fmaf(e2, y, e3);
  return (double)y - (double)__fdividef(res, 3.0f * p2);   // 2-ulp quotient of a ~1e-7 correction
}

// FP32 path: rho^(1/3) by cbrt_ff (the exchange term dominates E_xc), the
// VWN correlation (about 1% of it) in FP32.
__device__ __forceinline__ void lda_eps_v_f32(float rho, int xc, double* eps, double* v) {
  double e = 0.0, vv = 0.0;
  if (rho > 1e-15f) {
    const double y = cbrt_ff(rho);
    if (xc & JRG_XC_LDA_X) {
      const double ex = -0.7385587663820224 * y;   // (3/4) (3/pi)^(1/3) rho^(1/3)
      e += ex;
      vv += 4.0 / 3.0 * ex;
    }
    if (xc & JRG_XC_LDA_C_VWN) {
      const float A = 0.0310907f, b = 3.72744f, c = 12.9352f, x0 = -0.10498f;
      const float q = 6.15199081975907951f;        // sqrt(4c - b^2)
      const float xx0 = x0 * x0 + b * x0 + c;
      const float rs = 0.620350491f / (float)y;   // (3/(4 pi))^(1/3) / rho^(1/3)
      const float x = sqrtf(rs);
      const float xx = x * x + b * x + c;
      const float at = atanf(q / (2.0f * x + b));
      const float ec = A * (logf(x * x / xx) + 2.0f * b / q * at -
                            b * x0 / xx0 * (logf((x - x0) * (x - x0) / xx) + 2.0f * (b + 2.0f * x0) / q * at));
      const float den = (2.0f * x + b) * (2.0f * x + b) + q * q;
      const float dec = A * (2.0f / x - (2.0f * x + b) / xx - 4.0f * b / den -
                             b * x0 / xx0 * (2.0f / (x - x0) - (2.0f * x + b) / xx - 4.0f * (b + 2.0f * x0) / den));
      e += ec;
      vv += (double)(ec - x / 6.0f * dec);
    }
  }
  *eps = e;
  *v = vv;
}

template <typename R> __device__ __forceinline__ void lda_eps_v_t(R rho, int xc, double* eps, double* v) {
  if constexpr (sizeof(R) == 4) lda_eps_v_f32(rho, xc, eps, v);
  else lda_eps_v(rho, xc, eps, v);
}

// ------------------------------------------------------------------------
// Spin-polarised LDA (jrystal/_src/xc.py:40-64, polarised branches).
// Exchange by jrystal's scaling: eps_x = (e_x(2 rho_up) + e_x(2 rho_dn)) / 2
// per particle of the total density.  Correlation: the VWN (1980)
// interpolation of jax_xc's lda_c_vwn "pol" form,
//   eps_c = eps_P + alpha f(z) (1 - z^4) / f''(0) + (eps_F - eps_P) f(z) z^4,
// z = (rho_up - rho_dn) / rho, f(z) = ((1+z)^(4/3) + (1-z)^(4/3) - 2) /
// (2^(4/3) - 2), with the paramagnetic, ferromagnetic and spin-stiffness
// fits of the VWN5 parameterisation.  lda_pol gives eps and d eps / d rho_s;
// the energy path's potential is eps + rho d eps / d rho_s (the derivative
// of eps rho), the Kohn-Sham field of vxc_lda eps + rho_s d eps / d rho_s.
// T is the arithmetic type of the correlation (float on the FP32 path: it is
// about 1% of E_xc); exchange takes rho^(1/3) in FP64 on both paths.
// ------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void vwn_fit(T x, T A, T b, T c, T x0, T q, T* f, T* df) {
  const T xx0 = x0 * x0 + b * x0 + c;
  const T xx = x * x + b * x + c;
  const T at = atan(q / (T(2) * x + b));
  *f = A * (log(x * x / xx) + T(2) * b / q * at -
            b * x0 / xx0 * (log((x - x0) * (x - x0) / xx) + T(2) * (b + T(2) * x0) / q * at));
  const T den = (T(2) * x + b) * (T(2) * x + b) + q * q;
  *df = A * (T(2) / x - (T(2) * x + b) / xx - T(4) * b / den -
             b * x0 / xx0 * (T(2) / (x - x0) - (T(2) * x + b) / xx - T(4) * (b + T(2) * x0) / den));
}

// rho^(1/3) to FP64 accuracy (cbrt_ff on the FP32 path)
template <typename R> __device__ __forceinline__ double cbrt_t(R r) {
  if constexpr (sizeof(R) == 4) return cbrt_ff(r);
  else return cbrt((double)r);
}

template <typename R>
__device__ __forceinline__ void lda_pol(R ru, R rd, int xc, double* eps, double* du, double* dd) {
  using T = R;
  double e = 0.0, a = 0.0, b = 0.0;
  if (xc & JRG_XC_LDA_X) {
    constexpr double cx = 0.7385587663820224;   // (3/4) (3/pi)^(1/3)
    const R r2[2] = {R(2) * ru, R(2) * rd};
    double d[2] = {0.0, 0.0};
#pragma unroll
    for (int s = 0; s < 2; ++s)
      if (r2[s] > R(1e-15)) {
        const double ex = -cx * cbrt_t<R>(r2[s]);   // e_x(2 rho_s)
        e += 0.5 * ex;
        d[s] = ex / (3.0 * (double)r2[s]);         // e_x'(2 rho_s)
      }
    a += d[0];
    b += d[1];
  }
  const R rt = ru + rd;
  if ((xc & JRG_XC_LDA_C_VWN) && rt > R(1e-15)) {
    constexpr double kPi = 3.14159265358979323846;
    T z = (ru - rd) / rt;
    z = z > T(1) ? T(1) : (z < T(-1) ? T(-1) : z);
    const T x = sqrt(T(0.6203504908994001) / T(cbrt_t<R>(rt)));   // sqrt(rs), rs = (3/(4 pi rho))^(1/3)
    T ep, dep, ef, def, al, dal;
    vwn_fit<T>(x, T(0.0310907), T(3.72744), T(12.9352), T(-0.10498), T(6.15199081975907951), &ep, &dep);
    vwn_fit<T>(x, T(0.01554535), T(7.06042), T(18.0578), T(-0.32500), T(4.730926909560114), &ef, &def);
    vwn_fit<T>(x, T(-1.0 / (6.0 * kPi * kPi)), T(1.13107), T(13.0045), T(-0.0047584), T(7.123108917818118),
               &al, &dal);
    const T norm = T(0.5198420997897464);        // 2^(4/3) - 2
    const T fpp = T(1.7099209341613653);         // f''(0) = 4 / (9 (2^(1/3) - 1))
    const T cp = cbrt(T(1) + z), cm = cbrt(T(1) - z);
    const T fz = ((T(1) + z) * cp + (T(1) - z) * cm - T(2)) / norm;
    const T dfz = T(4) / T(3) * (cp - cm) / norm;
    const T z3 = z * z * z, z4 = z3 * z;
    const T ec = ep + al * fz * (T(1) - z4) / fpp + (ef - ep) * fz * z4;
    const T dx = dep + dal * fz * (T(1) - z4) / fpp + (def - dep) * fz * z4;
    const T dz = al / fpp * (dfz * (T(1) - z4) - T(4) * z3 * fz) + (ef - ep) * (dfz * z4 + T(4) * z3 * fz);
    // rho d eps / d rho_s = -(x/6) d eps/dx + (+-1 - z) d eps/dz
    const T t = -x / T(6) * dx;
    e += (double)ec;
    a += (double)(t + (T(1) - z) * dz) / (double)rt;
    b += (double)(t - (T(1) + z) * dz) / (double)rt;
  }
  *eps = e;
  *du = a;
  *dd = b;
}

// polarised form of k_potential: rho and vr are [2][ngrid]; the Hartree and
// external parts act on the total density, V_s = V_H + V_ext + eps + rho
// d eps / d rho_s; E_xc = vol/N sum eps rho, E_ext = vol/N sum V_ext rho
template <typename R>
__global__ void __launch_bounds__(kGridThreads) k_potential_pol(const R* __restrict__ rho,
                                                       const C_t<R>* __restrict__ vri, double vscale,
                                                       R* __restrict__ vr, double* __restrict__ slot_x,
                                                       long long ngrid, int xc, double pref,
                                                       const double* __restrict__ qscale,
                                                       const double* __restrict__ vext_r,
                                                       double* __restrict__ slot_e) {
  __shared__ double red[32];
  const double s = qscale ? *qscale : 1.0;
  double ex = 0.0, ee = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ngrid;
       i += (long long)gridDim.x * blockDim.x) {
    const double ru = s * (double)rho[i], rd = s * (double)rho[ngrid + i];
    const double rt = ru + rd;
    double eps, du, dd;
    lda_pol<R>((R)ru, (R)rd, xc, &eps, &du, &dd);
    ex += eps * rt;
    double ve = 0.0;
    if (vext_r) {
      ve = vext_r[i];
      ee += ve * rt;
    }
    const double base = (double)vri[i].x * vscale + eps + ve;
    vr[i] = (R)(base + rt * du);
    vr[ngrid + i] = (R)(base + rt * dd);
  }
  ex = block_sum(ex, red);
  if (threadIdx.x == 0) slot_x[blockIdx.x] = ex * pref;
  if (slot_e) {
    ee = block_sum(ee, red);
    if (threadIdx.x == 0) slot_e[blockIdx.x] = ee * pref;
  }
}

// polarised xc field of a [2][ngrid] density: eps (kohn_sham = 0, one grid),
// vxc_lda's eps + rho_s d eps / d rho_s per spin (kohn_sham = 1, two grids)
// or the derivative of eps rho, eps + rho d eps / d rho_s (kohn_sham = 2)
template <typename R>
__global__ void k_xc_field_pol(const R* __restrict__ rho, R* __restrict__ out, long long ngrid, int xc,
                               int kohn_sham) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ngrid;
       i += (long long)gridDim.x * blockDim.x) {
    const R ru = rho[i], rd = rho[ngrid + i];
    double eps, du, dd;
    lda_pol<R>(ru, rd, xc, &eps, &du, &dd);
    if (kohn_sham) {
      const double wu = kohn_sham == 2 ? (double)ru + (double)rd : (double)ru;
      const double wd = kohn_sham == 2 ? (double)ru + (double)rd : (double)rd;
      out[i] = (R)(eps + wu * du);
      out[ngrid + i] = (R)(eps + wd * dd);
    } else {
      out[i] = (R)eps;
    }
  }
}

// total density of a [2][ngrid] spin density
template <typename R>
__global__ void k_spin_total(const R* __restrict__ rho, R* __restrict__ out, long long ngrid) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ngrid;
       i += (long long)gridDim.x * blockDim.x)
    out[i] = (R)((double)rho[i] + (double)rho[ngrid + i]);
}

// ------------------------------------------------------------------------
// PBE (Perdew, Burke & Ernzerhof 1996), unpolarised, libxc parameters:
// f(rho, sigma) = rho (eps_x + eps_c) with exact partials f_rho, f_sigma from
// forward-mode dual numbers (value and the two partials carried together).
// Evaluated in FP64 on both precision paths.
// ------------------------------------------------------------------------
struct D2 {
  double v, r, s;   // value, d/d rho, d/d sigma
};
__device__ __forceinline__ D2 dconst(double c) { return D2{c, 0.0, 0.0}; }
__device__ __forceinline__ D2 operator+(D2 a, D2 b) { return D2{a.v + b.v, a.r + b.r, a.s + b.s}; }
__device__ __forceinline__ D2 operator-(D2 a, D2 b) { return D2{a.v - b.v, a.r - b.r, a.s - b.s}; }
__device__ __forceinline__ D2 operator*(D2 a, D2 b) {
  return D2{a.v * b.v, a.r * b.v + a.v * b.r, a.s * b.v + a.v * b.s};
}
__device__ __forceinline__ D2 operator/(D2 a, D2 b) {
  const double q = a.v / b.v;
  return D2{q, (a.r - q * b.r) / b.v, (a.s - q * b.s) / b.v};
}
__device__ __forceinline__ D2 operator*(double c, D2 a) { return D2{c * a.v, c * a.r, c * a.s}; }
__device__ __forceinline__ D2 operator+(double c, D2 a) { return D2{c + a.v, a.r, a.s}; }
__device__ __forceinline__ D2 operator-(double c, D2 a) { return D2{c - a.v, -a.r, -a.s}; }
__device__ __forceinline__ D2 dlog(D2 a) { return D2{log(a.v), a.r / a.v, a.s / a.v}; }
__device__ __forceinline__ D2 dexp(D2 a) { const double e = exp(a.v); return D2{e, e * a.r, e * a.s}; }
__device__ __forceinline__ D2 dsqrt(D2 a) {
  const double q = sqrt(a.v);
  return D2{q, 0.5 * a.r / q, 0.5 * a.s / q};
}
__device__ __forceinline__ D2 dcbrt(D2 a) {
  const double q = cbrt(a.v);
  return D2{q, q * a.r / (3.0 * a.v), q * a.s / (3.0 * a.v)};
}

__device__ D2 pbe_f(double rho_v, double sigma_v, int xc) {
  constexpr double kPi = 3.14159265358979323846;
  const D2 rho{rho_v, 1.0, 0.0}, sigma{sigma_v, 0.0, 1.0};
  const D2 kf = dcbrt((3.0 * kPi * kPi) * rho);
  D2 eps = dconst(0.0);
  if (xc & JRG_XC_GGA_X_PBE) {
    constexpr double kappa = 0.804, mu = 0.2195149727645171;
    const D2 s2 = sigma / (4.0 * (kf * kf) * (rho * rho));
    const D2 fx = (1.0 + kappa) - kappa * (dconst(1.0) / (1.0 + (mu / kappa) * s2));
    const double cx = -0.75 * cbrt(3.0 / kPi);
    eps = eps + cx * (dcbrt(rho) * fx);
  }
  if (xc & JRG_XC_GGA_C_PBE) {
    constexpr double A = 0.0310907, a1 = 0.21370, b1 = 7.5957, b2 = 3.5876, b3 = 1.6382,
                     b4 = 0.49294;
    constexpr double beta = 0.06672455060314922;
    const double gamma = (1.0 - log(2.0)) / (kPi * kPi);
    const D2 rs = dcbrt(dconst(3.0 / (4.0 * kPi)) / rho);
    const D2 srs = dsqrt(rs);
    const D2 den = (2.0 * A) * (b1 * srs + b2 * rs + b3 * (rs * srs) + b4 * (rs * rs));
    const D2 ec = (-2.0 * A) * ((1.0 + a1 * rs) * dlog(1.0 + dconst(1.0) / den));
    const D2 ks2 = (4.0 / kPi) * kf;
    const D2 t2 = sigma / (4.0 * ks2 * (rho * rho));
    const D2 aa = dconst(beta / gamma) / (dexp((-1.0 / gamma) * ec) - dconst(1.0));
    const D2 at2 = aa * t2;
    const D2 h = gamma * dlog(1.0 + (beta / gamma) * (t2 * (1.0 + at2) / (1.0 + at2 + at2 * at2)));
    eps = eps + ec + h;
  }
  return rho * eps;
}

// out = i G_a in * scale   (gradient component a in reciprocal space)
template <typename R>
__global__ void k_mul_ig(const C_t<R>* __restrict__ in, const double* __restrict__ gvec,
                         C_t<R>* __restrict__ out, int a, long long n, double scale) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double g = gvec[3 * i + a] * scale;
    const C_t<R> v = in[i];
    out[i] = cmk<C_t<R>>(-g * (double)v.y, g * (double)v.x);
  }
}

// Local PBE terms: sigma = |grad rho|^2 from the real parts of the three
// gradient grids; E_xc partials (vol/N sum f), vloc = f_rho, and the
// vector field h_a = f_sigma grad_a rho (0 where sigma = 0) written over the
// gradient grids.
// eps_only: write eps = f / rho (energy per particle) into vloc instead.
template <typename R>
__global__ void __launch_bounds__(256) k_gga_local(const R* __restrict__ rho, C_t<R>* __restrict__ g0,
                                                   C_t<R>* __restrict__ g1, C_t<R>* __restrict__ g2,
                                                   R* __restrict__ vloc, double* __restrict__ slot_x,
                                                   long long n, int xc, double pref, int eps_only,
                                                   const double* __restrict__ qscale,
                                                   const double* __restrict__ vext_r,
                                                   double* __restrict__ slot_e) {
  __shared__ double red[32];
  // renormalised density s rho and its gradients (ChargeFix), 1 without qscale
  const double s = qscale ? *qscale : 1.0;
  double ex = 0.0, ee = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double r = s * (double)rho[i];
    if (vext_r) ee += vext_r[i] * r;
    const double d0 = s * (double)g0[i].x, d1 = s * (double)g1[i].x, d2 = s * (double)g2[i].x;
    const double sig = d0 * d0 + d1 * d1 + d2 * d2;
    double fr = 0.0, fs = 0.0, fe = 0.0;
    if (r > 1e-15) {
      const D2 f = pbe_f(r, sig, xc);
      ex += f.v;
      fr = f.r;
      fs = sig > 0.0 ? f.s : 0.0;
      fe = f.v / r;
    }
    vloc[i] = (R)(eps_only ? fe : fr);
    g0[i] = cmk<C_t<R>>(fs * d0, 0.0);
    g1[i] = cmk<C_t<R>>(fs * d1, 0.0);
    g2[i] = cmk<C_t<R>>(fs * d2, 0.0);
  }
  ex = block_sum(ex, red);
  if (threadIdx.x == 0 && slot_x) slot_x[blockIdx.x] = ex * pref;
  if (slot_e) {
    ee = block_sum(ee, red);
    if (threadIdx.x == 0) slot_e[blockIdx.x] = ee * pref;
  }
}

// g0 = scale * sum_a i G_a h_a   (divergence in reciprocal space)
template <typename R>
__global__ void k_div_g(C_t<R>* __restrict__ g0, const C_t<R>* __restrict__ g1,
                        const C_t<R>* __restrict__ g2, const double* __restrict__ gvec, long long n,
                        double scale) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const C_t<R> h[3] = {g0[i], g1[i], g2[i]};
    double x = 0.0, y = 0.0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const double g = gvec[3 * i + a];
      x -= g * (double)h[a].y;
      y += g * (double)h[a].x;
    }
    g0[i] = cmk<C_t<R>>(x * scale, y * scale);
  }
}

// vr = Re(vri) * vscale + vr - 2 Re(div) + V_ext(r)   (vr holds f_rho on
// entry; vri and vext_r may be null)
template <typename R>
__global__ void k_potential_gga(const C_t<R>* __restrict__ vri, double vscale, R* __restrict__ vr,
                                const C_t<R>* __restrict__ div, long long n,
                                const double* __restrict__ vext_r) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    double base = vri ? (double)vri[i].x * vscale : 0.0;
    if (vext_r) base += vext_r[i];
    vr[i] = (R)(base + (double)vr[i] - 2.0 * (double)div[i].x);
  }
}

// For the density s rho (s = *qscale, 1 when null): V(r) = Re(vri)*vscale +
// v_xc + V_ext(r) (when vr is given), E_xc = vol/N sum eps s rho and, with
// vext_r, E_ext = vol/N sum V_ext(r) s rho (FP64 table, real-space form).
template <typename R>
__global__ void __launch_bounds__(kGridThreads, 4) k_potential(const R* __restrict__ rho,
                                                   const C_t<R>* __restrict__ vri, double vscale,
                                                   R* __restrict__ vr, double* __restrict__ slot_x,
                                                   long long ngrid, int xc, double pref,
                                                   const double* __restrict__ qscale,
                                                   const double* __restrict__ vext_r,
                                                   double* __restrict__ slot_e) {
  __shared__ double red[32];
  const double s = qscale ? *qscale : 1.0;
  double ex = 0.0, ee = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ngrid;
       i += (long long)gridDim.x * blockDim.x) {
    // the energy sums take s rho in FP64 (s - 1 is ~1e-8, below FP32
    // resolution); eps and v_xc are evaluated at its FP32 rounding
    const double r = s * (double)rho[i];
    const R rr = (R)r;
    double eps, v;
    lda_eps_v_t<R>(rr, xc, &eps, &v);
    ex += eps * r;
    double ve = 0.0;
    if (vext_r) {
      ve = vext_r[i];
      ee += ve * r;
    }
    if (vr) vr[i] = (R)((double)vri[i].x * vscale + v + ve);
  }
  ex = block_sum(ex, red);
  if (threadIdx.x == 0) slot_x[blockIdx.x] = ex * pref;
  if (slot_e) {
    ee = block_sum(ee, red);
    if (threadIdx.x == 0) slot_e[blockIdx.x] = ee * pref;
  }
}

// xc energy density (kohn_sham = 0) or v_xc (kohn_sham = 1) on the grid
template <typename R>
__global__ void k_xc_field(const R* __restrict__ rho, R* __restrict__ out, long long ngrid, int xc,
                           int kohn_sham) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ngrid;
       i += (long long)gridDim.x * blockDim.x) {
    double eps, v;
    lda_eps_v_t<R>(rho[i], xc, &eps, &v);
    out[i] = (R)(kohn_sham ? v : eps);
  }
}

// real part of a complex grid times a factor
template <typename R>
__global__ void k_real_part(const C_t<R>* __restrict__ in, R* __restrict__ out, long long n,
                            double fac) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    out[i] = (R)((double)in[i].x * fac);
}

// reciprocal Hartree potential (x fac) of a density transform
template <typename R>
__global__ void k_hartree_g(const C_t<R>* __restrict__ rhog, const double* __restrict__ ginv,
                            C_t<R>* __restrict__ out, long long n, double fac) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double g = ginv[i] * fac;
    C_t<R> o;
    o.x = (R)(g * rhog[i].x);
    o.y = (R)(g * rhog[i].y);
    out[i] = o;
  }
}

// kinetic energy per band: f * sum_g tk[k][g] |c[b][g]|^2, one block per band
template <typename R>
__global__ void __launch_bounds__(256) k_kinetic(const C_t<R>* __restrict__ coef,
                                                 const double* __restrict__ tk,
                                                 const double* __restrict__ occ,
                                                 double* __restrict__ slot, double* __restrict__ ekin,
                                                 int ng, int nb, int nk) {
  __shared__ double red[32];
  const int band = blockIdx.x;           // global (s, k, b)
  const int k = (band / nb) % nk;
  const C_t<R>* c = coef + (size_t)band * ng;
  const double* t = tk + (size_t)k * ng;
  R part = (R)0;
  for (int g = threadIdx.x; g < ng; g += blockDim.x) {
    const R x = c[g].x, y = c[g].y;
    part += (R)t[g] * (x * x + y * y);
  }
  const double acc = block_sum((double)part, red);
  if (threadIdx.x == 0) {
    slot[band] = acc * occ[band];
    if (ekin) ekin[band] = acc;
  }
}

// per band: FP64 sum of the kinetic block partials (precision R) of the
// forward rotation -> ekin[band], slot[band] = occ[band] * ekin[band]
template <typename R>
__global__ void k_kin_reduce(const R* __restrict__ part, int nblk, int nb, int nbt,
                             const double* __restrict__ occ, double* __restrict__ slot,
                             double* __restrict__ ekin) {
  // one warp per band: lanes take every 32nd block partial, then a shuffle sum
  const int band = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (band >= nbt) return;
  const int sk = band / nb, b = band - sk * nb;
  const R* p = part + (size_t)sk * nblk * nb + b;
  double acc = 0.0;
  for (int i = lane; i < nblk; i += 32) acc += (double)p[(size_t)i * nb];
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
  if (lane == 0) {
    slot[band] = acc * occ[band];
    if (ekin) ekin[band] = acc;
  }
}

constexpr int kSumThreads = 512;
// energies[t] = sum of its slots, t = 0..3; energies[4] = total
// energies[t] = sum of slots [slot_begin[t], slot_begin[t+1]) for t < nterms;
// with extra_term >= 0 the range [slot_begin[nterms], slot_begin[nterms+1])
// (the nonlocal pseudopotential energy) is added to term extra_term and also
// reported alone in energies[nterms + 3]; energies[nterms] = total.
__global__ void __launch_bounds__(kSumThreads) k_sum_slots(const double* __restrict__ slots,
                                                           const int* __restrict__ slot_begin,
                                                           double* __restrict__ energies, int nterms,
                                                           const int* __restrict__ flags, int extra_term) {
  // every thread sums its share of all ranges at once, then one two-level
  // reduction of the (nterms + 1) partial sums (one barrier)
  constexpr int kMaxT = 5;
  __shared__ double part[kSumThreads / 32][kMaxT];
  const int nt = nterms + (extra_term >= 0 ? 1 : 0);   // the extra range last
  double acc[kMaxT];
#pragma unroll
  for (int t = 0; t < kMaxT; ++t) {
    acc[t] = 0.0;
    if (t < nt)
      for (int i = slot_begin[t] + threadIdx.x; i < slot_begin[t + 1]; i += blockDim.x) acc[t] += slots[i];
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int t = 0; t < kMaxT; ++t) {
    double v = acc[t];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    if (lane == 0) part[wid][t] = v;
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int t = 0; t < kMaxT; ++t) {
      double v = lane < kSumThreads / 32 ? part[lane][t] : 0.0;
      for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
      acc[t] = v;
    }
    if (lane == 0) {
      const double extra = extra_term >= 0 ? acc[nterms] : 0.0;
      double tot = 0.0;
      for (int t = 0; t < nterms; ++t) {
        const double e = acc[t] + (t == extra_term ? extra : 0.0);
        energies[t] = e;
        tot += e;
      }
      energies[nterms] = tot;
      // the largest Gram condition estimate of the call (note_condition)
      energies[nterms + 1] = flags ? __longlong_as_double(*reinterpret_cast<const long long*>(flags + 2)) : 0.0;
      energies[nterms + 2] = flags ? (double)flags[0] : 0.0;
      energies[nterms + 3] = extra;
    }
  }
}

// band trace of a fixed Hamiltonian: out[0] = sum over (s,k,b) of Re A_bb
// with A = C^H g_C (g_C = w H c), out[1] = the kinetic part (slots [0, nkin))
__global__ void k_band_trace_sums(const double2* __restrict__ A, int nsk, int nb,
                                  const double* __restrict__ slots, int nkin, double* __restrict__ out) {
  __shared__ double red[32];
  double a = 0.0;
  for (int i = threadIdx.x; i < nsk * nb; i += blockDim.x) {
    const int sk = i / nb, b = i - sk * nb;
    a += A[((size_t)sk * nb + b) * nb + b].x;
  }
  a = block_sum(a, red);
  double k = 0.0;
  for (int i = threadIdx.x; i < nkin; i += blockDim.x) k += slots[i];
  k = block_sum(k, red);
  if (threadIdx.x == 0) {
    out[0] = a;
    out[1] = k;
  }
}

// ------------------------------------------------------------------------
// geometry tables (FP64): G vectors, 4 pi/|G|^2, external potential
//   Vext(G) = -(4 pi N/vol) sum_a Z_a exp(-i G.R_a)/(|G|^2 + 1e-10), 0 at G=0
// ------------------------------------------------------------------------
__device__ __forceinline__ int fftfreq_int(int i, int n) { return (i < (n + 1) / 2) ? i : i - n; }

template <typename R>
__global__ void k_geometry_tables(double* __restrict__ gvec, double* __restrict__ ginv,
                                  C_t<R>* __restrict__ vext, double2* __restrict__ vext64,
                                  const double* __restrict__ recip,
                                  const double* __restrict__ pos, const double* __restrict__ chg,
                                  int natom, int nx, int ny, int nz, double vol) {
  const long long n = (long long)nx * ny * nz;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int ix = (int)(i / ((long long)ny * nz));
    const int iy = (int)((i / nz) % ny);
    const int iz = (int)(i % nz);
    const double m0 = fftfreq_int(ix, nx), m1 = fftfreq_int(iy, ny), m2 = fftfreq_int(iz, nz);
    double g[3];
    for (int d = 0; d < 3; ++d) g[d] = m0 * recip[0 + d] + m1 * recip[3 + d] + m2 * recip[6 + d];
    gvec[3 * i + 0] = g[0]; gvec[3 * i + 1] = g[1]; gvec[3 * i + 2] = g[2];
    const double g2 = g[0] * g[0] + g[1] * g[1] + g[2] * g[2];
    const bool zero = (i == 0);
    ginv[i] = zero ? 0.0 : 4.0 * 3.14159265358979323846 / g2;
    double sx = 0.0, sy = 0.0;
    if (!zero) {
      for (int a = 0; a < natom; ++a) {
        const double ph = g[0] * pos[3 * a] + g[1] * pos[3 * a + 1] + g[2] * pos[3 * a + 2];
        double sn, cs;
        sincos(ph, &sn, &cs);
        sx += chg[a] * cs;
        sy -= chg[a] * sn;
      }
      const double f = -4.0 * 3.14159265358979323846 * (double)n / vol / (g2 + 1e-10);
      sx *= f; sy *= f;
    }
    vext[i] = cmk<C_t<R>>(sx, sy);
    if (vext64) vext64[i] = make_double2(sx, sy);
  }
}

// ------------------------------------------------------------------------
// Ewald nuclear repulsion (FP64)
// real space:  1/2 sum_ij Z_i Z_j sum_t erfc(eta d)/d,  d = |R_j - R_i - t| (d <= 1e-9 skipped)
// reciprocal:  (4 pi/vol) 1/2 sum_{G != 0} exp(-|G|^2/(4 eta^2))/|G|^2 |sum_i Z_i exp(i G.R_i)|^2
// ------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_ewald_real(const double* __restrict__ cell,
                                                    const double* __restrict__ pos,
                                                    const double* __restrict__ chg, int natom,
                                                    int nt, double eta, double* __restrict__ slot) {
  __shared__ double red[32];
  const long long ntot = (long long)nt * nt * nt;
  double acc = 0.0;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < ntot;
       t += (long long)gridDim.x * blockDim.x) {
    const int a0 = fftfreq_int((int)(t / ((long long)nt * nt)), nt);
    const int a1 = fftfreq_int((int)((t / nt) % nt), nt);
    const int a2 = fftfreq_int((int)(t % nt), nt);
    double tv[3];
    for (int d = 0; d < 3; ++d) tv[d] = a0 * cell[d] + a1 * cell[3 + d] + a2 * cell[6 + d];
    for (int i = 0; i < natom; ++i) {
      for (int j = 0; j < natom; ++j) {
        const double dx = pos[3 * j] - pos[3 * i] - tv[0];
        const double dy = pos[3 * j + 1] - pos[3 * i + 1] - tv[1];
        const double dz = pos[3 * j + 2] - pos[3 * i + 2] - tv[2];
        const double d = sqrt(dx * dx + dy * dy + dz * dz + 1e-20);
        if (d > 1e-9) acc += chg[i] * chg[j] * erfc(eta * d) / d;
      }
    }
  }
  acc = block_sum(acc, red);
  if (threadIdx.x == 0) slot[blockIdx.x] = 0.5 * acc;
}

__global__ void __launch_bounds__(256) k_ewald_recip(const double* __restrict__ gvec,
                                                     const double* __restrict__ pos,
                                                     const double* __restrict__ chg, int natom,
                                                     long long ngrid, double eta, double vol,
                                                     double* __restrict__ slot) {
  __shared__ double red[32];
  double acc = 0.0;
  for (long long i = 1 + blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ngrid;
       i += (long long)gridDim.x * blockDim.x) {
    const double gx = gvec[3 * i], gy = gvec[3 * i + 1], gz = gvec[3 * i + 2];
    const double g2 = gx * gx + gy * gy + gz * gz;
    const double kern = exp(-g2 / 4.0 / (eta * eta)) / g2;
    if (kern == 0.0) continue;
    double sx = 0.0, sy = 0.0;
    for (int a = 0; a < natom; ++a) {
      double sn, cs;
      sincos(gx * pos[3 * a] + gy * pos[3 * a + 1] + gz * pos[3 * a + 2], &sn, &cs);
      sx += chg[a] * cs;
      sy += chg[a] * sn;
    }
    acc += kern * (sx * sx + sy * sy);
  }
  acc = block_sum(acc, red);
  if (threadIdx.x == 0) slot[blockIdx.x] = 0.5 * 4.0 * 3.14159265358979323846 / vol * acc;
}

__global__ void k_ewald_finish(const double* __restrict__ slots, int nslots, const double* __restrict__ chg,
                               int natom, double eta, double vol, double* __restrict__ out) {
  __shared__ double red[32];
  double acc = 0.0;
  for (int i = threadIdx.x; i < nslots; i += blockDim.x) acc += slots[i];
  acc = block_sum(acc, red);
  if (threadIdx.x == 0) {
    double z2 = 0.0, z = 0.0;
    for (int a = 0; a < natom; ++a) { z2 += chg[a] * chg[a]; z += chg[a]; }
    const double pi = 3.14159265358979323846;
    double self = -z2 * 2.0 * eta / sqrt(pi) / 2.0;
    self -= z * z * pi / (eta * eta) / vol / 2.0;
    out[0] = acc + self;
  }
}

// ------------------------------------------------------------------------
// Adam (optax placement of eps) with optional elementwise update scale
// ------------------------------------------------------------------------

template <typename R>
__global__ void k_adam(R* __restrict__ p, const R* __restrict__ g, R* __restrict__ m,
                       R* __restrict__ v, const float* __restrict__ scale, long long n, R lr, R b1,
                       R b2, R c1, R c2, R eps, const int* __restrict__ guard,
                       const double* __restrict__ coefs) {
  // guard: the status word of the energy call that made g; non-zero (a
  // Cholesky breakdown) leaves the parameters and moments unchanged
  if (guard && *guard) return;
  // coefs: bias corrections (c1, c2) read from device memory instead of the
  // arguments (a step replayed from a CUDA graph, the step count on device)
  if (coefs) { c1 = (R)coefs[0]; c2 = (R)coefs[1]; }
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if constexpr (sizeof(R) == 4) {
    // four elements per thread with 16-byte accesses when the buffers are aligned
    const bool vec = (((uintptr_t)p | (uintptr_t)g | (uintptr_t)m | (uintptr_t)v |
                       (uintptr_t)scale) & 15) == 0;
    const long long n4 = vec ? n / 4 : 0;
    for (long long q = tid; q < n4; q += stride) {
      float4 pp = reinterpret_cast<float4*>(p)[q];
      const float4 gg = reinterpret_cast<const float4*>(g)[q];
      float4 mm = reinterpret_cast<float4*>(m)[q];
      float4 vv = reinterpret_cast<float4*>(v)[q];
      float4 u;
      u.x = adam_one<float>(gg.x, mm.x, vv.x, lr, b1, b2, c1, c2, eps);
      u.y = adam_one<float>(gg.y, mm.y, vv.y, lr, b1, b2, c1, c2, eps);
      u.z = adam_one<float>(gg.z, mm.z, vv.z, lr, b1, b2, c1, c2, eps);
      u.w = adam_one<float>(gg.w, mm.w, vv.w, lr, b1, b2, c1, c2, eps);
      if (scale) {
        const float4 s = reinterpret_cast<const float4*>(scale)[q];
        u.x *= s.x; u.y *= s.y; u.z *= s.z; u.w *= s.w;
      }
      pp.x += u.x; pp.y += u.y; pp.z += u.z; pp.w += u.w;
      reinterpret_cast<float4*>(p)[q] = pp;
      reinterpret_cast<float4*>(m)[q] = mm;
      reinterpret_cast<float4*>(v)[q] = vv;
    }
    for (long long i = 4 * n4 + tid; i < n; i += stride) {
      R mi = m[i], vi = v[i];
      R u = adam_one<R>(g[i], mi, vi, lr, b1, b2, c1, c2, eps);
      m[i] = mi; v[i] = vi;
      if (scale) u *= (R)scale[i];
      p[i] += u;
    }
  } else {
    for (long long i = tid; i < n; i += stride) {
      R mi = m[i], vi = v[i];
      R u = adam_one<R>(g[i], mi, vi, lr, b1, b2, c1, c2, eps);
      m[i] = mi; v[i] = vi;
      if (scale) u *= (R)scale[i];
      p[i] += u;
    }
  }
}

// Direct FP64 inverse DFT along one axis of an [n0][n1][n2] grid (plan setup
// only, no shared-memory size limit): out[.., k, ..] = sum_j in[.., j, ..]
// exp(+2 pi i j k / n), tw[t] = exp(-2 pi i t / n) of that axis.
__global__ void k_dft_axis_inv_f64(const double2* __restrict__ in, double2* __restrict__ out, int n0,
                                   int n1, int n2, int axis, const double2* __restrict__ tw) {
  const long long total = (long long)n0 * n1 * n2;
  const int n = axis == 0 ? n0 : (axis == 1 ? n1 : n2);
  const long long stride = axis == 0 ? (long long)n1 * n2 : (axis == 1 ? n2 : 1);
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const int k = (int)((idx / stride) % n);
    const long long base = idx - (long long)k * stride;
    double ax = 0.0, ay = 0.0;
    for (int j = 0; j < n; ++j) {
      const double2 w = tw[(int)(((long long)j * k) % n)];
      const double2 v = in[base + (long long)j * stride];
      ax += v.x * w.x + v.y * w.y;    // v * conj(w)
      ay += v.y * w.x - v.x * w.y;
    }
    out[idx] = make_double2(ax, ay);
  }
}

int launch_dft_axis_inv_f64(const double2* in, double2* out, int n0, int n1, int n2, int axis,
                            const double2* tw, cudaStream_t st) {
  k_dft_axis_inv_f64<<<1024, 256, 0, st>>>(in, out, n0, n1, n2, axis, tw);
  JRG_LAUNCH_CHECK("k_dft_axis_inv_f64");
  return JRG_OK;
}

// twiddle table W_n^t = exp(-2 pi i t/n), t < n, evaluated in FP64 (FP32
// tables: balanced_twiddle)
template <typename R>
__global__ void k_twiddles(int n, C_t<R>* __restrict__ out) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    double s, c;
    sincospi(-2.0 * (double)t / (double)n, &s, &c);
    if constexpr (sizeof(R) == 4) out[t] = balanced_twiddle(c, s);
    else out[t] = cmk<C_t<R>>(c, s);
  }
}

// ------------------------------------------------------------------------
// launch helpers
// ------------------------------------------------------------------------
static inline unsigned grid_for(long long n, int per = 256, int cap = 4096) {
  long long b = (n + per - 1) / per;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (unsigned)b;
}

template <typename R>
int launch_reduce_density(const void* part, void* rho, int groups_per_spin, int ns, long long ngrid,
                          const double* gscale, double* qpart, cudaStream_t st) {
  constexpr int W = Vec16<R>::n;
  if (ngrid % W == 0 && ((reinterpret_cast<uintptr_t>(part) | reinterpret_cast<uintptr_t>(rho)) & 15) == 0) {
    k_reduce_density_v<R><<<kQParts, 256, 0, st>>>(reinterpret_cast<const R*>(part), reinterpret_cast<R*>(rho),
                                                   groups_per_spin, ns, ngrid, gscale, qpart);
    JRG_LAUNCH_CHECK("k_reduce_density_v");
    return JRG_OK;
  }
  k_reduce_density<R><<<kQParts, 256, 0, st>>>(reinterpret_cast<const R*>(part), reinterpret_cast<R*>(rho),
                                               groups_per_spin, ns, ngrid, gscale, qpart);
  JRG_LAUNCH_CHECK("k_reduce_density");
  return JRG_OK;
}

template <typename R>
int launch_recip_terms(const void* rhog, const double* ginv, void* vg, double* slot_h, int nblocks,
                       long long ngrid, double pref, const ChargeFix& cf, cudaStream_t st) {
  k_recip_terms<R><<<nblocks, kGridThreads, 0, st>>>(reinterpret_cast<const C_t<R>*>(rhog), ginv,
                                            reinterpret_cast<C_t<R>*>(vg), slot_h, ngrid, pref, cf);
  JRG_LAUNCH_CHECK("k_recip_terms");
  return JRG_OK;
}

template <typename R>
int launch_potential(const void* rho, const void* vri, double vscale, void* vr, double* slot_x,
                     int nblocks, long long ngrid, int xc, double pref, const double* qscale,
                     const double* vext_r, double* slot_e, cudaStream_t st) {
  k_potential<R><<<nblocks, kGridThreads, 0, st>>>(reinterpret_cast<const R*>(rho),
                                          reinterpret_cast<const C_t<R>*>(vri), vscale,
                                          reinterpret_cast<R*>(vr), slot_x, ngrid, xc, pref, qscale,
                                          vext_r, slot_e);
  JRG_LAUNCH_CHECK("k_potential");
  return JRG_OK;
}

template <typename R>
int launch_potential_pol(const void* rho, const void* vri, double vscale, void* vr, double* slot_x,
                         int nblocks, long long ngrid, int xc, double pref, const double* qscale,
                         const double* vext_r, double* slot_e, cudaStream_t st) {
  k_potential_pol<R><<<nblocks, kGridThreads, 0, st>>>(reinterpret_cast<const R*>(rho),
                                              reinterpret_cast<const C_t<R>*>(vri), vscale,
                                              reinterpret_cast<R*>(vr), slot_x, ngrid, xc, pref, qscale,
                                              vext_r, slot_e);
  JRG_LAUNCH_CHECK("k_potential_pol");
  return JRG_OK;
}

template <typename R>
int launch_xc_field_pol(const void* rho, void* out, long long ngrid, int xc, int ks, cudaStream_t st) {
  k_xc_field_pol<R><<<grid_for(ngrid), 256, 0, st>>>(reinterpret_cast<const R*>(rho),
                                                     reinterpret_cast<R*>(out), ngrid, xc, ks);
  JRG_LAUNCH_CHECK("k_xc_field_pol");
  return JRG_OK;
}

template <typename R>
int launch_spin_total(const void* rho, void* out, long long ngrid, cudaStream_t st) {
  k_spin_total<R><<<grid_for(ngrid), 256, 0, st>>>(reinterpret_cast<const R*>(rho),
                                                   reinterpret_cast<R*>(out), ngrid);
  JRG_LAUNCH_CHECK("k_spin_total");
  return JRG_OK;
}

template <typename R>
int launch_xc_field(const void* rho, void* out, long long ngrid, int xc, int ks, cudaStream_t st) {
  k_xc_field<R><<<grid_for(ngrid), 256, 0, st>>>(reinterpret_cast<const R*>(rho),
                                                 reinterpret_cast<R*>(out), ngrid, xc, ks);
  JRG_LAUNCH_CHECK("k_xc_field");
  return JRG_OK;
}

template <typename R>
int launch_real_part(const void* in, void* out, long long n, double fac, cudaStream_t st) {
  k_real_part<R><<<grid_for(n), 256, 0, st>>>(reinterpret_cast<const C_t<R>*>(in),
                                              reinterpret_cast<R*>(out), n, fac);
  JRG_LAUNCH_CHECK("k_real_part");
  return JRG_OK;
}

template <typename R>
int launch_hartree_g(const void* rhog, const double* ginv, void* out, long long n, double fac,
                     cudaStream_t st) {
  k_hartree_g<R><<<grid_for(n), 256, 0, st>>>(reinterpret_cast<const C_t<R>*>(rhog), ginv,
                                               reinterpret_cast<C_t<R>*>(out), n, fac);
  JRG_LAUNCH_CHECK("k_hartree_g");
  return JRG_OK;
}

template <typename R>
int launch_kinetic(const void* coef, const double* tk, const double* occ, double* slot, double* ekin,
                   int nbands, int ng, int nb, int nk, cudaStream_t st) {
  k_kinetic<R><<<nbands, 256, 0, st>>>(reinterpret_cast<const C_t<R>*>(coef), tk, occ, slot, ekin, ng,
                                       nb, nk);
  JRG_LAUNCH_CHECK("k_kinetic");
  return JRG_OK;
}

template <typename R>
int launch_mul_ig(const void* in, const double* gvec, void* out, int a, long long n, double scale,
                  cudaStream_t st) {
  k_mul_ig<R><<<grid_for(n), 256, 0, st>>>(reinterpret_cast<const C_t<R>*>(in), gvec,
                                           reinterpret_cast<C_t<R>*>(out), a, n, scale);
  JRG_LAUNCH_CHECK("k_mul_ig");
  return JRG_OK;
}

template <typename R>
int launch_gga_local(const void* rho, void* g0, void* g1, void* g2, void* vloc, double* slot_x,
                     int nblocks, long long n, int xc, double pref, int eps_only, const double* qscale,
                     const double* vext_r, double* slot_e, cudaStream_t st) {
  k_gga_local<R><<<nblocks, 256, 0, st>>>(reinterpret_cast<const R*>(rho), reinterpret_cast<C_t<R>*>(g0),
                                          reinterpret_cast<C_t<R>*>(g1), reinterpret_cast<C_t<R>*>(g2),
                                          reinterpret_cast<R*>(vloc), slot_x, n, xc, pref, eps_only,
                                          qscale, vext_r, slot_e);
  JRG_LAUNCH_CHECK("k_gga_local");
  return JRG_OK;
}

template <typename R>
int launch_div_g(void* g0, const void* g1, const void* g2, const double* gvec, long long n,
                 double scale, cudaStream_t st) {
  k_div_g<R><<<grid_for(n), 256, 0, st>>>(reinterpret_cast<C_t<R>*>(g0), reinterpret_cast<const C_t<R>*>(g1),
                                          reinterpret_cast<const C_t<R>*>(g2), gvec, n, scale);
  JRG_LAUNCH_CHECK("k_div_g");
  return JRG_OK;
}

template <typename R>
int launch_potential_gga(const void* vri, double vscale, void* vr, const void* div, long long n,
                         const double* vext_r, cudaStream_t st) {
  k_potential_gga<R><<<grid_for(n), 256, 0, st>>>(reinterpret_cast<const C_t<R>*>(vri), vscale,
                                                  reinterpret_cast<R*>(vr),
                                                  reinterpret_cast<const C_t<R>*>(div), n, vext_r);
  JRG_LAUNCH_CHECK("k_potential_gga");
  return JRG_OK;
}

int launch_kin_reduce(int prec, const void* part, int nblk, int nb, int nbt, const double* occ,
                      double* slot, double* ekin, cudaStream_t st) {
  if (prec == 64)
    k_kin_reduce<double><<<(nbt * 32 + 255) / 256, 256, 0, st>>>(reinterpret_cast<const double*>(part), nblk,
                                                            nb, nbt, occ, slot, ekin);
  else
    k_kin_reduce<float><<<(nbt * 32 + 255) / 256, 256, 0, st>>>(reinterpret_cast<const float*>(part), nblk, nb,
                                                           nbt, occ, slot, ekin);
  JRG_LAUNCH_CHECK("k_kin_reduce");
  return JRG_OK;
}

int launch_band_trace_sums(const double2* A, int nsk, int nb, const double* slots, int nkin,
                          double* out, cudaStream_t st) {
  k_band_trace_sums<<<1, 256, 0, st>>>(A, nsk, nb, slots, nkin, out);
  JRG_LAUNCH_CHECK("k_band_trace_sums");
  return JRG_OK;
}

int launch_sum_slots(const double* slots, const int* slot_begin, double* energies, int nterms,
                     const int* flags, int extra_term, cudaStream_t st) {
  if (nterms < 1 || nterms + (extra_term >= 0 ? 1 : 0) > 5) return fail(JRG_ERR_INVALID, "k_sum_slots: too many terms");
  k_sum_slots<<<1, kSumThreads, 0, st>>>(slots, slot_begin, energies, nterms, flags, extra_term);
  JRG_LAUNCH_CHECK("k_sum_slots");
  return JRG_OK;
}

template <typename R>
int launch_geometry_tables(double* gvec, double* ginv, void* vext, double2* vext64, const double* recip,
                           const double* pos, const double* chg, int natom, int nx, int ny, int nz,
                           double vol, cudaStream_t st) {
  k_geometry_tables<R><<<grid_for((long long)nx * ny * nz), 256, 0, st>>>(
      gvec, ginv, reinterpret_cast<C_t<R>*>(vext), vext64, recip, pos, chg, natom, nx, ny, nz, vol);
  JRG_LAUNCH_CHECK("k_geometry_tables");
  return JRG_OK;
}

int launch_ewald(const double* cell, const double* gvec, const double* pos, const double* chg,
                 int natom, int nt, long long ngrid, double eta, double vol, double* slots,
                 int nslots_half, double* out, cudaStream_t st) {
  k_ewald_real<<<nslots_half, 256, 0, st>>>(cell, pos, chg, natom, nt, eta, slots);
  JRG_LAUNCH_CHECK("k_ewald_real");
  k_ewald_recip<<<nslots_half, 256, 0, st>>>(gvec, pos, chg, natom, ngrid, eta, vol,
                                             slots + nslots_half);
  JRG_LAUNCH_CHECK("k_ewald_recip");
  k_ewald_finish<<<1, 256, 0, st>>>(slots, 2 * nslots_half, chg, natom, eta, vol, out);
  JRG_LAUNCH_CHECK("k_ewald_finish");
  return JRG_OK;
}

template <typename R>
int launch_adam(void* p, const void* g, void* m, void* v, const float* scale, long long n, double lr,
                double b1, double b2, double c1, double c2, double eps, cudaStream_t st,
                const int* guard, const double* coefs) {
  k_adam<R><<<grid_for((n + 3) / 4, 256, 152 * 16), 256, 0, st>>>(
      reinterpret_cast<R*>(p), reinterpret_cast<const R*>(g), reinterpret_cast<R*>(m),
      reinterpret_cast<R*>(v), scale, n, (R)lr, (R)b1, (R)b2, (R)c1, (R)c2, (R)eps, guard, coefs);
  JRG_LAUNCH_CHECK("k_adam");
  return JRG_OK;
}

int launch_lda(int prec, long long n, int xc, int ks, const void* rho, void* out, cudaStream_t st) {
  if (prec == 64) return launch_xc_field<double>(rho, out, n, xc, ks, st);
  return launch_xc_field<float>(rho, out, n, xc, ks, st);
}

int launch_lda_pol(int prec, long long n, int xc, int ks, const void* rho, void* out, cudaStream_t st) {
  if (prec == 64) return launch_xc_field_pol<double>(rho, out, n, xc, ks, st);
  return launch_xc_field_pol<float>(rho, out, n, xc, ks, st);
}

int launch_twiddles(int n, int prec, void* out, cudaStream_t st) {
  if (prec == 64) k_twiddles<double><<<1, 128, 0, st>>>(n, reinterpret_cast<double2*>(out));
  else k_twiddles<float><<<1, 128, 0, st>>>(n, reinterpret_cast<float2*>(out));
  JRG_LAUNCH_CHECK("k_twiddles");
  return JRG_OK;
}

#define JRG_INST_GRID(R)                                                                        \
  template int launch_reduce_density<R>(const void*, void*, int, int, long long, const double*, \
                                        double*, cudaStream_t);                                  \
  template int launch_recip_terms<R>(const void*, const double*, void*, double*, int, long long,  \
                                     double, const ChargeFix&, cudaStream_t);                    \
  template int launch_potential<R>(const void*, const void*, double, void*, double*, int,         \
                                   long long, int, double, const double*, const double*, double*, \
                                   cudaStream_t);                                               \
  template int launch_xc_field<R>(const void*, void*, long long, int, int, cudaStream_t);         \
  template int launch_potential_pol<R>(const void*, const void*, double, void*, double*, int,     \
                                       long long, int, double, const double*, const double*,     \
                                       double*, cudaStream_t);                                  \
  template int launch_spin_total<R>(const void*, void*, long long, cudaStream_t);                 \
  template int launch_real_part<R>(const void*, void*, long long, double, cudaStream_t);          \
  template int launch_hartree_g<R>(const void*, const double*, void*, long long, double,          \
                                   cudaStream_t);                                               \
  template int launch_kinetic<R>(const void*, const double*, const double*, double*, double*, int, \
                                 int, int, int, cudaStream_t);                                  \
  template int launch_geometry_tables<R>(double*, double*, void*, double2*, const double*, const double*, \
                                         const double*, int, int, int, int, double, cudaStream_t); \
  template int launch_mul_ig<R>(const void*, const double*, void*, int, long long, double,        \
                                cudaStream_t);                                                  \
  template int launch_gga_local<R>(const void*, void*, void*, void*, void*, double*, int,          \
                                   long long, int, double, int, const double*, const double*,   \
                                   double*, cudaStream_t);                                      \
  template int launch_div_g<R>(void*, const void*, const void*, const double*, long long, double, \
                               cudaStream_t);                                                   \
  template int launch_potential_gga<R>(const void*, double, void*, const void*, long long,        \
                                       const double*, cudaStream_t);                            \
  template int launch_adam<R>(void*, const void*, void*, void*, const float*, long long, double,  \
                              double, double, double, double, double, cudaStream_t, const int*,  \
                              const double*);
JRG_INST_GRID(float)
JRG_INST_GRID(double)

}  // namespace jrg
