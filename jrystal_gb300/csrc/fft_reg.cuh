// Register-resident FFTs of compile-time length for the slab kernels.
//
// A line of length N = N1*N2 is transformed by N2 cooperating threads:
//   thread j2 holds x[N2*j1 + j2] (j1 < N1) in registers,
//   step A: N1-point DFT in registers, times W_N^(j2*k1),
//   exchange through shared memory,
//   step B: N1/N2 DFTs of N2 points per thread (k1 = r*N2 + j2),
// after which thread j2 holds X[k1 + N1*k2] = X[N2*(r + m*k2) + j2], i.e.
// again the elements N2*j + j2 (j = r + m*k2, m = N1/N2).  An inverse
// transform can therefore feed a forward transform (or an elementwise
// product) without a further exchange.
//
// Twiddle factors are compile-time constants: cos/sin(2 pi k/n) evaluated by
// a constexpr Taylor series after reduction to |phi| <= pi/4.
#pragma once
#include <utility>
#include "common.cuh"

namespace jrg {
namespace reg {

// ---- compile-time trigonometry -------------------------------------------
constexpr double kPi = 3.14159265358979323846264338327950288;

__host__ __device__ constexpr double taylor_sin(double x) {
  double term = x, sum = x;
  for (int k = 1; k < 14; ++k) {
    term *= -x * x / ((2.0 * k) * (2.0 * k + 1.0));
    sum += term;
  }
  return sum;
}
__host__ __device__ constexpr double taylor_cos(double x) {
  double term = 1.0, sum = 1.0;
  for (int k = 1; k < 14; ++k) {
    term *= -x * x / ((2.0 * k - 1.0) * (2.0 * k));
    sum += term;
  }
  return sum;
}
// cos and sin of 2 pi num / den
__host__ __device__ constexpr double cos2pi(long num, long den) {
  long r = ((num % den) + den) % den;
  // quadrant q and remainder: angle = 2 pi r/den = q pi/2 + phi
  long q = (4 * r + den / 2) / den;     // nearest multiple of pi/2
  double phi = 2.0 * kPi * (double)(4 * r - q * den) / (4.0 * (double)den);
  switch (q % 4) {
    case 0: return taylor_cos(phi);
    case 1: return -taylor_sin(phi);
    case 2: return -taylor_cos(phi);
    default: return taylor_sin(phi);
  }
}
__host__ __device__ constexpr double sin2pi(long num, long den) {
  long r = ((num % den) + den) % den;
  long q = (4 * r + den / 2) / den;
  double phi = 2.0 * kPi * (double)(4 * r - q * den) / (4.0 * (double)den);
  switch (q % 4) {
    case 0: return taylor_sin(phi);
    case 1: return taylor_cos(phi);
    case 2: return -taylor_sin(phi);
    default: return -taylor_cos(phi);
  }
}

// ---- compile-time loops -----------------------------------------------------
template <int... Is, class F>
__host__ __device__ __forceinline__ void sfor_impl(std::integer_sequence<int, Is...>, F&& f) {
  (f(std::integral_constant<int, Is>{}), ...);
}
template <int N, class F> __host__ __device__ __forceinline__ void sfor(F&& f) {
  sfor_impl(std::make_integer_sequence<int, N>{}, f);
}

// multiply by exp(DIR * 2 pi i K / N) (DIR = -1 forward, +1 inverse)
template <int DIR, int K, int N, typename C> __host__ __device__ __forceinline__ C twiddle_mul(C a) {
  constexpr int k = ((K % N) + N) % N;
  if constexpr (k == 0) {
    return a;
  } else if constexpr (4 * k == N) {           // exp(DIR i pi/2) = DIR * i
    C r;
    if (DIR > 0) { r.x = -a.y; r.y = a.x; } else { r.x = a.y; r.y = -a.x; }
    return r;
  } else if constexpr (2 * k == N) {
    C r; r.x = -a.x; r.y = -a.y; return r;
  } else if constexpr (4 * k == 3 * N) {
    C r;
    if (DIR > 0) { r.x = a.y; r.y = -a.x; } else { r.x = -a.y; r.y = a.x; }
    return r;
  } else {
    using R = decltype(a.x);
    constexpr double c = cos2pi(k, N);
    constexpr double s = DIR * sin2pi(k, N);
    C r;
    if constexpr (sizeof(R) == 8) {
      r.x = c * a.x - s * a.y;
      r.y = c * a.y + s * a.x;
    } else {
      // FP32: each constant as hi + lo.  A constant rounded to float scales
      // every product it touches by the same factor (sqrt(2)/2 rounds 1.7e-8
      // low, so |w|^2 = 1 - 3.4e-8): the transform loses norm by a fixed
      // fraction and the density by a fixed charge, which the energy sums
      // see at first order.  With the lo part the products carry only the
      // unbiased rounding of the arithmetic.
      constexpr float ch = (float)c, cl = (float)(c - (double)ch);
      constexpr float sh = (float)s, sl = (float)(s - (double)sh);
      if constexpr (ch == sh || ch == -sh) {
        // |cos| = |sin| (odd multiples of pi/4): w = ch (1 + i sign) (1 + lo/hi)
        constexpr float sg = ch == sh ? 1.f : -1.f;
        const float tx = a.x - sg * a.y, ty = a.y + sg * a.x;
        r.x = fmaf(ch, tx, cl * tx);
        r.y = fmaf(ch, ty, cl * ty);
      } else {
        r.x = fmaf(ch, a.x, fmaf(-sh, a.y, fmaf(cl, a.x, -sl * a.y)));
        r.y = fmaf(ch, a.y, fmaf(sh, a.x, fmaf(cl, a.y, sl * a.x)));
      }
    }
    return r;
  }
}


// ---- register DFTs ----------------------------------------------------------
template <int N, int DIR, typename C> __host__ __device__ __forceinline__ void dft(C (&v)[N]);

template <int DIR, typename C> __host__ __device__ __forceinline__ void dft2(C& a, C& b) {
  C t = a;
  a = cadd(t, b);
  b = csub(t, b);
}

template <int N, int DIR, typename C> __host__ __device__ __forceinline__ void dft(C (&v)[N]) {
  if constexpr (N == 1) {
    return;
  } else if constexpr (N == 2) {
    dft2<DIR>(v[0], v[1]);
  } else if constexpr (N == 3) {
    using R = decltype(v[0].x);
    constexpr double s3 = 0.86602540378443864676;
    C t1 = cadd(v[1], v[2]);
    C d = csub(v[1], v[2]);
    C t2 = csub(v[0], cscale(t1, (R)0.5));
    if constexpr (sizeof(R) == 4) {
      // sqrt(3)/2 as hi + lo (see twiddle_mul)
      constexpr float h = (float)s3, l = (float)(s3 - (double)h);
      d.x = fmaf(h, d.x, l * d.x);
      d.y = fmaf(h, d.y, l * d.y);
    } else {
      d.x *= s3;
      d.y *= s3;
    }
    C id;   // DIR * i * sqrt(3)/2 * (v1 - v2)
    if (DIR > 0) { id.x = -d.y; id.y = d.x; }
    else { id.x = d.y; id.y = -d.x; }
    v[0] = cadd(v[0], t1);
    v[1] = cadd(t2, id);
    v[2] = csub(t2, id);
  } else if constexpr (N == 4) {
    C a = cadd(v[0], v[2]), b = csub(v[0], v[2]);
    C c = cadd(v[1], v[3]), d = twiddle_mul<DIR, 1, 4>(csub(v[1], v[3]));
    v[0] = cadd(a, c);
    v[2] = csub(a, c);
    v[1] = cadd(b, d);
    v[3] = csub(b, d);
  } else {
    // N = P * Q: P-strided sub-DFTs of length Q, twiddles, then Q DFTs of length P
    constexpr int P = (N % 4 == 0 && N != 8) ? 4 : ((N % 3 == 0) ? 3 : 2);
    constexpr int Q = N / P;
    C y[P][Q];
    sfor<P>([&](auto pp) {
      constexpr int p = pp.value;
      sfor<Q>([&](auto qq) { constexpr int q = qq.value; y[p][q] = v[P * q + p]; });
      dft<Q, DIR>(y[p]);
    });
    sfor<Q>([&](auto kk) {
      constexpr int k = kk.value;
      C w[P];
      sfor<P>([&](auto pp) {
        constexpr int p = pp.value;
        w[p] = twiddle_mul<DIR, p * k, N>(y[p][k]);
      });
      dft<P, DIR>(w);
      sfor<P>([&](auto ss) { constexpr int s = ss.value; v[k + Q * s] = w[s]; });
    });
  }
}

// 8-point DFT of v with v[2..5] = 0 (a line of N = 32 or 64 points whose
// non-zero entries lie below N/4 and at or above 3N/4, held as 8 values per
// thread: x = N2 j1 + j2): the stages of dft<8> with the additions of the
// known zeros left out.
template <int DIR, typename C> __host__ __device__ __forceinline__ void dft8_in0167(C (&v)[8]) {
  // even and odd halves (v0, 0, 0, v6) and (v1, 0, 0, v7) through dft<4>'s stages
  const C te = twiddle_mul<DIR, 1, 4>(v[6]);
  const C to = twiddle_mul<DIR, 1, 4>(v[7]);
  C y[2][4];
  y[0][0] = cadd(v[0], v[6]);
  y[0][2] = csub(v[0], v[6]);
  y[0][1] = csub(v[0], te);
  y[0][3] = cadd(v[0], te);
  y[1][0] = cadd(v[1], v[7]);
  y[1][2] = csub(v[1], v[7]);
  y[1][1] = csub(v[1], to);
  y[1][3] = cadd(v[1], to);
  sfor<4>([&](auto kk) {
    constexpr int k = kk.value;
    C w0 = y[0][k], w1 = twiddle_mul<DIR, k, 8>(y[1][k]);
    dft2<DIR>(w0, w1);
    v[k] = w0;
    v[k + 4] = w1;
  });
}

// Split of a line length into N1 values per thread and N2 threads per line.
template <int N> struct Split;
template <> struct Split<16> { static constexpr int N1 = 4, N2 = 4; };
template <> struct Split<24> { static constexpr int N1 = 12, N2 = 2; };
template <> struct Split<27> { static constexpr int N1 = 9, N2 = 3; };
template <> struct Split<32> { static constexpr int N1 = 8, N2 = 4; };
template <> struct Split<36> { static constexpr int N1 = 6, N2 = 6; };
template <> struct Split<48> { static constexpr int N1 = 12, N2 = 4; };
template <> struct Split<64> { static constexpr int N1 = 8, N2 = 8; };
template <> struct Split<96> { static constexpr int N1 = 24, N2 = 4; };

// Step A of a line transform (see the file comment): N1-point DFT of the
// thread's registers, twiddle W_N^(j2*k1) from the table tw (tw[t] =
// exp(-2 pi i t/N), conjugated for the inverse), and write to the exchange
// buffer: element (k1, j2) of line l at ex[(k1*N2 + j2)*L + l].
template <int N, int DIR, typename C>
__host__ __device__ __forceinline__ void line_step_a(C (&v)[Split<N>::N1], const C* __restrict__ tw, int j2,
                                            C* ex, int L, int l) {
  constexpr int N1 = Split<N>::N1, N2 = Split<N>::N2;
  dft<N1, DIR>(v);
  sfor<N1>([&](auto kk) {
    constexpr int k1 = kk.value;
    C t = v[k1];
    if constexpr (k1 > 0) {
      C w = tw[j2 * k1];
      if (DIR > 0) w.y = -w.y;
      t = cmul(t, w);
    }
    ex[(k1 * N2 + j2) * L + l] = t;
  });
}

// line_step_a for the lengths held as 8 values per thread (N = 32, 64) with
// the thread's inputs v[2..5] known to be zero
template <int N, int DIR, typename C>
__host__ __device__ __forceinline__ void line_step_a_pruned8(C (&v)[8], const C* __restrict__ tw, int j2,
                                                    C* ex, int L, int l) {
  static_assert(Split<N>::N1 == 8, "pruned step for eight values per thread");
  constexpr int N2 = Split<N>::N2;
  dft8_in0167<DIR>(v);
  sfor<8>([&](auto kk) {
    constexpr int k1 = kk.value;
    C t = v[k1];
    if constexpr (k1 > 0) {
      C w = tw[j2 * k1];
      if (DIR > 0) w.y = -w.y;
      t = cmul(t, w);
    }
    ex[(k1 * N2 + j2) * L + l] = t;
  });
}

// Step B: after the exchange, the N1/N2 DFTs of length N2 of this thread;
// leaves v[j] = X[N2*j + j2].
template <int N, int DIR, typename C>
__host__ __device__ __forceinline__ void line_step_b(C (&v)[Split<N>::N1], int j2, const C* ex, int L,
                                            int l) {
  constexpr int N1 = Split<N>::N1, N2 = Split<N>::N2, M = N1 / N2;
  static_assert(N1 % N2 == 0, "N1 must be a multiple of N2");
  sfor<M>([&](auto rr) {
    constexpr int r = rr.value;
    const int k1 = r * N2 + j2;
    C u[N2];
    sfor<N2>([&](auto jj) {
      constexpr int jp = jj.value;
      u[jp] = ex[(k1 * N2 + jp) * L + l];
    });
    dft<N2, DIR>(u);
    sfor<N2>([&](auto kk) {
      constexpr int k2 = kk.value;
      v[r + M * k2] = u[k2];
    });
  });
}

}  // namespace reg
}  // namespace jrg
