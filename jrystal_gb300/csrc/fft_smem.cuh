// Shared-memory mixed-radix Stockham FFT engine.
//
// A CTA transforms a batch of lines that live in shared memory: element k of
// line l sits at base + line_start(l) + k*es, with line_start(l) = l*ls or
// rows[l]*ls when an indirect row list is given (pruned transforms over the
// rows of a plane that the plane-wave sphere touches).  Each radix stage reads
// one buffer and writes the other (autosort, natural order in and out), so a
// transform of n = r1*r2*... takes one shared-memory round trip per factor.
//
// Stage j (0 <= j < n/r) of a radix-r pass with Ns = product of the radices
// already applied reads src[j + q*(n/r)], multiplies input q by
// W_n^(q*(j mod Ns)*n/(Ns*r)), applies an r-point DFT and writes output q to
// dst[(j div Ns)*Ns*r + (j mod Ns) + q*Ns].  This is the Stockham autosort
// formulation used by Govindaraju et al., "High performance discrete Fourier
// transforms on graphics processors" (SC'08).
//
// Twiddles come from a per-axis table tw[t] = exp(-2 pi i t / n), t < n,
// computed in double precision on the host.  DIR = -1 is the forward
// (exp(-i...)) transform, DIR = +1 the inverse without the 1/n factor.
#pragma once
#include "common.cuh"

namespace jrg {

constexpr int kMaxRadices = 8;

struct FftAxis {
  int n;
  int nrad;
  int rad[kMaxRadices];
};

// Multiply by +i (s=+1) or -i (s=-1).
template <int S, typename C> __device__ __forceinline__ C mul_pm_i(C a) {
  C r;
  if (S > 0) { r.x = -a.y; r.y = a.x; } else { r.x = a.y; r.y = -a.x; }
  return r;
}

template <int DIR, typename C> __device__ __forceinline__ C twid(const C* tw, int t) {
  C w = tw[t];
  if (DIR > 0) w.y = -w.y;
  return w;
}

template <int RAD, int DIR, typename C>
__device__ __forceinline__ void small_dft(C (&v)[RAD], const C* tw, int n) {
  if constexpr (RAD == 2) {
    C a = v[0], b = v[1];
    v[0] = cadd(a, b); v[1] = csub(a, b);
  } else if constexpr (RAD == 3) {
    using R = decltype(v[0].x);
    constexpr double s3 = 0.86602540378443864676;   // sqrt(3)/2
    C t1 = cadd(v[1], v[2]);
    C d = csub(v[1], v[2]);
    C t2 = csub(v[0], cscale(t1, (R)0.5));
    if constexpr (sizeof(R) == 4) {
      // sqrt(3)/2 as hi + lo: a constant rounded to float would scale the
      // norm of every transform by the same factor
      constexpr float h = (float)s3, l = (float)(s3 - (double)h);
      d.x = fmaf(h, d.x, l * d.x);
      d.y = fmaf(h, d.y, l * d.y);
    } else {
      d.x *= s3;
      d.y *= s3;
    }
    C id = mul_pm_i<DIR>(d);                  // DIR*i*sqrt(3)/2*(v1-v2)
    v[0] = cadd(v[0], t1);
    v[1] = cadd(t2, id);
    v[2] = csub(t2, id);
  } else if constexpr (RAD == 4) {
    C a = cadd(v[0], v[2]), b = csub(v[0], v[2]);
    C c = cadd(v[1], v[3]), d = mul_pm_i<DIR>(csub(v[1], v[3]));
    v[0] = cadd(a, c); v[2] = csub(a, c);
    v[1] = cadd(b, d); v[3] = csub(b, d);
  } else {
    // generic O(r^2) DFT for radix 5 and 7 with table twiddles W_r^q = W_n^(q n/r)
    C out[RAD];
    const int step = n / RAD;
#pragma unroll
    for (int k = 0; k < RAD; ++k) {
      C acc = v[0];
#pragma unroll
      for (int q = 1; q < RAD; ++q) acc = cadd(acc, cmul(v[q], twid<DIR>(tw, ((k * q) % RAD) * step)));
      out[k] = acc;
    }
#pragma unroll
    for (int k = 0; k < RAD; ++k) v[k] = out[k];
  }
}

template <int RAD, int DIR, typename C>
__device__ __forceinline__ void fft_stage(const C* __restrict__ src, C* __restrict__ dst,
                                          const C* __restrict__ tw, int n, int Ns, int nlines,
                                          int es, int ls, const int* __restrict__ rows,
                                          bool lines_fast) {
  const int m = n / RAD;
  const int total = nlines * m;
  const int tstride = n / (Ns * RAD);
  for (int w = threadIdx.x; w < total; w += blockDim.x) {
    int line, j;
    if (lines_fast) { line = w % nlines; j = w / nlines; }
    else { j = w % m; line = w / m; }
    const int base = (rows ? rows[line] : line) * ls;
    C v[RAD];
#pragma unroll
    for (int q = 0; q < RAD; ++q) v[q] = src[base + (j + q * m) * es];
    const int jm = j % Ns;
    const int step = jm * tstride;
    if (step) {
#pragma unroll
      for (int q = 1; q < RAD; ++q) v[q] = cmul(v[q], twid<DIR>(tw, q * step));
    }
    small_dft<RAD, DIR>(v, tw, n);
    const int o = (j - jm) * RAD + jm;
#pragma unroll
    for (int q = 0; q < RAD; ++q) dst[base + (o + q * Ns) * es] = v[q];
  }
}

// Transforms the lines held in `a`, ping-ponging with `b`; returns the buffer
// holding the result.  Requires the input to be complete (caller syncs before)
// and leaves the CTA synchronised.  Elements of `b` outside the transformed
// lines are not touched.
template <int DIR, typename C>
__device__ C* fft_lines(C* a, C* b, const C* tw, const FftAxis& ax, int nlines, int es, int ls,
                        const int* rows, bool lines_fast) {
  int Ns = 1;
  for (int s = 0; s < ax.nrad; ++s) {
    const int r = ax.rad[s];
    switch (r) {
      case 2: fft_stage<2, DIR>(a, b, tw, ax.n, Ns, nlines, es, ls, rows, lines_fast); break;
      case 3: fft_stage<3, DIR>(a, b, tw, ax.n, Ns, nlines, es, ls, rows, lines_fast); break;
      case 4: fft_stage<4, DIR>(a, b, tw, ax.n, Ns, nlines, es, ls, rows, lines_fast); break;
      case 5: fft_stage<5, DIR>(a, b, tw, ax.n, Ns, nlines, es, ls, rows, lines_fast); break;
      default: fft_stage<7, DIR>(a, b, tw, ax.n, Ns, nlines, es, ls, rows, lines_fast); break;
    }
    __syncthreads();
    C* t = a; a = b; b = t;
    Ns *= r;
  }
  return a;
}

}  // namespace jrg
