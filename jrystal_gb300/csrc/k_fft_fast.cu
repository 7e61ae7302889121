// Fast slab kernels for cubic grids N^3, N in {16, 24, 27, 32, 36, 48, 64, 96}.
//
// Same data flow as the generic kernels in k_fft.cu (plane pass over y and z
// with the sphere scatter/gather fused in, line pass over x with the density
// or V(r) product fused in), but every 1-D transform is register-resident:
// a line of N points is held by N2 threads (N1 points each) and crosses
// shared memory once (see fft_reg.cuh).  Global loads and stores feed the
// first and leave the last register step directly.  Thread t of a CTA works
// on line l = t % L as worker j2 = t / L, so the lanes of a warp walk
// consecutive lines: consecutive z in global memory, consecutive addresses
// in the exchange buffers, and an odd row pitch (N + 1) in the [z][y] plane
// buffer keeps the column accesses free of bank conflicts.
#include "fast_dispatch.h"
#include "fft_reg.cuh"
#include <cstdlib>

#include "plan.h"
#include <type_traits>

namespace jrg {
namespace fast {

// kinetic table |G+k|^2/2 in the path's precision: the FP32 copy of the plan
// for the FP32 kernels (the same values as an FP32 cast of the FP64 table,
// without a conversion per coefficient and band)
template <typename R> using TK_t = std::conditional_t<sizeof(R) == 4, float, double>;
template <typename R> const TK_t<R>* tk_table(const jrg_plan* P) {
  if constexpr (sizeof(R) == 4) return P->d.tkf;
  else return P->d.tk;
}

using reg::Split;

template <int N> constexpr int threads_for() { return N * Split<N>::N2; }
// two resident CTAs per SM where the register file allows it (<= 64 registers
// per thread at 512 threads): hides the global-load latency of the band loop
template <typename R, int N> constexpr int min_blocks_for() {
  return (sizeof(R) == 4 && N <= 64) ? 2 : 1;
}

// byte offset of the prefetch row buffers in a line kernel's shared memory
// group weights of k_line_density, after the twiddles, exchange buffers and xact
template <typename R, int N> __host__ __device__ constexpr size_t line_w_offset() {
  return align16(sizeof(C_t<R>) * (size_t)(N + 2 * N * N) + sizeof(int) * N);
}
template <typename R, int N> __host__ __device__ constexpr size_t line_pf_offset() {
  return (sizeof(C_t<R>) * (size_t)(N + 2 * N * N) + sizeof(int) * N + 15) / 16 * 16;
}

// sphere -> y,z-transformed active planes
template <typename R, int N>
__global__ void __launch_bounds__(threads_for<N>()) k_plane_inv_sphere(
    const C_t<R>* __restrict__ coef, C_t<R>* __restrict__ planes, const int* __restrict__ plane_off,
    const int* __restrict__ sph_yz, const int* __restrict__ row_off, const int* __restrict__ rows,
    const C_t<R>* __restrict__ tw_g, int ng, int nact) {
  using C = C_t<R>;
  constexpr int N1 = Split<N>::N1, N2 = Split<N>::N2, P = N + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* tw = reinterpret_cast<C*>(smem_raw);
  C* A = tw + N;              // [z][y], pitch P
  C* ex = A + N * P;          // exchange, N*N
  int* srows = reinterpret_cast<int*>(ex + N * N);
  const int p = blockIdx.x, band = blockIdx.y, tid = threadIdx.x;
  for (int i = tid; i < N; i += blockDim.x) tw[i] = tw_g[i];
  const C z0 = czero<C>();
  for (int i = tid; i < N * P; i += blockDim.x) A[i] = z0;
  const int r0 = row_off[p], nr = row_off[p + 1] - r0;
  for (int i = tid; i < nr; i += blockDim.x) srows[i] = rows[r0 + i];
  __syncthreads();
  const C* cb = coef + (size_t)band * ng;
  for (int e = plane_off[p] + tid; e < plane_off[p + 1]; e += blockDim.x) {
    const int yz = sph_yz[e];
    const int y = yz / N, z = yz - y * N;
    A[z * P + y] = cb[e];
  }
  __syncthreads();
  // z transforms of the active rows (L = nr lines)
  C v[N1];
  {
    const bool act = tid < nr * N2;
    const int l = act ? tid % nr : 0, j2 = act ? tid / nr : 0;
    const int y = srows[l];
    if (act) {
#pragma unroll
      for (int j1 = 0; j1 < N1; ++j1) v[j1] = A[(N2 * j1 + j2) * P + y];
      reg::line_step_a<N, +1>(v, tw, j2, ex, nr, l);
    }
    __syncthreads();
    if (act) {
      reg::line_step_b<N, +1>(v, j2, ex, nr, l);
#pragma unroll
      for (int j = 0; j < N1; ++j) A[(N2 * j + j2) * P + y] = v[j];
    }
    __syncthreads();
  }
  // y transforms of all z columns (L = N lines), straight to global memory
  {
    const int z = tid % N, j2 = tid / N;
#pragma unroll
    for (int j1 = 0; j1 < N1; ++j1) v[j1] = A[z * P + N2 * j1 + j2];
    reg::line_step_a<N, +1>(v, tw, j2, ex, N, z);
    __syncthreads();
    reg::line_step_b<N, +1>(v, j2, ex, N, z);
    C* out = planes + ((size_t)band * nact + p) * (N * N);
#pragma unroll
    for (int j = 0; j < N1; ++j) out[(N2 * j + j2) * N + z] = v[j];
  }
}

// sphere -> y,z-transformed active planes, up to bpc bands per CTA: the
// gather of band i+1 (zero-filling cp.async through the dense row map: sphere
// values and zeros for the rest of every active row) runs under the transforms
// of band i; inactive rows of both [z][y] buffers stay zero.
// PR (8 values per thread: N = 32, 64): active rows y and sphere z lie below
// N/4 or at or above 3N/4, so the inputs v[2..5] of the z and y transforms are zero
template <typename R, int N, bool PR>
__global__ void __launch_bounds__(threads_for<N>()) k_plane_inv_sphere_mb(
    const C_t<R>* __restrict__ coef, C_t<R>* __restrict__ planes, const int* __restrict__ row_off,
    const int* __restrict__ rows, const int* __restrict__ rowmap, const C_t<R>* __restrict__ tw_g,
    int ng, int nact, int nbands, int bpc) {
  using C = C_t<R>;
  constexpr int N1 = Split<N>::N1, N2 = Split<N>::N2, P = N + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* tw = reinterpret_cast<C*>(smem_raw);
  C* A0 = tw + N;                                     // two [z][y] buffers, pitch P
  C* ex = A0 + 2 * N * P;                             // exchange, N*N
  int* srows = reinterpret_cast<int*>(ex + N * N);    // [N]
  int* smap = srows + N;                              // [nr][N]
  const int p = blockIdx.x, tid = threadIdx.x;
  const int b_begin = blockIdx.y * bpc, b_end = min(nbands, b_begin + bpc);
  const int r0 = row_off[p], nr = row_off[p + 1] - r0;
  for (int i = tid; i < N; i += blockDim.x) tw[i] = tw_g[i];
  for (int i = tid; i < nr; i += blockDim.x) srows[i] = rows[r0 + i];
  for (int i = tid; i < nr * N; i += blockDim.x) smap[i] = rowmap[(size_t)r0 * N + i];
  const C z0 = czero<C>();
  for (int i = tid; i < 2 * N * P; i += blockDim.x) A0[i] = z0;
  __syncthreads();
  auto gather = [&](C* A, int band) {
    const C* cb = coef + (size_t)band * ng;
    for (int i = tid; i < nr * N; i += blockDim.x) {
      const int r = i / N, z = i - r * N;
      const int e = smap[i];
      cp_async_zfill<sizeof(C)>(&A[z * P + srows[r]], e >= 0 ? cb + e : cb, e >= 0);
    }
    cp_async_commit();
  };
  if (b_begin < b_end) gather(A0, b_begin);
  C v[N1];
  for (int band = b_begin, it = 0; band < b_end; ++band, ++it) {
    C* A = A0 + (it & 1) * (N * P);
    if (band + 1 < b_end) {
      gather(A0 + ((it + 1) & 1) * (N * P), band + 1);   // last read before the previous exchange
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    // z transforms of the active rows (L = nr lines)
    {
      const bool act = tid < nr * N2;
      const int l = act ? tid % nr : 0, j2 = act ? tid / nr : 0;
      const int y = srows[l];
      if (act) {
#pragma unroll
        for (int j1 = 0; j1 < N1; ++j1) {
          if (PR && j1 >= 2 && j1 <= 5) continue;
          v[j1] = A[(N2 * j1 + j2) * P + y];
        }
        if constexpr (PR) reg::line_step_a_pruned8<N, +1>(v, tw, j2, ex, nr, l);
        else reg::line_step_a<N, +1>(v, tw, j2, ex, nr, l);
      }
      __syncthreads();
      if (act) {
        reg::line_step_b<N, +1>(v, j2, ex, nr, l);
#pragma unroll
        for (int j = 0; j < N1; ++j) A[(N2 * j + j2) * P + y] = v[j];
      }
      __syncthreads();
    }
    // y transforms of all z columns (L = N lines), straight to global memory
    {
      const int z = tid % N, j2 = tid / N;
#pragma unroll
      for (int j1 = 0; j1 < N1; ++j1) {
        if (PR && j1 >= 2 && j1 <= 5) continue;
        v[j1] = A[z * P + N2 * j1 + j2];
      }
      if constexpr (PR) reg::line_step_a_pruned8<N, +1>(v, tw, j2, ex, N, z);
      else reg::line_step_a<N, +1>(v, tw, j2, ex, N, z);
      __syncthreads();
      reg::line_step_b<N, +1>(v, j2, ex, N, z);
      C* out = planes + ((size_t)band * nact + p) * (N * N);
#pragma unroll
      for (int j = 0; j < N1; ++j) out[(N2 * j + j2) * N + z] = v[j];
    }
  }
}

// Rows [nact][N] of band b for line y go to shared memory with cp.async one
// band ahead of the transforms (PF, adjoint pass), so that the loads of the
// next band are in flight while the current one is transformed.
template <typename R, int N>
__device__ __forceinline__ void prefetch_row(const C_t<R>* __restrict__ planes, C_t<R>* dst, int b,
                                             int y, int nact) {
  using C = C_t<R>;
  const C* src = planes + (size_t)b * nact * (N * N) + (size_t)y * N;
  if constexpr ((N * sizeof(C)) % 16 == 0) {
    constexpr int PER = 16 / sizeof(C);
    for (int q = threadIdx.x; q < nact * (N / PER); q += blockDim.x) {
      const int s = q / (N / PER), zz = (q - s * (N / PER)) * PER;
      cp_async<16>(dst + s * N + zz, src + (size_t)s * (N * N) + zz);
    }
  } else {
    for (int q = threadIdx.x; q < nact * N; q += blockDim.x) {
      const int s = q / N, zz = q - s * N;
      cp_async<sizeof(C)>(dst + q, src + (size_t)s * (N * N) + zz);
    }
  }
  cp_async_commit();
}

// inverse x transform + occupation-weighted |psi|^2 of a band group (one
// transform per band: the row prefetch of the adjoint pass measured slower
// here, 0.30 vs 0.25 ms on the 64^3 Si8 cell).  The partial of a group holds
// sum_b (w_b / w_ref) |psi_b|^2 with w_ref the group's largest weight, and
// gscale[grp] = w_ref * wscale (FP64) is applied by the density reduction: a
// weight rounded to FP32 would scale the whole group's charge (the usual
// case, every occupied band of a k-point has the same weight) by one
// rounding error; the ratio of equal weights is exactly 1.
// PR (N = 32, 64): the thread's inputs v[2..5] (x = N/4 .. 3N/4 - 1) are known zero
template <typename R, int N, bool PR>
__global__ void __launch_bounds__(threads_for<N>(), min_blocks_for<R, N>()) k_line_density(
    const C_t<R>* __restrict__ planes, R* __restrict__ rho_part, const double* __restrict__ wband,
    double wscale, int band0, int nband, int bands_per_group, const int* __restrict__ xact,
    const C_t<R>* __restrict__ tw_g, int nact, double* __restrict__ gscale) {
  using C = C_t<R>;
  constexpr int N1 = Split<N>::N1, N2 = Split<N>::N2;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* tw = reinterpret_cast<C*>(smem_raw);
  C* ex0 = tw + N;
  C* ex1 = ex0 + N * N;
  int* sxact = reinterpret_cast<int*>(ex1 + N * N);
  R* sw = reinterpret_cast<R*>(smem_raw + line_w_offset<R, N>());   // [bands_per_group]
  const int y = blockIdx.x, grp = blockIdx.y, tid = threadIdx.x;
  const int z = tid % N, j2 = tid / N;
  const int b_begin = grp * bands_per_group;
  const int b_end = min(nband, b_begin + bands_per_group);
  for (int i = tid; i < N; i += blockDim.x) { tw[i] = tw_g[i]; sxact[i] = xact[i]; }
  group_weights<R>(wband + band0, b_begin, b_end, wscale, gscale, grp, sw);
  __syncthreads();
  int slot[N1];
#pragma unroll
  for (int j1 = 0; j1 < N1; ++j1) slot[j1] = sxact[N2 * j1 + j2];
  R acc[N1];
#pragma unroll
  for (int j = 0; j < N1; ++j) acc[j] = (R)0;
  const C z0 = czero<C>();
  C v[N1];
  // PR: the four non-zero inputs of the next band are loaded while the
  // current band is transformed
  C nxt[4];
  auto load4 = [&](int b) {
    const C* src = planes + (size_t)b * nact * (N * N) + y * N + z;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int j1 = q < 2 ? q : q + 4;
      nxt[q] = slot[j1] < 0 ? z0 : src[(size_t)slot[j1] * (N * N)];
    }
  };
  if (PR && b_begin < b_end) load4(b_begin);
  int parity = 0;
  for (int b = b_begin; b < b_end; ++b, parity ^= 1) {
    const R w = sw[b - b_begin];
    if constexpr (PR) {
      v[0] = nxt[0]; v[1] = nxt[1]; v[6] = nxt[2]; v[7] = nxt[3];
      if (b + 1 < b_end) load4(b + 1);
    } else {
      const C* src = planes + (size_t)b * nact * (N * N) + y * N + z;
#pragma unroll
      for (int j1 = 0; j1 < N1; ++j1) v[j1] = slot[j1] < 0 ? z0 : src[(size_t)slot[j1] * (N * N)];
    }
    C* ex = parity ? ex1 : ex0;
    if constexpr (PR) reg::line_step_a_pruned8<N, +1>(v, tw, j2, ex, N, z);
    else reg::line_step_a<N, +1>(v, tw, j2, ex, N, z);
    __syncthreads();
    reg::line_step_b<N, +1>(v, j2, ex, N, z);
#pragma unroll
    for (int j = 0; j < N1; ++j) acc[j] += w * (v[j].x * v[j].x + v[j].y * v[j].y);
  }
  R* out = rho_part + (size_t)grp * (N * N * N) + y * N + z;
#pragma unroll
  for (int j = 0; j < N1; ++j) out[(size_t)(N2 * j + j2) * (N * N)] = acc[j];
}

// adjoint line pass: inverse x transform, times V(r), forward x transform,
// active planes written back in place
// PR (N = 32, 64): x = N/4 .. 3N/4 - 1 (the thread's v[2..5]) are known zero
// on input and not written back
template <typename R, int N, bool PF, bool PR>
__global__ void __launch_bounds__(threads_for<N>(), min_blocks_for<R, N>()) k_line_apply_v(
    C_t<R>* __restrict__ planes, const R* __restrict__ vr, int nband, int bands_per_group,
    const int* __restrict__ xact, const C_t<R>* __restrict__ tw_g, int nact) {
  using C = C_t<R>;
  constexpr int N1 = Split<N>::N1, N2 = Split<N>::N2;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* tw = reinterpret_cast<C*>(smem_raw);
  C* ex0 = tw + N;
  C* ex1 = ex0 + N * N;
  int* sxact = reinterpret_cast<int*>(ex1 + N * N);
  C* rowbuf = reinterpret_cast<C*>(smem_raw + line_pf_offset<R, N>());   // [2][nact][N]
  const int y = blockIdx.x, grp = blockIdx.y, tid = threadIdx.x;
  const int z = tid % N, j2 = tid / N;
  for (int i = tid; i < N; i += blockDim.x) { tw[i] = tw_g[i]; sxact[i] = xact[i]; }
  const int b_begin = grp * bands_per_group;
  const int b_end = min(nband, b_begin + bands_per_group);
  if (PF && b_begin < b_end) prefetch_row<R, N>(planes, rowbuf, b_begin, y, nact);
  __syncthreads();
  int slot[N1];
  R vloc[N1];
#pragma unroll
  for (int j1 = 0; j1 < N1; ++j1) {
    slot[j1] = sxact[N2 * j1 + j2];
    vloc[j1] = vr[(size_t)(N2 * j1 + j2) * (N * N) + y * N + z];
  }
  const C z0 = czero<C>();
  C v[N1];
  // RP (pruned, no row buffer): the four non-zero inputs of the next band are
  // loaded into registers while the current band is transformed
  constexpr bool RP = PR && !PF;
  C nxt[4];
  auto load4 = [&](int b) {
    const C* src = planes + (size_t)b * nact * (N * N) + y * N + z;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int j1 = q < 2 ? q : q + 4;
      nxt[q] = slot[j1] < 0 ? z0 : src[(size_t)slot[j1] * (N * N)];
    }
  };
  if (RP && b_begin < b_end) load4(b_begin);
  int parity = 0;
  for (int b = b_begin; b < b_end; ++b, parity ^= 1) {
    C* base = planes + (size_t)b * nact * (N * N) + y * N + z;
    if constexpr (RP) {
      v[0] = nxt[0]; v[1] = nxt[1]; v[6] = nxt[2]; v[7] = nxt[3];
      if (b + 1 < b_end) load4(b + 1);
    } else if constexpr (PF) {
      if (b + 1 < b_end) {
        prefetch_row<R, N>(planes, rowbuf + (parity ^ 1) * nact * N, b + 1, y, nact);
        cp_async_wait<1>();
      } else {
        cp_async_wait<0>();
      }
      __syncthreads();
      const C* src = rowbuf + parity * nact * N + z;
#pragma unroll
      for (int j1 = 0; j1 < N1; ++j1) {
        if (PR && j1 >= 2 && j1 <= 5) continue;
        v[j1] = slot[j1] < 0 ? z0 : src[slot[j1] * N];
      }
    } else {
#pragma unroll
      for (int j1 = 0; j1 < N1; ++j1) {
        if (PR && j1 >= 2 && j1 <= 5) continue;
        v[j1] = slot[j1] < 0 ? z0 : base[(size_t)slot[j1] * (N * N)];
      }
    }
    if constexpr (PR) reg::line_step_a_pruned8<N, +1>(v, tw, j2, ex0, N, z);
    else reg::line_step_a<N, +1>(v, tw, j2, ex0, N, z);
    __syncthreads();
    reg::line_step_b<N, +1>(v, j2, ex0, N, z);
#pragma unroll
    for (int j = 0; j < N1; ++j) v[j] = cscale(v[j], vloc[j]);
    reg::line_step_a<N, -1>(v, tw, j2, ex1, N, z);
    __syncthreads();
    reg::line_step_b<N, -1>(v, j2, ex1, N, z);
#pragma unroll
    for (int j = 0; j < N1; ++j) {
      if (PR && j >= 2 && j <= 5) continue;   // the outputs left out are never formed
      if (slot[j] >= 0) base[(size_t)slot[j] * (N * N)] = v[j];
    }
  }
}

// forward: y, z transforms of an active plane, sphere gather and gradient
//   g[b][e] = f_b * (tk[k][e] * c[b][e] + scale * FFT(V psi_b)[e])
// PR (N = 32, 64): only rows y and sphere z below N/4 or at or above 3N/4 are
// needed, so the y and z transforms do not form the outputs v[2..5]
template <typename R, int N, bool PR>
__global__ void __launch_bounds__(threads_for<N>()) k_plane_fwd_sphere(
    const C_t<R>* __restrict__ planes, const C_t<R>* __restrict__ coef, C_t<R>* __restrict__ gcoef,
    const double* __restrict__ wband, const TK_t<R>* __restrict__ tk, int nb_per_k, int band0,
    const int* __restrict__ plane_off, const int* __restrict__ sph_yz, const int* __restrict__ row_off,
    const int* __restrict__ rows, const C_t<R>* __restrict__ tw_g, int ng, int nact, int nk,
    double scale) {
  using C = C_t<R>;
  constexpr int N1 = Split<N>::N1, N2 = Split<N>::N2, P = N + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* tw = reinterpret_cast<C*>(smem_raw);
  C* A = tw + N;
  C* ex = A + N * P;
  int* srows = reinterpret_cast<int*>(ex + N * N);
  const int p = blockIdx.x, band = blockIdx.y, tid = threadIdx.x;
  for (int i = tid; i < N; i += blockDim.x) tw[i] = tw_g[i];
  const int r0 = row_off[p], nr = row_off[p + 1] - r0;
  for (int i = tid; i < nr; i += blockDim.x) srows[i] = rows[r0 + i];
  __syncthreads();
  C v[N1];
  // y transforms of all z columns, from global memory
  {
    const int z = tid % N, j2 = tid / N;
    const C* in = planes + ((size_t)band * nact + p) * (N * N) + z;
#pragma unroll
    for (int j1 = 0; j1 < N1; ++j1) v[j1] = in[(N2 * j1 + j2) * N];
    reg::line_step_a<N, -1>(v, tw, j2, ex, N, z);
    __syncthreads();
    reg::line_step_b<N, -1>(v, j2, ex, N, z);
#pragma unroll
    for (int j = 0; j < N1; ++j) {
      if (PR && j >= 2 && j <= 5) continue;   // inactive rows are never read
      A[z * P + N2 * j + j2] = v[j];
    }
    __syncthreads();
  }
  // z transforms of the active rows
  {
    const bool act = tid < nr * N2;
    const int l = act ? tid % nr : 0, j2 = act ? tid / nr : 0;
    const int y = srows[l];
    if (act) {
#pragma unroll
      for (int j1 = 0; j1 < N1; ++j1) v[j1] = A[(N2 * j1 + j2) * P + y];
      reg::line_step_a<N, -1>(v, tw, j2, ex, nr, l);
    }
    __syncthreads();
    if (act) {
      reg::line_step_b<N, -1>(v, j2, ex, nr, l);
#pragma unroll
      for (int j = 0; j < N1; ++j) {
        if (PR && j >= 2 && j <= 5) continue;   // off-sphere z are never gathered
        A[(N2 * j + j2) * P + y] = v[j];
      }
    }
    __syncthreads();
  }
  const int gb = band0 + band;
  const int kidx = (gb / nb_per_k) % nk;
  const R w = (R)wband[gb];
  const R sc = (R)scale;
  const TK_t<R>* tkk = tk + (size_t)kidx * ng;
  const C* cb = coef + (size_t)band * ng;
  C* gout = gcoef + (size_t)band * ng;
  for (int e = plane_off[p] + tid; e < plane_off[p + 1]; e += blockDim.x) {
    const int yz = sph_yz[e];
    const int y = yz / N, z = yz - y * N;
    const C val = A[z * P + y];
    const C c = cb[e];
    const R t = (R)tkk[e];
    C g;
    g.x = w * (t * c.x + sc * val.x);
    g.y = w * (t * c.y + sc * val.y);
    gout[e] = g;
  }
}

// forward plane pass, up to bpc bands per CTA: each thread loads its eight
// values of the next band's plane into registers while the current band is
// transformed, gathered and weighted (PR as in k_plane_fwd_sphere).
template <typename R, int N, bool PR>
__global__ void __launch_bounds__(threads_for<N>()) k_plane_fwd_sphere_rp(
    const C_t<R>* __restrict__ planes, const C_t<R>* __restrict__ coef, C_t<R>* __restrict__ gcoef,
    const double* __restrict__ wband, const TK_t<R>* __restrict__ tk, int nb_per_k, int band0,
    const int* __restrict__ plane_off, const int* __restrict__ sph_yz, const int* __restrict__ row_off,
    const int* __restrict__ rows, const C_t<R>* __restrict__ tw_g, int ng, int nact, int nk,
    double scale, int nbands, int bpc) {
  using C = C_t<R>;
  constexpr int N1 = Split<N>::N1, N2 = Split<N>::N2, P = N + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* tw = reinterpret_cast<C*>(smem_raw);
  C* A = tw + N;
  C* ex = A + N * P;
  int* srows = reinterpret_cast<int*>(ex + N * N);
  const int p = blockIdx.x, tid = threadIdx.x;
  const int b_begin = blockIdx.y * bpc, b_end = min(nbands, b_begin + bpc);
  for (int i = tid; i < N; i += blockDim.x) tw[i] = tw_g[i];
  const int r0 = row_off[p], nr = row_off[p + 1] - r0;
  for (int i = tid; i < nr; i += blockDim.x) srows[i] = rows[r0 + i];
  const int zc = tid % N, jc = tid / N;   // column z and thread index j2 of the y transforms
  C nxt[N1];
  auto load = [&](int band) {
    const C* in = planes + ((size_t)band * nact + p) * (N * N) + zc;
#pragma unroll
    for (int j1 = 0; j1 < N1; ++j1) nxt[j1] = in[(N2 * j1 + jc) * N];
  };
  if (b_begin < b_end) load(b_begin);
  __syncthreads();
  const R sc = (R)scale;
  // first gather element of this thread: its map entry is band-independent,
  // its coefficient and kinetic value are loaded at the top of each band so
  // that their latency falls under the transforms
  const int e_lo = plane_off[p], e_hi = plane_off[p + 1];
  const int e0 = e_lo + tid;
  const bool has0 = e0 < e_hi;
  const int yz0 = has0 ? sph_yz[e0] : 0;
  C v[N1];
  for (int band = b_begin; band < b_end; ++band) {
    const int gb = band0 + band;
    const int kidx = (gb / nb_per_k) % nk;
    const TK_t<R>* tkk = tk + (size_t)kidx * ng;
    const C* cb = coef + (size_t)band * ng;
    C c0 = czero<C>();
    R t0 = (R)0;
    if (has0) {
      c0 = cb[e0];
      t0 = (R)tkk[e0];
    }
    // y transforms of all z columns
#pragma unroll
    for (int j1 = 0; j1 < N1; ++j1) v[j1] = nxt[j1];
    if (band + 1 < b_end) load(band + 1);
    reg::line_step_a<N, -1>(v, tw, jc, ex, N, zc);
    __syncthreads();
    reg::line_step_b<N, -1>(v, jc, ex, N, zc);
#pragma unroll
    for (int j = 0; j < N1; ++j) {
      if (PR && j >= 2 && j <= 5) continue;   // inactive rows are never read
      A[zc * P + N2 * j + jc] = v[j];
    }
    __syncthreads();
    // z transforms of the active rows
    {
      const bool act = tid < nr * N2;
      const int l = act ? tid % nr : 0, j2 = act ? tid / nr : 0;
      const int y = srows[l];
      if (act) {
#pragma unroll
        for (int j1 = 0; j1 < N1; ++j1) v[j1] = A[(N2 * j1 + j2) * P + y];
        reg::line_step_a<N, -1>(v, tw, j2, ex, nr, l);
      }
      __syncthreads();
      if (act) {
        reg::line_step_b<N, -1>(v, j2, ex, nr, l);
#pragma unroll
        for (int j = 0; j < N1; ++j) {
          if (PR && j >= 2 && j <= 5) continue;   // off-sphere z are never gathered
          A[(N2 * j + j2) * P + y] = v[j];
        }
      }
      __syncthreads();
    }
    const R w = (R)wband[gb];
    C* gout = gcoef + (size_t)band * ng;
    if (has0) {
      const int y = yz0 / N, z = yz0 - y * N;
      const C val = A[z * P + y];
      C g;
      g.x = w * (t0 * c0.x + sc * val.x);
      g.y = w * (t0 * c0.y + sc * val.y);
      gout[e0] = g;
    }
    for (int e = e0 + blockDim.x; e < e_hi; e += blockDim.x) {
      const int yz = sph_yz[e];
      const int y = yz / N, z = yz - y * N;
      const C val = A[z * P + y];
      const C c = cb[e];
      const R t = (R)tkk[e];
      C g;
      g.x = w * (t * c.x + sc * val.x);
      g.y = w * (t * c.y + sc * val.y);
      gout[e] = g;
    }
  }
}

// dense plane pass of whole grids [batch][x][y][z]: z then y transforms of
// plane x (input real or complex), result to `out` in the same layout
template <typename R, int N, int DIR, bool REAL_IN>
__global__ void __launch_bounds__(threads_for<N>()) k_plane_dense(const void* __restrict__ in_v,
                                                                   C_t<R>* __restrict__ out,
                                                                   const C_t<R>* __restrict__ tw_g) {
  using C = C_t<R>;
  constexpr int N1 = Split<N>::N1, N2 = Split<N>::N2, P = N + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* tw = reinterpret_cast<C*>(smem_raw);
  C* A = tw + N;
  C* ex = A + N * P;
  const int tid = threadIdx.x;
  const size_t base = ((size_t)blockIdx.y * N + blockIdx.x) * (N * N);
  for (int i = tid; i < N; i += blockDim.x) tw[i] = tw_g[i];
  for (int i = tid; i < N * N; i += blockDim.x) {
    const int y = i / N, z = i - y * N;
    C v;
    if constexpr (REAL_IN) { v.x = reinterpret_cast<const R*>(in_v)[base + i]; v.y = 0; }
    else v = reinterpret_cast<const C*>(in_v)[base + i];
    A[z * P + y] = v;
  }
  __syncthreads();
  C v[N1];
  {
    const int y = tid % N, j2 = tid / N;
#pragma unroll
    for (int j1 = 0; j1 < N1; ++j1) v[j1] = A[(N2 * j1 + j2) * P + y];
    reg::line_step_a<N, DIR>(v, tw, j2, ex, N, y);
    __syncthreads();
    reg::line_step_b<N, DIR>(v, j2, ex, N, y);
#pragma unroll
    for (int j = 0; j < N1; ++j) A[(N2 * j + j2) * P + y] = v[j];
    __syncthreads();
  }
  {
    const int z = tid % N, j2 = tid / N;
#pragma unroll
    for (int j1 = 0; j1 < N1; ++j1) v[j1] = A[z * P + N2 * j1 + j2];
    reg::line_step_a<N, DIR>(v, tw, j2, ex, N, z);
    __syncthreads();
    reg::line_step_b<N, DIR>(v, j2, ex, N, z);
#pragma unroll
    for (int j = 0; j < N1; ++j) out[base + (N2 * j + j2) * N + z] = v[j];
  }
}

// dense line pass: x transforms of row y of every (x, z) slab, times scale
template <typename R, int N, int DIR>
__global__ void __launch_bounds__(threads_for<N>()) k_line_dense(const C_t<R>* __restrict__ in,
                                                                  C_t<R>* __restrict__ out,
                                                                  const C_t<R>* __restrict__ tw_g,
                                                                  double scale) {
  using C = C_t<R>;
  constexpr int N1 = Split<N>::N1, N2 = Split<N>::N2;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* tw = reinterpret_cast<C*>(smem_raw);
  C* ex = tw + N;
  const int tid = threadIdx.x, y = blockIdx.x;
  const int z = tid % N, j2 = tid / N;
  const size_t base = (size_t)blockIdx.y * N * N * N + (size_t)y * N + z;
  for (int i = tid; i < N; i += blockDim.x) tw[i] = tw_g[i];
  __syncthreads();
  C v[N1];
#pragma unroll
  for (int j1 = 0; j1 < N1; ++j1) v[j1] = in[base + (size_t)(N2 * j1 + j2) * (N * N)];
  reg::line_step_a<N, DIR>(v, tw, j2, ex, N, z);
  __syncthreads();
  reg::line_step_b<N, DIR>(v, j2, ex, N, z);
  const R sc = (R)scale;
#pragma unroll
  for (int j = 0; j < N1; ++j) out[base + (size_t)(N2 * j + j2) * (N * N)] = cscale(v[j], sc);
}

// ------------------------------------------------------------------------
// dispatch: returns 1 when a fast kernel was launched, 0 when the grid is not
// covered (the caller then uses the generic kernels), <0 on a launch error.
// ------------------------------------------------------------------------
template <typename R, int N> size_t plane_smem() {
  return sizeof(C_t<R>) * (size_t)(N + N * (N + 1) + N * N) + sizeof(int) * (N + 1);
}
template <typename R, int N> size_t plane_mb_smem(int max_rows) {
  return sizeof(C_t<R>) * (size_t)(N + 2 * N * (N + 1) + N * N) + sizeof(int) * (size_t)N * (1 + max_rows);
}
template <typename R, int N> size_t line_smem() {
  return sizeof(C_t<R>) * (size_t)(N + 2 * N * N) + sizeof(int) * N;
}
template <typename R, int N> size_t line_pf_smem(int nact) {
  return line_pf_offset<R, N>() + 2 * sizeof(C_t<R>) * (size_t)nact * N;
}

static int optin_smem() {
  int dev = 0, v = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  return v;
}

// 1: ready to launch, 0: does not fit (use the generic kernels), <0: -status
template <typename K> static int prep(K kernel, size_t bytes) {
  if ((long long)bytes > optin_smem()) return 0;
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared);
  if (e != cudaSuccess) return -cuda_fail(e, "cudaFuncSetAttribute(fast slab kernel)");
  return 1;
}

#define FAST_LAUNCHED(what)                                  \
  do {                                                       \
    ::jrg::count_launch();                                   \
    cudaError_t e_ = cudaGetLastError();                     \
    if (e_ != cudaSuccess) return -::jrg::cuda_fail(e_, what); \
    return 1;                                                \
  } while (0)

static bool g_line_prefetch = true;   // cp.async row prefetch in the adjoint line kernel

// bands per CTA of the forward plane pass (register prefetch of the next
// band); JRG_PLANE_FWD_BANDS overrides the default for measurements
static int plane_fwd_bands_per_cta() {
  static int v = [] {
    const char* e = std::getenv("JRG_PLANE_FWD_BANDS");
    const int x = e ? std::atoi(e) : 8;
    return x < 1 ? 1 : (x > 64 ? 64 : x);
  }();
  return v;
}

// the pruned adjoint line kernel prefetches the next band into registers
// unless JRG_LINE_ROWBUF=1 selects the shared-memory row buffer (measurements)
static bool line_rowbuf() {
  static bool v = [] {
    const char* e = std::getenv("JRG_LINE_ROWBUF");
    return e && std::atoi(e) != 0;
  }();
  return v;
}

// bands per CTA of the inverse plane pass (1: one CTA per (plane, band));
// JRG_PLANE_BANDS overrides the default for measurements.  At the 64^3 Si8
// cell: 1 -> 0.253 ms, 4 -> 0.246, 8 -> 0.235, 16 -> 0.239 (best step time,
// 522.5 vs 512.9 evals/s), 32 -> 0.260.  In the forward plane pass a staged
// next plane (shared memory) was slower (0.33 vs 0.28 ms); the register
// prefetch (k_plane_fwd_sphere_rp) leaves the single-stream phase time as it
// was (0.266 vs 0.265 ms) but, with fewer CTAs per launch, overlaps the other
// pipeline stream better: 581.4 vs 576.7 evals/s over three runs each.
static int plane_bands_per_cta() {
  static int v = [] {
    const char* e = std::getenv("JRG_PLANE_BANDS");
    const int x = e ? std::atoi(e) : 16;
    return x < 1 ? 1 : (x > 64 ? 64 : x);
  }();
  return v;
}

template <typename R, int N, bool PR>
static int plane_inv_mb_launch(const jrg_plan* P, const Args& a, const C_t<R>* tw, int bpc, size_t smb,
                               cudaStream_t st) {
  using C = C_t<R>;
  constexpr int T = threads_for<N>();
  int rc;
  if ((rc = prep(k_plane_inv_sphere_mb<R, N, PR>, smb)) <= 0) return rc;
  k_plane_inv_sphere_mb<R, N, PR><<<dim3(P->nact, (a.nbands + bpc - 1) / bpc), T, smb, st>>>(
      reinterpret_cast<const C*>(a.in), reinterpret_cast<C*>(a.out), P->d.row_off, P->d.rows,
      P->d.rowmap, tw, P->ng, P->nact, a.nbands, bpc);
  FAST_LAUNCHED("fast::k_plane_inv_sphere_mb");
}

template <typename R, int N, bool PR>
static int plane_fwd_launch(const jrg_plan* P, const Args& a, const C_t<R>* tw, cudaStream_t st) {
  using C = C_t<R>;
  constexpr int T = threads_for<N>();
  int rc;
  const size_t sm = plane_smem<R, N>();
  int bpc = plane_fwd_bands_per_cta();
  while (bpc > 1 && (long long)a.nbands * P->nact < 2LL * 2 * 152 * bpc) bpc /= 2;
  if (bpc >= 2) {
    if ((rc = prep(k_plane_fwd_sphere_rp<R, N, PR>, sm)) <= 0) return rc;
    k_plane_fwd_sphere_rp<R, N, PR><<<dim3(P->nact, (a.nbands + bpc - 1) / bpc), T, sm, st>>>(
        reinterpret_cast<const C*>(a.in), reinterpret_cast<const C*>(a.aux), reinterpret_cast<C*>(a.out),
        a.w, tk_table<R>(P), P->nb, a.band0, P->d.plane_off, P->d.sph_yz, P->d.row_off, P->d.rows, tw, P->ng,
        P->nact, P->nk, a.wscale, a.nbands, bpc);
    FAST_LAUNCHED("fast::k_plane_fwd_sphere_rp");
  }
  if ((rc = prep(k_plane_fwd_sphere<R, N, PR>, sm)) <= 0) return rc;
  k_plane_fwd_sphere<R, N, PR><<<dim3(P->nact, a.nbands), T, sm, st>>>(
      reinterpret_cast<const C*>(a.in), reinterpret_cast<const C*>(a.aux), reinterpret_cast<C*>(a.out),
      a.w, tk_table<R>(P), P->nb, a.band0, P->d.plane_off, P->d.sph_yz, P->d.row_off, P->d.rows, tw, P->ng,
      P->nact, P->nk, a.wscale);
  FAST_LAUNCHED("fast::k_plane_fwd_sphere");
}

template <typename R, int N, bool PR>
static int line_density_launch(const jrg_plan* P, const Args& a, const C_t<R>* tw, cudaStream_t st) {
  using C = C_t<R>;
  constexpr int T = threads_for<N>();
  int rc;
  const size_t sm = line_w_offset<R, N>() + sizeof(R) * (size_t)a.bands_per_group;
  if ((rc = prep(k_line_density<R, N, PR>, sm)) <= 0) return rc;
  const int ngroups = (a.nbands + a.bands_per_group - 1) / a.bands_per_group;
  k_line_density<R, N, PR><<<dim3(N, ngroups), T, sm, st>>>(
      reinterpret_cast<const C*>(a.in), reinterpret_cast<R*>(a.out), a.w, a.wscale, a.band0,
      a.nbands, a.bands_per_group, P->d.xact, tw, P->nact, a.gscale);
  FAST_LAUNCHED("fast::k_line_density");
}

template <typename R, int N, bool PR>
static int line_apply_v_launch(const jrg_plan* P, const Args& a, const C_t<R>* tw, cudaStream_t st) {
  using C = C_t<R>;
  constexpr int T = threads_for<N>();
  int rc;
  const int ngroups = (a.nbands + a.bands_per_group - 1) / a.bands_per_group;
  const size_t smp = line_pf_smem<R, N>(P->nact);
  if (g_line_prefetch && !(PR && !line_rowbuf()) && (long long)smp <= optin_smem()) {
    if ((rc = prep(k_line_apply_v<R, N, true, PR>, smp)) <= 0) return rc;
    k_line_apply_v<R, N, true, PR><<<dim3(N, ngroups), T, smp, st>>>(
        reinterpret_cast<C*>(a.out), reinterpret_cast<const R*>(a.aux), a.nbands, a.bands_per_group,
        P->d.xact, tw, P->nact);
    FAST_LAUNCHED("fast::k_line_apply_v");
  }
  const size_t sm = line_smem<R, N>();
  if ((rc = prep(k_line_apply_v<R, N, false, PR>, sm)) <= 0) return rc;
  k_line_apply_v<R, N, false, PR><<<dim3(N, ngroups), T, sm, st>>>(
      reinterpret_cast<C*>(a.out), reinterpret_cast<const R*>(a.aux), a.nbands, a.bands_per_group,
      P->d.xact, tw, P->nact);
  FAST_LAUNCHED("fast::k_line_apply_v");
}

template <typename R, int N>
static int run(const jrg_plan* P, int op, const Args& a, cudaStream_t st) {
  using C = C_t<R>;
  const C* tw = reinterpret_cast<const C*>(P->d.tw);   // x table first; all axes equal
  constexpr int T = threads_for<N>();
  int rc;
  switch (op) {
    case OP_PLANE_INV: {
      // several bands per CTA only while the grid still fills the GPU twice
      // over at two CTAs per SM (152 SMs); a smaller call runs one band per CTA
      int bpc = plane_bands_per_cta();
      while (bpc > 1 && (long long)a.nbands * P->nact < 2LL * 2 * 152 * bpc) bpc /= 2;
      if (bpc < 4) bpc = 1;
      const size_t smb = plane_mb_smem<R, N>(P->max_rows);
      if (bpc > 1 && (long long)smb <= optin_smem()) {
        if constexpr (Split<N>::N1 == 8) {
          if (P->yzprune) return plane_inv_mb_launch<R, N, true>(P, a, tw, bpc, smb, st);
        }
        return plane_inv_mb_launch<R, N, false>(P, a, tw, bpc, smb, st);
      }
      const size_t sm = plane_smem<R, N>();
      if ((rc = prep(k_plane_inv_sphere<R, N>, sm)) <= 0) return rc;
      k_plane_inv_sphere<R, N><<<dim3(P->nact, a.nbands), T, sm, st>>>(
          reinterpret_cast<const C*>(a.in), reinterpret_cast<C*>(a.out), P->d.plane_off, P->d.sph_yz,
          P->d.row_off, P->d.rows, tw, P->ng, P->nact);
      FAST_LAUNCHED("fast::k_plane_inv_sphere");
    }
    case OP_LINE_DENSITY: {
      if constexpr (Split<N>::N1 == 8) {
        if (P->xprune) return line_density_launch<R, N, true>(P, a, tw, st);
      }
      return line_density_launch<R, N, false>(P, a, tw, st);
    }
    case OP_LINE_APPLY_V: {
      if constexpr (Split<N>::N1 == 8) {
        if (P->xprune) return line_apply_v_launch<R, N, true>(P, a, tw, st);
      }
      return line_apply_v_launch<R, N, false>(P, a, tw, st);
    }
    default: {
      if constexpr (Split<N>::N1 == 8) {
        if (P->yzprune) return plane_fwd_launch<R, N, true>(P, a, tw, st);
      }
      return plane_fwd_launch<R, N, false>(P, a, tw, st);
    }
  }
}

static bool g_fast_enabled = true;

template <typename R>
int dispatch(const jrg_plan* P, int op, const Args& a, cudaStream_t st) {
  if (!g_fast_enabled || !(P->nx == P->ny && P->ny == P->nz)) return 0;
  switch (P->nx) {
    case 16: return run<R, 16>(P, op, a, st);
    case 24: return run<R, 24>(P, op, a, st);
    case 27: return run<R, 27>(P, op, a, st);
    case 32: return run<R, 32>(P, op, a, st);
    case 36: return run<R, 36>(P, op, a, st);
    case 48: return run<R, 48>(P, op, a, st);
    case 64: return run<R, 64>(P, op, a, st);
    case 96: return run<R, 96>(P, op, a, st);
    default: return 0;
  }
}

template int dispatch<float>(const jrg_plan*, int, const Args&, cudaStream_t);
template int dispatch<double>(const jrg_plan*, int, const Args&, cudaStream_t);

template <typename R, int N, int DIR>
static int dense_run(const C_t<R>* tw, int batch, bool real_in, const void* in, C_t<R>* scratch,
                     C_t<R>* out, double scale, cudaStream_t st) {
  using C = C_t<R>;
  constexpr int T = threads_for<N>();
  const size_t smp = sizeof(C) * (size_t)(N + N * (N + 1) + N * N);
  const size_t sml = sizeof(C) * (size_t)(N + N * N);
  int rc;
  if (real_in) {
    if ((rc = prep(k_plane_dense<R, N, DIR, true>, smp)) <= 0) return rc;
    k_plane_dense<R, N, DIR, true><<<dim3(N, batch), T, smp, st>>>(in, scratch, tw);
  } else {
    if ((rc = prep(k_plane_dense<R, N, DIR, false>, smp)) <= 0) return rc;
    k_plane_dense<R, N, DIR, false><<<dim3(N, batch), T, smp, st>>>(in, scratch, tw);
  }
  {
    ::jrg::count_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return -::jrg::cuda_fail(e, "fast::k_plane_dense");
  }
  if ((rc = prep(k_line_dense<R, N, DIR>, sml)) <= 0) return rc;
  k_line_dense<R, N, DIR><<<dim3(N, batch), T, sml, st>>>(scratch, out, tw, scale);
  FAST_LAUNCHED("fast::k_line_dense");
}

template <typename R, int N>
static int dense_dir(const C_t<R>* tw, int batch, int dir, bool real_in, const void* in,
                     C_t<R>* scratch, C_t<R>* out, double scale, cudaStream_t st) {
  return dir < 0 ? dense_run<R, N, -1>(tw, batch, real_in, in, scratch, out, scale, st)
                 : dense_run<R, N, +1>(tw, batch, real_in, in, scratch, out, scale, st);
}

template <typename R>
int dispatch_dense(const FftAxis* ax, const C_t<R>* tw, int batch, int dir, bool real_in,
                   const void* in, C_t<R>* scratch, C_t<R>* out, double scale, cudaStream_t st) {
  if (!g_fast_enabled || !(ax[0].n == ax[1].n && ax[1].n == ax[2].n)) return 0;
  switch (ax[0].n) {
    case 16: return dense_dir<R, 16>(tw, batch, dir, real_in, in, scratch, out, scale, st);
    case 24: return dense_dir<R, 24>(tw, batch, dir, real_in, in, scratch, out, scale, st);
    case 27: return dense_dir<R, 27>(tw, batch, dir, real_in, in, scratch, out, scale, st);
    case 32: return dense_dir<R, 32>(tw, batch, dir, real_in, in, scratch, out, scale, st);
    case 36: return dense_dir<R, 36>(tw, batch, dir, real_in, in, scratch, out, scale, st);
    case 48: return dense_dir<R, 48>(tw, batch, dir, real_in, in, scratch, out, scale, st);
    case 64: return dense_dir<R, 64>(tw, batch, dir, real_in, in, scratch, out, scale, st);
    case 96: return dense_dir<R, 96>(tw, batch, dir, real_in, in, scratch, out, scale, st);
    default: return 0;
  }
}

template int dispatch_dense<float>(const FftAxis*, const C_t<float>*, int, int, bool, const void*,
                                   C_t<float>*, C_t<float>*, double, cudaStream_t);
template int dispatch_dense<double>(const FftAxis*, const C_t<double>*, int, int, bool, const void*,
                                    C_t<double>*, C_t<double>*, double, cudaStream_t);

}  // namespace fast
}  // namespace jrg

namespace jrg { void set_gram_rb(bool on); }

extern "C" int jrg_fast_paths(int enable) {
  const int prev = jrg::fast::g_fast_enabled ? 1 : 0;
  if (enable >= 0) {
    jrg::fast::g_fast_enabled = enable != 0;
    jrg::set_gram_rb(enable != 0);
  }
  return prev;
}
