// Plane-wave sphere <-> real-space grid transforms.
//
// A 3-D transform is split into two kernels so that each CTA holds a whole
// 2-D slab in shared memory:
//   plane kernels: one CTA per (band, x plane): the y and z transforms of the
//                  plane, with the sphere scatter/gather fused in;
//   line kernels:  one CTA per (band group, y row): the x transforms of an
//                  (x, z) slab, with |psi|^2 accumulation (density) or the
//                  multiply by V(r) between the inverse and forward x
//                  transforms (adjoint) fused in.
// Only x planes that intersect the sphere ("active planes") and, inside them,
// only y rows that hold sphere points are transformed where the data are
// known to be zero.  The intermediate between the two kernels holds only the
// active planes: [band][active plane][y][z].
#include "fast_dispatch.h"
#include "plan.h"

namespace jrg {

// ------------------------------------------------------------------------
// inverse: sphere coefficients -> active planes (y, z transformed)
// ------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(256) k_plane_inv_sphere(
    const C_t<R>* __restrict__ coef, C_t<R>* __restrict__ planes, const int* __restrict__ plane_off,
    const int* __restrict__ sph_yz, const int* __restrict__ row_off, const int* __restrict__ rows,
    const C_t<R>* __restrict__ tw_y, const C_t<R>* __restrict__ tw_z, FftAxis axy, FftAxis axz,
    int ny, int nz, int ng, int nact) {
  using C = C_t<R>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int plane = ny * nz;
  C* twy = reinterpret_cast<C*>(smem_raw);
  C* twz = twy + ny;
  C* A = twz + nz;
  C* B = A + plane;
  int* srows = reinterpret_cast<int*>(B + plane);
  const int p = blockIdx.x;
  const int band = blockIdx.y;
  for (int i = threadIdx.x; i < ny; i += blockDim.x) twy[i] = tw_y[i];
  for (int i = threadIdx.x; i < nz; i += blockDim.x) twz[i] = tw_z[i];
  const C z0 = czero<C>();
  for (int i = threadIdx.x; i < 2 * plane; i += blockDim.x) A[i] = z0;
  const int r0 = row_off[p], nr = row_off[p + 1] - r0;
  for (int i = threadIdx.x; i < nr; i += blockDim.x) srows[i] = rows[r0 + i];
  __syncthreads();
  const C* cb = coef + (size_t)band * ng;
  for (int e = plane_off[p] + threadIdx.x; e < plane_off[p + 1]; e += blockDim.x) A[sph_yz[e]] = cb[e];
  __syncthreads();
  C* r1 = fft_lines<+1>(A, B, twz, axz, nr, 1, nz, srows, false);
  C* o1 = (r1 == A) ? B : A;
  C* r2 = fft_lines<+1>(r1, o1, twy, axy, nz, nz, 1, nullptr, true);
  C* out = planes + ((size_t)band * nact + p) * plane;
  for (int i = threadIdx.x; i < plane; i += blockDim.x) out[i] = r2[i];
}

// ------------------------------------------------------------------------
// inverse x transform + occupation-weighted |psi|^2 of a band group
// ------------------------------------------------------------------------
// shared memory of the line kernels: twiddles, two slabs, extra reals and ints
template <typename R> __host__ __device__ size_t line_smem(int nx, int nz, int extra_real, int extra_int) {
  return sizeof(C_t<R>) * (size_t)(nx + 2 * nx * nz) + sizeof(R) * (size_t)extra_real +
         sizeof(int) * (size_t)extra_int;
}

constexpr int kLineThreads = 256;
constexpr int kMaxPtsPerThread = 48;   // nx*nz <= 256*48 (up to 96 x 128)

template <typename R>
__global__ void __launch_bounds__(kLineThreads) k_line_density(
    const C_t<R>* __restrict__ planes, R* __restrict__ rho_part, const double* __restrict__ wband,
    double wscale, int band0, int nband, int bands_per_group, const int* __restrict__ plane_x,
    const int* __restrict__ xact, const C_t<R>* __restrict__ tw_x, FftAxis axx, int nx, int ny,
    int nz, int nact, double* __restrict__ gscale) {
  using C = C_t<R>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int slab = nx * nz;
  C* twx = reinterpret_cast<C*>(smem_raw);
  C* A = twx + nx;
  C* B = A + slab;
  int* sxact = reinterpret_cast<int*>(B + slab);
  // weights relative to the group's largest (see the fast kernel)
  R* sw = reinterpret_cast<R*>(smem_raw + align16(line_smem<R>(nx, nz, 0, nx)));
  const int y = blockIdx.x;
  const int grp = blockIdx.y;
  const int b_begin = grp * bands_per_group;
  const int b_end = min(nband, b_begin + bands_per_group);
  for (int i = threadIdx.x; i < nx; i += blockDim.x) { twx[i] = tw_x[i]; sxact[i] = xact[i]; }
  group_weights<R>(wband + band0, b_begin, b_end, wscale, gscale, grp, sw);
  R acc[kMaxPtsPerThread];
#pragma unroll
  for (int k = 0; k < kMaxPtsPerThread; ++k) acc[k] = (R)0;
  __syncthreads();
  const C z0 = czero<C>();
  for (int b = b_begin; b < b_end; ++b) {
    const R w = sw[b - b_begin];
    // inactive x rows are zero; active rows come from the plane buffer
    for (int i = threadIdx.x; i < slab; i += blockDim.x) {
      const int x = i / nz, z = i - x * nz;
      const int pa = sxact[x];
      A[i] = (pa < 0) ? z0 : planes[(((size_t)b * nact + pa) * ny + y) * nz + z];
    }
    __syncthreads();
    C* res = fft_lines<+1>(A, B, twx, axx, nz, nz, 1, nullptr, true);
#pragma unroll
    for (int k = 0; k < kMaxPtsPerThread; ++k) {
      const int i = threadIdx.x + k * blockDim.x;
      if (i < slab) {
        const C v = res[i];
        acc[k] += w * (v.x * v.x + v.y * v.y);
      }
    }
    __syncthreads();
  }
  R* out = rho_part + (size_t)grp * nx * ny * nz;
#pragma unroll
  for (int k = 0; k < kMaxPtsPerThread; ++k) {
    const int i = threadIdx.x + k * blockDim.x;
    if (i < slab) {
      const int x = i / nz, z = i - x * nz;
      out[((size_t)x * ny + y) * nz + z] = acc[k];
    }
  }
}

// ------------------------------------------------------------------------
// adjoint line pass: inverse x transform, multiply by V(r), forward x
// transform, keep the active planes
// ------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(kLineThreads) k_line_apply_v(
    const C_t<R>* __restrict__ planes_in, C_t<R>* __restrict__ planes_out,
    const R* __restrict__ vr, int nband, int bands_per_group, const int* __restrict__ plane_x,
    const int* __restrict__ xact, const C_t<R>* __restrict__ tw_x, FftAxis axx, int nx, int ny,
    int nz, int nact) {
  using C = C_t<R>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int slab = nx * nz;
  C* twx = reinterpret_cast<C*>(smem_raw);
  C* A = twx + nx;
  C* B = A + slab;
  R* sv = reinterpret_cast<R*>(B + slab);
  int* sxact = reinterpret_cast<int*>(sv + slab);
  int* spx = sxact + nx;
  const int y = blockIdx.x;
  const int grp = blockIdx.y;
  for (int i = threadIdx.x; i < nx; i += blockDim.x) { twx[i] = tw_x[i]; sxact[i] = xact[i]; }
  for (int i = threadIdx.x; i < nact; i += blockDim.x) spx[i] = plane_x[i];
  for (int i = threadIdx.x; i < slab; i += blockDim.x) {
    const int x = i / nz, z = i - x * nz;
    sv[i] = vr[((size_t)x * ny + y) * nz + z];
  }
  __syncthreads();
  const int b_begin = grp * bands_per_group;
  const int b_end = min(nband, b_begin + bands_per_group);
  const C z0 = czero<C>();
  for (int b = b_begin; b < b_end; ++b) {
    for (int i = threadIdx.x; i < slab; i += blockDim.x) {
      const int x = i / nz, z = i - x * nz;
      const int pa = sxact[x];
      A[i] = (pa < 0) ? z0 : planes_in[(((size_t)b * nact + pa) * ny + y) * nz + z];
    }
    __syncthreads();
    C* res = fft_lines<+1>(A, B, twx, axx, nz, nz, 1, nullptr, true);
    for (int i = threadIdx.x; i < slab; i += blockDim.x) res[i] = cscale(res[i], sv[i]);
    __syncthreads();
    C* oth = (res == A) ? B : A;
    C* res2 = fft_lines<-1>(res, oth, twx, axx, nz, nz, 1, nullptr, true);
    for (int i = threadIdx.x; i < nact * nz; i += blockDim.x) {
      const int pa = i / nz, z = i - pa * nz;
      planes_out[(((size_t)b * nact + pa) * ny + y) * nz + z] = res2[spx[pa] * nz + z];
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------------
// forward: active planes -> y, z transforms -> sphere gather, combined with
// the kinetic term into the coefficient gradient
//   g[b][e] = f_b * (tk[k][e] * c[b][e] + scale * FFT(V psi_b)[e])
// ------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(256) k_plane_fwd_sphere(
    const C_t<R>* __restrict__ planes, const C_t<R>* __restrict__ coef, C_t<R>* __restrict__ gcoef,
    const double* __restrict__ wband, const double* __restrict__ tk, int nb_per_k, int band0,
    const int* __restrict__ plane_off, const int* __restrict__ sph_yz, const int* __restrict__ row_off,
    const int* __restrict__ rows, const C_t<R>* __restrict__ tw_y, const C_t<R>* __restrict__ tw_z,
    FftAxis axy, FftAxis axz, int ny, int nz, int ng, int nact, int nk, double scale) {
  using C = C_t<R>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int plane = ny * nz;
  C* twy = reinterpret_cast<C*>(smem_raw);
  C* twz = twy + ny;
  C* A = twz + nz;
  C* B = A + plane;
  int* srows = reinterpret_cast<int*>(B + plane);
  const int p = blockIdx.x;
  const int band = blockIdx.y;
  for (int i = threadIdx.x; i < ny; i += blockDim.x) twy[i] = tw_y[i];
  for (int i = threadIdx.x; i < nz; i += blockDim.x) twz[i] = tw_z[i];
  const int r0 = row_off[p], nr = row_off[p + 1] - r0;
  for (int i = threadIdx.x; i < nr; i += blockDim.x) srows[i] = rows[r0 + i];
  const C* in = planes + ((size_t)band * nact + p) * plane;
  for (int i = threadIdx.x; i < plane; i += blockDim.x) A[i] = in[i];
  __syncthreads();
  C* r1 = fft_lines<-1>(A, B, twy, axy, nz, nz, 1, nullptr, true);
  C* o1 = (r1 == A) ? B : A;
  C* r2 = fft_lines<-1>(r1, o1, twz, axz, nr, 1, nz, srows, false);
  const int gb = band0 + band;                 // global band index (s, k, b)
  const int kidx = (gb / nb_per_k) % nk;
  const R w = (R)wband[gb];
  const double* tkk = tk + (size_t)kidx * ng;
  const C* cb = coef + (size_t)band * ng;
  C* gout = gcoef + (size_t)band * ng;
  for (int e = plane_off[p] + threadIdx.x; e < plane_off[p + 1]; e += blockDim.x) {
    const C v = r2[sph_yz[e]];
    const C c = cb[e];
    const R t = (R)tkk[e];
    C g;
    g.x = w * (t * c.x + (R)scale * v.x);
    g.y = w * (t * c.y + (R)scale * v.y);
    gout[e] = g;
  }
}

// ------------------------------------------------------------------------
// dense transforms of whole grids [batch][nx][ny][nz]
// ------------------------------------------------------------------------
template <typename R, int DIR, bool REAL_IN>
__global__ void __launch_bounds__(256) k_plane_dense(const void* __restrict__ in_v,
                                                     C_t<R>* __restrict__ out,
                                                     const C_t<R>* __restrict__ tw_y,
                                                     const C_t<R>* __restrict__ tw_z, FftAxis axy,
                                                     FftAxis axz, int nx, int ny, int nz) {
  using C = C_t<R>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int plane = ny * nz;
  C* twy = reinterpret_cast<C*>(smem_raw);
  C* twz = twy + ny;
  C* A = twz + nz;
  C* B = A + plane;
  const int x = blockIdx.x;
  const size_t base = ((size_t)blockIdx.y * nx + x) * plane;
  for (int i = threadIdx.x; i < ny; i += blockDim.x) twy[i] = tw_y[i];
  for (int i = threadIdx.x; i < nz; i += blockDim.x) twz[i] = tw_z[i];
  if constexpr (REAL_IN) {
    const R* in = reinterpret_cast<const R*>(in_v) + base;
    for (int i = threadIdx.x; i < plane; i += blockDim.x) { C v; v.x = in[i]; v.y = 0; A[i] = v; }
  } else {
    const C* in = reinterpret_cast<const C*>(in_v) + base;
    for (int i = threadIdx.x; i < plane; i += blockDim.x) A[i] = in[i];
  }
  __syncthreads();
  C* r1 = fft_lines<DIR>(A, B, twz, axz, ny, 1, nz, nullptr, false);
  C* o1 = (r1 == A) ? B : A;
  C* r2 = fft_lines<DIR>(r1, o1, twy, axy, nz, nz, 1, nullptr, true);
  for (int i = threadIdx.x; i < plane; i += blockDim.x) out[base + i] = r2[i];
}

template <typename R, int DIR>
__global__ void __launch_bounds__(kLineThreads) k_line_dense(const C_t<R>* __restrict__ in,
                                                             C_t<R>* __restrict__ out,
                                                             const C_t<R>* __restrict__ tw_x,
                                                             FftAxis axx, int nx, int ny, int nz,
                                                             double scale) {
  using C = C_t<R>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int slab = nx * nz;
  C* twx = reinterpret_cast<C*>(smem_raw);
  C* A = twx + nx;
  C* B = A + slab;
  const int y = blockIdx.x;
  const size_t base = (size_t)blockIdx.y * nx * ny * nz;
  for (int i = threadIdx.x; i < nx; i += blockDim.x) twx[i] = tw_x[i];
  for (int i = threadIdx.x; i < slab; i += blockDim.x) {
    const int x = i / nz, z = i - x * nz;
    A[i] = in[base + ((size_t)x * ny + y) * nz + z];
  }
  __syncthreads();
  C* res = fft_lines<DIR>(A, B, twx, axx, nz, nz, 1, nullptr, true);
  for (int i = threadIdx.x; i < slab; i += blockDim.x) {
    const int x = i / nz, z = i - x * nz;
    out[base + ((size_t)x * ny + y) * nz + z] = cscale(res[i], (R)scale);
  }
}

// ------------------------------------------------------------------------
// host launchers
// ------------------------------------------------------------------------
template <typename R> size_t plane_smem(int ny, int nz, int max_rows) {
  return sizeof(C_t<R>) * (size_t)(ny + nz + 2 * ny * nz) + sizeof(int) * (size_t)(max_rows + 1);
}

template <typename K> static int set_smem(K kernel, size_t bytes) {
  if (bytes > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(smem)");
  }
  return JRG_OK;
}

template <typename R>
int launch_plane_inv_sphere(const jrg_plan* P, const void* coef, void* planes, int nbands,
                            cudaStream_t st) {
  using C = C_t<R>;
  {
    fast::Args a{coef, planes, nullptr, nullptr, 0.0, 0, nbands, 1};
    const int f = fast::dispatch<R>(P, fast::OP_PLANE_INV, a, st);
    if (f < 0) return -f;
    if (f > 0) return JRG_OK;
  }
  const C* tw = reinterpret_cast<const C*>(P->d.tw);
  size_t sm = plane_smem<R>(P->ny, P->nz, P->max_rows);
  int rc = set_smem(k_plane_inv_sphere<R>, sm);
  if (rc) return rc;
  dim3 grid(P->nact, nbands);
  k_plane_inv_sphere<R><<<grid, 256, sm, st>>>(
      reinterpret_cast<const C*>(coef), reinterpret_cast<C*>(planes), P->d.plane_off, P->d.sph_yz,
      P->d.row_off, P->d.rows, tw + P->nx, tw + P->nx + P->ny, P->ax[1], P->ax[2], P->ny, P->nz,
      P->ng, P->nact);
  JRG_LAUNCH_CHECK("k_plane_inv_sphere");
  return JRG_OK;
}

template <typename R>
int launch_line_density(const jrg_plan* P, const void* planes, void* rho_part, const double* wband,
                        double wscale, int band0, int nbands, int bands_per_group, double* gscale,
                        cudaStream_t st) {
  using C = C_t<R>;
  {
    fast::Args a{planes, rho_part, nullptr, wband, wscale, band0, nbands, bands_per_group, gscale};
    const int f = fast::dispatch<R>(P, fast::OP_LINE_DENSITY, a, st);
    if (f < 0) return -f;
    if (f > 0) return JRG_OK;
  }
  const C* tw = reinterpret_cast<const C*>(P->d.tw);
  size_t sm = align16(line_smem<R>(P->nx, P->nz, 0, P->nx)) + sizeof(R) * (size_t)bands_per_group;
  int rc = set_smem(k_line_density<R>, sm);
  if (rc) return rc;
  const int ngroups = (nbands + bands_per_group - 1) / bands_per_group;
  dim3 grid(P->ny, ngroups);
  k_line_density<R><<<grid, kLineThreads, sm, st>>>(
      reinterpret_cast<const C*>(planes), reinterpret_cast<R*>(rho_part), wband, wscale, band0, nbands,
      bands_per_group, P->d.plane_x, P->d.xact, tw, P->ax[0], P->nx, P->ny, P->nz, P->nact, gscale);
  JRG_LAUNCH_CHECK("k_line_density");
  return JRG_OK;
}

template <typename R>
int launch_line_apply_v(const jrg_plan* P, const void* planes_in, void* planes_out, const void* vr,
                        int nbands, int bands_per_group, cudaStream_t st) {
  using C = C_t<R>;
  if (planes_in == planes_out) {   // the fast kernel works in place
    fast::Args a{planes_in, planes_out, vr, nullptr, 0.0, 0, nbands, bands_per_group};
    const int f = fast::dispatch<R>(P, fast::OP_LINE_APPLY_V, a, st);
    if (f < 0) return -f;
    if (f > 0) return JRG_OK;
  }
  const C* tw = reinterpret_cast<const C*>(P->d.tw);
  size_t sm = line_smem<R>(P->nx, P->nz, P->nx * P->nz, P->nx + P->nact);
  int rc = set_smem(k_line_apply_v<R>, sm);
  if (rc) return rc;
  const int ngroups = (nbands + bands_per_group - 1) / bands_per_group;
  dim3 grid(P->ny, ngroups);
  k_line_apply_v<R><<<grid, kLineThreads, sm, st>>>(
      reinterpret_cast<const C*>(planes_in), reinterpret_cast<C*>(planes_out),
      reinterpret_cast<const R*>(vr), nbands, bands_per_group, P->d.plane_x, P->d.xact, tw,
      P->ax[0], P->nx, P->ny, P->nz, P->nact);
  JRG_LAUNCH_CHECK("k_line_apply_v");
  return JRG_OK;
}

template <typename R>
int launch_plane_fwd_sphere(const jrg_plan* P, const void* planes, const void* coef, void* gcoef,
                            const double* wband, int band0, int nbands, double scale,
                            cudaStream_t st) {
  using C = C_t<R>;
  {
    fast::Args a{planes, gcoef, coef, wband, scale, band0, nbands, 1};
    const int f = fast::dispatch<R>(P, fast::OP_PLANE_FWD, a, st);
    if (f < 0) return -f;
    if (f > 0) return JRG_OK;
  }
  const C* tw = reinterpret_cast<const C*>(P->d.tw);
  size_t sm = plane_smem<R>(P->ny, P->nz, P->max_rows);
  int rc = set_smem(k_plane_fwd_sphere<R>, sm);
  if (rc) return rc;
  dim3 grid(P->nact, nbands);
  k_plane_fwd_sphere<R><<<grid, 256, sm, st>>>(
      reinterpret_cast<const C*>(planes), reinterpret_cast<const C*>(coef),
      reinterpret_cast<C*>(gcoef), wband, P->d.tk, P->nb, band0, P->d.plane_off, P->d.sph_yz,
      P->d.row_off, P->d.rows, tw + P->nx, tw + P->nx + P->ny, P->ax[1], P->ax[2], P->ny, P->nz,
      P->ng, P->nact, P->nk, scale);
  JRG_LAUNCH_CHECK("k_plane_fwd_sphere");
  return JRG_OK;
}

// Dense batched 3-D transform with explicit axes/twiddles (used for single
// grids: density -> reciprocal density, potential -> real space, and the
// public jrg_fft3d).  `scratch` holds [batch][nx][ny][nz] complex.
template <typename R>
int launch_fft3d_dense(const FftAxis* ax, const C_t<R>* tw, int batch, int dir, bool real_in,
                       const void* in, C_t<R>* scratch, C_t<R>* out, double scale,
                       cudaStream_t st) {
  using C = C_t<R>;
  {
    const int f = fast::dispatch_dense<R>(ax, tw, batch, dir, real_in, in, scratch, out, scale, st);
    if (f < 0) return -f;
    if (f > 0) return JRG_OK;
  }
  const int nx = ax[0].n, ny = ax[1].n, nz = ax[2].n;
  size_t smp = plane_smem<R>(ny, nz, 0);
  size_t sml = line_smem<R>(nx, nz, 0, 0);
  dim3 gp(nx, batch), gl(ny, batch);
  int rc;
  if (dir < 0) {
    if (real_in) {
      if ((rc = set_smem(k_plane_dense<R, -1, true>, smp))) return rc;
      k_plane_dense<R, -1, true><<<gp, 256, smp, st>>>(in, scratch, tw + nx, tw + nx + ny, ax[1], ax[2], nx, ny, nz);
    } else {
      if ((rc = set_smem(k_plane_dense<R, -1, false>, smp))) return rc;
      k_plane_dense<R, -1, false><<<gp, 256, smp, st>>>(in, scratch, tw + nx, tw + nx + ny, ax[1], ax[2], nx, ny, nz);
    }
    JRG_LAUNCH_CHECK("k_plane_dense");
    if ((rc = set_smem(k_line_dense<R, -1>, sml))) return rc;
    k_line_dense<R, -1><<<gl, kLineThreads, sml, st>>>(scratch, out, tw, ax[0], nx, ny, nz, scale);
  } else {
    if (real_in) {
      if ((rc = set_smem(k_plane_dense<R, +1, true>, smp))) return rc;
      k_plane_dense<R, +1, true><<<gp, 256, smp, st>>>(in, scratch, tw + nx, tw + nx + ny, ax[1], ax[2], nx, ny, nz);
    } else {
      if ((rc = set_smem(k_plane_dense<R, +1, false>, smp))) return rc;
      k_plane_dense<R, +1, false><<<gp, 256, smp, st>>>(in, scratch, tw + nx, tw + nx + ny, ax[1], ax[2], nx, ny, nz);
    }
    JRG_LAUNCH_CHECK("k_plane_dense");
    if ((rc = set_smem(k_line_dense<R, +1>, sml))) return rc;
    k_line_dense<R, +1><<<gl, kLineThreads, sml, st>>>(scratch, out, tw, ax[0], nx, ny, nz, scale);
  }
  JRG_LAUNCH_CHECK("k_line_dense");
  return JRG_OK;
}

#define JRG_INST(R)                                                                              \
  template int launch_plane_inv_sphere<R>(const jrg_plan*, const void*, void*, int, cudaStream_t); \
  template int launch_line_density<R>(const jrg_plan*, const void*, void*, const double*, double, \
                                      int, int, int, double*, cudaStream_t);                     \
  template int launch_line_apply_v<R>(const jrg_plan*, const void*, void*, const void*, int, int,   \
                                      cudaStream_t);                                             \
  template int launch_plane_fwd_sphere<R>(const jrg_plan*, const void*, const void*, void*,        \
                                          const double*, int, int, double, cudaStream_t);        \
  template int launch_fft3d_dense<R>(const FftAxis*, const C_t<R>*, int, int, bool, const void*,   \
                                     C_t<R>*, C_t<R>*, double, cudaStream_t);
JRG_INST(float)
JRG_INST(double)

}  // namespace jrg
