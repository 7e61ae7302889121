// C ABI of the library: plan construction, workspace layout and the entry
// points declared in include/jrystal_gb300.h.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include "plan.h"

namespace jrg {

// ---- launchers implemented in the kernel files ----
template <typename R> int launch_plane_inv_sphere(const jrg_plan*, const void*, void*, int, cudaStream_t);
template <typename R> int launch_line_density(const jrg_plan*, const void*, void*, const double*, double, int, int, int, double*, cudaStream_t);
template <typename R> int launch_line_apply_v(const jrg_plan*, const void*, void*, const void*, int, int, cudaStream_t);
template <typename R> int launch_plane_fwd_sphere(const jrg_plan*, const void*, const void*, void*, const double*, int, int, double, cudaStream_t);
template <typename R> int launch_fft3d_dense(const FftAxis*, const C_t<R>*, int, int, bool, const void*, C_t<R>*, C_t<R>*, double, cudaStream_t);
template <typename R> int launch_pack_params(const void*, const void*, void*, int, int, int, bool, cudaStream_t);
template <typename R> int launch_unpack(const void*, void*, void*, void*, int, int, int, double, cudaStream_t);
template <typename R> int launch_gram(int, const void*, const void*, int, const void*, const void*, double2*, double2*, int, int, int, int, cudaStream_t, int* = nullptr, bool = false);
int launch_cholesky_inv(const double2*, double2*, double2*, int, int, int*, double*, cudaStream_t, double, bool);
int launch_adjoint_small(const double2*, const double2*, double2*, double2*, int, int, cudaStream_t,
                         const double* = nullptr, double* = nullptr);
template <typename R> int launch_rotate(int, int, const void*, const void*, const double2*, const void*, const double2*, void*, void*, int, int, int, double, void*, cudaStream_t, int = 0);
constexpr int kTriUpper = 1, kTriLower = 2;   // zero pattern of a rotation's first matrix: R^-1, R^-H
constexpr int kSplit = 0, kBand = 1;           // tall-operand layouts (k_orth.cu)
constexpr int kRotBand = 0, kRotGC = 1, kRotGSplit = 2;
template <typename R> int launch_reduce_density(const void*, void*, int, int, long long, const double*, double*, cudaStream_t);
template <typename R> int launch_recip_terms(const void*, const double*, void*, double*, int, long long, double, const ChargeFix&, cudaStream_t);
template <typename R> int launch_potential(const void*, const void*, double, void*, double*, int, long long, int, double, const double*, const double*, double*, cudaStream_t);
template <typename R> int launch_xc_field(const void*, void*, long long, int, int, cudaStream_t);
template <typename R> int launch_potential_pol(const void*, const void*, double, void*, double*, int, long long, int, double, const double*, const double*, double*, cudaStream_t);
template <typename R> int launch_spin_total(const void*, void*, long long, cudaStream_t);
template <typename R> int launch_real_part(const void*, void*, long long, double, cudaStream_t);
template <typename R> int launch_hartree_g(const void*, const double*, void*, long long, double, cudaStream_t);
template <typename R> int launch_kinetic(const void*, const double*, const double*, double*, double*, int, int, int, int, cudaStream_t);
int launch_precond_scale(const float*, const void*, const double*, const double*, const double*, int, int, int, long long, float, float, float*, cudaStream_t);
int launch_precond_scale_lut(const float*, const void*, const double*, const float*, float, const double*,
                             const double*, int, int, int, int, long long, float, float, float*, float*,
                             cudaStream_t);
size_t precond_lut_floats(int nb, int nbt);
int launch_sum_slots(const double*, const int*, double*, int, const int*, int, cudaStream_t);
int nl_splits(int ng, int nsk, int nb, int np);
int nl_chunks(int nb, int np);
template <typename R> int launch_nl_project(const void*, const void*, double2*, int, int, int, int, int, int, int, cudaStream_t);
int launch_nl_reduce(const double2*, double2*, const double*, const double*, double*, int, int, int, int, double, cudaStream_t);
template <typename R> int launch_nl_apply(void*, const void*, const double2*, int, int, int, int, int, int, cudaStream_t);
int launch_band_trace_sums(const double2*, int, int, const double*, int, double*, cudaStream_t);
int launch_kin_reduce(int, const void*, int, int, int, const double*, double*, double*, cudaStream_t);
template <typename R> int launch_rotate_kinetic(const void*, const void*, const double2*, void*, int, int, int, const double*, int, void*, cudaStream_t, int = 0);
template <typename R> int launch_mul_ig(const void*, const double*, void*, int, long long, double, cudaStream_t);
template <typename R> int launch_gga_local(const void*, void*, void*, void*, void*, double*, int, long long, int, double, int, const double*, const double*, double*, cudaStream_t);
template <typename R> int launch_div_g(void*, const void*, const void*, const double*, long long, double, cudaStream_t);
template <typename R> int launch_potential_gga(const void*, double, void*, const void*, long long, const double*, cudaStream_t);
constexpr int kXcGga = JRG_XC_GGA_X_PBE | JRG_XC_GGA_C_PBE;
template <typename R> int launch_geometry_tables(double*, double*, void*, double2*, const double*, const double*, const double*, int, int, int, int, double, cudaStream_t);
int launch_ewald(const double*, const double*, const double*, const double*, int, int, long long, double, double, double*, int, double*, cudaStream_t);
template <typename R> int launch_adam(void*, const void*, void*, void*, const float*, long long, double, double, double, double, double, double, cudaStream_t, const int* = nullptr, const double* = nullptr);
int launch_twiddles(int n, int prec, void* out, cudaStream_t st);
template <typename R> int launch_reorthonormalise(void*, void*, double2*, int, int, int, cudaStream_t);
int launch_dft_axis_inv_f64(const double2*, double2*, int, int, int, int, const double2*, cudaStream_t);
template <typename R> int launch_rotate_adam(const void*, const double2*, const void*, const double2*, const AdamArgs&, int, int, int, double, cudaStream_t);
int launch_lda(int prec, long long n, int xc, int ks, const void* rho, void* out, cudaStream_t st);
int launch_lda_pol(int prec, long long n, int xc, int ks, const void* rho, void* out, cudaStream_t st);

static thread_local std::string g_err;
static std::atomic<long long> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void set_error(const std::string& m) { g_err = m; }
int fail(int code, const std::string& m) { g_err = m; return code; }
int cuda_fail(cudaError_t e, const char* what) {
  g_err = std::string(what) + ": " + cudaGetErrorString(e);
  return JRG_ERR_CUDA;
}

bool factor_axis(int n, FftAxis* ax) {
  ax->n = n;
  ax->nrad = 0;
  int m = n;
  const int rads[5] = {4, 2, 3, 5, 7};
  for (int r : rads) {
    while (m % r == 0) {
      if (ax->nrad >= kMaxRadices) return false;
      ax->rad[ax->nrad++] = r;
      m /= r;
    }
  }
  return m == 1 && n >= 1;
}

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// energy slot layout
constexpr int kRecipBlocks = 256;   // CTAs (and energy slots) of the reciprocal-space terms
constexpr int kXcBlocks = 256;      // CTAs (and energy slots) of the xc terms (1024: 0.093 vs 0.081 ms)
constexpr int kEwaldBlocks = 512;

static int csize(int prec) { return prec == 64 ? 16 : 8; }
static int rsize(int prec) { return prec == 64 ? 8 : 4; }

static void layout_workspace_k(jrg_plan* P, int kc);

// Workspace layout; with a memory limit the plane buffer holds only as many
// (s,k) blocks as fit (at least one), and the energy entry points process the
// blocks in chunks, transforming each chunk's coefficients again for the
// adjoint instead of keeping all planes from the density pass.
static void layout_workspace(jrg_plan* P) {
  const int nsk = P->ns * P->nk;
  layout_workspace_k(P, nsk);
  if (P->mem_limit == 0 || P->ws.total <= P->mem_limit) return;
  const size_t per_k = (size_t)P->nb * P->nact * P->ny * P->nz * csize(P->prec);
  const size_t fixed = P->ws.total - P->ws.t_bytes;
  int kc = P->mem_limit > fixed ? (int)((P->mem_limit - fixed) / per_k) : 1;
  kc = std::max(1, std::min(kc, nsk));
  layout_workspace_k(P, kc);
}

static void layout_workspace_k(jrg_plan* P, int kc) {
  P->kchunk = kc;
  Workspace& w = P->ws;
  const size_t C = csize(P->prec), Rz = rsize(P->prec);
  const size_t nsk = (size_t)P->ns * P->nk, nbt = nsk * P->nb;
  const size_t b2 = (size_t)P->nb * P->nb * sizeof(double2);
  // enough (s,k,split) CTAs to fill the GPU several times over: ~256 G rows each
  w.gram_splits = std::max(1, std::min(512, (int)((P->ng + 255) / 256)));
  w.ngroups = (int)nsk;
  // slots: kinetic [nbt], external, Hartree, xc [256 each], nonlocal
  // [nsk * nl_chunks] (one per reduction CTA)
  w.nepart = (int)nbt + 2 * kRecipBlocks + kXcBlocks +
             (int)nsk * (P->nproj > 0 ? nl_chunks(P->nb, P->nproj) : 1);
  if (w.nepart < 2 * kEwaldBlocks) w.nepart = 2 * kEwaldBlocks;
  size_t o = 0;
  auto take = [&](size_t bytes) { size_t r = o; o += align256(bytes); return r; };
  w.wc = 0;                             // parameters are read in place
  w.c = take(nbt * P->ng * C);
  {
    // CUDA-core partials: nb^2 complex; tensor-core partials: (2nb rounded to 16)^2 real
    const size_t mp = (size_t)((2 * P->nb + 15) / 16 * 16);
    w.gram_part = take(nsk * w.gram_splits * std::max(b2, mp * mp * sizeof(double)));
  }
  w.gram = take(nsk * b2);
  w.rmat = take(nsk * b2);
  w.rinv = take(nsk * b2);
  w.adj = take(nsk * b2);
  w.kmat = take(2 * nsk * b2);          // R^{-H} and -K R^{-H}
  w.t_bytes = (size_t)kc * P->nb * P->nact * (size_t)P->ny * P->nz * C;
  w.t = take(w.t_bytes);
  w.u = w.t;                            // adjoint line pass works in place
  w.rho_part = take((size_t)w.ngroups * P->ngrid * Rz);
  w.rho_scale = take((size_t)w.ngroups * sizeof(double));
  w.rho_q = take((kQParts + 1) * sizeof(double));
  // spin-polarised: [up][down][total] (the total is transformed for the
  // Hartree term); the potential per spin
  w.rho = take((size_t)(P->ns == 2 ? 3 : 1) * P->ngrid * Rz);
  w.rhog = take((size_t)P->ngrid * C);
  w.fft_scratch = take((size_t)P->ngrid * C);
  w.vr = take((size_t)P->ns * P->ngrid * Rz);
  w.gc = take(nbt * P->ng * C);
  w.adj_part = w.gram_part;
  w.epart = take((size_t)w.nepart * sizeof(double));
  w.flags = take(64);
  w.ekin = take(nbt * sizeof(double));
  w.dinv = take(nbt * sizeof(double));
  w.rot_scratch = take(nsk * 2 * 128 * 64 * sizeof(uint32_t));   // split B of the TF32 rotations
  w.gga = (P->xc & kXcGga) ? take(3 * (size_t)P->ngrid * C) : 0;   // gradient / flux grids of PBE
  w.kin_part = take(nbt * (size_t)((P->ng + 255) / 256) * Rz);   // kinetic block partials
  // beta-projector contraction: G-split partials and the weighted F
  w.nl_splits = P->nproj > 0 ? nl_splits(P->ng, (int)nsk, P->nb, P->nproj) : 0;
  w.nl_part = P->nproj > 0 ? take(nsk * w.nl_splits * (size_t)P->nb * P->nproj * sizeof(double2)) : 0;
  w.nl_fw = P->nproj > 0 ? take(nbt * (size_t)P->nproj * sizeof(double2)) : 0;
  w.lut = take(precond_lut_floats(P->nb, (int)nbt) * sizeof(float));   // in-step preconditioner table
  w.total = o;
}

// V_ext(r) = Re IFFT(V_ext(G)) in FP64 from the FP64 table (plan setup; the
// external energy and potential of the energy path use it in real space).
// Three direct DFTs along the axes: N (nx + ny + nz) FP64 products once per
// table, with no shared-memory limit on the grid size.
static int make_vext_real(jrg_plan* P) {
  const size_t n = (size_t)P->ngrid;
  double2* tw = nullptr;
  double2* buf = nullptr;
  int rc = JRG_OK;
  cudaError_t e = cudaSuccess;
  if (!P->d.vext_r) e = cudaMalloc((void**)&P->d.vext_r, n * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc((void**)&tw, (size_t)(P->nx + P->ny + P->nz) * sizeof(double2));
  if (e == cudaSuccess) e = cudaMalloc((void**)&buf, 2 * n * sizeof(double2));
  if (e != cudaSuccess) rc = cuda_fail(e, "cudaMalloc(external potential table)");
  double2* twx = tw;
  double2* twy = tw + P->nx;
  double2* twz = tw + P->nx + P->ny;
  if (!rc) rc = launch_twiddles(P->nx, 64, twx, 0);
  if (!rc) rc = launch_twiddles(P->ny, 64, twy, 0);
  if (!rc) rc = launch_twiddles(P->nz, 64, twz, 0);
  if (!rc) rc = launch_dft_axis_inv_f64(P->d.vext64, buf, P->nx, P->ny, P->nz, 2, twz, 0);
  if (!rc) rc = launch_dft_axis_inv_f64(buf, buf + n, P->nx, P->ny, P->nz, 1, twy, 0);
  if (!rc) rc = launch_dft_axis_inv_f64(buf + n, buf, P->nx, P->ny, P->nz, 0, twx, 0);
  if (!rc) rc = launch_real_part<double>(buf, P->d.vext_r, (long long)n, 1.0 / (double)P->ngrid, 0);
  if (!rc) {
    e = cudaDeviceSynchronize();
    if (e != cudaSuccess) rc = cuda_fail(e, "external potential table");
  }
  if (tw) cudaFree(tw);
  if (buf) cudaFree(buf);
  return rc;
}

// first energy slot of the nonlocal (beta-projector) partials, one per (s,k)
static int nl_slot_begin(const jrg_plan* P) {
  return P->ns * P->nk * P->nb + 2 * kRecipBlocks + kXcBlocks;
}

// energy slot boundaries: kinetic, external, Hartree, xc, then the nonlocal
// range (empty without projectors) that k_sum_slots adds to the external term
static int upload_slot_layout(jrg_plan* P) {
  const int nbt = P->ns * P->nk * P->nb;
  const int nl0 = nl_slot_begin(P);
  const int sb[6] = {0, nbt, nbt + kRecipBlocks, nbt + 2 * kRecipBlocks, nl0,
                     nl0 + (P->nproj > 0 ? P->ns * P->nk * nl_chunks(P->nb, P->nproj) : 0)};
  if (!P->slot_begin) {
    cudaError_t e = cudaMalloc((void**)&P->slot_begin, sizeof(sb));
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(slot layout)");
  }
  cudaError_t e = cudaMemcpy(P->slot_begin, sb, sizeof(sb), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy(slot layout)");
  return JRG_OK;
}

}  // namespace jrg

using namespace jrg;

extern "C" {

int jrg_version(void) { return 1; }
long long jrg_launch_count(void) { return g_launches.load(); }
const char* jrg_last_error(void) { return g_err.c_str(); }

int jrg_plan_destroy(jrg_plan* P) {
  if (!P) return JRG_OK;
  void* ptrs[] = {P->d.gidx, P->d.sph_yz, P->d.plane_x, P->d.plane_off, P->d.row_off, P->d.rows,
                  P->d.xact, P->d.tk, P->d.tkf, P->d.tw, P->d.vext, P->d.ginv, P->d.gvec, P->d.proj,
                  P->d.rowmap};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (P->prec == 32 && P->d.vext64) cudaFree(P->d.vext64);
  if (P->d.vext_r) cudaFree(P->d.vext_r);
  if (P->slot_begin) cudaFree(P->slot_begin);
  if (P->d_cell) cudaFree(P->d_cell);
  if (P->d_atoms) cudaFree(P->d_atoms);
  if (P->d_ones) cudaFree(P->d_ones);
  if (P->fork_ev) cudaEventDestroy(P->fork_ev);
  if (P->join_ev) cudaEventDestroy(P->join_ev);
  if (P->side) cudaStreamDestroy(P->side);
  if (P->prof) {
    for (cudaEvent_t e : P->prof->ev) cudaEventDestroy(e);
    delete P->prof;
  }
  delete P;
  return JRG_OK;
}

int jrg_plan_create(const jrg_plan_desc* d, jrg_plan** out) {
  if (!d || !out) return fail(JRG_ERR_INVALID, "jrg_plan_create: null argument");
  *out = nullptr;
  if (d->precision != 32 && d->precision != 64)
    return fail(JRG_ERR_INVALID, "precision must be 32 or 64");
  if (d->num_spin != 1 && d->num_spin != 2) return fail(JRG_ERR_INVALID, "num_spin must be 1 or 2");
  if (d->num_kpt < 1 || d->num_band < 1 || d->num_g < 1 || d->num_atom < 0)
    return fail(JRG_ERR_INVALID, "num_kpt, num_band, num_g must be positive");
  if (d->num_band > d->num_g) return fail(JRG_ERR_INVALID, "num_band exceeds the sphere size");
  if (!d->sphere_index || !d->kpts || (d->num_atom > 0 && (!d->positions || !d->charges)))
    return fail(JRG_ERR_INVALID, "null table pointer");
  jrg_plan* P = new jrg_plan();
  P->prec = d->precision;
  P->nx = d->grid[0]; P->ny = d->grid[1]; P->nz = d->grid[2];
  for (int a = 0; a < 3; ++a) {
    if (!factor_axis(d->grid[a], &P->ax[a])) {
      delete P;
      return fail(JRG_ERR_UNSUPPORTED, "grid size must be a product of 2, 3, 5, 7");
    }
  }
  P->ngrid = (long long)P->nx * P->ny * P->nz;
  P->ns = d->num_spin; P->nk = d->num_kpt; P->nb = d->num_band; P->ng = d->num_g;
  P->xc = d->xc;
  if ((P->xc & ~15) || ((P->xc & 3) && (P->xc & kXcGga))) {
    delete P;
    return fail(JRG_ERR_UNSUPPORTED, "xc: LDA and PBE terms cannot be combined");
  }
  std::memcpy(P->cell, d->cell, sizeof(P->cell));
  {
    const double* a = d->cell;
    const double det = a[0] * (a[4] * a[8] - a[5] * a[7]) - a[1] * (a[3] * a[8] - a[5] * a[6]) +
                       a[2] * (a[3] * a[7] - a[4] * a[6]);
    if (!(std::fabs(det) > 0)) { delete P; return fail(JRG_ERR_INVALID, "singular cell"); }
    P->vol = std::fabs(det);
    // reciprocal vectors b = 2 pi inv(a)^T, rows b_i
    double inv[9];
    inv[0] = (a[4] * a[8] - a[5] * a[7]) / det; inv[1] = (a[2] * a[7] - a[1] * a[8]) / det;
    inv[2] = (a[1] * a[5] - a[2] * a[4]) / det; inv[3] = (a[5] * a[6] - a[3] * a[8]) / det;
    inv[4] = (a[0] * a[8] - a[2] * a[6]) / det; inv[5] = (a[2] * a[3] - a[0] * a[5]) / det;
    inv[6] = (a[3] * a[7] - a[4] * a[6]) / det; inv[7] = (a[1] * a[6] - a[0] * a[7]) / det;
    inv[8] = (a[0] * a[4] - a[1] * a[3]) / det;
    const double tpi = 2.0 * 3.14159265358979323846;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) P->recip[3 * i + j] = tpi * inv[3 * j + i];
  }
  P->pos.assign(d->positions, d->positions + 3 * d->num_atom);
  P->charge.assign(d->charges, d->charges + d->num_atom);
  P->kpts.assign(d->kpts, d->kpts + 3 * d->num_kpt);
  // sphere tables
  const int ng = P->ng;
  std::vector<int> gidx(d->sphere_index, d->sphere_index + ng), sph_yz(ng);
  std::vector<int> plane_x, plane_off, row_off, rows, xact(P->nx, -1);
  const long long nyz = (long long)P->ny * P->nz;
  for (int e = 0; e < ng; ++e) {
    if (gidx[e] < 0 || gidx[e] >= P->ngrid || (e > 0 && gidx[e] <= gidx[e - 1])) {
      delete P;
      return fail(JRG_ERR_INVALID, "sphere_index must be strictly increasing grid indices");
    }
    const int x = (int)(gidx[e] / nyz);
    const int yz = (int)(gidx[e] % nyz);
    const int y = yz / P->nz;
    sph_yz[e] = yz;
    if (plane_x.empty() || plane_x.back() != x) {
      xact[x] = (int)plane_x.size();
      plane_x.push_back(x);
      plane_off.push_back(e);
      row_off.push_back((int)rows.size());
      rows.push_back(y);
    } else if (rows.back() != y) {
      rows.push_back(y);
    }
  }
  plane_off.push_back(ng);
  row_off.push_back((int)rows.size());
  // dense map of every active row: sphere index per z, -1 off the sphere
  std::vector<int> rowmap(rows.size() * (size_t)P->nz, -1);
  {
    size_t r = 0;
    for (int e = 0; e < ng; ++e) {
      const int x = (int)(gidx[e] / nyz), y = sph_yz[e] / P->nz, z = sph_yz[e] % P->nz;
      const int pl = xact[x];
      if (r < (size_t)row_off[pl]) r = row_off[pl];
      while (rows[r] != y) ++r;    // rows of a plane are increasing, as the sphere order is
      rowmap[r * P->nz + z] = e;
    }
  }
  P->nact = (int)plane_x.size();
  {
    auto mid = [](int i, int n) { return i >= n / 4 && i < 3 * n / 4; };   // the zero blocks
    auto eight = [](int n) { return n == 32 || n == 64; };                 // 8 values per thread
    P->xprune = eight(P->nx);
    for (int x : plane_x)
      if (mid(x, P->nx)) P->xprune = false;
    P->yzprune = eight(P->ny) && P->ny == P->nz;
    for (int e = 0; e < ng; ++e) {
      const int y = sph_yz[e] / P->nz, z = sph_yz[e] % P->nz;
      if (mid(y, P->ny) || mid(z, P->nz)) P->yzprune = false;
    }
  }
  P->max_rows = 0;
  for (int p = 0; p < P->nact; ++p) P->max_rows = std::max(P->max_rows, row_off[p + 1] - row_off[p]);
  // kinetic table |G+k|^2/2
  std::vector<double> tk((size_t)P->nk * ng);
  auto ff = [](int i, int n) { return (i < (n + 1) / 2) ? i : i - n; };
  for (int e = 0; e < ng; ++e) {
    const int x = (int)(gidx[e] / nyz), y = (sph_yz[e]) / P->nz, z = sph_yz[e] % P->nz;
    const double m0 = ff(x, P->nx), m1 = ff(y, P->ny), m2 = ff(z, P->nz);
    double g[3];
    for (int c = 0; c < 3; ++c) g[c] = m0 * P->recip[c] + m1 * P->recip[3 + c] + m2 * P->recip[6 + c];
    for (int k = 0; k < P->nk; ++k) {
      double s = 0.0;
      for (int c = 0; c < 3; ++c) { const double v = g[c] + P->kpts[3 * k + c]; s += v * v; }
      tk[(size_t)k * ng + e] = 0.5 * s;
    }
  }
  // FP32 copy and maximum for the tabulated in-step preconditioner
  std::vector<float> tkf(tk.size());
  P->tk_max = 0.f;
  for (size_t i = 0; i < tk.size(); ++i) { tkf[i] = (float)tk[i]; P->tk_max = std::max(P->tk_max, tkf[i]); }
  // shared-memory limits of the slab kernels
  {
    int dev = 0;
    cudaError_t ce = cudaGetDevice(&dev);
    if (ce != cudaSuccess) { delete P; return cuda_fail(ce, "cudaGetDevice"); }
    P->device = dev;
    int optin = 0;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    const size_t C = csize(P->prec), Rz = rsize(P->prec);
    const size_t plane_b = C * (P->ny + P->nz + 2 * (size_t)P->ny * P->nz) + 4 * (P->max_rows + 1);
    const size_t line_b = C * (P->nx + 2 * (size_t)P->nx * P->nz) + Rz * P->nx * P->nz +
                          4 * (P->nx + P->nact);
    if ((long long)plane_b > optin || (long long)line_b > optin || P->nx * P->nz > 256 * 48) {
      delete P;
      return fail(JRG_ERR_UNSUPPORTED, "grid too large for the shared-memory slab kernels at this precision");
    }
  }
  // upload
  auto up = [&](void** dst, const void* src, size_t bytes) -> int {
    cudaError_t e = cudaMalloc(dst, bytes ? bytes : 4);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(plan table)");
    if (bytes) {
      e = cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice);
      if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy(plan table)");
    }
    return JRG_OK;
  };
  int rc = JRG_OK;
#define UP(field, vec) \
  if (!rc) rc = up((void**)&P->d.field, vec.data(), vec.size() * sizeof(vec[0]));
  UP(gidx, gidx) UP(sph_yz, sph_yz) UP(plane_x, plane_x) UP(plane_off, plane_off)
  UP(row_off, row_off) UP(rows, rows) UP(xact, xact) UP(tk, tk) UP(tkf, tkf) UP(rowmap, rowmap)
#undef UP
  // twiddles (host, double precision): x, y, z tables
  if (!rc) {
    const int nt = P->nx + P->ny + P->nz;
    std::vector<double> tw(2 * (size_t)nt);
    int o = 0;
    for (int a = 0; a < 3; ++a) {
      const int n = P->ax[a].n;
      for (int t = 0; t < n; ++t) {
        const double ang = -2.0 * 3.14159265358979323846 * (double)t / (double)n;
        tw[2 * (o + t)] = std::cos(ang);
        tw[2 * (o + t) + 1] = std::sin(ang);
      }
      o += n;
    }
    if (P->prec == 64) {
      rc = up(&P->d.tw, tw.data(), tw.size() * sizeof(double));
    } else {
      std::vector<float> twf(tw.size());
      for (size_t t = 0; t < tw.size() / 2; ++t) {
        const float2 w = balanced_twiddle(tw[2 * t], tw[2 * t + 1]);
        twf[2 * t] = w.x;
        twf[2 * t + 1] = w.y;
      }
      rc = up(&P->d.tw, twf.data(), twf.size() * sizeof(float));
    }
  }
  // geometry tables on the device (FP64)
  double* d_recip = nullptr; double* d_pos = nullptr; double* d_chg = nullptr;
  if (!rc) {
    std::vector<double> cr(18);
    std::memcpy(cr.data(), P->cell, 9 * sizeof(double));
    std::memcpy(cr.data() + 9, P->recip, 9 * sizeof(double));
    rc = up((void**)&P->d_cell, cr.data(), cr.size() * sizeof(double));
    d_recip = P->d_cell + 9;
  }
  std::vector<double> atoms(4 * std::max(1, d->num_atom), 0.0);
  for (int i = 0; i < d->num_atom; ++i) {
    for (int c = 0; c < 3; ++c) atoms[3 * i + c] = P->pos[3 * i + c];
    atoms[3 * d->num_atom + i] = P->charge[i];
  }
  if (!rc) rc = up((void**)&P->d_atoms, atoms.data(), atoms.size() * sizeof(double));
  if (!rc) { d_pos = P->d_atoms; d_chg = P->d_atoms + 3 * d->num_atom; }
  if (!rc) {
    std::vector<double> ones((size_t)P->ns * P->nk * P->nb, 1.0);
    rc = up((void**)&P->d_ones, ones.data(), ones.size() * sizeof(double));
  }
  if (!rc) {
    cudaError_t e = cudaStreamCreateWithFlags(&P->side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&P->fork_ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&P->join_ev, cudaEventDisableTiming);
    if (e != cudaSuccess) rc = cuda_fail(e, "stream/event creation");
  }
  if (!rc) {
    cudaError_t e = cudaMalloc((void**)&P->d.gvec, 3 * P->ngrid * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc((void**)&P->d.ginv, P->ngrid * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&P->d.vext, P->ngrid * csize(P->prec));
    if (e == cudaSuccess && P->prec == 32) e = cudaMalloc((void**)&P->d.vext64, P->ngrid * sizeof(double2));
    if (e == cudaSuccess && P->prec == 64) P->d.vext64 = (double2*)P->d.vext;
    if (e != cudaSuccess) rc = cuda_fail(e, "cudaMalloc(geometry tables)");
  }
  if (!rc) {
    if (P->prec == 64)
      rc = launch_geometry_tables<double>(P->d.gvec, P->d.ginv, P->d.vext, nullptr, d_recip, d_pos, d_chg,
                                          d->num_atom, P->nx, P->ny, P->nz, P->vol, 0);
    else
      rc = launch_geometry_tables<float>(P->d.gvec, P->d.ginv, P->d.vext, P->d.vext64, d_recip, d_pos, d_chg,
                                         d->num_atom, P->nx, P->ny, P->nz, P->vol, 0);
  }
  if (!rc) rc = make_vext_real(P);
  layout_workspace(P);
  if (!rc) rc = upload_slot_layout(P);
  if (!rc) {
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) rc = cuda_fail(e, "plan setup");
  }
  if (rc) { jrg_plan_destroy(P); return rc; }
  *out = P;
  return JRG_OK;
}

int jrg_plan_set_memory_limit(jrg_plan* P, size_t bytes) {
  if (!P) return fail(JRG_ERR_INVALID, "jrg_plan_set_memory_limit: null plan");
  P->mem_limit = bytes;
  layout_workspace(P);
  return upload_slot_layout(P);
}

int jrg_plan_memory_chunk(const jrg_plan* P, int* kchunk) {
  if (!P || !kchunk) return fail(JRG_ERR_INVALID, "jrg_plan_memory_chunk: null argument");
  *kchunk = P->kchunk;
  return JRG_OK;
}

int jrg_workspace_size(const jrg_plan* P, size_t* bytes) {
  if (!P || !bytes) return fail(JRG_ERR_INVALID, "null argument");
  *bytes = P->ws.total;
  return JRG_OK;
}

int jrg_plan_set_pseudopotential(jrg_plan* P, const double* v_local, int num_proj,
                                 const double* projectors) {
  if (!P || num_proj < 0 || (num_proj > 0 && !projectors))
    return fail(JRG_ERR_INVALID, "jrg_plan_set_pseudopotential: bad argument");
  // host FP64 interleaved complex -> device complex in the plan's precision
  auto upload = [&](const double* src, size_t n, void* dst) -> int {
    cudaError_t e;
    if (P->prec == 64) {
      e = cudaMemcpy(dst, src, n * 2 * sizeof(double), cudaMemcpyHostToDevice);
    } else {
      std::vector<float> f(2 * n);
      for (size_t i = 0; i < 2 * n; ++i) f[i] = (float)src[i];
      e = cudaMemcpy(dst, f.data(), n * 2 * sizeof(float), cudaMemcpyHostToDevice);
    }
    return e == cudaSuccess ? JRG_OK : cuda_fail(e, "cudaMemcpy(pseudopotential table)");
  };
  int rc;
  if (v_local && (rc = upload(v_local, (size_t)P->ngrid, P->d.vext))) return rc;
  if (v_local && P->prec == 32) {
    cudaError_t e = cudaMemcpy(P->d.vext64, v_local, (size_t)P->ngrid * sizeof(double2), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy(pseudopotential table)");
  }
  if (v_local && (rc = make_vext_real(P))) return rc;
  if (P->d.proj) {
    cudaFree(P->d.proj);
    P->d.proj = nullptr;
  }
  P->nproj = 0;
  if (num_proj > 0) {
    const size_t n = (size_t)P->nk * num_proj * P->ng;
    cudaError_t e = cudaMalloc(&P->d.proj, n * csize(P->prec));
    if (e != cudaSuccess) {
      P->d.proj = nullptr;
      return cuda_fail(e, "cudaMalloc(projector table)");
    }
    if ((rc = upload(projectors, n, P->d.proj))) return rc;
    P->nproj = num_proj;
  }
  layout_workspace(P);
  if ((rc = upload_slot_layout(P))) return rc;
  cudaError_t e = cudaDeviceSynchronize();
  return e == cudaSuccess ? JRG_OK : cuda_fail(e, "pseudopotential setup");
}

}  // extern "C"

namespace jrg {

static inline char* wsp(void* ws, size_t off) { return reinterpret_cast<char*>(ws) + off; }

// Cholesky pivots at or below this fraction of the Gram diagonal are a
// breakdown: the rounding level of the Gram (FP32 products: ~1e-8 relative)
static double min_pivot(const jrg_plan* P) { return P->prec == 64 ? 1e-14 : 1e-7; }

// phase timing: events of call `calls` (the call in progress)
struct PhaseScope {
  const jrg_plan* P;
  int ph;
  cudaStream_t st;
  PhaseScope(const jrg_plan* p, int phase, cudaStream_t s) : P(p), ph(phase), st(s) {
    Profiler* pr = P->prof;
    if (pr && pr->calls < pr->max_calls) {
      cudaEventRecord(pr->ev[((size_t)pr->calls * PH_COUNT + ph) * 2], st);
      pr->used[(size_t)pr->calls * PH_COUNT + ph] = 1;
    }
  }
  ~PhaseScope() {
    Profiler* pr = P->prof;
    if (pr && pr->calls < pr->max_calls)
      cudaEventRecord(pr->ev[((size_t)pr->calls * PH_COUNT + ph) * 2 + 1], st);
  }
};
#define PHASE(ph) PhaseScope phase_scope_##ph(P, ph, st)
static void profile_call_done(const jrg_plan* P) {
  if (P->prof && P->prof->calls < P->prof->max_calls) P->prof->calls++;
}

template <typename R>
static int orthonormalise(const jrg_plan* P, const void* w_re, const void* w_im, void* ws,
                          cudaStream_t st, int out_kind = kRotBand, void* out = nullptr,
                          int* kin_blocks = nullptr) {
  const Workspace& w = P->ws;
  const int nsk = P->ns * P->nk;
  int rc;
  {
    PHASE(PH_GRAM);
    if ((rc = launch_gram<R>(kSplit, w_re, w_im, kSplit, w_re, w_im, (double2*)wsp(ws, w.gram_part),
                             (double2*)wsp(ws, w.gram), nsk, P->ng, P->nb, w.gram_splits, st,
                             (int*)wsp(ws, w.flags))))
      return rc;
  }
  {
    PHASE(PH_CHOL);
    if ((rc = launch_cholesky_inv((double2*)wsp(ws, w.gram), (double2*)wsp(ws, w.rmat),
                                  (double2*)wsp(ws, w.rinv), nsk, P->nb, (int*)wsp(ws, w.flags),
                                  (double*)wsp(ws, w.dinv), st, min_pivot(P), P->prec == 32)))
      return rc;
  }
  PHASE(PH_ROTATE);
  if (kin_blocks) {
    // C and the kinetic block partials in one pass over the parameters
    *kin_blocks = launch_rotate_kinetic<R>(w_re, w_im, (double2*)wsp(ws, w.rinv), wsp(ws, w.c), nsk,
                                           P->ng, P->nb, P->d.tk, P->nk, wsp(ws, w.kin_part), st);
    if (*kin_blocks < 0) return -*kin_blocks;
    if (*kin_blocks > 0) return JRG_OK;
  }
  return launch_rotate<R>(out_kind, kSplit, w_re, w_im, (double2*)wsp(ws, w.rinv), nullptr, nullptr,
                          out ? out : wsp(ws, w.c), nullptr, nsk, P->ng, P->nb, 1.0,
                          wsp(ws, w.rot_scratch), st, kTriUpper);
}

// PBE terms of the grid phase.  Step 1 (from rho(G) in rhog, before it is
// overwritten): the three gradient grids grad_a rho = IFFT(i G_a rho(G))/N.
template <typename R>
static int gga_gradients(const jrg_plan* P, const C_t<R>* rhog, void* ws, cudaStream_t st) {
  using C = C_t<R>;
  const Workspace& w = P->ws;
  C* g = (C*)wsp(ws, w.gga);
  C* scratch = (C*)wsp(ws, w.fft_scratch);
  const C* tw = (const C*)P->d.tw;
  const double N = (double)P->ngrid;
  int rc;
  for (int a = 0; a < 3; ++a) {
    C* ga = g + (size_t)a * P->ngrid;
    if ((rc = launch_mul_ig<R>(rhog, P->d.gvec, ga, a, P->ngrid, 1.0 / N, st))) return rc;
    if ((rc = launch_fft3d_dense<R>(P->ax, tw, 1, +1, false, ga, scratch, ga, 1.0, st))) return rc;
  }
  return JRG_OK;
}

// Step 2: local terms (E_xc partials into slot_x, f_rho into vout) and, for the
// potential, vout = Re(vri) vscale + f_rho - 2 div(f_sigma grad rho) (+ V_ext(r)
// and its energy partials into slot_e when vext_r is given); with eps_only,
// vout = eps(rho, sigma) per particle instead.  qscale: the density factor of
// ChargeFix (null: 1).
template <typename R>
static int gga_potential(const jrg_plan* P, const void* rho, const C_t<R>* vri, double vscale,
                         void* vout, double* slot_x, int eps_only, void* ws, cudaStream_t st,
                         const double* qscale = nullptr, const double* vext_r = nullptr,
                         double* slot_e = nullptr) {
  using C = C_t<R>;
  const Workspace& w = P->ws;
  C* g = (C*)wsp(ws, w.gga);
  C* g1 = g + P->ngrid;
  C* g2 = g + 2 * (size_t)P->ngrid;
  C* scratch = (C*)wsp(ws, w.fft_scratch);
  const C* tw = (const C*)P->d.tw;
  const double N = (double)P->ngrid;
  int rc;
  if ((rc = launch_gga_local<R>(rho, g, g1, g2, vout, slot_x, kXcBlocks, P->ngrid, P->xc,
                                P->vol / N, eps_only, qscale, vext_r, slot_e, st)))
    return rc;
  if (eps_only) return JRG_OK;
  for (int a = 0; a < 3; ++a) {
    C* ga = g + (size_t)a * P->ngrid;
    if ((rc = launch_fft3d_dense<R>(P->ax, tw, 1, -1, false, ga, scratch, ga, 1.0, st))) return rc;
  }
  if ((rc = launch_div_g<R>(g, g1, g2, P->d.gvec, P->ngrid, 1.0 / N, st))) return rc;
  if ((rc = launch_fft3d_dense<R>(P->ax, tw, 1, +1, false, g, scratch, g, 1.0, st))) return rc;
  return launch_potential_gga<R>(vri, vscale, vout, g, P->ngrid, vext_r, st);
}

// Nonlocal pseudopotential term of the (s,k) blocks [k0, k0+n): F = C P and
// its energy partials (weights occ), and the weighted fw = wg / vol F used by
// nl_adjoint.  No-ops without projectors.
template <typename R>
static int nl_forward(const jrg_plan* P, void* ws, int k0, int n, const double* occ, const double* wg,
                      cudaStream_t st) {
  if (P->nproj <= 0) return JRG_OK;
  PHASE(PH_NL_PROJECT);
  const Workspace& w = P->ws;
  const size_t m = (size_t)P->nb * P->nproj;
  double2* part = (double2*)wsp(ws, w.nl_part) + (size_t)k0 * w.nl_splits * m;
  double2* fw = (double2*)wsp(ws, w.nl_fw) + (size_t)k0 * m;
  const C_t<R>* c = (const C_t<R>*)wsp(ws, w.c) + (size_t)k0 * P->nb * P->ng;
  double* slot = (double*)wsp(ws, w.epart) + nl_slot_begin(P) + (size_t)k0 * nl_chunks(P->nb, P->nproj);
  int rc;
  if ((rc = launch_nl_project<R>(c, P->d.proj, part, k0, n, P->nk, P->ng, P->nb, P->nproj, w.nl_splits,
                                 st)))
    return rc;
  return launch_nl_reduce(part, fw, occ + (size_t)k0 * P->nb, wg + (size_t)k0 * P->nb, slot, n, P->nb,
                          P->nproj, w.nl_splits, 1.0 / P->vol, st);
}

// g_C[k0, k0+n) += fw conj(P)
template <typename R>
static int nl_adjoint(const jrg_plan* P, void* ws, int k0, int n, cudaStream_t st) {
  if (P->nproj <= 0) return JRG_OK;
  PHASE(PH_NL_APPLY);
  const Workspace& w = P->ws;
  C_t<R>* gc = (C_t<R>*)wsp(ws, w.gc) + (size_t)k0 * P->nb * P->ng;
  const double2* fw = (const double2*)wsp(ws, w.nl_fw) + (size_t)k0 * P->nb * P->nproj;
  return launch_nl_apply<R>(gc, P->d.proj, fw, k0, n, P->nk, P->ng, P->nb, P->nproj, st);
}

static int sum_energy_slots(const jrg_plan* P, double* slots, double* energies, void* ws, cudaStream_t st) {
  return launch_sum_slots(slots, P->slot_begin, energies, 4, (int*)wsp(ws, P->ws.flags),
                          P->nproj > 0 ? 1 : -1, st);
}

// density of the band-major coefficients held in workspace slot c (qpart:
// the charge partials of ChargeFix, or null)
template <typename R>
static int density_from_c(const jrg_plan* P, const double* occ, void* ws, void* rho_out,
                          cudaStream_t st, double* qpart = nullptr) {
  using C = C_t<R>;
  const Workspace& w = P->ws;
  const int nsk = P->ns * P->nk;
  int rc;
  // (s,k) blocks in chunks of P->kchunk through the plane buffer
  for (int k0 = 0; k0 < nsk; k0 += P->kchunk) {
    const int n = std::min(P->kchunk, nsk - k0);
    {
      PHASE(PH_PLANE_INV);
      if ((rc = launch_plane_inv_sphere<R>(P, (C*)wsp(ws, w.c) + (size_t)k0 * P->nb * P->ng, wsp(ws, w.t),
                                           n * P->nb, st)))
        return rc;
    }
    {
      PHASE(PH_LINE_DENSITY);
      if ((rc = launch_line_density<R>(P, wsp(ws, w.t), (R*)wsp(ws, w.rho_part) + (size_t)k0 * P->ngrid, occ,
                                       1.0 / P->vol, k0 * P->nb, n * P->nb, P->nb,
                                       (double*)wsp(ws, w.rho_scale) + k0, st)))
        return rc;
    }
  }
  PHASE(PH_REDUCE_DENSITY);
  return launch_reduce_density<R>(wsp(ws, w.rho_part), rho_out, P->nk, P->ns, P->ngrid,
                                  (const double*)wsp(ws, w.rho_scale), qpart, st);
}

// Grid phase of the energy path on the density in workspace slot rho (with
// its charge partials in rho_q): rho(G); the charge factor s (ChargeFix);
// Hartree energy and potential in G space; xc and external energies and
// V(r) = V_H + v_xc + V_ext on the grid (external from the FP64 V_ext(r)
// table).  Energy partials go to the external, Hartree and xc slots.
template <typename R>
static int grid_phase(const jrg_plan* P, const double* occ, double* slots, void* ws, cudaStream_t st) {
  using C = C_t<R>;
  static_assert(kRecipBlocks == kXcBlocks, "external partials are written by the xc kernels");
  const Workspace& w = P->ws;
  const int nbt = P->ns * P->nk * P->nb;
  const double N = (double)P->ngrid;
  void* rho = wsp(ws, w.rho);
  C* rhog = (C*)wsp(ws, w.rhog);
  C* scratch = (C*)wsp(ws, w.fft_scratch);
  const C* tw = (const C*)P->d.tw;
  double* q = (double*)wsp(ws, w.rho_q);
  ChargeFix cf;
  cf.qpart = q;
  cf.occ = occ;
  cf.nocc = nbt;
  cf.dv = P->vol / N;
  cf.scale = q + kQParts;
  double* slot_e = slots + nbt;
  double* slot_h = slots + nbt + kRecipBlocks;
  double* slot_x = slots + nbt + 2 * kRecipBlocks;
  int rc;
  const void* rho_t = rho;   // the density the Hartree term transforms
  if (P->ns == 2) {
    void* tot = (char*)rho + 2 * (size_t)P->ngrid * rsize(P->prec);
    if ((rc = launch_spin_total<R>(rho, tot, P->ngrid, st))) return rc;
    rho_t = tot;
  }
  if ((rc = launch_fft3d_dense<R>(P->ax, tw, 1, -1, true, rho_t, scratch, rhog, 1.0, st))) return rc;
  const bool gga = (P->xc & kXcGga) != 0;
  if (gga && (rc = gga_gradients<R>(P, rhog, ws, st))) return rc;
  // Hartree energy and V_H(G) (in place)
  if ((rc = launch_recip_terms<R>(rhog, P->d.ginv, rhog, slot_h, kRecipBlocks, P->ngrid, P->vol / (N * N),
                                  cf, st)))
    return rc;
  if ((rc = launch_fft3d_dense<R>(P->ax, tw, 1, +1, false, rhog, scratch, rhog, 1.0 / N, st))) return rc;
  if (gga)
    return gga_potential<R>(P, rho, rhog, 1.0, wsp(ws, w.vr), slot_x, 0, ws, st, cf.scale, P->d.vext_r,
                            slot_e);
  if (P->ns == 2)
    return launch_potential_pol<R>(rho, rhog, 1.0, wsp(ws, w.vr), slot_x, kXcBlocks, P->ngrid, P->xc,
                                   P->vol / N, cf.scale, P->d.vext_r, slot_e, st);
  return launch_potential<R>(rho, rhog, 1.0, wsp(ws, w.vr), slot_x, kXcBlocks, P->ngrid, P->xc, P->vol / N,
                             cf.scale, P->d.vext_r, slot_e, st);
}

// Adjoint line pass over the (s,k) blocks k0 .. k0+n-1 held in the plane
// buffers t_in / t_out (block k0 first), with the potential of each block's
// spin (vr: [ns][grid]); one launch per spin.
template <typename R>
static int apply_v_blocks(const jrg_plan* P, void* t_in, void* t_out, const void* vr, int k0, int n,
                          cudaStream_t st) {
  using C = C_t<R>;
  const size_t per_block = (size_t)P->nb * P->nact * P->ny * P->nz;   // plane elements of one block
  int rc;
  for (int b = k0; b < k0 + n;) {
    const int s = b / P->nk;
    const int e = std::min(k0 + n, (s + 1) * P->nk);
    const size_t off = (size_t)(b - k0) * per_block;
    if ((rc = launch_line_apply_v<R>(P, (C*)t_in + off, (C*)t_out + off,
                                     (const R*)vr + (size_t)s * P->ngrid, (e - b) * P->nb, P->nb, st)))
      return rc;
    b = e;
  }
  return JRG_OK;
}

template <typename R>
static int energy_grad_impl(const jrg_plan* P, const void* w_re, const void* w_im, const double* occ,
                            double* energies, void* g_re, void* g_im, void* ws, cudaStream_t st,
                            const AdamArgs* adam = nullptr, double* band_e = nullptr) {
  using C = C_t<R>;
  const Workspace& w = P->ws;
  const int nsk = P->ns * P->nk;
  const int nbt = nsk * P->nb;
  const double N = (double)P->ngrid;
  int rc;
  JRG_CUDA(cudaMemsetAsync(wsp(ws, w.flags), 0, 64, st));
  int kin_blocks = 0;
  if ((rc = orthonormalise<R>(P, w_re, w_im, ws, st, kRotBand, nullptr, &kin_blocks))) return rc;
  double* slots = (double*)wsp(ws, w.epart);
  {
    PHASE(PH_KINETIC);
    if (kin_blocks > 0)
      rc = launch_kin_reduce(P->prec, wsp(ws, w.kin_part), kin_blocks, P->nb, nbt, occ, slots,
                             (double*)wsp(ws, w.ekin), st);
    else
      rc = launch_kinetic<R>(wsp(ws, w.c), P->d.tk, occ, slots, (double*)wsp(ws, w.ekin), nbt,
                             P->ng, P->nb, P->nk, st);
    if (rc) return rc;
  }
  if (adam && adam->mlp_w32) {
    // learned update scales from this step's band kinetic energies
    PHASE(PH_PRECOND);
    if ((rc = launch_precond_scale_lut(adam->mlp_w32, adam->mlp_wb, P->d.tk, P->d.tkf, P->tk_max,
                                       (const double*)wsp(ws, w.ekin), occ, P->nk, P->ng, P->nb, nbt,
                                       (long long)nbt * P->ng, adam->t_frac, adam->smax, adam->scale[0],
                                       (float*)wsp(ws, w.lut), st)))
      return rc;
  }
  if ((rc = nl_forward<R>(P, ws, 0, nsk, occ, band_e ? P->d_ones : occ, st))) return rc;
  if ((rc = density_from_c<R>(P, occ, ws, wsp(ws, w.rho), st, (double*)wsp(ws, w.rho_q)))) return rc;
  {
    PHASE(PH_GRID_TERMS);
    if ((rc = grid_phase<R>(P, occ, slots, ws, st))) return rc;
    if ((rc = sum_energy_slots(P, slots, energies, ws, st))) return rc;
  }
  if (!adam && !g_re && !g_im) return JRG_OK;
  if (!adam && (!g_re || !g_im)) return fail(JRG_ERR_INVALID, "grad_re and grad_im must both be given");
  // adjoint: planes -> x lines (x V) -> planes -> sphere gradient, per chunk
  // of (s,k) blocks; with more than one chunk the planes of each are
  // transformed again from the coefficients (the density pass overwrote them)
  for (int k0 = 0; k0 < nsk; k0 += P->kchunk) {
    const int n = std::min(P->kchunk, nsk - k0);
    const size_t co = (size_t)k0 * P->nb * P->ng;
    if (P->kchunk < nsk) {
      PHASE(PH_PLANE_INV);
      if ((rc = launch_plane_inv_sphere<R>(P, (C*)wsp(ws, w.c) + co, wsp(ws, w.t), n * P->nb, st))) return rc;
    }
    {
      PHASE(PH_LINE_APPLY_V);
      if ((rc = apply_v_blocks<R>(P, wsp(ws, w.t), wsp(ws, w.u), wsp(ws, w.vr), k0, n, st))) return rc;
    }
    {
      // with band energies requested, g_C = H c unweighted; the occupations
      // are folded into the small adjoint matrices below
      PHASE(PH_PLANE_FWD);
      if ((rc = launch_plane_fwd_sphere<R>(P, wsp(ws, w.u), (C*)wsp(ws, w.c) + co, (C*)wsp(ws, w.gc) + co,
                                           band_e ? P->d_ones : occ, k0 * P->nb, n * P->nb, 1.0 / N, st)))
        return rc;
    }
  }
  if ((rc = nl_adjoint<R>(P, ws, 0, nsk, st))) return rc;
  // orthonormalisation adjoint
  {
    PHASE(PH_ADJ_GRAM);
    if ((rc = launch_gram<R>(kBand, wsp(ws, w.c), nullptr, kBand, wsp(ws, w.gc), nullptr,
                             (double2*)wsp(ws, w.adj_part), (double2*)wsp(ws, w.adj), nsk, P->ng,
                             P->nb, w.gram_splits, st, (int*)wsp(ws, w.flags))))
      return rc;
  }
  double2* rh = (double2*)wsp(ws, w.kmat);
  double2* negm2 = rh + (size_t)nsk * P->nb * P->nb;
  {
    PHASE(PH_ADJ_SMALL);
    if ((rc = launch_adjoint_small((double2*)wsp(ws, w.adj), (double2*)wsp(ws, w.rinv), rh, negm2,
                                   nsk, P->nb, st, band_e ? occ : nullptr, band_e)))
      return rc;
  }
  PHASE(PH_ADJ_ROTATE);
  if (adam)
    return launch_rotate_adam<R>(wsp(ws, w.gc), rh, wsp(ws, w.c), negm2, *adam, nsk, P->ng, P->nb,
                                 2.0, st);
  return launch_rotate<R>(kRotGSplit, kBand, wsp(ws, w.gc), nullptr, rh, wsp(ws, w.c), negm2, g_re,
                          g_im, nsk, P->ng, P->nb, 2.0, wsp(ws, w.rot_scratch), st, kTriLower);
}

// Band trace of a fixed effective potential (band-structure objective):
// orthonormalise, kinetic, planes, x lines times v_eff, planes back to the
// sphere gradient, C^H g_C (= the weighted band Hamiltonian), its trace, and
// the orthonormalisation adjoint.
template <typename R>
static int band_trace_impl(const jrg_plan* P, const void* w_re, const void* w_im, const void* v_eff,
                           const double* wts, double* out, void* hmat, void* g_re, void* g_im,
                           void* ws, cudaStream_t st) {
  const Workspace& w = P->ws;
  const int nsk = P->ns * P->nk;
  const int nbt = nsk * P->nb;
  const double N = (double)P->ngrid;
  int rc;
  JRG_CUDA(cudaMemsetAsync(wsp(ws, w.flags), 0, 64, st));
  if ((rc = orthonormalise<R>(P, w_re, w_im, ws, st))) return rc;
  double* slots = (double*)wsp(ws, w.epart);
  {
    PHASE(PH_KINETIC);
    if ((rc = launch_kinetic<R>(wsp(ws, w.c), P->d.tk, wts, slots, (double*)wsp(ws, w.ekin), nbt,
                                P->ng, P->nb, P->nk, st)))
      return rc;
  }
  if ((rc = nl_forward<R>(P, ws, 0, nsk, wts, wts, st))) return rc;
  for (int k0 = 0; k0 < nsk; k0 += P->kchunk) {
    const int n = std::min(P->kchunk, nsk - k0);
    const size_t co = (size_t)k0 * P->nb * P->ng;
    {
      PHASE(PH_PLANE_INV);
      if ((rc = launch_plane_inv_sphere<R>(P, (C_t<R>*)wsp(ws, w.c) + co, wsp(ws, w.t), n * P->nb, st)))
        return rc;
    }
    {
      PHASE(PH_LINE_APPLY_V);
      if ((rc = apply_v_blocks<R>(P, wsp(ws, w.t), wsp(ws, w.u), v_eff, k0, n, st))) return rc;
    }
    {
      PHASE(PH_PLANE_FWD);
      if ((rc = launch_plane_fwd_sphere<R>(P, wsp(ws, w.u), (C_t<R>*)wsp(ws, w.c) + co,
                                           (C_t<R>*)wsp(ws, w.gc) + co, wts, k0 * P->nb, n * P->nb, 1.0 / N, st)))
        return rc;
    }
  }
  if ((rc = nl_adjoint<R>(P, ws, 0, nsk, st))) return rc;
  {
    PHASE(PH_ADJ_GRAM);
    if ((rc = launch_gram<R>(kBand, wsp(ws, w.c), nullptr, kBand, wsp(ws, w.gc), nullptr,
                             (double2*)wsp(ws, w.adj_part), (double2*)wsp(ws, w.adj), nsk, P->ng,
                             P->nb, w.gram_splits, st, (int*)wsp(ws, w.flags), true)))
      return rc;
  }
  if ((rc = launch_band_trace_sums((const double2*)wsp(ws, w.adj), nsk, P->nb, slots, nbt, out, st)))
    return rc;
  if (hmat)
    JRG_CUDA(cudaMemcpyAsync(hmat, wsp(ws, w.adj), sizeof(double2) * (size_t)nsk * P->nb * P->nb,
                             cudaMemcpyDeviceToDevice, st));
  if (!g_re && !g_im) return JRG_OK;
  if (!g_re || !g_im) return fail(JRG_ERR_INVALID, "grad_re and grad_im must both be given");
  double2* rh = (double2*)wsp(ws, w.kmat);
  double2* negm2 = rh + (size_t)nsk * P->nb * P->nb;
  {
    PHASE(PH_ADJ_SMALL);
    if ((rc = launch_adjoint_small((double2*)wsp(ws, w.adj), (double2*)wsp(ws, w.rinv), rh, negm2,
                                   nsk, P->nb, st)))
      return rc;
  }
  PHASE(PH_ADJ_ROTATE);
  return launch_rotate<R>(kRotGSplit, kBand, wsp(ws, w.gc), nullptr, rh, wsp(ws, w.c), negm2, g_re,
                          g_im, nsk, P->ng, P->nb, 2.0, wsp(ws, w.rot_scratch), st, kTriLower);
}

// Two-way k-point pipeline of the energy/gradient evaluation: the (s,k)
// blocks are split in two halves that run on the caller's stream and the
// plan's side stream, so that the latency-bound small kernels of one half
// (Cholesky, small adjoint matrices) overlap the bandwidth-bound kernels of
// the other.  The density reduction and the grid terms run once, on the
// caller's stream, between the two forks.
template <typename R>
static int phase_forward_range(const jrg_plan* P, const void* w_re, const void* w_im,
                               const double* occ, void* ws, int k0, int n, cudaStream_t st) {
  using C = C_t<R>;
  const Workspace& w = P->ws;
  const size_t nb2 = (size_t)P->nb * P->nb;
  const size_t po = (size_t)k0 * P->ng * P->nb;                         // parameter offset
  const size_t co = (size_t)k0 * P->nb * P->ng;                         // band-major offset
  const size_t to = (size_t)k0 * P->nb * P->nact * P->ny * P->nz;       // plane buffer offset
  const int nblk = (P->ng + 255) / 256;
  const R* wr = reinterpret_cast<const R*>(w_re) + po;
  const R* wi = reinterpret_cast<const R*>(w_im) + po;
  int* flags = (int*)wsp(ws, w.flags);
  int rc;
  if ((rc = launch_gram<R>(kSplit, wr, wi, kSplit, wr, wi,
                           (double2*)wsp(ws, w.gram_part) + (size_t)k0 * w.gram_splits * nb2,
                           (double2*)wsp(ws, w.gram) + k0 * nb2, n, P->ng, P->nb, w.gram_splits, st,
                           flags)))
    return rc;
  if ((rc = launch_cholesky_inv((double2*)wsp(ws, w.gram) + k0 * nb2, (double2*)wsp(ws, w.rmat) + k0 * nb2,
                                (double2*)wsp(ws, w.rinv) + k0 * nb2, n, P->nb, flags,
                                (double*)wsp(ws, w.dinv) + (size_t)k0 * P->nb, st, min_pivot(P), P->prec == 32)))
    return rc;
  const int kb = launch_rotate_kinetic<R>(wr, wi, (double2*)wsp(ws, w.rinv) + k0 * nb2,
                                          (C*)wsp(ws, w.c) + co, n, P->ng, P->nb, P->d.tk, P->nk,
                                          (R*)wsp(ws, w.kin_part) + (size_t)k0 * nblk * P->nb, st, k0);
  if (kb < 0) return -kb;
  if (kb == 0) return fail(JRG_ERR_UNSUPPORTED, "pipelined path needs the fused kinetic rotation");
  if ((rc = nl_forward<R>(P, ws, k0, n, occ, occ, st))) return rc;
  if ((rc = launch_plane_inv_sphere<R>(P, (C*)wsp(ws, w.c) + co, (C*)wsp(ws, w.t) + to, n * P->nb, st)))
    return rc;
  return launch_line_density<R>(P, (C*)wsp(ws, w.t) + to, (R*)wsp(ws, w.rho_part) + (size_t)k0 * P->ngrid,
                                occ, 1.0 / P->vol, k0 * P->nb, n * P->nb, P->nb,
                                (double*)wsp(ws, w.rho_scale) + k0, st);
}

// With adam given, the gradient of the half goes to adam->grad (when set) or
// into the half's own, now dead, plane-buffer range, and the half's
// parameters take their Adam step right there, in the half's stream.
template <typename R>
static int phase_adjoint_range(const jrg_plan* P, const double* occ, void* g_re, void* g_im, void* ws,
                               int k0, int n, cudaStream_t st, const AdamArgs* adam = nullptr) {
  using C = C_t<R>;
  const Workspace& w = P->ws;
  const int nsk = P->ns * P->nk;
  const size_t nb2 = (size_t)P->nb * P->nb;
  const size_t po = (size_t)k0 * P->ng * P->nb;
  const size_t co = (size_t)k0 * P->nb * P->ng;
  const size_t to = (size_t)k0 * P->nb * P->nact * P->ny * P->nz;
  const double N = (double)P->ngrid;
  C* t = (C*)wsp(ws, w.t) + to;
  C* c = (C*)wsp(ws, w.c) + co;
  C* gc = (C*)wsp(ws, w.gc) + co;
  int rc;
  if ((rc = apply_v_blocks<R>(P, t, t, wsp(ws, w.vr), k0, n, st))) return rc;
  if ((rc = launch_plane_fwd_sphere<R>(P, t, c, gc, occ, k0 * P->nb, n * P->nb, 1.0 / N, st))) return rc;
  if ((rc = nl_adjoint<R>(P, ws, k0, n, st))) return rc;
  if ((rc = launch_gram<R>(kBand, c, nullptr, kBand, gc, nullptr,
                           (double2*)wsp(ws, w.adj_part) + (size_t)k0 * w.gram_splits * nb2,
                           (double2*)wsp(ws, w.adj) + k0 * nb2, n, P->ng, P->nb, w.gram_splits, st,
                           (int*)wsp(ws, w.flags))))
    return rc;
  double2* rh = (double2*)wsp(ws, w.kmat);
  double2* negm2 = rh + (size_t)nsk * nb2;
  if ((rc = launch_adjoint_small((double2*)wsp(ws, w.adj) + k0 * nb2, (double2*)wsp(ws, w.rinv) + k0 * nb2,
                                 rh + k0 * nb2, negm2 + k0 * nb2, n, P->nb, st)))
    return rc;
  const size_t cnt = (size_t)n * P->ng * P->nb;
  R* gr = adam ? (adam->grad[0] ? reinterpret_cast<R*>(adam->grad[0]) + po : reinterpret_cast<R*>(t))
               : reinterpret_cast<R*>(g_re) + po;
  R* gi = adam ? (adam->grad[1] ? reinterpret_cast<R*>(adam->grad[1]) + po : reinterpret_cast<R*>(t) + cnt)
               : reinterpret_cast<R*>(g_im) + po;
  if ((rc = launch_rotate<R>(kRotGSplit, kBand, gc, nullptr, rh + k0 * nb2, c, negm2 + k0 * nb2, gr, gi,
                             n, P->ng, P->nb, 2.0, wsp(ws, w.rot_scratch), st, kTriLower)))
    return rc;
  if (!adam) return JRG_OK;
  for (int part = 0; part < 2; ++part) {
    const float* sc = adam->scale[part] ? adam->scale[part] + po : nullptr;
    if ((rc = launch_adam<R>(reinterpret_cast<R*>(adam->p[part]) + po, part ? gi : gr,
                             reinterpret_cast<R*>(adam->m[part]) + po,
                             reinterpret_cast<R*>(adam->v[part]) + po, sc, (long long)cnt, adam->lr,
                             adam->b1, adam->b2, adam->c1, adam->c2, adam->eps, st, adam->guard)))
      return rc;
  }
  return JRG_OK;
}

static bool g_pipeline = true;   // two-way k-point pipeline of jrg_energy_grad

static bool pipeline_ok(const jrg_plan* P) {
  // more than 32 bands: the thread-per-G rotations of mode 0 (fused kinetic partials)
  return P->ns * P->nk >= 2 && (P->nb <= 32 || jrg_tensor_core_paths(-1) == 0) && P->kchunk >= P->ns * P->nk &&
         (jrg_tensor_core_paths(-1) == 0 || jrg_tensor_core_paths(-1) == 3) &&
         jrg_fast_paths(-1) == 1 && !(P->prof && P->prof->max_calls > 0);
}

template <typename R>
static int energy_grad_pipelined(const jrg_plan* P, const void* w_re, const void* w_im,
                                 const double* occ, double* energies, void* g_re, void* g_im,
                                 void* ws, cudaStream_t st, const AdamArgs* adam = nullptr) {
  using C = C_t<R>;
  const Workspace& w = P->ws;
  const int nsk = P->ns * P->nk;
  const int nbt = nsk * P->nb;
  const int ka = (nsk + 1) / 2, kb = nsk - ka;
  const double N = (double)P->ngrid;
  int rc;
  auto fork = [&]() -> int {
    JRG_CUDA(cudaEventRecord(P->fork_ev, st));
    JRG_CUDA(cudaStreamWaitEvent(P->side, P->fork_ev, 0));
    return JRG_OK;
  };
  auto join = [&]() -> int {
    JRG_CUDA(cudaEventRecord(P->join_ev, P->side));
    JRG_CUDA(cudaStreamWaitEvent(st, P->join_ev, 0));
    return JRG_OK;
  };
  JRG_CUDA(cudaMemsetAsync(wsp(ws, w.flags), 0, 64, st));
  if ((rc = fork())) return rc;
  if ((rc = phase_forward_range<R>(P, w_re, w_im, occ, ws, 0, ka, st))) return rc;
  if ((rc = phase_forward_range<R>(P, w_re, w_im, occ, ws, ka, kb, P->side))) return rc;
  if ((rc = join())) return rc;
  double* slots = (double*)wsp(ws, w.epart);
  if ((rc = launch_kin_reduce(P->prec, wsp(ws, w.kin_part), (P->ng + 255) / 256, P->nb, nbt, occ, slots,
                              (double*)wsp(ws, w.ekin), st)))
    return rc;
  if (adam && adam->mlp_w32 &&
      (rc = launch_precond_scale_lut(adam->mlp_w32, adam->mlp_wb, P->d.tk, P->d.tkf, P->tk_max,
                                     (const double*)wsp(ws, w.ekin), occ, P->nk, P->ng, P->nb, nbt,
                                     (long long)nbt * P->ng, adam->t_frac, adam->smax, adam->scale[0],
                                     (float*)wsp(ws, w.lut), st)))
    return rc;
  if ((rc = launch_reduce_density<R>(wsp(ws, w.rho_part), wsp(ws, w.rho), P->nk, P->ns, P->ngrid,
                                     (const double*)wsp(ws, w.rho_scale), (double*)wsp(ws, w.rho_q), st)))
    return rc;
  if ((rc = grid_phase<R>(P, occ, slots, ws, st))) return rc;
  // the energy sums feed only the energies output: they run after the adjoint
  // halves, off the path between the two forks
  if (!adam && !g_re && !g_im) return sum_energy_slots(P, slots, energies, ws, st);
  if (!adam && (!g_re || !g_im)) return fail(JRG_ERR_INVALID, "grad_re and grad_im must both be given");
  if ((rc = fork())) return rc;
  if ((rc = phase_adjoint_range<R>(P, occ, g_re, g_im, ws, 0, ka, st, adam))) return rc;
  if ((rc = phase_adjoint_range<R>(P, occ, g_re, g_im, ws, ka, kb, P->side, adam))) return rc;
  if ((rc = join())) return rc;
  return sum_energy_slots(P, slots, energies, ws, st);
}

template <typename R>
static int energy_grad(const jrg_plan* P, const void* w_re, const void* w_im, const double* occ,
                       double* energies, void* g_re, void* g_im, void* ws, cudaStream_t st) {
  const int rc = pipeline_ok(P) && g_pipeline
                     ? energy_grad_pipelined<R>(P, w_re, w_im, occ, energies, g_re, g_im, ws, st)
                     : energy_grad_impl<R>(P, w_re, w_im, occ, energies, g_re, g_im, ws, st);
  profile_call_done(P);
  return rc;
}

template <typename R>
static int density_entry(const jrg_plan* P, const void* coeff, const double* occ, void* rho, void* ws,
                         cudaStream_t st) {
  const int nsk = P->ns * P->nk;
  int rc = launch_pack_params<R>(coeff, nullptr, wsp(ws, P->ws.c), nsk, P->ng, P->nb, true, st);
  if (rc) return rc;
  return density_from_c<R>(P, occ, ws, rho, st);
}

template <typename R>
static int coeff_entry(const jrg_plan* P, const void* w_re, const void* w_im, void* coeff, void* ws,
                       cudaStream_t st) {
  JRG_CUDA(cudaMemsetAsync(wsp(ws, P->ws.flags), 0, 64, st));
  return orthonormalise<R>(P, w_re, w_im, ws, st, kRotGC, coeff);
}

// Vector-Jacobian product of the coefficient map: g_W = (g_C - C K) R^-H with
// K the Hermitian completion of the upper triangle of C^H g_C (real diagonal);
// grad_coeff is the cotangent of C as torch reports it for a real loss,
// dL/dRe C + i dL/dIm C, and grad_re + i grad_im = g_W the same way.
template <typename R>
static int coeff_adjoint_entry(const jrg_plan* P, const void* w_re, const void* w_im, const void* gcoeff,
                               void* g_re, void* g_im, void* ws, cudaStream_t st) {
  const Workspace& w = P->ws;
  const int nsk = P->ns * P->nk;
  int rc;
  JRG_CUDA(cudaMemsetAsync(wsp(ws, w.flags), 0, 64, st));
  if ((rc = orthonormalise<R>(P, w_re, w_im, ws, st))) return rc;   // C band-major, R^-1
  if ((rc = launch_pack_params<R>(gcoeff, nullptr, wsp(ws, w.gc), nsk, P->ng, P->nb, true, st))) return rc;
  if ((rc = launch_gram<R>(kBand, wsp(ws, w.c), nullptr, kBand, wsp(ws, w.gc), nullptr,
                           (double2*)wsp(ws, w.adj_part), (double2*)wsp(ws, w.adj), nsk, P->ng, P->nb,
                           P->ws.gram_splits, st, (int*)wsp(ws, w.flags))))
    return rc;
  double2* rh = (double2*)wsp(ws, w.kmat);
  double2* negm2 = rh + (size_t)nsk * P->nb * P->nb;
  if ((rc = launch_adjoint_small((double2*)wsp(ws, w.adj), (double2*)wsp(ws, w.rinv), rh, negm2, nsk, P->nb,
                                 st)))
    return rc;
  return launch_rotate<R>(kRotGSplit, kBand, wsp(ws, w.gc), nullptr, rh, wsp(ws, w.c), negm2, g_re, g_im, nsk,
                          P->ng, P->nb, 1.0, wsp(ws, w.rot_scratch), st, kTriLower);
}

template <typename R>
static int potential_entry(const jrg_plan* P, const void* rho, int ks, void* out, void* ws,
                           cudaStream_t st) {
  using C = C_t<R>;
  const Workspace& w = P->ws;
  const double N = (double)P->ngrid;
  C* rhog = (C*)wsp(ws, w.rhog);
  C* scratch = (C*)wsp(ws, w.fft_scratch);
  const C* tw = (const C*)P->d.tw;
  R* o = (R*)out;
  int rc;
  const void* rho_t = rho;   // the density of the Hartree term
  if (P->ns == 2) {
    R* tot = (R*)wsp(ws, w.rho) + 2 * (size_t)P->ngrid;
    if ((rc = launch_spin_total<R>(rho, tot, P->ngrid, st))) return rc;
    rho_t = tot;
  }
  if ((rc = launch_fft3d_dense<R>(P->ax, tw, 1, -1, true, rho_t, scratch, rhog, 1.0, st))) return rc;
  if ((rc = launch_hartree_g<R>(rhog, P->d.ginv, rhog, P->ngrid, ks ? 1.0 : 0.5, st))) return rc;
  if ((rc = launch_fft3d_dense<R>(P->ax, tw, 1, +1, false, rhog, scratch, rhog, 1.0 / N, st))) return rc;
  if ((rc = launch_real_part<R>(rhog, o, P->ngrid, 1.0, st))) return rc;
  if ((rc = launch_fft3d_dense<R>(P->ax, tw, 1, +1, false, P->d.vext, scratch, rhog, 1.0 / N, st))) return rc;
  if ((rc = launch_real_part<R>(rhog, o + P->ngrid, P->ngrid, 1.0, st))) return rc;
  if (P->xc & kXcGga) {
    if ((rc = launch_fft3d_dense<R>(P->ax, tw, 1, -1, true, rho, scratch, rhog, 1.0, st))) return rc;
    if ((rc = gga_gradients<R>(P, rhog, ws, st))) return rc;
    return gga_potential<R>(P, rho, nullptr, 0.0, o + 2 * P->ngrid, nullptr, ks ? 0 : 1, ws, st);
  }
  if (P->ns == 2) {
    // xc part per spin: vxc_lda's field (Kohn-Sham), or eps in both grids
    if ((rc = launch_lda_pol(P->prec, P->ngrid, P->xc, ks, rho, o + 2 * P->ngrid, st))) return rc;
    if (!ks)
      JRG_CUDA(cudaMemcpyAsync(o + 3 * P->ngrid, o + 2 * P->ngrid, sizeof(R) * (size_t)P->ngrid,
                               cudaMemcpyDeviceToDevice, st));
    return JRG_OK;
  }
  return launch_xc_field<R>(rho, o + 2 * P->ngrid, P->ngrid, P->xc, ks, st);
}

}  // namespace jrg

extern "C" {

int jrg_coeff(const jrg_plan* P, const void* w_re, const void* w_im, void* coeff, void* ws,
              cudaStream_t st) {
  if (!P || !w_re || !w_im || !coeff || !ws) return fail(JRG_ERR_INVALID, "jrg_coeff: null argument");
  return P->prec == 64 ? coeff_entry<double>(P, w_re, w_im, coeff, ws, st)
                       : coeff_entry<float>(P, w_re, w_im, coeff, ws, st);
}

int jrg_coeff_adjoint(const jrg_plan* P, const void* w_re, const void* w_im, const void* grad_coeff,
                      void* grad_re, void* grad_im, void* ws, cudaStream_t st) {
  if (!P || !w_re || !w_im || !grad_coeff || !grad_re || !grad_im || !ws)
    return fail(JRG_ERR_INVALID, "jrg_coeff_adjoint: null argument");
  return P->prec == 64 ? coeff_adjoint_entry<double>(P, w_re, w_im, grad_coeff, grad_re, grad_im, ws, st)
                       : coeff_adjoint_entry<float>(P, w_re, w_im, grad_coeff, grad_re, grad_im, ws, st);
}

int jrg_density(const jrg_plan* P, const void* coeff, const double* occ, void* rho, void* ws,
                cudaStream_t st) {
  if (!P || !coeff || !occ || !rho || !ws) return fail(JRG_ERR_INVALID, "jrg_density: null argument");
  return P->prec == 64 ? density_entry<double>(P, coeff, occ, rho, ws, st)
                       : density_entry<float>(P, coeff, occ, rho, ws, st);
}

int jrg_energy_grad(const jrg_plan* P, const void* w_re, const void* w_im, const double* occ,
                    double* energies, void* g_re, void* g_im, void* ws, cudaStream_t st) {
  if (!P || !w_re || !w_im || !occ || !energies || !ws)
    return fail(JRG_ERR_INVALID, "jrg_energy_grad: null argument");
  if (P->ns == 2 && (P->xc & kXcGga))
    return fail(JRG_ERR_UNSUPPORTED, "jrg_energy_grad: spin-polarised PBE is not implemented");
  return P->prec == 64 ? energy_grad<double>(P, w_re, w_im, occ, energies, g_re, g_im, ws, st)
                       : energy_grad<float>(P, w_re, w_im, occ, energies, g_re, g_im, ws, st);
}

int jrg_energy_grad_bands(const jrg_plan* P, const void* w_re, const void* w_im, const double* occ,
                          double* energies, double* band_energies, void* g_re, void* g_im, void* ws,
                          cudaStream_t st) {
  if (!P || !w_re || !w_im || !occ || !energies || !band_energies || !g_re || !g_im || !ws)
    return fail(JRG_ERR_INVALID, "jrg_energy_grad_bands: null argument");
  if (P->ns == 2 && (P->xc & kXcGga))
    return fail(JRG_ERR_UNSUPPORTED, "jrg_energy_grad_bands: spin-polarised PBE is not implemented");
  int rc = P->prec == 64
               ? energy_grad_impl<double>(P, w_re, w_im, occ, energies, g_re, g_im, ws, st, nullptr, band_energies)
               : energy_grad_impl<float>(P, w_re, w_im, occ, energies, g_re, g_im, ws, st, nullptr, band_energies);
  profile_call_done(P);
  return rc;
}

int jrg_pipeline(int enable) {
  const int prev = jrg::g_pipeline ? 1 : 0;
  if (enable >= 0) jrg::g_pipeline = enable != 0;
  return prev;
}

int jrg_band_trace_grad(const jrg_plan* P, const void* w_re, const void* w_im, const void* v_eff,
                        const double* weights, double* out, void* hmat, void* grad_re, void* grad_im,
                        void* ws, cudaStream_t st) {
  if (!P || !w_re || !w_im || !v_eff || !weights || !out || !ws)
    return fail(JRG_ERR_INVALID, "jrg_band_trace_grad: null argument");
  int rc = P->prec == 64 ? band_trace_impl<double>(P, w_re, w_im, v_eff, weights, out, hmat, grad_re, grad_im, ws, st)
                         : band_trace_impl<float>(P, w_re, w_im, v_eff, weights, out, hmat, grad_re, grad_im, ws, st);
  profile_call_done(P);
  return rc;
}

int jrg_energy_grad_adam(const jrg_plan* P, void* params, void* m, void* v, const double* occ,
                         const jrg_adam_step* opt, double* energies, void* grad, void* ws,
                         cudaStream_t st) {
  if (!P || !params || !m || !v || !occ || !opt || !energies || !ws || opt->step < 1)
    return fail(JRG_ERR_INVALID, "jrg_energy_grad_adam: bad argument");
  if (opt->mlp_w32 && (!opt->mlp_wb || !opt->scale))
    return fail(JRG_ERR_INVALID, "jrg_energy_grad_adam: the learned scale needs mlp_wb and a scale buffer");
  if (P->ns == 2 && (P->xc & kXcGga))
    return fail(JRG_ERR_UNSUPPORTED, "jrg_energy_grad_adam: spin-polarised PBE is not implemented");
  if (P->nb > 32 && jrg_tensor_core_paths(-1) != 0)
    return fail(JRG_ERR_UNSUPPORTED, "jrg_energy_grad_adam: num_band > 32 needs contraction mode 0");
  const size_t n = (size_t)P->ns * P->nk * P->ng * P->nb;
  const size_t half = n * (P->prec == 64 ? 8 : 4);
  auto hi = [&](void* b) { return b ? (void*)((char*)b + half) : nullptr; };
  AdamArgs a;
  a.p[0] = params; a.p[1] = hi(params);
  a.m[0] = m; a.m[1] = hi(m);
  a.v[0] = v; a.v[1] = hi(v);
  a.scale[0] = opt->scale; a.scale[1] = opt->scale ? opt->scale + n : nullptr;
  a.grad[0] = grad; a.grad[1] = hi(grad);
  a.lr = opt->lr; a.b1 = opt->b1; a.b2 = opt->b2; a.eps = opt->eps;
  a.c1 = 1.0 - std::pow(opt->b1, opt->step);
  a.c2 = 1.0 - std::pow(opt->b2, opt->step);
  a.mlp_w32 = opt->mlp_w32; a.mlp_wb = opt->mlp_wb;
  a.t_frac = opt->t_frac; a.smax = opt->smax;
  a.guard = (const int*)((const char*)ws + P->ws.flags);
  int rc;
  if (pipeline_ok(P) && g_pipeline)   // per-half gradient + Adam in the two-stream pipeline
    rc = P->prec == 64 ? energy_grad_pipelined<double>(P, a.p[0], a.p[1], occ, energies, nullptr, nullptr, ws, st, &a)
                       : energy_grad_pipelined<float>(P, a.p[0], a.p[1], occ, energies, nullptr, nullptr, ws, st, &a);
  else   // Adam in the epilogue of the adjoint rotation
    rc = P->prec == 64 ? energy_grad_impl<double>(P, a.p[0], a.p[1], occ, energies, nullptr, nullptr, ws, st, &a)
                       : energy_grad_impl<float>(P, a.p[0], a.p[1], occ, energies, nullptr, nullptr, ws, st, &a);
  profile_call_done(P);
  return rc;
}

int jrg_reorthonormalise(const jrg_plan* P, void* w_re, void* w_im, void* ws, cudaStream_t st) {
  if (!P || !w_re || !w_im || !ws) return fail(JRG_ERR_INVALID, "jrg_reorthonormalise: null argument");
  const int nsk = P->ns * P->nk;
  // FP64 scratch for the column being projected: the plane buffer
  const size_t need = (size_t)nsk * P->ng * sizeof(double2);
  const size_t have = P->ws.t_bytes;
  if (need > have) return fail(JRG_ERR_UNSUPPORTED, "jrg_reorthonormalise: workspace too small for the scratch");
  double2* scratch = (double2*)wsp(ws, P->ws.t);
  return P->prec == 64 ? launch_reorthonormalise<double>(w_re, w_im, scratch, nsk, P->ng, P->nb, st)
                       : launch_reorthonormalise<float>(w_re, w_im, scratch, nsk, P->ng, P->nb, st);
}

int jrg_potential(const jrg_plan* P, const void* rho, int ks, void* out, void* ws, cudaStream_t st) {
  if (!P || !rho || !out || !ws) return fail(JRG_ERR_INVALID, "jrg_potential: null argument");
  if (P->ns == 2 && (P->xc & kXcGga))
    return fail(JRG_ERR_UNSUPPORTED, "jrg_potential: spin-polarised PBE is not implemented");
  return P->prec == 64 ? potential_entry<double>(P, rho, ks, out, ws, st)
                       : potential_entry<float>(P, rho, ks, out, ws, st);
}

int jrg_fft3d_workspace_size(int prec, const int grid[3], int batch, size_t* bytes) {
  if (!grid || !bytes || batch < 1 || (prec != 32 && prec != 64))
    return fail(JRG_ERR_INVALID, "jrg_fft3d_workspace_size: bad argument");
  const size_t c = csize(prec);
  *bytes = align256(c * (size_t)(grid[0] + grid[1] + grid[2])) +
           align256(c * (size_t)batch * grid[0] * grid[1] * grid[2]);
  return JRG_OK;
}

int jrg_fft3d(int prec, const int grid[3], int batch, int direction, const void* in, void* out,
              void* ws, cudaStream_t st) {
  if (!grid || !in || !out || !ws || batch < 1 || (direction != 1 && direction != -1) ||
      (prec != 32 && prec != 64))
    return fail(JRG_ERR_INVALID, "jrg_fft3d: bad argument");
  FftAxis ax[3];
  for (int a = 0; a < 3; ++a)
    if (!factor_axis(grid[a], &ax[a])) return fail(JRG_ERR_UNSUPPORTED, "grid size must be 7-smooth");
  {
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    const size_t c = csize(prec);
    const size_t pb = c * (grid[1] + grid[2] + 2 * (size_t)grid[1] * grid[2]) + 4;
    const size_t lb = c * (grid[0] + 2 * (size_t)grid[0] * grid[2]);
    if ((long long)pb > optin || (long long)lb > optin)
      return fail(JRG_ERR_UNSUPPORTED, "grid too large for the shared-memory slab kernels");
  }
  const int nt = grid[0] + grid[1] + grid[2];
  char* tw = (char*)ws;
  char* scratch = tw + align256((size_t)csize(prec) * nt);
  int rc = JRG_OK;
  int off = 0;
  for (int a = 0; a < 3 && !rc; ++a) {
    rc = launch_twiddles(grid[a], prec, tw + (size_t)csize(prec) * off, st);
    off += grid[a];
  }
  if (rc) return rc;
  const double scale = direction > 0 ? 1.0 / ((double)grid[0] * grid[1] * grid[2]) : 1.0;
  if (prec == 64)
    return launch_fft3d_dense<double>(ax, (const double2*)tw, batch, direction, false, in,
                                      (double2*)scratch, (double2*)out, scale, st);
  return launch_fft3d_dense<float>(ax, (const float2*)tw, batch, direction, false, in,
                                   (float2*)scratch, (float2*)out, scale, st);
}

int jrg_precond_scale(const jrg_plan* P, const float* w32, const void* wb, float t_frac, float smax,
                      const double* occ, float* scale, void* ws, cudaStream_t st) {
  if (!P || !w32 || !wb || !occ || !scale || !ws)
    return fail(JRG_ERR_INVALID, "jrg_precond_scale: null argument");
  const long long total = (long long)P->ns * P->nk * P->ng * P->nb;
  return launch_precond_scale(w32, wb, P->d.tk, (const double*)wsp(ws, P->ws.ekin), occ, P->nk, P->ng,
                              P->nb, total, t_frac, smax, scale, st);
}

int jrg_band_kinetic(const jrg_plan* P, const void* ws, double* out, cudaStream_t st) {
  if (!P || !ws || !out) return fail(JRG_ERR_INVALID, "jrg_band_kinetic: null argument");
  JRG_CUDA(cudaMemcpyAsync(out, (const char*)ws + P->ws.ekin,
                           sizeof(double) * (size_t)P->ns * P->nk * P->nb, cudaMemcpyDeviceToDevice, st));
  return JRG_OK;
}

int jrg_kinetic_table(const jrg_plan* P, double* out, cudaStream_t st) {
  if (!P || !out) return fail(JRG_ERR_INVALID, "jrg_kinetic_table: null argument");
  JRG_CUDA(cudaMemcpyAsync(out, P->d.tk, sizeof(double) * (size_t)P->nk * P->ng,
                           cudaMemcpyDeviceToDevice, st));
  return JRG_OK;
}

int jrg_lda(int prec, int64_t n, int xc, int kohn_sham, const void* rho, void* out, cudaStream_t st) {
  if (!rho || !out || n < 0 || (prec != 32 && prec != 64) || (xc & ~3) || !xc)
    return fail(JRG_ERR_INVALID, "jrg_lda: bad argument");
  return launch_lda(prec, n, xc, kohn_sham ? 1 : 0, rho, out, st);
}

int jrg_lda_polarized(int prec, int64_t n, int xc, int kohn_sham, const void* rho, void* out, cudaStream_t st) {
  if (!rho || !out || n < 0 || (prec != 32 && prec != 64) || (xc & ~3) || !xc)
    return fail(JRG_ERR_INVALID, "jrg_lda_polarized: bad argument");
  if (kohn_sham < 0 || kohn_sham > 2) return fail(JRG_ERR_INVALID, "jrg_lda_polarized: kohn_sham must be 0, 1 or 2");
  return launch_lda_pol(prec, n, xc, kohn_sham, rho, out, st);
}

int jrg_adam_update(int prec, int64_t n, void* param, const void* grad, void* m, void* v,
                    const float* scale, int step, double lr, double b1, double b2, double eps,
                    cudaStream_t st) {
  if (!param || !grad || !m || !v || n < 0 || step < 1 || (prec != 32 && prec != 64))
    return fail(JRG_ERR_INVALID, "jrg_adam_update: bad argument");
  const double c1 = 1.0 - std::pow(b1, step), c2 = 1.0 - std::pow(b2, step);
  if (prec == 64) return launch_adam<double>(param, grad, m, v, scale, n, lr, b1, b2, c1, c2, eps, st);
  return launch_adam<float>(param, grad, m, v, scale, n, lr, b1, b2, c1, c2, eps, st);
}

int jrg_ewald(const jrg_plan* P, double eta, double cutoff, double* result, void* ws, cudaStream_t st) {
  if (!P || !result || !ws || !(eta > 0) || !(cutoff > 0)) return fail(JRG_ERR_INVALID, "jrg_ewald: bad argument");
  // translation grid: n = ceil(cutoff / |a1 + a2 + a3|^2) per axis, fftfreq ordering
  double s[3] = {0, 0, 0};
  for (int i = 0; i < 3; ++i)
    for (int c = 0; c < 3; ++c) s[c] += P->cell[3 * i + c];
  const double nrm2 = s[0] * s[0] + s[1] * s[1] + s[2] * s[2];
  const int nt = (int)std::ceil(cutoff / nrm2);
  if (nt < 1 || nt > 4096) return fail(JRG_ERR_UNSUPPORTED, "jrg_ewald: translation grid out of range");
  const int na = (int)P->charge.size();
  return launch_ewald(P->d_cell, P->d.gvec, P->d_atoms, P->d_atoms + 3 * na, na, nt, P->ngrid, eta,
                      P->vol, (double*)wsp(ws, P->ws.epart), kEwaldBlocks, result, st);
}

}  // extern "C"

namespace {
const char* kPhaseNames[jrg::PH_COUNT] = {
  "pack_params", "gram", "cholesky_inv", "rotate", "kinetic", "plane_inv_sphere", "line_density",
  "reduce_density", "grid_terms", "line_apply_v", "plane_fwd_sphere", "adj_gram", "adj_small",
  "adj_rotate", "precond_scale", "nl_project", "nl_apply"};
}

extern "C" {

int jrg_profile_num_phases(void) { return jrg::PH_COUNT; }

const char* jrg_profile_phase_name(int ph) {
  return (ph >= 0 && ph < jrg::PH_COUNT) ? kPhaseNames[ph] : "";
}

int jrg_profile_enable(jrg_plan* P, int max_calls) {
  if (!P || max_calls < 0) return fail(JRG_ERR_INVALID, "jrg_profile_enable: bad argument");
  if (P->prof) {
    for (cudaEvent_t e : P->prof->ev) cudaEventDestroy(e);
    delete P->prof;
    P->prof = nullptr;
  }
  if (max_calls == 0) return JRG_OK;
  Profiler* pr = new Profiler();
  pr->max_calls = max_calls;
  pr->ev.resize((size_t)max_calls * PH_COUNT * 2);
  pr->used.assign((size_t)max_calls * PH_COUNT, 0);
  for (auto& e : pr->ev) {
    cudaError_t ce = cudaEventCreate(&e);
    if (ce != cudaSuccess) {
      delete pr;
      return cuda_fail(ce, "cudaEventCreate");
    }
  }
  P->prof = pr;
  return JRG_OK;
}

int jrg_profile_read(jrg_plan* P, double* ms, int* calls, int n) {
  if (!P || !ms || n < 1) return fail(JRG_ERR_INVALID, "jrg_profile_read: bad argument");
  for (int i = 0; i < n; ++i) ms[i] = 0.0;
  if (calls) *calls = 0;
  Profiler* pr = P->prof;
  if (!pr) return JRG_OK;
  for (int c = 0; c < pr->calls; ++c) {
    for (int ph = 0; ph < PH_COUNT && ph < n; ++ph) {
      if (!pr->used[(size_t)c * PH_COUNT + ph]) continue;
      cudaEvent_t a = pr->ev[((size_t)c * PH_COUNT + ph) * 2], b = pr->ev[((size_t)c * PH_COUNT + ph) * 2 + 1];
      JRG_CUDA(cudaEventSynchronize(b));
      float t = 0.f;
      JRG_CUDA(cudaEventElapsedTime(&t, a, b));
      ms[ph] += t;
    }
  }
  if (calls) *calls = pr->calls;
  return JRG_OK;
}

}  // extern "C"
