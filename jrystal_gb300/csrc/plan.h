// Internal plan layout shared by the kernels and the C ABI.
#pragma once
#include <string>
#include <vector>
#include "../../include/jrystal_gb300.h"
#include "fft_smem.cuh"

namespace jrg {

// Thread-local error reporting for the C ABI.
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

#define JRG_CUDA(call)                                   \
  do {                                                   \
    cudaError_t e_ = (call);                             \
    if (e_ != cudaSuccess) return ::jrg::cuda_fail(e_, #call); \
  } while (0)

void count_launch();

#define JRG_LAUNCH_CHECK(what)                           \
  do {                                                   \
    ::jrg::count_launch();                               \
    cudaError_t e_ = cudaGetLastError();                 \
    if (e_ != cudaSuccess) return ::jrg::cuda_fail(e_, what); \
  } while (0)

bool factor_axis(int n, FftAxis* ax);

// Charge renormalisation of the energy path's density.  The exact density of
// orthonormal coefficients integrates to sum_{s,k,b} occ (Parseval); the FP32
// density misses that by ~1e-8 (rounding of the coefficients and of the
// transforms), which the all-electron external energy (hundreds of Ha) turns
// into ~1e-6 Ha per atom.  k_reduce_density leaves FP64 partial sums of rho
// in qpart, k_recip_terms forms s = sum occ / (vol/N sum rho) (1 without
// qpart) and stores it in *scale, and the Hartree, external and xc terms use
// s rho.
constexpr int kQParts = 1024;   // CTAs of k_reduce_density, one charge partial each
struct ChargeFix {
  const double* qpart = nullptr;  // [kQParts]
  const double* occ = nullptr;    // [nocc]
  int nocc = 0;
  double dv = 0.0;                // vol / N
  double* scale = nullptr;        // s
};

// Device tables of one plan.
struct PlanTables {
  int* gidx = nullptr;        // [ng] flattened grid index
  int* sph_yz = nullptr;      // [ng] y*nz + z
  int* plane_x = nullptr;     // [nact] x index of each active plane
  int* plane_off = nullptr;   // [nact+1] sphere offsets per plane
  int* row_off = nullptr;     // [nact+1] offsets into rows
  int* rows = nullptr;        // active y rows per plane
  int* rowmap = nullptr;      // [total active rows][nz]: sphere index of (row, z), or -1
  int* xact = nullptr;        // [nx] active-plane slot of x, or -1
  double* tk = nullptr;       // [nk][ng] |G+k|^2 / 2
  float* tkf = nullptr;       // the same in FP32 (tabulated preconditioner)
  void* tw = nullptr;         // twiddles: x table, y table, z table (C_t<R>)
  void* vext = nullptr;       // [ngrid] complex V_ext(G) in precision R
  double2* vext64 = nullptr;  // [ngrid] the same table in FP64 (= vext at FP64)
  double* vext_r = nullptr;   // [ngrid] real-space V_ext(r) = Re IFFT(V_ext(G)), FP64
  double* ginv = nullptr;     // [ngrid] 4 pi / |G|^2, 0 at G = 0
  double* gvec = nullptr;     // [ngrid][3] cartesian G vectors
  void* proj = nullptr;       // [nk][nproj][ng] complex beta-projector table (precision R)
};

// Per-phase CUDA-event timing of the fused entry points (optional).
enum Phase {
  PH_PACK = 0, PH_GRAM, PH_CHOL, PH_ROTATE, PH_KINETIC, PH_PLANE_INV, PH_LINE_DENSITY,
  PH_REDUCE_DENSITY, PH_GRID_TERMS, PH_LINE_APPLY_V, PH_PLANE_FWD, PH_ADJ_GRAM, PH_ADJ_SMALL,
  PH_ADJ_ROTATE, PH_PRECOND, PH_NL_PROJECT, PH_NL_APPLY, PH_COUNT
};
struct Profiler {
  int max_calls = 0;
  int calls = 0;                         // calls recorded so far
  std::vector<cudaEvent_t> ev;           // [max_calls][PH_COUNT][2]
  std::vector<unsigned char> used;       // [max_calls][PH_COUNT]
};

// One fused optimiser step: Adam applied in the epilogue of the adjoint
// rotation (k_rotate_adam); all buffers [S][K][G][B], index 0 real parts,
// 1 imaginary parts.
struct AdamArgs {
  void* p[2];
  void* m[2];
  void* v[2];
  float* scale[2];        // per-element update scale (optional; learned scales when mlp_w32)
  void* grad[2];          // gradient output (optional)
  double lr, b1, b2, c1, c2, eps;
  const float* mlp_w32;   // learned preconditioner evaluated inside the step (optional)
  const void* mlp_wb;
  float t_frac, smax;
  const int* guard;       // status word of the call: no update when non-zero (optional)
};

// Workspace offsets (bytes) of one plan.
struct Workspace {
  size_t wc, c, gram_part, gram, rmat, rinv, t, u, rho_part, rho_scale, rho_q, rho, rhog, fft_scratch, vr,
      gc, adj_part, adj, kmat, epart, flags, ekin, dinv, rot_scratch, gga, kin_part, nl_part, nl_fw, lut,
      total;
  size_t t_bytes; // plane buffer
  int gram_splits;
  int nl_splits;  // G splits of the projector contraction
  int ngroups;    // density partial groups
  int nepart;     // energy partial slots
};

}  // namespace jrg

struct jrg_plan {
  int prec;                 // 32 or 64
  int nx, ny, nz;
  long long ngrid;
  int ns, nk, nb, ng;
  int nact;                 // active x planes
  int max_rows;             // max active rows in a plane
  // N = 32 or 64 (8 values per thread in the slab transforms) with every
  // active x plane (xprune) / active row y and sphere z (yzprune) below N/4 or
  // at or above 3N/4: the x (y, z) transforms skip the known zeros
  bool xprune = false;
  bool yzprune = false;
  double cell[9], recip[9], vol;
  std::vector<double> pos, charge, kpts;
  int xc;
  int nproj = 0;            // beta-projector rows of the pseudopotential (0: all-electron)
  size_t mem_limit = 0;     // workspace bound set by jrg_plan_set_memory_limit (0: none)
  int kchunk = 0;           // (s,k) blocks whose plane buffers are resident at once
  float tk_max = 0.f;       // largest |G+k|^2 / 2 of the plan
  jrg::FftAxis ax[3];
  jrg::PlanTables d;
  jrg::Workspace ws;
  int device;
  int* slot_begin = nullptr;  // energy slot boundaries [5]
  double* d_cell = nullptr;   // cell (9) then reciprocal vectors (9)
  double* d_atoms = nullptr;  // positions [natom][3] then charges [natom]
  double* d_ones = nullptr;   // [S*K*B] ones: unweighted band weights
  cudaStream_t side = nullptr;   // second stream of the two-way k-point pipeline
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
  jrg::Profiler* prof = nullptr;
};
