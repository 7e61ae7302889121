/*
 * jrystal_gb300 — C ABI of the GB300 (sm_103a) direct-minimisation
 * energy-and-gradient library.
 *
 * Every entry point takes caller-owned device pointers, plain sizes and a
 * cudaStream_t.  Plan set-up (jrg_plan_create, jrg_plan_set_pseudopotential)
 * allocates the plan's device tables; no other entry point allocates device
 * memory.  Scratch memory is a caller workspace of jrg_workspace_size() bytes
 * (256-byte aligned).  Functions
 * return a jrg_status; on failure jrg_last_error() gives a thread-local
 * message.  Numerical faults (Cholesky breakdown, non-finite values) are
 * reported through the status word of the call, never by trapping.
 *
 * The entry points replace the device work of these jrystal functions
 * (paths relative to the jrystal project):
 *   jrg_coeff          pw.coeff / unitary_module.unitary_matrix
 *                      jrystal/_src/pw.py:94-137, unitary_module.py:30-80
 *   jrg_density        pw.density_grid with occupation
 *                      jrystal/_src/pw.py:214-284 (+ utils.py:257-281 scatter)
 *   jrg_energy_grad    value_and_grad of total_energy in the ground-state
 *                      driver, calc/calc_ground_state_energy_all_electrons.py:119-181
 *                      (energy.kinetic/hartree/external/xc_energy,
 *                      jrystal/_src/energy.py:29-211)
 *   jrg_potential      potential.effective (non-Kohn-Sham and Kohn-Sham)
 *                      jrystal/_src/potential.py:203-279
 *   jrg_fft3d          spmd.fft.fftn3d / ifftn3d and jnp.fft.fftn over the
 *                      last three axes, jrystal/_src/spmd/fft.py:37-75
 *   jrg_adam_update    optax.adam update + apply_updates,
 *                      calc/opt_utils.py:153-168, calc driver :179-180
 *   jrg_ewald          ewald.ewald_coulomb_repulsion, jrystal/_src/ewald.py:21-86
 *   jrg_plan_set_pseudopotential  normcons.potential_local_reciprocal /
 *                      potential_nonlocal_psi_reciprocal tables consumed by
 *                      energy_local / energy_nonlocal in the norm-conserving
 *                      driver, calc/calc_ground_state_energy_normcons.py:115-192
 *   jrg_precond_*      learned diagonal preconditioner (no jrystal counterpart)
 */
#ifndef JRYSTAL_GB300_H_
#define JRYSTAL_GB300_H_

#include <stddef.h>
#include <stdint.h>
#include <cuda_runtime.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  JRG_OK = 0,
  JRG_ERR_INVALID = 1,      /* bad argument, shape or pointer */
  JRG_ERR_CUDA = 2,         /* a CUDA runtime call failed */
  JRG_ERR_NUMERIC = 3,      /* Cholesky breakdown or non-finite result */
  JRG_ERR_UNSUPPORTED = 4   /* size/precision the kernels do not cover */
} jrg_status;

/* exchange-correlation terms, OR-ed: "lda_x" and "lda_c_vwn" */
#define JRG_XC_LDA_X 1
#define JRG_XC_LDA_C_VWN 2
#define JRG_XC_GGA_X_PBE 4   /* PBE exchange (jax_xc gga_x_pbe); not combinable with the LDA flags */
#define JRG_XC_GGA_C_PBE 8   /* PBE correlation (jax_xc gga_c_pbe) */

typedef struct jrg_plan jrg_plan;

typedef struct {
  int precision;            /* 32: complex64/float32 arrays, 64: complex128/float64 */
  int grid[3];              /* FFT grid (x, y, z), each 7-smooth */
  double cell[9];           /* lattice vectors as rows, bohr */
  int num_atom;
  const double* positions;  /* host [num_atom][3], bohr */
  const double* charges;    /* host [num_atom] */
  int num_spin;             /* 1 (spin restricted) or 2 */
  int num_kpt;
  int num_band;
  const double* kpts;       /* host [num_kpt][3], cartesian */
  int num_g;                /* plane-wave sphere size */
  const int32_t* sphere_index; /* host [num_g]: (x*ny + y)*nz + z of each
                                  True entry of the frequency mask, strictly
                                  increasing (row-major mask order) */
  int xc;                   /* JRG_XC_* flags */
} jrg_plan_desc;

/* Library version, the last error message of the calling thread, and the
 * number of kernels this library has launched in the process so far. */
int jrg_version(void);
const char* jrg_last_error(void);
long long jrg_launch_count(void);

/* Plans: geometry tables (sphere maps, twiddles, kinetic and external
 * potential tables) on the current device.  Creating a plan allocates its
 * tables and synchronises the device; all other calls only enqueue work.
 * Concurrency: a plan serves one host thread at a time (its second stream,
 * fork/join events and phase profiler belong to the plan); threads that call
 * concurrently use a plan each.  Calls that may overlap on the device need
 * separate workspaces.  Distinct plans share no mutable state. */
int jrg_plan_create(const jrg_plan_desc* desc, jrg_plan** out);
int jrg_plan_destroy(jrg_plan* plan);
/* Caller workspace needed by the entry points below (bytes). */
int jrg_workspace_size(const jrg_plan* plan, size_t* bytes);

/* Bound on the workspace (bytes; 0 removes it).  The largest buffer holds
 * the plane transforms of every band (the reference keeps the whole wave
 * grid instead, jrystal/_src/pw.py:140-211); under a bound it holds as many
 * (s,k) blocks as fit, at least one, and the energy entry points run the
 * blocks in chunks, transforming each chunk's coefficients again for the
 * adjoint instead of keeping the planes of the density pass (about one more
 * inverse plane pass per band, no two-stream pipeline).  Query
 * jrg_workspace_size again afterwards; jrg_plan_memory_chunk gives the
 * blocks per chunk (the number of (s,k) blocks when nothing is recomputed). */
int jrg_plan_set_memory_limit(jrg_plan* plan, size_t bytes);
int jrg_plan_memory_chunk(const jrg_plan* plan, int* kchunk);

/* Norm-conserving pseudopotential of the plan's atoms (replaces the
 * all-electron Coulomb external potential; plan setup, allocates and
 * synchronises like jrg_plan_create):
 *   v_local     host double [nx][ny][nz] interleaved complex, the local part
 *               V_loc(G) of potential_local_reciprocal
 *               (jrystal/pseudopotential/local.py:32-132); NULL keeps the
 *               current table;
 *   projectors  host double [K][num_proj][G] interleaved complex, the rows
 *               of potential_nonlocal_psi_reciprocal on the plane-wave sphere
 *               (jrystal/pseudopotential/nloc.py:42-139); num_proj = 0
 *               removes the nonlocal term.
 * Every energy entry point then adds E_nl = sum f/vol sum_j |sum_G c P_j|^2
 * (nloc.py:143-157, 238-248) to the external energy (energies[1]; the
 * nonlocal part alone in energies[7]) and its gradient; jrg_potential's
 * external part becomes IFFT(V_loc).  The workspace grows: query
 * jrg_workspace_size again. */
int jrg_plan_set_pseudopotential(jrg_plan* plan, const double* v_local, int num_proj,
                                 const double* projectors);

/* Orthonormal coefficients from raw parameters.
 * w_re, w_im: [S][K][G][B] real; coeff: [S][K][G][B] interleaved complex.
 * Columns equal jnp.linalg.qr's Q up to a unit phase per band. */
int jrg_coeff(const jrg_plan* plan, const void* w_re, const void* w_im, void* coeff,
              void* workspace, cudaStream_t stream);

/* Vector-Jacobian product of jrg_coeff (the transpose rule of the QR in
 * unitary_module.py:74-80 as jax.grad applies it through pw.coeff,
 * jrystal/_src/pw.py:94-137): given W and the cotangent grad_coeff of the
 * coefficients ([S][K][G][B] complex, dL/dRe C + i dL/dIm C for a real loss
 * L), writes dL/dw_re and dL/dw_im ([S][K][G][B] real).  Recomputes the
 * orthonormalisation from W. */
int jrg_coeff_adjoint(const jrg_plan* plan, const void* w_re, const void* w_im,
                      const void* grad_coeff, void* grad_re, void* grad_im, void* workspace,
                      cudaStream_t stream);

/* Occupation-weighted density on the grid from sphere coefficients.
 * coeff: [S][K][G][B] complex; occupation: device double [S][K][B];
 * density: [S][nx][ny][nz] real. */
int jrg_density(const jrg_plan* plan, const void* coeff, const double* occupation,
                void* density, void* workspace, cudaStream_t stream);

/* Loss and gradient of the direct-minimisation path.
 * energies (device double[8]): kinetic, external, hartree, xc, total,
 *   then the Gram condition estimate max over (s,k) and k of S_kk / d_k (the
 *   Cholesky pivots d_k of S = W^H W: 1 for orthogonal columns, growing as
 *   the columns approach linear dependence, +inf at a breakdown), the status
 *   word (bit 0: a Cholesky pivot at or below the Gram's rounding level,
 *   1e-7 S_kk in FP32 and 1e-14 S_kk in FP64, or not finite, i.e. a
 *   rank-deficient or non-finite W; bit 1: a tensor-core Gram wait ran out),
 *   and the nonlocal pseudopotential part of the external energy (0 without
 *   projectors).  A non-zero status word is the JRG_ERR_NUMERIC condition of
 *   the call: it is left on the device (reading it would synchronise) for
 *   the caller to act on, e.g. with jrg_reorthonormalise.
 * grad_re/grad_im: [S][K][G][B] d total / d w_re, d w_im (may be NULL for
 * energy only).
 * num_spin 2 (spin-polarised, LDA only): occupation [2][K][B] holds each
 * channel's occupations; Hartree and external terms act on the total
 * density, E_xc = vol/N sum eps_xc(rho_up, rho_dn) (rho_up + rho_dn) with the
 * polarised LDA of jrg_lda_polarized (jrystal/_src/xc.py:40-64,
 * energy.py:185-211), and each channel's bands see their own potential
 * V_H + V_ext + d(eps_xc rho)/d rho_s. */
int jrg_energy_grad(const jrg_plan* plan, const void* w_re, const void* w_im,
                    const double* occupation, double* energies, void* grad_re,
                    void* grad_im, void* workspace, cudaStream_t stream);

/* jrg_energy_grad plus the band energies band_energies[s,k,b] =
 * <psi_skb| T + V_eff |psi_skb> = d total / d occupation[s,k,b] (device
 * double[S*K*B]), the occupation gradient the reference driver takes with
 * value_and_grad over its occupation parameters
 * (jrystal/calc/calc_ground_state_energy_all_electrons.py:119-147,175-181).
 * num_spin 1 or 2 as jrg_energy_grad. */
int jrg_energy_grad_bands(const jrg_plan* plan, const void* w_re, const void* w_im,
                          const double* occupation, double* energies, double* band_energies,
                          void* grad_re, void* grad_im, void* workspace, cudaStream_t stream);

/* Kohn-Sham band trace of a fixed effective potential, the objective of the
 * band-structure driver (jrystal/calc/calc_band_structure_all_electrons.py:78-92,
 * hamiltonian.hamiltonian_matrix_trace with kohn_sham=True,
 * jrystal/_src/hamiltonian.py:105-168):
 *   out[0] = sum_{s,k,b} w_skb <psi_skb| T + V_eff |psi_skb>,  out[1] = its kinetic part,
 * its gradient with respect to {w_re, w_im} (optional, both or neither), and
 * optionally the band Hamiltonian hmat[s,k][i][j] = w_skj <psi_i| T + V_eff |psi_j>
 * (jrystal/_src/hamiltonian.py:171-240; complex FP64 [S*K][B][B]).
 * v_eff: device [S][nx][ny][nz] real grids in the plan's precision, each
 * spin's V_H + V_ext + v_xc (e.g. the parts of jrg_potential with
 * kohn_sham = 1 summed per spin); the bands of spin s see grid s.
 * weights: device double [S*K*B] (ones for the band structure); out: device
 * double[2]. */
int jrg_band_trace_grad(const jrg_plan* plan, const void* w_re, const void* w_im,
                        const void* v_eff, const double* weights, double* out, void* hmat,
                        void* grad_re, void* grad_im, void* workspace, cudaStream_t stream);

/* One optimiser step (no counterpart in the reference as one call: it
 * fuses value_and_grad(total_energy) and optax.adam's update of
 * jrystal/calc/calc_ground_state_energy_all_electrons.py:175-190).
 * The energies (as jrg_energy_grad) are those of the parameters before the
 * update; the Adam update of jrg_adam_update runs in the epilogue of the
 * kernel that forms the gradient, so the gradient is written only when grad
 * is given.  params, m, v, grad: [2][S][K][G][B] (real parts, then
 * imaginary parts), updated in place.  scale, when given, multiplies each
 * update element ([2][S][K][G][B] FP32); with mlp_w32/mlp_wb given it is
 * first overwritten with the learned preconditioner's scales
 * (jrg_precond_scale at step fraction t_frac, cap smax) computed inside the
 * step from this step's band kinetic energies.  num_spin 1 or 2 as
 * jrg_energy_grad; more than 32 bands only with the default contraction
 * kernels (jrg_tensor_core_paths 0).
 * With a non-zero status word (energies[6]) no update is applied: params, m
 * and v keep their values. */
typedef struct {
  int step;                 /* 1-based Adam step */
  double lr, b1, b2, eps;
  float* scale;             /* optional */
  const float* mlp_w32;     /* optional learned preconditioner (FP32 and BF16 copies) */
  const void* mlp_wb;
  float t_frac, smax;
} jrg_adam_step;

int jrg_energy_grad_adam(const jrg_plan* plan, void* params, void* m, void* v,
                         const double* occupation, const jrg_adam_step* opt, double* energies,
                         void* grad, void* workspace, cudaStream_t stream);

/* Re-orthonormalisation of raw parameters in place, the recovery for a
 * non-zero status word or a large condition estimate of jrg_energy_grad
 * (Cholesky QR, unlike the Householder QR of unitary_module.py:74-80 in the
 * reference, breaks down on rank-deficient or non-finite W): per (s,k), W
 * becomes Q diag(n) with Q an orthonormal basis of W's columns (Gram-Schmidt
 * with a second projection pass, FP64) and n the original column norms.
 * For a full-rank W the coefficients of the next jrg_energy_grad, and so the
 * energy, are unchanged; a non-finite or dependent column is replaced by a
 * fixed pseudo-random direction orthogonal to the previous ones.  Uses the
 * plan workspace as scratch. */
int jrg_reorthonormalise(const jrg_plan* plan, void* w_re, void* w_im, void* workspace,
                         cudaStream_t stream);

/* Effective potential from a density [S][nx][ny][nz]:
 * out [2+S][nx][ny][nz] real = Hartree, external, then the xc part per spin
 * (split form) with jrystal's conventions: kohn_sham=0 halves Hartree and
 * gives the xc energy density, kohn_sham=1 gives the full Hartree and v_xc.
 * S = 2 (LDA only): Hartree of the total density; the xc part is vxc_lda's
 * eps + rho_s d eps / d rho_s per spin (kohn_sham=1) or eps in both grids
 * (jrystal/_src/potential.py:203-279 broadcasts it over the spin axis). */
int jrg_potential(const jrg_plan* plan, const void* density, int kohn_sham, void* out,
                  void* workspace, cudaStream_t stream);

/* Elementwise LDA on n real densities: the energy per particle eps_xc
 * (kohn_sham = 0) or the potential v_xc = d(rho eps_xc)/d rho (kohn_sham =
 * 1), summed over the JRG_XC_* terms; jrystal/_src/xc.py:54-64,109-124,222-253
 * (jax_xc lda_x and lda_c_vwn, unpolarised). */
int jrg_lda(int precision, int64_t n, int xc, int kohn_sham, const void* rho, void* out,
            cudaStream_t stream);

/* Spin-polarised LDA of a [2][n] density (up, down): eps_xc per particle of
 * the total density ([n], kohn_sham = 0), vxc_lda's per-spin field
 * eps_xc + rho_s d eps_xc / d rho_s ([2][n], kohn_sham = 1), or the
 * derivative of the energy density eps_xc (rho_up + rho_dn),
 * eps_xc + (rho_up + rho_dn) d eps_xc / d rho_s ([2][n], kohn_sham = 2: the
 * potential of jrg_energy_grad's polarised path).  Exchange by
 * jrystal's scaling (e_x(2 rho_up) + e_x(2 rho_dn)) / 2, correlation the VWN
 * spin interpolation of jax_xc's lda_c_vwn "pol" form;
 * jrystal/_src/xc.py:40-64,109-124. */
int jrg_lda_polarized(int precision, int64_t n, int xc, int kohn_sham, const void* rho, void* out,
                      cudaStream_t stream);

/* Batched complex 3-D FFT over the last three axes of [batch][nx][ny][nz].
 * direction -1: forward (unnormalised, jnp.fft.fftn); +1: inverse with the
 * 1/(nx ny nz) factor (jnp.fft.ifftn).  in and out may alias.  workspace
 * needs jrg_fft3d_workspace_size bytes. */
int jrg_fft3d_workspace_size(int precision, const int grid[3], int batch, size_t* bytes);
int jrg_fft3d(int precision, const int grid[3], int batch, int direction, const void* in,
              void* out, void* workspace, cudaStream_t stream);

/* jrg_fft3d without a workspace, for callers that cannot allocate device
 * memory (a runtime that owns the device memory, a fixed memory budget, or a
 * path that must avoid cudaMalloc's implicit synchronisation).  No
 * counterpart in the reference.  Scratch is a fixed 16 MiB device array
 * inside the library, held on every GPU that loads it until exit: the
 * twiddle tables (256-byte rounded) plus batch*nx*ny*nz complex elements
 * must fit, else JRG_ERR_INVALID.  All calls share that array, so calls that
 * overlap on the GPU race; nothing in it needs to start at zero.  The first
 * call on a device looks up the array's address (cudaGetSymbolAddress) and
 * should come before any stream capture; the address is kept with the
 * device's context and looked up again after that context is replaced
 * (cudaDeviceReset).  in and out may alias. */
int jrg_fft3d_noalloc(int precision, const int grid[3], int batch, int direction,
                      const void* in, void* out, cudaStream_t stream);

/* One Adam step over n elements (optax.adam: eps outside the sqrt after bias
 * correction).  step is the 1-based count after this update.  scale, when not
 * NULL, multiplies each update element (learned preconditioner). */
int jrg_adam_update(int precision, int64_t n, void* param, const void* grad, void* m, void* v,
                    const float* scale, int step, double lr, double b1, double b2, double eps,
                    cudaStream_t stream);

/* Ewald nuclear repulsion (FP64), the jrystal formula with the translation
 * grid of grid.translation_vectors(cell, cutoff) and the reciprocal sum over
 * the plan's FFT G grid.  result: device double[1]. */
int jrg_ewald(const jrg_plan* plan, double eta, double cutoff, double* result,
              void* workspace, cudaStream_t stream);

/* Learned diagonal preconditioner (no counterpart in the reference): an MLP
 * 3-64-64-64-1 (GELU, softplus) of x1 = |G+k|^2/E_kin,band, x2 = band/B,
 * x3 = step fraction, scaling each Adam update element.  Parameters: FP32
 * master copy (w32) and BF16 copy (wb) of jrg_mlp_num_params() values in the
 * order W1[64][3] b1 W2[64][64] b2 W3[64][64] b3 W4[64] b4.
 * jrg_precond_scale writes scale[2][S][K][G][B] (the same scale for w_re and
 * w_im of a coefficient, 1 for unoccupied bands, capped at smax) from the
 * per-band kinetic energies of the last jrg_energy_grad on this workspace.
 * jrg_mlp_train_eval runs the BF16/FP32 training forward over n records
 * x[n][3] -> s[n] and, given the one-step model terms a[n], c[n] (weights wt
 * optional), the summed loss sum wt (s a + s^2 c/2) and the gradient of its
 * mean with respect to the FP32 parameters. */
int jrg_mlp_num_params(void);
int jrg_mlp_to_bf16(const float* w32, void* wb, cudaStream_t stream);
int jrg_mlp_workspace_size(int n, size_t* bytes);
int jrg_mlp_train_eval(int n, const float* x, const float* w32, const void* wb, const float* a,
                       const float* c, const float* wt, float* s_out, double* loss, float* grad,
                       void* workspace, cudaStream_t stream);
int jrg_precond_scale(const jrg_plan* plan, const float* w32, const void* wb, float t_frac,
                      float smax, const double* occupation, float* scale, void* workspace,
                      cudaStream_t stream);
/* Per-band kinetic energies sum_G |G+k|^2/2 |c|^2 of the last jrg_energy_grad
 * (device double[S*K*B]) and the plan's |G+k|^2/2 table (double[K*G]). */
int jrg_band_kinetic(const jrg_plan* plan, const void* workspace, double* out, cudaStream_t stream);
int jrg_kinetic_table(const jrg_plan* plan, double* out, cudaStream_t stream);

/* Selects the specialised kernels (enable = 1, the default): register-
 * resident slab FFTs for cubic grids N^3 with N in {16, 24, 27, 32, 36, 48,
 * 64, 96} and register-blocked Gram contractions for num_band <= 32; or the
 * generic ones (enable = 0): shared-memory Stockham FFTs for every grid and
 * 32x32-tiled Gram contractions.  enable < 0 only queries.  Returns the
 * previous setting.  Process-wide; no reference counterpart. */
int jrg_fast_paths(int enable);

/* Selects the contraction kernels (Gram and rotations):
 * 0 = CUDA cores (the default: the only mode whose FP32 energies stay within
 * 1e-6 Ha/atom of the FP64 path at the 24-band Si8 cell; thread-per-G
 * rotations), 1 = mma.sync TF32 Gram and rotation with a three-product hi/lo
 * split (FP32 path, num_band <= 32), 2 = tcgen05 (5th-generation tensor
 * cores, tensor-memory accumulators) TF32 x 3 Gram with CUDA-core rotation
 * (FP32 path, num_band <= 32), 3 = CUDA cores with the register-blocked
 * shared-memory rotations of earlier versions; enable < 0 only queries.
 * Returns the previous setting.  Process-wide; no reference counterpart. */
int jrg_tensor_core_paths(int enable);

/* Two-way k-point pipeline of jrg_energy_grad (enable = 1, the default):
 * with at least two (s,k) blocks, the default contraction
 * and slab kernels and no phase profiling, the blocks are split in two
 * halves that run on the caller's stream and a second stream owned by the
 * plan (joined back before the call returns, in stream order), so that the
 * latency-bound small kernels of one half overlap the other half's
 * bandwidth-bound kernels.  enable = 0 runs everything on the caller's
 * stream; < 0 only queries.  Returns the previous setting.  Process-wide; no
 * reference counterpart. */
int jrg_pipeline(int enable);

/* Per-phase CUDA-event timing of jrg_energy_grad (no reference counterpart;
 * the reference only times whole steps, calc driver :207-211).  enable
 * creates events for up to max_calls calls (0 disables); read synchronises
 * on the recorded events and returns, per phase, the summed milliseconds and
 * the number of recorded calls; phase_name gives a phase's name. */
int jrg_profile_enable(jrg_plan* plan, int max_calls);
int jrg_profile_read(jrg_plan* plan, double* ms, int* calls, int num_phases);
const char* jrg_profile_phase_name(int phase);
int jrg_profile_num_phases(void);

/* Batched trajectory generation (no counterpart as one call: jrystal runs one
 * cell per driver loop, calc/calc_ground_state_energy_all_electrons.py:205-220,
 * each step being value_and_grad + optax.adam, :175-190).  A batch runs plain
 * Adam (jrg_energy_grad, then the jrg_adam_update rule) on many independent
 * cells at once -- any grids, k-sets and band counts, one plan each -- every
 * cell on its own stream branch forked from and joined back to the caller's
 * stream; with use_graph the fan-out of one step is captured into a CUDA
 * graph on the first such call and replayed after that, one graph launch per
 * step of every cell.  Each cell's trajectory equals the same steps taken one
 * cell at a time (energy and gradient, then Adam with no update on a non-zero
 * status word).  The step count lives on the device; a batch takes exactly
 * `steps` jrg_batch_step calls.  Records (per_step > 0): at every step t <
 * steps - 1, per_step occupied coefficients are drawn per cell (counter-based
 * hash of seed, cell, t, draw) and row t holds x = (|G+k|^2/2 / E_kin(band),
 * band/B, t/steps), a = g_t . u_t, c = max((g_{t+1} - g_t) . u_t, c_floor |a|)
 * (u_t the applied update of those elements, real and imaginary parts) and
 * w = (number of non-zero a) / sum |a| over the row -- the one-step secant
 * records of the learned preconditioner's training set.  Creation allocates
 * the batch's device state and streams and synchronises; steps only enqueue
 * (the first graph step also captures and instantiates).  The plans,
 * workspaces and buffers belong to the batch until it is destroyed. */
typedef struct jrg_batch jrg_batch;
typedef struct {
  int num_cells;
  jrg_plan* const* plans;            /* host array [num_cells]; num_spin 1 */
  void* const* workspaces;           /* device pointers, jrg_workspace_size bytes each */
  void* const* params;               /* [2][S][K][G][B] each, updated in place */
  void* const* m;                    /* Adam moments, zero before the first step */
  void* const* v;
  void* const* grads;                /* [2][S][K][G][B]: the last step's gradient */
  const double* const* occupations;  /* device [S*K*B] each */
  int steps;                         /* horizon */
  double lr, b1, b2, eps;
  double* energies;                  /* optional device [steps][num_cells][8] (as jrg_energy_grad) */
  int per_step;                      /* records per step and cell (0: none) */
  unsigned long long seed;
  double c_floor;
  float* rec_x;                      /* device [num_cells][steps-1][per_step][3] */
  float* rec_a;                      /* device [num_cells][steps-1][per_step] */
  float* rec_c;
  float* rec_w;
  int64_t* rec_idx;                  /* optional: flat element index of each draw in [S][K][G][B] */
} jrg_batch_desc;

int jrg_batch_create(const jrg_batch_desc* desc, jrg_batch** out);
int jrg_batch_step(jrg_batch* batch, int use_graph, cudaStream_t stream);
int jrg_batch_steps_done(const jrg_batch* batch, int* steps);
int jrg_batch_destroy(jrg_batch* batch);

#ifdef __cplusplus
}
#endif
#endif /* JRYSTAL_GB300_H_ */
