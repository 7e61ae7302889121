// Batched trajectory generation: plain Adam on many independent cells at once.
//
// jrystal optimises one cell per driver loop
// (calc/calc_ground_state_energy_all_electrons.py:205-220); generating training
// data for the learned preconditioner needs hundreds of steps on dozens of
// small cells (grids 24^3-48^3, 8-16 bands), where one cell's step is a chain
// of small, latency-bound kernels that leave most of the 152 SMs idle.  A batch
// puts every cell's step on its own stream branch -- energy and gradient
// (jrg_energy_grad), the record kernel below, Adam -- forked from and joined
// back to the caller's stream, and captures that whole fan-out once into a
// CUDA graph, so one graph launch runs one step of every cell and the GPU
// overlaps the cells' kernels.  The step count lives on the device (the
// record kernel advances it and copies the step's Adam bias corrections from a
// table made on the host at creation), so the same graph replays every step.
//
// Records (optional) are the one-step secant records of the preconditioner's
// training set: at step t, per_step occupied coefficients are drawn (a
// counter-based splitmix64 hash of seed, cell, step and draw); the record of
// step t holds the features x = (|G+k|^2/2 / E_kin,band, band/B, t/steps), the
// gradient g_t and the parameters at those elements, and at step t+1 it is
// completed with a = g_t . u_t and c = max((g_{t+1} - g_t) . u_t,
// c_floor |a|) for the applied update u_t, and the weight w = (number of
// non-zero a) / sum |a| shared by the step's draws.  Steps 0..steps-2 give
// rows.
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "plan.h"

namespace jrg {

template <typename R>
int launch_adam(void*, const void*, void*, void*, const float*, long long, double, double, double, double,
                double, double, cudaStream_t, const int*, const double*);

struct BatchCell {
  const void* params;       // [2][n] in the cell's precision
  const void* grad;         // [2][n]
  long long n;              // S*K*G*B
  const double* tk;         // [K][G] |G+k|^2 / 2
  const double* ekin;       // [S*K*B] band kinetic energies of the step's energy call
  const double* occ;        // [S*K*B]
  const double* energies;   // [8] of the step's energy call
  int K, G, B, nskb;
  int cell, ncells, steps, per_step;
  unsigned long long seed;
  double c_floor;
  int* t;                   // device step counter
  long long* prev_idx;      // [per_step]
  double* prev_g;           // [2][per_step]
  double* prev_p;           // [2][per_step]
  const double* coef_tab;   // [steps][2] Adam bias corrections 1 - b^t, t = 1..steps
  double* coef_cur;         // [2] read by k_adam
  double* hist;             // [steps][ncells][8] or null
  float* rec_x;             // [steps-1][per_step][3] of this cell
  float* rec_a;             // [steps-1][per_step]
  float* rec_c;
  float* rec_w;
  int64_t* rec_idx;         // [steps-1][per_step] or null
};

__device__ __forceinline__ unsigned long long splitmix64(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

constexpr int kRecThreads = 128;

template <typename R>
__global__ void __launch_bounds__(kRecThreads) k_batch_record(BatchCell c) {
  __shared__ double sabs[kRecThreads];
  __shared__ int skeep[kRecThreads];
  const int t = *c.t;
  const int tid = threadIdx.x;
  if (t >= c.steps) return;   // the host refuses steps past the horizon
  const R* p = reinterpret_cast<const R*>(c.params);
  const R* g = reinterpret_cast<const R*>(c.grad);
  const int P = c.per_step;
  if (P > 0 && t >= 1) {
    // complete the row of step t-1: p now holds the parameters after its update
    const long long row = t - 1;
    double s = 0.0;
    int keep = 0;
    for (int j = tid; j < P; j += kRecThreads) {
      const long long i = c.prev_idx[j];
      const double ur = (double)p[i] - c.prev_p[j], ui = (double)p[c.n + i] - c.prev_p[P + j];
      const double gr = c.prev_g[j], gi = c.prev_g[P + j];
      const double a = gr * ur + gi * ui;
      double cc = ((double)g[i] - gr) * ur + ((double)g[c.n + i] - gi) * ui;
      cc = fmax(cc, c.c_floor * fabs(a));
      c.rec_a[row * P + j] = (float)a;
      c.rec_c[row * P + j] = (float)cc;
      s += fabs(a);
      keep += fabs(a) > 0.0 ? 1 : 0;
    }
    sabs[tid] = s;
    skeep[tid] = keep;
    __syncthreads();
    for (int o = kRecThreads / 2; o > 0; o >>= 1) {
      if (tid < o) { sabs[tid] += sabs[tid + o]; skeep[tid] += skeep[tid + o]; }
      __syncthreads();
    }
    const float w = sabs[0] > 0.0 ? (float)(skeep[0] / sabs[0]) : 0.0f;
    for (int j = tid; j < P; j += kRecThreads) c.rec_w[row * P + j] = w;
  }
  if (P > 0 && t <= c.steps - 2) {
    // draw the elements of this step's row among the occupied bands
    int nocc = 0;
    for (int q = 0; q < c.nskb; ++q) nocc += c.occ[q] > 0.0 ? 1 : 0;
    for (int j = tid; j < P; j += kRecThreads) {
      const unsigned long long key = splitmix64(splitmix64(splitmix64(c.seed + (unsigned long long)c.cell) + t) + j);
      int r = nocc > 0 ? (int)(splitmix64(key) % (unsigned long long)nocc) : 0;
      int band = 0;
      for (int q = 0; q < c.nskb; ++q)
        if (c.occ[q] > 0.0) { if (r == 0) { band = q; break; } --r; }
      const int gi = (int)(splitmix64(key ^ 0x5851F42D4C957F2Dull) % (unsigned long long)c.G);
      const int sk = band / c.B, b = band % c.B, k = sk % c.K;
      const long long i = ((long long)sk * c.G + gi) * c.B + b;
      const long long o = (long long)t * P + j;
      c.rec_x[3 * o + 0] = (float)(c.tk[(long long)k * c.G + gi] / c.ekin[band]);
      c.rec_x[3 * o + 1] = (float)b / (float)c.B;
      c.rec_x[3 * o + 2] = (float)t / (float)c.steps;
      if (c.rec_idx) c.rec_idx[o] = i;
      c.prev_idx[j] = i;
      c.prev_g[j] = (double)g[i];
      c.prev_g[P + j] = (double)g[c.n + i];
      c.prev_p[j] = (double)p[i];
      c.prev_p[P + j] = (double)p[c.n + i];
    }
  }
  if (c.hist && tid < 8) c.hist[((long long)t * c.ncells + c.cell) * 8 + tid] = c.energies[tid];
  if (tid == 0) {
    c.coef_cur[0] = c.coef_tab[2 * t];
    c.coef_cur[1] = c.coef_tab[2 * t + 1];
  }
  __syncthreads();   // every thread has read *c.t
  if (tid == 0) *c.t = t + 1;
}

}  // namespace jrg

using namespace jrg;

struct jrg_batch {
  int ncells = 0, steps = 0, per_step = 0, device = 0;
  double lr = 0, b1 = 0, b2 = 0, eps = 0;
  std::vector<const jrg_plan*> plans;
  std::vector<void*> ws, params, m, v, grad;
  std::vector<const double*> occ;
  std::vector<BatchCell> cells;
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> done;
  cudaEvent_t fork = nullptr;
  cudaStream_t cap = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  void* dev = nullptr;        // device state of every cell
  double* energies = nullptr; // [ncells][8] energies of each cell's current call
  int* counters = nullptr;    // [ncells] device step counters
  int issued = 0;             // steps enqueued so far
};

static void batch_free(jrg_batch* b) {
  if (!b) return;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  if (b->cap) cudaStreamDestroy(b->cap);
  for (auto s : b->streams) if (s) cudaStreamDestroy(s);
  for (auto e : b->done) if (e) cudaEventDestroy(e);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->dev) cudaFree(b->dev);
  delete b;
}

// One step of every cell, forked from and joined back to st.
static int batch_enqueue(jrg_batch* b, cudaStream_t st) {
  JRG_CUDA(cudaEventRecord(b->fork, st));
  for (int c = 0; c < b->ncells; ++c) {
    const jrg_plan* P = b->plans[c];
    cudaStream_t s = b->streams[c];
    const size_t half = (size_t)b->cells[c].n * (P->prec == 64 ? 8 : 4);
    char* pr = (char*)b->params[c];
    char* gr = (char*)b->grad[c];
    JRG_CUDA(cudaStreamWaitEvent(s, b->fork, 0));
    int rc = jrg_energy_grad(P, pr, pr + half, b->occ[c], b->energies + 8 * c, gr, gr + half, b->ws[c], s);
    if (rc) return rc;
    if (P->prec == 64) k_batch_record<double><<<1, kRecThreads, 0, s>>>(b->cells[c]);
    else k_batch_record<float><<<1, kRecThreads, 0, s>>>(b->cells[c]);
    JRG_LAUNCH_CHECK("k_batch_record");
    const int* guard = (const int*)((const char*)b->ws[c] + P->ws.flags);
    rc = P->prec == 64 ? launch_adam<double>(pr, gr, b->m[c], b->v[c], nullptr, 2 * b->cells[c].n, b->lr, b->b1,
                                             b->b2, 1.0, 1.0, b->eps, s, guard, b->cells[c].coef_cur)
                       : launch_adam<float>(pr, gr, b->m[c], b->v[c], nullptr, 2 * b->cells[c].n, b->lr, b->b1,
                                            b->b2, 1.0, 1.0, b->eps, s, guard, b->cells[c].coef_cur);
    if (rc) return rc;
    JRG_CUDA(cudaEventRecord(b->done[c], s));
    JRG_CUDA(cudaStreamWaitEvent(st, b->done[c], 0));
  }
  return JRG_OK;
}

extern "C" {

int jrg_batch_create(const jrg_batch_desc* d, jrg_batch** out) {
  if (!d || !out) return fail(JRG_ERR_INVALID, "jrg_batch_create: null argument");
  *out = nullptr;
  if (d->num_cells < 1 || !d->plans || !d->workspaces || !d->params || !d->m || !d->v || !d->grads ||
      !d->occupations)
    return fail(JRG_ERR_INVALID, "jrg_batch_create: num_cells < 1 or a null per-cell array");
  if (d->steps < 1 || d->per_step < 0 || !(d->lr > 0.0) || !(d->b1 >= 0.0 && d->b1 < 1.0) ||
      !(d->b2 >= 0.0 && d->b2 < 1.0) || !(d->eps >= 0.0))
    return fail(JRG_ERR_INVALID, "jrg_batch_create: bad steps, per_step or Adam hyper-parameters");
  if (d->per_step > 0 && (!d->rec_x || !d->rec_a || !d->rec_c || !d->rec_w))
    return fail(JRG_ERR_INVALID, "jrg_batch_create: records requested without record buffers");
  int dev = 0;
  JRG_CUDA(cudaGetDevice(&dev));
  for (int c = 0; c < d->num_cells; ++c) {
    const jrg_plan* P = d->plans[c];
    if (!P || !d->workspaces[c] || !d->params[c] || !d->m[c] || !d->v[c] || !d->grads[c] || !d->occupations[c])
      return fail(JRG_ERR_INVALID, "jrg_batch_create: null plan or buffer of cell " + std::to_string(c));
    if (P->ns != 1) return fail(JRG_ERR_UNSUPPORTED, "jrg_batch_create: spin-polarised cells are not implemented");
    if (P->device != dev)
      return fail(JRG_ERR_INVALID, "jrg_batch_create: cell " + std::to_string(c) + " lives on another device");
    if (P->prof && P->prof->max_calls > 0)
      return fail(JRG_ERR_INVALID, "jrg_batch_create: phase profiling is on for cell " + std::to_string(c));
  }
  jrg_batch* b = new jrg_batch();
  b->ncells = d->num_cells;
  b->steps = d->steps;
  b->per_step = d->per_step;
  b->device = dev;
  b->lr = d->lr; b->b1 = d->b1; b->b2 = d->b2; b->eps = d->eps;
  const int nc = b->ncells, P = b->per_step, T = b->steps;
  for (int c = 0; c < nc; ++c) {
    b->plans.push_back(d->plans[c]);
    b->ws.push_back(d->workspaces[c]);
    b->params.push_back(d->params[c]);
    b->m.push_back(d->m[c]);
    b->v.push_back(d->v[c]);
    b->grad.push_back(d->grads[c]);
    b->occ.push_back(d->occupations[c]);
  }
  // device state: coefficient table, per cell: counter, energies, coef_cur,
  // prev_idx, prev_g, prev_p
  std::vector<double> tab(2 * (size_t)T);
  for (int t = 0; t < T; ++t) {
    tab[2 * t] = 1.0 - std::pow(d->b1, t + 1);
    tab[2 * t + 1] = 1.0 - std::pow(d->b2, t + 1);
  }
  const size_t tab_bytes = tab.size() * sizeof(double);
  const size_t per_cell = 8 * sizeof(double) + 2 * sizeof(double) + (size_t)P * sizeof(long long) +
                          4 * (size_t)P * sizeof(double);
  const size_t total = tab_bytes + (size_t)nc * per_cell + (size_t)nc * sizeof(int) + 256;
  cudaError_t e = cudaMalloc(&b->dev, total);
  if (e == cudaSuccess) e = cudaMemset(b->dev, 0, total);
  if (e == cudaSuccess) e = cudaMemcpy(b->dev, tab.data(), tab_bytes, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) { batch_free(b); return cuda_fail(e, "jrg_batch_create: device state"); }
  char* base = (char*)b->dev + tab_bytes;
  b->energies = (double*)base;
  double* coef_cur = b->energies + 8 * (size_t)nc;
  long long* prev_idx = (long long*)(coef_cur + 2 * (size_t)nc);
  double* prev_g = (double*)(prev_idx + (size_t)nc * P);
  double* prev_p = prev_g + 2 * (size_t)nc * P;
  b->counters = (int*)(prev_p + 2 * (size_t)nc * P);
  const long long rows = (long long)(T - 1) * P;
  for (int c = 0; c < nc; ++c) {
    const jrg_plan* Pl = b->plans[c];
    BatchCell x{};
    x.params = b->params[c];
    x.grad = b->grad[c];
    x.n = (long long)Pl->ns * Pl->nk * Pl->ng * Pl->nb;
    x.tk = Pl->d.tk;
    x.ekin = (const double*)((const char*)b->ws[c] + Pl->ws.ekin);
    x.occ = b->occ[c];
    x.energies = b->energies + 8 * (size_t)c;
    x.K = Pl->nk; x.G = Pl->ng; x.B = Pl->nb; x.nskb = Pl->ns * Pl->nk * Pl->nb;
    x.cell = c; x.ncells = nc; x.steps = T; x.per_step = P;
    x.seed = d->seed;
    x.c_floor = d->c_floor;
    x.t = b->counters + c;
    x.prev_idx = prev_idx + (size_t)c * P;
    x.prev_g = prev_g + 2 * (size_t)c * P;
    x.prev_p = prev_p + 2 * (size_t)c * P;
    x.coef_tab = (const double*)b->dev;
    x.coef_cur = coef_cur + 2 * (size_t)c;
    x.hist = d->energies;
    if (P > 0) {
      x.rec_x = d->rec_x + 3 * rows * c;
      x.rec_a = d->rec_a + rows * c;
      x.rec_c = d->rec_c + rows * c;
      x.rec_w = d->rec_w + rows * c;
      x.rec_idx = d->rec_idx ? d->rec_idx + rows * c : nullptr;
    }
    b->cells.push_back(x);
  }
  b->streams.assign(nc, nullptr);
  b->done.assign(nc, nullptr);
  for (int c = 0; c < nc && e == cudaSuccess; ++c) {
    e = cudaStreamCreateWithFlags(&b->streams[c], cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->done[c], cudaEventDisableTiming);
  }
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) { batch_free(b); return cuda_fail(e, "jrg_batch_create: streams"); }
  *out = b;
  return JRG_OK;
}

int jrg_batch_step(jrg_batch* b, int use_graph, cudaStream_t st) {
  if (!b) return fail(JRG_ERR_INVALID, "jrg_batch_step: null batch");
  if (b->issued >= b->steps)
    return fail(JRG_ERR_INVALID, "jrg_batch_step: the batch's " + std::to_string(b->steps) + " steps are done");
  int dev = 0;
  JRG_CUDA(cudaGetDevice(&dev));
  if (dev != b->device) return fail(JRG_ERR_INVALID, "jrg_batch_step: called with another device current");
  if (!use_graph) {
    const int rc = batch_enqueue(b, st);
    if (rc == JRG_OK) ++b->issued;
    return rc;
  }
  if (!b->exec) {
    JRG_CUDA(cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal));
    const int rc = batch_enqueue(b, b->cap);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(b->cap, &g);
    if (rc) { if (g) cudaGraphDestroy(g); return rc; }
    if (e != cudaSuccess) { if (g) cudaGraphDestroy(g); return cuda_fail(e, "jrg_batch_step: capture"); }
    b->graph = g;
    JRG_CUDA(cudaGraphInstantiate(&b->exec, b->graph, 0));
  }
  JRG_CUDA(cudaGraphLaunch(b->exec, st));
  ++b->issued;
  return JRG_OK;
}

int jrg_batch_steps_done(const jrg_batch* b, int* steps) {
  if (!b || !steps) return fail(JRG_ERR_INVALID, "jrg_batch_steps_done: null argument");
  *steps = b->issued;
  return JRG_OK;
}

int jrg_batch_destroy(jrg_batch* b) {
  if (!b) return JRG_OK;
  cudaError_t e = cudaDeviceSynchronize();
  batch_free(b);
  return e == cudaSuccess ? JRG_OK : cuda_fail(e, "jrg_batch_destroy");
}

}  // extern "C"
