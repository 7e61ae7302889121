// Dispatch into the register-resident slab kernels of k_fft_fast.cu.
#pragma once
#include "plan.h"

namespace jrg {
namespace fast {
enum Op { OP_PLANE_INV = 0, OP_LINE_DENSITY, OP_LINE_APPLY_V, OP_PLANE_FWD };
struct Args {
  const void* in;
  void* out;
  const void* aux;      // coefficients (plane fwd) or V(r) (apply_v)
  const double* w;
  double wscale;        // density weight scale, or the FFT scale of plane fwd
  int band0, nbands, bands_per_group;
  double* gscale;       // density: per band group, the FP64 factor of its partial
};
// 1: launched, 0: grid not covered (use the generic kernels), <0: -status
template <typename R> int dispatch(const jrg_plan* P, int op, const Args& a, cudaStream_t st);
// dense batched 3-D transform of cubic grids (same return convention)
template <typename R>
int dispatch_dense(const FftAxis* ax, const C_t<R>* tw, int batch, int dir, bool real_in,
                   const void* in, C_t<R>* scratch, C_t<R>* out, double scale, cudaStream_t st);
}  // namespace fast
}  // namespace jrg
