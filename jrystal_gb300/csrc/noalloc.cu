// jrg_fft3d_noalloc: the batched 3-D FFT of jrg_fft3d for callers that
// cannot allocate device memory.
//
// Some callers may not call cudaMalloc (or anything that allocates) when
// they need a transform: a runtime that embeds this library and owns the
// device memory (JAX/XLA preallocates most of the GPU and gives a custom
// call only the buffers it declared), a serving process that fixes its
// memory budget at start-up and forbids later allocations, or a
// latency-critical path that cannot afford the implicit device
// synchronisation a cudaMalloc/cudaFree pair may cause.  jrg_fft3d needs a
// caller workspace for its twiddle tables and its intermediate planes; this
// entry point uses a file-scope device array instead, so the caller passes
// only the input and output buffers.
//
// The array is kNoAllocScratchBytes (16 MiB) and lives on every GPU that
// loads this library until the process exits.  The twiddle tables (rounded
// up to 256 bytes) plus batch * nx * ny * nz complex elements must fit in it;
// larger requests are rejected with JRG_ERR_INVALID before any work is
// enqueued.  Every call shares the array: a call overwrites what the previous
// call left there (nothing in it has to start at zero -- the twiddles and
// every plane are written before they are read), and calls whose kernels
// overlap on the GPU (different streams, or different host threads on the
// same device) race on it.  Serialise them on one stream.
//
// Set-up: the first call on each device looks up the array's device address
// with cudaGetSymbolAddress while that device is current and caches it with
// the identity of the device's current context; a call that finds another
// context (the old one was destroyed, e.g. by cudaDeviceReset, and a new one
// created) looks the address up again.  Make the first call on a device
// before any stream capture begins.  in and out may alias.
#include <cuda.h>   // CUcontext / CUresult types of the two driver entry points below
#include <mutex>
#include "plan.h"

namespace jrg {

template <typename R>
int launch_fft3d_dense(const FftAxis*, const C_t<R>*, int, int, bool, const void*, C_t<R>*,
                       C_t<R>*, double, cudaStream_t);
int launch_twiddles(int n, int prec, void* out, cudaStream_t st);

constexpr size_t kNoAllocScratchBytes = (size_t)16 << 20;
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

static std::mutex g_noalloc_mu;
static void* g_noalloc_ptr[kNoAllocMaxDevices] = {};
static unsigned long long g_noalloc_ctx[kNoAllocMaxDevices] = {};   // context id of each cached address

// Unique id of the calling thread's current context (cuCtxGetId: ids are not
// reused within a process, unlike context handles), 0 when there is none or
// the driver does not provide the entry points.
static unsigned long long current_context_id() {
  typedef CUresult (*GetCurrent)(CUcontext*);
  typedef CUresult (*GetId)(CUcontext, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    cudaDriverEntryPointQueryResult q;
    void* f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<GetCurrent>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetId>(f);
  });
  if (!get_current || !get_id) return 0;
  CUcontext c = nullptr;
  if (get_current(&c) != CUDA_SUCCESS || !c) return 0;
  unsigned long long id = 0;
  return get_id(c, &id) == CUDA_SUCCESS ? id : 0;
}

// Device address of the scratch array on the current device: looked up once
// per device and context, and again when the device's context changed.
static int noalloc_scratch(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= kNoAllocMaxDevices)
    return fail(JRG_ERR_UNSUPPORTED, "jrg_fft3d_noalloc: device index beyond 63");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  const unsigned long long ctx = current_context_id();
  if (!g_noalloc_ptr[dev] || ctx == 0 || ctx != g_noalloc_ctx[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    g_noalloc_ptr[dev] = p;
    g_noalloc_ctx[dev] = current_context_id();   // the lookup made the context current if it was not
  }
  *out = g_noalloc_ptr[dev];
  return JRG_OK;
}

static size_t round256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace jrg

extern "C" int jrg_fft3d_noalloc(int prec, const int grid[3], int batch, int direction,
                                 const void* in, void* out, cudaStream_t st) {
  using namespace jrg;
  if (!grid || !in || !out || batch < 1 || (direction != 1 && direction != -1) ||
      (prec != 32 && prec != 64))
    return fail(JRG_ERR_INVALID, "jrg_fft3d_noalloc: bad argument");
  FftAxis ax[3];
  for (int a = 0; a < 3; ++a)
    if (grid[a] < 1 || !factor_axis(grid[a], &ax[a]))
      return fail(JRG_ERR_UNSUPPORTED, "jrg_fft3d_noalloc: grid size must be 7-smooth");
  const size_t c = prec == 64 ? 16 : 8;
  const size_t tw_bytes = round256(c * (size_t)(grid[0] + grid[1] + grid[2]));
  const size_t need = tw_bytes + c * (size_t)batch * grid[0] * grid[1] * grid[2];
  if (need > kNoAllocScratchBytes)
    return fail(JRG_ERR_INVALID,
                "jrg_fft3d_noalloc: batch x grid needs " + std::to_string(need) +
                    " bytes of scratch, above the fixed 16 MiB (16777216 bytes) array; "
                    "use jrg_fft3d with a workspace");
  int dev = 0, optin = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const size_t pb = c * (grid[1] + grid[2] + 2 * (size_t)grid[1] * grid[2]) + 4;
  const size_t lb = c * (grid[0] + 2 * (size_t)grid[0] * grid[2]);
  if ((long long)pb > optin || (long long)lb > optin)
    return fail(JRG_ERR_UNSUPPORTED, "jrg_fft3d_noalloc: grid too large for the slab kernels");
  void* base = nullptr;
  int rc = noalloc_scratch(&base);
  if (rc) return rc;
  char* tw = reinterpret_cast<char*>(base);
  char* scratch = tw + tw_bytes;
  int off = 0;
  for (int a = 0; a < 3; ++a) {
    if ((rc = launch_twiddles(grid[a], prec, tw + c * off, st))) return rc;
    off += grid[a];
  }
  const double scale = direction > 0 ? 1.0 / ((double)grid[0] * grid[1] * grid[2]) : 1.0;
  if (prec == 64)
    return launch_fft3d_dense<double>(ax, reinterpret_cast<const double2*>(tw), batch, direction,
                                      false, in, reinterpret_cast<double2*>(scratch),
                                      reinterpret_cast<double2*>(out), scale, st);
  return launch_fft3d_dense<float>(ax, reinterpret_cast<const float2*>(tw), batch, direction,
                                   false, in, reinterpret_cast<float2*>(scratch),
                                   reinterpret_cast<float2*>(out), scale, st);
}
