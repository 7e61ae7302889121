// Partial Gram S = X^H Y of the FP32 path on the 5th-generation tensor cores
// (tcgen05.mma, accumulator in tensor memory), num_band <= 32.
//
// Real embedding.  With x_i the interleaved (re, im) row of band i over a
// chunk of G vectors and x'_i = (im, -re), one real product
//   D = A B^T,  A = [x_0 .. x_{nb-1}, x'_0 .. x'_{nb-1}] (2nb rows),  B = [y_0 .. y_{nb-1}]
// gives Re S_ij = D_ij and Im S_ij = -D_{nb+i, j}.  The MMA shape is
// M = 128, N = 32, K = 8 (kind::tf32): rows 2nb..127 of A and columns nb..31
// of B are never stored and their products are never read.  Each FP32
// operand is split into TF32 hi and lo parts (cvt.rna), and the three MMAs
// lo*hi + hi*lo + hi*hi keep FP32 accuracy.
//
// Warp-specialised pipeline of one CTA (one (s,k), one G range, 512
// threads), coordinated by mbarriers only:
//   producers (warps 1-3, 6-15): stream chunks of 32 G vectors of X and Y into
//     a ring of raw shared-memory buffers with cp.async four chunks ahead
//     (named barrier 1 among the producers only), split each chunk into TF32
//     hi/lo parts in the no-swizzle K-major core-matrix layout of one of the
//     MMA stages, and arrive (one lane per warp) on the stage's "full" barrier;
//   MMA issuer (warp 0, one lane): waits "full", issues the chunk's 24 MMAs
//     into one of two 32-column tensor-memory accumulators and commits them
//     to the stage's "empty" barrier and the accumulator's "ready" barrier;
//   epilogue (warps 4-5, tensor-memory lanes 0-63): waits "ready", adds the
//     2nb accumulator rows (tcgen05.ld) into Kahan-compensated FP32 sums and
//     arrives on the accumulator's "free" barrier.
// Plain FP32 sums in tensor memory run over kFlush chunks (128 real terms x
// 3 products); across those groups the compensated sums keep the error at the
// level of the CUDA-core Gram's FP64 reduction.  Every wait is bounded: on a timeout
// the waiting thread sets bit 2 of the workspace flag word and a shared
// abort flag that ends every role's loop; the CTA then waits (bounded) for
// its issued MMAs, frees its tensor memory and returns.
#include <algorithm>
#include "plan.h"

namespace jrg {
namespace tc5 {

constexpr int kLaySplit = 0;             // parameters: re and im arrays [S][K][G][B]
constexpr int kLayBand = 1;              // band-major complex [S*K*B][G]

constexpr int kThreads = 512;
constexpr int kKC = 64;                  // K floats per chunk (32 complex G vectors)
constexpr int kGC = kKC / 2;             // G vectors per chunk
static_assert(kGC == 32, "the producer index arithmetic assumes 32 G vectors per chunk");
constexpr int kNKC = kKC / 4;            // core-matrix columns (16 bytes) per chunk
constexpr int kCore = 128;               // bytes per core matrix: 8 rows x 16 bytes
constexpr int kLBO = kCore;              // K-adjacent core matrices
constexpr int kSBO = kNKC * kCore;       // 8-row groups (2048 bytes)
constexpr int kM = 128, kN = 32;
// kind::tf32 instruction descriptor: F32 accumulator, TF32 A and B, both
// K-major, N >> 3 at bit 17, M >> 4 at bit 24
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(kN >> 3) << 17) |
                            ((uint32_t)(kM >> 4) << 24);
constexpr long kWaitLimit = 1L << 22;

constexpr int kMaxStages = 3;
constexpr int kNProd = 416;              // producer threads (warps 1-3 and 6-15)
constexpr int kRawDepth = 4;             // raw chunks in flight per CTA
constexpr int kRawPitch = kGC + 1;       // complex elements per raw row (padded)
constexpr int kFlush = 2;                // chunks accumulated per tensor-memory buffer

struct Layout {
  int ga, gb;                      // 8-row groups holding A (2nb rows) and B (nb rows)
  int a_hi, a_lo, b_hi, b_lo;      // part offsets inside a stage
  int stages;                      // MMA stages (3, or 2 when 3 do not fit)
  int stage;                       // bytes per MMA stage
  int raw, raw_stage;              // raw chunk ring
  int bars;                        // mbarriers: full[3], empty[3], ready[2], free[2]
  int total;
};

__host__ __device__ inline Layout layout_for(int nb) {
  Layout L;
  L.ga = (2 * nb + 7) / 8;
  L.gb = (nb + 7) / 8;
  L.a_hi = 0;
  L.a_lo = L.ga * kSBO;
  L.b_hi = 2 * L.ga * kSBO;
  L.b_lo = (2 * L.ga + L.gb) * kSBO;
  L.stage = 2 * (L.ga + L.gb) * kSBO;
  L.raw_stage = 2 * nb * kRawPitch * 8;
  L.stages = kMaxStages;
  for (;;) {
    // an MMA reads 16 row groups of A (4 of B) from a part's start: the span
    // past the last stage stays inside the allocation (pad before the raw ring)
    L.raw = L.stages * L.stage + 16 * kSBO;
    L.bars = L.raw + kRawDepth * L.raw_stage;
    L.total = L.bars + 192;
    if (L.total <= 227 * 1024 || L.stages == 2) break;
    --L.stages;
  }
  return L;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// shared-memory matrix descriptor: no swizzle, start >> 4, LBO >> 4, SBO >> 4,
// descriptor version 1 (bits 46-47)
__device__ __forceinline__ uint64_t mdesc(uint32_t addr) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)(kLBO >> 4) << 16) |
         ((uint64_t)(kSBO >> 4) << 32) | (1ull << 46);
}

// cp.async of BYTES bytes, or BYTES zero bytes when !valid (source size 0)
template <int BYTES>
__device__ __forceinline__ void cp_async_zfill(void* smem, const void* gmem, bool valid) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;" ::"r"(sa), "l"(gmem), "n"(BYTES),
               "r"(valid ? BYTES : 0)
               : "memory");
}

__device__ __forceinline__ uint32_t tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (long i = 0; i < kWaitLimit; ++i) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

__device__ __forceinline__ void mma(uint32_t tmem, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
      "l"(a), "l"(b), "r"(kIdesc), "r"(acc)
      : "memory");
}

// (hi, lo) TF32 parts of the pair (u, v) at (row, k), k even, of a part
__device__ __forceinline__ void put(unsigned char* hi, unsigned char* lo, int row, int k, float u,
                                    float v) {
  const int off = ((row >> 3) * kNKC + (k >> 2)) * kCore + (row & 7) * 16 + (k & 3) * 4;
  const uint32_t uh = tf32(u), vh = tf32(v);
  const uint32_t ul = tf32(u - __uint_as_float(uh)), vl = tf32(v - __uint_as_float(vh));
  *reinterpret_cast<uint2*>(hi + off) = make_uint2(uh, vh);
  *reinterpret_cast<uint2*>(lo + off) = make_uint2(ul, vl);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.shared::cta.b64 st, [%0];\n}\n" ::"r"(bar)
               : "memory");
}
__device__ __forceinline__ void commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
               : "memory");
}

template <int LAY>
__global__ void __launch_bounds__(kThreads, 1)
k_gram_tc5(const void* __restrict__ X0, const void* __restrict__ X1, const void* __restrict__ Y0,
           const void* __restrict__ Y1, double2* __restrict__ part, int ng, int nb, int split_len,
           int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  const Layout L = layout_for(nb);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int split = blockIdx.x, nsplit = gridDim.x;
  const size_t sk = blockIdx.z;
  const int g_begin = split * split_len;
  const int g_end = min(ng, g_begin + split_len);
  const int nchunk = g_end > g_begin ? (g_end - g_begin + kGC - 1) / kGC : 0;
  double2* out = part + (sk * nsplit + split) * (size_t)nb * nb;
  if (nchunk == 0) {
    for (int e = tid; e < nb * nb; e += kThreads) out[e] = make_double2(0.0, 0.0);
    return;
  }
  const uint32_t bar_base = smem_u32(sm + L.bars);
  auto full = [&](int s) { return bar_base + 8u * s; };
  const int S = L.stages;
  auto empty = [&](int s) { return bar_base + 8u * (kMaxStages + s); };
  auto ready = [&](int b) { return bar_base + 8u * (2 * kMaxStages + b); };
  auto freed = [&](int b) { return bar_base + 8u * (2 * kMaxStages + 2 + b); };
  volatile int* abort_flag = reinterpret_cast<volatile int*>(sm + L.bars + 160);
  int* issued = reinterpret_cast<int*>(sm + L.bars + 164);   // accumulator groups committed
  uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + L.bars + 168);
  if (tid == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(full(s), kNProd / 32);   // one arrival per producer warp
      mbar_init(empty(s), 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(ready(b), 1);
      mbar_init(freed(b), 2);            // one arrival per epilogue warp
    }

    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    *abort_flag = 0;
    *issued = 0;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 64;" ::"r"(
                     smem_u32(tslot))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;
  auto timed_out = [&]() {
    atomicOr(err, 2);
    *abort_flag = 1;
  };

  if (warp == 0) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      int open_grp = -1;   // group with MMAs issued but not yet committed to its ready barrier
      for (int c = 0; c < nchunk && !*abort_flag; ++c) {
        const int s = c % S, grp = c / kFlush, b = grp & 1;
        const bool first = (c % kFlush) == 0;
        const bool last = (c % kFlush) == kFlush - 1 || c == nchunk - 1;
        if (!mbar_wait(full(s), (c / S) & 1)) { timed_out(); break; }
        if (first && grp >= 2 && !mbar_wait(freed(b), ((grp - 2) >> 1) & 1)) { timed_out(); break; }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t base = smem_u32(sm + s * L.stage);
        const uint32_t d = tmem + (uint32_t)(b * 32);
#pragma unroll
        for (int k = 0; k < kKC / 8; ++k) {
          const uint32_t ko = k * 2 * kCore;
          const uint64_t ah = mdesc(base + L.a_hi + ko), al = mdesc(base + L.a_lo + ko);
          const uint64_t bh = mdesc(base + L.b_hi + ko), bl = mdesc(base + L.b_lo + ko);
          mma(d, al, bh, (first && k == 0) ? 0u : 1u);
          mma(d, ah, bl, 1u);
          mma(d, ah, bh, 1u);
        }
        commit(empty(s));
        open_grp = grp;
        if (last) {
          commit(ready(b));
          *issued = grp + 1;
          open_grp = -1;
        }
      }
      if (open_grp >= 0) {   // after an abort: track the open group's MMAs too
        commit(ready(open_grp & 1));
        *issued = open_grp + 1;
      }
    }
    __syncwarp();
  } else if (warp == 4 || warp == 5) {
    // ---------------- epilogue: accumulator rows 0..63, compensated sums ----------------
    float sum[32], comp[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) { sum[j] = 0.f; comp[j] = 0.f; }
    const int ngroup = (nchunk + kFlush - 1) / kFlush;
    for (int c = 0; c < ngroup; ++c) {
      const int b = c & 1;
      const bool ok = mbar_wait(ready(b), (c >> 1) & 1);
      if (!__all_sync(0xffffffffu, ok)) {   // warp-uniform exit before the warp-wide load
        if (lane == 0) timed_out();
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      uint32_t v[32];
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
          "%11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, "
          "%28, %29, %30, %31}, [%32];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
            "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]),
            "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]),
            "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]),
            "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]),
            "=r"(v[31])
          : "r"(tmem + ((uint32_t)((warp - 4) * 32) << 16) + (uint32_t)(b * 32))
          : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(freed(b));
#pragma unroll
      for (int j = 0; j < 32; ++j) {   // Kahan: sum - comp is the running total
        const float y = __uint_as_float(v[j]) - comp[j];
        const float t = sum[j] + y;
        comp[j] = (t - sum[j]) - y;
        sum[j] = t;
      }
    }
    const bool done = !*abort_flag;
    const int row = (warp - 4) * 32 + lane;
    if (row < nb) {
#pragma unroll
      for (int j = 0; j < 32; ++j)
        if (j < nb) out[row * nb + j].x = done ? (double)sum[j] - (double)comp[j] : 0.0;
    } else if (row < 2 * nb) {
#pragma unroll
      for (int j = 0; j < 32; ++j)
        if (j < nb) out[(row - nb) * nb + j].y = done ? (double)comp[j] - (double)sum[j] : 0.0;
    }
  } else {
    // ---------------- producers ----------------
    const int p = (warp < 4 ? warp - 1 : warp - 3) * 32 + lane;   // 0 .. kNProd-1
    auto prod_sync = [] { asm volatile("bar.sync 1, %0;" ::"n"(kNProd) : "memory"); };
    auto raw_x = [&](int q) { return reinterpret_cast<float2*>(sm + L.raw + q * L.raw_stage); };
    auto load_raw = [&](int c) {   // cp.async of chunk c into raw slot c % kRawDepth
      if (c < nchunk) {
        float2* xr = raw_x(c % kRawDepth);
        float2* yr = xr + nb * kRawPitch;
        const int g0 = g_begin + c * kGC;
        // element e: X then Y, 32 rows (bands, padded) x 32 G vectors; rows past
        // nb skipped, G vectors past the range zero-filled by the copy itself
        for (int e = p; e < 2 * 32 * kGC; e += kNProd) {
          const int which = e >> 10;
          const int rem = e & 1023;
          int r, gl;
          if (LAY == kLaySplit) { r = rem & 31; gl = rem >> 5; }   // consecutive bands: contiguous
          else { gl = rem & 31; r = rem >> 5; }                     // consecutive G: contiguous
          if (r >= nb) continue;
          const int g = g0 + gl;
          const bool in = g < g_end;
          float2* d = (which ? yr : xr) + r * kRawPitch + gl;
          if (LAY == kLaySplit) {
            const size_t o = in ? (sk * ng + g) * nb + r : 0;
            cp_async_zfill<4>(&d->x, reinterpret_cast<const float*>(which ? Y0 : X0) + o, in);
            cp_async_zfill<4>(&d->y, reinterpret_cast<const float*>(which ? Y1 : X1) + o, in);
          } else {
            const size_t o = in ? (sk * nb + r) * ng + g : 0;
            cp_async_zfill<8>(d, reinterpret_cast<const float2*>(which ? Y0 : X0) + o, in);
          }
        }
      }
      cp_async_commit();   // one group per chunk index, empty past the end
    };
    const int ncore = L.gb * kNKC * 16;    // (row, k pair) slots of an nb-row part
    for (int c = 0; c < kRawDepth - 1; ++c) load_raw(c);
    // Every producer runs all nchunk iterations and both named barriers of
    // each (an abort only skips the work), so the barriers always complete.
    for (int c = 0; c < nchunk; ++c) {
      const int s = c % S;
      prod_sync();                          // raw slot of chunk c - 1 has been converted
      load_raw(c + kRawDepth - 1);
      cp_async_wait<kRawDepth - 1>();
      prod_sync();                          // chunk c is in shared memory for every producer
      // warp-uniform decision: every lane polls, the warp acts together (the
      // per-warp arrival below needs all 32 lanes)
      const bool aborted = *abort_flag != 0;
      bool go = !aborted && (c < S || mbar_wait(empty(s), ((c / S) - 1) & 1));
      go = __all_sync(0xffffffffu, go);
      if (!go) {
        if (lane == 0 && !aborted) timed_out();
        continue;
      }
      const float2* xr = raw_x(c % kRawDepth);
      const float2* yr = xr + nb * kRawPitch;
      unsigned char* st = sm + s * L.stage;
      for (int e = p; e < ncore; e += kNProd) {
        const int cm = e >> 4, w = e & 15;
        const int rg = cm / kNKC, kc = cm - rg * kNKC;
        const int r = rg * 8 + (w >> 1), gl = 2 * kc + (w & 1);
        if (r < nb) {
          const float2 x = xr[r * kRawPitch + gl];
          const float2 y = yr[r * kRawPitch + gl];
          put(st + L.a_hi, st + L.a_lo, r, 2 * gl, x.x, x.y);
          put(st + L.a_hi, st + L.a_lo, nb + r, 2 * gl, x.y, -x.x);
          put(st + L.b_hi, st + L.b_lo, r, 2 * gl, y.x, y.y);
        }
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(full(s));
    }
    cp_async_wait<0>();
  }
  __syncthreads();
  // every issued MMA has completed before the tensor memory is released
  if (tid == 0) {
    const int last = *issued - 1;
    if (last >= 0 && !mbar_wait(ready(last & 1), (last >> 1) & 1)) atomicOr(err, 2);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 64;" ::"r"(tmem) : "memory");
}

}  // namespace tc5

// Launches the partial Gram into part ([nsk][nsplit][nb][nb], FP64); returns
// the split count used (> 0), 0 when not applicable, or -error.  The caller
// reduces the splits.
int launch_gram_tc5(int lay, const void* X0, const void* X1, const void* Y0, const void* Y1,
                    double2* part, int nsk, int ng, int nb, int nsplit, int* err,
                    cudaStream_t st) {
  using namespace tc5;
  if (nb > 32 || nb < 1 || !err) return 0;
  // one CTA per SM (150-220 KB of shared memory): about four waves
  nsplit = std::max(1, std::min(nsplit, (4 * 152 + nsk - 1) / nsk));
  const int split_len = (ng + nsplit - 1) / nsplit;
  const size_t sm = layout_for(nb).total;
  auto go = [&](auto kern) -> int {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return -cuda_fail(e, "cudaFuncSetAttribute(gram_tc5)");
    kern<<<dim3(nsplit, 1, nsk), kThreads, sm, st>>>(X0, X1, Y0, Y1, part, ng, nb, split_len, err);
    count_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess) return -cuda_fail(e, "k_gram_tc5");
    return nsplit;
  };
  return lay == kLaySplit ? go(k_gram_tc5<kLaySplit>) : go(k_gram_tc5<kLayBand>);
}

}  // namespace jrg
