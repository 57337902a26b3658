// common.cuh -- device layout, the per-solver control block and the inline-PTX helpers (mbarrier,
// TMA tensor loads) shared by the solver kernels.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "mhd_defs.cuh"

namespace mhdgb {

constexpr int NGH = 2;  // ghost layers, src_cpp_kokkos_host/config.hpp:56

// Boundary kind of a face shared with a neighbouring block of a decomposed grid: its ghost layers
// are copied from the neighbour (the MPI branch of SendRecvBoundary, boundary.cpp:222-318), so no
// local fill writes them.  Kinds 1..3 are the reference's (config.hpp:29-31).
constexpr int BC_EXCHANGE = 4;

// Device arrays use the reference FieldArray layout (src_cpp_kokkos_host/mhd.hpp:237-238,
// View(n1,nv,n2,n3) LayoutLeft: i fastest, then variable, then j, then k) with the i extent
// padded from itot = nx+2*ngh+1 to a pitch `ip` that makes every row 64-byte aligned (TMA needs
// 16-byte strides).  Index space is the reference's: cell i of the interior is i + ngh.
struct Layout {
  int nx, ny, nz;     // interior cells
  int itot, jtot, ktot;
  int ip;             // padded i pitch (elements)
  __host__ __device__ size_t at(int nv, int n, int k, int j, int i) const {
    return (size_t)i + (size_t)ip * ((size_t)n + (size_t)nv * ((size_t)j + (size_t)jtot * (size_t)k));
  }
  __host__ __device__ size_t count(int nv) const { return (size_t)ip * nv * jtot * ktot; }
};

// Status bits of the device status word (checked by the host at synchronisation points).
enum : unsigned { ST_NONFINITE = 1u, ST_NEGATIVE = 2u, ST_TIMEOUT = 4u, ST_TMA = 8u };

// Reduction slot: min of the per-cell CFL time and max of the per-cell signal speed, kept as the
// bit patterns of non-negative doubles (which order like unsigned integers).
struct RedSlot {
  unsigned long long dtmin_bits;
  unsigned long long chmax_bits;
};

// Per-solver control block in device memory.  Fused steps read the current step's dt and c_h
// from slot[step % 3], reduce the next step's values into slot[(step+1) % 3] and reset
// slot[(step+2) % 3]; the last CTA to finish advances step and time.
struct Ctrl {
  RedSlot slot[3];
  unsigned long long step;   // fused steps completed
  double time;               // accumulated simulated time (time_sim)
  double tmax;               // stop when time > tmax (the reference's main.cpp:265 test)
  unsigned long long max_step;
  unsigned done;             // set once time > tmax or step >= max_step: later steps do nothing
  unsigned status;           // ST_* bits
  unsigned blocks_done;      // CTA completion counter of the running launch
  unsigned work_next;        // dynamic tile queue head of the running launch
  double last_dt, last_ch;   // dt and c_h used by the latest completed step
};

__host__ __device__ inline unsigned long long dbits(double x) {
#ifdef __CUDA_ARCH__
  return (unsigned long long)__double_as_longlong(x);
#else
  union { double d; unsigned long long u; } v; v.d = x; return v.u;
#endif
}
__host__ __device__ inline double bitsd(unsigned long long u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  union { double d; unsigned long long u; } v; v.u = u; return v.d;
#endif
}
constexpr unsigned long long DT_RESET = 0x7FEFFFFFFFFFFFFFull;  // DBL_MAX
constexpr unsigned long long CH_RESET = 0x0ull;                 // +0.0

// ---------------------------------------------------------------------------------------------
// FP32 <-> FP64 conversions on the integer pipe.  On GB300 the F2F conversion instructions issue
// on the FP64 pipe (about 2 per clock per SM), which the mixed form cannot afford per cell; these
// bit manipulations give the same values for the numbers the solver produces.
//   f2d_exact: exact widening of a finite float (zero and denormals become a signed zero).
//   d2f_rne:   narrowing with round-to-nearest-even; magnitudes below the smallest normal float
//              flush to a signed zero, magnitudes beyond the float range (and inf/NaN) become inf.
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ double f2d_exact(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned s = u & 0x80000000u, em = u & 0x7FFFFFFFu;
  unsigned hi = s | ((em >> 3) + (896u << 20));
  unsigned lo = em << 29;
  if (em < 0x00800000u) { hi = s; lo = 0u; }
  return __hiloint2double((int)hi, (int)lo);
}

__device__ __forceinline__ float d2f_rne(double d) {
  const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
  const unsigned s = hi & 0x80000000u, ahi = hi & 0x7FFFFFFFu;
  unsigned r = ((ahi - (896u << 20)) << 3) | (lo >> 29);
  const unsigned rem = lo & 0x1FFFFFFFu;
  r += (unsigned)(rem > 0x10000000u) | ((unsigned)(rem == 0x10000000u) & r);
  if (ahi < (897u << 20)) r = 0u;
  if (ahi >= (1151u << 20)) r = 0x7F800000u;
  return __uint_as_float(s | r);
}

// ---------------------------------------------------------------------------------------------
// Block reductions of (min dt, max ch) with a non-finite check, then one atomic per CTA.
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ void warp_minmax(double& mn, double& mx) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    double a = __shfl_xor_sync(0xffffffffu, mn, o);
    double b = __shfl_xor_sync(0xffffffffu, mx, o);
    mn = smin(mn, a);
    mx = smax(mx, b);
  }
}

// All threads of the block must call.  scratch: >= 2*32 doubles of shared memory.
__device__ __forceinline__ void block_reduce_to_slot(double mn, double mx, double* scratch, RedSlot* slot) {
  warp_minmax(mn, mx);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  if (lane == 0) { scratch[wid] = mn; scratch[32 + wid] = mx; }
  __syncthreads();
  if (wid == 0) {
    mn = (lane < nw) ? scratch[lane] : 1.0e308;
    mx = (lane < nw) ? scratch[32 + lane] : 0.0;
    warp_minmax(mn, mx);
    if (lane == 0) {
      atomicMin(&slot->dtmin_bits, dbits(mn));
      atomicMax(&slot->chmax_bits, dbits(mx));
    }
  }
  __syncthreads();
}

// Named CTA barrier `id` (1..15) of `nthreads` threads (whole warps): warps that only signal
// arrive without waiting, warps that need the others' shared-memory writes wait (bar.sync) until
// every participant has arrived; writes made before an arrive are visible after the wait.  Each
// participating warp must reach its arrive or its wait exactly once per use, in uniform control
// flow, and a use must complete before the next one begins.
__device__ __forceinline__ void named_bar_arrive(int id, int nthreads) {
  asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}
__device__ __forceinline__ void named_bar_sync(int id, int nthreads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// ---------------------------------------------------------------------------------------------
// mbarrier + TMA (cp.async.bulk.tensor) helpers.  Waits are bounded: on timeout the waiter sets
// ST_TIMEOUT in the status word and gives up instead of spinning forever.
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Every wait of a kernel on an mbarrier gives up after this long (or after kWaitMaxSpins polls,
// whichever comes first), so a copy that never lands ends in a status the host reads instead of a
// hung context.
constexpr uint64_t kWaitLimitNs = 2000000000ull;
constexpr unsigned kWaitMaxSpins = 1u << 26;

// Returns false (and flags ST_TIMEOUT) if the phase did not complete within the limit.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, unsigned* status) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = globaltimer_ns();
  for (unsigned it = 0; it < kWaitMaxSpins; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 63u) == 63u && globaltimer_ns() - t0 > kWaitLimitNs) break;
    if (it > 64) __nanosleep(32);
  }
  atomicOr(status, ST_TIMEOUT);
  return false;
}

// 4-D tiled TMA load of one box into shared memory, completing on `bar`.
__device__ __forceinline__ void tma_load_4d(void* smem_dst, const CUtensorMap* map, int c0, int c1, int c2,
                                            int c3, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_u32(smem_dst)),
      "l"((uint64_t)map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
      : "memory");
}

// Division by a run-time divisor d that stays fixed over many numerators: q / d as the high half
// of 2q * ceil(2^31 / d), exact whenever q * d < 2^31 (the work-list decode has q, d < 2^15).
struct FastDiv {
  unsigned d, m;
  __device__ __forceinline__ explicit FastDiv(int d_) : d((unsigned)d_), m((0x80000000u + (unsigned)d_ - 1u) / (unsigned)d_) {}
  __device__ __forceinline__ int div(int q) const { return (int)__umulhi((unsigned)q << 1, m); }
};

__device__ __forceinline__ void prefetch_l2(const void* p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}
__device__ __forceinline__ void prefetch_tensormap(const CUtensorMap* map) {
  asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)map) : "memory");
}

}  // namespace mhdgb
