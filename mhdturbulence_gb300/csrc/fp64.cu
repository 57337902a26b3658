// fp64.cu -- the FP64 fused step with FMA contraction (last-bit differences from the reference's
// separately rounded arithmetic), in the tile shapes the autotuner chooses from.
#define MHDGB_FAST 1
#define MHDGB_VNS v_fast64
#include "fused.cuh"
#include "kernels.h"

namespace mhdgb {
namespace {

// The FP64 division, square root and reciprocal square root of the fast build against IEEE
// division and square root on log-uniform operands (both signs for the division) over
// [2^-60, 2^60]: the largest distance in units in the last place.
__global__ void k_fdiv_selftest(int n, unsigned long long seed, unsigned long long* max_ulp) {
  unsigned long long worst = 0;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    unsigned long long z = seed + 0x9E3779B97F4A7C15ull * (unsigned long long)(t + 1);
    auto next = [&]() {
      z ^= z >> 30; z *= 0xBF58476D1CE4E5B9ull; z ^= z >> 27; z *= 0x94D049BB133111EBull; z ^= z >> 31;
      return z;
    };
    const double ua = (double)(next() >> 11) * 0x1.0p-53, ub = (double)(next() >> 11) * 0x1.0p-53;
    const unsigned long long sg = next();
    const double a = ldexp(1.0 + ua, (int)(next() % 121) - 60) * ((sg & 1) ? -1.0 : 1.0);
    const double b = ldexp(1.0 + ub, (int)(next() % 121) - 60) * ((sg & 2) ? -1.0 : 1.0);
    const double q = v_fast64::fdiv(a, b), r = a / b;
    const long long d = (long long)__double_as_longlong(q) - (long long)__double_as_longlong(r);
    const unsigned long long ad = (unsigned long long)(d < 0 ? -d : d);
    if (ad > worst) worst = ad;
    // the square root of the fast form (and the reciprocal square root it also yields)
    const double x = fabs(a);
    double ix = 0.0;
    const double sq = v_fast64::sqrt_goldschmidt(x, &ix), sr = sqrt(x), ir = 1.0 / sr;
    const long long ds = (long long)__double_as_longlong(sq) - (long long)__double_as_longlong(sr);
    const long long di = (long long)__double_as_longlong(ix) - (long long)__double_as_longlong(ir);
    const unsigned long long ads = (unsigned long long)(ds < 0 ? -ds : ds);
    const unsigned long long adi = (unsigned long long)(di < 0 ? -di : di);
    if (ads > worst) worst = ads;
    if (adi > worst) worst = adi;
  }
  atomicMax(max_ulp, worst);
}

}  // namespace

namespace detail {

cudaError_t fdiv_selftest(int n, unsigned long long seed, unsigned long long* d_max_ulp, cudaStream_t s) {
  k_fdiv_selftest<<<304, 256, 0, s>>>(n, seed, d_max_ulp);
  return cudaGetLastError();
}

int variants_fp64(const FusedVariant** out) {
  static const FusedVariant v[] = {
      v_fast64::FusedLauncher<double, 32, 4, 128>::variant(FUSED_FP64),
      v_fast64::FusedLauncher<double, 28, 4, 128>::variant(FUSED_FP64),
      v_fast64::FusedLauncher<double, 16, 8, 128>::variant(FUSED_FP64),
      v_fast64::FusedLauncher<double, 32, 4, 256>::variant(FUSED_FP64),
      preferred_variant(v_fast64::FusedLauncher<double, 16, 8, 256>::variant(FUSED_FP64)),
      // the run-time solver kernel (HLLE / HLLC); not one of the tuned variants
      v_fast64::FusedLauncher<double, 16, 8, 256, 1, true>::variant(FUSED_FP64),
  };
  *out = v;
  return (int)(sizeof(v) / sizeof(v[0])) - 1;  // the last entry is the run-time solver kernel
}

cudaError_t recover_fp64(const FusedArgs& a, int which, RedSlot* slot, int nsm, cudaStream_t s, const double* uh_in,
                         double* uh_ghost_out) {
  return v_fast64::recover_launch<double>(a, which, slot, nsm, s, uh_in, uh_ghost_out);
}

}  // namespace detail
}  // namespace mhdgb
