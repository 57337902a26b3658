// mixed.cu -- the FP32-mixed fused step.  Built with fast FP32 division and square root
// (-prec-div=false -prec-sqrt=false -ftz=true): those only touch the FP32 reconstruction and Riemann
// solve; the FP64 state update and pressure recovery are unaffected, and the compensated sums use
// explicitly rounded intrinsics.
#define MHDGB_FAST 1
#define MHDGB_VNS v_mixed
#include "fused.cuh"
#include "fused_fs.cuh"
#include "kernels.h"

namespace mhdgb {
namespace detail {

int variants_mixed(const FusedVariant** out) {
  static const FusedVariant v[] = {
      v_mixed::FusedLauncher<float, 32, 4, 128>::variant(FUSED_MIXED),
      v_mixed::FusedLauncher<float, 32, 8, 256>::variant(FUSED_MIXED),
      v_mixed::FusedLauncher<float, 16, 8, 128>::variant(FUSED_MIXED),
      v_mixed::FusedLauncher<float, 64, 4, 256>::variant(FUSED_MIXED),
      v_mixed::FusedLauncher<float, 32, 4, 256, 2>::variant(FUSED_MIXED),
      v_mixed::FusedLauncher<float, 16, 8, 256, 2>::variant(FUSED_MIXED),
      preferred_variant(v_mixed::FusedLauncherFS<16, 8, 256, 2>::variant(FUSED_MIXED)),
      // the run-time solver kernel (HLLE / HLLC); not one of the tuned variants
      v_mixed::FusedLauncherFS<16, 8, 256, 2, true>::variant(FUSED_MIXED),
  };
  *out = v;
  return (int)(sizeof(v) / sizeof(v[0])) - 1;  // the last entry is the run-time solver kernel
}

cudaError_t recover_mixed(const FusedArgs& a, int which, RedSlot* slot, int nsm, cudaStream_t s, const double* uh_in,
                          double* uh_ghost_out) {
  return v_mixed::recover_launch<float>(a, which, slot, nsm, s, uh_in, uh_ghost_out);
}

}  // namespace detail
}  // namespace mhdgb
