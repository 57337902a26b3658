// fp64.cu -- the FP64 fused step with FMA contraction (last-bit differences from the reference's
// separately rounded arithmetic), in the tile shapes the autotuner chooses from.
#define MHDGB_VNS v_fast64
#include "fused.cuh"
#include "kernels.h"

namespace mhdgb {
namespace detail {

int variants_fp64(const FusedVariant** out) {
  static const FusedVariant v[] = {
      v_fast64::FusedLauncher<double, 32, 4, 128>::variant(FUSED_FP64),
      v_fast64::FusedLauncher<double, 28, 4, 128>::variant(FUSED_FP64),
      v_fast64::FusedLauncher<double, 16, 8, 128>::variant(FUSED_FP64),
  };
  *out = v;
  return (int)(sizeof(v) / sizeof(v[0]));
}

cudaError_t recover_fp64(const FusedArgs& a, int which, RedSlot* slot, int nsm, cudaStream_t s) {
  return v_fast64::recover_launch<double>(a, which, slot, nsm, s);
}

}  // namespace detail
}  // namespace mhdgb
