// fast.cu -- the fused step with FMA contraction: the FP64 form (last-bit differences from the
// reference's separately rounded arithmetic) and the FP32-mixed form.  Also the kind dispatch.
#define MHDGB_VNS v_fast
#include "fused.cuh"
#include "kernels.h"

namespace mhdgb {

using FastFP64 = v_fast::FusedLauncher<double, 32, 4>;
using FastMixed = v_fast::FusedLauncher<float, 32, 8>;

FusedShape fused_shape(FusedKind kind) {
  switch (kind) {
    case FUSED_FP64_EXACT: return detail::exact_shape();
    case FUSED_FP64: return FastFP64::shape();
    default: return FastMixed::shape();
  }
}

cudaError_t fused_prepare(FusedKind kind) {
  switch (kind) {
    case FUSED_FP64_EXACT: return detail::exact_prepare();
    case FUSED_FP64: return FastFP64::prepare();
    default: return FastMixed::prepare();
  }
}

int fused_ctas_per_sm(FusedKind kind) {
  switch (kind) {
    case FUSED_FP64_EXACT: return detail::exact_ctas_per_sm();
    case FUSED_FP64: return FastFP64::ctas_per_sm();
    default: return FastMixed::ctas_per_sm();
  }
}

cudaError_t launch_fused(FusedKind kind, const CUtensorMap maps[2], const FusedArgs& a, int grid, cudaStream_t s) {
  switch (kind) {
    case FUSED_FP64_EXACT: return detail::exact_launch(maps, a, grid, s);
    case FUSED_FP64: return FastFP64::launch(maps, a, grid, s);
    default: return FastMixed::launch(maps, a, grid, s);
  }
}

cudaError_t launch_recover(FusedKind kind, const double* U, void* P, const Layout& L, const int bc[6],
                           const double* dxs, const double* dys, const double* dzs, double gam, RedSlot* slot,
                           unsigned* status, int nsm, cudaStream_t s) {
  switch (kind) {
    case FUSED_FP64_EXACT: return detail::exact_recover(U, P, L, bc, dxs, dys, dzs, gam, slot, status, nsm, s);
    case FUSED_FP64: return v_fast::recover_launch<double>(U, P, L, bc, dxs, dys, dzs, gam, slot, status, nsm, s);
    default: return v_fast::recover_launch<float>(U, P, L, bc, dxs, dys, dzs, gam, slot, status, nsm, s);
  }
}

}  // namespace mhdgb
