// kernels.h -- host-side launchers of the device kernels (implemented in stages.cu / fast.cu).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include "common.cuh"
#include "fused_args.h"

namespace mhdgb {

// ---- stage kernels (stages.cu, FP64, separately rounded) ----
cudaError_t launch_flux(int dir, const double* P, double* F, const Layout& L, const double* chg, int riemann,
                        cudaStream_t s);
cudaError_t launch_update_conserv(const double* Fx, const double* Fy, const double* Fz, double* U, const Layout& L,
                                  const double* xinv, const double* yinv, const double* zinv, int quirk,
                                  const double* dt, cudaStream_t s);
cudaError_t launch_damp_psi(double* U, const Layout& L, const double* dxs, const double* dys, const double* dzs,
                            const double* dt, const double* chg, cudaStream_t s);
cudaError_t launch_update_prim(const double* U, double* P, const Layout& L, double gam, cudaStream_t s);
cudaError_t launch_reduce_dt_ch(const double* P, const Layout& L, const double* dxs, const double* dys,
                                const double* dzs, RedSlot* slot, unsigned* status, int nsm, cudaStream_t s);
cudaError_t launch_reset_slot(RedSlot* slot, cudaStream_t s);
cudaError_t launch_slot_to_scalars(const RedSlot* slot, double cfl, double* dt, double* ch, cudaStream_t s);
size_t pack_buffer_doubles(const Layout& L);
cudaError_t launch_ghost_fill(double* P, const Layout& L, const int bc[6], double* scratch, cudaStream_t s);
// Output snapshot [NSNAP][nz][ny][nx] of P (if non-null) or of the primitives recovered from U.
constexpr int NSNAP = 10;
cudaError_t launch_snapshot(const double* U, const double* P, const Layout& L, double gam, double* out,
                            cudaStream_t s);

// ---- fused step ----
// Compiled tile shapes of each kind (stages.cu: bit-exact FP64; fp64.cu: FP64; mixed.cu: mixed):
// returns n, the number of HLLD tile variants out[0..n-1]; out[n] is the kind's run-time solver
// kernel (HLLD, HLLE or HLLC from the arguments).
int fused_variants(FusedKind kind, const FusedVariant** out);
// The tile variant a grid starts with before any autotuning: the table entry marked preferred (the
// fastest measured on GB300 at the benchmark sizes, 150^3 and 256^3).
int fused_preferred_variant(FusedKind kind);
// Recover P (FP64 for FP64 kinds, FP32 for mixed) + ghost images from a.U into a.P[which];
// reduce dt/c_h into slot.
cudaError_t launch_recover(FusedKind kind, const FusedArgs& a, int which, RedSlot* slot, int nsm, cudaStream_t s,
                           const double* uh_in = nullptr, double* uh_ghost_out = nullptr);

namespace detail {
int variants_exact(const FusedVariant** out);
int variants_fp64(const FusedVariant** out);
int variants_mixed(const FusedVariant** out);
cudaError_t recover_exact(const FusedArgs& a, int which, RedSlot* slot, int nsm, cudaStream_t s, const double* uh_in,
                          double* uh_ghost_out);
cudaError_t recover_fp64(const FusedArgs& a, int which, RedSlot* slot, int nsm, cudaStream_t s, const double* uh_in,
                          double* uh_ghost_out);
cudaError_t recover_mixed(const FusedArgs& a, int which, RedSlot* slot, int nsm, cudaStream_t s, const double* uh_in,
                          double* uh_ghost_out);
cudaError_t fdiv_selftest(int n, unsigned long long seed, unsigned long long* d_max_ulp, cudaStream_t s);
}  // namespace detail

}  // namespace mhdgb
