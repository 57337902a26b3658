// mhd_defs.cuh -- variable indices of the reference (src_cpp_kokkos_host/mhd.hpp:249-268) and
// its std::min / std::max semantics.
#pragma once

#include <cuda_runtime.h>

namespace mhdgb {

// primitive indices, src_cpp_kokkos_host/mhd.hpp:250-253
enum : int { nden = 0, nve1 = 1, nve2 = 2, nve3 = 3, nene = 4, npre = 5, ncsp = 6,
             nbm1 = 7, nbm2 = 8, nbm3 = 9, nbps = 10, nst = 11, NPRIM = 12 };
// conserved / flux-vector indices, src_cpp_kokkos_host/mhd.hpp:255-268
enum : int { mudn = 0, muvu = 1, muvv = 2, muvw = 3, muet = 4, mubu = 5, mubv = 6, mubw = 7,
             mubp = 8, must = 9, mfdn = 10, mfvu = 11, mfvv = 12, mfvw = 13, mfet = 14,
             mfbu = 15, mfbv = 16, mfbw = 17, mfbp = 18, mfst = 19, mcsp = 20, mvel = 21,
             mpre = 22, NVEC = 23 };
enum : int { mden = 0, mrv1 = 1, mrv2 = 2, mrv3 = 3, meto = 4, mbm1 = 5, mbm2 = 6, mbm3 = 7,
             mbps = 8, mst = 9, NCONS = 10 };
// rotated (normal, tangential-1, tangential-2) aliases of the momentum and field slots
enum : int { mrvu = 1, mrvv = 2, mrvw = 3, mbmu = 5, mbmv = 6, mbmw = 7 };

// Riemann solvers: HLLD (the C++ path's, mhd.cpp:97-417) and the Fortran variant's alternatives
// HLLE and HLLC (src_f90_acc_device/mhd.f90:877-1141); values as MHDGB_RIEMANN_* in mhdgb.h.
enum : int { RIEMANN_HLLD = 0, RIEMANN_HLLE = 1, RIEMANN_HLLC = 2 };

// std::min / std::max of the reference: min(a,b) = (b<a)?b:a, max(a,b) = (a<b)?b:a.
template <class R> __device__ __forceinline__ R smin(R a, R b) { return (b < a) ? b : a; }
template <class R> __device__ __forceinline__ R smax(R a, R b) { return (a < b) ? b : a; }

}  // namespace mhdgb
