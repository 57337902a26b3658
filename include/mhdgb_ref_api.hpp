// mhdgb_ref_api.hpp -- the reference's solver-stage interface, backed by libmhdgb.so.
//
// A program written against the reference's src_cpp_kokkos_device headers (mhd.hpp, boundary.hpp)
// includes this header instead, keeps its own config.hpp (config:: and resolution_mod::, see
// src_cpp_kokkos_host/config.hpp:10-69) and its main loop (main.cpp:228-267), and links
// libmhdgb.so.  Names, signatures and the meaning of the globals follow the reference:
//   hydflux_mod::  GridArray, FieldArray, G, U, P, Fx, Fy, Fz, gam, chg,
//                  AllocateHydroVariables, DeallocateHydroVariables, GetNumericalFluxD,
//                  UpdateConservU, UpdatePrimitvP, ControlTimestep, EvaluateCh, DampPsi
//                  (mhd.hpp:117-359 of src_cpp_kokkos_host, device variant src_cpp_kokkos_device/mhd.hpp)
//   boundary_mod:: BoundaryArray, Bs, Br, boundary_xin..boundary_zout, AllocateBoundaryVariables,
//                  DeallocateBoundaryVariables, SetBoundaryCondition (boundary.hpp:14-145)
//   Output         the snapshot writer of output.hpp:93 (as mhdgb_ref::Output, and as the global
//                  Output when MHDGB_REF_OUTPUT is defined, in place of output.cpp)
// The arrays live on the GPU.  As in the reference's device build, the host mirror of a FieldArray
// is refreshed with d2h() and sent with h2d() (mhd.hpp:310-315); stages run on the device copies.
// resolution_mod::dt and hydflux_mod::chg stay the source of truth: ControlTimestep and EvaluateCh
// set them, and the stages that use them read the current host values.
// The reference reports no errors; here a failing call prints the library's message and aborts.
#ifndef MHDGB_REF_API_HPP_
#define MHDGB_REF_API_HPP_

#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "config.hpp"
#include "mhdgb.h"

namespace mhdgb_ref {

inline mhdgb_solver*& handle() {
  static mhdgb_solver* h = nullptr;
  return h;
}

inline void check(int rc, const char* what) {
  if (rc != MHDGB_OK) {
    std::fprintf(stderr, "mhdgb: %s failed: %s (%s)\n", what, mhdgb_status_string(rc),
                 handle() ? mhdgb_last_error(handle()) : "no handle");
    std::abort();
  }
}

// Which device array a FieldArray stands for.
enum class Role { none, cons, prim, flux1, flux2, flux3 };

}  // namespace mhdgb_ref

namespace hydflux_mod {
using index_t = int;
using size_t = std::size_t;

inline constexpr int ncomp{1};
inline constexpr int nprim{11 + ncomp};
inline constexpr int nden{0}, nve1{1}, nve2{2}, nve3{3}, nene{4}, npre{5}, ncsp{6}, nbm1{7}, nbm2{8}, nbm3{9},
    nbps{10}, nst{nprim - ncomp}, ned{nprim - 1};
inline constexpr int mconsv{9 + ncomp}, madd{3};
inline constexpr int mden{0}, mrv1{1}, mrv2{2}, mrv3{3}, meto{4}, mbm1{5}, mbm2{6}, mbm3{7}, mbps{8},
    mrvu{1}, mrvv{2}, mrvw{3}, mbmu{5}, mbmv{6}, mbmw{7}, mst{mconsv - ncomp}, med{mconsv - 1};

// Cell faces (x?a) and centres (x?b) of the three axes, host side; h2d() hands the faces to the
// solver (GridArray, mhd.hpp:22-182).
template <class T>
class GridArray {
 public:
  int n3 = 0, n2 = 0, n1 = 0;
  GridArray() = default;
  void allocate(int n3_, int n2_, int n1_) {
    n3 = n3_; n2 = n2_; n1 = n1_;
    a1.assign(n1, T(0)); b1.assign(n1, T(0));
    a2.assign(n2, T(0)); b2.assign(n2, T(0));
    a3.assign(n3, T(0)); b3.assign(n3, T(0));
  }
  void deallocate() { a1.clear(); b1.clear(); a2.clear(); b2.clear(); a3.clear(); b3.clear(); }
  T& x1a(int i) { return a1[i]; }
  T& x1b(int i) { return b1[i]; }
  T& x2a(int j) { return a2[j]; }
  T& x2b(int j) { return b2[j]; }
  T& x3a(int k) { return a3[k]; }
  T& x3b(int k) { return b3[k]; }
  const T& x1a(int i) const { return a1[i]; }
  const T& x1b(int i) const { return b1[i]; }
  const T& x2a(int j) const { return a2[j]; }
  const T& x2b(int j) const { return b2[j]; }
  const T& x3a(int k) const { return a3[k]; }
  const T& x3b(int k) const { return b3[k]; }
  void h2d() { mhdgb_ref::check(mhdgb_set_grid(mhdgb_ref::handle(), a1.data(), a2.data(), a3.data()), "GridArray::h2d"); }

 private:
  std::vector<T> a1, b1, a2, b2, a3, b3;
};

// A field in the reference layout (i fastest, then variable, then j, then k; mhd.hpp:237-238) with a
// host mirror; the device copy belongs to the solver (FieldArray, mhd.hpp:186-316).
template <class T>
class FieldArray {
 public:
  T* data = nullptr;
  int nv = 0, n3 = 0, n2 = 0, n1 = 0;
  size_t size = 0;
  mhdgb_ref::Role role = mhdgb_ref::Role::none;
  FieldArray() = default;
  void allocate(int nv_, int n3_, int n2_, int n1_, const std::string& = "F") {
    nv = nv_; n3 = n3_; n2 = n2_; n1 = n1_;
    size = (size_t)nv * n3 * n2 * n1;
    host.assign(size, T(0));
    data = host.data();
  }
  void deallocate() { host.clear(); data = nullptr; size = 0; }
  T& operator()(int n, int k, int j, int i) { return data[i + (size_t)n1 * (n + (size_t)nv * (j + (size_t)n2 * k))]; }
  const T& operator()(int n, int k, int j, int i) const {
    return data[i + (size_t)n1 * (n + (size_t)nv * (j + (size_t)n2 * k))];
  }
  T& href(int n, int k, int j, int i) const {
    return const_cast<T*>(data)[i + (size_t)n1 * (n + (size_t)nv * (j + (size_t)n2 * k))];
  }
  void h2d() {
    using mhdgb_ref::Role;
    if (role == Role::cons) mhdgb_ref::check(mhdgb_upload_cons(mhdgb_ref::handle(), data), "U.h2d");
    else if (role == Role::prim) mhdgb_ref::check(mhdgb_upload_prim(mhdgb_ref::handle(), data), "P.h2d");
  }
  void d2h() {
    using mhdgb_ref::Role;
    mhdgb_solver* h = mhdgb_ref::handle();
    if (role == Role::cons) mhdgb_ref::check(mhdgb_download_cons(h, data), "U.d2h");
    else if (role == Role::prim) mhdgb_ref::check(mhdgb_download_prim(h, data), "P.d2h");
    else if (role == Role::flux1) mhdgb_ref::check(mhdgb_download_flux(h, 1, data), "Fx.d2h");
    else if (role == Role::flux2) mhdgb_ref::check(mhdgb_download_flux(h, 2, data), "Fy.d2h");
    else if (role == Role::flux3) mhdgb_ref::check(mhdgb_download_flux(h, 3, data), "Fz.d2h");
  }

 private:
  std::vector<T> host;
};

inline GridArray<double> G;
inline FieldArray<double> U, Fx, Fy, Fz, P;
inline double gam = 1.4;  // mhd.cpp:27
inline double chg = 0.0;

}  // namespace hydflux_mod

namespace boundary_mod {
inline constexpr int periodicb = config::periodicb;
inline constexpr int reflection = config::reflection;
inline constexpr int outflow = config::outflow;
inline int boundary_xin = config::boundary_xin, boundary_xout = config::boundary_xout;
inline int boundary_yin = config::boundary_yin, boundary_yout = config::boundary_yout;
inline int boundary_zin = config::boundary_zin, boundary_zout = config::boundary_zout;

// The solver fills ghost layers in place on the device; the send/receive buffers of the
// reference's MPI exchange have no counterpart on one GPU (BoundaryArray, boundary.hpp:26-135).
template <class T>
class BoundaryArray {
 public:
  void allocate(int, int, int, int, int) {}
  void deallocate() {}
};
inline BoundaryArray<double> Bs, Br;
}  // namespace boundary_mod

namespace mhdgb_ref {
// Push the host globals the stages depend on (gam, boundary types, dt, chg) to the solver.
inline void sync_globals(bool dt_chg) {
  const int bc[6] = {boundary_mod::boundary_xin, boundary_mod::boundary_xout, boundary_mod::boundary_yin,
                     boundary_mod::boundary_yout, boundary_mod::boundary_zin, boundary_mod::boundary_zout};
  check(mhdgb_set_physics(handle(), hydflux_mod::gam, 0.05, bc), "set_physics");
  if (dt_chg) {
    check(mhdgb_set_dt(handle(), resolution_mod::dt), "set_dt");
    check(mhdgb_set_chg(handle(), hydflux_mod::chg), "set_chg");
  }
}
}  // namespace mhdgb_ref

namespace hydflux_mod {

// AllocateHydroVariables (mhd.cpp:33-77): one solver for the rank's grid (resolution_mod extents,
// config:: domain and boundaries) on device 0, plus the host mirrors.
inline void AllocateHydroVariables(GridArray<double>& G, FieldArray<double>& U, FieldArray<double>& Fx,
                                   FieldArray<double>& Fy, FieldArray<double>& Fz, FieldArray<double>& P) {
  using namespace resolution_mod;
  mhdgb_config c;
  mhdgb_config_default(&c);
  c.nx = ngrid1; c.ny = ngrid2; c.nz = ngrid3;
  c.x1min = config::x1min; c.x1max = config::x1max;
  c.x2min = config::x2min; c.x2max = config::x2max;
  c.x3min = config::x3min; c.x3max = config::x3max;
  c.bc[0] = boundary_mod::boundary_xin; c.bc[1] = boundary_mod::boundary_xout;
  c.bc[2] = boundary_mod::boundary_yin; c.bc[3] = boundary_mod::boundary_yout;
  c.bc[4] = boundary_mod::boundary_zin; c.bc[5] = boundary_mod::boundary_zout;
  c.gam = gam;
  c.cfl = 0.05;
  c.precision = MHDGB_FP64_EXACT;
  c.spacing_quirk = (ngrid1 <= ngrid2 && ngrid1 <= ngrid3) ? 1 : 0;  // mhd.cpp:1435-1436 where it is in bounds
  mhdgb_ref::check(mhdgb_create(&c, &mhdgb_ref::handle()), "AllocateHydroVariables");
  G.allocate(ktot, jtot, itot);
  U.allocate(mconsv, ktot, jtot, itot);
  P.allocate(nprim, ktot, jtot, itot);
  Fx.allocate(mconsv, ktot, jtot, itot);
  Fy.allocate(mconsv, ktot, jtot, itot);
  Fz.allocate(mconsv, ktot, jtot, itot);
  U.role = mhdgb_ref::Role::cons;
  P.role = mhdgb_ref::Role::prim;
  Fx.role = mhdgb_ref::Role::flux1;
  Fy.role = mhdgb_ref::Role::flux2;
  Fz.role = mhdgb_ref::Role::flux3;
}

// DeallocateHydroVariables (mhd.cpp:79-87).
inline void DeallocateHydroVariables(GridArray<double>& G, FieldArray<double>& U, FieldArray<double>& Fx,
                                     FieldArray<double>& Fy, FieldArray<double>& Fz, FieldArray<double>& P) {
  G.deallocate(); U.deallocate(); Fx.deallocate(); Fy.deallocate(); Fz.deallocate(); P.deallocate();
  mhdgb_destroy(mhdgb_ref::handle());
  mhdgb_ref::handle() = nullptr;
}

// GetNumericalFluxD (mhd.cpp:987-1410): the face fluxes of direction idir into F.
inline void GetNumericalFluxD(const int idir, const GridArray<double>&, const FieldArray<double>&, FieldArray<double>&) {
  mhdgb_ref::sync_globals(true);
  mhdgb_ref::check(mhdgb_flux(mhdgb_ref::handle(), idir), "GetNumericalFluxD");
}

// UpdateConservU (mhd.cpp:1412-1444).
inline void UpdateConservU(const GridArray<double>&, const FieldArray<double>&, const FieldArray<double>&,
                           const FieldArray<double>&, FieldArray<double>&) {
  mhdgb_ref::sync_globals(true);
  mhdgb_ref::check(mhdgb_update_conserv(mhdgb_ref::handle()), "UpdateConservU");
}

// UpdatePrimitvP (mhd.cpp:1447-1509).
inline void UpdatePrimitvP(const FieldArray<double>&, FieldArray<double>&) {
  mhdgb_ref::sync_globals(false);
  mhdgb_ref::check(mhdgb_update_prim(mhdgb_ref::handle()), "UpdatePrimitvP");
}

// ControlTimestep (mhd.cpp:1511-1561; device variant takes P as well): sets resolution_mod::dt.
inline void ControlTimestep(const GridArray<double>&) {
  mhdgb_ref::sync_globals(false);
  mhdgb_ref::check(mhdgb_control_timestep(mhdgb_ref::handle(), &resolution_mod::dt), "ControlTimestep");
}
inline void ControlTimestep(const GridArray<double>& G, const FieldArray<double>&) { ControlTimestep(G); }

// EvaluateCh (mhd.cpp:1563-1611): sets hydflux_mod::chg.
inline void EvaluateCh() {
  mhdgb_ref::sync_globals(false);
  mhdgb_ref::check(mhdgb_evaluate_ch(mhdgb_ref::handle(), &chg), "EvaluateCh");
}
inline void EvaluateCh(const FieldArray<double>&) { EvaluateCh(); }

// DampPsi (mhd.cpp:1613-1633).
inline void DampPsi(const GridArray<double>&, FieldArray<double>&) {
  mhdgb_ref::sync_globals(true);
  mhdgb_ref::check(mhdgb_damp_psi(mhdgb_ref::handle()), "DampPsi");
}

}  // namespace hydflux_mod

namespace boundary_mod {
using hydflux_mod::FieldArray;

inline void AllocateBoundaryVariables(BoundaryArray<double>& Bs, BoundaryArray<double>& Br) {
  Bs.allocate(0, 0, 0, 0, 0);
  Br.allocate(0, 0, 0, 0, 0);
}
inline void DeallocateBoundaryVariables(BoundaryArray<double>&, BoundaryArray<double>&) {}

// SetBoundaryCondition (boundary.cpp:750-893) with the single-rank fills of SendRecvBoundary.
inline void SetBoundaryCondition(FieldArray<double>&, BoundaryArray<double>&, BoundaryArray<double>&) {
  mhdgb_ref::sync_globals(false);
  mhdgb_ref::check(mhdgb_set_boundary(mhdgb_ref::handle()), "SetBoundaryCondition");
}
}  // namespace boundary_mod

namespace mhdgb_ref {
// Output(is_forced) of output.cpp:379-407: unless forced, only once time_sim has reached
// time_out + dtout; writes the current GPU state's snapshot files under the working directory
// (bindata/, and ascdata/ when config::asciiout), prints the reference's line, advances the index
// and sets time_out.  The state written is the device P (or U's primitives after steps), so no
// P.d2h() is needed first.
inline void Output(bool is_forced) {
  using namespace resolution_mod;
  static int index = 0;
  if (!is_forced && time_sim < time_out + dtout) return;
  check(mhdgb_output(handle(), ".", index, time_sim, dt, config::asciiout ? 1 : 0), "Output");
  std::printf("output index=%i, time=%e \n", index, time_sim);
  index += 1;
  time_out = time_sim;
}
}  // namespace mhdgb_ref

#ifdef MHDGB_REF_OUTPUT
inline void Output(bool is_forced) { mhdgb_ref::Output(is_forced); }
#endif

#endif
