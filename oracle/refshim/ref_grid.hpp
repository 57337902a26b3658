// ref_grid.hpp -- the reference's GenerateGrid (src_cpp_kokkos_host/main.cpp:26-65) for one rank
// (coords = 0, ntiles = 1), written out with the same operations in the same order, for the oracle
// harnesses.  Test infrastructure only.
#ifndef ORACLE_REFSHIM_REF_GRID_HPP_
#define ORACLE_REFSHIM_REF_GRID_HPP_

#include "config.hpp"
#include "mhd.hpp"

inline void ref_setup_grid(hydflux_mod::GridArray<double>& G) {
  using namespace resolution_mod;
  const double x1minloc = x1min + (x1max - x1min) / 1 * 0, x1maxloc = x1min + (x1max - x1min) / 1 * (0 + 1);
  const double dx1 = (x1maxloc - x1minloc) / double(ngrid1);
  for (int i = is - ngh; i <= ie + ngh + 1; i++) G.x1a(i) = dx1 * (i - (ngh + 1)) + x1minloc;
  for (int i = is - ngh; i <= ie + ngh; i++) G.x1b(i) = 0.5e0 * (G.x1a(i + 1) + G.x1a(i));
  const double x2minloc = x2min + (x2max - x2min) / 1 * 0, x2maxloc = x2min + (x2max - x2min) / 1 * (0 + 1);
  const double dx2 = (x2maxloc - x2minloc) / double(ngrid2);
  for (int j = js - ngh; j <= je + ngh + 1; j++) G.x2a(j) = dx2 * (j - (ngh + 1)) + x2minloc;
  for (int j = js - ngh; j <= je + ngh; j++) G.x2b(j) = 0.5e0 * (G.x2a(j + 1) + G.x2a(j));
  const double x3minloc = x3min + (x3max - x3min) / 1 * 0, x3maxloc = x3min + (x3max - x3min) / 1 * (0 + 1);
  const double dx3 = (x3maxloc - x3minloc) / double(ngrid3);
  for (int k = ks - ngh; k <= ke + ngh + 1; k++) G.x3a(k) = dx3 * (k - (ngh + 1)) + x3minloc;
  for (int k = ks - ngh; k <= ke + ngh; k++) G.x3b(k) = 0.5e0 * (G.x3a(k + 1) + G.x3a(k));
}

#endif
