// ref_harness.cpp -- drives the reference's own stage functions (src_cpp_kokkos_host/mhd.cpp,
// boundary.cpp, mpi_config.cpp, compiled unmodified from the reference tree) on a seeded input,
// in the stage order of src_cpp_kokkos_host/main.cpp:229-259, and dumps the results.  It exists
// only to pin the oracle restatement and to produce the golden vectors under tests/golden/.
//
// Input file (little endian):  int32 nx,ny,nz | float64 gam | int32 bc[6] | int32 nsteps |
//   int32 dump_flux | float64 U[10 * itot*jtot*ktot] in the reference FieldArray layout.
// Output file:  float64 dts[nsteps] | chgs[nsteps] | P0 (after UpdatePrimitvP on the input,
//   before any ghost fill) | P1 U1 (after step 1) | [Fx Fy Fz of step 1 if dump_flux] |
//   PN UN (after nsteps).  Arrays are full reference-layout arrays (ghosts included).
// The grid is the reference's GenerateGrid (main.cpp:26-65) for one rank.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "boundary.hpp"
#include "config.hpp"
#include "mhd.hpp"
#include "mpi_config.hpp"
#include "ref_grid.hpp"

using namespace resolution_mod;
using namespace hydflux_mod;

static void fail(const char* m) {
  std::fprintf(stderr, "ref_harness: %s\n", m);
  std::exit(2);
}

static void dump(FILE* f, const FieldArray<double>& A) {
  if (std::fwrite(A.data, sizeof(double), A.size, f) != A.size) fail("short write");
}

int main(int argc, char** argv) {
  if (argc != 3) fail("usage: ref_harness <in> <out>");
  FILE* in = std::fopen(argv[1], "rb");
  if (!in) fail("cannot open input");
  int dims[3], bc[6], nsteps, dump_flux;
  double g;
  if (std::fread(dims, sizeof(int), 3, in) != 3) fail("bad header");
  if (dims[0] != ngrid1 || dims[1] != ngrid2 || dims[2] != ngrid3) fail("grid does not match build");
  if (std::fread(&g, sizeof(double), 1, in) != 1) fail("bad header");
  if (std::fread(bc, sizeof(int), 6, in) != 6) fail("bad header");
  if (std::fread(&nsteps, sizeof(int), 1, in) != 1) fail("bad header");
  if (std::fread(&dump_flux, sizeof(int), 1, in) != 1) fail("bad header");

  mpi_config_mod::InitializeMPI();
  AllocateHydroVariables(G, U, Fx, Fy, Fz, P);
  boundary_mod::AllocateBoundaryVariables(boundary_mod::Bs, boundary_mod::Br);
  ref_setup_grid(G);
  gam = g;
  boundary_mod::boundary_xin = bc[0];
  boundary_mod::boundary_xout = bc[1];
  boundary_mod::boundary_yin = bc[2];
  boundary_mod::boundary_yout = bc[3];
  boundary_mod::boundary_zin = bc[4];
  boundary_mod::boundary_zout = bc[5];
  if (std::fread(U.data, sizeof(double), U.size, in) != U.size) fail("short U");
  std::fclose(in);

  UpdatePrimitvP(U, P);
  std::vector<double> P0(P.data, P.data + P.size);
  std::vector<double> dts(nsteps), chgs(nsteps);
  FILE* out = std::fopen(argv[2], "wb");
  if (!out) fail("cannot open output");
  std::vector<double> P1, U1, F1;
  const auto t0 = std::chrono::steady_clock::now();
  for (int step = 0; step < nsteps; step++) {
    ControlTimestep(G);
    boundary_mod::SetBoundaryCondition(P, boundary_mod::Bs, boundary_mod::Br);
    EvaluateCh();
    GetNumericalFluxD(1, G, P, Fx);
    GetNumericalFluxD(2, G, P, Fy);
    GetNumericalFluxD(3, G, P, Fz);
    UpdateConservU(G, Fx, Fy, Fz, U);
    DampPsi(G, U);
    UpdatePrimitvP(U, P);
    time_sim += dt;
    dts[step] = dt;
    chgs[step] = chg;
    if (step == 0) {
      P1.assign(P.data, P.data + P.size);
      U1.assign(U.data, U.data + U.size);
      if (dump_flux) {
        F1.insert(F1.end(), Fx.data, Fx.data + Fx.size);
        F1.insert(F1.end(), Fy.data, Fy.data + Fy.size);
        F1.insert(F1.end(), Fz.data, Fz.data + Fz.size);
      }
    }
  }
  // wall time of the step loop (the first step's copies of P, U and F included), reported the way
  // the reference's main.cpp:274-276 does
  const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  std::fprintf(stderr, "time/count/cell : %e\n", wall / ((double)ngrid1 * ngrid2 * ngrid3) / nsteps);
  std::fwrite(dts.data(), sizeof(double), nsteps, out);
  std::fwrite(chgs.data(), sizeof(double), nsteps, out);
  std::fwrite(P0.data(), sizeof(double), P0.size(), out);
  std::fwrite(P1.data(), sizeof(double), P1.size(), out);
  std::fwrite(U1.data(), sizeof(double), U1.size(), out);
  if (dump_flux) std::fwrite(F1.data(), sizeof(double), F1.size(), out);
  dump(out, P);
  dump(out, U);
  std::fclose(out);
  return 0;
}
