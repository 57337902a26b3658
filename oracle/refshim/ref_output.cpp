// ref_output.cpp -- runs the reference's own Output() (src_cpp_kokkos_host/output.cpp:379-407:
// MPI_IO_Pack, MPI_IO_Write, WriteXDMF, ASC_WRITE; compiled unmodified from the reference tree
// against the single-rank MPI-IO shim) on given primitive states, to pin the output oracle and to
// produce the golden output files under tests/golden/.  Test infrastructure only.
//
// Input file (little endian): int32 nx,ny,nz | int32 nsnap | nsnap x { float64 time, dt |
//   float64 P[12 * itot*jtot*ktot] in the reference FieldArray layout }.
// Each snapshot is written by a forced Output(true) in the current directory (bindata/, ascdata/).
#include <cstdio>
#include <cstdlib>

#include "config.hpp"
#include "mhd.hpp"
#include "mpi_config.hpp"
#include "output.hpp"
#include "ref_grid.hpp"

using namespace resolution_mod;
using namespace hydflux_mod;

static void fail(const char* m) {
  std::fprintf(stderr, "ref_output: %s\n", m);
  std::exit(2);
}

int main(int argc, char** argv) {
  if (argc != 2) fail("usage: ref_output <in>");
  FILE* in = std::fopen(argv[1], "rb");
  if (!in) fail("cannot open input");
  int dims[3], nsnap;
  if (std::fread(dims, sizeof(int), 3, in) != 3 || std::fread(&nsnap, sizeof(int), 1, in) != 1) fail("bad header");
  if (dims[0] != ngrid1 || dims[1] != ngrid2 || dims[2] != ngrid3) fail("grid does not match build");
  mpi_config_mod::InitializeMPI();
  AllocateHydroVariables(G, U, Fx, Fy, Fz, P);
  ref_setup_grid(G);
  for (int s = 0; s < nsnap; s++) {
    double td[2];
    if (std::fread(td, sizeof(double), 2, in) != 2) fail("short snapshot header");
    if (std::fread(P.data, sizeof(double), P.size, in) != P.size) fail("short P");
    time_sim = td[0];
    dt = td[1];
    Output(true);
  }
  std::fclose(in);
  return 0;
}
