// A program in the shape of the reference's src_cpp_kokkos_device/main.cpp, written against the
// drop-in header include/mhdgb_ref_api.hpp: grid, a KH state set in P and U on the host, h2d, the
// stage loop of main.cpp:317-351, d2h, and the forced snapshot outputs of main.cpp:219 and 279.
// Writes the initial P, U and the final U, P, dt, chg to the file named by argv[1] (read by
// tests/test_gpu_refapi.py); the snapshots go to bindata/ and ascdata/ in the working directory.
#include <cmath>
#include <cstdio>

#define MHDGB_REF_OUTPUT  // the header's Output() stands in for output.cpp's
#include "mhdgb_ref_api.hpp"

using namespace resolution_mod;
using namespace hydflux_mod;
using namespace boundary_mod;

static void write(FILE* f, const FieldArray<double>& A) { std::fwrite(A.data, sizeof(double), A.size, f); }

int main(int argc, char** argv) {
  const int nsteps = argc > 2 ? std::atoi(argv[2]) : 5;
  gam = 5.0 / 3.0;
  AllocateHydroVariables(G, U, Fx, Fy, Fz, P);
  AllocateBoundaryVariables(Bs, Br);
  const double dx1 = (x1max - x1min) / double(ngrid1), dx2 = (x2max - x2min) / double(ngrid2),
               dx3 = (x3max - x3min) / double(ngrid3);
  for (int i = 0; i < itot; i++) G.x1a(i) = dx1 * (i - (ngh + 1)) + x1min;
  for (int j = 0; j < jtot; j++) G.x2a(j) = dx2 * (j - (ngh + 1)) + x2min;
  for (int k = 0; k < ktot; k++) G.x3a(k) = dx3 * (k - (ngh + 1)) + x3min;
  for (int i = 0; i + 1 < itot; i++) G.x1b(i) = 0.5 * (G.x1a(i + 1) + G.x1a(i));
  for (int j = 0; j + 1 < jtot; j++) G.x2b(j) = 0.5 * (G.x2a(j + 1) + G.x2a(j));
  // a KH layer with B_x = 0.1, P and U consistent as GenerateProblem writes them (main.cpp:93-183)
  const double pi = std::acos(-1.0);
  for (int k = 0; k < ktot - 1; k++)
    for (int j = 0; j < jtot - 1; j++)
      for (int i = 0; i < itot - 1; i++) {
        const double x = G.x1b(i), y = G.x2b(j);
        P(nden, k, j, i) = 1.0;
        P(npre, k, j, i) = 1.0;
        P(nve1, k, j, i) = 0.5 * std::tanh(y / 0.05);
        P(nve2, k, j, i) = 0.02 * std::sin(2.0 * pi * x) * std::exp(-(y / 0.2) * (y / 0.2)) + 1e-3 * std::cos(3.0 * k);
        P(nve3, k, j, i) = 0.0;
        P(nbm1, k, j, i) = 0.1;
        P(nbm2, k, j, i) = 0.0;
        P(nbm3, k, j, i) = 0.0;
        P(nbps, k, j, i) = 0.0;
        P(nene, k, j, i) = P(npre, k, j, i) / (gam - 1.0);
        P(ncsp, k, j, i) = std::sqrt(gam * P(npre, k, j, i) / P(nden, k, j, i));
        P(nst, k, j, i) = 0.5 * (1.0 + std::tanh(y / 0.05));
        const double rho = P(nden, k, j, i);
        U(mden, k, j, i) = rho;
        U(mrv1, k, j, i) = rho * P(nve1, k, j, i);
        U(mrv2, k, j, i) = rho * P(nve2, k, j, i);
        U(mrv3, k, j, i) = rho * P(nve3, k, j, i);
        const double ekin = 0.5 * rho * (P(nve1, k, j, i) * P(nve1, k, j, i) + P(nve2, k, j, i) * P(nve2, k, j, i) +
                                         P(nve3, k, j, i) * P(nve3, k, j, i));
        const double emag = 0.5 * (P(nbm1, k, j, i) * P(nbm1, k, j, i));
        U(meto, k, j, i) = rho * P(nene, k, j, i) + ekin + emag;
        U(mbm1, k, j, i) = P(nbm1, k, j, i);
        U(mbm2, k, j, i) = 0.0;
        U(mbm3, k, j, i) = 0.0;
        U(mbps, k, j, i) = 0.0;
        U(mst, k, j, i) = rho * P(nst, k, j, i);
      }
  FILE* f = std::fopen(argv[1], "wb");
  write(f, P);
  write(f, U);
  G.h2d();
  P.h2d();
  U.h2d();
  Output(true);
  std::vector<double> dts, chgs;
  for (int step = 0; step < nsteps; step++) {
    ControlTimestep(G, P);
    SetBoundaryCondition(P, Bs, Br);
    EvaluateCh(P);
    GetNumericalFluxD(1, G, P, Fx);
    GetNumericalFluxD(2, G, P, Fy);
    GetNumericalFluxD(3, G, P, Fz);
    UpdateConservU(G, Fx, Fy, Fz, U);
    DampPsi(G, U);
    UpdatePrimitvP(U, P);
    time_sim += dt;
    dts.push_back(dt);
    chgs.push_back(chg);
  }
  Output(true);
  U.d2h();
  P.d2h();
  write(f, U);
  write(f, P);
  std::fwrite(dts.data(), sizeof(double), dts.size(), f);
  std::fwrite(chgs.data(), sizeof(double), chgs.size(), f);
  std::fclose(f);
  DeallocateHydroVariables(G, U, Fx, Fy, Fz, P);
  std::printf("time_sim %.17g\n", time_sim);
  return 0;
}
