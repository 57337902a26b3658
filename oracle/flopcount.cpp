// flopcount.cpp -- the oracle (mhd_oracle.c) compiled with an operation-counting double, to count
// the floating-point operations of the solver step per cell-update (test and measurement
// infrastructure; the product never links it).
//
// The oracle is C.  This file includes it as C++ with `double` replaced by Counted: a one-double
// wrapper whose operators count the operation and then perform exactly the same IEEE operation on
// the wrapped value.  So the arithmetic and its rounding are unchanged.  The tests check this by
// comparing the final state with the plain oracle's, bit for bit.  The build is single-threaded:
// without -fopenmp the pragmas are ignored, and the oracle guards its runtime calls.
//
// usage: flopcount NX NY NZ GAM CFL BXI BXO BYI BYO BZI BZO QUIRK RIEMANN XMIN XMAX YMIN YMAX ZMIN ZMAX
//                  U0.bin NSTEPS Uout.bin
//   U0.bin / Uout.bin: the 10 conserved fields in the reference layout (itot x jtot x ktot, FP64).
//   Step 1 runs stage by stage in the order of orc_step with the counters read between stages;
//   the remaining steps run through orc_run.  Prints one JSON line.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

namespace opcount {
struct Ops {
  unsigned long long add = 0, mul = 0, div = 0, sqrt = 0, cmp = 0, abs = 0, sign = 0;
};
Ops ops;
}  // namespace opcount

struct Counted {
  double v;
  Counted() = default;
  constexpr Counted(double x) : v(x) {}
  explicit constexpr operator double() const { return v; }
  Counted& operator+=(Counted b) { opcount::ops.add++; v += b.v; return *this; }
  Counted& operator-=(Counted b) { opcount::ops.add++; v -= b.v; return *this; }
  Counted& operator*=(Counted b) { opcount::ops.mul++; v *= b.v; return *this; }
  Counted& operator/=(Counted b) { opcount::ops.div++; v /= b.v; return *this; }
};
inline Counted operator+(Counted a, Counted b) { opcount::ops.add++; return Counted(a.v + b.v); }
inline Counted operator-(Counted a, Counted b) { opcount::ops.add++; return Counted(a.v - b.v); }
inline Counted operator*(Counted a, Counted b) { opcount::ops.mul++; return Counted(a.v * b.v); }
inline Counted operator/(Counted a, Counted b) { opcount::ops.div++; return Counted(a.v / b.v); }
inline Counted operator-(Counted a) { return Counted(-a.v); }  // a sign flip, not an operation
inline Counted operator+(Counted a) { return a; }
inline bool operator<(Counted a, Counted b) { opcount::ops.cmp++; return a.v < b.v; }
inline bool operator>(Counted a, Counted b) { opcount::ops.cmp++; return a.v > b.v; }
inline bool operator<=(Counted a, Counted b) { opcount::ops.cmp++; return a.v <= b.v; }
inline bool operator>=(Counted a, Counted b) { opcount::ops.cmp++; return a.v >= b.v; }
inline bool operator==(Counted a, Counted b) { opcount::ops.cmp++; return a.v == b.v; }
inline bool operator!=(Counted a, Counted b) { opcount::ops.cmp++; return a.v != b.v; }
inline Counted sqrt(Counted a) { opcount::ops.sqrt++; return Counted(std::sqrt(a.v)); }
inline Counted fabs(Counted a) { opcount::ops.abs++; return Counted(std::fabs(a.v)); }
inline Counted copysign(Counted a, Counted b) { opcount::ops.sign++; return Counted(std::copysign(a.v, b.v)); }

static_assert(sizeof(Counted) == sizeof(double), "Counted arrays are read and written as FP64 arrays");

// malloc/calloc results convert to any pointer type, as in C
struct AnyPtr {
  void* p;
  template <class T> operator T*() const { return static_cast<T*>(p); }
};

#define double Counted
#define malloc(n) AnyPtr{std::malloc(n)}
#define calloc(n, s) AnyPtr{std::calloc((n), (s))}
#include "mhd_oracle.c"
#undef calloc
#undef malloc
#undef double

namespace {

void put_ops(const opcount::Ops& a, const opcount::Ops& b, double cells, bool last) {
  const double add = (b.add - a.add) / cells, mul = (b.mul - a.mul) / cells, div = (b.div - a.div) / cells;
  const double sq = (b.sqrt - a.sqrt) / cells, cmp = (b.cmp - a.cmp) / cells;
  const double ab = (b.abs - a.abs) / cells, sg = (b.sign - a.sign) / cells;
  std::printf("{\"add\": %.3f, \"mul\": %.3f, \"div\": %.3f, \"sqrt\": %.3f, \"flops\": %.3f, \"cmp\": %.3f, "
              "\"abs\": %.3f, \"copysign\": %.3f}%s",
              add, mul, div, sq, add + mul + div + sq, cmp, ab, sg, last ? "" : ", ");
}

bool read_file(const char* path, void* dst, size_t bytes) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return false;
  const size_t got = std::fread(dst, 1, bytes, f);
  std::fclose(f);
  return got == bytes;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 23) {
    std::fprintf(stderr, "usage: flopcount NX NY NZ GAM CFL BC*6 QUIRK RIEMANN XMIN XMAX YMIN YMAX ZMIN ZMAX "
                         "U0.bin NSTEPS Uout.bin\n");
    return 2;
  }
  const int nx = std::atoi(argv[1]), ny = std::atoi(argv[2]), nz = std::atoi(argv[3]);
  orc_grid g;
  std::memset(&g, 0, sizeof(g));
  orc_grid_init(&g, nx, ny, nz);
  g.gam = std::atof(argv[4]);
  g.cfl = std::atof(argv[5]);
  for (int q = 0; q < 6; q++) g.bc[q] = std::atoi(argv[6 + q]);
  g.spacing_quirk = std::atoi(argv[12]);
  g.riemann = std::atoi(argv[13]);
  const double lo[3] = {std::atof(argv[14]), std::atof(argv[16]), std::atof(argv[18])};
  const double hi[3] = {std::atof(argv[15]), std::atof(argv[17]), std::atof(argv[19])};
  const int nsteps = std::atoi(argv[21]);
  const int ext[3] = {g.itot, g.jtot, g.ktot}, nn[3] = {nx, ny, nz};
  Counted* axes[3];
  for (int d = 0; d < 3; d++) {
    axes[d] = static_cast<Counted*>(std::calloc((size_t)ext[d], sizeof(Counted)));
    orc_generate_axis(axes[d], nn[d], lo[d], hi[d]);
  }
  g.x1a = axes[0];
  g.x2a = axes[1];
  g.x3a = axes[2];
  const size_t cells3 = (size_t)g.itot * g.jtot * g.ktot;
  const size_t nu = (size_t)ORC_NCONS * cells3, np = (size_t)ORC_NPRIM * cells3;
  Counted* U = static_cast<Counted*>(std::calloc(nu, sizeof(Counted)));
  Counted* P = static_cast<Counted*>(std::calloc(np, sizeof(Counted)));
  Counted* F[3];
  for (int d = 0; d < 3; d++) F[d] = static_cast<Counted*>(std::calloc(nu, sizeof(Counted)));
  if (!read_file(argv[20], U, nu * sizeof(double))) {
    std::fprintf(stderr, "flopcount: cannot read %s\n", argv[20]);
    return 1;
  }
  orc_update_prim(&g, U, P);  // the initial primitives (not part of a step)

  // step 1, stage by stage (orc_step's order, src_cpp_kokkos_host/main.cpp:229-259)
  const char* names[] = {"ControlTimestep", "SetBoundaryCondition", "EvaluateCh", "GetNumericalFlux1",
                         "GetNumericalFlux2", "GetNumericalFlux3", "UpdateConservU", "DampPsi", "UpdatePrimitvP"};
  opcount::Ops s[10];
  s[0] = opcount::ops;
  const Counted dt = orc_control_timestep(&g, P);
  s[1] = opcount::ops;
  orc_set_boundary(&g, P);
  s[2] = opcount::ops;
  const Counted chg = orc_evaluate_ch(&g, P);
  s[3] = opcount::ops;
  for (int d = 0; d < 3; d++) {
    orc_flux(d + 1, &g, P, F[d], chg);
    s[4 + d] = opcount::ops;
  }
  orc_update_conserv(&g, F[0], F[1], F[2], U, dt);
  s[7] = opcount::ops;
  orc_damp_psi(&g, U, dt, chg);
  s[8] = opcount::ops;
  orc_update_prim(&g, U, P);
  s[9] = opcount::ops;
  if (nsteps > 1) orc_run(&g, U, P, nsteps - 1, nullptr, nullptr);
  const opcount::Ops end = opcount::ops;

  const double cells = (double)nx * ny * nz;
  std::printf("{\"cells\": %.0f, \"steps\": %d, \"step1\": ", cells, nsteps);
  put_ops(s[0], s[9], cells, true);
  std::printf(", \"all_steps_per_step\": ");
  opcount::Ops per = s[0];
  put_ops(per, end, cells * nsteps, true);
  std::printf(", \"stages\": {");
  for (int q = 0; q < 9; q++) {
    std::printf("\"%s\": ", names[q]);
    put_ops(s[q], s[q + 1], cells, q == 8);
  }
  std::printf("}}\n");

  FILE* f = std::fopen(argv[22], "wb");
  if (!f || std::fwrite(U, sizeof(Counted), nu, f) != nu) {
    std::fprintf(stderr, "flopcount: cannot write %s\n", argv[22]);
    return 1;
  }
  std::fclose(f);
  return 0;
}
