// mhdgb_run -- C++ host driver of the GB300 solver: the reference's main loop
// (src_cpp_kokkos_host/main.cpp:188-291) on the Kelvin-Helmholtz problem, through the C ABI.
//
//   mhdgb_run [-n N | -nx X -ny Y -nz Z] [-p fp64|fp64_exact|mixed] [-t TMAX] [-s MAXSTEPS]
//             [-d DIAG_EVERY] [-o t-prof.csv] [--seed S] [--vshear V] [--bx B] [--amp A] [--noise E]
//             [--cfl C] [--autotune] [--output DIR [--dtout T] [--ascii]]
//             [--restart FILE] [--checkpoint FILE]
//
// Prints the reference's report lines ("sim time [s]:", "time/count/cell :", main.cpp:274-276).
// With -d > 0 the KH diagnostic of RealTimeAnalysis (src_cpp_kokkos_device/main.cpp:26-84) is
// appended to the t-prof.csv file every DIAG_EVERY steps, at the start and at the end; with -d 0
// (benchmark mode, config::benchmarkmode) only at the start and at the end.
// With --output the reference's snapshots (Output, output.cpp:379-407) are written under DIR: the
// forced ones at the start and the end (main.cpp:219, 279) and, with --dtout, one at the first step
// whose time reaches the previous snapshot's time + T (main.cpp:261).  Snapshots are written
// asynchronously while the following steps run.
// --restart starts from a checkpoint (state, grid, physics and clock) instead of the KH set-up;
// --checkpoint writes one at the end (mhdgb_checkpoint_save / _load).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "mhdgb.h"

namespace {

void die(mhdgb_solver* h, int rc, const char* what) {
  std::fprintf(stderr, "mhdgb_run: %s failed: %s (%s)\n", what, mhdgb_status_string(rc), h ? mhdgb_last_error(h) : "");
  std::exit(1);
}

struct TProf {
  FILE* fp = nullptr;
  void open(const char* path) {
    constexpr double Gamma = 1.49;
    fp = std::fopen(path, "w");
    if (fp) {
      std::fprintf(fp, "# Gamma= %24.16E\n", Gamma);
      std::fprintf(fp, "# 1:time 2:mix 3:v_y 4:exp(2Gamma*t)\n");
    }
  }
  void write(mhdgb_solver* h, double t) {
    constexpr double Amp = 1.2e-3, Gamma = 1.49;
    double d[3];
    const int rc = mhdgb_diag(h, d);
    if (rc) die(h, rc, "mhdgb_diag");
    if (fp) {
      std::fprintf(fp, " %24.16E %24.16E %24.16E %24.16E\n", t, d[1], d[2], Amp * std::exp(Gamma * t));
      std::fflush(fp);
    }
  }
  ~TProf() {
    if (fp) std::fclose(fp);
  }
};

}  // namespace

int main(int argc, char** argv) {
  mhdgb_config c;
  mhdgb_config_default(&c);
  double tmax = 15.0, vshear = 0.5, bx = 0.1, amp = 1e-2, noise = 1e-4;
  long long max_steps = 600000;  // config::stepmax
  int diag_every = 0;
  unsigned long long seed = 1;
  bool autotune = false, ascii = false;
  double dtout = 0.0;
  std::string tprof = "t-prof.csv", outdir, restart, checkpoint;
  for (int a = 1; a < argc; a++) {
    std::string s = argv[a];
    auto next = [&]() -> const char* {
      if (a + 1 >= argc) { std::fprintf(stderr, "missing value for %s\n", s.c_str()); std::exit(2); }
      return argv[++a];
    };
    if (s == "-n") c.nx = c.ny = c.nz = std::atoi(next());
    else if (s == "-nx") c.nx = std::atoi(next());
    else if (s == "-ny") c.ny = std::atoi(next());
    else if (s == "-nz") c.nz = std::atoi(next());
    else if (s == "-p") {
      std::string p = next();
      c.precision = p == "mixed" ? MHDGB_MIXED : (p == "fp64_exact" ? MHDGB_FP64_EXACT : MHDGB_FP64);
    } else if (s == "-t") tmax = std::atof(next());
    else if (s == "-s") max_steps = std::atoll(next());
    else if (s == "-d") diag_every = std::atoi(next());
    else if (s == "-o") tprof = next();
    else if (s == "--seed") seed = std::strtoull(next(), nullptr, 10);
    else if (s == "--vshear") vshear = std::atof(next());
    else if (s == "--bx") bx = std::atof(next());
    else if (s == "--amp") amp = std::atof(next());
    else if (s == "--noise") noise = std::atof(next());
    else if (s == "--cfl") c.cfl = std::atof(next());
    else if (s == "--autotune") autotune = true;
    else if (s == "--output") outdir = next();
    else if (s == "--dtout") dtout = std::atof(next());
    else if (s == "--ascii") ascii = true;
    else if (s == "--restart") restart = next();
    else if (s == "--checkpoint") checkpoint = next();
    else { std::fprintf(stderr, "unknown option %s\n", s.c_str()); return 2; }
  }
  mhdgb_solver* h = nullptr;
  int rc = mhdgb_create(&c, &h);
  if (rc) die(h, rc, "mhdgb_create");
  std::printf("grid size for x y z = %i %i %i\n", c.nx, c.ny, c.nz);
  if (!restart.empty()) {
    if ((rc = mhdgb_checkpoint_load(h, restart.c_str()))) die(h, rc, "mhdgb_checkpoint_load");
  } else if ((rc = mhdgb_init_kh(h, seed, vshear, 0.05, bx, amp, 0.2, noise))) {
    die(h, rc, "mhdgb_init_kh");
  }
  if (autotune) {
    int best = 0;
    if ((rc = mhdgb_autotune(h, 3, &best))) die(h, rc, "mhdgb_autotune");
  }
  mhdgb_report r{};
  if ((rc = mhdgb_sync(h, &r))) die(h, rc, "mhdgb_sync");   // the clock (non-zero after a restart)
  const long long step0 = r.step;
  TProf prof;
  prof.open(tprof.c_str());
  prof.write(h, r.time);
  // Output(forceoutput) at the initial state (resolution_mod::dt is still 0 there on a fresh start).
  int out_index = 0;
  double time_out = r.time;
  const bool output = !outdir.empty();
  auto snapshot = [&](double t, double dt) {
    int rc2 = mhdgb_output_begin(h, outdir.c_str(), out_index, t, dt, ascii ? 1 : 0);
    if (rc2) die(h, rc2, "mhdgb_output_begin");
    std::printf("output index=%i, time=%e \n", out_index, t);
    out_index += 1;
    time_out = t;
  };
  if (output) snapshot(r.time, r.dt);
  if ((rc = mhdgb_prepare(h))) die(h, rc, "mhdgb_prepare");
  std::printf("entering main loop\n");
  const auto t0 = std::chrono::high_resolution_clock::now();
  const int chunk = diag_every > 0 ? diag_every : 256;
  for (;;) {
    // Stop at tmax, or at the first step past the next regular snapshot time.
    const bool regular = output && dtout > 0.0;
    const double stop_t = regular ? std::min(tmax, time_out + dtout) : tmax;
    if ((rc = mhdgb_set_stop(h, stop_t, max_steps))) die(h, rc, "mhdgb_set_stop");
    for (;;) {
      if ((rc = mhdgb_step(h, chunk))) die(h, rc, "mhdgb_step");
      if ((rc = mhdgb_sync(h, &r))) die(h, rc, "mhdgb_sync");
      if (diag_every > 0 && !r.done) prof.write(h, r.time);
      if (r.done) break;
    }
    if (regular && r.time >= time_out + dtout) snapshot(r.time, r.dt);   // Output(usualoutput)
    if (r.time > tmax || r.step >= max_steps) break;
  }
  const auto t1 = std::chrono::high_resolution_clock::now();
  const double elapsed = std::chrono::duration<double>(t1 - t0).count();
  std::printf("exiting main loop time=%e, step=%lld\n", r.time, r.step);
  std::printf("sim time [s]: %e\n", elapsed);
  std::printf("time/count/cell : %e\n", elapsed / ((double)c.nx * c.ny * c.nz) / (double)(r.step - step0));
  prof.write(h, r.time);
  if (output) {
    snapshot(r.time, r.dt);   // Output(forceoutput) at the end
    if ((rc = mhdgb_output_end(h))) die(h, rc, "mhdgb_output_end");
  }
  if (!checkpoint.empty() && (rc = mhdgb_checkpoint_save(h, checkpoint.c_str()))) die(h, rc, "mhdgb_checkpoint_save");
  std::printf("program has been finished\n");
  mhdgb_destroy(h);
  return 0;
}
