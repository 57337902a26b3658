/*
 * mhdgb.h -- C ABI of the GB300 ideal-MHD solver step (libmhdgb.so).
 *
 * One handle = one grid on one CUDA device, with its own stream.  The library owns all device
 * memory; callers pass host arrays in the reference's FieldArray layout
 * (src_cpp_kokkos_host/mhd.hpp:186-245: element (n,k,j,i) at i + itot*(n + nv*(j + jtot*k)),
 * itot = nx + 2*ngh + 1, ngh = 2, src_cpp_kokkos_host/config.hpp:53-59).
 * Every function returns MHDGB_OK (0) or a negative status; mhdgb_last_error() gives the text.
 * A handle is not thread safe; different handles are independent.
 *
 * Three groups of entry points:
 *  - stage entry points, one per reference stage function (hydflux_mod / boundary_mod), which run
 *    the FP64 stage kernels on the handle's U / P / Fx,Fy,Fz arrays with the reference's rounding
 *    (bit-for-bit equal to the reference's CPU build);
 *  - the fused step (mhdgb_step / mhdgb_run_until): the whole main-loop body of
 *    src_cpp_kokkos_host/main.cpp:229-259 as one persistent kernel per step, CUDA-graph captured,
 *    in the FP64 form or the FP32-mixed form;
 *  - the ensemble: many independent grids of uneven size advanced together.
 */
#ifndef MHDGB_H_
#define MHDGB_H_

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define MHDGB_OK 0
#define MHDGB_ERR_ARG (-1)        /* invalid argument / configuration */
#define MHDGB_ERR_CUDA (-2)       /* CUDA runtime or driver error */
#define MHDGB_ERR_NONFINITE (-3)  /* a non-finite dt / c_h candidate was produced */
#define MHDGB_ERR_NEGATIVE (-4)   /* rho <= 0 or p <= 0 in some cell */
#define MHDGB_ERR_TIMEOUT (-5)    /* a bounded device-side wait gave up */
#define MHDGB_ERR_STATE (-6)      /* call out of order (e.g. no state uploaded) */
#define MHDGB_ERR_NOMEM (-7)      /* device allocation failed */
#define MHDGB_ERR_IO (-9)         /* a snapshot file could not be written */

/* boundary types, src_cpp_kokkos_host/config.hpp:29-31 */
#define MHDGB_BC_PERIODIC 1
#define MHDGB_BC_REFLECTION 2
#define MHDGB_BC_OUTFLOW 3
/* A face shared with another block of a decomposed grid (the reference's MPI neighbours,
 * mpi_config.cpp:61-69): no local fill writes its ghost layers, which the halo exchange copies from
 * the neighbour (mhdgb_halo_pack / _unpack, or a domain's own exchange); boundary.cpp:222-318. */
#define MHDGB_BC_EXCHANGE 4

/* precision of the fused step */
#define MHDGB_FP64 0        /* FP64 throughout, FMA contraction (last-bit differences) */
#define MHDGB_FP64_EXACT 1  /* FP64, separately rounded: bit-for-bit the reference's arithmetic */
#define MHDGB_MIXED 2       /* FP32 reconstruction + Riemann solve; FP64 state, update, pressure
                               recovery and reductions */

#define MHDGB_NPRIM 12 /* hydflux_mod::nprim, mhd.hpp:320 */
#define MHDGB_NCONS 10 /* hydflux_mod::mconsv, mhd.hpp:325 */

/* Compile-time parameters of src_cpp_kokkos_host/config.hpp:10-42 (one rank) plus hydflux_mod::gam
 * (mhd.cpp:27) and the CFL factor hard-coded at mhd.cpp:1560, as run-time values. */
typedef struct mhdgb_config {
  int nx, ny, nz;                  /* config::ngridtotal1..3 (interior cells) */
  double x1min, x1max, x2min, x2max, x3min, x3max; /* config::x?min / x?max */
  int bc[6];                       /* boundary_xin, _xout, _yin, _yout, _zin, _zout */
  double gam;                      /* hydflux_mod::gam */
  double cfl;                      /* dt = cfl * min_cells(...); the reference uses 0.05 */
  int precision;                   /* MHDGB_FP64, MHDGB_FP64_EXACT or MHDGB_MIXED */
  int spacing_quirk;               /* 1: UpdateConservU takes the y/z spacing at index i as
                                      mhd.cpp:1435-1436 does (requires nx <= ny, nx <= nz) */
  int device;                      /* CUDA device ordinal */
} mhdgb_config;

typedef struct mhdgb_solver mhdgb_solver;

/* Progress of the fused step (read by mhdgb_sync). */
typedef struct mhdgb_report {
  long long step;   /* fused steps completed */
  double time;      /* resolution_mod::time_sim */
  double dt;        /* dt of the latest step */
  double chg;       /* c_h of the latest step */
  double next_dt;   /* dt the next step will use */
  double next_chg;  /* c_h the next step will use */
  int done;         /* time > tmax or step >= max_steps reached */
  unsigned status;  /* device status bits: 1 non-finite, 2 non-positive rho/p, 4 wait timeout */
} mhdgb_report;

/* Defaults of src_cpp_kokkos_host/config.hpp (150^3, KH domain and boundaries) with gam = 5/3. */
int mhdgb_config_default(mhdgb_config* cfg);

/* AllocateHydroVariables + AllocateBoundaryVariables (mhd.cpp:33-77, boundary.cpp:36-95) and
 * GenerateGrid (main.cpp:26-65). */
int mhdgb_create(const mhdgb_config* cfg, mhdgb_solver** out);
/* DeallocateHydroVariables / DeallocateBoundaryVariables (mhd.cpp:79-87, boundary.cpp:98-104). */
int mhdgb_destroy(mhdgb_solver* h);
const char* mhdgb_last_error(const mhdgb_solver* h);
const char* mhdgb_status_string(int status);
/* itot, jtot, ktot of the handle (resolution_mod, config.hpp:57-59). */
int mhdgb_extents(const mhdgb_solver* h, int* itot, int* jtot, int* ktot);
/* Bytes of device memory held by the handle. */
size_t mhdgb_device_bytes(const mhdgb_solver* h);

/* Change gam (hydflux_mod::gam), the CFL factor and the boundary types (boundary_mod::boundary_xin
 * ... _zout, boundary.cpp:26-31) of an existing handle; bc may be NULL to keep them. */
int mhdgb_set_physics(mhdgb_solver* h, double gam, double cfl, const int* bc);

/* Riemann solver of the face fluxes, for the stage path and every fused form: HLLD (the C++ path's,
 * mhd.cpp:97-417; the default), or the Fortran variant's alternatives HLLE (src_f90_acc_device/
 * mhd.f90:877-907) and HLLC (mhd.f90:909-1141), selectable there by editing the calls at
 * mhd.f90:478-480, 665-667, 852-854.  The Fortran HLLC reads a passive-scalar star state it never
 * sets; here it is the scalar scaled by the star-state density ratio, as that routine scales the
 * transverse field. */
#define MHDGB_RIEMANN_HLLD 0
#define MHDGB_RIEMANN_HLLE 1
#define MHDGB_RIEMANN_HLLC 2
int mhdgb_set_riemann(mhdgb_solver* h, int solver);
int mhdgb_get_riemann(const mhdgb_solver* h);   /* the solver in use, or MHDGB_ERR_ARG */

/* GridArray G (mhd.hpp:22-182): cell faces x1a/x2a/x3a, lengths itot/jtot/ktot. */
int mhdgb_get_grid(const mhdgb_solver* h, double* x1a, double* x2a, double* x3a);
int mhdgb_set_grid(mhdgb_solver* h, const double* x1a, const double* x2a, const double* x3a);

/* State transfer (FieldArray::h2d / d2h, mhd.hpp:310-315).  U: 10 fields, P: 12 fields, F: 10. */
int mhdgb_upload_cons(mhdgb_solver* h, const double* U);
int mhdgb_upload_prim(mhdgb_solver* h, const double* P);
int mhdgb_download_cons(mhdgb_solver* h, double* U);
int mhdgb_download_prim(mhdgb_solver* h, double* P);
int mhdgb_download_flux(mhdgb_solver* h, int dir, double* F);

/* One variable at a time, for callers that keep one (itot, jtot, ktot) array per variable with i
 * fastest, as the Fortran variants do (src_f90_acc_device/mhd.f90:29-36: d, mv1..3, et, b1..3, bp,
 * Xcomp).  m is the reference's index: 0..9 for U (mden..mst), 0..11 for P (nden..nst). */
int mhdgb_upload_cons_field(mhdgb_solver* h, int m, const double* a);
int mhdgb_download_cons_field(mhdgb_solver* h, int m, double* a);
int mhdgb_upload_prim_field(mhdgb_solver* h, int n, const double* a);
int mhdgb_download_prim_field(mhdgb_solver* h, int n, double* a);

/* ---- stage entry points (synchronous, FP64, reference rounding) ---- */
/* ControlTimestep (mhd.cpp:1511-1561): dt = cfl * min over the interior; sets the handle's dt. */
int mhdgb_control_timestep(mhdgb_solver* h, double* dt);
/* SetBoundaryCondition (boundary.cpp:750-893) with the single-rank SendRecvBoundary fills. */
int mhdgb_set_boundary(mhdgb_solver* h);
/* EvaluateCh (mhd.cpp:1563-1611): sets the handle's chg. */
int mhdgb_evaluate_ch(mhdgb_solver* h, double* chg);
/* GetNumericalFluxD(dir) (mhd.cpp:987-1410), dir = 1, 2, 3: fills Fx, Fy or Fz. */
int mhdgb_flux(mhdgb_solver* h, int dir);
/* UpdateConservU (mhd.cpp:1412-1444). */
int mhdgb_update_conserv(mhdgb_solver* h);
/* DampPsi (mhd.cpp:1613-1633). */
int mhdgb_damp_psi(mhdgb_solver* h);
/* UpdatePrimitvP (mhd.cpp:1447-1509). */
int mhdgb_update_prim(mhdgb_solver* h);
/* resolution_mod::dt (config.hpp:49) and hydflux_mod::chg (mhd.cpp:26) of the stage path. */
int mhdgb_set_dt(mhdgb_solver* h, double dt);
int mhdgb_set_chg(mhdgb_solver* h, double chg);

/* ---- fused step ---- */
/* Recover P from U (UpdatePrimitvP over the interior, mhd.cpp:1480-1507), fill the ghosts and
 * reduce the first step's dt and c_h; called implicitly by the first mhdgb_step after an upload. */
int mhdgb_prepare(mhdgb_solver* h);
/* Enqueue nsteps steps of the main loop (main.cpp:229-259) on the handle's stream; returns
 * without waiting.  Steps after the stop condition (see mhdgb_set_stop) do nothing. */
int mhdgb_step(mhdgb_solver* h, int nsteps);
/* Stop condition of the loop, main.cpp:265: time > tmax or step >= max_steps. */
int mhdgb_set_stop(mhdgb_solver* h, double tmax, long long max_steps);
/* Run until the stop condition holds; report may be NULL. */
int mhdgb_run_until(mhdgb_solver* h, double tmax, long long max_steps, mhdgb_report* report);
/* Wait for the enqueued steps and report progress; returns a status for device-side errors. */
int mhdgb_sync(mhdgb_solver* h, mhdgb_report* report);
/* Reset time and step counters (resolution_mod::time_sim = 0). */
int mhdgb_reset_clock(mhdgb_solver* h);
/* One step on caller-owned host arrays: upload U (10 fields, reference layout), run nsteps fused
 * steps, download the new U and return the step's dt and c_h.  The drop-in form of the loop body
 * for callers that keep the state on the host.  Page-locked, mapped arrays (cudaHostAlloc,
 * cudaHostRegister, a pinned torch tensor) are read and written by the kernels themselves over the
 * host link: the recovery pass reads U_in, the last step writes each updated cell of U_out, and the
 * ghost cells of a separate U_out are copied from U_in.  Other arrays go through a device staging
 * buffer.  Both give the same U_out bit for bit; U_out may be U_in. */
int mhdgb_step_host(mhdgb_solver* h, const double* U_in, double* U_out, int nsteps, double* dt, double* chg);

/* Time nsteps fused steps with CUDA events recorded on the handle's stream around the enqueued
 * launches (synchronising before and after); *ms receives the elapsed device time. */
int mhdgb_time_steps(mhdgb_solver* h, int nsteps, double* ms);

/* Tile shapes of the fused kernel compiled for the handle's precision (the autotuner's choices):
 * columns tx x ty per tile, threads per CTA; current = 1 for the one in use. */
int mhdgb_variant_count(const mhdgb_solver* h);
int mhdgb_variant_info(const mhdgb_solver* h, int idx, int* tx, int* ty, int* threads, int* current);
int mhdgb_select_variant(mhdgb_solver* h, int idx);
/* Kernel form and tile shape of variant idx, e.g. "two-phase 16x8/256" or "fused-slope 16x8/256 x2"
 * (x2: compiled for two CTAs per SM); idx = -1 names the kernel in use, which for HLLE/HLLC is the
 * run-time solver kernel.  NULL for an invalid index. */
const char* mhdgb_variant_name(const mhdgb_solver* h, int idx);
/* Work decomposition of the fused step in use: tiles per axis, z chunks per tile column and, if
 * kstart is not NULL, the nchunks + 1 chunk boundaries (interior plane indices, 0 .. nz).  The work
 * queue hands out chunk 0 of every tile first; chunks that shrink towards the end of the queue even
 * out the CTAs' finish times. */
int mhdgb_work_layout(const mhdgb_solver* h, int* ntx, int* nty, int* nchunks, int* kstart);
/* The z chunking that the fused step plans for an nx x ny x nz grid cut into tx x ty tiles, on a
 * persistent launch of ctas CTAs: the host-side planner that mhdgb_work_layout reports the result
 * of (uniform, shrinking and geometric chunkings; the one whose simulated work queue finishes
 * first).  Writes the chunk lengths in planes (they sum to nz) to chunks[0 .. max_chunks) and
 * returns their number, or MHDGB_ERR_ARG for a bad size or too small an array.  Needs no device. */
int mhdgb_plan_zchunks(int nx, int ny, int nz, int tx, int ty, int ctas, int* chunks, int max_chunks);
/* Time every compiled tile shape on the handle's grid (steps fused steps each, from the current
 * state, which is restored afterwards) and keep the fastest.  The choice is remembered per
 * (precision, nx, ny, nz) for later handles in the process and, if the environment variable
 * MHDGB_TUNE_CACHE names a file, across processes. */
int mhdgb_autotune(mhdgb_solver* h, int steps, int* best);

/* Measured FP64 FMA throughput of a device (GFLOP/s, 2 flops per FMA): the denominator of the
 * FP64-pipe roofline of the FP64 form, which is bound by FP64 issue rather than by HBM. */
int mhdgb_measure_fp64_rate(int device, double* gflops);

/* Self-test of the FP64 division and square root used by the FMA-contracted FP64 form (FP32-seeded
 * reciprocal with two Newton-Raphson steps; FP32-seeded Goldschmidt square root and reciprocal
 * square root) against IEEE division and square root on n random operands; *max_ulp receives the
 * largest difference in units in the last place. */
int mhdgb_selftest_division(int device, int n, unsigned long long seed, double* max_ulp);
/* Self-test of failure detection (no reference counterpart): a kernel waits on a shared-memory
 * barrier that nothing completes; the bounded wait the fused step uses for its plane loads gives
 * up after about 2 s and returns with the timeout bit (4) set in *status, leaving the context
 * usable.  *seconds receives the kernel's duration.  Nothing faults or hangs. */
int mhdgb_selftest_wait_timeout(int device, double* seconds, unsigned* status);
/* Self-test of the fused step's abort path (no reference counterpart): on a 32x24x16 KH grid of the
 * given precision, one fused step runs with the first plane load of every work item expecting 16
 * bytes more than the load delivers, so each CTA's bounded wait for that plane gives up after about
 * 2 s, the CTA drains its other loads (bounded too) and returns.  *seconds is the step's duration and
 * *status its device status bits (4 = wait timeout).  The same handle then runs two ordinary steps
 * from a fresh state; *recovered = 1 if they report no error and equal those of a handle that never
 * saw the aborted step, bit for bit.  Nothing faults or hangs. */
int mhdgb_selftest_fused_abort(int device, int precision, double* seconds, unsigned* status, int* recovered);

/* KH diagnostic of RealTimeAnalysis (src_cpp_kokkos_device/main.cpp:26-84):
 * out = {volume, <X(1-X)>, sqrt(<v_y^2>)} over the interior, FP64 sums. */
int mhdgb_diag(mhdgb_solver* h, double out[3]);

/* Kelvin-Helmholtz initial state (single shear layer v_x = vshear*tanh(y/width), rho = 1, p = 1,
 * B = (bx,0,0), v_y = amp*sin(2 pi x) exp(-(y/sig)^2) + noise*(2u-1) with u seeded per cell,
 * scalar X = (1+tanh(y/width))/2) written into U; see mhdturbulence_gb300/ic.py. */
int mhdgb_init_kh(mhdgb_solver* h, unsigned long long seed, double vshear, double width, double bx, double amp,
                  double sig, double noise);
/* The same state for a block of a decomposed grid: the handle's cells are cells offset[a] ..
 * offset[a] + n[a] - 1 of a whole grid of whole[0] x whole[1] x whole[2] cells, whose seeded noise
 * they take (so the blocks together hold exactly the single grid's state).  The handle's cell faces
 * must already be the whole grid's (mhdgb_set_grid). */
int mhdgb_init_kh_block(mhdgb_solver* h, const int whole[3], const int offset[3], unsigned long long seed,
                        double vshear, double width, double bx, double amp, double sig, double noise);

/* ---- snapshot output ----
 * Output(true) of src_cpp_kokkos_host/output.cpp:379-407 for one rank: under root (NULL: "."),
 * bindata/unf%05d.dat, bindata/grid{1,2,3}D.bin, bindata/field%05d.bin ([10][nz][ny][nx] FP64:
 * d v1 v2 v3 b1 b2 b3 bp p X1), bindata/field%05d.xmf and, if ascii, ascdata/snap000-%05d.csv
 * (MPI_IO_Pack/MPI_IO_Write/WriteXDMF/ASC_WRITE, output.cpp:81-386), byte for byte the reference's
 * files for the same P, time and dt.  time/dt are the values written in the headers
 * (resolution_mod::time_sim and dt).  The state written is the primitive array the caller
 * uploaded, if it is still current, else the primitives recovered from U.
 * mhdgb_output_begin packs the state on the device after every step already enqueued, copies it to
 * pinned host memory on a second stream and writes the files on a host thread, so steps enqueued
 * after it overlap the copy and the file writing; mhdgb_output_end waits for that and returns the
 * writer's status (MHDGB_ERR_IO on a failed write).  A begin while a previous snapshot is still
 * being written waits for it first.  mhdgb_output = begin + end.  The first call allocates a
 * device and a pinned host buffer of 80 bytes per cell. */
int mhdgb_output_begin(mhdgb_solver* h, const char* root, int index, double time, double dt, int ascii);
int mhdgb_output_end(mhdgb_solver* h);
int mhdgb_output(mhdgb_solver* h, const char* root, int index, double time, double dt, int ascii);

/* ---- checkpoint / restart ----
 * No counterpart in the reference, which has none.  save writes the conserved state U (with
 * ghosts, FieldArray layout), the grid, gam, cfl, the boundary types, the Riemann solver and the
 * clock (step, time, latest dt and c_h, stop time and step) to one binary file; load restores all of
 * it into a handle of the same nx, ny, nz and spacing_quirk (any precision).  The next fused step
 * recovers P from U and
 * reduces dt and c_h as mhdgb_prepare does, so a run restarted in the same precision continues bit
 * for bit as if it had not stopped.  Errors: MHDGB_ERR_IO (file), MHDGB_ERR_ARG (not a checkpoint,
 * or another grid). */
int mhdgb_checkpoint_save(mhdgb_solver* h, const char* path);
int mhdgb_checkpoint_load(mhdgb_solver* h, const char* path);

/* ---- ensemble: many independent grids advanced together ----
 * Every member is an ordinary handle (upload/download/init/diag work on it; the ensemble owns it)
 * with its own grid, boundaries, gam and state; all members share one stream and one precision.
 * Each ensemble step is one persistent launch of the fused kernel that walks the work items of all
 * members, every member advancing by its own dt; launches are captured in a CUDA graph. */
typedef struct mhdgb_ensemble mhdgb_ensemble;
int mhdgb_ensemble_create(int n, const mhdgb_config* cfgs, mhdgb_ensemble** out);
int mhdgb_ensemble_destroy(mhdgb_ensemble* e);
const char* mhdgb_ensemble_last_error(const mhdgb_ensemble* e);
int mhdgb_ensemble_size(const mhdgb_ensemble* e);
int mhdgb_ensemble_member(mhdgb_ensemble* e, int i, mhdgb_solver** h);
long long mhdgb_ensemble_cells(const mhdgb_ensemble* e);
int mhdgb_ensemble_prepare(mhdgb_ensemble* e);
int mhdgb_ensemble_step(mhdgb_ensemble* e, int nsteps);
/* reports: array of size() entries or NULL. */
int mhdgb_ensemble_sync(mhdgb_ensemble* e, mhdgb_report* reports);
int mhdgb_ensemble_set_stop(mhdgb_ensemble* e, double tmax, long long max_steps);
int mhdgb_ensemble_time_steps(mhdgb_ensemble* e, int nsteps, double* ms);
int mhdgb_ensemble_select_variant(mhdgb_ensemble* e, int idx);
int mhdgb_ensemble_variant(const mhdgb_ensemble* e);
/* Times every compiled tile shape on the whole ensemble (states restored) and keeps the fastest. */
int mhdgb_ensemble_autotune(mhdgb_ensemble* e, int steps, int* best);

/* ---- allocation-free ghost fill ----
 * This entry point has no counterpart in the reference.  It performs SetBoundaryCondition
 * (boundary.cpp:750-893, single-rank fills) -- the same values as mhdgb_set_boundary, bit for bit --
 * on a primitive array that the caller owns, without a handle and without allocating device memory.
 * It is meant for callers that cannot let a library allocate on their call path: device memory under
 * a fixed budget or in the caller's own pool, or asynchronous work on other streams that the
 * device-wide synchronisation of cudaMalloc / cudaFree would stall.
 *
 * P      device pointer (on the current device) to the 12 primitive fields, element (n,k,j,i) at
 *        i + pitch*(n + 12*(j + (ny+5)*k)), i < nx+5 -- the reference's FieldArray layout when
 *        pitch = nx+5; pitch = 0 means nx+5.
 * nx..nz interior cells (each >= 2); bc: boundary_xin .. boundary_zout (MHDGB_BC_*).
 * stream a cudaStream_t (NULL: the legacy default stream).  The call only enqueues two kernels and
 *        returns; errors of the kernels themselves appear on that stream.
 *
 * Scratch: one fixed array of MHDGB_NOALLOC_SCRATCH_BYTES in the library's static device memory,
 * of which a call uses 1536*(nx+ny+nz+7) bytes; calls with nx+ny+nz > MHDGB_NOALLOC_MAX_EXTENT_SUM
 * return MHDGB_ERR_SCRATCH before touching the device.  No part of the scratch has to start at zero.
 * The first call on each device resolves the scratch address (cudaGetSymbolAddress, which also loads
 * the module): make that first call before any stream capture begins.  A device reset
 * (cudaDeviceReset) ends the context that address belongs to; the next call resolves it again, so
 * after a reset, too, make one call before capturing.  All calls on one device share
 * the one scratch array, so calls that overlap in time -- on different streams, or from several host
 * threads without ordering between their streams -- race on it and give wrong ghosts; order them. */
#define MHDGB_ERR_SCRATCH (-8) /* request larger than a fixed scratch area */
#define MHDGB_NOALLOC_SCRATCH_BYTES (4u << 20)
#define MHDGB_NOALLOC_MAX_EXTENT_SUM 2723
int mhdgb_fill_ghosts_noalloc(double* P, int nx, int ny, int nz, int pitch, const int* bc, void* stream);

/* ---- block decomposition (replaces the MPI topology and halo exchange of the reference) ----
 * The reference splits the grid over MPI ranks (MPI_Cart_create, mpi_config.cpp:61-69), exchanges
 * 2-deep primitive halos with its neighbours in SendRecvBoundary (boundary.cpp:222-318, 430-475,
 * 627-672, MPI_Waitall at :715) and reduces dt and c_h over ranks (MPIminfind / MPImaxfind,
 * mpi_config.cpp:83-99).  A block here is an ordinary handle whose faces shared with another block
 * have the kind MHDGB_BC_EXCHANGE.  Faces are numbered 0..5 = x-in, x-out, y-in, y-out, z-in, z-out;
 * a halo is the 12 primitives of the 2 cell layers next to a face over the face's interior extent,
 * ordered i fastest, then j, k and the variable.  Only that extent is exchanged: the solver never
 * reads the edge and corner ghosts.
 *
 * Per handle (one process per GPU, the caller's own transport, e.g. MPI or NCCL): after
 * mhdgb_prepare or a step, pack the layers next to each exchanged face, send them to the
 * neighbour, unpack what the neighbours sent into the ghost layers, replace the pending reduction
 * by its minimum / maximum over all blocks, and step once; repeat.
 * mhdgb_halo_bytes   bytes of face f's halo: 4-byte elements for a mixed handle prepared for fused
 *                    steps, 8-byte elements otherwise (the FP64 forms, and the stage path, which
 *                    works on FP64 primitives);
 * mhdgb_halo_pack    copies the 2 interior layers next to face f into buf (device memory, or mapped
 *                    page-locked host memory); mhdgb_halo_unpack copies buf into the 2 ghost layers
 *                    beyond face f.  Both act on the primitives the next fused step reads (or, if
 *                    the handle is not prepared for fused steps, on the stage path's) and return
 *                    once the copy is done;
 * mhdgb_get_reduction / mhdgb_set_reduction  read / replace the pending reduction of the next fused
 *                    step: the minimum over the block of the cell CFL time (dt = cfl * dtmin) and
 *                    the maximum signal speed (c_h).  The stage path reduces with
 *                    mhdgb_control_timestep / mhdgb_evaluate_ch and takes the global values through
 *                    mhdgb_set_dt / mhdgb_set_chg. */
size_t mhdgb_halo_bytes(const mhdgb_solver* h, int face);
int mhdgb_halo_pack(mhdgb_solver* h, int face, void* buf);
int mhdgb_halo_unpack(mhdgb_solver* h, int face, const void* buf);
int mhdgb_get_reduction(mhdgb_solver* h, double* dtmin, double* chmax);
int mhdgb_set_reduction(mhdgb_solver* h, double dtmin, double chmax);

/* A domain: one grid cut into ntiles[0] x ntiles[1] x ntiles[2] blocks inside one process.
 * Block b has coordinates (b / (nt1*nt2), (b / nt2) % nt1, b % nt2), the row-major rank order of
 * MPI_Cart_create; along each axis the first (n % nt) blocks take one cell more than the others.
 * Each block takes its cell faces from the whole grid (so results do not depend on the split:
 * a decomposed run equals the single-grid run bit for bit; the reference's ranks instead compute
 * their own faces from their extent, main.cpp:35-64, which can differ in the last bit).
 * Block b belongs to group b % ngroups, run on devices[b % ngroups] (ngroups = 0: one group on
 * cfg->device).  Each step, each group advances its blocks in one persistent launch of the fused
 * kernel; then, after every group's launch, each group copies the halos of its blocks' exchanged
 * faces straight from the neighbouring blocks' primitives (over NVLink when the neighbour is on
 * another GPU; peer access is enabled at creation) and reduces dt and c_h over all blocks.  Nothing
 * returns to the host between steps; a one-group domain captures its steps in CUDA graphs.
 * Requirements: spacing_quirk = 0, at least 2 cells per block and axis, boundary kinds 1..3.
 * Whole-grid arrays are in the reference layout with the whole grid's extents. */
typedef struct mhdgb_domain mhdgb_domain;
int mhdgb_domain_create(const mhdgb_config* cfg, const int ntiles[3], int ngroups, const int* devices,
                        mhdgb_domain** out);
int mhdgb_domain_destroy(mhdgb_domain* d);
const char* mhdgb_domain_last_error(const mhdgb_domain* d);
int mhdgb_domain_blocks(const mhdgb_domain* d);
/* Block b's handle (owned by the domain) and its first interior cell / extent in the whole grid. */
int mhdgb_domain_block(mhdgb_domain* d, int b, mhdgb_solver** h, int offset[3], int extent[3]);
int mhdgb_domain_upload_cons(mhdgb_domain* d, const double* U);
/* Writes the interior cells of the whole-grid array U; its ghost cells are left as they are. */
int mhdgb_domain_download_cons(mhdgb_domain* d, double* U);
/* The KH state of mhdgb_init_kh on the whole grid (the noise of a cell depends on its whole-grid
 * index, not on the split). */
int mhdgb_domain_init_kh(mhdgb_domain* d, unsigned long long seed, double vshear, double width, double bx,
                         double amp, double sig, double noise);
int mhdgb_domain_prepare(mhdgb_domain* d);
int mhdgb_domain_step(mhdgb_domain* d, int nsteps);
/* Waits for the steps; the report is block 0's (every block has the same step, time, dt and c_h)
 * with the status bits of all blocks. */
int mhdgb_domain_sync(mhdgb_domain* d, mhdgb_report* report);
int mhdgb_domain_set_stop(mhdgb_domain* d, double tmax, long long max_steps);
int mhdgb_domain_time_steps(mhdgb_domain* d, int nsteps, double* ms);
/* KH diagnostic of the whole grid (blocks' volume-weighted sums recombined; equal to the
 * single-grid diagnostic up to the order of the sums). */
int mhdgb_domain_diag(mhdgb_domain* d, double out[3]);

#ifdef __cplusplus
}
#endif
#endif
