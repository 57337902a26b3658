/*
 * mhd_oracle.h -- CPU restatement of the MHDTurbulence solver step (test infrastructure).
 *
 * THIS IS THE ORACLE, NOT THE PRODUCT.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline / reference legs may load it.  It restates, operation for operation, the FP64
 * arithmetic of the reference's src_cpp_kokkos_host path so that its results can be compared
 * bit for bit with the reference (pinned by the golden vectors under tests/golden/, which were
 * produced by the reference's own mhd.cpp/boundary.cpp compiled here) and within tolerance with
 * the CUDA path.
 *
 * Array layout is the reference FieldArray layout (src_cpp_kokkos_host/mhd.hpp:186-245,
 * View(n1,nv,n2,n3) LayoutLeft):  element (n,k,j,i) lives at  i + itot*(n + nv*(j + jtot*k)).
 * Extents are itot = nx + 2*ngh + 1 etc. (src_cpp_kokkos_host/config.hpp:57-59), ngh = 2.
 */
#ifndef MHD_ORACLE_H_
#define MHD_ORACLE_H_

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_NGH = 2, ORC_NPRIM = 12, ORC_NCONS = 10 };
enum { ORC_BC_PERIODIC = 1, ORC_BC_REFLECTION = 2, ORC_BC_OUTFLOW = 3 };

typedef struct orc_grid {
  int nx, ny, nz;          /* interior cells (ngrid1..3) */
  int itot, jtot, ktot;    /* allocated extents incl. ghosts: n + 2*ngh + 1 */
  double gam;              /* adiabatic index (hydflux_mod::gam) */
  double cfl;              /* dt = cfl * min(...); the reference hard-codes 0.05 */
  int bc[6];               /* xin, xout, yin, yout, zin, zout (1 periodic, 2 reflection, 3 outflow) */
  int spacing_quirk;       /* 1: UpdateConservU takes y/z spacings at index i, as mhd.cpp:1435-1436 */
  const double *x1a, *x2a, *x3a;  /* cell-face coordinates, length itot / jtot / ktot */
  int riemann;             /* 0 HLLD (mhd.cpp:97-417), 1 HLLE, 2 HLLC (src_f90_acc_device/mhd.f90:877-1141) */
} orc_grid;

/* Fill extents from nx,ny,nz (call before use). */
void orc_grid_init(orc_grid *g, int nx, int ny, int nz);
/* GenerateGrid (main.cpp:26-65) for one rank covering [xmin,xmax]: writes x?a of length ?tot. */
void orc_generate_axis(double *xa, int n, double xmin, double xmax);

/* Stages (all FP64).  P has 12 fields, U and F have 10. */
void orc_flux(int dir, const orc_grid *g, const double *P, double *F, double chg);
void orc_update_conserv(const orc_grid *g, const double *Fx, const double *Fy,
                        const double *Fz, double *U, double dt);
void orc_update_prim(const orc_grid *g, const double *U, double *P);
double orc_control_timestep(const orc_grid *g, const double *P);   /* returns dt */
double orc_evaluate_ch(const orc_grid *g, const double *P);        /* returns chg */
void orc_damp_psi(const orc_grid *g, double *U, double dt, double chg);
void orc_set_boundary(const orc_grid *g, double *P);

/* One full step in the order of main.cpp:229-259.  F is scratch (3 x 10 fields).
 * Writes dt and chg of the step. */
void orc_step(const orc_grid *g, double *U, double *P, double *Fx, double *Fy, double *Fz,
              double *dt_out, double *chg_out);
/* nsteps steps; dts/chgs may be NULL or arrays of nsteps. Returns the summed dt. */
double orc_run(const orc_grid *g, double *U, double *P, int nsteps, double *dts, double *chgs);

/* KH diagnostic (src_cpp_kokkos_device/main.cpp:26-84): out = {vol, mix, sqrt(<vy^2>)}. */
void orc_diag(const orc_grid *g, const double *P, double out[3]);

/* Thread control for the timed CPU baseline (0 = leave OpenMP default). */
void orc_set_threads(int n);
int orc_get_threads(void);

#ifdef __cplusplus
}
#endif
#endif
