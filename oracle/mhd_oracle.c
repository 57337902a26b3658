/*
 * mhd_oracle.c -- CPU restatement of the MHDTurbulence FP64 solver step.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle).  Nothing in the shipped library links or calls this
 * file; tests/, __graft_entry__.smoke() and bench.py's CPU legs use it as the reference for
 * comparisons and as the timed CPU baseline ("port").
 *
 * Every function restates one stage of the reference's src_cpp_kokkos_host path with the same
 * floating-point operation order (left-to-right evaluation as in the C++ source), so that built
 * with -ffp-contract=off it reproduces the reference bit for bit.  That claim is pinned by
 * tests/test_oracle_golden.py against vectors produced by the reference sources themselves
 * (oracle/refshim/, compiled from the reference tree against a small Kokkos/MPI shim).
 *
 * std::min / std::max semantics are kept exactly:  std::min(a,b) = (b<a)?b:a,
 * std::max(a,b) = (a<b)?b:a, and the initializer-list forms return the first extreme element.
 */
#include "mhd_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* primitive indices, src_cpp_kokkos_host/mhd.hpp:250-253 */
enum { nden = 0, nve1 = 1, nve2 = 2, nve3 = 3, nene = 4, npre = 5, ncsp = 6,
       nbm1 = 7, nbm2 = 8, nbm3 = 9, nbps = 10, nst = 11, nprim = 12 };
/* conserved / flux-vector indices, mhd.hpp:255-268 */
enum { mconsv = 10, madd = 3,
       mudn = 0, muvu = 1, muvv = 2, muvw = 3, muet = 4, mubu = 5, mubv = 6, mubw = 7, mubp = 8,
       must = 9,
       mfdn = 10, mfvu = 11, mfvv = 12, mfvw = 13, mfet = 14, mfbu = 15, mfbv = 16, mfbw = 17,
       mfbp = 18, mfst = 19, mcsp = 20, mvel = 21, mpre = 22, nvec = 23 };
enum { mden = 0, mrv1 = 1, mrv2 = 2, mrv3 = 3, meto = 4, mbm1 = 5, mbm2 = 6, mbm3 = 7, mbps = 8,
       mrvu = 1, mrvv = 2, mrvw = 3, mbmu = 5, mbmv = 6, mbmw = 7, mst = 9 };

#define SMIN(a, b) (((b) < (a)) ? (b) : (a)) /* std::min */
#define SMAX(a, b) (((a) < (b)) ? (b) : (a)) /* std::max */

static inline size_t ix(const orc_grid *g, int nv, int n, int k, int j, int i) {
  return (size_t)i + (size_t)g->itot * ((size_t)n + (size_t)nv * ((size_t)j + (size_t)g->jtot * (size_t)k));
}

void orc_grid_init(orc_grid *g, int nx, int ny, int nz) {
  g->nx = nx; g->ny = ny; g->nz = nz;
  g->itot = nx + 2 * ORC_NGH + 1;
  g->jtot = ny + 2 * ORC_NGH + 1;
  g->ktot = nz + 2 * ORC_NGH + 1;
  g->riemann = 0;
}

/* GenerateGrid, src_cpp_kokkos_host/main.cpp:35-44 (single rank: coords = 0, ntiles = 1). */
void orc_generate_axis(double *xa, int n, double xmin, double xmax) {
  const int ngh = ORC_NGH, is = ngh, ie = is + n - 1;
  double xminloc = xmin + (xmax - xmin) / 1 * 0;
  double xmaxloc = xmin + (xmax - xmin) / 1 * (0 + 1);
  double dx = (xmaxloc - xminloc) / (double)n;
  for (int i = is - ngh; i <= ie + ngh + 1; i++) xa[i] = dx * (i - (ngh + 1)) + xminloc;
}

/* vanLeer, src_cpp_kokkos_host/mhd.cpp:89-95 */
static inline double van_leer(double dsvp, double dsvm) {
  if (dsvp * dsvm > 0.0) return 2.0 * dsvp * dsvm / (dsvp + dsvm);
  return 0.0;
}

/* HLLD, src_cpp_kokkos_host/mhd.cpp:97-417 */
static void hlld(const double *leftst, const double *rigtst, double *nflux) {
  const double eps = 1.0e-30;
  double rol = leftst[mudn], eel = leftst[muet];
  double rxl = leftst[muvu], ryl = leftst[muvv], rzl = leftst[muvw];
  double vxl = leftst[muvu] / leftst[mudn];
  double vyl = leftst[muvv] / leftst[mudn];
  double vzl = leftst[muvw] / leftst[mudn];
  double byl = leftst[mubv], bzl = leftst[mubw], ptl = leftst[mpre];
  double scl = leftst[mst];

  double ror = rigtst[mudn], eer = rigtst[muet];
  double rxr = rigtst[muvu], ryr = rigtst[muvv], rzr = rigtst[muvw];
  double vxr = rigtst[muvu] / rigtst[mudn];
  double vyr = rigtst[muvv] / rigtst[mudn];
  double vzr = rigtst[muvw] / rigtst[mudn];
  double byr = rigtst[mubv], bzr = rigtst[mubw], ptr = rigtst[mpre];
  double scr = rigtst[mst];

  /* Step 1 (mhd.cpp:212-216) */
  double cfl = leftst[mcsp], cfr = rigtst[mcsp];
  double sl = SMIN(vxl, vxr) - SMAX(cfl, cfr);
  double sr = SMAX(vxl, vxr) + SMAX(cfl, cfr);

  /* Step 2 (mhd.cpp:221-243) */
  double frol = leftst[mfdn], feel = leftst[mfet], frxl = leftst[mfvu], fryl = leftst[mfvv];
  double frzl = leftst[mfvw], fbyl = leftst[mfbv], fbzl = leftst[mfbw], fscl = leftst[mfst];
  double fror = rigtst[mfdn], feer = rigtst[mfet], frxr = rigtst[mfvu], fryr = rigtst[mfvv];
  double frzr = rigtst[mfvw], fbyr = rigtst[mfbv], fbzr = rigtst[mfbw], fscr = rigtst[mfst];

  /* Step 4 (mhd.cpp:248-258) */
  double sdl = SMIN(-1e-20, sl - vxl);
  double sdr = SMAX(1e-20, sr - vxr);
  double rosdl = rol * sdl;
  double rosdr = ror * sdr;
  double temp = 1.0 / (rosdr - rosdl);
  double sm = (rosdr * vxr - rosdl * vxl - ptr + ptl) * temp;
  double sdml = SMIN(-1e-20, sl - sm);
  double isdml = 1.0 / sdml;
  double sdmr = SMAX(1e-20, sr - sm);
  double isdmr = 1.0 / sdmr;

  /* Step 5 (mhd.cpp:264) */
  double ptst = (rosdr * ptl - rosdl * ptr + rosdl * rosdr * (vxr - vxl)) * temp;

  /* Step 5A (mhd.cpp:269-300) */
  double bxs = 0.5 * (leftst[mubu] + rigtst[mubu]);
  double bxsq = bxs * bxs;
  double temp_fst = rosdl * sdml - bxsq;
  double sign1 = copysign(1.0, fabs(temp_fst) - eps);
  double maxs1 = SMAX(0.0, sign1);
  double mins1 = SMIN(0.0, sign1);
  double itf = 1.0 / (temp_fst + mins1);
  temp = bxs * (sdl - sdml) * itf;
  double rolst = maxs1 * (rosdl * isdml) - mins1 * rol;
  double sclst = rolst / rol * scl;
  double vxlst = maxs1 * sm - mins1 * vxl;
  double rxlst = rolst * vxlst;
  double vylst = maxs1 * (vyl - byl * temp) - mins1 * vyl;
  double rylst = rolst * vylst;
  double vzlst = maxs1 * (vzl - bzl * temp) - mins1 * vzl;
  double rzlst = rolst * vzlst;
  temp = (rosdl * sdl - bxsq) * itf;
  double bylst = maxs1 * (byl * temp) - mins1 * byl;
  double bzlst = maxs1 * (bzl * temp) - mins1 * bzl;
  double vdbstl = vxlst * bxs + vylst * bylst + vzlst * bzlst;
  double eelst = maxs1 * (sdl * eel - ptl * vxl + ptst * sm +
                          bxs * (vxl * bxs + vyl * byl + vzl * bzl - vdbstl)) * isdml
                 - mins1 * eel;

  /* Step 5B (mhd.cpp:305-333) */
  temp_fst = rosdr * sdmr - bxsq;
  sign1 = copysign(1.0, fabs(temp_fst) - eps);
  maxs1 = SMAX(0.0, sign1);
  mins1 = SMIN(0.0, sign1);
  itf = 1.0 / (temp_fst + mins1);
  temp = bxs * (sdr - sdmr) * itf;
  double rorst = maxs1 * (rosdr * isdmr) - mins1 * ror;
  double scrst = rorst / ror * scr;
  double vxrst = maxs1 * sm - mins1 * vxr;
  double rxrst = rorst * vxrst;
  double vyrst = maxs1 * (vyr - byr * temp) - mins1 * vyr;
  double ryrst = rorst * vyrst;
  double vzrst = maxs1 * (vzr - bzr * temp) - mins1 * vzr;
  double rzrst = rorst * vzrst;
  temp = (rosdr * sdr - bxsq) * itf;
  double byrst = maxs1 * (byr * temp) - mins1 * byr;
  double bzrst = maxs1 * (bzr * temp) - mins1 * bzr;
  double vdbstr = vxrst * bxs + vyrst * byrst + vzrst * bzrst;
  double eerst = maxs1 * ((sdr * eer - ptr * vxr + ptst * sm) * isdmr +
                          bxs * (vxr * bxs + vyr * byr + vzr * bzr - vdbstr) * isdmr)
                 - mins1 * eer;

  /* Step 5C (mhd.cpp:338-377) */
  double sqrtrol = sqrt(rolst);
  double sqrtror = sqrt(rorst);
  double abbx = fabs(bxs);
  double signbx = copysign(1.0, bxs);
  sign1 = copysign(1.0, abbx - eps);
  maxs1 = SMAX(0e0, sign1);
  mins1 = -SMIN(0e0, sign1);
  double invsumro = maxs1 / (sqrtrol + sqrtror);

  temp = invsumro * (sqrtrol * vylst + sqrtror * vyrst + signbx * (byrst - bylst));
  double vyldst = vylst * mins1 + temp;
  double ryldst = rylst * mins1 + rolst * temp;
  double ryrdst = ryrst * mins1 + rorst * temp;

  temp = invsumro * (sqrtrol * vzlst + sqrtror * vzrst + signbx * (bzrst - bzlst));
  double vzldst = vzlst * mins1 + temp;
  double rzldst = rzlst * mins1 + rolst * temp;
  double rzrdst = rzrst * mins1 + rorst * temp;

  temp = invsumro * (sqrtrol * byrst + sqrtror * bylst + signbx * sqrtrol * sqrtror * (vyrst - vylst));
  double byldst = bylst * mins1 + temp;
  double byrdst = byrst * mins1 + temp;

  temp = invsumro * (sqrtrol * bzrst + sqrtror * bzlst + signbx * sqrtrol * sqrtror * (vzrst - vzlst));
  double bzldst = bzlst * mins1 + temp;
  double bzrdst = bzrst * mins1 + temp;

  temp = sm * bxs + vyldst * byldst + vzldst * bzldst;
  double eeldst = eelst - sqrtrol * signbx * (vdbstl - temp) * maxs1;
  double eerdst = eerst + sqrtror * signbx * (vdbstr - temp) * maxs1;

  /* Step 6 (mhd.cpp:381-415) */
  double slst = (sm - abbx / sqrtrol) * maxs1;
  double srst = (sm + abbx / sqrtror) * maxs1;
  sign1 = copysign(1.0, sm);
  maxs1 = SMAX(0.0, sign1);
  mins1 = -SMIN(0.0, sign1);
  double msl = SMIN(sl, 0.0);
  double msr = SMAX(sr, 0.0);
  double mslst = SMIN(slst, 0.0);
  double msrst = SMAX(srst, 0.0);

  nflux[mden] = (frol + (rolst - rol) * msl) * maxs1 + (fror + (rorst - ror) * msr) * mins1;
  nflux[meto] = (feel + (eelst - eel) * msl + (eeldst - eelst) * mslst) * maxs1
              + (feer + (eerst - eer) * msr + (eerdst - eerst) * msrst) * mins1;
  nflux[mrvu] = (frxl + (rxlst - rxl) * msl) * maxs1 + (frxr + (rxrst - rxr) * msr) * mins1;
  nflux[mrvv] = (fryl + (rylst - ryl) * msl + (ryldst - rylst) * mslst) * maxs1
              + (fryr + (ryrst - ryr) * msr + (ryrdst - ryrst) * msrst) * mins1;
  nflux[mrvw] = (frzl + (rzlst - rzl) * msl + (rzldst - rzlst) * mslst) * maxs1
              + (frzr + (rzrst - rzr) * msr + (rzrdst - rzrst) * msrst) * mins1;
  nflux[mbmu] = 0e0;
  nflux[mbmv] = (fbyl + (bylst - byl) * msl + (byldst - bylst) * mslst) * maxs1
              + (fbyr + (byrst - byr) * msr + (byrdst - byrst) * msrst) * mins1;
  nflux[mbmw] = (fbzl + (bzlst - bzl) * msl + (bzldst - bzlst) * mslst) * maxs1
              + (fbzr + (bzrst - bzr) * msr + (bzrdst - bzrst) * msrst) * mins1;
  nflux[mst] = (fscl + (sclst - scl) * msl) * maxs1 + (fscr + (scrst - scr) * msr) * mins1;
  nflux[mbps] = 0.0; /* never read: the GLM pair overwrites it (mhd.cpp:1234-1237) */
}

/* HLLE, src_f90_acc_device/mhd.f90:877-907 (Fortran MIN/MAX written as std::min/std::max). */
static void hlle(const double *leftst, const double *rigtst, double *nflux) {
  const double csl = leftst[mcsp], csr = rigtst[mcsp];
  const double vl = leftst[mvel], vr = rigtst[mvel];
  double sl = SMIN(vl, vr) - SMAX(csl, csr);
  sl = SMIN(0.0, sl);
  double sr = SMAX(vl, vr) + SMAX(csl, csr);
  sr = SMAX(0.0, sr);
  for (int m = 0; m < mconsv; m++)
    nflux[m] = (sr * leftst[mconsv + m] - sl * rigtst[mconsv + m] + sl * sr * (rigtst[m] - leftst[m])) / (sr - sl);
}

/* HLLC, src_f90_acc_device/mhd.f90:909-1141.  The Fortran routine reads sclst, the passive-scalar
 * star state, without setting it; here it is scaled by rolst/rol like the transverse field. */
static void hllc(const double *leftst, const double *rigtst, double *nflux) {
  const double rol = leftst[mudn], eel = leftst[muet];
  const double rxl = leftst[muvu], ryl = leftst[muvv], rzl = leftst[muvw];
  const double vxl = leftst[muvu] / leftst[mudn], vyl = leftst[muvv] / leftst[mudn], vzl = leftst[muvw] / leftst[mudn];
  const double scl = leftst[must], byl = leftst[mubv], bzl = leftst[mubw], ptl = leftst[mpre];
  const double ror = rigtst[mudn], eer = rigtst[muet];
  const double rxr = rigtst[muvu], ryr = rigtst[muvv], rzr = rigtst[muvw];
  const double vxr = rigtst[muvu] / rigtst[mudn], vyr = rigtst[muvv] / rigtst[mudn], vzr = rigtst[muvw] / rigtst[mudn];
  const double scr = rigtst[must], byr = rigtst[mubv], bzr = rigtst[mubw], ptr = rigtst[mpre];
  const double cfl = leftst[mcsp], cfr = rigtst[mcsp];
  const double sl = SMIN(vxl, vxr) - SMAX(cfl, cfr);
  const double sr = SMAX(vxl, vxr) + SMAX(cfl, cfr);
  const double sdl = sl - vxl, sdr = sr - vxr;
  const double rosdl = rol * sdl, rosdr = ror * sdr;
  const double temp = 1.0 / (rosdr - rosdl);
  const double sm = (rosdr * vxr - rosdl * vxl - ptr + ptl) * temp;          /* eq. 45 */
  const double sdml = sl - sm, isdml = 1.0 / sdml;
  const double sdmr = sr - sm, isdmr = 1.0 / sdmr;
  const double ptst = (rosdr * ptl - rosdl * ptr + rosdl * rosdr * (vxr - vxl)) * temp;   /* eq. 49 */
  const double rolst = rol * sdl * isdml;
  const double rxlst = rolst * sm, rylst = rolst * vyl, rzlst = rolst * vzl;
  const double bylst = rolst / rol * byl, bzlst = rolst / rol * bzl, sclst = rolst / rol * scl;
  const double eelst = (sdl * eel - ptl * vxl + ptst * sm) * isdml;
  const double rorst = rosdr * isdmr;
  const double rxrst = rorst * sm, ryrst = rorst * vyr, rzrst = rorst * vzr;
  const double byrst = rorst / ror * byr, bzrst = rorst / ror * bzr, scrst = rorst / ror * scr;
  const double eerst = (sdr * eer - ptr * vxr + ptst * sm) * isdmr;
  const double sign1 = copysign(1.0, sm);
  const double maxs1 = SMAX(0.0, sign1), mins1 = -SMIN(0.0, sign1);
  const double msl = SMIN(sl, 0.0), msr = SMAX(sr, 0.0);
  nflux[mden] = (leftst[mfdn] + msl * (rolst - rol)) * maxs1 + (rigtst[mfdn] + msr * (rorst - ror)) * mins1;
  nflux[meto] = (leftst[mfet] + msl * (eelst - eel)) * maxs1 + (rigtst[mfet] + msr * (eerst - eer)) * mins1;
  nflux[mrvu] = (leftst[mfvu] + msl * (rxlst - rxl)) * maxs1 + (rigtst[mfvu] + msr * (rxrst - rxr)) * mins1;
  nflux[mrvv] = (leftst[mfvv] + msl * (rylst - ryl)) * maxs1 + (rigtst[mfvv] + msr * (ryrst - ryr)) * mins1;
  nflux[mrvw] = (leftst[mfvw] + msl * (rzlst - rzl)) * maxs1 + (rigtst[mfvw] + msr * (rzrst - rzr)) * mins1;
  nflux[mbmu] = 0.0;
  nflux[mbmv] = (leftst[mfbv] + msl * (bylst - byl)) * maxs1 + (rigtst[mfbv] + msr * (byrst - byr)) * mins1;
  nflux[mbmw] = (leftst[mfbw] + msl * (bzlst - bzl)) * maxs1 + (rigtst[mfbw] + msr * (bzrst - bzr)) * mins1;
  nflux[mbps] = 0.0;
  nflux[mst] = (leftst[mfst] + msl * (sclst - scl)) * maxs1 + (rigtst[mfst] + msr * (scrst - scr)) * mins1;
}

/* Direction maps of Prim2Cons1/2/3, src_cpp_kokkos_host/mhd.cpp:1078-1118. */
typedef struct dirmap {
  int muv1, muv2, muv3, mub1, mub2, mub3, mfv1, mfv2, mfv3, nved, nbmd, nvef, nbmf, nveb, nbmb;
} dirmap;
static const dirmap DMAP[3] = {
  {muvu, muvv, muvw, mubu, mubv, mubw, mfvu, mfvv, mfvw, nve1, nbm1, nve2, nbm2, nve3, nbm3},
  {muvw, muvu, muvv, mubw, mubu, mubv, mfvw, mfvu, mfvv, nve2, nbm2, nve3, nbm3, nve1, nbm1},
  {muvv, muvw, muvu, mubv, mubw, mubu, mfvv, mfvw, mfvu, nve3, nbm3, nve1, nbm1, nve2, nbm2},
};

/* Prim2ConsD, src_cpp_kokkos_host/mhd.cpp:997-1076 */
static void prim2cons(const double *Prim, double *Cons, const dirmap *d) {
  const double rho = Prim[nden];
  const double rhoinv = 1.0 / rho;
  const double vsq = Prim[nve1] * Prim[nve1] + Prim[nve2] * Prim[nve2] + Prim[nve3] * Prim[nve3];
  const double bsq = Prim[nbm1] * Prim[nbm1] + Prim[nbm2] * Prim[nbm2] + Prim[nbm3] * Prim[nbm3];
  Cons[mudn] = rho;
  Cons[d->muv1] = rho * Prim[nve1];
  Cons[d->muv2] = rho * Prim[nve2];
  Cons[d->muv3] = rho * Prim[nve3];
  Cons[muet] = rho * Prim[nene] + 0.5e0 * rho * vsq + 0.5e0 * bsq;
  Cons[d->mub1] = Prim[nbm1];
  Cons[d->mub2] = Prim[nbm2];
  Cons[d->mub3] = Prim[nbm3];
  Cons[mubp] = Prim[nbps];
  Cons[must] = rho * Prim[nst];
  double ptl = Prim[npre] + bsq / 2.0e0;
  Cons[mfdn] = rho * Prim[d->nved];
  Cons[d->mfv1] = rho * Prim[nve1] * Prim[d->nved] - Prim[nbm1] * Prim[d->nbmd];
  Cons[d->mfv2] = rho * Prim[nve2] * Prim[d->nved] - Prim[nbm2] * Prim[d->nbmd];
  Cons[d->mfv3] = rho * Prim[nve3] * Prim[d->nved] - Prim[nbm3] * Prim[d->nbmd];
  Cons[mfet] = (Cons[muet] + ptl) * Prim[d->nved] - bsq * Prim[d->nbmd];
  Cons[mfvu] += ptl;
  Cons[mfbu] = 0.0e0;
  Cons[mfbv] = Prim[d->nbmf] * Prim[d->nved] - Prim[d->nvef] * Prim[d->nbmd];
  Cons[mfbw] = Prim[d->nbmb] * Prim[d->nved] - Prim[d->nveb] * Prim[d->nbmd];
  Cons[mfbp] = 0.0e0;
  Cons[mfst] = rho * Prim[nst] * Prim[d->nved];
  double css = Prim[ncsp] * Prim[ncsp];
  double cts = css + bsq * rhoinv;
  Cons[mcsp] = sqrt((cts + sqrt(cts * cts - 4.0e0 * css * Prim[d->nbmd] * Prim[d->nbmd] * rhoinv)) / 2.0e0);
  Cons[mvel] = Prim[d->nved];
  Cons[mpre] = ptl;
}

/* CalcFlux, src_cpp_kokkos_host/mhd.cpp:1120-1158 */
static void calc_flux(const double *L1, const double *L2, const double *R1, const double *R2,
                      double *numflux, double *Cl, double *Cr, const dirmap *d, int riemann) {
  double Pl[nprim], Pr[nprim];
  for (int n = 0; n < nprim; n++) {
    double dsvp = R1[n] - L2[n];
    double dsvm = L2[n] - L1[n];
    Pl[n] = L2[n] + 0.5e0 * van_leer(dsvp, dsvm);
  }
  prim2cons(Pl, Cl, d);
  for (int n = 0; n < nprim; n++) {
    double dsvp = R2[n] - R1[n];
    double dsvm = R1[n] - L2[n];
    Pr[n] = R1[n] - 0.5e0 * van_leer(dsvp, dsvm);
  }
  prim2cons(Pr, Cr, d);
  if (riemann == 1) hlle(Cl, Cr, numflux);
  else if (riemann == 2) hllc(Cl, Cr, numflux);
  else hlld(Cl, Cr, numflux);
}

/* GetNumericalFluxD, src_cpp_kokkos_host/mhd.cpp:987-1410 (Flux1 1204-1241, Flux2 1287-1322,
 * Flux3 1370-1407).  dir is 1, 2 or 3. */
void orc_flux(int dir, const orc_grid *g, const double *P, double *F, double chg) {
  const int is = ORC_NGH, js = ORC_NGH, ks = ORC_NGH;
  const int ie = is + g->nx - 1, je = js + g->ny - 1, ke = ks + g->nz - 1;
  const int di = (dir == 1), dj = (dir == 2), dk = (dir == 3);
  const dirmap *d = &DMAP[dir - 1];
  /* output slots of the rotated HLLD vector, mhd.cpp:1225-1240 / 1306-1321 / 1391-1406 */
  int map_rv1, map_rv2, map_rv3, glm_b, map_b_a, map_b_b, src_b_a, src_b_b;
  if (dir == 1) {
    map_rv1 = mrvu; map_rv2 = mrvv; map_rv3 = mrvw; glm_b = mbm1;
    map_b_a = mbm2; src_b_a = mbmv; map_b_b = mbm3; src_b_b = mbmw;
  } else if (dir == 2) {
    map_rv1 = mrvw; map_rv2 = mrvu; map_rv3 = mrvv; glm_b = mbm2;
    map_b_a = mbm1; src_b_a = mbmw; map_b_b = mbm3; src_b_b = mbmv;
  } else {
    map_rv1 = mrvv; map_rv2 = mrvw; map_rv3 = mrvu; glm_b = mbm3;
    map_b_a = mbm1; src_b_a = mbmv; map_b_b = mbm2; src_b_b = mbmw;
  }
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = ks; k <= ke + dk; k++)
    for (int j = js; j <= je + dj; j++)
      for (int i = is; i <= ie + di; i++) {
        double L1[nprim], L2[nprim], R1[nprim], R2[nprim];
        double nf[mconsv], Cl[nvec], Cr[nvec];
        for (int n = 0; n < nprim; n++) {
          L1[n] = P[ix(g, nprim, n, k - 2 * dk, j - 2 * dj, i - 2 * di)];
          L2[n] = P[ix(g, nprim, n, k - dk, j - dj, i - di)];
          R1[n] = P[ix(g, nprim, n, k, j, i)];
          R2[n] = P[ix(g, nprim, n, k + dk, j + dj, i + di)];
        }
        calc_flux(L1, L2, R1, R2, nf, Cl, Cr, d, g->riemann);
        F[ix(g, mconsv, mden, k, j, i)] = nf[mden];
        F[ix(g, mconsv, mrv1, k, j, i)] = nf[map_rv1];
        F[ix(g, mconsv, mrv2, k, j, i)] = nf[map_rv2];
        F[ix(g, mconsv, mrv3, k, j, i)] = nf[map_rv3];
        F[ix(g, mconsv, meto, k, j, i)] = nf[meto];
        F[ix(g, mconsv, map_b_a, k, j, i)] = nf[src_b_a];
        F[ix(g, mconsv, map_b_b, k, j, i)] = nf[src_b_b];
        F[ix(g, mconsv, glm_b, k, j, i)] =
            0.5e0 * (Cl[mubp] + Cr[mubp]) - 0.5e0 * chg * (Cr[mubu] - Cl[mubu]);
        F[ix(g, mconsv, mbps, k, j, i)] =
            (0.5e0 * (Cl[mubu] + Cr[mubu]) - 0.5e0 / chg * (Cr[mubp] - Cl[mubp])) * chg * chg;
        F[ix(g, mconsv, mst, k, j, i)] = nf[mst];
      }
}

/* UpdateConservU, src_cpp_kokkos_host/mhd.cpp:1412-1444.  With spacing_quirk the y and z
 * spacings are taken at index i, as mhd.cpp:1435-1436 does. */
void orc_update_conserv(const orc_grid *g, const double *Fx, const double *Fy, const double *Fz,
                        double *U, double dt) {
  const int is = ORC_NGH, js = ORC_NGH, ks = ORC_NGH;
  const int ie = is + g->nx - 1, je = js + g->ny - 1, ke = ks + g->nz - 1;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = ks; k <= ke; k++)
    for (int j = js; j <= je; j++)
      for (int i = is; i <= ie; i++) {
        const int jy = g->spacing_quirk ? i : j;
        const int kz = g->spacing_quirk ? i : k;
        const double xinv = 1.0 / (g->x1a[i + 1] - g->x1a[i]);
        const double yinv = 1.0 / (g->x2a[jy + 1] - g->x2a[jy]);
        const double zinv = 1.0 / (g->x3a[kz + 1] - g->x3a[kz]);
        for (int m = 0; m < mconsv; m++) {
          size_t c = ix(g, mconsv, m, k, j, i);
          U[c] -= dt * ((Fx[ix(g, mconsv, m, k, j, i + 1)] - Fx[c]) * xinv
                      + (Fy[ix(g, mconsv, m, k, j + 1, i)] - Fy[c]) * yinv
                      + (Fz[ix(g, mconsv, m, k + 1, j, i)] - Fz[c]) * zinv);
        }
      }
}

/* UpdatePrimitvP, src_cpp_kokkos_host/mhd.cpp:1447-1509 */
void orc_update_prim(const orc_grid *g, const double *U, double *P) {
  const int is = ORC_NGH, js = ORC_NGH, ks = ORC_NGH;
  const int ie = is + g->nx - 1, je = js + g->ny - 1, ke = ks + g->nz - 1;
  const double gam = g->gam;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = ks; k <= ke; k++)
    for (int j = js; j <= je; j++)
      for (int i = is; i <= ie; i++) {
#define UU(m) U[ix(g, mconsv, (m), k, j, i)]
#define PP(n) P[ix(g, nprim, (n), k, j, i)]
        const double rho = UU(mden);
        const double rhoinv = 1.0 / rho;
        PP(nden) = rho;
        PP(nve1) = UU(mrv1) * rhoinv;
        PP(nve2) = UU(mrv2) * rhoinv;
        PP(nve3) = UU(mrv3) * rhoinv;
        double ekin = 0.5e0 * (UU(mrv1) * UU(mrv1) + UU(mrv2) * UU(mrv2) + UU(mrv3) * UU(mrv3)) * rhoinv;
        double emag = 0.5e0 * (UU(mbm1) * UU(mbm1) + UU(mbm2) * UU(mbm2) + UU(mbm3) * UU(mbm3));
        PP(nene) = (UU(meto) - ekin - emag) / UU(mden);
        PP(npre) = PP(nene) * PP(nden) * (gam - 1.0);
        PP(ncsp) = sqrt(PP(nene) * gam * (gam - 1.0));
        PP(nbm1) = UU(mbm1);
        PP(nbm2) = UU(mbm2);
        PP(nbm3) = UU(mbm3);
        PP(nbps) = UU(mbps);
        PP(nst) = UU(mst) * rhoinv;
#undef UU
#undef PP
      }
}

/* ControlTimestep, src_cpp_kokkos_host/mhd.cpp:1511-1561 (single rank: MPIminfind is the identity). */
double orc_control_timestep(const orc_grid *g, const double *P) {
  const int is = ORC_NGH, js = ORC_NGH, ks = ORC_NGH;
  const int ie = is + g->nx - 1, je = js + g->ny - 1, ke = ks + g->nz - 1;
  double dtminl = 1.0e90;
#pragma omp parallel
  {
    double loc = 1.0e90;
#pragma omp for collapse(2) schedule(static)
    for (int k = ks; k <= ke; k++)
      for (int j = js; j <= je; j++)
        for (int i = is; i <= ie; i++) {
#define PP(n) P[ix(g, nprim, (n), k, j, i)]
          double ctot = sqrt(PP(ncsp) * PP(ncsp)
                             + (PP(nbm1) * PP(nbm1) + PP(nbm2) * PP(nbm2) + PP(nbm3) * PP(nbm3)) / PP(nden));
          double a = (g->x1a[i + 1] - g->x1a[i]) / (fabs(PP(nve1)) + ctot);
          double b = (g->x2a[j + 1] - g->x2a[j]) / (fabs(PP(nve2)) + ctot);
          double c = (g->x3a[k + 1] - g->x3a[k]) / (fabs(PP(nve3)) + ctot);
          double dt = a;
          if (b < dt) dt = b;
          if (c < dt) dt = c;
          loc = SMIN(loc, dt);
#undef PP
        }
#pragma omp critical
    dtminl = SMIN(dtminl, loc);
  }
  return g->cfl * dtminl;
}

/* EvaluateCh, src_cpp_kokkos_host/mhd.cpp:1563-1611 */
double orc_evaluate_ch(const orc_grid *g, const double *P) {
  const int is = ORC_NGH, js = ORC_NGH, ks = ORC_NGH;
  const int ie = is + g->nx - 1, je = js + g->ny - 1, ke = ks + g->nz - 1;
  double chgloc = 0.0;
#pragma omp parallel
  {
    double loc = 0.0;
#pragma omp for collapse(2) schedule(static)
    for (int k = ks; k <= ke; k++)
      for (int j = js; j <= je; j++)
        for (int i = is; i <= ie; i++) {
#define PP(n) P[ix(g, nprim, (n), k, j, i)]
          double css = PP(ncsp) * PP(ncsp);
          double ca1 = PP(nbm1) * PP(nbm1) / PP(nden);
          double ca2 = PP(nbm2) * PP(nbm2) / PP(nden);
          double ca3 = PP(nbm3) * PP(nbm3) / PP(nden);
          double cts = css + ca1 + ca2 + ca3;
          double cm1 = sqrt((cts + sqrt(cts * cts - 4.0e0 * css * ca1)) / 2.0e0);
          double ch1 = (fabs(PP(nve1)) + cm1);
          double cm2 = sqrt((cts + sqrt(cts * cts - 4.0e0 * css * ca2)) / 2.0e0);
          double ch2 = (fabs(PP(nve2)) + cm2);
          double cm3 = sqrt((cts + sqrt(cts * cts - 4.0e0 * css * ca3)) / 2.0e0);
          double ch3 = (fabs(PP(nve3)) + cm3);
          double m = loc;
          if (m < ch1) m = ch1;
          if (m < ch2) m = ch2;
          if (m < ch3) m = ch3;
          loc = m;
#undef PP
        }
#pragma omp critical
    chgloc = SMAX(chgloc, loc);
  }
  return chgloc;
}

/* DampPsi, src_cpp_kokkos_host/mhd.cpp:1613-1633 */
void orc_damp_psi(const orc_grid *g, double *U, double dt, double chg) {
  const int is = ORC_NGH, js = ORC_NGH, ks = ORC_NGH;
  const int ie = is + g->nx - 1, je = js + g->ny - 1, ke = ks + g->nz - 1;
  const double alphabp = 0.1e0;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = ks; k <= ke; k++)
    for (int j = js; j <= je; j++)
      for (int i = is; i <= ie; i++) {
        double a = g->x1a[i + 1] - g->x1a[i];
        double b = g->x2a[j + 1] - g->x2a[j];
        double c = g->x3a[k + 1] - g->x3a[k];
        double dhl = a;
        if (b < dhl) dhl = b;
        if (c < dhl) dhl = c;
        double taui = alphabp * chg / dhl;
        size_t q = ix(g, mconsv, mbps, k, j, i);
        U[q] = U[q] * (1.0e0 - dt * taui);
      }
}

/* SetBoundaryCondition + the single-rank branch of SendRecvBoundary,
 * src_cpp_kokkos_host/boundary.cpp:750-893 and 106-747.  All three faces are packed from P
 * before any ghost is written (pack at 771-822, fill at 140-200 etc., unpack at 842-891), so
 * edge/corner ghosts keep values from before the call exactly as in the reference. */
void orc_set_boundary(const orc_grid *g, double *P) {
  const int ngh = ORC_NGH, is = ngh, js = ngh, ks = ngh;
  const int ie = is + g->nx - 1, je = js + g->ny - 1, ke = ks + g->nz - 1;
  const int it = g->itot, jt = g->jtot, kt = g->ktot;
  const size_t sx = (size_t)nprim * kt * jt * ngh, sy = (size_t)nprim * kt * ngh * it,
               sz = (size_t)nprim * ngh * jt * it;
  double *bsx_s = malloc(sx * sizeof(double)), *bsx_e = malloc(sx * sizeof(double));
  double *bsy_s = malloc(sy * sizeof(double)), *bsy_e = malloc(sy * sizeof(double));
  double *bsz_s = malloc(sz * sizeof(double)), *bsz_e = malloc(sz * sizeof(double));
#define BX(n, k, j, i) ((((size_t)(n) * kt + (k)) * jt + (j)) * ngh + (i))
#define BY(n, k, j, i) ((((size_t)(n) * kt + (k)) * ngh + (j)) * it + (i))
#define BZ(n, k, j, i) ((((size_t)(n) * ngh + (k)) * jt + (j)) * it + (i))
  /* pack (boundary.cpp:771-822) */
  for (int n = 0; n < nprim; n++)
    for (int k = 0; k < kt; k++)
      for (int j = 0; j < jt; j++)
        for (int i = 0; i < ngh; i++) {
          bsx_s[BX(n, k, j, i)] = P[ix(g, nprim, n, k, j, ie - ngh + 1 + i)];
          bsx_e[BX(n, k, j, i)] = P[ix(g, nprim, n, k, j, is + i)];
        }
  for (int n = 0; n < nprim; n++)
    for (int k = 0; k < kt; k++)
      for (int j = 0; j < ngh; j++)
        for (int i = 0; i < it; i++) {
          bsy_s[BY(n, k, j, i)] = P[ix(g, nprim, n, k, je - ngh + 1 + j, i)];
          bsy_e[BY(n, k, j, i)] = P[ix(g, nprim, n, k, js + j, i)];
        }
  for (int n = 0; n < nprim; n++)
    for (int k = 0; k < ngh; k++)
      for (int j = 0; j < jt; j++)
        for (int i = 0; i < it; i++) {
          bsz_s[BZ(n, k, j, i)] = P[ix(g, nprim, n, ke - ngh + 1 + k, j, i)];
          bsz_e[BZ(n, k, j, i)] = P[ix(g, nprim, n, ks + k, j, i)];
        }
  /* fill + unpack, x then y then z (boundary.cpp:140-200 etc., 842-891).  For each ghost
   * layer the source is: periodic -> the opposite side's send buffer at the same offset;
   * reflection -> this side's mirrored layer with the normal velocity negated;
   * outflow -> the first interior layer on this side. */
  const int bxi = g->bc[0], bxo = g->bc[1], byi = g->bc[2], byo = g->bc[3], bzi = g->bc[4], bzo = g->bc[5];
  for (int n = 0; n < nprim; n++)
    for (int k = 0; k < kt; k++)
      for (int j = 0; j < jt; j++)
        for (int i = 0; i < ngh; i++) {
          double vin = 0.0, vout = 0.0;
          if (bxi == ORC_BC_PERIODIC) vin = bsx_s[BX(n, k, j, i)];
          else if (bxi == ORC_BC_REFLECTION) { vin = bsx_e[BX(n, k, j, ngh - 1 - i)]; if (n == nve1) vin = -vin; }
          else if (bxi == ORC_BC_OUTFLOW) vin = bsx_e[BX(n, k, j, 0)];
          if (bxo == ORC_BC_PERIODIC) vout = bsx_e[BX(n, k, j, i)];
          else if (bxo == ORC_BC_REFLECTION) { vout = bsx_s[BX(n, k, j, ngh - 1 - i)]; if (n == nve1) vout = -vout; }
          else if (bxo == ORC_BC_OUTFLOW) vout = bsx_s[BX(n, k, j, ngh - 1)];
          P[ix(g, nprim, n, k, j, is - ngh + i)] = vin;
          P[ix(g, nprim, n, k, j, ie + 1 + i)] = vout;
        }
  for (int n = 0; n < nprim; n++)
    for (int k = 0; k < kt; k++)
      for (int j = 0; j < ngh; j++)
        for (int i = 0; i < it; i++) {
          double vin = 0.0, vout = 0.0;
          if (byi == ORC_BC_PERIODIC) vin = bsy_s[BY(n, k, j, i)];
          else if (byi == ORC_BC_REFLECTION) { vin = bsy_e[BY(n, k, ngh - 1 - j, i)]; if (n == nve2) vin = -vin; }
          else if (byi == ORC_BC_OUTFLOW) vin = bsy_e[BY(n, k, 0, i)];
          if (byo == ORC_BC_PERIODIC) vout = bsy_e[BY(n, k, j, i)];
          else if (byo == ORC_BC_REFLECTION) { vout = bsy_s[BY(n, k, ngh - 1 - j, i)]; if (n == nve2) vout = -vout; }
          else if (byo == ORC_BC_OUTFLOW) vout = bsy_s[BY(n, k, ngh - 1, i)];
          P[ix(g, nprim, n, k, js - ngh + j, i)] = vin;
          P[ix(g, nprim, n, k, je + 1 + j, i)] = vout;
        }
  for (int n = 0; n < nprim; n++)
    for (int k = 0; k < ngh; k++)
      for (int j = 0; j < jt; j++)
        for (int i = 0; i < it; i++) {
          double vin = 0.0, vout = 0.0;
          if (bzi == ORC_BC_PERIODIC) vin = bsz_s[BZ(n, k, j, i)];
          else if (bzi == ORC_BC_REFLECTION) { vin = bsz_e[BZ(n, ngh - 1 - k, j, i)]; if (n == nve3) vin = -vin; }
          else if (bzi == ORC_BC_OUTFLOW) vin = bsz_e[BZ(n, 0, j, i)];
          if (bzo == ORC_BC_PERIODIC) vout = bsz_e[BZ(n, k, j, i)];
          else if (bzo == ORC_BC_REFLECTION) { vout = bsz_s[BZ(n, ngh - 1 - k, j, i)]; if (n == nve3) vout = -vout; }
          else if (bzo == ORC_BC_OUTFLOW) vout = bsz_s[BZ(n, ngh - 1, j, i)];
          P[ix(g, nprim, n, ks - ngh + k, j, i)] = vin;
          P[ix(g, nprim, n, ke + 1 + k, j, i)] = vout;
        }
#undef BX
#undef BY
#undef BZ
  free(bsx_s); free(bsx_e); free(bsy_s); free(bsy_e); free(bsz_s); free(bsz_e);
}

/* One step in the order of src_cpp_kokkos_host/main.cpp:229-259. */
void orc_step(const orc_grid *g, double *U, double *P, double *Fx, double *Fy, double *Fz,
              double *dt_out, double *chg_out) {
  double dt = orc_control_timestep(g, P);
  orc_set_boundary(g, P);
  double chg = orc_evaluate_ch(g, P);
  orc_flux(1, g, P, Fx, chg);
  orc_flux(2, g, P, Fy, chg);
  orc_flux(3, g, P, Fz, chg);
  orc_update_conserv(g, Fx, Fy, Fz, U, dt);
  orc_damp_psi(g, U, dt, chg);
  orc_update_prim(g, U, P);
  if (dt_out) *dt_out = dt;
  if (chg_out) *chg_out = chg;
}

double orc_run(const orc_grid *g, double *U, double *P, int nsteps, double *dts, double *chgs) {
  size_t nf = (size_t)mconsv * g->itot * g->jtot * g->ktot;
  double *Fx = calloc(nf, sizeof(double)), *Fy = calloc(nf, sizeof(double)), *Fz = calloc(nf, sizeof(double));
  double t = 0.0;
  for (int s = 0; s < nsteps; s++) {
    double dt, chg;
    orc_step(g, U, P, Fx, Fy, Fz, &dt, &chg);
    if (dts) dts[s] = dt;
    if (chgs) chgs[s] = chg;
    t += dt;
  }
  free(Fx); free(Fy); free(Fz);
  return t;
}

/* RealTimeAnalysis, src_cpp_kokkos_device/main.cpp:26-84 (sums over k-planes in order). */
void orc_diag(const orc_grid *g, const double *P, double out[3]) {
  const int is = ORC_NGH, js = ORC_NGH, ks = ORC_NGH;
  const int ie = is + g->nx - 1, je = js + g->ny - 1, ke = ks + g->nz - 1;
  double vol = 0.0, mix = 0.0, avevy = 0.0;
  for (int k = ks; k <= ke; k++)
    for (int j = js; j <= je; j++)
      for (int i = is; i <= ie; i++) {
        const double dv = (g->x1a[i + 1] - g->x1a[i]) * (g->x2a[j + 1] - g->x2a[j]) * (g->x3a[k + 1] - g->x3a[k]);
        const double X = P[ix(g, nprim, nst, k, j, i)];
        const double vy = P[ix(g, nprim, nve2, k, j, i)];
        vol += dv;
        mix += X * (1.0 - X) * dv;
        avevy += vy * vy * dv;
      }
  out[0] = vol;
  out[1] = mix / vol;
  out[2] = sqrt(avevy / vol);
}

void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

int orc_get_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
