// fused.cuh -- the fused solver step: one persistent launch per time step.
//
// Work decomposition.  The interior is cut into column tiles of TX x TY cells, each split along z
// into chunks of kc planes; a (tile, chunk) pair is one work item and CTAs pull items from a queue
// in the control block.  A CTA marches through its chunk plane by plane:
//   * a 4-slot shared-memory ring receives planes of P (12 primitives, the tile plus 2 halo cells
//     in x and y) through 4-D TMA tensor loads completing on per-slot mbarriers; plane k+4 is
//     requested when plane k is retired, so each load has a whole plane of compute to land;
//   * phase A: every limited slope the plane needs (van Leer, once per cell and direction): x and y
//     slopes of plane k and the z slope of plane k+1, one work list;
//   * phase B: every face flux of the plane (prim->cons, HLLD, GLM): x and y faces of plane k and
//     the z face k+1/2, one work list;
//   * phase C: each cell thread completes U -= dt*(dFx*xinv + dFy*yinv + dFz*zinv) (the
//     reference's rounding order, mhd.cpp:1438-1440), damps psi (mhd.cpp:1630), recovers P
//     (mhd.cpp:1483-1506) into the other P buffer together with the ghost images the next step
//     needs, and folds the next step's dt / c_h candidates (mhd.cpp:1542-1550, 1589-1601) into a
//     block reduction; the lower z-face flux of its column stays in registers.
// The slope list is padded per direction to whole warps (no warp mixes two code paths) and handed
// out per warp from a shared counter; the face list is one unpadded list over all directions,
// each face read in its rotated frame by direction-generic code.  Masked-off lanes cost the FP64
// pipe as much as active ones, so padding is paid for in full.  In the FP64 form the warps that
// own no cell start the next plane's phase A as soon as their own faces are formed (a named
// barrier that only the owner warps wait at), into a second x/y slope buffer and a third z-slope
// buffer, so their FP64 pipe does not idle while the last faces are formed.
// Step n reads dt and c_h from ctrl->slot[n%3] (made by step n-1 or by the initial reduction),
// reduces into slot[(n+1)%3] and resets slot[(n+2)%3]; the last CTA to finish advances the step
// counter and the simulated time.  All launches of a run are identical and can be captured once in
// a CUDA graph.
//
// R is the arithmetic type of reconstruction, Riemann solve and the P buffers: double for the FP64
// form, float for the mixed form (whose fastest variant, k_fused_step_fs in fused_fs.cuh, forms the
// slopes inside the face phase instead).  The conserved state U and its update are FP64 in both forms; in
// the mixed form the flux-divergence terms are summed with compensation (TwoProd/TwoSum in FP32) and
// the pressure recovery e = (E - m^2/(2 rho) - B^2/2)/rho is FP64 (with 1/rho from an FP32 seed and
// one FP64 Newton step).
#pragma once

#include <cstdio>

#include "common.cuh"
#include "fused_args.h"
#include "mhd_physics.cuh"

namespace mhdgb {

// Bytes of the fused kernel's shared memory for nslb x/y slope buffers (see FusedSmem).
constexpr size_t fused_smem_bytes(int TX, int TY, size_t rsz, int nslb) {
  const size_t PLANE = (size_t)(TX + 4) * NPRIM * (TY + 4);
  const size_t NSLX = (size_t)NPRIM * TY * (TX + 2), NSLY = (size_t)NPRIM * (TY + 2) * TX,
               NSLZ = (size_t)NPRIM * TY * TX;
  const size_t NFX = (size_t)NCONS * TY * (TX + 1), NFY = (size_t)NCONS * (TY + 1) * TX, NFZ = (size_t)NCONS * TY * TX;
  auto a16 = [](size_t x) { return (x + 15) / 16 * 16; };
  return (4 * PLANE * rsz + 127) / 128 * 128 + nslb * (a16(NSLX * rsz) + a16(NSLY * rsz)) + a16(3 * NSLZ * rsz) +
         a16(NFX * rsz) + a16(NFY * rsz) + a16(NFZ * rsz) + 64 * sizeof(double) + 4 * sizeof(uint64_t) + 16 + 128;
}

template <class R, int TX, int TY, int NT, int MINB = 1>
struct FusedSmem {
  static constexpr int NBUF = 4;
  static constexpr int PX = TX + 4, PY = TY + 4;
  static constexpr int PLANE = PX * NPRIM * PY;             // elements of one ring plane
  static constexpr int NSLX = NPRIM * TY * (TX + 2);        // x slopes, cells i in [-1, TX]
  static constexpr int NSLY = NPRIM * (TY + 2) * TX;        // y slopes, cells j in [-1, TY]
  static constexpr int NSLZ = NPRIM * TY * TX;              // z slopes of one plane
  static constexpr int NFX = NCONS * TY * (TX + 1);         // x faces i in [0, TX]
  static constexpr int NFY = NCONS * (TY + 1) * TX;         // y faces j in [0, TY]
  static constexpr int NFZ = NCONS * TY * TX;               // z faces k+1/2
  // Owner threads: the whole warps that hold the tile's cell columns.  OV: the warps without a
  // column start the next plane's slopes as soon as their own faces are formed, while the others
  // still form faces, so the x and y slopes get one buffer per plane parity.  Only in the FP64 form
  // (where the faces' FP64-pipe time is uneven over the SM sub-partitions: 2 % faster at 150^3;
  // the FP32 variants ran 3 % slower), where there are such warps, and where the second buffer
  // keeps MINB CTAs per SM.
  static constexpr int NOWN = (TX * TY + 31) / 32 * 32;
  static constexpr bool OV = sizeof(R) == sizeof(double) && NT > NOWN &&
                             MINB * (fused_smem_bytes(TX, TY, sizeof(R), 2) + 1024) <= 228 * 1024;
  static constexpr int NSLB = OV ? 2 : 1;
  static constexpr size_t a16(size_t x) { return (x + 15) / 16 * 16; }
  static constexpr size_t ring_off = 0;
  static constexpr size_t slx_off = ((size_t)NBUF * PLANE * sizeof(R) + 127) / 128 * 128;
  static constexpr size_t sly_off = slx_off + NSLB * a16(NSLX * sizeof(R));
  static constexpr size_t slz_off = sly_off + NSLB * a16(NSLY * sizeof(R));
  // three z-slope planes, rotating: while the faces of plane k read the z slopes of planes k and
  // k+1, those of plane k+2 are formed; at the start of a chunk the third buffer holds plane kb-1's
  // (whose column-owned entries then hold the flux through face kb-1/2)
  static constexpr size_t fx_off = slz_off + a16(3 * NSLZ * sizeof(R));
  static constexpr size_t fy_off = fx_off + a16(NFX * sizeof(R));
  static constexpr size_t fz_off = fy_off + a16(NFY * sizeof(R));
  static constexpr size_t red_off = fz_off + a16(NFZ * sizeof(R));
  static constexpr size_t bar_off = red_off + 64 * sizeof(double);
  static constexpr size_t misc_off = bar_off + NBUF * sizeof(uint64_t);  // work item, abort flag, 2 slope counters
  static constexpr size_t used = misc_off + 16;
  static constexpr size_t total = used + 128;  // room to align the base to 128 bytes
  static constexpr unsigned plane_tx_bytes = (unsigned)(PLANE * sizeof(R));
  static_assert(total == fused_smem_bytes(TX, TY, sizeof(R), NSLB), "layout and size formula agree");
  static_assert(NT % 32 == 0 && NT >= TX * TY, "one owner thread per column, whole warps");
  static_assert((TX * sizeof(R)) % 16 == 0, "TMA x offsets must be 16-byte multiples");
  static_assert(((TX + 4) * sizeof(R)) % 16 == 0, "TMA box rows must be 16-byte multiples");
  static_assert((PLANE * sizeof(R)) % 128 == 0, "each ring slot is a TMA destination: 128-byte aligned");
  static_assert(total <= 227 * 1024, "shared memory budget");
};

namespace MHDGB_VNS {

// Accumulator of the flux divergence dFx*xinv + dFy*yinv + dFz*zinv of one cell.
// FP64 form: plain FP64 sums in the reference's order.  Mixed form: each FP32 product is split
// exactly into value + rounding error (TwoProd with an FMA) and the three terms are added with
// TwoSum, so the pair (hi, lo) carries the sum with compensated rounding.  __fmul_rn/__fadd_rn keep
// the compiler from fusing the steps.
template <class R> struct DivAcc;
template <> struct DivAcc<double> {
  double s[NCONS];
  __device__ __forceinline__ void first(int m, double df, double inv) { s[m] = df * inv; }
  __device__ __forceinline__ void add(int m, double df, double inv) { s[m] = s[m] + df * inv; }
};
template <> struct DivAcc<float> {
  float hi[NCONS], lo[NCONS];
  __device__ __forceinline__ void first(int m, float df, float inv) {
    const float p = __fmul_rn(df, inv);
    hi[m] = p;
    lo[m] = fmaf(df, inv, -p);
  }
  __device__ __forceinline__ void add(int m, float df, float inv) {
    const float p = __fmul_rn(df, inv);
    const float e = fmaf(df, inv, -p);
    const float s = __fadd_rn(hi[m], p);
    const float bp = __fadd_rn(s, -hi[m]);
    const float err = __fadd_rn(__fadd_rn(hi[m], -__fadd_rn(s, -bp)), __fadd_rn(p, -bp));
    hi[m] = s;
    lo[m] = __fadd_rn(lo[m], __fadd_rn(err, e));
  }
  __device__ __forceinline__ float total(int m) const { return __fadd_rn(hi[m], lo[m]); }
};

template <class R> __device__ __forceinline__ R inv_of(const FusedArgs& a, int d, int i);
template <> __device__ __forceinline__ double inv_of<double>(const FusedArgs& a, int d, int i) {
  return d == 0 ? a.xinv[i] : (d == 1 ? a.yinv[i] : a.zinv[i]);
}
template <> __device__ __forceinline__ float inv_of<float>(const FusedArgs& a, int d, int i) {
  return d == 0 ? a.xinvf[i] : (d == 1 ? a.yinvf[i] : a.zinvf[i]);
}
template <class R> __device__ __forceinline__ R spacing_of(const FusedArgs& a, int d, int i);
template <> __device__ __forceinline__ double spacing_of<double>(const FusedArgs& a, int d, int i) {
  return d == 0 ? a.dxs[i] : (d == 1 ? a.dys[i] : a.dzs[i]);
}
template <> __device__ __forceinline__ float spacing_of<float>(const FusedArgs& a, int d, int i) {
  return d == 0 ? a.dxsf[i] : (d == 1 ? a.dysf[i] : a.dzsf[i]);
}

// Ghost images of a freshly recovered interior cell: the values the reference's ghost fill
// (boundary.cpp:152-169 and equivalents) would copy from it at the start of the next step.
// ii/jj/kk are interior indices (0-based); pn holds the cell's 12 primitives.
template <class R>
__device__ __forceinline__ void write_ghost_images(R* __restrict__ Pout, const Layout& L, const int bc[6],
                                                   int ii, int jj, int kk, const R (&pn)[NPRIM]) {
  const int nx = L.nx, ny = L.ny, nz = L.nz;
  auto put = [&](int gi, int gj, int gk, int flip) {
#pragma unroll
    for (int n = 0; n < NPRIM; n++) {
      R v = pn[n];
      if (n == flip) v = -v;
      Pout[L.at(NPRIM, n, gk + NGH, gj + NGH, gi + NGH)] = v;
    }
  };
  if (bc[0] == 1) { if (ii >= nx - 2) put(ii - nx, jj, kk, -1); }
  else if (bc[0] == 2) { if (ii <= 1) put(-1 - ii, jj, kk, nve1); }
  else if (bc[0] == 3) { if (ii == 0) { put(-1, jj, kk, -1); put(-2, jj, kk, -1); } }
  if (bc[1] == 1) { if (ii <= 1) put(nx + ii, jj, kk, -1); }
  else if (bc[1] == 2) { if (ii >= nx - 2) put(2 * nx - 1 - ii, jj, kk, nve1); }
  else if (bc[1] == 3) { if (ii == nx - 1) { put(nx, jj, kk, -1); put(nx + 1, jj, kk, -1); } }
  if (bc[2] == 1) { if (jj >= ny - 2) put(ii, jj - ny, kk, -1); }
  else if (bc[2] == 2) { if (jj <= 1) put(ii, -1 - jj, kk, nve2); }
  else if (bc[2] == 3) { if (jj == 0) { put(ii, -1, kk, -1); put(ii, -2, kk, -1); } }
  if (bc[3] == 1) { if (jj <= 1) put(ii, ny + jj, kk, -1); }
  else if (bc[3] == 2) { if (jj >= ny - 2) put(ii, 2 * ny - 1 - jj, kk, nve2); }
  else if (bc[3] == 3) { if (jj == ny - 1) { put(ii, ny, kk, -1); put(ii, ny + 1, kk, -1); } }
  if (bc[4] == 1) { if (kk >= nz - 2) put(ii, jj, kk - nz, -1); }
  else if (bc[4] == 2) { if (kk <= 1) put(ii, jj, -1 - kk, nve3); }
  else if (bc[4] == 3) { if (kk == 0) { put(ii, jj, -1, -1); put(ii, jj, -2, -1); } }
  if (bc[5] == 1) { if (kk <= 1) put(ii, jj, nz + kk, -1); }
  else if (bc[5] == 2) { if (kk >= nz - 2) put(ii, jj, 2 * nz - 1 - kk, nve3); }
  else if (bc[5] == 3) { if (kk == nz - 1) { put(ii, jj, nz, -1); put(ii, jj, nz + 1, -1); } }
}

// Primitive recovery of one interior cell from its updated conserved state, written with its
// ghost images, plus the cell's dt and c_h candidates (in R) and the status checks.
template <class R>
__device__ __forceinline__ void recover_cell(const double (&u)[NCONS], double gam, R* __restrict__ Pout,
                                             const Layout& L, const int bc[6], int ii, int jj, int kk,
                                             R dx, R dy, R dz, R& dtc, R& chc, unsigned& bad);

// FP64 form: UpdatePrimitvP (mhd.cpp:1483-1506) and the reference candidates.
template <>
__device__ __forceinline__ void recover_cell<double>(const double (&u)[NCONS], double gam, double* __restrict__ Pout,
                                                     const Layout& L, const int bc[6], int ii, int jj, int kk,
                                                     double dx, double dy, double dz, double& dtc, double& chc,
                                                     unsigned& bad) {
  double p[NPRIM];
  cons2prim<double>(u, gam, p);
#pragma unroll
  for (int n = 0; n < NPRIM; n++) Pout[L.at(NPRIM, n, kk + NGH, jj + NGH, ii + NGH)] = p[n];
  write_ghost_images<double>(Pout, L, bc, ii, jj, kk, p);
  dtc = cell_dt<double>(p, dx, dy, dz);
  chc = cell_ch<double>(p);
  if constexpr (kFast) {  // the same tests on the integer pipe (dtc NaN; chc NaN or inf; rho, p > 0)
    const long long abs_mask = 0x7FFFFFFFFFFFFFFFLL, inf_bits = 0x7FF0000000000000LL;
    if ((__double_as_longlong(dtc) & abs_mask) > inf_bits || (__double_as_longlong(chc) & inf_bits) == inf_bits)
      bad |= ST_NONFINITE;
    if (!pos_nonzero(p[nden]) || !pos_nonzero(p[npre])) bad |= ST_NEGATIVE;
  } else {
    if (!(dtc == dtc) || !(chc == chc) || isinf(chc)) bad |= ST_NONFINITE;
    if (!(p[nden] > 0.0) || !(p[npre] > 0.0)) bad |= ST_NEGATIVE;
  }
}

// Mixed form: the specific internal energy e = (E - m^2/(2 rho) - B^2/2)/rho is computed in FP64
// (1/rho from an FP32 reciprocal refined by one FP64 Newton step, ~46 bits); the other primitives,
// which involve no cancellation, are formed in FP32 from the FP32-rounded conserved values;
// p = e*rho*(gam-1) and c_s = sqrt(e*gam*(gam-1)) as in mhd.cpp:1497-1499.
template <>
__device__ __forceinline__ void recover_cell<float>(const double (&u)[NCONS], double gam, float* __restrict__ Pout,
                                                    const Layout& L, const int bc[6], int ii, int jj, int kk,
                                                    float dx, float dy, float dz, float& dtc, float& chc,
                                                    unsigned& bad) {
  const float rho_f = d2f_rne(u[mden]);
  const float rinv_f = 1.0f / rho_f;
  const double r0 = f2d_exact(rinv_f);
  const double r = fma(r0, fma(-u[mden], r0, 1.0), r0);
  double m2 = u[mrv1] * u[mrv1];
  m2 = fma(u[mrv2], u[mrv2], m2);
  m2 = fma(u[mrv3], u[mrv3], m2);
  double b2 = u[mbm1] * u[mbm1];
  b2 = fma(u[mbm2], u[mbm2], b2);
  b2 = fma(u[mbm3], u[mbm3], b2);
  double t = fma(-m2, 0.5 * r, u[meto]);
  t = fma(-0.5, b2, t);
  const double e = t * r;
  const float gf = d2f_rne(gam);
  float p[NPRIM];
  p[nden] = rho_f;
  p[nve1] = d2f_rne(u[mrv1]) * rinv_f;
  p[nve2] = d2f_rne(u[mrv2]) * rinv_f;
  p[nve3] = d2f_rne(u[mrv3]) * rinv_f;
  p[nene] = d2f_rne(e);
  p[npre] = p[nene] * p[nden] * (gf - 1.0f);
  p[ncsp] = sqrtf(p[nene] * gf * (gf - 1.0f));
  p[nbm1] = d2f_rne(u[mbm1]);
  p[nbm2] = d2f_rne(u[mbm2]);
  p[nbm3] = d2f_rne(u[mbm3]);
  p[nbps] = d2f_rne(u[mbps]);
  p[nst] = d2f_rne(u[mst]) * rinv_f;
#pragma unroll
  for (int n = 0; n < NPRIM; n++) Pout[L.at(NPRIM, n, kk + NGH, jj + NGH, ii + NGH)] = p[n];
  write_ghost_images<float>(Pout, L, bc, ii, jj, kk, p);
  dtc = cell_dt<float>(p, dx, dy, dz);
  chc = cell_ch<float>(p);
  if (!(dtc == dtc) || !(chc == chc) || isinf(chc) || isinf(p[nene])) bad |= ST_NONFINITE;
  if (!(p[nden] > 0.0f) || !(p[npre] > 0.0f)) bad |= ST_NEGATIVE;
}

// U update of one cell from its summed flux divergence, then psi damping.
// FP64 form: U - dt*sum (mhd.cpp:1438-1440) and psi*(1 - dt*(0.1*c_h/min(dx,dy,dz))) (mhd.cpp:1628-1630).
// Mixed form: fma(-dt, sum, U) in FP64 with the compensated FP32 sum widened exactly; the damping
// factor is formed in FP32 with 1/min(dx,dy,dz) = max of the inverse spacings, applied in FP64.
__device__ __forceinline__ void update_cell(const DivAcc<double>& acc, const double* __restrict__ Uc, size_t fs,
                                            double dt, double chd, float, float, const FusedArgs& a, int i, int j,
                                            int k, double (&u)[NCONS]) {
#pragma unroll
  for (int m = 0; m < NCONS; m++) u[m] = Uc[m * fs] - dt * acc.s[m];
  double taui;
  if constexpr (kFast) {  // integer-pipe min of the (positive) spacings, Newton-reciprocal division
    const double dhl = imin(imin(a.dxs[i], a.dys[j]), a.dzs[k]);
    taui = fdiv(0.1 * chd, dhl);
  } else {
    double dhl = a.dxs[i];
    if (a.dys[j] < dhl) dhl = a.dys[j];
    if (a.dzs[k] < dhl) dhl = a.dzs[k];
    taui = 0.1 * chd / dhl;
  }
  u[mbps] = u[mbps] * (1.0 - dt * taui);
}

__device__ __forceinline__ void update_cell(const DivAcc<float>& acc, const double* __restrict__ Uc, size_t fs,
                                            double dt, double, float dtf, float chf, const FusedArgs& a, int i, int j,
                                            int k, double (&u)[NCONS]) {
#pragma unroll
  for (int m = 0; m < NCONS; m++) u[m] = fma(-dt, f2d_exact(acc.total(m)), Uc[m * fs]);
  const float imax = fmaxf(fmaxf(a.xinvf[i], a.yinvf[j]), a.zinvf[k]);
  u[mbps] = u[mbps] * f2d_exact(1.0f - dtf * (0.1f * chf * imax));
}

// Launch-wide steps shared by the fused-step kernels.
// Start of a launch: block 0 resets every live grid's reduction slot (step+2)%3 for the next launch
// (step n reduces into slot (n+1)%3).
__device__ __forceinline__ void fused_reset_next_slots(const InstanceDesc* __restrict__ desc, int ninst, int nt) {
  if (blockIdx.x != 0) return;
  for (int q = threadIdx.x; q < ninst; q += nt) {
    Ctrl* c = desc[q].a.ctrl;
    if (!c->done) {
      c->slot[(c->step + 2) % 3].dtmin_bits = DT_RESET;
      c->slot[(c->step + 2) % 3].chmax_bits = CH_RESET;
    }
  }
}
// The grid a queue item belongs to (the descriptors are sorted by item_begin).
__device__ __forceinline__ int fused_instance_of(const InstanceDesc* __restrict__ desc, int ninst, int gitem) {
  int inst = 0;
  for (int lo = 0, hi = ninst - 1; lo <= hi;) {
    const int mid = (lo + hi) >> 1;
    if (desc[mid].item_begin <= gitem) { inst = mid; lo = mid + 1; } else hi = mid - 1;
  }
  return inst;
}
// End of a CTA (thread 0): the last CTA to finish advances every live grid by one step and re-arms
// the work queue for the next launch.
__device__ __forceinline__ void fused_finish_cta(const InstanceDesc* __restrict__ desc, LaunchCtrl* __restrict__ lc,
                                                 int ninst) {
  __threadfence();
  const unsigned prev = atomicAdd(&lc->blocks_done, 1u);
  if (prev == gridDim.x - 1) {
    __threadfence();
    for (int q = 0; q < ninst; q++) {
      Ctrl* c = desc[q].a.ctrl;
      if (c->done) continue;
      const double dtq = desc[q].a.cfl * bitsd(c->slot[c->step % 3].dtmin_bits);
      c->last_dt = dtq;
      c->last_ch = bitsd(c->slot[c->step % 3].chmax_bits);
      c->time += dtq;
      c->step += 1;
      if (c->time > c->tmax || c->step >= c->max_step) c->done = 1;
    }
    lc->work_next = 0;
    lc->blocks_done = 0;
    __threadfence();
  }
}

// MINB: CTAs per SM the register allocation must allow (__launch_bounds__); 2 at 256 threads caps
// a thread at 128 registers, which the FP32 form meets without spills.
// GEN: false compiles HLLD alone (the tuned tile variants); true reads the Riemann solver from the
// arguments (one such kernel per form runs HLLE/HLLC), so adding solvers never changes the code,
// and hence the FMA contraction, of the HLLD kernels.
template <class R, int TX, int TY, int NT, int MINB, bool GEN>
__global__ void __launch_bounds__(NT, MINB)
k_fused_step(const InstanceDesc* __restrict__ desc, LaunchCtrl* __restrict__ lc) {
  using S = FusedSmem<R, TX, TY, NT, MINB>;
  constexpr int NBUF = S::NBUF, PX = S::PX;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char* smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);  // TMA destinations
  R* ring = reinterpret_cast<R*>(smem + S::ring_off);
  R* slx = reinterpret_cast<R*>(smem + S::slx_off);
  R* sly = reinterpret_cast<R*>(smem + S::sly_off);
  R* slz = reinterpret_cast<R*>(smem + S::slz_off);
  R* fxs = reinterpret_cast<R*>(smem + S::fx_off);
  R* fys = reinterpret_cast<R*>(smem + S::fy_off);
  R* fzs = reinterpret_cast<R*>(smem + S::fz_off);
  double* red = reinterpret_cast<double*>(smem + S::red_off);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + S::bar_off);
  int& s_item = *reinterpret_cast<int*>(smem + S::misc_off);
  int& s_abort = *reinterpret_cast<int*>(smem + S::misc_off + 4);
  int* s_aitem = reinterpret_cast<int*>(smem + S::misc_off + 8);  // next phase-A warp item, by plane parity

  const int tid = threadIdx.x;
  const int ninst = (int)lc->ninst, total = (int)lc->total_items;
  fused_reset_next_slots(desc, ninst, NT);
  if (tid == 0) {
    for (int s = 0; s < NBUF; s++) mbar_init(&bars[s], 1);
    fence_mbar_init();
    s_abort = 0;
    s_aitem[0] = 0;
    s_aitem[1] = 0;
  }
  __syncthreads();

  // Loads issued per slot, as bit masks (identical in every thread; registers, where an array
  // indexed by the run-time slot would live in local memory): bit s of odd = slot s has had an odd
  // number of loads, bit s of used = slot s has had one at all.  The wait for the latest load of
  // slot s is on mbarrier phase parity (count - 1) & 1 = 1 - odd bit.
  unsigned odd = 0, used = 0;
  auto fill = [&](int s) {
    odd ^= 1u << s;
    used |= 1u << s;
  };
  auto parity = [&](int s) { return ((odd >> s) & 1u) ^ 1u; };
  const int oi = tid % TX, oj = tid / TX;  // owner column of this thread (if oj < TY)

  for (;;) {
    if (tid == 0) s_item = (int)atomicAdd(&lc->work_next, 1u);
    __syncthreads();
    const int gitem = s_item;
    if (gitem >= total || s_abort) break;
    const int inst = fused_instance_of(desc, ninst, gitem);  // the grid this work item belongs to
    const FusedArgs& a = desc[inst].a;
    Ctrl* ctrl = a.ctrl;
    if (ctrl->done) { __syncthreads(); continue; }
    const Layout L = a.L;
    const size_t fsU = (size_t)L.ip;  // field stride of U in the (k, j, n, i) layout
    const unsigned long long step = ctrl->step;
    const int par = (int)(step & 1);
    R* __restrict__ Pout = reinterpret_cast<R*>(a.P[par ^ 1]);
    const CUtensorMap* tmap = &desc[inst].tmap[par];
    const RedSlot cur_slot = ctrl->slot[step % 3];
    const double dt = a.cfl * bitsd(cur_slot.dtmin_bits);
    const double chd = bitsd(cur_slot.chmax_bits);
    const R chg = (R)chd;
    const GlmConst<R> glm = glm_const(chg);
    const int riemann = GEN ? a.riemann : (int)RIEMANN_HLLD;
    const float dtf = (float)dt, chf = (float)chd;
    RedSlot* next = &ctrl->slot[(step + 1) % 3];
    R cmin = R(1e30), cmax = R(0);
    unsigned bad = 0;
    if (tid == 0) prefetch_tensormap(tmap);

    const int item = gitem - desc[inst].item_begin;
    const int bxi = item % a.ntx, byi = (item / a.ntx) % a.nty, bki = item / (a.ntx * a.nty);
    const int i0 = bxi * TX, j0 = byi * TY;
    const int kb = a.kst[bki], ke = a.kst[bki + 1];
    const int cx = min(TX, L.nx - i0), cy = min(TY, L.ny - j0);
    const bool own = oj < TY && oi < cx && oj < cy;
    const int ii = i0 + oi, jj = j0 + oj;

    auto slot_of = [&](int p) { return (p - (kb - 2)) % NBUF; };
    auto plane = [&](int p) -> const R* { return ring + (size_t)slot_of(p) * S::PLANE; };
    auto issue = [&](int p) {  // thread 0 only
      const int s = slot_of(p);
      mbar_arrive_expect_tx(&bars[s], S::plane_tx_bytes + (p == kb - 2 ? a.tx_extra : 0u));
      tma_load_4d(ring + (size_t)s * S::PLANE, tmap, i0, 0, j0, p + NGH, &bars[s]);
    };
    auto wait_plane = [&](int p) {
      const int s = slot_of(p);
      if (!mbar_wait(&bars[s], parity(s), &ctrl->status)) s_abort = 1;
    };
    auto PV = [&](const R* pl, int n, int i, int j) -> R { return pl[((j + 2) * NPRIM + n) * PX + (i + 2)]; };
    auto PV0 = [&](const R* pl, int i, int j) -> const R& { return pl[((j + 2) * NPRIM) * PX + (i + 2)]; };
    R* slxk = slx;  // the x and y slope buffers of the current plane (by plane parity with OV)
    R* slyk = sly;
    auto SLX = [&](int n, int i, int j) -> R& { return slxk[(n * TY + j) * (TX + 2) + (i + 1)]; };
    auto SLY = [&](int n, int i, int j) -> R& { return slyk[(n * (TY + 2) + (j + 1)) * TX + i]; };
    auto SLZ = [&](int b, int n, int i, int j) -> R& { return slz[((b * NPRIM + n) * TY + j) * TX + i]; };
    auto FXS = [&](int m, int i, int j) -> R& { return fxs[(m * TY + j) * (TX + 1) + i]; };
    auto FYS = [&](int m, int i, int j) -> R& { return fys[(m * (TY + 1) + j) * TX + i]; };
    auto FZS = [&](int m, int i, int j) -> R& { return fzs[(m * TY + j) * TX + i]; };

    // prologue: planes kb-2 .. kb+1 (ke >= kb+1 so all exist)
    if (tid == 0) {
      s_aitem[0] = 0;
      s_aitem[1] = 0;
      fence_proxy_async();
      for (int p = kb - 2; p < kb + 2; p++) issue(p);
    }
#pragma unroll
    for (int s = 0; s < NBUF; s++) fill(s);
    for (int p = kb - 2; p < kb + 2; p++) wait_plane(p);
    __syncthreads();
    if (s_abort) break;

    // z slopes of planes kb-1 and kb.  The flux through face kb-1/2 is formed in the first plane's
    // phase B by the same code as every other z face, so a face shared by two chunks comes out bit
    // for bit the same in both (the result cannot depend on the z-chunking).  The z slopes of plane
    // p live in slz buffer (p - kb + 1) % 3, tracked as zc, zn, zf = the buffers of planes k, k+1 and
    // k+2 (= k-1).
    R fz_lo[NCONS];  // flux through face k-1/2 of the owner's column
    int zc = 1, zn = 2, zf = 0;
    if (own) {
      const R *pm2 = plane(kb - 2), *pm1 = plane(kb - 1), *p0 = plane(kb), *pp1 = plane(kb + 1);
#pragma unroll
      for (int n = 0; n < NPRIM; n++) {
        const R a2 = PV(pm2, n, oi, oj), a1 = PV(pm1, n, oi, oj), b0 = PV(p0, n, oi, oj), b1 = PV(pp1, n, oi, oj);
        SLZ(zf, n, oi, oj) = van_leer(b0 - a1, a1 - a2);
        SLZ(zc, n, oi, oj) = van_leer(b1 - b0, b0 - a1);
      }
    }
    __syncthreads();  // plane kb-2 retired (kb-1 stays until the first plane's faces are formed)
    if (tid == 0) {
      fence_proxy_async();
      if (kb + 2 <= ke + 1) issue(kb + 2);
    }
    if (kb + 2 <= ke + 1) fill(slot_of(kb + 2));

    // work-list sizes (the slope sub-lists padded to whole warps) and the divisors of their decode
    const FastDiv dv0(cx), dv1(cx + 1), dv2(cx + 2);
    const int nxs = cy * (cx + 2), nys = (cy + 2) * cx, nzs = cy * cx;
    const int nxf = cy * (cx + 1), nyf = (cy + 1) * cx, nzf = cy * cx;
    const int pxs = (nxs + 31) & ~31, pys = (nys + 31) & ~31, pzs = (nzs + 31) & ~31;

    // Two barriers per plane.  Phase A writes only slope buffers that the previous plane's phase C
    // does not read, and phase C reads no ring plane, so neither the start nor the end of a plane
    // needs a barrier; the ring slot of plane k is reloaded once phase B has read it.
    // Phase A hands out whole-warp items from a shared counter: the warps without a cell (no phase
    // C) start on the slopes at once and the owner warps join when their cells are done.  With OV
    // the barrier after phase B is a named one that only the owner warps wait at: the others arrive
    // and go on to the next plane's slopes (into the other x/y slope buffer and the z-slope buffer
    // that plane k-1's faces read) while the owners' and other warps' last faces are formed.  On the
    // first plane of a chunk everyone waits, and again after the owners have taken the flux through
    // face kb-1/2, whose buffer the next plane's z slopes reuse.
    const int nwa = (pxs + pys + pzs) >> 5;
    for (int k = kb; k < ke; k++) {
      if constexpr (S::OV) {
        slxk = slx + (k & 1) * (size_t)S::NSLX;
        slyk = sly + (k & 1) * (size_t)S::NSLY;
      }
      if (own) {  // the cell's U is read in phase C, two phases from now: pull it into L2
        const double* u0 = a.U + L.at(NCONS, 0, k + NGH, jj + NGH, ii + NGH);
#pragma unroll
        for (int m = 0; m < NCONS; m++) prefetch_l2(u0 + m * fsU);
      }
      wait_plane(k + 2);
      const R *pk = plane(k), *pk1 = plane(k + 1), *pk2 = plane(k + 2);
      // ---- phase A: slopes ----
      for (;;) {
        int w = 0;
        if ((tid & 31) == 0) w = atomicAdd(&s_aitem[k & 1], 1);
        w = __shfl_sync(0xffffffffu, w, 0);
        if (w >= nwa) break;
        const int q = (w << 5) | (tid & 31);
        if (q < pxs) {
          if (q < nxs) {
            const int j = dv2.div(q), i = q - j * (cx + 2) - 1;
#pragma unroll
            for (int n = 0; n < NPRIM; n++) {
              const R m1 = PV(pk, n, i - 1, j), c0 = PV(pk, n, i, j), p1 = PV(pk, n, i + 1, j);
              SLX(n, i, j) = van_leer(p1 - c0, c0 - m1);
            }
          }
        } else if (q < pxs + pys) {
          const int r = q - pxs;
          if (r < nys) {
            const int jr = dv0.div(r), j = jr - 1, i = r - jr * cx;
#pragma unroll
            for (int n = 0; n < NPRIM; n++) {
              const R m1 = PV(pk, n, i, j - 1), c0 = PV(pk, n, i, j), p1 = PV(pk, n, i, j + 1);
              SLY(n, i, j) = van_leer(p1 - c0, c0 - m1);
            }
          }
        } else {
          const int r = q - pxs - pys;
          if (r < nzs) {
            const int j = dv0.div(r), i = r - j * cx;
#pragma unroll
            for (int n = 0; n < NPRIM; n++) {
              const R c0 = PV(pk, n, i, j), c1 = PV(pk1, n, i, j), c2 = PV(pk2, n, i, j);
              SLZ(zn, n, i, j) = van_leer(c2 - c1, c1 - c0);
            }
          }
        }
      }
      // the next plane's counter (last used by plane k-1's phase A, which every warp has left)
      if (tid == 0) s_aitem[(k + 1) & 1] = 0;
      __syncthreads();
      if (s_abort) break;  // a plane that never arrived (bounded wait): the data above is not used
      // ---- phase B: face fluxes (on the first plane also the faces kb-1/2, into slope buffer 2) ----
      // One list over the x, y and z faces (and the lower z faces on the first plane) with no
      // padding between directions: a thread reads its face's primitives and slopes in the rotated
      // order (normal, first and second tangential components), forms the flux with the
      // direction-generic code (Dir<0>) and stores it back into the unrotated slots.  Only the
      // last warp of the list has idle lanes.
      const int nfb = nxf + nyf + (k == kb ? 2 * nzf : nzf);
      for (int q = tid; q < ((nfb + 31) & ~31); q += NT) {
        if (q < nfb) {
          int rot, sstr, fstr;        // rotation (0, 1, 2 = x, y, z); slope and flux slot strides
          const R *pa, *pb, *sa, *sb;  // variable 0 of the left / right cell: primitive, slope
          R* fo;                      // flux slot 0 of the face
          if (q < nxf) {
            const int j = dv1.div(q), i = q - j * (cx + 1);
            rot = 0;
            pa = &PV0(pk, i - 1, j);
            pb = pa + 1;
            sa = &SLX(0, i - 1, j);
            sb = sa + 1;
            sstr = TY * (TX + 2);
            fo = &FXS(0, i, j);
            fstr = TY * (TX + 1);
          } else if (q < nxf + nyf) {
            const int r = q - nxf, j = dv0.div(r), i = r - j * cx;
            rot = 1;
            pa = &PV0(pk, i, j - 1);
            pb = pa + NPRIM * PX;
            sa = &SLY(0, i, j - 1);
            sb = sa + TX;
            sstr = (TY + 2) * TX;
            fo = &FYS(0, i, j);
            fstr = (TY + 1) * TX;
          } else {
            int r = q - nxf - nyf;
            const bool lower = r >= nzf;  // face kb-1/2 (first plane only)
            if (lower) r -= nzf;
            const int j = dv0.div(r), i = r - j * cx;
            rot = 2;
            pa = &PV0(lower ? plane(kb - 1) : pk, i, j);
            pb = &PV0(lower ? pk : pk1, i, j);
            sa = &SLZ(lower ? zf : zc, 0, i, j);
            sb = &SLZ(lower ? zc : zn, 0, i, j);
            sstr = TY * TX;
            // the lower face overwrites the slopes it alone read (column (i, j) of buffer 2)
            fo = lower ? &SLZ(zf, 0, i, j) : &FZS(0, i, j);
            fstr = TY * TX;
          }
          const int c1 = unrot_comp(1, rot), c2 = unrot_comp(2, rot);
          // unrotated variable read into rotated slot n (n is a constant after unrolling)
          auto var_of = [&](int n) {
            if (n == nve1 || n == nbm1) return n + rot;
            if (n == nve2 || n == nbm2) return n - 1 + c1;
            if (n == nve3 || n == nbm3) return n - 2 + c2;
            return n;
          };
          R pl[NPRIM], pr[NPRIM], f[NCONS];
#pragma unroll
          for (int n = 0; n < NPRIM; n++) {
            const int v = var_of(n);
            pl[n] = left_state(pa[v * PX], sa[v * sstr]);
            pr[n] = right_state(pb[v * PX], sb[v * sstr]);
          }
          face_flux<R, 0>(pl, pr, glm, f, riemann, rot);
          auto slot_of_flux = [&](int m) {
            if (m == mrv1 || m == mbm1) return m + rot;
            if (m == mrv2 || m == mbm2) return m - 1 + c1;
            if (m == mrv3 || m == mbm3) return m - 2 + c2;
            return m;
          };
#pragma unroll
          for (int m = 0; m < NCONS; m++) fo[slot_of_flux(m) * fstr] = f[m];
        }
      }
      // faces formed; plane k (and on the first plane kb-1) read for the last time
      if (k == kb) {
        __syncthreads();
        if (own) {
#pragma unroll
          for (int m = 0; m < NCONS; m++) fz_lo[m] = SLZ(zf, m, oi, oj);
        }
        __syncthreads();  // zf now takes plane kb+2's z slopes
      } else if constexpr (S::OV) {
        if (tid < S::NOWN) named_bar_sync(1, NT);
        else named_bar_arrive(1, NT);
      } else {
        __syncthreads();
      }
      if (k == kb && kb + 3 <= ke + 1) {  // plane kb-1's slot
        if (tid == 0) {
          fence_proxy_async();
          issue(kb + 3);
        }
        fill(slot_of(kb + 3));
      }
      if (k + 4 <= ke + 1) {  // plane k's slot
        if (tid == 0) {
          fence_proxy_async();
          issue(k + 4);
        }
        fill(slot_of(k + 4));
      }
      // ---- phase C: cell update, recovery, ghost images, candidates ----
      if (own) {
        DivAcc<R> acc;
        const R xi = inv_of<R>(a, 0, ii + NGH);
        const R yi = inv_of<R>(a, 1, (a.quirk ? ii : jj) + NGH);
        const R zi = inv_of<R>(a, 2, (a.quirk ? ii : k) + NGH);
#pragma unroll
        for (int m = 0; m < NCONS; m++) {
          acc.first(m, FXS(m, oi + 1, oj) - FXS(m, oi, oj), xi);
          acc.add(m, FYS(m, oi, oj + 1) - FYS(m, oi, oj), yi);
          const R fzh = FZS(m, oi, oj);
          acc.add(m, fzh - fz_lo[m], zi);
          fz_lo[m] = fzh;
        }
        const size_t c0 = L.at(NCONS, 0, k + NGH, jj + NGH, ii + NGH);
        double u[NCONS];
        update_cell(acc, a.U + c0, fsU, dt, chd, dtf, chf, a, ii + NGH, jj + NGH, k + NGH, u);
#pragma unroll
        for (int m = 0; m < NCONS; m++) a.U[c0 + m * fsU] = u[m];
        if (a.Uh) {  // the caller's host copy of U (end-to-end steps), field stride itot
          double* uh = a.Uh + ((size_t)(ii + NGH) + (size_t)L.itot * NCONS * ((size_t)(jj + NGH) +
                                                                            (size_t)L.jtot * (size_t)(k + NGH)));
#pragma unroll
          for (int m = 0; m < NCONS; m++) uh[(size_t)m * L.itot] = u[m];
        }
        R dtc, chc;
        recover_cell<R>(u, a.gam, Pout, L, a.bc, ii, jj, k, spacing_of<R>(a, 0, ii + NGH),
                        spacing_of<R>(a, 1, jj + NGH), spacing_of<R>(a, 2, k + NGH), dtc, chc, bad);
        if constexpr (kFast && std::is_same<R, double>::value) {  // integer-pipe min/max
          cmin = imin(cmin, dtc);
          cmax = imax(cmax, chc);
        } else {
          cmin = smin(cmin, dtc);
          cmax = smax(cmax, chc);
        }
      }
      const int z0 = zc;
      zc = zn;
      zn = zf;
      zf = z0;
    }
    if (bad) atomicOr(&ctrl->status, bad);
    block_reduce_to_slot((double)cmin, (double)cmax, red, next);
    if (s_abort) break;
  }

  if (s_abort) {
    // drain: wait (bounded) for any load still in flight before leaving
    for (int s = 0; s < NBUF; s++)
      if ((used >> s) & 1u) mbar_wait(&bars[s], parity(s), &desc[0].a.ctrl->status);
  }
  if (tid == 0) fused_finish_cta(desc, lc, ninst);
}

// Recovery of P from U for the interior (+ ghost images) and the dt/c_h reduction into slot: the
// state a fused run starts from.  uh_in null: from the device U.  Otherwise the state comes from the caller's
// host array (reference layout, itot x jtot x ktot, over the host link): every cell is copied into
// the device U on the way, interior cells are recovered, and ghost cells also go to uh_ghost_out
// when it is given (an output array other than the input).
template <class R>
__global__ void k_recover(FusedArgs a, int which, RedSlot* slot, const double* __restrict__ uh_in,
                          double* __restrict__ uh_ghost_out) {
  __shared__ double scratch[64];
  const Layout L = a.L;
  R mn = R(1e30), mx = R(0);
  unsigned bad = 0;
  R* Pout = reinterpret_cast<R*>(a.P[which]);
  const long long stride = (long long)gridDim.x * blockDim.x;
  if (!uh_in) {
    const long long n = (long long)L.nx * L.ny * L.nz;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += stride) {
      const int ii = (int)(t % L.nx), jj = (int)((t / L.nx) % L.ny), kk = (int)(t / ((long long)L.nx * L.ny));
      double u[NCONS];
#pragma unroll
      for (int m = 0; m < NCONS; m++) u[m] = a.U[L.at(NCONS, m, kk + NGH, jj + NGH, ii + NGH)];
      R dtc, chc;
      recover_cell<R>(u, a.gam, Pout, L, a.bc, ii, jj, kk, spacing_of<R>(a, 0, ii + NGH),
                      spacing_of<R>(a, 1, jj + NGH), spacing_of<R>(a, 2, kk + NGH), dtc, chc, bad);
      mn = smin(mn, dtc);
      mx = smax(mx, chc);
    }
  } else {
    const long long n = (long long)L.itot * L.jtot * L.ktot;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += stride) {
      const int i = (int)(t % L.itot), j = (int)((t / L.itot) % L.jtot), k = (int)(t / ((long long)L.itot * L.jtot));
      const size_t h0 = (size_t)i + (size_t)L.itot * NCONS * ((size_t)j + (size_t)L.jtot * (size_t)k);
      double u[NCONS];
#pragma unroll
      for (int m = 0; m < NCONS; m++) u[m] = uh_in[h0 + (size_t)m * L.itot];
#pragma unroll
      for (int m = 0; m < NCONS; m++) a.U[L.at(NCONS, m, k, j, i)] = u[m];
      const int ii = i - NGH, jj = j - NGH, kk = k - NGH;
      if ((unsigned)ii < (unsigned)L.nx && (unsigned)jj < (unsigned)L.ny && (unsigned)kk < (unsigned)L.nz) {
        R dtc, chc;
        recover_cell<R>(u, a.gam, Pout, L, a.bc, ii, jj, kk, spacing_of<R>(a, 0, i), spacing_of<R>(a, 1, j),
                        spacing_of<R>(a, 2, k), dtc, chc, bad);
        mn = smin(mn, dtc);
        mx = smax(mx, chc);
      } else if (uh_ghost_out) {
#pragma unroll
        for (int m = 0; m < NCONS; m++) uh_ghost_out[h0 + (size_t)m * L.itot] = u[m];
      }
    }
  }
  if (bad) atomicOr(&a.ctrl->status, bad);
  block_reduce_to_slot((double)mn, (double)mx, scratch, slot);
}

// Host side of one instantiation of the fused kernel.
template <class R, int TX, int TY, int NT, int MINB = 1, bool GEN = false>
struct FusedLauncher {
  using S = FusedSmem<R, TX, TY, NT, MINB>;
  static FusedShape shape() { return FusedShape{TX, TY, S::total, NT, (int)sizeof(R), MINB}; }
  static cudaError_t prepare() {
    return cudaFuncSetAttribute(k_fused_step<R, TX, TY, NT, MINB, GEN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)S::total);
  }
  static int ctas_per_sm() {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_fused_step<R, TX, TY, NT, MINB, GEN>, NT, S::total) != cudaSuccess)
      return 0;
    return n;
  }
  static cudaError_t launch(const InstanceDesc* desc, LaunchCtrl* lc, int grid, cudaStream_t s) {
    k_fused_step<R, TX, TY, NT, MINB, GEN><<<grid, NT, S::total, s>>>(desc, lc);
    return cudaGetLastError();
  }
  static const char* name() {
    static char buf[64];
    if (!buf[0])
      std::snprintf(buf, sizeof(buf), "two-phase %dx%d/%d%s%s", TX, TY, NT, MINB > 1 ? " x2" : "",
                    GEN ? " run-time solver" : "");
    return buf;
  }
  static FusedVariant variant(FusedKind kind) {
    return FusedVariant{kind, shape(), &prepare, &ctas_per_sm, &launch, name(), 0};
  }
};

template <class R>
cudaError_t recover_launch(const FusedArgs& a, int which, RedSlot* slot, int nsm, cudaStream_t s,
                           const double* uh_in, double* uh_ghost_out) {
  const int bs = 256;
  const long long n = uh_in ? (long long)a.L.itot * a.L.jtot * a.L.ktot : (long long)a.L.nx * a.L.ny * a.L.nz;
  long long g = (n + bs - 1) / bs;
  if (g > (long long)nsm * 8) g = (long long)nsm * 8;
  k_recover<R><<<(unsigned)g, bs, 0, s>>>(a, which, slot, uh_in, uh_ghost_out);
  return cudaGetLastError();
}

}  // namespace MHDGB_VNS
}  // namespace mhdgb
