// fused.cuh -- the fused solver step: one persistent launch per time step.
//
// Work decomposition.  The interior is cut into column tiles of TX x TY cells, each split along z
// into chunks of KC planes; a (tile, chunk) pair is one work item and CTAs pull items from a
// queue in the control block.  A CTA marches through its chunk plane by plane:
//   * a 4-slot shared-memory ring receives planes of P (12 primitives, the tile plus 2 halo cells
//     in x and y) through 4-D TMA tensor loads completing on per-slot mbarriers; plane k+4 is
//     requested when plane k is retired, so each load has a whole plane of compute to land;
//   * x pass: limited slopes of all 12 primitives (once per cell, van Leer) into shared memory,
//     then every x face of the plane (prim->cons, HLLD, GLM) into shared memory, then each cell
//     thread accumulates (F(i+1/2) - F(i-1/2)) * xinv;  y pass likewise;
//   * z pass: each cell thread owns its column, keeps the z slope and the lower z-face flux in
//     registers, computes the upper face from ring planes k..k+2, completes the update
//     U -= dt*(dFx*xinv + dFy*yinv + dFz*zinv) (the reference's rounding order, mhd.cpp:1438-1440),
//     damps psi (mhd.cpp:1630), recovers P (mhd.cpp:1483-1506) into the other P buffer together
//     with its ghost images for the next step, and folds the next step's dt / c_h candidates
//     into a block reduction (mhd.cpp:1542-1550, 1589-1601).
// Step n reads dt and c_h from ctrl->slot[n%3] (made by step n-1 or by the initial reduction),
// reduces into slot[(n+1)%3] and resets slot[(n+2)%3]; the last CTA to finish advances the step
// counter and the simulated time.  All launches of a run are therefore identical and can be
// captured once in a CUDA graph.
//
// R is the arithmetic type of reconstruction, Riemann solve and the P buffers (double for the
// FP64 form, float for the mixed form).  The conserved state U, the update, the psi damping and the
// pressure recovery are FP64 in both forms.
#pragma once

#include "common.cuh"
#include "fused_args.h"
#include "mhd_physics.cuh"

namespace mhdgb {

namespace MHDGB_VNS {

// Accumulator of the flux divergence dFx*xinv + dFy*yinv + dFz*zinv of one cell.
// FP64 form: plain FP64 sums in the reference's order.  Mixed form: each FP32 product is split
// exactly into value + rounding error (TwoProd with an FMA) and the three terms are added with
// TwoSum, so the pair (hi, lo) carries the sum with compensated rounding; it is rounded to FP64
// once, for the FP64 state update.  __fmul_rn/__fadd_rn keep the compiler from fusing the steps.
template <class R> struct DivAcc;
template <> struct DivAcc<double> {
  double s[NCONS];
  __device__ __forceinline__ void first(int m, double df, double inv) { s[m] = df * inv; }
  __device__ __forceinline__ void add(int m, double df, double inv) { s[m] = s[m] + df * inv; }
  __device__ __forceinline__ double total(int m) const { return s[m]; }
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
  __device__ __forceinline__ double total(int m) const { return (double)hi[m] + (double)lo[m]; }
};

template <class R> __device__ __forceinline__ R inv_of(const double* d, const float* f, int i);
template <> __device__ __forceinline__ double inv_of<double>(const double* d, const float*, int i) { return d[i]; }
template <> __device__ __forceinline__ float inv_of<float>(const double*, const float* f, int i) { return f[i]; }

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
  // x faces
  if (bc[0] == 1) { if (ii >= nx - 2) put(ii - nx, jj, kk, -1); }
  else if (bc[0] == 2) { if (ii <= 1) put(-1 - ii, jj, kk, nve1); }
  else if (bc[0] == 3) { if (ii == 0) { put(-1, jj, kk, -1); put(-2, jj, kk, -1); } }
  if (bc[1] == 1) { if (ii <= 1) put(nx + ii, jj, kk, -1); }
  else if (bc[1] == 2) { if (ii >= nx - 2) put(2 * nx - 1 - ii, jj, kk, nve1); }
  else if (bc[1] == 3) { if (ii == nx - 1) { put(nx, jj, kk, -1); put(nx + 1, jj, kk, -1); } }
  // y faces
  if (bc[2] == 1) { if (jj >= ny - 2) put(ii, jj - ny, kk, -1); }
  else if (bc[2] == 2) { if (jj <= 1) put(ii, -1 - jj, kk, nve2); }
  else if (bc[2] == 3) { if (jj == 0) { put(ii, -1, kk, -1); put(ii, -2, kk, -1); } }
  if (bc[3] == 1) { if (jj <= 1) put(ii, ny + jj, kk, -1); }
  else if (bc[3] == 2) { if (jj >= ny - 2) put(ii, 2 * ny - 1 - jj, kk, nve2); }
  else if (bc[3] == 3) { if (jj == ny - 1) { put(ii, ny, kk, -1); put(ii, ny + 1, kk, -1); } }
  // z faces
  if (bc[4] == 1) { if (kk >= nz - 2) put(ii, jj, kk - nz, -1); }
  else if (bc[4] == 2) { if (kk <= 1) put(ii, jj, -1 - kk, nve3); }
  else if (bc[4] == 3) { if (kk == 0) { put(ii, jj, -1, -1); put(ii, jj, -2, -1); } }
  if (bc[5] == 1) { if (kk <= 1) put(ii, jj, nz + kk, -1); }
  else if (bc[5] == 2) { if (kk >= nz - 2) put(ii, jj, 2 * nz - 1 - kk, nve3); }
  else if (bc[5] == 3) { if (kk == nz - 1) { put(ii, jj, nz, -1); put(ii, jj, nz + 1, -1); } }
}

// Recover P (type R) and its ghost images from U for one interior cell, and return the cell's dt
// and c_h candidates.  FP64 arithmetic for the recovery (the pressure e = (E - ekin - emag)/rho);
// the candidates are evaluated in R.
template <class R>
__device__ __forceinline__ void recover_cell(const double (&u)[NCONS], double gam, R* __restrict__ Pout,
                                             const Layout& L, const int bc[6], int ii, int jj, int kk,
                                             double dx, double dy, double dz, double& dtc, double& chc,
                                             unsigned& bad) {
  double pd[NPRIM];
  cons2prim<double>(u, gam, pd);
  R pr[NPRIM];
#pragma unroll
  for (int n = 0; n < NPRIM; n++) pr[n] = (R)pd[n];
#pragma unroll
  for (int n = 0; n < NPRIM; n++) Pout[L.at(NPRIM, n, kk + NGH, jj + NGH, ii + NGH)] = pr[n];
  write_ghost_images<R>(Pout, L, bc, ii, jj, kk, pr);
  dtc = (double)cell_dt<R>(pr, (R)dx, (R)dy, (R)dz);
  chc = (double)cell_ch<R>(pr);
  if (!(dtc == dtc) || !(chc == chc) || isinf(chc)) bad |= ST_NONFINITE;
  if (!(pd[nden] > 0.0) || !(pd[npre] > 0.0)) bad |= ST_NEGATIVE;
}

template <class R, int TX, int TY>
__global__ void __launch_bounds__(TX * TY, 1)
k_fused_step(const __grid_constant__ CUtensorMap tmap0, const __grid_constant__ CUtensorMap tmap1, FusedArgs a) {
  using S = FusedSmem<R, TX, TY>;
  constexpr int NBUF = S::NBUF, PX = S::PX, SX = S::SX, FX = S::FX, NT = TX * TY;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char* smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);  // TMA destinations
  R* ring = reinterpret_cast<R*>(smem + S::ring_off);
  R* slp = reinterpret_cast<R*>(smem + S::slope_off);
  R* flx = reinterpret_cast<R*>(smem + S::flux_off);
  double* red = reinterpret_cast<double*>(smem + S::red_off);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + S::bar_off);
  int& s_item = *reinterpret_cast<int*>(smem + S::misc_off);
  int& s_abort = *reinterpret_cast<int*>(smem + S::misc_off + 4);

  Ctrl* ctrl = a.ctrl;
  if (ctrl->done) return;
  const Layout L = a.L;
  const int tid = threadIdx.x;
  const unsigned long long step = ctrl->step;
  const int par = (int)(step & 1);
  const R* __restrict__ Pin = reinterpret_cast<const R*>(a.P[par]);
  R* __restrict__ Pout = reinterpret_cast<R*>(a.P[par ^ 1]);
  const CUtensorMap* tmap = par ? &tmap1 : &tmap0;
  (void)Pin;
  const RedSlot cur = ctrl->slot[step % 3];
  const double dt = a.cfl * bitsd(cur.dtmin_bits);
  const double chd = bitsd(cur.chmax_bits);
  const R chg = (R)chd;
  RedSlot* next = &ctrl->slot[(step + 1) % 3];
  if (blockIdx.x == 0 && tid == 0) {
    ctrl->slot[(step + 2) % 3].dtmin_bits = DT_RESET;
    ctrl->slot[(step + 2) % 3].chmax_bits = CH_RESET;
  }
  if (tid == 0) {
    prefetch_tensormap(tmap);
    for (int s = 0; s < NBUF; s++) mbar_init(&bars[s], 1);
    fence_mbar_init();
    s_abort = 0;
  }
  __syncthreads();

  unsigned fills[NBUF];  // loads issued per slot (identical in every thread)
#pragma unroll
  for (int s = 0; s < NBUF; s++) fills[s] = 0;

  const int tx = tid % TX, ty = tid / TX;
  double dmin = 1.0e308, cmax = 0.0;
  unsigned bad = 0;
  const int nitems = a.ntx * a.nty * a.nkc;

  for (;;) {
    if (tid == 0) s_item = (int)atomicAdd(&ctrl->work_next, 1u);
    __syncthreads();
    const int item = s_item;
    if (item >= nitems || s_abort) break;
    const int bxi = item % a.ntx, byi = (item / a.ntx) % a.nty, bki = item / (a.ntx * a.nty);
    const int i0 = bxi * TX, j0 = byi * TY;
    const int kb = bki * a.kc, ke = min(kb + a.kc, L.nz);
    const int cx = min(TX, L.nx - i0), cy = min(TY, L.ny - j0);
    const bool own = tx < cx && ty < cy;
    const int ii = i0 + tx, jj = j0 + ty;

    // ring slot of plane p (p relative to kb-2)
    auto slot_of = [&](int p) { return (p - (kb - 2)) % NBUF; };
    auto plane = [&](int p) -> R* { return ring + (size_t)slot_of(p) * S::PLANE; };
    auto issue = [&](int p) {  // thread 0 only
      const int s = slot_of(p);
      mbar_arrive_expect_tx(&bars[s], S::plane_tx_bytes);
      tma_load_4d(ring + (size_t)s * S::PLANE, tmap, i0, 0, j0, p + NGH, &bars[s]);
    };
    auto wait_plane = [&](int p) {
      const int s = slot_of(p);
      if (!mbar_wait(&bars[s], (fills[s] - 1) & 1, &ctrl->status)) s_abort = 1;
    };
    // P value of field n at local (i,j) of plane buffer pl; i,j in [-2, T+2)
    auto PV = [&](const R* pl, int n, int i, int j) -> R { return pl[((j + 2) * NPRIM + n) * PX + (i + 2)]; };

    // prologue: planes kb-2 .. kb+1
    if (tid == 0) {
      fence_proxy_async();
      for (int p = kb - 2; p < kb - 2 + NBUF; p++)
        if (p <= ke + 1) issue(p);
    }
#pragma unroll
    for (int s = 0; s < NBUF; s++) fills[s]++;  // every slot received one load (all p <= ke+1 here)
    for (int p = kb - 2; p <= kb + 1; p++) wait_plane(p);
    __syncthreads();
    if (s_abort) break;

    R zs_cur[NPRIM];   // z slope of the thread's cell at plane k
    R fz_lo[NCONS];    // flux through face k-1/2
    if (own) {
      const R *pm2 = plane(kb - 2), *pm1 = plane(kb - 1), *p0 = plane(kb), *pp1 = plane(kb + 1);
      R pl[NPRIM], pr[NPRIM];
#pragma unroll
      for (int n = 0; n < NPRIM; n++) {
        const R a2 = PV(pm2, n, tx, ty), a1 = PV(pm1, n, tx, ty), b0 = PV(p0, n, tx, ty), b1 = PV(pp1, n, tx, ty);
        const R zsm1 = van_leer(b0 - a1, a1 - a2);
        zs_cur[n] = van_leer(b1 - b0, b0 - a1);
        pl[n] = left_state(a1, zsm1);
        pr[n] = right_state(b0, zs_cur[n]);
      }
      face_flux<R, 3>(pl, pr, chg, fz_lo);
    }
    __syncthreads();  // planes kb-2, kb-1 retired
    if (tid == 0) {
      fence_proxy_async();
      if (kb + 2 <= ke + 1) issue(kb + 2);
      if (kb + 3 <= ke + 1) issue(kb + 3);
    }
    if (kb + 2 <= ke + 1) fills[slot_of(kb + 2)]++;
    if (kb + 3 <= ke + 1) fills[slot_of(kb + 3)]++;

    for (int k = kb; k < ke; k++) {
      const R* pk = plane(k);
      DivAcc<R> acc;
      // ---- x pass ----
      {
        const int nsl = cy * (cx + 2);
        for (int it = tid; it < nsl; it += NT) {
          const int j = it / (cx + 2), i = it % (cx + 2) - 1;
#pragma unroll
          for (int n = 0; n < NPRIM; n++) {
            const R m1 = PV(pk, n, i - 1, j), c0 = PV(pk, n, i, j), p1 = PV(pk, n, i + 1, j);
            slp[(n * S::SY + (j + 1)) * SX + (i + 1)] = van_leer(p1 - c0, c0 - m1);
          }
        }
        __syncthreads();
        const int nf = cy * (cx + 1);
        for (int it = tid; it < nf; it += NT) {
          const int j = it / (cx + 1), i = it % (cx + 1);
          R pl[NPRIM], pr[NPRIM], f[NCONS];
#pragma unroll
          for (int n = 0; n < NPRIM; n++) {
            pl[n] = left_state(PV(pk, n, i - 1, j), slp[(n * S::SY + (j + 1)) * SX + i]);
            pr[n] = right_state(PV(pk, n, i, j), slp[(n * S::SY + (j + 1)) * SX + (i + 1)]);
          }
          face_flux<R, 1>(pl, pr, chg, f);
#pragma unroll
          for (int m = 0; m < NCONS; m++) flx[(m * S::FY + j) * FX + i] = f[m];
        }
        __syncthreads();
        if (own) {
          const R xi = inv_of<R>(a.xinv, a.xinvf, ii + NGH);
#pragma unroll
          for (int m = 0; m < NCONS; m++)
            acc.first(m, flx[(m * S::FY + ty) * FX + tx + 1] - flx[(m * S::FY + ty) * FX + tx], xi);
        }
        __syncthreads();
      }
      // ---- y pass ----
      {
        const int nsl = (cy + 2) * cx;
        for (int it = tid; it < nsl; it += NT) {
          const int j = it / cx - 1, i = it % cx;
#pragma unroll
          for (int n = 0; n < NPRIM; n++) {
            const R m1 = PV(pk, n, i, j - 1), c0 = PV(pk, n, i, j), p1 = PV(pk, n, i, j + 1);
            slp[(n * S::SY + (j + 1)) * SX + (i + 1)] = van_leer(p1 - c0, c0 - m1);
          }
        }
        __syncthreads();
        const int nf = (cy + 1) * cx;
        for (int it = tid; it < nf; it += NT) {
          const int j = it / cx, i = it % cx;
          R pl[NPRIM], pr[NPRIM], f[NCONS];
#pragma unroll
          for (int n = 0; n < NPRIM; n++) {
            pl[n] = left_state(PV(pk, n, i, j - 1), slp[(n * S::SY + j) * SX + (i + 1)]);
            pr[n] = right_state(PV(pk, n, i, j), slp[(n * S::SY + (j + 1)) * SX + (i + 1)]);
          }
          face_flux<R, 2>(pl, pr, chg, f);
#pragma unroll
          for (int m = 0; m < NCONS; m++) flx[(m * S::FY + j) * FX + i] = f[m];
        }
        __syncthreads();
        if (own) {
          const R yi = inv_of<R>(a.yinv, a.yinvf, (a.quirk ? ii : jj) + NGH);
#pragma unroll
          for (int m = 0; m < NCONS; m++)
            acc.add(m, flx[(m * S::FY + ty + 1) * FX + tx] - flx[(m * S::FY + ty) * FX + tx], yi);
        }
      }
      // ---- z pass + update ----
      wait_plane(k + 2);
      if (own && !s_abort) {
        const R *p1 = plane(k + 1), *p2 = plane(k + 2);
        R zs_nx[NPRIM], pl[NPRIM], pr[NPRIM], fz_hi[NCONS];
#pragma unroll
        for (int n = 0; n < NPRIM; n++) {
          const R c0 = PV(pk, n, tx, ty), c1 = PV(p1, n, tx, ty), c2 = PV(p2, n, tx, ty);
          zs_nx[n] = van_leer(c2 - c1, c1 - c0);
          pl[n] = left_state(c0, zs_cur[n]);
          pr[n] = right_state(c1, zs_nx[n]);
        }
        face_flux<R, 3>(pl, pr, chg, fz_hi);
        const R zi = inv_of<R>(a.zinv, a.zinvf, (a.quirk ? ii : k) + NGH);
        double u[NCONS];
#pragma unroll
        for (int m = 0; m < NCONS; m++) {
          acc.add(m, fz_hi[m] - fz_lo[m], zi);
          const size_t c = L.at(NCONS, m, k + NGH, jj + NGH, ii + NGH);
          u[m] = a.U[c] - dt * acc.total(m);
        }
        // DampPsi (mhd.cpp:1628-1630)
        double dhl = a.dxs[ii + NGH];
        if (a.dys[jj + NGH] < dhl) dhl = a.dys[jj + NGH];
        if (a.dzs[k + NGH] < dhl) dhl = a.dzs[k + NGH];
        const double taui = 0.1 * chd / dhl;
        u[mbps] = u[mbps] * (1.0 - dt * taui);
#pragma unroll
        for (int m = 0; m < NCONS; m++) a.U[L.at(NCONS, m, k + NGH, jj + NGH, ii + NGH)] = u[m];
        double dtc, chc;
        recover_cell<R>(u, a.gam, Pout, L, a.bc, ii, jj, k, a.dxs[ii + NGH], a.dys[jj + NGH], a.dzs[k + NGH],
                        dtc, chc, bad);
        dmin = smin(dmin, dtc);
        cmax = smax(cmax, chc);
#pragma unroll
        for (int n = 0; n < NPRIM; n++) zs_cur[n] = zs_nx[n];
#pragma unroll
        for (int m = 0; m < NCONS; m++) fz_lo[m] = fz_hi[m];
      }
      __syncthreads();  // plane k retired
      if (s_abort) break;
      if (k + 4 <= ke + 1) {
        if (tid == 0) {
          fence_proxy_async();
          issue(k + 4);
        }
        fills[slot_of(k + 4)]++;
      }
    }
    if (s_abort) break;
    __syncthreads();
  }

  if (s_abort) {
    // drain: wait (bounded) for any load still in flight before leaving
    for (int s = 0; s < NBUF; s++)
      if (fills[s]) mbar_wait(&bars[s], (fills[s] - 1) & 1, &ctrl->status);
  }
  if (bad) atomicOr(&ctrl->status, bad);
  block_reduce_to_slot(dmin, cmax, red, next);
  if (tid == 0) {
    __threadfence();
    const unsigned prev = atomicAdd(&ctrl->blocks_done, 1u);
    if (prev == gridDim.x - 1) {
      __threadfence();
      ctrl->last_dt = dt;
      ctrl->last_ch = chd;
      ctrl->time += dt;
      ctrl->step = step + 1;
      ctrl->work_next = 0;
      ctrl->blocks_done = 0;
      if (ctrl->time > ctrl->tmax || ctrl->step >= ctrl->max_step) ctrl->done = 1;
      __threadfence();
    }
  }
}

// Recovery of P from U for the interior (+ ghost images) and the dt/c_h reduction into
// ctrl->slot[step % 3]: the state a fused run starts from.
template <class R>
__global__ void k_recover(const double* __restrict__ U, void* P, Layout L, int bc0, int bc1, int bc2, int bc3,
                          int bc4, int bc5, const double* __restrict__ dxs, const double* __restrict__ dys,
                          const double* __restrict__ dzs, double gam, RedSlot* slot, unsigned* status) {
  __shared__ double scratch[64];
  const int bc[6] = {bc0, bc1, bc2, bc3, bc4, bc5};
  const long long n = (long long)L.nx * L.ny * L.nz;
  double mn = 1.0e308, mx = 0.0;
  unsigned bad = 0;
  R* Pout = reinterpret_cast<R*>(P);
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int ii = (int)(t % L.nx), jj = (int)((t / L.nx) % L.ny), kk = (int)(t / ((long long)L.nx * L.ny));
    double u[NCONS];
#pragma unroll
    for (int m = 0; m < NCONS; m++) u[m] = U[L.at(NCONS, m, kk + NGH, jj + NGH, ii + NGH)];
    double dtc, chc;
    recover_cell<R>(u, gam, Pout, L, bc, ii, jj, kk, dxs[ii + NGH], dys[jj + NGH], dzs[kk + NGH], dtc, chc, bad);
    mn = smin(mn, dtc);
    mx = smax(mx, chc);
  }
  if (bad) atomicOr(status, bad);
  block_reduce_to_slot(mn, mx, scratch, slot);
}

// Host side of one instantiation of the fused kernel.
template <class R, int TX, int TY>
struct FusedLauncher {
  using S = FusedSmem<R, TX, TY>;
  static FusedShape shape() { return FusedShape{TX, TY, S::total, TX * TY, (int)sizeof(R)}; }
  static cudaError_t prepare() {
    return cudaFuncSetAttribute(k_fused_step<R, TX, TY>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::total);
  }
  static int ctas_per_sm() {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_fused_step<R, TX, TY>, TX * TY, S::total) != cudaSuccess)
      return 0;
    return n;
  }
  static cudaError_t launch(const CUtensorMap maps[2], const FusedArgs& a, int grid, cudaStream_t s) {
    k_fused_step<R, TX, TY><<<grid, TX * TY, S::total, s>>>(maps[0], maps[1], a);
    return cudaGetLastError();
  }
};

template <class R>
cudaError_t recover_launch(const double* U, void* P, const Layout& L, const int bc[6], const double* dxs,
                           const double* dys, const double* dzs, double gam, RedSlot* slot, unsigned* status,
                           int nsm, cudaStream_t s) {
  const int bs = 256;
  const long long n = (long long)L.nx * L.ny * L.nz;
  long long g = (n + bs - 1) / bs;
  if (g > (long long)nsm * 8) g = (long long)nsm * 8;
  k_recover<R><<<(unsigned)g, bs, 0, s>>>(U, P, L, bc[0], bc[1], bc[2], bc[3], bc[4], bc[5], dxs, dys, dzs, gam,
                                          slot, status);
  return cudaGetLastError();
}

}  // namespace MHDGB_VNS
}  // namespace mhdgb
