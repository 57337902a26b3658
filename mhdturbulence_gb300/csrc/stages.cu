// stages.cu -- one CUDA kernel per reference stage (the stage-exact path behind the reference's
// hydflux_mod / boundary_mod functions).  Built with -fmad=false: every operation is rounded
// separately, as in the reference's CPU build, so the FP64 results match the reference bit for bit.
//
//   GetNumericalFluxD  (mhd.cpp:987-1410)    -> k_flux<DIR>
//   UpdateConservU     (mhd.cpp:1412-1444)   -> k_update_conserv
//   DampPsi            (mhd.cpp:1613-1633)   -> k_damp_psi
//   UpdatePrimitvP     (mhd.cpp:1447-1509)   -> k_update_prim
//   ControlTimestep / EvaluateCh (mhd.cpp:1511-1611, + MPIminfind/MPImaxfind) -> k_reduce_dt_ch
//   SetBoundaryCondition (boundary.cpp:750-893, single-rank SendRecvBoundary) -> k_pack + k_unpack
#define MHDGB_FAST 0
#define MHDGB_VNS v_exact
#include "fused.cuh"
#include "kernels.h"

namespace mhdgb {
namespace v_exact {

// One thread per face.  Faces of direction DIR cover i in [is, ie+di], j in [js, je+dj],
// k in [ks, ke+dk] (mhd.cpp:1205, 1288, 1371); the flux is stored at the face's upper cell index.
template <int DIR>
__global__ void k_flux(const double* __restrict__ P, double* __restrict__ F, Layout L,
                       const double* __restrict__ chg_ptr, int riemann) {
  constexpr int di = DIR == 1, dj = DIR == 2, dk = DIR == 3;
  const int nfx = L.nx + di, nfy = L.ny + dj, nfz = L.nz + dk;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)nfx * nfy * nfz) return;
  const int i = NGH + (int)(t % nfx);
  const int j = NGH + (int)((t / nfx) % nfy);
  const int k = NGH + (int)(t / ((long long)nfx * nfy));
  const double chg = *chg_ptr;
  double L1[NPRIM], L2[NPRIM], R1[NPRIM], R2[NPRIM], Pl[NPRIM], Pr[NPRIM];
#pragma unroll
  for (int n = 0; n < NPRIM; n++) {
    L1[n] = P[L.at(NPRIM, n, k - 2 * dk, j - 2 * dj, i - 2 * di)];
    L2[n] = P[L.at(NPRIM, n, k - dk, j - dj, i - di)];
    R1[n] = P[L.at(NPRIM, n, k, j, i)];
    R2[n] = P[L.at(NPRIM, n, k + dk, j + dj, i + di)];
  }
  // CalcFlux, mhd.cpp:1134-1154
#pragma unroll
  for (int n = 0; n < NPRIM; n++) {
    Pl[n] = left_state(L2[n], van_leer(R1[n] - L2[n], L2[n] - L1[n]));
    Pr[n] = right_state(R1[n], van_leer(R2[n] - R1[n], R1[n] - L2[n]));
  }
  double f[NCONS];
  face_flux<double, DIR>(Pl, Pr, glm_const(chg), f, riemann);
#pragma unroll
  for (int m = 0; m < NCONS; m++) F[L.at(NCONS, m, k, j, i)] = f[m];
}

// U -= dt * (dFx*xinv + dFy*yinv + dFz*zinv), mhd.cpp:1431-1442.  yinv/zinv are indexed by
// jsel/ksel: the cell's own j/k, or its i when reproducing mhd.cpp:1435-1436.
__global__ void k_update_conserv(const double* __restrict__ Fx, const double* __restrict__ Fy,
                                 const double* __restrict__ Fz, double* __restrict__ U, Layout L,
                                 const double* __restrict__ xinv, const double* __restrict__ yinv,
                                 const double* __restrict__ zinv, int quirk, const double* __restrict__ dt_ptr) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)L.nx * L.ny * L.nz) return;
  const int i = NGH + (int)(t % L.nx);
  const int j = NGH + (int)((t / L.nx) % L.ny);
  const int k = NGH + (int)(t / ((long long)L.nx * L.ny));
  const double dt = *dt_ptr;
  const double xi = xinv[i], yi = yinv[quirk ? i : j], zi = zinv[quirk ? i : k];
#pragma unroll
  for (int m = 0; m < NCONS; m++) {
    const size_t c = L.at(NCONS, m, k, j, i);
    U[c] = U[c] - dt * ((Fx[L.at(NCONS, m, k, j, i + 1)] - Fx[c]) * xi
                      + (Fy[L.at(NCONS, m, k, j + 1, i)] - Fy[c]) * yi
                      + (Fz[L.at(NCONS, m, k + 1, j, i)] - Fz[c]) * zi);
  }
}

// psi <- psi * (1 - dt * alpha * chg / min(dx,dy,dz)), mhd.cpp:1625-1631.
__global__ void k_damp_psi(double* __restrict__ U, Layout L, const double* __restrict__ dxs,
                           const double* __restrict__ dys, const double* __restrict__ dzs,
                           const double* __restrict__ dt_ptr, const double* __restrict__ chg_ptr) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)L.nx * L.ny * L.nz) return;
  const int i = NGH + (int)(t % L.nx);
  const int j = NGH + (int)((t / L.nx) % L.ny);
  const int k = NGH + (int)(t / ((long long)L.nx * L.ny));
  const double alphabp = 0.1;
  double dhl = dxs[i];
  if (dys[j] < dhl) dhl = dys[j];
  if (dzs[k] < dhl) dhl = dzs[k];
  const double taui = alphabp * *chg_ptr / dhl;
  const size_t c = L.at(NCONS, mbps, k, j, i);
  U[c] = U[c] * (1.0 - *dt_ptr * taui);
}

// UpdatePrimitvP over the interior, mhd.cpp:1480-1507.
__global__ void k_update_prim(const double* __restrict__ U, double* __restrict__ P, Layout L, double gam) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)L.nx * L.ny * L.nz) return;
  const int i = NGH + (int)(t % L.nx);
  const int j = NGH + (int)((t / L.nx) % L.ny);
  const int k = NGH + (int)(t / ((long long)L.nx * L.ny));
  double u[NCONS], p[NPRIM];
#pragma unroll
  for (int m = 0; m < NCONS; m++) u[m] = U[L.at(NCONS, m, k, j, i)];
  cons2prim<double>(u, gam, p);
#pragma unroll
  for (int n = 0; n < NPRIM; n++) P[L.at(NPRIM, n, k, j, i)] = p[n];
}

// Snapshot of the interior primitives in the order of the reference's output (MPI_IO_Pack,
// output.cpp:247-260): out[v][k][j][i] (dense nz*ny*nx per variable) for v = d, v1, v2, v3, b1, b2,
// b3, bp, p, X1.  Copies P when given, else recovers the primitives from U with UpdatePrimitvP's
// arithmetic (the values P holds after a step).  One thread per interior cell, i fastest.
__global__ void k_snapshot(const double* __restrict__ U, const double* __restrict__ P, Layout L, double gam,
                           double* __restrict__ out) {
  const long long ncell = (long long)L.nx * L.ny * L.nz;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ncell) return;
  const int i = NGH + (int)(t % L.nx);
  const int j = NGH + (int)((t / L.nx) % L.ny);
  const int k = NGH + (int)(t / ((long long)L.nx * L.ny));
  double p[NPRIM];
  if (P) {
#pragma unroll
    for (int n = 0; n < NPRIM; n++) p[n] = P[L.at(NPRIM, n, k, j, i)];
  } else {
    double u[NCONS];
#pragma unroll
    for (int m = 0; m < NCONS; m++) u[m] = U[L.at(NCONS, m, k, j, i)];
    cons2prim<double>(u, gam, p);
  }
  const int order[NSNAP] = {nden, nve1, nve2, nve3, nbm1, nbm2, nbm3, nbps, npre, nst};
#pragma unroll
  for (int v = 0; v < NSNAP; v++) out[v * ncell + t] = p[order[v]];
}


// a reduction slot; cells with a non-finite value, rho <= 0 or p <= 0 raise status bits.
__global__ void k_reduce_dt_ch(const double* __restrict__ P, Layout L, const double* __restrict__ dxs,
                               const double* __restrict__ dys, const double* __restrict__ dzs,
                               RedSlot* slot, unsigned* status) {
  __shared__ double scratch[64];
  const long long n = (long long)L.nx * L.ny * L.nz;
  double mn = 1.0e308, mx = 0.0;
  unsigned bad = 0;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int i = NGH + (int)(t % L.nx);
    const int j = NGH + (int)((t / L.nx) % L.ny);
    const int k = NGH + (int)(t / ((long long)L.nx * L.ny));
    double p[NPRIM];
#pragma unroll
    for (int q = 0; q < NPRIM; q++) p[q] = P[L.at(NPRIM, q, k, j, i)];
    const double dt = cell_dt<double>(p, dxs[i], dys[j], dzs[k]);
    const double ch = cell_ch<double>(p);
    if (!(dt == dt) || !(ch == ch) || isinf(ch)) bad |= ST_NONFINITE;
    if (!(p[nden] > 0.0) || !(p[npre] > 0.0)) bad |= ST_NEGATIVE;
    mn = smin(mn, dt);
    mx = smax(mx, ch);
  }
  if (bad) atomicOr(status, bad);
  block_reduce_to_slot(mn, mx, scratch, slot);
}

__global__ void k_reset_slot(RedSlot* slot) {
  slot->dtmin_bits = DT_RESET;
  slot->chmax_bits = CH_RESET;
}

// dt = cfl * min and chg = max of a slot, written as plain doubles for the stage kernels.
__global__ void k_slot_to_scalars(const RedSlot* slot, double cfl, double* dt_out, double* ch_out) {
  *dt_out = cfl * bitsd(slot->dtmin_bits);
  *ch_out = bitsd(slot->chmax_bits);
}

// ---------------------------------------------------------------------------------------------
// Ghost fill with the reference's pack -> fill -> unpack semantics (boundary.cpp:771-891 and the
// ntiles==1 branches of SendRecvBoundary): all three directions are packed from P before any
// ghost is written, then x, y and z ghost layers are written in that order over the full
// transverse extents.  This reproduces even the edge/corner ghost values of the reference.
// Pack buffers: X [nprim][ktot][jtot][2] per side, Y [nprim][ktot][2][itot], Z [nprim][2][jtot][itot].
// ---------------------------------------------------------------------------------------------
struct PackBufs {
  double *xs, *xe, *ys, *ye, *zs, *ze;
};

__global__ void k_pack(const double* __restrict__ P, Layout L, PackBufs B) {
  const int it = L.itot, jt = L.jtot, kt = L.ktot;
  const int ie = NGH + L.nx - 1, je = NGH + L.ny - 1, ke = NGH + L.nz - 1;
  const long long nX = (long long)NPRIM * kt * jt * NGH, nY = (long long)NPRIM * kt * NGH * it,
                  nZ = (long long)NPRIM * NGH * jt * it;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < nX + nY + nZ;
       t += (long long)gridDim.x * blockDim.x) {
    if (t < nX) {  // X[n][k][j][i]
      const int i = (int)(t % NGH), j = (int)((t / NGH) % jt), k = (int)((t / (NGH * jt)) % kt),
                n = (int)(t / ((long long)NGH * jt * kt));
      B.xs[t] = P[L.at(NPRIM, n, k, j, ie - NGH + 1 + i)];
      B.xe[t] = P[L.at(NPRIM, n, k, j, NGH + i)];
    } else if (t < nX + nY) {  // Y[n][k][j][i]
      const long long s = t - nX;
      const int i = (int)(s % it), j = (int)((s / it) % NGH), k = (int)((s / (it * NGH)) % kt),
                n = (int)(s / ((long long)it * NGH * kt));
      B.ys[s] = P[L.at(NPRIM, n, k, je - NGH + 1 + j, i)];
      B.ye[s] = P[L.at(NPRIM, n, k, NGH + j, i)];
    } else {  // Z[n][k][j][i]
      const long long s = t - nX - nY;
      const int i = (int)(s % it), j = (int)((s / it) % jt), k = (int)((s / ((long long)it * jt)) % NGH),
                n = (int)(s / ((long long)it * jt * NGH));
      B.zs[s] = P[L.at(NPRIM, n, ke - NGH + 1 + k, j, i)];
      B.ze[s] = P[L.at(NPRIM, n, NGH + k, j, i)];
    }
  }
}

// Ghost value of one side: periodic copies the opposite side's layer at the same offset,
// reflection mirrors this side's layers and negates the normal velocity, outflow repeats the
// first interior layer (boundary.cpp:152-169 and equivalents).
__device__ __forceinline__ double fill_value(int bc, const double* same, const double* opp, long long at_same,
                                             long long at_mirror, long long at_first, int n, int nvel) {
  if (bc == 1) return opp[at_same];
  if (bc == 2) { const double v = same[at_mirror]; return n == nvel ? -v : v; }
  if (bc == 3) return same[at_first];
  return 0.0;
}

template <int AX>
__global__ void k_unpack(double* __restrict__ P, Layout L, PackBufs B, int bc_in, int bc_out) {
  const int it = L.itot, jt = L.jtot, kt = L.ktot;
  const int ie = NGH + L.nx - 1, je = NGH + L.ny - 1, ke = NGH + L.nz - 1;
  const long long n1 = AX == 0 ? NGH : it, n2 = AX == 1 ? NGH : jt, n3 = AX == 2 ? NGH : kt;
  const long long tot = NPRIM * n1 * n2 * n3;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < tot; t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t % n1), j = (int)((t / n1) % n2), k = (int)((t / (n1 * n2)) % n3),
              n = (int)(t / (n1 * n2 * n3));
    long long mir, first, last;
    if (AX == 0) {
      mir = (((long long)n * kt + k) * jt + j) * NGH + (NGH - 1 - i);
      first = (((long long)n * kt + k) * jt + j) * NGH;
      last = first + NGH - 1;
      // Br.Xs <- Bs.Xs (periodic) / Bs.Xe mirrored / Bs.Xe(0);  Br.Xe <- Bs.Xe / Bs.Xs mirrored / Bs.Xs(ngh-1)
      const double vin = bc_in == 3 ? B.xe[first] : fill_value(bc_in, B.xe, B.xs, t, mir, first, n, nve1);
      const double vout = bc_out == 3 ? B.xs[last] : fill_value(bc_out, B.xs, B.xe, t, mir, first, n, nve1);
      if (bc_in != BC_EXCHANGE) P[L.at(NPRIM, n, k, j, i)] = vin;
      if (bc_out != BC_EXCHANGE) P[L.at(NPRIM, n, k, j, ie + 1 + i)] = vout;
    } else if (AX == 1) {
      mir = (((long long)n * kt + k) * NGH + (NGH - 1 - j)) * it + i;
      first = (((long long)n * kt + k) * NGH + 0) * it + i;
      last = (((long long)n * kt + k) * NGH + (NGH - 1)) * it + i;
      const double vin = bc_in == 3 ? B.ye[first] : fill_value(bc_in, B.ye, B.ys, t, mir, first, n, nve2);
      const double vout = bc_out == 3 ? B.ys[last] : fill_value(bc_out, B.ys, B.ye, t, mir, first, n, nve2);
      if (bc_in != BC_EXCHANGE) P[L.at(NPRIM, n, k, j, i)] = vin;
      if (bc_out != BC_EXCHANGE) P[L.at(NPRIM, n, k, je + 1 + j, i)] = vout;
    } else {
      mir = (((long long)n * NGH + (NGH - 1 - k)) * jt + j) * it + i;
      first = (((long long)n * NGH + 0) * jt + j) * it + i;
      last = (((long long)n * NGH + (NGH - 1)) * jt + j) * it + i;
      const double vin = bc_in == 3 ? B.ze[first] : fill_value(bc_in, B.ze, B.zs, t, mir, first, n, nve3);
      const double vout = bc_out == 3 ? B.zs[last] : fill_value(bc_out, B.zs, B.ze, t, mir, first, n, nve3);
      if (bc_in != BC_EXCHANGE) P[L.at(NPRIM, n, k, j, i)] = vin;
      if (bc_out != BC_EXCHANGE) P[L.at(NPRIM, n, ke + 1 + k, j, i)] = vout;
    }
  }
}

}  // namespace v_exact

// ---------------------------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------------------------
using namespace v_exact;

static inline unsigned nblk(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

cudaError_t launch_flux(int dir, const double* P, double* F, const Layout& L, const double* chg, int riemann,
                        cudaStream_t s) {
  const int bs = 128;
  if (dir == 1) k_flux<1><<<nblk((long long)(L.nx + 1) * L.ny * L.nz, bs), bs, 0, s>>>(P, F, L, chg, riemann);
  else if (dir == 2) k_flux<2><<<nblk((long long)L.nx * (L.ny + 1) * L.nz, bs), bs, 0, s>>>(P, F, L, chg, riemann);
  else k_flux<3><<<nblk((long long)L.nx * L.ny * (L.nz + 1), bs), bs, 0, s>>>(P, F, L, chg, riemann);
  return cudaGetLastError();
}

cudaError_t launch_update_conserv(const double* Fx, const double* Fy, const double* Fz, double* U, const Layout& L,
                                  const double* xinv, const double* yinv, const double* zinv, int quirk,
                                  const double* dt, cudaStream_t s) {
  const int bs = 256;
  k_update_conserv<<<nblk((long long)L.nx * L.ny * L.nz, bs), bs, 0, s>>>(Fx, Fy, Fz, U, L, xinv, yinv, zinv, quirk, dt);
  return cudaGetLastError();
}

cudaError_t launch_damp_psi(double* U, const Layout& L, const double* dxs, const double* dys, const double* dzs,
                            const double* dt, const double* chg, cudaStream_t s) {
  const int bs = 256;
  k_damp_psi<<<nblk((long long)L.nx * L.ny * L.nz, bs), bs, 0, s>>>(U, L, dxs, dys, dzs, dt, chg);
  return cudaGetLastError();
}

cudaError_t launch_update_prim(const double* U, double* P, const Layout& L, double gam, cudaStream_t s) {
  const int bs = 256;
  k_update_prim<<<nblk((long long)L.nx * L.ny * L.nz, bs), bs, 0, s>>>(U, P, L, gam);
  return cudaGetLastError();
}

cudaError_t launch_reduce_dt_ch(const double* P, const Layout& L, const double* dxs, const double* dys,
                                const double* dzs, RedSlot* slot, unsigned* status, int nsm, cudaStream_t s) {
  k_reset_slot<<<1, 1, 0, s>>>(slot);
  const int bs = 256;
  long long n = (long long)L.nx * L.ny * L.nz;
  unsigned g = nblk(n, bs);
  if (g > (unsigned)(nsm * 8)) g = nsm * 8;
  k_reduce_dt_ch<<<g, bs, 0, s>>>(P, L, dxs, dys, dzs, slot, status);
  return cudaGetLastError();
}

cudaError_t launch_slot_to_scalars(const RedSlot* slot, double cfl, double* dt, double* ch, cudaStream_t s) {
  k_slot_to_scalars<<<1, 1, 0, s>>>(slot, cfl, dt, ch);
  return cudaGetLastError();
}

cudaError_t launch_reset_slot(RedSlot* slot, cudaStream_t s) {
  k_reset_slot<<<1, 1, 0, s>>>(slot);
  return cudaGetLastError();
}

cudaError_t launch_snapshot(const double* U, const double* P, const Layout& L, double gam, double* out,
                            cudaStream_t s) {
  const int bs = 256;
  k_snapshot<<<nblk((long long)L.nx * L.ny * L.nz, bs), bs, 0, s>>>(U, P, L, gam, out);
  return cudaGetLastError();
}

size_t pack_buffer_doubles(const Layout& L) {
  return 2 * ((size_t)NPRIM * L.ktot * L.jtot * NGH + (size_t)NPRIM * L.ktot * NGH * L.itot +
              (size_t)NPRIM * NGH * L.jtot * L.itot);
}

cudaError_t launch_ghost_fill(double* P, const Layout& L, const int bc[6], double* scratch, cudaStream_t s) {
  PackBufs B;
  const size_t nX = (size_t)NPRIM * L.ktot * L.jtot * NGH, nY = (size_t)NPRIM * L.ktot * NGH * L.itot,
               nZ = (size_t)NPRIM * NGH * L.jtot * L.itot;
  B.xs = scratch; B.xe = B.xs + nX;
  B.ys = B.xe + nX; B.ye = B.ys + nY;
  B.zs = B.ye + nY; B.ze = B.zs + nZ;
  const int bs = 256;
  k_pack<<<nblk((long long)(nX + nY + nZ), bs), bs, 0, s>>>(P, L, B);
  k_unpack<0><<<nblk((long long)nX, bs), bs, 0, s>>>(P, L, B, bc[0], bc[1]);
  k_unpack<1><<<nblk((long long)nY, bs), bs, 0, s>>>(P, L, B, bc[2], bc[3]);
  k_unpack<2><<<nblk((long long)nZ, bs), bs, 0, s>>>(P, L, B, bc[4], bc[5]);
  return cudaGetLastError();
}

namespace detail {
int variants_exact(const FusedVariant** out) {
  static const FusedVariant v[] = {
      preferred_variant(v_exact::FusedLauncher<double, 32, 4, 128>::variant(FUSED_FP64_EXACT)),
      // the run-time solver kernel (HLLE / HLLC); not one of the tuned variants
      v_exact::FusedLauncher<double, 32, 4, 128, 1, true>::variant(FUSED_FP64_EXACT),
  };
  *out = v;
  return (int)(sizeof(v) / sizeof(v[0])) - 1;  // the last entry is the run-time solver kernel
}
cudaError_t recover_exact(const FusedArgs& a, int which, RedSlot* slot, int nsm, cudaStream_t s, const double* uh_in,
                          double* uh_ghost_out) {
  return v_exact::recover_launch<double>(a, which, slot, nsm, s, uh_in, uh_ghost_out);
}
}  // namespace detail

int fused_preferred_variant(FusedKind kind) {
  const FusedVariant* v = nullptr;
  const int n = fused_variants(kind, &v);
  for (int i = 0; i < n; i++)
    if (v[i].preferred) return i;
  return 0;
}

int fused_variants(FusedKind kind, const FusedVariant** out) {
  switch (kind) {
    case FUSED_FP64_EXACT: return detail::variants_exact(out);
    case FUSED_FP64: return detail::variants_fp64(out);
    default: return detail::variants_mixed(out);
  }
}

cudaError_t launch_recover(FusedKind kind, const FusedArgs& a, int which, RedSlot* slot, int nsm, cudaStream_t s,
                           const double* uh_in, double* uh_ghost_out) {
  switch (kind) {
    case FUSED_FP64_EXACT: return detail::recover_exact(a, which, slot, nsm, s, uh_in, uh_ghost_out);
    case FUSED_FP64: return detail::recover_fp64(a, which, slot, nsm, s, uh_in, uh_ghost_out);
    default: return detail::recover_mixed(a, which, slot, nsm, s, uh_in, uh_ghost_out);
  }
}

}  // namespace mhdgb
