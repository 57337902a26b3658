// fused_fs.cuh -- the mixed form's fused step with the limited slopes formed inside the face phase.
//
// Same work items, TMA plane loads, cell phase and end-of-step protocol as k_fused_step (fused.cuh),
// with two differences:
//   * no slope phase: each face reads the 4-cell stencil across it and forms the two van Leer
//     slopes it needs itself, with the slope phase's expressions, so its states are the same;
//   * the face fluxes go to one of two buffers by plane parity, so the owner warps' cell phase of
//     plane k runs while the other warps already form the faces of plane k+1: one barrier per plane.
// The faces of plane k read planes k-1 .. k+2; the ring holds six planes, so each load is issued a
// whole plane before its first use.  In FP32 the second evaluation of each slope costs less than
// the barrier and the slope round trip through shared memory; the FP64 form keeps the slope phase,
// where every slope costs FP64 divisions.
#pragma once

#include "fused.cuh"

namespace mhdgb {

template <int TX, int TY, int NT>
struct FusedSmemFS {
  using R = float;
  static constexpr int NBUF = 6;
  static constexpr int PX = TX + 4, PY = TY + 4;
  static constexpr int PLANE = PX * NPRIM * PY;
  static constexpr int NFX = NCONS * TY * (TX + 1);  // x faces i in [0, TX]
  static constexpr int NFY = NCONS * (TY + 1) * TX;  // y faces j in [0, TY]
  static constexpr int NFZ = NCONS * TY * TX;        // z faces k+1/2
  static constexpr int NXY = NFX + NFY;              // one buffer of x and y faces
  static constexpr size_t a16(size_t x) { return (x + 15) / 16 * 16; }
  static constexpr size_t ring_off = 0;
  static constexpr size_t f_off = ((size_t)NBUF * PLANE * sizeof(R) + 127) / 128 * 128;
  // z faces in three buffers by plane: the cells of plane k read faces k-1/2 and k+1/2 while the
  // faces k+3/2 of the next plane are formed
  static constexpr size_t z_off = f_off + a16(2 * (size_t)NXY * sizeof(R));
  static constexpr size_t red_off = z_off + a16(3 * (size_t)NFZ * sizeof(R));
  static constexpr size_t bar_off = red_off + 64 * sizeof(double);
  static constexpr size_t misc_off = bar_off + NBUF * sizeof(uint64_t);  // item, abort, 2 face counters
  static constexpr size_t used = misc_off + 16;
  static constexpr size_t total = used + 128;  // room to align the base to 128 bytes
  static constexpr unsigned plane_tx_bytes = (unsigned)(PLANE * sizeof(R));
  static_assert(NT % 32 == 0 && NT >= TX * TY, "one owner thread per column, whole warps");
  static_assert((TX * sizeof(R)) % 16 == 0, "TMA x offsets must be 16-byte multiples");
  static_assert(((TX + 4) * sizeof(R)) % 16 == 0, "TMA box rows must be 16-byte multiples");
  static_assert((PLANE * sizeof(R)) % 128 == 0, "each ring slot is a TMA destination: 128-byte aligned");
  static_assert(total <= 227 * 1024, "shared memory budget");
};

namespace MHDGB_VNS {

template <int TX, int TY, int NT, int MINB, bool GEN>
__global__ void __launch_bounds__(NT, MINB)
k_fused_step_fs(const InstanceDesc* __restrict__ desc, LaunchCtrl* __restrict__ lc) {
  using R = float;
  using S = FusedSmemFS<TX, TY, NT>;
  constexpr int NBUF = S::NBUF, PX = S::PX;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char* smem = smem_raw + ((128u - (smem_u32(smem_raw) & 127u)) & 127u);  // TMA destinations
  R* ring = reinterpret_cast<R*>(smem + S::ring_off);
  R* fbuf = reinterpret_cast<R*>(smem + S::f_off);
  R* zbuf = reinterpret_cast<R*>(smem + S::z_off);
  double* red = reinterpret_cast<double*>(smem + S::red_off);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + S::bar_off);
  int& s_item = *reinterpret_cast<int*>(smem + S::misc_off);
  int& s_abort = *reinterpret_cast<int*>(smem + S::misc_off + 4);
  int* s_fitem = reinterpret_cast<int*>(smem + S::misc_off + 8);  // next face warp item, by plane parity

  const int tid = threadIdx.x;
  const int ninst = (int)lc->ninst, total = (int)lc->total_items;
  fused_reset_next_slots(desc, ninst, NT);
  if (tid == 0) {
    for (int s = 0; s < NBUF; s++) mbar_init(&bars[s], 1);
    fence_mbar_init();
    s_abort = 0;
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
    auto PV0 = [&](const R* pl, int i, int j) -> const R& { return pl[((j + 2) * NPRIM) * PX + (i + 2)]; };
    auto FXS = [&](int b, int m, int i, int j) -> R& { return fbuf[b * S::NXY + (m * TY + j) * (TX + 1) + i]; };
    auto FYS = [&](int b, int m, int i, int j) -> R& {
      return fbuf[b * S::NXY + S::NFX + (m * (TY + 1) + j) * TX + i];
    };
    // z face p+1/2 (p = kb-1 .. ke-1) lives in z buffer (p - kb + 1) % 3
    auto zslot = [&](int p) { return (p - kb + 1) % 3; };
    auto FZS = [&](int z, int m, int i, int j) -> R& { return zbuf[z * S::NFZ + (m * TY + j) * TX + i]; };

    // prologue: planes kb-2 .. kb+3 (those up to ke+1; ke >= kb+1, so kb+2 always exists)
    if (tid == 0) {
      s_fitem[0] = 0;
      s_fitem[1] = 0;
      fence_proxy_async();
      for (int p = kb - 2; p <= kb + 3 && p <= ke + 1; p++) issue(p);
    }
    for (int p = kb - 2; p <= kb + 3 && p <= ke + 1; p++) fill(slot_of(p));
    for (int p = kb - 2; p <= kb + 2; p++) wait_plane(p);
    __syncthreads();
    if (s_abort) break;

    const int nxf = cy * (cx + 1), nyf = (cy + 1) * cx, nzf = cy * cx;
    const FastDiv dv0(cx), dv1(cx + 1);

    for (int k = kb; k < ke; k++) {
      if (own) {  // the cell's U is read after the faces of this plane: pull it into L2 now
        const double* u0 = a.U + L.at(NCONS, 0, k + NGH, jj + NGH, ii + NGH);
#pragma unroll
        for (int m = 0; m < NCONS; m++) prefetch_l2(u0 + m * fsU);
      }
      if (k > kb) wait_plane(k + 2);
      const int fb = k & 1;
      // ---- faces of plane k (on the first plane also the faces kb-1/2) ----
      // One unpadded list over x, y and z faces, each read in its rotated frame (see k_fused_step).
      // Warp items come from counter fb; thread 0 clears the other one, which plane k-1 used and
      // plane k+1 will use, and the barrier below publishes it.
      if (tid == 0) s_fitem[fb ^ 1] = 0;
      const int nfb = nxf + nyf + (k == kb ? 2 * nzf : nzf);
      const int nwb = (nfb + 31) >> 5;
      for (;;) {
        int w = 0;
        if ((tid & 31) == 0) w = atomicAdd(&s_fitem[fb], 1);
        w = __shfl_sync(0xffffffffu, w, 0);
        if (w >= nwb) break;
        const int q = (w << 5) | (tid & 31);
        if (q < nfb) {
          int rot, fstr;              // rotation (0, 1, 2 = x, y, z); flux slot stride
          const R *c0, *c1, *c2, *c3;  // variable 0 of the stencil cells -2, -1 (left), 0 (right), +1
          R* fo;                      // flux slot 0 of the face
          if (q < nxf) {
            const int j = dv1.div(q), i = q - j * (cx + 1);
            rot = 0;
            c0 = &PV0(plane(k), i - 2, j);
            c1 = c0 + 1;
            c2 = c0 + 2;
            c3 = c0 + 3;
            fo = &FXS(fb, 0, i, j);
            fstr = TY * (TX + 1);
          } else if (q < nxf + nyf) {
            const int r = q - nxf, j = dv0.div(r), i = r - j * cx;
            rot = 1;
            c0 = &PV0(plane(k), i, j - 2);
            c1 = c0 + NPRIM * PX;
            c2 = c1 + NPRIM * PX;
            c3 = c2 + NPRIM * PX;
            fo = &FYS(fb, 0, i, j);
            fstr = (TY + 1) * TX;
          } else {
            int r = q - nxf - nyf;
            const bool lower = r >= nzf;  // face kb-1/2 (first plane only)
            if (lower) r -= nzf;
            const int j = dv0.div(r), i = r - j * cx;
            rot = 2;
            const int kl = lower ? k - 1 : k;  // the face lies between planes kl and kl+1
            c0 = &PV0(plane(kl - 1), i, j);
            c1 = &PV0(plane(kl), i, j);
            c2 = &PV0(plane(kl + 1), i, j);
            c3 = &PV0(plane(kl + 2), i, j);
            fo = &FZS(zslot(kl), 0, i, j);
            fstr = TY * TX;
          }
          const int u1 = unrot_comp(1, rot), u2 = unrot_comp(2, rot);
          // unrotated variable read into rotated slot n (n is a constant after unrolling)
          auto var_of = [&](int n) {
            if (n == nve1 || n == nbm1) return n + rot;
            if (n == nve2 || n == nbm2) return n - 1 + u1;
            if (n == nve3 || n == nbm3) return n - 2 + u2;
            return n;
          };
          R pl[NPRIM], pr[NPRIM], f[NCONS];
#pragma unroll
          for (int n = 0; n < NPRIM; n++) {
            const int v = var_of(n) * PX;
            const float2 st = van_leer_states_pair(c0[v], c1[v], c2[v], c3[v]);  // both cells' slopes
            pl[n] = st.x;
            pr[n] = st.y;
          }
          face_flux<R, 0>(pl, pr, glm, f, riemann, rot);
          auto slot_of_flux = [&](int m) {
            if (m == mrv1 || m == mbm1) return m + rot;
            if (m == mrv2 || m == mbm2) return m - 1 + u1;
            if (m == mrv3 || m == mbm3) return m - 2 + u2;
            return m;
          };
#pragma unroll
          for (int m = 0; m < NCONS; m++) fo[slot_of_flux(m) * fstr] = f[m];
        }
      }
      __syncthreads();  // faces of plane k formed; plane k-1 (and on the first plane kb-2) read for the last time
      if (s_abort) break;
      // the freed slots take the planes the faces of plane k+3 (and on the first plane k+2) first need
      if (k == kb && kb + 4 <= ke + 1) {  // plane kb-2's slot
        if (tid == 0) {
          fence_proxy_async();
          issue(kb + 4);
        }
        fill(slot_of(kb + 4));
      }
      if (k + 5 <= ke + 1) {  // plane k-1's slot
        if (tid == 0) {
          fence_proxy_async();
          issue(k + 5);
        }
        fill(slot_of(k + 5));
      }
      // ---- cells of plane k: update, recovery, ghost images, candidates (as k_fused_step) ----
      if (own) {
        const int zl = zslot(k - 1), zh = zslot(k);
        DivAcc<R> acc;
        const R xi = inv_of<R>(a, 0, ii + NGH);
        const R yi = inv_of<R>(a, 1, (a.quirk ? ii : jj) + NGH);
        const R zi = inv_of<R>(a, 2, (a.quirk ? ii : k) + NGH);
#pragma unroll
        for (int m = 0; m < NCONS; m++) {
          acc.first(m, FXS(fb, m, oi + 1, oj) - FXS(fb, m, oi, oj), xi);
          acc.add(m, FYS(fb, m, oi, oj + 1) - FYS(fb, m, oi, oj), yi);
          acc.add(m, FZS(zh, m, oi, oj) - FZS(zl, m, oi, oj), zi);
        }
        const size_t cu = L.at(NCONS, 0, k + NGH, jj + NGH, ii + NGH);
        double u[NCONS];
        update_cell(acc, a.U + cu, fsU, dt, chd, dtf, chf, a, ii + NGH, jj + NGH, k + NGH, u);
#pragma unroll
        for (int m = 0; m < NCONS; m++) a.U[cu + m * fsU] = u[m];
        if (a.Uh) {  // the caller's host copy of U (end-to-end steps), field stride itot
          double* uh = a.Uh + ((size_t)(ii + NGH) + (size_t)L.itot * NCONS * ((size_t)(jj + NGH) +
                                                                            (size_t)L.jtot * (size_t)(k + NGH)));
#pragma unroll
          for (int m = 0; m < NCONS; m++) uh[(size_t)m * L.itot] = u[m];
        }
        R dtc, chc;
        recover_cell<R>(u, a.gam, Pout, L, a.bc, ii, jj, k, spacing_of<R>(a, 0, ii + NGH),
                        spacing_of<R>(a, 1, jj + NGH), spacing_of<R>(a, 2, k + NGH), dtc, chc, bad);
        cmin = smin(cmin, dtc);
        cmax = smax(cmax, chc);
      }
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

// Host side of one instantiation of k_fused_step_fs (the FusedLauncher interface).
template <int TX, int TY, int NT, int MINB = 1, bool GEN = false>
struct FusedLauncherFS {
  using S = FusedSmemFS<TX, TY, NT>;
  static FusedShape shape() { return FusedShape{TX, TY, S::total, NT, (int)sizeof(float), MINB}; }
  static cudaError_t prepare() {
    return cudaFuncSetAttribute(k_fused_step_fs<TX, TY, NT, MINB, GEN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)S::total);
  }
  static int ctas_per_sm() {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_fused_step_fs<TX, TY, NT, MINB, GEN>, NT, S::total) !=
        cudaSuccess)
      return 0;
    return n;
  }
  static cudaError_t launch(const InstanceDesc* desc, LaunchCtrl* lc, int grid, cudaStream_t s) {
    k_fused_step_fs<TX, TY, NT, MINB, GEN><<<grid, NT, S::total, s>>>(desc, lc);
    return cudaGetLastError();
  }
  static const char* name() {
    static char buf[64];
    if (!buf[0])
      std::snprintf(buf, sizeof(buf), "fused-slope %dx%d/%d%s%s", TX, TY, NT, MINB > 1 ? " x2" : "",
                    GEN ? " run-time solver" : "");
    return buf;
  }
  static FusedVariant variant(FusedKind kind) {
    return FusedVariant{kind, shape(), &prepare, &ctas_per_sm, &launch, name(), 0};
  }
};

}  // namespace MHDGB_VNS
}  // namespace mhdgb
