// fused_args.h -- launch arguments and shared-memory plan of the fused step kernel.
#pragma once

#include "common.cuh"

namespace mhdgb {

enum FusedKind { FUSED_FP64_EXACT = 0, FUSED_FP64 = 1, FUSED_MIXED = 2 };

struct FusedShape {
  int tx, ty;          // columns of a tile
  size_t smem;         // dynamic shared memory per CTA
  int threads;         // threads per CTA
  int elem;            // bytes per P element (8 or 4)
};

struct FusedArgs {
  double* U;                      // conserved state, NCONS fields
  void* P[2];                     // primitive buffers (type R), NPRIM fields, step parity selects
  Layout L;
  const double *xinv, *yinv, *zinv;  // 1/(x?a(i+1)-x?a(i)) per index of the reference index space
  const double *dxs, *dys, *dzs;     // x?a(i+1)-x?a(i)
  const float *xinvf, *yinvf, *zinvf;  // the inverse spacings rounded to FP32 (mixed form)
  double gam, cfl;
  int bc[6];
  int quirk;                      // y/z inverse spacing taken at index i (mhd.cpp:1435-1436)
  int ntx, nty, nkc, kc;          // tiles in x, y; chunks in z; planes per chunk
  Ctrl* ctrl;
};

template <class R, int TX, int TY>
struct FusedSmem {
  static constexpr int NBUF = 4;
  static constexpr int PX = TX + 4, PY = TY + 4;
  static constexpr int PLANE = PX * NPRIM * PY;               // elements of one ring plane
  static constexpr int SX = TX + 2, SY = TY + 2;              // slope buffer extents
  static constexpr int FX = TX + 1, FY = TY + 1;              // face-flux buffer extents
  static constexpr size_t ring_bytes = (size_t)NBUF * PLANE * sizeof(R);
  static constexpr size_t slope_bytes = (size_t)NPRIM * SY * SX * sizeof(R);
  static constexpr size_t flux_bytes = (size_t)NCONS * FY * FX * sizeof(R);
  static constexpr size_t ring_off = 0;
  static constexpr size_t slope_off = (ring_bytes + 127) / 128 * 128;
  static constexpr size_t flux_off = slope_off + (slope_bytes + 15) / 16 * 16;
  static constexpr size_t red_off = flux_off + (flux_bytes + 15) / 16 * 16;
  static constexpr size_t bar_off = red_off + 64 * sizeof(double);
  static constexpr size_t misc_off = bar_off + NBUF * sizeof(uint64_t);  // work item, abort flag
  static constexpr size_t used = misc_off + 16;
  static constexpr size_t total = used + 128;  // room to align the base to 128 bytes
  static constexpr unsigned plane_tx_bytes = (unsigned)(PLANE * sizeof(R));
};

}  // namespace mhdgb
