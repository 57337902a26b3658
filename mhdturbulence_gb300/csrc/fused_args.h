// fused_args.h -- launch arguments of the fused step kernel and the table entry describing one
// compiled tile shape of it (used by the host-side autotuner).
#pragma once

#include "common.cuh"

namespace mhdgb {

enum FusedKind { FUSED_FP64_EXACT = 0, FUSED_FP64 = 1, FUSED_MIXED = 2 };

constexpr int MAX_ZCHUNKS = 64;  // z chunks per tile column

struct FusedShape {
  int tx, ty;          // columns of a tile
  size_t smem;         // dynamic shared memory per CTA
  int threads;         // threads per CTA
  int elem;            // bytes per P element (8 or 4)
  int min_ctas;        // CTAs per SM the kernel's register budget was compiled for
};

struct FusedArgs {
  double* U;                           // conserved state, NCONS fields
  void* P[2];                          // primitive buffers (R), NPRIM fields; step parity selects
  Layout L;
  const double *xinv, *yinv, *zinv;    // 1/(x?a(i+1)-x?a(i)) per index of the reference index space
  const double *dxs, *dys, *dzs;       // x?a(i+1)-x?a(i)
  const float *xinvf, *yinvf, *zinvf;  // the same rounded to FP32 (mixed form)
  const float *dxsf, *dysf, *dzsf;
  double gam, cfl;
  int bc[6];
  int quirk;                           // y/z inverse spacing taken at index i (mhd.cpp:1435-1436)
  int riemann;                         // RIEMANN_HLLD / _HLLE / _HLLC
  int ntx, nty, nkc;                   // tiles in x, y; chunks in z
  // chunk c of every tile column covers planes [kst[c], kst[c+1]) (interior index); the work queue
  // takes all tiles of chunk 0 first, so chunks that shrink with c even out the CTAs' finish times
  int kst[MAX_ZCHUNKS + 1];
  Ctrl* ctrl;
  // End-to-end steps: the caller's host array of U (reference layout, itot x jtot x ktot, reached
  // over the host link), written by the step's cell updates besides U; null otherwise.
  double* Uh;
  // Bytes the first plane load of each work item is expected to deliver beyond the plane itself:
  // 0 in every step; mhdgb_selftest_fused_abort sets it so that the wait for that plane runs out
  // and the kernel's abort-and-drain path runs.
  unsigned tx_extra;
};

// One grid of a launch: its arguments, the TMA maps of its two primitive buffers and its range of
// the launch's work queue.  Kept in device memory (tensor maps need 64-byte alignment).
struct alignas(64) InstanceDesc {
  CUtensorMap tmap[2];
  FusedArgs a;
  int item_begin;   // first work item of this grid in the launch's queue
  int nitems;       // ntx * nty * nkc
};

// Launch-wide control of the fused kernel: the work-queue head and the CTA completion counter.
struct LaunchCtrl {
  unsigned work_next;
  unsigned blocks_done;
  unsigned ninst;
  unsigned total_items;
};

// One compiled instantiation of the fused kernel.
struct FusedVariant {
  FusedKind kind;
  FusedShape shape;
  cudaError_t (*prepare)();    // set the kernel's shared-memory attribute on the current device
  int (*ctas_per_sm)();        // occupancy
  cudaError_t (*launch)(const InstanceDesc* desc, LaunchCtrl* lc, int grid, cudaStream_t s);
  const char* name;            // kernel form and tile shape, e.g. "two-phase 16x8/256"
  int preferred;               // 1: the entry a grid starts on before any autotuning
};

// Marks the table entry a grid starts on: the fastest measured on GB300 at the benchmark sizes.
inline FusedVariant preferred_variant(FusedVariant v) {
  v.preferred = 1;
  return v;
}

}  // namespace mhdgb
