// ghost_noalloc.cu -- mhdgb_fill_ghosts_noalloc: the ghost fill of mhdgb_set_boundary on a
// caller-owned device array, with no device allocation on the call path.
//
// Who needs it.  mhdgb_set_boundary works on a handle, and creating a handle allocates the solver's
// whole state (U, both P buffers, the flux arrays, the pack buffers).  Some callers own their
// primitive array already and cannot let a library allocate device memory when they call it: a code
// whose device memory sits under a fixed budget or in a pool it manages itself (an OpenACC program
// that placed its arrays with a data region, a framework with its own caching allocator), and a code
// that keeps asynchronous work running on other streams, which cudaMalloc / cudaFree would stall
// because they synchronise the whole device.  This entry point takes the array, its extents, the
// six boundary types and a stream, and allocates nothing: its only scratch is a fixed-size array in
// the module's static device memory.
//
// Algorithm.  The reference fills ghosts by packing the boundary layers of all three directions
// from P, then writing the x, y and z ghost layers in that order, each over the full transverse
// extent (boundary.cpp:771-891 with the single-rank SendRecvBoundary).  Later directions overwrite
// the edge and corner ghosts of earlier ones, and a pack taken before any write makes some edge
// ghosts copy the ghost values P held before the call.  The same result comes from two kernels:
//   k_edge_snapshot  saves the only packed values that the x and y writes would change: the old
//                    x-ghost columns of the y edge rows, and the old x-ghost columns and y-ghost
//                    rows of the z edge layers (192 * (nx + ny + nz + 7) doubles in all);
//   k_fill_owned     writes every ghost cell once, with the value of the direction that writes it
//                    last in the reference (z where k is a ghost index, else y where j is, else x),
//                    read from the snapshot where the reference's pack held an overwritten ghost and
//                    from P's interior cells otherwise.  It reads no cell it writes.
// The result equals mhdgb_set_boundary's bit for bit (values are only copied or negated).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "common.cuh"
#include "mhd_defs.cuh"
#include "mhdgb.h"

namespace mhdgb {
namespace {

constexpr size_t kScratchDoubles = MHDGB_NOALLOC_SCRATCH_BYTES / sizeof(double);

// The fixed scratch.  No part of it needs to start at zero: every call writes the snapshot it reads.
__device__ __align__(256) double g_edge_scratch[kScratchDoubles];

// Snapshot arrays inside the scratch (per field n, "slots" as below):
//   ys [n][kk][r][c]   kk < nz+1 non-ghost k, r < 4 y edge rows, c < 4 x-ghost columns
//   za [n][r][j][c]    r < 4 z edge layers, j < jtot, c < 4 x-ghost columns
//   zb [n][r][q][u]    r < 4 z edge layers, q < 4 y-ghost rows, u < nx+1 non-ghost i
struct EdgeSnap {
  double *ys, *za, *zb;
};

size_t snapshot_doubles(int nx, int ny, int nz) {
  return (size_t)NPRIM * 16 * ((size_t)nz + 1 + (size_t)ny + 5 + (size_t)nx + 1);
}

// Index sets of one axis with n interior cells and end index e = n + 1 (ngh = 2, extent n + 5):
//   ghost slots g = 0..3   -> 0, 1, e+1, e+2
//   edge slots  r = 0..3   -> 2, 3, e-1, e   (the layers the reference packs)
//   non-ghost   u = 0..n   -> 2 .. e, then e+3 (the extra index of itot = n + 2*ngh + 1)
__device__ __forceinline__ int ghost_at(int g, int e) { return g < 2 ? g : e + g - 1; }
__device__ __forceinline__ int edge_at(int r, int e) { return r < 2 ? 2 + r : e + r - 3; }
__device__ __forceinline__ int nonghost_at(int u, int e) { return u < e - 1 ? 2 + u : e + 3; }
__device__ __forceinline__ bool is_ghost(int c, int e) { return c < 2 || (c > e && c < e + 3); }
__device__ __forceinline__ int ghost_slot(int c, int e) { return c < 2 ? c : c - e + 1; }
__device__ __forceinline__ int nonghost_slot(int c, int e) { return c <= e ? c - 2 : e - 1; }

// Edge slot a ghost slot copies from, and whether the normal velocity changes sign:
// periodic takes the opposite side's layer at the same offset, reflection mirrors this side's
// layers, outflow repeats the first interior layer (boundary.cpp:152-169 and equivalents).
__device__ __forceinline__ int source_edge(int g, int bc_in, int bc_out, bool& flip) {
  const int bc = g < 2 ? bc_in : bc_out;
  flip = bc == MHDGB_BC_REFLECTION;
  if (g < 2) return bc == MHDGB_BC_PERIODIC ? 2 + g : (bc == MHDGB_BC_REFLECTION ? 1 - g : 0);
  const int m = g - 2;
  return bc == MHDGB_BC_PERIODIC ? m : (bc == MHDGB_BC_REFLECTION ? 3 - m : 3);
}

__global__ void k_edge_snapshot(const double* __restrict__ P, Layout L, EdgeSnap S) {
  const int ie = L.nx + 1, je = L.ny + 1, ke = L.nz + 1;
  const long long nys = 16LL * (L.nz + 1), nza = 16LL * L.jtot, nzb = 16LL * (L.nx + 1);
  const long long per_n = nys + nza + nzb;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= NPRIM * per_n) return;
  const int n = (int)(t / per_n);
  long long s = t - n * per_n;
  if (s < nys) {
    const int c = (int)(s % 4), r = (int)((s / 4) % 4), kk = (int)(s / 16);
    S.ys[n * nys + s] = P[L.at(NPRIM, n, nonghost_at(kk, ke), edge_at(r, je), ghost_at(c, ie))];
    return;
  }
  s -= nys;
  if (s < nza) {
    const int c = (int)(s % 4), j = (int)((s / 4) % L.jtot), r = (int)(s / (4LL * L.jtot));
    S.za[n * nza + s] = P[L.at(NPRIM, n, edge_at(r, ke), j, ghost_at(c, ie))];
    return;
  }
  s -= nza;
  const int u = (int)(s % (L.nx + 1)), q = (int)((s / (L.nx + 1)) % 4), r = (int)(s / (4LL * (L.nx + 1)));
  S.zb[n * nzb + s] = P[L.at(NPRIM, n, edge_at(r, ke), ghost_at(q, je), nonghost_at(u, ie))];
}

__global__ void k_fill_owned(double* __restrict__ P, Layout L, EdgeSnap S, int bx0, int bx1, int by0, int by1,
                             int bz0, int bz1) {
  const int it = L.itot, jt = L.jtot;
  const int ie = L.nx + 1, je = L.ny + 1, ke = L.nz + 1;
  const long long nzr = 4LL * jt * it, nyr = 4LL * (L.nz + 1) * it, nxr = 4LL * (L.nz + 1) * (L.ny + 1);
  const long long per_n = nzr + nyr + nxr;
  const long long nys = 16LL * (L.nz + 1), nza = 16LL * jt, nzb = 16LL * (L.nx + 1);
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= NPRIM * per_n) return;
  const int n = (int)(t / per_n);
  long long s = t - n * per_n;
  bool flip;
  double v;
  if (s < nzr) {  // z ghost layers over the full (j, i) plane
    const int i = (int)(s % it), j = (int)((s / it) % jt), g = (int)(s / ((long long)it * jt));
    const int r = source_edge(g, bz0, bz1, flip);
    if (is_ghost(i, ie)) v = S.za[n * nza + ((long long)r * jt + j) * 4 + ghost_slot(i, ie)];
    else if (is_ghost(j, je)) v = S.zb[n * nzb + ((long long)r * 4 + ghost_slot(j, je)) * (L.nx + 1) + nonghost_slot(i, ie)];
    else v = P[L.at(NPRIM, n, edge_at(r, ke), j, i)];
    P[L.at(NPRIM, n, ghost_at(g, ke), j, i)] = (flip && n == nve3) ? -v : v;
    return;
  }
  s -= nzr;
  if (s < nyr) {  // y ghost rows at non-ghost k, full i
    const int i = (int)(s % it), g = (int)((s / it) % 4), kk = (int)(s / (4LL * it));
    const int r = source_edge(g, by0, by1, flip);
    const int k = nonghost_at(kk, ke);
    if (is_ghost(i, ie)) v = S.ys[n * nys + ((long long)kk * 4 + r) * 4 + ghost_slot(i, ie)];
    else v = P[L.at(NPRIM, n, k, edge_at(r, je), i)];
    P[L.at(NPRIM, n, k, ghost_at(g, je), i)] = (flip && n == nve2) ? -v : v;
    return;
  }
  s -= nyr;
  {  // x ghost columns at non-ghost (k, j)
    const int g = (int)(s % 4), jj = (int)((s / 4) % (L.ny + 1)), kk = (int)(s / (4LL * (L.ny + 1)));
    const int r = source_edge(g, bx0, bx1, flip);
    const int k = nonghost_at(kk, ke), j = nonghost_at(jj, je);
    v = P[L.at(NPRIM, n, k, j, edge_at(r, ie))];
    P[L.at(NPRIM, n, k, j, ghost_at(g, ie))] = (flip && n == nve1) ? -v : v;
  }
}

// Identity of the calling thread's current context, 0 if it cannot be read.  cudaDeviceReset (or
// any other end of the primary context) destroys the context the scratch address was resolved in;
// the context that replaces it loads the module again and may place g_edge_scratch elsewhere, and
// it has a new identity.
unsigned long long current_context_id() {
  static PFN_cuCtxGetCurrent_v4000 get_current = nullptr;
  static PFN_cuCtxGetId_v12000 get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(p);
    p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<PFN_cuCtxGetId_v12000>(p);
  });
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS)
    return 0;
  return id;
}

// Address of g_edge_scratch on each device, resolved on the first call in each context of it.
constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
struct ScratchAddr {
  unsigned long long ctx_id;
  double* addr;
};
ScratchAddr g_scratch_addr[kMaxDevices] = {};

cudaError_t scratch_address(int dev, double** out) {
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  const unsigned long long ctx = current_context_id();
  if (dev < kMaxDevices && ctx != 0 && g_scratch_addr[dev].addr && g_scratch_addr[dev].ctx_id == ctx) {
    *out = g_scratch_addr[dev].addr;
    return cudaSuccess;
  }
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_edge_scratch);
  if (e != cudaSuccess) return e;
  if (dev < kMaxDevices) g_scratch_addr[dev] = ScratchAddr{current_context_id(), static_cast<double*>(p)};
  *out = static_cast<double*>(p);
  return cudaSuccess;
}

}  // namespace
}  // namespace mhdgb

extern "C" int mhdgb_fill_ghosts_noalloc(double* P, int nx, int ny, int nz, int pitch, const int* bc,
                                         void* stream) {
  using namespace mhdgb;
  if (!P || !bc || nx < 2 || ny < 2 || nz < 2) return MHDGB_ERR_ARG;
  for (int q = 0; q < 6; q++)
    if (bc[q] < MHDGB_BC_PERIODIC || bc[q] > MHDGB_BC_OUTFLOW) return MHDGB_ERR_ARG;
  const int itot = nx + 5;
  if (pitch == 0) pitch = itot;
  if (pitch < itot || reinterpret_cast<uintptr_t>(P) % alignof(double) != 0) return MHDGB_ERR_ARG;
  // The size check comes before anything touches the device.
  if ((long long)nx + ny + nz > (long long)MHDGB_NOALLOC_MAX_EXTENT_SUM ||
      snapshot_doubles(nx, ny, nz) > kScratchDoubles)
    return MHDGB_ERR_SCRATCH;

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return MHDGB_ERR_CUDA;
  // makes the device's primary context current on this thread (no allocation), so its identity can
  // be read
  if (cudaSetDevice(dev) != cudaSuccess) return MHDGB_ERR_CUDA;
  cudaPointerAttributes attr{};
  if (cudaPointerGetAttributes(&attr, P) != cudaSuccess) {
    cudaGetLastError();
    return MHDGB_ERR_ARG;
  }
  if ((attr.type != cudaMemoryTypeDevice && attr.type != cudaMemoryTypeManaged) || attr.device != dev)
    return MHDGB_ERR_ARG;
  double* scratch = nullptr;
  if (scratch_address(dev, &scratch) != cudaSuccess) return MHDGB_ERR_CUDA;

  Layout L;
  L.nx = nx; L.ny = ny; L.nz = nz;
  L.itot = itot; L.jtot = ny + 5; L.ktot = nz + 5;
  L.ip = pitch;
  EdgeSnap S;
  S.ys = scratch;
  S.za = S.ys + (size_t)NPRIM * 16 * (nz + 1);
  S.zb = S.za + (size_t)NPRIM * 16 * L.jtot;
  const cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int bs = 256;
  const long long nsnap = (long long)snapshot_doubles(nx, ny, nz);
  const long long nfill = (long long)NPRIM * (4LL * L.jtot * L.itot + 4LL * (nz + 1) * L.itot + 4LL * (nz + 1) * (ny + 1));
  // cudaLaunchKernel returns the status of its own launch, so an error left pending by an earlier,
  // unrelated call on this thread is neither reported as ours nor cleared
  const double* Pc = P;
  void* snap_args[] = {(void*)&Pc, (void*)&L, (void*)&S};
  if (cudaLaunchKernel((const void*)k_edge_snapshot, dim3((unsigned)((nsnap + bs - 1) / bs)), dim3(bs), snap_args, 0,
                       s) != cudaSuccess)
    return MHDGB_ERR_CUDA;
  int b[6] = {bc[0], bc[1], bc[2], bc[3], bc[4], bc[5]};
  void* fill_args[] = {(void*)&P, (void*)&L, (void*)&S, &b[0], &b[1], &b[2], &b[3], &b[4], &b[5]};
  if (cudaLaunchKernel((const void*)k_fill_owned, dim3((unsigned)((nfill + bs - 1) / bs)), dim3(bs), fill_args, 0,
                       s) != cudaSuccess)
    return MHDGB_ERR_CUDA;
  return MHDGB_OK;
}
