// solver.cu -- host side of the C ABI declared in include/mhdgb.h.
//
// A handle owns, on its device: the conserved state U (FP64), two primitive buffers per precision
// (the fused step reads one and writes the other), the three face-flux arrays and the pack buffers
// of the stage path, the per-axis spacing tables, and the control block (Ctrl).  All arrays use
// the reference FieldArray layout with a padded i pitch.  Host arrays (dense rows of itot) move
// through a device staging buffer and a row-repacking kernel; page-locked host arrays given to
// mhdgb_step_host are instead read and written by the kernels themselves over the host link.
#include <cudaTypedefs.h>

#include <algorithm>
#include <array>
#include <cstdint>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <numeric>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "../../include/mhdgb.h"
#include "kernels.h"
#include "output.h"

using namespace mhdgb;

// Diagnostic and initial-state kernels (no FP contraction concerns: FP64 sums in fixed order).
namespace {

template <class R>
__global__ void k_diag_planes(const R* __restrict__ P, Layout L, const double* __restrict__ dxs,
                              const double* __restrict__ dys, const double* __restrict__ dzs, double* planes) {
  // one block per interior k plane; fixed-order tree sum of (dv, X(1-X)dv, vy^2 dv)
  __shared__ double sh[3][256];
  const int k = blockIdx.x;
  double s0 = 0.0, s1 = 0.0, s2 = 0.0;
  for (int t = threadIdx.x; t < L.nx * L.ny; t += blockDim.x) {
    const int i = t % L.nx, j = t / L.nx;
    const double dv = dxs[i + NGH] * dys[j + NGH] * dzs[k + NGH];
    const double X = (double)P[L.at(NPRIM, nst, k + NGH, j + NGH, i + NGH)];
    const double vy = (double)P[L.at(NPRIM, nve2, k + NGH, j + NGH, i + NGH)];
    s0 += dv;
    s1 += X * (1.0 - X) * dv;
    s2 += vy * vy * dv;
  }
  sh[0][threadIdx.x] = s0; sh[1][threadIdx.x] = s1; sh[2][threadIdx.x] = s2;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o)
      for (int q = 0; q < 3; q++) sh[q][threadIdx.x] += sh[q][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int q = 0; q < 3; q++) planes[3 * k + q] = sh[q][0];
}

__global__ void k_diag_final(const double* planes, int nz, double* out) {
  double v = 0.0, m = 0.0, a = 0.0;
  for (int k = 0; k < nz; k++) { v += planes[3 * k]; m += planes[3 * k + 1]; a += planes[3 * k + 2]; }
  out[0] = v;
  out[1] = m / v;
  out[2] = sqrt(a / v);
}

__global__ void k_ctrl_reset(Ctrl* c, int keep_clock) {
  for (int s = 0; s < 3; s++) { c->slot[s].dtmin_bits = DT_RESET; c->slot[s].chmax_bits = CH_RESET; }
  if (!keep_clock) { c->step = 0; c->time = 0.0; c->last_dt = 0.0; c->last_ch = 0.0; }
  c->done = 0;
  c->status = 0;
  c->blocks_done = 0;
  c->work_next = 0;
}

// Clock of a restart: the step count, time and latest dt/c_h of a checkpoint, with fresh reduction
// slots (the first step after the restart reduces them again, as prepare does).
__global__ void k_ctrl_restore(Ctrl* c, unsigned long long step, double time, double last_dt, double last_ch,
                               double tmax, unsigned long long max_step) {
  for (int s = 0; s < 3; s++) { c->slot[s].dtmin_bits = DT_RESET; c->slot[s].chmax_bits = CH_RESET; }
  c->step = step;
  c->time = time;
  c->last_dt = last_dt;
  c->last_ch = last_ch;
  c->tmax = tmax;
  c->max_step = max_step;
  c->done = (time > tmax || step >= max_step) ? 1u : 0u;
  c->status = 0;
  c->blocks_done = 0;
  c->work_next = 0;
}

// Point the step's host copy of U at v (null: none), in the launch descriptor on the device.
__global__ void k_set_host_u(InstanceDesc* d, double* v) { d->a.Uh = v; }

// Test hook of the abort self-test: extra bytes the first plane load of each work item expects.
__global__ void k_set_tx_extra(InstanceDesc* d, unsigned v) { d->a.tx_extra = v; }

// Failure-detection self-test: one thread waits on an mbarrier that no arrival or copy ever
// completes.  The bounded wait (the one the fused step uses for its plane loads) gives up, sets
// ST_TIMEOUT in *status, and the kernel returns normally.
__global__ void k_wait_selftest(unsigned* status) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
    mbar_wait(&bar, 0u, status);
  }
}

__global__ void k_ctrl_set_stop(Ctrl* c, double tmax, unsigned long long max_step) {
  c->tmax = tmax;
  c->max_step = max_step;
  c->done = (c->time > tmax || c->step >= max_step) ? 1u : 0u;
}

// One variable between a dense (k, j, i) host array and its rows in the (k, j, n, i) device layout.
__global__ void k_field(const double* __restrict__ src, double* __restrict__ dst, int itot, int ip, int nv, int n,
                        size_t rows, int to_device) {
  const size_t tot = rows * (size_t)itot;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < tot; t += (size_t)gridDim.x * blockDim.x) {
    const size_t r = t / itot, i = t % itot;  // r = j + jtot*k
    const size_t d = (r * nv + n) * ip + i;
    if (to_device) dst[d] = src[t];
    else dst[t] = src[d];
  }
}

// Row repack between the dense host layout (row length itot) and the padded device pitch ip.
__global__ void k_repack(const double* __restrict__ src, double* __restrict__ dst, int itot, int ip, size_t rows,
                         int to_pitched) {
  const size_t n = rows * (size_t)itot;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const size_t r = t / itot, i = t % itot;
    if (to_pitched) dst[r * ip + i] = src[t];
    else dst[t] = src[r * ip + i];
  }
}

// FP64 FMA issue-rate probe: 8 independent dependent-chains per thread, grid-strided.
__global__ void k_dfma_rate(double* out, int iters) {
  double a[8];
  for (int i = 0; i < 8; i++) a[i] = 1.0 + 1e-9 * threadIdx.x + 0.01 * i;
  for (int it = 0; it < iters; it++)
#pragma unroll
    for (int i = 0; i < 8; i++) a[i] = fma(a[i], 0.9999999, 1e-7);
  double s = 0.0;
  for (int i = 0; i < 8; i++) s += a[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

uint64_t splitmix64(uint64_t x) {
  uint64_t z = x + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

struct KhParams {
  unsigned long long seed;
  double vshear, width, bx, amp, sig, noise;
};

// Kelvin-Helmholtz initial state (the set-up of mhdturbulence_gb300/ic.py.kh_prim) on the device,
// for the interior cells of a block whose first cell is cell (i0, j0, k0) of a gnx x gny x ... grid
// (the noise of a cell is a counter hash of its whole-grid index, so it does not depend on the
// split); xa / ya are the block's cell faces.  Ghost cells are left as they are.
__global__ void k_init_kh(double* __restrict__ U, Layout L, const double* __restrict__ xa,
                          const double* __restrict__ ya, int gnx, int gny, int i0, int j0, int k0, uint64_t key,
                          double gam, double vshear, double width, double bx, double amp, double sig, double noise) {
  const long long n = (long long)L.nx * L.ny * L.nz;
  const double pi = 3.14159265358979323846;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t % L.nx), j = (int)((t / L.nx) % L.ny), k = (int)(t / ((long long)L.nx * L.ny));
    const double x = 0.5 * (xa[i + NGH + 1] + xa[i + NGH]);
    const double y = 0.5 * (ya[j + NGH + 1] + ya[j + NGH]);
    const uint64_t idx = ((uint64_t)(k + k0) * gny + (uint64_t)(j + j0)) * gnx + (uint64_t)(i + i0);
    uint64_t z = (idx ^ key) + 0x9E3779B97F4A7C15ull;  // splitmix64
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    const double u = (double)(z >> 11) * (1.0 / 9007199254740992.0);
    const double th = tanh(y / width);
    const double rho = 1.0, p = 1.0;
    const double vx = vshear * th;
    const double ys = y / sig;
    const double vy = amp * sin(2.0 * pi * x) * exp(-(ys * ys)) + noise * (2.0 * u - 1.0);
    const double X = 0.5 * (1.0 + th);
    const double e = p / (rho * (gam - 1.0));
    const double ekin = 0.5 * rho * (vx * vx + vy * vy);
    const double emag = 0.5 * (bx * bx);
    const size_t c = L.at(NCONS, 0, k + NGH, j + NGH, i + NGH), fs = (size_t)L.ip;
    U[c + mden * fs] = rho;
    U[c + mrv1 * fs] = rho * vx;
    U[c + mrv2 * fs] = rho * vy;
    U[c + mrv3 * fs] = 0.0;
    U[c + meto * fs] = rho * e + ekin + emag;
    U[c + mbm1 * fs] = bx;
    U[c + mbm2 * fs] = 0.0;
    U[c + mbm3 * fs] = 0.0;
    U[c + mbps * fs] = 0.0;
    U[c + mst * fs] = rho * X;
  }
}

uint64_t kh_key(unsigned long long seed) {
  return splitmix64((uint64_t)seed * 0xD1B54A32D192ED03ull + 0ull * 0x8CB92BA72F3D8DD7ull);
}

}  // namespace

struct mhdgb_solver {
  mhdgb_config cfg{};
  FusedKind kind = FUSED_FP64;
  FusedShape shape{};
  Layout L{};
  cudaStream_t stream = nullptr;
  int nsm = 0;
  // device memory
  double* U = nullptr;
  double* P64[2] = {nullptr, nullptr};
  float* P32[2] = {nullptr, nullptr};
  double* F[3] = {nullptr, nullptr, nullptr};
  double* pack = nullptr;
  double *xinv = nullptr, *yinv = nullptr, *zinv = nullptr, *dxs = nullptr, *dys = nullptr, *dzs = nullptr;
  float *xinvf = nullptr, *yinvf = nullptr, *zinvf = nullptr, *dxsf = nullptr, *dysf = nullptr, *dzsf = nullptr;
  double* scal = nullptr;   // [0] dt, [1] chg of the stage path, [2..4] diagnostic, [8..] diag planes
  double* faces = nullptr;  // x1a (itot) then x2a (jtot): the cell faces the KH initial state needs
  RedSlot* sslot = nullptr; // stage-path reduction slot
  Ctrl* ctrl = nullptr;
  size_t bytes = 0;
  // host state
  std::vector<double> x1a, x2a, x3a;
  CUtensorMap tmap[2];
  const FusedVariant* vars = nullptr;  // compiled HLLD tile shapes of this precision; vars[nvars] is
  int nvars = 0, vidx = 0;             // the run-time solver kernel; vidx: the kernel in use
  int hlld_vidx = 0;                   // the HLLD variant to return to from HLLE/HLLC
  int grid = 0, ntx = 0, nty = 0, nkc = 0;
  std::vector<int> kst;      // z chunk boundaries (FusedArgs::kst)
  long long cur_step = 0;    // device step count as of the last sync (selects the current P)
  bool have_state = false;   // U uploaded
  bool prepared = false;     // fused buffers consistent with U
  bool p64_valid = false;    // P64[cur] holds the primitives of U (stage path view)
  bool p_user = false;       // P64[cur] was uploaded by the caller and not superseded since
  cudaGraphExec_t gexec = nullptr;
  int gsteps = 0;
  InstanceDesc* d_desc = nullptr;  // this grid as a one-instance launch of the fused kernel
  LaunchCtrl* d_lc = nullptr;
  double* stage = nullptr;         // dense host-layout staging buffer (allocated on first transfer)
  bool own_stream = true;          // false for the members of an ensemble (they share its stream)
  int riemann = 0;                 // MHDGB_RIEMANN_*
  unsigned desc_version = 0;       // bumped whenever the kernel arguments change (ensembles re-read)
  std::string err;
  // snapshot output (allocated on first use): device pack -> copy stream -> pinned host -> writer
  double* d_snap = nullptr;
  double* h_snap = nullptr;
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t ev_packed = nullptr, ev_copied = nullptr;
  std::thread writer;
  int writer_rc = MHDGB_OK;
  std::string writer_err;
};

namespace {

int fail(mhdgb_solver* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  return code;
}

int cuda_fail(mhdgb_solver* h, cudaError_t e, const char* what) {
  return fail(h, MHDGB_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(h, call)                                          \
  do {                                                       \
    cudaError_t e_ = (call);                                 \
    if (e_ != cudaSuccess) return cuda_fail((h), e_, #call); \
  } while (0)

// cudaMemset and cudaMemcpy from pageable host memory run on the legacy default stream and may
// still be in flight when they return; the handles' streams are non-blocking, so nothing orders
// that work before theirs.  Every such call is followed by this wait.
inline cudaError_t legacy_fence() { return cudaStreamSynchronize(cudaStreamLegacy); }

template <class T>
cudaError_t dalloc(mhdgb_solver* h, T** p, size_t n) {
  cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
  if (e == cudaSuccess) {
    h->bytes += n * sizeof(T);
    e = cudaMemset(*p, 0, n * sizeof(T));
  }
  if (e == cudaSuccess) e = legacy_fence();
  return e;
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
  }
  return fn;
}

// 4-D map over a primitive buffer: dims (i, n, j, k) = (itot, 12, jtot, ktot); box (tx+4, 12, ty+4, 1).
int make_tmap(mhdgb_solver* h, CUtensorMap* map, void* base, int elem) {
  auto fn = encode_fn();
  if (!fn) return fail(h, MHDGB_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
  const Layout& L = h->L;
  cuuint64_t dims[4] = {(cuuint64_t)L.itot, (cuuint64_t)NPRIM, (cuuint64_t)L.jtot, (cuuint64_t)L.ktot};
  cuuint64_t strides[3] = {(cuuint64_t)L.ip * elem, (cuuint64_t)L.ip * elem * NPRIM,
                           (cuuint64_t)L.ip * elem * NPRIM * L.jtot};
  cuuint32_t box[4] = {(cuuint32_t)(h->shape.tx + 4), (cuuint32_t)NPRIM, (cuuint32_t)(h->shape.ty + 4), 1u};
  cuuint32_t estr[4] = {1, 1, 1, 1};
  CUresult r = fn(map, elem == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, base, dims,
                  strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(h, MHDGB_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
  return MHDGB_OK;
}

void set_spacing_tables(mhdgb_solver* h, std::vector<double>& hx, std::vector<double>& hinv,
                        const std::vector<double>& xa, int n) {
  hx.assign(n, 0.0);
  hinv.assign(n, 0.0);
  for (int i = 0; i + 1 < (int)xa.size(); i++) {
    hx[i] = xa[i + 1] - xa[i];
    hinv[i] = 1.0 / (xa[i + 1] - xa[i]);
  }
}

int upload_grid(mhdgb_solver* h) {
  const int n = std::max(h->L.itot, std::max(h->L.jtot, h->L.ktot));
  std::vector<double> dx, ix, dy, iy, dz, iz;
  set_spacing_tables(h, dx, ix, h->x1a, n);
  set_spacing_tables(h, dy, iy, h->x2a, n);
  set_spacing_tables(h, dz, iz, h->x3a, n);
  std::vector<float> fx(n), fy(n), fz(n), sx(n), sy(n), sz(n);
  for (int i = 0; i < n; i++) {
    fx[i] = (float)ix[i]; fy[i] = (float)iy[i]; fz[i] = (float)iz[i];
    sx[i] = (float)dx[i]; sy[i] = (float)dy[i]; sz[i] = (float)dz[i];
  }
  const size_t b = n * sizeof(double), bf = n * sizeof(float);
  CK(h, cudaMemcpy(h->dxs, dx.data(), b, cudaMemcpyHostToDevice));
  CK(h, cudaMemcpy(h->dys, dy.data(), b, cudaMemcpyHostToDevice));
  CK(h, cudaMemcpy(h->dzs, dz.data(), b, cudaMemcpyHostToDevice));
  CK(h, cudaMemcpy(h->xinv, ix.data(), b, cudaMemcpyHostToDevice));
  CK(h, cudaMemcpy(h->yinv, iy.data(), b, cudaMemcpyHostToDevice));
  CK(h, cudaMemcpy(h->zinv, iz.data(), b, cudaMemcpyHostToDevice));
  CK(h, cudaMemcpy(h->xinvf, fx.data(), bf, cudaMemcpyHostToDevice));
  CK(h, cudaMemcpy(h->yinvf, fy.data(), bf, cudaMemcpyHostToDevice));
  CK(h, cudaMemcpy(h->zinvf, fz.data(), bf, cudaMemcpyHostToDevice));
  CK(h, cudaMemcpy(h->dxsf, sx.data(), bf, cudaMemcpyHostToDevice));
  CK(h, cudaMemcpy(h->dysf, sy.data(), bf, cudaMemcpyHostToDevice));
  CK(h, cudaMemcpy(h->dzsf, sz.data(), bf, cudaMemcpyHostToDevice));
  CK(h, cudaMemcpy(h->faces, h->x1a.data(), h->L.itot * sizeof(double), cudaMemcpyHostToDevice));
  CK(h, cudaMemcpy(h->faces + h->L.itot, h->x2a.data(), h->L.jtot * sizeof(double), cudaMemcpyHostToDevice));
  CK(h, legacy_fence());
  return MHDGB_OK;
}

// GenerateGrid (main.cpp:35-64) for one rank.
std::vector<double> face_axis(int n, double lo, double hi) {
  const int ngh = NGH, is = ngh, ie = is + n - 1;
  std::vector<double> xa(n + 2 * ngh + 1);
  const double xminloc = lo + (hi - lo) / 1 * 0;
  const double xmaxloc = lo + (hi - lo) / 1 * (0 + 1);
  const double dx = (xmaxloc - xminloc) / double(n);
  for (int i = is - ngh; i <= ie + ngh + 1; i++) xa[i] = dx * (i - (ngh + 1)) + xminloc;
  return xa;
}

int set_device(mhdgb_solver* h) {
  CK(h, cudaSetDevice(h->cfg.device));
  return MHDGB_OK;
}

// 2-D pitched copy of a reference-layout host array (row = itot elements) to/from a device array.
int copy_h2d(mhdgb_solver* h, void* dst, const void* src, int nv, size_t elem) {
  const Layout& L = h->L;
  CK(h, cudaMemcpy2DAsync(dst, L.ip * elem, src, L.itot * elem, L.itot * elem, (size_t)nv * L.jtot * L.ktot,
                          cudaMemcpyHostToDevice, h->stream));
  return MHDGB_OK;
}

int copy_d2h(mhdgb_solver* h, void* dst, const void* src, int nv, size_t elem) {
  const Layout& L = h->L;
  CK(h, cudaMemcpy2DAsync(dst, L.itot * elem, src, L.ip * elem, L.itot * elem, (size_t)nv * L.jtot * L.ktot,
                          cudaMemcpyDeviceToHost, h->stream));
  return MHDGB_OK;
}

// State transfers: one dense copy through a staging buffer, then a repack kernel (much faster than
// a pitched 2-D copy with ~1 KB rows).
double* staging(mhdgb_solver* h) {
  if (!h->stage) {
    const size_t n = (size_t)NPRIM * h->L.itot * h->L.jtot * h->L.ktot;
    if (dalloc(h, &h->stage, n) != cudaSuccess) return nullptr;
  }
  return h->stage;
}

int upload_u(mhdgb_solver* h, const double* U) {
  const Layout& L = h->L;
  const size_t rows = (size_t)NCONS * L.jtot * L.ktot;
  double* st = staging(h);
  if (!st) return fail(h, MHDGB_ERR_NOMEM, "staging buffer");
  CK(h, cudaMemcpyAsync(st, U, rows * L.itot * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  k_repack<<<h->nsm * 8, 256, 0, h->stream>>>(st, h->U, L.itot, L.ip, rows, 1);
  CK(h, cudaGetLastError());
  return MHDGB_OK;
}

int download_u(mhdgb_solver* h, double* U) {
  const Layout& L = h->L;
  const size_t rows = (size_t)NCONS * L.jtot * L.ktot;
  double* st = staging(h);
  if (!st) return fail(h, MHDGB_ERR_NOMEM, "staging buffer");
  k_repack<<<h->nsm * 8, 256, 0, h->stream>>>(h->U, st, L.itot, L.ip, rows, 0);
  CK(h, cudaGetLastError());
  CK(h, cudaMemcpyAsync(U, st, rows * L.itot * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  return MHDGB_OK;
}

int read_ctrl(mhdgb_solver* h, Ctrl* c) {
  CK(h, cudaMemcpyAsync(c, h->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  return MHDGB_OK;
}

// Wait for enqueued work and refresh the host's view of the step parity.
int settle(mhdgb_solver* h) {
  Ctrl c;
  int rc = read_ctrl(h, &c);
  if (rc) return rc;
  if ((long long)c.step != h->cur_step) {
    h->cur_step = (long long)c.step;
    h->p64_valid = false;
  }
  return MHDGB_OK;
}

int status_to_code(mhdgb_solver* h, unsigned st) {
  if (st & ST_TIMEOUT) return fail(h, MHDGB_ERR_TIMEOUT, "a device-side wait gave up (TMA load did not complete)");
  if (st & ST_NONFINITE) return fail(h, MHDGB_ERR_NONFINITE, "non-finite dt or c_h candidate in the state");
  if (st & ST_NEGATIVE) return fail(h, MHDGB_ERR_NEGATIVE, "non-positive density or pressure in the state");
  return MHDGB_OK;
}

int cur_index(const mhdgb_solver* h) { return (int)(h->cur_step & 1); }

// Buffers of the stage path, allocated on first use.
int ensure_stage_bufs(mhdgb_solver* h) {
  const Layout& L = h->L;
  for (int q = 0; q < 3; q++)
    if (!h->F[q] && dalloc(h, &h->F[q], L.count(NCONS)) != cudaSuccess) return fail(h, MHDGB_ERR_NOMEM, "flux arrays");
  if (!h->pack && dalloc(h, &h->pack, pack_buffer_doubles(L)) != cudaSuccess)
    return fail(h, MHDGB_ERR_NOMEM, "pack buffers");
  for (int q = 0; q < 2; q++)
    if (!h->P64[q] && dalloc(h, &h->P64[q], L.count(NPRIM)) != cudaSuccess)
      return fail(h, MHDGB_ERR_NOMEM, "FP64 primitive arrays");
  return MHDGB_OK;
}

// Make P64[cur] the primitives of U (interior + ghosts), for the stage path and downloads.
int ensure_p64(mhdgb_solver* h) {
  int rc = ensure_stage_bufs(h);
  if (rc) return rc;
  if (h->p64_valid) return MHDGB_OK;
  if (!h->have_state) return fail(h, MHDGB_ERR_STATE, "no state uploaded");
  double* P = h->P64[cur_index(h)];
  if (h->prepared && h->kind != FUSED_MIXED) {
    // P64[cur] is the fused step's own recovery of U: recovering it again with the stage kernels'
    // rounding could change its last bits under the running fused steps; only the ghost layers
    // still need the reference's fill
    CK(h, launch_ghost_fill(P, h->L, h->cfg.bc, h->pack, h->stream));
    h->p64_valid = true;
    return MHDGB_OK;
  }
  CK(h, launch_update_prim(h->U, P, h->L, h->cfg.gam, h->stream));
  CK(h, launch_ghost_fill(P, h->L, h->cfg.bc, h->pack, h->stream));
  h->p64_valid = true;
  return MHDGB_OK;
}

int destroy_graph(mhdgb_solver* h) {
  if (h->gexec) cudaGraphExecDestroy(h->gexec);
  h->gexec = nullptr;
  h->gsteps = 0;
  return MHDGB_OK;
}

FusedArgs fused_args(mhdgb_solver* h) {
  FusedArgs a{};
  a.U = h->U;
  if (h->kind == FUSED_MIXED) { a.P[0] = h->P32[0]; a.P[1] = h->P32[1]; }
  else { a.P[0] = h->P64[0]; a.P[1] = h->P64[1]; }
  a.L = h->L;
  a.xinv = h->xinv; a.yinv = h->yinv; a.zinv = h->zinv;
  a.dxs = h->dxs; a.dys = h->dys; a.dzs = h->dzs;
  a.xinvf = h->xinvf; a.yinvf = h->yinvf; a.zinvf = h->zinvf;
  a.dxsf = h->dxsf; a.dysf = h->dysf; a.dzsf = h->dzsf;
  a.gam = h->cfg.gam;
  a.cfl = h->cfg.cfl;
  for (int q = 0; q < 6; q++) a.bc[q] = h->cfg.bc[q];
  a.quirk = h->cfg.spacing_quirk;
  a.riemann = h->riemann;
  a.ntx = h->ntx; a.nty = h->nty; a.nkc = h->nkc;
  for (int c = 0; c <= h->nkc && c < (int)h->kst.size(); c++) a.kst[c] = h->kst[c];
  a.ctrl = h->ctrl;
  return a;
}

InstanceDesc host_desc(mhdgb_solver* h, int item_begin) {
  InstanceDesc d;
  std::memset(&d, 0, sizeof(d));
  d.tmap[0] = h->tmap[0];
  d.tmap[1] = h->tmap[1];
  d.a = fused_args(h);
  d.item_begin = item_begin;
  d.nitems = h->ntx * h->nty * h->nkc;
  return d;
}

// The handle as a one-instance launch: descriptor and launch control in device memory.
int upload_desc(mhdgb_solver* h) {
  h->desc_version++;
  const InstanceDesc d = host_desc(h, 0);
  const LaunchCtrl lc{0u, 0u, 1u, (unsigned)d.nitems};
  CK(h, cudaMemcpyAsync(h->d_desc, &d, sizeof(d), cudaMemcpyHostToDevice, h->stream));
  CK(h, cudaMemcpyAsync(h->d_lc, &lc, sizeof(lc), cudaMemcpyHostToDevice, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  return MHDGB_OK;
}

int launch_one(mhdgb_solver* h) {
  CK(h, h->vars[h->vidx].launch(h->d_desc, h->d_lc, h->grid, h->stream));
  return MHDGB_OK;
}

// Relative cost of one plane of a cx x cy tile: its face and slope work against a full tile's, plus
// a fixed part (barriers, loads).  Only the ratios matter.
double tile_plane_cost(int cx, int cy, int tx, int ty) {
  auto warps = [](int n) { return (double)((n + 31) / 32); };
  const double f = (double)(cy * (cx + 1) + (cy + 1) * cx + cy * cx), ff = (double)(ty * (tx + 1) + (ty + 1) * tx + ty * tx);
  const double sl = warps(cy * (cx + 2)) + warps((cy + 2) * cx) + warps(cy * cx);
  const double sf = warps(ty * (tx + 2)) + warps((ty + 2) * tx) + warps(ty * tx);
  return 0.1 + 0.9 * (0.75 * f / ff + 0.25 * sl / sf);
}

// Finish time of the slowest of `grid` CTAs that take the work items in queue order (chunk-major,
// then tile rows, then tiles), each CTA the next item when it finishes its last.  A chunk's start
// costs about kOverheadPlanes planes more (prologue loads, the extra z faces of its first plane);
// 1.2 fits the measured times of KH ensembles with 8- to 64-plane items and of eleven chunkings of
// a 150^3 grid in both forms.
double simulate_queue(const std::vector<double>& tile_cost, const std::vector<int>& chunks, int grid) {
  constexpr double kOverheadPlanes = 1.2;
  std::vector<double> heap(grid, 0.0);  // min-heap of CTA finish times
  auto cmp = [](double a, double b) { return a > b; };
  for (int c : chunks)
    for (double tc : tile_cost) {
      std::pop_heap(heap.begin(), heap.end(), cmp);
      heap.back() += tc * (c + kOverheadPlanes);
      std::push_heap(heap.begin(), heap.end(), cmp);
    }
  return *std::max_element(heap.begin(), heap.end());
}

// z chunks of a grid for a persistent launch of `grid` CTAs: among uniform chunkings and chunkings
// whose sizes shrink (each chunk about remaining * tiles / (K * grid) planes, or a few chunks each
// a factor r shorter than the one before, so the queue ends on small items that fill the CTAs'
// last gaps), the one with the earliest simulated finish.
std::vector<int> choose_chunks(const Layout& L, int tx, int ty, int ntx, int nty, int grid) {
  std::vector<double> cost;
  for (int by = 0; by < nty; by++)
    for (int bx = 0; bx < ntx; bx++)
      cost.push_back(tile_plane_cost(std::min(tx, L.nx - bx * tx), std::min(ty, L.ny - by * ty), tx, ty));
  const int tiles = ntx * nty, nz = L.nz;
  std::vector<std::vector<int>> cand;
  for (int n = 1; n <= std::min(nz, 32); n++) {
    const int kc = (nz + n - 1) / n;
    std::vector<int> c;
    for (int k = 0; k < nz; k += kc) c.push_back(std::min(kc, nz - k));
    if ((int)c.size() <= MAX_ZCHUNKS) cand.push_back(c);
  }
  const double Ks[] = {1.25, 1.5, 2.0, 2.5, 3.0, 4.0, 6.0};
  for (double K : Ks)
    for (int minc : {2, 4, 8}) {
      std::vector<int> c;
      int rem = nz;
      while (rem > 0) {
        int s = std::max(minc, (int)std::ceil(rem * (double)tiles / (K * grid)));
        s = std::min(s, rem);
        if (rem - s < minc) s = rem;
        c.push_back(s);
        rem -= s;
      }
      if ((int)c.size() <= MAX_ZCHUNKS) cand.push_back(c);
    }
  for (int m = 2; m <= 7 && m <= nz; m++)
    for (double r : {1.5, 2.0, 2.5, 3.0, 4.0}) {
      std::vector<double> w(m);
      double tot = 0.0;
      for (int i = 0; i < m; i++) tot += (w[i] = std::pow(r, -i));
      std::vector<int> c(m);
      int sum = 0;
      for (int i = 0; i < m; i++) sum += (c[i] = std::max(1, (int)std::lround(nz * w[i] / tot)));
      c[0] += nz - sum;
      if (c[0] >= 1) cand.push_back(c);
    }
  double best = 1e300;
  std::vector<int> pick{nz};
  for (const auto& c : cand) {
    const double t = simulate_queue(cost, c, grid);
    if (t < best * (1.0 - 1e-9)) { best = t; pick = c; }
  }
  return pick;
}

// Make variant idx the one in use: kernel attribute, grid, work decomposition, tensor maps.
// kc_fixed > 0 cuts z into equal chunks of at most kc_fixed planes (ensembles, whose queue is
// ordered by item length across their grids); otherwise the chunking with the best simulated
// balance is taken (choose_chunks).
int use_variant(mhdgb_solver* h, int idx, int kc_fixed = 0) {
  if (idx < 0 || idx > h->nvars) return fail(h, MHDGB_ERR_ARG, "no such variant");
  const FusedVariant& v = h->vars[idx];
  CK(h, v.prepare());
  const int cps = v.ctas_per_sm();
  if (cps < 1) return fail(h, MHDGB_ERR_CUDA, "fused kernel variant does not fit on an SM");
  h->vidx = idx;
  if (idx < h->nvars) h->hlld_vidx = idx;
  h->shape = v.shape;
  h->grid = h->nsm * cps;
  const Layout& L = h->L;
  h->ntx = (L.nx + h->shape.tx - 1) / h->shape.tx;
  h->nty = (L.ny + h->shape.ty - 1) / h->shape.ty;
  std::vector<int> chunks;
  if (kc_fixed > 0) {
    const int nc = std::min((L.nz + kc_fixed - 1) / kc_fixed, MAX_ZCHUNKS);
    const int kc = (L.nz + nc - 1) / nc;
    for (int k = 0; k < L.nz; k += kc) chunks.push_back(std::min(kc, L.nz - k));
  } else {
    chunks = choose_chunks(L, h->shape.tx, h->shape.ty, h->ntx, h->nty, h->grid);
  }
  h->nkc = (int)chunks.size();
  h->kst.assign(1, 0);
  for (int c : chunks) h->kst.push_back(h->kst.back() + c);
  void* pbase[2] = {h->kind == FUSED_MIXED ? (void*)h->P32[0] : (void*)h->P64[0],
                    h->kind == FUSED_MIXED ? (void*)h->P32[1] : (void*)h->P64[1]};
  int rc;
  for (int q = 0; q < 2; q++)
    if ((rc = make_tmap(h, &h->tmap[q], pbase[q], h->shape.elem))) return rc;
  destroy_graph(h);
  return upload_desc(h);
}

// Process-wide autotune results: (kind, nx, ny, nz) -> variant index; optionally persisted in the
// file named by MHDGB_TUNE_CACHE (lines "kind nx ny nz index").
std::mutex g_tune_mu;
std::map<std::tuple<int, int, int, int>, int>& tune_cache() {
  static std::map<std::tuple<int, int, int, int>, int> m;
  static bool loaded = false;
  if (!loaded) {
    loaded = true;
    if (const char* f = std::getenv("MHDGB_TUNE_CACHE")) {
      if (FILE* fp = std::fopen(f, "r")) {
        int k, x, y, z, i;
        while (std::fscanf(fp, "%d %d %d %d %d", &k, &x, &y, &z, &i) == 5) m[std::make_tuple(k, x, y, z)] = i;
        std::fclose(fp);
      }
    }
  }
  return m;
}

void tune_cache_store(int kind, const Layout& L, int idx) {
  std::lock_guard<std::mutex> g(g_tune_mu);
  auto& m = tune_cache();
  m[std::make_tuple(kind, L.nx, L.ny, L.nz)] = idx;
  if (const char* f = std::getenv("MHDGB_TUNE_CACHE")) {
    if (FILE* fp = std::fopen(f, "w")) {
      for (auto& kv : m)
        std::fprintf(fp, "%d %d %d %d %d\n", std::get<0>(kv.first), std::get<1>(kv.first), std::get<2>(kv.first),
                     std::get<3>(kv.first), kv.second);
      std::fclose(fp);
    }
  }
}

int build_graph(mhdgb_solver* h, int nsteps) {
  destroy_graph(h);
  cudaGraph_t g = nullptr;
  CK(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  int rc = MHDGB_OK;
  for (int s = 0; s < nsteps && rc == MHDGB_OK; s++) rc = launch_one(h);
  cudaError_t e = cudaStreamEndCapture(h->stream, &g);
  if (rc != MHDGB_OK) { if (g) cudaGraphDestroy(g); return rc; }
  if (e != cudaSuccess) return cuda_fail(h, e, "cudaStreamEndCapture");
  e = cudaGraphInstantiate(&h->gexec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_fail(h, e, "cudaGraphInstantiate");
  h->gsteps = nsteps;
  return MHDGB_OK;
}

}  // namespace

extern "C" {

int mhdgb_config_default(mhdgb_config* c) {
  if (!c) return MHDGB_ERR_ARG;
  std::memset(c, 0, sizeof(*c));
  c->nx = c->ny = c->nz = 150;
  c->x1min = -0.5; c->x1max = 0.5;
  c->x2min = -1.0; c->x2max = 1.0;
  c->x3min = -0.5; c->x3max = 0.5;
  c->bc[0] = c->bc[1] = MHDGB_BC_PERIODIC;
  c->bc[2] = c->bc[3] = MHDGB_BC_REFLECTION;
  c->bc[4] = c->bc[5] = MHDGB_BC_PERIODIC;
  c->gam = 5.0 / 3.0;
  c->cfl = 0.05;
  c->precision = MHDGB_FP64;
  c->spacing_quirk = 0;
  c->device = 0;
  return MHDGB_OK;
}

const char* mhdgb_status_string(int s) {
  switch (s) {
    case MHDGB_OK: return "ok";
    case MHDGB_ERR_ARG: return "invalid argument";
    case MHDGB_ERR_CUDA: return "CUDA error";
    case MHDGB_ERR_NONFINITE: return "non-finite value in the state";
    case MHDGB_ERR_NEGATIVE: return "non-positive density or pressure";
    case MHDGB_ERR_TIMEOUT: return "device-side wait timed out";
    case MHDGB_ERR_STATE: return "call out of order";
    case MHDGB_ERR_NOMEM: return "device allocation failed";
    case MHDGB_ERR_SCRATCH: return "grid too large for the fixed scratch of mhdgb_fill_ghosts_noalloc";
    case MHDGB_ERR_IO: return "file output failed";
    default: return "unknown status";
  }
}

const char* mhdgb_last_error(const mhdgb_solver* h) { return h ? h->err.c_str() : "null handle"; }

}  // extern "C"

namespace {
int create_impl(const mhdgb_config* cfg, cudaStream_t shared, mhdgb_solver** out) {
  if (!cfg || !out) return MHDGB_ERR_ARG;
  *out = nullptr;
  if (cfg->nx < 2 || cfg->ny < 2 || cfg->nz < 2) return MHDGB_ERR_ARG;
  if (!(cfg->gam > 1.0) || !(cfg->cfl > 0.0)) return MHDGB_ERR_ARG;
  for (int q = 0; q < 6; q++)
    if (cfg->bc[q] < MHDGB_BC_PERIODIC || cfg->bc[q] > MHDGB_BC_EXCHANGE) return MHDGB_ERR_ARG;
  if (cfg->precision < MHDGB_FP64 || cfg->precision > MHDGB_MIXED) return MHDGB_ERR_ARG;
  if (cfg->spacing_quirk && (cfg->nx > cfg->ny || cfg->nx > cfg->nz)) return MHDGB_ERR_ARG;
  mhdgb_solver* h = new mhdgb_solver();
  h->cfg = *cfg;
  int rc = set_device(h);
  if (rc) { delete h; return rc; }
  h->kind = cfg->precision == MHDGB_MIXED ? FUSED_MIXED : (cfg->precision == MHDGB_FP64_EXACT ? FUSED_FP64_EXACT : FUSED_FP64);
  h->nvars = fused_variants(h->kind, &h->vars);
  Layout& L = h->L;
  L.nx = cfg->nx; L.ny = cfg->ny; L.nz = cfg->nz;
  L.itot = cfg->nx + 2 * NGH + 1; L.jtot = cfg->ny + 2 * NGH + 1; L.ktot = cfg->nz + 2 * NGH + 1;
  L.ip = (L.itot + 7) / 8 * 8;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, cfg->device) != cudaSuccess) { delete h; return MHDGB_ERR_CUDA; }
  h->nsm = prop.multiProcessorCount;
  auto cleanup = [&](int code) { mhdgb_destroy(h); return code; };
  if (shared) {
    h->stream = shared;
    h->own_stream = false;
  } else if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
    return cleanup(MHDGB_ERR_CUDA);
  }
  const int nmax = std::max(L.itot, std::max(L.jtot, L.ktot));
  // Working set of the fused step: U and the two primitive buffers of its precision.  The stage
  // path's flux and pack buffers (and FP64 primitives for the mixed form) come on first use.
  bool ok = dalloc(h, &h->U, L.count(NCONS)) == cudaSuccess;
  if (h->kind == FUSED_MIXED)
    for (int q = 0; q < 2 && ok; q++) ok = dalloc(h, &h->P32[q], L.count(NPRIM)) == cudaSuccess;
  else
    for (int q = 0; q < 2 && ok; q++) ok = dalloc(h, &h->P64[q], L.count(NPRIM)) == cudaSuccess;
  ok = ok && dalloc(h, &h->d_desc, 1) == cudaSuccess && dalloc(h, &h->d_lc, 1) == cudaSuccess;
  ok = ok && dalloc(h, &h->xinv, nmax) == cudaSuccess && dalloc(h, &h->yinv, nmax) == cudaSuccess &&
       dalloc(h, &h->zinv, nmax) == cudaSuccess && dalloc(h, &h->dxs, nmax) == cudaSuccess &&
       dalloc(h, &h->dys, nmax) == cudaSuccess && dalloc(h, &h->dzs, nmax) == cudaSuccess &&
       dalloc(h, &h->xinvf, nmax) == cudaSuccess && dalloc(h, &h->yinvf, nmax) == cudaSuccess &&
       dalloc(h, &h->zinvf, nmax) == cudaSuccess && dalloc(h, &h->dxsf, nmax) == cudaSuccess &&
       dalloc(h, &h->dysf, nmax) == cudaSuccess && dalloc(h, &h->dzsf, nmax) == cudaSuccess;
  ok = ok && dalloc(h, &h->scal, 8 + 3 * (size_t)L.nz) == cudaSuccess;
  ok = ok && dalloc(h, &h->faces, (size_t)L.itot + L.jtot) == cudaSuccess;
  ok = ok && dalloc(h, &h->sslot, 1) == cudaSuccess && dalloc(h, &h->ctrl, 1) == cudaSuccess;
  if (!ok) return cleanup(MHDGB_ERR_NOMEM);
  h->x1a = face_axis(cfg->nx, cfg->x1min, cfg->x1max);
  h->x2a = face_axis(cfg->ny, cfg->x2min, cfg->x2max);
  h->x3a = face_axis(cfg->nz, cfg->x3min, cfg->x3max);
  if ((rc = upload_grid(h))) return cleanup(rc);
  {
    int idx = fused_preferred_variant(h->kind);
    if (idx >= h->nvars) idx = 0;
    std::lock_guard<std::mutex> g(g_tune_mu);
    auto& m = tune_cache();
    auto it = m.find(std::make_tuple((int)h->kind, L.nx, L.ny, L.nz));
    if (it != m.end() && it->second < h->nvars) idx = it->second;
    if ((rc = use_variant(h, idx)) && (idx == 0 || (rc = use_variant(h, 0)))) return cleanup(rc);
  }
  k_ctrl_reset<<<1, 1, 0, h->stream>>>(h->ctrl, 0);
  k_ctrl_set_stop<<<1, 1, 0, h->stream>>>(h->ctrl, 1.0e300, ~0ull);
  if (cudaStreamSynchronize(h->stream) != cudaSuccess) return cleanup(MHDGB_ERR_CUDA);
  *out = h;
  return MHDGB_OK;
}

}  // namespace

extern "C" {

int mhdgb_create(const mhdgb_config* cfg, mhdgb_solver** out) { return create_impl(cfg, nullptr, out); }

int mhdgb_destroy(mhdgb_solver* h) {
  if (!h) return MHDGB_OK;
  if (h->writer.joinable()) h->writer.join();
  cudaSetDevice(h->cfg.device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->copy_stream) cudaStreamSynchronize(h->copy_stream);
  destroy_graph(h);
  void* ptrs[] = {h->U, h->P64[0], h->P64[1], h->P32[0], h->P32[1], h->F[0], h->F[1], h->F[2], h->pack,
                  h->xinv, h->yinv, h->zinv, h->dxs, h->dys, h->dzs, h->xinvf, h->yinvf, h->zinvf,
                  h->dxsf, h->dysf, h->dzsf, h->scal, h->faces, h->sslot, h->ctrl, h->d_desc, h->d_lc, h->stage,
                  h->d_snap};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (h->h_snap) cudaFreeHost(h->h_snap);
  if (h->ev_packed) cudaEventDestroy(h->ev_packed);
  if (h->ev_copied) cudaEventDestroy(h->ev_copied);
  if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
  if (h->stream && h->own_stream) cudaStreamDestroy(h->stream);
  delete h;
  return MHDGB_OK;
}

int mhdgb_extents(const mhdgb_solver* h, int* itot, int* jtot, int* ktot) {
  if (!h) return MHDGB_ERR_ARG;
  if (itot) *itot = h->L.itot;
  if (jtot) *jtot = h->L.jtot;
  if (ktot) *ktot = h->L.ktot;
  return MHDGB_OK;
}

size_t mhdgb_device_bytes(const mhdgb_solver* h) { return h ? h->bytes : 0; }

int mhdgb_get_grid(const mhdgb_solver* h, double* x1a, double* x2a, double* x3a) {
  if (!h) return MHDGB_ERR_ARG;
  if (x1a) std::memcpy(x1a, h->x1a.data(), h->x1a.size() * sizeof(double));
  if (x2a) std::memcpy(x2a, h->x2a.data(), h->x2a.size() * sizeof(double));
  if (x3a) std::memcpy(x3a, h->x3a.data(), h->x3a.size() * sizeof(double));
  return MHDGB_OK;
}

int mhdgb_set_physics(mhdgb_solver* h, double gam, double cfl, const int* bc) {
  if (!h || !(gam > 1.0) || !(cfl > 0.0)) return MHDGB_ERR_ARG;
  if (bc)
    for (int q = 0; q < 6; q++)
      if (bc[q] < MHDGB_BC_PERIODIC || bc[q] > MHDGB_BC_EXCHANGE) return MHDGB_ERR_ARG;
  int rc = set_device(h);
  if (rc || (rc = settle(h))) return rc;
  const bool same = h->cfg.gam == gam && h->cfg.cfl == cfl &&
                    (!bc || std::equal(bc, bc + 6, h->cfg.bc));
  if (same) return MHDGB_OK;
  h->cfg.gam = gam;
  h->cfg.cfl = cfl;
  if (bc) std::copy(bc, bc + 6, h->cfg.bc);
  h->prepared = false;
  h->p64_valid = h->p_user;
  destroy_graph(h);
  return upload_desc(h);
}

int mhdgb_set_riemann(mhdgb_solver* h, int solver) {
  if (!h || solver < MHDGB_RIEMANN_HLLD || solver > MHDGB_RIEMANN_HLLC) return MHDGB_ERR_ARG;
  int rc = set_device(h);
  if (rc || (rc = settle(h))) return rc;
  if (h->riemann == solver) return MHDGB_OK;
  h->riemann = solver;
  // HLLD runs on the tuned HLLD variants, HLLE/HLLC on the run-time solver kernel
  const int want = solver == MHDGB_RIEMANN_HLLD ? h->hlld_vidx : h->nvars;
  if (want != h->vidx) return use_variant(h, want);
  destroy_graph(h);
  return upload_desc(h);
}

int mhdgb_get_riemann(const mhdgb_solver* h) { return h ? h->riemann : MHDGB_ERR_ARG; }

int mhdgb_set_grid(mhdgb_solver* h, const double* x1a, const double* x2a, const double* x3a) {
  if (!h || !x1a || !x2a || !x3a) return MHDGB_ERR_ARG;
  int rc = set_device(h);
  if (rc) return rc;
  h->x1a.assign(x1a, x1a + h->L.itot);
  h->x2a.assign(x2a, x2a + h->L.jtot);
  h->x3a.assign(x3a, x3a + h->L.ktot);
  h->prepared = false;
  return upload_grid(h);
}

int mhdgb_upload_cons(mhdgb_solver* h, const double* U) {
  if (!h || !U) return MHDGB_ERR_ARG;
  int rc = set_device(h);
  if (rc || (rc = settle(h)) || (rc = upload_u(h, U))) return rc;
  h->have_state = true;
  h->prepared = false;
  h->p64_valid = h->p_user;  // a P the caller uploaded stays in force, as the reference's P array does
  CK(h, cudaStreamSynchronize(h->stream));
  return MHDGB_OK;
}

int mhdgb_upload_prim(mhdgb_solver* h, const double* P) {
  if (!h || !P) return MHDGB_ERR_ARG;
  int rc = set_device(h);
  if (rc || (rc = settle(h)) || (rc = ensure_stage_bufs(h)) ||
      (rc = copy_h2d(h, h->P64[cur_index(h)], P, NPRIM, sizeof(double))))
    return rc;
  h->p64_valid = true;
  h->p_user = true;
  h->prepared = false;
  CK(h, cudaStreamSynchronize(h->stream));
  return MHDGB_OK;
}

int mhdgb_download_cons(mhdgb_solver* h, double* U) {
  if (!h || !U) return MHDGB_ERR_ARG;
  int rc = set_device(h);
  if (rc || (rc = settle(h)) || (rc = download_u(h, U))) return rc;
  CK(h, cudaStreamSynchronize(h->stream));
  return MHDGB_OK;
}

int mhdgb_download_prim(mhdgb_solver* h, double* P) {
  if (!h || !P) return MHDGB_ERR_ARG;
  int rc = set_device(h);
  if (rc || (rc = mhdgb_sync(h, nullptr)) < 0) {
    if (rc != MHDGB_ERR_NONFINITE && rc != MHDGB_ERR_NEGATIVE) return rc;
  }
  if ((rc = ensure_p64(h))) return rc;
  if ((rc = copy_d2h(h, P, h->P64[cur_index(h)], NPRIM, sizeof(double)))) return rc;
  CK(h, cudaStreamSynchronize(h->stream));
  return MHDGB_OK;
}

}  // extern "C"

namespace {
int field_transfer(mhdgb_solver* h, bool cons, int n, const double* in, double* out) {
  const int nv = cons ? NCONS : NPRIM;
  if (!h || n < 0 || n >= nv || (!in && !out)) return MHDGB_ERR_ARG;
  int rc = set_device(h);
  if (rc || (rc = settle(h))) return rc;
  if (!cons && (rc = ensure_stage_bufs(h))) return rc;
  const Layout& L = h->L;
  const size_t rows = (size_t)L.jtot * L.ktot, bytes = rows * L.itot * sizeof(double);
  double* st = staging(h);
  if (!st) return fail(h, MHDGB_ERR_NOMEM, "staging buffer");
  double* arr = cons ? h->U : h->P64[cur_index(h)];
  if (in) {
    if (!cons && !h->p64_valid && (rc = ensure_p64(h))) return rc;  // keep the other fields consistent
    CK(h, cudaMemcpyAsync(st, in, bytes, cudaMemcpyHostToDevice, h->stream));
    k_field<<<h->nsm * 8, 256, 0, h->stream>>>(st, arr, L.itot, L.ip, nv, n, rows, 1);
    CK(h, cudaGetLastError());
    if (cons) { h->have_state = true; h->prepared = false; h->p64_valid = h->p_user; }
    else { h->p64_valid = true; h->p_user = true; h->prepared = false; }
  } else {
    if (!cons && (rc = ensure_p64(h))) return rc;
    k_field<<<h->nsm * 8, 256, 0, h->stream>>>(arr, st, L.itot, L.ip, nv, n, rows, 0);
    CK(h, cudaGetLastError());
    CK(h, cudaMemcpyAsync(out, st, bytes, cudaMemcpyDeviceToHost, h->stream));
  }
  CK(h, cudaStreamSynchronize(h->stream));
  return MHDGB_OK;
}
}  // namespace

extern "C" {

int mhdgb_upload_cons_field(mhdgb_solver* h, int m, const double* a) { return field_transfer(h, true, m, a, nullptr); }
int mhdgb_download_cons_field(mhdgb_solver* h, int m, double* a) { return field_transfer(h, true, m, nullptr, a); }
int mhdgb_upload_prim_field(mhdgb_solver* h, int n, const double* a) { return field_transfer(h, false, n, a, nullptr); }
int mhdgb_download_prim_field(mhdgb_solver* h, int n, double* a) { return field_transfer(h, false, n, nullptr, a); }

int mhdgb_download_flux(mhdgb_solver* h, int dir, double* F) {
  if (!h || !F || dir < 1 || dir > 3) return MHDGB_ERR_ARG;
  int rc = set_device(h);
  if (rc || (rc = ensure_stage_bufs(h)) || (rc = copy_d2h(h, F, h->F[dir - 1], NCONS, sizeof(double)))) return rc;
  CK(h, cudaStreamSynchronize(h->stream));
  return MHDGB_OK;
}

// ---- stage entry points ----
int mhdgb_control_timestep(mhdgb_solver* h, double* dt) {
  if (!h) return MHDGB_ERR_ARG;
  int rc = set_device(h);
  if (rc || (rc = ensure_p64(h))) return rc;
  CK(h, launch_reduce_dt_ch(h->P64[cur_index(h)], h->L, h->dxs, h->dys, h->dzs, h->sslot, &h->ctrl->status, h->nsm,
                            h->stream));
  double tmp[2];
  CK(h, launch_slot_to_scalars(h->sslot, h->cfg.cfl, h->scal + 2, h->scal + 3, h->stream));
  CK(h, cudaMemcpyAsync(h->scal + 0, h->scal + 2, sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  CK(h, cudaMemcpyAsync(tmp, h->scal + 2, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  if (dt) *dt = tmp[0];
  return MHDGB_OK;
}

int mhdgb_set_boundary(mhdgb_solver* h) {
  if (!h) return MHDGB_ERR_ARG;
  int rc = set_device(h);
  if (rc || (rc = ensure_p64(h))) return rc;
  CK(h, launch_ghost_fill(h->P64[cur_index(h)], h->L, h->cfg.bc, h->pack, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  return MHDGB_OK;
}

int mhdgb_evaluate_ch(mhdgb_solver* h, double* chg) {
  if (!h) return MHDGB_ERR_ARG;
  int rc = set_device(h);
  if (rc || (rc = ensure_p64(h))) return rc;
  CK(h, launch_reduce_dt_ch(h->P64[cur_index(h)], h->L, h->dxs, h->dys, h->dzs, h->sslot, &h->ctrl->status, h->nsm,
                            h->stream));
  double tmp[2];
  CK(h, launch_slot_to_scalars(h->sslot, h->cfg.cfl, h->scal + 2, h->scal + 3, h->stream));
  CK(h, cudaMemcpyAsync(h->scal + 1, h->scal + 3, sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  CK(h, cudaMemcpyAsync(tmp, h->scal + 2, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  if (chg) *chg = tmp[1];
  return MHDGB_OK;
}

int mhdgb_flux(mhdgb_solver* h, int dir) {
  if (!h || dir < 1 || dir > 3) return MHDGB_ERR_ARG;
  int rc = set_device(h);
  if (rc || (rc = ensure_p64(h))) return rc;
  CK(h, launch_flux(dir, h->P64[cur_index(h)], h->F[dir - 1], h->L, h->scal + 1, h->riemann, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  return MHDGB_OK;
}

int mhdgb_update_conserv(mhdgb_solver* h) {
  if (!h) return MHDGB_ERR_ARG;
  int rc = set_device(h);
  if (rc) return rc;
  if ((rc = ensure_stage_bufs(h))) return rc;
  if (!h->have_state) return fail(h, MHDGB_ERR_STATE, "no state uploaded");
  CK(h, launch_update_conserv(h->F[0], h->F[1], h->F[2], h->U, h->L, h->xinv, h->yinv, h->zinv,
                              h->cfg.spacing_quirk, h->scal + 0, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  h->prepared = false;
  return MHDGB_OK;
}

int mhdgb_damp_psi(mhdgb_solver* h) {
  if (!h) return MHDGB_ERR_ARG;
  int rc = set_device(h);
  if (rc) return rc;
  if ((rc = ensure_stage_bufs(h))) return rc;
  if (!h->have_state) return fail(h, MHDGB_ERR_STATE, "no state uploaded");
  CK(h, launch_damp_psi(h->U, h->L, h->dxs, h->dys, h->dzs, h->scal + 0, h->scal + 1, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  h->prepared = false;
  return MHDGB_OK;
}

int mhdgb_update_prim(mhdgb_solver* h) {
  if (!h) return MHDGB_ERR_ARG;
  int rc = set_device(h);
  if (rc) return rc;
  if ((rc = ensure_stage_bufs(h))) return rc;
  if (!h->have_state) return fail(h, MHDGB_ERR_STATE, "no state uploaded");
  CK(h, launch_update_prim(h->U, h->P64[cur_index(h)], h->L, h->cfg.gam, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  h->p64_valid = true;
  h->p_user = false;
  h->prepared = false;
  return MHDGB_OK;
}

int mhdgb_set_dt(mhdgb_solver* h, double dt) {
  if (!h) return MHDGB_ERR_ARG;
  int rc = set_device(h);
  if (rc) return rc;
  CK(h, cudaMemcpy(h->scal + 0, &dt, sizeof(double), cudaMemcpyHostToDevice));
  CK(h, legacy_fence());
  return MHDGB_OK;
}

int mhdgb_set_chg(mhdgb_solver* h, double chg) {
  if (!h) return MHDGB_ERR_ARG;
  int rc = set_device(h);
  if (rc) return rc;
  CK(h, cudaMemcpy(h->scal + 1, &chg, sizeof(double), cudaMemcpyHostToDevice));
  CK(h, legacy_fence());
  return MHDGB_OK;
}

// ---- fused step ----
int mhdgb_prepare(mhdgb_solver* h) {
  if (!h) return MHDGB_ERR_ARG;
  int rc = set_device(h);
  if (rc) return rc;
  if (!h->have_state) return fail(h, MHDGB_ERR_STATE, "no state uploaded");
  Ctrl c;
  if ((rc = read_ctrl(h, &c))) return rc;
  h->cur_step = (long long)c.step;
  const int cur = cur_index(h);
  CK(h, launch_reset_slot(&h->ctrl->slot[c.step % 3], h->stream));
  CK(h, launch_reset_slot(&h->ctrl->slot[(c.step + 1) % 3], h->stream));
  FusedArgs a = fused_args(h);
  CK(h, launch_recover(h->kind, a, cur, &h->ctrl->slot[c.step % 3], h->nsm, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  h->prepared = true;
  h->p64_valid = h->kind != FUSED_MIXED;
  return MHDGB_OK;
}

int mhdgb_step(mhdgb_solver* h, int nsteps) {
  if (!h || nsteps < 0) return MHDGB_ERR_ARG;
  int rc = set_device(h);
  if (rc) return rc;
  if (!h->prepared && (rc = mhdgb_prepare(h))) return rc;
  const int G = 16;
  if (nsteps >= G && !h->gexec && (rc = build_graph(h, G))) return rc;
  while (nsteps >= G) {
    CK(h, cudaGraphLaunch(h->gexec, h->stream));
    nsteps -= G;
  }
  for (; nsteps > 0; nsteps--)
    if ((rc = launch_one(h))) return rc;
  h->p64_valid = false;
  h->p_user = false;
  return MHDGB_OK;
}

int mhdgb_set_stop(mhdgb_solver* h, double tmax, long long max_steps) {
  if (!h) return MHDGB_ERR_ARG;
  int rc = set_device(h);
  if (rc) return rc;
  k_ctrl_set_stop<<<1, 1, 0, h->stream>>>(h->ctrl, tmax, max_steps < 0 ? ~0ull : (unsigned long long)max_steps);
  CK(h, cudaGetLastError());
  CK(h, cudaStreamSynchronize(h->stream));
  return MHDGB_OK;
}

int mhdgb_sync(mhdgb_solver* h, mhdgb_report* r) {
  if (!h) return MHDGB_ERR_ARG;
  int rc = set_device(h);
  if (rc) return rc;
  Ctrl c;
  if ((rc = read_ctrl(h, &c))) return rc;
  if ((long long)c.step != h->cur_step) {
    h->cur_step = (long long)c.step;
    h->p64_valid = false;
  }
  if (r) {
    r->step = (long long)c.step;
    r->time = c.time;
    r->dt = c.last_dt;
    r->chg = c.last_ch;
    r->next_dt = h->cfg.cfl * bitsd(c.slot[c.step % 3].dtmin_bits);
    r->next_chg = bitsd(c.slot[c.step % 3].chmax_bits);
    r->done = (int)c.done;
    r->status = c.status;
  }
  return status_to_code(h, c.status);
}

int mhdgb_run_until(mhdgb_solver* h, double tmax, long long max_steps, mhdgb_report* r) {
  int rc = mhdgb_set_stop(h, tmax, max_steps);
  if (rc) return rc;
  mhdgb_report rep;
  for (;;) {
    if ((rc = mhdgb_step(h, 64))) return rc;
    if ((rc = mhdgb_sync(h, &rep))) return rc;
    if (rep.done) break;
  }
  if (r) *r = rep;
  return MHDGB_OK;
}

int mhdgb_reset_clock(mhdgb_solver* h) {
  if (!h) return MHDGB_ERR_ARG;
  int rc = set_device(h);
  if (rc) return rc;
  k_ctrl_reset<<<1, 1, 0, h->stream>>>(h->ctrl, 0);
  CK(h, cudaGetLastError());
  CK(h, cudaStreamSynchronize(h->stream));
  h->cur_step = 0;
  h->prepared = false;
  h->p64_valid = false;
  return MHDGB_OK;
}

}  // extern "C"

namespace {

// Device address of a host array of n doubles that is page-locked and mapped (cudaHostAlloc,
// cudaHostRegister), or null.  Both ends are checked, so a registration that covers only part of
// the array is not taken.
const double* mapped_view(const double* p, size_t n) {
  cudaPointerAttributes a0{}, a1{};
  if (cudaPointerGetAttributes(&a0, p) != cudaSuccess || cudaPointerGetAttributes(&a1, p + n - 1) != cudaSuccess) {
    cudaGetLastError();  // an unknown pointer is not an error here
    return nullptr;
  }
  if (a0.type != cudaMemoryTypeHost || a1.type != cudaMemoryTypeHost || !a0.devicePointer || !a1.devicePointer)
    return nullptr;
  const double* d0 = static_cast<const double*>(a0.devicePointer);
  if (static_cast<const double*>(a1.devicePointer) != d0 + (n - 1)) return nullptr;
  return d0;
}

// mhdgb_step_host with page-locked, mapped arrays: the recovery pass reads U_in over the host link
// (copying every cell into the device U and, for a separate U_out, the ghost cells into U_out), and
// the last step's cell updates write U_out as they are made, so the transfers overlap the work and
// no staging copy or repacking pass runs.
int step_host_mapped(mhdgb_solver* h, const double* din, double* dout, bool same, int nsteps) {
  Ctrl c;
  int rc = read_ctrl(h, &c);
  if (rc) return rc;
  h->cur_step = (long long)c.step;
  h->have_state = true;
  h->p_user = false;
  CK(h, launch_reset_slot(&h->ctrl->slot[c.step % 3], h->stream));
  CK(h, launch_reset_slot(&h->ctrl->slot[(c.step + 1) % 3], h->stream));
  const FusedArgs a = fused_args(h);
  CK(h, launch_recover(h->kind, a, cur_index(h), &h->ctrl->slot[c.step % 3], h->nsm, h->stream, din,
                       same ? nullptr : dout));
  h->prepared = true;
  h->p64_valid = h->kind != FUSED_MIXED;
  if (nsteps > 1 && (rc = mhdgb_step(h, nsteps - 1))) return rc;
  k_set_host_u<<<1, 1, 0, h->stream>>>(h->d_desc, dout);
  CK(h, cudaGetLastError());
  rc = mhdgb_step(h, 1);
  k_set_host_u<<<1, 1, 0, h->stream>>>(h->d_desc, nullptr);
  CK(h, cudaGetLastError());
  return rc;
}

}  // namespace

extern "C" {

int mhdgb_step_host(mhdgb_solver* h, const double* U_in, double* U_out, int nsteps, double* dt, double* chg) {
  if (!h || !U_in || !U_out || nsteps < 1) return MHDGB_ERR_ARG;
  int rc = set_device(h);
  if (rc) return rc;
  const Layout& L = h->L;
  const size_t n = (size_t)NCONS * L.itot * L.jtot * L.ktot;
  const double* din = mapped_view(U_in, n);
  const double* dout = mapped_view(U_out, n);
  // arrays that overlap without being the same one take the staged route: the recovery pass writes
  // U_out's ghost cells while it is still reading U_in
  const bool partial_overlap = U_in != U_out && U_in < U_out + n && U_out < U_in + n;
  if (din && dout && !partial_overlap) {
    if ((rc = step_host_mapped(h, din, const_cast<double*>(dout), din == dout, nsteps))) return rc;
  } else {
    if ((rc = settle(h)) || (rc = upload_u(h, U_in))) return rc;
    h->have_state = true;
    h->prepared = false;
    h->p_user = false;
    if ((rc = mhdgb_prepare(h)) || (rc = mhdgb_step(h, nsteps))) return rc;
    if ((rc = settle(h)) || (rc = download_u(h, U_out))) return rc;
  }
  mhdgb_report rep;
  rc = mhdgb_sync(h, &rep);
  if (dt) *dt = rep.dt;
  if (chg) *chg = rep.chg;
  return rc;
}

int mhdgb_time_steps(mhdgb_solver* h, int nsteps, double* ms) {
  if (!h || nsteps < 1 || !ms) return MHDGB_ERR_ARG;
  int rc = set_device(h);
  if (rc) return rc;
  if (!h->prepared && (rc = mhdgb_prepare(h))) return rc;
  const int G = 16;
  if (nsteps >= G && !h->gexec && (rc = build_graph(h, G))) return rc;
  cudaEvent_t e0, e1;
  CK(h, cudaEventCreate(&e0));
  CK(h, cudaEventCreate(&e1));
  CK(h, cudaStreamSynchronize(h->stream));
  CK(h, cudaEventRecord(e0, h->stream));
  rc = mhdgb_step(h, nsteps);
  CK(h, cudaEventRecord(e1, h->stream));
  CK(h, cudaEventSynchronize(e1));
  float t = 0.0f;
  CK(h, cudaEventElapsedTime(&t, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms = t;
  return rc;
}

int mhdgb_measure_fp64_rate(int device, double* gflops) {
  if (!gflops) return MHDGB_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return MHDGB_ERR_CUDA;
  int nsm = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
  const int bs = 256, grid = nsm * 8, iters = 4000;
  double* out = nullptr;
  if (cudaMalloc(&out, sizeof(double) * grid * bs) != cudaSuccess) return MHDGB_ERR_NOMEM;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_dfma_rate<<<grid, bs>>>(out, 50);
  cudaDeviceSynchronize();
  float best = 1e30f;
  for (int rep = 0; rep < 3; rep++) {
    cudaEventRecord(e0);
    k_dfma_rate<<<grid, bs>>>(out, iters);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    best = std::min(best, ms);
  }
  const cudaError_t e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (e != cudaSuccess) return MHDGB_ERR_CUDA;
  *gflops = 2.0 * 8.0 * iters * (double)grid * bs / (best * 1e-3) / 1e9;  // 2 flops per FMA
  return MHDGB_OK;
}

int mhdgb_selftest_division(int device, int n, unsigned long long seed, double* max_ulp) {
  if (!max_ulp || n < 1) return MHDGB_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return MHDGB_ERR_CUDA;
  unsigned long long* d = nullptr;
  if (cudaMalloc(&d, sizeof(*d)) != cudaSuccess) return MHDGB_ERR_NOMEM;
  unsigned long long h = 0;
  cudaError_t e = cudaMemset(d, 0, sizeof(*d));
  if (e == cudaSuccess) e = detail::fdiv_selftest(n, seed, d, nullptr);
  if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return MHDGB_ERR_CUDA;
  *max_ulp = (double)h;
  return MHDGB_OK;
}

int mhdgb_selftest_wait_timeout(int device, double* seconds, unsigned* status) {
  if (!seconds || !status) return MHDGB_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return MHDGB_ERR_CUDA;
  unsigned* d = nullptr;
  if (cudaMalloc(&d, sizeof(*d)) != cudaSuccess) return MHDGB_ERR_NOMEM;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaMemset(d, 0, sizeof(*d));
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e == cudaSuccess) e = cudaEventRecord(e0);
  if (e == cudaSuccess) {
    k_wait_selftest<<<1, 32>>>(d);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaEventRecord(e1);
  if (e == cudaSuccess) e = cudaEventSynchronize(e1);
  float ms = 0.0f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  unsigned h = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(d);
  if (e != cudaSuccess) return MHDGB_ERR_CUDA;
  *seconds = ms * 1e-3;
  *status = h;
  return MHDGB_OK;
}

int mhdgb_variant_count(const mhdgb_solver* h) { return h ? h->nvars : 0; }

int mhdgb_variant_info(const mhdgb_solver* h, int idx, int* tx, int* ty, int* threads, int* current) {
  if (!h || idx < 0 || idx >= h->nvars) return MHDGB_ERR_ARG;
  if (tx) *tx = h->vars[idx].shape.tx;
  if (ty) *ty = h->vars[idx].shape.ty;
  if (threads) *threads = h->vars[idx].shape.threads;
  if (current) *current = idx == h->vidx;
  return MHDGB_OK;
}

int mhdgb_work_layout(const mhdgb_solver* h, int* ntx, int* nty, int* nchunks, int* kstart) {
  if (!h) return MHDGB_ERR_ARG;
  if (ntx) *ntx = h->ntx;
  if (nty) *nty = h->nty;
  if (nchunks) *nchunks = h->nkc;
  if (kstart)
    for (size_t c = 0; c < h->kst.size(); c++) kstart[c] = h->kst[c];
  return MHDGB_OK;
}

int mhdgb_plan_zchunks(int nx, int ny, int nz, int tx, int ty, int ctas, int* chunks, int max_chunks) {
  if (nx < 1 || ny < 1 || nz < 1 || tx < 1 || ty < 1 || ctas < 1 || !chunks || max_chunks < 1) return MHDGB_ERR_ARG;
  Layout L{};
  L.nx = nx;
  L.ny = ny;
  L.nz = nz;
  const std::vector<int> c = choose_chunks(L, tx, ty, (nx + tx - 1) / tx, (ny + ty - 1) / ty, ctas);
  if ((int)c.size() > max_chunks) return MHDGB_ERR_ARG;
  for (size_t i = 0; i < c.size(); i++) chunks[i] = c[i];
  return (int)c.size();
}

const char* mhdgb_variant_name(const mhdgb_solver* h, int idx) {
  if (!h) return nullptr;
  if (idx == -1) idx = h->vidx;
  if (idx < 0 || idx > h->nvars) return nullptr;
  return h->vars[idx].name;
}

int mhdgb_select_variant(mhdgb_solver* h, int idx) {
  if (!h || idx < 0 || idx >= h->nvars) return MHDGB_ERR_ARG;
  int rc = set_device(h);
  if (rc || (rc = mhdgb_sync(h, nullptr)) == MHDGB_ERR_CUDA) return rc;
  if (h->riemann != MHDGB_RIEMANN_HLLD) {  // HLLE/HLLC keep their kernel; the choice applies to HLLD
    h->hlld_vidx = idx;
    return MHDGB_OK;
  }
  const bool was_prepared = h->prepared;
  if ((rc = use_variant(h, idx))) return rc;
  h->prepared = was_prepared;  // the P buffers and reduction slots do not depend on the tile shape
  return MHDGB_OK;
}

int mhdgb_autotune(mhdgb_solver* h, int steps, int* best) {
  if (!h || steps < 1) return MHDGB_ERR_ARG;
  int rc = set_device(h);
  if (rc) return rc;
  if (!h->have_state) return fail(h, MHDGB_ERR_STATE, "autotune needs an uploaded state");
  if (h->riemann != MHDGB_RIEMANN_HLLD) {  // one kernel runs HLLE/HLLC: nothing to choose
    if (best) *best = h->hlld_vidx;
    return MHDGB_OK;
  }
  Ctrl saved;
  if ((rc = read_ctrl(h, &saved))) return rc;
  const Layout& L = h->L;
  const size_t rows = (size_t)NCONS * L.jtot * L.ktot;
  double* st = staging(h);
  if (!st) return fail(h, MHDGB_ERR_NOMEM, "staging buffer");
  k_repack<<<h->nsm * 8, 256, 0, h->stream>>>(h->U, st, L.itot, L.ip, rows, 0);  // keep U
  CK(h, cudaGetLastError());
  auto restore = [&]() -> int {
    k_repack<<<h->nsm * 8, 256, 0, h->stream>>>(st, h->U, L.itot, L.ip, rows, 1);
    CK(h, cudaGetLastError());
    CK(h, cudaMemcpyAsync(h->ctrl, &saved, sizeof(Ctrl), cudaMemcpyHostToDevice, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    h->cur_step = (long long)saved.step;
    h->prepared = false;
    h->p64_valid = false;
    return MHDGB_OK;
  };
  double best_ms = 1e300;
  int bidx = h->vidx;
  for (int v = 0; v < h->nvars; v++) {
    if ((rc = use_variant(h, v)) || (rc = restore())) return rc;
    double ms = 0.0;
    if ((rc = mhdgb_time_steps(h, 2, &ms)) || (rc = mhdgb_time_steps(h, steps, &ms))) return rc;
    if (ms < best_ms) { best_ms = ms; bidx = v; }
  }
  if ((rc = use_variant(h, bidx)) || (rc = restore())) return rc;
  tune_cache_store((int)h->kind, h->L, bidx);
  if (best) *best = bidx;
  return MHDGB_OK;
}

int mhdgb_diag(mhdgb_solver* h, double out[3]) {
  if (!h || !out) return MHDGB_ERR_ARG;
  int rc = set_device(h);
  if (rc || (rc = mhdgb_sync(h, nullptr)) == MHDGB_ERR_CUDA) return rc;
  const Layout& L = h->L;
  double* planes = h->scal + 8;
  if (h->kind == FUSED_MIXED && h->prepared) {
    k_diag_planes<float><<<L.nz, 256, 0, h->stream>>>(h->P32[cur_index(h)], L, h->dxs, h->dys, h->dzs, planes);
  } else if (h->prepared) {  // the fused step's FP64 primitives, read as they are
    k_diag_planes<double><<<L.nz, 256, 0, h->stream>>>(h->P64[cur_index(h)], L, h->dxs, h->dys, h->dzs, planes);
  } else {
    if ((rc = ensure_p64(h))) return rc;
    k_diag_planes<double><<<L.nz, 256, 0, h->stream>>>(h->P64[cur_index(h)], L, h->dxs, h->dys, h->dzs, planes);
  }
  CK(h, cudaGetLastError());
  k_diag_final<<<1, 1, 0, h->stream>>>(planes, L.nz, h->scal + 4);
  CK(h, cudaGetLastError());
  CK(h, cudaMemcpyAsync(out, h->scal + 4, 3 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  return MHDGB_OK;
}

}  // extern "C"

namespace {
// The KH state of cell block (i0, j0, k0) + (nx, ny, nz) of a gnx x gny x ... grid into h's U
// (ghost cells zero).
int init_kh_block(mhdgb_solver* h, int gnx, int gny, int i0, int j0, int k0, const KhParams& kp) {
  int rc = set_device(h);
  if (rc || (rc = settle(h))) return rc;
  const Layout& L = h->L;
  CK(h, cudaMemsetAsync(h->U, 0, L.count(NCONS) * sizeof(double), h->stream));
  const long long n = (long long)L.nx * L.ny * L.nz;
  const unsigned g = (unsigned)std::min<long long>((n + 255) / 256, (long long)h->nsm * 16);
  k_init_kh<<<g, 256, 0, h->stream>>>(h->U, L, h->faces, h->faces + L.itot, gnx, gny, i0, j0, k0, kh_key(kp.seed),
                                      h->cfg.gam, kp.vshear, kp.width, kp.bx, kp.amp, kp.sig, kp.noise);
  CK(h, cudaGetLastError());
  CK(h, cudaStreamSynchronize(h->stream));
  h->have_state = true;
  h->prepared = false;
  h->p64_valid = h->p_user;
  return MHDGB_OK;
}
}  // namespace

extern "C" {

int mhdgb_init_kh(mhdgb_solver* h, unsigned long long seed, double vshear, double width, double bx, double amp,
                  double sig, double noise) {
  if (!h) return MHDGB_ERR_ARG;
  return init_kh_block(h, h->L.nx, h->L.ny, 0, 0, 0, KhParams{seed, vshear, width, bx, amp, sig, noise});
}

int mhdgb_init_kh_block(mhdgb_solver* h, const int whole[3], const int offset[3], unsigned long long seed,
                        double vshear, double width, double bx, double amp, double sig, double noise) {
  if (!h || !whole || !offset) return MHDGB_ERR_ARG;
  if (offset[0] < 0 || offset[1] < 0 || offset[2] < 0 || offset[0] + h->L.nx > whole[0] ||
      offset[1] + h->L.ny > whole[1] || offset[2] + h->L.nz > whole[2])
    return fail(h, MHDGB_ERR_ARG, "block does not lie inside the whole grid");
  return init_kh_block(h, whole[0], whole[1], offset[0], offset[1], offset[2],
                       KhParams{seed, vshear, width, bx, amp, sig, noise});
}

int mhdgb_selftest_fused_abort(int device, int precision, double* seconds, unsigned* status, int* recovered) {
  if (!seconds || !status || !recovered) return MHDGB_ERR_ARG;
  if (precision < MHDGB_FP64 || precision > MHDGB_MIXED) return MHDGB_ERR_ARG;
  mhdgb_config cfg;
  mhdgb_config_default(&cfg);
  cfg.nx = 32; cfg.ny = 24; cfg.nz = 16;
  cfg.precision = precision;
  cfg.device = device;
  mhdgb_solver *h = nullptr, *ref = nullptr;
  int rc = mhdgb_create(&cfg, &h);
  if (rc) return rc;
  if ((rc = mhdgb_create(&cfg, &ref))) { mhdgb_destroy(h); return rc; }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  auto done = [&](int code) {
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    mhdgb_destroy(h);
    mhdgb_destroy(ref);
    return code;
  };
  auto init = [](mhdgb_solver* s) { return mhdgb_init_kh(s, 1, 0.5, 0.05, 0.1, 1e-2, 0.2, 1e-4); };
  if ((rc = init(h)) || (rc = mhdgb_prepare(h))) return done(rc);
  // one step whose first plane load per work item expects 16 bytes more than the plane: every CTA
  // with a work item waits for that plane until the bounded wait gives up, then drains and returns
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) return done(MHDGB_ERR_CUDA);
  k_set_tx_extra<<<1, 1, 0, h->stream>>>(h->d_desc, 16u);
  if (cudaGetLastError() != cudaSuccess || cudaEventRecord(e0, h->stream) != cudaSuccess) return done(MHDGB_ERR_CUDA);
  if ((rc = launch_one(h))) return done(rc);
  if (cudaEventRecord(e1, h->stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess)
    return done(MHDGB_ERR_CUDA);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, e0, e1);
  Ctrl c;
  if ((rc = read_ctrl(h, &c))) return done(rc);
  *seconds = ms * 1e-3;
  *status = c.status;
  // the same handle then runs two ordinary steps from a fresh state, which must equal a handle that
  // never saw the aborted launch bit for bit
  k_set_tx_extra<<<1, 1, 0, h->stream>>>(h->d_desc, 0u);
  if (cudaGetLastError() != cudaSuccess) return done(MHDGB_ERR_CUDA);
  if ((rc = mhdgb_reset_clock(h)) || (rc = init(h)) || (rc = mhdgb_step(h, 2))) return done(rc);
  const int sync_rc = mhdgb_sync(h, nullptr);
  if ((rc = init(ref)) || (rc = mhdgb_step(ref, 2)) || (rc = mhdgb_sync(ref, nullptr))) return done(rc);
  const size_t n = (size_t)NCONS * h->L.itot * h->L.jtot * h->L.ktot;
  std::vector<double> a(n), b(n);
  if ((rc = mhdgb_download_cons(h, a.data())) || (rc = mhdgb_download_cons(ref, b.data()))) return done(rc);
  *recovered = sync_rc == MHDGB_OK && std::memcmp(a.data(), b.data(), n * sizeof(double)) == 0;
  return done(MHDGB_OK);
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------
// Ensemble: many independent grids (uneven sizes, own parameters) advanced together, one persistent
// launch of the fused kernel per step walking all grids' work items.
// ---------------------------------------------------------------------------------------------
struct mhdgb_ensemble {
  int device = 0;
  FusedKind kind = FUSED_FP64;
  cudaStream_t stream = nullptr;
  int nsm = 0;
  std::vector<mhdgb_solver*> m;
  const FusedVariant* vars = nullptr;
  int nvars = 0, vidx = 0, grid = 0;   // vidx: the HLLD tile variant selected
  int active = 0;                      // the kernel launched: vidx, or nvars (run-time solver) when
                                       // a member uses HLLE/HLLC
  // Planes per work item (at most; a grid's z is cut into equal chunks).  A chunk's start costs
  // about half a plane (the ring's prologue, the lower z faces), so long items pay: on the 64-grid
  // KH ensemble 8 planes gave 6.41 Gcell/s mixed and 0.361 FP64, 24 gave 7.03 / 0.380, 64 gave
  // 7.19 / 0.381, flat from 32 on.  The queue takes the grids with the longest items first, so it
  // ends on short ones.
  int kc = 64;
  InstanceDesc* d_desc = nullptr;
  LaunchCtrl* d_lc = nullptr;
  int total_items = 0;
  cudaGraphExec_t gexec = nullptr;
  std::vector<unsigned> desc_seen;  // members' desc_version as last copied into d_desc
  std::string err;
};

namespace {

int efail(mhdgb_ensemble* e, int code, const std::string& msg) {
  if (e) e->err = msg;
  return code;
}

#define ECK(e, call)                                                                      \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess) return efail((e), MHDGB_ERR_CUDA, std::string(#call) + ": " + \
                                        cudaGetErrorString(e_));                          \
  } while (0)

int ens_member_rc(mhdgb_ensemble* e, int i, int rc) {
  if (rc) e->err = "member " + std::to_string(i) + ": " + e->m[i]->err;
  return rc;
}

// Use tile shape idx for every member and rebuild the launch's instance table.
bool ens_any_general_solver(const mhdgb_ensemble* e) {
  for (const auto* h : e->m)
    if (h->riemann != MHDGB_RIEMANN_HLLD) return true;
  return false;
}

int ens_use_variant(mhdgb_ensemble* e, int idx) {
  if (idx < 0 || idx >= e->nvars) return efail(e, MHDGB_ERR_ARG, "no such variant");
  const int eff = ens_any_general_solver(e) ? e->nvars : idx;
  for (size_t i = 0; i < e->m.size(); i++) {
    const bool was = e->m[i]->prepared;
    int rc = use_variant(e->m[i], eff, e->kc);
    if (rc) return ens_member_rc(e, (int)i, rc);
    e->m[i]->prepared = was;
  }
  // queue order: the grids with the longest items (first chunk, in planes) first
  std::vector<size_t> order(e->m.size());
  std::iota(order.begin(), order.end(), size_t(0));
  std::stable_sort(order.begin(), order.end(),
                   [&](size_t x, size_t y) { return e->m[x]->kst[1] > e->m[y]->kst[1]; });
  std::vector<InstanceDesc> d;
  d.reserve(e->m.size());
  int begin = 0;
  for (size_t i : order) {
    d.push_back(host_desc(e->m[i], begin));
    begin += d.back().nitems;
  }
  e->desc_seen.resize(e->m.size());
  for (size_t i = 0; i < e->m.size(); i++) e->desc_seen[i] = e->m[i]->desc_version;
  e->vidx = idx;
  e->active = eff;
  e->total_items = begin;
  e->grid = e->m[0]->grid;
  const LaunchCtrl lc{0u, 0u, (unsigned)e->m.size(), (unsigned)begin};
  ECK(e, cudaMemcpyAsync(e->d_desc, d.data(), d.size() * sizeof(InstanceDesc), cudaMemcpyHostToDevice, e->stream));
  ECK(e, cudaMemcpyAsync(e->d_lc, &lc, sizeof(lc), cudaMemcpyHostToDevice, e->stream));
  ECK(e, cudaStreamSynchronize(e->stream));
  if (e->gexec) cudaGraphExecDestroy(e->gexec);
  e->gexec = nullptr;
  return MHDGB_OK;
}

int ens_launch(mhdgb_ensemble* e) {
  ECK(e, e->vars[e->active].launch(e->d_desc, e->d_lc, e->grid, e->stream));
  return MHDGB_OK;
}

int ens_prepare_all(mhdgb_ensemble* e, bool force) {
  // a member whose arguments changed (mhdgb_set_physics, mhdgb_set_riemann) since the ensemble's
  // descriptors were built: rebuild them all
  for (size_t i = 0; i < e->m.size(); i++)
    if (i >= e->desc_seen.size() || e->desc_seen[i] != e->m[i]->desc_version) {
      int rc = ens_use_variant(e, e->vidx);
      if (rc) return rc;
      break;
    }
  for (size_t i = 0; i < e->m.size(); i++) {
    if (!force && e->m[i]->prepared) continue;
    int rc = mhdgb_prepare(e->m[i]);
    if (rc) return ens_member_rc(e, (int)i, rc);
  }
  return MHDGB_OK;
}

}  // namespace

extern "C" {

int mhdgb_ensemble_create(int n, const mhdgb_config* cfgs, mhdgb_ensemble** out) {
  if (n < 1 || !cfgs || !out) return MHDGB_ERR_ARG;
  *out = nullptr;
  for (int i = 1; i < n; i++)
    if (cfgs[i].precision != cfgs[0].precision || cfgs[i].device != cfgs[0].device) return MHDGB_ERR_ARG;
  mhdgb_ensemble* e = new mhdgb_ensemble();
  e->device = cfgs[0].device;
  if (cudaSetDevice(e->device) != cudaSuccess) { delete e; return MHDGB_ERR_CUDA; }
  if (cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) != cudaSuccess) { delete e; return MHDGB_ERR_CUDA; }
  cudaDeviceGetAttribute(&e->nsm, cudaDevAttrMultiProcessorCount, e->device);
  for (int i = 0; i < n; i++) {
    mhdgb_solver* h = nullptr;
    int rc = create_impl(&cfgs[i], e->stream, &h);
    if (rc) { mhdgb_ensemble_destroy(e); return rc; }
    e->m.push_back(h);
  }
  e->kind = e->m[0]->kind;
  e->vars = e->m[0]->vars;
  e->nvars = e->m[0]->nvars;
  if (cudaMalloc(&e->d_desc, n * sizeof(InstanceDesc)) != cudaSuccess ||
      cudaMalloc(&e->d_lc, sizeof(LaunchCtrl)) != cudaSuccess) {
    mhdgb_ensemble_destroy(e);
    return MHDGB_ERR_NOMEM;
  }
  const int pref = fused_preferred_variant(e->kind);
  int rc = ens_use_variant(e, pref < e->nvars ? pref : 0);
  if (rc && pref != 0) rc = ens_use_variant(e, 0);
  if (rc) { mhdgb_ensemble_destroy(e); return rc; }
  *out = e;
  return MHDGB_OK;
}

int mhdgb_ensemble_destroy(mhdgb_ensemble* e) {
  if (!e) return MHDGB_OK;
  cudaSetDevice(e->device);
  if (e->stream) cudaStreamSynchronize(e->stream);
  if (e->gexec) cudaGraphExecDestroy(e->gexec);
  for (auto* h : e->m) mhdgb_destroy(h);
  if (e->d_desc) cudaFree(e->d_desc);
  if (e->d_lc) cudaFree(e->d_lc);
  if (e->stream) cudaStreamDestroy(e->stream);
  delete e;
  return MHDGB_OK;
}

const char* mhdgb_ensemble_last_error(const mhdgb_ensemble* e) { return e ? e->err.c_str() : "null ensemble"; }

int mhdgb_ensemble_size(const mhdgb_ensemble* e) { return e ? (int)e->m.size() : 0; }

int mhdgb_ensemble_member(mhdgb_ensemble* e, int i, mhdgb_solver** h) {
  if (!e || !h || i < 0 || i >= (int)e->m.size()) return MHDGB_ERR_ARG;
  *h = e->m[i];
  return MHDGB_OK;
}

long long mhdgb_ensemble_cells(const mhdgb_ensemble* e) {
  long long c = 0;
  if (e)
    for (auto* h : e->m) c += (long long)h->L.nx * h->L.ny * h->L.nz;
  return c;
}

int mhdgb_ensemble_select_variant(mhdgb_ensemble* e, int idx) {
  if (!e) return MHDGB_ERR_ARG;
  if (cudaSetDevice(e->device) != cudaSuccess) return MHDGB_ERR_CUDA;
  ECK(e, cudaStreamSynchronize(e->stream));
  return ens_use_variant(e, idx);
}

int mhdgb_ensemble_variant(const mhdgb_ensemble* e) { return e ? e->vidx : -1; }

int mhdgb_ensemble_prepare(mhdgb_ensemble* e) {
  if (!e) return MHDGB_ERR_ARG;
  if (cudaSetDevice(e->device) != cudaSuccess) return MHDGB_ERR_CUDA;
  return ens_prepare_all(e, true);
}

int mhdgb_ensemble_step(mhdgb_ensemble* e, int nsteps) {
  if (!e || nsteps < 0) return MHDGB_ERR_ARG;
  if (cudaSetDevice(e->device) != cudaSuccess) return MHDGB_ERR_CUDA;
  int rc = ens_prepare_all(e, false);
  if (rc) return rc;
  const int G = 16;
  if (nsteps >= G && !e->gexec) {
    cudaGraph_t g = nullptr;
    ECK(e, cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
    for (int s = 0; s < G && rc == MHDGB_OK; s++) rc = ens_launch(e);
    cudaError_t ce = cudaStreamEndCapture(e->stream, &g);
    if (rc) { if (g) cudaGraphDestroy(g); return rc; }
    if (ce != cudaSuccess) return efail(e, MHDGB_ERR_CUDA, "cudaStreamEndCapture");
    ce = cudaGraphInstantiate(&e->gexec, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) return efail(e, MHDGB_ERR_CUDA, "cudaGraphInstantiate");
  }
  while (nsteps >= G) {
    ECK(e, cudaGraphLaunch(e->gexec, e->stream));
    nsteps -= G;
  }
  for (; nsteps > 0; nsteps--)
    if ((rc = ens_launch(e))) return rc;
  for (auto* h : e->m) { h->p64_valid = false; h->p_user = false; }
  return MHDGB_OK;
}

int mhdgb_ensemble_sync(mhdgb_ensemble* e, mhdgb_report* reports) {
  if (!e) return MHDGB_ERR_ARG;
  if (cudaSetDevice(e->device) != cudaSuccess) return MHDGB_ERR_CUDA;
  int first = MHDGB_OK;
  for (size_t i = 0; i < e->m.size(); i++) {
    const int rc = mhdgb_sync(e->m[i], reports ? &reports[i] : nullptr);
    if (rc && first == MHDGB_OK) first = ens_member_rc(e, (int)i, rc);
  }
  return first;
}

int mhdgb_ensemble_set_stop(mhdgb_ensemble* e, double tmax, long long max_steps) {
  if (!e) return MHDGB_ERR_ARG;
  for (size_t i = 0; i < e->m.size(); i++) {
    const int rc = mhdgb_set_stop(e->m[i], tmax, max_steps);
    if (rc) return ens_member_rc(e, (int)i, rc);
  }
  return MHDGB_OK;
}

int mhdgb_ensemble_time_steps(mhdgb_ensemble* e, int nsteps, double* ms) {
  if (!e || nsteps < 1 || !ms) return MHDGB_ERR_ARG;
  if (cudaSetDevice(e->device) != cudaSuccess) return MHDGB_ERR_CUDA;
  int rc = ens_prepare_all(e, false);
  if (rc) return rc;
  if (nsteps >= 16 && !e->gexec && (rc = mhdgb_ensemble_step(e, 0))) return rc;
  cudaEvent_t e0, e1;
  ECK(e, cudaEventCreate(&e0));
  ECK(e, cudaEventCreate(&e1));
  ECK(e, cudaStreamSynchronize(e->stream));
  ECK(e, cudaEventRecord(e0, e->stream));
  rc = mhdgb_ensemble_step(e, nsteps);
  ECK(e, cudaEventRecord(e1, e->stream));
  ECK(e, cudaEventSynchronize(e1));
  float t = 0.0f;
  ECK(e, cudaEventElapsedTime(&t, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms = t;
  return rc;
}

int mhdgb_ensemble_autotune(mhdgb_ensemble* e, int steps, int* best) {
  if (!e || steps < 1) return MHDGB_ERR_ARG;
  if (cudaSetDevice(e->device) != cudaSuccess) return MHDGB_ERR_CUDA;
  if (ens_any_general_solver(e)) {  // HLLE/HLLC members: the one run-time solver kernel runs all
    if (best) *best = e->vidx;
    return MHDGB_OK;
  }
  // keep every member's U and control block, time each tile shape, restore
  std::vector<Ctrl> saved(e->m.size());
  for (size_t i = 0; i < e->m.size(); i++) {
    mhdgb_solver* h = e->m[i];
    if (!h->have_state) return efail(e, MHDGB_ERR_STATE, "autotune needs every member's state");
    int rc = read_ctrl(h, &saved[i]);
    if (rc) return ens_member_rc(e, (int)i, rc);
    double* st = staging(h);
    if (!st) return efail(e, MHDGB_ERR_NOMEM, "staging buffer");
    k_repack<<<h->nsm * 8, 256, 0, e->stream>>>(h->U, st, h->L.itot, h->L.ip,
                                                 (size_t)NCONS * h->L.jtot * h->L.ktot, 0);
    ECK(e, cudaGetLastError());
  }
  auto restore = [&]() -> int {
    for (size_t i = 0; i < e->m.size(); i++) {
      mhdgb_solver* h = e->m[i];
      k_repack<<<h->nsm * 8, 256, 0, e->stream>>>(h->stage, h->U, h->L.itot, h->L.ip,
                                                   (size_t)NCONS * h->L.jtot * h->L.ktot, 1);
      ECK(e, cudaGetLastError());
      ECK(e, cudaMemcpyAsync(h->ctrl, &saved[i], sizeof(Ctrl), cudaMemcpyHostToDevice, e->stream));
      h->cur_step = (long long)saved[i].step;
      h->prepared = false;
      h->p64_valid = false;
    }
    ECK(e, cudaStreamSynchronize(e->stream));
    return MHDGB_OK;
  };
  double best_ms = 1e300;
  int bidx = e->vidx, rc;
  for (int v = 0; v < e->nvars; v++) {
    if ((rc = ens_use_variant(e, v)) || (rc = restore())) return rc;
    double ms = 0.0;
    if ((rc = mhdgb_ensemble_time_steps(e, 2, &ms)) || (rc = mhdgb_ensemble_time_steps(e, steps, &ms))) return rc;
    if (ms < best_ms) { best_ms = ms; bidx = v; }
  }
  if ((rc = ens_use_variant(e, bidx)) || (rc = restore())) return rc;
  if (best) *best = bidx;
  return MHDGB_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------
// Snapshot output (Output, src_cpp_kokkos_host/output.cpp:379-407)
// ---------------------------------------------------------------------------------------------
namespace {

int join_writer(mhdgb_solver* h) {
  if (!h->writer.joinable()) return MHDGB_OK;
  h->writer.join();
  if (h->writer_rc) return fail(h, h->writer_rc, h->writer_err);
  return MHDGB_OK;
}

int ensure_snapshot_bufs(mhdgb_solver* h) {
  const size_t n = (size_t)NSNAP * h->L.nx * h->L.ny * h->L.nz;
  if (!h->d_snap && dalloc(h, &h->d_snap, n) != cudaSuccess) return fail(h, MHDGB_ERR_NOMEM, "snapshot buffer");
  if (!h->h_snap && cudaMallocHost((void**)&h->h_snap, n * sizeof(double)) != cudaSuccess) {
    h->h_snap = nullptr;
    return fail(h, MHDGB_ERR_NOMEM, "pinned snapshot buffer");
  }
  if (!h->copy_stream) CK(h, cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
  if (!h->ev_packed) CK(h, cudaEventCreateWithFlags(&h->ev_packed, cudaEventDisableTiming));
  if (!h->ev_copied) CK(h, cudaEventCreateWithFlags(&h->ev_copied, cudaEventDisableTiming));
  return MHDGB_OK;
}

}  // namespace

extern "C" {

int mhdgb_output_begin(mhdgb_solver* h, const char* root, int index, double time, double dt, int ascii) {
  if (!h || index < 0 || index > 99999) return MHDGB_ERR_ARG;
  int rc = set_device(h);
  if (rc || (rc = join_writer(h))) return rc;
  if (!h->have_state && !h->p_user) return fail(h, MHDGB_ERR_STATE, "no state uploaded");
  if ((rc = ensure_snapshot_bufs(h))) return rc;
  // A primitive array the caller uploaded is written as it is (the reference writes its P, which
  // for the initial state is GenerateProblem's), and so is the FP64 fused step's own recovery once
  // the handle steps fused (the P that mhdgb_download_prim returns; the parity of the current
  // buffer is known after the steps already enqueued have run); otherwise the primitives are
  // recovered from U in stream order, after every step already enqueued.
  const double* P = nullptr;
  if (h->p_user) {
    P = h->P64[cur_index(h)];
  } else if (h->prepared && h->kind != FUSED_MIXED) {
    if ((rc = settle(h))) return rc;
    P = h->P64[cur_index(h)];
  }
  CK(h, launch_snapshot(h->U, P, h->L, h->cfg.gam, h->d_snap, h->stream));
  CK(h, cudaEventRecord(h->ev_packed, h->stream));
  CK(h, cudaStreamWaitEvent(h->copy_stream, h->ev_packed, 0));
  const size_t bytes = (size_t)NSNAP * h->L.nx * h->L.ny * h->L.nz * sizeof(double);
  CK(h, cudaMemcpyAsync(h->h_snap, h->d_snap, bytes, cudaMemcpyDeviceToHost, h->copy_stream));
  CK(h, cudaEventRecord(h->ev_copied, h->copy_stream));
  SnapshotMeta m;
  m.root = root ? root : ".";
  m.index = index;
  m.time = time;
  m.dt = dt;
  m.ascii = ascii != 0;
  m.nx = h->L.nx; m.ny = h->L.ny; m.nz = h->L.nz;
  m.x1a = h->x1a; m.x2a = h->x2a; m.x3a = h->x3a;
  h->writer_rc = MHDGB_OK;
  h->writer_err.clear();
  h->writer = std::thread([h, m = std::move(m)]() {
    cudaSetDevice(h->cfg.device);
    const cudaError_t e = cudaEventSynchronize(h->ev_copied);
    if (e != cudaSuccess) {
      h->writer_rc = MHDGB_ERR_CUDA;
      h->writer_err = std::string("snapshot copy: ") + cudaGetErrorString(e);
      return;
    }
    std::string err;
    if (write_snapshot_files(m, h->h_snap, &err)) {
      h->writer_rc = MHDGB_ERR_IO;
      h->writer_err = err;
    }
  });
  return MHDGB_OK;
}

int mhdgb_output_end(mhdgb_solver* h) {
  if (!h) return MHDGB_ERR_ARG;
  return join_writer(h);
}

int mhdgb_output(mhdgb_solver* h, const char* root, int index, double time, double dt, int ascii) {
  const int rc = mhdgb_output_begin(h, root, index, time, dt, ascii);
  return rc ? rc : mhdgb_output_end(h);
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------
// Checkpoint / restart (the reference has none).  File layout, little endian:
//   char[8] "MHDGBCK1" | int32 version, nx, ny, nz, precision, spacing_quirk, bc[6], riemann |
//   float64 x1min, x1max, x2min, x2max, x3min, x3max, gam, cfl |
//   int64 step | uint64 max_step | float64 time, last_dt, last_ch, tmax |
//   float64 x1a[itot], x2a[jtot], x3a[ktot] | float64 U[ktot][jtot][10][itot] (FieldArray layout)
// ---------------------------------------------------------------------------------------------
namespace {
constexpr char kCkMagic[8] = {'M', 'H', 'D', 'G', 'B', 'C', 'K', '1'};
constexpr int kCkVersion = 2;

struct CkHead {
  int32_t ints[13];   // version, nx, ny, nz, precision, spacing_quirk, bc[6], riemann
  double reals[8];    // domain, gam, cfl
  int64_t step;
  uint64_t max_step;
  double clock[4];    // time, last_dt, last_ch, tmax
};

bool wr(FILE* f, const void* p, size_t n) { return std::fwrite(p, 1, n, f) == n; }
bool rd(FILE* f, void* p, size_t n) { return std::fread(p, 1, n, f) == n; }
}  // namespace

extern "C" {

int mhdgb_checkpoint_save(mhdgb_solver* h, const char* path) {
  if (!h || !path) return MHDGB_ERR_ARG;
  int rc = set_device(h);
  if (rc || (rc = settle(h))) return rc;
  if (!h->have_state) return fail(h, MHDGB_ERR_STATE, "no state to checkpoint");
  Ctrl c;
  if ((rc = read_ctrl(h, &c))) return rc;
  const Layout& L = h->L;
  std::vector<double> U((size_t)NCONS * L.itot * L.jtot * L.ktot);
  if ((rc = download_u(h, U.data()))) return rc;
  CK(h, cudaStreamSynchronize(h->stream));
  CkHead hd{};
  const mhdgb_config& g = h->cfg;
  const int32_t ints[13] = {kCkVersion, g.nx, g.ny, g.nz, g.precision, g.spacing_quirk,
                            g.bc[0], g.bc[1], g.bc[2], g.bc[3], g.bc[4], g.bc[5], h->riemann};
  std::copy(ints, ints + 13, hd.ints);
  const double reals[8] = {g.x1min, g.x1max, g.x2min, g.x2max, g.x3min, g.x3max, g.gam, g.cfl};
  std::copy(reals, reals + 8, hd.reals);
  hd.step = (int64_t)c.step;
  hd.max_step = c.max_step;
  hd.clock[0] = c.time; hd.clock[1] = c.last_dt; hd.clock[2] = c.last_ch; hd.clock[3] = c.tmax;
  FILE* f = std::fopen(path, "wb");
  if (!f) return fail(h, MHDGB_ERR_IO, std::string("cannot create ") + path);
  bool ok = wr(f, kCkMagic, 8) && wr(f, hd.ints, sizeof(hd.ints)) && wr(f, hd.reals, sizeof(hd.reals)) &&
            wr(f, &hd.step, 8) && wr(f, &hd.max_step, 8) && wr(f, hd.clock, sizeof(hd.clock)) &&
            wr(f, h->x1a.data(), 8 * h->x1a.size()) && wr(f, h->x2a.data(), 8 * h->x2a.size()) &&
            wr(f, h->x3a.data(), 8 * h->x3a.size()) && wr(f, U.data(), 8 * U.size());
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) return fail(h, MHDGB_ERR_IO, std::string("cannot write ") + path);
  return MHDGB_OK;
}

int mhdgb_checkpoint_load(mhdgb_solver* h, const char* path) {
  if (!h || !path) return MHDGB_ERR_ARG;
  int rc = set_device(h);
  if (rc || (rc = settle(h))) return rc;
  FILE* f = std::fopen(path, "rb");
  if (!f) return fail(h, MHDGB_ERR_IO, std::string("cannot open ") + path);
  char magic[8];
  CkHead hd{};
  bool ok = rd(f, magic, 8) && std::equal(magic, magic + 8, kCkMagic) && rd(f, hd.ints, sizeof(hd.ints)) &&
            rd(f, hd.reals, sizeof(hd.reals)) && rd(f, &hd.step, 8) && rd(f, &hd.max_step, 8) &&
            rd(f, hd.clock, sizeof(hd.clock)) && hd.ints[0] == kCkVersion;
  if (!ok) {
    std::fclose(f);
    return fail(h, MHDGB_ERR_ARG, std::string(path) + " is not a checkpoint of this library");
  }
  const mhdgb_config& g = h->cfg;
  if (hd.ints[1] != g.nx || hd.ints[2] != g.ny || hd.ints[3] != g.nz || hd.ints[5] != g.spacing_quirk) {
    std::fclose(f);
    return fail(h, MHDGB_ERR_ARG, "checkpoint grid " + std::to_string(hd.ints[1]) + "x" + std::to_string(hd.ints[2]) +
                                      "x" + std::to_string(hd.ints[3]) + " (or its spacing_quirk) differs from the handle's");
  }
  const Layout& L = h->L;
  std::vector<double> x1a(L.itot), x2a(L.jtot), x3a(L.ktot), U((size_t)NCONS * L.itot * L.jtot * L.ktot);
  ok = rd(f, x1a.data(), 8 * x1a.size()) && rd(f, x2a.data(), 8 * x2a.size()) && rd(f, x3a.data(), 8 * x3a.size()) &&
       rd(f, U.data(), 8 * U.size());
  std::fclose(f);
  if (!ok) return fail(h, MHDGB_ERR_IO, std::string(path) + " is truncated");
  const int bc[6] = {hd.ints[6], hd.ints[7], hd.ints[8], hd.ints[9], hd.ints[10], hd.ints[11]};
  if ((rc = mhdgb_set_physics(h, hd.reals[6], hd.reals[7], bc))) return rc;
  if ((rc = mhdgb_set_riemann(h, hd.ints[12]))) return rc;
  h->cfg.x1min = hd.reals[0]; h->cfg.x1max = hd.reals[1];
  h->cfg.x2min = hd.reals[2]; h->cfg.x2max = hd.reals[3];
  h->cfg.x3min = hd.reals[4]; h->cfg.x3max = hd.reals[5];
  if ((rc = mhdgb_set_grid(h, x1a.data(), x2a.data(), x3a.data()))) return rc;
  if ((rc = upload_u(h, U.data()))) return rc;
  k_ctrl_restore<<<1, 1, 0, h->stream>>>(h->ctrl, (unsigned long long)hd.step, hd.clock[0], hd.clock[1], hd.clock[2],
                                          hd.clock[3], hd.max_step);
  CK(h, cudaGetLastError());
  CK(h, cudaStreamSynchronize(h->stream));
  h->cur_step = (long long)hd.step;
  h->have_state = true;
  h->prepared = false;
  h->p64_valid = false;
  h->p_user = false;
  return MHDGB_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------
// Block decomposition.  The reference splits the grid over MPI ranks with MPI_Cart_create
// (mpi_config.cpp:61-69), swaps 2-deep primitive halos with its neighbours inside SendRecvBoundary
// (boundary.cpp:222-318, 430-475, 627-672) and reduces dt and c_h with MPI_MINLOC / MPI_MAXLOC
// allreduces (mpi_config.cpp:83-99).  Here a block is an ordinary handle whose shared faces have
// the kind MHDGB_BC_EXCHANGE (no local fill writes their ghosts).  Two ways to drive blocks:
//   * per handle (one process per GPU, any transport): mhdgb_halo_pack / _unpack move a face's
//     2-deep slab between the handle's primitives and a contiguous buffer, and
//     mhdgb_get_reduction / _set_reduction read and replace the pending dt / c_h reduction;
//   * a domain (one process, one or more GPUs): the blocks of each group advance in one persistent
//     launch of the fused kernel, then one kernel per group copies every exchanged halo straight
//     from the neighbouring block's primitives (a peer read over NVLink when the neighbour is on
//     another GPU; no staging buffer), and one thread reduces dt and c_h over all blocks into the
//     group's own control blocks.  Nothing leaves the devices between steps.
// Only the interior transverse extent of a face is exchanged: the solver never reads the edge and
// corner ghosts that the reference's full-extent buffers also carry.
// ---------------------------------------------------------------------------------------------
namespace {

// The 2-deep box of face f (0..5 = x-in, x-out, y-in, y-out, z-in, z-out) in the reference index
// space: the interior layers next to the face (ghost = false) or the ghost layers beyond it.
struct FaceBox {
  int lo[3], n[3];  // start and count along i, j, k
};

__host__ __device__ inline FaceBox face_box(const Layout& L, int face, bool ghost) {
  FaceBox b{{NGH, NGH, NGH}, {L.nx, L.ny, L.nz}};
  const int ax = face >> 1, hi = face & 1;
  b.lo[ax] = ghost ? (hi ? NGH + b.n[ax] : 0) : (hi ? NGH + b.n[ax] - 2 : NGH);
  b.n[ax] = 2;
  return b;
}

__host__ __device__ inline long long box_count(const FaceBox& b) {
  return (long long)NPRIM * b.n[0] * b.n[1] * b.n[2];
}

// Element e of a box (i fastest, then j, k, variable) as an offset into a primitive array.
__host__ __device__ inline size_t box_at(const Layout& L, const FaceBox& b, long long e) {
  const int i = (int)(e % b.n[0]);
  const int j = (int)((e / b.n[0]) % b.n[1]);
  const int k = (int)((e / ((long long)b.n[0] * b.n[1])) % b.n[2]);
  const int n = (int)(e / ((long long)b.n[0] * b.n[1] * b.n[2]));
  return L.at(NPRIM, n, b.lo[2] + k, b.lo[1] + j, b.lo[0] + i);
}

// Face slab <-> contiguous buffer (box order).
template <class R>
__global__ void k_halo_copy(R* __restrict__ P, Layout L, FaceBox b, R* __restrict__ buf, int to_buf) {
  const long long n = box_count(b);
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const size_t o = box_at(L, b, e);
    if (to_buf) buf[e] = P[o];
    else P[o] = buf[e];
  }
}

// One exchanged face of a domain: the source block's interior slab goes to the destination block's
// ghost layers, in the primitive buffer of the current step's parity.
struct HaloXfer {
  const void* src[2];
  void* dst[2];
  Layout Ls, Ld;
  FaceBox bs, bd;
  const Ctrl* ctrl;   // the destination's control block (its step selects the parity)
  long long begin;    // first element of this transfer in the launch's element range
};

template <class R>
__global__ void k_halo_exchange(const HaloXfer* __restrict__ x, int nx, long long total) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    int t = 0;
    for (int lo = 0, hi = nx - 1; lo <= hi;) {
      const int mid = (lo + hi) >> 1;
      if (x[mid].begin <= e) { t = mid; lo = mid + 1; } else hi = mid - 1;
    }
    const HaloXfer& q = x[t];
    const int par = (int)(q.ctrl->step & 1);
    const long long r = e - q.begin;
    static_cast<R*>(q.dst[par])[box_at(q.Ld, q.bd, r)] = static_cast<const R*>(q.src[par])[box_at(q.Ls, q.bs, r)];
  }
}

// dt / c_h over all blocks of a domain, written into the pending slot of this group's blocks.  The
// pending slot of a block is slot[step % 3]: the one its next fused step takes dt and c_h from.
__global__ void k_domain_reduce(Ctrl* const* __restrict__ all, int nall, Ctrl* const* __restrict__ own, int nown) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  unsigned long long dtmin = DT_RESET, chmax = CH_RESET;
  for (int q = 0; q < nall; q++) {
    const Ctrl* c = all[q];
    const RedSlot s = c->slot[c->step % 3];
    dtmin = s.dtmin_bits < dtmin ? s.dtmin_bits : dtmin;
    chmax = s.chmax_bits > chmax ? s.chmax_bits : chmax;
  }
  for (int q = 0; q < nown; q++) {
    Ctrl* c = own[q];
    c->slot[c->step % 3].dtmin_bits = dtmin;
    c->slot[c->step % 3].chmax_bits = chmax;
  }
}

__global__ void k_get_slot(const Ctrl* c, RedSlot* out) { *out = c->slot[c->step % 3]; }
__global__ void k_set_slot(Ctrl* c, RedSlot v) { c->slot[c->step % 3] = v; }

// The primitive array a halo call works on: the fused step's current buffer once the handle is
// prepared for fused steps, else the stage path's FP64 primitives.
int halo_target(mhdgb_solver* h, void** P, int* elem) {
  int rc;
  if ((rc = settle(h))) return rc;
  if (h->prepared) {
    const int c = cur_index(h);
    *P = h->kind == FUSED_MIXED ? (void*)h->P32[c] : (void*)h->P64[c];
    *elem = h->kind == FUSED_MIXED ? 4 : 8;
    return MHDGB_OK;
  }
  if ((rc = ensure_p64(h))) return rc;
  *P = h->P64[cur_index(h)];
  *elem = 8;
  return MHDGB_OK;
}

// The address a kernel reaches buf at: device (or managed) memory as it is, page-locked host
// memory through its device mapping; null for pageable host memory, which no kernel can reach.
void* kernel_view(void* buf) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, buf) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) return buf;
  if (a.type == cudaMemoryTypeHost && a.devicePointer) return a.devicePointer;
  return nullptr;
}

int halo_copy(mhdgb_solver* h, int face, void* buf, int to_buf) {
  if (!h || !buf || face < 0 || face > 5) return MHDGB_ERR_ARG;
  int rc = set_device(h);
  void* P = nullptr;
  int elem = 8;
  if (rc || (rc = halo_target(h, &P, &elem))) return rc;
  buf = kernel_view(buf);
  if (!buf) return fail(h, MHDGB_ERR_ARG, "halo buffer is neither device memory nor page-locked host memory");
  const FaceBox b = face_box(h->L, face, !to_buf);
  const long long n = box_count(b);
  const int bs = 256;
  const unsigned g = (unsigned)std::min<long long>((n + bs - 1) / bs, (long long)h->nsm * 8);
  if (elem == 4) k_halo_copy<float><<<g, bs, 0, h->stream>>>((float*)P, h->L, b, (float*)buf, to_buf);
  else k_halo_copy<double><<<g, bs, 0, h->stream>>>((double*)P, h->L, b, (double*)buf, to_buf);
  CK(h, cudaGetLastError());
  CK(h, cudaStreamSynchronize(h->stream));
  if (!to_buf) h->p_user = false;
  return MHDGB_OK;
}

}  // namespace

extern "C" {

size_t mhdgb_halo_bytes(const mhdgb_solver* h, int face) {
  if (!h || face < 0 || face > 5) return 0;
  const size_t elem = (h->prepared && h->kind == FUSED_MIXED) ? 4 : 8;
  return (size_t)box_count(face_box(h->L, face, false)) * elem;
}

int mhdgb_halo_pack(mhdgb_solver* h, int face, void* buf) { return halo_copy(h, face, buf, 1); }

int mhdgb_halo_unpack(mhdgb_solver* h, int face, const void* buf) {
  return halo_copy(h, face, const_cast<void*>(buf), 0);
}

int mhdgb_get_reduction(mhdgb_solver* h, double* dtmin, double* chmax) {
  if (!h || !dtmin || !chmax) return MHDGB_ERR_ARG;
  int rc = set_device(h);
  if (rc) return rc;
  if (!h->prepared) return fail(h, MHDGB_ERR_STATE, "no pending reduction: call mhdgb_prepare or step first");
  RedSlot* d = h->sslot;  // the stage path's slot doubles as the transfer cell
  k_get_slot<<<1, 1, 0, h->stream>>>(h->ctrl, d);
  CK(h, cudaGetLastError());
  RedSlot v;
  CK(h, cudaMemcpyAsync(&v, d, sizeof(v), cudaMemcpyDeviceToHost, h->stream));
  CK(h, cudaStreamSynchronize(h->stream));
  *dtmin = bitsd(v.dtmin_bits);
  *chmax = bitsd(v.chmax_bits);
  return MHDGB_OK;
}

int mhdgb_set_reduction(mhdgb_solver* h, double dtmin, double chmax) {
  if (!h || !(dtmin >= 0.0) || !(chmax >= 0.0)) return MHDGB_ERR_ARG;
  int rc = set_device(h);
  if (rc) return rc;
  if (!h->prepared) return fail(h, MHDGB_ERR_STATE, "no pending reduction: call mhdgb_prepare or step first");
  k_set_slot<<<1, 1, 0, h->stream>>>(h->ctrl, RedSlot{dbits(dtmin), dbits(chmax)});
  CK(h, cudaGetLastError());
  CK(h, cudaStreamSynchronize(h->stream));
  return MHDGB_OK;
}

}  // extern "C"

// A grid cut into blocks on one or more devices, advanced as one.
struct mhdgb_domain {
  mhdgb_config cfg{};                       // the whole grid
  int nt[3] = {1, 1, 1};                    // blocks per axis
  std::vector<double> x1a, x2a, x3a;        // the whole grid's faces
  std::vector<mhdgb_ensemble*> groups;      // one persistent launch per group and step
  std::vector<int> group_dev;
  std::vector<mhdgb_solver*> blocks;        // block b at coords (b / (nt1*nt2), (b / nt2) % nt1, b % nt2)
  std::vector<int> block_group;
  std::vector<std::array<int, 3>> off, ext; // first interior cell (whole-grid index) and extent
  struct Group {
    HaloXfer* d_xfer = nullptr;
    int nxfer = 0;
    long long total = 0;
    Ctrl** d_all = nullptr;
    Ctrl** d_own = nullptr;
    int nown = 0;
    cudaEvent_t ev_step = nullptr, ev_halo = nullptr;
    cudaGraphExec_t gexec = nullptr;
  };
  std::vector<Group> g;
  bool prepared = false;
  std::string err;
};

namespace {

int dfail(mhdgb_domain* d, int code, const std::string& msg) {
  if (d) d->err = msg;
  return code;
}

#define DCK(d, call)                                                                      \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess) return dfail((d), MHDGB_ERR_CUDA, std::string(#call) + ": " + \
                                        cudaGetErrorString(e_));                          \
  } while (0)

// Cells of block c (of nt) along an axis of n cells: the first n % nt blocks take one more.
void split_axis(int n, int nt, int c, int* off, int* len) {
  const int base = n / nt, rem = n % nt;
  *len = base + (c < rem ? 1 : 0);
  *off = c * base + std::min(c, rem);
}

int block_of(const mhdgb_domain* d, int c0, int c1, int c2) { return (c0 * d->nt[1] + c1) * d->nt[2] + c2; }

// Enqueue the halo copies and the reduction of group q on its stream.
int domain_exchange(mhdgb_domain* d, int q) {
  mhdgb_domain::Group& G = d->g[q];
  mhdgb_ensemble* e = d->groups[q];
  if (G.total > 0) {
    const int bs = 256;
    const unsigned grid = (unsigned)std::min<long long>((G.total + bs - 1) / bs, (long long)e->nsm * 8);
    if (e->kind == FUSED_MIXED) k_halo_exchange<float><<<grid, bs, 0, e->stream>>>(G.d_xfer, G.nxfer, G.total);
    else k_halo_exchange<double><<<grid, bs, 0, e->stream>>>(G.d_xfer, G.nxfer, G.total);
    DCK(d, cudaGetLastError());
  }
  k_domain_reduce<<<1, 32, 0, e->stream>>>(G.d_all, (int)d->blocks.size(), G.d_own, G.nown);
  DCK(d, cudaGetLastError());
  return MHDGB_OK;
}

// One domain step: every group's launch, then (after all launches) every group's exchange.  With
// one group everything is on one stream; with more, events order the groups' streams.
int domain_step_once(mhdgb_domain* d) {
  const int ng = (int)d->groups.size();
  for (int q = 0; q < ng; q++) {
    mhdgb_ensemble* e = d->groups[q];
    DCK(d, cudaSetDevice(e->device));
    if (ng > 1)
      for (int r = 0; r < ng; r++)
        if (r != q) DCK(d, cudaStreamWaitEvent(e->stream, d->g[r].ev_halo, 0));
    int rc = ens_launch(e);
    if (rc) return dfail(d, rc, e->err);
    if (ng > 1) DCK(d, cudaEventRecord(d->g[q].ev_step, e->stream));
  }
  for (int q = 0; q < ng; q++) {
    mhdgb_ensemble* e = d->groups[q];
    DCK(d, cudaSetDevice(e->device));
    if (ng > 1)
      for (int r = 0; r < ng; r++)
        if (r != q) DCK(d, cudaStreamWaitEvent(e->stream, d->g[r].ev_step, 0));
    int rc = domain_exchange(d, q);
    if (rc) return rc;
    if (ng > 1) DCK(d, cudaEventRecord(d->g[q].ev_halo, e->stream));
  }
  return MHDGB_OK;
}

int domain_sync_streams(mhdgb_domain* d) {
  for (auto* e : d->groups) {
    DCK(d, cudaSetDevice(e->device));
    DCK(d, cudaStreamSynchronize(e->stream));
  }
  return MHDGB_OK;
}

int domain_destroy_graphs(mhdgb_domain* d);

// Recover every block's primitives from its U, then exchange the halos and reduce the first dt.
// (A re-prepare may change a group's kernel, e.g. after mhdgb_set_riemann on a block: the captured
// steps are dropped.)
int domain_prepare(mhdgb_domain* d) {
  domain_destroy_graphs(d);
  for (auto* e : d->groups) {
    DCK(d, cudaSetDevice(e->device));
    int rc = ens_prepare_all(e, true);
    if (rc) return dfail(d, rc, e->err);
  }
  const int ng = (int)d->groups.size();
  for (int q = 0; q < ng; q++) {
    mhdgb_ensemble* e = d->groups[q];
    DCK(d, cudaSetDevice(e->device));
    int rc = domain_exchange(d, q);
    if (rc) return rc;
    if (ng > 1) DCK(d, cudaEventRecord(d->g[q].ev_halo, e->stream));
  }
  int rc = domain_sync_streams(d);
  if (rc) return rc;
  d->prepared = true;
  return MHDGB_OK;
}

int domain_destroy_graphs(mhdgb_domain* d) {
  for (auto& G : d->g)
    if (G.gexec) { cudaGraphExecDestroy(G.gexec); G.gexec = nullptr; }
  return MHDGB_OK;
}

}  // namespace

extern "C" {

int mhdgb_domain_create(const mhdgb_config* cfg, const int ntiles[3], int ngroups, const int* devices,
                        mhdgb_domain** out) {
  if (!cfg || !ntiles || !out) return MHDGB_ERR_ARG;
  *out = nullptr;
  for (int a = 0; a < 3; a++)
    if (ntiles[a] < 1) return MHDGB_ERR_ARG;
  const int nb = ntiles[0] * ntiles[1] * ntiles[2];
  if (cfg->nx / ntiles[0] < 2 || cfg->ny / ntiles[1] < 2 || cfg->nz / ntiles[2] < 2) return MHDGB_ERR_ARG;
  for (int q = 0; q < 6; q++)
    if (cfg->bc[q] < MHDGB_BC_PERIODIC || cfg->bc[q] > MHDGB_BC_OUTFLOW) return MHDGB_ERR_ARG;
  if (cfg->spacing_quirk) return MHDGB_ERR_ARG;  // index-i spacings do not survive a split
  if (ngroups < 0 || (ngroups > 0 && !devices) || ngroups > nb) return MHDGB_ERR_ARG;
  if (ngroups == 0) ngroups = 1;
  mhdgb_domain* d = new mhdgb_domain();
  d->cfg = *cfg;
  for (int a = 0; a < 3; a++) d->nt[a] = ntiles[a];
  d->x1a = face_axis(cfg->nx, cfg->x1min, cfg->x1max);
  d->x2a = face_axis(cfg->ny, cfg->x2min, cfg->x2max);
  d->x3a = face_axis(cfg->nz, cfg->x3min, cfg->x3max);
  const int n[3] = {cfg->nx, cfg->ny, cfg->nz};
  // block configurations, grouped: block b goes to group b % ngroups
  std::vector<std::vector<mhdgb_config>> gcfg(ngroups);
  std::vector<std::vector<int>> gblocks(ngroups);
  d->off.resize(nb);
  d->ext.resize(nb);
  d->block_group.resize(nb);
  for (int b = 0; b < nb; b++) {
    const int c[3] = {b / (ntiles[1] * ntiles[2]), (b / ntiles[2]) % ntiles[1], b % ntiles[2]};
    mhdgb_config bc = *cfg;
    int* dims[3] = {&bc.nx, &bc.ny, &bc.nz};
    for (int a = 0; a < 3; a++) {
      split_axis(n[a], ntiles[a], c[a], &d->off[b][a], dims[a]);
      d->ext[b][a] = *dims[a];
      // a face on the whole grid's boundary keeps its kind unless it wraps around to another block
      // (periodic with more than one block along the axis); every inner face is exchanged
      for (int side = 0; side < 2; side++) {
        const bool edge = side == 0 ? c[a] == 0 : c[a] == ntiles[a] - 1;
        const int f = 2 * a + side;
        if (!edge || (cfg->bc[f] == MHDGB_BC_PERIODIC && ntiles[a] > 1)) bc.bc[f] = MHDGB_BC_EXCHANGE;
      }
    }
    const int q = b % ngroups;
    bc.device = devices ? devices[q] : cfg->device;
    gcfg[q].push_back(bc);
    gblocks[q].push_back(b);
    d->block_group[b] = q;
  }
  d->blocks.assign(nb, nullptr);
  d->g.resize(ngroups);
  auto cleanup = [&](int code) { mhdgb_domain_destroy(d); return code; };
  for (int q = 0; q < ngroups; q++) {
    mhdgb_ensemble* e = nullptr;
    int rc = mhdgb_ensemble_create((int)gcfg[q].size(), gcfg[q].data(), &e);
    if (rc) return cleanup(rc);
    d->groups.push_back(e);
    d->group_dev.push_back(gcfg[q][0].device);
    for (size_t i = 0; i < gblocks[q].size(); i++) d->blocks[gblocks[q][i]] = e->m[i];
  }
  // peer access between the groups' distinct devices (each group reads its neighbours' slabs)
  for (int q = 0; q < ngroups; q++)
    for (int r = 0; r < ngroups; r++) {
      const int a = d->group_dev[q], b = d->group_dev[r];
      if (a == b) continue;
      int ok = 0;
      if (cudaDeviceCanAccessPeer(&ok, a, b) != cudaSuccess || !ok) {
        d->err = "devices " + std::to_string(a) + " and " + std::to_string(b) + " have no peer access";
        return cleanup(MHDGB_ERR_ARG);
      }
      cudaSetDevice(a);
      const cudaError_t pe = cudaDeviceEnablePeerAccess(b, 0);
      if (pe != cudaSuccess && pe != cudaErrorPeerAccessAlreadyEnabled) return cleanup(MHDGB_ERR_CUDA);
      cudaGetLastError();
    }
  // each block's faces are the whole grid's, sliced: results do not depend on the split
  for (int b = 0; b < nb; b++) {
    const auto& o = d->off[b];
    int rc = mhdgb_set_grid(d->blocks[b], d->x1a.data() + o[0], d->x2a.data() + o[1], d->x3a.data() + o[2]);
    if (rc) return cleanup(rc);
  }
  // halo transfer tables and reduction lists per group
  std::vector<Ctrl*> all(nb);
  for (int b = 0; b < nb; b++) all[b] = d->blocks[b]->ctrl;
  for (int q = 0; q < ngroups; q++) {
    mhdgb_domain::Group& G = d->g[q];
    mhdgb_ensemble* e = d->groups[q];
    if (cudaSetDevice(e->device) != cudaSuccess) return cleanup(MHDGB_ERR_CUDA);
    std::vector<HaloXfer> xs;
    std::vector<Ctrl*> own;
    long long total = 0;
    for (int b : gblocks[q]) {
      mhdgb_solver* dst = d->blocks[b];
      own.push_back(dst->ctrl);
      const int c[3] = {b / (ntiles[1] * ntiles[2]), (b / ntiles[2]) % ntiles[1], b % ntiles[2]};
      for (int f = 0; f < 6; f++) {
        if (dst->cfg.bc[f] != MHDGB_BC_EXCHANGE) continue;
        const int a = f >> 1, side = f & 1;
        int cn[3] = {c[0], c[1], c[2]};
        cn[a] = (c[a] + (side ? 1 : -1) + ntiles[a]) % ntiles[a];
        mhdgb_solver* src = d->blocks[block_of(d, cn[0], cn[1], cn[2])];
        HaloXfer t{};
        const bool mixed = dst->kind == FUSED_MIXED;
        for (int p = 0; p < 2; p++) {
          t.src[p] = mixed ? (const void*)src->P32[p] : (const void*)src->P64[p];
          t.dst[p] = mixed ? (void*)dst->P32[p] : (void*)dst->P64[p];
        }
        t.Ls = src->L;
        t.Ld = dst->L;
        t.bs = face_box(src->L, f ^ 1, false);  // the neighbour's layers next to its opposite face
        t.bd = face_box(dst->L, f, true);
        t.ctrl = dst->ctrl;
        t.begin = total;
        total += box_count(t.bd);
        xs.push_back(t);
      }
    }
    G.nxfer = (int)xs.size();
    G.total = total;
    G.nown = (int)own.size();
    if ((!xs.empty() && cudaMalloc(&G.d_xfer, xs.size() * sizeof(HaloXfer)) != cudaSuccess) ||
        cudaMalloc(&G.d_all, nb * sizeof(Ctrl*)) != cudaSuccess ||
        cudaMalloc(&G.d_own, own.size() * sizeof(Ctrl*)) != cudaSuccess)
      return cleanup(MHDGB_ERR_NOMEM);
    if ((!xs.empty() && cudaMemcpy(G.d_xfer, xs.data(), xs.size() * sizeof(HaloXfer), cudaMemcpyHostToDevice) != cudaSuccess) ||
        cudaMemcpy(G.d_all, all.data(), nb * sizeof(Ctrl*), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(G.d_own, own.data(), own.size() * sizeof(Ctrl*), cudaMemcpyHostToDevice) != cudaSuccess ||
        legacy_fence() != cudaSuccess)
      return cleanup(MHDGB_ERR_CUDA);
    if (cudaEventCreateWithFlags(&G.ev_step, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&G.ev_halo, cudaEventDisableTiming) != cudaSuccess)
      return cleanup(MHDGB_ERR_CUDA);
  }
  *out = d;
  return MHDGB_OK;
}

int mhdgb_domain_destroy(mhdgb_domain* d) {
  if (!d) return MHDGB_OK;
  for (size_t q = 0; q < d->groups.size(); q++) {
    cudaSetDevice(d->group_dev[q]);
    cudaStreamSynchronize(d->groups[q]->stream);
  }
  domain_destroy_graphs(d);
  for (size_t q = 0; q < d->g.size(); q++) {
    auto& G = d->g[q];
    if (q < d->group_dev.size()) cudaSetDevice(d->group_dev[q]);
    if (G.d_xfer) cudaFree(G.d_xfer);
    if (G.d_all) cudaFree(G.d_all);
    if (G.d_own) cudaFree(G.d_own);
    if (G.ev_step) cudaEventDestroy(G.ev_step);
    if (G.ev_halo) cudaEventDestroy(G.ev_halo);
  }
  for (auto* e : d->groups) mhdgb_ensemble_destroy(e);
  delete d;
  return MHDGB_OK;
}

const char* mhdgb_domain_last_error(const mhdgb_domain* d) { return d ? d->err.c_str() : "null domain"; }

int mhdgb_domain_blocks(const mhdgb_domain* d) { return d ? (int)d->blocks.size() : 0; }

int mhdgb_domain_block(mhdgb_domain* d, int b, mhdgb_solver** h, int offset[3], int extent[3]) {
  if (!d || b < 0 || b >= (int)d->blocks.size()) return MHDGB_ERR_ARG;
  if (h) *h = d->blocks[b];
  for (int a = 0; a < 3; a++) {
    if (offset) offset[a] = d->off[b][a];
    if (extent) extent[a] = d->ext[b][a];
  }
  return MHDGB_OK;
}

// Whole-grid arrays: reference layout with the whole grid's extents (nx+5, ny+5, nz+5).
int mhdgb_domain_upload_cons(mhdgb_domain* d, const double* U) {
  if (!d || !U) return MHDGB_ERR_ARG;
  const int IT = d->cfg.nx + 5, JT = d->cfg.ny + 5;
  for (size_t b = 0; b < d->blocks.size(); b++) {
    mhdgb_solver* h = d->blocks[b];
    const auto& o = d->off[b];
    const int it = h->L.itot, jt = h->L.jtot, kt = h->L.ktot;
    std::vector<double> Ub((size_t)NCONS * it * jt * kt);
    for (int k = 0; k < kt; k++)
      for (int j = 0; j < jt; j++)
        for (int m = 0; m < NCONS; m++)
          std::memcpy(&Ub[(size_t)it * (m + (size_t)NCONS * (j + (size_t)jt * k))],
                      &U[(size_t)o[0] + (size_t)IT * (m + (size_t)NCONS * ((j + o[1]) + (size_t)JT * (k + o[2])))],
                      sizeof(double) * it);
    int rc = mhdgb_upload_cons(h, Ub.data());
    if (rc) return dfail(d, rc, "block " + std::to_string(b) + ": " + h->err);
  }
  d->prepared = false;
  return MHDGB_OK;
}

// Interior cells of every block into the whole-grid array (its ghost cells are left as they are).
int mhdgb_domain_download_cons(mhdgb_domain* d, double* U) {
  if (!d || !U) return MHDGB_ERR_ARG;
  const int IT = d->cfg.nx + 5, JT = d->cfg.ny + 5;
  for (size_t b = 0; b < d->blocks.size(); b++) {
    mhdgb_solver* h = d->blocks[b];
    const auto& o = d->off[b];
    const auto& x = d->ext[b];
    const int it = h->L.itot, jt = h->L.jtot, kt = h->L.ktot;
    std::vector<double> Ub((size_t)NCONS * it * jt * kt);
    int rc = mhdgb_download_cons(h, Ub.data());
    if (rc) return dfail(d, rc, "block " + std::to_string(b) + ": " + h->err);
    for (int k = NGH; k < NGH + x[2]; k++)
      for (int j = NGH; j < NGH + x[1]; j++)
        for (int m = 0; m < NCONS; m++)
          std::memcpy(&U[(size_t)(o[0] + NGH) + (size_t)IT * (m + (size_t)NCONS * ((j + o[1]) + (size_t)JT * (k + o[2])))],
                      &Ub[(size_t)NGH + (size_t)it * (m + (size_t)NCONS * (j + (size_t)jt * k))], sizeof(double) * x[0]);
  }
  return MHDGB_OK;
}

int mhdgb_domain_init_kh(mhdgb_domain* d, unsigned long long seed, double vshear, double width, double bx,
                         double amp, double sig, double noise) {
  if (!d) return MHDGB_ERR_ARG;
  const KhParams kp{seed, vshear, width, bx, amp, sig, noise};
  for (size_t b = 0; b < d->blocks.size(); b++) {
    const auto& o = d->off[b];
    int rc = init_kh_block(d->blocks[b], d->cfg.nx, d->cfg.ny, o[0], o[1], o[2], kp);
    if (rc) return dfail(d, rc, "block " + std::to_string(b) + ": " + d->blocks[b]->err);
  }
  d->prepared = false;
  return MHDGB_OK;
}

int mhdgb_domain_prepare(mhdgb_domain* d) {
  if (!d) return MHDGB_ERR_ARG;
  return domain_prepare(d);
}

int mhdgb_domain_step(mhdgb_domain* d, int nsteps) {
  if (!d || nsteps < 0) return MHDGB_ERR_ARG;
  int rc;
  // a block that lost its prepared state (new U, new physics) or whose kernel arguments changed
  // since its group's launch table was built: prepare the whole domain again
  bool stale = !d->prepared;
  for (auto* h : d->blocks) stale = stale || !h->prepared;
  for (auto* e : d->groups)
    for (size_t i = 0; i < e->m.size(); i++)
      stale = stale || i >= e->desc_seen.size() || e->desc_seen[i] != e->m[i]->desc_version;
  if (stale && (rc = domain_prepare(d))) return rc;
  const int G = 16;
  if (d->groups.size() == 1 && nsteps >= G) {
    mhdgb_ensemble* e = d->groups[0];
    auto& Gr = d->g[0];
    DCK(d, cudaSetDevice(e->device));
    if (!Gr.gexec) {
      cudaGraph_t graph = nullptr;
      DCK(d, cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
      rc = MHDGB_OK;
      for (int s = 0; s < G && rc == MHDGB_OK; s++) rc = domain_step_once(d);
      cudaError_t ce = cudaStreamEndCapture(e->stream, &graph);
      if (rc) { if (graph) cudaGraphDestroy(graph); return rc; }
      if (ce != cudaSuccess) return dfail(d, MHDGB_ERR_CUDA, "cudaStreamEndCapture");
      ce = cudaGraphInstantiate(&Gr.gexec, graph, 0);
      cudaGraphDestroy(graph);
      if (ce != cudaSuccess) return dfail(d, MHDGB_ERR_CUDA, "cudaGraphInstantiate");
    }
    while (nsteps >= G) {
      DCK(d, cudaGraphLaunch(Gr.gexec, e->stream));
      nsteps -= G;
    }
  }
  for (; nsteps > 0; nsteps--)
    if ((rc = domain_step_once(d))) return rc;
  for (auto* h : d->blocks) { h->p64_valid = false; h->p_user = false; }
  return MHDGB_OK;
}

int mhdgb_domain_sync(mhdgb_domain* d, mhdgb_report* r) {
  if (!d) return MHDGB_ERR_ARG;
  int rc = domain_sync_streams(d);
  if (rc) return rc;
  int first = MHDGB_OK;
  unsigned status = 0;
  mhdgb_report r0{};
  for (size_t b = 0; b < d->blocks.size(); b++) {
    mhdgb_report rb{};
    rc = mhdgb_sync(d->blocks[b], &rb);
    status |= rb.status;
    if (b == 0) r0 = rb;
    if (rc && first == MHDGB_OK) first = dfail(d, rc, "block " + std::to_string(b) + ": " + d->blocks[b]->err);
  }
  r0.status = status;
  if (r) *r = r0;
  return first;
}

int mhdgb_domain_set_stop(mhdgb_domain* d, double tmax, long long max_steps) {
  if (!d) return MHDGB_ERR_ARG;
  for (size_t b = 0; b < d->blocks.size(); b++) {
    int rc = mhdgb_set_stop(d->blocks[b], tmax, max_steps);
    if (rc) return dfail(d, rc, d->blocks[b]->err);
  }
  return MHDGB_OK;
}

int mhdgb_domain_time_steps(mhdgb_domain* d, int nsteps, double* ms) {
  if (!d || nsteps < 1 || !ms) return MHDGB_ERR_ARG;
  int rc;
  if (!d->prepared && (rc = domain_prepare(d))) return rc;
  if (nsteps >= 16 && d->groups.size() == 1 && !d->g[0].gexec && (rc = mhdgb_domain_step(d, 16))) return rc;
  if ((rc = domain_sync_streams(d))) return rc;
  mhdgb_ensemble* e0 = d->groups[0];
  DCK(d, cudaSetDevice(e0->device));
  cudaEvent_t a, b;
  DCK(d, cudaEventCreate(&a));
  DCK(d, cudaEventCreate(&b));
  DCK(d, cudaEventRecord(a, e0->stream));
  // every group's stream starts after the first event, and the last event follows every group
  for (size_t q = 1; q < d->groups.size(); q++) {
    DCK(d, cudaSetDevice(d->groups[q]->device));
    DCK(d, cudaStreamWaitEvent(d->groups[q]->stream, a, 0));
  }
  rc = mhdgb_domain_step(d, nsteps);
  for (size_t q = 1; q < d->groups.size() && rc == MHDGB_OK; q++) {
    DCK(d, cudaSetDevice(d->groups[q]->device));
    DCK(d, cudaEventRecord(d->g[q].ev_step, d->groups[q]->stream));
    DCK(d, cudaSetDevice(e0->device));
    DCK(d, cudaStreamWaitEvent(e0->stream, d->g[q].ev_step, 0));
  }
  DCK(d, cudaSetDevice(e0->device));
  DCK(d, cudaEventRecord(b, e0->stream));
  DCK(d, cudaEventSynchronize(b));
  float t = 0.0f;
  DCK(d, cudaEventElapsedTime(&t, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  *ms = t;
  return rc;
}

// KH diagnostic of the whole grid from the blocks' sums (each block's volume-weighted means,
// recombined by volume).
int mhdgb_domain_diag(mhdgb_domain* d, double out[3]) {
  if (!d || !out) return MHDGB_ERR_ARG;
  double v = 0.0, m = 0.0, a = 0.0;
  for (size_t b = 0; b < d->blocks.size(); b++) {
    double o[3];
    int rc = mhdgb_diag(d->blocks[b], o);
    if (rc) return dfail(d, rc, d->blocks[b]->err);
    v += o[0];
    m += o[1] * o[0];
    a += o[2] * o[2] * o[0];
  }
  out[0] = v;
  out[1] = m / v;
  out[2] = std::sqrt(a / v);
  return MHDGB_OK;
}

}  // extern "C"
