// noalloc.cu -- pdfs_sweep_static(): one FSM ordering that allocates nothing.
//
// Callers that cannot allocate device memory while they run -- code confined
// to a pre-sized pool or arena handed over by a host application, real-time
// loops that must not call the allocator (cudaMalloc can block and
// synchronise the device), plugins whose host process forbids allocation
// after its own set-up -- get the sweep of pdfs_sweep() without any call to
// cudaMalloc, cudaFree or an allocating library routine.  Everything the
// sweep kernel needs besides the caller's field lives in g_scratch below, a
// file-scope device array of PDFS_STATIC_SCRATCH_BYTES that each GPU loading
// this library holds until the process exits.
//
// Host code must not pass g_scratch itself to a kernel: in host code the
// name is only a host-side stand-in for the symbol.  Its device address is
// looked up with cudaGetSymbolAddress once per device context, with that
// device current (the first call in a context does it, so make that call
// before any stream capture), and that address is what the kernel receives.
// The address is cached per device together with the id of the context it
// belongs to, under a lock: after a cudaDeviceReset (a new primary context,
// into which the module and its array are loaded again) or under another
// driver context the lookup is repeated, so a stale address is never used.
// CUDA loads modules lazily by default, so the array is reserved during the
// first call on each device: make one call (a 1 x 1 x 1 grid is enough)
// during set-up, before the phase in which nothing may be allocated.
// All calls share the array and leave their contents behind; each call
// zeroes the words that must start at zero (column progress, ticket,
// status), and calls that overlap on the GPU race on the array, so the
// caller serialises them.
#include <cuda.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "internal.h"

namespace pdfs {
namespace {

constexpr int kTY = 4;   // FP64 tile of the sweep (32 x 4 columns, one row per compute warp)
constexpr int kR = 1;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_scratch[PDFS_STATIC_SCRATCH_BYTES];

// Device address of g_scratch per device, with the id of the context it was
// looked up in (0 = none yet).  Guarded by g_scratch_mu.
struct ScratchAddr {
  unsigned long long ctx_id;
  void *ptr;
};
static ScratchAddr g_scratch_dev[kMaxDevices];
static std::mutex g_scratch_mu;

using CtxGetCurrentFn = CUresult (*)(CUcontext *);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long *);

template <class F>
F driver_fn(const char *name, int version) {
  void *p = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion(name, &p, version, cudaEnableDefault, &q) == cudaSuccess &&
      q == cudaDriverEntryPointSuccess)
    return reinterpret_cast<F>(p);
  cudaGetLastError();
  return nullptr;
}

// Id of the calling thread's current driver context, 0 if it cannot be told.
unsigned long long current_ctx_id() {
  static const CtxGetCurrentFn get_cur = driver_fn<CtxGetCurrentFn>("cuCtxGetCurrent", 4000);
  static const CtxGetIdFn get_id = driver_fn<CtxGetIdFn>("cuCtxGetId", 12000);
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (!get_cur || !get_id || get_cur(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// g_scratch's device address in the current context of device dev.  The
// lookup runs once per context (cudaGetSymbolAddress also makes the device's
// primary context current if no context was); without a context id the
// lookup runs on every call.
cudaError_t scratch_address(int dev, unsigned char **out) {
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  unsigned long long id = current_ctx_id();
  ScratchAddr &e = g_scratch_dev[dev];
  if (id != 0 && e.ctx_id == id && e.ptr) {
    *out = static_cast<unsigned char *>(e.ptr);
    return cudaSuccess;
  }
  void *ptr = nullptr;
  cudaError_t err = cudaGetSymbolAddress(&ptr, g_scratch);
  if (err != cudaSuccess) return err;
  if (!ptr) return cudaErrorInvalidSymbol;
  if (id == 0) id = current_ctx_id();  // the lookup may have made the primary context current
  e.ctx_id = id;
  e.ptr = ptr;
  *out = static_cast<unsigned char *>(ptr);
  return cudaSuccess;
}

// Offsets of the scratch regions (256-byte aligned) for one grid.
struct ScratchPlan {
  size_t status, ticket, order, prog, xbox, ybox, total;
  long long xstride, ystride;
  int nbands;
};

size_t up256(size_t v) { return (v + 255) & ~size_t(255); }

ScratchPlan plan_for(const Layout &L, int nz) {
  ScratchPlan p;
  const size_t ncol = (size_t)L.ncx * L.ncy;
  p.nbands = mailbox_chunks(nz);
  p.xstride = (long long)p.nbands * kMailboxChunk * L.ty;
  p.ystride = (long long)p.nbands * kMailboxChunk * L.tx;
  p.status = 0;
  p.ticket = up256(p.status + sizeof(DevStatus));
  p.order = up256(p.ticket + 16);
  p.prog = up256(p.order + ncol * 4);
  p.xbox = up256(p.prog + ncol * L.ty * 4);
  p.ybox = up256(p.xbox + ncol * (size_t)p.xstride * 8);
  p.total = up256(p.ybox + ncol * (size_t)p.ystride * 8);
  return p;
}

// Ticket order of the columns, computed on the device so that nothing is
// staged from the host: column c's ticket is its rank by (expected start
// step lcx*(TX+12) + lcy*(TY+12), column id) -- the order the allocating path
// builds on the host.
__global__ void k_static_order(int *order, int ncx, int ncy, int tx, int ty) {
  const int n = ncx * ncy;
  const long long wx = tx + 12, wy = ty + 12;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    const long long kc = (c % ncx) * wx + (c / ncx) * wy;
    int rank = 0;
    for (int d = 0; d < n; ++d) {
      const long long kd = (d % ncx) * wx + (d / ncx) * wy;
      rank += (kd < kc || (kd == kc && d < c)) ? 1 : 0;
    }
    order[rank] = c;
  }
}

int status_of(cudaError_t e) {
  if (e == cudaSuccess) return PDFS_OK;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return PDFS_ERR_NO_DEVICE;
  return PDFS_ERR_CUDA;
}

bool valid_grid(const pdfs_grid *g) {
  return g && g->nx >= 1 && g->ny >= 1 && g->nz >= 1 && g->ny + 2 <= 65535 && g->nz + 2 <= 65535 &&
         g->nx + 2 <= (1 << 20) && g->dx > 0 && g->dy > 0 && g->dz > 0;
}

}  // namespace
}  // namespace pdfs

using namespace pdfs;

extern "C" int pdfs_static_layout(const pdfs_grid *g, long long *px, long long *ry, long long *elems,
                                  long long *scratch_bytes) {
  if (!valid_grid(g)) return PDFS_ERR_INVALID;
  const Layout L = make_layout(*g, 32, kTY, 8);
  const ScratchPlan p = plan_for(L, g->nz);
  if (px) *px = L.px;
  if (ry) *ry = L.ry;
  if (elems) *elems = (long long)L.elems;
  if (scratch_bytes) *scratch_bytes = (long long)p.total;
  return p.total > PDFS_STATIC_SCRATCH_BYTES ? PDFS_ERR_TOO_LARGE : PDFS_OK;
}

extern "C" int pdfs_sweep_static(const pdfs_grid *g, double *field_dev, int sn, double *max_change, void *stream) {
  if (!valid_grid(g) || !field_dev || sn < 1 || sn > 8) return PDFS_ERR_INVALID;
  const Layout L = make_layout(*g, 32, kTY, 8);
  const ScratchPlan p = plan_for(L, g->nz);
  if (p.total > PDFS_STATIC_SCRATCH_BYTES) return PDFS_ERR_TOO_LARGE;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return status_of(e);
  if (dev < 0 || dev >= kMaxDevices) return PDFS_ERR_INVALID;
  unsigned char *base = nullptr;
  if ((e = scratch_address(dev, &base)) != cudaSuccess) return status_of(e);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int sms = 0;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return status_of(e);

  SweepArgs a;
  std::memset(&a, 0, sizeof(a));
  a.u = field_dev;
  a.px = L.px;
  a.plane = L.plane;
  a.nx = g->nx;
  a.ny = g->ny;
  a.nz = g->nz;
  ordering_signs(sn, &a.sx, &a.sy, &a.sz);
  a.ncx = L.ncx;
  a.ncy = L.ncy;
  a.nbands = p.nbands;
  a.xstride = p.xstride;
  a.ystride = p.ystride;
  DevStatus *status = reinterpret_cast<DevStatus *>(base + p.status);
  a.order = reinterpret_cast<const int *>(base + p.order);
  a.prog = reinterpret_cast<int *>(base + p.prog);
  a.xbox = base + p.xbox;
  a.ybox = base + p.ybox;
  a.ticket = reinterpret_cast<int *>(base + p.ticket);
  a.err = status->err;
  a.maxchg = &status->chg;
  a.hmin = (float)std::min(g->dx, std::min(g->dy, g->dz));
  // the same wait bound and test hook as the allocating path: PDFS_WAIT_MS
  // (default 4 s, counted at the highest SM clock) and PDFS_TEST_POISON_COLUMN
  // (a column that never publishes, so that the bounded waits give up)
  long long wait_ms = 4000;
  if (const char *w = getenv("PDFS_WAIT_MS")) wait_ms = atoll(w);
  a.wait_cycles = wait_ms * 1000000LL * 21 / 10;
  a.poison_col = getenv("PDFS_TEST_POISON_COLUMN") ? atoi(getenv("PDFS_TEST_POISON_COLUMN")) : -1;
  const double h[3] = {g->dx, g->dy, g->dz};
  for (int i = 0; i < 3; ++i) {
    a.k64.h[i] = h[i];
    a.k64.h2[i] = h[i] * h[i];
    a.k64.q[i] = 1.0 / (h[i] * h[i]);
  }
  a.k64.qsum = a.k64.q[0] + a.k64.q[1] + a.k64.q[2];
  a.k64.iqsum = 1.0 / a.k64.qsum;

  // words that must start at zero; the mailboxes are written before they are read
  const size_t ncol = (size_t)L.ncx * L.ncy;
  if ((e = cudaMemsetAsync(base + p.status, 0, sizeof(DevStatus), st)) != cudaSuccess) return status_of(e);
  if ((e = cudaMemsetAsync(base + p.ticket, 0, 16, st)) != cudaSuccess) return status_of(e);
  if ((e = cudaMemsetAsync(base + p.prog, 0, ncol * L.ty * 4, st)) != cudaSuccess) return status_of(e);
  k_static_order<<<(int)std::min<size_t>((ncol + 127) / 128, 1024), 128, 0, st>>>(
      reinterpret_cast<int *>(base + p.order), L.ncx, L.ncy, L.tx, L.ty);
  if ((e = cudaGetLastError()) != cudaSuccess) return status_of(e);
  int grid = 0;
  // tile id 1 of the FP64 kernels is TY = 4, one row per compute warp
  if ((e = launch_sweep(1, 1, ARITH_REF, false, a, L, nullptr, sms, st, &grid)) != cudaSuccess) return status_of(e);
  DevStatus hs;
  if ((e = cudaMemcpyAsync(&hs, status, sizeof(hs), cudaMemcpyDeviceToHost, st)) != cudaSuccess) return status_of(e);
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return status_of(e);
  if (hs.err[0]) return hs.err[0] == DEV_ERR_TIMEOUT ? PDFS_ERR_TIMEOUT : PDFS_ERR_CUDA;
  if (max_change) {
    double d;
    std::memcpy(&d, &hs.chg, 8);
    *max_change = d;
  }
  return PDFS_OK;
}
