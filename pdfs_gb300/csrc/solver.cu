// solver.cu -- host driver of the GB300 FSM solve and the C ABI of include/pdfs.h.
//
// Replaces run_fsm (single_gpu_cuda/src/phi3D_fsm.cu:64-106): the field is
// copied once into a padded device layout, swept by the persistent column
// kernels until convergence (the reference runs a fixed single round,
// single_gpu_cuda/src/phi3D.c:118-119, and has no convergence test), and
// copied back.  Errors are returned, never exit()ed (phi3D_fsm.h:39-46 exits).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstddef>
#include <cstring>
#include <mutex>
#include <utility>
#include <vector>

#include "internal.h"

namespace pdfs {

Layout make_layout(const pdfs_grid &g, int tx, int ty, int esize, int xo) {
  Layout L;
  L.tx = tx;
  L.ty = ty;
  L.esize = esize;
  L.V = 16 / esize;
  L.xo = xo < 0 ? L.V - 1 : xo;
  L.ncx = (g.nx + tx - 1) / tx;
  L.ncy = (g.ny + ty - 1) / ty;
  const long long need = (long long)L.ncx * tx + 2 * L.V;
  const long long align = 128 / esize;
  L.px = (need + align - 1) / align * align;
  L.ry = (long long)L.ncy * ty + 2;
  L.plane = L.px * L.ry;
  L.elems = (size_t)L.plane * (size_t)(g.nz + 2);
  return L;
}

Layout make_layout_zc(const pdfs_grid &g, int rows, int esize) {
  Layout L;
  L.zc = 1;
  L.tx = kLcLanes;
  L.ty = rows;
  L.esize = esize;
  L.V = 16 / esize;
  L.ncx = (g.nx + 1 + kLcLanes - 1) / kLcLanes;  // lanes 0..30 of the last tile reach lx = nx - 1
  L.ncy = (g.ny + 30) / rows + 1;                // lane 30 of the last tile row reaches ly = ny - 1
  L.px = g.nx + 2;
  L.ry = g.ny + 2;
  // the traversal runs over z = 0 .. 8 ceil(nz/8) + 7 (going down it passes
  // every block's top boundary z == 0 mod 8); q_last == 7 (mod 8), T == 0 (mod 8)
  L.q_last = kLcZ0 + 8 * ((g.nz + 7) / 8) + 7;
  L.T = L.q_last - kLcZ0 + 1;
  L.qz = L.q_last + 25;  // room for the look-ahead of the rows past the last step
  L.plane = 0;
  L.elems = (size_t)L.ry * (size_t)L.px * (size_t)L.qz;
  return L;
}

// Expected start level of each tile: it trails the tile above by R + c
// levels (its row 0 needs that tile's row R-1 at the same position) and the
// tiles to the left by the offset of the rows it reads from them plus c
// (c: a few levels of hand-off latency).  Every wait then points to a
// strictly earlier start, so sorting by start lists each tile after the
// tiles it waits on: the tickets are deadlock-free.
std::vector<int> lc_order(int ntx, int nty, int rows) {
  const int c = 4;
  std::vector<long long> start((size_t)ntx * nty, 0);
  for (int tx = 0; tx < ntx; ++tx)
    for (int ty = 0; ty < nty; ++ty) {
      long long st = 0;
      if (ty > 0) st = std::max(st, start[(size_t)(ty - 1) * ntx + tx] + rows + c);
      if (tx > 0)
        for (int r = 0; r < rows; ++r) {
          const int k = rows * ty + r + 30, ty2 = k / rows, r2 = k % rows;  // lane 30, row r2 of tile (tx-1, ty2)
          if (ty2 < nty) st = std::max(st, start[(size_t)ty2 * ntx + tx - 1] + std::max(1, r2 - r + c));
        }
      start[(size_t)ty * ntx + tx] = st;
    }
  std::vector<int> o((size_t)ntx * nty);
  for (size_t i = 0; i < o.size(); ++i) o[i] = (int)i;
  std::stable_sort(o.begin(), o.end(), [&](int a, int b) { return start[a] < start[b]; });
  return o;
}

MaskLayout make_mask_layout(const pdfs_grid &g) {
  MaskLayout M;
  M.fy = ((long long)g.ny + 32 + 3) / 4 * 4;
  M.fw = (g.nx + 31) / 32 + 1;
  M.fplane = M.fy * M.fw;
  M.words = (size_t)M.fplane * (size_t)(g.nz + 2);
  return M;
}

// ---- layout conversion kernels (one thread per node of a row; grid (rows, planes)) ----
template <class T>
__global__ void k_fill(T *p, size_t n, T v) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) p[i] = v;
}

// reference layout (double) -> internal layout of T
template <class T>
__global__ void k_pack(const double *__restrict__ ref, T *__restrict__ dst, int nx, int ny, Layout L, int z0) {
  const int y = blockIdx.x, z = blockIdx.y + z0;
  const double *row = ref + ((size_t)z * (ny + 2) + y) * (size_t)(nx + 2);
  for (int x = threadIdx.x; x < nx + 2; x += blockDim.x) dst[L.index(x, y, z)] = (T)row[x];
}

// internal layout -> reference layout (double).  FP32 source: frozen nodes
// (mask bit set) take the exact FP64 input instead of the rounded value.
template <class T>
__global__ void k_unpack(const T *__restrict__ src, Layout L, const double *__restrict__ in64, Layout L64,
                         const uint32_t *__restrict__ fmask, MaskLayout M, double *__restrict__ ref, int nx, int ny,
                         int z0) {
  const int y = blockIdx.x, z = blockIdx.y + z0;
  double *row = ref + ((size_t)z * (ny + 2) + y) * (size_t)(nx + 2);
  for (int x = threadIdx.x; x < nx + 2; x += blockDim.x) {
    double v = (double)src[L.index(x, y, z)];
    if (L.zc) v = fabs(v);  // z-column fields mark frozen nodes with the sign
    if (fmask && x >= 1 && x <= nx && y >= 1 && y <= ny) {
      const uint32_t w = fmask[M.word(x, y, z)];
      if ((w >> ((x - 1) & 31)) & 1u) v = in64[L64.index(x, y, z)];
    }
    row[x] = v;
  }
}

// internal layout of S -> internal layout of D, every halo-padded node
// (one warp per halo-padded row: row r = blockIdx.x * 8 + warp is (y, z) =
// (r % (ny + 2), r / (ny + 2)))
constexpr int kRowWarps = 8;
template <class S, class D>
__global__ void __launch_bounds__(32 * kRowWarps) k_convert(const S *__restrict__ src, Layout Ls, D *__restrict__ dst,
                                                            Layout Ld, int nx, int ny, int nz) {
  const long long r = (long long)blockIdx.x * kRowWarps + (threadIdx.x >> 5);
  if (r >= (long long)(ny + 2) * (nz + 2)) return;
  const int y = (int)(r % (ny + 2)), z = (int)(r / (ny + 2));
  const long long is = Ls.index(0, y, z), id = Ld.index(0, y, z);
#pragma unroll 4
  for (int x = threadIdx.x & 31; x < nx + 2; x += 32) dst[id + x] = (D)src[is + x];
}

inline unsigned row_blocks(const pdfs_grid &g) {
  return (unsigned)(((long long)(g.ny + 2) * (g.nz + 2) + kRowWarps - 1) / kRowWarps);
}

// Every element of a z-column (ZC) working field, in column order: the
// input's value (FP32, or its nearest pair) -- or, with from32, the FP32
// field's value as a pair -- with the sign bit set on the nodes the sweeps
// must not change (frozen nodes and the halo: their exact input, as a pair
// for pairs), and -inf in the padding at both ends of each column.
template <class T>
__global__ void k_zc_fill(T *__restrict__ dst, Layout Ld, const double *__restrict__ in64, Layout L64,
                          const float *__restrict__ u32, Layout L32, bool from32, const uint32_t *__restrict__ fmask,
                          MaskLayout M, int nx, int ny, int nz, int *neg) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < Ld.elems; i += (size_t)gridDim.x * blockDim.x) {
    const long long col = (long long)(i / (size_t)Ld.qz);
    const int z = (int)(i - (size_t)col * (size_t)Ld.qz) - kLcZ0;
    const int y = (int)(col / Ld.px), x = (int)(col - (long long)y * Ld.px);
    if (z < 0 || z > nz + 1) {
      if constexpr (sizeof(T) == 4)
        dst[i] = -INFINITY;
      else
        dst[i] = p_make(-INFINITY, 0.0f);
      continue;
    }
    bool frz = x < 1 || x > nx || y < 1 || y > ny || z < 1 || z > nz;
    if (!frz && fmask) frz = (fmask[M.word(x, y, z)] >> ((x - 1) & 31)) & 1u;
    // the sign bit marks frozen nodes: a node the sweeps update must not carry one
    if (!frz && signbit(in64[L64.index(x, y, z)])) *neg = 1;
    if constexpr (sizeof(T) == 4) {
      const float v = (float)in64[L64.index(x, y, z)];
      dst[i] = frz ? -fabsf(v) : v;
    } else {
      double pv;
      if (frz || !from32) {
        pv = p_from_double(in64[L64.index(x, y, z)]);
      } else {
        pv = p_make(fabsf(u32[L32.index(x, y, z)]), 0.0f);
      }
      if (frz) pv = __longlong_as_double(__double_as_longlong(pv) | 0x80000000LL);  // hi's sign bit
      dst[i] = pv;
    }
  }
}

// FP32 working field -> FP64 working field (polish start): frozen nodes and
// the halo keep the exact FP64 input.
__global__ void __launch_bounds__(32 * kRowWarps) k_widen(const float *__restrict__ u32, Layout L32,
                                                          const double *__restrict__ in64, double *__restrict__ u64,
                                                          Layout L64, const uint32_t *__restrict__ fmask, MaskLayout M,
                                                          int nx, int ny, int nz) {
  const long long r = (long long)blockIdx.x * kRowWarps + (threadIdx.x >> 5);
  if (r >= (long long)(ny + 2) * (nz + 2)) return;
  const int y = (int)(r % (ny + 2)), z = (int)(r / (ny + 2));
  const bool irow = y >= 1 && y <= ny && z >= 1 && z <= nz;
  const long long i32 = L32.index(0, y, z), i64 = L64.index(0, y, z);
#pragma unroll 4
  for (int x = threadIdx.x & 31; x < nx + 2; x += 32) {
    const float v = u32[i32 + x];
    const bool interior = irow && x >= 1 && x <= nx;
    bool frz = !interior;
    if (interior && fmask) frz = (__ldg(fmask + M.word(x, y, z)) >> ((x - 1) & 31)) & 1u;
    u64[i64 + x] = frz ? in64[i64 + x] : (double)v;
  }
}

__device__ __forceinline__ double to_pair(double d) { return p_from_double(d); }

// every element of an FP64 buffer -> the pair nearest it (the start of an
// FP64-precision solve in pair arithmetic)
__global__ void k_to_pair(const double *__restrict__ src, double *__restrict__ dst, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    dst[i] = to_pair(src[i]);
}

// FP32 working field -> pair working field (polish start): (u32, 0) for the
// nodes the sweeps update, the input's nearest pair for frozen nodes and the halo
__global__ void __launch_bounds__(32 * kRowWarps) k_widen_pair(const float *__restrict__ u32, Layout L32,
                                                               const double *__restrict__ in64,
                                                               double *__restrict__ u64, Layout L64,
                                                               const uint32_t *__restrict__ fmask, MaskLayout M,
                                                               int nx, int ny, int nz) {
  const long long r = (long long)blockIdx.x * kRowWarps + (threadIdx.x >> 5);
  if (r >= (long long)(ny + 2) * (nz + 2)) return;
  const int y = (int)(r % (ny + 2)), z = (int)(r / (ny + 2));
  const bool irow = y >= 1 && y <= ny && z >= 1 && z <= nz;
  const long long i32 = L32.index(0, y, z), i64 = L64.index(0, y, z);
#pragma unroll 4
  for (int x = threadIdx.x & 31; x < nx + 2; x += 32) {
    const float v = u32[i32 + x];
    const bool interior = irow && x >= 1 && x <= nx;
    bool frz = !interior;
    if (interior && fmask) frz = (__ldg(fmask + M.word(x, y, z)) >> ((x - 1) & 31)) & 1u;
    u64[i64 + x] = frz ? to_pair(in64[i64 + x]) : p_make(v, 0.0f);
  }
}

// pair working field -> reference layout: hi + lo (exact in FP64) for the
// updated nodes; frozen nodes and the halo take the exact FP64 input
__global__ void k_unpack_pair(const double *__restrict__ src, Layout L, const double *__restrict__ in64,
                              const uint32_t *__restrict__ fmask, MaskLayout M, double *__restrict__ ref, int nx,
                              int ny, int nz, int z0) {
  const int y = blockIdx.x, z = blockIdx.y + z0;
  double *row = ref + ((size_t)z * (ny + 2) + y) * (size_t)(nx + 2);
  for (int x = threadIdx.x; x < nx + 2; x += blockDim.x) {
    const long long i = L.index(x, y, z);
    const bool interior = x >= 1 && x <= nx && y >= 1 && y <= ny && z >= 1 && z <= nz;
    bool frz = !interior;
    if (interior && fmask) {
      const uint32_t w = fmask[M.word(x, y, z)];
      frz = (w >> ((x - 1) & 31)) & 1u;
    }
    const double v = src[i];
    row[x] = frz ? in64[i] : (double)p_hi(v) + (double)p_lo(v);
  }
}

// Per 8^3 block: the smallest input value (the replace-update's cap) of the
// nodes the sweeps update (+inf if every node is frozen), and the same rounded
// down to float.  One warp per block, blocks b0 .. b1-1: lane (x, y) = (lane %
// 8, lane / 8) of a 8 x 4 quarter plane loads its 16 nodes before reducing.
__global__ void k_block_capmin(const double *__restrict__ in64, Layout L, const uint32_t *__restrict__ fmask,
                               MaskLayout M, int nx, int ny, int nz, int nbx, int nby, long long b0, long long b1,
                               double *__restrict__ b64, float *__restrict__ b32) {
  const int lane = threadIdx.x & 31;
  for (long long b = b0 + ((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5); b < b1;
       b += ((long long)gridDim.x * blockDim.x) >> 5) {
    const int bx = (int)(b % nbx), by = (int)((b / nbx) % nby), bz = (int)(b / ((long long)nbx * nby));
    const int x = 1 + bx * 8 + (lane & 7);
    double v[16];
    bool use[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      const int y = 1 + by * 8 + (lane >> 3) + 4 * (k & 1), z = 1 + bz * 8 + (k >> 1);
      use[k] = x <= nx && y <= ny && z <= nz;
      v[k] = use[k] ? in64[L.index(x, y, z)] : INFINITY;
      if (use[k] && fmask) use[k] = !((fmask[M.word(x, y, z)] >> ((x - 1) & 31)) & 1u);
    }
    double m = INFINITY;
#pragma unroll
    for (int k = 0; k < 16; ++k)
      if (use[k] && dkey(v[k]) < dkey(m)) m = v[k];  // integer keys: off the FP64 pipe
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const double o = __shfl_xor_sync(0xffffffffu, m, off);
      m = dkey(o) < dkey(m) ? o : m;
    }
    if (lane == 0) {
      b64[b] = m;
      b32[b] = __double2float_rd(m);
    }
  }
}

// uint8 mask in the reference layout -> frozen bitmask (interior nodes only)
__global__ void k_pack_mask(const uint8_t *__restrict__ m, uint32_t *__restrict__ bits, MaskLayout M, int nx,
                            int ny) {
  const int y = blockIdx.x + 1, z = blockIdx.y + 1;  // interior rows only
  const uint8_t *row = m + ((size_t)z * (ny + 2) + y) * (size_t)(nx + 2);
  const int nwords = (nx + 31) / 32;
  for (int w = threadIdx.x; w < nwords; w += blockDim.x) {
    uint32_t v = 0;
    for (int b = 0; b < 32; ++b) {
      const int x = 1 + w * 32 + b;
      if (x <= nx && row[x]) v |= 1u << b;
    }
    bits[M.word(1 + w * 32, y, z)] = v;
  }
}

// Ticket order of columns: ticket -> local column id (lcy*ncx + lcx), sorted
// by the column's expected start step, lcx*(TX+12) + lcy*(TY+12): a column
// trails its x-upwind neighbour by about TX steps and its y-upwind one by
// about TY, plus a few steps of hand-off latency.  Any order with positive
// weights lists both upwind neighbours first, which is all the deadlock
// argument needs.
std::vector<int> wavefront_order(int ncx, int ncy, int tx, int ty) {
  std::vector<int> o((size_t)ncx * ncy);
  for (size_t i = 0; i < o.size(); ++i) o[i] = (int)i;
  const long long wx = tx + 12, wy = ty + 12;
  std::stable_sort(o.begin(), o.end(), [&](int a, int b) {
    const long long ka = (a % ncx) * wx + (a / ncx) * wy, kb = (b % ncx) * wx + (b / ncx) * wy;
    return ka < kb;
  });
  return o;
}

}  // namespace pdfs

using namespace pdfs;

static int cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return PDFS_OK;
  if (e == cudaErrorMemoryAllocation) return PDFS_ERR_OOM;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return PDFS_ERR_NO_DEVICE;
  return PDFS_ERR_CUDA;
}
#define CK(call)                                 \
  do {                                           \
    cudaError_t e_ = (call);                     \
    if (e_ != cudaSuccess) {                     \
      if (getenv("PDFS_LOG"))                    \
        fprintf(stderr, "pdfs: %s:%d %s: %s\n", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); \
      return cuda_status(e_);                    \
    }                                            \
  } while (0)

static bool is_device_ptr(const void *p) {
  if (!p) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

static bool verbose(const pdfs_opts &o) { return o.verbose || getenv("PDFS_LOG"); }

extern "C" void pdfs_default_opts(pdfs_opts *o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->precision = PDFS_PREC_FP64;
  o->arith = PDFS_ARITH_REFERENCE;
  o->freeze = PDFS_FREEZE_NONE;
  o->scheduler = PDFS_SCHED_NONE;
  o->tol = 0.0;
}

extern "C" const char *pdfs_status_string(int s) {
  switch (s) {
    case PDFS_OK: return "ok";
    case PDFS_ERR_INVALID: return "invalid argument";
    case PDFS_ERR_OOM: return "out of memory";
    case PDFS_ERR_CUDA: return "CUDA error";
    case PDFS_ERR_TIMEOUT: return "inter-tile wait timed out";
    case PDFS_ERR_NOT_CONVERGED: return "not converged within max_sweeps";
    case PDFS_ERR_IO: return "I/O error";
    case PDFS_ERR_NO_DEVICE: return "no CUDA device";
    case PDFS_ERR_TOO_LARGE: return "grid too large for the fixed scratch of pdfs_sweep_static";
    default: return "unknown status";
  }
}

extern "C" const char *pdfs_version(void) { return "pdfs-gb300 0.1 (sm_103a)"; }

// Context blocks (the arena of a context's buffers, the transfer stage) are
// kept in a per-process cache when a context is destroyed, up to a quarter of
// the device's memory, and handed to the next context that needs a block of
// about that size: a repeated solve pays neither cudaMalloc nor cudaFree (which
// synchronises the device; 10 ms for the 15 GB of a 768^3 solve) again.  Every
// block is idle when cached: destroy and the stage's reallocation synchronise
// the context's streams first.  An allocation that finds the device full
// empties the cache and retries.
namespace {
struct CachedBlock {
  int dev;
  void *p;
  size_t bytes;
};
struct BlockCache {
  std::mutex m;
  std::vector<CachedBlock> blocks;
  size_t held[64] = {};
};
BlockCache &block_cache() {
  static BlockCache *bc = new BlockCache();  // never destroyed: the driver frees device memory at exit
  return *bc;
}
size_t cache_cap(int dev) {
  static size_t cap[64] = {};
  if (dev < 0 || dev >= 64) return 0;
  if (!cap[dev]) {
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
      cudaGetLastError();
      return 0;
    }
    cap[dev] = tot / 4;
  }
  return cap[dev];
}
void cache_release(int dev) {
  std::vector<void *> drop;
  {
    BlockCache &bc = block_cache();
    std::lock_guard<std::mutex> lk(bc.m);
    for (size_t i = 0; i < bc.blocks.size();) {
      if (bc.blocks[i].dev == dev) {
        drop.push_back(bc.blocks[i].p);
        bc.held[dev] -= bc.blocks[i].bytes;
        bc.blocks[i] = bc.blocks.back();
        bc.blocks.pop_back();
      } else {
        ++i;
      }
    }
  }
  for (void *p : drop) cudaFree(p);
}
}  // namespace

// A block of at least `bytes` (a cached one of at most 1/8 more, else new).
template <class P>
static cudaError_t ctx_malloc(pdfs_ctx *c, P **out, size_t bytes) {
  const int dev = c->dev;
  if (dev >= 0 && dev < 64) {
    BlockCache &bc = block_cache();
    std::lock_guard<std::mutex> lk(bc.m);
    int best = -1;
    for (size_t i = 0; i < bc.blocks.size(); ++i) {
      const CachedBlock &b = bc.blocks[i];
      if (b.dev == dev && b.bytes >= bytes && b.bytes - bytes <= bytes / 8 &&
          (best < 0 || b.bytes < bc.blocks[best].bytes))
        best = (int)i;
    }
    if (best >= 0) {
      *out = reinterpret_cast<P *>(bc.blocks[best].p);
      bc.held[dev] -= bc.blocks[best].bytes;
      bc.blocks[best] = bc.blocks.back();
      bc.blocks.pop_back();
      return cudaSuccess;
    }
  }
  void *p = nullptr;
  cudaError_t e = cudaMalloc(&p, bytes);
  if (e == cudaErrorMemoryAllocation) {  // give the cached blocks back and try once more
    cudaGetLastError();
    cache_release(dev);
    e = cudaMalloc(&p, bytes);
  }
  *out = reinterpret_cast<P *>(p);
  return e;
}
// Returns an idle block of `bytes` to the cache (or to the device when the
// cache is full).
static void ctx_free(pdfs_ctx *c, void *p, size_t bytes) {
  if (!p) return;
  const int dev = c->dev;
  if (dev >= 0 && dev < 64) {
    const size_t cap = cache_cap(dev);
    BlockCache &bc = block_cache();
    std::lock_guard<std::mutex> lk(bc.m);
    if (bc.held[dev] + bytes <= cap) {
      bc.blocks.push_back({dev, p, bytes});
      bc.held[dev] += bytes;
      return;
    }
  }
  cudaFree(p);
}

extern "C" int pdfs_release_cached(int device) {
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return PDFS_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= ndev) return PDFS_ERR_INVALID;
  CK(cudaSetDevice(device));
  cache_release(device);
  return PDFS_OK;
}

static int validate(const pdfs_grid *g, const pdfs_opts *o) {
  if (!g || !o) return PDFS_ERR_INVALID;
  if (g->nx < 1 || g->ny < 1 || g->nz < 1) return PDFS_ERR_INVALID;
  if ((long long)g->nx + 2 > (1 << 20) || (long long)g->ny + 2 > 65535 || (long long)g->nz + 2 > 65535)
    return PDFS_ERR_INVALID;
  if (!(g->dx > 0) || !(g->dy > 0) || !(g->dz > 0) || !std::isfinite(g->dx) || !std::isfinite(g->dy) ||
      !std::isfinite(g->dz))
    return PDFS_ERR_INVALID;
  if (o->precision < 0 || o->precision > 2 || o->arith < 0 || o->arith > 3 || o->freeze < 0 || o->freeze > 1 ||
      o->scheduler < 0 || o->scheduler > 3 || o->tol < 0 || !std::isfinite(o->tol) || o->fixed_sweeps < 0 ||
      o->max_sweeps < 0 || o->first_ordering < 0 || o->first_ordering > 8)
    return PDFS_ERR_INVALID;
  const int t32 = o->tile & 0xff, t64 = (o->tile >> 8) & 0xff;
  if (t32 > tile_count32() || t64 > tile_count64()) return PDFS_ERR_INVALID;
  // FP64 kernels: columns 1 and 4 for the mixed arithmetic; 1-3 for the
  // reference one (polish: 1-2); 1-4 for the fast one (polish: 1, 2, 4);
  // bricks (5: 16 x 16 x 16, 7: 16 x 16 x 32) and pencils (6) for every
  // arithmetic; FP32 pairs on bricks and pencils only
  if ((t64 == 9 || t64 == 10) && o->arith != PDFS_ARITH_PAIR) return PDFS_ERR_INVALID;  // lane columns: pairs only
  if (o->arith == PDFS_ARITH_PAIR) {
    if (t64 != 0 && t64 < 5) return PDFS_ERR_INVALID;  // FP32 pairs: bricks, pencils and lane columns
  } else if (o->arith == PDFS_ARITH_MIXED) {
    if (t64 == 2 || t64 == 3) return PDFS_ERR_INVALID;
  } else {
    if (t64 == 4 && o->arith != PDFS_ARITH_FAST) return PDFS_ERR_INVALID;
    if (o->precision == PDFS_PREC_FP32_POLISH64 && t64 == 3) return PDFS_ERR_INVALID;
  }
  if (o->scheduler == PDFS_SCHED_LEARNED && !o->mlp_weights && !default_mlp_blob()) return PDFS_ERR_INVALID;
  return PDFS_OK;
}

// Default tile choice (pdfs_autotune may override through opts.tile).
// FP32: 16 x 16 pencils (tile 10: 3.6 ms per 768^3 sweep, against 3.9 ms for
// 16 x 16 x 32 bricks and 7.9 ms for the best column tile); their masked
// sweeps run on 16 x 16 x 32 bricks.
// FP64: pencils (tile 6) for every arithmetic: 6.9 ms per 768^3 pair polish
// sweep, against 8.1 ms for 16 x 16 x 16 bricks and 15.9 ms for mixed 32 x 6
// columns; 51 ms per plain fast-arithmetic sweep against 55 ms for 32 x 4
// columns (the reference arithmetic is even: both are FP64-pipe-bound).
// The lane-column tiles (FP32 12/13, pairs 9/10) measured 6.1 / 3.7 ms per
// FP32 sweep and 26.6 / 11.6 ms per pair polish sweep (8 / 4 rows): they stay
// selectable (and autotuned), not the default.
static void pick_tiles(pdfs_ctx *c) {
  const int t32 = c->o.tile & 0xff, t64 = (c->o.tile >> 8) & 0xff;
  c->t32 = t32 ? t32 : 10;
  c->t64 = t64 ? t64 : 6;
}

extern "C" int pdfs_ctx_create(const pdfs_grid *g, const pdfs_opts *o_in, pdfs_ctx **out) {
  if (!out) return PDFS_ERR_INVALID;
  *out = nullptr;
  pdfs_opts o;
  if (o_in)
    o = *o_in;
  else
    pdfs_default_opts(&o);
  int s = validate(g, &o);
  if (s) return s;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return PDFS_ERR_NO_DEVICE;
  }
  if (o.device < 0 || o.device >= ndev) return PDFS_ERR_INVALID;
  const auto t_start = std::chrono::steady_clock::now();
  CK(cudaSetDevice(o.device));
  pdfs_ctx *c = new pdfs_ctx();
  c->g = *g;
  c->o = o;
  c->dev = o.device;
  pick_tiles(c);
  const TileShape s32 = tile32(c->t32), s64 = tile64(c->t64);
  // bricks and pencils (c == 0) index from the halo node; columns from the
  // interior; lane-column tiles use the z-column layout
  c->L32 = s32.lc ? make_layout_zc(*g, s32.lc, 4) : make_layout(*g, s32.tx, s32.ty, 4, s32.c == 0 ? 0 : -1);
  c->L64 = s64.lc ? make_layout_zc(*g, s64.lc, 8) : make_layout(*g, s64.tx, s64.ty, 8, s64.c == 0 ? 0 : -1);
  c->M = make_mask_layout(*g);
  int rc = PDFS_OK;
  auto fail = [&](cudaError_t e) {
    rc = cuda_status(e);
    pdfs_ctx_destroy(c);
    return rc;
  };
  std::vector<std::pair<const char *, std::chrono::steady_clock::time_point>> marks;
  auto mark = [&](const char *what) {
    if (verbose(o)) marks.emplace_back(what, std::chrono::steady_clock::now());
  };
  cudaError_t e;
  if ((e = cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, c->dev)) != cudaSuccess) return fail(e);
  if ((e = cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking)) != cudaSuccess) return fail(e);
  mark("stream");
  // Host tables first, then every device buffer of the context carved from
  // one allocation (a batch creates hundreds of contexts: one allocation, or
  // one cached block, per context keeps their set-up short).
  c->nbx = (g->nx + 7) / 8;
  c->nby = (g->ny + 7) / 8;
  c->nbz = (g->nz + 7) / 8;
  c->nblocks = (long long)c->nbx * c->nby * c->nbz;
  std::vector<uint16_t> wb;
  if (o.scheduler == PDFS_SCHED_LEARNED) {
    const float *blob = o.mlp_weights ? o.mlp_weights : default_mlp_blob();
    wb.resize(PDFS_MLP_PARAMS);
    for (int i = 0; i < PDFS_MLP_PARAMS; ++i) {  // bf16 values: the upper half of the float
      uint32_t u;
      std::memcpy(&u, &blob[i], 4);
      wb[i] = (uint16_t)(u >> 16);
    }
    c->mlp_thr = blob[PDFS_MLP_PARAMS];
  }
  // brick tiles: ticket orders and the completion flags (epoch 0 = never)
  std::vector<int> bo[2];
  size_t nflags = 0;
  for (int k = 0; k < 2; ++k) {
    const TileShape ts = k ? s64 : s32;
    if (ts.bz == 0) continue;
    int *nt = k ? c->nt64 : c->nt32;
    nt[0] = (g->nx + ts.tx - 1) / ts.tx;
    nt[1] = (g->ny + ts.ty - 1) / ts.ty;
    nt[2] = (g->nz + ts.bz - 1) / ts.bz;
    bo[k] = brick_order(nt[0], nt[1], nt[2]);
    nflags = std::max(nflags, bo[k].size());
  }
  mark("brick orders");
  const std::vector<int> w32 = wavefront_order(c->L32.ncx, c->L32.ncy, c->L32.tx, c->L32.ty),
                         w64 = wavefront_order(c->L64.ncx, c->L64.ncy, c->L64.tx, c->L64.ty);
  std::vector<int> lo32, lo64;
  if (s32.lc) lo32 = lc_order(c->L32.ncx, c->L32.ncy, s32.lc);
  if (s64.lc) lo64 = lc_order(c->L64.ncx, c->L64.ncy, s64.lc);
  mark("columns");
  // lane-column tiles: per tile, row R-1's face for every traversal step (32
  // lanes); per tile column, lane 30's face by (ly + 32, step); FP32 values
  // take one tagged word, pairs two
  size_t lc_y = 0, lc_x = 0;
  for (int k = 0; k < 2; ++k) {
    const TileShape ts = k ? s64 : s32;
    if (!ts.lc) continue;
    const Layout &L = k ? c->L64 : c->L32;
    const size_t wv = k ? 2 : 1;
    lc_y = std::max(lc_y, (size_t)L.ncx * L.ncy * (size_t)L.T * 32 * wv);
    lc_x = std::max(lc_x, (size_t)L.ncx * (size_t)(ts.lc * L.ncy + 2) * (size_t)L.T * wv);
  }
  // per-row progress words and face mailboxes, sized for the larger of the two layouts
  {
    const int nb = mailbox_chunks(g->nz) * kMailboxChunk;
    size_t prog = 0, mb = 0;
    for (int k = 0; k < 2; ++k) {
      const Layout &L = k ? c->L64 : c->L32;
      const size_t ncol = (size_t)L.ncx * L.ncy;
      prog = std::max(prog, ncol * (size_t)L.ty);
      mb = std::max(mb, ncol * (size_t)nb * (size_t)(L.tx + L.ty) * (size_t)L.esize);
    }
    c->progress_ints = prog;
    c->mailbox_bytes = mb;
  }
  // pencils: two faces of prow diagonals x 16 entries x 2 words per pencil
  // (tag 0 never matches: epochs start at 1)
  size_t pmail_words = 0;
  if (s32.pencil || s64.pencil) {
    c->prow = g->nz + 15;
    pmail_words = (size_t)((g->nx + 15) / 16) * ((g->ny + 15) / 16) * 2 * (size_t)c->prow * 16 * 2;
  }
  std::vector<std::pair<void **, size_t>> plan;
  auto want = [&](auto **p, size_t bytes) {
    if (bytes) plan.emplace_back(reinterpret_cast<void **>(p), bytes);
  };
  const bool need32 = o.precision != PDFS_PREC_FP64;
  want(&c->in64, c->L64.elems * 8);  // the FP64 input is always resident
  if (o.precision != PDFS_PREC_FP32) want(&c->u64, c->L64.elems * 8);
  if (o.precision == PDFS_PREC_FP32_POLISH64) {  // polish: the per-block cap bounds
    want(&c->bcap64, (size_t)c->nblocks * 8);
    want(&c->bcap32, (size_t)c->nblocks * 4);
  }
  if (need32) want(&c->u32, c->L32.elems * 4);
  want(&c->fmask, c->M.words * 4);
  want(&c->progress, c->progress_ints * 4);
  want(&c->mailbox, c->mailbox_bytes);
  want(&c->ticket, 16);
  want(&c->dstat, sizeof(DevStatus));
  want(&c->bchg, (size_t)c->nblocks * kRing * 4);
  want(&c->bact, (size_t)c->nblocks);
  if (need32) want(&c->omask, (size_t)c->nblocks);  // the polish's octant masks (pdfs_ctx_orderings)
  // octant rounds: FP32 on 16 x 16 x 32 bricks, the polish on 16 x 16 x 16 ones
  c->oct32_ok = o.precision != PDFS_PREC_FP64 && s32.bz == 32 && s32.ty == 16 && s32.tx == 16;
  c->oct64_ok = o.precision == PDFS_PREC_FP32_POLISH64 && s64.bz == 16 && s64.ty == 16 && s64.tx == 16;
  if (c->oct32_ok || c->oct64_ok) {
    want(&c->toct, (size_t)std::max(octant_scratch_ints(c->nt32[0], c->nt32[1], c->nt32[2]),
                                    octant_scratch_ints(c->nt64[0], c->nt64[1], c->nt64[2])) * 4);
    want(&c->ochg, kOctWords * 8);
  }
  if (!wb.empty()) {
    want(&c->mlp_w, PDFS_MLP_PARAMS * 2);
    want(&c->bmin, (size_t)c->nblocks * 4);
  }
  want(&c->tord32, bo[0].size() * 4);
  want(&c->tord64, bo[1].size() * 4);
  want(&c->tflag, nflags * 4);
  want(&c->tact, nflags);
  want(&c->tsparse, nflags ? (nflags + 1) * 4 : 0);
  want(&c->pmail, pmail_words * 8);
  want(&c->order32, w32.size() * 4);
  want(&c->order64, w64.size() * 4);
  want(&c->lcord32, lo32.size() * 4);
  want(&c->lcord64, lo64.size() * 4);
  want(&c->lc_ymail, lc_y * 8);
  want(&c->lc_xmail, lc_x * 8);
  {
    size_t total = 0;
    for (auto &r : plan) total += (r.second + 255) & ~(size_t)255;  // 256-byte aligned pieces
    if ((e = ctx_malloc(c, &c->arena, total)) != cudaSuccess) return fail(e);
    c->arena_bytes = total;
    char *p = reinterpret_cast<char *>(c->arena);
    for (auto &r : plan) {
      *r.first = p;
      p += (r.second + 255) & ~(size_t)255;
    }
  }
  mark("allocation");
  if ((e = cudaHostAlloc(&c->hstat, sizeof(DevStatus), cudaHostAllocDefault)) != cudaSuccess) return fail(e);
  if (!wb.empty() &&
      (e = cudaMemcpyAsync(c->mlp_w, wb.data(), PDFS_MLP_PARAMS * 2, cudaMemcpyHostToDevice, c->st)) != cudaSuccess)
    return fail(e);
  for (int k = 0; k < 2; ++k) {
    int *dst = k ? c->tord64 : c->tord32;
    if (!bo[k].empty() &&
        (e = cudaMemcpyAsync(dst, bo[k].data(), bo[k].size() * 4, cudaMemcpyHostToDevice, c->st)) != cudaSuccess)
      return fail(e);
  }
  if (nflags && (e = cudaMemsetAsync(c->tflag, 0, nflags * 4, c->st)) != cudaSuccess) return fail(e);
  if (pmail_words && (e = cudaMemsetAsync(c->pmail, 0, pmail_words * 8, c->st)) != cudaSuccess) return fail(e);
  // lane-column mailboxes: tag 0 never matches (epochs start at 1)
  if (lc_y && (e = cudaMemsetAsync(c->lc_ymail, 0, lc_y * 8, c->st)) != cudaSuccess) return fail(e);
  if (lc_x && (e = cudaMemsetAsync(c->lc_xmail, 0, lc_x * 8, c->st)) != cudaSuccess) return fail(e);
  for (int k = 0; k < 2; ++k) {
    const std::vector<int> &lo = k ? lo64 : lo32;
    int *dst = k ? c->lcord64 : c->lcord32;
    if (!lo.empty() && (e = cudaMemcpyAsync(dst, lo.data(), lo.size() * 4, cudaMemcpyHostToDevice, c->st)) != cudaSuccess)
      return fail(e);
  }
  if ((e = cudaMemcpyAsync(c->order32, w32.data(), w32.size() * 4, cudaMemcpyHostToDevice, c->st)) != cudaSuccess)
    return fail(e);
  if ((e = cudaMemcpyAsync(c->order64, w64.data(), w64.size() * 4, cudaMemcpyHostToDevice, c->st)) != cudaSuccess)
    return fail(e);
  const auto t_alloc = std::chrono::steady_clock::now();
  // padding outside the halo-padded grid is never written by the sweeps; fill it with +inf once
  if (c->in64) k_fill<double><<<2 * c->sms, 256, 0, c->st>>>(c->in64, c->L64.elems, INFINITY);
  if (c->u64) k_fill<double><<<2 * c->sms, 256, 0, c->st>>>(c->u64, c->L64.elems, INFINITY);
  if (c->u32) k_fill<float><<<2 * c->sms, 256, 0, c->st>>>(c->u32, c->L32.elems, INFINITY);
  if ((e = cudaMemsetAsync(c->fmask, 0, c->M.words * 4, c->st)) != cudaSuccess) return fail(e);
  if ((e = cudaEventCreate(&c->e0)) != cudaSuccess) return fail(e);
  if ((e = cudaEventCreate(&c->e1)) != cudaSuccess) return fail(e);
  if ((e = cudaEventCreate(&c->k0)) != cudaSuccess) return fail(e);
  if ((e = cudaEventCreate(&c->k1)) != cudaSuccess) return fail(e);
  if ((e = cudaEventCreate(&c->q0)) != cudaSuccess) return fail(e);
  if ((e = cudaEventCreate(&c->q1)) != cudaSuccess) return fail(e);
  if ((e = cudaEventCreate(&c->r0)) != cudaSuccess) return fail(e);
  if ((e = cudaEventCreate(&c->r1)) != cudaSuccess) return fail(e);
  if ((e = cudaStreamSynchronize(c->st)) != cudaSuccess) return fail(e);
  if (verbose(o)) {
    const auto t_end = std::chrono::steady_clock::now();
    auto ms = [](auto a, auto b) { return std::chrono::duration<double, std::milli>(b - a).count(); };
    fprintf(stderr, "pdfs: create %.1f ms (", ms(t_start, t_end));
    auto t = t_start;
    for (auto &m : marks) {
      fprintf(stderr, "%s %.1f, ", m.first, ms(t, m.second));
      t = m.second;
    }
    fprintf(stderr, "tables %.1f, fills %.1f)\n", ms(t, t_alloc), ms(t_alloc, t_end));
  }
  *out = c;
  return PDFS_OK;
}

extern "C" void pdfs_ctx_destroy(pdfs_ctx *c) {
  if (!c) return;
  cudaSetDevice(c->dev);
  // every block is idle before it goes back to the cache
  if (c->st2) cudaStreamSynchronize(c->st2);
  if (c->st) cudaStreamSynchronize(c->st);
  ctx_free(c, c->arena, c->arena_bytes);
  ctx_free(c, c->stage, c->stage_bytes);
  if (c->hstat) cudaFreeHost(c->hstat);
  if (c->e0) cudaEventDestroy(c->e0);
  if (c->e1) cudaEventDestroy(c->e1);
  if (c->k0) cudaEventDestroy(c->k0);
  if (c->k1) cudaEventDestroy(c->k1);
  if (c->q0) cudaEventDestroy(c->q0);
  if (c->q1) cudaEventDestroy(c->q1);
  if (c->r0) cudaEventDestroy(c->r0);
  if (c->r1) cudaEventDestroy(c->r1);
  for (cudaEvent_t ev : c->slab_ev)
    if (ev) cudaEventDestroy(ev);
  if (c->st2) cudaStreamDestroy(c->st2);
  if (c->st) cudaStreamDestroy(c->st);
  cudaGetLastError();
  delete c;
}

static size_t ref_nodes(const pdfs_grid &g) { return (size_t)(g.nx + 2) * (g.ny + 2) * (g.nz + 2); }

// The stage holds a field in the reference layout and, after it, a mask.
static int ensure_stage(pdfs_ctx *c) {
  const size_t b = ref_nodes(c->g) * 9;
  if (c->stage_bytes >= b) return PDFS_OK;
  if (c->stage) CK(cudaStreamSynchronize(c->st));  // the old stage is idle
  ctx_free(c, c->stage, c->stage_bytes);
  c->stage = nullptr;
  c->stage_bytes = 0;
  CK(ctx_malloc(c, &c->stage, b));
  c->stage_bytes = b;
  return PDFS_OK;
}

// Planes per slab of the load / store pipelines: at most kSlabs slabs, and
// one slab (no pipeline) for fields under 256 MB, where the layout kernels
// that a pipeline would hide take a few tens of microseconds.
static int slab_planes(const pdfs_grid &g) {
  const int planes = g.nz + 2;
  if (ref_nodes(g) * 8 < (256u << 20)) return planes;
  return std::max(16, (planes + pdfs_ctx::kSlabs - 1) / pdfs_ctx::kSlabs);
}

// The pipeline's second stream and slab events, made on first use.
static int ensure_pipeline(pdfs_ctx *c) {
  if (c->st2) return PDFS_OK;
  CK(cudaStreamCreateWithFlags(&c->st2, cudaStreamNonBlocking));
  for (cudaEvent_t &ev : c->slab_ev) CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  return PDFS_OK;
}

static double ms_between(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0;
  cudaEventElapsedTime(&ms, a, b);
  return ms;
}

// Host -> device.  The mask goes first (the cap bounds need it), then the
// field in z-slabs on c->st; c->st2 packs each slab as it lands and takes the
// cap bounds of the 8^3 blocks whose planes are all packed, so that only the
// last slab's kernels trail the copies.
static int load_impl(pdfs_ctx *c, const double *field, const uint8_t *frozen, double *ms_h2d) {
  if (!c || !field) return PDFS_ERR_INVALID;
  CK(cudaSetDevice(c->dev));
  const pdfs_grid &g = c->g;
  const size_t n = ref_nodes(g);
  const size_t plane = (size_t)(g.nx + 2) * (g.ny + 2);
  const bool dev_field = is_device_ptr(field);
  const bool use_mask = c->o.freeze == PDFS_FREEZE_MASK && frozen;
  const bool dev_mask = use_mask && is_device_ptr(frozen);
  const auto t_start = std::chrono::steady_clock::now();
  int s;
  if (!dev_field || (use_mask && !dev_mask)) {
    if ((s = ensure_stage(c))) return s;
  }
  const double *src = dev_field ? field : (const double *)c->stage;
  const int planes = g.nz + 2, per = dev_field ? planes : slab_planes(g);
  const bool pipe = per < planes;  // else every step runs on c->st
  if (pipe && (s = ensure_pipeline(c))) return s;
  cudaStream_t ks = pipe ? c->st2 : c->st;  // the layout kernels' stream
  auto handoff = [&](cudaEvent_t ev) -> cudaError_t {  // ks waits for the copies issued so far
    if (!pipe) return cudaSuccess;
    cudaError_t e = cudaEventRecord(ev, c->st);
    return e != cudaSuccess ? e : cudaStreamWaitEvent(ks, ev, 0);
  };
  const auto t_stage = std::chrono::steady_clock::now();
  CK(cudaEventRecord(c->e0, c->st));
  if (pipe) CK(cudaStreamWaitEvent(ks, c->e0, 0));
  CK(cudaMemsetAsync(c->fmask, 0, c->M.words * 4, ks));
  if (use_mask) {
    const uint8_t *m = frozen;
    if (!dev_mask) {
      m = (const uint8_t *)c->stage + n * 8;
      CK(cudaMemcpyAsync((void *)m, frozen, n, cudaMemcpyHostToDevice, c->st));
      CK(handoff(c->slab_ev[pdfs_ctx::kSlabs]));
    }
    dim3 mg(g.ny, g.nz);
    k_pack_mask<<<mg, 64, 0, ks>>>(m, c->fmask, c->M, g.nx, g.ny);
    CK(cudaGetLastError());
  }
  const long long blocks_per_z = (long long)c->nbx * c->nby;
  int bz_done = 0;
  for (int z0 = 0, k = 0; z0 < planes; z0 += per, ++k) {
    const int z1 = std::min(planes, z0 + per);
    if (!dev_field) {
      CK(cudaMemcpyAsync((char *)c->stage + z0 * plane * 8, field + z0 * plane, (size_t)(z1 - z0) * plane * 8,
                         cudaMemcpyHostToDevice, c->st));
      CK(handoff(c->slab_ev[k]));
    }
    dim3 grid(g.ny + 2, z1 - z0);
    k_pack<double><<<grid, 128, 0, ks>>>(src, c->in64, g.nx, g.ny, c->L64, z0);
    CK(cudaGetLastError());
    if (c->bcap64) {
      // block bz holds planes 8 bz + 1 .. min(8 bz + 8, nz): complete once plane z1 - 1 is packed
      const int bz_ready = z1 >= g.nz + 1 ? c->nbz : std::min(c->nbz, (z1 - 1) / 8);
      if (bz_ready > bz_done) {
        k_block_capmin<<<8 * c->sms, 256, 0, ks>>>(c->in64, c->L64, use_mask ? c->fmask : nullptr, c->M, g.nx,
                                                        g.ny, g.nz, c->nbx, c->nby, bz_done * blocks_per_z,
                                                        bz_ready * blocks_per_z, c->bcap64, c->bcap32);
        CK(cudaGetLastError());
        bz_done = bz_ready;
      }
    }
  }
  CK(cudaEventRecord(c->e1, ks));
  if (pipe) CK(cudaStreamWaitEvent(c->st, c->e1, 0));
  CK(cudaStreamSynchronize(c->st));
  if (ms_h2d) *ms_h2d = ms_between(c->e0, c->e1);
  if (verbose(c->o))
    fprintf(stderr, "pdfs: load %.1f ms (stage allocation %.1f, copies and layout kernels %.1f)\n",
            std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count(),
            std::chrono::duration<double, std::milli>(t_stage - t_start).count(), ms_between(c->e0, c->e1));
  c->has_mask = use_mask;
  c->loaded = true;
  c->last_prec = -1;
  return PDFS_OK;
}

extern "C" int pdfs_ctx_load(pdfs_ctx *c, const double *field, const uint8_t *frozen) {
  return load_impl(c, field, frozen, nullptr);
}

// One sweep of ordering sn on the FP32 (which = 0) or FP64 (1 min, 2 replace)
// working field.  *chg receives the sweep's max change (relative for FP32,
// absolute for FP64).  active: per-block visit mask or nullptr.
// The sweep arguments of context c: which 0 = FP32, 1 = FP64 min, 2 = FP64 replace.
void pdfs::fill_sweep_args(const pdfs_ctx *c, int which, int sn, const uint8_t *active, unsigned int *blk_chg,
                           SweepArgs *out) {
  const pdfs_grid &g = c->g;
  const bool f32 = which == 0;
  const Layout &L = f32 ? c->L32 : c->L64;
  SweepArgs &a = *out;
  std::memset(&a, 0, sizeof(a));
  a.u = f32 ? (void *)c->u32 : (void *)c->u64;
  a.fmask = c->has_mask ? c->fmask : nullptr;
  a.px = L.px;
  a.plane = L.plane;
  a.mask_fy = c->M.fy;
  a.mask_fw = c->M.fw;
  a.nx = g.nx;
  a.ny = g.ny;
  a.nz = g.nz;
  ordering_signs(sn, &a.sx, &a.sy, &a.sz);
  a.ncx = L.ncx;
  a.ncy = L.ncy;
  a.order = f32 ? c->order32 : c->order64;
  a.prog = c->progress;
  a.nbands = mailbox_chunks(g.nz);
  a.xstride = (long long)a.nbands * kMailboxChunk * L.ty;
  a.ystride = (long long)a.nbands * kMailboxChunk * L.tx;
  a.xbox = c->mailbox;
  a.ybox = (char *)c->mailbox + (size_t)L.ncx * L.ncy * a.xstride * L.esize;
  a.ticket = c->ticket;
  a.err = c->dstat->err;
  a.maxchg = &c->dstat->chg;
  a.blk_active = active;
  a.blk_chg = blk_chg;
  a.cap = which == 2 ? (const void *)c->in64 : nullptr;  // FP64; pair kernels convert the rare cap they read
  a.bcap64 = which == 2 ? c->bcap64 : nullptr;
  a.bcap32 = which == 2 ? c->bcap32 : nullptr;
  a.nbx = c->nbx;
  a.nby = c->nby;
  a.nbz = c->nbz;
  a.hmin = (float)std::min(g.dx, std::min(g.dy, g.dz));
  const int *nt = f32 ? c->nt32 : c->nt64;
  a.tflag = c->tflag;
  a.torder = f32 ? c->tord32 : c->tord64;
  a.tact = active ? c->tact : nullptr;
  a.nticket = active ? c->tsparse : nullptr;
  a.ntx = nt[0];
  a.nty = nt[1];
  a.ntz = nt[2];
  a.epoch = c->epoch;
  a.pmail = c->pmail;
  a.prow = c->prow;
  long long wait_ms = c->o.spin_limit > 0 ? c->o.spin_limit : 4000;
  if (getenv("PDFS_WAIT_MS")) wait_ms = atoll(getenv("PDFS_WAIT_MS"));
  a.wait_cycles = wait_ms * 1000000LL * 21 / 10;  // at most 2.07 GHz: never shorter than wait_ms
  a.poison_col = getenv("PDFS_TEST_POISON_COLUMN") ? atoi(getenv("PDFS_TEST_POISON_COLUMN")) : -1;
  const double h[3] = {g.dx, g.dy, g.dz};
  for (int i = 0; i < 3; ++i) {
    a.k64.h[i] = h[i];
    a.k64.h2[i] = h[i] * h[i];
    a.k64.q[i] = 1.0 / (h[i] * h[i]);
    a.k32.h[i] = (float)h[i];
    a.k32.q[i] = (float)(1.0 / (h[i] * h[i]));
  }
  a.k64.qsum = a.k64.q[0] + a.k64.q[1] + a.k64.q[2];
  a.k64.iqsum = 1.0 / a.k64.qsum;
  a.k32.iqsum = (float)a.k64.iqsum;
  a.k32.iso_h = (float)g.dx;
  a.k32.iso_2h2 = (float)(2.0 * g.dx * g.dx);
  a.k32.iso_h2 = (float)(g.dx * g.dx);
}

static int run_sweep(pdfs_ctx *c, int which, int sn, const uint8_t *active, unsigned int *blk_chg, double *chg);
static int octant_round(pdfs_ctx *c, int which, int first, int nsw, unsigned full, double *chg, long long *active,
                        long long *updates);
int pdfs::ctx_sweep_once(pdfs_ctx *c, int which, int sn, const uint8_t *active, unsigned int *blk_chg, double *chg) {
  return run_sweep(c, which, sn, active, blk_chg, chg);
}

// The lane-column kernel's arguments from the sweep arguments a of context c.
static void fill_lc_args(const pdfs_ctx *c, int which, const SweepArgs &a, LcArgs *out) {
  const bool f32 = which == 0;
  const Layout &L = f32 ? c->L32 : c->L64;
  LcArgs &l = *out;
  std::memset(&l, 0, sizeof(l));
  l.u = a.u;
  l.cap = which == 2 ? c->in64 : nullptr;
  l.bcap32 = which == 2 ? c->bcap32 : nullptr;
  l.cxp = L.px;
  l.qz = L.qz;
  l.q_last = L.q_last;
  l.T = L.T;
  l.nx = a.nx;
  l.ny = a.ny;
  l.nz = a.nz;
  l.sx = a.sx;
  l.sy = a.sy;
  l.sz = a.sz;
  l.ntx = L.ncx;
  l.nty = L.ncy;
  l.order = f32 ? c->lcord32 : c->lcord64;
  l.ticket = a.ticket;
  l.err = a.err;
  l.maxchg = a.maxchg;
  l.hmin = a.hmin;
  l.ymail = c->lc_ymail;
  l.xmail = c->lc_xmail;
  l.xrows = L.ty * L.ncy + 2;
  l.epoch = a.epoch;
  l.wait_cycles = a.wait_cycles;
  l.poison_tile = a.poison_col;
  l.blk_active = a.blk_active;
  l.blk_chg = a.blk_chg;
  l.nbx = a.nbx;
  l.nby = a.nby;
  l.nbz = a.nbz;
  l.k32 = a.k32;
}

static int run_sweep(pdfs_ctx *c, int which, int sn, const uint8_t *active, unsigned int *blk_chg, double *chg) {
  const pdfs_grid &g = c->g;
  const bool f32 = which == 0;
  const Layout &L = f32 ? c->L32 : c->L64;
  SweepArgs a;
  fill_sweep_args(c, which, sn, active, blk_chg, &a);
  const bool iso = g.dx == g.dy && g.dy == g.dz;

  const int tile = f32 ? c->t32 : c->t64;
  const TileShape ts = f32 ? tile32(tile) : tile64(tile);
  if (ts.lc) {
    // lane-column tiles: every sweep, with or without a block mask
    CK(cudaMemsetAsync(c->dstat, 0, offsetof(DevStatus, active_blocks), c->st));
    if (blk_chg) CK(cudaMemsetAsync(blk_chg, 0, (size_t)c->nblocks * 4, c->st));
    CK(cudaMemsetAsync(c->ticket, 0, 4, c->st));
    a.epoch = ++c->epoch;  // mailbox words of every earlier sweep carry a smaller tag
    LcArgs l;
    fill_lc_args(c, which, a, &l);
    int grid = 0;
    CK(cudaEventRecord(c->k0, c->st));
    CK(launch_sweep_lanecol(f32 ? 0 : (which == 2 ? 2 : 1), ts.lc, iso, l, c->sms, c->st, &grid));
    CK(cudaEventRecord(c->k1, c->st));
    CK(cudaMemcpyAsync(c->hstat, c->dstat, sizeof(DevStatus), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    c->kern_ms += ms_between(c->k0, c->k1);
    c->launches++;
    if (c->hstat->err[0]) {
      if (verbose(c->o))
        fprintf(stderr, "pdfs: sweep sn=%d device error %d (tile %d)\n", sn, c->hstat->err[0], c->hstat->err[2]);
      return c->hstat->err[0] == DEV_ERR_TIMEOUT ? PDFS_ERR_TIMEOUT : PDFS_ERR_CUDA;
    }
    if (chg) {
      if (f32) {
        unsigned int b = (unsigned int)c->hstat->chg;
        float f;
        std::memcpy(&f, &b, 4);
        *chg = f;
      } else {
        double d;
        std::memcpy(&d, &c->hstat->chg, 8);
        *chg = d;
      }
    }
    return PDFS_OK;
  }
  // pencils sweep unmasked sweeps; a block mask or block-change output goes to bricks
  // (pencils that recorded block changes measured no faster: 37.4 against 36.9 ms
  // for the 8 recording sweeps of the 768^3 headline solve)
  const bool pencil = ts.pencil && !active && !blk_chg;
  if (ts.bz == 0 || pencil) CK(cudaMemsetAsync(c->progress, 0, (size_t)L.ncx * L.ncy * L.ty * 4, c->st));
  CK(cudaMemsetAsync(c->dstat, 0, offsetof(DevStatus, active_blocks), c->st));
  if (blk_chg) CK(cudaMemsetAsync(blk_chg, 0, (size_t)c->nblocks * 4, c->st));
  CK(cudaMemsetAsync(c->ticket, 0, 4, c->st));
  const int arith = c->o.arith == PDFS_ARITH_REFERENCE ? ARITH_REF
                    : c->o.arith == PDFS_ARITH_MIXED   ? ARITH_MIXED
                    : c->o.arith == PDFS_ARITH_PAIR    ? ARITH_PAIR
                                                       : ARITH_FAST;
  int grid = 0;
  CK(cudaEventRecord(c->k0, c->st));
  if (pencil) {
    a.epoch = ++c->epoch;  // mailbox words of every earlier sweep carry a smaller tag
    CK(launch_sweep_pencils(which, arith, iso, a, L, c->sms, c->st, &grid));
  } else if (ts.bz > 0) {
    a.epoch = ++c->epoch;  // the flags of every earlier sweep are below it
    CK(launch_sweep_bricks(which, ts.ty, ts.bz, arith, iso, a, L, c->sms, c->st, &grid));
  } else {
    CK(launch_sweep(which, tile, arith, iso, a, L, which == 2 ? (const void *)c->in64 : nullptr, c->sms, c->st,
                    &grid));
  }
  CK(cudaEventRecord(c->k1, c->st));
  CK(cudaMemcpyAsync(c->hstat, c->dstat, sizeof(DevStatus), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  c->kern_ms += ms_between(c->k0, c->k1);
  c->launches++;
  if (c->hstat->err[0]) {
    if (verbose(c->o))
      fprintf(stderr, "pdfs: sweep sn=%d device error %d (column %d)\n", sn, c->hstat->err[0], c->hstat->err[2]);
    return c->hstat->err[0] == DEV_ERR_TIMEOUT ? PDFS_ERR_TIMEOUT : PDFS_ERR_CUDA;
  }
  if (chg) {
    if (f32) {
      unsigned int b = (unsigned int)c->hstat->chg;
      float f;
      std::memcpy(&f, &b, 4);
      *chg = f;
    } else {
      double d;
      std::memcpy(&d, &c->hstat->chg, 8);
      *chg = d;
    }
  }
  return PDFS_OK;
}

// A z-column working field from the input (FP32, or pairs) or, for pairs
// with from32, from the FP32 field: frozen nodes and the halo signed.
// Lane-column tiles take fields whose updated nodes are >= 0 (distances):
// a negative input there returns PDFS_ERR_INVALID (the pencil tiles take any sign).
template <class T>
static int zc_fill(pdfs_ctx *c, T *dst, const Layout &Ld, bool from32) {
  const pdfs_grid &g = c->g;
  int *neg = &c->dstat->err[3];
  CK(cudaMemsetAsync(neg, 0, 4, c->st));
  k_zc_fill<T><<<8 * c->sms, 256, 0, c->st>>>(dst, Ld, c->in64, c->L64, c->u32, c->L32, from32,
                                              c->has_mask ? c->fmask : nullptr, c->M, g.nx, g.ny, g.nz, neg);
  c->launches++;
  CK(cudaGetLastError());
  int h = 0;
  CK(cudaMemcpyAsync(&h, neg, 4, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  if (h) {
    if (verbose(c->o)) fprintf(stderr, "pdfs: lane-column tiles need a field >= 0 at the nodes they update\n");
    return PDFS_ERR_INVALID;
  }
  return PDFS_OK;
}

int pdfs::ctx_fp64_start(pdfs_ctx *c) {  // FP64 working field <- the input
  if (c->L64.zc) return zc_fill<double>(c, c->u64, c->L64, false);
  if (c->o.arith == PDFS_ARITH_PAIR) {
    k_to_pair<<<4 * c->sms, 256, 0, c->st>>>(c->in64, c->u64, c->L64.elems);
    c->launches++;
    CK(cudaGetLastError());
  } else {
    CK(cudaMemcpyAsync(c->u64, c->in64, c->L64.elems * 8, cudaMemcpyDeviceToDevice, c->st));
  }
  return PDFS_OK;
}

int pdfs::ctx_widen(pdfs_ctx *c) {
  const pdfs_grid &g = c->g;
  if (c->L64.zc) return zc_fill<double>(c, c->u64, c->L64, true);
  const unsigned grid = row_blocks(g);
  if (c->o.arith == PDFS_ARITH_PAIR) {
    k_widen_pair<<<grid, 32 * kRowWarps, 0, c->st>>>(c->u32, c->L32, c->in64, c->u64, c->L64,
                                          c->has_mask ? c->fmask : nullptr, c->M, g.nx, g.ny, g.nz);
    c->launches++;
    CK(cudaGetLastError());
    return PDFS_OK;
  }
  k_widen<<<grid, 32 * kRowWarps, 0, c->st>>>(c->u32, c->L32, c->in64, c->u64, c->L64, c->has_mask ? c->fmask : nullptr, c->M,
                                   g.nx, g.ny, g.nz);
  c->launches++;
  CK(cudaGetLastError());
  return PDFS_OK;
}

int pdfs::ctx_narrow(pdfs_ctx *c) {  // FP64 input -> FP32 working field
  const pdfs_grid &g = c->g;
  if (c->L32.zc) return zc_fill<float>(c, c->u32, c->L32, false);
  k_convert<double, float><<<row_blocks(g), 32 * kRowWarps, 0, c->st>>>(c->in64, c->L64, c->u32, c->L32, g.nx, g.ny,
                                                                         g.nz);
  c->launches++;
  CK(cudaGetLastError());
  return PDFS_OK;
}

extern "C" int pdfs_ctx_run(pdfs_ctx *c, pdfs_stats *stats) {
  if (!c || !c->loaded) return PDFS_ERR_INVALID;
  CK(cudaSetDevice(c->dev));
  const auto t0 = std::chrono::steady_clock::now();
  CK(cudaEventRecord(c->r0, c->st));
  pdfs_stats st;
  std::memset(&st, 0, sizeof(st));
  st.tile = c->t32 | (c->t64 << 8);
  c->launches = 0;
  const pdfs_opts &o = c->o;
  const pdfs_grid &g = c->g;
  const long long nodes = (long long)g.nx * g.ny * g.nz;
  const int max_sweeps = o.max_sweeps > 0 ? o.max_sweeps : 100000;
  const int first = o.first_ordering ? o.first_ordering - 1 : 0;
  int rc = PDFS_OK;
  double chg = 0.0;

  // One phase of sweeps (which: 0 FP32 min-update, 1 FP64 min-update, 2 FP64
  // replace-update).  tol bounds the phase's change metric.  With a
  // scheduler, the first round and every judging sweep visit all blocks;
  // the phase ends only at a full sweep whose change is <= tol.
  // FP32 + polish: the polish's full sweeps certify the fixed point, so the
  // FP32 phase may end on a quiet scheduled sweep (no judging sweep), and the
  // polish -- one full cycle and a certifying sweep -- visits every block.
  // (Scheduling the polish as well was measured: its changes are small and
  // spread, blocks skipped below tol drift, and the certifying sweeps kept
  // finding them -- 36 to 54 polish sweeps instead of 9 on the 768^3 grid.)
  const bool polish = o.precision == PDFS_PREC_FP32_POLISH64;
  auto phase = [&](int which, double tol, int *count, double *ms, double *kms) -> int {
    c->kern_ms = 0.0;
    CK(cudaEventRecord(c->e0, c->st));
    // PDFS_SCHED_OCTANT, FP32 phase: the first cycle as one unmasked round (8
    // full sweeps in one launch), then cycles as octant rounds over masks from
    // the field (at most three, until a round's last two sweeps change by at
    // most 16 x the phase tolerance)
    const bool oct32 = o.scheduler == PDFS_SCHED_OCTANT && which == 0 && o.fixed_sweeps == 0 && c->oct32_ok;
    const bool sched = o.scheduler != PDFS_SCHED_NONE && o.scheduler != PDFS_SCHED_OCTANT && o.fixed_sweeps == 0 &&
                       !(polish && which == 2);
    // the polish under a scheduler: its first cycle visits, in each ordering,
    // only the blocks that ordering matters to (octant masks of the FP32
    // result); full sweeps follow until one certifies
    const bool octant = o.scheduler != PDFS_SCHED_NONE && o.fixed_sweeps == 0 && polish && which == 2;
    const bool certify = !(polish && which == 0);  // must the phase end on a full sweep?
    const int nfull = 8;  // sweeps that visit every block before the scheduler starts
    const float thr = (float)tol;
    // per-block changes: ring slot cur = this sweep, (cur - k) mod kRing = k sweeps ago
    int cur = 0;
    if (sched) CK(cudaMemsetAsync(c->bchg, 0, (size_t)c->nblocks * kRing * 4, c->st));
    if (sched || octant) CK(cudaMemsetAsync(&c->dstat->sched_err, 0, 4, c->st));
    if (octant && !c->oct64_ok) {  // the masks of the one-launch-per-sweep path (the round computes its own)
      CK(octant_mask(c->u32, c->L32, c->has_mask ? c->fmask : nullptr, c->M, g, kOctSlack64, INFINITY, c->nbx,
                     c->nby, c->nbz, c->omask, c->st));
      c->launches++;
    }
    bool need_full = true;
    int s = 0;
    int oct_rounds = 0;
    bool oct_done = false;
    int band_sweep = -1;  // learned scheduler: the sweep of the last block-minimum pass
    for (;;) {
      const bool round64 = octant && s == 0 && c->oct64_ok && max_sweeps > 8;
      const bool full32 = oct32 && s == 0 && max_sweeps >= 8;
      const bool round32 = oct32 && s >= 8 && !oct_done && s + 8 < max_sweeps;
      if (round64 || round32 || full32) {
        // a cycle of 8 orderings in one launch, each on its octant mask (or on
        // every block).  (The polish's first certifying full sweep run as a
        // ninth sweep of its round was measured: the round grew by the 6.1 ms
        // of a full pencil sweep, 72.9 ms either way on the 768^3 grid.)
        const int nsw = 8;
        const unsigned full = full32 ? 0xffu : 0u;
        double ch8[kOctMax];
        long long nb_act = 0, upd = 0;
        const double kms0 = c->kern_ms;
        int r = octant_round(c, which, (first + s) % 8, nsw, full, ch8, &nb_act, &upd);
        if (r) return r;
        const int *nt = which == 0 ? c->nt32 : c->nt64;
        const long long bnodes = (long long)nt[0] * nt[1] * nt[2];
        if (verbose(o))
          for (int j = 0; j < nsw; ++j)
            fprintf(stderr, "pdfs: phase %d sweep %d sn=%d %s change=%.3e (one launch: %.3f ms for %d sweeps, "
                            "%lld of %lld brick visits)\n",
                    which, s + j, (first + s + j) % 8 + 1, ((full >> j) & 1u) ? "full, in round" : "octant",
                    ch8[j], c->kern_ms - kms0, nsw, nb_act, nsw * bnodes);
        st.voxel_updates += upd;
        if (which != 0) st.voxel_updates_fp64 += upd;
        chg = ch8[nsw - 1];
        s += nsw;
        if (full32) {
          st.full_sweeps += 8;
          // the sweep-by-sweep phase would have ended at its first sweep within tol
          bool quiet = false;
          for (int j = 0; j < 8; ++j) quiet = quiet || ch8[j] <= tol;
          if (quiet) break;
          continue;
        }
        (which == 0 ? st.ms_kern_masked_fp32 : st.ms_kern_masked_fp64) += c->kern_ms - kms0;
        (which == 0 ? st.updates_masked_fp32 : st.updates_masked_fp64) += upd;
        (which == 0 ? st.masked_sweeps_fp32 : st.masked_sweeps_fp64) += nsw;
        if (round32) {
          ++oct_rounds;
          const bool quiet = std::max(ch8[6], ch8[7]) <= 16.0 * tol;
          if (quiet || oct_rounds == 3) {
            if (!certify) break;  // the polish's full sweeps certify the fixed point
            oct_done = true;      // full sweeps follow until one is within tol
          }
        }
        continue;
      }
      if (o.fixed_sweeps > 0 && s >= o.fixed_sweeps) break;
      if (o.fixed_sweeps == 0 && s >= max_sweeps) {
        rc = PDFS_ERR_NOT_CONVERGED;
        break;
      }
      const int sn = (first + s) % 8 + 1;
      const bool full = octant ? s >= 8 : (!sched || s < nfull || need_full);  // oct32: its full sweeps
      const uint8_t *act = nullptr;
      long long nact = c->nblocks;
      if (!full) {
        CK(cudaEventRecord(c->q0, c->st));
        CK(cudaMemsetAsync(&c->dstat->active_blocks, 0, 4, c->st));
        if (octant) {
          CK(octant_active(c->omask, sn, kOctDilate, c->bact, c->nbx, c->nby, c->nbz, &c->dstat->active_blocks,
                           c->sms, c->st));
          c->launches++;
        } else if (o.scheduler == PDFS_SCHED_LEARNED) {
          const bool f32 = which == 0;
          // the band feature (per-block field minimum) moves little once the
          // scheduler runs: it is refreshed every kBandEvery scheduled sweeps
          if (band_sweep < 0 || s - band_sweep >= kBandEvery) {
            CK(block_min(f32 ? (const void *)c->u32 : (const void *)c->u64,
                         f32 ? 0 : (o.arith == PDFS_ARITH_PAIR ? 2 : 1), f32 ? c->L32 : c->L64, g, c->nbx, c->nby,
                         c->nbz, c->bmin, c->st));
            band_sweep = s;
            c->launches++;
          }
          CK(sched_learned(c->mlp_w, c->mlp_thr, c->bchg, cur, std::min(s, kHist), c->bmin, c->nbx, c->nby,
                           c->nbz, sn, s, f32 ? 0 : 1, thr, (float)std::min(g.dx, std::min(g.dy, g.dz)), c->bact,
                           &c->dstat->active_blocks, &c->dstat->sched_err, c->sms, c->st));
          c->launches++;
        } else {
          CK(sched_change(c->bchg, cur, std::min(s, kHist), thr, c->bact, c->nbx, c->nby, c->nbz,
                          &c->dstat->active_blocks, c->sms, c->st));
          c->launches++;
        }
        CK(cudaEventRecord(c->q1, c->st));
        act = c->bact;
      }
      const double kms0 = c->kern_ms;
      int r = run_sweep(c, which, sn, act, sched ? c->bchg + (size_t)cur * c->nblocks : nullptr, &chg);
      if (r) return r;
      if (!full) {
        nact = c->hstat->active_blocks;
        st.ms_sched += ms_between(c->q0, c->q1);
        if (c->hstat->sched_err) return PDFS_ERR_TIMEOUT;
      }
      if (verbose(o))
        fprintf(stderr, "pdfs: phase %d sweep %d sn=%d %s change=%.3e active=%lld/%lld kernel %.3f ms\n", which, s,
                sn, full ? "full" : "skip", chg, nact, c->nblocks, c->kern_ms - kms0);
      ++s;
      const long long upd = full ? nodes : (long long)((double)nodes * (double)nact / (double)c->nblocks);
      st.voxel_updates += upd;
      if (which != 0) st.voxel_updates_fp64 += upd;
      if (full) {
        st.full_sweeps++;
      } else {
        st.blocks_skipped += c->nblocks - nact;
        (which == 0 ? st.ms_kern_masked_fp32 : st.ms_kern_masked_fp64) += c->kern_ms - kms0;
        (which == 0 ? st.updates_masked_fp32 : st.updates_masked_fp64) += upd;
        (which == 0 ? st.masked_sweeps_fp32 : st.masked_sweeps_fp64)++;
      }
      if (o.fixed_sweeps == 0 && (full || !certify) && chg <= tol) break;
      need_full = !full && chg <= tol;  // a quiet skipped sweep calls for a judging full sweep
      cur = (cur + 1) % kRing;          // this sweep's changes become history
    }
    CK(cudaEventRecord(c->e1, c->st));
    CK(cudaEventSynchronize(c->e1));
    *count += s;
    *ms += ms_between(c->e0, c->e1);
    *kms += c->kern_ms;
    st.final_change = chg;
    return PDFS_OK;
  };

  int r = PDFS_OK;
  if (o.precision == PDFS_PREC_FP64) {
    if ((r = ctx_fp64_start(c))) return r;
    r = phase(1, o.tol, &st.sweeps_fp64, &st.ms_fp64, &st.ms_kern_fp64);
    c->last_prec = 1;
  } else {
    if ((r = ctx_narrow(c))) return r;
    r = phase(0, kTol32, &st.sweeps_fp32, &st.ms_fp32, &st.ms_kern_fp32);
    c->last_prec = 0;
    if (!r && o.precision == PDFS_PREC_FP32_POLISH64 && o.fixed_sweeps == 0) {
      if ((r = ctx_widen(c))) return r;
      r = phase(2, o.tol, &st.sweeps_fp64, &st.ms_fp64, &st.ms_kern_fp64);
      c->last_prec = 1;
    }
  }
  if (!r) r = rc;
  st.status = r;
  st.launches = c->launches;
  if (cudaEventRecord(c->r1, c->st) == cudaSuccess && cudaEventSynchronize(c->r1) == cudaSuccess)
    st.ms_device = ms_between(c->r0, c->r1);
  st.ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (stats) *stats = st;
  if (verbose(o))
    fprintf(stderr, "pdfs: run status=%d fp32 sweeps=%d (%.2f ms) fp64 sweeps=%d (%.2f ms) final change=%g\n", r,
            st.sweeps_fp32, st.ms_fp32, st.sweeps_fp64, st.ms_fp64, st.final_change);
  return r;
}

// Device -> host: c->st converts the result to the reference layout slab by
// slab, c->st2 copies each converted slab out.
static int store_impl(pdfs_ctx *c, double *field, double *ms_d2h) {
  if (!c || !field || c->last_prec < 0) return PDFS_ERR_INVALID;
  CK(cudaSetDevice(c->dev));
  const pdfs_grid &g = c->g;
  const size_t plane = (size_t)(g.nx + 2) * (g.ny + 2);
  const bool dev = is_device_ptr(field);
  double *dst = field;
  int s;
  if (!dev) {
    if ((s = ensure_stage(c))) return s;
    dst = (double *)c->stage;
  }
  const int planes = g.nz + 2, per = dev ? planes : slab_planes(g);
  const bool pipe = per < planes;  // else the copy runs on c->st
  if (pipe && (s = ensure_pipeline(c))) return s;
  cudaStream_t cs = pipe ? c->st2 : c->st;  // the copies' stream
  CK(cudaEventRecord(c->e0, c->st));
  const uint32_t *fm = c->has_mask ? c->fmask : nullptr;
  for (int z0 = 0, k = 0; z0 < planes; z0 += per, ++k) {
    const int z1 = std::min(planes, z0 + per);
    dim3 grid(g.ny + 2, z1 - z0);
    if (c->last_prec == 1 && c->o.arith == PDFS_ARITH_PAIR)
      k_unpack_pair<<<grid, 128, 0, c->st>>>(c->u64, c->L64, c->in64, fm, c->M, dst, g.nx, g.ny, g.nz, z0);
    else if (c->last_prec == 1)
      k_unpack<double><<<grid, 128, 0, c->st>>>(c->u64, c->L64, c->in64, c->L64, nullptr, c->M, dst, g.nx, g.ny, z0);
    else
      k_unpack<float><<<grid, 128, 0, c->st>>>(c->u32, c->L32, c->in64, c->L64, fm, c->M, dst, g.nx, g.ny, z0);
    CK(cudaGetLastError());
    if (!dev) {
      if (pipe) {
        CK(cudaEventRecord(c->slab_ev[k], c->st));
        CK(cudaStreamWaitEvent(cs, c->slab_ev[k], 0));
      }
      CK(cudaMemcpyAsync(field + z0 * plane, (char *)c->stage + z0 * plane * 8, (size_t)(z1 - z0) * plane * 8,
                         cudaMemcpyDeviceToHost, cs));
    }
  }
  if (pipe) {
    CK(cudaEventRecord(c->slab_ev[pdfs_ctx::kSlabs], cs));
    CK(cudaStreamWaitEvent(c->st, c->slab_ev[pdfs_ctx::kSlabs], 0));
  }
  CK(cudaEventRecord(c->e1, c->st));
  CK(cudaStreamSynchronize(c->st));
  if (ms_d2h) *ms_d2h = ms_between(c->e0, c->e1);
  return PDFS_OK;
}

extern "C" int pdfs_ctx_store(pdfs_ctx *c, double *field) { return store_impl(c, field, nullptr); }

extern "C" int pdfs_solve(const pdfs_grid *g, double *field, const uint8_t *frozen, const pdfs_opts *o,
                          pdfs_stats *stats) {
  const auto t0 = std::chrono::steady_clock::now();
  if (!field) return PDFS_ERR_INVALID;
  pdfs_ctx *c = nullptr;
  int s = pdfs_ctx_create(g, o, &c);
  if (s) {
    if (stats) stats->status = s;
    return s;
  }
  double h2d = 0, d2h = 0;
  pdfs_stats st;
  std::memset(&st, 0, sizeof(st));
  s = load_impl(c, field, frozen, &h2d);
  if (!s) {
    s = pdfs_ctx_run(c, &st);
    if (!s || s == PDFS_ERR_NOT_CONVERGED) {
      int s2 = store_impl(c, field, &d2h);
      if (s2) s = s2;
    }
  }
  pdfs_ctx_destroy(c);
  st.status = s;
  st.ms_h2d = h2d;
  st.ms_d2h = d2h;
  st.ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (stats) *stats = st;
  return s;
}

extern "C" int pdfs_ctx_blocks(const pdfs_ctx *c, int *nbx, int *nby, int *nbz) {
  if (!c) return PDFS_ERR_INVALID;
  if (nbx) *nbx = c->nbx;
  if (nby) *nby = c->nby;
  if (nbz) *nbz = c->nbz;
  return PDFS_OK;
}

// A cycle of 8 orderings as one launch (an octant round on bricks,
// tile3d.cuh OCT): orderings (first + j) % 8 + 1, j = 0..7, each over the
// blocks its octant mask (from the FP32 field) names.  which: 0 = FP32
// min-update (16 x 16 x 32 bricks), 2 = the polish (16 x 16 x 16).  chg: the 8
// sweeps' max changes; *active: the bricks visited, summed over the 8 sweeps;
// *updates: the node updates of the active blocks, summed alike.
// nsw sweeps (orderings first + 1, first + 2, ..) in one launch: sweep j
// visits every block when bit j of full is set, else the blocks whose octant
// masks (computed here from the FP32 field) name its ordering.  chg[j]: sweep
// j's change; active: tickets run; updates: node updates.
static int octant_round(pdfs_ctx *c, int which, int first, int nsw, unsigned full, double *chg, long long *active,
                        long long *updates) {
  const pdfs_grid &g = c->g;
  const bool f32 = which == 0;
  const uint8_t *bits = c->omask;
  const unsigned every = (1u << nsw) - 1u;
  int kernels = 6;  // nodes, brick bits, tickets, plan, merge, round
  if ((full & every) == every) {  // no sweep reads the masks
    CK(cudaMemsetAsync(c->bact, 0xff, (size_t)c->nblocks, c->st));
    bits = c->bact;
  } else {
    CK(octant_mask(c->u32, c->L32, c->has_mask ? c->fmask : nullptr, c->M, g, f32 ? kOctSlack32 : kOctSlack64,
                   INFINITY, c->nbx, c->nby, c->nbz, c->omask, c->st));
    ++kernels;
    if (kOctDilate) {
      CK(octant_union(c->omask, c->bact, c->nbx, c->nby, c->nbz, c->sms, c->st));
      bits = c->bact;
      ++kernels;
    }
  }
  SweepArgs a;
  fill_sweep_args(c, which, first % 8 + 1, nullptr, nullptr, &a);
  a.oct_first = first % 8;
  a.oct_full = full & every;
  a.oct_bits = bits;
  a.oct_tbits = c->tact;
  a.maxchg = c->ochg;
  a.epoch = c->epoch + 1;  // sweep j publishes epoch + j
  c->epoch += kOctMax;
  const int *nt = f32 ? c->nt32 : c->nt64;
  const int nb = nt[0] * nt[1] * nt[2];
  int *cnt_off = c->toct + kOctMax * (size_t)nb;
  CK(cudaMemsetAsync(c->dstat, 0, offsetof(DevStatus, active_blocks), c->st));
  CK(cudaMemsetAsync(c->ochg, 0, kOctWords * 8, c->st));  // change words, then 8 node counts
  CK(cudaMemsetAsync(c->ticket, 0, 4, c->st));
  CK(octant_nodes(bits, c->nbx, c->nby, c->nbz, g.nx, g.ny, g.nz, c->ochg + kOctMax, c->sms, c->st));
  const bool iso = g.dx == g.dy && g.dy == g.dz;
  const int arith = c->o.arith == PDFS_ARITH_REFERENCE ? ARITH_REF
                    : c->o.arith == PDFS_ARITH_MIXED   ? ARITH_MIXED
                    : c->o.arith == PDFS_ARITH_PAIR    ? ARITH_PAIR
                                                       : ARITH_FAST;
  int grid = 0;
  CK(cudaEventRecord(c->k0, c->st));
  CK(launch_octant_round(which, arith, iso, nsw, a, f32 ? c->L32 : c->L64, c->toct, cnt_off, c->sms, c->st,
                         &grid));
  CK(cudaEventRecord(c->k1, c->st));
  unsigned long long h[kOctWords];
  int cnt[kOctMax];
  CK(cudaMemcpyAsync(c->hstat, c->dstat, sizeof(DevStatus), cudaMemcpyDeviceToHost, c->st));
  CK(cudaMemcpyAsync(h, c->ochg, sizeof h, cudaMemcpyDeviceToHost, c->st));
  CK(cudaMemcpyAsync(cnt, cnt_off, sizeof cnt, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  c->kern_ms += ms_between(c->k0, c->k1);
  c->launches += kernels;
  if (c->hstat->err[0]) return c->hstat->err[0] == DEV_ERR_TIMEOUT ? PDFS_ERR_TIMEOUT : PDFS_ERR_CUDA;
  *active = 0;
  *updates = 0;
  const long long nodes = (long long)g.nx * g.ny * g.nz;
  for (int j = 0; j < nsw; ++j)  // sweep j runs ordering first + j + 1
    *updates += ((full >> j) & 1u) ? nodes : (long long)h[kOctMax + (first + j) % 8];
  for (int j = 0; j < nsw; ++j) {
    if (f32) {  // float bits in the slot's low word
      const unsigned b32 = (unsigned)h[j];
      float f;
      std::memcpy(&f, &b32, 4);
      chg[j] = f;
    } else {  // the double's bits (pairs: their hi word as a double)
      std::memcpy(&chg[j], &h[j], 8);
    }
    *active += (long long)cnt[j];
  }
  return PDFS_OK;
}

extern "C" int pdfs_ctx_orderings(pdfs_ctx *c, uint8_t *orderings) {
  if (!c || !c->loaded || !c->u32 || !c->omask || !orderings || c->last_prec < 0) return PDFS_ERR_INVALID;
  CK(cudaSetDevice(c->dev));
  const uint8_t *buf = c->omask;
  CK(octant_mask(c->u32, c->L32, c->has_mask ? c->fmask : nullptr, c->M, c->g, kOctSlack32, INFINITY, c->nbx,
                 c->nby, c->nbz, c->omask, c->st));
  if (kOctDilate) {  // the polish's widened masks: bit sn of a block or of a face neighbour
    CK(octant_union(c->omask, c->bact, c->nbx, c->nby, c->nbz, c->sms, c->st));
    buf = c->bact;
  }
  CK(cudaMemcpyAsync(orderings, buf, (size_t)c->nblocks, cudaMemcpyDefault, c->st));
  CK(cudaStreamSynchronize(c->st));
  return PDFS_OK;
}

extern "C" int pdfs_ctx_sweep(pdfs_ctx *c, int sn, const uint8_t *active, float *block_change, double *max_change) {
  if (!c || !c->loaded || sn < 1 || sn > 8) return PDFS_ERR_INVALID;
  CK(cudaSetDevice(c->dev));
  const int prec = c->o.precision == PDFS_PREC_FP32 ? 0 : 1;
  if (c->last_prec != prec) {  // start from the loaded input
    if (prec == 1) {
      int r = ctx_fp64_start(c);
      if (r) return r;
    } else {
      int r = ctx_narrow(c);
      if (r) return r;
    }
    c->last_prec = prec;
  }
  const size_t nb = (size_t)c->nblocks;
  const uint8_t *act = nullptr;
  if (active) {
    if (is_device_ptr(active)) {
      act = active;
    } else {
      CK(cudaMemcpyAsync(c->bact, active, nb, cudaMemcpyHostToDevice, c->st));
      act = c->bact;
    }
  }
  unsigned int *bc = block_change ? c->bchg : nullptr;  // bits of non-negative floats
  double chg = 0.0;
  int r = run_sweep(c, prec == 0 ? 0 : 1, sn, act, bc, &chg);
  if (r) return r;
  if (block_change)
    CK(cudaMemcpyAsync(block_change, c->bchg, nb * 4, cudaMemcpyDefault, c->st));
  CK(cudaStreamSynchronize(c->st));
  if (max_change) *max_change = chg;
  return PDFS_OK;
}

extern "C" int pdfs_sweep(const pdfs_grid *g, double *field, const uint8_t *frozen, int sn, const pdfs_opts *o_in,
                          double *max_change) {
  if (sn < 1 || sn > 8 || !field) return PDFS_ERR_INVALID;
  pdfs_opts o;
  if (o_in)
    o = *o_in;
  else
    pdfs_default_opts(&o);
  o.precision = PDFS_PREC_FP64;
  o.fixed_sweeps = 1;
  o.first_ordering = sn;
  o.scheduler = PDFS_SCHED_NONE;
  pdfs_stats st;
  int s = pdfs_solve(g, field, frozen, &o, &st);
  if (max_change) *max_change = st.final_change;
  return s;
}
