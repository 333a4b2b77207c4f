// sweep.cuh -- warp-specialised, TMA-fed, column-pipelined sweep of one FSM ordering.
//
// The reference sweeps one hyperplane x+y+z = level per kernel launch
// (single_gpu_cuda/src/phi3D_fsm.cu:161-185, mpi_openacc/src/phi3D_fsm.c:92-117):
// 8*(nx+ny+nz-2) launches per round, each touching one strided diagonal slice.
// Any topological order of an ordering's dependency DAG gives the same
// result (each node reads the new values of its three upwind neighbours and
// the old values of its three downwind ones), so this kernel uses a blocked
// order instead.
//
// Decomposition.  The x-y plane is cut into columns of 32 x TY nodes that run
// the whole z extent.  A persistent CTA owns one column at a time (tickets in
// wavefront order) and marches it along the sweep's z direction:
//   * compute warp `ly` (row ly of the column in sweep order) has lane `lx`
//     update plane lz = t - lx - ly at its step t: a skewed wavefront in which
//     lane lx-1 produced the upwind x value one step earlier (same warp) and
//     warp ly-1 produced the upwind y value one step earlier;
//   * warps chain through per-warp step counters in shared memory (release /
//     acquire), so there is no CTA-wide barrier per step;
//   * a loader warp streams planes (field and frozen-mask words) into a ring
//     of D shared-memory slots with TMA (cp.async.bulk.tensor, mbarrier
//     full/empty pairs), as far ahead as the ring allows; the polish's
//     per-node cap is read by each lane straight from global memory a few
//     steps ahead, so the ring (and the CTA's shared memory) stays small;
//   * a communication warp fetches the upwind faces of the neighbouring
//     columns (all chunks that are ready, in one round trip) and publishes
//     this column's per-row progress, so the compute warps never wait on a
//     global fence or a global round trip;
//   * faces cross columns through diagonal-indexed mailboxes in global memory:
//     item (row, z) of a column's downwind x face is stored at [z + row][row]
//     and item (x, z) of its downwind y face at [z + x][x].  A downstream
//     column at step t needs exactly mailbox row d = t, so each step's halo is
//     one contiguous run that is written and read with coalesced accesses, and
//     the downstream column trails its upstream by about TX (or TY) steps;
//   * every wait is bounded (in SM cycles): on expiry the kernel records
//     DEV_ERR_TIMEOUT, raises an abort flag, drains its own TMA loads and
//     returns, so the host gets PDFS_ERR_TIMEOUT and the context stays usable.
//
// Memory layout (internal, per element type T, V = 16/sizeof(T)):
//   element (x, y, z) of the halo-padded grid (0 <= x <= nx+1, ...) lives at
//   z*plane + y*px + x + (V-1), so interior x = 1 + cx*32 starts on a 16-byte
//   boundary (a legal TMA x coordinate); px >= ncx*32 + 2V, rows ry =
//   ncy*TY + 2, planes nz + 2.
#pragma once
#include <cuda.h>

#include <cstdint>
#include <type_traits>

#include "godunov.cuh"

namespace pdfs {

enum { MODE_MIN = 0, MODE_REPLACE = 1 };

// Lane-column tiles (lanecol.cuh) and their z-column ("ZC") field layout.
constexpr int kLcZ0 = 16;     // column position of the halo plane z = 0
constexpr int kLcLanes = 31;  // computing lanes of a tile

enum { ARITH_REF = 0, ARITH_FAST = 1, ARITH_MIXED = 2, ARITH_PAIR = 3 };
enum { DEV_ERR_TIMEOUT = 1, DEV_ERR_SMEM_ALIGN = 2 };

struct SweepArgs {
  void *u;                // working field (internal layout)
  const uint32_t *fmask;  // frozen bit per node (MaskLayout), or nullptr
  long long px;           // row pitch (elements)
  long long plane;        // plane stride (elements)
  long long mask_fy;      // frozen mask: words per 32-wide column of a plane
  long long mask_fw;      // frozen mask: word columns per plane
  int nx, ny, nz;
  int sx, sy, sz;         // +1 / -1 sweep direction per axis
  int ncx, ncy;           // columns
  int nbands;             // mailbox chunks per column
  const int *order;       // ticket -> local column id (lcy*ncx + lcx), wavefront order
  int *prog;              // [column][row]: steps published by each row of each column
  void *xbox;             // x-face mailboxes, [column][d][row]
  void *ybox;             // y-face mailboxes, [column][d][x]
  long long xstride, ystride;  // mailbox elements per column
  int *ticket;            // column ticket counter
  int *err;               // [0] error code, [1] abort flag, [2] column that timed out
  void *maxchg;           // FP32: uint bits of max relative change; FP64: u64 bits of max abs change
  float hmin;             // smallest spacing (relative-change floor)
  const uint8_t *blk_active;  // per 8^3 block (x fastest): update its nodes?  nullptr = all
  unsigned int *blk_chg;  // per 8^3 block: float bits of this sweep's max change (nullptr = off)
  int nbx, nby, nbz;      // 8^3 block grid
  long long wait_cycles;  // bound on any single wait, in SM cycles
  int poison_col;         // test hook: this column never publishes (-1 = off)
  GodConst64 k64;
  GodConst32 k32;
  const struct BatchDesc *batch;  // many grids in one launch (nullptr = this grid only)
  const void *cap;        // replace-update: per-node upper bound (the input), field layout
  // 3-D brick sweep (tile3d.cuh)
  int *tflag;             // per brick: epoch of the last sweep that completed it
  const int *torder;      // ticket -> local brick id in sweep order, wavefront order
  int ntx, nty, ntz;      // brick grid
  int epoch;              // this sweep's flag value (increases every launch)
  // pencils (pencil.cuh): per pencil, its downwind x and y faces as epoch-tagged
  // 64-bit words, [pencil][face][prow diagonals][16][words per value]
  unsigned long long *pmail;
  int prow;
  // replace-update on bricks and pencils: per 8^3 block, the smallest cap of
  // its updated nodes (+inf if none), exact and rounded down to float.  A new
  // value below it is below every cap of the block, so the cap is not read.
  const double *bcap64;
  const float *bcap32;
  // block-masked brick sweeps: per brick (global brick id), does it hold an
  // active 8^3 block; the tickets then list only those bricks (torder holds
  // them in wavefront order, *nticket of them)
  const uint8_t *tact;
  const int *nticket;
  // an octant round on bricks (tile3d.cuh, OCT): up to kOctMax sweeps in one
  // launch, ordering (oct_first + j) % 8 + 1 for sweep j; oct_bits: per 8^3
  // block, bit sn-1 = ordering sn visits it; oct_tbits: the same per brick
  // (the union of its blocks); oct_full: bit j = sweep j visits every block;
  // torder: the merged ticket list ((j << 27) | brick), *nticket of them
  int oct_first;
  unsigned oct_full;
  const uint8_t *oct_bits;
  const uint8_t *oct_tbits;
};

// Arguments of the lane-column sweep (lanecol.cuh).
struct LcArgs {
  void *u;               // working field (ZC layout): FP32, or FP32 pairs in 64-bit slots
  const double *cap;     // replace-update: the FP64 input in the same ZC layout
  const float *bcap32;   // replace-update: per 8^3 block, the smallest cap rounded down
  long long cxp;         // columns per row of columns (nx + 2)
  long long qz;          // elements per column
  int q_last;            // position of the last traversal step in +z order (== 7 mod 8)
  int T;                 // traversal steps per column (== 0 mod 8)
  int nx, ny, nz;
  int sx, sy, sz;        // +1 / -1 sweep direction per axis
  int ntx, nty;          // tiles
  const int *order;      // ticket -> tile id (ty * ntx + tx), every tile after the tiles it waits on
  int *ticket;
  int *err;              // [0] error code, [1] abort flag, [2] tile that timed out
  void *maxchg;          // FP32: uint bits of the max relative change; pairs: u64 bits of the max change
  float hmin;
  unsigned long long *ymail;  // [tile][T][32][words]: row R-1 of each tile
  unsigned long long *xmail;  // [tx][xrows][T][words]: lane 30 of each tile, by ly + 32
  int xrows;
  int epoch;
  long long wait_cycles;
  int poison_tile;       // test hook: this tile never publishes (-1 = off)
  const uint8_t *blk_active;  // per 8^3 block: update its nodes?  (nullptr = all)
  unsigned int *blk_chg;      // per 8^3 block: float bits of this sweep's max change (nullptr = off)
  int nbx, nby, nbz;
  GodConst32 k32;
};

// A batched sweep: tickets enumerate (grid, local column) pairs, each grid's
// columns in wavefront order; args[g] / maps[3g..3g+2] describe grid g.
struct BatchDesc {
  int nticket;
  const int2 *tickets;      // (grid, local column id); pencil rounds: (grid * 8 + sweep, local pencil id)
  const SweepArgs *args;    // per grid (sx/sy/sz are taken from the launch)
  const CUtensorMap *maps;  // per grid: field, cap, mask
  // Pencil rounds (pencil.cuh): one launch runs all 8 orderings of a round
  // for every grid; sweep s of a grid starts once its sweep s - 1 is done.
  int ngrid;                // grids in args; the change words are [sweep][grid]
  int *done;                // [grid * 8 + sweep]: pencils finished this round
  const int *round;         // rounds run before this one (mailbox epochs advance 8 per round)
};

// Shared-memory plan of one kernel variant: columns of 32 x TY nodes, R rows
// per compute warp (TY/R compute warps).
template <class T, int TY, int R_, int MODE>
struct WsGeo {
  static constexpr int TX = 32;
  static constexpr int RW = R_;        // rows per compute warp
  static constexpr int NW = TY / R_;   // compute warps
  static constexpr int V = 16 / (int)sizeof(T);
  static constexpr int W = TX + 2 * V;  // slot row: x0-V .. x0+TX+V-1
  static constexpr int R = TY + 2;      // slot rows: y0-1 .. y0+TY
  static constexpr int SK = TX + TY - 2;
  static constexpr int LOOK = sizeof(T) == 8 ? 4 : 8;  // planes the producer may run ahead
  static constexpr int D = SK + 3 + LOOK;               // ring depth (planes)
  static constexpr int ALIGN = 128 / (int)sizeof(T);
  static constexpr int SLOT = ((R * W + ALIGN - 1) / ALIGN) * ALIGN;
  static constexpr int C = 4;   // steps per mailbox chunk
  static constexpr int HB = sizeof(T) == 8 ? 4 : 8;  // mailbox chunk ring depth
  static constexpr int NT = (NW + 2) * 32;  // NW compute warps, a TMA loader warp, a communication warp
  static constexpr int CP = 4;  // replace-update: caps each lane prefetches ahead (registers)
  static constexpr size_t OFF_RING = 0;
  static constexpr size_t OFF_FR = OFF_RING + (size_t)D * SLOT * sizeof(T);
  static constexpr int MSL = 32;  // mask words per slot: 128 bytes, a legal TMA destination
  static constexpr size_t OFF_XB = OFF_FR + (size_t)D * MSL * 4;
  static constexpr size_t OFF_YB = OFF_XB + (size_t)HB * C * TY * sizeof(T);
  static constexpr size_t OFF_BAR = (OFF_YB + (size_t)HB * C * TX * sizeof(T) + 15) & ~size_t(15);
  static constexpr size_t OFF_DONE = OFF_BAR + (size_t)(2 * D + 2 * HB) * 8;
  static constexpr size_t BYTES = OFF_DONE + (size_t)NW * 4 + 16;
  static_assert(TY % R_ == 0, "rows per warp must divide TY");
  static constexpr unsigned TX_BYTES = (unsigned)(R * W * sizeof(T));
  // mask words per plane load: the column's rows, from a 16-byte aligned
  // start (a TMA copy's innermost coordinate must be a 16-byte multiple, so
  // a TY that is not a multiple of 4 reads from (y0-1) rounded down to 4)
  static constexpr int MBOX = TY % 4 == 0 ? TY : (TY + 6) / 4 * 4;
  static constexpr unsigned MASK_BYTES = MBOX * 4;
  // every TMA destination (field slot, mask slot) starts on 128 bytes
  static_assert((SLOT * sizeof(T)) % 128 == 0 && OFF_FR % 128 == 0, "TMA alignment");
  static_assert(MBOX * 4 >= 16 && MBOX <= MSL, "TMA box");
};

// ---- PTX helpers ---------------------------------------------------------------------
__device__ __forceinline__ unsigned saddr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t *b, unsigned n) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(saddr(b)), "r"(n) : "memory");
}
__device__ __forceinline__ void mbar_inval(uint64_t *b) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];\n" ::"r"(saddr(b)) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive(uint64_t *b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(saddr(b)) : "memory");
}
__device__ __forceinline__ void mbar_arrive_tx(uint64_t *b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(saddr(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t *b, unsigned parity) {
  unsigned r;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(r)
      : "r"(saddr(b)), "r"(parity)
      : "memory");
  return r != 0;
}
__device__ __forceinline__ bool mbar_try(uint64_t *b, unsigned parity) {
  unsigned r;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(r)
      : "r"(saddr(b)), "r"(parity)
      : "memory");
  return r != 0;
}
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y, int z, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];\n" ::"r"(saddr(dst)),
      "l"(map), "r"(x), "r"(y), "r"(z), "r"(saddr(bar))
      : "memory");
}
// An L2 prefetch of a tensor-map box (no shared memory, no completion).
__device__ __forceinline__ void tma_prefetch_3d(const CUtensorMap *map, int x, int y, int z) {
  asm volatile("cp.async.bulk.prefetch.tensor.3d.L2.global.tile [%0, {%1, %2, %3}];\n" ::"l"(map), "r"(x), "r"(y),
               "r"(z)
               : "memory");
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }
__device__ __forceinline__ int ld_acquire_gpu(const int *p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed_gpu(int *p, int v) {
  asm volatile("st.relaxed.gpu.global.s32 [%0], %1;\n" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int ld_acquire_cta_s(const int *p) {
  int v;
  asm volatile("ld.acquire.cta.shared.s32 %0, [%1];\n" : "=r"(v) : "r"(saddr(p)) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_cta_s(int *p, int v) {
  asm volatile("st.release.cta.shared.s32 [%0], %1;\n" ::"r"(saddr(p)), "r"(v) : "memory");
}
// Wait bounds are counted in SM cycles (clock64() is a register read).
__device__ __forceinline__ long long cycles() { return clock64(); }

template <class T>
__device__ __forceinline__ T tmin(T a, T b) {  // the reference's min macro: a < b ? a : b
  return a < b ? a : b;
}

// Minimum, "changed" test and running max of a variant: the mixed FP64
// kernels do them on integer keys / bit patterns, off the FP64 pipe.
// FP32-pair variants (ARITH_PAIR, FP64 slots holding pairs) work on the two floats.
template <class T, int ARITH>
__device__ __forceinline__ T vmin(T a, T b) {
  if constexpr (sizeof(T) == 8 && ARITH == ARITH_MIXED)
    return kmin(a, b);
  else if constexpr (sizeof(T) == 8 && ARITH == ARITH_PAIR)
    return pmin(a, b);
  else
    return tmin(a, b);
}
template <class T, int ARITH>
__device__ __forceinline__ bool vdiffers(T a, T b) {
  if constexpr (sizeof(T) == 8 && ARITH == ARITH_MIXED)
    return __double_as_longlong(a) != __double_as_longlong(b);
  else if constexpr (sizeof(T) == 8 && ARITH == ARITH_PAIR)
    return p_hi(a) != p_hi(b) || p_lo(a) != p_lo(b);
  else
    return a != b;
}
template <class T, int ARITH>
__device__ __forceinline__ T vmax_nonneg(T a, T b) {  // a, b >= 0
  if constexpr (sizeof(T) == 8 && ARITH == ARITH_MIXED)
    return __double_as_longlong(a) < __double_as_longlong(b) ? b : a;
  else if constexpr (sizeof(T) == 8 && ARITH == ARITH_PAIR)
    return p_hi(a) < p_hi(b) ? b : a;
  else
    return fmax(a, b);
}

// The cap bound of a block in the form a variant compares with: float for
// FP32 pairs (rounded down), double otherwise.
template <class T, int ARITH>
struct CapBound {
  using type = typename std::conditional<sizeof(T) == 8 && ARITH == ARITH_PAIR, float, double>::type;
  __device__ __forceinline__ static type load(const SweepArgs &a, long long b) {
    if constexpr (sizeof(T) == 8 && ARITH == ARITH_PAIR)
      return __ldg(a.bcap32 + b);
    else
      return __ldg(a.bcap64 + b);
  }
  // v < bound, so min(cap, v) == v for every cap of the block
  __device__ __forceinline__ static bool below(T v, type bnd) {
    if constexpr (sizeof(T) == 8 && ARITH == ARITH_PAIR)
      return p_hi(v) < bnd;  // hi < the rounded-down bound: hi + lo is below the exact one
    else if constexpr (sizeof(T) == 8 && ARITH == ARITH_MIXED)
      return dkey(v) < dkey(bnd);
    else
      return (double)v < bnd;
  }
};

// A node's cap (the input, FP64) in the variant's representation.
template <class T, int ARITH>
__device__ __forceinline__ T cap_value(const T *p) {
  if constexpr (sizeof(T) == 8 && ARITH == ARITH_PAIR)
    return p_from_double(__ldg(p));
  else
    return __ldg(p);
}

// A node's change as a kernel accumulates it: relative for FP32, absolute
// for FP64, absolute as the pair (|change|, 0) for FP32 pairs.
template <class T, int ARITH>
__device__ __forceinline__ T node_change(T cv, T nv, float hmin) {
  if constexpr (sizeof(T) == 4)
    return __fdividef(fabsf(cv - nv), fmaxf(nv, hmin));
  else if constexpr (ARITH == ARITH_PAIR)
    return p_make(fabsf(p_sub(cv, nv)), 0.0f);
  else
    return fabs(cv - nv);
}
template <class T, int ARITH>
__device__ __forceinline__ float change_f(T d) {  // as a float (per-block change words)
  if constexpr (sizeof(T) == 8 && ARITH == ARITH_PAIR)
    return p_hi(d);
  else
    return (float)d;
}
template <class T, int ARITH>
__device__ __forceinline__ bool change_pos(T d) {
  if constexpr (sizeof(T) == 8 && ARITH == ARITH_PAIR)
    return p_hi(d) > 0.0f;
  else
    return d > T(0);
}
template <class T, int ARITH>
__device__ __forceinline__ unsigned long long change_u64(T d) {  // the FP64 phases' max-change word
  if constexpr (ARITH == ARITH_PAIR)
    return (unsigned long long)__double_as_longlong((double)p_hi(d));
  else
    return (unsigned long long)__double_as_longlong((double)d);
}

// The local solver of a kernel variant.  k64 / k32 are the compute warps'
// register copies of the per-sweep constants.
template <class T, int MODE, int ARITH, bool ISO>
__device__ __forceinline__ T local_update(T m0, T m1, T m2, const GodConst64 &k64, const GodConst32 &k32);
template <>
__device__ __forceinline__ float local_update<float, MODE_MIN, ARITH_FAST, true>(float m0, float m1, float m2,
                                                                                  const GodConst64 &,
                                                                                  const GodConst32 &k32) {
  return god32s<true>(m0, m1, m2, k32);
}
template <>
__device__ __forceinline__ float local_update<float, MODE_MIN, ARITH_FAST, false>(float m0, float m1, float m2,
                                                                                   const GodConst64 &,
                                                                                   const GodConst32 &k32) {
  return god32s<false>(m0, m1, m2, k32);
}
#define PDFS_LU64(MODE_, ARITH_, FN)                                                                  \
  template <>                                                                                         \
  __device__ __forceinline__ double local_update<double, MODE_, ARITH_, false>(                      \
      double m0, double m1, double m2, const GodConst64 &k64, const GodConst32 &) {                  \
    return FN(m0, m1, m2, k64);                                                                       \
  }
PDFS_LU64(MODE_MIN, ARITH_REF, god_ref64)
PDFS_LU64(MODE_MIN, ARITH_FAST, god_fast64)
PDFS_LU64(MODE_REPLACE, ARITH_REF, god_ref64)
PDFS_LU64(MODE_REPLACE, ARITH_FAST, god_fast64)
#undef PDFS_LU64
#define PDFS_LUMX(MODE_, ISO_)                                                                       \
  template <>                                                                                       \
  __device__ __forceinline__ double local_update<double, MODE_, ARITH_MIXED, ISO_>(                 \
      double m0, double m1, double m2, const GodConst64 &, const GodConst32 &k32) {                 \
    return god_mixed64<ISO_>(m0, m1, m2, k32);                                                      \
  }
PDFS_LUMX(MODE_MIN, true)
PDFS_LUMX(MODE_MIN, false)
PDFS_LUMX(MODE_REPLACE, true)
PDFS_LUMX(MODE_REPLACE, false)
#undef PDFS_LUMX
#define PDFS_LUPR(MODE_, ISO_)                                                                       \
  template <>                                                                                       \
  __device__ __forceinline__ double local_update<double, MODE_, ARITH_PAIR, ISO_>(                  \
      double m0, double m1, double m2, const GodConst64 &, const GodConst32 &k32) {                 \
    return god_pair<ISO_>(m0, m1, m2, k32);                                                         \
  }
PDFS_LUPR(MODE_MIN, true)
PDFS_LUPR(MODE_MIN, false)
PDFS_LUPR(MODE_REPLACE, true)
PDFS_LUPR(MODE_REPLACE, false)
#undef PDFS_LUPR

// Records a timeout and raises the abort flags (global and CTA).
__device__ __forceinline__ void raise_timeout(const SweepArgs &a, int col, volatile int *s_abort) {
  atomicCAS(a.err, 0, DEV_ERR_TIMEOUT);
  atomicExch(a.err + 2, col);
  atomicExch(a.err + 1, 1);
  *s_abort = 1;
}

// Bounded wait on an mbarrier phase; false on abort or timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t *b, unsigned parity, const SweepArgs &a, int col,
                                          volatile int *s_abort) {
  if (mbar_try(b, parity)) return true;
  const long long t0 = cycles();
  for (;;) {
    if (mbar_try(b, parity)) return true;
    if (*s_abort) return false;
    if (cycles() - t0 > a.wait_cycles) {
      raise_timeout(a, col, s_abort);
      return false;
    }
  }
}

template <class T, int TY, int R, int MODE, int ARITH, bool ISO>
__global__ void __launch_bounds__((TY / R + 2) * 32) ws_sweep_kernel(const __grid_constant__ CUtensorMap tm_u,
                                                                     const __grid_constant__ CUtensorMap tm_unused,
                                                                     const __grid_constant__ CUtensorMap tm_mask,
                                                                     const __grid_constant__ SweepArgs a0) {
  using G = WsGeo<T, TY, R, MODE>;
  constexpr int TX = G::TX, V = G::V, W = G::W, D = G::D, SLOT = G::SLOT, C = G::C, HB = G::HB, NW = G::NW;
  static_assert((C & (C - 1)) == 0 && (HB & (HB - 1)) == 0, "power-of-two chunk sizes");
  extern __shared__ __align__(1024) unsigned char sm[];
  T *ring = reinterpret_cast<T *>(sm + G::OFF_RING);
  uint32_t *fring = reinterpret_cast<uint32_t *>(sm + G::OFF_FR);
  T *xband = reinterpret_cast<T *>(sm + G::OFF_XB);
  T *yband = reinterpret_cast<T *>(sm + G::OFF_YB);
  uint64_t *full = reinterpret_cast<uint64_t *>(sm + G::OFF_BAR);
  uint64_t *empty = full + D;
  uint64_t *bfull = empty + D;
  uint64_t *bempty = bfull + HB;
  int *done = reinterpret_cast<int *>(sm + G::OFF_DONE);  // per compute warp: steps completed
  __shared__ int s_ticket, s_grid, s_lc, s_zlo, s_zhi;
  __shared__ volatile int s_abort;
  __shared__ SweepArgs s_a;  // the current column's grid
  __shared__ const CUtensorMap *s_maps;

  // TMA needs 128-byte aligned shared-memory destinations: refuse to start otherwise
  if ((saddr(sm) & 127u) != 0) {
    if (threadIdx.x == 0) {
      atomicCAS(a0.err, 0, DEV_ERR_SMEM_ALIGN);
      atomicExch(a0.err + 1, 1);
    }
    return;
  }

  const SweepArgs &a = s_a;
  const BatchDesc *batch = a0.batch;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int ntick = batch ? batch->nticket : a0.ncx * a0.ncy;
  int cur_grid = -1;

  if (tid == 0) s_abort = 0;
  for (int ncols_done = 0;; ++ncols_done) {
    if (tid == 0) {
      const int tk = atomicAdd(a0.ticket, 1);
      s_ticket = tk;
      if (tk < ntick) {
        if (batch) {
          const int2 e = batch->tickets[tk];
          s_grid = e.x;
          s_lc = e.y;
        } else {
          s_grid = 0;
          s_lc = a0.order[tk];
        }
      }
      if (*(volatile int *)(a0.err + 1)) s_abort = 1;
      s_zlo = 0x7fffffff;
      s_zhi = 0;
      for (int i = 0; i < D; ++i) {
        if (ncols_done) {
          mbar_inval(full + i);
          mbar_inval(empty + i);
        }
        mbar_init(full + i, 1);
        mbar_init(empty + i, NW);
      }
      for (int i = 0; i < HB; ++i) {
        if (ncols_done) {
          mbar_inval(bfull + i);
          mbar_inval(bempty + i);
        }
        mbar_init(bfull + i, 1);
        mbar_init(bempty + i, NW);
      }
      mbar_fence_init();
    }
    __syncthreads();
    if (s_ticket >= ntick || s_abort) break;
    if (s_grid != cur_grid) {  // stage the column's grid description in shared memory
      cur_grid = s_grid;
      const SweepArgs *src = batch ? batch->args + cur_grid : &a0;
      const int *ws = reinterpret_cast<const int *>(src);
      int *wd = reinterpret_cast<int *>(&s_a);
      for (int i = tid; i < (int)(sizeof(SweepArgs) / 4); i += blockDim.x) wd[i] = ws[i];
      __syncthreads();
      if (tid == 0) {
        s_a.sx = a0.sx;
        s_a.sy = a0.sy;
        s_a.sz = a0.sz;
        s_a.err = a0.err;
        s_a.ticket = a0.ticket;
        if (batch) s_a.maxchg = reinterpret_cast<unsigned long long *>(a0.maxchg) + cur_grid;
        s_maps = batch ? batch->maps + 3 * cur_grid : nullptr;
      }
      __syncthreads();
    }
    const CUtensorMap *mp_u = batch ? s_maps : &tm_u;
    const CUtensorMap *mp_mask = batch ? s_maps + 2 : &tm_mask;
    T *__restrict__ u = reinterpret_cast<T *>(a.u);
    T *__restrict__ xbox = reinterpret_cast<T *>(a.xbox);
    T *__restrict__ ybox = reinterpret_cast<T *>(a.ybox);
    const int nz = a.nz, NP = nz + 2, NB = a.nbands;
    const int tsteps = max(nz + TX + TY + 1, NB * C);  // steps every compute warp runs per column
    const bool masked = a.fmask != nullptr;
    T tmax = T(0);
    const int lc = s_lc;
    const int lcx = lc % a.ncx, lcy = lc / a.ncx;
    const int cx = a.sx > 0 ? lcx : a.ncx - 1 - lcx;
    const int cy = a.sy > 0 ? lcy : a.ncy - 1 - lcy;
    const int col = cy * a.ncx + cx;
    const int upx = lcx > 0 ? col - a.sx : -1;
    const int upy = lcy > 0 ? col - a.sy * a.ncx : -1;
    const bool has_dnx = lcx < a.ncx - 1, has_dny = lcy < a.ncy - 1;
    const int x0 = 1 + cx * TX, y0 = 1 + cy * TY;
    const long long rowbase = (long long)cx * TX;  // internal x index of x0 - V
    const int mstart = TY % 4 == 0 ? y0 - 1 : (y0 - 1) & ~3;  // first mask word a plane load reads
    const int moff = (y0 - 1) - mstart;                        // this column's first row within it

    // Active z range [zlo, zhi) of the column, in sweep order, under a block
    // mask: the union of its active 8^3 blocks.  Nodes outside it keep their
    // values this sweep, so only the steps that reach the range run; the
    // column's face items outside the range are copied from the field.
    constexpr int SKW = TX + TY - 2;  // lane (TX-1, TY-1) trails lane (0, 0) by SKW planes
    int zlo = 0, zhi = nz;
    if (a.blk_active) {
      const int bx0 = (x0 - 1) >> 3, bx1 = min(a.nbx, (x0 - 1 + TX + 7) >> 3);
      const int by0 = (y0 - 1) >> 3, by1 = min(a.nby, (y0 - 1 + TY + 7) >> 3);
      const int nbxf = bx1 - bx0, nbf = nbxf * (by1 - by0);
      int lo = 0x7fffffff, hi = 0;
      for (int i = tid; i < nbf * a.nbz; i += blockDim.x) {
        const int bz = i / nbf, rem = i - bz * nbf;
        const int by = by0 + rem / nbxf, bx = bx0 + rem % nbxf;
        if (__ldg(a.blk_active + ((long long)bz * a.nby + by) * a.nbx + bx)) {
          const int g0 = 8 * bz + 1, g1 = min(8 * bz + 8, nz);  // global z planes of the block
          lo = min(lo, a.sz > 0 ? g0 - 1 : nz - g1);
          hi = max(hi, (a.sz > 0 ? g1 - 1 : nz - g0) + 1);
        }
      }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, off));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, off));
      }
      if (lane == 0) {
        atomicMin(&s_zlo, lo);
        atomicMax(&s_zhi, hi);
      }
      __syncthreads();
      zlo = s_zlo;
      zhi = s_zhi;
    }
    // steps [t_start, t_end) and planes [p_start, p_end] this column works on
    const bool any = zlo < zhi;
    const int t_start = any ? zlo : 0;
    const int t_end = any ? min(tsteps, zhi + SKW + 1) : 0;
    const int p_start = any ? max(0, t_start - SKW) : 0;
    const int p_end = any ? min(NP - 1, t_end + 1) : -1;
    const int kb0 = t_start / C;                          // first mailbox chunk consumed
    const int kb_end = any ? min(NB, (t_end - 1) / C + 1) : kb0;  // one past the last
    if (a.blk_active) {
      // face items outside the rows the steps write: x face rows
      // [t_start-TX+1, t_end-TX+1), y face rows [t_start-TY+1, t_end-TY+1)
      const int xl = a.sx > 0 ? TX - 1 : 0;  // lane holding the downwind x face
      if (has_dnx) {
        T *xout = reinterpret_cast<T *>(a.xbox) + (long long)col * a.xstride;
        const int w0 = any ? t_start - TX + 1 : 0, w1 = any ? t_end - TX + 1 : 0;
        const int dmax = nz + TY - 1;
        for (int i = tid; i < dmax * TY; i += blockDim.x) {
          const int d = i / TY, row = i - d * TY, z = d - row;
          if ((d >= w0 && d < w1) || z < 0 || z >= nz) continue;
          const int gy = a.sy > 0 ? row : TY - 1 - row;
          if (y0 + gy > a.ny) continue;
          const int gz = a.sz > 0 ? z + 1 : nz - z;
          xout[i] = u[(long long)gz * a.plane + (long long)(y0 + gy) * a.px + rowbase + V + xl];
        }
      }
      if (has_dny) {
        T *yout = reinterpret_cast<T *>(a.ybox) + (long long)col * a.ystride;
        const int w0 = any ? t_start - TY + 1 : 0, w1 = any ? t_end - TY + 1 : 0;
        const int dmax = nz + TX - 1;
        const int gyl = a.sy > 0 ? TY - 1 : 0;
        for (int i = tid; i < dmax * TX; i += blockDim.x) {
          const int d = i / TX, lx = i - d * TX, z = d - lx;
          if ((d >= w0 && d < w1) || z < 0 || z >= nz) continue;
          const int ln = a.sx > 0 ? lx : TX - 1 - lx;
          if (x0 + ln > a.nx) continue;
          const int gz = a.sz > 0 ? z + 1 : nz - z;
          yout[i] = u[(long long)gz * a.plane + (long long)(y0 + gyl) * a.px + rowbase + V + ln];
        }
      }
    }
    if (tid < NW) done[tid] = t_start;
    __syncthreads();

    if (warp == NW) {
      // ---------------------------- TMA loader warp (lane 0) ----------------------------
      if (lane == 0) {
        int pl = p_start;  // planes p_start..p_end go to ring slots (p - p_start) % D
        long long t_last = cycles();
        while (pl <= p_end) {
          const int s = (pl - p_start) % D, use = (pl - p_start) / D;
          // try_wait suspends the thread in hardware until the slot is free
          // (or a short time limit passes), so the loader does not spin
          if (use == 0 || mbar_try(empty + s, (use - 1) & 1)) {
            const int gz = a.sz > 0 ? pl : nz + 1 - pl;
            mbar_arrive_tx(full + s, G::TX_BYTES + (masked ? G::MASK_BYTES : 0u));
            tma_load_3d(ring + (size_t)s * SLOT, mp_u, (int)rowbase, y0 - 1, gz, full + s);
            if (masked) tma_load_3d(fring + s * G::MSL, mp_mask, mstart, cx, gz, full + s);
            ++pl;
            t_last = cycles();
          } else {
            if (s_abort) break;
            if (cycles() - t_last > a.wait_cycles) {
              raise_timeout(a, col, &s_abort);
              break;
            }
          }
        }
        if (s_abort) {
          // drain the TMA loads still in flight before the CTA leaves
          for (int q = max(p_start, pl - D); q < pl; ++q) {
            const long long t0 = cycles();
            while (!mbar_try(full + (q - p_start) % D, ((q - p_start) / D) & 1) && cycles() - t0 < 4000000000ll) {
            }
          }
        }
      }
    } else if (warp == NW + 1) {
      // ------------------------------ communication warp ------------------------------
      // Fills the mailbox-chunk ring from the upwind columns' mailboxes (every
      // ready chunk with a free slot, in one round trip) and publishes this
      // column's per-row progress.
      int kb = kb0, pub = 0;  // chunk k goes to slot (k - kb0) % HB
      unsigned nap = 32;      // idle back-off (ns), doubled up to 1 us while nothing moves
      long long t_last = cycles();
      for (;;) {
        bool moved = false;
        if (kb < kb_end) {
          // chunk k is complete once the row's progress >= k*C + C + TX - 1
          // (x face) / + TY - 1 (y face), or once the column is done
          int rdy = NB;
          if (upx >= 0 && lane < TY) {
            const int v = ld_acquire_gpu(a.prog + (long long)upx * TY + lane);
            rdy = v >= tsteps ? NB : max(0, (v - TX + 1) / C);
          }
          if (upy >= 0 && lane == TY) {
            const int v = ld_acquire_gpu(a.prog + (long long)upy * TY + (TY - 1));
            rdy = v >= tsteps ? NB : max(0, (v - TY + 1) / C);
          }
#pragma unroll
          for (int off = 16; off > 0; off >>= 1) rdy = min(rdy, __shfl_xor_sync(0xffffffffu, rdy, off));
          int n = 0;  // chunks to fill now: ready and with a free slot
          while (kb + n < min(rdy, kb_end) && n < HB) {
            const int k = kb + n, useb = (k - kb0) / HB;
            if (useb > 0 && !mbar_test(bempty + (k - kb0) % HB, (useb - 1) & 1)) break;
            ++n;
          }
          if (n > 0) {
            if (upx >= 0)
              for (int i = lane; i < n * C * TY; i += 32) {
                const int k = kb + i / (C * TY);
                xband[((k - kb0) % HB) * C * TY + i % (C * TY)] =
                    __ldcg(xbox + (long long)upx * a.xstride + (long long)kb * C * TY + i);
              }
            if (upy >= 0)
              for (int i = lane; i < n * C * TX; i += 32) {
                const int k = kb + i / (C * TX);
                yband[((k - kb0) % HB) * C * TX + i % (C * TX)] =
                    __ldcg(ybox + (long long)upy * a.ystride + (long long)kb * C * TX + i);
              }
            __syncwarp();
            if (lane < n) mbar_arrive(bfull + (kb + lane - kb0) % HB);
            kb += n;
            moved = true;
          }
        }
        {  // publish this column's progress, row by row (row ly belongs to compute warp ly / R)
          bool need = false;
          int dv = 0;
          if (lane < TY) {
            dv = ld_acquire_cta_s(done + lane / R);
            need = dv > pub;
          }
          if (__any_sync(0xffffffffu, need)) {
            __threadfence();
            if (need) {
              if (col != a.poison_col) st_relaxed_gpu(a.prog + (long long)col * TY + lane, dv);
              pub = dv;
            }
            moved = true;
          }
        }
        const bool published = __all_sync(0xffffffffu, lane >= TY || pub == tsteps);
        if (kb >= kb_end && published) break;
        if (moved) {
          t_last = cycles();
          nap = 32;
        } else {
          if (s_abort || *(volatile int *)(a.err + 1)) {
            s_abort = 1;
            break;
          }
          if (cycles() - t_last > a.wait_cycles) {
            if (lane == 0) raise_timeout(a, col, &s_abort);
            s_abort = 1;
            break;
          }
          __nanosleep(nap);
          nap = min(nap * 2, 1024u);
        }
      }
    } else {
      // ------------------------------- compute warps -------------------------------
      // warp w owns rows ly = w*R + r (sweep order); lane = global x offset.
      // At step t, lane lx of row ly updates plane lz = t - lx - ly.
      //
      // The per-sweep values live in registers: the SweepArgs copy sits in
      // shared memory and every mbarrier / fence asm is a compiler barrier,
      // so reading it inside the loop would reload it each step.
      const int w = warp;
      const int ly0 = w * R;
      const int sxd = a.sx, syd = a.sy, szd = a.sz;
      const long long plane = a.plane;
      const float hmin = a.hmin;
      const GodConst64 k64 = a.k64;
      const GodConst32 k32 = a.k32;
      const uint8_t *__restrict__ blk_active = a.blk_active;
      unsigned int *__restrict__ blk_chg = a.blk_chg;
      const int nbx = a.nbx, nby = a.nby;
      const int lx = sxd > 0 ? lane : TX - 1 - lane;
      int o[R], gy[R];
      bool valid[R];
      long long grow[R];  // global row offset of my node (without the plane term)
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int ly = ly0 + r;
        gy[r] = syd > 0 ? ly : TY - 1 - ly;
        valid[r] = (y0 + gy[r] <= a.ny) && (x0 + lane <= a.nx);
        o[r] = (gy[r] + 1) * W + lane + V;
        grow[r] = (long long)(y0 + gy[r]) * a.px + rowbase + V + lane;
      }
      // 8^3 block bookkeeping: x and y block indices are fixed per lane/row,
      // the z block changes every 8 planes
      const bool track = blk_active != nullptr || blk_chg != nullptr;
      const int bxl = (x0 - 1 + lane) >> 3;
      int byr[R], bzr[R];
      bool actb[R];
      T accb[R];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        byr[r] = (y0 - 1 + gy[r]) >> 3;
        bzr[r] = -1;
        actb[r] = true;
        accb[r] = T(0);
      }
      const bool band_x = (lx == 0) && (upx >= 0);
      const bool band_y = (w == 0) && (upy >= 0);
      const bool wr_x = (lx == TX - 1) && has_dnx;
      const bool wr_y = (w == NW - 1) && has_dny;
      const int xm = sxd > 0 ? -1 : 1;  // smem offset of the upwind x neighbour
      // the upwind lane's node exists (a descending sweep's upwind lane lies
      // at x+1, past nx in a ragged last column: then the ring's halo is used)
      const bool upx_lane_ok = sxd > 0 || x0 + lane + 1 <= a.nx;
      const int ym = syd > 0 ? -W : W;  // smem offset of the upwind y neighbour
      T *xout = xbox + (long long)col * a.xstride;
      T *yout = ybox + (long long)col * a.ystride;
      // ring slot of plane p = lz + 1 of row 0 at step t (per lane), and of
      // the write-back plane of row 0 (lane TX-1's plane, uniform); plane p
      // sits in slot (p - p_start) mod D, so the sweep's upwind z plane of a
      // node is one slot below its own and the downwind one a slot above
      int s0 = (t_start + 1 - lx - ly0 - p_start) % D;
      if (s0 < 0) s0 += D;
      int swb = (t_start + 1 - (TX - 1) - ly0 - p_start) % D;
      if (swb < 0) swb += D;
      int qw = p_start, qslot = 0, qpar = 0;  // next plane to wait for, its slot and phase parity
      int rel = p_start, rslot = 0;           // next plane to release and its slot
      bool finished = true;
      // replace-update: the caps of my nodes for the next CP steps, per row,
      // prefetched from global memory (lanes sit on different planes, so the
      // cap is not worth a ring of its own)
      const T *__restrict__ capg = reinterpret_cast<const T *>(a.cap);
      T capq[R][G::CP];
      auto cap_at = [&](int r, int t) -> T {
        const int lz = t - lx - ly0 - r;
        if (MODE != MODE_REPLACE || !valid[r] || (unsigned)lz >= (unsigned)nz) return T(0);
        const int gz = szd > 0 ? lz + 1 : nz - lz;
        return __ldg(capg + (long long)gz * plane + grow[r]);
      };
#pragma unroll
      for (int r = 0; r < R; ++r)
#pragma unroll
        for (int k = 0; k < G::CP; ++k) capq[r][k] = MODE == MODE_REPLACE ? cap_at(r, t_start + k) : T(0);
      // Values a step hands to the next one in registers: prev[r] is my row
      // r's result of the previous step -- the sweep's upwind z neighbour of
      // my next node, the upwind x neighbour of lane lx+1's next node (passed
      // by shuffle) and, within the warp, the upwind y neighbour of row r+1's
      // next node.  The frozen-mask word of my node's plane travels down the
      // warp the same way: lane lx receives from lane lx-1 the word it used a
      // step earlier, so only lane lx = 0 reads it (all lanes reading it
      // would hit one shared-memory bank 32 times).
      T prev[R];
      uint32_t mw[R];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        prev[r] = T(0);
        mw[r] = 0;
      }
      for (int t = t_start; t < t_end; ++t) {
        if (w > 0 && ld_acquire_cta_s(done + w - 1) < t) {
          const long long t0 = cycles();
          while (ld_acquire_cta_s(done + w - 1) < t) {
            if (s_abort) break;
            if (cycles() - t0 > a.wait_cycles) {
              if (lane == 0) raise_timeout(a, col, &s_abort);
              break;
            }
          }
          if (__any_sync(0xffffffffu, s_abort != 0)) {
            finished = false;
            break;
          }
        }
        const int qneed = min(t - ly0 + 2, p_end);
        bool ok = true;
        while (ok && qw <= qneed) {
          ok = mbar_wait(full + qslot, qpar, a, col, &s_abort);
          ++qw;
          if (++qslot == D) {
            qslot = 0;
            qpar ^= 1;
          }
        }
        const int kb = t / C;
        const int tc = t & (C - 1);
        const int rkb = kb - kb0;  // chunk kb sits in slot rkb % HB
        if (ok && (tc == 0 || t == t_start) && kb < kb_end)
          ok = mbar_wait(bfull + (rkb & (HB - 1)), (rkb / HB) & 1, a, col, &s_abort);
        if (!__all_sync(0xffffffffu, ok)) {
          finished = false;
          break;
        }

        // the upwind x values (lane lx-1's results of the previous step)
        T upx_sh[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
          upx_sh[r] = sxd > 0 ? __shfl_up_sync(0xffffffffu, prev[r], 1) : __shfl_down_sync(0xffffffffu, prev[r], 1);
          if (masked)
            mw[r] = sxd > 0 ? __shfl_up_sync(0xffffffffu, mw[r], 1) : __shfl_down_sync(0xffffffffu, mw[r], 1);
        }
        const bool first = t == t_start;  // registers hold no previous step yet

        // Rows of one step are independent (different planes), so the step is
        // split into a load phase, a compute phase and a store phase: the R
        // update chains then overlap instead of waiting on each other's stores.
        bool act[R];
        T cv[R], m0[R], m1[R], m2[R], capv[R];
        int sr[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const int lz = t - lx - ly0 - r;
          int sx_ = s0 - r;
          if (sx_ < 0) sx_ += D;
          sr[r] = sx_;
          act[r] = valid[r] && (unsigned)lz < (unsigned)nz;
          if (track && act[r]) {
            const int gz = szd > 0 ? lz + 1 : nz - lz;
            const int bz = (gz - 1) >> 3;
            if (bz != bzr[r]) {  // entering a new z block: flush the old one, fetch the new flag
              const long long base = ((long long)bz * nby + byr[r]) * nbx + bxl;
              if (blk_chg && bzr[r] >= 0 && accb[r] > T(0))
                atomicMax(blk_chg + ((long long)bzr[r] * nby + byr[r]) * nbx + bxl, __float_as_uint((float)accb[r]));
              accb[r] = T(0);
              bzr[r] = bz;
              actb[r] = blk_active ? __ldg(blk_active + base) != 0 : true;
            }
            act[r] = actb[r];
          }
          if (masked) {
            if (lx == 0 || first) mw[r] = fring[sx_ * G::MSL + moff + gy[r]];
            if (act[r]) act[r] = !((mw[r] >> lane) & 1u);
          }
          cv[r] = T(0);
          m0[r] = m1[r] = m2[r] = capv[r] = T(0);
          if (valid[r] && (unsigned)lz < (unsigned)nz) {
            const T *sl = ring + sx_ * SLOT + o[r];
            cv[r] = sl[0];
            const T dn_x = sl[-xm], dn_y = sl[-ym];
            // upwind neighbours: registers where a previous step of this warp
            // produced them, else the ring / the mailbox chunk
            T up_x = upx_sh[r];
            if (lx == 0 || first || !upx_lane_ok)
              up_x = band_x ? xband[(rkb & (HB - 1)) * C * TY + tc * TY + ly0 + r] : sl[xm];
            T up_y;
            if (r > 0 && !first && valid[r > 0 ? r - 1 : 0])  // the upwind row's node exists
              up_y = prev[r > 0 ? r - 1 : 0];
            else if (r == 0 && band_y)
              up_y = yband[(rkb & (HB - 1)) * C * TX + tc * TX + lx];
            else
              up_y = sl[ym];
            int s_up = sx_ - 1, s_dn = sx_ + 1;
            s_up = s_up < 0 ? s_up + D : s_up;
            s_dn = s_dn >= D ? s_dn - D : s_dn;
            const T z_up = (lz == 0 || first) ? ring[s_up * SLOT + o[r]] : prev[r];
            const T z_dn = ring[s_dn * SLOT + o[r]];
            // the reference's minima keep global orientation: min(u[x-1], u[x+1])
            const T xl = sxd > 0 ? up_x : dn_x, xr = sxd > 0 ? dn_x : up_x;
            const T yd = syd > 0 ? up_y : dn_y, yu = syd > 0 ? dn_y : up_y;
            const T zd = szd > 0 ? z_up : z_dn, zu = szd > 0 ? z_dn : z_up;
            m0[r] = vmin<T, ARITH>(xl, xr);
            m1[r] = vmin<T, ARITH>(yd, yu);
            m2[r] = vmin<T, ARITH>(zd, zu);
            if (MODE == MODE_REPLACE) capv[r] = capq[r][0];
          }
        }
        T nv[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
          nv[r] = cv[r];
          if (act[r]) {
            const T g = local_update<T, MODE, ARITH, ISO>(m0[r], m1[r], m2[r], k64, k32);
            nv[r] = MODE == MODE_REPLACE ? vmin<T, ARITH>(capv[r], g) : vmin<T, ARITH>(cv[r], g);
          }
          prev[r] = nv[r];
        }
        if (MODE == MODE_REPLACE) {
#pragma unroll
          for (int r = 0; r < R; ++r) {
#pragma unroll
            for (int k = 0; k + 1 < G::CP; ++k) capq[r][k] = capq[r][k + 1];
            capq[r][G::CP - 1] = cap_at(r, t + G::CP);
          }
        }
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const int lz = t - lx - ly0 - r;
          if (act[r] && vdiffers<T, ARITH>(nv[r], cv[r])) {
            ring[sr[r] * SLOT + o[r]] = nv[r];
            T d;
            if (sizeof(T) == 4)
              d = (T)__fdividef(fabsf((float)cv[r] - (float)nv[r]), fmaxf((float)nv[r], hmin));
            else
              d = (T)fabs((double)cv[r] - (double)nv[r]);
            tmax = vmax_nonneg<T, ARITH>(tmax, d);
            accb[r] = vmax_nonneg<T, ARITH>(accb[r], d);
          }
          if (valid[r] && (unsigned)lz < (unsigned)nz) {
            if (wr_x) xout[(long long)(t - (TX - 1)) * TY + ly0 + r] = nv[r];
            if (wr_y && r == R - 1) yout[(long long)(lz + lx) * TX + lx] = nv[r];
          }
        }
        __syncwarp();
        // rows completed by lane lx = TX-1 at this step: write them back
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const int lzw = t - (TX - 1) - ly0 - r;
          if (valid[r] && lzw >= zlo && lzw < zhi) {  // planes outside [zlo, zhi) are unchanged
            int s = swb - r;
            if (s < 0) s += D;
            const int gz = szd > 0 ? lzw + 1 : nz - lzw;
            u[(long long)gz * plane + grow[r]] = ring[s * SLOT + o[r]];
          }
        }
        // ring plane t-(TX-1)-ly0-(R-1) is no longer touched by this warp; a
        // mailbox chunk is released after its last step
        fence_proxy_async();
        __syncwarp();
        if (lane == 0) {
          // release every plane up to q (several at the first step of a
          // column whose range starts late: the planes below its first
          // step's release point were loaded and waited for, never used)
          const int q = min(t - (TX - 1) - ly0 - (R - 1), p_end);
          while (rel <= q) {
            mbar_arrive(empty + rslot);
            ++rel;
            if (++rslot == D) rslot = 0;
          }
          if (tc == C - 1 && kb < kb_end) mbar_arrive(bempty + (rkb & (HB - 1)));
          st_release_cta_s(done + w, t + 1);
        }
        if (++s0 == D) s0 = 0;
        if (++swb == D) swb = 0;
      }
      // the column is complete: the face items past the range were copied up front
      if (finished && lane == 0) st_release_cta_s(done + w, tsteps);
      if (blk_chg) {
#pragma unroll
        for (int r = 0; r < R; ++r)
          if (bzr[r] >= 0 && accb[r] > T(0))
            atomicMax(blk_chg + ((long long)bzr[r] * nby + byr[r]) * nbx + bxl, __float_as_uint((float)accb[r]));
      }
    }
    // the column's max change -> its grid's counter (one atomic per compute warp)
    if (warp < NW) {
      T v = tmax;
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, off));
      if (lane == 0 && v > T(0)) {
        if (sizeof(T) == 4)
          atomicMax(reinterpret_cast<unsigned int *>(a.maxchg), __float_as_uint((float)v));
        else
          atomicMax(reinterpret_cast<unsigned long long *>(a.maxchg),
                    (unsigned long long)__double_as_longlong((double)v));
      }
    }
    __syncthreads();
    if (s_abort) break;
  }
}

}  // namespace pdfs
