// internal.h -- declarations shared by the host-side translation units of libpdfs.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <algorithm>
#include <vector>
#include <cstdint>

#include "../../include/pdfs.h"
#include "sweep.cuh"

namespace pdfs {

// Internal padded layout of one element type for one tile shape
// (see sweep.cuh for the indexing rule).
// xo is the x offset of the index: V - 1 for the column kernels (interior x =
// 1 + tx*cx on a 16-byte boundary), 0 for bricks and pencils (their boxes
// start at the halo node x0 - 1 = 16*cx, on a 16-byte boundary).
// zc != 0: the z-column layout of the lane-column tiles (lanecol.cuh), node
// (x, y, z) at (y * px + x) * qz + kLcZ0 + z with px = nx + 2 columns per row
// of columns; traversal steps T, last traversal position q_last; ncx x ncy
// tiles of tx = 31 lanes by ty rows.
struct Layout {
  int tx = 0, ty = 0, V = 0, esize = 0, xo = 0;
  int ncx = 0, ncy = 0;
  long long px = 0, ry = 0, plane = 0;
  size_t elems = 0;  // total elements including padding
  int zc = 0, q_last = 0, T = 0;
  long long qz = 0;
  __host__ __device__ long long index(int x, int y, int z) const {
    return zc ? ((long long)y * px + x) * qz + kLcZ0 + z : (long long)z * plane + (long long)y * px + x + xo;
  }
};

// xo < 0: the column kernels' offset V - 1
Layout make_layout(const pdfs_grid &g, int tx, int ty, int esize, int xo = -1);
// The z-column layout of lane-column tiles of `rows` rows.
Layout make_layout_zc(const pdfs_grid &g, int rows, int esize);
// Ticket order of lane-column tiles: every tile after the tiles it waits on,
// by expected start level.
std::vector<int> lc_order(int ntx, int nty, int rows);

// Frozen bitmask layout, independent of the tile: node (x, y, z) is bit
// (x-1)%32 of word z*fplane + ((x-1)/32)*fy + (y-1).  The rows of one 32-wide
// column are contiguous, so a column's mask words for one plane are a single
// TMA box; fy is a multiple of 4 (16-byte strides).
struct MaskLayout {
  long long fy = 0, fw = 0, fplane = 0;
  size_t words = 0;
  __host__ __device__ long long word(int x, int y, int z) const {
    return (long long)z * fplane + (long long)((x - 1) >> 5) * fy + (y - 1);
  }
};
MaskLayout make_mask_layout(const pdfs_grid &g);

// A sweep kernel variant: a column tile (tx x ty, c rows per compute warp,
// bz = 0), a brick (tx x ty x bz, tile3d.cuh) or a pencil (tx x ty along z,
// pencil.cuh; block-masked sweeps on bricks of depth bz).
struct TileShape {
  int tx, ty, c;
  int bz = 0;
  int pencil = 0;
  int lc = 0;  // lane-column tile (lanecol.cuh): its rows; the field is in the ZC layout
};
// Tile ids (1-based) for FP32 and FP64 kernels.
int tile_count32();
int tile_count64();
TileShape tile32(int id);
TileShape tile64(int id);

// Launches one sweep; grid is chosen from the occupancy of the variant.
// which: 0 = FP32 min (iso / aniso from `iso`), 1 = FP64 min, 2 = FP64 replace
// (cap = upper bound field in the same layout).
cudaError_t launch_sweep(int which, int tile, int arith, bool iso, const SweepArgs &a, const Layout &L,
                         const void *cap, int sms, cudaStream_t st, int *grid_used);
// One sweep by the brick kernel (tile3d.cu): bricks of 16 x by x bz, a.tflag /
// a.torder / a.ntx.. / a.epoch filled in.
cudaError_t launch_sweep_bricks(int which, int by, int bz, int arith, bool iso, const SweepArgs &a, const Layout &L,
                                int sms, cudaStream_t st, int *grid_used);
// One unmasked sweep by the pencil kernel (pencil.cu): 16 x 16 pencils, the
// column order / progress words of a 16 x 16 layout.
cudaError_t launch_sweep_pencils(int which, int arith, bool iso, const SweepArgs &a, const Layout &L, int sms,
                                 cudaStream_t st, int *grid_used);
cudaError_t encode_mask_map(CUtensorMap *m, const SweepArgs &a, int ty);
// One round of a batch on pencils (pencil_batch.cu): the 8 orderings of every
// grid that a0.batch describes, in one launch (at most max_ticks tickets).
cudaError_t launch_pencil_round(int which, int arith, bool iso, const SweepArgs &a0, int max_ticks, int sms,
                                cudaStream_t st, int *grid_used);
cudaError_t encode_pencil_maps(int which, const SweepArgs &a, const Layout &L, CUtensorMap m[3]);
// One sweep by the lane-column kernel (lanecol.cu): which 0 = FP32 min, 1 =
// pair min, 2 = pair replace; tiles of rows = 4 or 8 rows.
cudaError_t launch_sweep_lanecol(int which, int rows, bool iso, const LcArgs &a, int sms, cudaStream_t st,
                                 int *grid_used);
// nsw <= kOctMax sweeps (orderings oct_first + 1, ..) as one launch on bricks
// over octant masks (tile3d.cu): which 0 = FP32 min-update (16 x 16 x 32
// bricks), 2 = the polish's replace-update (16 x 16 x 16).  a0 as for such a
// sweep, with oct_first, oct_full (the unmasked sweeps), oct_bits (per block)
// and oct_tbits (per brick, filled here) set, a0.epoch the first of nsw epochs
// and a0.maxchg nsw change words; list: the start of the scratch
// (octant_scratch_ints), cnt_off: list + kOctMax x bricks.
constexpr int kOctMax = 8;
// pdfs_ctx::ochg: kOctMax change words, then the node counts of the 8 orderings
constexpr int kOctWords = kOctMax + 8;
// ints of an octant round's ticket scratch (pdfs_ctx::toct) for ntx x nty x ntz bricks
int octant_scratch_ints(int ntx, int nty, int ntz);
cudaError_t launch_octant_round(int which, int arith, bool iso, int nsw, const SweepArgs &a0, const Layout &L,
                                int *list, int *cnt_off, int sms, cudaStream_t st, int *grid_used);
// Ticket order of bricks: local brick ids (lk * nty + lj) * ntx + li by level li + lj + lk.
std::vector<int> brick_order(int ntx, int nty, int ntz);
cudaError_t encode_field_map(CUtensorMap *m, void *base, int esize, const Layout &L, int nplanes, int bx, int by,
                             int bz);

// Change-based active set: blocks that changed by more than thr in any of
// the last hist sweeps, or whose face neighbour did in the last one (ring as
// for sched_learned).  *count += active blocks.
cudaError_t sched_change(const unsigned int *ring, int cur, int hist, float thr, uint8_t *active, int nbx, int nby,
                         int nbz, int *count, int sms, cudaStream_t st);
// Polish orderings per 8^3 block (bit sn-1: ordering sn matters to the
// block), from the FP32 result; and the active mask of one ordering.
cudaError_t octant_mask(const float *u32, const Layout &L, const uint32_t *fmask, const MaskLayout &M,
                        const pdfs_grid &g, float slack, float far, int nbx, int nby, int nbz, uint8_t *omask,
                        cudaStream_t st);
cudaError_t octant_active(const uint8_t *omask, int sn, int dilate, uint8_t *active, int nbx, int nby, int nbz,
                          int *count, int sms, cudaStream_t st);
cudaError_t octant_union(const uint8_t *omask, uint8_t *out, int nbx, int nby, int nbz, int sms, cudaStream_t st);
// nodes[j] += grid nodes of the blocks with bit j (ordering j + 1) set.
cudaError_t octant_nodes(const uint8_t *bits, int nbx, int nby, int nbz, int nx, int ny, int nz,
                         unsigned long long *nodes, int sms, cudaStream_t st);

// Status words a sweep writes on the device (read back after each sweep).
struct DevStatus {
  int err[4];
  unsigned long long chg;
  int active_blocks;  // blocks the scheduler activated for this sweep
  int sched_err;      // the learned scheduler's inference gave up (a bounded wait)
};


// FP32 phase convergence: max relative change of a full sweep (FP32
// rounding creep stays around 1e-7).
constexpr float kTol32 = 4.0e-6f;

// Schedulers keep the per-block max change of the current sweep and of the
// kHist sweeps before it in a ring of kHist + 1 slots (one full cycle of
// orderings: a block that changes again has, in practice, changed within
// the last cycle).
constexpr int kHist = 8;
constexpr int kRing = kHist + 1;
// The learned scheduler recomputes its band feature every kBandEvery
// scheduled sweeps (a pass over the field each time).
constexpr int kBandEvery = 4;
// Octant masks: an axis whose two neighbours differ by at most kOctSlack * h
// accepts both sweep directions (FP32 rounds / the polish); kOctDilate = 1
// adds each block's face neighbours' orderings.  Measured on the 768^3
// headline grid under the octant scheduler (solve time; always 16 FP32 and 9
// polish sweeps): FP32 slack 0.25 with polish slack 0.25 102.0 ms, 0.15 100.4,
// 0.1 99.9, 0.05 99.5, 0 99.1 ms (0.05 keeps a margin for the characteristics
// nearly parallel to a face); FP32 slack 0.2 / 0.3 within 0.3 ms of 0.25, 0.1
// needs a second FP32 round (122.6 ms), 0.5 103.0 ms; without the
// widening the FP32 phase needs a second round (127 ms).  Earlier, for the
// polish alone run one masked sweep at a time: slack 0.25 widened 52.1 ms and
// 9 sweeps, not widened 54.4 ms and 10; slack 0.5 56.4 / 57.3 ms.
constexpr float kOctSlack32 = 0.25f;
constexpr float kOctSlack64 = 0.05f;
constexpr int kOctDilate = 1;

// Weights of the learned scheduler compiled into the library (a blob of
// PDFS_MLP_BLOB floats), or nullptr when none were built in.
const float *default_mlp_blob();
// Learned scheduler (mlp.cu): per-block minimum of a working field, and the
// fused feature + network + decision kernel (active[b], *count += actives).
// kind: 0 FP32 field, 1 FP64 field, 2 FP32-pair field
cudaError_t block_min(const void *u, int kind, const Layout &L, const pdfs_grid &g, int nbx, int nby, int nbz,
                      float *bmin, cudaStream_t st);
// ring: kRing slots of nblocks change words, slot cur = the sweep about to
// run, slot (cur - k) mod kRing = k sweeps ago, hist = sweeps of history.
// The network runs on the tensor cores (tcgen05); *err is set if one of its
// accumulator waits gives up.
cudaError_t sched_learned(const uint16_t *w, float thr, const unsigned int *ring, int cur, int hist,
                          const float *bmin, int nbx, int nby, int nbz, int sn, int sweep, int phase, float tol,
                          float hmin, uint8_t *active, int *count, int *err, int sms, cudaStream_t st);

// Steps per mailbox chunk (matches WsGeo::C).
constexpr int kMailboxChunk = 4;
inline int mailbox_chunks(int nz) { return (nz + 32 + kMailboxChunk - 1) / kMailboxChunk; }

}  // namespace pdfs

// The context behind the opaque pdfs_ctx handle of the C ABI.
struct pdfs_ctx {
  pdfs_grid g{};
  pdfs_opts o{};
  int dev = 0, sms = 0;
  cudaStream_t st = nullptr;
  int t32 = 1, t64 = 1;
  pdfs::Layout L32, L64;
  pdfs::MaskLayout M;
  double *in64 = nullptr;   // exact input, internal FP64 layout (also the polish cap)
  double *u64 = nullptr;    // FP64 working field (FP32 pairs under PDFS_ARITH_PAIR)
  double *bcap64 = nullptr; // polish: per 8^3 block, the smallest cap of its updated nodes
  float *bcap32 = nullptr;  // the same rounded down to float
  float *u32 = nullptr;     // FP32 working field
  uint32_t *fmask = nullptr;
  void *arena = nullptr;    // every device buffer below but the stage, as one allocation
  size_t arena_bytes = 0;
  void *stage = nullptr;    // reference-layout staging buffer for host transfers
  size_t stage_bytes = 0;
  int *order32 = nullptr, *order64 = nullptr, *progress = nullptr, *ticket = nullptr;
  // brick tiles (tile3d.cuh): per-brick completion epochs, ticket orders, brick grids
  int *tflag = nullptr, *tord32 = nullptr, *tord64 = nullptr;
  // block-masked brick sweeps: per brick, an active block?  and [count, tickets...]
  uint8_t *tact = nullptr;
  int *tsparse = nullptr;
  int nt32[3] = {0, 0, 0}, nt64[3] = {0, 0, 0};
  int epoch = 0;  // flag value of the last brick or pencil sweep
  unsigned long long *pmail = nullptr;  // pencils: epoch-tagged face mailboxes
  int prow = 0;                          // their diagonals per face
  // lane-column tiles: ticket orders, and the epoch-tagged face mailboxes
  int *lcord32 = nullptr, *lcord64 = nullptr;
  unsigned long long *lc_ymail = nullptr, *lc_xmail = nullptr;
  void *mailbox = nullptr;  // x- and y-face mailboxes of every column
  size_t mailbox_bytes = 0;
  size_t progress_ints = 0;
  pdfs::DevStatus *dstat = nullptr;
  pdfs::DevStatus *hstat = nullptr;  // pinned
  // 8^3 block bookkeeping for the scheduler
  int nbx = 0, nby = 0, nbz = 0;
  long long nblocks = 0;
  unsigned int *bchg = nullptr;  // [kRing][nblocks] float bits of per-block max change, rotating
  uint8_t *bact = nullptr;       // [nblocks] active mask of the next sweep
  uint8_t *omask = nullptr;      // [nblocks] polish: the orderings that matter to each block
  int *toct = nullptr;           // octant rounds: [8][bricks] tickets, 17 counts / offsets, the merged
                                 // ticket list and its plan (octant_scratch_ints)
  bool oct32_ok = false, oct64_ok = false;  // octant rounds available (FP32 / polish brick shapes)
  unsigned long long *ochg = nullptr;  // its 8 change words
  float *bmin = nullptr;         // [nblocks] per-block field minimum (learned scheduler)
  uint16_t *mlp_w = nullptr;     // learned scheduler: bf16 network weights
  float mlp_thr = 0.0f;          // its decision threshold on the logit
  bool loaded = false, has_mask = false;
  int last_prec = -1;      // which working field holds the last result
  cudaEvent_t e0 = nullptr, e1 = nullptr, k0 = nullptr, k1 = nullptr, q0 = nullptr, q1 = nullptr;
  cudaEvent_t r0 = nullptr, r1 = nullptr;  // around a whole pdfs_ctx_run
  // load / store pipeline: slab copies on st, layout kernels on st2
  cudaStream_t st2 = nullptr;
  static constexpr int kSlabs = 32;
  cudaEvent_t slab_ev[kSlabs + 1] = {};
  double kern_ms = 0.0;  // accumulated sweep-kernel time since the last reset
  int launches = 0;      // kernels launched since the last reset
};

namespace pdfs {
void fill_sweep_args(const pdfs_ctx *c, int which, int sn, const uint8_t *active, unsigned int *blk_chg,
                     SweepArgs *out);
// Sweep direction of ordering sn (1..8), +1 ascending, from makeSweepInfo
// (mpi_openacc/src/phi3D_fsm.c:206-218): a reflection offset reverses its
// axis, descending levels reverse all three.
__host__ __device__ inline void ordering_signs(int sn, int *sx, int *sy, int *sz) {
  const int desc = (sn == 2 || sn == 5 || sn == 7 || sn == 8) ? -1 : 1;
  *sx = ((sn == 4 || sn == 8) ? -1 : 1) * desc;
  *sy = ((sn == 2 || sn == 6) ? -1 : 1) * desc;
  *sz = ((sn == 3 || sn == 7) ? -1 : 1) * desc;
}
std::vector<int> wavefront_order(int ncx, int ncy, int tx, int ty);
// One sweep of context c (which: 0 FP32 min, 1 FP64 min, 2 FP64 replace):
// active = block mask or nullptr, blk_chg = per-block change or nullptr.
int ctx_sweep_once(pdfs_ctx *c, int which, int sn, const uint8_t *active, unsigned int *blk_chg, double *chg);
// FP64 input -> FP32 working field / FP32 result -> FP64 polish start
int ctx_narrow(pdfs_ctx *c);
int ctx_widen(pdfs_ctx *c);
// the FP64 working field <- the input (a copy, or its pairs)
int ctx_fp64_start(pdfs_ctx *c);
// Tensor maps of one grid for a sweep kernel variant: field, cap, mask.
cudaError_t encode_sweep_maps(int which, int tile, const SweepArgs &a, const Layout &L, const void *cap,
                              CUtensorMap maps[3]);
// One batched sweep over the grids that a0.batch describes (ntick tickets).
cudaError_t launch_sweep_batch(int which, int tile, int arith, bool iso, const SweepArgs &a0, int ntick, int sms,
                               cudaStream_t st, int *grid_used);
}  // namespace pdfs
