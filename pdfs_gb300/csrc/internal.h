// internal.h -- declarations shared by the host-side translation units of libpdfs.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <algorithm>
#include <cstdint>

#include "../../include/pdfs.h"
#include "sweep.cuh"

namespace pdfs {

// Internal padded layout of one element type for one tile shape
// (see sweep.cuh for the indexing rule).
struct Layout {
  int tx = 0, ty = 0, V = 0, esize = 0;
  int ncx = 0, ncy = 0;
  long long px = 0, ry = 0, plane = 0;
  size_t elems = 0;  // total elements including padding
  __host__ __device__ long long index(int x, int y, int z) const { return (long long)z * plane + (long long)y * px + x + (V - 1); }
};

Layout make_layout(const pdfs_grid &g, int tx, int ty, int esize);

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

// A sweep kernel variant: element type, tile, chunk depth.
struct TileShape {
  int tx, ty, c;
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

// Change-based active set: blocks (or their face neighbours) that changed by
// more than thr in either of the last two sweeps.  *count += active blocks.
cudaError_t sched_change(const unsigned int *chg1, const unsigned int *chg2, float thr, uint8_t *active, int nbx,
                         int nby, int nbz, int *count, int sms, cudaStream_t st);

// Steps per mailbox chunk (matches WsGeo::C).
constexpr int kMailboxChunk = 4;
inline int mailbox_chunks(int nz) { return (nz + 32 + kMailboxChunk - 1) / kMailboxChunk; }

}  // namespace pdfs
