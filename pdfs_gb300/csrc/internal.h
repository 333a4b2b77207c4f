// internal.h -- declarations shared by the host-side translation units of libpdfs.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
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

// Frozen bitmask layout: bit (x-1) of word row (z, y); independent of the tile.
struct MaskLayout {
  long long fpw = 0, fry = 0, fplane = 0;
  size_t words = 0;
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
// which: 0 = FP32 min (iso / aniso from `iso`), 1 = FP64 min, 2 = FP64 replace.
cudaError_t launch_sweep(int which, int tile, int arith, bool iso, const SweepArgs &a, int sms,
                         cudaStream_t st, int *grid_used);

}  // namespace pdfs
