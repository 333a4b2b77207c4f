// sweep.cu -- instantiations and launcher of the column-pipelined sweep kernels.
#include "internal.h"

namespace pdfs {

// FP32 tiles: 32 lanes span x so each warp reads one smem row (bank-conflict
// free without a swizzle); TY sets the skew (TX+TY-2) and the column count.
static const TileShape kTiles32[] = {{32, 8, 4}, {32, 4, 4}, {32, 16, 2}, {32, 8, 2}};
// FP64 tiles: a 16-lane half warp reads 128 contiguous bytes per row.
static const TileShape kTiles64[] = {{16, 8, 2}, {32, 8, 2}, {16, 16, 2}, {32, 4, 2}};

int tile_count32() { return (int)(sizeof(kTiles32) / sizeof(kTiles32[0])); }
int tile_count64() { return (int)(sizeof(kTiles64) / sizeof(kTiles64[0])); }
TileShape tile32(int id) { return kTiles32[(id >= 1 && id <= tile_count32()) ? id - 1 : 0]; }
TileShape tile64(int id) { return kTiles64[(id >= 1 && id <= tile_count64()) ? id - 1 : 0]; }

template <class T, int TX, int TY, int C, int MODE, int ARITH, bool ISO>
static cudaError_t launch_one(const SweepArgs &a, int sms, cudaStream_t st, int *grid_used) {
  auto kern = col_sweep_kernel<T, TX, TY, C, MODE, ARITH, ISO>;
  const size_t smem = ColGeo<T, TX, TY, C>::smem_bytes(MODE == MODE_REPLACE);
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, TX * TY, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  const int ncol = a.ncx * a.ncy;
  int grid = per_sm * sms;
  if (grid > ncol) grid = ncol;
  kern<<<grid, TX * TY, smem, st>>>(a);
  if (grid_used) *grid_used = grid;
  return cudaGetLastError();
}

#define PDFS_T32(ID, TX, TY, C)                                                               \
  case ID:                                                                                    \
    return iso ? launch_one<float, TX, TY, C, MODE_MIN, ARITH_FAST, true>(a, sms, st, g)      \
               : launch_one<float, TX, TY, C, MODE_MIN, ARITH_FAST, false>(a, sms, st, g);
#define PDFS_T64(ID, TX, TY, C, MODE)                                                          \
  case ID:                                                                                     \
    return arith == ARITH_REF ? launch_one<double, TX, TY, C, MODE, ARITH_REF, false>(a, sms, st, g) \
                              : launch_one<double, TX, TY, C, MODE, ARITH_FAST, false>(a, sms, st, g);

cudaError_t launch_sweep(int which, int tile, int arith, bool iso, const SweepArgs &a, int sms,
                         cudaStream_t st, int *g) {
  if (which == 0) {
    switch (tile) {
      PDFS_T32(1, 32, 8, 4)
      PDFS_T32(2, 32, 4, 4)
      PDFS_T32(3, 32, 16, 2)
      PDFS_T32(4, 32, 8, 2)
      default:
        return cudaErrorInvalidValue;
    }
  } else if (which == 1) {
    switch (tile) {
      PDFS_T64(1, 16, 8, 2, MODE_MIN)
      PDFS_T64(2, 32, 8, 2, MODE_MIN)
      PDFS_T64(3, 16, 16, 2, MODE_MIN)
      PDFS_T64(4, 32, 4, 2, MODE_MIN)
      default:
        return cudaErrorInvalidValue;
    }
  } else {
    switch (tile) {
      PDFS_T64(1, 16, 8, 2, MODE_REPLACE)
      PDFS_T64(2, 32, 8, 2, MODE_REPLACE)
      PDFS_T64(3, 16, 16, 2, MODE_REPLACE)
      PDFS_T64(4, 32, 4, 2, MODE_REPLACE)
      default:
        return cudaErrorInvalidValue;
    }
  }
}
#undef PDFS_T32
#undef PDFS_T64

}  // namespace pdfs
