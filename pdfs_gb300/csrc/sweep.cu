// sweep.cu -- instantiations and launcher of the warp-specialised sweep kernels.
#include <cudaTypedefs.h>

#include <cstring>


#include "internal.h"

namespace pdfs {

// Tile variants.  Columns (sweep.cuh) are 32 nodes wide (one warp lane per
// x); TY rows, R rows per compute warp: {tx, ty, rows per warp}.  Bricks
// (tile3d.cuh) are 16 x 16 x BZ: {16, 16, 0, BZ}.
// Bricks may also be 16 x 8 x BZ.  Pencils (pencil.cuh) are 16 x 16
// cross-sections marched along z: {16, 16, 0, BZ, 1}; their block-masked
// sweeps run on 16 x 16 x BZ bricks.
// Lane-column tiles (lanecol.cuh): 31 lanes x R rows of z-columns (R = 8 or
// 4), {31, R, 0, 0, 0, R}; their block-masked sweeps run on the same kernel.
static const TileShape kT32[] = {{32, 8, 2},  {32, 8, 4},  {32, 16, 4},     {32, 8, 1},      {32, 4, 2},
                                 {32, 6, 1},  {32, 10, 1}, {16, 16, 0, 16}, {16, 16, 0, 32}, {16, 16, 0, 32, 1},
                                 {16, 8, 0, 48}, {31, 8, 0, 0, 0, 8},      {31, 4, 0, 0, 0, 4}};
// tile 4 (32 x 6, one row per warp) exists for the fast and mixed arithmetic
static const TileShape kT64[] = {{32, 4, 1},      {32, 4, 2},         {32, 8, 2},     {32, 6, 1},
                                 {16, 16, 0, 16}, {16, 16, 0, 16, 1}, {16, 16, 0, 32}, {16, 8, 0, 32},
                                 {31, 8, 0, 0, 0, 8}, {31, 4, 0, 0, 0, 4}};

int tile_count32() { return (int)(sizeof(kT32) / sizeof(kT32[0])); }
int tile_count64() { return (int)(sizeof(kT64) / sizeof(kT64[0])); }
TileShape tile32(int id) { return kT32[(id >= 1 && id <= tile_count32()) ? id - 1 : 0]; }
TileShape tile64(int id) { return kT64[(id >= 1 && id <= tile_count64()) ? id - 1 : 0]; }

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

// 3-D tiled map over an internal-layout field: dims {px, ry, nz+2}, box {bx, by, bz}.
cudaError_t encode_field_map(CUtensorMap *m, void *base, int esize, const Layout &L, int nplanes, int bx, int by,
                             int bz) {
  auto fn = encode_fn();
  if (!fn) return cudaErrorNotSupported;
  cuuint64_t dims[3] = {(cuuint64_t)L.px, (cuuint64_t)L.ry, (cuuint64_t)nplanes};
  cuuint64_t strides[2] = {(cuuint64_t)L.px * esize, (cuuint64_t)L.plane * esize};
  cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)by, (cuuint32_t)bz};
  cuuint32_t es[3] = {1, 1, 1};
  CUresult r = fn(m, esize == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, base, dims,
                  strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

// Frozen-mask map: 32-bit words, dims {fy, fw, nz+2}, box {MBOX, 1, 1} (the
// column's TY rows rounded up to a 16-byte box).
cudaError_t encode_mask_map(CUtensorMap *m, const SweepArgs &a, int ty) {
  auto fn = encode_fn();
  if (!fn) return cudaErrorNotSupported;
  cuuint64_t dims[3] = {(cuuint64_t)a.mask_fy, (cuuint64_t)a.mask_fw, (cuuint64_t)(a.nz + 2)};
  cuuint64_t strides[2] = {(cuuint64_t)a.mask_fy * 4, (cuuint64_t)(a.mask_fy * a.mask_fw) * 4};
  cuuint32_t box[3] = {(cuuint32_t)ty, 1, 1};
  cuuint32_t es[3] = {1, 1, 1};
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_UINT32, 3, const_cast<uint32_t *>(a.fmask), dims, strides, box, es,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

// The tensor maps a variant reads: field slots, (unused), mask words.
template <class T, int TY, int R, int MODE>
static cudaError_t encode_maps(const SweepArgs &a, const Layout &L, const void *cap, CUtensorMap m[3]) {
  using G = WsGeo<T, TY, R, MODE>;
  cudaError_t e = encode_field_map(&m[0], a.u, sizeof(T), L, a.nz + 2, G::W, G::R, 1);
  if (e != cudaSuccess) return e;
  (void)cap;  // the polish cap is read through a.cap, not a map
  m[1] = m[0];
  if (a.fmask) {
    e = encode_mask_map(&m[2], a, G::MBOX);
    if (e != cudaSuccess) return e;
  } else {
    m[2] = m[0];
  }
  return cudaSuccess;
}

// Single grid (a.batch == nullptr): maps from a and L.  Batched: the maps
// live with each grid's description in device memory, ntick tickets.
template <class T, int TY, int R, int MODE, int ARITH, bool ISO>
static cudaError_t launch_one(const SweepArgs &a, const Layout *L, const void *cap, int ntick, int sms,
                              cudaStream_t st, int *grid_used) {
  using G = WsGeo<T, TY, R, MODE>;
  auto kern = ws_sweep_kernel<T, TY, R, MODE, ARITH, ISO>;
  CUtensorMap m[3];
  cudaError_t e = cudaSuccess;
  if (a.batch == nullptr) {
    e = encode_maps<T, TY, R, MODE>(a, *L, cap, m);
    if (e != cudaSuccess) return e;
  } else {
    std::memset(m, 0, sizeof(m));
  }
  const size_t smem = G::BYTES;
  e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, G::NT, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  int grid = per_sm * sms;
  if (grid > ntick) grid = ntick;
  if (grid < 1) grid = 1;
  kern<<<grid, G::NT, smem, st>>>(m[0], m[1], m[2], a);
  if (grid_used) *grid_used = grid;
  return cudaGetLastError();
}

#define PDFS_T32(ID, TY, R)                                                                           \
  case ID:                                                                                            \
    return iso ? launch_one<float, TY, R, MODE_MIN, ARITH_FAST, true>(a, L, cap, ntick, sms, st, g)   \
               : launch_one<float, TY, R, MODE_MIN, ARITH_FAST, false>(a, L, cap, ntick, sms, st, g);
#define PDFS_T64(ID, TY, R, MODE)                                                                            \
  case ID:                                                                                                   \
    return arith == ARITH_REF ? launch_one<double, TY, R, MODE, ARITH_REF, false>(a, L, cap, ntick, sms, st, g) \
                              : launch_one<double, TY, R, MODE, ARITH_FAST, false>(a, L, cap, ntick, sms, st, g);
// FP64 field with FP32 increments: tiles 1 (TY = 4) and 4 (TY = 6), one row per warp
#define PDFS_T64M(TY, MODE)                                                                              \
  return iso ? launch_one<double, TY, 1, MODE, ARITH_MIXED, true>(a, L, cap, ntick, sms, st, g)         \
             : launch_one<double, TY, 1, MODE, ARITH_MIXED, false>(a, L, cap, ntick, sms, st, g);

static cudaError_t dispatch(int which, int tile, int arith, bool iso, const SweepArgs &a, const Layout *L,
                            const void *cap, int ntick, int sms, cudaStream_t st, int *g) {
  if (which == 0) {
    switch (tile) {
      PDFS_T32(1, 8, 2)
      PDFS_T32(2, 8, 4)
      PDFS_T32(3, 16, 4)
      PDFS_T32(4, 8, 1)
      PDFS_T32(5, 4, 2)
      PDFS_T32(6, 6, 1)
      PDFS_T32(7, 10, 1)
      default:
        return cudaErrorInvalidValue;
    }
  } else if (arith == ARITH_MIXED) {
    if (tile == 1) {
      if (which == 1) {
        PDFS_T64M(4, MODE_MIN)
      } else {
        PDFS_T64M(4, MODE_REPLACE)
      }
    } else if (tile == 4) {
      if (which == 1) {
        PDFS_T64M(6, MODE_MIN)
      } else {
        PDFS_T64M(6, MODE_REPLACE)
      }
    }
    return cudaErrorInvalidValue;
  } else if (tile == 4) {  // fast arithmetic only (validated by the caller)
    if (which == 1)
      return launch_one<double, 6, 1, MODE_MIN, ARITH_FAST, false>(a, L, cap, ntick, sms, st, g);
    return launch_one<double, 6, 1, MODE_REPLACE, ARITH_FAST, false>(a, L, cap, ntick, sms, st, g);
  } else if (which == 1) {
    switch (tile) {
      PDFS_T64(1, 4, 1, MODE_MIN)
      PDFS_T64(2, 4, 2, MODE_MIN)
      PDFS_T64(3, 8, 2, MODE_MIN)
      default:
        return cudaErrorInvalidValue;
    }
  } else {
    switch (tile) {
      PDFS_T64(1, 4, 1, MODE_REPLACE)
      PDFS_T64(2, 4, 2, MODE_REPLACE)
      default:
        return cudaErrorInvalidValue;
    }
  }
}
#undef PDFS_T32
#undef PDFS_T64
#undef PDFS_T64M

cudaError_t launch_sweep(int which, int tile, int arith, bool iso, const SweepArgs &a, const Layout &L,
                         const void *cap, int sms, cudaStream_t st, int *g) {
  return dispatch(which, tile, arith, iso, a, &L, cap, a.ncx * a.ncy, sms, st, g);
}

cudaError_t launch_sweep_batch(int which, int tile, int arith, bool iso, const SweepArgs &a0, int ntick, int sms,
                               cudaStream_t st, int *g) {
  if (!a0.batch || ntick < 1) return cudaErrorInvalidValue;
  return dispatch(which, tile, arith, iso, a0, nullptr, nullptr, ntick, sms, st, g);
}

#define PDFS_M32(ID, TY, R) \
  case ID:                  \
    return encode_maps<float, TY, R, MODE_MIN>(a, L, cap, m);
#define PDFS_M64(ID, TY, R, MODE) \
  case ID:                        \
    return encode_maps<double, TY, R, MODE>(a, L, cap, m);

cudaError_t encode_sweep_maps(int which, int tile, const SweepArgs &a, const Layout &L, const void *cap,
                              CUtensorMap m[3]) {
  if (which == 0) {
    switch (tile) {
      PDFS_M32(1, 8, 2)
      PDFS_M32(2, 8, 4)
      PDFS_M32(3, 16, 4)
      PDFS_M32(4, 8, 1)
      PDFS_M32(5, 4, 2)
      PDFS_M32(6, 6, 1)
      PDFS_M32(7, 10, 1)
      default:
        return cudaErrorInvalidValue;
    }
  } else if (which == 1) {
    switch (tile) {
      PDFS_M64(1, 4, 1, MODE_MIN)
      PDFS_M64(2, 4, 2, MODE_MIN)
      PDFS_M64(3, 8, 2, MODE_MIN)
      PDFS_M64(4, 6, 1, MODE_MIN)
      default:
        return cudaErrorInvalidValue;
    }
  } else {
    switch (tile) {
      PDFS_M64(1, 4, 1, MODE_REPLACE)
      PDFS_M64(2, 4, 2, MODE_REPLACE)
      PDFS_M64(4, 6, 1, MODE_REPLACE)
      default:
        return cudaErrorInvalidValue;
    }
  }
}
#undef PDFS_M32
#undef PDFS_M64

}  // namespace pdfs
