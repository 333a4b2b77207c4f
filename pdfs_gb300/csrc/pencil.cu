// pencil.cu -- instantiations and launcher of the pencil sweep kernel (pencil.cuh).
#include <algorithm>

#include "internal.h"
#include "pencil.cuh"

namespace pdfs {

template <class T, int MODE, int ARITH, bool ISO>
static cudaError_t launch_pc(const SweepArgs &a, const Layout &L, int sms, cudaStream_t st, int *grid_used) {
  using G = PcGeo<T>;
  auto kern = pc_sweep_kernel<T, MODE, ARITH, ISO>;
  CUtensorMap m[2];
  cudaError_t e = encode_field_map(&m[0], a.u, sizeof(T), L, a.nz + 2, G::W, G::RY, 1);
  if (e != cudaSuccess) return e;
  if (a.fmask) {
    e = encode_mask_map(&m[1], a, G::BY);
    if (e != cudaSuccess) return e;
  } else {
    m[1] = m[0];
  }
  const size_t smem = G::BYTES;
  e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, G::NT, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  int grid = std::min(per_sm * sms, a.ncx * a.ncy);
  if (grid < 1) grid = 1;
  kern<<<grid, G::NT, smem, st>>>(m[0], m[1], a);
  if (grid_used) *grid_used = grid;
  return cudaGetLastError();
}

cudaError_t launch_sweep_pencils(int which, int arith, bool iso, const SweepArgs &a, const Layout &L, int sms,
                                 cudaStream_t st, int *g) {
  if (L.tx != 16 || L.ty != 16 || L.xo != 0 || a.blk_active || a.blk_chg || !a.pmail || a.prow < a.nz + 15 ||
      (which == 2 && (!a.bcap64 || !a.bcap32)))
    return cudaErrorInvalidValue;
  if (which == 0)
    return iso ? launch_pc<float, MODE_MIN, ARITH_FAST, true>(a, L, sms, st, g)
               : launch_pc<float, MODE_MIN, ARITH_FAST, false>(a, L, sms, st, g);
  const bool rep = which == 2;
  switch (arith) {
    case ARITH_REF:
      return rep ? launch_pc<double, MODE_REPLACE, ARITH_REF, false>(a, L, sms, st, g)
                 : launch_pc<double, MODE_MIN, ARITH_REF, false>(a, L, sms, st, g);
    case ARITH_FAST:
      return rep ? launch_pc<double, MODE_REPLACE, ARITH_FAST, false>(a, L, sms, st, g)
                 : launch_pc<double, MODE_MIN, ARITH_FAST, false>(a, L, sms, st, g);
    case ARITH_MIXED:
      if (iso)
        return rep ? launch_pc<double, MODE_REPLACE, ARITH_MIXED, true>(a, L, sms, st, g)
                   : launch_pc<double, MODE_MIN, ARITH_MIXED, true>(a, L, sms, st, g);
      return rep ? launch_pc<double, MODE_REPLACE, ARITH_MIXED, false>(a, L, sms, st, g)
                 : launch_pc<double, MODE_MIN, ARITH_MIXED, false>(a, L, sms, st, g);
    case ARITH_PAIR:
      if (iso)
        return rep ? launch_pc<double, MODE_REPLACE, ARITH_PAIR, true>(a, L, sms, st, g)
                   : launch_pc<double, MODE_MIN, ARITH_PAIR, true>(a, L, sms, st, g);
      return rep ? launch_pc<double, MODE_REPLACE, ARITH_PAIR, false>(a, L, sms, st, g)
                 : launch_pc<double, MODE_MIN, ARITH_PAIR, false>(a, L, sms, st, g);
    default:
      return cudaErrorInvalidValue;
  }
}

}  // namespace pdfs
