// tile3d.cu -- instantiations and launcher of the brick sweep kernel (tile3d.cuh).
#include <algorithm>

#include "internal.h"
#include "tile3d.cuh"

namespace pdfs {

std::vector<int> brick_order(int ntx, int nty, int ntz) {
  // a brick waits for one brick a level below in each axis: listing bricks by
  // level (x + y + z), in index order within a level, lists all three first,
  // which is all the deadlock argument needs.  A counting sort by level.
  const size_t n = (size_t)ntx * nty * ntz;
  const int levels = ntx + nty + ntz - 2;
  std::vector<size_t> start((size_t)levels + 1, 0);
  for (int z = 0; z < ntz; ++z)
    for (int y = 0; y < nty; ++y)
      for (int x = 0; x < ntx; ++x) ++start[x + y + z + 1];
  for (int l = 0; l < levels; ++l) start[l + 1] += start[l];
  std::vector<int> o(n);
  int i = 0;
  for (int z = 0; z < ntz; ++z)
    for (int y = 0; y < nty; ++y)
      for (int x = 0; x < ntx; ++x) o[start[x + y + z]++] = i++;
  return o;
}

template <class T, int BY, int BZ, int MODE, int ARITH, bool ISO>
static cudaError_t launch_t3(const SweepArgs &a, const Layout &L, int sms, cudaStream_t st, int *grid_used) {
  using G = T3Geo<T, BY, BZ>;
  auto kern = t3_sweep_kernel<T, BY, BZ, MODE, ARITH, ISO>;
  CUtensorMap m;
  cudaError_t e = encode_field_map(&m, a.u, sizeof(T), L, a.nz + 2, G::W, G::RY, G::RZ);
  if (e != cudaSuccess) return e;
  const size_t smem = G::BYTES;
  e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, G::NT, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  const int ntile = a.ntx * a.nty * a.ntz;
  int grid = std::min(per_sm * sms, ntile);
  if (grid < 1) grid = 1;
  kern<<<grid, G::NT, smem, st>>>(m, a);
  if (grid_used) *grid_used = grid;
  return cudaGetLastError();
}

template <int BY, int BZ>
static cudaError_t dispatch_t3(int which, int arith, bool iso, const SweepArgs &a, const Layout &L, int sms,
                               cudaStream_t st, int *g) {
  if (which == 0)
    return iso ? launch_t3<float, BY, BZ, MODE_MIN, ARITH_FAST, true>(a, L, sms, st, g)
               : launch_t3<float, BY, BZ, MODE_MIN, ARITH_FAST, false>(a, L, sms, st, g);
  {
    if (which == 1) {
      if (arith == ARITH_REF) return launch_t3<double, BY, BZ, MODE_MIN, ARITH_REF, false>(a, L, sms, st, g);
      if (arith == ARITH_FAST) return launch_t3<double, BY, BZ, MODE_MIN, ARITH_FAST, false>(a, L, sms, st, g);
      if (arith == ARITH_PAIR)
        return iso ? launch_t3<double, BY, BZ, MODE_MIN, ARITH_PAIR, true>(a, L, sms, st, g)
                   : launch_t3<double, BY, BZ, MODE_MIN, ARITH_PAIR, false>(a, L, sms, st, g);
      return iso ? launch_t3<double, BY, BZ, MODE_MIN, ARITH_MIXED, true>(a, L, sms, st, g)
                 : launch_t3<double, BY, BZ, MODE_MIN, ARITH_MIXED, false>(a, L, sms, st, g);
    }
    if (arith == ARITH_REF) return launch_t3<double, BY, BZ, MODE_REPLACE, ARITH_REF, false>(a, L, sms, st, g);
    if (arith == ARITH_FAST) return launch_t3<double, BY, BZ, MODE_REPLACE, ARITH_FAST, false>(a, L, sms, st, g);
    if (arith == ARITH_PAIR)
      return iso ? launch_t3<double, BY, BZ, MODE_REPLACE, ARITH_PAIR, true>(a, L, sms, st, g)
                 : launch_t3<double, BY, BZ, MODE_REPLACE, ARITH_PAIR, false>(a, L, sms, st, g);
    return iso ? launch_t3<double, BY, BZ, MODE_REPLACE, ARITH_MIXED, true>(a, L, sms, st, g)
               : launch_t3<double, BY, BZ, MODE_REPLACE, ARITH_MIXED, false>(a, L, sms, st, g);
  }
}

cudaError_t launch_sweep_bricks(int which, int by, int bz, int arith, bool iso, const SweepArgs &a, const Layout &L,
                                int sms, cudaStream_t st, int *g) {
  if (!a.tflag || !a.torder || a.ntx < 1 || a.nty < 1 || a.ntz < 1 || L.ty != by || L.tx != 16 || L.xo != 0 ||
      (which == 2 && (!a.bcap64 || !a.bcap32)))
    return cudaErrorInvalidValue;
  if (by == 16 && bz == 16) return dispatch_t3<16, 16>(which, arith, iso, a, L, sms, st, g);
  if (by == 16 && bz == 32) return dispatch_t3<16, 32>(which, arith, iso, a, L, sms, st, g);
  if (by == 8 && bz == 32) return dispatch_t3<8, 32>(which, arith, iso, a, L, sms, st, g);
  if (by == 8 && bz == 48 && which == 0)  // FP32 only
    return iso ? launch_t3<float, 8, 48, MODE_MIN, ARITH_FAST, true>(a, L, sms, st, g)
               : launch_t3<float, 8, 48, MODE_MIN, ARITH_FAST, false>(a, L, sms, st, g);
  return cudaErrorInvalidValue;
}

}  // namespace pdfs
