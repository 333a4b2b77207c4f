// pencil_batch.cu -- the pencil kernel's batched rounds (pencil.cuh, BATCH):
// one launch sweeps the 8 orderings of a round for every grid of a batch.
#include <algorithm>
#include <cstring>

#include "internal.h"
#include "pencil.cuh"

namespace pdfs {

template <class T, int MODE, int ARITH, bool ISO>
static cudaError_t launch_round(const SweepArgs &a0, int max_ticks, int sms, cudaStream_t st, int *grid_used) {
  using G = PcGeo<T>;
  auto kern = pc_sweep_kernel<T, MODE, ARITH, ISO, true>;
  CUtensorMap unused;  // the grids' maps come from the batch description
  std::memset(&unused, 0, sizeof unused);
  const size_t smem = G::BYTES;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, G::NT, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  // every CTA resident at once: a ticket waits only on smaller tickets, which
  // running CTAs hold
  int grid = std::min(per_sm * sms, max_ticks);
  if (grid < 1) grid = 1;
  kern<<<grid, G::NT, smem, st>>>(unused, unused, a0);
  if (grid_used) *grid_used = grid;
  return cudaGetLastError();
}

cudaError_t launch_pencil_round(int which, int arith, bool iso, const SweepArgs &a0, int max_ticks, int sms,
                                cudaStream_t st, int *g) {
  if (!a0.batch || max_ticks < 1) return cudaErrorInvalidValue;
  if (which == 0)
    return iso ? launch_round<float, MODE_MIN, ARITH_FAST, true>(a0, max_ticks, sms, st, g)
               : launch_round<float, MODE_MIN, ARITH_FAST, false>(a0, max_ticks, sms, st, g);
  const bool rep = which == 2;
  switch (arith) {
    case ARITH_REF:
      return rep ? launch_round<double, MODE_REPLACE, ARITH_REF, false>(a0, max_ticks, sms, st, g)
                 : launch_round<double, MODE_MIN, ARITH_REF, false>(a0, max_ticks, sms, st, g);
    case ARITH_FAST:
      return rep ? launch_round<double, MODE_REPLACE, ARITH_FAST, false>(a0, max_ticks, sms, st, g)
                 : launch_round<double, MODE_MIN, ARITH_FAST, false>(a0, max_ticks, sms, st, g);
    case ARITH_MIXED:
      if (iso)
        return rep ? launch_round<double, MODE_REPLACE, ARITH_MIXED, true>(a0, max_ticks, sms, st, g)
                   : launch_round<double, MODE_MIN, ARITH_MIXED, true>(a0, max_ticks, sms, st, g);
      return rep ? launch_round<double, MODE_REPLACE, ARITH_MIXED, false>(a0, max_ticks, sms, st, g)
                 : launch_round<double, MODE_MIN, ARITH_MIXED, false>(a0, max_ticks, sms, st, g);
    case ARITH_PAIR:
      if (iso)
        return rep ? launch_round<double, MODE_REPLACE, ARITH_PAIR, true>(a0, max_ticks, sms, st, g)
                   : launch_round<double, MODE_MIN, ARITH_PAIR, true>(a0, max_ticks, sms, st, g);
      return rep ? launch_round<double, MODE_REPLACE, ARITH_PAIR, false>(a0, max_ticks, sms, st, g)
                 : launch_round<double, MODE_MIN, ARITH_PAIR, false>(a0, max_ticks, sms, st, g);
    default:
      return cudaErrorInvalidValue;
  }
}

// A grid's tensor maps for the pencils: its field (plane boxes of the pencil's
// slot), [1] unused (the cap is read directly), its frozen mask.
cudaError_t encode_pencil_maps(int which, const SweepArgs &a, const Layout &L, CUtensorMap m[3]) {
  if (L.tx != 16 || L.ty != 16 || L.xo != 0) return cudaErrorInvalidValue;
  cudaError_t e = which == 0 ? encode_field_map(&m[0], a.u, 4, L, a.nz + 2, PcGeo<float>::W, PcGeo<float>::RY, 1)
                             : encode_field_map(&m[0], a.u, 8, L, a.nz + 2, PcGeo<double>::W, PcGeo<double>::RY, 1);
  if (e != cudaSuccess) return e;
  m[1] = m[0];
  if (a.fmask) return encode_mask_map(&m[2], a, PcGeo<float>::BY);
  m[2] = m[0];
  return cudaSuccess;
}

}  // namespace pdfs
