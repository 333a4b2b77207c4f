// lanecol.cu -- FP32 instantiations of the lane-column sweep (lanecol.cuh)
// and its dispatcher; the FP32-pair variants are compiled in lanecol_pmin.cu
// (min-update) and lanecol_prep.cu (replace-update).
#include "internal.h"
#include "lanecol.cuh"

namespace pdfs {

template cudaError_t launch_lc_dir<float, 8, MODE_MIN>(bool, bool, const LcArgs &, int, cudaStream_t, int *);
template cudaError_t launch_lc_dir<float, 4, MODE_MIN>(bool, bool, const LcArgs &, int, cudaStream_t, int *);
extern template cudaError_t launch_lc_dir<double, 8, MODE_MIN>(bool, bool, const LcArgs &, int, cudaStream_t, int *);
extern template cudaError_t launch_lc_dir<double, 4, MODE_MIN>(bool, bool, const LcArgs &, int, cudaStream_t, int *);
extern template cudaError_t launch_lc_dir<double, 8, MODE_REPLACE>(bool, bool, const LcArgs &, int, cudaStream_t,
                                                                   int *);
extern template cudaError_t launch_lc_dir<double, 4, MODE_REPLACE>(bool, bool, const LcArgs &, int, cudaStream_t,
                                                                   int *);

cudaError_t launch_sweep_lanecol(int which, int rows, bool iso, const LcArgs &a, int sms, cudaStream_t st, int *g) {
  const bool blk = a.blk_active != nullptr || a.blk_chg != nullptr;
  if (a.ntx < 1 || a.nty < 1 || a.T % 8 != 0 || (a.q_last & 7) != 7 || !a.order || !a.ymail || !a.xmail ||
      (rows != 4 && rows != 8))
    return cudaErrorInvalidValue;
  if (which == 0)
    return rows == 8 ? launch_lc_dir<float, 8, MODE_MIN>(iso, blk, a, sms, st, g)
                     : launch_lc_dir<float, 4, MODE_MIN>(iso, blk, a, sms, st, g);
  if (which == 1)
    return rows == 8 ? launch_lc_dir<double, 8, MODE_MIN>(iso, blk, a, sms, st, g)
                     : launch_lc_dir<double, 4, MODE_MIN>(iso, blk, a, sms, st, g);
  if (!a.cap || !a.bcap32) return cudaErrorInvalidValue;
  return rows == 8 ? launch_lc_dir<double, 8, MODE_REPLACE>(iso, blk, a, sms, st, g)
                   : launch_lc_dir<double, 4, MODE_REPLACE>(iso, blk, a, sms, st, g);
}

}  // namespace pdfs
