// lanecol_prep.cu -- FP32-pair replace-update (polish) instantiations of the lane-column sweep.
#include "internal.h"
#include "lanecol.cuh"

namespace pdfs {
template cudaError_t launch_lc_dir<double, 8, MODE_REPLACE>(bool, bool, const LcArgs &, int, cudaStream_t, int *);
}  // namespace pdfs
