// lanecol_pmin.cu -- FP32-pair min-update instantiations of the lane-column sweep.
#include "internal.h"
#include "lanecol.cuh"

namespace pdfs {
template cudaError_t launch_lc_dir<double, 8, MODE_MIN>(bool, bool, const LcArgs &, int, cudaStream_t, int *);
}  // namespace pdfs
