// sched.cu -- active-block scheduling of the sweeps (8^3 node blocks).
//
// The reference sweeps every node in every ordering (single_gpu_cuda/src/
// phi3D_fsm.cu:144-189).  A block whose nodes and face neighbours did not
// change recently is unlikely to change in the next sweep; skipping it is
// always safe for the answer because a solve only terminates after a sweep
// that visits every block and changes nothing (or less than the tolerance),
// which certifies the plain method's fixed point.
#include "internal.h"

namespace pdfs {

// active[b] = block b changed by more than thr in one of the last hist
// sweeps, or one of its six face neighbours did in the last sweep.  count
// receives the number of active blocks.
__global__ void k_sched_change(const unsigned int *__restrict__ ring, int cur, int hist, float thr,
                               uint8_t *__restrict__ active, int nbx, int nby, int nbz, int *__restrict__ count) {
  const long long n = (long long)nbx * nby * nbz;
  const unsigned int *c1 = ring + (size_t)((cur - 1 + kRing) % kRing) * n;
  int local = 0;
  for (long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x; b < n; b += (long long)gridDim.x * blockDim.x) {
    const int bx = (int)(b % nbx), by = (int)((b / nbx) % nby), bz = (int)(b / ((long long)nbx * nby));
    auto hot = [&](long long i) { return __uint_as_float(c1[i]) > thr; };
    bool on = false;
    for (int k = 1; k <= hist && !on; ++k)
      on = __uint_as_float(ring[(size_t)((cur - k + kRing) % kRing) * n + b]) > thr;
    if (!on && bx > 0) on = hot(b - 1);
    if (!on && bx < nbx - 1) on = hot(b + 1);
    if (!on && by > 0) on = hot(b - nbx);
    if (!on && by < nby - 1) on = hot(b + nbx);
    if (!on && bz > 0) on = hot(b - (long long)nbx * nby);
    if (!on && bz < nbz - 1) on = hot(b + (long long)nbx * nby);
    active[b] = on ? 1 : 0;
    local += on ? 1 : 0;
  }
  for (int off = 16; off > 0; off >>= 1) local += __shfl_xor_sync(0xffffffffu, local, off);
  if ((threadIdx.x & 31) == 0 && local) atomicAdd(count, local);
}

cudaError_t sched_change(const unsigned int *ring, int cur, int hist, float thr, uint8_t *active, int nbx, int nby,
                         int nbz, int *count, int sms, cudaStream_t st) {
  const long long n = (long long)nbx * nby * nbz;
  int grid = (int)std::min<long long>((n + 255) / 256, (long long)sms * 8);
  if (grid < 1) grid = 1;
  k_sched_change<<<grid, 256, 0, st>>>(ring, cur, hist, thr, active, nbx, nby, nbz, count);
  return cudaGetLastError();
}

}  // namespace pdfs
