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

// Polish orderings.  Along a characteristic of |grad u| = 1 (a straight line
// from the nearest interface point) a node's upwind neighbours lie on the
// side of the smaller value on every axis its Godunov update uses; an
// ordering whose sweep directions agree with those sides carries the node's
// whole upwind chain into it in one sweep (the fast sweeping argument, Zhao,
// Math. Comp. 74 (2005) 603-627).  From a nearly converged field this gives
// each 8^3 block the set of orderings that matter to it: bit sn-1 of omask
// is set where some node of the block accepts ordering sn.  An axis accepts
// both directions where the update does not use it (its smaller neighbour is
// not below the node) or where its two neighbours differ by at most
// slack * h (a characteristic nearly parallel to the faces).  Frozen nodes
// and nodes not yet reached (>= far) accept none.  One warp covers four
// blocks along x, lane = node x offset.
__global__ void k_octant_mask(const float *__restrict__ u, Layout L, const uint32_t *__restrict__ fmask,
                              MaskLayout M, int nx, int ny, int nz, float hx, float hy, float hz, float slack,
                              float far, int nbx, int nby, int nbz, uint8_t *__restrict__ omask) {
  const long long wid = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int nwx = (nbx + 3) / 4;
  if (wid >= (long long)nwx * nby * nbz) return;  // whole warps leave together
  const int wx = (int)(wid % nwx), by = (int)((wid / nwx) % nby), bz = (int)(wid / ((long long)nwx * nby));
  const int x = 1 + wx * 32 + lane;
  const bool have = x <= nx + 1;  // the node, or the halo node right of the grid
  // accepted directions of one axis: bit 0 ascending, bit 1 descending
  auto axis = [](float c, float lo, float hi, float tie) -> unsigned {
    const float m = fminf(lo, hi);
    if (!(m < c) || fabsf(lo - hi) <= tie) return 3u;
    return lo < hi ? 1u : 2u;
  };
  auto at = [&](int xx, int yy, int zz) { return fabsf(u[L.index(xx, yy, zz)]); };
  // the (x, y, z) direction sets met in the block, as 27 bits: bit 9(ax-1) + 3(ay-1) + (az-1)
  unsigned combos = 0;
  const int z0 = 1 + bz * 8, z1 = min(nz, bz * 8 + 8);
  for (int y = 1 + by * 8; y <= min(ny, by * 8 + 8); ++y) {
    // a sliding window along z: the planes below, at and above the node
    float cm = have ? at(x, y, z0 - 1) : INFINITY;
    float c = have ? at(x, y, z0) : INFINITY;
    for (int z = z0; z <= z1; ++z) {
      const float cp = have ? at(x, y, z + 1) : INFINITY;
      // x neighbours from the adjacent lanes; the warp's edge lanes read theirs
      float xl = __shfl_up_sync(0xffffffffu, c, 1), xr = __shfl_down_sync(0xffffffffu, c, 1);
      if (lane == 0 && have) xl = at(x - 1, y, z);
      if (lane == 31 && x <= nx) xr = at(x + 1, y, z);
      // frozen bits of the warp's 32 x: one word, when the warp holds a grid node
      const unsigned fw = (fmask && 1 + wx * 32 <= nx) ? fmask[M.word(1 + wx * 32, y, z)] : 0u;
      if (x <= nx && !((fw >> lane) & 1u) && c < far) {
        const unsigned ax = axis(c, xl, xr, slack * hx);
        const unsigned ay = axis(c, at(x, y - 1, z), at(x, y + 1, z), slack * hy);
        const unsigned az = axis(c, cm, cp, slack * hz);
        combos |= 1u << ((ax - 1) * 9 + (ay - 1) * 3 + (az - 1));
      }
      cm = c;
      c = cp;
    }
  }
#pragma unroll
  for (int off = 1; off < 8; off <<= 1) combos |= __shfl_xor_sync(0xffffffffu, combos, off);
  const int bx = wx * 4 + (lane >> 3);
  if ((lane & 7) == 0 && bx < nbx) {
    unsigned acc = 0;
    for (int k = 0; k < 27; ++k) {
      if (!((combos >> k) & 1u)) continue;
      const unsigned ax = k / 9 + 1, ay = (k / 3) % 3 + 1, az = k % 3 + 1;
#pragma unroll
      for (int sn = 1; sn <= 8; ++sn) {
        int sx, sy, sz;
        ordering_signs(sn, &sx, &sy, &sz);
        if ((ax & (sx > 0 ? 1u : 2u)) && (ay & (sy > 0 ? 1u : 2u)) && (az & (sz > 0 ? 1u : 2u)))
          acc |= 1u << (sn - 1);
      }
    }
    omask[((long long)bz * nby + by) * nbx + bx] = (uint8_t)acc;
  }
}

// active[b] = ordering sn matters to block b or to one of its six face
// neighbours (dilate) ; count receives the number of active blocks.
__global__ void k_octant_active(const uint8_t *__restrict__ omask, int sn, int dilate, uint8_t *__restrict__ active,
                                int nbx, int nby, int nbz, int *__restrict__ count) {
  const long long n = (long long)nbx * nby * nbz;
  const unsigned bit = 1u << (sn - 1);
  int local = 0;
  for (long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x; b < n; b += (long long)gridDim.x * blockDim.x) {
    const int bx = (int)(b % nbx), by = (int)((b / nbx) % nby), bz = (int)(b / ((long long)nbx * nby));
    bool on = (omask[b] & bit) != 0;
    if (dilate && !on) {
      const long long pl = (long long)nbx * nby;
      on = (bx > 0 && (omask[b - 1] & bit)) || (bx < nbx - 1 && (omask[b + 1] & bit)) ||
           (by > 0 && (omask[b - nbx] & bit)) || (by < nby - 1 && (omask[b + nbx] & bit)) ||
           (bz > 0 && (omask[b - pl] & bit)) || (bz < nbz - 1 && (omask[b + pl] & bit));
    }
    active[b] = on ? 1 : 0;
    local += on ? 1 : 0;
  }
  for (int off = 16; off > 0; off >>= 1) local += __shfl_xor_sync(0xffffffffu, local, off);
  if ((threadIdx.x & 31) == 0 && local) atomicAdd(count, local);
}

cudaError_t octant_mask(const float *u32, const Layout &L, const uint32_t *fmask, const MaskLayout &M,
                        const pdfs_grid &g, float slack, float far, int nbx, int nby, int nbz, uint8_t *omask,
                        cudaStream_t st) {
  const long long warps = (long long)((nbx + 3) / 4) * nby * nbz;
  const int grid = (int)((warps * 32 + 255) / 256);
  k_octant_mask<<<grid, 256, 0, st>>>(u32, L, fmask, M, g.nx, g.ny, g.nz, (float)g.dx, (float)g.dy, (float)g.dz, slack,
                                      far, nbx, nby, nbz, omask);
  return cudaGetLastError();
}

// out[b] = omask of block b | omask of its six face neighbours (the widened
// masks that octant_active(dilate = 1) applies one ordering at a time).
__global__ void k_octant_union(const uint8_t *__restrict__ omask, uint8_t *__restrict__ out, int nbx, int nby,
                               int nbz) {
  const long long n = (long long)nbx * nby * nbz, pl = (long long)nbx * nby;
  for (long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x; b < n; b += (long long)gridDim.x * blockDim.x) {
    const int bx = (int)(b % nbx), by = (int)((b / nbx) % nby), bz = (int)(b / pl);
    unsigned m = omask[b];
    if (bx > 0) m |= omask[b - 1];
    if (bx < nbx - 1) m |= omask[b + 1];
    if (by > 0) m |= omask[b - nbx];
    if (by < nby - 1) m |= omask[b + nbx];
    if (bz > 0) m |= omask[b - pl];
    if (bz < nbz - 1) m |= omask[b + pl];
    out[b] = (uint8_t)m;
  }
}

// nodes[j] += the grid nodes of the blocks whose bit j is set (the node
// updates a masked sweep of ordering j + 1 executes).
__global__ void k_octant_nodes(const uint8_t *__restrict__ bits, int nbx, int nby, int nbz, int nx, int ny, int nz,
                               unsigned long long *__restrict__ nodes) {
  const long long n = (long long)nbx * nby * nbz;
  unsigned long long local[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x; b < n; b += (long long)gridDim.x * blockDim.x) {
    const int bx = (int)(b % nbx), by = (int)((b / nbx) % nby), bz = (int)(b / ((long long)nbx * nby));
    const unsigned long long v = (unsigned long long)min(8, nx - 8 * bx) * min(8, ny - 8 * by) * min(8, nz - 8 * bz);
    const unsigned m = bits[b];
#pragma unroll
    for (int j = 0; j < 8; ++j)
      if ((m >> j) & 1u) local[j] += v;
  }
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    unsigned long long v = local[j];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(nodes + j, v);
  }
}

cudaError_t octant_nodes(const uint8_t *bits, int nbx, int nby, int nbz, int nx, int ny, int nz,
                         unsigned long long *nodes, int sms, cudaStream_t st) {
  const long long n = (long long)nbx * nby * nbz;
  int grid = (int)std::min<long long>((n + 255) / 256, (long long)sms * 8);
  if (grid < 1) grid = 1;
  k_octant_nodes<<<grid, 256, 0, st>>>(bits, nbx, nby, nbz, nx, ny, nz, nodes);
  return cudaGetLastError();
}

cudaError_t octant_union(const uint8_t *omask, uint8_t *out, int nbx, int nby, int nbz, int sms, cudaStream_t st) {
  const long long n = (long long)nbx * nby * nbz;
  int grid = (int)std::min<long long>((n + 255) / 256, (long long)sms * 8);
  if (grid < 1) grid = 1;
  k_octant_union<<<grid, 256, 0, st>>>(omask, out, nbx, nby, nbz);
  return cudaGetLastError();
}

cudaError_t octant_active(const uint8_t *omask, int sn, int dilate, uint8_t *active, int nbx, int nby, int nbz,
                          int *count, int sms, cudaStream_t st) {
  const long long n = (long long)nbx * nby * nbz;
  int grid = (int)std::min<long long>((n + 255) / 256, (long long)sms * 8);
  if (grid < 1) grid = 1;
  k_octant_active<<<grid, 256, 0, st>>>(omask, sn, dilate, active, nbx, nby, nbz, count);
  return cudaGetLastError();
}

}  // namespace pdfs
