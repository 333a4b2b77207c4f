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
// and nodes not yet reached (>= far) accept none.

// The orderings that sweep axis `axis` (0 x, 1 y, 2 z) in direction `sign`,
// one bit per ordering (bit sn-1), from ordering_signs' table.
__host__ __device__ constexpr unsigned orderings_along(int axis, int sign) {
  unsigned m = 0;
  for (int sn = 1; sn <= 8; ++sn) {
    const int desc = (sn == 2 || sn == 5 || sn == 7 || sn == 8) ? -1 : 1;
    const int s = axis == 0 ? ((sn == 4 || sn == 8) ? -1 : 1) * desc
                  : axis == 1 ? ((sn == 2 || sn == 6) ? -1 : 1) * desc
                              : ((sn == 3 || sn == 7) ? -1 : 1) * desc;
    if (s == sign) m |= 1u << (sn - 1);
  }
  return m;
}

// accepted directions of one axis: bit 0 ascending, bit 1 descending
__device__ __forceinline__ unsigned octant_axis(float c, float lo, float hi, float tie) {
  const float m = fminf(lo, hi);
  if (!(m < c) || fabsf(lo - hi) <= tie) return 3u;
  return lo < hi ? 1u : 2u;
}

// the orderings a node with direction sets (ax, ay, az) accepts
__device__ __forceinline__ unsigned octant_orderings(unsigned ax, unsigned ay, unsigned az) {
  constexpr unsigned XP = orderings_along(0, 1), XM = orderings_along(0, -1);
  constexpr unsigned YP = orderings_along(1, 1), YM = orderings_along(1, -1);
  constexpr unsigned ZP = orderings_along(2, 1), ZM = orderings_along(2, -1);
  static_assert((XP | XM) == 0xffu && (XP & XM) == 0u && (YP & ZP & XP) == 1u, "ordering table");
  return (((ax & 1u) ? XP : 0u) | ((ax & 2u) ? XM : 0u)) & (((ay & 1u) ? YP : 0u) | ((ay & 2u) ? YM : 0u)) &
         (((az & 1u) ? ZP : 0u) | ((az & 2u) ? ZM : 0u));
}

__global__ void __launch_bounds__(256) k_octant_mask(const float *__restrict__ u, Layout L,
                                                     const uint32_t *__restrict__ fmask, MaskLayout M, int nx, int ny,
                                                     int nz, float hx, float hy, float hz, float slack, float far,
                                                     int nbx, int nby, int nbz, uint8_t *__restrict__ omask) {
  // one CTA per 4 x 1 x 1 blocks (32 x of one block row and plane): warp w
  // takes row y = 8 by + w + 1, lane = x offset, and walks the block's 8 planes
  // with a window along z held in registers
  __shared__ unsigned s_c[8][4];
  const int nwx = (nbx + 3) / 4;
  const int wx = (int)(blockIdx.x % nwx), by = (int)((blockIdx.x / nwx) % nby), bz = (int)(blockIdx.x / ((long long)nwx * nby));
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int x = 1 + wx * 32 + lane, y = 1 + by * 8 + w;
  const bool row = y <= ny;
  const bool have = row && x <= nx + 1;  // the node, or the halo node right of the grid
  auto at = [&](int xx, int yy, int zz) { return fabsf(u[L.index(xx, yy, zz)]); };
  unsigned acc = 0;  // the orderings my nodes accept
  const int z0 = 1 + bz * 8, z1 = min(nz, bz * 8 + 8);
  const bool wgrid = row && 1 + wx * 32 <= nx;  // the warp holds grid nodes (its frozen word exists)
  float cm = have ? at(x, y, z0 - 1) : INFINITY;
  float c = have ? at(x, y, z0) : INFINITY;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const int z = z0 + k;
    const bool zin = z <= z1;
    const float cp = (have && zin) ? at(x, y, z + 1) : INFINITY;
    // x neighbours from the adjacent lanes; the warp's edge lanes read theirs
    float xl = __shfl_up_sync(0xffffffffu, c, 1), xr = __shfl_down_sync(0xffffffffu, c, 1);
    if (lane == 0 && have && zin) xl = at(x - 1, y, z);
    if (lane == 31 && x <= nx && row && zin) xr = at(x + 1, y, z);
    // frozen bits of the warp's 32 x: one word
    const unsigned fw = (fmask && wgrid && zin) ? fmask[M.word(1 + wx * 32, y, z)] : 0u;
    if (zin && row && x <= nx && !((fw >> lane) & 1u) && c < far)
      acc |= octant_orderings(octant_axis(c, xl, xr, slack * hx),
                              octant_axis(c, at(x, y - 1, z), at(x, y + 1, z), slack * hy),
                              octant_axis(c, cm, cp, slack * hz));
    cm = c;
    c = cp;
  }
#pragma unroll
  for (int off = 1; off < 8; off <<= 1) acc |= __shfl_xor_sync(0xffffffffu, acc, off);
  if ((lane & 7) == 0) s_c[w][lane >> 3] = acc;
  __syncthreads();
  const int bx = wx * 4 + threadIdx.x;
  if (threadIdx.x < 4 && bx < nbx) {
    unsigned all = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) all |= s_c[k][threadIdx.x];
    omask[((long long)bz * nby + by) * nbx + bx] = (uint8_t)all;
  }
}

// The same masks from shared-memory copies of the field: one CTA per
// 16 x 16 column of 2 x 2 blocks and kOmChunks blocks along z, each block's
// box (one-node halo) fetched by one TMA copy into one of two buffers, the
// next box in flight while a block is evaluated; thread (lx, ly) walks its
// column's 8 planes of each block.  For the layouts whose interior x starts
// 16-byte aligned (pencils, bricks).
constexpr int kOmW = 20, kOmRY = 18, kOmRZ = 10;  // box: x0-1 .. x0+16 rounded to 16 bytes, y0-1 .. y0+16, z0-1 .. z0+8
constexpr int kOmChunks = 4;
// floats of one buffer: the box rounded up to 128 bytes (TMA destinations are 128-byte aligned)
constexpr int kOmBuf = (kOmRZ * kOmRY * kOmW * 4 + 127) / 128 * 32;
__global__ void __launch_bounds__(256) k_octant_mask_tma(const __grid_constant__ CUtensorMap tm, const uint32_t *__restrict__ fmask,
                                                         MaskLayout M, int nx, int ny, int nz, float hx, float hy,
                                                         float hz, float slack, float far, int nbx, int nby, int nbz,
                                                         uint8_t *__restrict__ omask) {
  __shared__ __align__(128) float sbox[2][kOmBuf];
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ unsigned s_c[4];
  const int nrx = (nbx + 1) / 2, nry = (nby + 1) / 2;
  const int rx = (int)(blockIdx.x % nrx), ry = (int)((blockIdx.x / nrx) % nry);
  const int bz0 = kOmChunks * (int)(blockIdx.x / ((long long)nrx * nry));
  const int nch = min(kOmChunks, nbz - bz0);
  const int tid = threadIdx.x, lx = tid & 15, ly = tid >> 4, lane = tid & 31;
  const int x0 = 1 + 16 * rx, y0 = 1 + 16 * ry;
  constexpr unsigned kBox = (unsigned)(sizeof(float) * kOmRZ * kOmRY * kOmW);
  static_assert((kOmBuf * 4) % 128 == 0 && kOmBuf * 4 >= (int)kBox, "buffer size");
  auto box = [&](int b, int k, int r, int xx) { return sbox[b][(k * kOmRY + r) * kOmW + xx]; };
  if (tid < 4) s_c[tid] = 0u;
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_fence_init();
  }
  __syncthreads();
  int last[2] = {-1, -1};  // thread 0: the last block copied into each buffer
  if (tid == 0)
    for (int c = 0; c < min(2, nch); ++c) {
      mbar_arrive_tx(&bar[c], kBox);
      tma_load_3d(&sbox[c][0], &tm, x0 - 1, y0 - 1, 8 * (bz0 + c), &bar[c]);
      last[c] = c;
    }
  const int x = x0 + lx, y = y0 + ly;
  bool ok = true;  // every copy so far landed
  for (int c = 0; c < nch; ++c) {
    const int b = c & 1, bz = bz0 + c, z0 = 1 + 8 * bz;
    // bounded wait for the copy; on expiry every ordering is kept (always safe)
    bool landed = ok && mbar_try(&bar[b], (c >> 1) & 1);
    if (ok && !landed) {
      const long long t0 = clock64();
      while (!(landed = mbar_try(&bar[b], (c >> 1) & 1)) && clock64() - t0 < 4000000000ll) {
      }
    }
    ok = landed;
    unsigned acc = 0;  // the orderings my nodes accept
    if (landed && x <= nx && y <= ny) {
      const int z1 = min(nz, z0 + 7);
      for (int z = z0; z <= z1; ++z) {
        const int k = z - z0 + 1;
        if (fmask && ((fmask[M.word(x, y, z)] >> ((x - 1) & 31)) & 1u)) continue;
        const float cc = fabsf(box(b, k, ly + 1, lx + 1));
        if (!(cc < far)) continue;
        acc |= octant_orderings(
            octant_axis(cc, fabsf(box(b, k, ly + 1, lx)), fabsf(box(b, k, ly + 1, lx + 2)), slack * hx),
            octant_axis(cc, fabsf(box(b, k, ly, lx + 1)), fabsf(box(b, k, ly + 2, lx + 1)), slack * hy),
            octant_axis(cc, fabsf(box(b, k - 1, ly + 1, lx + 1)), fabsf(box(b, k + 1, ly + 1, lx + 1)), slack * hz));
      }
    }
    // the 4 blocks: lanes 0-7 and 16-23 of a warp (rows 2w, 2w + 1) hold x block
    // 2 rx, lanes 8-15 and 24-31 x block 2 rx + 1; both rows are in y block ly / 8
#pragma unroll
    for (int off = 1; off <= 16; off <<= 1)
      if (off != 8) acc |= __shfl_xor_sync(0xffffffffu, acc, off);
    if ((lane & 23) == 0 && acc) atomicOr(&s_c[((ly >> 3) << 1) | (lane >> 3)], acc);
    __syncthreads();  // the box is read and the block sums are complete
    if (tid < 4) {
      const int bx = 2 * rx + (tid & 1), by = 2 * ry + (tid >> 1);
      if (bx < nbx && by < nby) omask[((long long)bz * nby + by) * nbx + bx] = (uint8_t)(landed ? s_c[tid] : 0xffu);
      s_c[tid] = 0u;
    }
    if (tid == 0 && ok && c + 2 < nch) {  // the buffer's next box
      fence_proxy_async();
      mbar_arrive_tx(&bar[b], kBox);
      tma_load_3d(&sbox[b][0], &tm, x0 - 1, y0 - 1, 8 * (bz + 2), &bar[b]);
      last[b] = c + 2;
    }
    __syncthreads();  // the sums are reset before the next block's
  }
  // a copy that did not land in time is still drained (bounded) before the CTA leaves
  if (tid == 0 && !ok) {
    for (int b = 0; b < 2; ++b) {
      if (last[b] < 0) continue;
      const long long t0 = clock64();
      while (!mbar_try(&bar[b], (last[b] >> 1) & 1) && clock64() - t0 < 4000000000ll) {
      }
    }
  }
}

// active[b] = ordering sn matters to block b or (dilate) to the face
// neighbour it sweeps from along some axis; count receives the number of
// active blocks.
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
      int sx, sy, sz;
      ordering_signs(sn, &sx, &sy, &sz);
      const int ux = bx - sx, uy = by - sy, uz = bz - sz;  // the upwind neighbour along each axis
      on = (ux >= 0 && ux < nbx && (omask[b - sx] & bit)) ||
           (uy >= 0 && uy < nby && (omask[b - (long long)sy * nbx] & bit)) ||
           (uz >= 0 && uz < nbz && (omask[b - (long long)sz * pl] & bit));
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
  if (L.xo == 0 && !L.zc && L.tx % 16 == 0) {  // the box's x start is 16-byte aligned: the TMA kernel
    CUtensorMap m;
    cudaError_t e = encode_field_map(&m, (void *)u32, 4, L, g.nz + 2, kOmW, kOmRY, kOmRZ);
    if (e != cudaSuccess) return e;
    const long long ctas = (long long)((nbx + 1) / 2) * ((nby + 1) / 2) * ((nbz + kOmChunks - 1) / kOmChunks);
    k_octant_mask_tma<<<(unsigned)ctas, 256, 0, st>>>(m, fmask, M, g.nx, g.ny, g.nz, (float)g.dx, (float)g.dy,
                                                      (float)g.dz, slack, far, nbx, nby, nbz, omask);
    return cudaGetLastError();
  }
  const long long ctas = (long long)((nbx + 3) / 4) * nby * nbz;
  k_octant_mask<<<(unsigned)ctas, 256, 0, st>>>(u32, L, fmask, M, g.nx, g.ny, g.nz, (float)g.dx, (float)g.dy,
                                                (float)g.dz, slack, far, nbx, nby, nbz, omask);
  return cudaGetLastError();
}

// out[b] = omask of block b, widened: ordering sn also where it matters to the
// face neighbour that sn sweeps into b from (the lower-x neighbour for an
// ordering that sweeps +x, ...) -- the characteristics that cross the face
// into b.  octant_active(dilate = 1) applies the same rule one ordering at a
// time.  (Widening by all six neighbours' masks, whatever the direction: the
// 768^3 octant solve took 70.8 ms against 69.0, with the same sweeps.)
__global__ void k_octant_union(const uint8_t *__restrict__ omask, uint8_t *__restrict__ out, int nbx, int nby,
                               int nbz) {
  const long long n = (long long)nbx * nby * nbz, pl = (long long)nbx * nby;
  for (long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x; b < n; b += (long long)gridDim.x * blockDim.x) {
    const int bx = (int)(b % nbx), by = (int)((b / nbx) % nby), bz = (int)(b / pl);
    constexpr unsigned XP = orderings_along(0, 1), XM = orderings_along(0, -1);
    constexpr unsigned YP = orderings_along(1, 1), YM = orderings_along(1, -1);
    constexpr unsigned ZP = orderings_along(2, 1), ZM = orderings_along(2, -1);
    unsigned m = omask[b];
    if (bx > 0) m |= omask[b - 1] & XP;
    if (bx < nbx - 1) m |= omask[b + 1] & XM;
    if (by > 0) m |= omask[b - nbx] & YP;
    if (by < nby - 1) m |= omask[b + nbx] & YM;
    if (bz > 0) m |= omask[b - pl] & ZP;
    if (bz < nbz - 1) m |= omask[b + pl] & ZM;
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
