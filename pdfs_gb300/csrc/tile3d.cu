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

// Block-masked sweeps: per brick (global brick id), whether one of its 8^3
// blocks is active -- one thread per brick ...
__global__ void k_brick_active(int ntx, int nty, int ntz, int bx, int by, int bz, const uint8_t *__restrict__ active,
                               int nbx, int nby, int nbz, uint8_t *__restrict__ tact) {
  const int n = ntx * nty * ntz;
  for (int tile = blockIdx.x * blockDim.x + threadIdx.x; tile < n; tile += gridDim.x * blockDim.x) {
    const int bi = tile % ntx, bj = (tile / ntx) % nty, bk = tile / (ntx * nty);
    bool act = false;
    for (int q = 0; q < bz && !act; ++q)
      for (int p = 0; p < by && !act; ++p)
        for (int o = 0; o < bx && !act; ++o) {
          const int X = bi * bx + o, Y = bj * by + p, Z = bk * bz + q;
          act = X < nbx && Y < nby && Z < nbz && active[((long long)Z * nby + Y) * nbx + X];
        }
    tact[tile] = act ? 1 : 0;
  }
}

// ... and the tickets of the active bricks in the sweep's wavefront order
// (out, *count of them).  One CTA: each thread takes a contiguous run of
// tickets, the counts are scanned, the runs are written in order -- so the
// compacted list keeps every brick after its upwind bricks.
__global__ void k_brick_compact(const int *__restrict__ torder, int ntx, int nty, int ntz, int sx, int sy, int sz,
                                const uint8_t *__restrict__ tact, int *__restrict__ out, int *__restrict__ count) {
  __shared__ int s_sum[1024];
  const int n = ntx * nty * ntz, tid = threadIdx.x, nt = blockDim.x;
  const int per = (n + nt - 1) / nt, t0 = min(n, tid * per), t1 = min(n, t0 + per);
  auto active = [&](int tk) {
    const int lt = torder[tk], li = lt % ntx, lj = (lt / ntx) % nty, lk = lt / (ntx * nty);
    const int bi = sx > 0 ? li : ntx - 1 - li, bj = sy > 0 ? lj : nty - 1 - lj, bk = sz > 0 ? lk : ntz - 1 - lk;
    return tact[(bk * nty + bj) * ntx + bi] != 0;
  };
  int cnt = 0;
  for (int tk = t0; tk < t1; ++tk) cnt += active(tk) ? 1 : 0;
  s_sum[tid] = cnt;
  __syncthreads();
  for (int off = 1; off < nt; off <<= 1) {  // inclusive scan of the counts
    const int v = tid >= off ? s_sum[tid - off] : 0;
    __syncthreads();
    s_sum[tid] += v;
    __syncthreads();
  }
  int pos = s_sum[tid] - cnt;
  for (int tk = t0; tk < t1; ++tk)
    if (active(tk)) out[pos++] = torder[tk];
  if (tid == nt - 1) *count = s_sum[tid];
}

// ---- octant rounds (the polish's first cycle in one launch, tile3d.cuh OCT) ----

// Per brick, the union of its 8^3 blocks' ordering bits.
__global__ void k_brick_bits(int ntx, int nty, int ntz, int bx, int by, int bz, const uint8_t *__restrict__ bits,
                             int nbx, int nby, int nbz, uint8_t *__restrict__ tbits) {
  const int n = ntx * nty * ntz;
  for (int tile = blockIdx.x * blockDim.x + threadIdx.x; tile < n; tile += gridDim.x * blockDim.x) {
    const int bi = tile % ntx, bj = (tile / ntx) % nty, bk = tile / (ntx * nty);
    unsigned m = 0;
    for (int q = 0; q < bz; ++q)
      for (int p = 0; p < by; ++p)
        for (int o = 0; o < bx; ++o) {
          const int X = bi * bx + o, Y = bj * by + p, Z = bk * bz + q;
          if (X < nbx && Y < nby && Z < nbz) m |= bits[((long long)Z * nby + Y) * nbx + X];
        }
    tbits[tile] = (uint8_t)m;
  }
}

// Sweep j's tickets (CTA j): the bricks whose bits name ordering
// (first + j) % 8 + 1 (every brick when bit j of full is set), in that
// ordering's wavefront order, to out[j][...]; their count to cnt[j].  The
// scan keeps the order (as k_brick_compact).
__global__ void k_oct_tickets(const int *__restrict__ torder, int ntx, int nty, int ntz, int first, unsigned full,
                              const uint8_t *__restrict__ tbits, int *__restrict__ out, int *__restrict__ cnt) {
  __shared__ int s_sum[1024];
  const int j = blockIdx.x, n = ntx * nty * ntz, tid = threadIdx.x, nt = blockDim.x;
  const int sn = (first + j) % 8 + 1;
  const unsigned bit = 1u << (sn - 1);
  const bool all = (full >> j) & 1u;
  int sx, sy, sz;
  ordering_signs(sn, &sx, &sy, &sz);
  const int per = (n + nt - 1) / nt, t0 = min(n, tid * per), t1 = min(n, t0 + per);
  auto active = [&](int tk) {
    if (all) return true;
    const int lt = torder[tk], li = lt % ntx, lj = (lt / ntx) % nty, lk = lt / (ntx * nty);
    const int bi = sx > 0 ? li : ntx - 1 - li, bj = sy > 0 ? lj : nty - 1 - lj, bk = sz > 0 ? lk : ntz - 1 - lk;
    return (tbits[(bk * nty + bj) * ntx + bi] & bit) != 0;
  };
  int c = 0;
  for (int tk = t0; tk < t1; ++tk) c += active(tk) ? 1 : 0;
  s_sum[tid] = c;
  __syncthreads();
  for (int off = 1; off < nt; off <<= 1) {
    const int v = tid >= off ? s_sum[tid - off] : 0;
    __syncthreads();
    s_sum[tid] += v;
    __syncthreads();
  }
  int pos = s_sum[tid] - c;
  int *o = out + (long long)j * n;
  for (int tk = t0; tk < t1; ++tk)
    if (active(tk)) o[pos++] = torder[tk];
  if (tid == nt - 1) cnt[j] = s_sum[tid];
}

// The round's ticket order.  Sweep j's brick at wavefront level w (its
// local x + y + z) gets key T[j] + w; tickets are listed by key, then by
// sweep, so sweep j + 1 starts at its first corner while sweep j is still
// finishing elsewhere instead of after all of sweep j.  The host picks T so
// that every wait is on a smaller key: a brick of sweep j waits for its
// upwind bricks (key - 1) and for itself and its face neighbours in an
// earlier sweep j', whose keys are at most T[j'] + w + 1 + the summed extents
// (bricks - 1) of the axes j' and j sweep in opposite directions.
struct OctKeys {
  int T[kOctMax];
};

__device__ __forceinline__ int oct_level(int lt, int ntx, int nty) {
  return lt % ntx + (lt / ntx) % nty + lt / (ntx * nty);
}

// One CTA: off[0..nsw] (prefix sums of the nsw counts), start[j][w] (the
// first of sweep j's listed tickets at level >= w; the lists are in level
// order) and base[j][w] (where sweep j's level-w tickets begin in the merged
// order).
__global__ void __launch_bounds__(1024) k_oct_plan(const int *__restrict__ lists, const int *__restrict__ cnt,
                                                   int *__restrict__ off, int nsw, int ntx, int nty, int ntz,
                                                   OctKeys K, int *__restrict__ start, int *__restrict__ base) {
  __shared__ int s_sum[1024];
  const int n = ntx * nty * ntz, WL = ntx + nty + ntz - 2, tid = threadIdx.x;
  if (tid == 0) {
    off[0] = 0;
    for (int j = 0; j < nsw; ++j) off[j + 1] = off[j] + cnt[j];
  }
  for (int idx = tid; idx < nsw * (WL + 1); idx += blockDim.x) {
    const int j = idx / (WL + 1), w = idx % (WL + 1);
    const int *l = lists + (long long)j * n;
    int lo = 0, hi = cnt[j];  // first listed ticket with level >= w
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (oct_level(l[mid], ntx, nty) < w)
        lo = mid + 1;
      else
        hi = mid;
    }
    start[idx] = lo;
  }
  __syncthreads();
  // cells (key k, sweep j) in order; cell size = sweep j's tickets at level k - T[j]
  const int ncell = (K.T[nsw - 1] + WL) * nsw;
  const int per = (ncell + blockDim.x - 1) / blockDim.x, c0 = min(ncell, tid * per), c1 = min(ncell, c0 + per);
  auto size = [&](int c) {
    const int j = c % nsw, w = c / nsw - K.T[j];
    return (w >= 0 && w < WL) ? start[j * (WL + 1) + w + 1] - start[j * (WL + 1) + w] : 0;
  };
  int sum = 0;
  for (int c = c0; c < c1; ++c) sum += size(c);
  s_sum[tid] = sum;
  __syncthreads();
  for (int o = 1; o < (int)blockDim.x; o <<= 1) {
    const int v = tid >= o ? s_sum[tid - o] : 0;
    __syncthreads();
    s_sum[tid] += v;
    __syncthreads();
  }
  int pos = s_sum[tid] - sum;
  for (int c = c0; c < c1; ++c) {
    const int j = c % nsw, w = c / nsw - K.T[j];
    if (w >= 0 && w < WL) base[j * WL + w] = pos;
    pos += size(c);
  }
}

// merged[base[j][w] + i - start[j][w]] = (j << 27) | brick, for sweep j's
// i-th listed ticket (level w)
__global__ void k_oct_merge(const int *__restrict__ lists, const int *__restrict__ cnt, int nsw, int ntx, int nty,
                            int ntz, const int *__restrict__ start, const int *__restrict__ base,
                            int *__restrict__ merged) {
  const int n = ntx * nty * ntz, WL = ntx + nty + ntz - 2;
  for (int j = 0; j < nsw; ++j) {
    const int m = cnt[j];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
      const int lt = lists[(long long)j * n + i], w = oct_level(lt, ntx, nty);
      merged[base[j * WL + w] + i - start[j * (WL + 1) + w]] = (j << 27) | lt;
    }
  }
}

// [kOctMax][n] per-sweep lists, kOctMax counts, kOctMax + 1 offsets, the
// merged list, start [kOctMax][WL + 1], base [kOctMax][WL]
int octant_scratch_ints(int ntx, int nty, int ntz) {
  const int n = ntx * nty * ntz, WL = ntx + nty + ntz - 2;
  return 2 * kOctMax * n + 2 * kOctMax + 1 + kOctMax * (WL + 1) + kOctMax * WL;
}

template <class T, int BZ, int MODE, int ARITH, bool ISO>
static cudaError_t launch_oct(const SweepArgs &a, const Layout &L, int sms, cudaStream_t st, int *grid_used) {
  using G = T3Geo<T, 16, BZ>;
  auto kern = t3_sweep_kernel<T, 16, BZ, MODE, ARITH, ISO, true>;
  CUtensorMap m;
  cudaError_t e = encode_field_map(&m, a.u, sizeof(T), L, a.nz + 2, G::W, G::RY, G::RZ);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G::BYTES);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, G::NT, G::BYTES);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  // every CTA resident: a ticket waits only on smaller tickets
  int grid = std::min(per_sm * sms, kOctMax * a.ntx * a.nty * a.ntz);
  if (grid < 1) grid = 1;
  kern<<<grid, G::NT, G::BYTES, st>>>(m, a);
  if (grid_used) *grid_used = grid;
  return cudaGetLastError();
}

cudaError_t launch_octant_round(int which, int arith, bool iso, int nsw, const SweepArgs &a0, const Layout &L,
                                int *list, int *cnt_off, int sms, cudaStream_t st, int *g) {
  // FP32 min-update rounds on the FP32 masked bricks (16 x 16 x 32), FP64
  // replace-update (polish) rounds on the FP64 ones (16 x 16 x 16).  (FP32
  // rounds on 16^3 bricks, 8 CTAs per SM instead of 4, were measured slower
  // on the 768^3 grid: full round 22.4 -> 25.9 ms, masked 13.8 -> 15.0 ms.)
  const int bz = which == 0 ? 32 : 16;
  if (!a0.tflag || !a0.torder || !a0.oct_bits || !a0.oct_tbits || a0.ntx < 1 || L.ty != 16 || L.tx != 16 ||
      L.xo != 0 || which == 1 || (which == 2 && (!a0.bcap64 || !a0.bcap32)) || a0.ntz != (a0.nz + bz - 1) / bz ||
      nsw < 1 || nsw > kOctMax || (long long)a0.ntx * a0.nty * a0.ntz >= (1ll << 27))
    return cudaErrorInvalidValue;
  const int n = a0.ntx * a0.nty * a0.ntz;
  k_brick_bits<<<std::min((n + 255) / 256, 4 * sms), 256, 0, st>>>(a0.ntx, a0.nty, a0.ntz, 2, 2, bz / 8, a0.oct_bits,
                                                                  a0.nbx, a0.nby, a0.nbz,
                                                                  const_cast<uint8_t *>(a0.oct_tbits));
  k_oct_tickets<<<nsw, 1024, 0, st>>>(a0.torder, a0.ntx, a0.nty, a0.ntz, a0.oct_first, a0.oct_full, a0.oct_tbits,
                                      list, cnt_off);
  // the keys' sweep offsets: T[j] >= T[j'] + 2 + the extents of the axes
  // sweeps j' and j run in opposite directions, for every j' < j
  OctKeys K;
  const int ext[3] = {a0.ntx - 1, a0.nty - 1, a0.ntz - 1};
  int sg[kOctMax][3];
  for (int j = 0; j < nsw; ++j) ordering_signs((a0.oct_first + j) % 8 + 1, &sg[j][0], &sg[j][1], &sg[j][2]);
  for (int j = 0; j < nsw; ++j) {
    K.T[j] = 0;
    for (int q = 0; q < j; ++q) {
      int d = 2;
      for (int ax = 0; ax < 3; ++ax)
        if (sg[q][ax] != sg[j][ax]) d += ext[ax];
      K.T[j] = std::max(K.T[j], K.T[q] + d);
    }
  }
  const int WL = a0.ntx + a0.nty + a0.ntz - 2;
  int *off = cnt_off + kOctMax, *merged = off + kOctMax + 1;
  int *start = merged + kOctMax * (size_t)n, *base = start + kOctMax * (WL + 1);
  k_oct_plan<<<1, 1024, 0, st>>>(list, cnt_off, off, nsw, a0.ntx, a0.nty, a0.ntz, K, start, base);
  k_oct_merge<<<std::max(1, std::min((n + 255) / 256, 4 * sms)), 256, 0, st>>>(list, cnt_off, nsw, a0.ntx, a0.nty,
                                                                               a0.ntz, start, base, merged);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  SweepArgs a = a0;
  a.torder = merged;
  a.nticket = off + nsw;  // the round's ticket count
  a.blk_active = nullptr;
  a.tact = nullptr;
  if (which == 0)
    return iso ? launch_oct<float, 32, MODE_MIN, ARITH_FAST, true>(a, L, sms, st, g)
               : launch_oct<float, 32, MODE_MIN, ARITH_FAST, false>(a, L, sms, st, g);
  switch (arith) {
    case ARITH_PAIR:
      return iso ? launch_oct<double, 16, MODE_REPLACE, ARITH_PAIR, true>(a, L, sms, st, g)
                 : launch_oct<double, 16, MODE_REPLACE, ARITH_PAIR, false>(a, L, sms, st, g);
    case ARITH_MIXED:
      return iso ? launch_oct<double, 16, MODE_REPLACE, ARITH_MIXED, true>(a, L, sms, st, g)
                 : launch_oct<double, 16, MODE_REPLACE, ARITH_MIXED, false>(a, L, sms, st, g);
    case ARITH_FAST:
      return launch_oct<double, 16, MODE_REPLACE, ARITH_FAST, false>(a, L, sms, st, g);
    case ARITH_REF:
      return launch_oct<double, 16, MODE_REPLACE, ARITH_REF, false>(a, L, sms, st, g);
    default:
      return cudaErrorInvalidValue;
  }
}

cudaError_t launch_sweep_bricks(int which, int by, int bz, int arith, bool iso, const SweepArgs &a0, const Layout &L,
                                int sms, cudaStream_t st, int *g) {
  if (!a0.tflag || !a0.torder || a0.ntx < 1 || a0.nty < 1 || a0.ntz < 1 || L.ty != by || L.tx != 16 ||
      L.xo != 0 || (which == 2 && (!a0.bcap64 || !a0.bcap32)))
    return cudaErrorInvalidValue;
  SweepArgs a = a0;
  if (a0.blk_active && a0.tact && a0.nticket) {
    // block-masked: tickets for the bricks that hold an active block only
    int *list = const_cast<int *>(a0.nticket) + 1;  // the compacted order follows the count
    const int n = a0.ntx * a0.nty * a0.ntz;
    k_brick_active<<<std::min((n + 255) / 256, 4 * sms), 256, 0, st>>>(a0.ntx, a0.nty, a0.ntz, 2, by / 8, bz / 8,
                                                                      a0.blk_active, a0.nbx, a0.nby, a0.nbz,
                                                                      const_cast<uint8_t *>(a0.tact));
    k_brick_compact<<<1, 1024, 0, st>>>(a0.torder, a0.ntx, a0.nty, a0.ntz, a0.sx, a0.sy, a0.sz, a0.tact, list,
                                        const_cast<int *>(a0.nticket));
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    a.torder = list;
  } else {
    a.tact = nullptr;
    a.nticket = nullptr;
  }
  if (by == 16 && bz == 16) return dispatch_t3<16, 16>(which, arith, iso, a, L, sms, st, g);
  if (by == 16 && bz == 32) return dispatch_t3<16, 32>(which, arith, iso, a, L, sms, st, g);
  if (by == 8 && bz == 32) return dispatch_t3<8, 32>(which, arith, iso, a, L, sms, st, g);
  if (by == 8 && bz == 48 && which == 0)  // FP32 only
    return iso ? launch_t3<float, 8, 48, MODE_MIN, ARITH_FAST, true>(a, L, sms, st, g)
               : launch_t3<float, 8, 48, MODE_MIN, ARITH_FAST, false>(a, L, sms, st, g);
  return cudaErrorInvalidValue;
}

}  // namespace pdfs
