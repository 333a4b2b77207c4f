// tile3d.cuh -- the 3-D tile sweep: each CTA sweeps a 16 x BY x BZ brick of
// the grid held whole in shared memory, hyperplane by hyperplane.
//
// The reference sweeps one hyperplane x+y+z = level of the whole grid per
// kernel launch (single_gpu_cuda/src/phi3D_fsm.cu:161-185,
// mpi_openacc/src/phi3D_fsm.c:92-117).  Any topological order of an
// ordering's dependency DAG gives the same result (each node reads the new
// values of its three upwind neighbours and the old values of its three
// downwind ones), so this kernel cuts the grid into bricks and orders them
// twice over:
//   * inside a brick, level by level: thread (lx, ly) -- brick-local
//     coordinates in sweep order -- updates node (lx, ly, L - lx - ly) at
//     level L, and a CTA barrier separates levels.  A level reads the
//     previous level's results and the next level's old values straight from
//     the shared-memory copy of the brick;
//   * across bricks, by per-brick completion flags in global memory: a brick
//     starts its levels once its (at most three) upwind bricks have published
//     this sweep's epoch, and publishes its own after its stores are visible.
//     Persistent CTAs take bricks by ticket in wavefront order (every upwind
//     brick holds a smaller ticket), so the wait always ends.
//
// A brick's old values do not depend on its upwind bricks, so its whole box
// (the brick and a one-node halo, rows rounded up to 16 bytes) is requested
// by one TMA copy as soon as the ticket is taken; only the upwind halo faces
// are read again, from L2, after the flags.  Updated nodes are stored to
// global memory as they are computed (unchanged nodes are not written).
//
// Against the column kernel (sweep.cuh) this trades the cross-column
// mailboxes, the plane ring and the per-step warp hand-offs for one barrier
// per level and a 1.5-2x halo read, and it keeps a brick's every level in
// one CTA's shared memory.
//
// Every wait is bounded (SweepArgs::wait_cycles): on expiry the kernel
// records DEV_ERR_TIMEOUT, raises the abort flag, lets its own TMA copy land
// and returns.
#pragma once
#include "sweep.cuh"

namespace pdfs {

template <class T, int BY_, int BZ>
struct T3Geo {
  static constexpr int BX = 16, BY = BY_;
  // box row: x0-1 .. x0+BX, rounded up to 16 bytes; the field's index has no
  // x offset, so x0 - 1 = 16*bi starts the row on a 16-byte boundary
  static constexpr int W = (int)((((BX + 2) * sizeof(T)) + 15) / 16 * 16 / sizeof(T));
  static constexpr int RY = BY + 2;       // box rows: y0-1 .. y0+BY
  static constexpr int RZ = BZ + 2;       // box planes: z0-1 .. z0+BZ
  static constexpr int PL = RY * W;       // plane stride in shared memory
  static constexpr int NL = BX + BY + BZ - 2;  // levels of one brick
  static constexpr int NT = BX * BY;      // one thread per (x, y) of the brick
  static constexpr int NZB = BZ / 8;      // 8^3 scheduler blocks per brick column
  static constexpr unsigned BOX_BYTES = (unsigned)(W * RY * RZ * sizeof(T));
  static constexpr size_t OFF_MASK = ((size_t)BOX_BYTES + 127) & ~size_t(127);
  static constexpr size_t OFF_BAR = OFF_MASK + (size_t)BZ * BY * 4;
  static constexpr size_t BYTES = OFF_BAR + 16;
  static_assert(BZ % 8 == 0 && BY % 8 == 0, "bricks hold whole 8^3 blocks");
  static constexpr int NBX = BX / 8, NBY = BY / 8;  // 8^3 blocks per brick in x and y
  static_assert((W * sizeof(T)) % 16 == 0, "TMA rows are 16-byte multiples");
};

__device__ __forceinline__ void st_release_gpu(int *p, int v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;\n" ::"l"(p), "r"(v) : "memory");
}
// A brick's completion: the CTA barrier before it orders every thread's
// stores before thread 0's acquire-release fence at GPU scope, which orders
// them before the relaxed flag store (the fence-then-relaxed-store pattern of
// CUTLASS's arrival barriers).
__device__ __forceinline__ void publish_gpu(int *p, int v) {
  asm volatile("fence.acq_rel.gpu;\n" ::: "memory");
  asm volatile("st.relaxed.gpu.global.s32 [%0], %1;\n" ::"l"(p), "r"(v) : "memory");
}

// Column of thread tid when the brick's 16 x BY columns are listed by
// diagonal d = lx + ly (then by ly).  Column (lx, ly) holds a node of level L
// for L - lx - ly in [0, BZ), so a warp whose 32 columns span diagonals
// d0 .. d1 runs the level body on BZ + d1 - d0 levels: BZ + 2 to BZ + 7 for
// 16 x 16 columns listed by diagonal, BZ + 16 for the row-major warp of two
// rows (158 against 256 warp-level bodies per 16^3 brick).
template <int BX, int BY>
__device__ __forceinline__ int2 diag_column(int tid) {
  int base = 0;
#pragma unroll 1
  for (int d = 0; d <= BX + BY - 2; ++d) {
    const int lo = d - (BX - 1) > 0 ? d - (BX - 1) : 0, hi = d < BY - 1 ? d : BY - 1;  // ly on diagonal d
    if (tid < base + hi - lo + 1) return make_int2(d - (lo + tid - base), lo + tid - base);
    base += hi - lo + 1;
  }
  return make_int2(0, 0);
}

// OCT: an octant round -- up to kOctMax sweeps in one launch (a cycle of the
// 8 orderings).  A ticket
// names (sweep j, brick); ordering (oct_first + j) % 8 + 1 visits the bricks
// and blocks whose bits name it, or every brick when bit j of oct_full is
// set.  Before its box is read, a
// brick waits until it and its six face neighbours have finished their latest
// earlier sweep of the round (their values are this sweep's old values), then
// for its upwind bricks in this sweep as usual.  Flags carry epoch + j, so
// "finished sweep j" is a flag >= epoch + j; the ticket list (k_oct_plan,
// k_oct_merge) interleaves the sweeps by wavefront level with every brick
// after the ones it waits on, so every wait is on a smaller ticket.  The
// result is the sequential sweeps', bit for bit.
template <class T, int BY_, int BZ, int MODE, int ARITH, bool ISO, bool OCT = false>
__global__ void __launch_bounds__(16 * BY_) t3_sweep_kernel(const __grid_constant__ CUtensorMap tm_u,
                                                            const __grid_constant__ SweepArgs a) {
  using G = T3Geo<T, BY_, BZ>;
  constexpr int BX = G::BX, BY = G::BY, W = G::W, PL = G::PL, NL = G::NL, NZB = G::NZB;
  extern __shared__ __align__(1024) unsigned char sm[];
  T *box = reinterpret_cast<T *>(sm);
  uint32_t *smask = reinterpret_cast<uint32_t *>(sm + G::OFF_MASK);  // [BZ][BY] frozen words of the brick
  uint64_t *bar = reinterpret_cast<uint64_t *>(sm + G::OFF_BAR);
  __shared__ int s_next, s_lo, s_hi;  // s_lo / s_hi: a masked brick's active planes (sweep order)
  __shared__ volatile int s_abort;

  if ((saddr(sm) & 127u) != 0) {  // TMA destinations must be 128-byte aligned
    if (threadIdx.x == 0) {
      atomicCAS(a.err, 0, DEV_ERR_SMEM_ALIGN);
      atomicExch(a.err + 1, 1);
    }
    return;
  }
  const int tid = threadIdx.x, lane = tid & 31;
  // brick-local x, y in sweep order; an octant round orders them by diagonal
  const int lx = OCT ? diag_column<BX, BY>(tid).x : tid & (BX - 1);
  const int ly = OCT ? diag_column<BX, BY>(tid).y : tid / BX;
  int sxd = a.sx, syd = a.sy, szd = a.sz;  // OCT: set per ticket
  int gxl = sxd > 0 ? lx : BX - 1 - lx;      // brick-local x, y in grid order
  int gyl = syd > 0 ? ly : BY - 1 - ly;
  const int nx = a.nx, ny = a.ny, nz = a.nz;
  const int ntx = a.ntx, nty = a.nty, ntz = a.ntz;
  // a block-masked sweep takes tickets only for the bricks with an active block
  const int ntile = a.nticket ? *a.nticket : ntx * nty * ntz;
  const uint8_t *__restrict__ tact = a.tact;
  const long long plane = a.plane, px = a.px;
  const float hmin = a.hmin;
  const GodConst64 k64 = a.k64;
  const GodConst32 k32 = a.k32;
  const uint8_t *__restrict__ blk_active = a.blk_active;
  unsigned int *__restrict__ blk_chg = a.blk_chg;
  const bool masked = a.fmask != nullptr;
  T *__restrict__ u = reinterpret_cast<T *>(a.u);
  const T *__restrict__ capg = reinterpret_cast<const T *>(a.cap);
  int epoch = a.epoch;  // OCT: epoch + the ticket's sweep
  T tmax = T(0);

  if (tid == 0) {
    s_abort = 0;
    mbar_init(bar, 1);
    mbar_fence_init();
    s_next = atomicAdd(a.ticket, 1);
  }
  __syncthreads();
  unsigned par = 0;  // phase parity of the box barrier
  for (;;) {
    const int tk = s_next;
    if (tid == 0) {
      s_lo = BZ;
      s_hi = -1;
    }
    // a uniform decision (s_abort may change under the reads); the barrier
    // also orders every read of s_next before its next write
    if (__syncthreads_or(tk >= ntile || s_abort)) break;
    int lt, osw = 0;
    unsigned obit = 0;   // OCT: the ticket's ordering bit
    bool sfull = false;  // OCT: the ticket's sweep visits every block
    if constexpr (OCT) {  // (sweep << 27) | brick in sweep order
      const int e = a.torder[tk];
      osw = e >> 27;
      lt = e & 0x07ffffff;
      sfull = (a.oct_full >> osw) & 1u;
      const int sn = (a.oct_first + osw) % 8 + 1;
      obit = 1u << (sn - 1);
      ordering_signs(sn, &sxd, &syd, &szd);
      gxl = sxd > 0 ? lx : BX - 1 - lx;
      gyl = syd > 0 ? ly : BY - 1 - ly;
      epoch = a.epoch + osw;
    } else {
      lt = a.torder[tk];  // local brick id in sweep order: (lk * nty + lj) * ntx + li
    }
    const int li = lt % ntx, lj = (lt / ntx) % nty, lk = lt / (ntx * nty);
    const int bi = sxd > 0 ? li : ntx - 1 - li;
    const int bj = syd > 0 ? lj : nty - 1 - lj;
    const int bk = szd > 0 ? lk : ntz - 1 - lk;
    const int tile = (bk * nty + bj) * ntx + bi;
    const int x0 = 1 + bi * BX, y0 = 1 + bj * BY, z0 = 1 + bk * BZ;

    // block mask: a brick none of whose 8^3 blocks is active keeps its values
    // and publishes at once (its faces are the old values its neighbours need);
    // otherwise only the levels that reach its active planes run
    bool run = true;
    int lev0 = 0, lev1 = NL;  // levels [lev0, lev1) of this brick
    if (OCT || blk_active) {
      bool act = false;
      if (tid < G::NBX * G::NBY * NZB) {
        const int q = tid / (G::NBX * G::NBY);
        const int bx = G::NBX * bi + tid % G::NBX, by = G::NBY * bj + (tid / G::NBX) % G::NBY;
        const int bz = bk * NZB + q;
        if (bx < a.nbx && by < a.nby && bz < a.nbz)
          act = OCT ? sfull || (__ldg(a.oct_bits + ((long long)bz * a.nby + by) * a.nbx + bx) & obit) != 0
                    : __ldg(blk_active + ((long long)bz * a.nby + by) * a.nbx + bx) != 0;
        if (act) {  // the block's planes 8q .. 8q+7 (grid order) in sweep order
          const int lo = szd > 0 ? 8 * q : BZ - 8 * q - 8;
          atomicMin(&s_lo, lo);
          atomicMax(&s_hi, lo + 7);
        }
      }
      run = __syncthreads_or(act) != 0;
      lev0 = s_lo;                        // thread (0, 0) reaches the first active plane
      lev1 = min(NL, s_hi + BX + BY - 1);  // thread (15, 15) leaves the last one
    }
    if (tid == 32) s_next = atomicAdd(a.ticket, 1);  // the next brick's ticket, fetched ahead
    if (!run) {
      if (tid == 0 && tile != a.poison_col) st_release_gpu(a.tflag + tile, epoch);
      __syncthreads();
      continue;
    }

    if constexpr (OCT) {
      // the round's earlier sweeps: this brick and its six face neighbours
      // (lanes 0..6 of warp 0, one each) finish their latest earlier sweep first
      bool okp = true;
      if (tid < 7) {
        int n = -1;
        if (tid == 0) n = tile;
        if (tid == 1 && bi > 0) n = tile - 1;
        if (tid == 2 && bi < ntx - 1) n = tile + 1;
        if (tid == 3 && bj > 0) n = tile - ntx;
        if (tid == 4 && bj < nty - 1) n = tile + ntx;
        if (tid == 5 && bk > 0) n = tile - ntx * nty;
        if (tid == 6 && bk < ntz - 1) n = tile + ntx * nty;
        int need = -1;
        if (n >= 0) {
          const unsigned tb = __ldg(a.oct_tbits + n);
          for (int j = osw - 1; j >= 0 && need < 0; --j)
            if (((a.oct_full >> j) & 1u) || ((tb >> ((a.oct_first + j) % 8)) & 1u)) need = j;
        }
        if (need >= 0 && ld_acquire_gpu(a.tflag + n) < a.epoch + need) {
          const long long t0 = cycles();
          unsigned nap = 32;
          while (ld_acquire_gpu(a.tflag + n) < a.epoch + need) {
            if (s_abort || *(volatile int *)(a.err + 1)) {
              s_abort = 1;
              okp = false;
              break;
            }
            if (cycles() - t0 > a.wait_cycles) {
              raise_timeout(a, tile, &s_abort);
              okp = false;
              break;
            }
            __nanosleep(nap);
            nap = min(nap * 2, 256u);
          }
        }
      }
      if (!__syncthreads_and(okp)) break;
    }
    // the box: TMA from (x0 - 1, y0 - 1, z0 - 1); out-of-range rows and planes read 0 (never used)
    fence_proxy_async();  // this CTA's generic accesses to the box come before the copy's writes
    __syncthreads();
    if (tid == 0) {
      mbar_arrive_tx(bar, G::BOX_BYTES);
      tma_load_3d(box, &tm_u, bi * BX, y0 - 1, z0 - 1, bar);
    }
    const bool vxy = (x0 + gxl <= nx) && (y0 + gyl <= ny);
    const int zcnt = min(BZ, nz - z0 + 1);  // planes of the brick inside the grid
    // frozen words of the brick's rows: node bit (x0 - 1 + gx) & 31
    if (masked) {
      for (int q = tid; q < BZ * BY; q += G::NT) {
        const int p = q / BY, r = q % BY;
        uint32_t w = 0;
        if (p < zcnt && y0 + r <= ny)
          w = __ldg(a.fmask + (long long)(z0 + p) * (a.mask_fy * a.mask_fw) + (long long)(bi >> 1) * a.mask_fy +
                    (y0 - 1 + r));
        smask[q] = w;
      }
    }
    const int mshift = 16 * (bi & 1) + gxl;
    // active 8^3 blocks of my (x, y) column, one bit per z block of the brick
    unsigned actz = (1u << NZB) - 1u;
    if ((OCT || blk_active) && vxy) {
      actz = 0;
      const int bx = (x0 - 1 + gxl) >> 3, by = (y0 - 1 + gyl) >> 3;
#pragma unroll
      for (int q = 0; q < NZB; ++q) {
        const int bz = bk * NZB + q;
        if (bz < a.nbz && (OCT ? sfull || (__ldg(a.oct_bits + ((long long)bz * a.nby + by) * a.nbx + bx) & obit) != 0
                                : __ldg(blk_active + ((long long)bz * a.nby + by) * a.nbx + bx) != 0))
          actz |= 1u << q;
      }
    }
    const long long gbase = (long long)z0 * plane + (long long)(y0 + gyl) * px + (x0 + gxl);
    // replace-update: the cap bounds of my column's 8^3 blocks in this brick
    using CB = CapBound<T, ARITH>;
    typename CB::type bnd[NZB];
#pragma unroll
    for (int q = 0; q < NZB; ++q) {
      bnd[q] = 0;
      if (MODE == MODE_REPLACE && vxy && bk * NZB + q < a.nbz)
        bnd[q] = CB::load(a, ((long long)(bk * NZB + q) * a.nby + ((y0 - 1 + gyl) >> 3)) * a.nbx + ((x0 - 1 + gxl) >> 3));
    }

    // wait for the upwind bricks (lanes 0..2 of warp 0, one each)
    bool ok = true;
    if (tid < 3) {
      int up = -1;
      if (tid == 0 && li > 0) up = tile - sxd;
      if (tid == 1 && lj > 0) up = tile - syd * ntx;
      if (tid == 2 && lk > 0) up = tile - szd * ntx * nty;
      // an upwind brick without an active block keeps its values: nothing to wait for
      if constexpr (OCT) {
        if (up >= 0 && !sfull && !(__ldg(a.oct_tbits + up) & obit)) up = -1;
      } else {
        if (up >= 0 && tact && !tact[up]) up = -1;
      }
      if (up >= 0 && ld_acquire_gpu(a.tflag + up) < epoch) {
        const long long t0 = cycles();
        unsigned nap = 32;
        while (ld_acquire_gpu(a.tflag + up) < epoch) {
          if (s_abort || *(volatile int *)(a.err + 1)) {
            s_abort = 1;
            ok = false;
            break;
          }
          if (cycles() - t0 > a.wait_cycles) {
            raise_timeout(a, tile, &s_abort);
            ok = false;
            break;
          }
          __nanosleep(nap);
          nap = min(nap * 2, 256u);
        }
      }
    }
    ok = __syncthreads_and(ok) != 0;
    // the box copy has landed (bounded wait; on abort it is still drained below)
    bool landed = mbar_wait(bar, par, a, tile, &s_abort);
    if (!__syncthreads_and(ok && landed)) {
      if (!landed && tid == 0) {  // let the copy land before the CTA leaves
        const long long t0 = cycles();
        while (!mbar_try(bar, par) && cycles() - t0 < 4000000000ll) {
        }
      }
      break;
    }
    par ^= 1u;
    // upwind halo faces: this sweep's values, written by the upwind bricks (L2)
    if (li > 0) {  // x face
      const int xu = sxd > 0 ? x0 - 1 : x0 + BX;
      const int sxo = sxd > 0 ? 0 : BX + 1;
      for (int q = tid; q < BZ * BY; q += G::NT) {
        const int p = q / BY, r = q % BY;
        if (p < zcnt && y0 + r <= ny)
          box[(1 + p) * PL + (1 + r) * W + sxo] =
              __ldcg(u + (long long)(z0 + p) * plane + (long long)(y0 + r) * px + xu);
      }
    }
    if (lj > 0) {  // y face
      const int yu = syd > 0 ? y0 - 1 : y0 + BY;
      const int syo = syd > 0 ? 0 : BY + 1;
      for (int q = tid; q < BZ * BX; q += G::NT) {
        const int p = q / BX, xx = q % BX;
        if (p < zcnt && x0 + xx <= nx)
          box[(1 + p) * PL + syo * W + 1 + xx] =
              __ldcg(u + (long long)(z0 + p) * plane + (long long)yu * px + x0 + xx);
      }
    }
    if (lk > 0) {  // z face
      const int zu = szd > 0 ? z0 - 1 : z0 + BZ;
      const int szo = szd > 0 ? 0 : BZ + 1;
      for (int q = tid; q < BY * BX; q += G::NT) {
        const int r = q / BX, xx = q % BX;
        if (y0 + r <= ny && x0 + xx <= nx)
          box[szo * PL + (1 + r) * W + 1 + xx] =
              __ldcg(u + (long long)zu * plane + (long long)(y0 + r) * px + x0 + xx);
      }
    }
    __syncthreads();

    // the levels: node (lx, ly, lz = L - lx - ly), sweep order
    const int obase = (1 + gyl) * W + 1 + gxl + (szd > 0 ? PL : BZ * PL);  // lz = 0
    const int dzo = szd > 0 ? PL : -PL;
    T accb[NZB];
#pragma unroll
    for (int q = 0; q < NZB; ++q) accb[q] = T(0);
    const int lxy = lx + ly;
    // pair-arithmetic rounds: the planes of my column that update, one bit per
    // plane in sweep order (inside the grid, in an active 8^3 block, not
    // frozen), read once per brick, off the levels' dependency chain (768^3
    // polish round 22.0 -> 20.5 ms; the FP32 kernels were slower that way and
    // test each node as they reach it)
    constexpr bool kPlaneBits = OCT && ARITH == ARITH_PAIR;
    using PlaneBits = typename std::conditional<(BZ > 32), unsigned long long, unsigned>::type;
    PlaneBits live = 0;
    if (kPlaneBits && vxy) {
#pragma unroll 4
      for (int lz = 0; lz < BZ; ++lz) {
        const int gz = szd > 0 ? lz : BZ - 1 - lz;
        bool on = gz < zcnt && ((actz >> (gz >> 3)) & 1u);
        if (masked && on) on = !((smask[gz * BY + gyl] >> mshift) & 1u);
        if (on) live |= PlaneBits(1) << lz;
      }
    }
    for (int L = lev0; L < lev1; ++L) {
      const int lz = L - lxy;
      if ((unsigned)lz < (unsigned)BZ) {
        const int gz = szd > 0 ? lz : BZ - 1 - lz;
        if (kPlaneBits ? ((live >> lz) & 1u) != 0 : (vxy && gz < zcnt)) {
          const int o = obase + lz * dzo;
          const T cv = box[o];
          // the reference's minima keep grid orientation: min(u[x-1], u[x+1])
          const T m0 = vmin<T, ARITH>(box[o - 1], box[o + 1]);
          const T m1 = vmin<T, ARITH>(box[o - W], box[o + W]);
          const T m2 = vmin<T, ARITH>(box[o - PL], box[o + PL]);
          bool act = true;
          if constexpr (!kPlaneBits) {
            act = (actz >> (gz >> 3)) & 1u;
            if (masked && act) act = !((smask[gz * BY + gyl] >> mshift) & 1u);
          }
          if (act) {
            const T g = local_update<T, MODE, ARITH, ISO>(m0, m1, m2, k64, k32);
            T nv;
            if constexpr (MODE == MODE_REPLACE) {
              typename CB::type b = bnd[0];
#pragma unroll
              for (int q = 1; q < NZB; ++q)
                if ((gz >> 3) == q) b = bnd[q];
              nv = CB::below(g, b) ? g : vmin<T, ARITH>(cap_value<T, ARITH>(capg + gbase + (long long)gz * plane), g);
            } else {
              nv = vmin<T, ARITH>(cv, g);
            }
            if (vdiffers<T, ARITH>(nv, cv)) {
              box[o] = nv;
              u[gbase + (long long)gz * plane] = nv;
              const T d = node_change<T, ARITH>(cv, nv, hmin);
              tmax = vmax_nonneg<T, ARITH>(tmax, d);
              if (!OCT && blk_chg) {
#pragma unroll
                for (int q = 0; q < NZB; ++q)
                  if ((gz >> 3) == q) accb[q] = vmax_nonneg<T, ARITH>(accb[q], d);
              }
            }
          }
        }
      }
      __syncthreads();
    }
    // per-block change: lanes of one warp with the same 8^3 block are lx in
    // [0, 8) or [8, 16) of the warp's two rows (rounds record none)
    if (!OCT && blk_chg) {
#pragma unroll
      for (int q = 0; q < NZB; ++q) {
        T v = accb[q];
#pragma unroll
        for (int off = 1; off <= 16; off <<= 1) {
          if (off == 8) continue;
          const T w2 = __shfl_xor_sync(0xffffffffu, v, off);
          v = vmax_nonneg<T, ARITH>(v, w2);
        }
        // only nodes inside the grid change, so v > 0 names a block of the grid
        const int bz = bk * NZB + q;
        if ((lane == 0 || lane == 8) && change_pos<T, ARITH>(v) && bz < a.nbz) {
          const int bx = (x0 - 1 + gxl) >> 3, by = (y0 - 1 + gyl) >> 3;
          atomicMax(blk_chg + ((long long)bz * a.nby + by) * a.nbx + bx, __float_as_uint(change_f<T, ARITH>(v)));
        }
      }
    }
    if constexpr (OCT) {  // this sweep's change word (one per sweep of the round)
      T v = tmax;
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) v = vmax_nonneg<T, ARITH>(v, __shfl_xor_sync(0xffffffffu, v, off));
      if (lane == 0 && change_pos<T, ARITH>(v)) {
        if constexpr (sizeof(T) == 4)  // the low word of the sweep's 64-bit slot
          atomicMax(reinterpret_cast<unsigned int *>(reinterpret_cast<unsigned long long *>(a.maxchg) + osw),
                    __float_as_uint(v));
        else
          atomicMax(reinterpret_cast<unsigned long long *>(a.maxchg) + osw, change_u64<T, ARITH>(v));
      }
      tmax = T(0);
    }
    // publish: the barrier orders every thread's stores before thread 0's
    // GPU-scope fence, which orders them before the flag
    __syncthreads();
    if (tid == 0 && tile != a.poison_col) publish_gpu(a.tflag + tile, epoch);
  }
  // the CTA's max change -> the grid's counter (one atomic per warp)
  {
    T v = tmax;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v = vmax_nonneg<T, ARITH>(v, __shfl_xor_sync(0xffffffffu, v, off));
    if (lane == 0 && change_pos<T, ARITH>(v)) {
      if constexpr (sizeof(T) == 4)
        atomicMax(reinterpret_cast<unsigned int *>(a.maxchg), __float_as_uint(v));
      else
        atomicMax(reinterpret_cast<unsigned long long *>(a.maxchg), change_u64<T, ARITH>(v));
    }
  }
}

}  // namespace pdfs
