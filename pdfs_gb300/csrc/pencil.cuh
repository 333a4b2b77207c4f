// pencil.cuh -- the pencil sweep: a CTA marches a 16 x 16 pencil of the grid
// through the whole z extent, one CTA barrier per level.
//
// The reference sweeps one hyperplane x+y+z = level of the whole grid per
// kernel launch (single_gpu_cuda/src/phi3D_fsm.cu:161-185,
// mpi_openacc/src/phi3D_fsm.c:92-117).  Any topological order of an
// ordering's dependency DAG gives the same result (each node reads the new
// values of its three upwind neighbours and the old values of its three
// downwind ones).  This kernel's order:
//   * compute thread (lx, ly) -- pencil-local coordinates in sweep order --
//     updates node (lx, ly, lz = G - lx - ly) at level G; a named barrier of
//     the 256 compute threads separates levels.  Every thread is busy on all
//     but SK = 30 of the nz + 30 levels, where a brick (tile3d.cuh) idles its
//     threads for 30 of every BZ + 30;
//   * planes stream through a ring of D shared-memory slots (TMA,
//     cp.async.bulk.tensor; one mbarrier per slot), as far ahead as the slot
//     of the plane SK + 1 levels back allows;
//   * faces cross pencils through mailboxes of epoch-tagged 64-bit words: the
//     threads on a pencil's downwind x (y) face write each node's final value
//     of the sweep, tagged with the sweep's epoch, to entry [lz + ly][ly]
//     ([lz + lx][lx]).  A 64-bit store is single-copy atomic, so a reader that
//     sees the tag sees the value: no GPU-scope fence and no progress counter.
//     Thread (0, ly) at level G reads the upwind x pencil's node (15, ly,
//     G - ly), entry [G][ly], which that pencil wrote at its level G + 15, so
//     a pencil runs about 16 levels behind its neighbours;
//   * a loader warp requests the planes and reports them landed, and a face
//     warp polls the upwind mailboxes a few diagonals ahead and patches the
//     tagged values into the landed planes;
//   * pencils are taken by ticket in wavefront order, so an upwind pencil is
//     always running or done; every wait is bounded (SweepArgs::wait_cycles)
//     and ends in DEV_ERR_TIMEOUT plus the abort flag, never in a hang.
// Sweeps with a block mask or block-change output run on bricks instead.
#pragma once
#include "sweep.cuh"


namespace pdfs {

template <class T>
struct PcGeo {
  static constexpr int BX = 16, BY = 16;
  // slot row: x0-1 .. x0+BX rounded up to 16 bytes (the field's index has no x
  // offset, so x0 - 1 = 16*cx starts the row on a 16-byte boundary)
  static constexpr int W = (int)((((BX + 2) * sizeof(T)) + 15) / 16 * 16 / sizeof(T));
  static constexpr int RY = BY + 2;        // slot rows: y0-1 .. y0+BY
  static constexpr int SK = BX + BY - 2;   // thread (15, 15) trails thread (0, 0) by SK planes
  // planes requested ahead of use; FP32 publishes its done count every other level
  static constexpr int LOOK = sizeof(T) == 4 ? 11 : 7;
  static constexpr int PUB = sizeof(T) == 4 ? 1 : 0;
  static constexpr int D = SK + 3 + LOOK;  // ring slots
  // planes requested into L2 (a TMA prefetch) this far ahead of their load:
  // the FP64 ring's 7-plane look-ahead does not cover a DRAM round trip (768^3
  // pair polish sweep 6.91 -> 6.54 ms with 12 planes); the FP32 ring's 11 do
  // (3.54 -> 3.62 ms with 16: the prefetch only costs there)
  static constexpr int PF = sizeof(T) == 4 ? 0 : 12;
  static constexpr unsigned FIELD_BYTES = (unsigned)(W * RY * sizeof(T));
  static constexpr unsigned MASK_OFF = (FIELD_BYTES + 127u) & ~127u;  // the plane's 16 frozen words
  static constexpr unsigned SLOT_BYTES = MASK_OFF + 128u;
  static constexpr int NC = BX * BY;       // compute threads
  static constexpr int NT = NC + 64;       // and the loader and face warps
  static constexpr int WV = (int)sizeof(T) / 4 > 1 ? 2 : 1;  // mailbox words per value (32 value bits each)
  static constexpr int C = 8;              // levels the face warp prepares per round, at most
  static constexpr size_t OFF_BAR = (size_t)D * SLOT_BYTES;
  static constexpr size_t BYTES = OFF_BAR + (size_t)D * 8 + 16;
  static_assert(SLOT_BYTES % 128 == 0, "TMA destinations stay 128-byte aligned");
};

__device__ __forceinline__ void compute_bar() { asm volatile("bar.sync 1, 256;\n" ::: "memory"); }

__device__ __forceinline__ void st_relaxed_gpu_u64(unsigned long long *p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;\n" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_relaxed_gpu_u64(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];\n" : "=l"(v) : "l"(p) : "memory");
  return v;
}
// A value's 32-bit pieces, each tagged with the epoch in the upper word.
template <class T>
__device__ __forceinline__ void mail_put(unsigned long long *e, T v, int epoch) {
  const unsigned long long tag = (unsigned long long)(unsigned)epoch << 32;
  if constexpr (sizeof(T) == 4) {
    st_relaxed_gpu_u64(e, tag | __float_as_uint(v));
  } else {
    st_relaxed_gpu_u64(e, tag | (unsigned)__double2loint(v));
    st_relaxed_gpu_u64(e + 1, tag | (unsigned)__double2hiint(v));
  }
}
template <class T>
__device__ __forceinline__ bool mail_get(const unsigned long long *e, int epoch, T &v) {
  const unsigned tag = (unsigned)epoch;
  const unsigned long long w0 = ld_relaxed_gpu_u64(e);
  if constexpr (sizeof(T) == 4) {
    v = __uint_as_float((unsigned)w0);
    return (unsigned)(w0 >> 32) == tag;
  } else {
    const unsigned long long w1 = ld_relaxed_gpu_u64(e + 1);
    v = __hiloint2double((int)(unsigned)w1, (int)(unsigned)w0);
    return (unsigned)(w0 >> 32) == tag && (unsigned)(w1 >> 32) == tag;
  }
}

// A warp's max change -> the change word (FP32: float bits; FP64: the u64
// key of change_u64), one atomic per warp.
template <class T, int ARITH>
__device__ __forceinline__ void warp_change_out(T v, void *maxchg, int lane) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v = vmax_nonneg<T, ARITH>(v, __shfl_xor_sync(0xffffffffu, v, off));
  if (lane == 0 && change_pos<T, ARITH>(v)) {
    if constexpr (sizeof(T) == 4)
      atomicMax(reinterpret_cast<unsigned int *>(maxchg), __float_as_uint(v));
    else
      atomicMax(reinterpret_cast<unsigned long long *>(maxchg), change_u64<T, ARITH>(v));
  }
}

// One idle round of a helper warp: lane 0 decides, for the whole warp, to give
// up on the abort flag or after wait_cycles without progress.
__device__ __forceinline__ bool helper_idle(const SweepArgs &a, int col, volatile int *s_abort, long long t_last,
                                            unsigned &nap) {
  int stop = 0;
  if ((threadIdx.x & 31) == 0) {
    if (*s_abort || *(volatile int *)(a.err + 1)) {
      stop = 1;
    } else if (cycles() - t_last > a.wait_cycles) {
      raise_timeout(a, col, s_abort);
      stop = 1;
    }
  }
  if (__shfl_sync(0xffffffffu, stop, 0)) {
    *s_abort = 1;
    return true;
  }
  if (nap) __nanosleep(nap);
  nap = min(nap + 32u, 128u);
  return false;
}

// Batched rounds: the grid description of the current ticket, staged in
// shared memory (a function-scope __shared__ object, so the single-grid
// instantiations do not carry it).
__device__ __forceinline__ SweepArgs &pc_batch_args() {
  __shared__ SweepArgs s;
  return s;
}
template <bool BATCH>
__device__ __forceinline__ const SweepArgs &pc_args(const SweepArgs &a0) {
  if constexpr (BATCH)
    return pc_batch_args();
  else
    return a0;
}
__device__ __forceinline__ void fence_proxy_async_global() {
  asm volatile("fence.proxy.async.global;\n" ::: "memory");
}

// BATCH: one launch runs a whole round -- the 8 orderings of every grid of a
// batch (BatchDesc).  A ticket names (grid, sweep, pencil); sweep s of a grid
// starts once every pencil of its sweep s - 1 has finished (a per-(grid,
// sweep) counter, bounded wait), and tickets list every grid's sweep s before
// any grid's sweep s + 1, so every wait is on smaller tickets.
template <class T, int MODE, int ARITH, bool ISO, bool BATCH = false>
__global__ void __launch_bounds__(PcGeo<T>::NT) pc_sweep_kernel(const __grid_constant__ CUtensorMap tm_u,
                                                               const __grid_constant__ CUtensorMap tm_mask,
                                                               const __grid_constant__ SweepArgs a0) {
  const SweepArgs &a = pc_args<BATCH>(a0);
  using G = PcGeo<T>;
  constexpr int BX = G::BX, BY = G::BY, W = G::W, SK = G::SK, D = G::D;
  constexpr int SE = (int)(G::SLOT_BYTES / sizeof(T));  // slot stride in elements
  extern __shared__ __align__(1024) unsigned char sm[];
  T *ring = reinterpret_cast<T *>(sm);
  uint64_t *full = reinterpret_cast<uint64_t *>(sm + G::OFF_BAR);
  __shared__ int s_ticket, s_stop, s_done, s_ready, s_landed;
  __shared__ int s_gs, s_lc;                // BATCH: the ticket's grid * 8 + sweep, and its pencil
  __shared__ const CUtensorMap *s_maps;     // BATCH: the grid's tensor maps
  __shared__ volatile int s_abort;

  if ((saddr(sm) & 127u) != 0) {  // TMA destinations must be 128-byte aligned
    if (threadIdx.x == 0) {
      atomicCAS(a0.err, 0, DEV_ERR_SMEM_ALIGN);
      atomicExch(a0.err + 1, 1);
    }
    return;
  }
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  int ntick;
  if constexpr (BATCH)
    ntick = a0.batch->nticket;
  else
    ntick = a0.ncx * a0.ncy;
  int cur_gs = -1;  // BATCH: the (grid, sweep) staged in shared memory
  T tmax = T(0);

  if (tid == 0) s_abort = 0;
  for (int npen = 0;; ++npen) {
    if (tid == 0) {
      const int tk = atomicAdd(a0.ticket, 1);
      s_ticket = tk;
      if constexpr (BATCH) {
        if (tk < ntick) {
          const int2 e = a0.batch->tickets[tk];
          s_gs = e.x;
          s_lc = e.y;
        }
      }
      if (*(volatile int *)(a0.err + 1)) s_abort = 1;
      s_stop = (tk >= ntick || s_abort) ? 1 : 0;
      s_done = 0;
      s_ready = 0;
      s_landed = 0;
      for (int i = 0; i < D; ++i) {
        if (npen) mbar_inval(full + i);
        mbar_init(full + i, 1);
      }
      mbar_fence_init();
    }
    __syncthreads();
    if (s_stop) break;
    if constexpr (BATCH) {
      if (s_gs != cur_gs) {  // stage the grid's description; set the sweep's direction, epoch, change word
        cur_gs = s_gs;
        const int g = cur_gs >> 3, sw = cur_gs & 7;
        const int *ws = reinterpret_cast<const int *>(a0.batch->args + g);
        int *wd = reinterpret_cast<int *>(&pc_batch_args());
        for (int i = tid; i < (int)(sizeof(SweepArgs) / 4); i += blockDim.x) wd[i] = ws[i];
        __syncthreads();
        if (tid == 0) {
          SweepArgs &S = pc_batch_args();
          ordering_signs(sw + 1, &S.sx, &S.sy, &S.sz);
          S.epoch += 8 * *a0.batch->round + sw;
          S.err = a0.err;
          S.ticket = a0.ticket;
          S.maxchg = reinterpret_cast<unsigned long long *>(a0.maxchg) + (size_t)sw * a0.batch->ngrid + g;
          s_maps = a0.batch->maps + 3 * g;
          // the grid's previous sweep must be complete: its stores, then its count (release)
          if (sw > 0) {
            const int *cnt = a0.batch->done + cur_gs - 1;
            const int need = S.ncx * S.ncy;
            if (ld_acquire_gpu(cnt) < need) {
              const long long t0 = cycles();
              unsigned nap = 32;
              while (ld_acquire_gpu(cnt) < need) {
                if (s_abort || *(volatile int *)(a0.err + 1)) {
                  s_abort = 1;
                  break;
                }
                if (cycles() - t0 > S.wait_cycles) {
                  raise_timeout(S, -1, &s_abort);
                  break;
                }
                __nanosleep(nap);
                nap = min(nap * 2, 256u);
              }
            }
          }
        }
        __syncthreads();
        if (s_abort) break;
      }
    }
    const int sxd = a.sx, syd = a.sy, szd = a.sz;
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    const int NP = nz + 2, t_end = nz + SK;  // planes (sweep order, halo planes included), levels
    const long long plane = a.plane, px = a.px;
    const bool masked = a.fmask != nullptr;
    const int epoch = a.epoch;
    const CUtensorMap *mp_u, *mp_mask;
    if constexpr (BATCH) {
      mp_u = s_maps;
      mp_mask = s_maps + 2;
    } else {
      mp_u = &tm_u;
      mp_mask = &tm_mask;
    }
    int lc;
    if constexpr (BATCH)
      lc = s_lc;
    else
      lc = a.order[s_ticket];
    const int lcx = lc % a.ncx, lcy = lc / a.ncx;
    const int cx = sxd > 0 ? lcx : a.ncx - 1 - lcx;
    const int cy = syd > 0 ? lcy : a.ncy - 1 - lcy;
    const int col = cy * a.ncx + cx;
    const int upx = lcx > 0 ? col - sxd : -1;
    const int upy = lcy > 0 ? col - syd * a.ncx : -1;
    const int x0 = 1 + cx * BX, y0 = 1 + cy * BY;

    if (warp == G::NC / 32) {
      // ------------------------------- loader warp (lane 0) -------------------------------
      int q_issue = 0, q_land = 0;  // planes requested / seen landed (plane q in slot q % D)
      const unsigned tx_bytes = G::FIELD_BYTES + (masked ? 64u : 0u);
      long long t_last = cycles();
      unsigned nap = 0;
      bool failed = false;
      // a round's earlier sweep was written by other CTAs of this launch:
      // order the acquire of its count before these async-proxy reads
      if constexpr (BATCH) fence_proxy_async_global();
      for (;;) {
        int moved = 0;
        if (lane == 0) {
          const int done = ld_acquire_cta_s(&s_done);
          // plane q reuses the slot of plane q - D, last read at level q - D + SK
          while (q_issue < NP && (q_issue < D || done >= q_issue - D + SK + 1)) {
            const int s = q_issue % D;
            const int gz = szd > 0 ? q_issue : nz + 1 - q_issue;
            unsigned char *dst = sm + (size_t)s * G::SLOT_BYTES;
            mbar_arrive_tx(full + s, tx_bytes);
            tma_load_3d(dst, mp_u, cx * BX, y0 - 1, gz, full + s);
            if (masked) tma_load_3d(dst + G::MASK_OFF, mp_mask, cy * BY, cx >> 1, gz, full + s);
            if constexpr (G::PF > 0) {
              const int qp = q_issue + G::PF;
              if (qp < NP) {
                const int gzp = szd > 0 ? qp : nz + 1 - qp;
                tma_prefetch_3d(mp_u, cx * BX, y0 - 1, gzp);
                if (masked) tma_prefetch_3d(mp_mask, cy * BY, cx >> 1, gzp);
              }
            }
            ++q_issue;
            moved = 1;
          }
          const int q0 = q_land;
          while (q_land < q_issue && mbar_try(full + q_land % D, (q_land / D) & 1)) ++q_land;
          if (q_land > q0) {
            st_release_cta_s(&s_landed, q_land);
            moved = 1;
          }
        }
        moved = __shfl_sync(0xffffffffu, moved, 0);  // lane 0 decides for the warp
        q_issue = __shfl_sync(0xffffffffu, q_issue, 0);
        q_land = __shfl_sync(0xffffffffu, q_land, 0);
        if (q_land >= NP) break;
        if (moved) {
          t_last = cycles();
          nap = 0;
        } else if (helper_idle(a, col, &s_abort, t_last, nap)) {
          failed = true;
          break;
        }
      }
      if (failed && lane == 0) {  // let the copies in flight land before the CTA leaves
        for (int q = q_land; q < q_issue; ++q) {
          const long long t0 = cycles();
          while (!mbar_try(full + q % D, (q / D) & 1) && cycles() - t0 < 4000000000ll) {
          }
        }
      }
    } else if (warp == G::NC / 32 + 1) {
      // -------------------------------------- face warp --------------------------------------
      // Level g needs planes up to min(g + 2, NP - 1) and diagonal g of the
      // upwind pencils' face mailboxes.
      int g_ready = 0;
      const int sxo = sxd > 0 ? 0 : BX + 1;  // x face: slot x
      const int syo = syd > 0 ? 0 : BY + 1;  // y face: slot row
      const int k = lane & 15;
      const bool xl = lane < 16;  // lane < 16: x face row ly = lane; else y face column lx = lane - 16
      const int up = xl ? upx : upy;
      const int gk = xl ? (syd > 0 ? k : BY - 1 - k) : (sxd > 0 ? k : BX - 1 - k);
      const bool need = up >= 0 && (xl ? (y0 + gk <= ny) : (x0 + gk <= nx));
      const unsigned long long *box =
          need ? a.pmail + (((size_t)up * 2 + (xl ? 0 : 1)) * a.prow * 16 + k) * G::WV : nullptr;
      long long t_last = cycles();
      unsigned nap = 0;
      while (g_ready < t_end) {
        const int landed = __shfl_sync(0xffffffffu, ld_acquire_cta_s(&s_landed), 0);
        const int plim = landed >= NP ? t_end : landed - 2;
        int lim = min(min(t_end, plim), g_ready + G::C);
        T v[G::C];
        unsigned okm = 0;  // bit i: level g_ready + i is ready for this lane
#pragma unroll
        for (int i = 0; i < G::C; ++i) {
          const int g = g_ready + i, lz = g - k;
          bool ok = true;
          if (need && g < lim && lz >= 0 && lz < nz) ok = mail_get<T>(box + (size_t)g * 16 * G::WV, epoch, v[i]);
          if (ok) okm |= 1u << i;
        }
        okm = __reduce_and_sync(0xffffffffu, okm);
        lim = min(lim, g_ready + __ffs(~okm) - 1);  // the ready prefix
        if (lim > g_ready) {
#pragma unroll
          for (int i = 0; i < G::C; ++i) {
            const int g = g_ready + i, lz = g - k;
            if (need && g < lim && lz >= 0 && lz < nz)
              ring[((lz + 1) % D) * SE + (xl ? (1 + gk) * W + sxo : syo * W + 1 + gk)] = v[i];
          }
          __syncwarp();
          fence_proxy_async();  // these halo stores come before a later TMA write into the slots
          __syncwarp();
          if (lane == 0) st_release_cta_s(&s_ready, lim);
          g_ready = lim;
          t_last = cycles();
          nap = 0;
        } else if (helper_idle(a, col, &s_abort, t_last, nap)) {
          break;
        }
      }
    } else {
      // ------------------------------------ compute threads ------------------------------------
      const int lx = tid & (BX - 1), ly = tid / BX, lxy = lx + ly;  // sweep order
      const int gx = sxd > 0 ? lx : BX - 1 - lx, gy = syd > 0 ? ly : BY - 1 - ly;
      const bool vxy = (x0 + gx <= nx) && (y0 + gy <= ny);
      const int orow = (1 + gy) * W + 1 + gx;  // my node within a slot
      const int mbyte = (int)G::MASK_OFF + 4 * gy, mshift = 16 * (cx & 1) + gx;
      const long long grow = (long long)(y0 + gy) * px + (x0 + gx);
      // downwind faces: my node's final value goes to a mailbox when a pencil is downwind
      const bool poisoned = col == a.poison_col;
      const bool mx = lx == BX - 1 && lcx < a.ncx - 1 && !poisoned;
      const bool my = ly == BY - 1 && lcy < a.ncy - 1 && !poisoned;
      unsigned long long *xmail = a.pmail + ((size_t)col * 2 + 0) * a.prow * 16 * G::WV;
      unsigned long long *ymail = a.pmail + ((size_t)col * 2 + 1) * a.prow * 16 * G::WV;
      const float hmin = a.hmin;
      const GodConst64 k64 = a.k64;
      const GodConst32 k32 = a.k32;
      T *__restrict__ u = reinterpret_cast<T *>(a.u);
      const T *__restrict__ capg = reinterpret_cast<const T *>(a.cap);
      auto gz_of = [&](int lz) { return szd > 0 ? lz + 1 : nz - lz; };
      // replace-update: the cap bound of my node's 8^3 block, and of the next
      // block in sweep order (loaded one block ahead)
      using CB = CapBound<T, ARITH>;
      typename CB::type bcur = 0, bnxt = 0;
      int bzc = 0;
      const long long bxy = (long long)((y0 - 1 + gy) >> 3) * a.nbx + ((x0 - 1 + gx) >> 3);
      const int dbz = szd > 0 ? 1 : -1;
      auto bnd_at = [&](int bz) -> typename CB::type {
        return (bz >= 0 && bz < a.nbz) ? CB::load(a, (long long)bz * a.nby * a.nbx + bxy) : typename CB::type(0);
      };
      if (MODE == MODE_REPLACE && vxy) {
        bzc = (gz_of(0) - 1) >> 3;
        bcur = bnd_at(bzc);
        bnxt = bnd_at(bzc + dbz);
      }
      int sl = (1 - lxy) % D;  // slot of my node's plane (lz + 1) at level 0
      if (sl < 0) sl += D;
      int ready = 0;  // thread 0: levels below it are prepared (re-read only when reached)
      bool stop = false;
      for (int g = 0; g < t_end; ++g) {
        if (tid == 0 && ready <= g) {
          ready = ld_acquire_cta_s(&s_ready);
          const long long t0 = cycles();
          while (ready <= g) {
            if (s_abort) {
              stop = true;
              break;
            }
            if (cycles() - t0 > a.wait_cycles) {
              raise_timeout(a, col, &s_abort);
              stop = true;
              break;
            }
            ready = ld_acquire_cta_s(&s_ready);
          }
        }
        if (tid == 0 && stop) s_stop = 1;
        compute_bar();
        if (s_stop) {
          stop = true;
          break;
        }
        // levels below g are complete (FP32: published every other level; its ring looks further ahead)
        if (tid == 0 && (g & G::PUB) == 0) st_release_cta_s(&s_done, g);
        const int lz = g - lxy;
        if ((unsigned)lz < (unsigned)nz) {
          if (vxy) {
            const int sp = sl == 0 ? D - 1 : sl - 1, sn = sl == D - 1 ? 0 : sl + 1;
            T *cur = ring + sl * SE;
            const T *prv = ring + sp * SE, *nxt = ring + sn * SE;
            const T cv = cur[orow];
            const T m0 = vmin<T, ARITH>(cur[orow - 1], cur[orow + 1]);
            const T m1 = vmin<T, ARITH>(cur[orow - W], cur[orow + W]);
            // grid orientation: min(u[z-1], u[z+1]); the sweep's previous plane is z-1 when sz > 0
            const T m2 = szd > 0 ? vmin<T, ARITH>(prv[orow], nxt[orow]) : vmin<T, ARITH>(nxt[orow], prv[orow]);
            bool act = true;
            if (masked) {
              const uint32_t w = *reinterpret_cast<const uint32_t *>(sm + (size_t)sl * G::SLOT_BYTES + mbyte);
              act = !((w >> mshift) & 1u);
            }
            if constexpr (MODE == MODE_REPLACE) {
              // my nodes are consecutive in sweep order: the block moves one step at a time
              const int bz = (gz_of(lz) - 1) >> 3;
              if (bz != bzc) {
                bzc = bz;
                bcur = bnxt;
                bnxt = bnd_at(bz + dbz);
              }
            }
            T fin = cv;  // the node's value at the end of the sweep
            if (act) {
              const T gv = local_update<T, MODE, ARITH, ISO>(m0, m1, m2, k64, k32);
              T nv;
              if constexpr (MODE == MODE_REPLACE) {
                nv = CB::below(gv, bcur) ? gv
                                         : vmin<T, ARITH>(cap_value<T, ARITH>(capg + (long long)gz_of(lz) * plane + grow), gv);
              } else {
                nv = vmin<T, ARITH>(cv, gv);
              }
              if (vdiffers<T, ARITH>(nv, cv)) {
                fin = nv;
                cur[orow] = nv;
                u[(long long)gz_of(lz) * plane + grow] = nv;
                tmax = vmax_nonneg<T, ARITH>(tmax, node_change<T, ARITH>(cv, nv, hmin));
                fence_proxy_async();  // this store comes before a later TMA write into the slot
              }
            }
            if (mx) mail_put<T>(xmail + ((size_t)(lz + ly) * 16 + ly) * G::WV, fin, epoch);
            if (my) mail_put<T>(ymail + ((size_t)(lz + lx) * 16 + lx) * G::WV, fin, epoch);
          }
        }
        sl = sl == D - 1 ? 0 : sl + 1;
      }
      compute_bar();
      if (tid == 0 && !stop) st_release_cta_s(&s_done, t_end);
      if constexpr (BATCH) {
        // this pencil's change -> its (grid, sweep) word; my stores come
        // before the next sweep's plane copies, which another CTA may issue
        warp_change_out<T, ARITH>(tmax, a.maxchg, lane);
        tmax = T(0);
        fence_proxy_async_global();
      }
    }
    __syncthreads();
    if (s_abort) break;
    if constexpr (BATCH) {  // the pencil is done: count it (release)
      if (tid == 0) {
        __threadfence();
        atomicAdd(a0.batch->done + cur_gs, 1);
      }
    }
  }
  // the CTA's max change -> the grid's counter (one atomic per warp)
  if constexpr (!BATCH) warp_change_out<T, ARITH>(tmax, a.maxchg, lane);
}

}  // namespace pdfs
