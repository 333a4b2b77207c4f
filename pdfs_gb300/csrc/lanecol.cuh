// lanecol.cuh -- the lane-column sweep: one warp per sheared tile of z-columns,
// every dependency inside the warp carried by registers and shuffles.
//
// The reference sweeps one hyperplane x+y+z = level of the whole grid per
// kernel launch (single_gpu_cuda/src/phi3D_fsm.cu:161-185,
// mpi_openacc/src/phi3D_fsm.c:92-117).  Any topological order of an
// ordering's dependency DAG gives the same result (each node reads the new
// values of its three upwind neighbours and the old values of its three
// downwind ones), so this kernel uses its own order:
//
// Layout ("ZC", z-columns).  The working field is stored z fastest: node
// (x, y, z) of the halo-padded grid is element (y*cxp + x)*QZ + Z0 + z, so a
// lane walking its own column reads consecutive elements, 16 or 32 bytes
// (four positions) per vector load, every byte of each sector used.  Nodes
// the sweeps must not change -- frozen nodes, the halo, and the padding at
// both ends of a column (-inf) -- carry the sign bit (of the hi word for FP32
// pairs); every neighbour is read as its absolute value, so a frozen node
// costs nothing and the min-update leaves it alone by itself.
//
// Tiles.  In sweep-local coordinates (lx, ly, lz), lane i and row r of tile
// (tx, ty) own the column (lx, ly) = (31 tx + i - 1, R ty + r - i - 1): the
// lanes of a row lie on an anti-diagonal of the x-y plane, so lx + ly is the
// same for every lane and all 32 lanes of row r sit on the same z (traversal
// position t = g - r) at tile level g.  The dependencies of node (lane i,
// row r) at level g are then:
//   x-upwind (new):  lane i-1, row r-1, level g-1    -> __shfl_up of res[r-1]
//   y-upwind (new):  lane i,   row r-1, level g-1    -> res[r-1]
//   z-upwind (new):  lane i,   row r,   level g-1    -> res[r]
//   x-downwind (old): lane i+1, row r+1, its next position -> __shfl_down
//   y-downwind (old): lane i,   row r+1, its next position -> register
//   z-downwind (old): lane i,   row r,   next position     -> register
// Row 0's upwind values come from the tile above (its row R-1, face
// mailbox), lane 0's x-upwind value from the tile to the left (its lane 30).
// Lane 31 is the downwind x halo (the next tile's lane 0 column: read, never
// written) and row R the downwind y halo (read, never computed), so a tile
// computes 31 x R columns.
//
// Faces cross tiles through mailboxes of epoch-tagged 64-bit words (value
// bits in the low word, the sweep's epoch in the high word; an FP32 pair is
// two such words): a 64-bit store is single-copy atomic, so a reader that
// sees the tag sees the value, and no fence or progress counter is needed.
// Tiles are taken by ticket in an order where every tile follows the tiles
// it waits on; every wait is bounded (wait_cycles) and ends in
// DEV_ERR_TIMEOUT plus the abort flag, never in a hang.
#pragma once
#include "sweep.cuh"

namespace pdfs {



// ---- memory helpers: one 16-byte vector of a column (four FP32 values or two
// pairs); the L2::256B hint has L2 fetch the next 256 bytes of the column too
// The field loads and stores are ordinary (schedulable) accesses: a lane
// reads each element of its columns once, before it or any other tile writes
// it, and writes only its own columns.
__device__ __forceinline__ void lc_ld(float (&v)[4], const float *p) {
  asm("ld.global.L2::256B.v4.f32 {%0, %1, %2, %3}, [%4];\n"
      : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3])
      : "l"(p));
}
__device__ __forceinline__ void lc_ld(double (&v)[2], const double *p) {
  asm("ld.global.L2::256B.v2.f64 {%0, %1}, [%2];\n" : "=d"(v[0]), "=d"(v[1]) : "l"(p));
}
__device__ __forceinline__ void lc_st(float *p, const float (&v)[4]) {
  *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
__device__ __forceinline__ void lc_st(double *p, const double (&v)[2]) {
  *reinterpret_cast<double2 *>(p) = make_double2(v[0], v[1]);
}
// Mailbox words: relaxed at GPU scope (single-copy atomic 64-bit words); a
// poll re-reads the word every time (volatile asm), nothing else is ordered.
__device__ __forceinline__ void lc_put(unsigned long long *p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;\n" ::"l"(p), "l"(v));
}
__device__ __forceinline__ unsigned long long lc_get(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];\n" : "=l"(v) : "l"(p));
  return v;
}

// ---- value helpers: FP32, or FP32 pairs (hi in the low word) ------------------------
template <class T>
struct LcVal;
template <>
struct LcVal<float> {
  static constexpr int WV = 1;  // mailbox words per value
  __device__ __forceinline__ static float ninf() { return -INFINITY; }
  __device__ __forceinline__ static float absv(float v) { return fabsf(v); }
  __device__ __forceinline__ static bool frozen(float v) { return __float_as_uint(v) >> 31; }
  __device__ __forceinline__ static unsigned word(float v, int) { return __float_as_uint(v); }
  __device__ __forceinline__ static float from(unsigned w0, unsigned) { return __uint_as_float(w0); }
};
template <>
struct LcVal<double> {
  static constexpr int WV = 2;
  __device__ __forceinline__ static double ninf() { return p_make(-INFINITY, 0.0f); }
  __device__ __forceinline__ static double absv(double v) {
    return __longlong_as_double(__double_as_longlong(v) & ~0x80000000LL);  // hi's sign bit
  }
  __device__ __forceinline__ static bool frozen(double v) { return (__double2loint(v) >> 31) & 1; }
  __device__ __forceinline__ static unsigned word(double v, int k) {
    return k ? (unsigned)__double2hiint(v) : (unsigned)__double2loint(v);
  }
  __device__ __forceinline__ static double from(unsigned w0, unsigned w1) {
    return __hiloint2double((int)w1, (int)w0);
  }
};

// The reference's min(a, b) = a < b ? a : b of the grid-oriented pair (u[k-1],
// u[k+1]) given the sweep-oriented (upwind, downwind) values: for FP32 the
// operands are non-negative and the result is the same either way; FP32 pairs
// keep the operand order so that equal values return the same bits.
template <class T>
__device__ __forceinline__ T lc_min(T upw, T dnw, bool fwd) {
  if constexpr (sizeof(T) == 4) {
    (void)fwd;
    return fminf(upw, dnw);
  } else {
    const bool lt = p_lt(upw, dnw), gt = p_lt(dnw, upw);
    return lt ? upw : (gt ? dnw : (fwd ? dnw : upw));
  }
}

template <class T, bool ISO>
__device__ __forceinline__ T lc_godunov(T m0, T m1, T m2, const GodConst32 &k) {
  if constexpr (sizeof(T) == 4)
    return god32s<ISO>(m0, m1, m2, k);
  else
    return god_pair<ISO>(m0, m1, m2, k);
}

// One warp per tile; T = float (FP32 min-update) or double (FP32 pairs, min
// or replace-update).  R rows per tile; VW positions per vector load (four
// FP32 values or two pairs: 16 bytes).  SZ is the sweep's z direction.  BLK:
// block mask and per-block change output in use.
// Four-row tiles fit 16 warps per SM (128 registers), eight-row tiles 12.
template <class T, int R, int MODE, bool ISO, int SZ, bool BLK>
__global__ void __launch_bounds__(128, R <= 4 ? 4 : 3) lc_sweep_kernel(const __grid_constant__ LcArgs a) {
  using V = LcVal<T>;
  constexpr int WV = V::WV;
  constexpr int VW = 16 / (int)sizeof(T);
  constexpr int ARITH = sizeof(T) == 4 ? ARITH_FAST : ARITH_PAIR;
  constexpr int NR = R + 1;  // rows with windows: R computed rows and the downwind halo row
  constexpr unsigned FULL = 0xffffffffu;
  static_assert(R >= 2 && R <= 8 && (8 % VW) == 0, "tile shape");
  const int lane = threadIdx.x & 31;
  const int ntiles = a.ntx * a.nty;
  const unsigned etag = (unsigned)a.epoch;
  const unsigned long long tag = (unsigned long long)etag << 32;
  const float hmin = a.hmin;
  const GodConst32 k32 = a.k32;
  const bool fx = a.sx > 0, fy = a.sy > 0;
  T *__restrict__ u = reinterpret_cast<T *>(a.u);
  const int T_ = a.T;
  const long long ys = a.cxp * a.qz;  // elements per +1 in y
  T tmx[R];  // each row's max change (separate chains, folded at the end)
#pragma unroll
  for (int r = 0; r < R; ++r) tmx[r] = T(0);

  for (;;) {
    int tk = 0, ab = 0;
    if (lane == 0) {
      tk = atomicAdd(a.ticket, 1);
      ab = *(volatile int *)(a.err + 1);
    }
    tk = __shfl_sync(FULL, tk, 0);
    ab = __shfl_sync(FULL, ab, 0);
    if (tk >= ntiles || ab) break;
    const int tile = a.order[tk];
    const int tx = tile % a.ntx, ty = tile / a.ntx;
    const bool publish = tile != a.poison_tile;

    // ---- this lane's columns: row r at (lx, ly0 + r) in sweep-local coordinates ----
    const int lx = kLcLanes * tx + lane - 1;
    const int ly0 = R * ty - lane - 1;
    const int gx = fx ? lx + 1 : a.nx - lx;
    const int gy0 = fy ? ly0 + 1 : a.ny - ly0;
    // the lane's row-0 column as a pointer; rows and positions as 32-bit offsets
    T *const ubase = u + ((long long)gy0 * ys + (long long)gx * a.qz);
    const int ys32 = fy ? (int)ys : -(int)ys;
    unsigned rowok = 0;  // bit r: row r's column lies in the halo-padded grid
#pragma unroll
    for (int r = 0; r < NR; ++r) {
      const int ly = ly0 + r;
      if (lx >= -1 && lx <= a.nx && ly >= -1 && ly <= a.ny) rowok |= 1u << r;
    }
    // vector v holds traversal positions VW v .. VW v + VW-1: column position
    // kLcZ0 + t going up, q_last - t going down (memory order reversed)
    const int qv0 = SZ > 0 ? kLcZ0 : a.q_last - (VW - 1);  // column position of vector 0
    auto vaddr = [&](int r, int v) -> T * { return ubase + (r * ys32 + qv0 + SZ * VW * v); };
    // Each row's window: cur = the vector of its position t, nxt = the next
    // one (in flight until the row reaches the last element of cur).  A row
    // entering a vector moves nxt into cur and loads the vector after it.
    T cur[NR][VW], nxt[NR][VW];
    T res[R];          // each row's new value of the previous level (its z-upwind value)
    bool chg[R];       // row r changed a node of its current vector
#pragma unroll
    for (int r = 0; r < R; ++r) chg[r] = false;
#pragma unroll
    for (int r = 0; r < NR; ++r) {
#pragma unroll
      for (int e = 0; e < VW; ++e) cur[r][e] = nxt[r][e] = V::ninf();
      const int v0 = -((r + VW - 1) / VW);  // vector of position t = -r (row r at level 0)
      if ((rowok >> r) & 1) {
        if (((-r) & (VW - 1)) == 0) {
          lc_ld(nxt[r], vaddr(r, v0));  // level 0 moves it into cur
        } else {
          lc_ld(cur[r], vaddr(r, v0));
          lc_ld(nxt[r], vaddr(r, v0 + 1));
        }
      }
    }
    // ---- 8^3 block bookkeeping: the row's current block (-1 outside the interior) ----
    int bxy[R], bcur[R];
    float bch[R], bnd[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int ly = ly0 + r, gy = fy ? ly + 1 : a.ny - ly;
      const bool in = lx >= 0 && lx < a.nx && ly >= 0 && ly < a.ny;
      bxy[r] = in ? ((gy - 1) >> 3) * a.nbx + ((gx - 1) >> 3) : -1;
      bcur[r] = -1;
      bch[r] = 0.0f;
      bnd[r] = -INFINITY;  // replace-update: read every cap until the row enters a block
    }

    // ---- face mailboxes ----
    const bool has_up = ty > 0;
    const unsigned long long *ybox = a.ymail + ((size_t)(has_up ? tile - a.ntx : 0) * T_ * 32 + lane) * WV;
    unsigned long long *ypub = a.ymail + ((size_t)tile * T_ * 32 + lane) * WV;
    // lane r < R reads row r's x-face entry, written by lane 30 of the tile to
    // the left (tile row (R ty + r + 30) / R), xmail row ly + 32 = R ty + 31 + r
    const int xrow_in = R * ty + 31 + lane;
    const bool has_left = lane < R && tx > 0 && (R * ty + lane + 30) / R < a.nty && xrow_in < a.xrows;
    const unsigned long long *xbox =
        a.xmail + ((size_t)(tx > 0 ? tx - 1 : 0) * a.xrows + (size_t)(has_left ? xrow_in : 0)) * T_ * WV;
    unsigned long long *xpub = a.xmail + ((size_t)tx * a.xrows + (size_t)R * ty + 1) * T_ * WV;

    // Mailbox words.  The x face of level g is fetched at the end of level
    // g-1; the y face (row 0's upwind row) is fetched at the start of level
    // g and only needed after rows R-1..1 of the level are done, so its
    // latency hides behind them.
    unsigned long long py0, py1, px0, px1;
    auto need_y = [&](int g) { return has_up && g < T_; };
    auto need_x = [&](int g) { return has_left && g - lane >= 0 && g - lane < T_; };
    auto fetch_y = [&](int g) {
      const bool n = need_y(g);
      py0 = n ? lc_get(ybox + (size_t)g * 32 * WV) : (tag | 0x7f800000ull);
      py1 = (WV == 2 && n) ? lc_get(ybox + (size_t)g * 32 * WV + 1) : tag;
    };
    auto fetch_x = [&](int g) {
      const bool n = need_x(g);
      px0 = n ? lc_get(xbox + (size_t)(g - lane) * WV) : (tag | 0x7f800000ull);
      px1 = (WV == 2 && n) ? lc_get(xbox + (size_t)(g - lane) * WV + 1) : tag;
    };
    auto ok_y = [&]() { return (unsigned)(py0 >> 32) == etag && (WV == 1 || (unsigned)(py1 >> 32) == etag); };
    auto ok_x = [&]() { return (unsigned)(px0 >> 32) == etag && (WV == 1 || (unsigned)(px1 >> 32) == etag); };
    // Bounded wait until the words of level g carry this sweep's tag: a few
    // tight polls (each an L2 round trip), then sleeps of growing length.
    // false: the wait gave up (timeout recorded) or another tile aborted.
    auto wait_faces = [&](int g, bool ys) -> bool {
      const long long t0 = clock64();
      unsigned nap = 0;
      for (int it = 0;; ++it) {
        if (ys) {
          if (need_y(g)) {
            py0 = lc_get(ybox + (size_t)g * 32 * WV);
            if (WV == 2) py1 = lc_get(ybox + (size_t)g * 32 * WV + 1);
          }
          if (__all_sync(FULL, ok_y())) return true;
        } else {
          if (need_x(g)) {
            px0 = lc_get(xbox + (size_t)(g - lane) * WV);
            if (WV == 2) px1 = lc_get(xbox + (size_t)(g - lane) * WV + 1);
          }
          if (__all_sync(FULL, ok_x())) return true;
        }
        int stop = 0;
        if (lane == 0) {
          if (*(volatile int *)(a.err + 1)) {
            stop = 1;
          } else if (clock64() - t0 > a.wait_cycles) {
            atomicCAS(a.err, 0, DEV_ERR_TIMEOUT);
            atomicExch(a.err + 2, tile);
            atomicExch(a.err + 1, 1);
            stop = 1;
          }
        }
        if (__shfl_sync(FULL, stop, 0)) return false;
        if (it >= 8) {
          __nanosleep(nap);
          nap = nap < 32 ? 32 : min(nap * 2u, 256u);
        }
      }
    };
    fetch_x(0);

    const int M = (T_ + R - 1 + VW - 1) / VW;  // row R-1 reaches the last position T-1 at level T + R - 2
    for (int m = 0; m < M; ++m) {
#pragma unroll
      for (int j = 0; j < VW; ++j) {
        const int g = VW * m + j;
        // -------- 1. faces: the x face of this level (fetched last level), the y face's fetch --------
        if (!__all_sync(FULL, ok_x()) && !wait_faces(g, false)) return;  // the warp leaves; nothing in flight
        const T xv = V::from((unsigned)px0, (unsigned)px1);
        fetch_x(g + 1);
        fetch_y(g);

        // -------- 2. a row entering a vector takes the next one and loads the one after --------
#pragma unroll
        for (int r = 0; r < NR; ++r) {
          if (((j - r) & (VW - 1)) == 0) {
            const int c = (j - r + 16) / VW - 16 / VW;  // floor((j - r) / VW)
#pragma unroll
            for (int e = 0; e < VW; ++e) cur[r][e] = nxt[r][e];
            if ((rowok >> r) & 1) lc_ld(nxt[r], vaddr(r, m + c + 1));
          }
        }

        // -------- 3. the nodes of this level: rows R-1..1, then row 0 --------
        // The rows of a level do not depend on one another (row r reads row
        // r-1's value of the previous level and row r+1's old values); rows
        // R-1..1 need nothing from the tile above, row 0 needs its y face.
        // Each stage runs across the pass's rows, giving the scheduler
        // independent operations.
#pragma unroll
        for (int pass = 0; pass < 2; ++pass) {
          if (pass == 1) {
            // publish what rows R-1..1 computed: row R-1 is the next tile's y face
            if (publish) {
              const int tb = g - (R - 1);
              if (tb >= 0 && tb < T_) {
                unsigned long long *pp = ypub + (size_t)tb * 32 * WV;
                lc_put(pp, tag | V::word(res[R - 1], 0));
                if (WV == 2) lc_put(pp + 1, tag | V::word(res[R - 1], 1));
              }
            }
            if (!__all_sync(FULL, ok_y()) && !wait_faces(g, true)) return;
          }
          const T yv = V::from((unsigned)py0, (unsigned)py1);
          T cvv[R], up[R], dn[R], zdn[R], xup[R], xdn[R], gv[R];
#pragma unroll
          for (int r = 0; r < R; ++r) {
            if ((pass == 0) == (r == 0)) continue;
            const int p = (j - r) & (VW - 1);  // t mod VW
            const int pn = (p + 1) & (VW - 1);
            const int e = SZ > 0 ? p : VW - 1 - p, en = SZ > 0 ? pn : VW - 1 - pn;
            // row r+1 sits one position behind: its next position is our t
            const int p1 = (j - r - 1) & (VW - 1);
            const int pn1 = (p1 + 1) & (VW - 1);
            const int en1 = SZ > 0 ? pn1 : VW - 1 - pn1;
            cvv[r] = cur[r][e];
            zdn[r] = p < VW - 1 ? cur[r][en] : nxt[r][en];
            dn[r] = p1 < VW - 1 ? cur[r + 1][en1] : nxt[r + 1][en1];
            up[r] = r == 0 ? yv : res[r - 1];
          }
#pragma unroll
          for (int r = 0; r < R; ++r) {
            if ((pass == 0) == (r == 0)) continue;
            xup[r] = __shfl_up_sync(FULL, up[r], 1);
          }
#pragma unroll
          for (int r = 0; r < R; ++r) {
            if ((pass == 0) == (r == 0)) continue;
            const T xl = __shfl_sync(FULL, xv, r);
            if (lane == 0) xup[r] = xl;
          }
#pragma unroll
          for (int r = 0; r < R; ++r) {
            if ((pass == 0) == (r == 0)) continue;
            xdn[r] = __shfl_down_sync(FULL, dn[r], 1);
          }
#pragma unroll
          for (int r = 0; r < R; ++r) {
            if ((pass == 0) == (r == 0)) continue;
            const T m0 = lc_min<T>(V::absv(xup[r]), V::absv(xdn[r]), fx);
            const T m1 = lc_min<T>(V::absv(up[r]), V::absv(dn[r]), fy);
            const T m2 = lc_min<T>(V::absv(res[r]), V::absv(zdn[r]), SZ > 0);
            gv[r] = lc_godunov<T, ISO>(m0, m1, m2, k32);
          }
#pragma unroll
          for (int r = 0; r < R; ++r) {
            if ((pass == 0) == (r == 0)) continue;
            const int p = (j - r) & (VW - 1);
            const int c = (j - r + 16) / VW - 16 / VW;  // vector of t, relative to m
            const int e = SZ > 0 ? p : VW - 1 - p;
            const T cv = cvv[r];
            const int t = g - r;
            if constexpr (BLK || MODE == MODE_REPLACE) {
              // entering an 8^3 block: z == 1 (mod 8) going up, z == 0 (mod 8)
              // going down (the column's padding puts z = 8 ceil(nz/8) on the path)
              if (((t - (SZ > 0 ? 1 : 7)) & 7) == 0) {
                const int z = SZ > 0 ? t : a.q_last - kLcZ0 - t;
                const int bz = (z - 1) >> 3;
                const int nb = (bz >= 0 && bz < a.nbz && bxy[r] >= 0) ? bz * a.nby * a.nbx + bxy[r] : -1;
                if constexpr (BLK) {
                  // the change of the block the row leaves: the lanes of a row
                  // that share a block form one contiguous run (both block
                  // coordinates are monotone in the lane), reduced in-warp
                  if (a.blk_chg && __any_sync(FULL, bch[r] > 0.0f)) {
                    const int key = lane < kLcLanes ? bcur[r] : -1;
                    float mv = bch[r];
#pragma unroll
                    for (int off = 1; off < 32; off <<= 1) {
                      const float ov = __shfl_down_sync(FULL, mv, off);
                      const int ko = __shfl_down_sync(FULL, key, off);
                      if (lane + off < 32 && ko == key) mv = fmaxf(mv, ov);
                    }
                    const int kp = __shfl_up_sync(FULL, key, 1);
                    if (key >= 0 && mv > 0.0f && (lane == 0 || kp != key))
                      atomicMax(a.blk_chg + key, __float_as_uint(mv));
                  }
                  bch[r] = 0.0f;
                }
                bcur[r] = nb;
                if constexpr (MODE == MODE_REPLACE) bnd[r] = nb >= 0 ? __ldg(a.bcap32 + nb) : -INFINITY;
              }
            }
            T nv;
            if constexpr (MODE == MODE_MIN) {
              if constexpr (sizeof(T) == 4)
                nv = fminf(cv, gv[r]);  // frozen values are negative: they stay
              else
                nv = V::frozen(cv) ? cv : pmin(cv, gv[r]);
            } else {
              if (V::frozen(cv)) {
                nv = cv;
              } else if (CapBound<T, ARITH>::below(gv[r], bnd[r])) {
                nv = gv[r];
              } else {
                const long long q = SZ > 0 ? (long long)kLcZ0 + t : (long long)a.q_last - t;
                nv = pmin(cap_value<T, ARITH>(reinterpret_cast<const T *>(a.cap) + (ubase - u) + (r * ys32 + (int)q)),
                          gv[r]);
              }
            }
            if constexpr (BLK) {
              if (a.blk_active && !(bcur[r] >= 0 && __ldg(a.blk_active + bcur[r]))) nv = cv;
            }
            const bool changed = vdiffers<T, ARITH>(nv, cv);
            if (changed) {
              const T d = node_change<T, ARITH>(cv, nv, hmin);
              tmx[r] = vmax_nonneg<T, ARITH>(tmx[r], d);
              if constexpr (BLK) bch[r] = fmaxf(bch[r], change_f<T, ARITH>(d));
            }
            chg[r] = chg[r] || changed;
            cur[r][e] = nv;
            res[r] = nv;
            // leaving the vector: write it back if one of its nodes changed
            if (p == VW - 1) {
              if (chg[r] && lane < kLcLanes) lc_st(vaddr(r, m + c), cur[r]);
              chg[r] = false;
            }
            // lane 30's value is the next tile's x face
            if (publish && lane == kLcLanes - 1 && t >= 0 && t < T_) {
              unsigned long long *pp = xpub + ((size_t)r * T_ + t) * WV;
              lc_put(pp, tag | V::word(nv, 0));
              if (WV == 2) lc_put(pp + 1, tag | V::word(nv, 1));
            }
          }
        }
      }
    }
    if constexpr (BLK) {  // the blocks the rows end in
      if (a.blk_chg) {
#pragma unroll
        for (int r = 0; r < R; ++r)
          if (lane < kLcLanes && bcur[r] >= 0 && bch[r] > 0.0f) atomicMax(a.blk_chg + bcur[r], __float_as_uint(bch[r]));
      }
    }
  }
  // the warp's max change -> the grid's counter (lane 31 only copies the next tile's column)
  T tmax = tmx[0];
#pragma unroll
  for (int r = 1; r < R; ++r) tmax = vmax_nonneg<T, ARITH>(tmax, tmx[r]);
  T v = lane < kLcLanes ? tmax : T(0);
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v = vmax_nonneg<T, ARITH>(v, __shfl_xor_sync(FULL, v, off));
  if (lane == 0 && change_pos<T, ARITH>(v)) {
    if constexpr (sizeof(T) == 4)
      atomicMax(reinterpret_cast<unsigned int *>(a.maxchg), __float_as_uint(v));
    else
      atomicMax(reinterpret_cast<unsigned long long *>(a.maxchg), change_u64<T, ARITH>(v));
  }
}

// Launch of one variant: persistent warps (four per block) over the tiles.
template <class T, int R, int MODE, bool ISO, int SZ, bool BLK>
cudaError_t launch_lc_t(const LcArgs &a, int sms, cudaStream_t st, int *grid_used) {
  auto kern = lc_sweep_kernel<T, R, MODE, ISO, SZ, BLK>;
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 128, 0);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  const int ntiles = a.ntx * a.nty;
  int grid = per_sm * sms < (ntiles + 3) / 4 ? per_sm * sms : (ntiles + 3) / 4;
  if (grid < 1) grid = 1;
  kern<<<grid, 128, 0, st>>>(a);
  if (grid_used) *grid_used = grid;
  return cudaGetLastError();
}

// The variant of a sweep: z direction, isotropy and block bookkeeping.
template <class T, int R, int MODE>
cudaError_t launch_lc_dir(bool iso, bool blk, const LcArgs &a, int sms, cudaStream_t st, int *g) {
  if (a.sz > 0) {
    if (blk)
      return iso ? launch_lc_t<T, R, MODE, true, 1, true>(a, sms, st, g)
                 : launch_lc_t<T, R, MODE, false, 1, true>(a, sms, st, g);
    return iso ? launch_lc_t<T, R, MODE, true, 1, false>(a, sms, st, g)
               : launch_lc_t<T, R, MODE, false, 1, false>(a, sms, st, g);
  }
  if (blk)
    return iso ? launch_lc_t<T, R, MODE, true, -1, true>(a, sms, st, g)
               : launch_lc_t<T, R, MODE, false, -1, true>(a, sms, st, g);
  return iso ? launch_lc_t<T, R, MODE, true, -1, false>(a, sms, st, g)
             : launch_lc_t<T, R, MODE, false, -1, false>(a, sms, st, g);
}

}  // namespace pdfs
