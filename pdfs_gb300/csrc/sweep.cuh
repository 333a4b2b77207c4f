// sweep.cuh -- persistent column-pipelined sweep of one FSM ordering.
//
// The reference sweeps one hyperplane x+y+z = level per kernel launch
// (single_gpu_cuda/src/phi3D_fsm.cu:161-185, mpi_openacc/src/phi3D_fsm.c:92-117):
// 8*(nx+ny+nz-2) launches per round, each touching one strided diagonal slice.
// Any topological order of an ordering's dependency DAG gives the same
// result (each node reads the new values of its three upwind neighbours and
// the old values of its three downwind ones), so this kernel uses a blocked
// order instead:
//
//   * the x-y plane is cut into TX*TY columns that run the whole z extent;
//     a CTA owns one column at a time and marches it along z in the sweep's
//     z direction;
//   * inside a column, thread (lx, ly) (coordinates in the sweep's direction)
//     updates plane lz = step - lx - ly at each step, so all TX*TY threads work
//     on every step (a skewed wavefront, one __syncthreads per step);
//   * planes stream through a shared-memory ring of D slots by cp.async
//     (16-byte L2 loads), C planes per chunk, two chunks ahead;
//   * columns depend on their upwind x and y neighbours only.  Each column
//     publishes how many planes it has finished (release store); a column
//     loads a chunk only once both upwind columns have published it (acquire
//     load, bounded by wall time).  CTAs take columns from an atomic ticket in
//     wavefront order, so every column a CTA waits on is held by a CTA that is
//     already running: no deadlock, whatever the grid size.
//
// Memory layout (internal, per element type T, V = 16/sizeof(T)):
//   element (x, y, z) of the halo-padded grid (0 <= x <= nx+1, ...) lives at
//   z*plane + y*px + x + (V-1), so interior x = 1 + cx*TX starts on a 16-byte
//   boundary; px >= ncx*TX + 2V, rows ry = ncy*TY + 2, planes nz + 2.
#pragma once
#include <cstdint>

#include "godunov.cuh"

namespace pdfs {

enum { MODE_MIN = 0, MODE_REPLACE = 1 };
enum { ARITH_REF = 0, ARITH_FAST = 1 };
enum { DEV_ERR_TIMEOUT = 1 };

struct SweepArgs {
  void *u;                // working field (internal layout)
  const void *cap;        // MODE_REPLACE: upper bound per node (internal layout, same T)
  const uint32_t *fmask;  // frozen bit per node, or nullptr
  long long px;           // row pitch (elements)
  long long plane;        // plane stride (elements)
  long long fpw;          // frozen mask words per row
  long long fplane;       // frozen mask words per plane
  int nx, ny, nz;
  int sx, sy, sz;         // +1 / -1 sweep direction per axis
  int ncx, ncy;           // columns
  const int *order;       // ticket -> local column id (lcy*ncx + lcx), wavefront order
  int *progress;          // per global column id: planes finished in this sweep
  int *ticket;            // column ticket counter
  int *err;               // [0] error code, [1] abort flag, [2] column that timed out
  void *maxchg;           // FP32: uint bits of max relative change; FP64: u64 bits of max abs change
  const uint8_t *blk_active;  // per 8^3 block: visit it (nullptr = all)
  float *blk_chg;         // per 8^3 block: max change in this sweep (nullptr = not tracked)
  int nbx, nby, nbz;      // block grid
  float hmin;             // smallest spacing (relative-change floor)
  long long wait_ns;      // bound on a single inter-column wait
  int poison_col;         // test hook: this column never publishes (-1 = off)
  GodConst64 k64;
  GodConst32 k32;
};

template <class T, int TX, int TY, int C>
struct ColGeo {
  static constexpr int V = 16 / (int)sizeof(T);
  static constexpr int W = TX + 2 * V;  // smem row: x0-V .. x0+TX+V-1
  static constexpr int R = TY + 2;      // rows y0-1 .. y0+TY
  static constexpr int SK = TX + TY - 2;
  static constexpr int D = SK + 3 * C;  // ring depth (planes)
  static constexpr int ALIGN = 128 / (int)sizeof(T);
  static constexpr int SLOT = ((R * W + ALIGN - 1) / ALIGN) * ALIGN;
  static constexpr int NT = TX * TY;
  static constexpr int CAPSLOT = TX * TY;
  static size_t smem_bytes(bool with_cap) {
    size_t b = (size_t)D * SLOT * sizeof(T) + (size_t)D * TY * sizeof(uint32_t);
    b = (b + 127) & ~size_t(127);
    if (with_cap) b += (size_t)D * CAPSLOT * sizeof(T);
    return b;
  }
};

// ---- small PTX helpers -------------------------------------------------------------
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async4(void *smem, const void *gmem) {
  unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }
__device__ __forceinline__ int ld_acquire(const int *p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(int *p, int v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;\n" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
  return t;
}

// Bounded wait until progress[col] >= need.  On timeout: record the error and
// raise the abort flag so every CTA of the launch drains and returns.
static __device__ __noinline__ bool wait_progress(const SweepArgs &a, int col, int need) {
  if (col < 0 || need <= 0) return true;
  const int *p = a.progress + col;
  if (ld_acquire(p) >= need) return true;
  const unsigned long long t0 = globaltimer();
  unsigned ns = 32;
  for (;;) {
    if (ld_acquire(p) >= need) return true;
    if (*(volatile int *)(a.err + 1)) return false;
    if (globaltimer() - t0 > (unsigned long long)a.wait_ns) {
      atomicCAS(a.err, 0, DEV_ERR_TIMEOUT);
      atomicExch(a.err + 2, col);
      atomicExch(a.err + 1, 1);
      return false;
    }
    __nanosleep(ns);
    if (ns < 256) ns <<= 1;
  }
}

template <class T>
__device__ __forceinline__ T tmin(T a, T b) {  // the reference's min macro: a < b ? a : b
  return a < b ? a : b;
}

template <class T, int MODE, int ARITH, bool ISO>
__device__ __forceinline__ T local_update(T m0, T m1, T m2, const SweepArgs &a);
template <>
__device__ __forceinline__ float local_update<float, MODE_MIN, ARITH_FAST, true>(float m0, float m1, float m2,
                                                                                  const SweepArgs &a) {
  return god32<true>(m0, m1, m2, a.k32);
}
template <>
__device__ __forceinline__ float local_update<float, MODE_MIN, ARITH_FAST, false>(float m0, float m1, float m2,
                                                                                   const SweepArgs &a) {
  return god32<false>(m0, m1, m2, a.k32);
}
#define PDFS_LU64(MODE_, ARITH_, FN)                                                                  \
  template <>                                                                                         \
  __device__ __forceinline__ double local_update<double, MODE_, ARITH_, false>(double m0, double m1, \
                                                                              double m2,             \
                                                                              const SweepArgs &a) {  \
    return FN(m0, m1, m2, a.k64);                                                                     \
  }
PDFS_LU64(MODE_MIN, ARITH_REF, god_ref64)
PDFS_LU64(MODE_MIN, ARITH_FAST, god_fast64)
PDFS_LU64(MODE_REPLACE, ARITH_REF, god_ref64)
PDFS_LU64(MODE_REPLACE, ARITH_FAST, god_fast64)
#undef PDFS_LU64

template <class T, int TX, int TY, int C, int MODE, int ARITH, bool ISO>
__global__ void __launch_bounds__(TX *TY) col_sweep_kernel(const SweepArgs a) {
  using G = ColGeo<T, TX, TY, C>;
  constexpr int V = G::V, W = G::W, R = G::R, SK = G::SK, D = G::D, SLOT = G::SLOT, NT = G::NT;
  constexpr int NV = W / V;  // 16-byte vectors per smem row
  extern __shared__ __align__(128) unsigned char smem_raw[];
  T *ring = reinterpret_cast<T *>(smem_raw);
  uint32_t *fring = reinterpret_cast<uint32_t *>(ring + (size_t)D * SLOT);
  T *cring = reinterpret_cast<T *>(smem_raw + ((((size_t)D * SLOT * sizeof(T) + (size_t)D * TY * 4) + 127) & ~size_t(127)));
  __shared__ int s_ticket;
  __shared__ int s_stop;      // written by thread 0 before the ticket barrier
  __shared__ int s_stopk[2];  // per chunk parity: a slot is rewritten only two chunks later
  __shared__ T s_red[NT / 32];

  T *__restrict__ u = reinterpret_cast<T *>(a.u);
  const T *__restrict__ capg = reinterpret_cast<const T *>(a.cap);
  const int tid = threadIdx.x;
  const int gxo = tid % TX, gyo = tid / TX;  // position in global orientation
  const int lx = a.sx > 0 ? gxo : TX - 1 - gxo;
  const int ly = a.sy > 0 ? gyo : TY - 1 - gyo;
  const int skew = lx + ly;
  const int ncol = a.ncx * a.ncy;
  const int nz = a.nz;
  const int nplanes = nz + 2;
  const int nsteps = nz + SK;
  const int nphase = (nsteps + C - 1) / C;
  const int o = (gyo + 1) * W + gxo + V;  // my node inside a ring slot
  // global-orientation z neighbours: local p-1 is global z-1 when sz > 0
  const int zlo = a.sz > 0 ? -1 : 1;
  T tmax = T(0);

  for (;;) {
    if (tid == 0) {
      s_ticket = atomicAdd(a.ticket, 1);
      s_stop = *(volatile int *)(a.err + 1);
    }
    __syncthreads();
    const int tk = s_ticket;
    if (tk >= ncol || s_stop) break;
    const int lc = a.order[tk];
    const int lcx = lc % a.ncx, lcy = lc / a.ncx;
    const int cx = a.sx > 0 ? lcx : a.ncx - 1 - lcx;
    const int cy = a.sy > 0 ? lcy : a.ncy - 1 - lcy;
    const int col = cy * a.ncx + cx;
    const int upx = lcx > 0 ? col - a.sx : -1;
    const int upy = lcy > 0 ? col - a.sy * a.ncx : -1;
    const int x0 = 1 + cx * TX, y0 = 1 + cy * TY;
    const bool valid = (x0 + gxo <= a.nx) && (y0 + gyo <= a.ny);
    const long long rowbase = (long long)cx * TX;  // internal x index of x0 - V

    // Issues the loads of chunk k (planes p = k*C .. k*C+C-1, p = lz + 1) once
    // the upwind columns have finished them.  Collective; false = abort.
    auto load_chunk = [&](int k) -> bool {
      const int p0 = k * C;
      if (p0 < nplanes) {
        if (tid == 0) {
          const int need = min(nz, p0 + C - 1);
          const bool ok = wait_progress(a, upx, need) && wait_progress(a, upy, need);
          s_stopk[k & 1] = ok ? 0 : 1;
        }
        __syncthreads();
        if (s_stopk[k & 1]) return false;
        for (int i = tid; i < C * R * NV; i += NT) {
          const int v = i % NV;
          const int rr = (i / NV) % R;
          const int p = p0 + i / (NV * R);
          if (p < nplanes) {
            const int gz = a.sz > 0 ? p : nz + 1 - p;
            const T *src = u + (long long)gz * a.plane + (long long)(y0 - 1 + rr) * a.px + rowbase + v * V;
            cp_async16(ring + (p % D) * SLOT + rr * W + v * V, src);
          }
        }
        if (a.fmask) {
          for (int i = tid; i < C * TY; i += NT) {
            const int p = p0 + i / TY, r = i % TY;
            if (p < nplanes) {
              const int gz = a.sz > 0 ? p : nz + 1 - p;
              cp_async4(fring + (p % D) * TY + r,
                        a.fmask + (long long)gz * a.fplane + (long long)(y0 + r) * a.fpw + (x0 - 1) / 32);
            }
          }
        }
        if (MODE == MODE_REPLACE) {
          constexpr int CV = TX / V;
          for (int i = tid; i < C * TY * CV; i += NT) {
            const int v = i % CV;
            const int r = (i / CV) % TY;
            const int p = p0 + i / (CV * TY);
            if (p < nplanes) {
              const int gz = a.sz > 0 ? p : nz + 1 - p;
              const T *src = capg + (long long)gz * a.plane + (long long)(y0 + r) * a.px + rowbase + V + v * V;
              cp_async16(cring + (p % D) * G::CAPSLOT + r * TX + v * V, src);
            }
          }
        }
      }
      cp_async_commit();
      return true;
    };

    bool ok = load_chunk(0) && load_chunk(1);
    for (int k = 0; ok && k < nphase; ++k) {
      if (!load_chunk(k + 2)) {
        ok = false;
        break;
      }
      cp_async_wait<1>();
      __syncthreads();
#pragma unroll
      for (int s = 0; s < C; ++s) {
        const int lz = k * C + s - skew;
        if (valid && lz >= 0 && lz < nz) {
          const int p = lz + 1;
          T *sl = ring + (p % D) * SLOT;
          const T c = sl[o];
          bool frz = false;
          if (a.fmask) frz = (fring[(p % D) * TY + gyo] >> ((x0 - 1 + gxo) & 31)) & 1u;
          if (!frz) {
            const T *zl = ring + ((p + zlo) % D) * SLOT;  // global z-1
            const T *zh = ring + ((p - zlo) % D) * SLOT;  // global z+1
            const T m0 = tmin(sl[o - 1], sl[o + 1]);
            const T m1 = tmin(sl[o - W], sl[o + W]);
            const T m2 = tmin(zl[o], zh[o]);
            const T g = local_update<T, MODE, ARITH, ISO>(m0, m1, m2, a);
            T nv;
            if (MODE == MODE_REPLACE)
              nv = tmin(cring[(p % D) * G::CAPSLOT + gyo * TX + gxo], g);
            else
              nv = tmin(c, g);
            if (nv != c) {
              sl[o] = nv;
              T d;
              if (sizeof(T) == 4)
                d = (T)(fabsf((float)c - (float)nv) / fmaxf((float)nv, a.hmin));
              else
                d = (T)fabs((double)c - (double)nv);
              tmax = fmax(tmax, d);
            }
          }
        }
        __syncthreads();
      }
      // planes lz in [kC-SK, kC+C-SK) are now complete: write my nodes back
#pragma unroll
      for (int j = 0; j < C; ++j) {
        const int lz = k * C - SK + j;
        if (valid && lz >= 0 && lz < nz) {
          const int p = lz + 1;
          const int gz = a.sz > 0 ? p : nz + 1 - p;
          u[(long long)gz * a.plane + (long long)(y0 + gyo) * a.px + rowbase + V + gxo] =
              ring[(p % D) * SLOT + o];
        }
      }
      __syncthreads();
      if (tid == 0) {
        __threadfence();
        if (col != a.poison_col) st_release(a.progress + col, max(0, min(nz, k * C + C - SK)));
      }
    }
    cp_async_wait_all();
    __syncthreads();
    if (!ok) break;
  }

  // CTA max-change reduction -> one atomic per CTA
  T v = tmax;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, off));
  if ((tid & 31) == 0) s_red[tid >> 5] = v;
  __syncthreads();
  if (tid == 0) {
    T m = s_red[0];
    for (int w = 1; w < NT / 32; ++w) m = fmax(m, s_red[w]);
    if (m > T(0)) {
      if (sizeof(T) == 4)
        atomicMax(reinterpret_cast<unsigned int *>(a.maxchg), __float_as_uint((float)m));
      else
        atomicMax(reinterpret_cast<unsigned long long *>(a.maxchg),
                  (unsigned long long)__double_as_longlong((double)m));
    }
  }
}

}  // namespace pdfs
