// mlp.cu -- the learned active-block scheduler: features, the fused
// inference on the tensor cores (tcgen05 MMAs into TMEM), the bf16 training
// kernels (forward, backward, Adam) with FP32 accumulation, and the trainer
// that learns from plain-sweep traces.
//
// The reference has no scheduler: every ordering visits every node
// (single_gpu_cuda/src/phi3D_fsm.cu:144-189, mpi_openacc/src/phi3D_fsm.c:83-119).
// The network predicts, per 8^3 block, whether the next sweep changes the
// block by more than the phase's tolerance.  Skipping a block is always safe
// for the answer: a solve ends only on a sweep that visits every block and
// stays within the tolerance (solver.cu).
//
// Arithmetic of the network (shared by training and inference):
//   x  = bf16(features)
//   h1 = bf16(relu(W1 x + b1)),  h2 = bf16(relu(W2 h1 + b2)),  z = w3 . h2 + b3
// with bf16 weights and every dot product accumulated in FP32.  Training
// minimises the mean weighted binary cross-entropy of z against the label
// (positives weigh pos_weight) with Adam on FP32 master weights.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <random>
#include <vector>

#include "internal.h"

namespace pdfs {
namespace {

constexpr int NI = PDFS_MLP_IN, NH = PDFS_MLP_HIDDEN, NP = PDFS_MLP_PARAMS;
// parameter offsets
constexpr int OW1 = 0, OB1 = OW1 + NH * NI, OW2 = OB1 + NH, OB2 = OW2 + NH * NH, OW3 = OB2 + NH, OB3 = OW3 + NH;
static_assert(OB3 + 1 == NP, "parameter layout");
constexpr int TB = 128;  // training samples per CTA

__device__ __forceinline__ float bfr(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }
__device__ __forceinline__ float bf2f(uint16_t b) { return __uint_as_float((unsigned)b << 16); }
__device__ __forceinline__ uint16_t f2bf(float v) {
  const __nv_bfloat16 h = __float2bfloat16_rn(v);
  return *reinterpret_cast<const uint16_t *>(&h);
}

// Weights of one network as floats in shared memory (all bf16 values).
__device__ __forceinline__ void load_weights(float *sw, const uint16_t *__restrict__ w) {
  for (int i = threadIdx.x; i < NP; i += blockDim.x) sw[i] = bf2f(w[i]);
}

// Forward pass of one sample; h1 (bf16 values) is kept for the backward
// pass, h2 goes to h2_out when given and its positive entries to *mask.
__device__ __forceinline__ float mlp_forward(const float *sw, const float x[NI], float h1[NH], float *h2_out,
                                             unsigned long long *mask) {
#pragma unroll
  for (int j = 0; j < NH; ++j) {
    float acc = sw[OB1 + j];
#pragma unroll
    for (int k = 0; k < NI; ++k) acc = fmaf(sw[OW1 + j * NI + k], x[k], acc);
    h1[j] = bfr(fmaxf(acc, 0.0f));
  }
  float z = sw[OB3];
  unsigned long long m = 0;
#pragma unroll 1
  for (int j = 0; j < NH; ++j) {
    float acc = sw[OB2 + j];
#pragma unroll
    for (int k = 0; k < NH; ++k) acc = fmaf(sw[OW2 + j * NH + k], h1[k], acc);
    const float h2 = bfr(fmaxf(acc, 0.0f));
    if (h2 > 0.0f) m |= 1ull << j;
    if (h2_out) h2_out[j] = h2;
    z = fmaf(sw[OW3 + j], h2, z);
  }
  if (mask) *mask = m;
  return z;
}

// ---- features ----------------------------------------------------------------------
struct FeatArgs {
  const unsigned int *ring;     // float bits of block max changes, kRing slots of nb (see internal.h)
  long long nb;
  int cur, hist;                // slot of the upcoming sweep; sweeps of history
  const float *bmin;            // per block: min of the field
  int nbx, nby, nbz;
  int sx, sy, sz, sn;           // upcoming ordering
  int sweep, phase;
  float tol, hband;             // phase tolerance; 8 * smallest spacing
};

__device__ __forceinline__ float lchg(float c, float tol) {
  if (!(c > 0.0f)) return -2.0f;
  return fminf(fmaxf(__log2f(c / tol), -32.0f), 32.0f) * (1.0f / 16.0f);
}

// Change of block i k sweeps ago (0 beyond the recorded history).
__device__ __forceinline__ float hist_chg(const FeatArgs &f, int k, long long i) {
  if (k > f.hist) return 0.0f;
  return __uint_as_float(f.ring[(size_t)((f.cur - k + kRing) % kRing) * f.nb + i]);
}

__device__ __forceinline__ void block_features(const FeatArgs &f, long long b, float x[NI]) {
  const int bx = (int)(b % f.nbx), by = (int)((b / f.nbx) % f.nby), bz = (int)(b / ((long long)f.nbx * f.nby));
  const long long sxs = 1, sys = f.nbx, szs = (long long)f.nbx * f.nby;
  const float c1 = hist_chg(f, 1, b), c2 = hist_chg(f, 2, b), c8 = hist_chg(f, kHist, b);
  int age = kHist + 1;  // sweeps since the block last changed by more than tol
  for (int k = kHist; k >= 1; --k)
    if (hist_chg(f, k, b) > f.tol) age = k;
  // face neighbours upwind of the block in this ordering lie at -s
  float up = 0.0f;
  const int ux = bx - f.sx, uy = by - f.sy, uz = bz - f.sz;
  if (ux >= 0 && ux < f.nbx) up = fmaxf(up, hist_chg(f, 1, b - f.sx * sxs));
  if (uy >= 0 && uy < f.nby) up = fmaxf(up, hist_chg(f, 1, b - f.sy * sys));
  if (uz >= 0 && uz < f.nbz) up = fmaxf(up, hist_chg(f, 1, b - f.sz * szs));
  const float band = fminf(fmaxf(f.bmin[b], 0.0f) / f.hband, 1073741824.0f);
  x[0] = __log2f(1.0f + band) * 0.125f;
  x[1] = lchg(c1, f.tol);
  x[2] = lchg(c2, f.tol);
  x[3] = (float)age * (1.0f / (kHist + 1));
  x[4] = (float)f.phase;
  x[5] = (float)min(f.sweep, 64) * (1.0f / 64.0f);
#pragma unroll
  for (int k = 0; k < 8; ++k) x[6 + k] = (k == f.sn - 1) ? 1.0f : 0.0f;
  x[14] = lchg(up, f.tol);
  x[15] = lchg(c8, f.tol);
#pragma unroll
  for (int k = 0; k < NI; ++k) x[k] = bfr(x[k]);
}

// The history rule of the change scheduler (sched.cu): the block changed by
// more than tol within the recorded history, or a face neighbour did in the
// last sweep.  Blocks outside it have, in practice, settled.
__device__ __forceinline__ bool history_rule(const FeatArgs &f, long long b) {
  for (int k = 1; k <= f.hist; ++k)
    if (hist_chg(f, k, b) > f.tol) return true;
  const int bx = (int)(b % f.nbx), by = (int)((b / f.nbx) % f.nby), bz = (int)(b / ((long long)f.nbx * f.nby));
  const long long sys = f.nbx, szs = (long long)f.nbx * f.nby;
  return (bx > 0 && hist_chg(f, 1, b - 1) > f.tol) || (bx < f.nbx - 1 && hist_chg(f, 1, b + 1) > f.tol) ||
         (by > 0 && hist_chg(f, 1, b - sys) > f.tol) || (by < f.nby - 1 && hist_chg(f, 1, b + sys) > f.tol) ||
         (bz > 0 && hist_chg(f, 1, b - szs) > f.tol) || (bz < f.nbz - 1 && hist_chg(f, 1, b + szs) > f.tol);
}

// Per-block minimum of a working field (interior nodes): one warp covers
// four blocks along x, lane = node x offset.
template <class T, bool PAIR = false>
__global__ void k_block_min(const T *__restrict__ u, Layout L, int nx, int ny, int nz, int nbx, int nby, int nbz,
                            float *__restrict__ bmin) {
  const long long wid = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int nwx = (nbx + 3) / 4;
  if (wid >= (long long)nwx * nby * nbz) return;
  const int wx = (int)(wid % nwx), by = (int)((wid / nwx) % nby), bz = (int)(wid / ((long long)nwx * nby));
  const int x = 1 + wx * 32 + lane;
  float m = INFINITY;
  if (x <= nx) {
    for (int z = 1 + bz * 8; z <= min(nz, bz * 8 + 8); ++z)
      for (int y = 1 + by * 8; y <= min(ny, by * 8 + 8); ++y) {
        const T v = u[L.index(x, y, z)];
        float f;
        if constexpr (PAIR)
          f = p_hi(v);
        else
          f = (float)v;
        m = fminf(m, fabsf(f));  // z-column fields mark frozen nodes with the sign
      }
  }
#pragma unroll
  for (int off = 1; off < 8; off <<= 1) m = fminf(m, __shfl_xor_sync(0xffffffffu, m, off));
  const int bx = wx * 4 + (lane >> 3);
  if ((lane & 7) == 0 && bx < nbx) bmin[((long long)bz * nby + by) * nbx + bx] = m;
}

// Trace recording, before a sweep: the features (bf16) of every block the
// history rule nominates -- the blocks the network decides about.
__global__ void k_features(FeatArgs f, uint16_t *__restrict__ xout, uint8_t *__restrict__ cand) {
  const long long n = (long long)f.nbx * f.nby * f.nbz;
  for (long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x; b < n; b += (long long)gridDim.x * blockDim.x) {
    const bool c = history_rule(f, b);
    cand[b] = c ? 1 : 0;
    if (!c) continue;
    float x[NI];
    block_features(f, b, x);
#pragma unroll
    for (int k = 0; k < NI; ++k) xout[b * NI + k] = f2bf(x[k]);
  }
}

// After the sweep: append (features, change > tol) of the nominated blocks
// to the sample store (order is irrelevant: training shuffles).
__global__ void k_append(const uint16_t *__restrict__ xin, const uint8_t *__restrict__ cand,
                         const unsigned int *__restrict__ chg, long long n, float tol, uint16_t *__restrict__ xs,
                         uint8_t *__restrict__ ys, unsigned long long *__restrict__ count) {
  for (long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x; b < n; b += (long long)gridDim.x * blockDim.x) {
    if (!cand[b]) continue;
    const unsigned long long i = atomicAdd(count, 1ull);
#pragma unroll
    for (int k = 0; k < NI; ++k) xs[i * NI + k] = xin[b * NI + k];
    ys[i] = __uint_as_float(chg[b]) > tol ? 1 : 0;
  }
}

// ---- fused inference on the tensor cores (tcgen05, accumulators in TMEM) ---------------
// A persistent loop over tiles of 128 rows (blocks, or given samples).  Row r
// of a tile belongs to thread r: it writes its 16 bf16 features into the A
// tile, reads its row of each accumulator back from TMEM (warp w owns TMEM
// lanes 32w..32w+31) and finishes the 64 -> 1 output layer on the CUDA cores.
//   layer 1: D1[128 x 64] = X[128 x 16] W1^T    one K = 16 MMA
//   layer 2: D2[128 x 64] = H1[128 x 64] W2^T   four K = 16 MMAs
// Operands are bf16 in the canonical K-major layout without swizzle: core
// matrices of 8 rows x 16 bytes (rows contiguous), 128 bytes apart along K
// (leading byte offset) and 16 K bytes apart along M / N (stride byte offset).
// Accumulation is FP32; h1 is rounded to bf16 on its way back to shared
// memory, as in the training kernels.
namespace tc {
constexpr int TM = 128;              // rows per tile (the MMA's M)
constexpr uint32_t TMEM_COLS = 128;  // D1 in columns 0..63, D2 in 64..127
constexpr size_t OFF_B1 = 0, OFF_B2 = OFF_B1 + NH * NI * 2, OFF_A1 = OFF_B2 + NH * NH * 2,
                 OFF_A2 = OFF_A1 + TM * NI * 2, OFF_P = OFF_A2 + TM * NH * 2;
constexpr size_t SMEM = OFF_P + (3 * NH + 1) * 4;
// requested dynamic shared memory: at most 3 CTAs per SM, so their TMEM
// allocations (3 x 128 of 512 columns) never wait on each other
constexpr size_t SMEM_ALLOC = 64 * 1024;
static_assert(SMEM <= SMEM_ALLOC, "tile layout");
// kind::f16 instruction descriptor: D FP32 (bits 4-5), A and B bf16 (bits
// 7-9, 10-12), both K-major, N / 8 at bits 17-22, M / 16 at bits 24-28
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(NH >> 3) << 17) |
                           ((uint32_t)(TM >> 4) << 24);
}  // namespace tc

// Byte offset of element (row, k) of a K-major operand with K columns.
__device__ __forceinline__ uint32_t kmaj(int row, int k, int K) {
  return (uint32_t)((row >> 3) * (16 * K) + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}
// Shared-memory matrix descriptor: start, leading and stride byte offsets
// (each >> 4, 14 bits), descriptor version 1 at bit 46, no swizzle.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr_, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr_ >> 4) & 0x3fffu) | ((uint64_t)((lbo >> 4) & 0x3fffu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3fffu) << 32) | (1ull << 46);
}
__device__ __forceinline__ void tc_mma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, int accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void tc_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(saddr(bar))
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
// 16 consecutive accumulator columns of this thread's TMEM lane; the wait is
// in the same statement so no use of the registers can move above it.
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float v[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];\n"
      "tcgen05.wait::ld.sync.aligned;\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
// Bounded wait on an mbarrier phase (SM cycles).
__device__ __forceinline__ bool tc_wait(uint64_t *bar, uint32_t parity) {
  const long long t0 = clock64();
  while (!mbar_try(bar, parity))
    if (clock64() - t0 > 4000000000ll) return false;
  return true;
}

// SCHED: rows are the grid's blocks -- features, history rule, network and
// decision (active[b], *count += actives).  Otherwise rows are the samples
// xin[n][16] and the logits go to out.  *err is set if an accumulator wait
// ever gives up (the CTA then stops and frees its TMEM).
template <bool SCHED>
__global__ void __launch_bounds__(128) k_mlp_tc(const uint16_t *__restrict__ w, float thr, FeatArgs f,
                                                const uint16_t *__restrict__ xin, long long n,
                                                uint8_t *__restrict__ active, int *__restrict__ count,
                                                float *__restrict__ out, int *__restrict__ err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ uint64_t bar;
  __shared__ uint32_t s_tmem;
  const int tid = threadIdx.x, warp = tid >> 5;
  unsigned char *B1 = sm + tc::OFF_B1, *B2 = sm + tc::OFF_B2, *A1 = sm + tc::OFF_A1, *A2 = sm + tc::OFF_A2;
  float *pb = reinterpret_cast<float *>(sm + tc::OFF_P);  // b1 | b2 | w3 | b3
  for (int i = tid; i < NH * NI; i += blockDim.x) *reinterpret_cast<uint16_t *>(B1 + kmaj(i / NI, i % NI, NI)) = w[OW1 + i];
  for (int i = tid; i < NH * NH; i += blockDim.x) *reinterpret_cast<uint16_t *>(B2 + kmaj(i / NH, i % NH, NH)) = w[OW2 + i];
  for (int i = tid; i < NH; i += blockDim.x) {
    pb[i] = bf2f(w[OB1 + i]);
    pb[NH + i] = bf2f(w[OB2 + i]);
    pb[2 * NH + i] = bf2f(w[OW3 + i]);
  }
  if (tid == 0) {
    pb[3 * NH] = bf2f(w[OB3]);
    mbar_init(&bar, 1);
    mbar_fence_init();
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(saddr(&s_tmem)),
                 "r"(tc::TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  fence_proxy_async();  // the weight tiles, written by threads, are read by the tensor cores
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = s_tmem;
  const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
  uint32_t par = 0;
  int local = 0;
  bool failed = false;
  for (long long base = (long long)blockIdx.x * tc::TM; base < n; base += (long long)gridDim.x * tc::TM) {
    const long long b = base + tid;
    const bool valid = b < n;
    float x[NI];
    bool rule = false;
#pragma unroll
    for (int k = 0; k < NI; ++k) x[k] = 0.0f;
    if (valid) {
      if (SCHED) {
        rule = history_rule(f, b);
        block_features(f, b, x);
      } else {
#pragma unroll
        for (int k = 0; k < NI; ++k) x[k] = bf2f(xin[b * NI + k]);
      }
    }
#pragma unroll
    for (int k = 0; k < NI; ++k) *reinterpret_cast<uint16_t *>(A1 + kmaj(tid, k, NI)) = f2bf(x[k]);
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
      tc_mma(tmem, sdesc(saddr(A1), 128, 16 * NI), sdesc(saddr(B1), 128, 16 * NI), tc::IDESC, 0);
      tc_commit(&bar);
    }
    if (__syncthreads_or(!tc_wait(&bar, par))) {
      failed = true;
      break;
    }
    par ^= 1;
    tc_fence_after();
    // h1 = bf16(relu(D1 + b1)) -> row tid of the layer-2 operand
#pragma unroll
    for (int c = 0; c < NH; c += 16) {
      float v[16];
      tc_ld16(tmem + lane_base + c, v);
#pragma unroll
      for (int i = 0; i < 16; ++i)
        *reinterpret_cast<uint16_t *>(A2 + kmaj(tid, c + i, NH)) = f2bf(fmaxf(v[i] + pb[c + i], 0.0f));
    }
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
#pragma unroll
      for (int kk = 0; kk < NH / 16; ++kk)
        tc_mma(tmem + NH, sdesc(saddr(A2) + kk * 256, 128, 16 * NH), sdesc(saddr(B2) + kk * 256, 128, 16 * NH),
               tc::IDESC, kk > 0);
      tc_commit(&bar);
    }
    if (__syncthreads_or(!tc_wait(&bar, par))) {
      failed = true;
      break;
    }
    par ^= 1;
    tc_fence_after();
    float z = pb[3 * NH];
#pragma unroll
    for (int c = 0; c < NH; c += 16) {
      float v[16];
      tc_ld16(tmem + lane_base + NH + c, v);
#pragma unroll
      for (int i = 0; i < 16; ++i) z = fmaf(pb[2 * NH + c + i], bfr(fmaxf(v[i] + pb[NH + c + i], 0.0f)), z);
    }
    if (SCHED) {
      const bool on = valid && rule && z > thr;
      if (valid) active[b] = on ? 1 : 0;
      local += on ? 1 : 0;
    } else if (valid) {
      out[b] = z;
    }
    tc_fence_before();
    __syncthreads();  // the next tile overwrites the operand tiles and the accumulators
  }
  if (SCHED) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) local += __shfl_xor_sync(0xffffffffu, local, off);
    if ((tid & 31) == 0 && local) atomicAdd(count, local);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(tc::TMEM_COLS) : "memory");
  if (failed && tid == 0) atomicExch(err, 1);
}

// ---- training ----------------------------------------------------------------------
// Sample order of an epoch: i -> (a*i + c) mod n with gcd(a, n) = 1.
struct Perm {
  unsigned long long a, c, n;
  __device__ __forceinline__ long long at(long long i) const { return (long long)((a * (unsigned long long)i + c) % n); }
};

// Shared memory of k_train: weights (floats), then per sample x, h1, h2,
// dh1 (bf16) and dz (float).
constexpr size_t TRAIN_SMEM = (size_t)((NP + 3) & ~3) * 4 + (size_t)TB * (NI + 3 * NH) * 2 + (size_t)TB * 4;

// One mini-batch slice of TB samples per CTA: forward, backward, and the
// CTA's share of the weight gradient (FP32 sums), added into grad.  dz is
// pre-divided by the mini-batch size so grad is the mean's gradient.
__global__ void __launch_bounds__(TB) k_train(const uint16_t *__restrict__ w, const uint16_t *__restrict__ xs,
                                              const uint8_t *__restrict__ ys, Perm perm, long long first,
                                              int batch, float pos_weight, float *__restrict__ grad,
                                              float *__restrict__ loss_sum) {
  extern __shared__ __align__(16) unsigned char smem[];
  float *sw = reinterpret_cast<float *>(smem);
  uint16_t *sx = reinterpret_cast<uint16_t *>(smem + (size_t)((NP + 3) & ~3) * 4);
  uint16_t *sh1 = sx + TB * NI;
  uint16_t *sh2 = sh1 + TB * NH;
  uint16_t *sdh1 = sh2 + TB * NH;
  float *sdz = reinterpret_cast<float *>(sdh1 + TB * NH);
  load_weights(sw, w);
  __syncthreads();

  const int t = threadIdx.x;
  const long long i = (long long)blockIdx.x * TB + t;  // position in the mini-batch
  const float inv_b = 1.0f / (float)batch;
  float loss = 0.0f;
  if (i < batch) {
    const long long idx = perm.at(first + i);
    float x[NI], h1[NH], h2[NH];
#pragma unroll
    for (int k = 0; k < NI; ++k) x[k] = bf2f(xs[idx * NI + k]);
    unsigned long long mask;
    const float z = mlp_forward(sw, x, h1, h2, &mask);
    const float y = ys[idx] ? 1.0f : 0.0f;
    const float wy = ys[idx] ? pos_weight : 1.0f;
    const float p = 1.0f / (1.0f + __expf(-z));
    loss = wy * (fmaxf(z, 0.0f) - z * y + log1pf(__expf(-fabsf(z)))) * inv_b;
    const float dz = wy * (p - y) * inv_b;
    // dh1[k] = [h1_k > 0] sum_j [h2_j > 0] w3_j dz W2[j][k]
    for (int k = 0; k < NH; ++k) {
      float acc = 0.0f;
      if (h1[k] > 0.0f) {
        unsigned long long m = mask;
        while (m) {
          const int j = __ffsll((long long)m) - 1;
          m &= m - 1;
          acc = fmaf(sw[OW3 + j], sw[OW2 + j * NH + k], acc);
        }
      }
      sdh1[t * NH + k] = f2bf(acc * dz);
    }
#pragma unroll
    for (int k = 0; k < NI; ++k) sx[t * NI + k] = f2bf(x[k]);
    for (int k = 0; k < NH; ++k) {
      sh1[t * NH + k] = f2bf(h1[k]);
      sh2[t * NH + k] = f2bf(h2[k]);
    }
    sdz[t] = dz;
  } else {
    for (int k = 0; k < NI; ++k) sx[t * NI + k] = 0;
    for (int k = 0; k < NH; ++k) sh1[t * NH + k] = sh2[t * NH + k] = sdh1[t * NH + k] = 0;
    sdz[t] = 0.0f;
  }
  __syncthreads();

  // weight gradients: thread pair (2j, 2j+1) owns output row j
  const int j = t >> 1, half = t & 1;
  const float w3j = sw[OW3 + j];
  {
    float acc[32];
#pragma unroll
    for (int k = 0; k < 32; ++k) acc[k] = 0.0f;
    float db2 = 0.0f, dw3 = 0.0f;
    for (int s = 0; s < TB; ++s) {
      const float h2 = bf2f(sh2[s * NH + j]);
      const float dz = sdz[s];
      dw3 = fmaf(dz, h2, dw3);
      if (h2 > 0.0f) {
        const float g = w3j * dz;
        db2 += g;
        const uint16_t *h1 = sh1 + s * NH + half * 32;
#pragma unroll
        for (int k = 0; k < 32; ++k) acc[k] = fmaf(g, bf2f(h1[k]), acc[k]);
      }
    }
#pragma unroll
    for (int k = 0; k < 32; ++k)
      if (acc[k] != 0.0f) atomicAdd(grad + OW2 + j * NH + half * 32 + k, acc[k]);
    if (half == 0) {
      if (db2 != 0.0f) atomicAdd(grad + OB2 + j, db2);
    } else if (dw3 != 0.0f) {
      atomicAdd(grad + OW3 + j, dw3);
    }
  }
  {
    float acc[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) acc[k] = 0.0f;
    float db1 = 0.0f;
    for (int s = 0; s < TB; ++s) {
      const float d = bf2f(sdh1[s * NH + j]);
      if (d != 0.0f) {
        db1 += d;
        const uint16_t *x = sx + s * NI + half * 8;
#pragma unroll
        for (int k = 0; k < 8; ++k) acc[k] = fmaf(d, bf2f(x[k]), acc[k]);
      }
    }
#pragma unroll
    for (int k = 0; k < 8; ++k)
      if (acc[k] != 0.0f) atomicAdd(grad + OW1 + j * NI + half * 8 + k, acc[k]);
    if (half == 0 && db1 != 0.0f) atomicAdd(grad + OB1 + j, db1);
  }
  // db3 and the loss: CTA sums
  float dzs = sdz[t];
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    dzs += __shfl_xor_sync(0xffffffffu, dzs, off);
    loss += __shfl_xor_sync(0xffffffffu, loss, off);
  }
  if ((t & 31) == 0) {
    if (dzs != 0.0f) atomicAdd(grad + OB3, dzs);
    if (loss_sum) atomicAdd(loss_sum, loss);
  }
}

// Adam on FP32 master weights; refreshes the bf16 copy and clears the gradient.
__global__ void k_adam(float *__restrict__ p, float *__restrict__ m, float *__restrict__ v, float *__restrict__ g,
                       uint16_t *__restrict__ pb, int n, float lr, float b1, float b2, float eps, float bc1, float bc2) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float pi = p[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    p[i] = pi;
    if (pb) pb[i] = f2bf(pi);
    g[i] = 0.0f;
  }
}

__global__ void k_to_bf16(const float *__restrict__ p, uint16_t *__restrict__ pb, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) pb[i] = f2bf(p[i]);
}

int cstat(cudaError_t e) {
  if (e == cudaSuccess) return PDFS_OK;
  if (e == cudaErrorMemoryAllocation) return PDFS_ERR_OOM;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return PDFS_ERR_NO_DEVICE;
  return PDFS_ERR_CUDA;
}
#define MK(call)                              \
  do {                                        \
    cudaError_t e_ = (call);                  \
    if (e_ != cudaSuccess) return cstat(e_);  \
  } while (0)

// Scoped device buffer.
template <class T>
struct DBuf {
  T *p = nullptr;
  ~DBuf() { cudaFree(p); }
  cudaError_t alloc(size_t n) {
    cudaFree(p);
    p = nullptr;
    return cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T));
  }
};

cudaError_t set_smem_attrs() {
  cudaError_t e = cudaFuncSetAttribute(k_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TRAIN_SMEM);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_mlp_tc<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc::SMEM_ALLOC);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_mlp_tc<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc::SMEM_ALLOC);
}

// Logits of n samples (bf16 features) on the tensor cores; *err as k_mlp_tc.
cudaError_t mlp_logits(const uint16_t *w, const uint16_t *x, long long n, float *out, int *err, int sms,
                       cudaStream_t st) {
  const int grid = (int)std::max<long long>(1, std::min<long long>((n + tc::TM - 1) / tc::TM, (long long)sms * 3));
  FeatArgs none;
  std::memset(&none, 0, sizeof(none));
  k_mlp_tc<false><<<grid, 128, tc::SMEM_ALLOC, st>>>(w, 0.0f, none, x, n, nullptr, nullptr, out, err);
  return cudaGetLastError();
}

// Gradient of the mean loss over n samples (in order) into grad (cleared here).
cudaError_t train_grad(const uint16_t *w, const uint16_t *x, const uint8_t *y, long long n, Perm perm,
                       long long first, int batch, float pos_weight, float *grad, float *loss, cudaStream_t st) {
  (void)n;
  const int grid = (batch + TB - 1) / TB;
  k_train<<<grid, TB, TRAIN_SMEM, st>>>(w, x, y, perm, first, batch, pos_weight, grad, loss);
  return cudaGetLastError();
}

unsigned long long gcdu(unsigned long long a, unsigned long long b) {
  while (b) {
    const unsigned long long t = a % b;
    a = b;
    b = t;
  }
  return a;
}

Perm random_perm(unsigned long long n, std::mt19937_64 &rng) {
  Perm p{1, 0, n};
  if (n <= 1) return p;
  std::uniform_int_distribution<unsigned long long> d(1, n - 1);
  do {
    p.a = d(rng);
  } while (gcdu(p.a, n) != 1);
  p.c = d(rng);
  return p;
}

}  // namespace

// ---- scheduler hook used by the solve (solver.cu) ------------------------------------
#if __has_include("mlp_default.h")
#include "mlp_default.h"  // kDefaultMlpBlob: weights trained by pdfs_gb300/train_scheduler.py
const float *default_mlp_blob() { return kDefaultMlpBlob; }
#else
const float *default_mlp_blob() { return nullptr; }
#endif

cudaError_t block_min(const void *u, int kind, const Layout &L, const pdfs_grid &g, int nbx, int nby, int nbz,
                      float *bmin, cudaStream_t st) {
  const long long warps = (long long)((nbx + 3) / 4) * nby * nbz;
  const int grid = (int)((warps * 32 + 255) / 256);
  if (kind == 0)
    k_block_min<float><<<grid, 256, 0, st>>>((const float *)u, L, g.nx, g.ny, g.nz, nbx, nby, nbz, bmin);
  else if (kind == 2)
    k_block_min<double, true><<<grid, 256, 0, st>>>((const double *)u, L, g.nx, g.ny, g.nz, nbx, nby, nbz, bmin);
  else
    k_block_min<double><<<grid, 256, 0, st>>>((const double *)u, L, g.nx, g.ny, g.nz, nbx, nby, nbz, bmin);
  return cudaGetLastError();
}

static FeatArgs feat_args(const unsigned int *ring, int cur, int hist, const float *bmin, int nbx, int nby,
                          int nbz, int sn, int sweep, int phase, float tol, float hmin) {
  FeatArgs f;
  f.ring = ring;
  f.nb = (long long)nbx * nby * nbz;
  f.cur = cur;
  f.hist = hist;
  f.bmin = bmin;
  f.nbx = nbx;
  f.nby = nby;
  f.nbz = nbz;
  ordering_signs(sn, &f.sx, &f.sy, &f.sz);
  f.sn = sn;
  f.sweep = sweep;
  f.phase = phase;
  f.tol = tol;
  f.hband = 8.0f * hmin;
  return f;
}

cudaError_t sched_learned(const uint16_t *w, float thr, const unsigned int *ring, int cur, int hist,
                          const float *bmin, int nbx, int nby, int nbz, int sn, int sweep, int phase, float tol,
                          float hmin, uint8_t *active, int *count, int *err, int sms, cudaStream_t st) {
  static bool attrs = false;
  if (!attrs) {
    cudaError_t e = set_smem_attrs();
    if (e != cudaSuccess) return e;
    attrs = true;
  }
  const FeatArgs f = feat_args(ring, cur, hist, bmin, nbx, nby, nbz, sn, sweep, phase, tol, hmin);
  const long long n = (long long)nbx * nby * nbz;
  const int grid = (int)std::max<long long>(1, std::min<long long>((n + tc::TM - 1) / tc::TM, (long long)sms * 3));
  k_mlp_tc<true><<<grid, 128, tc::SMEM_ALLOC, st>>>(w, thr, f, nullptr, n, active, count, nullptr, err);
  return cudaGetLastError();
}

}  // namespace pdfs

using namespace pdfs;

// ---- trainer ---------------------------------------------------------------------------
struct pdfs_mlp_trainer {
  int dev = 0;
  cudaStream_t st = nullptr;
  std::mt19937_64 rng;
  long long n = 0, cap = 0;  // samples collected / capacity
  uint16_t *x = nullptr;     // [cap][16] bf16 features
  uint8_t *y = nullptr;      // [cap] labels
  float *p = nullptr, *m = nullptr, *v = nullptr, *g = nullptr;  // FP32 master, Adam moments, gradient
  uint16_t *pb = nullptr;   // bf16 weights
  float *loss = nullptr;    // device loss accumulator
  unsigned long long *count = nullptr;  // device copy of n while recording
  int step = 0;
};

static int trainer_grow(pdfs_mlp_trainer *t, long long need) {
  if (t->n + need <= t->cap) return PDFS_OK;
  long long nc = std::max<long long>(t->cap * 2, t->n + need);
  nc = std::max<long long>(nc, 1 << 20);
  uint16_t *nx = nullptr;
  uint8_t *ny = nullptr;
  MK(cudaMalloc(&nx, (size_t)nc * NI * 2));
  if (cudaMalloc(&ny, (size_t)nc) != cudaSuccess) {
    cudaFree(nx);
    return PDFS_ERR_OOM;
  }
  if (t->n) {
    MK(cudaMemcpyAsync(nx, t->x, (size_t)t->n * NI * 2, cudaMemcpyDeviceToDevice, t->st));
    MK(cudaMemcpyAsync(ny, t->y, (size_t)t->n, cudaMemcpyDeviceToDevice, t->st));
    MK(cudaStreamSynchronize(t->st));
  }
  cudaFree(t->x);
  cudaFree(t->y);
  t->x = nx;
  t->y = ny;
  t->cap = nc;
  return PDFS_OK;
}

extern "C" int pdfs_mlp_trainer_create(int device, unsigned seed, pdfs_mlp_trainer **out) {
  if (!out) return PDFS_ERR_INVALID;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return PDFS_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= ndev) return PDFS_ERR_INVALID;
  MK(cudaSetDevice(device));
  MK(set_smem_attrs());
  auto *t = new pdfs_mlp_trainer();
  t->dev = device;
  t->rng.seed(seed);
  auto fail = [&](cudaError_t e) {
    pdfs_mlp_trainer_destroy(t);
    return cstat(e);
  };
  cudaError_t e;
  if ((e = cudaStreamCreateWithFlags(&t->st, cudaStreamNonBlocking)) != cudaSuccess) return fail(e);
  for (float **q : {&t->p, &t->m, &t->v, &t->g})
    if ((e = cudaMalloc(q, NP * 4)) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&t->pb, NP * 2)) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&t->loss, 4)) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&t->count, 8)) != cudaSuccess) return fail(e);
  // He-uniform initialisation of the hidden layers, small output layer
  std::vector<float> h(NP, 0.0f);
  auto fill = [&](int off, int fan_out, int fan_in, float gain) {
    const float a = gain * std::sqrt(6.0f / (float)fan_in);
    std::uniform_real_distribution<float> d(-a, a);
    for (int i = 0; i < fan_out * fan_in; ++i) h[off + i] = d(t->rng);
  };
  fill(OW1, NH, NI, 1.0f);
  fill(OW2, NH, NH, 1.0f);
  fill(OW3, 1, NH, 0.5f);
  for (float &q : h) q = __bfloat162float(__float2bfloat16_rn(q));  // start from bf16-exact values
  if ((e = cudaMemcpy(t->p, h.data(), NP * 4, cudaMemcpyHostToDevice)) != cudaSuccess) return fail(e);
  for (float *q : {t->m, t->v, t->g})
    if ((e = cudaMemset(q, 0, NP * 4)) != cudaSuccess) return fail(e);
  k_to_bf16<<<(NP + 255) / 256, 256, 0, t->st>>>(t->p, t->pb, NP);
  if ((e = cudaStreamSynchronize(t->st)) != cudaSuccess) return fail(e);
  *out = t;
  return PDFS_OK;
}

extern "C" void pdfs_mlp_trainer_destroy(pdfs_mlp_trainer *t) {
  if (!t) return;
  cudaSetDevice(t->dev);
  if (t->st) cudaStreamSynchronize(t->st);
  cudaFree(t->x);
  cudaFree(t->y);
  cudaFree(t->p);
  cudaFree(t->m);
  cudaFree(t->v);
  cudaFree(t->g);
  cudaFree(t->pb);
  cudaFree(t->loss);
  cudaFree(t->count);
  if (t->st) cudaStreamDestroy(t->st);
  cudaGetLastError();
  delete t;
}

// Records the sweeps of one phase of a plain solve of context c: from the
// sweep after the first full cycle on (when the solve's schedulers start),
// one sample per block the history rule nominates.
static int trace_phase(pdfs_mlp_trainer *t, pdfs_ctx *c, int which, float tol, float *bmin, uint16_t *tx,
                       uint8_t *cand) {
  const bool f32 = which == 0;
  const long long nb = c->nblocks;
  MK(cudaMemsetAsync(c->bchg, 0, (size_t)nb * kRing * 4, c->st));
  const float hmin = (float)std::min(c->g.dx, std::min(c->g.dy, c->g.dz));
  const int first = c->o.first_ordering ? c->o.first_ordering - 1 : 0;
  const int grid = std::max(1, (int)std::min<long long>((nb + 255) / 256, (long long)c->sms * 8));
  int cur = 0;
  for (int s = 0; s < 400; ++s) {
    const int sn = (first + s) % 8 + 1;
    const bool rec = s >= kHist;
    if (rec) {
      int r = trainer_grow(t, nb);
      if (r) return r;
      MK(cudaMemcpyAsync(t->count, &t->n, 8, cudaMemcpyHostToDevice, c->st));
      MK(block_min(f32 ? (const void *)c->u32 : (const void *)c->u64,
                   f32 ? 0 : (c->o.arith == PDFS_ARITH_PAIR ? 2 : 1), f32 ? c->L32 : c->L64, c->g, c->nbx,
                   c->nby, c->nbz, bmin, c->st));
      const FeatArgs f = feat_args(c->bchg, cur, kHist, bmin, c->nbx, c->nby, c->nbz, sn, s, f32 ? 0 : 1, tol, hmin);
      k_features<<<grid, 256, 0, c->st>>>(f, tx, cand);
      MK(cudaGetLastError());
    }
    unsigned int *now = c->bchg + (size_t)cur * nb;
    double chg = 0.0;
    int r = ctx_sweep_once(c, which, sn, nullptr, now, &chg);
    if (r) return r;
    if (rec) {
      k_append<<<grid, 256, 0, c->st>>>(tx, cand, now, nb, tol, t->x, t->y, t->count);
      MK(cudaGetLastError());
      unsigned long long n = 0;
      MK(cudaMemcpyAsync(&n, t->count, 8, cudaMemcpyDeviceToHost, c->st));
      MK(cudaStreamSynchronize(c->st));
      t->n = (long long)n;
    }
    cur = (cur + 1) % kRing;
    if (chg <= tol) break;
  }
  MK(cudaStreamSynchronize(c->st));
  return PDFS_OK;
}

extern "C" int pdfs_mlp_trainer_add_solve(pdfs_mlp_trainer *t, const pdfs_grid *g, const double *field,
                                          const uint8_t *frozen, const pdfs_opts *o_in, long long *samples) {
  if (!t || !g || !field) return PDFS_ERR_INVALID;
  pdfs_opts o;
  if (o_in)
    o = *o_in;
  else
    pdfs_default_opts(&o);
  const bool polish = o.precision == PDFS_PREC_FP32_POLISH64, fp64 = o.precision == PDFS_PREC_FP64;
  o.scheduler = PDFS_SCHED_NONE;
  o.fixed_sweeps = 0;
  o.device = t->dev;
  pdfs_ctx *c = nullptr;
  int s = pdfs_ctx_create(g, &o, &c);
  if (s) return s;
  float *bmin = nullptr;
  uint16_t *tx = nullptr;
  uint8_t *cand = nullptr;
  do {
    if ((s = pdfs_ctx_load(c, field, frozen)) != PDFS_OK) break;
    if (cudaMalloc(&bmin, (size_t)c->nblocks * 4) != cudaSuccess ||
        cudaMalloc(&tx, (size_t)c->nblocks * NI * 2) != cudaSuccess ||
        cudaMalloc(&cand, (size_t)c->nblocks) != cudaSuccess) {
      s = PDFS_ERR_OOM;
      break;
    }
    if (fp64) {  // plain FP64 solve to o.tol
      if ((s = ctx_fp64_start(c)) != PDFS_OK) break;
      s = trace_phase(t, c, 1, (float)o.tol, bmin, tx, cand);
      break;
    }
    if ((s = ctx_narrow(c)) != PDFS_OK) break;
    if ((s = trace_phase(t, c, 0, kTol32, bmin, tx, cand)) != PDFS_OK) break;
    if (polish) {
      if ((s = ctx_widen(c)) != PDFS_OK) break;
      if ((s = trace_phase(t, c, 2, (float)o.tol, bmin, tx, cand)) != PDFS_OK) break;
    }
  } while (0);
  cudaFree(bmin);
  cudaFree(tx);
  cudaFree(cand);
  cudaGetLastError();
  pdfs_ctx_destroy(c);
  if (samples) *samples = t->n;
  return s;
}

extern "C" int pdfs_mlp_trainer_fit(pdfs_mlp_trainer *t, int epochs, int batch, float lr, float pos_weight,
                                    float *loss_out) {
  if (!t || epochs < 1 || batch < 1 || !(lr > 0.0f) || !(pos_weight > 0.0f)) return PDFS_ERR_INVALID;
  if (t->n < 1) return PDFS_ERR_INVALID;
  MK(cudaSetDevice(t->dev));
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  float last = 0.0f;
  for (int ep = 0; ep < epochs; ++ep) {
    const Perm perm = random_perm((unsigned long long)t->n, t->rng);
    MK(cudaMemsetAsync(t->loss, 0, 4, t->st));
    long long nbatch = 0;
    for (long long first = 0; first < t->n; first += batch) {
      const int b = (int)std::min<long long>(batch, t->n - first);
      MK(train_grad(t->pb, t->x, t->y, t->n, perm, first, b, pos_weight, t->g, t->loss, t->st));
      ++t->step;
      const float bc1 = 1.0f - std::pow(b1, (float)t->step), bc2 = 1.0f - std::pow(b2, (float)t->step);
      k_adam<<<(NP + 255) / 256, 256, 0, t->st>>>(t->p, t->m, t->v, t->g, t->pb, NP, lr, b1, b2, eps, bc1, bc2);
      MK(cudaGetLastError());
      ++nbatch;
    }
    float ls = 0.0f;
    MK(cudaMemcpyAsync(&ls, t->loss, 4, cudaMemcpyDeviceToHost, t->st));
    MK(cudaStreamSynchronize(t->st));
    last = ls / (float)nbatch;
  }
  if (loss_out) *loss_out = last;
  return PDFS_OK;
}

extern "C" int pdfs_mlp_trainer_weights(pdfs_mlp_trainer *t, float recall, float *blob, float *recall_out,
                                        float *active_out) {
  if (!t || !blob || !(recall > 0.0f) || recall > 1.0f || t->n < 1) return PDFS_ERR_INVALID;
  MK(cudaSetDevice(t->dev));
  std::vector<uint16_t> hb(NP);
  MK(cudaMemcpy(hb.data(), t->pb, NP * 2, cudaMemcpyDeviceToHost));
  for (int i = 0; i < NP; ++i) {
    const uint32_t u = (uint32_t)hb[i] << 16;
    std::memcpy(&blob[i], &u, 4);
  }
  // logits of (up to) 4M samples spread over the collection
  const long long ns = std::min<long long>(t->n, 1 << 22);
  const long long stride = t->n / ns;
  DBuf<uint16_t> xs;
  DBuf<uint8_t> ys;
  DBuf<float> lg;
  MK(xs.alloc((size_t)ns * NI));
  MK(ys.alloc((size_t)ns));
  MK(lg.alloc((size_t)ns));
  MK(cudaMemcpy2DAsync(xs.p, NI * 2, t->x, (size_t)stride * NI * 2, NI * 2, (size_t)ns, cudaMemcpyDeviceToDevice,
                       t->st));
  MK(cudaMemcpy2DAsync(ys.p, 1, t->y, (size_t)stride, 1, (size_t)ns, cudaMemcpyDeviceToDevice, t->st));
  DBuf<int> derr;
  MK(derr.alloc(1));
  MK(cudaMemsetAsync(derr.p, 0, 4, t->st));
  int sms = 0;
  MK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, t->dev));
  MK(mlp_logits(t->pb, xs.p, ns, lg.p, derr.p, sms, t->st));
  int herr = 0;
  MK(cudaMemcpyAsync(&herr, derr.p, 4, cudaMemcpyDeviceToHost, t->st));
  std::vector<float> hl((size_t)ns);
  std::vector<uint8_t> hy((size_t)ns);
  MK(cudaMemcpyAsync(hl.data(), lg.p, (size_t)ns * 4, cudaMemcpyDeviceToHost, t->st));
  MK(cudaMemcpyAsync(hy.data(), ys.p, (size_t)ns, cudaMemcpyDeviceToHost, t->st));
  MK(cudaStreamSynchronize(t->st));
  if (herr) return PDFS_ERR_TIMEOUT;
  std::vector<float> pos;
  for (long long i = 0; i < ns; ++i)
    if (hy[i]) pos.push_back(hl[i]);
  float thr = -INFINITY;
  if (!pos.empty()) {
    std::sort(pos.begin(), pos.end());
    // keep the top `recall` fraction of the positives: threshold just below
    const size_t k = (size_t)std::floor((1.0 - (double)recall) * (double)pos.size());
    thr = std::nextafter(pos[std::min(k, pos.size() - 1)], -INFINITY);
  }
  blob[NP] = thr;
  if (recall_out || active_out) {
    long long tp = 0, act = 0;
    for (long long i = 0; i < ns; ++i) {
      const bool on = hl[i] > thr;
      act += on;
      tp += on && hy[i];
    }
    if (recall_out) *recall_out = pos.empty() ? 1.0f : (float)tp / (float)pos.size();
    if (active_out) *active_out = (float)act / (float)ns;
  }
  return PDFS_OK;
}

// ---- kernel-level entry points for checks ------------------------------------------------
extern "C" int pdfs_mlp_grad(const float *params, const uint16_t *x, const uint8_t *y, int n, float pos_weight,
                             float *grad, float *loss) {
  if (!params || !x || !y || n < 1 || !grad || !(pos_weight > 0.0f)) return PDFS_ERR_INVALID;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return PDFS_ERR_NO_DEVICE;
  }
  MK(set_smem_attrs());
  DBuf<float> dp, dg, dl;
  DBuf<uint16_t> dpb, dx;
  DBuf<uint8_t> dy;
  MK(dp.alloc(NP));
  MK(dg.alloc(NP));
  MK(dl.alloc(1));
  MK(dpb.alloc(NP));
  MK(dx.alloc((size_t)n * NI));
  MK(dy.alloc((size_t)n));
  MK(cudaMemcpy(dp.p, params, NP * 4, cudaMemcpyHostToDevice));
  MK(cudaMemcpy(dx.p, x, (size_t)n * NI * 2, cudaMemcpyHostToDevice));
  MK(cudaMemcpy(dy.p, y, (size_t)n, cudaMemcpyHostToDevice));
  MK(cudaMemset(dg.p, 0, NP * 4));
  MK(cudaMemset(dl.p, 0, 4));
  k_to_bf16<<<(NP + 255) / 256, 256>>>(dp.p, dpb.p, NP);
  MK(cudaGetLastError());
  MK(train_grad(dpb.p, dx.p, dy.p, n, Perm{1, 0, (unsigned long long)n}, 0, n, pos_weight, dg.p, dl.p, 0));
  MK(cudaMemcpy(grad, dg.p, NP * 4, cudaMemcpyDeviceToHost));
  if (loss) MK(cudaMemcpy(loss, dl.p, 4, cudaMemcpyDeviceToHost));
  return PDFS_OK;
}

extern "C" int pdfs_mlp_adam(float *params, float *m, float *v, const float *grad, int step, float lr, float beta1,
                             float beta2, float eps, uint16_t *params_bf16) {
  if (!params || !m || !v || !grad || step < 1) return PDFS_ERR_INVALID;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return PDFS_ERR_NO_DEVICE;
  }
  DBuf<float> dp, dm, dv, dg;
  DBuf<uint16_t> dpb;
  MK(dp.alloc(NP));
  MK(dm.alloc(NP));
  MK(dv.alloc(NP));
  MK(dg.alloc(NP));
  MK(dpb.alloc(NP));
  MK(cudaMemcpy(dp.p, params, NP * 4, cudaMemcpyHostToDevice));
  MK(cudaMemcpy(dm.p, m, NP * 4, cudaMemcpyHostToDevice));
  MK(cudaMemcpy(dv.p, v, NP * 4, cudaMemcpyHostToDevice));
  MK(cudaMemcpy(dg.p, grad, NP * 4, cudaMemcpyHostToDevice));
  const float bc1 = 1.0f - std::pow(beta1, (float)step), bc2 = 1.0f - std::pow(beta2, (float)step);
  k_adam<<<(NP + 255) / 256, 256>>>(dp.p, dm.p, dv.p, dg.p, dpb.p, NP, lr, beta1, beta2, eps, bc1, bc2);
  MK(cudaGetLastError());
  MK(cudaMemcpy(params, dp.p, NP * 4, cudaMemcpyDeviceToHost));
  MK(cudaMemcpy(m, dm.p, NP * 4, cudaMemcpyDeviceToHost));
  MK(cudaMemcpy(v, dv.p, NP * 4, cudaMemcpyDeviceToHost));
  if (params_bf16) MK(cudaMemcpy(params_bf16, dpb.p, NP * 2, cudaMemcpyDeviceToHost));
  return PDFS_OK;
}

extern "C" int pdfs_mlp_infer(const float *blob, const uint16_t *x, int n, float *logits) {
  if (!blob || !x || n < 1 || !logits) return PDFS_ERR_INVALID;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return PDFS_ERR_NO_DEVICE;
  }
  MK(set_smem_attrs());
  DBuf<float> dp, dl;
  DBuf<uint16_t> dpb, dx;
  MK(dp.alloc(NP));
  MK(dpb.alloc(NP));
  MK(dx.alloc((size_t)n * NI));
  MK(dl.alloc((size_t)n));
  MK(cudaMemcpy(dp.p, blob, NP * 4, cudaMemcpyHostToDevice));
  MK(cudaMemcpy(dx.p, x, (size_t)n * NI * 2, cudaMemcpyHostToDevice));
  k_to_bf16<<<(NP + 255) / 256, 256>>>(dp.p, dpb.p, NP);
  DBuf<int> derr;
  MK(derr.alloc(1));
  MK(cudaMemset(derr.p, 0, 4));
  int dev = 0, sms = 0;
  MK(cudaGetDevice(&dev));
  MK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  MK(mlp_logits(dpb.p, dx.p, n, dl.p, derr.p, sms, 0));
  int herr = 0;
  MK(cudaMemcpy(&herr, derr.p, 4, cudaMemcpyDeviceToHost));
  if (herr) return PDFS_ERR_TIMEOUT;
  MK(cudaMemcpy(logits, dl.p, (size_t)n * 4, cudaMemcpyDeviceToHost));
  return PDFS_OK;
}
