// batch.cu -- many independent grids per launch, and the tile autotuner.
//
// The reference solves one grid per process (single_gpu_cuda/src/main.c:56-106).
// pdfs_solve_batch() keeps every grid resident in its own context and runs
// each sweep as ONE persistent launch over the columns of all grids that are
// still sweeping: the ticket table lists (grid, column) pairs, each grid's
// columns in wavefront order, so the deadlock-free argument of the single-grid
// sweep carries over unchanged.  A round of 8 orderings is captured once in a
// CUDA graph and replayed; after each round the per-grid, per-sweep changes
// come back in one copy, and converged grids leave the ticket table.
#include <chrono>
#include <cstdio>
#include <cstring>
#include <vector>

#include "internal.h"

using namespace pdfs;

namespace {

struct BatchState {
  int n = 0;
  int dev = 0, sms = 0;
  cudaStream_t st = nullptr;
  SweepArgs *d_args = nullptr;
  CUtensorMap *d_maps = nullptr;
  int2 *d_tickets = nullptr;
  BatchDesc *d_desc = nullptr;
  int *d_prog = nullptr;
  size_t prog_ints = 0;
  unsigned long long *d_chg = nullptr;  // [8][n]
  unsigned long long *h_chg = nullptr;  // pinned copy
  int *d_err = nullptr;                 // [4]
  int *h_err = nullptr;                 // pinned
  int *d_ticket = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
  ~BatchState() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    cudaFree(d_args);
    cudaFree(d_maps);
    cudaFree(d_tickets);
    cudaFree(d_desc);
    cudaFree(d_prog);
    cudaFree(d_chg);
    cudaFree(d_err);
    cudaFree(d_ticket);
    if (h_chg) cudaFreeHost(h_chg);
    if (h_err) cudaFreeHost(h_err);
    if (st) cudaStreamDestroy(st);
  }
};

int cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return PDFS_OK;
  if (e == cudaErrorMemoryAllocation) return PDFS_ERR_OOM;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return PDFS_ERR_NO_DEVICE;
  return PDFS_ERR_CUDA;
}
#define BK(call)                            \
  do {                                      \
    cudaError_t e_ = (call);                \
    if (e_ != cudaSuccess) {                \
      if (getenv("PDFS_LOG"))               \
        fprintf(stderr, "pdfs batch: %s:%d %s: %s\n", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); \
      return cuda_status(e_);               \
    }                                       \
  } while (0)

double chg_value(unsigned long long bits, bool f32) {
  if (f32) {
    unsigned int b = (unsigned int)bits;
    float f;
    std::memcpy(&f, &b, 4);
    return f;
  }
  double d;
  std::memcpy(&d, &bits, 8);
  return d;
}

// One phase (which: 0 FP32, 1 FP64 min, 2 FP64 replace) over every grid in
// `todo`, rounds of 8 sweeps until each grid has a sweep with change <= tol.
int batch_phase(BatchState &B, std::vector<pdfs_ctx *> &ctx, const std::vector<int> &todo, int which, double tol,
                int max_sweeps, std::vector<pdfs_stats> &st, double *kern_ms, int *launches) {
  const int n = B.n;
  const bool f32 = which == 0;
  const pdfs_opts &o = ctx[0]->o;
  const int tile = f32 ? ctx[0]->t32 : ctx[0]->t64;
  const int arith = o.arith == PDFS_ARITH_REFERENCE ? ARITH_REF : (o.arith == PDFS_ARITH_MIXED ? ARITH_MIXED : ARITH_FAST);
  bool iso = true;
  // per-grid sweep arguments and tensor maps
  std::vector<SweepArgs> args(n);
  std::vector<CUtensorMap> maps(3 * (size_t)n);
  std::vector<size_t> prog_off(n, 0);
  size_t prog = 0;
  for (int g = 0; g < n; ++g) {
    const pdfs_ctx *c = ctx[g];
    const Layout &L = f32 ? c->L32 : c->L64;
    prog_off[g] = prog;
    prog += (size_t)L.ncx * L.ncy * L.ty;
    iso = iso && c->g.dx == c->g.dy && c->g.dy == c->g.dz;
  }
  if (prog > B.prog_ints) {
    cudaFree(B.d_prog);
    B.d_prog = nullptr;
    BK(cudaMalloc(&B.d_prog, prog * 4));
    B.prog_ints = prog;
  }
  for (int g = 0; g < n; ++g) {
    pdfs_ctx *c = ctx[g];
    fill_sweep_args(c, which, 1, nullptr, nullptr, &args[g]);
    args[g].prog = B.d_prog + prog_off[g];
    args[g].err = B.d_err;
    args[g].ticket = B.d_ticket;
    const Layout &L = f32 ? c->L32 : c->L64;
    BK(encode_sweep_maps(which, tile, args[g], L, which == 2 ? (const void *)c->in64 : nullptr, &maps[3 * (size_t)g]));
    if (!(c->g.dx == c->g.dy && c->g.dy == c->g.dz) && f32) iso = false;
  }
  BK(cudaMemcpyAsync(B.d_args, args.data(), sizeof(SweepArgs) * n, cudaMemcpyHostToDevice, B.st));
  BK(cudaMemcpyAsync(B.d_maps, maps.data(), sizeof(CUtensorMap) * 3 * n, cudaMemcpyHostToDevice, B.st));

  std::vector<int> active(todo);
  std::vector<int> sweeps(n, 0);
  std::vector<int2> tickets;
  auto rebuild = [&]() -> int {
    tickets.clear();
    for (int g : active) {
      const pdfs_ctx *c = ctx[g];
      const Layout &L = f32 ? c->L32 : c->L64;
      std::vector<int> ord = wavefront_order(L.ncx, L.ncy, L.tx, L.ty);
      for (int lc : ord) tickets.push_back(make_int2(g, lc));
    }
    if (tickets.empty()) return PDFS_OK;
    BK(cudaMemcpyAsync(B.d_tickets, tickets.data(), sizeof(int2) * tickets.size(), cudaMemcpyHostToDevice, B.st));
    BatchDesc desc{(int)tickets.size(), B.d_tickets, B.d_args, B.d_maps};
    BK(cudaMemcpyAsync(B.d_desc, &desc, sizeof(desc), cudaMemcpyHostToDevice, B.st));
    return PDFS_OK;
  };
  int r = rebuild();
  if (r) return r;
  const int max_ticks = (int)tickets.size();

  // one round = 8 sweeps: reset progress and tickets, launch, collect changes
  SweepArgs a0;
  std::memset(&a0, 0, sizeof(a0));
  a0.err = B.d_err;
  a0.ticket = B.d_ticket;
  a0.batch = B.d_desc;
  auto enqueue_round = [&]() -> int {
    for (int s = 0; s < 8; ++s) {
      ordering_signs(s + 1, &a0.sx, &a0.sy, &a0.sz);
      a0.maxchg = B.d_chg + (size_t)s * n;
      BK(cudaMemsetAsync(B.d_prog, 0, prog * 4, B.st));
      BK(cudaMemsetAsync(B.d_ticket, 0, 4, B.st));
      int grid = 0;
      BK(launch_sweep_batch(which, tile, arith, iso, a0, max_ticks, B.sms, B.st, &grid));
    }
    BK(cudaMemcpyAsync(B.h_chg, B.d_chg, sizeof(unsigned long long) * 8 * n, cudaMemcpyDeviceToHost, B.st));
    BK(cudaMemcpyAsync(B.h_err, B.d_err, 16, cudaMemcpyDeviceToHost, B.st));
    return PDFS_OK;
  };

  cudaEvent_t e0, e1;
  BK(cudaEventCreate(&e0));
  BK(cudaEventCreate(&e1));
  bool captured = false;
  for (int round = 0; !active.empty(); ++round) {
    if (round * 8 >= max_sweeps) {
      for (int g : active) st[g].status = PDFS_ERR_NOT_CONVERGED;
      break;
    }
    BK(cudaMemsetAsync(B.d_chg, 0, sizeof(unsigned long long) * 8 * n, B.st));
    BK(cudaEventRecord(e0, B.st));
    if (round == 0) {
      // the first round runs eagerly (it also sets the kernel attributes);
      // the following rounds replay the same work from a graph
      if ((r = enqueue_round())) return r;
    } else {
      if (!captured) {
        if (B.exec) {
          cudaGraphExecDestroy(B.exec);
          B.exec = nullptr;
        }
        if (B.graph) {
          cudaGraphDestroy(B.graph);
          B.graph = nullptr;
        }
        BK(cudaStreamBeginCapture(B.st, cudaStreamCaptureModeThreadLocal));
        r = enqueue_round();
        cudaGraph_t gph = nullptr;
        cudaError_t ce = cudaStreamEndCapture(B.st, &gph);
        if (r) return r;
        BK(ce);
        B.graph = gph;
        BK(cudaGraphInstantiate(&B.exec, B.graph, 0));
        captured = true;
      }
      BK(cudaGraphLaunch(B.exec, B.st));
    }
    BK(cudaEventRecord(e1, B.st));
    BK(cudaStreamSynchronize(B.st));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    *kern_ms += ms;
    *launches += 8;
    if (B.h_err[0]) return B.h_err[0] == DEV_ERR_TIMEOUT ? PDFS_ERR_TIMEOUT : PDFS_ERR_CUDA;
    std::vector<int> still;
    const long long nodes_of = 0;
    (void)nodes_of;
    for (int g : active) {
      int conv = -1;
      double last = 0.0;
      for (int s = 0; s < 8; ++s) {
        last = chg_value(B.h_chg[(size_t)s * n + g], f32);
        if (last <= tol) {
          conv = s;
          break;
        }
      }
      const int done_sweeps = conv >= 0 ? conv + 1 : 8;
      sweeps[g] += 8;  // the round ran all 8 sweeps on every active grid
      pdfs_stats &S = st[g];
      const long long nodes = (long long)ctx[g]->g.nx * ctx[g]->g.ny * ctx[g]->g.nz;
      S.voxel_updates += nodes * 8;
      if (!f32) S.voxel_updates_fp64 += nodes * 8;
      S.full_sweeps += 8;
      if (f32)
        S.sweeps_fp32 += 8;
      else
        S.sweeps_fp64 += 8;
      S.final_change = last;
      (void)done_sweeps;
      if (conv < 0) still.push_back(g);
    }
    if (still.size() != active.size()) {
      active.swap(still);
      if ((r = rebuild())) return r;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return PDFS_OK;
}

}  // namespace

extern "C" int pdfs_solve_batch(int n, const pdfs_grid *grids, double *const *fields, const uint8_t *const *frozen,
                                const pdfs_opts *o_in, pdfs_stats *stats) {
  if (n < 1 || !grids || !fields) return PDFS_ERR_INVALID;
  const auto t0 = std::chrono::steady_clock::now();
  pdfs_opts o;
  if (o_in)
    o = *o_in;
  else
    pdfs_default_opts(&o);
  if (o.fixed_sweeps != 0) return PDFS_ERR_INVALID;  // the batch runs whole rounds to convergence
  o.scheduler = PDFS_SCHED_NONE;
  {
    // a batched launch runs the column kernels (one ticket space across the
    // grids); brick tiles and the default choice map to the column defaults
    int t32 = o.tile & 0xff, t64 = (o.tile >> 8) & 0xff;
    if (t32 == 0 || tile32(t32).bz || tile32(t32).lc) t32 = 4;
    // FP32 pairs live on bricks only: the batch polishes in the mixed arithmetic
    if (o.arith == PDFS_ARITH_PAIR) o.arith = PDFS_ARITH_MIXED;
    if (t64 == 0 || tile64(t64).bz || tile64(t64).lc) t64 = o.arith == PDFS_ARITH_MIXED ? 4 : 1;
    o.tile = t32 | (t64 << 8);
  }
  std::vector<pdfs_ctx *> ctx(n, nullptr);
  std::vector<pdfs_stats> st(n);
  std::memset(st.data(), 0, sizeof(pdfs_stats) * n);
  int rc = PDFS_OK;
  BatchState B;
  B.n = n;
  auto cleanup = [&](int s) {
    for (auto *c : ctx) pdfs_ctx_destroy(c);
    if (stats) {
      const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
      for (int g = 0; g < n; ++g) {
        st[g].ms_total = ms;
        if (!st[g].status) st[g].status = s;
        stats[g] = st[g];
      }
    }
    return s;
  };
  for (int g = 0; g < n; ++g) {
    if (!fields[g]) return cleanup(PDFS_ERR_INVALID);
    if ((rc = pdfs_ctx_create(&grids[g], &o, &ctx[g]))) return cleanup(rc);
    if ((rc = pdfs_ctx_load(ctx[g], fields[g], frozen ? frozen[g] : nullptr))) return cleanup(rc);
  }
  B.dev = ctx[0]->dev;
  B.sms = ctx[0]->sms;
  cudaError_t e;
#define BQ(call)                        \
  do {                                  \
    if ((e = (call)) != cudaSuccess) {  \
      return cleanup(cuda_status(e));   \
    }                                   \
  } while (0)
  BQ(cudaStreamCreateWithFlags(&B.st, cudaStreamNonBlocking));
  size_t total_cols = 0;
  for (auto *c : ctx) total_cols += std::max((size_t)c->L32.ncx * c->L32.ncy, (size_t)c->L64.ncx * c->L64.ncy);
  BQ(cudaMalloc(&B.d_args, sizeof(SweepArgs) * n));
  BQ(cudaMalloc(&B.d_maps, sizeof(CUtensorMap) * 3 * n));
  BQ(cudaMalloc(&B.d_tickets, sizeof(int2) * total_cols));
  BQ(cudaMalloc(&B.d_desc, sizeof(BatchDesc)));
  BQ(cudaMalloc(&B.d_chg, sizeof(unsigned long long) * 8 * n));
  BQ(cudaMalloc(&B.d_err, 16));
  BQ(cudaMalloc(&B.d_ticket, 16));
  BQ(cudaMemset(B.d_err, 0, 16));
  BQ(cudaHostAlloc(&B.h_chg, sizeof(unsigned long long) * 8 * n, cudaHostAllocDefault));
  BQ(cudaHostAlloc(&B.h_err, 16, cudaHostAllocDefault));
  double kms32 = 0, kms64 = 0;
  int launches = 0;
  std::vector<int> all(n);
  for (int g = 0; g < n; ++g) all[g] = g;
  const int max_sweeps = o.max_sweeps > 0 ? o.max_sweeps : 100000;
  if (o.precision == PDFS_PREC_FP64) {
    for (auto *c : ctx)
      BQ(cudaMemcpyAsync(c->u64, c->in64, c->L64.elems * 8, cudaMemcpyDeviceToDevice, c->st));
    for (auto *c : ctx) BQ(cudaStreamSynchronize(c->st));
    rc = batch_phase(B, ctx, all, 1, o.tol, max_sweeps, st, &kms64, &launches);
    for (auto *c : ctx) c->last_prec = 1;
  } else {
    for (auto *c : ctx) {
      if ((rc = ctx_narrow(c))) return cleanup(rc);
    }
    for (auto *c : ctx) BQ(cudaStreamSynchronize(c->st));
    rc = batch_phase(B, ctx, all, 0, 4.0e-6, max_sweeps, st, &kms32, &launches);
    for (auto *c : ctx) c->last_prec = 0;
    if (!rc && o.precision == PDFS_PREC_FP32_POLISH64) {
      for (auto *c : ctx) {
        if ((rc = ctx_widen(c))) return cleanup(rc);
      }
      for (auto *c : ctx) BQ(cudaStreamSynchronize(c->st));
      rc = batch_phase(B, ctx, all, 2, o.tol, max_sweeps, st, &kms64, &launches);
      for (auto *c : ctx) c->last_prec = 1;
    }
  }
  if (rc) return cleanup(rc);
  for (int g = 0; g < n; ++g) {
    if ((rc = pdfs_ctx_store(ctx[g], fields[g]))) return cleanup(rc);
    st[g].ms_kern_fp32 = kms32;
    st[g].ms_kern_fp64 = kms64;
    st[g].ms_fp32 = kms32;
    st[g].ms_fp64 = kms64;
    st[g].launches = launches;
    st[g].tile = ctx[g]->t32 | (ctx[g]->t64 << 8);
  }
  int first_bad = PDFS_OK;
  for (int g = 0; g < n && !first_bad; ++g) first_bad = st[g].status;
  return cleanup(first_bad);
#undef BQ
}

extern "C" int pdfs_autotune(const pdfs_grid *g, const pdfs_opts *o_in, int *tile) {
  if (!g || !tile) return PDFS_ERR_INVALID;
  pdfs_opts o;
  if (o_in)
    o = *o_in;
  else
    pdfs_default_opts(&o);
  o.scheduler = PDFS_SCHED_NONE;
  o.freeze = PDFS_FREEZE_NONE;
  // a synthetic field: unknown everywhere except a thin slab of seeds
  const size_t n = (size_t)(g->nx + 2) * (g->ny + 2) * (g->nz + 2);
  std::vector<double> f(n, 1.0e10);
  for (int z = 0; z < g->nz + 2; ++z)
    for (int y = 0; y < g->ny + 2; ++y)
      for (int x = 0; x < g->nx + 2; ++x) {
        const bool halo = x == 0 || y == 0 || z == 0 || x == g->nx + 1 || y == g->ny + 1 || z == g->nz + 1;
        double &v = f[((size_t)z * (g->ny + 2) + y) * (g->nx + 2) + x];
        if (halo) v = INFINITY;
        else if (z == (g->nz + 1) / 2) v = 0.0;
      }
  auto time_tile = [&](int prec, int t, double *ms) -> int {
    pdfs_opts q = o;
    q.precision = prec;
    q.tile = prec == PDFS_PREC_FP32 ? t : (t << 8);
    q.fixed_sweeps = 2;
    pdfs_ctx *c = nullptr;
    int s = pdfs_ctx_create(g, &q, &c);
    if (s) return s;
    pdfs_stats st;
    s = pdfs_ctx_load(c, f.data(), nullptr);
    if (!s) s = pdfs_ctx_run(c, &st);  // first run: allocation and attribute set-up
    if (!s) s = pdfs_ctx_run(c, &st);
    pdfs_ctx_destroy(c);
    *ms = st.ms_kern_fp32 + st.ms_kern_fp64;
    return s;
  };
  int best32 = 1, best64 = 1;
  double b = 1e30;
  for (int t = 1; t <= tile_count32(); ++t) {
    double ms = 0;
    if (time_tile(PDFS_PREC_FP32, t, &ms) == PDFS_OK && ms < b) {
      b = ms;
      best32 = t;
    }
  }
  b = 1e30;
  // FP64 candidates: the tiles valid for the arithmetic (see validate() in solver.cu)
  std::vector<int> c64;
  if (o.arith == PDFS_ARITH_MIXED)
    c64 = {1, 4};
  else
    for (int t = 1; t <= (o.precision == PDFS_PREC_FP32_POLISH64 ? 2 : 3); ++t) c64.push_back(t);
  if (o.arith == PDFS_ARITH_FAST) c64.push_back(4);
  for (int t : {5, 6, 7, 8}) c64.push_back(t);  // bricks and pencils: every arithmetic
  if (o.arith == PDFS_ARITH_PAIR)
    for (int t : {9, 10}) c64.push_back(t);  // lane columns: FP32 pairs
  for (int t : c64) {
    double ms = 0;
    if (time_tile(PDFS_PREC_FP64, t, &ms) == PDFS_OK && ms < b) {
      b = ms;
      best64 = t;
    }
  }
  *tile = best32 | (best64 << 8);
  return PDFS_OK;
}
