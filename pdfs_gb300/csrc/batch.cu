// batch.cu -- many independent grids per launch, and the tile autotuner.
//
// The reference solves one grid per process (single_gpu_cuda/src/main.c:56-106).
// pdfs_solve_batch() keeps every grid resident in its own context.  On
// pencils (the default) each round of 8 orderings is ONE persistent launch
// over the pencils of every grid still sweeping: the ticket table lists
// (grid, sweep, pencil) triples, every grid's sweep s before any grid's sweep
// s + 1 and each grid's pencils in wavefront order, and a pencil of sweep s
// starts once its grid's sweep s - 1 is complete -- so every wait is on a
// smaller ticket held by a running CTA.  On column tiles each sweep is one
// launch over (grid, column) pairs.  Rounds after the first replay a captured
// CUDA graph; after each round the per-grid, per-sweep changes come back in
// one copy, and converged grids leave the ticket table.
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
  int *d_done = nullptr;   // pencil rounds: [grid * 8 + sweep] pencils finished
  int *d_round = nullptr;  // pencil rounds: rounds run in this phase
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
    cudaFree(d_done);
    cudaFree(d_round);
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


__global__ void k_add(int *p, int v) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *p += v;
}

// One phase on pencils (which: 0 FP32, 1 FP64 min, 2 FP64 replace): rounds
// of 8 orderings over every grid in `todo`, ONE launch per round (the
// pencil kernel's batched mode), until each grid has a sweep with change
// <= tol.  The first round runs eagerly; the following rounds replay a
// captured graph (counter resets, the launch, the round count, the copy of
// the changes).
int batch_phase_pencils(BatchState &B, std::vector<pdfs_ctx *> &ctx, const std::vector<int> &todo, int which,
                        double tol, int max_sweeps, std::vector<pdfs_stats> &st, double *kern_ms, int *launches) {
  const int n = B.n;
  const bool f32 = which == 0;
  const pdfs_opts &o = ctx[0]->o;
  const int arith = o.arith == PDFS_ARITH_REFERENCE ? ARITH_REF
                    : o.arith == PDFS_ARITH_MIXED   ? ARITH_MIXED
                    : o.arith == PDFS_ARITH_PAIR    ? ARITH_PAIR
                                                    : ARITH_FAST;
  bool iso = true;
  std::vector<SweepArgs> args(n);
  std::vector<CUtensorMap> maps(3 * (size_t)n);
  for (int g = 0; g < n; ++g) {
    pdfs_ctx *c = ctx[g];
    iso = iso && c->g.dx == c->g.dy && c->g.dy == c->g.dz;
    fill_sweep_args(c, which, 1, nullptr, nullptr, &args[g]);
    // the round's sweep s tags its mailbox words epoch + 8 * round + s: above
    // every tag this context has used
    args[g].epoch = c->epoch + 1;
    args[g].err = B.d_err;
    args[g].ticket = B.d_ticket;
    const Layout &L = f32 ? c->L32 : c->L64;
    BK(encode_pencil_maps(which, args[g], L, &maps[3 * (size_t)g]));
  }
  BK(cudaMemcpyAsync(B.d_args, args.data(), sizeof(SweepArgs) * n, cudaMemcpyHostToDevice, B.st));
  BK(cudaMemcpyAsync(B.d_maps, maps.data(), sizeof(CUtensorMap) * 3 * n, cudaMemcpyHostToDevice, B.st));
  BK(cudaMemsetAsync(B.d_round, 0, 4, B.st));

  std::vector<int> active(todo);
  std::vector<int2> tickets;
  auto rebuild = [&]() -> int {
    // every grid's sweep s before any grid's sweep s + 1; a grid's pencils in
    // its wavefront order
    tickets.clear();
    std::vector<std::vector<int>> ord(n);
    for (int g : active) {
      const Layout &L = f32 ? ctx[g]->L32 : ctx[g]->L64;
      ord[g] = wavefront_order(L.ncx, L.ncy, L.tx, L.ty);
    }
    for (int s = 0; s < 8; ++s)
      for (int g : active)
        for (int lc : ord[g]) tickets.push_back(make_int2(g * 8 + s, lc));
    if (tickets.empty()) return PDFS_OK;
    BK(cudaMemcpyAsync(B.d_tickets, tickets.data(), sizeof(int2) * tickets.size(), cudaMemcpyHostToDevice, B.st));
    BatchDesc desc{(int)tickets.size(), B.d_tickets, B.d_args, B.d_maps, n, B.d_done, B.d_round};
    BK(cudaMemcpyAsync(B.d_desc, &desc, sizeof(desc), cudaMemcpyHostToDevice, B.st));
    return PDFS_OK;
  };
  int r = rebuild();
  if (r) return r;
  const int max_ticks = (int)tickets.size();

  SweepArgs a0;
  std::memset(&a0, 0, sizeof(a0));
  a0.err = B.d_err;
  a0.ticket = B.d_ticket;
  a0.maxchg = B.d_chg;
  a0.batch = B.d_desc;
  auto enqueue_round = [&]() -> int {
    BK(cudaMemsetAsync(B.d_done, 0, sizeof(int) * 8 * n, B.st));
    BK(cudaMemsetAsync(B.d_ticket, 0, 4, B.st));
    int grid = 0;
    BK(launch_pencil_round(which, arith, iso, a0, max_ticks, B.sms, B.st, &grid));
    k_add<<<1, 32, 0, B.st>>>(B.d_round, 1);
    BK(cudaGetLastError());
    BK(cudaMemcpyAsync(B.h_chg, B.d_chg, sizeof(unsigned long long) * 8 * n, cudaMemcpyDeviceToHost, B.st));
    BK(cudaMemcpyAsync(B.h_err, B.d_err, 16, cudaMemcpyDeviceToHost, B.st));
    return PDFS_OK;
  };

  cudaEvent_t e0, e1;
  BK(cudaEventCreate(&e0));
  BK(cudaEventCreate(&e1));
  bool captured = false;
  int rounds = 0;
  for (int round = 0; !active.empty(); ++round) {
    if (round * 8 >= max_sweeps) {
      for (int g : active) st[g].status = PDFS_ERR_NOT_CONVERGED;
      break;
    }
    BK(cudaMemsetAsync(B.d_chg, 0, sizeof(unsigned long long) * 8 * n, B.st));
    BK(cudaEventRecord(e0, B.st));
    if (round == 0) {
      if ((r = enqueue_round())) return r;  // eagerly: it also sets the kernel attributes
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
    ++rounds;
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    *kern_ms += ms;
    *launches += 2;  // the round and the round count
    if (B.h_err[0]) return B.h_err[0] == DEV_ERR_TIMEOUT ? PDFS_ERR_TIMEOUT : PDFS_ERR_CUDA;
    std::vector<int> still;
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
      if (conv < 0) still.push_back(g);
    }
    if (still.size() != active.size()) {
      active.swap(still);
      if ((r = rebuild())) return r;
    }
  }
  // every context's later sweeps tag above this phase's words
  for (int g = 0; g < n; ++g) ctx[g]->epoch += 8 * rounds + 8;
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
  bool pen32 = true, pen64 = true;
  {
    // A batch runs on pencils -- one launch per round of 8 orderings over all
    // grids (the default, and for brick or lane-column tiles) -- or, when a
    // column tile is asked for, on columns, one launch per sweep.
    auto column = [](const TileShape &t) { return !t.pencil && !t.bz && !t.lc; };
    int t32 = o.tile & 0xff, t64 = (o.tile >> 8) & 0xff;
    if (t32 >= 1 && t32 <= tile_count32() && column(tile32(t32))) pen32 = false;
    if (t64 >= 1 && t64 <= tile_count64() && column(tile64(t64))) pen64 = false;
    if (pen32) t32 = 10;
    if (pen64) t64 = 6;
    // the column kernels have no FP32-pair arithmetic: they polish in the mixed one
    if (!pen64 && o.arith == PDFS_ARITH_PAIR) o.arith = PDFS_ARITH_MIXED;
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
  size_t total_cols = 0;  // tickets: columns of a sweep, or pencils of a round's 8 sweeps
  for (auto *c : ctx) total_cols += 8 * std::max((size_t)c->L32.ncx * c->L32.ncy, (size_t)c->L64.ncx * c->L64.ncy);
  BQ(cudaMalloc(&B.d_args, sizeof(SweepArgs) * n));
  BQ(cudaMalloc(&B.d_maps, sizeof(CUtensorMap) * 3 * n));
  BQ(cudaMalloc(&B.d_tickets, sizeof(int2) * total_cols));
  BQ(cudaMalloc(&B.d_desc, sizeof(BatchDesc)));
  BQ(cudaMalloc(&B.d_chg, sizeof(unsigned long long) * 8 * n));
  BQ(cudaMalloc(&B.d_err, 16));
  BQ(cudaMalloc(&B.d_ticket, 16));
  BQ(cudaMalloc(&B.d_done, sizeof(int) * 8 * n));
  BQ(cudaMalloc(&B.d_round, 16));
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
    rc = (pen64 ? batch_phase_pencils : batch_phase)(B, ctx, all, 1, o.tol, max_sweeps, st, &kms64, &launches);
    for (auto *c : ctx) c->last_prec = 1;
  } else {
    for (auto *c : ctx) {
      if ((rc = ctx_narrow(c))) return cleanup(rc);
    }
    for (auto *c : ctx) BQ(cudaStreamSynchronize(c->st));
    rc = (pen32 ? batch_phase_pencils : batch_phase)(B, ctx, all, 0, 4.0e-6, max_sweeps, st, &kms32, &launches);
    for (auto *c : ctx) c->last_prec = 0;
    if (!rc && o.precision == PDFS_PREC_FP32_POLISH64) {
      for (auto *c : ctx) {
        if ((rc = ctx_widen(c))) return cleanup(rc);
      }
      for (auto *c : ctx) BQ(cudaStreamSynchronize(c->st));
      rc = (pen64 ? batch_phase_pencils : batch_phase)(B, ctx, all, 2, o.tol, max_sweeps, st, &kms64, &launches);
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
