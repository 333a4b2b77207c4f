/*
 * pdfs.h -- C ABI of the GB300 Fast Sweeping Method solver (libpdfs.so).
 *
 * Drop-in for the FSM solve of GEM3D/PDFS.  Plain C types only: pointers,
 * sizes, ints and doubles.  No function calls exit(); every entry point
 * returns a status code (PDFS_OK = 0, negative on failure).
 *
 * Field layout everywhere in this ABI is the reference's: a halo-padded
 * array of (nx+2)*(ny+2)*(nz+2) doubles, x fastest, then y, then z
 * (single_gpu_cuda/src/phi3D.c:66-68, mpi_openacc/src/phi3D_fsm.c:86-112).
 * Interior nodes have 1-based coordinates; halo values are read, never written.
 */
#ifndef PDFS_H
#define PDFS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes --------------------------------------------------------- */
#define PDFS_OK 0
#define PDFS_ERR_INVALID (-1)       /* bad argument (sizes, spacings, options)      */
#define PDFS_ERR_OOM (-2)           /* device or pinned host allocation failed      */
#define PDFS_ERR_CUDA (-3)          /* a CUDA runtime call failed                   */
#define PDFS_ERR_TIMEOUT (-4)       /* a bounded inter-tile wait gave up            */
#define PDFS_ERR_NOT_CONVERGED (-5) /* max_sweeps reached before the tolerance      */
#define PDFS_ERR_IO (-6)            /* file could not be read or written            */
#define PDFS_ERR_NO_DEVICE (-7)     /* no CUDA device (the library never falls back) */
#define PDFS_ERR_TOO_LARGE (-8)     /* grid exceeds the fixed scratch of pdfs_sweep_static */

/* ---- problem description ----------------------------------------------------- */
typedef struct {
  int nx, ny, nz;    /* interior nodes per axis (>= 1)        */
  double dx, dy, dz; /* node spacings (> 0)                   */
} pdfs_grid;

/* Arithmetic of the sweeps. */
enum {
  PDFS_PREC_FP64 = 0,          /* every sweep in FP64                                        */
  PDFS_PREC_FP32 = 1,          /* FP32 sweeps until a full sweep's max relative change
                                  |u_new - u_old| / max(u_new, h) is <= 4e-6 (FP32 rounding
                                  keeps sweeps changing by about 1e-7 relative), widened
                                  to FP64                                                    */
  PDFS_PREC_FP32_POLISH64 = 2, /* FP32 bulk sweeps, then FP64 replace-update polish sweeps    */
};

/* FP64 local-solver arithmetic. */
enum {
  PDFS_ARITH_REFERENCE = 0, /* the reference's expression trees, no fused multiply-add:
                               bit-identical to phi3D_fsm.c compiled with -ffp-contract=off */
  PDFS_ARITH_FAST = 1,      /* shifted quadratic with fused multiply-add (about 1e-15 rel.)  */
  PDFS_ARITH_MIXED = 2,     /* FP64 field, minima, update and convergence test; the local
                               solve's increment above the smallest minimum (at most about
                               h) in FP32: within about 1e-7 relative of the FP64 fixed
                               point, a few FP64 operations per update (tile 1 only).  The
                               increments' rounding keeps sweeps changing by ~1e-7 h: use
                               a tol of 1e-6 h or more                                    */
  PDFS_ARITH_PAIR = 3,      /* as MIXED, with the field, minima and update held as FP32
                               pairs hi + lo (48 significant bits, Knuth/Dekker error-free
                               sums) instead of FP64: no FP64 instruction in the sweeps.
                               FP64 bricks and pencils only (tiles 5-8; 6 is the
                               default); frozen nodes and the halo come back as the
                               exact FP64 input.  Same tol rule                          */
};

/* Which nodes are updated. */
enum {
  PDFS_FREEZE_NONE = 0, /* every interior node is min-updated, as the reference does        */
  PDFS_FREEZE_MASK = 1, /* nodes with frozen[i] != 0 keep their input value                 */
};

/* Active-block scheduling of the sweeps (8^3 node blocks). */
enum {
  PDFS_SCHED_NONE = 0,    /* every sweep visits every block                               */
  PDFS_SCHED_CHANGE = 1,  /* visit blocks that changed in one of the last 8 sweeps (one
                             cycle of orderings) or whose face neighbour changed in the
                             last sweep                                                   */
  PDFS_SCHED_LEARNED = 2, /* of the blocks PDFS_SCHED_CHANGE would visit, those the MLP
                             predicts will change                                         */
  PDFS_SCHED_OCTANT = 3,  /* FP32 and polish phases: the first FP32 cycle runs as one
                             launch of 8 full sweeps, each later cycle of 8 orderings as
                             one launch over the blocks whose characteristic directions
                             (from the FP32 field) agree with each ordering; FP64-only
                             solves sweep every block                                 */
};
/* Whatever the scheduler, a solve only terminates after a sweep that visits
 * every block and changes by at most the phase's tolerance (FP32: the
 * relative 4e-6; FP64: tol).  Under PDFS_PREC_FP32_POLISH64 with a scheduler,
 * the scheduler runs the FP32 phase, which may then end on a quiet scheduled
 * sweep; the polish's first cycle of 8 orderings visits, in each ordering,
 * only the blocks whose characteristic directions (from the FP32 result)
 * agree with that ordering's sweep directions, and full sweeps follow until
 * one certifies the fixed point. */

typedef struct {
  int precision;         /* PDFS_PREC_*                                           */
  int arith;             /* PDFS_ARITH_* (FP64 sweeps)                            */
  int freeze;            /* PDFS_FREEZE_*                                         */
  int scheduler;         /* PDFS_SCHED_*                                          */
  double tol;            /* FP64 convergence: stop at a full sweep whose max
                            |u_new - u_old| <= tol                                */
  int max_sweeps;        /* bound on sweeps of each phase (0 = 100000)             */
  int fixed_sweeps;      /* > 0: run exactly this many sweeps, orderings 1,2,..,8,1,..
                            with no convergence test (run_fsm semantics)          */
  int first_ordering;    /* 1..8: ordering of the first sweep (0 = 1)               */
  int tile;              /* sweep tile variant (0 = autotuned choice)               */
  int device;            /* CUDA device ordinal                                   */
  const float *mlp_weights; /* PDFS_SCHED_LEARNED: packed bf16-exact FP32 weights,
                               NULL = the weights compiled into the library        */
  long long spin_limit;  /* bound on polls of an inter-tile wait (0 = default)       */
  int verbose;           /* 0 quiet, 1 per-phase summary on stderr                 */
  int reserved[8];
} pdfs_opts;

typedef struct {
  int status;
  int sweeps_fp32;            /* FP32 sweeps run                                    */
  int sweeps_fp64;            /* FP64 sweeps run                                    */
  int full_sweeps;            /* sweeps that visited every block                    */
  long long voxel_updates;    /* node updates executed (skipped blocks excluded)   */
  long long blocks_skipped;   /* 8^3 blocks skipped by the scheduler, all sweeps   */
  double final_change;        /* max change of the last sweep                       */
  double ms_total;            /* wall time of the call                              */
  double ms_h2d, ms_d2h;      /* host<->device copies (host pointers only)          */
  double ms_fp32, ms_fp64;    /* device time of the two sweep phases                */
  double ms_sched;            /* device time of scheduler inference                 */
  double ms_kern_fp32;        /* summed durations of the FP32 sweep kernels alone    */
  double ms_kern_fp64;        /* summed durations of the FP64 sweep kernels alone    */
  int tile;                   /* tile variant used (FP32 id | FP64 id << 8)         */
  int launches;               /* kernels this call launched                          */
  double ms_device;           /* pdfs_ctx_run: device time from its first to its last
                                 kernel (CUDA events on the context's stream)        */
  long long voxel_updates_fp64; /* the part of voxel_updates done by FP64 sweeps     */
  /* the block-masked (scheduled) sweeps, a part of the sums above: their
   * kernels' summed durations and the node updates they executed */
  double ms_kern_masked_fp32, ms_kern_masked_fp64;
  long long updates_masked_fp32, updates_masked_fp64;
  int masked_sweeps_fp32, masked_sweeps_fp64;
} pdfs_stats;

/* Fills *o with the defaults: FP64, reference arithmetic, no freezing, no
 * scheduler, tol = 0 (exact fixed point), device 0. */
void pdfs_default_opts(pdfs_opts *o);

/* Solves |grad u| = 1 on the grid, in place.  field and frozen may be host
 * or device pointers (frozen may be NULL; it is read only with
 * PDFS_FREEZE_MASK).  Replaces run_fsm (single_gpu_cuda/src/phi3D_fsm.cu:64-106)
 * with a convergent, status-returning call. */
int pdfs_solve(const pdfs_grid *g, double *field, const uint8_t *frozen, const pdfs_opts *o,
               pdfs_stats *stats);

/* One ordering sn (1..8) of the plain FSM, in place: the GPU counterpart of
 * runFSM(pf, sn) (mpi_openacc/src/phi3D_fsm.c:67).  *max_change (nullable)
 * receives the sweep's max |u_new - u_old|.  o may be NULL (FP64 reference
 * arithmetic). */
int pdfs_sweep(const pdfs_grid *g, double *field, const uint8_t *frozen, int sn, const pdfs_opts *o,
               double *max_change);

/* ---- device-resident context ----------------------------------------------------
 * A context owns the device buffers of one grid so repeated solves re-use
 * them.  pdfs_solve() is create + load + run + store + destroy. */
typedef struct pdfs_ctx pdfs_ctx;

int pdfs_ctx_create(const pdfs_grid *g, const pdfs_opts *o, pdfs_ctx **out);
/* Copies the input field (and mask) into the context; host or device pointers. */
int pdfs_ctx_load(pdfs_ctx *c, const double *field, const uint8_t *frozen);
/* Solves from the loaded input; the input stays resident, so it can be re-run. */
int pdfs_ctx_run(pdfs_ctx *c, pdfs_stats *stats);
/* Copies the solution into field (host or device pointer, reference layout). */
int pdfs_ctx_store(pdfs_ctx *c, double *field);
/* Frees the context.  Its device blocks go to a per-process cache (at most a
 * quarter of the device's memory), from which the next context of about the
 * same size takes them: repeated solves skip cudaMalloc and cudaFree. */
void pdfs_ctx_destroy(pdfs_ctx *c);
/* Returns every cached block of the device to CUDA (for callers that need
 * the memory elsewhere).  Contexts still alive keep their blocks. */
int pdfs_release_cached(int device);

/* The 8^3 node blocks of a context's grid: nbx = ceil(nx/8), nby, nbz alike.
 * Block (bx, by, bz) has index (bz*nby + by)*nbx + bx and holds interior
 * nodes x = 8bx+1 .. 8bx+8 (and likewise in y and z). */
int pdfs_ctx_blocks(const pdfs_ctx *c, int *nbx, int *nby, int *nbz);

/* One ordering sn (1..8) on the context's working field, continuing from the
 * previous pdfs_ctx_sweep; the first call after pdfs_ctx_load starts from the
 * input.  FP32 min-update if opts.precision is PDFS_PREC_FP32, else FP64
 * min-update.  active (nullable; host or device; one byte per block): nodes
 * of blocks with active[b] == 0 keep their values.  block_change (nullable;
 * host or device; one float per block) receives each block's max change
 * (FP32: relative, FP64: absolute), *max_change the sweep's.  pdfs_ctx_store
 * reads the field.  No counterpart in the reference, which sweeps every node
 * (phi3D_fsm.c:83-119): this is the building block of block schedulers and
 * of the traces their models learn from. */
int pdfs_ctx_sweep(pdfs_ctx *c, int sn, const uint8_t *active, float *block_change, double *max_change);

/* Per 8^3 block, the orderings that matter to it, from the context's FP32
 * working field (after a PDFS_PREC_FP32 run or sweeps, or the FP32 phase of a
 * PDFS_PREC_FP32_POLISH64 run): bit sn-1 of orderings[b] is set where, at some
 * updated node of the block, every axis the Godunov update uses has its
 * smaller neighbour on the side ordering sn sweeps from (an axis the update
 * does not use, or whose neighbours differ by at most h/4, accepts both), or
 * where that holds in the face-neighbour block ordering sn sweeps into the
 * block from (along any axis).  These are the masks of the
 * FP32 octant rounds (PDFS_SCHED_OCTANT); the polish's round uses a band of
 * h/20 instead of h/4.  orderings: one byte per block,
 * host or device.  PDFS_ERR_INVALID for a context without an FP32 field. */
int pdfs_ctx_orderings(pdfs_ctx *c, uint8_t *orderings);

/* Solves n independent grids together (the batched configuration).  On
 * pencil tiles (the default; brick and lane-column tiles map to it) each
 * round of 8 orderings is ONE persistent launch over the pencils of every
 * grid still sweeping; on column tiles (asked for in opts.tile) each sweep is
 * one launch.  Rounds after the first replay a CUDA graph, and a grid leaves
 * once one of its sweeps changes by <= the phase tolerance (the round's
 * later sweeps still run on it).
 * fields[i] / frozen[i] as in pdfs_solve (frozen may be NULL, or hold NULL
 * entries).  stats: NULL or n entries.  opts.fixed_sweeps must be 0 and the
 * scheduler is not used.  Returns the first failing grid's status. */
int pdfs_solve_batch(int n, const pdfs_grid *grids, double *const *fields, const uint8_t *const *frozen,
                     const pdfs_opts *o, pdfs_stats *stats);

/* Times the sweep tile variants on grid g (two sweeps each, synthetic field)
 * and returns the fastest pair as an opts.tile value (FP32 id | FP64 id << 8). */
int pdfs_autotune(const pdfs_grid *g, const pdfs_opts *o, int *tile);

/* ---- learned active-block scheduler ---------------------------------------------
 * No counterpart in the reference (it sweeps every node).  A small MLP
 * predicts, per 8^3 block, whether the block changes by more than the
 * phase's tolerance in the next sweep.  PDFS_SCHED_LEARNED asks it about the
 * blocks the history rule of PDFS_SCHED_CHANGE nominates, sweeps the ones
 * it predicts active, and certifies the answer with full sweeps.
 *
 * Network: 16 features -> 64 (ReLU) -> 64 (ReLU) -> 1 logit; weights and
 * activations in bf16, every sum accumulated in FP32.  Parameter order
 * (row-major, [out][in]): W1[64][16], b1[64], W2[64][64], b2[64], w3[64], b3.
 * A weight blob (opts.mlp_weights) is PDFS_MLP_PARAMS floats, each a bf16
 * value, followed by the decision threshold on the logit.
 *
 * Features of block b before sweep s of a phase (ordering sn, phase
 * tolerance tol; ck = the block's max change in sweep s-k, 0 before the
 * phase's first sweep; L(c) = clamp(log2(c/tol), -32, 32)/16 for c > 0,
 * else -2):
 *   0 band: log2(1 + min(field over b) / (8 h)) / 8   (h = smallest spacing)
 *   1 L(c1)   2 L(c2)
 *   3 age / 9: the least k in 1..8 with ck > tol, else 9
 *   4 phase (0 FP32 bulk, 1 FP64 polish)   5 min(s, 64) / 64
 *   6..13 one-hot of sn
 *   14 L(max c1 of the 3 face neighbours upwind of b in ordering sn)
 *   15 L(c8): the block's change one cycle of orderings ago
 * Label: the block's max change in sweep s > tol. */
#define PDFS_MLP_IN 16
#define PDFS_MLP_HIDDEN 64
#define PDFS_MLP_PARAMS (64 * 16 + 64 + 64 * 64 + 64 + 64 + 1)
#define PDFS_MLP_BLOB (PDFS_MLP_PARAMS + 1)

/* Trainer: collects (features, label) samples from plain solves on the GPU
 * and fits the network with the library's own bf16 forward / backward /
 * Adam kernels. */
typedef struct pdfs_mlp_trainer pdfs_mlp_trainer;
int pdfs_mlp_trainer_create(int device, unsigned seed, pdfs_mlp_trainer **out);
/* Solves (g, field, frozen) with every block swept -- FP32 to its fixed
 * point, then the FP64 polish to o->tol when o->precision is
 * PDFS_PREC_FP32_POLISH64; FP64 to o->tol when it is PDFS_PREC_FP64 (the
 * phase feature is 1 for both FP64 phases) -- and, from the ninth sweep of each phase on
 * (where the schedulers start), records one sample per block the history
 * rule nominates.  *samples (nullable) receives the trainer's total. */
int pdfs_mlp_trainer_add_solve(pdfs_mlp_trainer *t, const pdfs_grid *g, const double *field, const uint8_t *frozen,
                               const pdfs_opts *o, long long *samples);
/* Adam over the collected samples in shuffled mini-batches; positives
 * weigh pos_weight.  *loss (nullable) receives the last epoch's mean
 * weighted cross-entropy. */
int pdfs_mlp_trainer_fit(pdfs_mlp_trainer *t, int epochs, int batch, float lr, float pos_weight, float *loss);
/* The trained weights as a blob; the threshold is set so that the given
 * fraction of the positive samples is predicted active.  *recall_out and
 * *active_out (nullable) receive the recall and the predicted-active
 * fraction on the collected samples. */
int pdfs_mlp_trainer_weights(pdfs_mlp_trainer *t, float recall, float *blob, float *recall_out, float *active_out);
void pdfs_mlp_trainer_destroy(pdfs_mlp_trainer *t);

/* Kernel-level entry points (host pointers), for gradient checks: n samples
 * of bf16 features x[n][16] and labels y[n].  grad receives the gradient of
 * the mean weighted cross-entropy (PDFS_MLP_PARAMS floats), loss the loss. */
int pdfs_mlp_grad(const float *params, const uint16_t *x, const uint8_t *y, int n, float pos_weight, float *grad,
                  float *loss);
/* One Adam step (bias-corrected, step >= 1) on FP32 master parameters with
 * moments m and v; params_bf16 (nullable) receives the bf16 copy. */
int pdfs_mlp_adam(float *params, float *m, float *v, const float *grad, int step, float lr, float beta1, float beta2,
                  float eps, uint16_t *params_bf16);
/* Logits of n samples under a blob (the fused inference arithmetic). */
int pdfs_mlp_infer(const float *blob, const uint16_t *x, int n, float *logits);

/* ---- allocation-free sweep ----------------------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory while they run: code that executes inside a pre-sized memory pool
 * or arena handed to it by a host application, real-time or embedded loops
 * that must not call the allocator after start-up (cudaMalloc can block and
 * synchronise the device), and plugins whose host process forbids device
 * allocation after its own set-up.  pdfs_sweep_static() runs one ordering
 * of the plain FSM (FP64, the reference's arithmetic, every node
 * min-updated: the same result as pdfs_sweep) without calling cudaMalloc,
 * cudaFree or any allocating routine.  Its scratch -- column progress words,
 * the column ticket, the status words and the face mailboxes -- lives in one
 * fixed device array of PDFS_STATIC_SCRATCH_BYTES that every GPU which loads
 * the library keeps until the process exits.  The caller passes the field.
 *
 * Field: a device array in the sweep's internal layout.  Node (x, y, z) of
 * the halo-padded grid (0 <= x <= nx+1, ...) is element
 * z*ry*px + y*px + x + 1; pdfs_static_layout() gives px, ry and the element
 * count; entries outside the halo-padded grid are not read for any result
 * (fill them with +inf).
 *
 * The first call in a device's context looks up the array's device address
 * (once per context, with that device current; after a cudaDeviceReset the
 * next call looks it up again); make that first call before any stream
 * capture.  CUDA loads modules lazily by default, so the array itself is
 * reserved during that first call: make one call (a 1 x 1 x 1 grid will do)
 * on each device during set-up, before the phase in which nothing may be
 * allocated.  The wait bound and the test hook of the allocating path apply
 * (PDFS_WAIT_MS, PDFS_TEST_POISON_COLUMN; a wait that gives up returns
 * PDFS_ERR_TIMEOUT).  Every call shares the one array and leaves its contents behind:
 * each call clears the words that must start at zero, but calls whose work
 * overlaps on the GPU (concurrent streams, other host threads) race on it and
 * must be serialised by the caller. */
#define PDFS_STATIC_SCRATCH_BYTES (32ull << 20)

/* Internal layout of the field for pdfs_sweep_static: row pitch px, rows per
 * plane ry, total elements, and the scratch bytes the grid needs.  Returns
 * PDFS_ERR_TOO_LARGE if the scratch exceeds PDFS_STATIC_SCRATCH_BYTES. */
int pdfs_static_layout(const pdfs_grid *g, long long *px, long long *ry, long long *elems,
                       long long *scratch_bytes);

/* One ordering sn (1..8), in place on field_dev, on `stream` (a
 * cudaStream_t, NULL = the default stream); waits for the stream, then
 * stores the sweep's max change in *max_change (nullable). */
int pdfs_sweep_static(const pdfs_grid *g, double *field_dev, int sn, double *max_change, void *stream);

/* Human-readable text of a status code (static storage). */
const char *pdfs_status_string(int status);
/* Library version string. */
const char *pdfs_version(void);

#ifdef __cplusplus
}
#endif
#endif /* PDFS_H */
