"""Benchmark of the GB300 FSM distance-field solve.

Metric (the reference's headline, printed identically by both arms):
time-to-converge and Gvoxel-updates/s of the block-scheduled FP32-bulk +
FP64-precision-polish solve against the plain FP64 FSM, at <= 1e-6
relative error (the octant scheduler by default; the none, history-rule and
learned schedulers are timed beside it).  Gvox-updates/s are plain-equivalent: the plain FP64 FSM's
node updates on the same input (interior nodes x its sweep count) divided by
the time to converge.  The reference arm runs the plain FP64 FSM itself, so
its rate is its own per-ordering rate.

One step = one complete solve of the workload to convergence, from the input
already resident in HBM (pdfs_ctx_run), timed on the device by CUDA events
on the solve's stream.  e2e = the same through pdfs_solve() with pinned host
buffers, host<->device copies and layout passes inside the timed region,
averaged over the same number of steps.

Default workload: 768^3, dx = 1, union of 150 seeded spheres (radii
log-uniform 4..50 cells), interface nodes frozen; inputs (3.6 GB) are larger
than L2 (129 MB), so no flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload C4|C2|C3|C1|spheresN] [--mode polish|fp32|fp64|fp64ref]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402


METRIC = "time-to-converge & Gvox-updates/s: scheduled FP32+polish vs plain FP64 FSM at 1e-6 err"
UNIT = "Gvox-updates/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="C4")
    p.add_argument("--mode", default="polish", choices=["polish", "fp32", "fp64", "fp64ref"])
    p.add_argument("--scheduler", default="octant", choices=["none", "change", "learned", "octant"])
    p.add_argument("--tol", type=float, default=1e-5, help="FP64 polish tolerance (max change)")
    p.add_argument("--polish-arith", default="pair", choices=["mixed", "pair", "fast"],
                   help="polish arithmetic: FP32 increments over an FP64 field (mixed) or an FP32-pair "
                        "field (pair), or all FP64 (fast)")
    p.add_argument("--no-sched-table", action="store_true", help="skip timing the three schedulers")
    p.add_argument("--configs", action="store_true",
                   help="accuracy report: every config's FP32 + polish solve against the plain FP64 FSM")
    p.add_argument("--config-list", default="", help="--configs: which configs (comma-separated, default C1..C4)")
    p.add_argument("--tile", type=int, default=0)
    p.add_argument("--fixed-sweeps", type=int, default=0, help="profiling: run exactly this many sweeps")
    p.add_argument("--no-plain", action="store_true", help="skip the plain FP64 FSM comparison solve")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    p.add_argument("--no-fp64-polish", action="store_true", help="skip the all-FP64 polish comparison solve")
    p.add_argument("--cpu-sweeps", type=int, default=0, help="CPU sample: sweeps of the full grid")
    return p.parse_args()


def workload(name, seed=0):
    from pdfs_gb300 import workloads as W
    if name.startswith("spheres"):
        n = int(name[len("spheres"):])
        return W.random_spheres(n, n, n, 1.0, 1.0, 1.0, max(8, int(150 * (n / 768) ** 3)), 4.0,
                                max(6.0, 50.0 * n / 768), seed=seed + 4, name=f"spheres_{n}^3")
    return W.config(name, seed=seed)


# ---- distributed plumbing (one process per GPU; replicas: the single-grid path does not shard) ----
def dist_init(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        backend = "nccl"
        try:
            import torch
            if not torch.cuda.is_available():
                backend = "gloo"
            else:
                torch.cuda.set_device(local)
        except Exception:
            backend = "gloo"
        dist.init_process_group(backend=backend)
        pg = dist
    return rank, world, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, v):
    if pg is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.p = None
        self.lines = []

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.p = None

    def _read(self):
        for line in self.p.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.p:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.t.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return {}


# sweep kernel variants by tile id: columns (TY, rows per warp), bricks (BY, BZ), pencils
COLUMNS32 = {1: (8, 2), 2: (8, 4), 3: (16, 4), 4: (8, 1), 5: (4, 2), 6: (6, 1), 7: (10, 1)}
COLUMNS64 = {1: (4, 1), 2: (4, 2), 3: (8, 2), 4: (6, 1)}
BRICKS32 = {8: (16, 16), 9: (16, 32), 11: (8, 48)}
BRICKS64 = {5: (16, 16), 7: (16, 32), 8: (8, 32)}
PENCILS32, PENCILS64 = (10,), (6,)
LANECOL32, LANECOL64 = {12: 8, 13: 4}, {9: 8, 10: 4}  # lane-column tiles: rows per tile


def kernel_kind(kind, tile):
    t = tile & 0xff if kind == "fp32" else tile >> 8
    if t in (LANECOL32 if kind == "fp32" else LANECOL64):
        return "lanecol"
    if t in (BRICKS32 if kind == "fp32" else BRICKS64):
        return "brick"
    if t in (PENCILS32 if kind == "fp32" else PENCILS64):
        return "pencil"
    return "column"


def kernel_name(kind, tile, prec, arith):
    """The dominant sweep kernel's template name, as ncu lists it."""
    from pdfs_gb300 import _lib as L
    mode = "MIN" if kind == "fp32" or prec != L.PREC_FP32_POLISH64 else "REPLACE"
    ar = "FAST" if kind == "fp32" else {L.ARITH_MIXED: "MIXED", L.ARITH_PAIR: "PAIR",
                                        L.ARITH_FAST: "FAST"}.get(arith, "REF")
    t = "float" if kind == "fp32" else "double"
    tid = tile & 0xff if kind == "fp32" else tile >> 8
    k = kernel_kind(kind, tile)
    if k == "brick":
        by, bz = (BRICKS32 if kind == "fp32" else BRICKS64)[tid]
        return "t3_sweep_kernel<%s, %d, %d, %s, %s>" % (t, by, bz, mode, ar)
    if k == "pencil":
        return "pc_sweep_kernel<%s, %s, %s>" % (t, mode, ar)
    if k == "lanecol":
        rows = (LANECOL32 if kind == "fp32" else LANECOL64)[tid]
        return "lc_sweep_kernel<%s, %d, %s>" % (t, rows, mode)
    ty = (COLUMNS32 if kind == "fp32" else COLUMNS64).get(tid, (0, 0))
    return "ws_sweep_kernel<%s, %d, %d, %s, %s>" % ((t,) + ty + (mode, ar))


def traffic_per_launch(kind, prec, nodes, tile, masked=False, full_round=False):
    """DRAM bytes of one launch of the dominant sweep kernel: the per-update
    traffic an ncu capture measured (profiles/traffic.json, dram__bytes_read
    + dram__bytes_write over the capture's executed voxel updates) times this
    launch's updates; None without a capture for that kernel.  masked: the
    block-masked sweeps (bricks), whose traffic per executed update differs
    from a full sweep's; full_round: the FP32 first cycle as one unmasked round."""
    from pdfs_gb300 import _lib as L
    try:
        t = json.load(open(os.path.join(ROOT, "profiles", "traffic.json")))
    except (OSError, ValueError):
        return None
    key = "fp32" if kind == "fp32" else ("fp64_replace" if prec == L.PREC_FP32_POLISH64 else "fp64_min")
    key += "_masked_brick" if masked else ("_round" if full_round else "_" + kernel_kind(kind, tile))
    e = t.get(key)
    return None if not e else float(e["dram_bytes_per_update"]) * nodes


def _cpu_fsm(w, threads):
    """The reference's CPU FSM path for one ordering of the full grid:
    its own OpenACC loop built for host multicore (oracle/_ref, where the
    reference's sources were present to build it), else the oracle port (OpenMP
    over each hyperplane).  Returns (sweep(a, sn), kind, what)."""
    from oracle import oracle as O
    sp = (w.dx, w.dy, w.dz)
    O.build(ref=False)
    if O.have_ref(omp=True):
        os.environ.setdefault("OMP_NUM_THREADS", str(threads))
        return (lambda a, sn: O.ref_sweep_raw(a, sp, sn, omp=True)), "reference", \
            "the reference's mpi_openacc phi3D_fsm.c, OpenACC loop as OpenMP (interface not frozen: it has no mask)"
    return (lambda a, sn: O.sweep(a, sp, sn, frozen=w.frozen, threads=threads)), "port", \
        "the oracle port of the reference's FSM (OpenMP over hyperplanes)"


def cpu_baseline(w, sweeps, threads):
    """The reference's CPU FSM path timed on the host cores on `sweeps`
    orderings of the full grid."""
    run, kind, what = _cpu_fsm(w, threads)
    a = w.field.copy()
    t0 = time.perf_counter()
    for s in range(sweeps):
        run(a, s % 8 + 1)
    dt = time.perf_counter() - t0
    return w.interior * sweeps / dt / 1e9, dt, kind, what


def run_reference(args, rank, world, pg):
    """Reference arm: the reference's CPU FSM path on the host cores, one
    ordering of the full grid per step.  The plain FP64 FSM's plain-equivalent
    rate is its own rate, so the line carries the same metric and unit as our
    arm's."""
    if rank != 0:
        return
    w = workload(args.workload)
    threads = os.cpu_count() or 1
    run, kind, what = _cpu_fsm(w, threads)
    a = w.field.copy()
    for s in range(args.warmup):
        run(a, s % 8 + 1)
    times = []
    for s in range(args.steps):
        t0 = time.perf_counter()
        run(a, (args.warmup + s) % 8 + 1)
        times.append(time.perf_counter() - t0)
    t = float(np.mean(times))
    v = w.interior / t / 1e9
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": w.name, "nx": w.nx, "ny": w.ny, "nz": w.nz, "parallelism": "host threads",
                       "step": "one plain FP64 ordering of the full grid"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": kind,
                             "sample": f"one FP64 ordering over the full {w.nx}x{w.ny}x{w.nz} grid per step: {what}"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_batch(args, rank, world, pg, device):
    """C5: 256 independent grids (per-axis sizes log-uniform 32..256, 1..20
    spheres; under torchrun every rank solves its own batch, so value is the
    whole job's grids/s) solved in one batched solve -- persistent launches over a
    per-grid ticket table, rounds replayed from a CUDA graph -- against
    looping the plain FP64 solver (and our own single-grid solve) over them.
    Host buffers on both sides (the batch API takes host or device fields)."""
    from pdfs_gb300 import _lib as L
    from pdfs_gb300 import api
    from pdfs_gb300 import workloads as W
    ws = W.batch_c5()
    sps = [(w.dx, w.dy, w.dz) for w in ws]
    nodes = sum(w.interior for w in ws)
    arith = {"mixed": L.ARITH_MIXED, "pair": L.ARITH_PAIR}.get(args.polish_arith, L.ARITH_FAST)
    kw = dict(freeze=L.FREEZE_MASK, precision=L.PREC_FP32_POLISH64, arith=arith, tol=args.tol, device=device)
    import torch
    dev = torch.device("cuda", device)
    # value: the inputs resident in HBM (device tensors; each step reloads them
    # from a pristine device copy outside the timed region)
    d_in = [torch.from_numpy(w.field).to(dev) for w in ws]
    d_fz = [torch.from_numpy(w.frozen).to(dev) for w in ws]
    d_work = [x.clone() for x in d_in]
    for _ in range(max(3, args.warmup)):
        for a, b in zip(d_work, d_in):
            a.copy_(b)
        torch.cuda.synchronize()
        api.solve_batch(d_work, sps, frozen=d_fz, **kw)
    dtimes, dst = [], None
    for _ in range(args.steps):
        for a, b in zip(d_work, d_in):
            a.copy_(b)
        torch.cuda.synchronize()
        barrier(pg)
        t0 = time.perf_counter()
        dst = api.solve_batch(d_work, sps, frozen=d_fz, **kw)
        torch.cuda.synchronize()
        dtimes.append(time.perf_counter() - t0)
    t_dev = max_over_ranks(pg, float(np.mean(dtimes)))
    del d_in, d_fz, d_work
    # e2e: host buffers through the same call (host<->device copies inside)
    api.solve_batch([w.field.copy() for w in ws], sps, frozen=[w.frozen for w in ws], **kw)
    times, outs = [], None
    for _ in range(args.steps):
        fs = [w.field.copy() for w in ws]
        barrier(pg)
        t0 = time.perf_counter()
        st = api.solve_batch(fs, sps, frozen=[w.frozen for w in ws], **kw)
        times.append(time.perf_counter() - t0)
        outs = fs
    t_batch = max_over_ranks(pg, float(np.mean(times)))
    # looping the plain FP64 solver (the reference's method, on the GPU)
    t0 = time.perf_counter()
    plain_sweeps, err = 0, 0.0
    for w, o in zip(ws, outs):
        ref = w.field.copy()
        ps = api.solve(ref, (w.dx, w.dy, w.dz), frozen=w.frozen, freeze=L.FREEZE_MASK, precision=L.PREC_FP64,
                       arith=L.ARITH_FAST, tol=1e-12, device=device)
        plain_sweeps += ps["sweeps_fp64"] * w.interior
        i = (slice(1, -1),) * 3
        err = max(err, float(np.max(np.abs(o[i] - ref[i]) / np.maximum(np.abs(ref[i]), 1.0))))
    t_plain = time.perf_counter() - t0
    # looping our own single-grid solve
    t0 = time.perf_counter()
    for w in ws:
        api.solve(w.field.copy(), (w.dx, w.dy, w.dz), frozen=w.frozen, **kw)
    t_loop = time.perf_counter() - t0
    # the same batch on column tiles: one launch per sweep, mixed polish
    kc = dict(kw, tile=4 | (4 << 8), arith=L.ARITH_MIXED)
    api.solve_batch([w.field.copy() for w in ws], sps, frozen=[w.frozen for w in ws], **kc)
    t0 = time.perf_counter()
    api.solve_batch([w.field.copy() for w in ws], sps, frozen=[w.frozen for w in ws], **kc)
    t_cols = time.perf_counter() - t0
    if rank == 0:
        line = {
            "metric": "grids/s of the batched FP32 + FP64-polish solve (256 grids) vs looping the plain FP64 solver",
            "value": world * len(ws) / t_dev, "unit": "grids/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_dev * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f32pair" if arith == L.ARITH_PAIR else "f32+f64",
            "data": "synthetic (seeded spheres)",
            "config": {"workload": "C5_256_grids_32-256", "grids": len(ws), "interior_nodes": nodes,
                       "polish_tol": args.tol, "polish_arith": args.polish_arith,
                       "l2": "inputs larger than L2 (no flush needed)"},
            "gvox_updates_per_s_plain_equivalent": plain_sweeps / t_dev / 1e9,
            "inputs": "device tensors (value); host arrays (e2e)",
            "device_step_ms": {"total": t_dev * 1e3, "sweep_kernels": dst[0]["ms_kern_fp32"] + dst[0]["ms_kern_fp64"],
                               "fp32_kernels": dst[0]["ms_kern_fp32"], "fp64_kernels": dst[0]["ms_kern_fp64"]},
            "plain_fp64_loop": {"grids_per_s": len(ws) / t_plain, "time_s": t_plain},
            "own_single_grid_loop": {"grids_per_s": len(ws) / t_loop, "time_s": t_loop},
            "batch_on_columns": {"grids_per_s": len(ws) / t_cols, "time_s": t_cols,
                                 "kernel": "columns 32x8 / mixed polish, one launch per sweep"},
            "batch_kernel": "pencil rounds: one launch per round of 8 orderings over every grid",
            "launches_per_step": int(max(x["launches"] for x in st)),
            "speedup_vs_plain_loop": t_plain / t_batch, "max_rel_err_vs_plain": err,  # both from host arrays
            "sweeps_per_grid": {"fp32": float(np.mean([x["sweeps_fp32"] for x in st])),
                                "fp64": float(np.mean([x["sweeps_fp64"] for x in st]))},
            "e2e": {"value": world * len(ws) / t_batch, "unit": "grids/s", "ms_per_step": t_batch * 1e3,
                    "h2d_bytes_per_step": int(world * sum(w.field.nbytes + w.frozen.nbytes for w in ws)),
                    "d2h_bytes_per_step": int(world * sum(w.field.nbytes for w in ws))},
            "roofline": None, "cpu_baseline": None,
            "gpu_launches": int(max(x["launches"] for x in st)),  # one batched launch serves every grid
        }
        print(json.dumps(line), flush=True)


def run_configs(args, device):
    """One JSON line per config (C1..C4): against the oracle's FP64 plain-FSM
    fixed point (tol 1e-12, every host core), the max and RMS relative error
    of the plain FP64 GPU solve, the FP32 + pair-polish, FP32 + FP64-polish
    and FP32-only solves, and the learned-scheduler headline solve, with their
    times end to end through pdfs_solve (host buffers).  C1 also runs the FP64
    reference arithmetic, which must be bit-exact."""
    from oracle import oracle as O
    from pdfs_gb300 import _lib as L
    from pdfs_gb300 import api
    from pdfs_gb300 import workloads as W
    threads = os.cpu_count() or 1
    names = args.config_list.split(",") if args.config_list else ["C1", "C2", "C3", "C4"]
    for name in names:
        w = W.config(name)
        sp = (w.dx, w.dy, w.dz)
        h = min(sp)
        fz = dict(frozen=w.frozen, freeze=L.FREEZE_MASK, device=device)
        orc = w.field.copy()
        t0 = time.perf_counter()
        o_sweeps, _ = O.solve(orc, sp, tol=1e-12, frozen=w.frozen, threads=threads)
        t_orc = time.perf_counter() - t0
        i = (slice(1, -1),) * 3
        den = np.maximum(np.abs(orc[i]), h)

        def err(f):
            e = np.abs(f[i] - orc[i]) / den
            return float(e.max()), float(np.sqrt(np.mean(e * e)))

        out = {"config": name, "workload": w.name, "nx": w.nx, "ny": w.ny, "nz": w.nz, "spacing": list(sp),
               "oracle": {"sweeps": o_sweeps, "time_s": t_orc, "threads": threads, "tol": 1e-12}}
        cases = [("plain_fp64_fast", dict(precision=L.PREC_FP64, arith=L.ARITH_FAST, tol=1e-12)),
                 ("fp32_polish_pair", dict(precision=L.PREC_FP32_POLISH64, arith=L.ARITH_PAIR, tol=1e-5 * h)),
                 ("fp32_polish_pair_learned", dict(precision=L.PREC_FP32_POLISH64, arith=L.ARITH_PAIR,
                                                   tol=1e-5 * h, scheduler=L.SCHED_LEARNED)),
                 ("fp32_polish_pair_octant", dict(precision=L.PREC_FP32_POLISH64, arith=L.ARITH_PAIR,
                                                  tol=1e-5 * h, scheduler=L.SCHED_OCTANT)),
                 ("fp32_polish_fp64", dict(precision=L.PREC_FP32_POLISH64, arith=L.ARITH_FAST, tol=1e-5 * h)),
                 ("fp32_only", dict(precision=L.PREC_FP32))]
        if name in ("C1", "C2"):
            cases.append(("fp64_reference_arith", dict(precision=L.PREC_FP64, arith=L.ARITH_REFERENCE, tol=1e-12)))
        t_plain = None
        for label, kw in cases:
            f = w.field.copy()
            api.solve(f, sp, **kw, **fz)  # warm (allocations, module loads)
            f[:] = w.field
            t0 = time.perf_counter()
            st = api.solve(f, sp, **kw, **fz)
            t = time.perf_counter() - t0
            mx, rms = err(f)
            out[label] = {"max_rel_err": mx, "rms_rel_err": rms, "sweeps_fp32": st["sweeps_fp32"],
                          "sweeps_fp64": st["sweeps_fp64"], "time_s": t, "run_ms_device": st["ms_device"]}
            if label == "plain_fp64_fast":
                t_plain = t
            elif t_plain:
                out[label]["speedup_vs_plain_fp64"] = t_plain / t
            if label == "fp64_reference_arith":
                out[label]["bit_exact"] = bool(f.tobytes() == orc.tobytes())
            del f
        print(json.dumps(out), flush=True)
        del w, orc, den


def main():
    args = parse()
    rank, world, local, pg = dist_init(args)
    if args.configs:
        from pdfs_gb300 import build as B
        B.build()
        if rank == 0:
            run_configs(args, local)
        return
    if args.impl == "reference":
        run_reference(args, rank, world, pg)
        return
    if args.workload == "C5":
        from pdfs_gb300 import build as B
        B.build()
        run_batch(args, rank, world, pg, local)
        if pg is not None:
            pg.destroy_process_group()
        return
    from pdfs_gb300 import _lib as L
    from pdfs_gb300 import api
    from pdfs_gb300 import build as B
    B.build()
    device = local
    w = workload(args.workload)
    sp = (w.dx, w.dy, w.dz)
    freeze = L.FREEZE_MASK
    prec = {"polish": L.PREC_FP32_POLISH64, "fp32": L.PREC_FP32, "fp64": L.PREC_FP64,
            "fp64ref": L.PREC_FP64}[args.mode]
    arith = L.ARITH_REFERENCE if args.mode == "fp64ref" else L.ARITH_FAST
    if args.mode == "polish" and args.polish_arith in ("mixed", "pair"):
        arith = L.ARITH_MIXED if args.polish_arith == "mixed" else L.ARITH_PAIR
    sched = {"none": L.SCHED_NONE, "change": L.SCHED_CHANGE, "learned": L.SCHED_LEARNED,
             "octant": L.SCHED_OCTANT}[args.scheduler]
    if args.mode in ("fp64", "fp64ref"):
        sched = L.SCHED_NONE
    opts = dict(precision=prec, arith=arith, freeze=freeze, scheduler=sched, tol=args.tol, tile=args.tile,
                fixed_sweeps=args.fixed_sweeps, device=device)
    ctx = api.Context(w.nx, w.ny, w.nz, sp, **opts)
    ctx.load(w.field, w.frozen)
    for _ in range(args.warmup):
        ctx.run()
    clocks = Clocks(device)
    barrier(pg)
    clocks.start()
    t0 = time.perf_counter()
    stats = []
    for _ in range(args.steps):
        # each run synchronises its stream before returning; ms_device is the
        # run's CUDA-event time on the solve's stream, first kernel to last
        stats.append(ctx.run())
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    barrier(pg)
    t_dev = sum(x["ms_device"] for x in stats) / 1e3
    t_dev = max_over_ranks(pg, t_dev)
    wall = max_over_ranks(pg, wall)
    t_step = t_dev / args.steps
    out = np.empty_like(w.field)
    ctx.store(out)
    ctx.close()
    st = stats[-1]
    i = (slice(1, -1),) * 3

    # plain FP64 FSM on the same input: sweep count (for the plain-equivalent
    # rate), its time, and the error of our answer against it
    plain, ref = None, None
    if not args.no_plain and args.fixed_sweeps == 0:
        ref = w.field.copy()
        ps = api.solve(ref, sp, frozen=w.frozen, freeze=freeze, precision=L.PREC_FP64, arith=L.ARITH_FAST,
                       tol=1e-12, device=device)
        e = np.abs(out[i] - ref[i]) / np.maximum(np.abs(ref[i]), min(sp))
        plain = {"sweeps": ps["sweeps_fp64"], "time_s": (ps["ms_fp64"] + 0.0) / 1e3,
                 "kernel_ms": ps["ms_kern_fp64"], "max_rel_err_vs_plain": float(e.max()),
                 "rms_rel_err_vs_plain": float(np.sqrt(np.mean(e * e)))}
        del e
    plain_sweeps = plain["sweeps"] if plain else (st["sweeps_fp32"] + st["sweeps_fp64"])
    # whole-job aggregate: every rank solves its own replica of the workload
    # (a single grid does not shard), timed by the slowest rank
    value = world * w.interior * plain_sweeps / t_step / 1e9

    # the same solve with the polish in true FP64 arithmetic (ARITH_FAST), one warm run
    fp64_polish = None
    if (not args.no_fp64_polish and args.fixed_sweeps == 0 and args.mode == "polish"
            and args.polish_arith != "fast"):
        o2 = dict(opts, arith=L.ARITH_FAST)
        with api.Context(w.nx, w.ny, w.nz, sp, **o2) as c2:
            c2.load(w.field, w.frozen)
            c2.run()
            s2 = c2.run()
            o64 = np.empty_like(w.field)
            c2.store(o64)
        fp64_polish = {"time_s": s2["ms_device"] / 1e3, "sweeps_fp32": s2["sweeps_fp32"],
                       "sweeps_fp64": s2["sweeps_fp64"], "arith": "fast (FP64)"}
        if ref is not None:
            e = np.abs(o64[i] - ref[i]) / np.maximum(np.abs(ref[i]), min(sp))
            fp64_polish.update(max_rel_err=float(e.max()), rms_rel_err=float(np.sqrt(np.mean(e * e))))
            del e
        del o64

    # e2e through pdfs_solve with pinned host buffers, averaged over the timed steps
    e2e = None
    if not args.no_e2e and args.fixed_sweeps == 0:
        try:
            import torch
            hf = torch.empty(w.field.shape, dtype=torch.float64).pin_memory()
            hm = torch.empty(w.frozen.shape, dtype=torch.uint8).pin_memory()
            hf.numpy()[:] = w.field
            hm.numpy()[:] = w.frozen
            f_np, m_np = hf.numpy(), hm.numpy()
            pinned = True
        except Exception:
            f_np, m_np = w.field.copy(), w.frozen
            pinned = False
        api.solve(f_np, sp, frozen=m_np, **opts)  # warm
        ts = []
        for k in range(args.steps):
            f_np[:] = w.field  # the step's input, outside the timed region
            barrier(pg)
            t1 = time.perf_counter()
            api.solve(f_np, sp, frozen=m_np, **opts)
            ts.append(time.perf_counter() - t1)
        te = max_over_ranks(pg, float(np.mean(ts)))
        e2e = {"value": world * w.interior * plain_sweeps / te / 1e9, "unit": UNIT,
               "h2d_bytes_per_step": int(world * (w.field.nbytes + w.frozen.nbytes)),
               "d2h_bytes_per_step": int(world * w.field.nbytes), "time_to_converge_s": te,
               "steps": len(ts), "host_buffers": "pinned" if pinned else "pageable"}

    # roofline of the dominant kernel: the sweep kernels by phase and kind (full
    # sweeps on the tile's kernel, block-masked sweeps on bricks), each with its
    # executed updates, launches and summed CUDA-event durations
    pk = peaks()
    hbm = pk.get("hbm_gbs", 6800.0)
    mask_b = 1.0 / 8.0
    k32, k64 = st["ms_kern_fp32"], st["ms_kern_fp64"]
    s32, s64 = st["sweeps_fp32"], st["sweeps_fp64"]
    vu64 = st["voxel_updates_fp64"]
    vu32 = st["voxel_updates"] - vu64
    parts = []
    # octant rounds run a masked cycle of 8 sweeps as one launch
    per_round = 8 if args.scheduler == "octant" or (args.scheduler in ("change", "learned") and
                                                    prec == L.PREC_FP32_POLISH64) else 1
    for phase, kt, kmask, n, nmask, upd, umask, per in (
            ("fp32", k32, st["ms_kern_masked_fp32"], s32, st["masked_sweeps_fp32"], vu32,
             st["updates_masked_fp32"], 8 + mask_b),
            ("fp64", k64, st["ms_kern_masked_fp64"], s64, st["masked_sweeps_fp64"], vu64,
             st["updates_masked_fp64"], 16 + mask_b)):
        if n - nmask > 0:
            # the octant scheduler runs the FP32 phase's first cycle as one unmasked round
            full_round = phase == "fp32" and args.scheduler == "octant" and n - nmask >= 8
            parts.append({"phase": phase, "kind": "full", "ms": kt - kmask, "sweeps": n - nmask,
                          "launches": 1 + (n - nmask - 8) if full_round else n - nmask,
                          "updates": upd - umask, "bytes_per_update": per, "full_round": full_round})
        if nmask > 0:
            rounds = (phase == "fp64" and per_round == 8) or (phase == "fp32" and args.scheduler == "octant")
            parts.append({"phase": phase, "kind": "masked", "ms": kmask, "sweeps": nmask,
                          "launches": max(1, nmask // 8) if rounds else nmask, "updates": umask,
                          "bytes_per_update": per, "one_launch_per_8_sweeps": rounds})
    for q in parts:
        q["kernel"] = kernel_name(q["phase"], st["tile"], prec, arith) if q["kind"] == "full" else \
            ("t3_sweep_kernel<float, 16, 32, MIN, FAST>" if q["phase"] == "fp32" else
             f"t3_sweep_kernel<double, 16, 16, {'REPLACE' if prec == L.PREC_FP32_POLISH64 else 'MIN'}, "
             f"{ {L.ARITH_PAIR: 'PAIR', L.ARITH_MIXED: 'MIXED', L.ARITH_FAST: 'FAST'}.get(arith, 'REF')}>")
        if q.get("full_round"):
            q["kernel"] = "t3_sweep_kernel<float, 16, 32, MIN, FAST, octant round (every block)>"
        if q.get("one_launch_per_8_sweeps"):
            q["kernel"] = q["kernel"][:-1] + ", octant round>"
        q["ms_per_launch"] = q["ms"] / q["launches"]
        q["achieved_gbs"] = q["updates"] * q["bytes_per_update"] / (q["ms"] / 1e3) / 1e9 if q["ms"] > 0 else 0.0
        q["frac"] = q["achieved_gbs"] / hbm
        q["share_of_sweep_time"] = q["ms"] / max(k32 + k64, 1e-9)
    dom = max(parts, key=lambda q: q["ms"]) if parts else None
    roof = None
    if dom is not None:
        # traffic: ncu DRAM bytes per update of this kernel (profiles/traffic.json) x its updates per launch
        tr = traffic_per_launch(dom["phase"], prec, dom["updates"] / dom["launches"], st["tile"],
                                masked=dom["kind"] == "masked", full_round=bool(dom.get("full_round")))
        roof = {"bound": "hbm", "achieved": dom["achieved_gbs"], "peak": hbm, "unit": "GB/s", "frac": dom["frac"],
                "traffic": tr, "kernel": dom["kernel"],
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (burst copy)" if "hbm_gbs" in pk else "fallback 6800 GB/s",
                "bytes_per_update": dom["bytes_per_update"], "launches_per_step": dom["launches"],
                "ms_per_launch": dom["ms_per_launch"], "sweep_kind": dom["kind"]}
    fp32_roof = None
    full32 = [q for q in parts if q["phase"] == "fp32" and q["kind"] == "full"]
    if full32:
        fp32_roof = {"achieved": full32[0]["achieved_gbs"], "frac": full32[0]["frac"],
                     "ms_per_sweep": full32[0]["ms"] / full32[0]["sweeps"]}

    # the same solve under each scheduler (one timed run each, after one warm run)
    sched_table = None
    if not args.no_sched_table and args.fixed_sweeps == 0 and args.mode in ("polish", "fp32"):
        sched_table = {}
        for name, sv in (("none", L.SCHED_NONE), ("change", L.SCHED_CHANGE), ("learned", L.SCHED_LEARNED),
                         ("octant", L.SCHED_OCTANT)):
            o2 = dict(opts, scheduler=sv)
            try:
                with api.Context(w.nx, w.ny, w.nz, sp, **o2) as c2:
                    c2.load(w.field, w.frozen)
                    c2.run()
                    s2 = c2.run()
                    sched_table[name] = {"time_s": s2["ms_device"] / 1e3,
                                         "sweeps": s2["sweeps_fp32"] + s2["sweeps_fp64"],
                                         "full_sweeps": s2["full_sweeps"],
                                         "voxel_updates_per_node": s2["voxel_updates"] / w.interior}
            except api.PdfsError as e:
                sched_table[name] = {"unavailable": str(e)}

    cpu = None
    if rank == 0 and world >= 1 and not args.no_cpu and args.fixed_sweeps == 0:
        threads = os.cpu_count() or 1
        sweeps = args.cpu_sweeps or 2
        v, dt, kind, what = cpu_baseline(w, sweeps, threads)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": kind,
               "sample": f"{sweeps} FP64 orderings of the full grid ({dt:.1f} s): {what}"}

    # the reference's own CUDA solver beside the CPU baseline: its sweep kernel
    # built unmodified from its sources (a cubin), its host level loop (one
    # launch per hyperplane, a device synchronisation after each), one
    # run_fsm round of the 8 orderings on the same input
    ref_gpu = None
    if rank == 0 and not args.no_cpu and args.fixed_sweeps == 0:
        from oracle import oracle as O
        if O.have_ref_cuda("nvcc"):
            try:
                ms_sw, ms_all = O.ref_cuda_run(w.field.copy(), sp, first=1, nsweeps=8, sync_each=True)
                ms_q, _ = O.ref_cuda_run(w.field.copy(), sp, first=1, nsweeps=8, sync_each=False)
                per = ms_sw / 8
                ref_gpu = {"kernel": "fast_sweep_kernel (single_gpu_cuda/src/phi3D_fsm.cu), nvcc defaults, sm_103a",
                           "ms_per_sweep": per, "ms_per_sweep_no_level_sync": ms_q / 8,
                           "round_ms_with_copies": ms_all,
                           "gvox_updates_per_s": w.interior * 8 / (ms_sw / 1e3) / 1e9,
                           "time_to_converge_s_est": per * plain_sweeps / 1e3,
                           "ours_speedup": per * plain_sweeps / 1e3 / t_step}
            except Exception as e:
                ref_gpu = {"unavailable": str(e)[:200]}
        else:
            ref_gpu = {"unavailable": "the reference's CUDA kernel was not built (no reference sources at build time)"}

    if rank == 0:
        dtype = {L.ARITH_PAIR: "f32+f32pair", L.ARITH_MIXED: "f32+f64mixed"}.get(arith, "f32+f64") \
            if prec == L.PREC_FP32_POLISH64 else ("f32" if prec == L.PREC_FP32 else "f64")
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": dtype, "data": "synthetic (seeded spheres)",
            "config": {"workload": w.name, "nx": w.nx, "ny": w.ny, "nz": w.nz, "spacing": list(sp),
                       "mode": args.mode, "scheduler": args.scheduler, "polish_tol": args.tol,
                       "polish_arith": args.polish_arith if args.mode == "polish" else None,
                       "parallelism": "replicas" if world > 1 else "single GPU",
                       "l2": "inputs larger than L2 (no flush needed)"},
            "time_to_converge_s": t_step, "wall_s_per_step": wall / args.steps,
            "sweeps": {"fp32": s32, "fp64": s64, "full": st["full_sweeps"],
                       "voxel_updates": st["voxel_updates"], "blocks_skipped": st["blocks_skipped"]},
            "plain_fp64": plain,
            "speedup_vs_plain_fp64": (plain["time_s"] / t_step) if plain else None,
            "fp64_polish": fp64_polish,
            "roofline": roof, "roofline_fp32_sweep": fp32_roof, "roofline_by_kernel": parts,
            "schedulers": sched_table,
            "cpu_baseline": cpu, "reference_gpu": ref_gpu, "e2e": e2e, "gpu_launches": int(sum(s["launches"] for s in stats)),
            "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
