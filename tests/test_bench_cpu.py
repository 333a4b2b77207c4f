"""The measurement plumbing of bench.py on the CPU: its kernel tables agree
with the library's tile tables (pdfs_gb300/csrc/sweep.cu), the default tiles
name the kernels the profiles cover, and the DRAM traffic it reports comes
from the committed ncu captures."""
import importlib.util
import json
import os
import re

import pytest

from pdfs_gb300 import _lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def tile_table(name):
    """Entries {tx, ty, c[, bz[, pencil[, lc]]]} of kT32 / kT64 in sweep.cu
    (named row counts from sweep.cuh)."""
    src = open(os.path.join(ROOT, "pdfs_gb300", "csrc", "sweep.cu")).read()
    hdr = open(os.path.join(ROOT, "pdfs_gb300", "csrc", "sweep.cuh")).read()
    consts = {m.group(1): int(m.group(2)) for m in re.finditer(r"constexpr int (kLc\w+) = (\d+);", hdr)}
    body = re.search(r"static const TileShape %s\[\] = \{(.*?)\};" % name, src, re.S).group(1)
    out = []
    for m in re.finditer(r"\{([^{}]*)\}", body):
        v = [consts[x.strip()] if x.strip() in consts else int(x) for x in m.group(1).split(",")]
        v += [0] * (6 - len(v))
        out.append(tuple(v))
    return out


def default_tiles():
    """The default tile ids (pick_tiles in solver.cu)."""
    src = open(os.path.join(ROOT, "pdfs_gb300", "csrc", "solver.cu")).read()
    t32 = int(re.search(r"c->t32 = t32 \? t32 : (\d+);", src).group(1))
    t64 = int(re.search(r"c->t64 = t64 \? t64 : (\d+);", src).group(1))
    return t32, t64


@pytest.mark.parametrize("kind", ["fp32", "fp64"])
def test_bench_kernel_tables_match_library(bench, kind):
    table = tile_table("kT32" if kind == "fp32" else "kT64")
    cols = bench.COLUMNS32 if kind == "fp32" else bench.COLUMNS64
    bricks = bench.BRICKS32 if kind == "fp32" else bench.BRICKS64
    pencils = bench.PENCILS32 if kind == "fp32" else bench.PENCILS64
    lanecols = bench.LANECOL32 if kind == "fp32" else bench.LANECOL64
    for tid, (tx, ty, c, bz, pencil, lc) in enumerate(table, start=1):
        tile = tid if kind == "fp32" else tid << 8
        k = bench.kernel_kind(kind, tile)
        if lc:
            assert k == "lanecol" and lanecols[tid] == lc
        elif pencil:
            assert k == "pencil" and tid in pencils
        elif bz:
            assert k == "brick" and bricks[tid] == (ty, bz)
        else:
            assert k == "column" and cols[tid] == (ty, c)
    assert set(cols) | set(bricks) | set(pencils) | set(lanecols) == set(range(1, len(table) + 1))


def test_default_kernels_have_profiles_and_traffic(bench):
    t32, t64 = default_tiles()
    tile = t32 | (t64 << 8)
    n32 = bench.kernel_name("fp32", tile, L.PREC_FP32_POLISH64, L.ARITH_PAIR)
    n64 = bench.kernel_name("fp64", tile, L.PREC_FP32_POLISH64, L.ARITH_PAIR)
    assert n32 == "pc_sweep_kernel<float, MIN, FAST>"
    assert n64 == "pc_sweep_kernel<double, REPLACE, PAIR>"
    traffic = json.load(open(os.path.join(ROOT, "profiles", "traffic.json")))
    for kind, name in (("fp32", n32), ("fp64", n64)):
        t = bench.traffic_per_launch(kind, L.PREC_FP32_POLISH64, 1000, tile)
        assert t is not None and t > 0
        entry = [e for e in traffic.values() if e["kernel"].startswith(name.split(">")[0])]
        assert entry, name
        # a capture's bytes per update, and the capture's summary exists
        assert abs(t / 1000 - entry[0]["dram_bytes"] / entry[0]["updates"]) < 1e-3
        assert os.path.exists(os.path.join(ROOT, entry[0]["capture"]))


def test_launch_list_profile_names_the_default_kernels():
    text = open(os.path.join(ROOT, "profiles", "launches_C4_768_pair.md")).read()
    assert "pc_sweep_kernel<double, REPLACE, PAIR, ISO>" in text
    assert "pc_sweep_kernel<float, MIN, FAST, ISO>" in text
    assert "--clock-control none" in text
