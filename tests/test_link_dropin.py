"""Link-level drop-in: the reference's own CUDA-program sources
(single_gpu_cuda/src/main.c, phi3D.c, vti_parser.c, file_writer.c), compiled
unmodified, link against libpdfs.so in place of phi3D_fsm.cu -- the change
INTEGRATION.md section 1 gives a maintainer.  run_fsm (phi3D_fsm.h:69-71,
called from phi3D.c:118-119) must be left undefined in the program and be
resolved from libpdfs.

The reference tree is needed to build the program: $PDFS_REF_ROOT, else the
default that oracle/Makefile names.  Where it is absent the test is skipped.
The program is built into pytest's temporary directory, never into the repo."""
import os
import subprocess

import pytest

from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "pdfs_gb300")
SRCS = ("main.c", "phi3D.c", "vti_parser.c", "file_writer.c")


def ref_cuda_src():
    d = os.path.join(O.ref_root(), "single_gpu_cuda", "src")
    if not all(os.path.exists(os.path.join(d, f)) for f in SRCS):
        pytest.skip("the reference's single_gpu_cuda sources are not present")
    return d


@pytest.fixture(scope="module")
def program(tmp_path_factory):
    src = ref_cuda_src()
    out = tmp_path_factory.mktemp("dropin")
    exe = str(out / "PDFS_with_libpdfs")
    cmd = (["gcc", "-std=gnu99", "-O2", "-w", "-I" + src] + [os.path.join(src, f) for f in SRCS] +
           ["-o", exe, "-L" + PKG, "-lpdfs", "-Wl,-rpath," + PKG, "-lm"])
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe, out


def test_reference_program_links_against_libpdfs(program):
    exe, _ = program
    undef = subprocess.run(["nm", "-u", exe], capture_output=True, text=True, check=True).stdout
    assert any(line.split()[-1] == "run_fsm" for line in undef.splitlines() if line.strip())
    defined = subprocess.run(["nm", "-D", "--defined-only", os.path.join(PKG, "libpdfs.so")], capture_output=True,
                             text=True, check=True).stdout
    assert any(line.split()[-1] == "run_fsm" for line in defined.splitlines() if line.strip())
    deps = subprocess.run(["ldd", exe], capture_output=True, text=True, check=True).stdout
    assert "libpdfs.so" in deps


def test_reference_program_runs_through_libpdfs_without_a_gpu(program):
    """Without a GPU the reference's main runs end to end through libpdfs's
    run_fsm, which reports the missing device instead of exiting (no CPU
    fallback), and writes its output file.  On a GPU the same run_fsm is
    bit-exact with the reference (tests/test_gpu_pipeline.py)."""
    from tests.conftest import have_gpu
    if have_gpu():
        pytest.skip("a GPU is present: the pipeline tests cover the run")
    exe, out = program
    vti = os.path.join(ROOT, "tests", "golden", "vti", "sphere_in.vti")
    r = subprocess.run([exe, vti, str(out / "sphere")], capture_output=True, text=True, timeout=120,
                       env=dict(os.environ, CUDA_VISIBLE_DEVICES=""))
    assert "run_fsm" in r.stdout + r.stderr and "device" in (r.stdout + r.stderr).lower(), r.stdout + r.stderr
