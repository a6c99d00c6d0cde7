"""A C program written against the drop-in headers (tests/c_caller/
embed_solve.c: layout setup, smearFat7, shift, createStaggeredSolver,
solve2, dslash2, the embedqop.c pattern, and makeU's entry points)
compiles and links against
-lqll_gb300 on the CPU; on a GPU it runs and reaches the tolerance."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "c_caller", "embed_solve.c")
LIBDIR = os.path.join(ROOT, "qll_gb300")


def _build(tmp_path):
    exe = str(tmp_path / "embed_solve")
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cmd = ["gcc", "-std=gnu11", "-O2", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "include"),
           SRC, "-o", exe, "-L" + LIBDIR, "-lqll_gb300", "-Wl,-rpath," + LIBDIR,
           "-L" + os.path.join(cuda, "lib64"), "-Wl,-rpath," + os.path.join(cuda, "lib64"),
           "-lcudart", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_c_program_compiles_and_links(tmp_path):
    assert os.path.exists(_build(tmp_path))


@pytest.mark.gpu
def test_c_program_solves(tmp_path):
    exe = _build(tmp_path)
    r = subprocess.run([exe, "8", "8", "8", "8", "0.1"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    words = r.stdout.split()
    its, resid = int(words[words.index("its") + 1]), float(words[words.index("resid") + 1])
    assert abs(its - 86) <= 1            # the FP64 CG's count at 8^4, m = 0.1 (the oracle's)
    assert resid < 1.01e-8
