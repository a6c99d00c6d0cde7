"""Build libqll_gb300.so in place: C host code with gcc, CUDA kernels with
nvcc for sm_103a only, linked into qll_gb300/libqll_gb300.so."""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libqll_gb300.so")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
INC = ["-I" + os.path.join(ROOT, "include"), "-I" + CSRC, "-I" + os.path.join(CUDA, "include")]


def _sources():
    c = sorted(f for f in os.listdir(CSRC) if f.endswith(".c"))
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    return c, cu


def _cmd(src):
    out = os.path.join(OBJ, src + ".o")
    path = os.path.join(CSRC, src)
    if src.endswith(".cu"):
        cmd = [NVCC] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC"] + INC
    else:
        # no floating-point contraction: host results (the input generator,
        # host-side reductions) are then the same on x86_64 and aarch64
        cmd = ["gcc", "-O3", "-std=gnu11", "-fPIC", "-fopenmp", "-Wall",
               "-Wno-unused-function", "-ffp-contract=off"] + INC
    return out, cmd + ["-c", path, "-o", out]


def _stale(out, src):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    deps = [os.path.join(CSRC, src)] + [os.path.join(CSRC, f) for f in os.listdir(CSRC)
                                        if f.endswith((".h", ".cuh"))]
    deps += [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, jobs=None):
    os.makedirs(OBJ, exist_ok=True)
    c, cu = _sources()
    todo = []
    objs = []
    for src in cu + c:
        out, cmd = _cmd(src)
        objs.append(out)
        if _stale(out, src):
            todo.append((src, cmd))

    def run(item):
        src, cmd = item
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile of %s failed:\n%s%s" % (src, r.stdout, r.stderr))
        return src

    with ThreadPoolExecutor(max_workers=jobs or min(16, os.cpu_count() or 4)) as ex:
        list(ex.map(run, todo))
    if todo or not os.path.exists(LIB):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + [
            "-Xcompiler", "-fopenmp", "-lcudart", "-lgomp", "-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
