"""Builds the reference library itself (QLL, C) as a second CPU oracle:
test infrastructure, never shipped or measured as the product.

The reference's own build needs three sources generated by Lua scripts
(lib/vla0.c, lib/vlaw0.c, include/vec_ops_c.h; lib/Makefile:40-44,
include/Makefile:1-2) and the QMP message-passing library
(include/common.h:2).  Neither Lua nor QMP is installed, so this recipe
  1. runs the reference's generator scripts unchanged with the small Lua
     interpreter in lua51.py;
  2. compiles the reference's lib/*.c (the D/F wrappers and the files they
     include, the object list of lib/Makefile:11-33) from the reference's
     own sources, with refstub/qmp.h standing in for QMP (one rank: no
     message is ever exchanged, the global sum is the identity) and
     refstub/rdtsc.h for the x86/PowerPC tick counter of
     include/rdtsc.h, which has no aarch64 branch; the staged
     include/thread.h takes the reference's own PowerPC memory barrier on
     aarch64 as well (stage() says why);
  3. links them with ref_harness.c (this repository's C entry points that
     drive the reference API the way its test programs do) into
     _ref/libqllref.so.
Builds: _ref/libqllref.so with -DC1 (one SIMD lane: the reference's
one-lane layout, the same site order as the oracle and the GPU library),
without floating-point contraction, for parity; and _ref/libqllref_fast.so
with -DC4 (four sites per vector, the reference's portable GCC-vector SIMD
path) and host-native flags (-O3 -mcpu=native on aarch64, -march=native on
x86_64), the reference's own kind of timing build (its make.inc:18-24),
for the CPU timing arm; refh_convert moves fields between the one-lane
order and its layout.

The reference's sources are staged, with the generated ones, under
_ref/src (git-ignored, never committed), so that a machine without the
reference tree (the GPU host) can compile the same sources for its own
architecture: run with the reference present once to stage, then anywhere.
Usage: python oracle/ref_build.py [--reference DIR]
"""
import argparse
import glob
import os
import platform
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
SRC = os.path.join(OUT, "src")
STUB = os.path.join(HERE, "refstub")

# the object list of the reference's lib/Makefile:11-33
UNITS = ["common", "gather", "layout", "shifts", "vlaD", "vlaF", "vlawD", "vlawF", "fieldD",
         "fieldF", "gaugeD", "gaugeF", "transporterF", "transporterD", "stagDslashF",
         "stagDslashD", "wilsonDslashF", "wilsonDslashD", "cgF", "cgD", "cgmsF", "cgmsD"]
GENERATED = [("lib/vla0.c.lua", "lib/vla0.c"), ("lib/vlaw0.c.lua", "lib/vlaw0.c"),
             ("include/vec_ops_c.h.lua", "include/vec_ops_c.h")]


def stage(ref):
    """copies the reference's library sources and headers under _ref/src
    and generates the Lua outputs there"""
    sys.path.insert(0, HERE)
    import lua51
    for sub in ("lib", "include"):
        os.makedirs(os.path.join(SRC, sub), exist_ok=True)
        for f in glob.glob(os.path.join(ref, sub, "*")):
            name = os.path.basename(f)
            # the tick counter is replaced by the portable stand-in
            if name == "rdtsc.h" or not name.endswith((".c", ".h", ".lua")):
                continue
            shutil.copyfile(f, os.path.join(SRC, sub, name))
    # include/thread.h:83-88 makes its thread-reduction fence SYNC a full
    # memory barrier on PowerPC only and empty elsewhere, which relies on
    # x86's store and load ordering: on aarch64 the threads of its global
    # sums (lib/common.c:30-72) can read a partner's partial sum before it
    # is visible, and the sums come out wrong (observed on the aarch64 GPU
    # host: the 16-thread CG at 32^3x64 did not converge).  The staged copy
    # takes the reference's own PowerPC barrier on aarch64 too.
    th = os.path.join(SRC, "include", "thread.h")
    with open(th) as fh:
        text = fh.read()
    text = text.replace("#ifdef __powerpc__", "#if defined(__powerpc__) || defined(__aarch64__)", 1)
    with open(th, "w") as fh:
        fh.write(text)
    for script, out in GENERATED:
        path = os.path.join(SRC, script)
        tmp = os.path.join(SRC, out + ".tmp")
        with open(tmp, "w") as fh:
            lua51.run_script(path, fh)
        os.replace(tmp, os.path.join(SRC, out))


def native_flags():
    return ["-mcpu=native"] if platform.machine() in ("aarch64", "arm64") else ["-march=native"]


def compile_lib(name, extra, jobs=None):
    obj = os.path.join(OUT, "obj_" + name)
    os.makedirs(obj, exist_ok=True)
    base = ["gcc", "-std=gnu99", "-fPIC", "-fopenmp", "-w",
            "-I" + STUB, "-I" + os.path.join(SRC, "include"), "-I" + os.path.join(SRC, "lib")]
    cmds = []
    objs = []
    for u in UNITS:
        o = os.path.join(obj, u + ".o")
        objs.append(o)
        cmds.append(base + extra + ["-c", os.path.join(SRC, "lib", u + ".c"), "-o", o])
    o = os.path.join(obj, "ref_harness.o")
    objs.append(o)
    cmds.append(base + extra + ["-c", os.path.join(HERE, "ref_harness.c"), "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("reference build failed: %s\n%s%s" % (" ".join(cmd), r.stdout,
                                                                      r.stderr))
    with ThreadPoolExecutor(max_workers=jobs or min(16, os.cpu_count() or 4)) as ex:
        list(ex.map(run, cmds))
    lib = os.path.join(OUT, name + ".so")
    r = subprocess.run(["gcc", "-shared", "-fopenmp", "-o", lib] + objs + ["-lm"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference link failed:\n%s%s" % (r.stdout, r.stderr))
    return lib


def build(ref=None):
    """stages (when the reference tree is present) and compiles; returns
    the parity library's path, or None when neither the reference tree nor
    staged sources exist"""
    ref = ref or os.environ.get("QLL_REFERENCE", "/root/reference")
    if os.path.isdir(os.path.join(ref, "lib")):
        stage(ref)
    if not os.path.exists(os.path.join(SRC, "lib", "vla0.c")):
        return None
    lib = compile_lib("libqllref", ["-DC1", "-O2", "-ffp-contract=off"])
    compile_lib("libqllref_fast", ["-DC4", "-O3"] + native_flags())
    return lib


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=None)
    a = ap.parse_args()
    print(build(a.reference))
