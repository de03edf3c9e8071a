"""Build recipe of the reference runner (test infrastructure only).

Reads pxlengine's FLIP shader where it lies in the reference checkout (shaders/fluid.slang under
PXF_REFERENCE_ROOT, default /root/reference), applies four mechanical edits so that g++ accepts
it, and compiles oracle/ref_fluid.cpp, which includes the result, with oracle/slang_shim.h
force-included (OpenMP). Outputs go to oracle/_ref/ only (git-ignored, carried to the GPU machine with
the working tree): fluid_slang.inc and libref_fluid.so. Without the checkout, a fluid_slang.inc
made earlier from it is compiled for this machine; with neither, nothing is built and None is
returned.

The edits (nothing else of the shader changes):
  [shader("compute")]        -> removed     (Slang entry-point attribute)
  [numthreads(256, 1, 1)]    -> removed     (the host dispatches the invocations itself)
  : SV_DispatchThreadID      -> removed     (the invocation index is the kernel's argument)
  out T x (parameter)        -> T& x        (an out parameter is a reference)
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT_DIR, "libref_fluid.so")
INC = os.path.join(OUT_DIR, "fluid_slang.inc")
SHIM = os.path.join(HERE, "slang_shim.h")
DRIVER = os.path.join(HERE, "ref_fluid.cpp")

EDITS = [
    (re.compile(r'\[shader\("compute"\)\]'), ""),
    (re.compile(r"\[numthreads\([^\]]*\)\]"), ""),
    (re.compile(r":\s*SV_DispatchThreadID"), ""),
    (re.compile(r"([(,]\s*)out\s+(\w+)\s+"), r"\1\2& "),
]


def shader_path():
    root = os.environ.get("PXF_REFERENCE_ROOT", "/root/reference")
    path = os.path.join(root, "shaders", "fluid.slang")
    return path if os.path.exists(path) else None


def _machine():
    return os.uname().machine


def build(force: bool = False):
    src = shader_path()
    if src is None and not os.path.exists(INC):
        return None
    os.makedirs(OUT_DIR, exist_ok=True)
    stamp = os.path.join(OUT_DIR, "machine")
    same_machine = os.path.exists(stamp) and open(stamp).read().strip() == _machine()
    deps = [SHIM, DRIVER, os.path.abspath(__file__)] + ([src] if src else [INC])
    if (not force and same_machine and os.path.exists(LIB)
            and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps)):
        return LIB
    if src is not None:
        text = open(src).read()
        for pat, rep in EDITS:
            text = pat.sub(rep, text)
        with open(INC, "w") as f:
            f.write(text)
    cxx = os.environ.get("CXX", "g++")
    cmd = [cxx, "-std=c++17", "-O2", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fsingle-precision-constant",
           "-Wno-attributes", "-include", SHIM, "-I", OUT_DIR, "-shared", "-fPIC", "-o", LIB + ".tmp", DRIVER]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    with open(stamp, "w") as f:
        f.write(_machine())
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
