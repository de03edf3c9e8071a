"""Build recipe of the reference runner (test infrastructure only).

Reads pxlengine's FLIP shader and agent-simulation shader where they lie in the reference checkout
(shaders/fluid.slang and shaders/sim.slang under PXF_REFERENCE_ROOT, default /root/reference),
applies a few mechanical edits so that g++ accepts them, and compiles oracle/ref_fluid.cpp and
oracle/ref_sim.cpp, which include the results, with oracle/slang_shim.h force-included (OpenMP).
Outputs go to oracle/_ref/ only (git-ignored, carried to the GPU machine with the working tree):
fluid_slang.inc, sim_slang.inc and libref_shaders.so. Without the checkout, .inc files made earlier
from it are compiled for this machine; with neither, nothing is built and None is returned.

The edits (nothing else of the shaders changes):
  [shader("compute")]        -> removed     (Slang entry-point attribute)
  [numthreads(256, 1, 1)]    -> removed     (the host dispatches the invocations itself)
  : SV_DispatchThreadID etc. -> removed     (the invocation / group index is the kernel's argument)
  out T x (parameter)        -> T& x        (an out parameter is a reference)
  groupshared                -> removed     (the array is shared by the threads of one workgroup)
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT_DIR, "libref_shaders.so")
SHIM = os.path.join(HERE, "slang_shim.h")
SHADERS = {"fluid.slang": "fluid_slang.inc", "sim.slang": "sim_slang.inc"}
DRIVERS = [os.path.join(HERE, "ref_fluid.cpp"), os.path.join(HERE, "ref_sim.cpp")]

EDITS = [
    (re.compile(r'\[shader\("compute"\)\]'), ""),
    (re.compile(r"\[numthreads\([^\]]*\)\]"), ""),
    (re.compile(r":\s*SV_\w+"), ""),
    (re.compile(r"([(,]\s*)out\s+(\w+)\s+"), r"\1\2& "),
    (re.compile(r"\bgroupshared\s+"), ""),
]


def shader_root():
    root = os.environ.get("PXF_REFERENCE_ROOT", "/root/reference")
    ok = all(os.path.exists(os.path.join(root, "shaders", s)) for s in SHADERS)
    return root if ok else None


def _machine():
    return os.uname().machine


def build(force: bool = False):
    root = shader_root()
    incs = [os.path.join(OUT_DIR, inc) for inc in SHADERS.values()]
    if root is None and not all(os.path.exists(i) for i in incs):
        return None
    os.makedirs(OUT_DIR, exist_ok=True)
    srcs = [os.path.join(root, "shaders", s) for s in SHADERS] if root else incs
    stamp = os.path.join(OUT_DIR, "machine")
    same_machine = os.path.exists(stamp) and open(stamp).read().strip() == _machine()
    deps = [SHIM, os.path.abspath(__file__)] + DRIVERS + srcs
    if (not force and same_machine and os.path.exists(LIB)
            and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps)):
        return LIB
    if root is not None:
        for shader, inc in SHADERS.items():
            text = open(os.path.join(root, "shaders", shader)).read()
            for pat, rep in EDITS:
                text = pat.sub(rep, text)
            with open(os.path.join(OUT_DIR, inc), "w") as f:
                f.write(text)
    cxx = os.environ.get("CXX", "g++")
    cmd = [cxx, "-std=c++17", "-O2", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fsingle-precision-constant",
           "-Wno-attributes", "-include", SHIM, "-I", OUT_DIR, "-shared", "-fPIC", "-o", LIB + ".tmp"] + DRIVERS
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    with open(stamp, "w") as f:
        f.write(_machine())
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
