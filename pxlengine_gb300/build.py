"""Build recipe of libpxlflip.so (CUDA for sm_103a + C++ host engine), in-tree.

Every translation unit compiles in parallel with one -gencode (compute_103a -> sm_103a) and
-fmad=false: the FLIP arithmetic must not be contracted into FMAs, so that it rounds exactly like
the reference's FP32 expressions. The output lands in pxlengine_gb300/_lib/.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libpxlflip.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    if os.path.exists(cand):
        return cand
    found = shutil.which("nvcc")
    if not found:
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libpxlflip.so")
    return found


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def _deps():
    return _sources() + glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        [os.path.join(HERE, "..", "include", "pxlflip.h"), os.path.abspath(__file__)]


def _compile(src: str, obj: str, nvcc: str, extra):
    if src.endswith(".cu"):
        cmd = [nvcc, "-std=c++17", *ARCH, "-O3", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC",
               "-Xcompiler", "-fvisibility=hidden", *extra, "-c", src, "-o", obj]
    else:
        cxx = os.environ.get("CXX", "g++")
        cmd = [cxx, "-std=c++17", "-O2", "-fPIC", "-fvisibility=hidden", "-ffp-contract=off",
               "-I", os.path.join(os.path.dirname(nvcc), "..", "include"), "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False, extra=()) -> str:
    os.makedirs(OUT, exist_ok=True)
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(p) <= t for p in _deps() if os.path.exists(p)):
            return LIB
    nvcc = nvcc_path()
    objdir = os.path.join(OUT, "obj")
    os.makedirs(objdir, exist_ok=True)
    srcs = _sources()
    objs = [os.path.join(objdir, os.path.basename(s) + ".o") for s in srcs]
    with cf.ThreadPoolExecutor(max_workers=max(2, min(len(srcs), os.cpu_count() or 2))) as ex:
        list(ex.map(lambda so: _compile(so[0], so[1], nvcc, list(extra)), zip(srcs, objs)))
    tmp = LIB + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-cudart", "static", "-Xlinker", "--no-undefined"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
