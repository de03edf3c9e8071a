"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/flip_oracle.cpp into oracle/_build/liborc_flip.so. Flags: -O3, OpenMP, no FMA
contraction (-ffp-contract=off) and no -march=native, so x86_64 and aarch64 produce the same bits.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "flip_oracle.cpp")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liborc_flip.so")


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cxx = os.environ.get("CXX", "g++")
    cmd = [cxx, "-std=c++17", "-O3", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
           "-shared", "-fPIC", "-o", LIB + ".tmp", SRC]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
