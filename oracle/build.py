"""Build recipe for the CPU oracle (test infrastructure only).

Compiles ``oracle/oracle.cc`` into ``oracle/_build/liboracle.so`` with the host C++
compiler and OpenMP.  Chroma itself cannot be compiled here (its configure step
requires QDP++, QMP and libxml2, none of which are present), so there is no
``oracle/_ref`` build: the oracle is a restatement of Chroma's algorithms.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "oracle.cc")
OUT_DIR = os.path.join(HERE, "_build")
OUT = os.path.join(OUT_DIR, "liboracle.so")


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(OUT) and os.path.getmtime(OUT) >= os.path.getmtime(SRC):
        return OUT
    cxx = os.environ.get("CXX", "g++")
    cmd = [cxx, "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-Wall",
           "-Wno-unused-function", SRC, "-o", OUT + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(OUT + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
