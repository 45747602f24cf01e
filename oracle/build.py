"""Builds the CPU oracle shared library (test infrastructure only).

The oracle is a C++ restatement of FLEXI's DGSEM Navier-Stokes operator used by tests/,
__graft_entry__.smoke() and bench.py's cpu_baseline leg as the checker. Output goes to
oracle/_build/liboracle.so (git-ignored); FLEXI's own sources are Fortran 2008 with CMake,
MPI and HDF5 dependencies and are not compiled here.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SOURCES = ["oracle_capi.cpp"]
HEADERS = ["basis.hpp", "mesh.hpp", "dg.hpp"]


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    deps = [os.path.join(HERE, f) for f in SOURCES + HEADERS]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-o", LIB + ".tmp"]
    cmd += [os.path.join(HERE, s) for s in SOURCES]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
