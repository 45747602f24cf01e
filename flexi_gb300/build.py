"""Builds libflexigpu.so in-tree (flexi_gb300/_build/) for sm_103a.

CUDA translation units are compiled in parallel with nvcc
(-gencode arch=compute_103a,code=sm_103a -lineinfo), the host mesh preparation with g++/OpenMP,
and everything is linked into one shared library exposing the C ABI of include/flexi_gpu.h.
"""
import concurrent.futures
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libflexigpu.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU = ["fg_host.cu", "fg_noalloc.cu"] + [f"fg_inst_n{n}.cu" for n in range(2, 13)]
CPP = ["fg_mesh.cpp", "fg_io.cpp"]
HEADERS = ["fg_common.cuh", "fg_kernels.cuh", "fg_launch.cuh", "fg_inst.cuh", "fg_basis.hpp", "fg_mesh.hpp", "fg_adjoint_point.cuh", "fg_adjoint.cuh", "fg_h5.hpp"]
# host-only harness of the point-wise physics and its adjoints, for the CPU tests
POINT_SRC = "fg_point_test.cu"
POINT_LIB = os.path.join(OUT, "libfgpoint.so")


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def _stale(obj, src):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "flexi_gpu.h")]
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src):
    path = os.path.join(CSRC, src)
    obj = os.path.join(OUT, src + ".o")
    if not _stale(obj, path):
        return obj
    if src.endswith(".cu"):
        cmd = [_nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fopenmp", "-I", INCLUDE, "-c", path, "-o", obj + ".tmp"]
    else:
        cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-fopenmp", "-I", INCLUDE, "-c", path, "-o", obj + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {src}\n{r.stdout}\n{r.stderr}")
    os.replace(obj + ".tmp", obj)
    return obj


def build(force: bool = False, jobs: int = 0) -> str:
    os.makedirs(OUT, exist_ok=True)
    if force:
        for f in os.listdir(OUT):
            if f.endswith(".o"):
                os.remove(os.path.join(OUT, f))
    srcs = CU + CPP
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with concurrent.futures.ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(_compile, srcs))
    if force or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [_nvcc(), *ARCH, "-shared", "-o", LIB + ".tmp", *objs, "-lgomp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed\n{r.stdout}\n{r.stderr}")
        os.replace(LIB + ".tmp", LIB)
    build_point_harness()
    return LIB


def build_point_harness() -> str:
    """libfgpoint.so: the point-wise functions compiled as host code (no device code, no GPU needed)."""
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(CSRC, POINT_SRC)
    if _stale(POINT_LIB, src):
        cmd = [_nvcc(), "-O2", "-std=c++17", "-shared", "-Xcompiler", "-fPIC", "-I", INCLUDE, src, "-o", POINT_LIB + ".tmp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {POINT_SRC}\n{r.stdout}\n{r.stderr}")
        os.replace(POINT_LIB + ".tmp", POINT_LIB)
    return POINT_LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
