"""Builds the in-tree shared libraries of imodel_gb300.

* ``_lib/libimodel_mesh.so`` -- the host C++ grid builder (g++, OpenMP).
* ``_lib/libimodel_swm.so``  -- the sm_103a CUDA time step and its C ABI.

Objects are compiled in parallel; a library is rebuilt only when one of its
sources or headers is newer than it.  No CPU fallback of the time step is
built: on a machine without nvcc ``build_all`` raises.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
LIB_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(HERE, "_lib", "obj")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
               "-I" + INCLUDE, "-I" + CSRC] + ARCH
CXX_COMMON = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I" + INCLUDE]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build imodel_gb300")
    return cand


def _cuda_lib_dir() -> str:
    nvcc = _nvcc()
    root = os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    for sub in ("lib64", "lib", "targets/sbsa-linux/lib", "targets/x86_64-linux/lib"):
        d = os.path.join(root, sub)
        if os.path.exists(os.path.join(d, "libcudart.so")):
            return d
    return os.path.join(root, "lib64")


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run_parallel(jobs):
    procs = []
    for cmd in jobs:
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE,
                                            stderr=subprocess.STDOUT)))
    failed = []
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((cmd, out.decode(errors="replace")))
    if failed:
        msg = "\n".join(" ".join(c) + "\n" + o for c, o in failed)
        raise RuntimeError("build failed:\n" + msg)


def build_mesh_lib(force: bool = False) -> str:
    """The grid builder: topology and host geometry (mesh.cpp, OpenMP) and
    the GPU geometry kernels (mesh_gpu.cu, no multiply-add contraction)."""
    os.makedirs(OBJ_DIR, exist_ok=True)
    out = os.path.join(LIB_DIR, "libimodel_mesh.so")
    headers = glob.glob(os.path.join(INCLUDE, "*.h")) + [os.path.join(CSRC, "mesh_internal.h")]
    cpp = os.path.join(CSRC, "mesh.cpp")
    cu = os.path.join(CSRC, "mesh_gpu.cu")
    cpp_obj = os.path.join(OBJ_DIR, "mesh.o")
    cu_obj = os.path.join(OBJ_DIR, "mesh_gpu.cu.o")
    jobs = []
    if force or _stale(cpp_obj, [cpp] + headers):
        jobs.append(["g++"] + CXX_COMMON + ["-fopenmp", "-I" + CSRC, "-c", cpp, "-o", cpp_obj])
    if force or _stale(cu_obj, [cu] + headers):
        jobs.append([_nvcc()] + NVCC_COMMON + ["--fmad=false", "-c", cu, "-o", cu_obj])
    if jobs:
        _run_parallel(jobs)
    if force or _stale(out, [cpp_obj, cu_obj]):
        _run_parallel([[_nvcc(), "-shared"] + ARCH + [cpp_obj, cu_obj] +
                       ["-o", out, "-Xcompiler", "-fopenmp", "-L" + _cuda_lib_dir(), "-lcudart"]])
    return out


def build_swm_lib(force: bool = False) -> str:
    os.makedirs(OBJ_DIR, exist_ok=True)
    out = os.path.join(LIB_DIR, "libimodel_swm.so")
    headers = glob.glob(os.path.join(INCLUDE, "*.h")) + \
        glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh"))
    units = {
        # FP64 reference-order kernels: no multiply-add contraction
        "swm_k64.cu": ["--fmad=false"],
        "swm_k32.cu": [],
        "swm_capi.cu": [],
        "swm_ens.cu": [],
        "mlp.cu": [],
        # moist shallow-water model: reference operation order, no contraction
        "swm_moist.cu": ["--fmad=false"],
        # allocation-free weighted sums: compensated summation, no contraction
        "swm_noalloc.cu": ["--fmad=false"],
    }
    nvcc = _nvcc()
    jobs, objs = [], []
    for name, extra in units.items():
        src = os.path.join(CSRC, name)
        obj = os.path.join(OBJ_DIR, name + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append([nvcc] + NVCC_COMMON + extra + ["-c", src, "-o", obj])
    src = os.path.join(CSRC, "swm_layout.cpp")
    obj = os.path.join(OBJ_DIR, "swm_layout.o")
    objs.append(obj)
    if force or _stale(obj, [src] + headers):
        jobs.append(["g++"] + CXX_COMMON + ["-fopenmp", "-I" + CSRC, "-c", src, "-o", obj])
    if jobs:
        _run_parallel(jobs)
    if force or _stale(out, objs):
        _run_parallel([[nvcc, "-shared"] + ARCH + objs +
                       ["-o", out, "-Xcompiler", "-fopenmp", "-L" + _cuda_lib_dir(), "-lcudart"]])
    return out


def build_all(force: bool = False) -> list:
    return [build_mesh_lib(force), build_swm_lib(force)]


if __name__ == "__main__":
    print("\n".join(build_all(force="--force" in sys.argv)))
