"""Builds libjmg.so (the CUDA solver, sm_103a) in-tree with nvcc.

The translation units are compiled in parallel and linked into
``jsolver_gb300/libjmg.so``. Nothing is installed outside the source tree.
"""
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libjmg.so")
SOURCES = ["mg_kernels.cu", "mg_hierarchy.cu", "mg_aux.cu", "mg_driver.cu", "mg_noalloc.cu", "mg_coarse.cu", "mg_tile2d.cu",
           "mg_adjoint_kernels.cu", "mg_adjoint.cu", "mg_net.cu", "mg_krylov.cu", "mg_tangent.cu",
           "mg_batch.cu", "mg_fused.cu", "mg_tile3d.cu", "mg_fusedops2d.cu", "mg_coarse_staged.cu",
           "mg_mid2d.cu", "mg_sweep_tma3d.cu",
           "mg_fusedops3d.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall"]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build jsolver_gb300")
    return exe


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    """Compile the CUDA sources (if changed) and link ``libjmg.so``. Returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "jmg.h"))
    exe = nvcc()

    def compile_one(src):
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        if force or _stale(o, [s] + headers):
            cmd = [exe] + ARCH + FLAGS + ["-c", s, "-o", o]
            if verbose:
                print(" ".join(cmd))
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        return o

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    if force or _stale(LIB, objs):
        cmd = [exe] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
