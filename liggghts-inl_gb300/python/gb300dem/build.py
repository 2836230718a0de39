"""Builds libdemgpu.so (CUDA kernels + C ABI) in-tree for sm_103a.

Each translation unit is compiled in parallel with nvcc, then linked with
-shared.  Output: liggghts-inl_gb300/_build/libdemgpu.so (git-ignored).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "libdemgpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-ffp-contract=off",
                  "-Xptxas", "-warn-spills"]
SOURCES = ["dem_kernels.cu", "dem_capi.cu", "dem_probe.cu", "dem_noalloc.cu", "dem_mesh_host.cu",
           "dem_adjoint.cu"]


def nvcc():
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _deps_mtime():
    m = 0.0
    for f in os.listdir(CSRC):
        m = max(m, os.path.getmtime(os.path.join(CSRC, f)))
    m = max(m, os.path.getmtime(os.path.join(PKG, "..", "include", "liggghts_gb300.h")))
    return m


def build(force=False, verbose=False):
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps_mtime():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()

    def comp(src):
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        cmd = [nv] + NVFLAGS + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
        if verbose:
            print(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(comp, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nv] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="-f" in sys.argv, verbose=True))
