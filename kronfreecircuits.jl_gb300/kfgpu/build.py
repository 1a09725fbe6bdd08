"""Build libkfgpu.so in-tree with nvcc for sm_103a (GB300).

Each translation unit under csrc/ compiles to an object in parallel, then one link step makes
kfgpu/libkfgpu.so.  A source newer than the library (or `force=True`) triggers a rebuild.
`check=True` builds the bounds-recording variant kfgpu/libkfgpu_check.so (-DKF_CHECK: kernels test
their indices and record the first failing site instead of accessing; load it with KF_LIB).
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(ROOT, "csrc")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(PKG, "libkfgpu.so")
LIB_CHECK = os.path.join(PKG, "libkfgpu_check.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr", "-DNDEBUG"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: libkfgpu.so cannot be built")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _stale(lib=LIB):
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    deps = sources() + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    deps += glob.glob(os.path.join(os.path.dirname(ROOT), "include", "*.h"))
    return any(os.path.getmtime(p) > t for p in deps if os.path.exists(p))


def build_library(force=False, verbose=False, check=False):
    """Compile csrc/*.cu|*.cpp for sm_103a and link kfgpu/libkfgpu.so (check=True:
    kfgpu/libkfgpu_check.so with -DKF_CHECK); returns its path."""
    lib = LIB_CHECK if check else LIB
    bdir = BUILD + ("_check" if check else "")
    flags = FLAGS + (["-DKF_CHECK"] if check else [])
    if not force and not _stale(lib):
        return lib
    os.makedirs(bdir, exist_ok=True)
    cc = nvcc()
    inc = ["-I", os.path.join(os.path.dirname(ROOT), "include")]

    def compile_one(src):
        obj = os.path.join(bdir, os.path.basename(src) + ".o")
        lang = ["-x", "cu"] if src.endswith(".cu") else ["-x", "c++"]
        cmd = [cc] + ARCH + flags + inc + lang + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, sources()))
    tmp = lib + ".tmp"
    cmd = [cc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build_library(force=True, verbose=True))
