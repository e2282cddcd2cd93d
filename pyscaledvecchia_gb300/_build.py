"""Build libsvgpu.so (the sm_103a kernels behind the C ABI of include/svgpu.h).

The library is compiled in-tree with nvcc: every ``csrc/*.cu`` translation
unit in parallel, then one shared-object link.  Only ``sm_103a`` code is
generated.  A stamp with the hash of the sources and flags lets the loader
detect a stale build.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OUTDIR = os.path.join(PKG, "_lib")
LIBNAME = "libsvgpu.so"
LIBPATH = os.path.join(OUTDIR, LIBNAME)
STAMP = os.path.join(OUTDIR, "libsvgpu.stamp")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
              "-I" + INCLUDE]


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libsvgpu.so")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _digest() -> str:
    h = hashlib.sha256()
    files = sources() + sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh"))
    files.append(os.path.join(INCLUDE, "svgpu.h"))
    for f in files:
        h.update(os.path.basename(f).encode())
        with open(f, "rb") as fh:
            h.update(fh.read())
    # flags without the include path: the same tree reached through another
    # path (a symlink) is the same build
    h.update(" ".join(ARCH + [f for f in NVCC_FLAGS if not f.startswith("-I")]).encode())
    return h.hexdigest()


def is_current() -> bool:
    if not os.path.exists(LIBPATH) or not os.path.exists(STAMP):
        return False
    with open(STAMP) as fh:
        return fh.read().strip() == _digest()


def build(force: bool = False, verbose: bool = False, jobs: int | None = None) -> str:
    """Compile csrc/*.cu for sm_103a and link libsvgpu.so; returns its path."""
    if not force and is_current():
        return LIBPATH
    nvcc = nvcc_path()
    os.makedirs(OUTDIR, exist_ok=True)
    objdir = os.path.join(OUTDIR, "obj")
    os.makedirs(objdir, exist_ok=True)

    def compile_one(src):
        obj = os.path.join(objdir, os.path.basename(src)[:-3] + ".o")
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)
        return obj

    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=jobs or min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIBPATH + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIBPATH)
    with open(STAMP, "w") as fh:
        fh.write(_digest())
    return LIBPATH


if __name__ == "__main__":
    print(build(force=True, verbose=True))
