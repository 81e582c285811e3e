"""In-tree build of the CUDA library (sm_103a only) with nvcc, no cmake.

Each .cu translation unit compiles in parallel to an object, then one link
step produces persiansph_gb300/_build/libpsph_gb300.so, which the ctypes
boundary (persiansph_gb300.abi) loads.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libpsph_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              f"-I{REPO}/include", f"-I{CSRC}"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _stale(lib, deps):
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra_flags=(), out_dir=None) -> str:
    """Compiles the library into out_dir (default persiansph_gb300/_build)."""
    out = out_dir or OUT
    lib_path = os.path.join(out, "libpsph_gb300.so")
    os.makedirs(out, exist_ok=True)
    srcs = sources()
    deps = srcs + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))] + \
        [os.path.join(REPO, "include", f) for f in os.listdir(os.path.join(REPO, "include"))]
    if not force and not _stale(lib_path, deps):
        return lib_path
    nv = nvcc()

    def compile_one(src):
        obj = os.path.join(out, os.path.basename(src)[:-3] + ".o")
        cmd = [nv, *ARCH, *NVCC_FLAGS, *extra_flags, "-c", src, "-o", obj]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{res.stderr}")
        if verbose and res.stderr:
            sys.stderr.write(res.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = lib_path + ".tmp"
    cmd = [nv, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart", "-lpthread"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stderr}")
    os.replace(tmp, lib_path)
    return lib_path


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
