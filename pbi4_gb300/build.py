"""Build libpbi4gpu.so (the C-ABI CUDA library) in-tree for sm_103a.

Each .cu translation unit is compiled in parallel with nvcc, then linked into
pbi4_gb300/_build/libpbi4gpu.so against cuFFT.  Runs the same on x86_64 (cross
compilation, no GPU needed) and on the aarch64 GPU hosts.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libpbi4gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
              "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]


def nvcc() -> str:
    cand = [os.environ.get("NVCC", ""), shutil.which("nvcc") or "", "/usr/local/cuda/bin/nvcc"]
    for c in cand:
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps_mtime():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(os.path.dirname(HERE), "include", "pbi4gpu.h"))
    files.append(os.path.abspath(__file__))
    return max(os.path.getmtime(f) for f in files if os.path.exists(f))


def up_to_date() -> bool:
    return os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps_mtime()


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile and link the library (in parallel, one nvcc per .cu).  Extra
    nvcc flags (e.g. -D tuning macros) may come from the environment variable
    PBI4G_NVCC_EXTRA; the library is rebuilt when they change."""
    extra = os.environ.get("PBI4G_NVCC_EXTRA", "").split()
    stamp = os.path.join(OUT, "nvcc_extra.txt")
    prev = open(stamp).read() if os.path.exists(stamp) else ""
    if not force and up_to_date() and prev == " ".join(extra):
        return LIB
    os.makedirs(OUT, exist_ok=True)
    nv = nvcc()
    srcs = sources()

    def compile_one(src):
        obj = os.path.join(OUT, os.path.basename(src)[:-3] + ".o")
        cmd = [nv, *ARCH, *NVCC_FLAGS, *extra, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr, file=sys.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + ".tmp"
    cmd = [nv, *ARCH, "-shared", "-o", tmp, *objs, "-lcufft", "-lcuda"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    with open(stamp, "w") as f:
        f.write(" ".join(extra))
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
