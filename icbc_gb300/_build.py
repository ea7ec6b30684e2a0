"""Builds libicbc_gpu.so (the CUDA kernels + C ABI) in-tree for sm_103a.

Every encoder translation unit is compiled with ``-fmad=false``: the reference
rounds every multiply and add separately, so FMA contraction would change
results.  The ten per-level kernels compile as separate objects in parallel.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)
INCLUDE = os.path.join(ROOT, "include")
OUT_DIR = os.path.join(HERE, "_lib")
LIB_NAME = "libicbc_gpu.so"
LIB_PATH = os.path.join(OUT_DIR, LIB_NAME)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-prec-div=true", "-prec-sqrt=true",
              "-ftz=false", "-Xcompiler", "-fPIC", "-Xcompiler", "-fno-fast-math", "-I" + INCLUDE]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _units():
    """(source, extra flags, object name) of every translation unit."""
    # The all-levels units (batch, SIMD profiles, no-alloc) compile longest: start them first.
    units = [(os.path.join(CSRC, "bc1_batch.cu"), ["-DICBC_BATCH_BYTES=%d" % v], "bc1_batch%d.o" % v) for v in (1, 0)]
    units += [(os.path.join(CSRC, n), [], n.replace(".cu", ".o")) for n in ("bc1_simd.cu", "bc1_noalloc.cu")]
    units += [(os.path.join(CSRC, "bc1_level.cu"), ["-DICBC_LEVEL=%d" % lv], "bc1_level%d.o" % lv)
              for lv in range(9, -1, -1)]
    units += [(os.path.join(CSRC, n), [], n.replace(".cu", ".o"))
              for n in ("bc1_decode.cu", "icbc_gpu_api.cu", "icbc_gpu_serve.cu", "icbc_compat.cu", "bc1_refine.cu",
                        "icbc_containers.cu", "bc1_ingest.cu")]
    return [u for u in units if os.path.exists(u[0])]


def _sources_digest() -> str:
    h = hashlib.sha256()
    files = sorted(os.listdir(CSRC)) + ["icbc_gpu.h", "icbc_compat.hpp"]
    for name in files:
        path = os.path.join(CSRC, name) if os.path.exists(os.path.join(CSRC, name)) else os.path.join(INCLUDE, name)
        if os.path.isfile(path):
            h.update(name.encode())
            with open(path, "rb") as f:
                h.update(f.read())
    h.update(" ".join(ARCH + NVCC_FLAGS).encode())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False, jobs: int | None = None) -> str:
    """Compiles and links the library if any source changed; returns its path."""
    os.makedirs(OUT_DIR, exist_ok=True)
    stamp = os.path.join(OUT_DIR, "build.stamp")
    digest = _sources_digest()
    if not force and os.path.exists(LIB_PATH) and os.path.exists(stamp):
        with open(stamp) as f:
            if f.read().strip() == digest:
                return LIB_PATH
    exe = nvcc()
    objs_dir = os.path.join(OUT_DIR, "obj")
    os.makedirs(objs_dir, exist_ok=True)

    def compile_one(unit):
        src, extra, obj = unit
        out = os.path.join(objs_dir, obj)
        cmd = [exe] + ARCH + NVCC_FLAGS + extra + ["-c", src, "-o", out]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (os.path.basename(src), r.stdout, r.stderr))
        if verbose:
            sys.stderr.write(r.stderr)
        return out

    units = _units()
    workers = jobs or min(len(units), max(1, os.cpu_count() or 1))
    with cf.ThreadPoolExecutor(max_workers=workers) as ex:
        objs = list(ex.map(compile_one, units))
    tmp = LIB_PATH + ".%d.tmp" % os.getpid()
    cmd = [exe] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB_PATH)
    with open(stamp, "w") as f:
        f.write(digest)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
