"""In-tree build of libmeshhash.so with nvcc for sm_103a.

Every translation unit is compiled in parallel with
``-gencode arch=compute_103a,code=sm_103a -O3 -lineinfo --fmad=false``:
FMA contraction is off on the device and on the host (``-ffp-contract=off``)
so single-precision results are reproducible by a CPU restatement; division
and square root stay IEEE (no fast-math).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libmeshhash.so")
OBJ = os.path.join(HERE, "_build")
SOURCES = ["mh_volume.cu", "mh_alloc.cu", "mh_integrate.cu", "mh_mesh.cu", "mh_raycast.cu", "mh_gc.cu",
           "mh_tv.cu",
           "mh_batch.cu", "mh_pose.cu",
           "mh_compact.cu", "mh_io.cu", "mh_huber.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
         "--expt-relaxed-constexpr"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh", ".h", ".inc"))]
    files.append(os.path.join(HERE, "..", "include", "meshhash.h"))
    return files


def up_to_date() -> bool:
    if not os.path.exists(OUT):
        return False
    t = os.path.getmtime(OUT)
    return all(os.path.getmtime(f) <= t for f in _deps())


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    if not force and up_to_date():
        return OUT
    os.makedirs(OBJ, exist_ok=True)
    cc = nvcc()
    extra = ["-Xptxas", "-v"] if ptxas_info else []

    def compile_one(src):
        obj = os.path.join(OBJ, src.replace(".cu", ".o"))
        cmd = [cc, "-c", os.path.join(CSRC, src), "-o", obj] + ARCH + FLAGS + extra
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        return obj, r.stderr

    with cf.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        results = list(ex.map(compile_one, SOURCES))
    if verbose or ptxas_info:
        for _, err in results:
            if err:
                sys.stderr.write(err)
    tmp = OUT + ".tmp"
    cmd = [cc, "-shared", "-o", tmp] + [o for o, _ in results] + ARCH + ["-Xcompiler", "-fPIC"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv)
    print(OUT)
