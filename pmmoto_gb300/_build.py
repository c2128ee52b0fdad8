"""Build the CUDA library in-tree: pmmoto_gb300/_lib/libpmmoto_gb300.so.

Every ``csrc/*.cu`` translation unit is compiled for sm_103a only, in
parallel, then linked into one shared library with a plain C ABI
(``include/pmmoto_gb300.h``).  ``--fmad=false`` keeps nvcc from fusing
multiply-adds: the library reproduces a reference whose float arithmetic is
not contracted.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT_DIR, "libpmmoto_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = [os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"]
    for c in cand:
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _flags(verbose: bool):
    f = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-Xcompiler", "-fPIC",
                "-I", os.path.join(REPO, "include")]
    if verbose:
        f += ["-Xptxas", "-v"]
    return f


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    srcs = sources()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(REPO, "include", "pmmoto_gb300.h"))
    newest_hdr = max(os.path.getmtime(h) for h in headers)
    objs, jobs = [], []
    for s in srcs:
        o = os.path.join(OUT_DIR, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if force or not os.path.exists(o) or os.path.getmtime(o) < max(os.path.getmtime(s), newest_hdr):
            jobs.append((s, o))
    if jobs:
        cmd0 = nvcc()

        def run(job):
            s, o = job
            r = subprocess.run([cmd0, *_flags(verbose), "-c", s, "-o", o], capture_output=True, text=True)
            return s, r

        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            for s, r in ex.map(run, jobs):
                if verbose and r.stderr:
                    sys.stderr.write(r.stderr)
                if r.returncode != 0:
                    raise RuntimeError(f"nvcc failed for {s}:\n{r.stdout}\n{r.stderr}")
    if jobs or not os.path.exists(LIB):
        r = subprocess.run([nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
