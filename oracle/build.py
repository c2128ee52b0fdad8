"""ORACLE build recipe -- test infrastructure only.

Builds, into ``oracle/_ref/`` (git-ignored):

* ``liboracle.so`` -- the C/C++ restatement (``pmg_oracle.c``,
  ``pmg_oracle_cc.cpp``), compiled with ``-ffp-contract=off`` so that no
  multiply-add is fused, and with OpenMP over independent lines.
* ``libpmref.so`` -- PMMoTo's own C++ line kernels compiled from the
  reference source tree through ``ref_shim.cpp``; built only where the
  reference sources are present (the ``PMMOTO_REF_SRC`` environment
  variable, or the path the caller passes).

Run ``python -m oracle.build`` or call :func:`build_oracle`.
"""

from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
REF_SRC = os.environ.get("PMMOTO_REF_SRC")


def _run(cmd):
    subprocess.run(cmd, check=True)


def build_oracle(force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    so = os.path.join(OUT, "liboracle.so")
    srcs = [os.path.join(HERE, "pmg_oracle.c"), os.path.join(HERE, "pmg_oracle_cc.cpp")]
    if force or not os.path.exists(so) or any(os.path.getmtime(s) > os.path.getmtime(so) for s in srcs):
        objs = []
        for s in srcs:
            o = os.path.join(OUT, os.path.basename(s) + ".o")
            cc = "gcc" if s.endswith(".c") else "g++"
            std = "-std=c11" if s.endswith(".c") else "-std=c++17"
            _run([cc, std, "-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-c", s, "-o", o])
            objs.append(o)
        _run(["g++", "-shared", "-fopenmp", "-o", so] + objs)
    return so


def build_reference(force: bool = False, ref_src: str | None = None) -> str | None:
    """Compile the reference's own line kernels from its source tree
    (``ref_src``, else ``$PMMOTO_REF_SRC``); None when no tree is given or
    it has no line kernels."""
    ref_src = ref_src or REF_SRC
    if not ref_src:
        return None
    dist = os.path.join(ref_src, "filters", "distance")
    core = os.path.join(ref_src, "core")
    parts = os.path.join(ref_src, "particles")
    if not os.path.isdir(dist):
        return None
    os.makedirs(OUT, exist_ok=True)
    so = os.path.join(OUT, "libpmref.so")
    shim = os.path.join(HERE, "ref_shim.cpp")
    if force or not os.path.exists(so) or os.path.getmtime(shim) > os.path.getmtime(so):
        # the reference's setup.py uses -O3 -std=c++17; contraction is made
        # explicit so the x86 and Arm builds round identically
        _run(["g++", "-std=c++17", "-O3", "-fPIC", "-shared", "-ffp-contract=off",
              "-I", dist, "-I", core, "-I", parts, shim, "-o", so])
    return so


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_reference(force="--force" in sys.argv))
