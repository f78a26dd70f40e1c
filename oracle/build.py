"""Build recipe of the CPU oracle (test infrastructure only).

Two builds of the same source:
  * ``_build/liboracle.so``       -O2 -ffp-contract=off -fopenmp: the parity build. No FMA is
    contracted, matching gfortran -O2 on generic x86-64 (the reference's build,
    source/CMakeLists.txt:12). OpenMP does not change results: every loop writes disjoint cells
    and the only reduction is a max.
  * ``_build/liboracle_timed.so`` -O2 -fopenmp: the CPU baseline as a C compiler would build it
    for the host (FMA contraction allowed where the host has FMA).
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
SRC = os.path.join(HERE, "dense_oracle.cpp")

VARIANTS = {
    "liboracle.so": ["-O2", "-ffp-contract=off", "-fopenmp"],
    "liboracle_timed.so": ["-O2", "-fopenmp"],
}


def build(force: bool = False) -> dict[str, str]:
    os.makedirs(BUILD, exist_ok=True)
    out = {}
    procs = []
    for name, flags in VARIANTS.items():
        dst = os.path.join(BUILD, name)
        out[name] = dst
        if (not force and os.path.exists(dst)
                and os.path.getmtime(dst) >= os.path.getmtime(SRC)
                and os.path.getmtime(dst) >= os.path.getmtime(
                    os.path.join(HERE, "..", "include", "dense2d.h"))):
            continue
        cmd = ["g++", "-std=c++17", "-fPIC", "-shared", *flags, "-o", dst, SRC]
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    for cmd, p in procs:
        txt = p.communicate()[0].decode()
        if p.returncode != 0:
            raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{txt}")
    return out


if __name__ == "__main__":
    print(build(force=True))
