"""Build of the in-tree shared library ``csrc/_build/libdense2d.so`` (sm_103a only).

Translation units, compiled in parallel:
  kernels.cu  three times: -DDENSE_VARIANT_STRICT=0 (fast: FMA contraction),
              -DDENSE_VARIANT_STRICT=1 -fmad=false (strict: the reference's rounding) and
              -DDENSE_VARIANT_STRICT=0 -DDENSE_CHECK=1 (checked: fast with every index checked)
  capi.cu     the C ABI (handles, graphs, copies)
  batch.cu    the batched form (many blocks per launch)
  adjoint.cu  the discrete adjoint of the time step
  setup_device.cu  device-side setups of the variant benchmarks, vortex error norms
  io.cu       the save path: Tecplot and checkpoint files, the driver loop with device-side saves
  noalloc.cu, probe.cu  the allocation-free stage and the FP64 throughput probes
  host_setup.cpp  namelist reader and initial setups, g++ -ffp-contract=off so the initial
              state rounds exactly like the reference's gfortran -O2 build on x86-64
The ptxas resource report of each kernel (registers, spills, shared memory) is written to
``csrc/_build/ptxas_<unit>.log``.
"""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(CSRC, "_build")
LIB = os.path.join(BUILD, "libdense2d.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xptxas", "-v",
              "--expt-relaxed-constexpr"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources() -> list[str]:
    out = []
    for d in (CSRC, INCLUDE):
        for f in os.listdir(d):
            if f.endswith((".cu", ".cuh", ".h", ".cpp")):
                out.append(os.path.join(d, f))
    return out


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(s) > t for s in _sources()) or os.path.getmtime(__file__) > t


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile libdense2d.so if any source is newer than it. Returns its path."""
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    units = {
        "kernels_fast": [nvcc, *ARCH, *NVCC_FLAGS, "-DDENSE_VARIANT_STRICT=0", "-c",
                         os.path.join(CSRC, "kernels.cu")],
        "kernels_strict": [nvcc, *ARCH, *NVCC_FLAGS, "-DDENSE_VARIANT_STRICT=1", "-fmad=false",
                           "-c", os.path.join(CSRC, "kernels.cu")],
        "kernels_checked": [nvcc, *ARCH, *NVCC_FLAGS, "-DDENSE_VARIANT_STRICT=0", "-DDENSE_CHECK=1", "-c",
                            os.path.join(CSRC, "kernels.cu")],
        "capi": [nvcc, *ARCH, *NVCC_FLAGS, "-c", os.path.join(CSRC, "capi.cu")],
        "probe": [nvcc, *ARCH, *NVCC_FLAGS, "-c", os.path.join(CSRC, "probe.cu")],
        "noalloc": [nvcc, *ARCH, *NVCC_FLAGS, "-c", os.path.join(CSRC, "noalloc.cu")],
        "batch": [nvcc, *ARCH, *NVCC_FLAGS, "-c", os.path.join(CSRC, "batch.cu")],
        "adjoint": [nvcc, *ARCH, *NVCC_FLAGS, "-c", os.path.join(CSRC, "adjoint.cu")],
        "setup_device": [nvcc, *ARCH, *NVCC_FLAGS, "-c", os.path.join(CSRC, "setup_device.cu")],
        "io": [nvcc, *ARCH, *NVCC_FLAGS, "-c", os.path.join(CSRC, "io.cu")],
        "host_setup": ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-c",
                       os.path.join(CSRC, "host_setup.cpp")],
    }
    procs = []
    for name, cmd in units.items():
        obj = os.path.join(BUILD, name + ".o")
        full = cmd + ["-o", obj]
        procs.append((name, obj, full, subprocess.Popen(full, stdout=subprocess.PIPE,
                                                        stderr=subprocess.STDOUT)))
    objs = []
    for name, obj, cmd, p in procs:
        txt = p.communicate()[0].decode(errors="replace")
        with open(os.path.join(BUILD, f"ptxas_{name}.log"), "w") as f:
            f.write(txt)
        if p.returncode != 0:
            raise RuntimeError(f"build of {name} failed:\n{' '.join(cmd)}\n{txt}")
        if verbose:
            print(txt)
        objs.append(obj)
    tmp = LIB + ".tmp"
    link = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcuda", "-lpthread", "-ldl"]
    r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{' '.join(link)}\n{r.stdout.decode()}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=False))
