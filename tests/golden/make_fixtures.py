"""Regenerate the committed fixtures under tests/golden/.

Run from the repository root where the reference checkout is available:

    python tests/golden/make_fixtures.py /path/to/reference

It writes:
  inputs/*.in            the reference's shipped input.in files (its only configuration data),
                         used to pin the namelist reader;
  shock_relation.json    the output of the reference's shock_relation.py (a Python helper that
                         computes the post-shock state used by init_shockvortex_general.f90:264-267);
  flop_counts.json       floating-point operations per cell-update of the reference algorithm,
                         counted on the CPU oracle for each scheme and for the bench workloads;
  oracle_step.npz        one-step oracle states of small cases (regression pin of the oracle).
Nothing under tests/ reads the reference at run time: the tests read these files.
"""
from __future__ import annotations

import json
import os
import shutil
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

INPUTS = {
    "root": "input.in",
    "build": "build/input.in",
    "ivc": "examples/ivc/input.in",
    "rt": "examples/rt/input.in",
    "double_mach": "examples/double_mach/input.in",
}

# (name, benchmark, splitting, recon, ni, nj) of the per-scheme FLOP counts
FLOP_CASES = [
    ("LLF+upwind5", 11, 101, 251, 64, 64),
    ("LLF+WENO-JS5", 11, 101, 253, 64, 64),
    ("LLF+WENO-Z5", 11, 101, 255, 64, 64),
    ("GLF+WENO-JS5", 11, 102, 253, 64, 64),
    ("SW+WENO-JS5", 11, 103, 253, 64, 64),
    ("CH (104)", 11, 104, 0, 64, 64),
    ("AdaWENO (105) smooth vortex", 11, 105, 0, 64, 64),
]
# the bench workloads at full size
BENCH_CASES = [
    ("C1 IVC 200x200 LLF+WENO-JS5", 11, 101, 253, 200, 200),
    ("C2 DMR 1920x480 AdaWENO", 5, 105, 0, 1920, 480),
    ("C3 RT 256x1024 CH", 13, 104, 0, 256, 1024),
]

ONE_STEP = [
    ("ivc_ref_101_253", 1, 101, 253, 20, 16),
    ("vortex_105", 11, 105, 0, 16, 20),
    ("dmr_104", 5, 104, 0, 32, 12),
    ("rt_104", 3, 104, 0, 12, 32),
    ("sedov_103_251", 2, 103, 251, 16, 16),
]


def main(ref: str) -> None:
    from oracle import oracle as orc

    os.makedirs(os.path.join(HERE, "inputs"), exist_ok=True)
    for name, rel in INPUTS.items():
        shutil.copyfile(os.path.join(ref, rel), os.path.join(HERE, "inputs", f"{name}.in"))

    out = subprocess.run([sys.executable, os.path.join(ref, "shock_relation.py")],
                         capture_output=True, text=True, check=True).stdout
    vals = dict(line.split("=") for line in out.split() if "=" in line)
    with open(os.path.join(HERE, "shock_relation.json"), "w") as f:
        json.dump({"mach": 1.1, "gamma": 1.4, "stdout": out,
                   **{k: float(v) for k, v in vals.items()}}, f, indent=1)

    counts = {"convention": "add/sub, mul, div, sqrt on field values each count 1, as written "
                            "in the reference; operations on scalars only (gamma, dt, dx) are not "
                            "counted; one full TVD-RK3 step from the benchmark's initial state, "
                            "divided by ni*nj", "schemes": {}, "bench": {}}
    for name, b, s, r, ni, nj in FLOP_CASES + BENCH_CASES:
        cfg = orc.default_config(ni=ni, nj=nj, benchmark=b, splitting=s, recon=r, cfl=0.5,
                                 var_eps=5.0, var_xc=5.0, var_yc=5.0)
        c = orc.count_step_flops(cfg)
        key = "bench" if (name, b, s, r, ni, nj) in BENCH_CASES else "schemes"
        counts[key][name] = {"benchmark": b, "splitting": s, "recon": r, "ni": ni, "nj": nj,
                             "flops_per_cell_update": c["flops_per_cell_update"],
                             "flux_per_cell_update": c["phase"]["flux"] / c["cells"],
                             "flux_xi_per_cell_update": c["flux_dir"]["xi"] / c["cells"],
                             "flux_eta_per_cell_update": c["flux_dir"]["eta"] / c["cells"],
                             "div_per_cell_update": c["div"] / c["cells"],
                             "sqrt_per_cell_update": c["sqrt"] / c["cells"],
                             "phase_per_cell_update": {k: v / c["cells"] for k, v in c["phase"].items()}}
        if s == 105:
            # AdaWENO's work depends on the data only through the branch taken at each
            # (interface, sign): record the price of each branch and the rest as a base
            bc = orc.branch_costs(cfg.gamma)
            br = c["adaweno_branches"]
            e = counts[key][name]
            e["adaweno"] = {
                "smooth_branch_flops": bc["smooth"], "char_branch_flops": bc["char"],
                "base_per_cell_update": (c["flops"] - bc["smooth"] * br["smooth"]
                                         - bc["char"] * br["char"]) / c["cells"],
                "base_xi_per_cell_update": (c["flux_dir"]["xi"] - bc["smooth"] * br["smooth_xi"]
                                            - bc["char"] * br["char_xi"]) / c["cells"],
                "base_eta_per_cell_update": (c["flux_dir"]["eta"] - bc["smooth"] * br["smooth_eta"]
                                             - bc["char"] * br["char_eta"]) / c["cells"],
                "branches_at_setup": br}
        print(name, round(c["flops_per_cell_update"], 1))
    with open(os.path.join(HERE, "flop_counts.json"), "w") as f:
        json.dump(counts, f, indent=1)

    arrays = {}
    for name, b, s, r, ni, nj in ONE_STEP:
        cfg = orc.default_config(ni=ni, nj=nj, benchmark=b, splitting=s, recon=r, cfl=0.5,
                                 var_eps=5.0, var_xc=5.0, var_yc=5.0)
        o = orc.OracleSolver(cfg)
        c0, _ = o.get_state()
        o.steps(1)
        c1, _ = o.get_state()
        arrays[f"{name}__cfg"] = np.array([b, s, r, ni, nj])
        arrays[f"{name}__before"] = c0
        arrays[f"{name}__after"] = c1
        arrays[f"{name}__dt"] = np.array([o.scalars()["dt"]])
    np.savez_compressed(os.path.join(HERE, "oracle_step.npz"), **arrays)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_fixtures.py /path/to/reference-checkout")
    main(sys.argv[1])
