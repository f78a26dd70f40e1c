"""Autotuner of the batched form's launch schedule.

A schedule is (xi tile variant, eta tile variant, block order, launch mode): the thread-block
shape of each direction sweep (``batch_tile_shape`` in csrc/kernels.cu: 4 xi and 5 eta shapes,
from short wide tiles that give small instances more blocks to tall narrow ones that stage fewer
halo cells per interface), the order in which the instances' blocks are laid out (instance-major,
largest instance first, or round-robin) and how a step is launched (one launch per phase, or one
persistent launch whose blocks take the step's pieces in that order, each waiting only for its
own instance's previous phase) -- 60 schedules per launch mode, counted by the library
(``dense_batch_schedule_space``); the persistent mode exists for the component-wise schemes of
the fast variant. None of them changes any result -- every interface's arithmetic is the same --
so the tuner is free to pick whichever is fastest for the batch at hand.

The search is a coordinate descent (launch mode, order, xi tile, eta tile, repeated until a pass
changes nothing, at most three passes), each candidate timed on a scratch copy of the batch (same
configurations, same initial states) so the caller's solution is untouched. The winner is cached
in a JSON file keyed by device, scheme and the histogram of instance sizes, so a second batch of
the same shape reuses it without timing.
"""
from __future__ import annotations

import ctypes
import hashlib
import json
import os
import time

from . import _abi
from .solver import BatchSolver, init_general

CACHE = os.environ.get("DENSE2D_AUTOTUNE_CACHE",
                       os.path.join(os.path.expanduser("~"), ".cache", "dense2d_gb300", "autotune.json"))


def schedule_space() -> tuple[int, int, int]:
    """(xi tile variants, eta tile variants, block orders) of dense_batch_set_schedule."""
    lib = _abi.load_library()
    n = [ctypes.c_int() for _ in range(3)]
    lib.dense_batch_schedule_space(*[ctypes.byref(x) for x in n])
    return n[0].value, n[1].value, n[2].value


def launch_modes(cfgs) -> tuple[int, ...]:
    """Launch modes the batch supports: the persistent step (1) covers the component-wise
    schemes (101-103 with 251/253/255) of the fast variant."""
    c0 = cfgs[0]
    return (0, 1) if c0.splitting <= 103 and c0.strict == 0 else (0,)


def _device_key() -> str:
    try:
        import torch
        p = torch.cuda.get_device_properties(torch.cuda.current_device())
        return f"{p.name}|{p.multi_processor_count}"
    except Exception:  # no torch: the key still separates schemes and shapes
        return "cuda"


def batch_key(cfgs) -> str:
    sizes = sorted((c.ni, c.nj) for c in cfgs)
    h = hashlib.sha1(json.dumps(sizes).encode()).hexdigest()[:16]
    c0 = cfgs[0]
    return f"{_device_key()}|{c0.splitting}|{c0.recon}|{c0.strict}|n{len(cfgs)}|{h}|modes"


def _load_cache() -> dict:
    try:
        with open(CACHE) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store_cache(d: dict) -> None:
    try:
        os.makedirs(os.path.dirname(CACHE), exist_ok=True)
        tmp = CACHE + ".tmp"
        with open(tmp, "w") as f:
            json.dump(d, f, indent=1, sort_keys=True)
        os.replace(tmp, CACHE)
    except OSError:
        pass


def _time_schedule(b: BatchSolver, sched, steps: int, reps: int) -> float:
    b.set_schedule(*sched)
    b.steps(1)  # warm-up: builds the graph for this schedule
    best = float("inf")
    for _ in range(reps):
        t0 = time.perf_counter()
        b.steps(steps)
        best = min(best, time.perf_counter() - t0)
    return best


def tune(cfgs, setups=None, steps: int = 2, reps: int = 2, use_cache: bool = True):
    """Best (xi_variant, eta_variant, order, launch mode) for this batch, and the timings tried.

    ``setups`` is the list of (cfg, cons, prim, x, y) the batch starts from (init_general of each
    configuration when omitted)."""
    key = batch_key(cfgs)
    cache = _load_cache() if use_cache else {}
    if key in cache:
        e = cache[key]
        return tuple(e["schedule"]), {"cached": True, "key": key, "trials": e.get("trials", {})}
    if setups is None:
        setups = [init_general(c) for c in cfgs]
    trials = {}
    scratch = BatchSolver([s[0] for s in setups])
    try:
        for i, (c, cons, prim, x, y) in enumerate(setups):
            scratch.upload(i, cons, prim, x, y)
        best = (0, 0, 0, 0)

        def run(sched):
            if sched not in trials:
                trials[sched] = _time_schedule(scratch, sched, steps, reps)
            return trials[sched]

        def along(dim, values):
            nonlocal best
            for x in values:
                cand = tuple(x if d == dim else best[d] for d in range(4))
                if run(cand) < run(best):
                    best = cand

        n_xi, n_eta, n_order = schedule_space()
        for _ in range(3):
            start = best
            along(3, launch_modes(cfgs))
            along(2, range(n_order))
            along(0, range(n_xi))
            along(1, range(n_eta))
            if best == start:
                break
    finally:
        scratch.close()
    named = {",".join(str(x) for x in k): v for k, v in trials.items()}
    if use_cache:
        cache = _load_cache()
        cache[key] = {"schedule": list(best), "trials": named}
        _store_cache(cache)
    return best, {"cached": False, "key": key, "trials": named}
