"""Autotuner for the fused sweep kernel: tile shape and half-sweeps per launch.

The fused kernel has four tile shapes (16x64, 16x128, 32x64 rows x z-cells, and 16x128 row
pairs for even fused depths) and fuses 1..4 half-sweeps per launch; which pair is fastest
depends on the volume's shape and the GPU. The
tuner times every candidate on the solver's own volumes with CUDA events (a few launches
each), restores the field afterwards and keeps the fastest. Results are cached per
(operator, shape, batch, device) in memory and, if ``TAUFACTOR_GB300_CACHE`` names a file, on
disk as JSON. Every candidate computes the same half-sweeps bit for bit, so tuning never
changes results.
"""
from __future__ import annotations

import json
import os

import torch

CANDIDATES = [(tile, k) for k in (4, 3, 2) for tile in (0, 1, 2)] + [(3, 4), (3, 2)]
_MEMO: dict = {}


def _key(solver) -> str:
    return json.dumps([solver._op.kind, solver._op.periodic, solver.batch_size, solver.Nx, solver.Ny, solver.Nz,
                       torch.cuda.get_device_name(solver.device)])


def _load_disk() -> dict:
    path = os.environ.get("TAUFACTOR_GB300_CACHE")
    if not path or not os.path.exists(path):
        return {}
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store_disk(key: str, value) -> None:
    path = os.environ.get("TAUFACTOR_GB300_CACHE")
    if not path:
        return
    data = _load_disk()
    data[key] = value
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(data, f)
    os.replace(tmp, path)


def default_config(solver):
    """Shape-based choice used when no tuning result exists. The multiphase kind fuses 3
    half-sweeps per launch: its per-lane face lookups make the 4-deep march large enough to miss
    in the instruction cache (on GB300, 0.112 against 0.141 ms per half-sweep at 320^3; 0.304
    against 0.332 on 4 x 256^3 periodic). The other kinds are fastest at 4."""
    if solver._op.kind == 0 and solver.Nz >= 128:
        return 1, 4
    if solver._op.kind == 2:
        return 0, 3
    return 0, 4


def apply(solver, tile: int, k: int) -> None:
    solver._op.tile = int(tile)
    solver._op.k_max = int(k)


def tune(solver, half_sweeps: int = 48, candidates=None) -> dict:
    """Time the candidates on `solver`, apply the fastest and return {(tile, k): ms per half-sweep}."""
    key = _key(solver)
    if key in _MEMO:
        apply(solver, *_MEMO[key])
        return {}
    disk = _load_disk()
    if key in disk:
        _MEMO[key] = tuple(disk[key])
        apply(solver, *_MEMO[key])
        return {}
    cands = candidates or CANDIDATES
    if solver._op.kind != 0:
        cands = [(0, k) for k in (4, 3, 2)]
    saved = solver._cur.clone()
    saved_iter = solver.iter
    times = {}
    with torch.cuda.device(solver.device):
        for tile, k in cands:
            apply(solver, tile, k)
            n = max(k, (half_sweeps // k) * k)
            solver._advance(k)  # warm-up launch
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            solver._advance(n)
            e1.record()
            e1.synchronize()
            times[(tile, k)] = e0.elapsed_time(e1) / n
        solver._cur.copy_(saved)
    solver.iter = saved_iter
    best = min(times, key=times.get)
    apply(solver, *best)
    _MEMO[key] = best
    _store_disk(key, list(best))
    return times
