"""Autotuner for the fast kernel's launch shape (configurations per block, threads per block).

The best shape depends on the robot (FK slots, spheres, self pairs), the scene (primitives vs a
point cloud), whether per-sphere distances are requested and the batch size.  ``autotune``
times every supported shape on the caller's batch with CUDA events and keeps the fastest; the
choice is cached in a JSON file keyed by that signature and the device name, so later runs of
the same workload skip the sweep.
"""
from __future__ import annotations

import json
import os
from pathlib import Path
from typing import Optional, Tuple

SHAPES = [(16, 128), (32, 128), (16, 256), (32, 256), (64, 256), (32, 512), (64, 512), (128, 512)]


def cache_path() -> Path:
    p = os.environ.get("PMGPU_AUTOTUNE_CACHE")
    if p:
        return Path(p)
    return Path(os.path.expanduser("~")) / ".cache" / "plainmp_gb300" / "autotune.json"


def signature(cst, batch: int, distances: bool) -> str:
    import torch

    g = cst.groups()
    sdf = cst.get_sdf()
    scene = type(sdf).__name__ if sdf is not None else "none"
    return (f"{torch.cuda.get_device_name()}|q{cst.q_dim()}|s{cst.n_spheres}|g{cst.n_groups}|sg{int(g['only_self'].sum())}|"
            f"c{cst.cst_dim()}|{scene}|B{batch}|d{int(distances)}")


def _load() -> dict:
    try:
        return json.loads(cache_path().read_text())
    except (OSError, ValueError):
        return {}


def _save(d: dict) -> None:
    p = cache_path()
    try:
        p.parent.mkdir(parents=True, exist_ok=True)
        p.write_text(json.dumps(d, indent=1, sort_keys=True))
    except OSError:
        pass  # a read-only home directory only costs the cache


def autotune(cst, Q, distances: bool = False, reps: int = 5, use_cache: bool = True, verbose: bool = False
             ) -> Tuple[Tuple[int, int], dict]:
    """Pick and set the fastest launch shape for is_valid_fast on the batch Q (a CUDA tensor).
    Returns ((configs_per_block, threads_per_block), {shape: ms})."""
    import torch

    key = signature(cst, int(Q.shape[0]), distances)
    cache = _load() if use_cache else {}
    if key in cache:
        cpb, nt = cache[key]["shape"]
        cst.set_fast_launch(cpb, nt)
        return (cpb, nt), cache[key].get("ms", {})
    times = {}
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for cpb, nt in SHAPES:
        cst.set_fast_launch(cpb, nt)
        try:
            cst.is_valid_fast(Q, distances=distances)
        except Exception:  # shape not launchable for this table size (shared memory)
            continue
        torch.cuda.synchronize()
        ms = []
        for _ in range(reps):
            start.record()
            cst.is_valid_fast(Q, distances=distances)
            end.record()
            end.synchronize()
            ms.append(start.elapsed_time(end))
        ms.sort()
        times[f"{cpb}x{nt}"] = ms[len(ms) // 2]
        if verbose:
            print(f"  shape {cpb}x{nt}: {times[f'{cpb}x{nt}']:.3f} ms")
    best = min(times, key=times.get)
    cpb, nt = (int(v) for v in best.split("x"))
    cst.set_fast_launch(cpb, nt)
    if use_cache:
        cache = _load()
        cache[key] = {"shape": [cpb, nt], "ms": times}
        _save(cache)
    return (cpb, nt), times
