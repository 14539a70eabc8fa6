"""Autotuner of the fast kernels.

Dimensions: the fast kernel's launch shape (configurations per block, threads per block) and its
sphere tile (spheres of one configuration per warp row of sphere tasks), the hard cloud-query
kernel's blocks per SM (distances only), and the edge kernel's launch shape.  The best values
depend on the robot (FK slots, spheres, self pairs), the scene (primitives vs a point cloud),
whether per-sphere distances are requested and the batch size.  ``autotune`` and
``autotune_edges`` time the candidates on the caller's batch with CUDA events and keep the
fastest; the choice is cached in a JSON file keyed by that signature and the device name, so
later runs of the same workload skip the sweep.
"""
from __future__ import annotations

import json
import os
from pathlib import Path
from typing import List, Optional, Tuple

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


def sphere_tiles(cpb: int) -> List[int]:
    """The sphere tiles worth trying at a shape: 0 (the least, 32 / cpb) and every larger power of two."""
    least = max(1, 32 // cpb)
    return [0] + [t for t in (2, 4, 8, 16, 32) if t > least]


def _time(fn, reps: int) -> float:
    import torch

    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    fn()
    torch.cuda.synchronize()
    ms = []
    for _ in range(reps):
        start.record()
        fn()
        end.record()
        end.synchronize()
        ms.append(start.elapsed_time(end))
    ms.sort()
    return ms[len(ms) // 2]


def autotune(cst, Q, distances: bool = False, reps: int = 5, use_cache: bool = True, verbose: bool = False
             ) -> Tuple[Tuple[int, int], dict]:
    """Pick and set the fastest launch shape and sphere tile for is_valid_fast on the batch Q (a CUDA
    tensor), and with distances the hard-query kernel's blocks per SM.  Returns
    ((configs_per_block, threads_per_block), {candidate: ms}); cst.get_fast_tuning() gives the rest."""
    key = signature(cst, int(Q.shape[0]), distances)
    _, _, ecpb, ent = cst.get_fast_tuning()
    cache = _load() if use_cache else {}
    if key in cache and "sphere_tile" in cache[key]:
        c = cache[key]
        cst.set_fast_launch(*c["shape"])
        cst.set_fast_tuning(c["sphere_tile"], c["hq_blocks_per_sm"], ecpb, ent)
        return tuple(c["shape"]), c.get("ms", {})
    times = {}
    best, best_ms = None, float("inf")
    for cpb, nt in SHAPES:
        cst.set_fast_launch(cpb, nt)
        for st in sphere_tiles(cpb):
            cst.set_fast_tuning(st, 4, ecpb, ent)
            try:
                ms = _time(lambda: cst.is_valid_fast(Q, distances=distances), reps)
            except Exception:  # shape not launchable for this table size (shared memory)
                break
            times[f"{cpb}x{nt}/st{st}"] = ms
            if verbose:
                print(f"  shape {cpb}x{nt} sphere tile {st}: {ms:.3f} ms")
            if ms < best_ms:
                best, best_ms = (cpb, nt, st), ms
    cpb, nt, st = best
    cst.set_fast_launch(cpb, nt)
    hq = 4
    if distances:  # the hard-query kernel's occupancy at the chosen shape
        best_ms = float("inf")
        for b in (2, 3, 4, 8):
            cst.set_fast_tuning(st, b, ecpb, ent)
            ms = _time(lambda: cst.is_valid_fast(Q, distances=True), reps)
            times[f"hq{b}"] = ms
            if ms < best_ms:
                hq, best_ms = b, ms
    cst.set_fast_tuning(st, hq, ecpb, ent)
    if use_cache:
        cache = _load()
        cache[key] = {"shape": [cpb, nt], "sphere_tile": st, "hq_blocks_per_sm": hq, "ms": times}
        _save(cache)
    return (cpb, nt), times


EDGE_SHAPES = [(16, 128), (32, 128), (32, 256), (64, 256)]


def autotune_edges(validator, S1, S2, reps: int = 5, use_cache: bool = True, verbose: bool = False
                   ) -> Tuple[Tuple[int, int], dict]:
    """Pick and set the fastest launch shape of the edge kernel for validator.check_motion_fast on
    the edges (S1, S2) (CUDA tensors).  Returns ((waypoints_per_block, threads_per_block), {shape: ms})."""
    cst = validator.cst
    key = signature(cst, int(S1.shape[0]), False) + f"|edges|{type(validator).__name__}"
    st, hq, _, _ = cst.get_fast_tuning()
    cache = _load() if use_cache else {}
    if key in cache:
        c = cache[key]
        cst.set_fast_tuning(st, hq, *c["shape"])
        return tuple(c["shape"]), c.get("ms", {})
    out = None
    times = {}
    for ecpb, ent in EDGE_SHAPES:
        cst.set_fast_tuning(st, hq, ecpb, ent)
        try:
            if out is None:
                out = validator.check_motion_fast(S1, S2)
            ms = _time(lambda: validator.check_motion_fast(S1, S2, out=out), reps)
        except Exception:  # not launchable for this table size (shared memory)
            continue
        times[f"{ecpb}x{ent}"] = ms
        if verbose:
            print(f"  edge shape {ecpb}x{ent}: {ms:.3f} ms")
    best = min(times, key=times.get)
    ecpb, ent = (int(v) for v in best.split("x"))
    cst.set_fast_tuning(st, hq, ecpb, ent)
    if use_cache:
        cache = _load()
        cache[key] = {"shape": [ecpb, ent], "ms": times}
        _save(cache)
    return (ecpb, ent), times
