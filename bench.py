"""Benchmark of the collision-checking hot path on GB300.

Headline workload (one "step" = one pass of the hot path over one batch, inputs resident in
HBM): the 14-DOF dual arm (two 7-joint chains, 120 spheres, cross-arm self pairs) against a
200,000-point cloud on 12 box surfaces, 65,536 joint configurations per batch.  A step is
``SphereCollisionCst.is_valid_fast`` with per-sphere signed distances: validity booleans
identical to the reference plus the FP32 nearest-point signed distance of every sphere
(clamped at the reference's 0.1 m cutoff).  metric = configurations checked per second.

Reported beside it: the plain FP64 method (one thread per configuration, launch per batch)
on the same batch, the validity-only fast path, the end-to-end rate through the public API
with pinned host buffers (copies inside the timed region), the CPU restatement of the
reference on all host cores, kernel timing and the dominant kernel's roofline, and the SM
clocks sampled during the timed region.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Multi-GPU (torchrun, one rank per GPU): configurations are independent, so every rank checks
its own batch (replicas, weak scaling) and the reported time is the maximum over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

PEAKS = ROOT / "MEASURED_PEAKS.json"
FALLBACK_HBM_GBS = 6800.0
L2_FLUSH_BYTES = 512 << 20  # > 129 MB L2
B = 65536


def workload():
    from plainmp_gb300 import workloads as W

    robot = W.dualarm_robot()
    scene = W.Scene(cloud=W.box_surface_cloud(), cloud_radius=0.0)
    q = W.dualarm_configs(B)
    return robot, scene, q


def config_dict(extra=None):
    d = {
        "workload": "dual-arm 14-DOF, 120 spheres, 59 self-collision group pairs, 200k-point box-surface cloud (sigma 2 mm, float32)",
        "batch_configs": B,
        "outputs": "validity (identical to the reference) + per-sphere FP32 signed distance clamped at 0.1 m",
        "l2": "flushed between timed steps (512 MB write)",
        "parallelism": "replicas (independent configurations, one batch per GPU)",
    }
    if extra:
        d.update(extra)
    return d


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = "clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown," \
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 6:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[2:6]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    if PEAKS.exists():
        d = json.loads(PEAKS.read_text())
        return float(d.get("hbm_gbs", FALLBACK_HBM_GBS)), "measured"
    return FALLBACK_HBM_GBS, "fallback"


def cpu_baseline(robot, scene, q, seconds: float = 6.0):
    """The oracle (CPU FP64 restatement of the reference's is_valid loop) on all host cores,
    over a bounded sample of the batch: validity only, as the reference computes it."""
    from oracle import pyoracle

    threads = os.cpu_count() or 1
    _, oc, _ = pyoracle.make_constraint(robot, scene)
    n = 4096
    t0 = time.perf_counter()
    oc.is_valid(q[:n], threads=threads)
    dt = time.perf_counter() - t0
    reps = max(1, min(64, int(seconds / max(dt, 1e-6))))
    done = 0
    t0 = time.perf_counter()
    for r in range(reps):
        off = (r * n) % (B - n)
        oc.is_valid(q[off:off + n], threads=threads)
        done += n
    dt = time.perf_counter() - t0
    return {"value": done / dt, "unit": "configs/s", "cores": threads, "kind": "port",
            "sample": f"{done} configs of the same batch ({reps} x {n}), validity only (the reference has no per-sphere distance output)"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    robot, scene, q = workload()
    from oracle import pyoracle

    threads = os.cpu_count() or 1
    _, oc, _ = pyoracle.make_constraint(robot, scene)
    n = 8192
    for w in range(args.warmup):
        oc.is_valid(q[:n], threads=threads)
    times = []
    for k in range(args.steps):
        off = (k * n) % (B - n)
        t0 = time.perf_counter()
        oc.is_valid(q[off:off + n], threads=threads)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = n * args.steps / total
    line = {
        "impl": "reference", "metric": "configs checked/sec", "value": value, "unit": "configs/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": config_dict({"reference_sample_per_step": n}),
        "cpu_baseline": {"value": value, "unit": "configs/s", "cores": threads, "kind": "port",
                         "sample": f"{n} configs per step of the same batch, validity only"},
        "e2e": {"value": value, "unit": "configs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)

    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    import plainmp_gb300 as pm
    from plainmp_gb300 import _lib, scenes

    robot, scene, qh = workload()
    kin, cst, sdf = scenes.make_constraint(robot, scene)
    dev = torch.device("cuda", local)
    Q = torch.tensor(qh, device=dev)
    ns = cst.n_spheres
    out = torch.empty(B, dtype=torch.uint8, device=dev)
    dout = torch.empty((B, ns), dtype=torch.float32, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)

    from plainmp_gb300 import autotune

    shape_dist, _ = autotune.autotune(cst, Q, distances=True)
    shape_valid, _ = autotune.autotune(cst, Q, distances=False)
    cst.set_fast_launch(*shape_dist)

    def step():
        cst.is_valid_fast(Q, distances=True, out=out, dist_out=dout)

    def barrier():
        torch.cuda.synchronize(dev)
        if dist is not None:
            dist.barrier()

    for _ in range(args.warmup):
        step()
    barrier()
    _lib.profile_read("*")
    _lib.profile_enable(True)
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    total_ms = 0.0
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.fill_(1.0)
            barrier()
            start.record(stream)
            step()
            end.record(stream)
            end.synchronize()
            total_ms += start.elapsed_time(end)
    barrier()
    _lib.profile_enable(False)
    k_ms, k_n = _lib.profile_read("k_fast_valid")
    r_ms, r_n = _lib.profile_read("k_fast_recheck")
    rest_ms, rest_n = _lib.profile_read("*")
    all_n = k_n + r_n + rest_n
    t = torch.tensor([total_ms], device=dev)
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    total_ms = float(t.item())
    ms_per_step = total_ms / args.steps
    value = world * B * args.steps / (total_ms / 1e3)

    # validity-only fast path and the plain FP64 method on the same batch
    def timed(fn, n):
        fn()
        torch.cuda.synchronize(dev)
        tt = 0.0
        for _ in range(n):
            flush.fill_(1.0)
            torch.cuda.synchronize(dev)
            start.record(stream)
            fn()
            end.record(stream)
            end.synchronize()
            tt += start.elapsed_time(end)
        return tt / n

    cst.set_fast_launch(*shape_valid)
    ms_valid = timed(lambda: cst.is_valid_fast(Q, out=out), 5)
    cst.set_fast_launch(*shape_dist)
    ms_plain = timed(lambda: cst.is_valid_batch(Q), 3)
    ok_fast = cst.is_valid_fast(Q).cpu().numpy()
    ok_plain = cst.is_valid_batch(Q).cpu().numpy()
    mismatches = int((ok_fast != ok_plain).sum())
    _, st = cst.is_valid_fast(Q, stats=True)

    # end to end through the public API with pinned host buffers (copies inside the region)
    qpin = torch.from_numpy(qh).pin_memory()
    opin = torch.empty(B, dtype=torch.uint8).pin_memory()
    dpin = torch.empty((B, ns), dtype=torch.float32).pin_memory()
    e2e_fn = lambda: cst.is_valid_fast(qpin.numpy(), distances=True, out=opin.numpy(), dist_out=dpin.numpy())  # noqa: E731
    e2e_fn()
    e_tot = 0.0
    for _ in range(max(3, args.steps // 2)):
        flush.fill_(1.0)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        e2e_fn()
        e_tot += time.perf_counter() - t0
    e_n = max(3, args.steps // 2)
    e2e_value = world * B * e_n / e_tot
    h2d = qh.nbytes
    d2h = B + B * ns * 4

    hbm, hbm_kind = peaks()
    kernel_ms = k_ms / max(k_n, 1)
    # algorithmic bytes of one k_fast_valid launch: q (FP64) in, validity and FP32 distances out
    alg_bytes = B * (cst.q_dim() * 8 + 1 + ns * 4)
    achieved = alg_bytes / (kernel_ms / 1e3) / 1e9
    prof = ROOT / "profiles" / "k_fast_valid_dualarm65536.traffic.json"
    traffic = None
    if prof.exists():
        traffic = json.loads(prof.read_text()).get("dram_bytes_per_launch")

    if rank != 0:
        return
    cpu = None if args.no_cpu_baseline else cpu_baseline(robot, scene, qh)
    line = {
        "metric": "configs checked/sec",
        "value": value,
        "unit": "configs/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_per_step,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 (FP64 FK and FP64 recheck of uncertain decisions)",
        "data": "synthetic (seeded generators in plainmp_gb300/workloads.py)",
        "config": config_dict({"launch_shape": {"with_distances": list(shape_dist), "validity_only": list(shape_valid)}}),
        "e2e": {"value": e2e_value, "unit": "configs/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": all_n,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": traffic, "peak_kind": hbm_kind,
                     "kernel": "k_fast_valid", "kernel_ms": kernel_ms, "launches": k_n,
                     "note": "HBM is not the binding resource: the kernel is issue/latency bound (see profiles/)"},
        "clocks": clk.summary(),
        "plain_fp64": {"value": B / (ms_plain / 1e3), "unit": "configs/s", "ms_per_batch": ms_plain,
                       "what": "plain FP64 method, one thread per configuration, validity only"},
        "fast_validity_only": {"value": B / (ms_valid / 1e3), "unit": "configs/s", "ms_per_batch": ms_valid},
        "speedup_vs_plain": {"with_distances": ms_plain / ms_per_step, "validity_only": ms_plain / ms_valid},
        "validity_mismatches_fast_vs_plain": mismatches,
        "recheck": {"terms": st["rechecked_terms"], "configs_full": st["rechecked_configs"], "recheck_kernel_ms": r_ms / max(r_n, 1)},
    }
    if cpu is not None:
        line["cpu_baseline"] = cpu
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
