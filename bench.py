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


def _workloads():
    """The seeded generators (plainmp_gb300/workloads.py), loaded by file path: importing the
    package would load the product library, which the CPU arms must not touch."""
    import importlib.util

    name = "_pm_workloads"
    if name not in sys.modules:
        spec = importlib.util.spec_from_file_location(name, ROOT / "plainmp_gb300" / "workloads.py")
        mod = importlib.util.module_from_spec(spec)
        sys.modules[name] = mod
        spec.loader.exec_module(mod)
    return sys.modules[name]


def workload():
    W = _workloads()

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


class NvmlPoller:
    """SM clock and clock-event reasons read from NVML (the library nvidia-smi reads) every ~1 ms
    in a thread: a timed region of a few tens of ms gets many samples, where nvidia-smi's 200 ms
    period gets one or two.  Read-only queries; summary() is None when NVML cannot be loaded."""

    # nvmlClocksEventReason bits (nvml.h)
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown",
               0x80: "hw_power_brake_slowdown"}

    def __init__(self, index: int, uuid: str = "", period_s: float = 0.001):
        self.index, self.period = index, period_s
        self.uuid = uuid if not uuid or uuid.startswith("GPU-") else "GPU-" + uuid  # NVML's form of the CUDA device's UUID
        self.samples, self.max_mhz, self.lib, self.dev = [], None, None, None
        self._stop = threading.Event()
        self.t = None

    def __enter__(self):
        import ctypes as C

        try:
            lib = C.CDLL("libnvidia-ml.so.1")
            if lib.nvmlInit_v2() != 0:
                return self
            dev = C.c_void_p()
            # the CUDA device itself (NVML may number the GPUs differently), else the same index
            if not (self.uuid and lib.nvmlDeviceGetHandleByUUID(self.uuid.encode(), C.byref(dev)) == 0) and \
                    lib.nvmlDeviceGetHandleByIndex_v2(C.c_uint(self.index), C.byref(dev)) != 0:
                lib.nvmlShutdown()
                return self
            mx = C.c_uint(0)
            if lib.nvmlDeviceGetMaxClockInfo(dev, C.c_int(1), C.byref(mx)) == 0:  # NVML_CLOCK_SM
                self.max_mhz = float(mx.value)
            self.reasons_fn = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
                lib.nvmlDeviceGetCurrentClocksThrottleReasons
            self.lib, self.dev = lib, dev
        except (OSError, AttributeError):
            return self
        self.t = threading.Thread(target=self._run, daemon=True)
        self.t.start()
        return self

    def _run(self):
        import ctypes as C

        clk, rs = C.c_uint(0), C.c_ulonglong(0)
        while not self._stop.is_set():
            if self.lib.nvmlDeviceGetClockInfo(self.dev, C.c_int(1), C.byref(clk)) == 0 and \
                    self.reasons_fn(self.dev, C.byref(rs)) == 0:
                self.samples.append((float(clk.value), int(rs.value)))
            time.sleep(self.period)

    def __exit__(self, *a):
        self._stop.set()
        if self.t is not None:
            self.t.join(timeout=5)
        if self.lib is not None:
            self.lib.nvmlShutdown()

    def summary(self):
        if not self.samples:
            return None
        reasons = sorted({name for _, r in self.samples for bit, name in self.REASONS.items() if r & bit})
        return {"sm_mhz": statistics.median(s for s, _ in self.samples), "sm_max_mhz": self.max_mhz, "reasons": reasons,
                "samples": len(self.samples), "source": "NVML, every ~1 ms during the timed region"}


def issue_rate(warp_inst, kernel_ms, sm_mhz, n_sm):
    """Issue utilisation of an issue-bound kernel: warp instructions per launch (ncu
    smsp__inst_executed.sum) over the launch's CUDA-event duration, against the SM's ceiling of 4
    schedulers x 1 warp instruction per cycle at the SM clock sampled during the timed region.
    None when a figure is missing."""
    if not warp_inst or not kernel_ms or not sm_mhz or not n_sm:
        return None
    achieved = warp_inst / (kernel_ms / 1e3) / 1e9
    peak = 4.0 * n_sm * sm_mhz / 1e3
    return {"achieved": achieved, "peak": peak, "unit": "G warp instructions/s", "frac": achieved / peak}


def peaks():
    if PEAKS.exists():
        d = json.loads(PEAKS.read_text())
        return float(d.get("hbm_gbs", FALLBACK_HBM_GBS)), "measured"
    return FALLBACK_HBM_GBS, "fallback"


def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else the platform string)."""
    import platform

    try:
        r = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10)
        for ln in r.stdout.splitlines():
            if ln.startswith("Model name:"):
                return ln.split(":", 1)[1].strip() + f" ({platform.machine()})"
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for ln in Path("/proc/cpuinfo").read_text().splitlines():
            if ln.lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def _oracle_rate(oc, q, threads: int, n: int, seconds: float):
    """configs/s of the oracle's is_valid loop over slices of n configurations of q, repeated for
    about `seconds`: (rate, configurations done, repetitions)."""
    t0 = time.perf_counter()
    oc.is_valid(q[:n], threads=threads)
    dt = time.perf_counter() - t0
    reps = max(1, min(64, int(seconds / max(dt, 1e-6))))
    done = 0
    t0 = time.perf_counter()
    for r in range(reps):
        off = (r * n) % max(len(q) - n, 1)
        oc.is_valid(q[off:off + n], threads=threads)
        done += n
    return done / (time.perf_counter() - t0), done, reps


def cpu_row(seconds: float = 4.0) -> dict:
    """All-core oracle rate on the headline batch in this process (PM_ORACLE_CONTRACT selects the
    build); run by cpu_baseline in a child process for the contraction-on build."""
    from oracle import pyoracle

    robot, scene, q = workload()
    threads = os.cpu_count() or 1
    _, oc, _ = pyoracle.make_constraint(robot, scene)
    rate, done, reps = _oracle_rate(oc, q, threads, 4096, seconds)
    return {"value": rate, "unit": "configs/s", "cores": threads, "sample": f"{done} configs ({reps} x 4096)",
            "build": "-O3 -ffp-contract=fast" if pyoracle.CONTRACT else "-O3 -ffp-contract=off"}


def cpu_baseline(robot, scene, q, seconds: float = 6.0):
    """The oracle (CPU FP64 restatement of the reference's is_valid loop) on all host cores,
    over a bounded sample of the batch: validity only, as the reference computes it.  Rows: the
    bit-exact build (-ffp-contract=off, the headline figure), one core of it, and the build with
    contraction on (-ffp-contract=fast, timed in a child process)."""
    from oracle import pyoracle

    threads = os.cpu_count() or 1
    _, oc, _ = pyoracle.make_constraint(robot, scene)
    rate, done, reps = _oracle_rate(oc, q, threads, 4096, seconds)
    out = {"value": rate, "unit": "configs/s", "cores": threads, "kind": "port", "cpu_model": cpu_model(),
           "build": "-O3 -ffp-contract=off",
           "sample": f"{done} configs of the same batch ({reps} x 4096), validity only (the reference has no per-sphere distance output)"}
    # one core, as one planner process runs the reference's is_valid loop
    r1, done1, reps1 = _oracle_rate(oc, q, 1, 1024, seconds / 3)
    out["single_core"] = {"value": r1, "unit": "configs/s", "cores": 1, "sample": f"{done1} configs ({reps1} x 1024)"}
    try:
        env = dict(os.environ, PM_ORACLE_CONTRACT="1")
        r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--cpu-row"], capture_output=True, text=True, env=env,
                           timeout=600)
        out["contract_build"] = json.loads(r.stdout.strip().splitlines()[-1]) if r.returncode == 0 else \
            {"error": (r.stderr.strip().splitlines() or ["failed"])[-1]}
    except (OSError, subprocess.SubprocessError, ValueError, IndexError) as e:
        out["contract_build"] = {"error": f"{type(e).__name__}: {e}"}
    return out


C0_FLOP = 7 * 90 + 8 * 24 + 56 * 18 + 56 * (35 * 10 + 11 * 5 + 30 * 5) + 960 * 11  # per configuration, the counting rule
FP32_NOMINAL_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12  # 152 SMs x 128 FP32 lanes x FMA x 2.07 GHz


def _timer(dev, flush, stream):
    import torch

    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)

    def timed(fn, n):
        """Mean ms of fn over n runs, L2 flushed before each, CUDA events on torch's stream."""
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

    return timed


def bench_chain7(dev, timed):
    """C0 (4096 configurations) and C1 (1024 edges of 1-120 waypoints) on the 7-joint chain
    against 10 boxes, 5 spheres and 5 cylinders: the plain FP64 method vs the fast path."""
    import torch

    from plainmp_gb300 import BoxMotionValidator, scenes
    from plainmp_gb300 import workloads as W

    robot, scene = W.chain7_robot(), W.chain7_scene()
    _, cst, _ = scenes.make_constraint(robot, scene)
    from plainmp_gb300 import autotune

    Q = torch.tensor(W.chain7_configs(4096), device=dev)
    ms_plain = timed(lambda: cst.is_valid_batch(Q), 5)
    shape0, _ = autotune.autotune(cst, Q, distances=True)
    cst.set_fast_launch(*shape0)
    ms_fast = timed(lambda: cst.is_valid_fast(Q, distances=True), 10)
    same = bool(torch.equal(cst.is_valid_fast(Q), cst.is_valid_batch(Q)))
    s1, s2 = W.chain7_edges(1024)
    # waypoints checked per edge without early exit (box validator, width 0.05): floor(max|dq| / w) + 1
    wp = np.floor(np.abs(s2 - s1).max(axis=1) / 0.05).astype(np.int64) + 1
    wp_hist = {"min": int(wp.min()), "max": int(wp.max()), "mean": float(wp.mean()), "total": int(wp.sum()),
               "deciles": [int(x) for x in np.percentile(wp, np.arange(10, 100, 10))]}
    S1, S2 = torch.tensor(s1, device=dev), torch.tensor(s2, device=dev)
    mv = BoxMotionValidator(cst, [0.05] * 7)
    edge_shape, _ = autotune.autotune_edges(mv, S1, S2)
    ms_e_plain = timed(lambda: mv.check_motion_batch(S1, S2), 5)
    eout = torch.empty(S1.shape[0], dtype=torch.uint8, device=dev)
    ms_e_fast = timed(lambda: mv.check_motion_fast(S1, S2, out=eout), 10)
    same_e = bool(torch.equal(mv.check_motion_fast(S1, S2), mv.check_motion_batch(S1, S2)))
    try:  # the whole edge pipeline (setup, scan, persistent kernel, recheck) as one CUDA graph
        eg = _capture(lambda: mv.check_motion_fast(S1, S2, out=eout))
        ms_e_graph = timed(eg.replay, 10)
    except Exception:  # noqa: BLE001 - reported as null
        ms_e_graph = None
    # the composite (IneqCompositeCst) of the collision constraint and an end-link height bound:
    # one fused launch vs the members one after the other (fast collision path, plain bound)
    from plainmp_gb300 import BaseType, IneqCompositeCst, LinkPositionBoundCst

    bound = LinkPositionBoundCst(cst.get_kin(), robot.control_joints, BaseType.FIXED, robot.end_link, 2, lb=0.0)
    comp = IneqCompositeCst([cst, bound])
    cout = torch.empty(Q.shape[0], dtype=torch.uint8, device=dev)
    ms_c_fused = timed(lambda: comp.is_valid_fast(Q, out=cout), 10)
    ms_c_members = timed(lambda: cst.is_valid_fast(Q) & bound.is_valid_batch(Q), 10)
    same_c = bool(torch.equal(comp.is_valid_fast(Q), cst.is_valid_batch(Q) & bound.is_valid_batch(Q)))
    return {
        "C0": {"workload": "7-joint chain, 56 spheres, 10 boxes + 5 spheres + 5 cylinders, 4096 configurations",
               "unit": "configs/s", "plain_fp64": 4096 / (ms_plain / 1e3), "fast_with_distances": 4096 / (ms_fast / 1e3),
               "ms": {"plain_fp64": ms_plain, "fast_with_distances": ms_fast}, "validity_identical": same,
               "launch_shape": list(shape0),
               # algorithmic work per configuration with no early exit and no broad phase: FK 7 x 90,
               # rotations 8 x 24, sphere transforms 56 x 18, narrow phase 56 x (35 x 10 + 11 x 5 + 30 x 5),
               # self pairs 960 x 11; the kernels skip most of it (culling, early exit), so these
               # "effective" rates exceed the arithmetic peaks by design
               "effective": {"kflop_per_config": C0_FLOP / 1e3,
                             "fast_tflops": 4096 / (ms_fast / 1e3) * C0_FLOP / 1e12,
                             "plain_tflops": 4096 / (ms_plain / 1e3) * C0_FLOP / 1e12}},
        "C0_composite": {"workload": "the C0 batch against IneqCompositeCst([collision, end-link z >= 0])", "unit": "configs/s",
                         "fused": 4096 / (ms_c_fused / 1e3), "members_in_turn": 4096 / (ms_c_members / 1e3),
                         "ms": {"fused": ms_c_fused, "members_in_turn": ms_c_members}, "validity_identical": same_c,
                         "valid_fraction": float(comp.is_valid_fast(Q).float().mean())},
        "C1": {"workload": "1024 straight edges on the C0 chain and scene, box validator width 0.05 rad, 1-120 waypoints",
               "unit": "edges/s", "plain_fp64": 1024 / (ms_e_plain / 1e3), "fast_persistent": 1024 / (ms_e_fast / 1e3),
               "fast_cuda_graph": 1024 / (ms_e_graph / 1e3) if ms_e_graph else None,
               "ms": {"plain_fp64": ms_e_plain, "fast_persistent": ms_e_fast, "fast_cuda_graph": ms_e_graph},
               "edge_validity_identical": same_e, "waypoints_per_edge": wp_hist,
               "edge_launch_shape": list(edge_shape)},
    }


def _capture(fn):
    """A CUDA graph of fn (warmed up on a side stream first), or the capture error."""
    import torch

    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        for _ in range(2):
            fn()
    torch.cuda.current_stream().wait_stream(s)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        fn()
    return g


def ik_grad_check(cst, link, q, tgt, dev, h=1e-6, w_rot=0.1, margin=0.02):
    """Max relative error of the FP32 adjoint gradient of the C3 cost on a sample of problems, against
    central differences (h = 1e-6, FP64) of the same cost evaluated in FP64 by the library's plain
    device method (sin/cos FK link pose, exact per-sphere SDF distances).  Error per problem:
    |g - g_fd|_inf / max(1, |g_fd|_inf); problems where differences at h and h/2 disagree (a hinge
    switching inside the step) are left out, as in the gradient tests."""
    import torch

    from plainmp_gb300 import diff

    if cst.groups()["only_self"].any():  # the hinge would need the active-sphere mask
        return None
    q32 = torch.tensor(q, dtype=torch.float32, device=dev)
    Q = q32.double()  # the FD runs at exactly the FP32 point the kernel sees
    T = tgt.double()

    def qmul(a, b):
        ax, ay, az, aw = a.unbind(-1)
        bx, by, bz, bw = b.unbind(-1)
        return torch.stack([aw * bx + ax * bw + ay * bz - az * by, aw * by + ay * bw + az * bx - ax * bz,
                            aw * bz + az * bw + ax * by - ay * bx, aw * bw - ax * bx - ay * by - az * bz], -1)

    def cost64(P, Tr):
        pose = diff.link_poses(cst, P, link)
        c = ((pose[:, :3] - Tr[:, :3]) ** 2).sum(1)
        e = qmul(Tr[:, 3:] * torch.tensor([-1.0, -1.0, -1.0, 1.0], dtype=torch.float64, device=dev), pose[:, 3:])
        e = torch.where(e[:, 3:4] < 0, -e, e)
        sn = e[:, :3].norm(dim=1)
        k = torch.where(sn > 1e-12, 2.0 * torch.atan2(sn, e[:, 3]) / sn.clamp_min(1e-300), 2.0 / e[:, 3])
        c = c + w_rot * ((k[:, None] * e[:, :3]) ** 2).sum(1)
        d = torch.as_tensor(cst.sphere_distances(P, high_accuracy=True), device=dev)
        return c + (torch.clamp(margin - d, min=0.0) ** 2).sum(1)

    def fd(step):
        B, d = Q.shape
        P = Q[:, None, :].repeat(1, 2 * d, 1)
        for j in range(d):
            P[:, 2 * j, j] += step
            P[:, 2 * j + 1, j] -= step
        v = cost64(P.reshape(-1, d), T.repeat_interleave(2 * d, dim=0)).reshape(B, 2 * d)
        return (v[:, 0::2] - v[:, 1::2]) / (2 * step)

    def rel(g, ref):
        return (g - ref).abs().amax(1) / ref.abs().amax(1).clamp_min(1.0)

    g1, g2 = fd(h), fd(h / 2)
    keep = rel(g1, g2) < 1e-5
    _, g = diff.ik_cost_grad(cst, q32, tgt, link)
    err = rel(g.double(), g1)[keep]
    return {"problems": int(Q.shape[0]), "smooth": int(keep.sum()), "max_rel_err": float(err.max()) if err.numel() else None,
            "tolerance": 1e-4,
            "reference": "central differences (h = 1e-6) of the cost in FP64 by the plain device method"}


def bench_ik(dev, timed, steps=50, lr=0.05, fp32_peak=None):
    """C3: 8192 collision-aware IK problems on the C0 chain and scene, `steps` gradient steps
    each.  One gradient eval = cost + adjoint gradient of one problem at one step."""
    import torch

    from plainmp_gb300 import diff, scenes
    from plainmp_gb300 import workloads as W

    robot, scene = W.chain7_robot(), W.chain7_scene()
    kin, cst, _ = scenes.make_constraint(robot, scene)
    link = kin.get_link_ids([robot.end_link])[0]
    q0, q_star = W.ik_problems(8192)
    n = q0.shape[0]
    tgt = diff.link_poses(cst, torch.tensor(q_star, device=dev), link).float()
    Q0 = torch.tensor(q0, dtype=torch.float32, device=dev)
    lo, hi = np.array(kin.get_joint_position_limits(kin.get_joint_ids(robot.control_joints))).T
    lo_t, hi_t = torch.tensor(lo, dtype=torch.float32, device=dev), torch.tensor(hi, dtype=torch.float32, device=dev)
    ms_fused = timed(lambda: diff.ik_descend(cst, Q0, tgt, link, steps=steps, lr=lr), 5)
    c_init = diff.ik_cost_grad(cst, Q0, tgt, link, want_grad=False)
    _, c_final = diff.ik_descend(cst, Q0, tgt, link, steps=steps, lr=lr)
    qbuf = Q0.clone()

    def autograd_loop():
        q = qbuf
        for _ in range(steps):
            qq = q.detach().requires_grad_(True)
            c = diff.ik_cost(cst, qq, tgt, link)
            (g,) = torch.autograd.grad(c.sum(), qq)
            q = torch.minimum(torch.maximum(q - lr * g, lo_t), hi_t)
        return q

    ms_eager = timed(autograd_loop, 2)
    graph = None
    try:
        graph = _capture(autograd_loop)
        ms_graph = timed(graph.replay, 5)
    except Exception as e:  # noqa: BLE001 - reported in the JSON line
        ms_graph = None
        graph_err = f"{type(e).__name__}: {e}"
    grad_check = ik_grad_check(cst, link, q0[:64], tgt[:64], dev)
    evals = n * steps
    # algorithmic flops per eval (no broad phase, no early exit): forward FK 7 x 90 + 8 links x 24,
    # 56 sphere transforms x 18, narrow phase 56 x (35 x 10 boxes + 11 x 5 spheres + 30 x 5
    # cylinders); forward + adjoint counted as 3 x forward
    fwd = 7 * 90 + 8 * 24 + 56 * 18 + 56 * (35 * 10 + 11 * 5 + 30 * 5)
    flops = 3 * fwd
    achieved = evals * flops / (ms_fused / 1e3) / 1e12
    out = {
        "workload": "8192 IK problems, 7-joint chain (56 spheres) vs 10 boxes + 5 spheres + 5 cylinders, "
                    f"{steps} gradient steps, lr {lr}, cost |p-p*|^2 + 0.1 |log(R*^T R)|^2 + sum max(0, 0.02 - d_s)^2",
        "unit": "gradient evals/s",
        "fused_descent": evals / (ms_fused / 1e3),
        "autograd_eager": evals / (ms_eager / 1e3),
        "autograd_cuda_graph": evals / (ms_graph / 1e3) if ms_graph else None,
        "ms": {"fused_descent": ms_fused, "autograd_eager": ms_eager, "autograd_cuda_graph": ms_graph},
        "median_cost": {"initial": float(c_init.median()), "after_descent": float(c_final.median())},
        "gradient_check": grad_check,
        "roofline": {"bound": "fp32 issue", "achieved": achieved, "peak": fp32_peak or FP32_NOMINAL_TFLOPS, "unit": "TFLOP/s",
                     "frac": achieved / (fp32_peak or FP32_NOMINAL_TFLOPS),
                     "peak_kind": "measured (FP32 FMA microbenchmark k_fma_peak)" if fp32_peak else "nominal (FP32 FMA, 2.07 GHz)",
                     "flops_per_eval": flops, "kernel": "k_ik_cost (fused descent)"},
    }
    if ms_graph is None:
        out["autograd_cuda_graph_error"] = graph_err
    return out


def traj_cost_check(cst, q32, off, margin=0.03, n=16):
    """Relative error of the FP32 trajectory costs against the same cost in FP64, on the first n
    trajectories, at the FP32 waypoints the kernel sees: the acceleration smoothing term on the
    host, the hinge from the library's plain device method (exact FP64 per-sphere SDF distances,
    sin/cos FK).  Error per trajectory: |c - c64| / max(1, |c64|)."""
    from plainmp_gb300 import diff

    if cst.groups()["only_self"].any():  # the hinge would need the active-sphere mask
        return None
    c32 = diff.traj_cost_grad(cst, q32[:off[n]], off[:n + 1], want_grad=False)
    q = q32.astype(np.float64)
    errs = []
    for i in range(n):
        P = q[off[i]:off[i + 1]]
        d = np.asarray(cst.sphere_distances(P, high_accuracy=True))
        acc = P[2:] - 2.0 * P[1:-1] + P[:-2]
        ref = float((np.maximum(margin - d, 0.0) ** 2).sum() + (acc ** 2).sum())
        errs.append(abs(float(c32[i]) - ref) / max(1.0, abs(ref)))
    return {"trajectories": n, "max_rel_err": max(errs),
            "reference": "the same cost in FP64: smoothing on the host, hinge from the plain method's FP64 distances"}


def bench_traj(dev, timed):
    """C4: 512 trajectories (20-100 waypoints) of the planar-base chain (x, y, yaw + 7 joints)
    against the 200k-point cloud; one eval = cost + gradient of one trajectory (FK recomputed
    in the backward pass), through the torch.autograd.Function, captured in a CUDA graph."""
    import torch

    from plainmp_gb300 import diff, scenes
    from plainmp_gb300 import workloads as W

    robot = W.planar_chain7_robot()
    scene = W.Scene(cloud=W.box_surface_cloud(), cloud_radius=0.0)
    _, cst, _ = scenes.make_constraint(robot, scene)
    trajs = W.trajectories(512)
    Qh = np.concatenate(trajs, axis=0).astype(np.float32)
    off = np.concatenate([[0], np.cumsum([len(t) for t in trajs])]).astype(np.int64)
    Q = torch.tensor(Qh, device=dev)
    O = torch.tensor(off, device=dev)
    gout = torch.empty_like(Q)
    cout = torch.empty(len(trajs), device=dev)

    def fwd_bwd():
        q = Q.detach().requires_grad_(True)
        c = diff.trajectory_cost(cst, q, O)
        (g,) = torch.autograd.grad(c.sum(), q)
        gout.copy_(g)
        cout.copy_(c)

    ms_eager = timed(fwd_bwd, 5)
    try:
        graph = _capture(fwd_bwd)
        ms_graph = timed(graph.replay, 10)
        err = None
    except Exception as e:  # noqa: BLE001
        ms_graph, err = None, f"{type(e).__name__}: {e}"
    ms_direct = timed(lambda: diff.traj_cost_grad(cst, Q, O), 10)
    best = ms_graph or ms_eager
    out = {
        "workload": f"512 trajectories, {len(Qh)} waypoints (20-100 each), planar base + 7 joints (56 spheres) vs the "
                    "200k-point cloud, hinge margin 0.03 + acceleration smoothing",
        "unit": "trajectory gradient evals/s",
        "value": len(trajs) / (best / 1e3),
        "waypoints_per_s": len(Qh) / (best / 1e3),
        "ms": {"autograd_eager": ms_eager, "autograd_cuda_graph": ms_graph, "cost_and_grad_one_call": ms_direct},
    }
    if err:
        out["autograd_cuda_graph_error"] = err
    try:
        out["fp64_check"] = traj_cost_check(cst, Qh, off)
    except Exception as e:  # noqa: BLE001  (reported in the line; the rates above stand)
        out["fp64_check"] = {"error": f"{type(e).__name__}: {e}"}
    return out


def bench_single_calls(n: int = 2000):
    """Per-call latency of the calls OMPL's callbacks make, one state or one edge at a time, through
    the C ABI with host memory: the state-validity hook calls is_valid per state
    (ompl_thin_wrap.hpp:114-120), the motion validator checkMotion per edge (motion_validator.cpp:
    17-79).  Beside each, the oracle's single-core time per state or edge (its own C loop over the
    same inputs, no binding in between).  The library's figures go through ctypes (about 1 us of
    binding per call)."""
    import ctypes as C

    from oracle import pyoracle
    from plainmp_gb300 import _lib, scenes

    W = _workloads()
    lib = _lib.lib
    out = {}
    cases = [("C0", W.chain7_robot(), W.chain7_scene(), W.chain7_configs(n, seed=41)),
             ("C2", W.dualarm_robot(), W.Scene(cloud=W.box_surface_cloud(), cloud_radius=0.0), W.dualarm_configs(n, seed=42))]
    for name, robot, scene, qs in cases:
        _, cst, _ = scenes.make_constraint(robot, scene)
        _, oc, _ = pyoracle.make_constraint(robot, scene)
        qs = np.ascontiguousarray(qs)
        ok = np.zeros(1, np.uint8)
        optr = C.c_void_p(ok.ctypes.data)
        ptrs = [C.c_void_p(qs[i].ctypes.data) for i in range(n)]
        got = np.empty(n, np.uint8)
        got_f = np.empty(n, np.uint8)

        def plain(i):
            return lib.pmgpu_cst_is_valid(cst._h, ptrs[i], 1, optr, _lib.MEM_HOST, None)

        def fast(i):
            return lib.pmgpu_cst_is_valid_fast(cst._h, ptrs[i], 1, optr, None, None, _lib.MEM_HOST, None)

        per_call = {}
        for label, fn, dst in (("plain", plain, got), ("fast", fast, got_f)):
            for i in range(min(n, 50)):  # warm-up (tables, staging buffers)
                fn(i)
            t0 = time.perf_counter()
            for i in range(n):
                if fn(i) != 0:
                    raise RuntimeError(lib.pmgpu_last_error().decode())
                dst[i] = ok[0]
            per_call[label] = (time.perf_counter() - t0) / n * 1e6
        t0 = time.perf_counter()
        ref = oc.is_valid(qs, threads=1)
        cpu_us = (time.perf_counter() - t0) / n * 1e6
        out[name] = {"is_valid_per_call_us": per_call["plain"], "is_valid_fast_per_call_us": per_call["fast"],
                     "oracle_single_core_us": cpu_us,
                     "identical": bool(np.array_equal(got, ref) and np.array_equal(got_f, ref)), "calls": n}
    # one edge at a time: checkMotion of the box validator (width 0.05) on the chain's edges
    robot, scene = W.chain7_robot(), W.chain7_scene()
    _, cst, _ = scenes.make_constraint(robot, scene)
    _, oc, _ = pyoracle.make_constraint(robot, scene)
    s1, s2 = W.chain7_edges(1024)
    s1, s2 = np.ascontiguousarray(s1), np.ascontiguousarray(s2)
    width = np.full(7, 0.05)
    wptr = C.c_void_p(width.ctypes.data)
    ok = np.zeros(1, np.uint8)
    optr = C.c_void_p(ok.ctypes.data)
    ne = s1.shape[0]
    p1 = [C.c_void_p(s1[i].ctypes.data) for i in range(ne)]
    p2 = [C.c_void_p(s2[i].ctypes.data) for i in range(ne)]

    def plain_e(i):
        return lib.pmgpu_check_motion(cst._h, p1[i], p2[i], 1, 0, wptr, 0.0, optr, None, _lib.MEM_HOST, None)

    def fast_e(i):
        return lib.pmgpu_check_motion_fast(cst._h, p1[i], p2[i], 1, 0, wptr, 0.0, optr, None, _lib.MEM_HOST, None)

    per_call, outs = {}, {}
    for label, fn in (("plain", plain_e), ("fast", fast_e)):
        got = np.empty(ne, np.uint8)
        for i in range(20):
            fn(i)
        t0 = time.perf_counter()
        for i in range(ne):
            if fn(i) != 0:
                raise RuntimeError(lib.pmgpu_last_error().decode())
            got[i] = ok[0]
        per_call[label] = (time.perf_counter() - t0) / ne * 1e6
        outs[label] = got
    t0 = time.perf_counter()
    ref, _ = oc.check_motion(s1, s2, 0, width, threads=1)
    cpu_us = (time.perf_counter() - t0) / ne * 1e6
    out["C1"] = {"check_motion_per_call_us": per_call["plain"], "check_motion_fast_per_call_us": per_call["fast"],
                 "oracle_single_core_us": cpu_us,
                 "identical": bool(np.array_equal(outs["plain"], ref) and np.array_equal(outs["fast"], ref)), "calls": ne}
    out["what"] = ("per-call latency through the C ABI with host memory (one state / one edge per call, as OMPL's callbacks "
                   "call), against the oracle's single-core time per state / edge")
    return out


def bench_exact_queries(dev, timed):
    """The exact FP64 cloud queries outside the fast path: sphere_distances of 4,096 dual-arm
    configurations (120 spheres each) against the 200k-point cloud, and KDTree.sqdist_batch on 10^5
    queries near the cloud and 10^5 far from it; beside them the oracle's KD-tree (kdtree.cpp:67-96)
    on all host cores over the same queries, and whether the squared distances are identical."""
    import torch

    from oracle import pyoracle
    from plainmp_gb300 import KDTree, scenes

    W = _workloads()
    robot, scene = W.dualarm_robot(), W.Scene(cloud=W.box_surface_cloud(), cloud_radius=0.0)
    _, cst, _ = scenes.make_constraint(robot, scene)
    _, oc, osdf = pyoracle.make_constraint(robot, scene)
    Q = torch.tensor(W.dualarm_configs(4096, seed=43), device=dev)
    ms_sd = timed(lambda: cst.sphere_distances(Q), 5)
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    ref_sd = oc.sphere_distances(Q.cpu().numpy(), threads=threads)
    cpu_sd = time.perf_counter() - t0
    same_sd = bool(np.array_equal(np.asarray(cst.sphere_distances(Q).cpu()), ref_sd))
    cloud = scene.cloud.astype(np.float64)
    rng = np.random.default_rng(44)
    near = cloud[rng.integers(0, len(cloud), 100000)] + rng.normal(0.0, 0.05, (100000, 3))
    lo, hi = cloud.min(0), cloud.max(0)
    far = rng.uniform(lo - 1.5, hi + 1.5, (100000, 3))
    far = far[np.abs(far - (lo + hi) / 2).max(1) > (hi - lo).max() / 2 + 0.3][:100000]
    tree = KDTree(cloud)
    ref_cloud = pyoracle.Sdf.cloud(cloud, 0.0)
    res = {}
    for name, pts in (("near", near), ("far", far)):
        P = torch.tensor(pts, device=dev)
        ms = timed(lambda: tree.sqdist_batch(P), 5)
        t0 = time.perf_counter()
        rsq, _ = ref_cloud.nearest(pts)
        cpu_s = time.perf_counter() - t0
        res[name] = {"queries": len(pts), "gpu_ms": ms, "queries_per_s": len(pts) / (ms / 1e3),
                     "oracle_kdtree_queries_per_s_1_core": len(pts) / cpu_s,
                     "identical": bool(np.array_equal(np.asarray(tree.sqdist_batch(P).cpu()), rsq))}
    return {"sphere_distances": {"configs": 4096, "spheres": cst.n_spheres, "gpu_ms": ms_sd,
                                 "configs_per_s": 4096 / (ms_sd / 1e3), "oracle_configs_per_s": 4096 / cpu_sd,
                                 "oracle_cores": threads, "identical": same_sd},
            "kdtree_sqdist_batch": res,
            "what": "exact FP64 nearest-point queries (cell lists near the cloud, super-blocks elsewhere) vs the oracle KD-tree"}


def run_reference(args):
    """The reference arm: the CPU restatement of the reference's is_valid loop (kind "port"; the
    reference itself does not build here) on all host cores, over the whole 65,536-configuration
    batch per step.  It loads the oracle alone: the seeded generators come by file path, so the
    product library stays out of this process."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    robot, scene, q = workload()
    from oracle import pyoracle

    threads = os.cpu_count() or 1
    _, oc, _ = pyoracle.make_constraint(robot, scene)
    for w in range(args.warmup):
        oc.is_valid(q, threads=threads)
    times = []
    for k in range(args.steps):
        t0 = time.perf_counter()
        oc.is_valid(q, threads=threads)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = B * args.steps / total
    line = {
        "impl": "reference", "metric": "configs checked/sec", "value": value, "unit": "configs/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": config_dict({"l2": "not applicable (CPU)"}),
        "cpu_baseline": {"value": value, "unit": "configs/s", "cores": threads, "kind": "port", "cpu_model": cpu_model(),
                         "build": "-O3 -ffp-contract=off",
                         "sample": f"the whole {B}-configuration batch per step, validity only (the reference has no "
                                   "per-sphere distance output)"},
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
    ap.add_argument("--headline-only", action="store_true", help="skip the C0/C1/C3/C4 side measurements")
    ap.add_argument("--cpu-row", action="store_true", help=argparse.SUPPRESS)
    args = ap.parse_args()
    if args.cpu_row:
        print(json.dumps(cpu_row()), flush=True)
        return
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

    from plainmp_gb300 import replicas

    robot, scene, _ = workload()
    # weak scaling: every rank checks its own B-configuration slice of a world * B batch
    from plainmp_gb300 import workloads as W

    a, b = replicas.shard(world * B, rank, world)
    qh = W.dualarm_configs(world * B)[a:b] if world > 1 else W.dualarm_configs(B)
    kin, cst, sdf = scenes.make_constraint(robot, scene)
    dev = torch.device("cuda", local)
    Q = torch.tensor(qh, device=dev)
    ns = cst.n_spheres
    out = torch.empty(B, dtype=torch.uint8, device=dev)
    dout = torch.empty((B, ns), dtype=torch.float32, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)

    from plainmp_gb300 import autotune

    shape_valid, _ = autotune.autotune(cst, Q, distances=False)
    tune_valid = cst.get_fast_tuning()
    shape_dist, _ = autotune.autotune(cst, Q, distances=True)
    tune_dist = cst.get_fast_tuning()

    def step():
        cst.is_valid_fast(Q, distances=True, out=out, dist_out=dout)

    def barrier():
        torch.cuda.synchronize(dev)
        if dist is not None:
            dist.barrier()

    for _ in range(args.warmup):
        step()
    barrier()
    # The step as a CUDA graph of the same API call (captured after the warm-up): the replay launches
    # its memsets and kernels without the per-call host work in between.  The eager call is timed
    # below as well.
    graph = _capture(step)
    for _ in range(args.warmup):
        graph.replay()
    barrier()
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    total_ms = 0.0
    with ClockSampler(local) as clk, NvmlPoller(local, str(getattr(torch.cuda.get_device_properties(dev), "uuid", "") or "")) as nv:
        for _ in range(args.steps):
            flush.fill_(1.0)
            barrier()
            start.record(stream)
            graph.replay()
            end.record(stream)
            end.synchronize()
            total_ms += start.elapsed_time(end)
    barrier()
    total_ms = replicas.max_over_ranks(total_ms, dist, dev)
    ms_per_step = total_ms / args.steps
    value = world * B * args.steps / (total_ms / 1e3)
    # the same steps eagerly (one API call each), with the library's per-kernel event timing: the
    # kernel durations of the roofline and the launch count
    _lib.profile_read("*")
    _lib.profile_enable(True)
    eager_ms = 0.0
    for _ in range(args.steps):
        flush.fill_(1.0)
        barrier()
        start.record(stream)
        step()
        end.record(stream)
        end.synchronize()
        eager_ms += start.elapsed_time(end)
    barrier()
    _lib.profile_enable(False)
    k_ms, k_n = _lib.profile_read("k_fast_valid")
    h_ms, h_n = _lib.profile_read("k_hard_queries")
    r_ms, r_n = _lib.profile_read("k_fast_recheck")
    rest_ms, rest_n = _lib.profile_read("*")
    all_n = k_n + h_n + r_n + rest_n
    eager_ms = replicas.max_over_ranks(eager_ms, dist, dev) / args.steps

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
    cst.set_fast_tuning(*tune_valid)
    ms_valid_eager = timed(lambda: cst.is_valid_fast(Q, out=out), 5)
    # validity only as a CUDA graph of the same call, as the headline step; and its kernel time
    g_valid = _capture(lambda: cst.is_valid_fast(Q, out=out))
    ms_valid = timed(g_valid.replay, 5)
    _lib.profile_read("*")
    _lib.profile_enable(True)
    for _ in range(3):
        cst.is_valid_fast(Q, out=out)
    torch.cuda.synchronize(dev)
    _lib.profile_enable(False)
    kv_ms, kv_n = _lib.profile_read("k_fast_valid")
    kvr_ms, kvr_n = _lib.profile_read("k_fast_recheck")
    _lib.profile_read("*")
    del g_valid
    cst.set_fast_launch(*shape_dist)
    cst.set_fast_tuning(*tune_dist)
    ms_plain = timed(lambda: cst.is_valid_batch(Q), 3)
    ok_fast = cst.is_valid_fast(Q).cpu().numpy()
    ok_plain = cst.is_valid_batch(Q).cpu().numpy()
    mismatches = int((ok_fast != ok_plain).sum())
    _, st = cst.is_valid_fast(Q, stats=True)
    # FP32 distance error on a sample: the fast path's per-sphere distances against the plain FP64
    # method's (both clamped at the 0.1 m cutoff)
    n_err = min(B, 4096)
    _, d32 = cst.is_valid_fast(Q[:n_err], distances=True)
    d64 = torch.clamp(torch.as_tensor(cst.sphere_distances(Q[:n_err])), max=0.1)
    dist_err = float((d32.double() - d64).abs().max())

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
    # the step's two main kernels: k_fast_valid, then k_hard_queries answering its hard cloud queries
    kernel_ms = (k_ms + h_ms) / max(k_n, 1)
    # algorithmic bytes of one step's kernels: q (FP64) in, validity and FP32 distances out
    alg_bytes = B * (cst.q_dim() * 8 + 1 + ns * 4)
    achieved = alg_bytes / (kernel_ms / 1e3) / 1e9
    prof = ROOT / "profiles" / "k_fast_valid_dualarm65536.traffic.json"
    traffic, issue, inst, l2 = None, None, {}, None
    if prof.exists():
        pj = json.loads(prof.read_text())
        traffic, issue = pj.get("dram_bytes_per_launch"), pj.get("issue_active_pct")
        inst = {k: v.get("warp_instructions") for k, v in pj.get("per_kernel", {}).items()}
        l2 = pj.get("l2_bytes_per_launch")
    clocks = nv.summary()
    if clocks is None:
        clocks = clk.summary()
    else:
        clocks["nvidia_smi"] = clk.summary()
    n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
    k_each = {"k_fast_valid": k_ms / max(k_n, 1), "k_hard_queries": h_ms / max(h_n, 1)}
    issue_each = {k: issue_rate(inst.get(k), k_each[k], clocks["sm_mhz"], n_sm) for k in k_each}
    issue_step = issue_rate(sum(v or 0 for v in inst.values()), kernel_ms, clocks["sm_mhz"], n_sm)
    if issue_step is not None:
        issue_step.update({"per_kernel": issue_each,
                           "instructions": "ncu smsp__inst_executed.sum of one launch of each kernel at launch shape (16, 256), "
                                           "profiles/k_fast_valid_dualarm65536.traffic.json"})

    side = None
    fma_peaks = None
    if rank == 0 and not args.headline_only:
        # measured FMA throughput of this GPU: the denominator of the arithmetic-bound rooflines
        fma_peaks = {"fp32_fma_tflops": _lib.measure_fma_peak(False), "fp64_fma_tflops": _lib.measure_fma_peak(True),
                 "how": "k_fma_peak: 8 independent FMA chains per thread, 64 warps per SM, best of 5 launches (CUDA events)"}
        timed2 = _timer(dev, flush, stream)
        side = bench_chain7(dev, timed2)
        side["C3"] = bench_ik(dev, timed2, fp32_peak=fma_peaks["fp32_fma_tflops"])
        side["C4"] = bench_traj(dev, timed2)
        side["exact_queries"] = bench_exact_queries(dev, timed2)
        side["single_calls"] = bench_single_calls()

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
        "config": config_dict({"launch_shape": {"with_distances": list(shape_dist), "validity_only": list(shape_valid)},
                               "autotuned": {
                                   "with_distances": {"k_fast_valid": {"configs_per_block": shape_dist[0], "threads": shape_dist[1],
                                                                       "sphere_tile": tune_dist[0]},
                                                      "k_hard_queries": {"blocks_per_sm": tune_dist[1], "threads": 256}},
                                   "validity_only": {"k_fast_valid": {"configs_per_block": shape_valid[0], "threads": shape_valid[1],
                                                                      "sphere_tile": tune_valid[0]}},
                                   "sphere_tile_0": "the least tile, 32 / configs_per_block spheres per warp row"},
                               "cloud_grid": sdf.stats()}),
        "e2e": {"value": e2e_value, "unit": "configs/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "step": "one CUDA-graph replay of is_valid_fast(Q, distances=True) on the resident batch (memsets, k_fast_valid, "
                "k_hard_queries, k_fast_recheck); kernel durations from the same steps run eagerly right after",
        "api_eager": {"value": world * B / (eager_ms / 1e3), "unit": "configs/s", "ms_per_step": eager_ms,
                      "what": "the same step as one eager API call (host work between the launches included)"},
        "gpu_launches": all_n,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": traffic, "peak_kind": hbm_kind,
                     "kernel": "k_fast_valid + k_hard_queries", "kernel_ms": kernel_ms, "launches": k_n,
                     "kernel_ms_each": {"k_fast_valid": k_ms / max(k_n, 1), "k_hard_queries": h_ms / max(h_n, 1),
                                        "k_fast_recheck": r_ms / max(r_n, 1)},
                     "note": "HBM is not the binding resource: the kernel is issue/latency bound"
                             + (f" (ncu: SM issue active {issue} %, profiles/k_fast_valid_dualarm65536.md)" if issue else ""),
                     "issue": issue_step,
                     "l2": None if not l2 else {"bytes": l2, "achieved_gbs": l2 / (kernel_ms / 1e3) / 1e9,
                                                "sector_pct_of_peak_ncu": {k: v.get("l2_sector_pct_of_peak")
                                                                           for k, v in pj.get("per_kernel", {}).items()},
                                                "bytes_from": "ncu lts__t_sectors.sum x 32 B of one launch of each kernel"}},
        "clocks": clocks,
        "plain_fp64": {"value": B / (ms_plain / 1e3), "unit": "configs/s", "ms_per_batch": ms_plain,
                       "what": "plain FP64 method, one thread per configuration, validity only"},
        "fast_validity_only": {"value": B / (ms_valid / 1e3), "unit": "configs/s", "ms_per_batch": ms_valid,
                               "ms_per_batch_eager_call": ms_valid_eager,
                               "kernel_ms": {"k_fast_valid": kv_ms / max(kv_n, 1), "k_fast_recheck": kvr_ms / max(kvr_n, 1)},
                               "how": "CUDA graph replay of is_valid_fast (as the headline step); the eager call beside it"},
        "speedup_vs_plain": {"with_distances": ms_plain / ms_per_step, "validity_only": ms_plain / ms_valid},
        "validity_mismatches_fast_vs_plain": mismatches,
        "recheck": {"terms": st["rechecked_terms"], "terms_per_config": st["rechecked_terms"] / B,
                    "configs_full": st["rechecked_configs"], "recheck_kernel_ms": r_ms / max(r_n, 1)},
        "distance_error": {"sample_configs": n_err, "max_abs_m": dist_err,
                           "vs": "plain FP64 per-sphere distances, both clamped at 0.1 m"},
    }
    if cpu is not None:
        line["cpu_baseline"] = cpu
    if fma_peaks is not None:
        line["measured_peaks"] = fma_peaks
    if side is not None:
        line["workloads"] = side
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
