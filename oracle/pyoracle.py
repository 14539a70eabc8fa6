"""Test infrastructure only -- NOT part of the product.

ctypes glue for the CPU FP64 restatement in oracle/oracle.cpp.  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg import this module.  The URDF is read
here with xml.etree (independently of the product's C++ reader) and handed to the oracle as
arrays; the urdfdom semantics (number parsing, axis default, joint-name child order) are
restated by the oracle.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import xml.etree.ElementTree as ET
from pathlib import Path
from typing import List, Optional, Sequence, Tuple

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
# PM_ORACLE_CONTRACT=1 selects a second build with floating-point contraction on
# (-ffp-contract=fast: FMA where the compiler finds one, the GNU dialects' default).  Its results
# may differ from the restatement's in the last bits; it exists only as a CPU timing row.
CONTRACT = os.environ.get("PM_ORACLE_CONTRACT", "") == "1"
LIB = BUILD / ("liboracle_contract.so" if CONTRACT else "liboracle.so")

_TYPES = {"revolute": 1, "continuous": 2, "prismatic": 3, "floating": 4, "planar": 5, "fixed": 6}


def build(force: bool = False, contract: bool = CONTRACT) -> Path:
    """Compile the oracle (g++, -O3 -ffp-contract=off; with contract, -ffp-contract=fast)."""
    BUILD.mkdir(exist_ok=True)
    src = HERE / "oracle.cpp"
    lib_path = BUILD / ("liboracle_contract.so" if contract else "liboracle.so")
    if lib_path.exists() and not force and lib_path.stat().st_mtime > src.stat().st_mtime:
        return lib_path
    tmp = BUILD / f"{lib_path.stem}.{os.getpid()}.so"
    cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-O3", "-ffp-contract=fast" if contract else "-ffp-contract=off", "-fPIC",
           "-shared", "-pthread", str(src), "-o", str(tmp)]
    subprocess.run(cmd, check=True)
    os.replace(tmp, lib_path)
    return lib_path


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        L.orc_last_error.restype = C.c_char_p
        _lib = L
    return _lib


def _chk(rc):
    if rc != 0:
        raise RuntimeError(lib().orc_last_error().decode())


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _i32(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _strs(names):
    arr = (C.c_char_p * max(len(names), 1))()
    for i, n in enumerate(names):
        arr[i] = n.encode()
    return arr


def _vec3(s: Optional[str], default):
    if s is None:
        return list(default)
    parts = [p for p in s.split(" ") if p != ""]
    if len(parts) != 3:
        raise ValueError(f"expected 3 numbers in {s!r}")
    return [float(p) for p in parts]


def parse_urdf(xml: str):
    root = ET.fromstring(xml)
    links = [l.get("name") for l in root.findall("link")]
    idx = {n: i for i, n in enumerate(links)}
    joints = []
    for j in root.findall("joint"):
        t = _TYPES[j.get("type")]
        o = j.find("origin")
        xyz = _vec3(o.get("xyz") if o is not None else None, (0, 0, 0))
        rpy_s = o.get("rpy") if o is not None else None
        rpy = _vec3(rpy_s, (0, 0, 0))
        ax = j.find("axis")
        axis = [1.0, 0.0, 0.0]
        if t not in (4, 6) and ax is not None and ax.get("xyz") is not None:
            axis = _vec3(ax.get("xyz"), (1, 0, 0))
        lim = j.find("limit")
        lo = float(lim.get("lower", 0.0)) if lim is not None else 0.0
        hi = float(lim.get("upper", 0.0)) if lim is not None else 0.0
        joints.append(dict(name=j.get("name"), type=t, parent=idx[j.find("parent").get("link")],
                           child=idx[j.find("child").get("link")], xyz=xyz, rpy=rpy, has_rpy=rpy_s is not None, axis=axis,
                           lower=lo, upper=hi))
    return links, joints


class Model:
    def __init__(self, urdf: str):
        links, joints = parse_urdf(urdf)
        n = len(joints)
        xyz = np.array([j["xyz"] for j in joints] or np.zeros((0, 3)), dtype=np.float64).reshape(-1)
        rpy = np.array([j["rpy"] for j in joints] or np.zeros((0, 3)), dtype=np.float64).reshape(-1)
        axis = np.array([j["axis"] for j in joints] or np.zeros((0, 3)), dtype=np.float64).reshape(-1)
        has = np.array([1 if j["has_rpy"] else 0 for j in joints] or [0], dtype=np.int32)
        types = np.array([j["type"] for j in joints] or [0], dtype=np.int32)
        par = np.array([j["parent"] for j in joints] or [0], dtype=np.int32)
        chi = np.array([j["child"] for j in joints] or [0], dtype=np.int32)
        lo = np.array([j["lower"] for j in joints] or [0.0], dtype=np.float64)
        hi = np.array([j["upper"] for j in joints] or [0.0], dtype=np.float64)
        h = C.c_void_p()
        _chk(lib().orc_model_create(len(links), _strs(links), n, _strs([j["name"] for j in joints]), _i32(types), _i32(par), _i32(chi),
                                    _d(xyz), _d(rpy), _i32(has), _d(axis), _d(lo), _d(hi), C.byref(h)))
        self.h = h
        nl, nd = C.c_int(), C.c_int()
        lib().orc_model_counts(h, C.byref(nl), C.byref(nd))
        self.n_link, self.n_dof = nl.value, nd.value

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_model_destroy(self.h)

    def link_id(self, name: str) -> int:
        out = C.c_int()
        _chk(lib().orc_model_link_id(self.h, name.encode(), C.byref(out)))
        return out.value

    def joint_id(self, name: str) -> int:
        out = C.c_int()
        _chk(lib().orc_model_joint_id(self.h, name.encode(), C.byref(out)))
        return out.value

    def structure(self):
        par = np.empty(self.n_link, dtype=np.int32)
        jc = np.empty(max(self.n_dof, 1), dtype=np.int32)
        jq = np.empty(max(self.n_dof, 1), dtype=np.int32)
        tf = np.empty((self.n_link, 7))
        tq = np.empty(self.n_link, dtype=np.int32)
        lib().orc_model_structure(self.h, _i32(par), _i32(jc), _i32(jq), _d(tf), _i32(tq))
        return {"link_parent": par, "joint_child": jc[: self.n_dof], "joint_origin_qid": jq[: self.n_dof], "link_tf7": tf,
                "link_tf_qid": tq}

    def set_joint_positions(self, ids, q, accurate=True):
        ids = np.asarray(ids, dtype=np.int32)
        q = np.ascontiguousarray(q, dtype=np.float64)
        _chk(lib().orc_model_set_joint_positions(self.h, _i32(ids), len(ids), _d(q), int(accurate)))

    def set_base_pose(self, pose7):
        p = np.ascontiguousarray(pose7, dtype=np.float64)
        _chk(lib().orc_model_set_base_pose(self.h, _d(p)))

    def link_pose(self, link: int) -> np.ndarray:
        out = np.empty(7)
        _chk(lib().orc_model_link_pose(self.h, link, _d(out)))
        return out

    def link_jacobian(self, elink: int, ids, rot_type: int = 0, base_type: int = 0) -> np.ndarray:
        ids = np.asarray(ids, dtype=np.int32)
        dimj = 3 + (rot_type == 1) * 3 + (rot_type == 2) * 4
        dof = len(ids) + (base_type == 1) * 6 + (base_type == 2) * 3
        out = np.empty(dimj * dof)
        _chk(lib().orc_model_link_jacobian(self.h, elink, _i32(ids), len(ids), rot_type, base_type, _d(out)))
        return out.reshape(dof, dimj).T


class Sdf:
    def __init__(self, h, keep=()):
        self.h = h
        self.keep = list(keep)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_sdf_destroy(self.h)

    @staticmethod
    def box(width, pos, rot):
        h = C.c_void_p()
        _chk(lib().orc_sdf_box(_d(np.ascontiguousarray(width, dtype=np.float64)), _d(np.ascontiguousarray(pos, dtype=np.float64)),
                               _d(np.ascontiguousarray(rot, dtype=np.float64)), C.byref(h)))
        return Sdf(h)

    @staticmethod
    def cylinder(r, hgt, pos, rot):
        h = C.c_void_p()
        _chk(lib().orc_sdf_cylinder(C.c_double(r), C.c_double(hgt), _d(np.ascontiguousarray(pos, dtype=np.float64)),
                                    _d(np.ascontiguousarray(rot, dtype=np.float64)), C.byref(h)))
        return Sdf(h)

    @staticmethod
    def sphere(r, pos, rot):
        h = C.c_void_p()
        _chk(lib().orc_sdf_sphere(C.c_double(r), _d(np.ascontiguousarray(pos, dtype=np.float64)),
                                  _d(np.ascontiguousarray(rot, dtype=np.float64)), C.byref(h)))
        return Sdf(h)

    @staticmethod
    def ground(height):
        h = C.c_void_p()
        _chk(lib().orc_sdf_ground(C.c_double(height), C.byref(h)))
        return Sdf(h)

    @staticmethod
    def cloud(points, radius):
        p = np.ascontiguousarray(points, dtype=np.float64)
        h = C.c_void_p()
        _chk(lib().orc_sdf_cloud(_d(p), C.c_longlong(p.shape[0]), C.c_double(radius), C.byref(h)))
        return Sdf(h)

    @staticmethod
    def union(members: Sequence["Sdf"]):
        arr = (C.c_void_p * max(len(members), 1))(*[m.h for m in members])
        h = C.c_void_p()
        _chk(lib().orc_sdf_union(arr, len(members), C.byref(h)))
        return Sdf(h, members)

    def translate(self, t):
        _chk(lib().orc_sdf_translate(self.h, _d(np.ascontiguousarray(t, dtype=np.float64))))

    def rotate_z(self, a):
        _chk(lib().orc_sdf_rotate_z(self.h, C.c_double(a)))

    def info(self):
        lb, ub = np.empty(3), np.empty(3)
        fl = np.empty(2, dtype=np.int32)
        lib().orc_sdf_info(self.h, _d(lb), _d(ub), _i32(fl))
        return lb, ub, bool(fl[0]), bool(fl[1])

    def evaluate(self, pts):
        p = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 3)
        out = np.empty(p.shape[0])
        lib().orc_sdf_evaluate(self.h, _d(p), C.c_longlong(p.shape[0]), _d(out))
        return out

    def is_outside(self, pts, radii):
        p = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 3)
        r = np.ascontiguousarray(np.broadcast_to(radii, (p.shape[0],)), dtype=np.float64)
        out = np.empty(p.shape[0], dtype=np.uint8)
        lib().orc_sdf_is_outside(self.h, _d(p), C.c_longlong(p.shape[0]), _d(r), out.ctypes.data_as(C.POINTER(C.c_ubyte)))
        return out

    def is_outside_aabb(self, pts, radii):
        p = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 3)
        r = np.ascontiguousarray(np.broadcast_to(radii, (p.shape[0],)), dtype=np.float64)
        out = np.empty(p.shape[0], dtype=np.uint8)
        lib().orc_sdf_is_outside_aabb(self.h, _d(p), C.c_longlong(p.shape[0]), _d(r), out.ctypes.data_as(C.POINTER(C.c_ubyte)))
        return out

    def nearest(self, pts):
        p = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 3)
        sq = np.empty(p.shape[0])
        nr = np.empty((p.shape[0], 3))
        _chk(lib().orc_cloud_nearest(self.h, _d(p), C.c_longlong(p.shape[0]), _d(sq), _d(nr)))
        return sq, nr


class Cst:
    """SphereCollisionCst restatement (primitive_sphere_collision.cpp)."""

    def __init__(self, model: Model, joints: Sequence[str], base_type: int, specs, pairs: Sequence[Tuple[str, str]],
                 fixed_sdf: Optional[Sdf] = None, reorder: bool = True):
        self.model = model
        counts = np.array([s.radii.shape[0] for s in specs], dtype=np.int32)
        rel = np.ascontiguousarray(np.concatenate([np.asarray(s.relative_positions, dtype=np.float64).T for s in specs], axis=0)
                                   if specs else np.zeros((0, 3)))
        radii = np.ascontiguousarray(np.concatenate([np.asarray(s.radii, dtype=np.float64) for s in specs]) if specs else np.zeros(0))
        only = np.array([1 if s.only_self_collision else 0 for s in specs] or [0], dtype=np.int32)
        h = C.c_void_p()
        _chk(lib().orc_cst_create(model.h, _strs(list(joints)), len(joints), base_type, len(specs),
                                  _strs([s.parent_link_name for s in specs]), _i32(counts), _d(rel), _d(radii), _i32(only), len(pairs),
                                  _strs([a for a, _ in pairs]), _strs([b for _, b in pairs]), fixed_sdf.h if fixed_sdf else None,
                                  int(reorder), C.byref(h)))
        self.h = h
        self.sdf = None
        qd, cd, ns = C.c_int(), C.c_int(), C.c_int()
        lib().orc_cst_dims(h, C.byref(qd), C.byref(cd), C.byref(ns))
        self.q_dim, self.n_spheres = qd.value, ns.value
        self.n_groups = len(specs)
        # per sphere: its group is self-only (group order is the spec order; reordering is within a group)
        self._self_only = np.repeat(np.array([bool(s.only_self_collision) for s in specs], dtype=bool), counts) \
            if specs else np.zeros(0, dtype=bool)

    def sphere_self_only(self) -> np.ndarray:
        return self._self_only

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_cst_destroy(self.h)

    def set_sdf(self, sdf: Optional[Sdf]):
        self.sdf = sdf
        lib().orc_cst_set_sdf(self.h, sdf.h if sdf else None)

    @property
    def cst_dim(self):
        qd, cd, ns = C.c_int(), C.c_int(), C.c_int()
        lib().orc_cst_dims(self.h, C.byref(qd), C.byref(cd), C.byref(ns))
        return cd.value

    def groups(self):
        ng, ns = self.n_groups, self.n_spheres
        link = np.empty(max(ng, 1), dtype=np.int32)
        gr = np.empty(max(ng, 1))
        grel = np.empty((max(ng, 1), 3))
        only = np.empty(max(ng, 1), dtype=np.int32)
        rel = np.empty((max(ns, 1), 3))
        radii = np.empty(max(ns, 1))
        lib().orc_cst_groups(self.h, _i32(link), _d(gr), _d(grel), _i32(only), _d(rel), _d(radii))
        return {"link": link[:ng], "radius": gr[:ng], "centre": grel[:ng], "only_self": only[:ng], "rel": rel[:ns], "radii": radii[:ns]}

    def is_valid(self, Q, threads: int = 1) -> np.ndarray:
        Q = np.ascontiguousarray(Q, dtype=np.float64).reshape(-1, self.q_dim)
        out = np.empty(Q.shape[0], dtype=np.uint8)
        _chk(lib().orc_cst_is_valid(self.h, _d(Q), C.c_longlong(Q.shape[0]), out.ctypes.data_as(C.POINTER(C.c_ubyte)), threads))
        return out

    def evaluate(self, Q, threads: int = 1):
        Q = np.ascontiguousarray(Q, dtype=np.float64).reshape(-1, self.q_dim)
        m = self.cst_dim
        vals = np.empty((Q.shape[0], m))
        jac = np.empty((Q.shape[0], m, self.q_dim))
        _chk(lib().orc_cst_evaluate(self.h, _d(Q), C.c_longlong(Q.shape[0]), _d(vals), _d(jac), threads))
        return vals, jac

    def sphere_distances(self, Q, high_accuracy=False, threads: int = 1, centres=False):
        Q = np.ascontiguousarray(Q, dtype=np.float64).reshape(-1, self.q_dim)
        dist = np.empty((Q.shape[0], self.n_spheres))
        cen = np.empty((Q.shape[0], self.n_spheres, 3))
        _chk(lib().orc_cst_sphere_distances(self.h, _d(Q), C.c_longlong(Q.shape[0]), int(high_accuracy), _d(dist), _d(cen), threads))
        return (dist, cen) if centres else dist

    def link_poses(self, Q, link: int, threads: int = 1) -> np.ndarray:
        """(B, 7) [x y z qx qy qz qw] of `link` after update_kintree(q, high_accuracy=True)."""
        Q = np.ascontiguousarray(Q, dtype=np.float64).reshape(-1, self.q_dim)
        out = np.empty((Q.shape[0], 7))
        _chk(lib().orc_cst_link_poses(self.h, _d(Q), C.c_longlong(Q.shape[0]), int(link), _d(out), threads))
        return out

    def check_motion(self, S1, S2, kind: int = 0, width=None, resolution: float = 0.05, threads: int = 1):
        S1 = np.ascontiguousarray(S1, dtype=np.float64).reshape(-1, self.q_dim)
        S2 = np.ascontiguousarray(S2, dtype=np.float64).reshape(-1, self.q_dim)
        w = np.ascontiguousarray(width if width is not None else np.zeros(self.q_dim), dtype=np.float64)
        out = np.empty(S1.shape[0], dtype=np.uint8)
        cnt = C.c_longlong(0)
        _chk(lib().orc_check_motion(self.h, _d(S1), _d(S2), C.c_longlong(S1.shape[0]), kind, _d(w), C.c_double(resolution),
                                    out.ctypes.data_as(C.POINTER(C.c_ubyte)), C.byref(cnt), threads))
        return out, int(cnt.value)

    def update_kintree(self, q, high_accuracy=True):
        q = np.ascontiguousarray(q, dtype=np.float64)
        _chk(lib().orc_cst_update_kintree(self.h, _d(q), int(high_accuracy)))


def sequence_table(n_max: int = 128) -> np.ndarray:
    out = np.empty((n_max, n_max), dtype=np.int64)
    lib().orc_sequence_table(n_max, out.ctypes.data_as(C.POINTER(C.c_longlong)))
    return out


def approx_sin_cos(x) -> Tuple[np.ndarray, np.ndarray]:
    x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1)
    s, c = np.empty_like(x), np.empty_like(x)
    lib().orc_approx_sin_cos(_d(x), C.c_longlong(x.shape[0]), _d(s), _d(c))
    return s, c


def scene_sdf(scene) -> Optional[Sdf]:
    """Oracle SDF for a plainmp_gb300.workloads.Scene."""
    if scene is None:
        return None
    if scene.cloud is not None:
        return Sdf.cloud(scene.cloud.astype(np.float64), scene.cloud_radius)
    members = []
    for p in scene.primitives:
        if p.kind == "box":
            members.append(Sdf.box(p.size, p.position, p.rotation))
        elif p.kind == "sphere":
            members.append(Sdf.sphere(p.size[0], p.position, p.rotation))
        else:
            members.append(Sdf.cylinder(p.size[0], p.size[1], p.position, p.rotation))
    return Sdf.union(members) if members else None


def make_constraint(robot, scene=None, self_collision: bool = True, reorder: bool = True):
    base = {"FIXED": 0, "FLOATING": 1, "PLANAR": 2}[robot.base_type]
    m = Model(robot.urdf)
    c = Cst(m, robot.control_joints, base, robot.spheres, robot.self_pairs if self_collision else [], None, reorder)
    sdf = scene_sdf(scene)
    if sdf is not None:
        c.set_sdf(sdf)
    return m, c, sdf


# ------------------------------------------------------------------ FP64 costs (differentiable paths)
def _qmul(a, b):
    ax, ay, az, aw = np.moveaxis(a, -1, 0)
    bx, by, bz, bw = np.moveaxis(b, -1, 0)
    return np.stack([aw * bx + ax * bw + ay * bz - az * by, aw * by + ay * bw + az * bx - ax * bz,
                     aw * bz + az * bw + ax * by - ay * bx, aw * bw - ax * bx - ay * by - az * bz], axis=-1)


def rotvec_error(q, qt):
    """phi = log(R(qt)^T R(q)) as a rotation vector (shortest arc), quaternions [x y z w]."""
    e = _qmul(qt * np.array([-1.0, -1.0, -1.0, 1.0]), q)
    e = np.where(e[..., 3:4] < 0, -e, e)
    s = np.linalg.norm(e[..., :3], axis=-1)
    k = np.where(s > 1e-12, 2.0 * np.arctan2(s, e[..., 3]) / np.maximum(s, 1e-300), 2.0 / e[..., 3])
    return k[..., None] * e[..., :3]


def ik_cost(cst: "Cst", Q, target, link: int, w_pos=1.0, w_rot=0.1, w_col=1.0, margin=0.02, threads: int = 1):
    """FP64 collision-aware IK cost: w_pos ||p - p*||^2 + w_rot ||log(R*^T R)||^2 of `link`
    plus w_col sum_s max(0, margin - d_s)^2, d_s the per-sphere min of SDF.evaluate - r
    (orc_cst_sphere_distances with sin/cos FK).  target: (B, 7) [x y z qx qy qz qw]."""
    Q = np.ascontiguousarray(Q, dtype=np.float64).reshape(-1, cst.q_dim)
    cost = np.zeros(Q.shape[0])
    if link >= 0 and target is not None:
        pose = cst.link_poses(Q, link, threads=threads)
        T = np.asarray(target, dtype=np.float64).reshape(-1, 7)
        cost += w_pos * np.sum((pose[:, :3] - T[:, :3]) ** 2, axis=1)
        cost += w_rot * np.sum(rotvec_error(pose[:, 3:], T[:, 3:]) ** 2, axis=1)
    if w_col != 0.0:
        d = cst.sphere_distances(Q, high_accuracy=True, threads=threads)
        active = ~np.asarray(cst.sphere_self_only(), dtype=bool)
        h = np.maximum(margin - d[:, active], 0.0)
        cost += w_col * np.sum(h * h, axis=1)
    return cost


def smooth_cost(Q, dof_weights=None):
    """sum_t sum_d w_d^2 (q[t+1] - 2 q[t] + q[t-1])_d^2 = x^T A x with A of smoothcost_fullmat
    (src/plainmp/nlp_solver/sqp_based_solver.py:74-97)."""
    Q = np.asarray(Q, dtype=np.float64)
    if Q.shape[0] < 3:
        return 0.0
    acc = Q[2:] - 2.0 * Q[1:-1] + Q[:-2]
    w2 = np.ones(Q.shape[1]) if dof_weights is None else np.asarray(dof_weights, dtype=np.float64) ** 2
    return float(np.sum(acc * acc * w2))


def traj_cost(cst: "Cst", Q, offsets, w_col=1.0, margin=0.03, w_smooth=1.0, dof_weights=None, threads: int = 1):
    """FP64 per-trajectory cost: w_smooth * smooth_cost + w_col * hinge sum over all waypoints."""
    Q = np.ascontiguousarray(Q, dtype=np.float64).reshape(-1, cst.q_dim)
    col = ik_cost(cst, Q, None, -1, w_col=w_col, margin=margin, threads=threads)
    out = np.empty(len(offsets) - 1)
    for i in range(len(offsets) - 1):
        a, b = int(offsets[i]), int(offsets[i + 1])
        out[i] = w_smooth * smooth_cost(Q[a:b], dof_weights) + np.sum(col[a:b])
    return out
