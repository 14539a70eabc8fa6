"""Shared helpers for the parity tests."""
import json
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"


def golden(name: str):
    return json.loads((GOLDEN / name).read_text())


def plainmp_numbering(dump: dict):
    """Restates KinematicModel's stack-DFS numbering (kinematics.cpp:192-206, 66-145) from a
    urdfdom dump: link order, parent ids, movable joint order."""
    links = dump["links"]
    order = []
    st = [dump["root"]]
    while st:
        l = st.pop()
        order.append(l)
        st.extend(links[l]["children"])
    lid = {n: i for i, n in enumerate(order)}
    parent = [lid[links[n]["parent"]] if links[n]["parent"] is not None else -1 for n in order]
    joints = dump["joints"]
    jorder = []
    js = list(links[dump["root"]]["child_joints"])
    while js:
        j = js.pop()
        if joints[j]["type"] in (1, 2, 3):
            jorder.append(j)
        js.extend(links[joints[j]["child"]]["child_joints"])
    return order, parent, jorder


def rotz(a):
    c, s = np.cos(a), np.sin(a)
    return np.array([[c, -s, 0], [s, c, 0], [0, 0, 1.0]])


def rpy_matrix(yaw, pitch, roll):
    """skrobot's rpy_matrix(az, ay, ax) = Rz(az) Ry(ay) Rx(ax)."""
    cy, sy = np.cos(yaw), np.sin(yaw)
    cp, sp = np.cos(pitch), np.sin(pitch)
    cr, sr = np.cos(roll), np.sin(roll)
    rz = np.array([[cy, -sy, 0], [sy, cy, 0], [0, 0, 1]])
    ry = np.array([[cp, 0, sp], [0, 1, 0], [-sp, 0, cp]])
    rx = np.array([[1, 0, 0], [0, cr, -sr], [0, sr, cr]])
    return rz @ ry @ rx
