"""Generate the golden fixtures in tests/golden/ from the reference itself.

Run where the reference checkout is available, its root given as the argument or in PLAINMP_REF:

    python tests/golden/make_golden.py [reference_root]

* sequence_table.json -- SEQUENCE_TABLE rows for n = 1..128 computed by the reference's own
  generator function (cpp/plainmp/ompl/generate_sequence.py: find_farthest_sequence_fast),
  imported from the reference checkout.
* urdf_*.json -- what the reference's vendored urdfdom parser reads from a URDF (root, child
  order, origin quaternions, axes, limits), dumped by oracle/_ref/urdf_dump (built by
  oracle/ref/build_ref.sh from the reference sources); each fixture embeds its URDF text.
"""
from __future__ import annotations

import importlib.util
import json
import os
import subprocess
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO))

EDGE_URDF = """<?xml version="1.0"?>
<!-- branching tree; joint names out of link order; mixed joint types -->
<robot name="edge">
  <link name="root"/>
  <link name="b_link"/>
  <link name="a_link"/>
  <link name="c_link"/>
  <link name="tip"/>
  <link name="slider"/>
  <link name="wheel"/>
  <link name="tool"/>
  <joint name="zz_first" type="revolute">
    <parent link="root"/><child link="b_link"/>
    <origin xyz="0.1 -0.2 0.3" rpy="0.3 -0.2 1.1"/>
    <axis xyz="0 0 2"/>
    <limit lower="-1.5" upper="1.5" effort="1" velocity="1"/>
  </joint>
  <joint name="aa_second" type="revolute">
    <parent link="root"/><child link="a_link"/>
    <origin xyz="-0.25 0.05 0.125"/>
    <axis xyz="0.6 0.8 0"/>
    <limit upper="2.0" effort="1" velocity="1"/>
  </joint>
  <joint name="mm_cont" type="continuous">
    <parent link="a_link"/><child link="c_link"/>
    <origin xyz="0 0 0.2" rpy="1.5707963267948966 0 0"/>
  </joint>
  <joint name="bb_fixed" type="fixed">
    <parent link="c_link"/><child link="tip"/>
    <origin xyz="0.05 0 0" rpy="0 0.7 0"/>
  </joint>
  <joint name="cc_pris" type="prismatic">
    <parent link="b_link"/><child link="slider"/>
    <origin xyz="0.0 0.1 0.0" rpy="0 0 -0.4"/>
    <axis xyz="1 0 0"/>
    <limit lower="-0.1" upper="0.4" effort="1" velocity="1"/>
  </joint>
  <joint name="ab_wheel" type="continuous">
    <parent link="b_link"/><child link="wheel"/>
  </joint>
  <joint name="ba_tool" type="revolute">
    <parent link="slider"/><child link="tool"/>
    <origin xyz="1e-3 2.5e-1 -3.75E-2" rpy="-2.5 0.1 3.0"/>
    <axis xyz="0.0 -1.0 0.0"/>
    <limit lower="-3.14159" upper="3.14159" effort="1" velocity="1"/>
  </joint>
</robot>
"""


def sequence_table(ref: Path) -> None:
    spec = importlib.util.spec_from_file_location("generate_sequence", ref / "cpp/plainmp/ompl/generate_sequence.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    rows = [mod.find_farthest_sequence_fast(n) for n in range(1, 129)]
    (HERE / "sequence_table.json").write_text(json.dumps({"source": "cpp/plainmp/ompl/generate_sequence.py:11-63", "rows": rows},
                                                         separators=(",", ":")) + "\n")


def urdf_fixture(name: str, urdf: str, dump: Path) -> None:
    with tempfile.NamedTemporaryFile("w", suffix=".urdf", delete=False) as f:
        f.write(urdf)
        path = f.name
    out = subprocess.run([str(dump), path], capture_output=True, text=True, check=True).stdout
    data = json.loads(out)
    data["urdf"] = urdf
    (HERE / f"urdf_{name}.json").write_text(json.dumps(data, indent=1) + "\n")


def main() -> None:
    arg = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PLAINMP_REF")
    if not arg:
        sys.exit("usage: make_golden.py REFERENCE_ROOT (or set PLAINMP_REF to the plainmp checkout)")
    ref = Path(arg)
    sequence_table(ref)
    subprocess.run([str(REPO / "oracle/ref/build_ref.sh"), str(ref)], check=True)
    dump = REPO / "oracle/_ref/urdf_dump"
    from plainmp_gb300 import workloads as W

    urdf_fixture("chain7", W.chain7_robot().urdf, dump)
    urdf_fixture("dualarm", W.dualarm_robot().urdf, dump)
    urdf_fixture("edge", EDGE_URDF, dump)


if __name__ == "__main__":
    main()
