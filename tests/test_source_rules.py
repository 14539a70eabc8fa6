"""Source rules, checked on the text (no GPU, no compiler): warp intrinsics in the CUDA kernels, and
the commands the profile summaries give.

A warp intrinsic with a full member mask (`__shfl_sync(0xffffffff, ...)`, `__any_sync`,
`__ballot_sync`, ...) must be executed by every non-exited lane the mask names, at the same call.
If some lanes skip it, the behaviour is undefined. The warp's lanes can then pair up at different
sync points, and later shuffles return values from lanes that run other code.

The usual way to break this is a conditionally evaluated call: `have && __shfl_sync(...)` or
`c ? __shfl_sync(...) : x`, or an unbraced `if (c) v = __shfl_sync(...)`. A lane whose condition is
false skips the call. The rule below rejects a warp intrinsic that is preceded in its own
statement by `&&`, `||`, `?` or an `if (...)` header. A second rule rejects a warp intrinsic
anywhere inside a braced branch taken by one lane (`if (lane == 0) { ... }`, also `hl`, `sub`,
`tid`, `threadIdx.x`, `(threadIdx.x & 31)`): the other lanes the mask names never reach it. Loops
and braced branches whose condition is warp-uniform are left to review.
"""
import re
from pathlib import Path

import pytest

CSRC = Path(__file__).resolve().parent.parent / "plainmp_gb300" / "csrc"

_INTRINSIC = re.compile(
    r"__(?:shfl|shfl_up|shfl_down|shfl_xor|any|all|ballot|match_any|match_all|reduce_[a-z]+|syncwarp)(?:_sync)?\s*\("
)


def _strip_comments(src: str) -> str:
    src = re.sub(r"/\*.*?\*/", lambda m: "\n" * m.group(0).count("\n"), src, flags=re.S)
    return re.sub(r"//[^\n]*", "", src)


def conditional_warp_calls(src: str):
    """(line, statement prefix) of every warp intrinsic that its own statement evaluates conditionally."""
    s = _strip_comments(src)
    found = []
    for m in _INTRINSIC.finditer(s):
        i = m.start()
        start = max(s.rfind(";", 0, i), s.rfind("{", 0, i), s.rfind("}", 0, i))
        prefix = s[start + 1 : i]
        # a `for (init; cond; step)` header splits at its semicolons; the prefix is then the rest
        # of the header, which is unconditional when the intrinsic sits in the loop condition
        cond = re.search(r"&&|\|\||\?", prefix) or re.match(r"\s*(?:else\s+)?if\s*\(.*\)\s*\S", prefix, flags=re.S)
        if cond:
            found.append((s.count("\n", 0, i) + 1, " ".join(prefix.split())[-80:]))
    return found


_ONE_LANE = re.compile(r"\bif\s*\(\s*(?:lane|hl|sub|tid|threadIdx\.x|\(threadIdx\.x\s*&\s*31\))\s*==\s*0\s*\)\s*\{")


def one_lane_warp_calls(src: str):
    """Line of every warp intrinsic inside a braced `if (<lane> == 0) { ... }` branch."""
    s = _strip_comments(src)
    found = []
    for m in _ONE_LANE.finditer(s):
        depth, j = 1, m.end()
        while j < len(s) and depth:
            depth += {"{": 1, "}": -1}.get(s[j], 0)
            j += 1
        for c in _INTRINSIC.finditer(s, m.end(), j):
            found.append(s.count("\n", 0, c.start()) + 1)
    return found


def test_rule_catches_one_lane_branches():
    planted = """
    __device__ void f(int lane, int v, bool need) {
      if (lane == 0) {
        atomicAdd(&g, __popc(__ballot_sync(0xffffffffu, need)));   // only lane 0 arrives
      }
      const unsigned b = __ballot_sync(0xffffffffu, need);           // fine
      if ((threadIdx.x & 31) == 0) { if (v) { v = __shfl_sync(0xffffffffu, v, 0); } }
    }
    """
    assert one_lane_warp_calls(planted) == [4, 7]


def test_rule_catches_conditional_calls():
    planted = """
    __device__ void f(bool have, int v) {
      const bool want = have && __shfl_sync(0xffffffffu, v, 0, 16) != 0;   // skipped where !have
      int w = have ? __shfl_sync(0xffffffffu, v, 0) : 0;
      if (have) v = __shfl_xor_sync(0xffffffffu, v, 1);
      const int ok = __shfl_sync(0xffffffffu, have ? 1 : 0, 0);             // fine: the argument only
      while (__any_sync(0xffffffffu, v > 0)) { v--; }                      // fine
    }
    """
    lines = [ln for ln, _ in conditional_warp_calls(planted)]
    assert lines == [3, 4, 5], lines


@pytest.mark.parametrize("path", sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cuh")), ids=lambda p: p.name)
def test_warp_intrinsics_are_unconditional(path):
    bad = conditional_warp_calls(path.read_text())
    assert not bad, f"{path.name}: warp intrinsic evaluated conditionally at " + "; ".join(
        f"line {ln}: ...{ctx}" for ln, ctx in bad
    )


@pytest.mark.parametrize("path", sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cuh")), ids=lambda p: p.name)
def test_no_warp_intrinsics_in_one_lane_branches(path):
    bad = one_lane_warp_calls(path.read_text())
    assert not bad, f"{path.name}: warp intrinsic inside a one-lane branch at lines {bad}"


def test_profile_commands_run_committed_files():
    """Every profiles/ summary gives the command that made it, and that command runs committed
    files: the scripts and modules it names exist here, and profile_cases knows the case it asks for."""
    import re
    import subprocess

    repo = CSRC.parent.parent
    tracked = set(subprocess.run(["git", "ls-files"], cwd=repo, capture_output=True, text=True).stdout.split())
    if not tracked:
        pytest.skip("not a git checkout")
    cases = set(re.findall(r'which in \(([^)]*)\)', (repo / "profile_cases.py").read_text()))
    known = {c.strip().strip('"') for group in cases for c in group.split(",") if c.strip()}
    summaries = sorted((repo / "profiles").glob("*.md"))
    assert summaries
    for md in summaries:
        text = md.read_text()
        cmds = re.findall(r"python3? (-m [\w.]+(?: \w+)?|[\w./]+\.py(?: \w+)?)", text)
        assert cmds, f"{md.name} gives no command"
        for c in cmds:
            if c.startswith("-m "):
                parts = c[3:].split()
                path = parts[0].replace(".", "/") + ".py"
                assert path in tracked, (md.name, c)
            else:
                parts = c.split()
                assert parts[0] in tracked, (md.name, c)
                if parts[0] == "profile_cases.py" and len(parts) > 1:
                    assert parts[1] in known, (md.name, c)
