"""Build the in-tree native library ``plainmp_gb300/libpmgpu.so``.

CUDA sources are compiled for sm_103a only (``-gencode arch=compute_103a,code=sm_103a``) with
``--fmad=false`` so FP64 results are bit-identical to the CPU restatement; C++ host sources are
compiled with ``-ffp-contract=off`` for the same reason (the Arm host contracts by default).
Translation units compile in parallel; objects are rebuilt when a source or header changes.
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
BUILD = PKG / "_build"
LIB = PKG / "libpmgpu.so"

CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "--fmad=false", "-std=c++17", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
    f"-I{CSRC}", f"-I{INCLUDE}",
]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall",
             f"-I{CSRC}", f"-I{INCLUDE}", f"-I{CUDA_HOME / 'include'}"]


def _headers_digest() -> str:
    h = hashlib.sha1()
    for p in sorted(list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))):
        h.update(p.read_bytes())
    return h.hexdigest()


def _compile(src: Path, digest: str, extra: list[str]) -> Path:
    tag = hashlib.sha1((digest + src.read_text() + " ".join(extra)).encode()).hexdigest()[:16]
    obj = BUILD / f"{src.stem}.{tag}.o"
    if obj.exists():
        return obj
    if src.suffix == ".cu":
        cmd = [NVCC, *NVCC_FLAGS, *extra, "-c", str(src), "-o", str(obj)]
    else:
        cmd = [os.environ.get("CXX", "g++"), *CXX_FLAGS, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False, ptxas_info: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    digest = _headers_digest()
    srcs = sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    with ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, digest, extra if s.suffix == ".cu" else []), srcs))
    for stale in set(BUILD.glob("*.o")) - set(objs):  # objects of earlier source versions
        stale.unlink()
    link_tag = hashlib.sha1("".join(o.name for o in objs).encode()).hexdigest()[:16]
    stamp = BUILD / f"link.{link_tag}"
    if LIB.exists() and stamp.exists():
        return LIB
    tmp = BUILD / "libpmgpu.so.tmp"
    cmd = [NVCC, *ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *map(str, objs), "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    shutil.move(str(tmp), str(LIB))
    for old in BUILD.glob("link.*"):
        old.unlink()
    stamp.write_text("ok")
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_info="--ptxas" in sys.argv)
