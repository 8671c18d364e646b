"""Build the in-tree CUDA solver library ``_lib/libobe_gb300.so`` for sm_103a.

Two translation units compiled in parallel: the host packer (g++) and the CUDA solver
(nvcc, ``-gencode arch=compute_103a,code=sm_103a``), linked with nvcc into one shared library
with the C ABI of include/obe_gb300.h.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
import tempfile
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = ROOT / "csrc"
INCLUDE = ROOT.parent / "include"
OUT = PKG / "_lib" / "libobe_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the GB300 solver needs the CUDA toolkit to build")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp")) + sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [INCLUDE / "obe_gb300.h"]


def up_to_date() -> bool:
    if not OUT.exists():
        return False
    mtime = OUT.stat().st_mtime
    return all(src.stat().st_mtime <= mtime for src in sources())


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and up_to_date():
        return OUT
    nvcc = _nvcc()
    OUT.parent.mkdir(parents=True, exist_ok=True)
    with tempfile.TemporaryDirectory(prefix="obe_build_") as tmp:
        tmp = Path(tmp)
        cmds = [
            [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", f"-I{INCLUDE}",
             "-c", str(CSRC / "obe_solver.cu"), "-o", str(tmp / "obe_solver.o")],
            ["g++", "-O2", "-std=c++17", "-fPIC", f"-I{INCLUDE}", "-c", str(CSRC / "obe_plan.cpp"),
             "-o", str(tmp / "obe_plan.o")],
        ]

        def run(cmd):
            res = subprocess.run(cmd, capture_output=True, text=True)
            if res.returncode != 0:
                raise RuntimeError(f"build failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
            if verbose:
                sys.stdout.write(res.stdout + res.stderr)

        with ThreadPoolExecutor(max_workers=2) as pool:
            list(pool.map(run, cmds))
        tmp_out = tmp / "libobe_gb300.so"
        run([nvcc, *ARCH, "-shared", "-o", str(tmp_out), str(tmp / "obe_solver.o"), str(tmp / "obe_plan.o")])
        shutil.copy2(tmp_out, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
