"""Build the in-tree CUDA solver library ``_lib/libobe_gb300.so`` for sm_103a.

Translation units compiled in parallel: the host packer (g++), the host side of the CUDA solver
and one object per integrator kernel shape (nvcc, ``-gencode arch=compute_103a,code=sm_103a``),
linked with nvcc into one shared library with the C ABI of include/obe_gb300.h.
"""

from __future__ import annotations

import os
import platform
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
# integrator shapes (threads per trajectory, elements per thread); the RHS kernel is built with
# the first shape of each width.  Must match OBE_FOR_EACH_SHAPE / OBE_FOR_EACH_RHS in obe_kernels.cuh.
SHAPES = [(32, 8), (32, 16), (64, 4), (64, 16), (128, 2), (128, 12), (128, 16), (256, 24), (256, 32), (512, 12), (512, 16)]
RHS_SHAPES = [(32, 8), (64, 16), (128, 16), (256, 32), (512, 16)]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the GB300 solver needs the CUDA toolkit to build")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp")) + sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [INCLUDE / "obe_gb300.h"]


HASH = OUT.with_name("libobe_gb300.sources.sha256")


def sources_hash() -> str:
    import hashlib

    h = hashlib.sha256()
    for src in sources():
        h.update(src.name.encode())
        h.update(src.read_bytes())
    h.update(" ".join(ARCH).encode())
    h.update(platform.machine().encode())  # a hash written on another architecture never matches
    return h.hexdigest()


def up_to_date() -> bool:
    # by content, not by time stamps: a library built from other sources (or on a machine whose
    # clock disagrees with the sources' time stamps) is rebuilt
    return OUT.exists() and HASH.exists() and HASH.read_text().strip() == sources_hash()


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and up_to_date():
        return OUT
    nvcc = _nvcc()
    OUT.parent.mkdir(parents=True, exist_ok=True)
    with tempfile.TemporaryDirectory(prefix="obe_build_") as tmp:
        tmp = Path(tmp)
        common = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", f"-I{INCLUDE}"]
        objs = [tmp / "obe_solver.o", tmp / "obe_plan.o", tmp / "obe_dense.o"]
        cmds = [
            common + ["-c", str(CSRC / "obe_solver.cu"), "-o", str(objs[0])],
            common + ["-c", str(CSRC / "obe_dense.cu"), "-o", str(objs[2])],
            ["g++", "-O2", "-std=c++17", "-fPIC", f"-I{INCLUDE}", "-c", str(CSRC / "obe_plan.cpp"), "-o", str(objs[1])],
        ]
        # one object per kernel shape (threads per trajectory, elements per thread), compiled in parallel
        for tpt, ept in SHAPES:
            obj = tmp / f"obe_instance_{tpt}_{ept}.o"
            defs = [f"-DOBE_TPT={tpt}", f"-DOBE_EPT={ept}"] + (["-DOBE_RHS"] if (tpt, ept) in RHS_SHAPES else [])
            cmds.append(common + defs + ["-c", str(CSRC / "obe_instance.cu"), "-o", str(obj)])
            objs.append(obj)

        def run(cmd):
            res = subprocess.run(cmd, capture_output=True, text=True)
            if res.returncode != 0:
                raise RuntimeError(f"build failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
            if verbose:
                sys.stdout.write(res.stdout + res.stderr)

        with ThreadPoolExecutor(max_workers=min(len(cmds), os.cpu_count() or 4)) as pool:
            list(pool.map(run, cmds))
        tmp_out = tmp / "libobe_gb300.so"
        run([nvcc, *ARCH, "-shared", "-o", str(tmp_out), *map(str, objs)])
        shutil.copy2(tmp_out, OUT)
    HASH.write_text(sources_hash() + "\n")
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
