"""Builds libtrayracer.so (CUDA kernels + C ABI) for sm_103a.

Every translation unit is compiled by nvcc in parallel into ``_build/`` and
linked into ``trayracer_gb300/libtrayracer.so`` next to this file. A stamp of
the source hashes and flags skips the rebuild when nothing changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
BUILD = PKG / "_build"
LIB = PKG / "libtrayracer.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC"]
HOST_FLAGS = ["-O2", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off,-pthread"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libtrayracer.so")
    return cand


def _sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))


def _stamp() -> str:
    h = hashlib.sha256()
    for p in _sources() + _headers():
        h.update(p.name.encode())
        h.update(p.read_bytes())
    h.update(" ".join(ARCH + CUDA_FLAGS + HOST_FLAGS).encode())
    h.update(os.uname().machine.encode())
    return h.hexdigest()


def build(verbose: bool = False, force: bool = False) -> Path:
    """Compiles and links the library; returns the path of the .so."""
    BUILD.mkdir(exist_ok=True)
    stamp_file = BUILD / "stamp.txt"
    stamp = _stamp()
    if not force and LIB.exists() and stamp_file.exists() and stamp_file.read_text() == stamp:
        return LIB
    nvcc = _nvcc()
    objs = []
    cmds = []
    for src in _sources():
        obj = BUILD / (src.name + ".o")
        flags = CUDA_FLAGS if src.suffix == ".cu" else HOST_FLAGS
        cmd = [nvcc, *ARCH, *flags, "-I", str(CSRC), "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)]
        if src.suffix == ".cu" and verbose:
            cmd.insert(1, "-Xptxas=-v")
        cmds.append(cmd)
        objs.append(obj)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    workers = max(1, min(len(cmds), os.cpu_count() or 4))
    with cf.ThreadPoolExecutor(workers) as ex:
        for cmd, r in ex.map(run, cmds):
            if verbose and (r.stdout or r.stderr):
                sys.stderr.write(r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{r.stdout}{r.stderr}")
    tmp = LIB.with_suffix(".so.tmp")
    link = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart", "-Xlinker", "-rpath,$ORIGIN"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{' '.join(link)}\n{r.stdout}{r.stderr}")
    os.replace(tmp, LIB)
    stamp_file.write_text(stamp)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
