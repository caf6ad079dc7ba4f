"""Builds the CPU oracle (test infrastructure).

* ``oracle/liboracle.so`` - the restated oracle (oracle.cpp), g++ with
  -ffp-contract=off so host float arithmetic rounds where the source says.
* ``oracle/_ref/libtrref.so`` - only where the reference sources are present
  (``TRAYRACER_REFERENCE`` or /root/reference): the reference's own raygen
  programs (Tracer/Optix/GPU/optix.cu) and path-tracing shade kernel
  (Tracer/CUDA/GPU/Shade/PathTracing.h) compiled as host C++ from where they
  lie, with the host shims in ref_shim/. Nothing from the reference is copied.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
CUDA_INC = os.environ.get("CUDA_HOME", "/usr/local/cuda") + "/include"
COMMON = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-pthread", "-I", CUDA_INC]


def _stale(out: Path, srcs: list[Path]) -> bool:
    if not out.exists():
        return True
    m = out.stat().st_mtime
    return any(s.stat().st_mtime > m for s in srcs)


def build_oracle() -> Path:
    out = HERE / "liboracle.so"
    srcs = [HERE / "oracle.cpp", HERE / "oracle.h", HERE.parent / "include" / "trayracer.h"]
    if _stale(out, srcs):
        tmp = out.with_suffix(".tmp.so")
        cmd = COMMON + [str(HERE / "oracle.cpp"), "-o", str(tmp)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{' '.join(cmd)}\n{r.stderr}")
        os.replace(tmp, out)
    return out


def reference_root() -> Path | None:
    root = Path(os.environ.get("TRAYRACER_REFERENCE", "/root/reference"))
    return root if (root / "Tracer" / "CUDA" / "GPU" / "Shade" / "PathTracing.h").exists() else None


def build_reference() -> Path | None:
    """Compiles the reference's kernels as host C++ into oracle/_ref; None when absent."""
    root = reference_root()
    if root is None:
        return None
    outdir = HERE / "_ref"
    outdir.mkdir(exist_ok=True)
    out = outdir / "libtrref.so"
    shim = HERE / "ref_shim"
    srcs = sorted(shim.glob("*.cpp")) + sorted(shim.glob("*.h")) + [HERE / "oracle.cpp", HERE / "oracle.h"]
    if not _stale(out, srcs):
        return out
    inc = [
        "-I", str(shim),
        "-I", str(root / "Tracer"),
        "-I", str(root / "Tracer" / "CUDA" / "GPU"),
        "-I", str(root / "Tracer" / "CUDA" / "GPU" / "Shade"),
        "-I", str(root / "thirdparty"),
    ]
    tmp = out.with_suffix(".tmp.so")
    units = [str(p) for p in sorted(shim.glob("*.cpp"))] + [str(HERE / "oracle.cpp")]
    cmd = COMMON + ["-w"] + inc + units + ["-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference build failed:\n{' '.join(cmd)}\n{r.stderr}")
    os.replace(tmp, out)
    return out


if __name__ == "__main__":
    print(build_oracle())
    print(build_reference())
    sys.exit(0)
