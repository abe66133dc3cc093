"""Build the in-tree native libraries of qmprs_gb300.

* ``_lib/libqmprs_gb300.so``   the CUDA library (sm_103a), C ABI declared in
  ``include/qmprs_gb300.h``; every ``.cu`` in ``csrc/`` is compiled in
  parallel with ``nvcc -gencode arch=compute_103a,code=sm_103a`` and linked
  with ``-shared``.
* ``_lib/libqmprs_hostcheck.so``  host-only build (g++) of the FP64 small
  linear algebra the kernels use, for CPU tests.

Usage: ``python -m qmprs_gb300.build`` (or ``build()`` from Python).  Only
sources newer than their objects are recompiled.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_lib"
OBJ = PKG / "_build"
INCLUDE = ROOT / "include"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              f"-I{CSRC}", f"-I{INCLUDE}"]

CUDA_LIB = "libqmprs_gb300.so"
HOST_LIB = "libqmprs_hostcheck.so"


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _headers_mtime() -> float:
    hs = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    return max(h.stat().st_mtime for h in hs)


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")


def build_cuda(verbose: bool = False, extra: list[str] | None = None) -> Path:
    OUT.mkdir(exist_ok=True)
    OBJ.mkdir(exist_ok=True)
    nvcc = _nvcc()
    hdr = _headers_mtime()
    srcs = sorted(CSRC.glob("*.cu"))
    jobs = []
    for src in srcs:
        obj = OBJ / (src.stem + ".o")
        if obj.exists() and obj.stat().st_mtime >= max(src.stat().st_mtime, hdr):
            continue
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, *(extra or []), "-c", str(src), "-o", str(obj)]
        jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        for fut in [ex.submit(_run, j) for j in jobs]:
            fut.result()
    lib = OUT / CUDA_LIB
    objs = [str(OBJ / (s.stem + ".o")) for s in srcs]
    if (not lib.exists()) or jobs or lib.stat().st_mtime < max(Path(o).stat().st_mtime for o in objs):
        _run([nvcc, *ARCH, "-shared", "-o", str(lib), *objs, "-lcudart"])
    if verbose:
        print(f"built {lib}")
    return lib


def build_hostcheck() -> Path:
    OUT.mkdir(exist_ok=True)
    lib = OUT / HOST_LIB
    src = CSRC / "host_check.cpp"
    if lib.exists() and lib.stat().st_mtime >= max(src.stat().st_mtime, _headers_mtime()):
        return lib
    cxx = shutil.which("g++") or "g++"
    _run([cxx, "-O2", "-std=c++17", "-fPIC", "-shared", f"-I{CSRC}", str(src), "-o", str(lib)])
    return lib


def build(verbose: bool = False) -> None:
    build_hostcheck()
    build_cuda(verbose=verbose)


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
