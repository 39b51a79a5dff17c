"""In-tree build of the GB300 TeaLeaf backend.

Produces, under exploringsycl_gb300/_build/:
  libtealeaf_gb300.so         CUDA kernels + C ABI (include/tealeaf_gb300.h), sm_103a
  tealeaf_gb300               TeaLeaf host driver + GB300 run_* backend (executable)
  libtealeaf_gb300_driver.so  the same driver as a library exporting tl_main()

Every .cu file is compiled separately (in parallel) with
``-gencode arch=compute_103a,code=sm_103a -lineinfo``; the double-precision
kernels additionally with ``--fmad=false`` so that no multiply-add is fused
(their results are compared bit for bit with the CPU oracle).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
BUILD = PKG / "_build"
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
HOST = PKG / "host"
BACKEND = PKG / "backend"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
              f"-I{INCLUDE}", f"-I{CSRC}"]
# Per-file extra flags: exact double precision for the drop-in kernels.
EXTRA = {
    "tl_fp64.cu": ["--fmad=false"],
}
HOST_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall",
              "-Wno-unused-result"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the GB300 backend cannot be built")


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_library(verbose: bool = False) -> Path:
    """Compile every csrc/*.cu and link libtealeaf_gb300.so."""
    BUILD.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    sources = sorted(CSRC.glob("*.cu"))
    headers = sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))
    objs = []
    jobs = []
    for src in sources:
        obj = BUILD / (src.stem + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            cmd = [nvcc, *ARCH, *NVCC_FLAGS, *EXTRA.get(src.name, []), "-c", str(src),
                   "-o", str(obj)]
            jobs.append(cmd)
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for fut in [ex.submit(_run, c) for c in jobs]:
                fut.result()
    lib = BUILD / "libtealeaf_gb300.so"
    if _stale(lib, objs):
        _run([nvcc, *ARCH, "-shared", "-o", str(lib), *map(str, objs)])
    if verbose:
        print(f"built {lib}")
    return lib


def build_driver(verbose: bool = False) -> tuple[Path, Path]:
    """Link the TeaLeaf host driver with the GB300 backend (exe and .so)."""
    lib = build_library(verbose)
    cxx = os.environ.get("CXX", "g++")
    deps = [HOST / "tl_driver.cpp", HOST / "tl_main.cpp", BACKEND / "kernel_interface.cpp",
            *HOST.glob("*.h"), BACKEND / "chunk_extension.h", lib]
    inc = [f"-I{HOST}", f"-I{BACKEND}", f"-I{INCLUDE}"]
    link = [f"-L{BUILD}", "-ltealeaf_gb300", "-Wl,-rpath,$ORIGIN"]
    exe = BUILD / "tealeaf_gb300"
    if _stale(exe, deps):
        _run([cxx, *HOST_FLAGS, *inc, str(HOST / "tl_driver.cpp"), str(HOST / "tl_main.cpp"),
              str(BACKEND / "kernel_interface.cpp"), *link, "-o", str(exe)])
    dso = BUILD / "libtealeaf_gb300_driver.so"
    if _stale(dso, deps):
        _run([cxx, *HOST_FLAGS, "-shared", *inc, str(HOST / "tl_driver.cpp"),
              str(BACKEND / "kernel_interface.cpp"), *link, "-o", str(dso)])
    if verbose:
        print(f"built {exe} and {dso}")
    return exe, dso


def build_all(verbose: bool = False) -> None:
    build_driver(verbose)


if __name__ == "__main__":
    build_all(verbose=True)
    sys.exit(0)
