"""The GB300 run_* backend compiles unchanged against the reference's own
driver headers and links with the reference's own driver objects (no GPU is
needed to link). Skipped where the reference sources are absent."""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
REF = Path(os.environ.get("TEALEAF_REF",
                         Path(__file__).resolve().parents[2] / "reference" / "TeaLeaf"))


@pytest.mark.skipif(not REF.is_dir(), reason="reference sources not present")
def test_reference_driver_links_with_gb300_backend(tmp_path, backend_built):
    gb = ROOT / "exploringsycl_gb300"
    inc = [f"-I{REF}", f"-I{gb / 'backend'}", f"-I{ROOT / 'include'}"]
    srcs = sorted(str(p) for p in list(REF.glob("*.c")) + list((REF / "drivers").glob("*.c")))
    subprocess.run(["g++", "-x", "c++", "-O1", "-DNO_MPI", "-w", *inc, "-c", *srcs],
                   cwd=tmp_path, check=True, capture_output=True)
    subprocess.run(["g++", "-std=c++17", "-O1", *inc, "-c",
                    str(gb / "backend" / "kernel_interface.cpp"), "-o", "gb300_backend.o"],
                   cwd=tmp_path, check=True, capture_output=True)
    objs = sorted(str(p) for p in tmp_path.glob("*.o"))
    res = subprocess.run(["g++", *objs, f"-L{gb / '_build'}", "-ltealeaf_gb300",
                          f"-Wl,-rpath,{gb / '_build'}", "-o", "tealeaf"],
                         cwd=tmp_path, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    assert (tmp_path / "tealeaf").exists()
