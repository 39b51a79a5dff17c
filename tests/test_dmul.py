"""CPU: the integer-pipe FP64 multiplication (exploringsycl_gb300/csrc/tl_dmul.cuh)
against the host's IEEE multiplication, bit for bit, on random operands of
every class, on short significands whose products fall on rounding ties,
and at the edges of the normal range (the fast path and its fall-back)."""
from __future__ import annotations

import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_dmul_matches_ieee_multiplication(tmp_path):
    exe = tmp_path / "dmul_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off",
                    f"-I{ROOT / 'exploringsycl_gb300' / 'csrc'}",
                    str(ROOT / "tests" / "dmul_check.cpp"), "-o", str(exe)], check=True)
    for seed in (1, 2, 3):
        res = subprocess.run([str(exe), "400000", str(seed)], capture_output=True, text=True)
        assert res.returncode == 0, res.stdout + res.stderr
        cases, fast, bad = (int(v) for v in res.stdout.split()[1::2])
        assert bad == 0 and fast > cases // 2
