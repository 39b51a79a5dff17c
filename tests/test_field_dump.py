"""Field dumps (TL_DUMP_DIR): VisIt brick-of-values pairs written at every
field summary, as the reference's write_to_visit (TeaLeaf/shared.c:114-150)
lays them out. The oracle backend's dumps are checked against its own
field-summary sums on the CPU; the GB300 backend's must equal the oracle's
byte for byte."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

from exploringsycl_gb300 import deck as dk

from .drivers import run_driver


def read_bov(path: Path) -> tuple[dict, np.ndarray]:
    header = {}
    for line in path.read_text().splitlines():
        key, _, value = line.partition(":")
        header[key.strip()] = value.strip()
    nx, ny, nz = (int(v) for v in header["DATA_SIZE"].split())
    data = np.fromfile(path.parent / header["DATA_FILE"], dtype="<f8")
    assert data.size == nx * ny * nz
    return header, data.reshape(ny, nx)


def test_oracle_dump_reproduces_field_summary(tmp_path, oracle_built):
    n = 24
    d = dk.five_state(n, end_step=2)
    out = tmp_path / "dumps"
    out.mkdir()
    run = run_driver(oracle_built.DRIVER, d, tmp_path / "run", env={"TL_DUMP_DIR": str(out)})
    assert run.returncode == 0, run.stdout[-2000:]
    # one summary at start-up and one after the last step (summary_frequency 10)
    assert len(run.summaries) >= 2
    cell_volume = (10.0 / n) ** 2
    for i, (vol, mass, ie, temp) in enumerate(run.summaries):
        hdr, rho = read_bov(out / f"density{i}.bov")
        _, e = read_bov(out / f"energy{i}.bov")
        _, u = read_bov(out / f"u{i}.bov")
        assert hdr["DATA_FORMAT"] == "DOUBLE" and hdr["DATA_ENDIAN"] == "LITTLE"
        assert hdr["VARIABLE"] == "density" and hdr["CENTERING"] == "zone"
        assert rho.shape == (n, n)
        assert np.isclose(rho.size * cell_volume, vol, rtol=1e-12)
        assert np.isclose(np.sum(rho) * cell_volume, mass, rtol=1e-12)
        assert np.isclose(np.sum(rho * e) * cell_volume, ie, rtol=1e-12)
        assert np.isclose(np.sum(rho * u) * cell_volume, temp, rtol=1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("make", [lambda: dk.five_state(40, end_step=3),
                                  lambda: dk.random_deck(48, seed=5, end_step=2)])
def test_gpu_dump_equals_oracle_dump(make, tmp_path, backend_built, oracle_built):
    from exploringsycl_gb300 import DRIVER_EXE

    d = make()
    dumps = {}
    for name, exe in (("gpu", DRIVER_EXE), ("cpu", oracle_built.DRIVER)):
        out = tmp_path / f"{name}_dumps"
        out.mkdir()
        run = run_driver(exe, d, tmp_path / name, env={"TL_DUMP_DIR": str(out)})
        assert run.returncode == 0, run.stdout[-2000:]
        dumps[name] = {p.name: p.read_bytes() for p in sorted(out.iterdir())}
    assert dumps["gpu"].keys() == dumps["cpu"].keys() and dumps["gpu"]
    for fname, blob in dumps["gpu"].items():
        assert blob == dumps["cpu"][fname], fname
