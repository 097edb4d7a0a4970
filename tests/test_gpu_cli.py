"""The command-line driver (CManager / CController over the C ABI) with the
reference's output options: VTK snapshots after every step (-g) and the
benchmark .ini record (-b)."""
from __future__ import annotations

import configparser
import subprocess
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent


def parse_vtk(path):
    lines = path.read_text().splitlines()
    assert lines[:3] == ["# vtk DataFile Version 3.1", "Turbulent Fluid Simulation on MultiGPU.", "ASCII"]
    assert lines[4] == "DATASET STRUCTURED_GRID"
    dims = [int(v) for v in lines[5].split()[1:]]
    npts = int(lines[6].split()[1])
    assert npts == dims[0] * dims[1] * dims[2]
    at = 8 + npts + 1
    ncell = int(lines[at].split()[1])
    rho = np.array(lines[at + 3:at + 3 + ncell], dtype=np.float64)
    at += 3 + ncell + 1
    assert lines[at] == "SCALARS flag INT 1 "
    flags = np.array(lines[at + 2:at + 2 + ncell], dtype=np.int64)
    at += 2 + ncell + 1
    assert lines[at] == "VECTORS velocity float"
    vel = np.array([ln.split() for ln in lines[at + 1:at + 1 + ncell]], dtype=np.float64)
    return [d - 1 for d in dims], rho, flags, vel


def test_cli_writes_vtk_snapshots_and_benchmark_record(capi, tmp_path):
    exe = ROOT / "turbulent_lbm_multigpu_gb300" / "lbm_gb300"
    out = subprocess.run([str(exe), "-x", "16", "-y", "16", "-z", "16", "-X", "2", "-l", "3", "-g", "-b"],
                         cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "MLUPS:" in out.stdout
    for uid in (0, 1):
        for step in range(3):
            assert (tmp_path / "output" / "vtk" / f"OUTPUT.{uid}.{step}.vtk").exists()
    dims, rho, flags, vel = parse_vtk(tmp_path / "output" / "vtk" / "OUTPUT.0.2.vtk")
    assert dims == [8, 16, 16]
    f = flags.reshape(16, 16, 8)  # z, y, x
    # subdomain 0 of a 2x1x1 split: walls at x = 0 and on the y / z faces,
    # the ghost layer at x = 7, the lid plane y = 14 (x in [1, 6], z in [1, 14])
    assert (f[:, :, 0] == 1).all() and (f[1:-1, 1:-1, 7] == 8).all()
    assert (f[1:-1, 14, 1:7] == 4).all() and (f[1:-1, 1:14, 1:7] == 2).all()
    assert np.isfinite(rho).all() and np.isfinite(vel).all()
    assert np.abs(vel[f.reshape(-1) == 4, 0]).max() > 0  # the lid moves
    ini = configparser.ConfigParser()
    text = (tmp_path / "output" / "benchmark" / "benchmark_2.ini").read_text()
    ini.read_string("[EXP1]\n" + text)
    e = ini["EXP1"]
    assert (int(e["CUBE_X"]), int(e["CUBE_Y"]), int(e["CUBE_Z"])) == (16, 16, 16)
    assert float(e["MLUPS"]) > 0 and float(e["SECONDS"]) > 0 and float(e["FPS"]) > 0


def test_cli_domain_view_equals_controller_loop(capi, tmp_path):
    """The lock-step loop through the domain view (one step launch, one halo
    launch per axis) writes the same VTK snapshots, byte for byte, as the
    controllers' own simulationStep / syncAlpha / syncBeta loop."""
    import os

    exe = ROOT / "turbulent_lbm_multigpu_gb300" / "lbm_gb300"
    outs = []
    for loop in ("0", "1"):
        d = tmp_path / f"loop{loop}"
        d.mkdir()
        env = dict(os.environ, LBM_GB300_CONTROLLER_LOOP=loop)
        out = subprocess.run([str(exe), "-x", "24", "-y", "16", "-z", "16", "-X", "2", "-Y", "2", "-l", "5", "-g"],
                             cwd=d, capture_output=True, text=True, timeout=300, env=env)
        assert out.returncode == 0, out.stdout + out.stderr
        outs.append(d / "output" / "vtk")
    files = sorted(p.name for p in outs[0].iterdir())
    assert len(files) == 4 * 5 and files == sorted(p.name for p in outs[1].iterdir())
    for name in files:
        assert (outs[0] / name).read_bytes() == (outs[1] / name).read_bytes(), name


@pytest.mark.parametrize("loop", ["0", "1"])
def test_cli_validate_mode_passes(capi, tmp_path, loop):
    """The reference's validate mode (src/main.cpp:309-408) through conf.xml:
    the decomposed run's interior velocity equals the single domain's, cell
    for cell, through the domain view (graph replay) and the controller loop."""
    import os
    import re

    conf = (ROOT / "conf.xml").read_text()
    for tag, val in (("loops", "30"), ("validate", "1")):
        conf = re.sub(rf"<{tag}>[^<]*</{tag}>", f"<{tag}>{val}</{tag}>", conf, count=1)
    conf = re.sub(r"<domain-size>.*?</domain-size>",
                  "<domain-size><x>40</x><y>32</y><z>16</z></domain-size>", conf, flags=re.S)
    conf = re.sub(r"<perturbation>[^<]*</perturbation>", "<perturbation>0</perturbation>", conf)
    (tmp_path / "conf.xml").write_text(conf)
    exe = ROOT / "turbulent_lbm_multigpu_gb300" / "lbm_gb300"
    env = dict(os.environ, LBM_GB300_CONTROLLER_LOOP=loop)
    out = subprocess.run([str(exe), "-c", "conf.xml"], cwd=tmp_path, capture_output=True, text=True,
                         timeout=300, env=env)
    assert out.returncode == 0, out.stdout + out.stderr
    m = re.search(r"NUMBER OF FAILED CELLS/TOTAL NUMBER OF CELLS: (\d+)/(\d+)", out.stdout)
    assert m and int(m.group(1)) == 0 and int(m.group(2)) == 18 * 14 * 14, out.stdout
