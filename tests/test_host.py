"""Host-side checks that need no GPU: the C ABI library's exports, the C++
headers, the conf.xml reader, the CLbmSkeleton formulas, the decomposition
geometry and the multi-rank bench logic."""
from __future__ import annotations

import os
import re
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    text = (ROOT / "include" / "lbm_gb300.h").read_text()
    return sorted(set(re.findall(r"\b(lbm_cu_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol(capi):
    from turbulent_lbm_multigpu_gb300.build import LIB

    out = subprocess.run(["nm", "-D", "--defined-only", str(LIB)], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (lbm_cu_\w+)", out))
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, f"declared but not exported: {missing}"
    assert len(declared_symbols()) >= 20


def test_library_refuses_to_run_without_a_gpu(capi):
    """No CPU fallback: without a device every compute call reports an error."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(capi.LbmError):
        capi.Lattice(8, 8, 8)


@pytest.fixture(scope="module")
def probe(tmp_path_factory):
    exe = tmp_path_factory.mktemp("probe") / "host_probe"
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", f"-I{ROOT / 'include'}",
                    str(ROOT / "tests" / "cpp" / "host_probe.cpp"), "-o", str(exe)], check=True)
    return exe


def test_cpp_headers_instantiate_for_float_and_double(tmp_path):
    src = tmp_path / "inst.cpp"
    src.write_text('#include "lbm_gb300/CManager.hpp"\n'
                   "template class CLbmSolver<float>; template class CLbmSolver<double>;\n"
                   "template class CController<float>; template class CController<double>;\n"
                   "template class CManager<float>; template class CManager<double>;\nint main(){return 0;}\n")
    cuda_inc = Path(shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc").resolve().parent.parent / "include"
    subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-Werror", f"-I{ROOT / 'include'}",
                    f"-I{cuda_inc}", str(src)], check=True)


def parse_probe(text):
    return {line.split()[0]: line.split()[1:] for line in text.strip().splitlines()}


def test_conf_xml_reader(probe):
    out = subprocess.run([str(probe), "conf", str(ROOT / "conf.xml")], capture_output=True, text=True, check=True)
    d = parse_probe(out.stdout)
    assert d["domain"] == ["256", "256", "256"]
    assert d["subdomains"] == ["2", "2", "1"]
    assert d["loops"] == ["2000"] and d["kernels"] == ["128"] and d["validate"] == ["0"]
    assert float(d["viscosity"][0]) == pytest.approx(0.001308)
    lat = d["lattice"]
    assert lat[0] == "1" and float(lat[2]) == 10000 and float(lat[3]) == pytest.approx(0.1)
    assert float(lat[4]) == pytest.approx(0.17) and lat[5] == "f32" and lat[6] == "1234"


def test_conf_xml_reader_errors(probe, tmp_path):
    bad = tmp_path / "bad.xml"
    bad.write_text("<lbm-configuration><physics></physics></lbm-configuration>")
    r = subprocess.run([str(probe), "conf", str(bad)], capture_output=True, text=True)
    assert r.returncode == 3 and "missing element" in r.stdout
    r = subprocess.run([str(probe), "conf", str(tmp_path / "absent.xml")], capture_output=True, text=True)
    assert r.returncode == 3 and "Loading XML file failed" in r.stdout


def test_skeleton_formulas_match_reference_arithmetic(probe):
    """CLbmSkeleton::init / updateValues (src/CLbmSkeleton.hpp:81-190) in float,
    restated with numpy float32 in the reference's operand order."""
    out = subprocess.run([str(probe), "skeleton"], capture_output=True, text=True, check=True).stdout
    d = {k: [float.fromhex(x) for x in v if x.startswith(("0x", "-0x"))] for k, v in
         parse_probe("\n".join(l for l in out.splitlines() if not l.startswith(("limiting", "dim")))).items()}
    f = np.float32
    dx = f(0.1) / f(32)
    nu, tau = f(0.001308), f(0.953575)
    dt = (dx * dx) * (f(2.0) * tau - f(1.0)) / (f(6.0) * nu * np.sqrt(f(1.0)))
    g = np.array([0, -9.81, 0], f)
    grav = g * ((dt * dt) / dx)
    glen = np.sqrt(grav[0] * grav[0] + grav[1] * grav[1] + grav[2] * grav[2])
    if glen >= f(0.0001):
        dt = np.sqrt((f(0.0001) * dx) / np.sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]))
        grav = g * ((dt * dt) / dx)
        tau = f(0.5) * (dt * nu * np.sqrt(f(1.0)) * f(6.0)) / (dx * dx) + f(0.5)
    assert d["tau"][0] == tau
    assert d["inv_tau"][0] == f(1.0) / tau
    assert d["dt"][0] == dt
    assert d["gravity"][1] == grav[1]
    assert d["lid"][0] == f(100) * dt


def test_decomposition_geometry_matches_cmanager():
    """CComm geometry of CManager::initSimulation (src/CManager.hpp:122-199)."""
    from oracle import oracle as O

    sub, layout = O.manager_layout((64, 48, 32), (2, 3, 2))
    assert sub == (32, 16, 16)
    coords, bc, comms, lid = layout[3]  # (1, 1, 0)
    assert coords == (1, 1, 0)
    assert bc == [O.FLAG_GHOST, O.FLAG_OBSTACLE, O.FLAG_GHOST, O.FLAG_GHOST, O.FLAG_OBSTACLE, O.FLAG_GHOST]
    assert [(c.dst, c.axis, c.direction) for c in comms] == [(2, 0, (1, 0, 0)), (1, 1, (0, 1, 0)),
                                                             (5, 1, (0, -1, 0)), (9, 2, (0, 0, -1))]
    x_lower = comms[0]
    assert x_lower.send_origin == (1, 0, 0) and x_lower.recv_origin == (0, 0, 0)
    assert x_lower.send_size == (1, 16, 16)
    assert not lid and layout[5][3]
    with pytest.raises(ValueError, match="does not match"):
        O.manager_layout((30, 20, 10), (4, 1, 1))


def _rank_main(rank, world, port, q):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    ms = bench.max_over_ranks(10.0 + rank, dist)
    q.put((rank, ms, bench.whole_job_mlups(1000, 4, ms, world)))
    dist.destroy_process_group()


def test_bench_multirank_aggregation_gloo():
    """Weak scaling over replicas: max time over ranks, units of all ranks."""
    import multiprocessing as mp
    import socket

    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(60)
    assert [r[1] for r in res] == [11.0, 11.0]
    assert res[0][2] == pytest.approx(1000 * 4 * 2 / 11e-3 / 1e6)


def _vtk_expected(nx, ny, nz):
    """The reference's VTK text (src/libvis/CLbmVisualizationVTK.hpp:27-99 and
    VTK_Common.hpp:31-46) for the probe's synthetic subdomain, built in
    float32 like the C++ writer and printed with C's %f."""
    f = np.float32
    n = nx * ny * nz
    a = np.arange(n)
    rho = (f(1.0) + f(0.001) * a.astype(f) - f(0.0375) * (a % 7).astype(f)).astype(f)
    vx = (f(0.01) * ((a * 37) % 101 - 50).astype(f) / f(7.0)).astype(f)
    vy = (f(-0.02) * (a % 5).astype(f) / f(3.0)).astype(f)
    vz = (f(1e-7) * a.astype(f)).astype(f)
    fl = 1 << (a % 4)
    dx = f(0.1) / f(32.0)
    ox, oy, oz = f(2) * dx, f(0) * dx, f(6) * dx
    out = ["# vtk DataFile Version 3.1\n", "Turbulent Fluid Simulation on MultiGPU.\n", "ASCII\n", "\n",
           "DATASET STRUCTURED_GRID\n", f"DIMENSIONS  {nx + 1} {ny + 1} {nz + 1} \n",
           f"POINTS {(nx + 1) * (ny + 1) * (nz + 1)} float\n", "\n"]
    for k in range(nz + 1):
        for j in range(ny + 1):
            for i in range(nx + 1):
                out.append("%f %f %f\n" % (float(f(ox + f(i) * dx)), float(f(oy + f(j) * dx)), float(f(oz + f(k) * dx))))
    out += ["\n", f"CELL_DATA {n} \n", "SCALARS density float 1 \n", "LOOKUP_TABLE default \n"]
    out += ["%f\n" % float(v) for v in rho]
    out += ["\n", "SCALARS flag INT 1 \n", "LOOKUP_TABLE default \n"]
    out += ["%i\n" % int(v) for v in fl]
    out += ["\n", "VECTORS velocity float\n"]
    out += ["%f %f %f\n" % (float(x), float(y), float(z)) for x, y, z in zip(vx, vy, vz)]
    return "".join(out)


@pytest.mark.parametrize("threads,dims", [(1, (5, 4, 3)), (3, (40, 30, 20))])
def test_vtk_writer_matches_reference_layout(probe, tmp_path, threads, dims):
    """Byte-identical to the reference's serial fprintf output, also when the
    text is formatted by several threads (the 40x30x20 case splits every
    section)."""
    path = tmp_path / "OUTPUT.0.1.vtk"
    subprocess.run([str(probe), "vtk", str(path), str(threads), *map(str, dims)], check=True)
    assert path.read_text() == _vtk_expected(*dims)


def test_scaling_records_follow_the_reference_layout(tmp_path):
    """The sweep's .ini records and their analysis (benchmark.py analyse():
    averages per key over the [EXPn] sections, keyed by NP)."""
    from turbulent_lbm_multigpu_gb300 import scaling

    p = tmp_path / "benchmark_4.ini"
    scaling.append_record(p, 1, 4, (256, 256, 256), 2.0, 100, 4)
    scaling.append_record(p, 2, 4, (256, 256, 256), 4.0, 100, 4)
    text = p.read_text()
    assert text.startswith("[EXP1]\nNP : 4\nCUBE_X : 256\n")
    r = scaling.analyse([str(p)])[4]
    assert r["SECONDS"] == pytest.approx(3.0) and r["FPS"] == pytest.approx(37.5)
    assert r["MLUPS"] == pytest.approx(37.5 * 256 ** 3 * 1e-6)
    assert r["BANDWIDTH"] == pytest.approx(r["MLUPS"] * 39 * 4)
