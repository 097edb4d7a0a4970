"""Benchmark of the D3Q19 hot path on GB300 (one JSON line on stdout).

Workload (the reference-derived plain configuration at scale): lid-driven
cavity, 256^3 cells decomposed into 2x2x1 subdomains of 128x128x256 held on
one GPU, D3Q19 BGK + Smagorinsky (Cs 0.17), Re 10000 on lid length 256, lid
speed 0.1, FP32 populations, seeded start-up velocity uniform on +-1e-3
(Philox, seed 1234).  A "step" is one time step of the whole domain: the
alternating beta/alpha step kernel over all four subdomains plus the CComm
halo exchange in x, y, z order (CController::computeNextStep).

Reported:
  value      MLUPS over all cells (walls and ghost layers included, the
             reference's count), device-resident fields, timed with CUDA
             events on the launching stream around K steps replayed as one
             captured graph (CUDA-event pairs around the step kernels of a
             beta/alpha pair in every 10 steps are part of that graph and
             give the roofline's kernel time);
  roofline   the step kernel against the measured HBM copy bandwidth;
             algorithmic bytes = 2*19*4 = 152 per cell update;
  e2e        the same metric through the C ABI with host buffers: upload of
             the initial populations from pinned host memory, K steps, and
             the final velocity field read back to the host, all timed;
  cpu_baseline  the oracle port of the reference kernels on the host cores.

--impl reference times the CPU implementation (the oracle port of the
reference's kernels, all host threads) on the same configuration.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "D3Q19 MLUPS & % HBM roofline; served solves/s, p50/p99 latency vs plain"
SIZE = (256, 256, 256)
NUMS = (2, 2, 1)
U_LID, RE, CS, SEED, AMP = 0.1, 10000.0, 0.17, 1234, 1e-3
BYTES_PER_CELL = {"f32": 152, "f64": 304, "f16": 76, "bf16": 76, "c16": 76}
HALO_MODE = 1  # after alpha, exchange the 5 populations the ghost layer's inner neighbours read
TIMED_EVERY = 10  # step kernels timed by CUDA events: a beta/alpha pair in every 10 steps


def lattice_params(dtype):
    import numpy as np

    tau = 3.0 * U_LID * SIZE[0] / RE + 0.5
    t = dtype(tau)
    return dict(inv_tau=float(dtype(1) / t), tau0=float(t),
                les_c=float(dtype(18.0 * math.sqrt(2.0) * CS * CS)), lid=float(dtype(U_LID)))


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def init_dist(ws, backend):
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group(backend=backend)
        return dist
    return None


def max_over_ranks(ms: float, dist) -> float:
    """The slowest rank's time (the whole job ends with it)."""
    if dist is None:
        return ms
    import torch

    t = torch.tensor([ms], dtype=torch.float64)
    if dist.get_backend() == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_mlups(cells: int, steps: int, ms: float, world: int) -> float:
    """Cell updates of all ranks (independent replicas) per second, in millions."""
    return cells * steps * world / (ms * 1e-3) / 1e6


def measured_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic():
    """DRAM bytes per cell update of the step kernel from the committed ncu
    summary (profiles/roofline_inputs.txt), or None."""
    f = ROOT / "profiles" / "roofline_inputs.txt"
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.startswith("dram_bytes_per_cell_update_f32:"):
            return float(line.split(":", 1)[1].split()[0])
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index, self.rows, self.proc = index, [], None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) == 6:
                self.rows.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(2)
            except Exception:
                self.proc.kill()
            self.t.join(1)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[2 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


# ------------------------------------------------------------ CPU (oracle)
def cpu_run(cells_z: int, steps: int, warmup: int, threads: int):
    """Oracle port of the reference kernels on the host cores, same
    configuration with a shorter z extent; returns (MLUPS, seconds, cells)."""
    os.environ["OMP_NUM_THREADS"] = str(threads)
    import numpy as np

    from oracle import oracle as O

    size = (SIZE[0], SIZE[1], cells_z)
    pp = lattice_params(np.float32)
    p = O.Params(inv_tau=pp["inv_tau"], tau0=pp["tau0"], les_c=pp["les_c"], lid=pp["lid"],
                 store_vel=False, store_rho=False)
    D = O.Domain(lambda d: O.OracleKernels("f32"), size, NUMS, p, "f32")
    D.perturb(SEED, AMP)
    for _ in range(warmup):
        D.step()
    t0 = time.perf_counter()
    for _ in range(steps):
        D.step()
    dt = time.perf_counter() - t0
    cells = size[0] * size[1] * size[2]
    return cells * steps / dt / 1e6, dt, cells


def cpu_baseline_sample(target_s=12.0):
    """Full 256^3 domain, as many timed steps as fit in about target_s seconds."""
    threads = os.cpu_count() or 1
    m0, _, _ = cpu_run(SIZE[2], 1, 1, threads)
    steps = int(max(2, min(200, target_s * m0 * 1e6 / (SIZE[0] * SIZE[1] * SIZE[2]))))
    z = SIZE[2]
    mlups, dt, cells = cpu_run(z, steps, 0, threads)
    return {"value": round(mlups, 2), "unit": "MLUPS", "cores": threads, "kind": "port",
            "sample": f"oracle port (C, OpenMP) of the reference kernels on the same 256^3 2x2x1 cavity, "
                      f"{steps} timed steps after 2 warm-up steps ({dt:.1f} s)"}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    # calibrate so that warm-up + timed steps take about 90 s in total
    m0, _, _ = cpu_run(8, 2, 1, threads)
    per_cell_s = 1.0 / (m0 * 1e6)
    budget = 90.0 / max(1, args.steps + args.warmup)
    z = int(max(6, min(SIZE[2], budget / (per_cell_s * SIZE[0] * SIZE[1]))))
    mlups, dt, cells = cpu_run(z, args.steps, args.warmup, threads)
    line = {
        "impl": "reference", "metric": METRIC, "value": round(mlups, 3), "unit": "MLUPS", "n_gpus": 0,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt / args.steps * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": config_dict("reference CPU arm: same cavity, z extent %d per step sample" % z),
        "cpu_baseline": {"value": round(mlups, 3), "unit": "MLUPS", "cores": threads, "kind": "port",
                         "sample": f"256x256x{z} slab of the 2x2x1 cavity per step ({cells} cells)"},
        "e2e": {"value": round(mlups, 3), "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def config_dict(note=None):
    d = {"workload": "lid-driven cavity 256^3, 2x2x1 subdomains of 128x128x256 on one GPU, D3Q19 BGK + "
                     "Smagorinsky Cs=0.17, Re=10000, lid u=0.1, seeded start-up +-1e-3",
         "size": list(SIZE), "subdomains": list(NUMS), "storage": "f32", "cs": CS, "re": RE, "lid": U_LID,
         "l2": "inputs larger than L2 (1.27 GB of populations per step vs 129 MB L2)",
         "halo": "after beta the 5 inward populations (reference); after alpha the 5 populations the ghost "
                 "layer's inner neighbours gather (fluid and lid cells identical to the 19-population exchange)"}
    if note:
        d["note"] = note
    return d


# ------------------------------------------------------------------ GPU arm
def make_params(api, storage):
    import numpy as np

    pp = lattice_params(np.float64 if storage == "f64" else np.float32)
    return api.Params.make(pp["inv_tau"], pp["tau0"], pp["les_c"], (0.0, 0.0, 0.0), pp["lid"])


def measure(api, size, nums, storage, steps, warmup, dist=None, clocks=None, shape=None, halo_mode=HALO_MODE,
            fp64_fma=False, fused=True):
    """K timed steps of one domain, replayed as one captured CUDA graph with a
    CUDA-event pair around every step kernel; returns (ms of the K steps,
    step-kernel ms per launch, MLUPS of the same K steps launched one by one
    without graph, cells)."""
    import torch

    D = api.Domain(size, nums, api.STORAGE_NAMES[storage], store_velocity=False, store_density=False)
    D.set_params(make_params(api, storage))
    D.set_halo_mode(halo_mode)
    if shape:
        D.set_kernel_shape(shape)
    if fp64_fma:
        D.set_fp64_contraction(True)
    if not fused:
        D.set_fused_exchange(False)
    D.reset()
    D.perturb(SEED, AMP)
    D.run(warmup, use_graph=False)
    D.profile(True)
    D.kernel_time(reset=True)
    # capture only, nothing runs; event pairs around a beta/alpha pair of step
    # kernels in every TIMED_EVERY steps (an event record in the graph costs ~1 %)
    D.prepare_timed_run(steps, TIMED_EVERY)
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ctx = clocks if clocks is not None else _Null()
    with ctx:
        start.record()
        D.run(steps, use_graph=True)
        stop.record()
        torch.cuda.synchronize()
    ms = start.elapsed_time(stop)
    (b_ms, b_n), (a_ms, a_n) = D.kernel_time_by_step()
    k_ms, k_n = D.kernel_time(reset=True)
    want = sum(1 for k in range(steps) if k % TIMED_EVERY < 2)
    if k_n != want:
        raise SystemExit(f"timed run recorded {k_n} step kernels, expected {want}")
    D.profile(False)
    g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    g0.record()
    D.run(steps, use_graph=False)
    g1.record()
    torch.cuda.synchronize()
    cells = D.cells
    eager_mlups = cells * steps / (g0.elapsed_time(g1) * 1e-3) / 1e6
    del D
    measure.split = (b_ms / max(1, b_n), a_ms / max(1, a_n))  # beta, alpha ms per launch
    return ms, k_ms / max(1, k_n), eager_mlups, cells


class _Null:
    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False


def run_gpu(args):
    ws, rank, local = dist_env()
    import torch

    torch.cuda.set_device(local)
    dist = init_dist(ws, "nccl")
    from turbulent_lbm_multigpu_gb300 import build, capi as api

    if rank == 0 or not build.LIB.exists():
        build.build()
    if dist:
        dist.barrier()

    with ClockSampler(local) as clk:
        ms, k_ms, eager_mlups, cells = measure(api, args.size, args.nums, args.storage, args.steps, args.warmup, dist,
                                               shape=args.shape, fp64_fma=args.fp64_fma)
        beta_ms, alpha_ms = measure.split
    ms = max_over_ranks(ms, dist)
    mlups = whole_job_mlups(cells, args.steps, ms, ws)
    if args.steps < 2:
        raise SystemExit("need at least 2 timed steps")

    # roofline of the step kernel
    peak, peak_kind = measured_peak()
    alg_bytes = BYTES_PER_CELL[args.storage] * cells
    achieved = alg_bytes / (k_ms * 1e-3) / 1e9
    traffic = profiled_traffic() if args.storage == "f32" else None
    ctype = {"f32": "float", "f64": "double", "f16": "half", "bf16": "bfloat16", "c16": "c16_t"}[args.storage]
    shape = args.shape or (3 if args.storage in ("f16", "bf16", "c16") else 1)
    kname = {1: f"k_beta/k_alpha<{ctype},LES> (one cell per thread)",
             2: f"k_beta2/k_alpha2<{ctype},LES> (two cells per thread)",
             3: f"k_step_staged<{ctype},LES> (TMA-staged tiles)"}[shape]
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": round(traffic * cells) if traffic else None,
                "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else
                "fallback 6.8 TB/s", "kernel": kname,
                "kernel_ms_per_launch": round(k_ms, 4), "alg_bytes_per_launch": alg_bytes,
                "by_step": {"beta_ms": round(beta_ms, 4), "beta_frac": round(alg_bytes / (beta_ms * 1e-3) / 1e9 / peak, 4),
                            "alpha_ms": round(alpha_ms, 4),
                            "alpha_frac": round(alg_bytes / (alpha_ms * 1e-3) / 1e9 / peak, 4),
                            "note": "the alpha kernel also copies the x faces of the exchange that follows it"}}

    prm = make_params(api, "f32")
    e2e = None if args.no_e2e else run_e2e(api, prm, args.steps)

    extra = {}
    if not args.no_extra and tuple(args.size) == SIZE:
        n = max(50, min(args.steps, 400))
        for label, size, nums, st, hm, fma, fu in (
                ("f32 256^3 2x2x1, x faces after alpha in their own launch", SIZE, NUMS, "f32", HALO_MODE, False, False),
                ("f32 256^3 2x2x1, reference exchange (19 populations after alpha)", SIZE, NUMS, "f32", 0, False, True),
                ("f64 256^3 2x2x1", SIZE, NUMS, "f64", HALO_MODE, False, True),
                ("f64 256^3 2x2x1, contracted multiply-adds (<= 1e-12 per step)", SIZE, NUMS, "f64", HALO_MODE, True, True),
                ("f16-shifted 256^3 2x2x1", SIZE, NUMS, "f16", HALO_MODE, False, True),
                ("bf16-shifted 256^3 2x2x1", SIZE, NUMS, "bf16", HALO_MODE, False, True),
                ("c16-shifted 256^3 2x2x1 (13-bit significand)", SIZE, NUMS, "c16", HALO_MODE, False, True),
                ("f32 512^3", (512, 512, 512), (1, 1, 1), "f32", HALO_MODE, False, True),
                ("f16-shifted 512^3", (512, 512, 512), (1, 1, 1), "f16", HALO_MODE, False, True),
                ("c16-shifted 512^3", (512, 512, 512), (1, 1, 1), "c16", HALO_MODE, False, True)):
            xms, xk, xg, xc = measure(api, size, nums, st, n, 4, halo_mode=hm, fp64_fma=fma, fused=fu)
            xa = BYTES_PER_CELL[st] * xc / (xk * 1e-3) / 1e9
            xb, xa_ = measure.split
            extra[label] = {"mlups": round(xc * n / (xms * 1e-3) / 1e6, 1), "eager_mlups": round(xg, 1),
                            "beta_ms": round(xb, 4), "alpha_ms": round(xa_, 4),
                            "kernel_ms": round(xk, 4), "achieved_gbs": round(xa, 1),
                            "frac_of_measured_hbm": round(xa / peak, 4), "steps": n,
                            "alg_bytes_per_cell": BYTES_PER_CELL[st]}

    if not args.no_extra and tuple(args.size) == SIZE:
        from turbulent_lbm_multigpu_gb300 import experiments as ex

        b = ex.batch(count=512, scale=10.0, check=2)
        extra["batch 512 cavities (steps/10)"] = {k: (round(v, 3) if isinstance(v, float) else v)
                                                 for k, v in b.items() if k != "config"}
        extra["batch 512 cavities (steps/10)"]["cell_updates"] = b["config"]["cell_updates"]
        sv = ex.serve(requests=24, scale=4.0, rates=(100, 400), accuracy_samples=0, f32_rate=None)
        extra["serving 24 requests (steps/4)"] = {
            "sequential_plain_f32_solves_per_s": round(sv["sequential_plain_f32"]["solves_per_s"], 3),
            "served": [{k: round(v, 4) for k, v in r.items()} for r in sv["served"]],
            "speedup_solves_per_s": [round(x, 3) for x in sv["speedup_solves_per_s"]],
            "f16_share": sv["config"]["f16_share"]}

    line = {
        "metric": METRIC, "value": round(mlups, 1), "unit": "MLUPS", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 5), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": args.storage, "data": "synthetic",
        "config": config_dict(None if tuple(args.size) == SIZE and args.storage == "f32"
                              else f"profiling size {args.size}, storage {args.storage}"),
        "roofline": roofline, "e2e": e2e,
        "gpu_launches": launches_per_run(args),
        "clocks": clk.summary(),
        "eager_mlups": round(eager_mlups, 1),
    }
    if extra:
        line["extra"] = extra
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline_sample()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def launches_per_run(args):
    """Kernel launches of the timed K steps: one step kernel per step and one
    exchange launch per decomposed axis, except the x part after alpha steps,
    which the one-cell alpha kernel does itself (kernel shape 1: float and
    double storage by default)."""
    axes = [a for a in range(3) if args.nums[a] > 1]
    fused = 0 in axes and (args.shape or (3 if args.storage in ("f16", "bf16", "c16") else 1)) == 1
    n = 0
    for k in range(args.steps):
        alpha = (args.warmup + k) & 1  # the counter starts at 0 and the warm-up steps come first
        n += 1 + len(axes) - (1 if alpha and fused else 0)
    return n


def run_e2e(api, prm, steps):
    """Upload the start-up field from pinned host memory, run, read the velocity back."""
    import numpy as np
    import torch

    D = api.Domain(SIZE, NUMS, api.F32, store_velocity=True, store_density=False)
    D.set_params(prm)
    D.set_halo_mode(HALO_MODE)
    D.reset()
    D.perturb(SEED, AMP)
    D.set_store_interval(0)  # velocity written on the last step only
    sub = D.sub
    n = sub[0] * sub[1] * sub[2]
    host_in = [torch.empty(19 * n, dtype=torch.float32).pin_memory().numpy() for _ in D.subdomains]
    host_out = [torch.empty(3 * n, dtype=torch.float32).pin_memory().numpy() for _ in D.subdomains]
    for L, h in zip(D.subdomains, host_in):
        L.read(api.FIELD_DD, out=h.reshape(19, sub[2], sub[1], sub[0]))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for L, h in zip(D.subdomains, host_in):
        L.write(api.FIELD_DD, h)
    D.run(steps, use_graph=True)
    for L, h in zip(D.subdomains, host_out):
        L.read(api.FIELD_VELOCITY, out=h.reshape(3, sub[2], sub[1], sub[0]))
    e1.record()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    ms = e0.elapsed_time(e1)
    h2d = sum(h.nbytes for h in host_in)
    d2h = sum(h.nbytes for h in host_out)
    del D
    return {"value": round(D_cells() * steps / (ms * 1e-3) / 1e6, 1), "unit": "MLUPS",
            "h2d_bytes_per_step": int(h2d // steps), "d2h_bytes_per_step": int(d2h // steps),
            "wall_s": round(wall, 4),
            "note": "start-up populations uploaded once and velocity read once per run of `steps` steps; "
                    "bytes per step are those totals divided by the step count"}


def D_cells():
    return SIZE[0] * SIZE[1] * SIZE[2]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end run (profiling)")
    ap.add_argument("--no-extra", action="store_true", help="skip the extra storage / size measurements")
    ap.add_argument("--size", type=int, nargs=3, default=list(SIZE), help="domain size (profiling only)")
    ap.add_argument("--nums", type=int, nargs=3, default=list(NUMS), help="subdomains (profiling only)")
    ap.add_argument("--storage", default="f32", choices=["f32", "f64", "f16", "bf16", "c16"],
                    help="population storage of the main measurement (profiling only)")
    ap.add_argument("--shape", type=int, default=None, choices=[1, 2, 3],
                    help="step kernel shape of the main measurement (profiling only)")
    ap.add_argument("--fp64-fma", action="store_true",
                    help="double storage: contracted multiply-add kernels in the main measurement (profiling only)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
