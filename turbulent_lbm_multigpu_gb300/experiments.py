"""Measurements of the three systems patterns on one GPU.

    python -m turbulent_lbm_multigpu_gb300.experiments precision [--size 768 --steps 5000]
    python -m turbulent_lbm_multigpu_gb300.experiments batch [--count 512 --scale 1]
    python -m turbulent_lbm_multigpu_gb300.experiments serve [--requests 256 --scale 1]

Each prints one JSON object.  Inputs are synthetic and seeded: lid-driven
cavities drawn with the seeds and distributions of the configurations
(precision: 768^3, Re 2e4, lid 0.1, Cs 0.17, seed 1234, start-up +-1e-3;
batch: 512 cavities, seed 42, edges log-uniform on [32, 128], Re on
[100, 5000], lid on [0.02, 0.1], steps on {500..5000}, f32 or shifted f16;
serving: Poisson arrivals at 50-400 /s, seed 7, edges log-uniform on
[32, 256], Re on [100, 2e4], steps on {500..20000}, f32 or shifted f16,
150 GB HBM budget).  `--scale` divides the step counts (the default bench
runs reduced samples; the full runs are recorded under profiles/).
"""
from __future__ import annotations

import argparse
import json
import math
import time

import numpy as np

from . import capi as api

CS = 0.17


def tau_for(u: float, length: float, re: float) -> float:
    """tau = 3 nu + 1/2 with nu = U L / Re (lattice units)."""
    return 3.0 * u * length / re + 0.5


def _sync():
    api.check(api.lib().lbm_cu_synchronize(None))


def _lattice_params(storage: int, tau: float, cs: float, lid: float):
    if storage == api.F64:
        t = float(np.float64(tau))
        inv = 1.0 / t
    else:
        t32 = np.float32(tau)
        t, inv = float(t32), float(np.float32(1) / t32)
    return api.Params.make(inv, t, api.les_coefficient(cs), (0.0, 0.0, 0.0), lid)


def cavity_lattice(dims, storage, tau, cs, lid, seed, amp, store_velocity=False):
    """A lone lid-driven cavity at step 0 (walls, lid plane, seeded start-up)."""
    L = api.Lattice(*dims, storage, store_velocity, False)
    L.set_params(_lattice_params(storage, tau, cs, lid))
    L.init([api.FLAG_OBSTACLE] * 6)
    nx, ny, nz = dims
    L.write(api.FIELD_FLAGS, np.full((nz - 2) * (nx - 2), api.FLAG_VELOCITY_INJECTION, np.int32),
            origin=(1, ny - 2, 1), size=(nx - 2, 1, nz - 2))
    if amp:
        L.perturb((0, 0, 0), dims, seed, amp)
    return L


def centerline_ux(L: api.Lattice, layout: int):
    """u_x along the vertical line x = nx/2, z = nz/2, from the populations."""
    nx, ny, nz = L.dims
    f = L.read(api.FIELD_DD, origin=(nx // 2, 0, nz // 2), size=(1, ny, 1))[:, 0, :, 0].astype(np.float64)
    ex = np.array([1, -1, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0, 0, 0, 0], dtype=np.float64)
    if layout:
        f = f[[i ^ 1 if i < 18 else 18 for i in range(19)]]
    return ex @ f


# ------------------------------------------------------------- precision
def precision(size=768, steps=5000, every=100, compare_every=1000, storages=("f64", "f32", "f16", "bf16", "c16"),
              re=20000.0, lid=0.1, seed=1234, amp=1e-3):
    dims = (size, size, size)
    tau = tau_for(lid, size, re)
    lats, ms, series = {}, {}, {}
    for name in storages:
        st = api.STORAGE_NAMES[name]
        lats[name] = cavity_lattice(dims, st, tau, CS, lid, seed, amp)
        ms[name] = 0.0
        series[name] = []
    ref = storages[0]
    errors = []
    step = 0
    ev0, ev1 = None, None
    try:
        import torch

        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    except Exception:
        pass
    while step < steps:
        n = min(every, steps - step)
        layout = (step + n - 1) & 1  # after the chunk: last step beta -> 0, alpha -> 1
        for name, L in lats.items():
            _sync()
            if ev0 is not None:
                ev0.record()
                L.run(step, n)
                ev1.record()
                ev1.synchronize()
                ms[name] += ev0.elapsed_time(ev1)
            else:
                t0 = time.perf_counter()
                L.run(step, n)
                _sync()
                ms[name] += (time.perf_counter() - t0) * 1e3
            m = L.reduce_conserved(layout)
            series[name].append({"step": step + n, "mass": m[0], "jx": m[1], "jy": m[2], "jz": m[3], "energy": m[4]})
        step += n
        if step % compare_every == 0 or step == steps:
            row = {"step": step}
            for name, L in lats.items():
                if name != ref:
                    row[name] = api.compare_velocity(L, layout, lats[ref], layout)
            errors.append(row)
    cells = size ** 3
    out = {"config": {"size": dims, "steps": steps, "re": re, "lid": lid, "tau": tau, "cs": CS, "seed": seed,
                      "amp": amp, "reference": ref},
           "mlups": {k: cells * steps / (v * 1e-3) / 1e6 for k, v in ms.items()},
           "final_error_vs_" + ref: errors[-1], "error_series": errors}
    out["deviation_stats"] = {k: api.deviation_stats(L) for k, L in lats.items() if k in ("f16", "bf16", "c16")}
    layout = (steps - 1) & 1
    prof = {k: centerline_ux(L, layout) for k, L in lats.items()}
    out["centerline_ux"] = {k: {"mean": float(v.mean()), "rms": float(np.sqrt((v ** 2).mean())),
                                "max_rel_diff_vs_ref": float(np.max(np.abs(v - prof[ref])) /
                                                             max(np.max(np.abs(prof[ref])), 1e-30))}
                            for k, v in prof.items()}
    m0 = {k: s[0]["mass"] for k, s in series.items()}
    out["mass_drift"] = {k: [(r["step"], (r["mass"] - m0[k]) / m0[k]) for r in s] for k, s in series.items()}
    out["kinetic_energy"] = {k: [(r["step"], r["energy"]) for r in s] for k, s in series.items()}
    e_ref = series[ref][-1]["energy"]
    out["energy_rel_diff_vs_ref"] = {k: (s[-1]["energy"] - e_ref) / e_ref for k, s in series.items()}
    return out


# ----------------------------------------------------------------- batch
def batch_specs(count=512, seed=42, scale=1.0):
    rng = np.random.default_rng(seed)
    specs = []
    for _ in range(count):
        edges = np.exp(rng.uniform(math.log(32), math.log(128), 3)).round().astype(int)
        re = rng.uniform(100, 5000)
        u = rng.uniform(0.02, 0.1)
        steps = int(rng.integers(500, 5001))
        storage = api.F16 if rng.random() < 0.5 else api.F32
        steps = max(2, int(round(steps / scale)))
        specs.append(api.Cavity.make(tuple(int(e) for e in edges), storage, tau_for(u, float(edges[0]), re), CS,
                                     float(u), steps, int(rng.integers(0, 2 ** 32)), 1e-3))
    return specs


def batch(count=512, seed=42, scale=1.0, check=4):
    specs = batch_specs(count, seed, scale)
    updates = sum(c.nx * c.ny * c.nz * c.steps for c in specs)
    B = api.Batch(specs, store_velocity=False)
    shape, tune_ms = B.tune(trial_steps=10)
    B.reset()
    _sync()
    t0 = time.perf_counter()
    B.run(use_graph=True)
    _sync()
    t_batch = time.perf_counter() - t0

    # the same cavities one by one: one lattice at a time, one launch per step
    t_seq = 0.0
    same = True
    for i, c in enumerate(specs):
        L = cavity_lattice((c.nx, c.ny, c.nz), c.storage, c.tau0, c.cs, c.lid, c.seed, c.amp)
        _sync()
        t0 = time.perf_counter()
        L.run(0, c.steps)
        _sync()
        t_seq += time.perf_counter() - t0
        if i < check:
            a, b = L.read(api.FIELD_DD), B.lattices[i].read(api.FIELD_DD)
            same = same and bool(np.array_equal(a.view(np.uint8), b.view(np.uint8)))
        del L
    # one by one again, each cavity's steps replayed from a captured graph (a
    # one-subdomain domain): separates the launch overhead from the packing
    t_graph = 0.0
    for i, c in enumerate(specs):
        D = api.Domain((c.nx, c.ny, c.nz), (1, 1, 1), c.storage)
        D.set_params(_lattice_params(c.storage, c.tau0, c.cs, c.lid))
        D.reset()
        D.perturb(c.seed, c.amp)
        _sync()
        t0 = time.perf_counter()
        D.run(c.steps, use_graph=True)
        _sync()
        t_graph += time.perf_counter() - t0
        if i < check:
            a, b = D.subdomains[0].read(api.FIELD_DD), B.lattices[i].read(api.FIELD_DD)
            same = same and bool(np.array_equal(a.view(np.uint8), b.view(np.uint8)))
        D.close()
    return {"config": {"cavities": count, "seed": seed, "step_scale": scale, "cell_updates": updates,
                       "f16_share": sum(c.storage == api.F16 for c in specs) / count},
            "tuned_cells_per_thread": shape, "tune_ms_per_step": tune_ms,
            "batched_s": t_batch, "batched_mlups": updates / t_batch / 1e6,
            "one_by_one_s": t_seq, "one_by_one_mlups": updates / t_seq / 1e6,
            "one_by_one_graph_s": t_graph, "one_by_one_graph_mlups": updates / t_graph / 1e6,
            "speedup": t_seq / t_batch, "speedup_vs_graph_replay": t_graph / t_batch,
            f"first_{check}_identical": same}


# ----------------------------------------------------------------- serving
def serve_specs(requests=64, seed=7, scale=1.0):
    rng = np.random.default_rng(seed)
    specs = []
    for _ in range(requests):
        edges = np.exp(rng.uniform(math.log(32), math.log(256), 3)).round().astype(int)
        re = rng.uniform(100, 20000)
        u = 0.1
        steps = max(2, int(round(int(rng.integers(500, 20001)) / scale)))
        storage = api.F16 if rng.random() < 0.5 else api.F32
        specs.append(api.Cavity.make(tuple(int(e) for e in edges), storage, tau_for(u, float(edges[0]), re), CS,
                                     u, steps, int(rng.integers(0, 2 ** 32)), 1e-3))
    return specs


def serve_run(specs, rate, seed=7, budget=150e9, quantum=64, keep=()):
    """Poisson arrivals at `rate` per second into the continuous-batching
    server.  Per request: arrival, admission (the tick whose admission step
    took it: the server admits in arrival order), completion.  The
    populations and flags of the requests in `keep` are read back at
    completion (for the accuracy check)."""
    rng = np.random.default_rng(seed + int(rate))
    arrivals = np.cumsum(rng.exponential(1.0 / rate, len(specs)))
    S = api.Server(budget, store_velocity=False)
    submitted = 0
    waiting = []  # submitted, not yet admitted, in arrival order
    t0 = time.perf_counter()
    done_at, admit_at, sid_of, kept = {}, {}, {}, {}
    ticks = 0
    while len(done_at) < len(specs):
        now = time.perf_counter() - t0
        while submitted < len(specs) and arrivals[submitted] <= now:
            sid_of[S.submit(specs[submitted])] = submitted
            waiting.append(submitted)
            submitted += 1
        st = S.status()
        if st["active"] == 0 and st["queued"] == 0:
            # idle until the next arrival
            time.sleep(max(0.0, arrivals[submitted] - now))
            continue
        t_tick = time.perf_counter() - t0
        n_adm = S.tick(max_steps=quantum)
        ticks += 1
        for i in waiting[:n_adm]:
            admit_at[i] = t_tick
        del waiting[:n_adm]
        for sid in S.poll():
            i = sid_of[sid]
            done_at[i] = time.perf_counter() - t0
            if i in keep:
                L = S.lattice(sid)
                kept[i] = (L.read(api.FIELD_DD), L.read(api.FIELD_FLAGS)[0])
            S.release(sid)
    lat = np.array([done_at[i] - arrivals[i] for i in range(len(specs))])
    wait = np.array([admit_at[i] - arrivals[i] for i in range(len(specs))]).clip(min=0.0)
    service = np.array([done_at[i] - admit_at[i] for i in range(len(specs))])
    elapsed = max(done_at.values()) - arrivals[0]
    admitted_span = max(admit_at.values()) - min(admit_at.values())
    updates = S.status()["cell_updates"]
    pct = lambda a, q: float(np.percentile(a, q))  # noqa: E731
    out = {"rate": rate, "p50_s": pct(lat, 50), "p99_s": pct(lat, 99),
           "queue_wait_p50_s": pct(wait, 50), "queue_wait_p99_s": pct(wait, 99),
           "service_p50_s": pct(service, 50), "service_p99_s": pct(service, 99),
           "offered_per_s": len(specs) / (arrivals[-1] - arrivals[0]),
           "admitted_per_s": (len(specs) - 1) / admitted_span if admitted_span > 0 else float("inf"),
           "solves_per_s": len(specs) / elapsed, "mlups": updates / elapsed / 1e6, "elapsed_s": elapsed,
           "ticks": ticks}
    return out, kept


def sequential_plain(specs):
    """Every request alone, f32, one after the other, one launch per step."""
    t = 0.0
    updates = 0
    for c in specs:
        L = cavity_lattice((c.nx, c.ny, c.nz), api.F32, c.tau0, c.cs, c.lid, c.seed, c.amp)
        _sync()
        t0 = time.perf_counter()
        L.run(0, c.steps)
        _sync()
        t += time.perf_counter() - t0
        updates += c.nx * c.ny * c.nz * c.steps
        del L
    return {"solves_per_s": len(specs) / t, "mlups": updates / t / 1e6, "elapsed_s": t}


_EXYZ = np.array([[1, -1, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0, 0, 0, 0],
                  [0, 0, 1, -1, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 0],
                  [0, 0, 0, 0, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1, 1, -1, 0]], dtype=np.float64)


def _velocity_error(dd, dd_ref, flags):
    """Relative RMS and max error of the momentum sum_i e_i f_i over the fluid
    cells (both populations in the same slot layout)."""
    m = flags == api.FLAG_FLUID
    j = _EXYZ @ dd[:, m].astype(np.float64)
    r = _EXYZ @ dd_ref[:, m].astype(np.float64)
    d = np.sqrt(((j - r) ** 2).sum(0))
    nr = np.sqrt((r ** 2).sum(0))
    return {"rel_rms": float(np.sqrt((d ** 2).sum() / (nr ** 2).sum())), "rel_max": float(d.max() / nr.max())}


def served_accuracy(specs, kept):
    """Velocity error of served 16-bit solves (read back at completion)
    against the same solve in FP64 alone, beside the error of the same solve
    in plain FP32 alone."""
    rows = []
    for i, (dd, flags) in sorted(kept.items()):
        c = specs[i]
        ref = cavity_lattice((c.nx, c.ny, c.nz), api.F64, c.tau0, c.cs, c.lid, c.seed, c.amp)
        ref.run(0, c.steps)
        f64 = ref.read(api.FIELD_DD)
        del ref
        L32 = cavity_lattice((c.nx, c.ny, c.nz), api.F32, c.tau0, c.cs, c.lid, c.seed, c.amp)
        L32.run(0, c.steps)
        f32 = L32.read(api.FIELD_DD)
        del L32
        rows.append({"request": i, "dims": [c.nx, c.ny, c.nz], "steps": c.steps, "storage": int(c.storage),
                     "served_vs_f64": _velocity_error(dd, f64, flags),
                     "plain_f32_vs_f64": _velocity_error(f32, f64, flags)})
    return rows


def serve(requests=256, seed=7, scale=1.0, rates=(50, 100, 200, 400), budget=150e9, accuracy_samples=6,
          f32_rate=100):
    specs = serve_specs(requests, seed, scale)
    seq = sequential_plain(specs)
    # the accuracy sample: the first 16-bit requests of at most ~2.1 M cells
    keep = [i for i, c in enumerate(specs) if c.storage != api.F32 and c.nx * c.ny * c.nz <= 2_100_000]
    keep = set(keep[:accuracy_samples])
    runs, kept = [], {}
    for r in rates:
        out, k = serve_run(specs, r, seed, budget, keep=keep if r == rates[0] else ())
        runs.append(out)
        kept.update(k)
    # the same requests all in plain f32, served: packing without the 16-bit share
    specs32 = [api.Cavity.make((c.nx, c.ny, c.nz), api.F32, c.tau0, c.cs, c.lid, c.steps, c.seed, c.amp)
               for c in specs]
    out = {"config": {"requests": requests, "seed": seed, "step_scale": scale, "budget_bytes": budget,
                      "f16_share": sum(c.storage == api.F16 for c in specs) / requests,
                      "cell_updates": sum(c.nx * c.ny * c.nz * c.steps for c in specs)},
           "sequential_plain_f32": seq, "served": runs,
           "speedup_solves_per_s": [r["solves_per_s"] / seq["solves_per_s"] for r in runs]}
    if f32_rate:
        served32, _ = serve_run(specs32, f32_rate, seed, budget)
        out["served_all_f32"] = served32
        out["speedup_all_f32"] = served32["solves_per_s"] / seq["solves_per_s"]
    if kept:
        out["accuracy"] = served_accuracy(specs, kept)
    return out


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("what", choices=["precision", "batch", "serve"])
    ap.add_argument("--size", type=int, default=768)
    ap.add_argument("--steps", type=int, default=5000)
    ap.add_argument("--count", type=int, default=512)
    ap.add_argument("--requests", type=int, default=256)
    ap.add_argument("--scale", type=float, default=1.0)
    a = ap.parse_args()
    from . import build

    build.build()
    if a.what == "precision":
        r = precision(a.size, a.steps)
    elif a.what == "batch":
        r = batch(a.count, scale=a.scale)
    else:
        r = serve(a.requests, scale=a.scale)
    print(json.dumps(r, default=float))


if __name__ == "__main__":
    main()
