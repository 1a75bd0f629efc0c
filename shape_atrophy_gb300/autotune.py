"""Launch-shape autotuner.

Measures the launch shapes (and the mixed-precision inner floor) of the CUDA library on the current device and
writes them to ``tuning.json`` beside this file, keyed by device name and SM
count; ``api.context()`` applies the entry for its device the first time a
context is made (``SA_TUNING=off`` keeps the compiled defaults).

Shapes and the workload each is timed on (one coordinate pass, each value
timed ``reps`` times, the median kept; the other shapes stay at their best so
far):

* ``persistMaxWarps`` -- warps per CTA cap of the persistent cooperative CG
  (the CTA count is the slice count over it).  Workload: stepwise solve of the
  layered icosphere-5 shell (8 prism layers), FP64 and mixed precision, time
  per step summed over the two.
* ``vfdCtasPerSm`` -- CTAs per SM of the varifold pair sums (sets the number of
  column chunks).  Workload: the varifold objective of the same shell, FP64 and
  mixed.
* ``mixedInnerFloor`` -- the lowest squared relative residual (10^-k) the FP32
  inner solves of mixed precision aim for before the FP64 refinement takes
  over.  Workload: mixed-precision steps of the same shell.
* ``batchBlock`` x ``batchSlicesPerWarp`` -- CTA size of the batched serving CG
  and the rows per warp that size each solve's share of CTAs.  Workload: a
  seeded batch of shell requests (icosphere 3-5, 4-12 layers, 20 steps)
  submitted at once to the continuous-batching server, FP64 and mixed; time to
  drain.

Every value is a valid launch shape: the kernels fall back (persistent CG to
the two-kernel CG) when a shape does not fit, so the autotuner only ever picks
among measured, working configurations.  Results for a fixed table are
reproducible run to run (partial sums are grouped by the table and the
problem size only).

Usage: ``python -m shape_atrophy_gb300.autotune [--reps 3] [--out PATH] [--dry-run]``.
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np

from . import api, problems

CANDIDATES = {
    "persistMaxWarps": [8, 12, 16, 20],
    "vfdCtasPerSm": [2, 4, 8, 16, 32],
    "mixedInnerFloor": [8, 9, 10, 11, 12],
    "batchBlock": [128, 256],
    "batchSlicesPerWarp": [1, 2, 4],
}


def _median(f, reps):
    return float(np.median([f() for _ in range(reps)]))


def time_steps(spec, precision, steps=10, warm=3, device=0):
    """Seconds per step of a stepwise solve (each step call is synchronous)."""
    s = api.Session(spec, precision=precision, objective=False, device=device)
    s.step(warm)
    t0 = time.perf_counter()
    s.step(steps)
    dt = (time.perf_counter() - t0) / steps
    s.close()
    return dt


def time_objective(spec, precision, calls=5, device=0):
    """Seconds per varifold objective evaluation at the initial shape."""
    s = api.Session(spec, precision=precision, objective=True, device=device)
    s.objective()
    t0 = time.perf_counter()
    for _ in range(calls):
        s.objective()
    dt = (time.perf_counter() - t0) / calls
    s.close()
    return dt


def serving_batch(n=16, seed=11, steps=20):
    rng = np.random.default_rng(seed)
    cache, out = {}, []
    for _ in range(n):
        level = int(rng.choice([3, 4, 5], p=[0.4, 0.4, 0.2]))
        layers = int(rng.choice([4, 8, 12]))
        key = (level, layers)
        if key not in cache:
            cache[key] = problems.shell_layered(level=level, lyrCntNum=layers + 1, steps=steps, native=True)
        sp = dict(cache[key])
        lam = 10.0 ** rng.uniform(np.log10(0.5), 1.0, 3)
        sp["modVec"] = np.column_stack([lam, lam / 2]).reshape(-1)
        sp["spdLyrVec"] = 10.0 ** rng.uniform(np.log10(0.005), np.log10(0.1), 3)
        c = rng.normal(size=3)
        c /= np.linalg.norm(c)
        sp["tauVarVec"] = np.array([c[0], c[1], c[2], 1.0, 0.15])
        out.append(sp)
    return out


def time_served(reqs, precision, device=0):
    """Seconds to drain a batch of requests submitted at once."""
    sv = api.Server(hbm_budget=100e9, max_instances=64, device=device)
    t0 = time.perf_counter()
    ids = [sv.submit(sp, precision=precision) for sp in reqs]
    res = [sv.result(i) for i in ids]
    dt = time.perf_counter() - t0
    sv.close()
    if any(r["info"]["status"] != 0 for r in res):
        raise RuntimeError("a served solve failed during tuning")
    return dt


def tune(reps=3, device=0, log=print):
    api.context(device)                       # load the library; the table is ignored below
    best = dict(api.get_tuning())
    shell = problems.shell_layered(level=5, lyrCntNum=9, steps=20, native=True)
    reqs = serving_batch()
    meas = {}

    def sweep(name, score):
        rows = {}
        for v in CANDIDATES[name]:
            api.set_tuning(**{**best, name: v})
            rows[v] = _median(score, reps)
            log(f"  {name}={v}: {1e3 * rows[v]:.3f} ms")
        best[name] = min(rows, key=rows.get)
        api.set_tuning(**best)
        meas[name] = {str(k): 1e3 * t for k, t in rows.items()}

    log("persistent CG (icosphere-5 shell, ms per step, FP64 + mixed)")
    sweep("persistMaxWarps", lambda: time_steps(shell, "fp64", device=device) +
          time_steps(shell, "mixed", device=device))
    log("varifold pair sums (icosphere-5 shell, ms per objective, FP64 + mixed)")
    sweep("vfdCtasPerSm", lambda: time_objective(shell, "fp64", device=device) +
          time_objective(shell, "mixed", device=device))
    log("mixed-precision inner floor (icosphere-5 shell, ms per mixed step)")
    sweep("mixedInnerFloor", lambda: time_steps(shell, "mixed", device=device))
    log("batched CG (16 shell requests at once, ms to drain, FP64 + mixed)")
    time_served(reqs[:2], "fp64", device=device)     # warm the server path
    for name in ("batchBlock", "batchSlicesPerWarp"):
        sweep(name, lambda: time_served(reqs, "fp64", device=device) + time_served(reqs, "mixed", device=device))
    name, sms = api.device_name(device)
    return {"name": name, "smCount": sms, "values": best, "ms": meas, "reps": reps,
            "workloads": {"persistMaxWarps": "icosphere-5 shell, 8 prism layers, 10 steps after 3, FP64 + mixed",
                          "vfdCtasPerSm": "varifold objective of the same shell, 5 calls, FP64 + mixed",
                          "mixedInnerFloor": "mixed-precision steps of the same shell, 10 steps after 3",
                          "batchBlock": "16 seeded shell requests (icosphere 3-5, 4-12 layers, 20 steps) "
                                        "drained by the server, FP64 + mixed",
                          "batchSlicesPerWarp": "as batchBlock"}}


def write_entry(entry, path=api.TUNING_FILE):
    table = {"devices": []}
    if os.path.exists(path):
        with open(path) as f:
            table = json.load(f)
    table["devices"] = [e for e in table.get("devices", [])
                        if not (e.get("name") == entry["name"] and e.get("smCount") == entry["smCount"])]
    table["devices"].append(entry)
    with open(path, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
        f.write("\n")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--out", default=api.TUNING_FILE)
    ap.add_argument("--dry-run", action="store_true", help="print the entry, do not write the table")
    args = ap.parse_args()
    os.environ["SA_TUNING"] = "off"           # tune from the compiled defaults
    entry = tune(reps=args.reps, device=args.device)
    print(json.dumps(entry), flush=True)
    if not args.dry_run:
        write_entry(entry, args.out)


if __name__ == "__main__":
    main()
