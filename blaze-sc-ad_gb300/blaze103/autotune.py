"""Autotuner of the launch shape, per workload shape.

For each named shape (a query-length profile, a batch size and a database
size) it times the search over a grid of launch settings with CUDA events --
the subject staging bound (subjects up to `stage_bytes` residues are staged in
shared memory, longer ones are read from global memory), warps per scan block,
residues per batched tile and the batched launch mode (tiles of many queries
per launch, or one launch per query) -- checks that every setting returns the
same HSPs, and writes the fastest setting per shape to ``tuning.json`` beside
this file. ``lookup`` returns the entry of the nearest shape; ``PrelimSearch``
applies it to batched runs unless a tuning was set explicitly.

Run on the GPU:  python blaze-sc-ad_gb300/blaze103/autotune.py [--quick]
"""
from __future__ import annotations

import argparse
import itertools
import json
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TUNING_PATH = os.path.join(HERE, "tuning.json")

# shapes: (kind, synthetic workload, scale of its database, queries, grid,
# timed repetitions). Knobs: the subject staging bound, warps per scan block
# (0: as many as registers allow), residues per warp of a batched tile (0:
# several tiles' worth per warp) and the batched launch mode (1: tiles of
# many queries per launch, 2: one scan launch per query).
_SMALL_BATCH_GRID = {
    "stage_bytes": (1024, 2048),
    "max_warps_per_block": (16, 0),
    "tile_residues": (0, 4096, 65536),
    "batch_launch": (1, 2),
}
SHAPES = {
    "plain-db-scale": ("plain", "plain-db-scale", 1.0, 8,
                       {"stage_bytes": (1024, 2048, 4096), "max_warps_per_block": (8, 16, 0)}, 3),
    "batched-512": ("batched", "batched", 0.02, 512, _SMALL_BATCH_GRID, 3),
    "batched-512-full": ("batched", "batched", 1.0, 512, {"stage_bytes": (1024, 2048), "batch_launch": (1, 2)}, 1),
    "batched-64": ("batched", "batched", 0.02, 64, _SMALL_BATCH_GRID, 3),
    "serving-32": ("batched", "serving", 0.01, 32, _SMALL_BATCH_GRID, 3),
    "serving-4-large": ("batched", "serving", 0.1, 4, {"stage_bytes": (1024, 2048), "batch_launch": (1, 2)}, 3),
}
DEFAULT = {"stage_bytes": 1024, "max_warps_per_block": 0, "tile_residues": 0, "batch_launch": 0}

_cache = None


def load_table(path: str = TUNING_PATH) -> dict:
    global _cache
    if _cache is None:
        try:
            with open(path) as f:
                _cache = json.load(f)
        except (OSError, ValueError):
            _cache = {"shapes": {}}
    return _cache


def lookup(kind: str, n_queries: int, median_qlen: float, db_residues: int) -> dict | None:
    """Tuning of the nearest tuned shape of this kind (log distance over batch
    size, median query length and database residues), or None."""
    best, best_d = None, math.inf
    for entry in load_table().get("shapes", {}).values():
        if entry.get("kind") != kind:
            continue
        d = (abs(math.log(max(n_queries, 1) / entry["n_queries"]))
             + abs(math.log(max(median_qlen, 1) / entry["median_qlen"]))
             + 0.5 * abs(math.log(max(db_residues, 1) / entry["db_residues"])))
        if d < best_d:
            best, best_d = entry, d
    return dict(best["tuning"]) if best else None


def _time_setting(ps, run, tuning, reps):
    ps.set_tuning(**tuning)
    out = run()  # warm: buffers sized, graph captured
    ms = []
    for _ in range(reps):
        run()
        ms.append(ps.stats()["device_ms"])
    return float(np.median(ms)), out


def tune_shape(name: str, reps: int | None = None, quick: bool = False) -> dict:
    import blaze103
    from blaze103 import synth

    kind, workload, scale, nq, grid, shape_reps = SHAPES[name]
    reps = shape_reps if reps is None else reps
    seed = synth.WORKLOADS[workload]["index"]
    w = synth.make_workload(workload, scale=scale, n_queries=nq, seed=seed)
    rng = np.random.default_rng(seed)
    queries = list(w.queries)
    while len(queries) < nq:  # workloads with fewer queries than the batch: draw more
        queries.append(synth.random_residues(rng, int(synth.lognormal_lengths(rng, 1, 350, 0.82, 30, 5000)[0])))
    queries = queries[:nq]
    db = blaze103.SeqSrc(w.residues, w.offsets)
    ps = blaze103.PrelimSearch(db, autotune=False)
    params = [blaze103.default_params(len(q), db) for q in queries]
    if kind == "batched":
        batch = blaze103.QueryBatch(db, queries)

        def run():
            return ps.run_batch(batch, params)
    else:
        singles = [blaze103.Query(db, q) for q in queries]

        def run():
            total = 0.0
            outs = []
            for q, p in zip(singles, params):
                ps.run_query(q, p)
                outs.append(ps.results())
                total += ps.stats()["device_ms"]
            run.ms = total
            return outs

    grid = dict(grid)
    if quick:
        grid = {k: v[:2] for k, v in grid.items()}
    rows, ref = [], None
    for vals in itertools.product(*grid.values()):
        tuning = dict(DEFAULT)
        tuning.update(zip(grid.keys(), vals))
        if kind == "plain":
            ps.set_tuning(**tuning)
            out = run()
            ms = float(np.median([(run(), run.ms)[1] for _ in range(reps)]))
        else:
            ms, out = _time_setting(ps, run, tuning, reps)
        if ref is None:
            ref = out
        same = (np.array_equal(out, ref) if kind == "batched"
                else all(np.array_equal(a, b) for a, b in zip(out, ref)))
        if not same:
            raise RuntimeError(f"{name}: tuning {tuning} changed the results")
        rows.append({"tuning": tuning, "ms": ms})
        print(f"{name} {tuning} {ms:.2f} ms", file=sys.stderr, flush=True)
    rows.sort(key=lambda r: r["ms"])
    lengths = [len(q) for q in queries]
    entry = {"kind": kind, "n_queries": nq, "median_qlen": float(np.median(lengths)),
             "db_residues": int(w.total_residues), "db_subjects": int(w.n_subjects),
             "tuning": rows[0]["tuning"], "ms": rows[0]["ms"],
             "default_ms": next((r["ms"] for r in rows
                                 if all(r["tuning"][k] == DEFAULT[k] for k in ("stage_bytes", "max_warps_per_block",
                                                                                "tile_residues"))), None),
             "grid": rows}
    if kind == "batched":
        batch.close()
    else:
        for q in singles:
            q.close()
    ps.close()
    db.close()
    return entry


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--shapes", default=",".join(SHAPES))
    ap.add_argument("--reps", type=int, default=None, help="timed repetitions (default: per shape)")
    ap.add_argument("--quick", action="store_true", help="two values per knob")
    ap.add_argument("--out", default=TUNING_PATH)
    args = ap.parse_args()
    sys.path.insert(0, os.path.dirname(HERE))
    table = {"generated": time.strftime("%Y-%m-%d %H:%M:%S"), "shapes": {}}
    try:
        import torch  # noqa: F401  (device name for the record only)
        table["device"] = torch.cuda.get_device_name(0)
    except Exception:  # noqa: BLE001
        pass
    for name in args.shapes.split(","):
        table["shapes"][name] = tune_shape(name, args.reps, args.quick)
    with open(args.out, "w") as f:
        json.dump(table, f, indent=1)
    print(json.dumps({k: (v["tuning"], v["ms"], v["default_ms"]) for k, v in table["shapes"].items()}))


if __name__ == "__main__":
    main()
