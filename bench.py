#!/usr/bin/env python3
"""Benchmark of the BLASTP preliminary search stage on GB300.

Workload (N=1): the plain GPU drop-in at database scale -- 8 queries of 100,
200, 300, 500, 700, 800, 900 and 1,000 residues, each searched on its own
(one launch sequence per query) against a 2M-subject, ~0.7G-residue synthetic
database resident in HBM (seeded; log-normal lengths, median 250, sorted;
1% planted homologs). A step is one pass of all 8 queries over the database.

metric  DB residues/s per query, aggregated: (queries x DB residues) / time.
value   device time (CUDA events on the search stream, summed over the runs)
        with the database and the query tables already resident.
e2e     the same metric through blaze_prelim_search with host query buffers:
        lookup build, H2D of the tables and D2H of the HSPs inside the timed
        region (wall clock).
roofline  the scan kernel (word finder + two-hit + ungapped), HBM-bound:
        algorithmic bytes per launch = residues (1 B) + offsets (8 B each).

parity  the oracle's HSPs for the cpu_baseline sample (every 4th subject,
        whole-database statistics) compared field by field with the e2e
        path's HSPs for the same OIDs.
batched / serve  sub-records at N=1: the batched form on the 512-query,
        5M-subject workload against the plain path on the same GPU (with
        batched == plain and oracle checks on a subject sample), and the
        serving loop's p50/p99 latency under Poisson arrivals.

`--impl reference` times the CPU implementation of the path (the oracle port:
NCBI blastp 2.13.0 is not installed on this machine) on the host cores, on the
same bounded subject sample of the same workload per step as cpu_baseline.

With N>1 (torchrun) every rank searches its own database of the same size
(weak scaling, E-values over the global size) and the slowest rank's time
counts; no collective touches the data path.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for p in (ROOT, os.path.join(ROOT, "blaze-sc-ad_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

import numpy as np  # noqa: E402

METRIC = "DB residues/s per query (aggregate over queries)"
UNIT = "residues/s"
PEAKS_PATH = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


class Group:
    """Barrier and max-reduction across ranks (torch.distributed when N>1)."""

    def __init__(self, world, device):
        self.world = world
        self.dist = None
        if world > 1:
            import torch
            import torch.distributed as dist

            backend = "nccl" if torch.cuda.is_available() else "gloo"
            if backend == "nccl":
                torch.cuda.set_device(device)
            dist.init_process_group(backend=backend)
            self.dist, self.torch, self.backend = dist, torch, backend

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def max(self, x: float) -> float:
        if not self.dist:
            return x
        dev = "cuda" if self.backend == "nccl" else "cpu"
        t = self.torch.tensor([float(x)], dtype=self.torch.float64, device=dev)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.dist:
            self.dist.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.reader = threading.Thread(target=self._read, daemon=True)
            self.reader.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.reader.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for name, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak():
    try:
        with open(PEAKS_PATH) as f:
            pk = json.load(f)
        return float(pk["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback"


def subject_sample(workload, k: int):
    """Every k-th subject of the database (a bounded sample with the same
    length distribution): (OIDs, residues, offsets)."""
    off = workload.offsets
    idx = np.arange(0, workload.n_subjects, k)
    lens = (off[idx + 1] - off[idx]).astype(np.int64)
    sub_off = np.zeros(len(idx) + 1, dtype=np.uint64)
    np.cumsum(lens, out=sub_off[1:])
    if k == 1:
        return idx, workload.residues, sub_off
    res = workload.residues
    return idx, np.concatenate([res[int(off[i]):int(off[i + 1])] for i in idx]), sub_off


def cpu_sample_run(workload, queries, frac: float, threads: int, db_total: int, db_n: int, keep: bool = False):
    """Time the oracle on every k-th subject of the database (k = 1/frac);
    returns (residues/s, seconds, residues, subjects, sample). With keep, the
    sample is (OIDs, per-query oracle HSPs with E-values and reap, subject =
    position in the sample); the finishing step is outside the timed span."""
    import oracle

    k = max(int(round(1.0 / frac)), 1)
    idx, res, sub_off = subject_sample(workload, k)
    raw = []
    t0 = time.perf_counter()
    for q in queries:
        p = oracle.default_params(len(q), db_total, db_n)
        hs, _ = oracle.search_db(q, res, sub_off, p, threads=threads)
        raw.append((hs, p))
    dt = time.perf_counter() - t0
    n_res = int(sub_off[-1]) * len(queries)
    sample = (idx, [oracle.finish(hs, p) for hs, p in raw]) if keep else None
    return n_res / dt, dt, n_res, len(idx), sample


PARITY_FIELDS = [("oid", "subject"), ("score", "score"), ("q_start", "q_start"), ("q_end", "q_end"),
                 ("s_start", "s_start"), ("s_end", "s_end"), ("q_gapped_start", "q_gstart"),
                 ("s_gapped_start", "s_gstart")]


def parity_check(idx, ref_lists, got_lists, k: int) -> dict:
    """Field-by-field comparison of GPU HSPs (HSP_DTYPE, all subjects) with
    the oracle's HSPs of the subject sample (OIDs idx = every k-th), per
    query; a record counts as a mismatch when it is missing on either side
    or differs in any field (E-values: relative 1e-12)."""
    from collections import Counter

    mism = hsps = ev_bad = 0
    for ref, got in zip(ref_lists, got_lists):
        g = got[(got["oid"] % k) == 0] if k > 1 else got
        r = ref.copy()
        r["subject"] = idx[r["subject"]].astype(r["subject"].dtype)
        hsps += len(r)
        if len(g) == len(r):
            same = np.ones(len(r), dtype=bool)
            for gf, rf in PARITY_FIELDS:
                same &= g[gf].astype(np.int64) == r[rf].astype(np.int64)
            if len(r):
                ev_ok = np.abs(g["evalue"] - r["evalue"]) <= 1e-12 * np.abs(r["evalue"])
                ev_bad += int((~ev_ok & same).sum())
                same &= ev_ok
            mism += int((~same).sum())
            continue
        tg = Counter(tuple(int(x[f]) for f, _ in PARITY_FIELDS) for x in g)
        tr = Counter(tuple(int(x[f]) for _, f in PARITY_FIELDS) for x in r)
        mism += sum(((tg - tr) + (tr - tg)).values())
    return {"hsps": hsps, "mismatches": mism, "evalue_mismatches": ev_bad,
            "fields": [f for f, _ in PARITY_FIELDS] + ["evalue (rtol 1e-12)"]}


def plain_config(w, world) -> dict:
    """The workload description both arms report (same config)."""
    return {"workload": "plain drop-in: 8 queries (100-1000 aa) vs 2M subjects / 0.7G residues, "
                        "one query per search",
            "db_subjects": w.n_subjects, "db_residues": w.total_residues,
            "queries": [len(q) for q in w.queries],
            "parallelism": f"weak x{world} (one database per rank)" if world > 1 else "single process",
            "l2": "inputs larger than L2 (0.7 GB database vs 129 MB L2), no flush"}


def run_reference(args, rank, world):
    """CPU implementation of the path on the host cores (oracle port)."""
    from blaze103 import synth

    if rank != 0:
        return
    threads = os.cpu_count() or 1
    w = synth.make_workload("plain-db-scale", scale=args.scale, seed=1)
    frac = args.ref_frac if args.ref_frac else args.cpu_frac
    for _ in range(args.warmup):
        cpu_sample_run(w, w.queries, frac, threads, w.total_residues * world, w.n_subjects * world)
    t_all = 0.0
    n_all = 0
    sample = None
    for _ in range(args.steps):
        rate, dt, n_res, n_subj, _ = cpu_sample_run(w, w.queries, frac, threads,
                                                    w.total_residues * world, w.n_subjects * world)
        t_all += dt
        n_all += n_res
        k = max(int(round(1 / frac)), 1)
        which = "all subjects" if k == 1 else f"every {k}th subject"
        sample = (f"8 queries x {which} of the "
                  f"{w.n_subjects}-subject database ({n_subj} subjects, "
                  f"{n_res // 8} residues) per step, the cpu_baseline sample")
    value = n_all / t_all
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_all / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic (seeded; 20 standard residues at Robinson-Robinson frequencies, "
                "log-normal lengths, 1% planted homologs)",
        "config": plain_config(w, world),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "NCBI blastp 2.13.0 (the reference's CPU path) is not installed on this machine; "
                "the oracle restatement of the same algorithm is timed instead",
    }
    print(json.dumps(line), flush=True)


# The batched records' workloads: name, seed and description.
BATCHED_WORKLOADS = {
    "batched": (2, "batched", "log-normal median 350, 50-2000 aa", "10% planted homologs"),
    "overflow-stress": (3, "extension and overflow stress", "2000-5000 aa",
                        "lengths log-normal (median 250) with the longest 0.1% at 15000-35000 aa, 20% with "
                        "low-complexity runs, 25% planted homologs at 30-60% identity"),
}


def batched_record(local, rank, world, scale: float, n_queries, warmup: int, passes: int,
                   check_subjects: int = 5000, workload: str = "batched") -> dict:
    """Batched form vs the plain path on the same queries and database, both
    timed with CUDA events on the search stream: the batched workload (512
    queries, lengths log-normal, median 350, clipped 50-2,000; 5M subjects at
    scale 1; 10% planted homologs) or the extension and overflow stress (64
    queries of 2,000-5,000 residues; 500,000 subjects up to 35,000 residues,
    low-complexity runs, 25% homologs at 30-60% identity). Also checked: the
    batched HSPs equal the plain path's for every query, and both equal the
    oracle's on every k-th subject (about check_subjects of them,
    whole-database statistics)."""
    import blaze103
    import oracle
    from blaze103 import synth

    seed0, label, qdesc, ddesc = BATCHED_WORKLOADS[workload]
    w = synth.make_workload(workload, scale=scale, n_queries=n_queries, seed=seed0 + 7919 * rank)
    db_total, db_n = w.total_residues * world, w.n_subjects * world
    db = blaze103.SeqSrc(w.residues, w.offsets, device=local)
    ps = blaze103.PrelimSearch(db)
    params = [blaze103.default_params(len(q), db_residues=db_total, db_subjects=db_n) for q in w.queries]
    batch = blaze103.QueryBatch(db, w.queries)
    singles = [blaze103.Query(db, q) for q in w.queries]
    R, nq = w.total_residues, len(w.queries)
    last = {}

    def batch_step():
        out = ps.run_batch(batch, params)
        st = ps.stats()
        last.update(st)
        return st["device_ms"], out

    for _ in range(warmup):
        batch_step()
    clocks = ClockSampler(local)
    clocks.start()
    b_ms, got_b = [], None
    for _ in range(passes):
        ms, got_b = batch_step()
        b_ms.append(ms)
    clk = clocks.stop()
    p_ms, plain_lists = 0.0, []
    for q, p in zip(singles, params):
        ps.run_query(q, p)
        p_ms += ps.stats()["device_ms"]
        plain_lists.append(ps.results())
    b_s, p_s = sum(b_ms) / len(b_ms) / 1e3, p_ms / 1e3

    # batched == plain, query by query, every field
    bounds = np.searchsorted(got_b["query"], np.arange(nq + 1))
    same = sum(int(not np.array_equal(got_b[bounds[i]:bounds[i + 1]][list(blaze103.HSP_DTYPE.names)]
                                      .astype(blaze103.HSP_DTYPE), plain_lists[i])) for i in range(nq))
    # both against the oracle on a subject sample
    k = max(w.n_subjects // max(check_subjects, 1), 1)
    idx, res, sub_off = subject_sample(w, k)
    ref_lists = []
    for q in w.queries:
        pd = oracle.default_params(len(q), db_total, db_n)
        hs, _ = oracle.search_db(q, res, sub_off, pd, threads=os.cpu_count() or 1)
        ref_lists.append(oracle.finish(hs, pd))
    par = parity_check(idx, ref_lists, plain_lists, k)
    par.update({"subjects_checked": int(len(idx)), "queries": nq, "sample": f"every {k}th subject",
                "queries_batched_differs_from_plain": same,
                "batched_hsps": int(len(got_b)), "plain_hsps": int(sum(len(x) for x in plain_lists))})
    rec = {
        "metric": "DB residues/s per query, batched form (aggregate over queries)",
        "value": nq * R / b_s, "unit": UNIT, "passes": passes, "warmup": warmup,
        "ms_per_pass": b_s * 1e3,
        "config": {"workload": f"{label}: {nq} queries ({qdesc}) vs "
                               f"{w.n_subjects} subjects / {R} residues, {ddesc}",
                   "db_subjects": w.n_subjects, "db_residues": R, "queries": nq, "database_scale": scale,
                   "longest_subject": int(np.diff(w.offsets.astype(np.int64)).max()),
                   "query_lengths": [min(len(q) for q in w.queries), max(len(q) for q in w.queries)]},
        "plain_same_workload": {"value": nq * R / p_s, "ms_per_pass": p_s * 1e3,
                                "form": "one search per query (scan + gapped launch sequence each)"},
        "batched_over_plain": p_s / b_s,
        "stages_ms_per_pass": {"scan": last["scan_ms"], "gapped": last["gapped_ms"]},
        "work_per_pass": {k_: last[k_] for k_ in ("word_hits", "ungapped_extensions", "init_hsps",
                                                  "gapped_extensions", "dp_cells", "hsps")},
        "dp_cells_per_s": last["dp_cells"] / (last["gapped_ms"] / 1e3) if last["gapped_ms"] else None,
        "parity": par,
        "clocks": clk,
    }
    for q in singles:
        q.close()
    batch.close()
    ps.close()
    db.close()
    return rec


def serve_record(local, rank, scale: float, rates, duration: float, max_queries: int, server_cfg: dict) -> dict:
    """Serving loop under Poisson arrivals (serving workload: query lengths
    log-normal, median 350, 30-5,000; 10M subjects at scale 1): for each
    offered rate, queries arrive at exponential gaps, are batched on the fly
    by the library's serving loop and completed; reports throughput and
    p50/p99 latency (submission to completion), beside the same arrivals
    served one query at a time."""
    import blaze103
    from blaze103 import synth

    w = synth.make_workload("serving", scale=scale, seed=4 + 7919 * rank)
    rng = np.random.default_rng(44 + rank)
    pool = [synth.random_residues(rng, int(L))
            for L in synth.lognormal_lengths(rng, 512, 350, 0.82, 30, 5000)]
    db = blaze103.SeqSrc(w.residues, w.offsets, device=local)
    R = w.total_residues

    def arrivals(rate):
        n = max(20, min(int(rate * duration), max_queries))
        return rng.exponential(1.0 / rate, n), rng.integers(0, len(pool), n)

    def serve(rate, arr, **cfg):
        srv = blaze103.Server(db, **cfg)
        gaps, picks = arr
        n = len(gaps)
        tickets = []
        due = time.perf_counter()
        for g, k in zip(gaps, picks):
            due += g
            d = due - time.perf_counter()
            if d > 0:
                time.sleep(d)
            tickets.append(srv.submit(pool[k]))
        for t in tickets:
            srv.wait(t)
        st = srv.stats()
        srv.close()
        return {"offered_qps": rate, "queries": n, "completed_qps": n / st["busy_s"],
                "residues_per_s": st["residues"] / st["busy_s"], "batches": st["batches"],
                "p50_ms": st["latency_p50_ms"], "p99_ms": st["latency_p99_ms"], "max_ms": st["latency_max_ms"]}

    serve(rates[0], arrivals(rates[0]), **server_cfg)  # warm-up: contexts, buffers
    clocks = ClockSampler(local)
    clocks.start()
    sweep = []
    for r in rates:
        arr = arrivals(r)  # both services see the same queries at the same times
        row = {"served": serve(r, arr, **server_cfg)}
        row["one_at_a_time"] = serve(r, arr, slots=1, max_batch=1, batch_window_us=0)
        sweep.append(row)
    clk = clocks.stop()
    db.close()
    top = sweep[-1]["served"]
    return {
        "metric": "DB residues/s per query, served under Poisson arrivals (aggregate); p50/p99 latency",
        "value": top["residues_per_s"], "unit": UNIT,
        "config": {"workload": f"serving: Poisson arrivals at {','.join(str(r) for r in rates)} q/s, query lengths "
                               f"log-normal (median 350, 30-5000) vs {w.n_subjects} subjects / {R} residues",
                   "db_subjects": w.n_subjects, "db_residues": R, "database_scale": scale, "server": server_cfg},
        "p50_ms": top["p50_ms"], "p99_ms": top["p99_ms"],
        "sweep": sweep,
        "clocks": clk,
    }


def _standalone(rec: dict, world: int, steps: int, warmup: int) -> dict:
    line = {"metric": rec["metric"], "value": rec["value"], "unit": UNIT, "n_gpus": world, "steps": steps,
            "warmup": warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int32", "data": "synthetic (seeded)"}
    line.update({k: v for k, v in rec.items() if k not in line})
    return line


def run_batched(args, rank, world, local):
    scale = args.scale if args.scale != 1.0 else 0.02
    rec = batched_record(local, rank, world, scale, args.queries, args.warmup, args.steps)
    if rank == 0:
        print(json.dumps(_standalone(rec, world, args.steps, args.warmup)), flush=True)


def server_config(args) -> dict:
    return dict(slots=args.slots, max_batch=args.max_batch, batch_window_us=args.window_us,
                memory_budget=args.memory_budget)


def run_serve(args, rank, world, local):
    scale = args.scale if args.scale != 1.0 else 0.01
    rates = [float(x) for x in args.rates.split(",")]
    rec = serve_record(local, rank, scale, rates, args.duration, args.max_queries, server_config(args))
    if rank == 0:
        print(json.dumps(_standalone(rec, world, len(rates), 1)), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="blaze", choices=["blaze", "reference"])
    ap.add_argument("--scale", type=float, default=1.0, help="database size relative to the default workload (2M subjects)")
    ap.add_argument("--cpu-frac", type=float, default=1.0,
                    help="cpu_baseline (and parity) sample: this fraction of the subjects (1: all)")
    ap.add_argument("--ref-frac", type=float, default=None,
                    help="reference arm sample fraction per step (default: the cpu_baseline fraction)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="plain line without its batched sub-record")
    ap.add_argument("--no-serve", action="store_true", help="plain line without its serving sub-record")
    ap.add_argument("--no-stress", action="store_true", help="plain line without its overflow-stress sub-record")
    ap.add_argument("--stress-scale", type=float, default=1.0,
                    help="overflow-stress sub-record: database size relative to 500,000 subjects")
    ap.add_argument("--batched-scale", type=float, default=1.0,
                    help="batched sub-record: database size relative to 5M subjects")
    ap.add_argument("--serve-scale", type=float, default=0.1,
                    help="serving sub-record: database size relative to 10M subjects")
    ap.add_argument("--serve-rates", default="20,100,400", help="serving sub-record: arrival rates, queries/s")
    ap.add_argument("--serve-small-scale", type=float, default=0.01,
                    help="second serving sub-record (serve_small): a database where one query leaves the GPU "
                         "mostly idle (0: none)")
    ap.add_argument("--serve-small-rates", default="100,2000", help="serve_small: arrival rates, queries/s")
    ap.add_argument("--mode", default="plain", choices=["plain", "batched", "serve"],
                    help="plain: the drop-in, one query per launch sequence (the headline line); "
                         "batched: many queries per launch against a 5M-subject-shaped database, scaled")
    ap.add_argument("--queries", type=int, default=512, help="batched mode: queries per batch")
    ap.add_argument("--rates", default="10,100,500,2000", help="serve mode: arrival rates, queries/s")
    ap.add_argument("--duration", type=float, default=2.0, help="serve mode: seconds of arrivals per rate")
    ap.add_argument("--max-queries", type=int, default=3000, help="serve mode: arrivals per rate at most")
    ap.add_argument("--slots", type=int, default=3, help="serve mode: batches in flight")
    ap.add_argument("--max-batch", type=int, default=64, help="serve mode: queries per batch at most")
    ap.add_argument("--window-us", type=int, default=1000, help="serve mode: batching window")
    ap.add_argument("--memory-budget", type=int, default=0, help="serve mode: device bytes (0: none)")
    args = ap.parse_args()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.mode == "batched":
        run_batched(args, rank, world, local)
        return
    if args.mode == "serve":
        run_serve(args, rank, world, local)
        return

    import blaze103
    from blaze103 import synth

    group = Group(world, local)
    w = synth.make_workload("plain-db-scale", scale=args.scale, seed=1 + 7919 * rank)
    db_total, db_n = w.total_residues * world, w.n_subjects * world  # E-values over the global DB
    db = blaze103.SeqSrc(w.residues, w.offsets, device=local)
    ps = blaze103.PrelimSearch(db)
    params = [blaze103.default_params(len(q), db_residues=db_total, db_subjects=db_n) for q in w.queries]
    queries = [blaze103.Query(db, q, p.word_threshold) for q, p in zip(w.queries, params)]
    R, N = w.total_residues, w.n_subjects

    def one_step(acc):
        for q, p in zip(queries, params):
            ps.run_query(q, p)
            st = ps.stats()
            for k in ("device_ms", "scan_ms", "gapped_ms"):
                acc[k] += st[k]
            for k in ("kernel_launches", "dp_cells", "hsps", "word_hits", "ungapped_extensions",
                      "gapped_extensions", "reruns"):
                acc[k] += st[k]

    def fresh():
        return {k: 0 for k in ("device_ms", "scan_ms", "gapped_ms", "kernel_launches", "dp_cells",
                               "hsps", "word_hits", "ungapped_extensions", "gapped_extensions",
                               "reruns")}

    for _ in range(args.warmup):
        one_step(fresh())
    acc = fresh()
    clocks = ClockSampler(local)
    group.barrier()
    clocks.start()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        one_step(acc)
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    group.barrier()
    dev_s = group.max(acc["device_ms"] / 1e3)
    wall_s = group.max(wall)
    units = args.steps * len(queries) * R * world
    value = units / dev_s

    # e2e: the one-call C ABI path with host query buffers
    cap = max(4 * acc["hsps"] // max(args.steps, 1) + 1024, 1 << 16)
    for _ in range(1):
        for q, p in zip(w.queries, params):
            ps.prelim_search(q, p, cap)
    h2d = d2h = 0
    e2e_out = [None] * len(w.queries)
    group.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for i, (q, p) in enumerate(zip(w.queries, params)):
            e2e_out[i] = ps.prelim_search(q, p, cap)
            st = ps.stats()
            h2d += st["h2d_bytes"]
            d2h += st["d2h_bytes"]
    e2e_s = group.max(time.perf_counter() - t0)
    group.barrier()
    e2e_value = units / e2e_s

    # traceback stage (after the timed region): every query's HSPs traced
    # again with the final X-drop, timed with CUDA events
    tb_ms, tb_hsps, tb_cells, tb_out = 0.0, 0, 0, 0
    for q, p in zip(w.queries, params):
        ps.run(q, p)
        tb_out += len(ps.traceback(q, p))
        st = ps.stats()
        tb_ms += st["traceback_ms"]
        tb_hsps += st["traceback_hsps"]
        tb_cells += st["traceback_cells"]

    # roofline of the scan kernel
    peak, peak_kind = measured_peak()
    scan_launches = args.steps * len(queries)
    scan_avg_s = acc["scan_ms"] / 1e3 / scan_launches
    alg_bytes = R * 1 + (N + 1) * 8
    achieved = alg_bytes / scan_avg_s / 1e9
    traffic = None
    prof = os.path.join(ROOT, "profiles", "scan_kernel_traffic.json")
    if os.path.exists(prof):
        try:
            with open(prof) as f:
                pj = json.load(f)
            # one capture on a smaller database, scaled by residues processed
            # (the scan's traffic is the residues plus per-subject offsets)
            cap_bytes = pj["dram_bytes_read"] + pj["dram_bytes_write"]
            traffic = cap_bytes * R / pj["captured_residues"]
        except (OSError, ValueError, KeyError, ZeroDivisionError):
            traffic = None

    # the scan's real bound: integer issue. Warp instructions per step from
    # the committed ncu count (scaled by residues), against the SMs' issue
    # rate (4 schedulers per SM, one warp instruction per cycle each, at the
    # maximum SM clock)
    issue = None
    iprof = os.path.join(ROOT, "profiles", "scan_kernel_issue.json")
    if os.path.exists(iprof):
        try:
            import torch

            with open(iprof) as f:
                ij = json.load(f)
            if [x["query_length"] for x in ij["per_query"]] == [len(q) for q in w.queries]:
                inst = ij["warp_inst_per_step"] * R / ij["captured_residues"]
                n_sm = torch.cuda.get_device_properties(local).multi_processor_count
                mhz = clk.get("sm_max_mhz") or 2070.0
                peak_rate = n_sm * 4 * mhz * 1e6
                rate = inst / (acc["scan_ms"] / 1e3 / args.steps)
                issue = {"kernel": "scan_kernel", "warp_inst_per_step": inst,
                         "warp_inst_per_residue": inst / (R * len(queries)),
                         "achieved_warp_inst_per_s": rate, "peak_warp_inst_per_s": peak_rate,
                         "frac": rate / peak_rate,
                         "source": "profiles/scan_kernel_issue.json (ncu sm__inst_executed.sum, scaled by residues)"}
        except (OSError, ValueError, KeyError, ImportError, RuntimeError):
            issue = None

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * dev_s / args.steps,
        "wall_ms_per_step": 1e3 * wall_s / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic (seeded; 20 standard residues at Robinson-Robinson frequencies, "
                "log-normal lengths, 1% planted homologs)",
        "config": plain_config(w, world),
        "placement": "database and query tables resident in HBM; one scan + gapped launch sequence per query",
        "e2e": {"value": e2e_value, "unit": UNIT,
                "h2d_bytes_per_step": h2d // args.steps, "d2h_bytes_per_step": d2h // args.steps,
                "path": "blaze_prelim_search with host query and result buffers"},
        "gpu_launches": int(acc["kernel_launches"]),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_kind": f"{peak_kind} hbm_gbs",
                     "kernel": "scan_kernel", "alg_bytes_per_launch": alg_bytes,
                     "avg_launch_ms": scan_avg_s * 1e3},
        "issue_roofline": issue,
        "stages_ms_per_step": {"scan": acc["scan_ms"] / args.steps,
                               "gapped": acc["gapped_ms"] / args.steps},
        "dp_cells_per_s": acc["dp_cells"] / (acc["gapped_ms"] / 1e3) if acc["gapped_ms"] else None,
        "counts_per_step": {k: acc[k] // args.steps for k in ("hsps", "word_hits", "ungapped_extensions",
                                                               "gapped_extensions", "dp_cells", "reruns")},
        "traceback": {"ms_per_step": tb_ms, "hsps_traced": tb_hsps, "aligned_hsps": tb_out,
                      "dp_cells": tb_cells, "dp_cells_per_s": tb_cells / (tb_ms / 1e3) if tb_ms else None,
                      "final_xdrop": 64, "timed": "separately, after the timed steps"},
        "clocks": clk,
    }
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        rate, dt, n_res, n_subj, sample = cpu_sample_run(w, w.queries, args.cpu_frac, threads, db_total, db_n,
                                                         keep=True)
        k = max(int(round(1.0 / args.cpu_frac)), 1)
        which = "all subjects" if k == 1 else f"every {k}th subject"
        line["cpu_baseline"] = {
            "value": rate, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"8 queries x {which} "
                      f"({n_subj} subjects, {n_res // 8} residues), {dt:.1f} s",
        }
        # the oracle's HSPs of that sample against the e2e path's, same OIDs
        par = parity_check(sample[0], sample[1], e2e_out, k)
        par.update({"subjects_checked": n_subj, "queries": len(w.queries),
                    "sample": f"{which}, whole-database statistics",
                    "path": "e2e (blaze_prelim_search)", "oracle": "oracle/blaze_oracle.c"})
        line["parity"] = par
    for q in queries:
        q.close()
    ps.close()
    db.close()
    # sub-records (N=1 only): the batched form and the serving loop
    if world == 1 and not args.no_batched:
        line["batched"] = batched_record(local, rank, world, args.batched_scale, args.queries, 1, 1)
    if world == 1 and not args.no_stress:
        line["stress"] = batched_record(local, rank, world, args.stress_scale, None, 1, 1,
                                        workload="overflow-stress")
    if world == 1 and not args.no_serve:
        rates = [float(x) for x in args.serve_rates.split(",")]
        line["serve"] = serve_record(local, rank, args.serve_scale, rates, args.duration, args.max_queries,
                                     server_config(args))
        if args.serve_small_scale > 0:
            rates = [float(x) for x in args.serve_small_rates.split(",")]
            line["serve_small"] = serve_record(local, rank, args.serve_small_scale, rates, args.duration,
                                               args.max_queries, server_config(args))
    if rank == 0:
        print(json.dumps(line), flush=True)
    group.close()


if __name__ == "__main__":
    main()
