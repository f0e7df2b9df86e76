"""CPU tests of bench.py's contract: the reference arm prints one well-formed
JSON line from the host cores, and the product arm fails loudly (no number)
where no GPU is usable instead of falling back to the CPU."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SMALL = ["--scale", "0.001", "--steps", "1", "--warmup", "1"]


def _bench(args):
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], capture_output=True, text=True,
                          timeout=600, cwd=ROOT)


def test_reference_arm_prints_the_contract_line():
    r = _bench(["--impl", "reference", *SMALL])
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["value"] > 0 and line["higher_is_better"] is True
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}


def test_product_arm_fails_loudly_without_a_gpu():
    import blaze103

    if blaze103.device_count() > 0:
        pytest.skip("a GPU is present: the product arm runs")
    r = _bench(SMALL)
    assert r.returncode != 0
    assert not [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert "no usable CUDA device" in r.stderr


def test_reference_arm_under_torchrun_prints_once():
    # two ranks on the host: rank 0 times and prints, the other exits 0 without work
    import socket

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
                        "--impl", "reference", "--gpus", "2", *SMALL],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(l) for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1 and lines[0]["impl"] == "reference" and lines[0]["n_gpus"] == 2


def _bench_module():
    import importlib.util

    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_parity_check_counts_every_differing_record():
    # the oracle's own HSPs stand in for the GPU's; a planted change in the
    # oracle side must show up as mismatches
    import numpy as np

    import blaze103
    import oracle
    from blaze103 import synth

    bench = _bench_module()
    w = synth.make_workload("plain-small", scale=0.1)
    q = w.queries[0]
    pd = oracle.default_params(len(q), w.total_residues, w.n_subjects)
    whole, _ = oracle.search_db(q, w.residues, w.offsets, pd, threads=2)
    whole = oracle.finish(whole, pd)
    got = np.zeros(len(whole), dtype=blaze103.HSP_DTYPE)
    for gf, rf in bench.PARITY_FIELDS:
        got[gf] = whole[rf]
    got["evalue"] = whole["evalue"]
    k = 3
    idx, res, off = bench.subject_sample(w, k)
    assert np.array_equal(off[1:] - off[:-1], (w.offsets[idx + 1] - w.offsets[idx]))
    hs, _ = oracle.search_db(q, res, off, pd, threads=2)
    ref = oracle.finish(hs, pd)
    assert len(ref) >= 10
    par = bench.parity_check(idx, [ref], [got], k)
    assert par["mismatches"] == 0 and par["hsps"] == len(ref)
    bad = ref.copy()
    bad["score"][0] += 1
    assert bench.parity_check(idx, [bad], [got], k)["mismatches"] == 1
    assert bench.parity_check(idx, [ref[1:]], [got], k)["mismatches"] == 1
    ev = ref.copy()
    ev["evalue"][2] *= 1.0 + 1e-9
    p2 = bench.parity_check(idx, [ev], [got], k)
    assert p2["mismatches"] == 1 and p2["evalue_mismatches"] == 1


def test_both_arms_report_the_same_config():
    r = _bench(["--impl", "reference", *SMALL])
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads([l for l in r.stdout.splitlines() if l.startswith("{")][0])
    from blaze103 import synth

    bench = _bench_module()
    w = synth.make_workload("plain-db-scale", scale=0.001, seed=1)
    assert line["config"] == bench.plain_config(w, 1)
    assert "all subjects" in line["cpu_baseline"]["sample"]  # the cpu_baseline sample: the whole database
