"""GPU tests of the serving loop (blaze_server_*): a query's HSP lists must be
the same whether it runs alone through the plain path or arrives among other
queries and is batched with them, whatever the number of batches in flight,
the batch size or the memory budget; two of them are checked against the
oracle as well."""
import threading
import time

import numpy as np
import pytest

import blaze103
from blaze103 import synth

from _parity import concat, oracle_run, params_for

pytestmark = pytest.mark.gpu

EVALUE = 10.0


def _workload(seed=31, n_subjects=2500, n_queries=24):
    rng = np.random.default_rng(seed)
    lengths = [int(x) for x in rng.integers(20, 1200, n_queries)] + [3, 9000]
    qs = [synth.random_residues(rng, L) for L in lengths]
    seqs = [synth.random_residues(rng, int(L)) for L in synth.lognormal_lengths(rng, n_subjects, 250, 0.82, 30, 4000)]
    for i in range(0, len(seqs), 5):
        q = qs[i % len(qs)]
        w = min(len(q), int(rng.integers(30, 300)))
        s0 = int(rng.integers(0, len(q) - w + 1))
        seqs[i] = np.concatenate([seqs[i], synth.mutate(rng, q[s0:s0 + w], 0.45)])
    res, off = concat(seqs)
    return qs, res, off


@pytest.fixture(scope="module")
def served():
    qs, res, off = _workload()
    db = blaze103.SeqSrc(res, off)
    ps = blaze103.PrelimSearch(db)
    alone = [ps.run(q, blaze103.default_params(len(q), db, EVALUE)).hsps for q in qs]
    ps.close()
    yield qs, res, off, db, alone
    db.close()


def _serve(db, qs, submitters=3, **cfg):
    srv = blaze103.Server(db, **cfg)
    tickets = [None] * len(qs)

    def submit(idx):
        for i in idx:
            tickets[i] = srv.submit(qs[i])

    threads = [threading.Thread(target=submit, args=(range(k, len(qs), submitters),)) for k in range(submitters)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    got = [srv.wait(t, timeout_ms=600_000) for t in tickets]
    st = srv.stats()
    srv.close()
    return got, st


@pytest.mark.parametrize("cfg", [dict(slots=1, max_batch=1), dict(slots=2, max_batch=8),
                                 dict(slots=3, max_batch=64, batch_window_us=5000),
                                 dict(slots=4, max_batch=16, memory_budget=8 << 20)])
def test_results_identical_alone_and_in_the_mix(served, cfg):
    qs, _, _, db, alone = served
    got, st = _serve(db, qs, **cfg)
    for i, (g, a) in enumerate(zip(got, alone)):
        for f in blaze103.HSP_DTYPE.names:
            assert np.array_equal(g[f], a[f]), (i, f)
    assert st["completed"] == st["submitted"] == len(qs)
    assert st["residues"] == len(qs) * db.tot_len
    assert 0 < st["latency_p50_ms"] <= st["latency_p99_ms"] <= st["latency_max_ms"]
    if cfg["max_batch"] == 1:
        assert st["batches"] == len(qs)
    assert sum(len(a) for a in alone) > 100


def test_served_results_match_oracle(served):
    qs, res, off, db, _ = served
    got, _ = _serve(db, qs[:6], slots=2, max_batch=4)
    for i in (1, 4):
        _, pd = params_for(len(qs[i]), int(off[-1]), len(off) - 1)
        ref, _ = oracle_run(qs[i], res, off, pd)
        assert np.array_equal(got[i]["oid"], ref["subject"])
        for f in ("score", "q_start", "q_end", "s_start", "s_end"):
            assert np.array_equal(got[i][f], ref[f]), f


def test_server_rejects_bad_input(served):
    qs, _, _, db, _ = served
    srv = blaze103.Server(db, slots=1)
    with pytest.raises(ValueError):
        srv.submit(np.array([1, 0, 3], dtype=np.uint8))
    with pytest.raises(blaze103.BlazeError) as e:
        srv.wait(12345)
    assert e.value.status == 1
    t = srv.submit(qs[0])
    assert len(srv.wait(t)) >= 0
    with pytest.raises(blaze103.BlazeError):  # a ticket is released once taken
        srv.wait(t)
    srv.close()
    with pytest.raises(blaze103.BlazeError) as e:  # more worker threads than the library runs
        blaze103.Server(db, slots=65)
    assert e.value.status == 6  # BLAZE_ERR_LIMIT


def test_concurrent_search_contexts(served):
    # several host threads, each with its own search context, running queries
    # whose launches need different amounts of shared memory at the same time
    qs, _, _, db, alone = served
    errors = []

    def work(order):
        ps = blaze103.PrelimSearch(db)
        try:
            for _ in range(3):
                for i in order:
                    got = ps.run(qs[i], blaze103.default_params(len(qs[i]), db, EVALUE)).hsps
                    if not np.array_equal(got, alone[i]):
                        errors.append(i)
        except Exception as e:  # noqa: BLE001 - reported below
            errors.append(repr(e))
        finally:
            ps.close()

    rng = np.random.default_rng(0)
    threads = [threading.Thread(target=work, args=(rng.permutation(len(qs)),)) for _ in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert errors == []


@pytest.mark.parametrize("seed", range(7000, 7012))
def test_random_server_settings(seed):
    # random slots, batch cap, memory budget (down to 1 byte: one query at a
    # time next to a running batch), batching window, launch mode and tile
    # size; queries from three threads with random gaps; each result equals
    # the query's plain run
    rng = np.random.default_rng(seed)
    seqs = [synth.random_residues(rng, int(L))
            for L in synth.lognormal_lengths(rng, int(rng.choice([50, 500])), 250, 0.9, 1, 4000)]
    qs = [synth.random_residues(rng, int(rng.integers(1, 3000))) for _ in range(int(rng.integers(1, 40)))]
    for i in range(0, len(seqs), 5):
        q = qs[int(rng.integers(0, len(qs)))]
        if len(q) > 30:
            w = min(len(q), int(rng.integers(30, 300)))
            s0 = int(rng.integers(0, len(q) - w + 1))
            seqs[i] = np.concatenate([seqs[i], synth.mutate(rng, q[s0:s0 + w], 0.5)])
    res, off = concat(seqs)
    db = blaze103.SeqSrc(res, off)
    ps = blaze103.PrelimSearch(db, autotune=False)
    want = [ps.run(q).hsps for q in qs]
    ps.close()
    srv = blaze103.Server(db, slots=int(rng.integers(1, 5)), max_batch=int(rng.choice([1, 2, 7, 64])),
                          memory_budget=int(rng.choice([0, 1, 1 << 20, 64 << 20])),
                          batch_window_us=int(rng.choice([0, 100, 2000])),
                          tuning=dict(launch_mode=int(rng.integers(0, 3)), tile_residues=int(rng.choice([0, 1, 4096]))))
    tickets = [None] * len(qs)
    gaps = rng.exponential(0.0005, len(qs))

    def submit(idx):
        for i in idx:
            time.sleep(float(gaps[i]))
            tickets[i] = srv.submit(qs[i])

    threads = [threading.Thread(target=submit, args=(list(range(k, len(qs), 3)),)) for k in range(3)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    for i, tk in enumerate(tickets):
        got = srv.wait(tk, 60000)
        for f in blaze103.HSP_DTYPE.names:
            assert np.array_equal(got[f], want[i][f]), (i, f)
    srv.close()
    db.close()
