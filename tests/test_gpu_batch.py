"""GPU tests of the batched form: many queries in one launch per stage must
give, query by query, exactly the HSP lists of the plain one-query path (and
of the oracle), whatever the tile size, staging size and block shape."""
import numpy as np
import pytest

import blaze103
from blaze103 import synth

from _parity import concat, oracle_run, params_for

pytestmark = pytest.mark.gpu


def _db(seed=21, n=3000, with_homologs_of=None):
    rng = np.random.default_rng(seed)
    seqs = [synth.random_residues(rng, int(L)) for L in synth.lognormal_lengths(rng, n, 250, 0.82, 30, 5000)]
    for i in range(0, len(seqs), 7):
        if with_homologs_of:
            q = with_homologs_of[i % len(with_homologs_of)]
            w = min(len(q), int(rng.integers(40, 300)))
            s0 = int(rng.integers(0, len(q) - w + 1))
            seqs[i] = np.concatenate([seqs[i], synth.mutate(rng, q[s0:s0 + w], 0.45)])
    seqs.sort(key=len)
    return concat(seqs)


def _queries(seed=22, lengths=(5, 50, 120, 300, 333, 700, 1000, 1500, 2600, 9000)):
    rng = np.random.default_rng(seed)
    return [synth.random_residues(rng, L) for L in lengths]


def _plain(ps, db, q, p):
    qq = blaze103.Query(db, q)
    try:
        ps.run_query(qq, p)
        return ps.results()
    finally:
        qq.close()


def _check_batch_equals_plain(tuning=None, qs=None, **override):
    qs = qs or _queries()
    res, off = _db(with_homologs_of=qs)
    db = blaze103.SeqSrc(res, off)
    ps = blaze103.PrelimSearch(db)
    params = [params_for(len(q), db.tot_len, db.num_seqs, **override)[0] for q in qs]
    want = [_plain(ps, db, q, p) for q, p in zip(qs, params)]
    if tuning:
        ps.set_tuning(**tuning)
    batch = blaze103.QueryBatch(db, qs)
    got = ps.run_batch(batch, params)
    assert np.all(np.diff(got["query"].astype(np.int64)) >= 0)
    total = 0
    for i, w in enumerate(want):
        g = got[got["query"] == i]
        for f in blaze103.HSP_DTYPE.names:
            assert np.array_equal(g[f], w[f]), (i, f)
        total += len(w)
    assert total == len(got) and total > 50
    batch.close()
    ps.close()
    db.close()
    return qs, res, off, params, got


def test_batch_equals_plain_per_query():
    qs, res, off, params, got = _check_batch_equals_plain()
    # and two of the queries against the oracle directly
    for i in (3, 6):
        pd = params_for(len(qs[i]), int(off[-1]), len(off) - 1)[1]
        ref, _ = oracle_run(qs[i], res, off, pd)
        g = got[got["query"] == i]
        assert np.array_equal(g["oid"], ref["subject"])
        for f in ("score", "q_start", "q_end", "s_start", "s_end"):
            assert np.array_equal(g[f], ref[f]), f


@pytest.mark.parametrize("tuning", [dict(batch_launch=2), dict(batch_launch=1, tile_residues=64),
                                    dict(batch_launch=2, launch_mode=1, stage_bytes=256),
                                    dict(tile_residues=1), dict(tile_residues=1 << 24),
                                    dict(stage_bytes=512, max_warps_per_block=3),
                                    dict(stage_bytes=8192, tile_residues=3000)])
def test_batch_tuning_does_not_change_results(tuning):
    _check_batch_equals_plain(tuning)


def test_batch_capacity_regrowth(monkeypatch):
    monkeypatch.setenv("BLAZE_INITIAL_SCRATCH_CAP", "2")
    monkeypatch.setenv("BLAZE_INITIAL_INIT_CAP", "5")
    monkeypatch.setenv("BLAZE_INITIAL_OUT_CAP", "5")
    monkeypatch.setenv("BLAZE_INITIAL_WORK_CAP", "3")
    _check_batch_equals_plain()


# Batches of at least 16 queries run the gapped stage with one lane per DP
# (prep, DP and finishing kernels); these batches must give the plain path's
# lists too, including DPs whose band outgrows the lane's 64-column ring or
# whose gap costs the packed ring cells cannot hold (rerun warp-parallel).
def _queries20(seed=23):
    rng = np.random.default_rng(seed)
    lengths = (5, 50, 120, 300, 333, 700, 1000, 1500, 2600, 9000,
               64, 90, 150, 210, 260, 410, 520, 640, 880, 1200)
    return [synth.random_residues(rng, L) for L in lengths]


@pytest.mark.parametrize("tuning", [None, dict(launch_mode=1), dict(launch_mode=2, batch_launch=1),
                                    dict(batch_launch=2)])
def test_lane_dp_batch_equals_plain(tuning):
    _check_batch_equals_plain(tuning, qs=_queries20())


def test_lane_dp_capacity_regrowth(monkeypatch):
    monkeypatch.setenv("BLAZE_INITIAL_SCRATCH_CAP", "2")
    monkeypatch.setenv("BLAZE_INITIAL_INIT_CAP", "5")
    monkeypatch.setenv("BLAZE_INITIAL_OUT_CAP", "5")
    monkeypatch.setenv("BLAZE_INITIAL_WORK_CAP", "3")
    _check_batch_equals_plain(qs=_queries20())


@pytest.mark.parametrize("override", [dict(gapped_xdrop=100), dict(gap_open=40), dict(gap_open=0, gap_extend=2)])
def test_lane_dp_fallbacks_and_gap_costs(override):
    _check_batch_equals_plain(qs=_queries20(), **override)


def test_batch_rejects_mixed_search_settings():
    qs = _queries(lengths=(100, 200))
    res, off = _db(n=200)
    db = blaze103.SeqSrc(res, off)
    ps = blaze103.PrelimSearch(db)
    p = [params_for(len(q), db.tot_len, db.num_seqs)[0] for q in qs]
    p[1].window = 30
    batch = blaze103.QueryBatch(db, qs)
    with pytest.raises(blaze103.BlazeError) as e:
        ps.run_batch(batch, p)
    assert e.value.status == 1
    batch.close()
    ps.close()
    db.close()


def test_graph_replay_matches_direct_launches():
    qs = _queries(lengths=(40, 300, 700, 1200))
    res, off = _db(n=1500, with_homologs_of=qs)
    db = blaze103.SeqSrc(res, off)
    ps = blaze103.PrelimSearch(db)
    params = [params_for(len(q), db.tot_len, db.num_seqs)[0] for q in qs]
    ps.set_tuning(launch_mode=1)
    batch = blaze103.QueryBatch(db, qs)
    direct = ps.run_batch(batch, params)
    assert ps.stats()["graph_builds"] == 0 and ps.stats()["graph_replays"] == 0
    ps.set_tuning(launch_mode=0)  # batched runs go through the graph
    first = ps.run_batch(batch, params)
    assert ps.stats()["graph_builds"] == 1
    again = ps.run_batch(batch, params)
    assert ps.stats()["graph_replays"] == 1 and ps.stats()["graph_builds"] == 0
    assert np.array_equal(first, direct) and np.array_equal(again, direct)
    # a different batch changes the arguments: the graph is updated, not reused
    sub = blaze103.QueryBatch(db, qs[1:3])
    got = ps.run_batch(sub, params[1:3])
    assert ps.stats()["graph_builds"] >= 1
    for i in range(2):
        w = direct[direct["query"] == i + 1]
        g = got[got["query"] == i]
        for f in blaze103.HSP_DTYPE.names:
            assert np.array_equal(g[f], w[f]), f
    # single queries through the graph as well
    ps.set_tuning(launch_mode=2)
    one = ps.run(qs[2], params[2]).hsps
    ps.set_tuning(launch_mode=1)
    assert np.array_equal(one, ps.run(qs[2], params[2]).hsps)
    with pytest.raises(blaze103.BlazeError):
        ps.set_tuning(launch_mode=3)
    sub.close()
    batch.close()
    ps.close()
    db.close()


def test_batch_culling_per_query():
    # hitlist_size, max_hsps and the preliminary reap differ per query; each
    # query's records equal its plain run with the same parameters, and the
    # plain run equals the oracle's reap and culling
    qs = _queries()
    res, off = _db(with_homologs_of=qs)
    db = blaze103.SeqSrc(res, off)
    ps = blaze103.PrelimSearch(db)
    settings = [dict(hitlist_size=3), dict(max_hsps=1), dict(prelim_evalue=1e-3), {},
                dict(hitlist_size=5, max_hsps=2, prelim_evalue=0.5), dict(hitlist_size=1),
                dict(hitlist_size=100000), dict(prelim_evalue=1e-30), dict(max_hsps=3), dict(hitlist_size=2)]
    params = [params_for(len(q), db.tot_len, db.num_seqs, **k)[0] for q, k in zip(qs, settings)]
    want = [_plain(ps, db, q, p) for q, p in zip(qs, params)]
    batch = blaze103.QueryBatch(db, qs)
    got = ps.run_batch(batch, params)
    for i, w in enumerate(want):
        g = got[got["query"] == i]
        for f in blaze103.HSP_DTYPE.names:
            assert np.array_equal(g[f], w[f]), (i, f)
    for i in (0, 4):
        pd = params_for(len(qs[i]), int(off[-1]), len(off) - 1, **settings[i])[1]
        ref, _ = oracle_run(qs[i], res, off, pd)
        assert np.array_equal(want[i]["oid"], ref["subject"])
        assert np.array_equal(want[i]["score"], ref["score"])
    assert len(np.unique(got[got["query"] == 0]["oid"])) <= 3
    batch.close()
    ps.close()
    db.close()


def test_config2_batched_against_oracle_on_a_subject_sample():
    # the batched workload's 512 queries (log-normal, median 350, 50-2,000)
    # against a 5% slice of its 5M-subject database (10% planted homologs):
    # every query's batched HSPs on every 50th subject equal the oracle's,
    # under the statistics of the whole slice
    import os

    import oracle

    w = synth.make_workload("batched", scale=0.05)
    assert len(w.queries) == 512
    db = blaze103.SeqSrc(w.residues, w.offsets)
    ps = blaze103.PrelimSearch(db)
    params = [params_for(len(q), db.tot_len, db.num_seqs)[0] for q in w.queries]
    batch = blaze103.QueryBatch(db, w.queries)
    got = ps.run_batch(batch, params)
    k = 50
    idx = np.arange(0, w.n_subjects, k)
    sres = np.concatenate([w.residues[int(w.offsets[i]):int(w.offsets[i + 1])] for i in idx])
    soff = np.zeros(len(idx) + 1, dtype=np.uint64)
    np.cumsum((w.offsets[idx + 1] - w.offsets[idx]).astype(np.int64), out=soff[1:])
    bounds = np.searchsorted(got["query"], np.arange(len(w.queries) + 1))
    checked = 0
    for i, q in enumerate(w.queries):
        pd = params_for(len(q), db.tot_len, db.num_seqs)[1]
        hs, _ = oracle.search_db(q, sres, soff, pd, threads=os.cpu_count() or 1)
        ref = oracle.finish(hs, pd)
        g = got[bounds[i]:bounds[i + 1]]
        g = g[(g["oid"] % k) == 0]
        assert np.array_equal(g["oid"], idx[ref["subject"]].astype(np.uint32)), i
        for f in ("score", "q_start", "q_end", "s_start", "s_end"):
            assert np.array_equal(g[f], ref[f]), (i, f)
        assert np.array_equal(g["q_gapped_start"], ref["q_gstart"]), i
        assert np.array_equal(g["s_gapped_start"], ref["s_gstart"]), i
        assert np.allclose(g["evalue"], ref["evalue"], rtol=1e-12, atol=0.0), i
        checked += len(ref)
    assert checked > 500
    batch.close()
    ps.close()
    db.close()
