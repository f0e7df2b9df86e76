"""GPU parity: libblaze103 (through its C ABI, on cuda:0) against the oracle,
bit for bit on HSP offsets and scores, init hits included; E-values within a
relative 1e-12 (double arithmetic of identical integer scores)."""
import os

import numpy as np
import pytest

import blaze103
from blaze103 import synth

from _parity import compare, concat, params_for

pytestmark = pytest.mark.gpu


def test_config0_full_size():
    # the plain small workload at its stated size: 1 query of 300 residues,
    # 20,000 subjects (~7M residues), 1% planted homologs
    w = synth.make_workload("plain-small", scale=1.0)
    assert w.n_subjects == 20_000
    got, ref, stats = compare(w.queries[0], w.residues, w.offsets)
    assert len(got) > 100 and stats["dp_cells"] > 0
    assert np.isin(w.planted, got["oid"]).mean() > 0.9


def test_config1_queries_on_a_database_slice():
    # the eight database-scale queries (100-1,000 residues) against a 2%
    # slice of that database's shape (40,000 subjects)
    w = synth.make_workload("plain-db-scale", scale=0.02)
    for q in w.queries:
        compare(q, w.residues, w.offsets)


def test_config3_slice_long_queries_long_and_low_complexity_subjects():
    # the overflow-stress workload's own queries (2,000-5,000 residues)
    # against a slice with its longest subjects (up to 35,000 residues) and
    # its low-complexity runs: 3-letter stretches in 20% of subjects
    # (a 20% database's 2,000 longest subjects plus 3,000 others, and three
    # subjects at the workload's length bound -- 20,000, 30,000 and 35,000
    # residues -- each with homologs of the queries and low-complexity runs)
    w = synth.make_workload("overflow-stress", scale=0.2, n_queries=3)
    rng = np.random.default_rng(33)
    pick = np.concatenate([np.arange(w.n_subjects - 2000, w.n_subjects),
                           rng.choice(w.n_subjects - 2000, size=3000, replace=False)])
    pick.sort()
    seqs = [w.residues[int(w.offsets[i]):int(w.offsets[i + 1])] for i in pick]
    alpha = np.array([1, 11, 17], dtype=np.uint8)
    for L in (20_000, 30_000, 35_000):
        s = synth.random_residues(rng, L)
        for k, q in enumerate(w.queries):
            hom = synth.mutate(rng, q[100 * k:100 * k + 600], 0.45)
            p = int(rng.integers(0, L - len(hom)))
            s[p:p + len(hom)] = hom
        for _ in range(6):
            p = int(rng.integers(0, L - 200))
            s[p:p + 150] = alpha[rng.integers(0, 3, 150)]
        seqs.append(s)
    res, off = concat(seqs)
    assert int(np.diff(off.astype(np.int64)).max()) == 35_000 and min(len(q) for q in w.queries) >= 2000
    runs = 0
    for q in w.queries:
        got, _, stats = compare(q, res, off)
        assert len(got) > 0
        runs += stats["ungapped_extensions"]
    assert runs > 10_000


@pytest.mark.parametrize("qlen", [3, 11, 64, 100, 300, 1000, 2500])
def test_query_lengths(qlen):
    rng = np.random.default_rng(qlen)
    q = synth.random_residues(rng, qlen)
    seqs = [synth.random_residues(rng, int(L)) for L in synth.lognormal_lengths(rng, 1500, 250, 0.82, 30, 3000)]
    for i in range(0, len(seqs), 10):  # 10% homologs
        w = min(len(q), int(rng.integers(30, 300)))
        s0 = int(rng.integers(0, len(q) - w + 1))
        hom = synth.mutate(rng, q[s0:s0 + w], 0.45)
        pos = int(rng.integers(0, len(seqs[i]) + 1))
        seqs[i] = np.concatenate([seqs[i][:pos], hom, seqs[i][pos:]])
    res, off = concat(seqs)
    compare(q, res, off)


def test_edge_subjects():
    rng = np.random.default_rng(5)
    q = synth.random_residues(rng, 150)
    seqs = [q[:0], q[:1], q[:2], q[:3], q[:4], q.copy(), q[::-1].copy(), q[50:53].copy(),
            np.concatenate([q, q]), synth.random_residues(rng, 3000)]
    res, off = concat(seqs)
    got, _, _ = compare(q, res, off)
    assert 5 in set(got["oid"].tolist())  # the identical subject


def test_tiny_queries():
    rng = np.random.default_rng(6)
    seqs = [synth.random_residues(rng, 200) for _ in range(50)]
    res, off = concat(seqs)
    for L in (1, 2, 3, 4):
        compare(seqs[3][10:10 + L], res, off)


def test_unsorted_database_keeps_oids():
    w = synth.make_workload("plain-small", scale=0.05)
    n = w.n_subjects
    perm = np.random.default_rng(9).permutation(n)
    seqs = [w.residues[int(w.offsets[i]):int(w.offsets[i + 1])] for i in perm]
    res, off = concat(seqs)
    got, ref, _ = compare(w.queries[0], res, off)
    assert len(got) > 0


def test_low_complexity_seed_storm():
    rng = np.random.default_rng(11)
    alpha = np.array([1, 11, 17], dtype=np.uint8)  # A, L, S
    q = np.concatenate([alpha[rng.integers(0, 3, 400)], synth.random_residues(rng, 200)])
    seqs = []
    for i in range(300):
        s = synth.random_residues(rng, int(rng.integers(100, 1500)))
        if i % 2 == 0:
            run = alpha[rng.integers(0, 3, int(rng.integers(50, 400)))]
            p = int(rng.integers(0, len(s)))
            s = np.concatenate([s[:p], run, s[p:]])
        seqs.append(s)
    res, off = concat(seqs)
    got, _, stats = compare(q, res, off)
    assert stats["ungapped_extensions"] > 1000


def test_capacity_regrowth(monkeypatch):
    # tiny starting buffers force every grow-and-repeat path
    monkeypatch.setenv("BLAZE_INITIAL_SCRATCH_CAP", "2")
    monkeypatch.setenv("BLAZE_INITIAL_INIT_CAP", "3")
    monkeypatch.setenv("BLAZE_INITIAL_OUT_CAP", "3")
    w = synth.make_workload("plain-small", scale=0.05)
    got, _, stats = compare(w.queries[0], w.residues, w.offsets)
    assert stats["reruns"] >= 1 and len(got) > 3


def test_long_subjects_and_queries():
    w = synth.make_workload("overflow-stress", scale=0.001, n_queries=2)
    for q in w.queries:
        compare(q, w.residues, w.offsets)


def test_one_call_host_buffers_and_small_output():
    w = synth.make_workload("plain-small", scale=0.05)
    q = w.queries[0]
    db = blaze103.SeqSrc(w.residues, w.offsets)
    ps = blaze103.PrelimSearch(db)
    p, _ = params_for(len(q), w.total_residues, w.n_subjects)
    full = ps.run(q, p).hsps
    one = ps.prelim_search(q, p, capacity=len(full) + 10)
    assert np.array_equal(full, one)
    if len(full) > 1:
        with pytest.raises(blaze103.BlazeError) as e:
            ps.prelim_search(q, p, capacity=len(full) - 1)
        assert e.value.status == 5  # BLAZE_ERR_OUTPUT_TOO_SMALL
    again = ps.run(q, p).hsps
    assert np.array_equal(full, again)
    ps.close()
    db.close()


def test_one_call_reuses_its_tables_across_query_lengths():
    # the one-call entry point keeps its query tables between calls: longer,
    # shorter and degenerate queries in turn must each equal the regular path
    rng = np.random.default_rng(4242)
    seqs = [synth.random_residues(rng, int(L)) for L in synth.lognormal_lengths(rng, 800, 250, 0.82, 30, 3000)]
    qs = [synth.random_residues(rng, L) for L in (700, 5, 1200, 300, 3, 9000, 50, 1)]
    for i in range(0, len(seqs), 4):
        q = qs[i % len(qs)]
        if len(q) > 40:
            s0 = int(rng.integers(0, len(q) - 40))
            seqs[i] = np.concatenate([seqs[i], synth.mutate(rng, q[s0:s0 + 40], 0.6)])
    res, off = concat(seqs)
    db = blaze103.SeqSrc(res, off)
    ps = blaze103.PrelimSearch(db)
    for q in qs + qs[::-1]:
        p, _ = params_for(len(q), db.tot_len, db.num_seqs)
        one = ps.prelim_search(q, p, capacity=1 << 16)
        assert np.array_equal(ps.run(q, p).hsps, one)
    ps.close()
    db.close()


def test_invalid_inputs_rejected():
    w = synth.make_workload("plain-small", scale=0.01)
    db = blaze103.SeqSrc(w.residues, w.offsets)
    bad = np.array([1, 2, 0, 4], dtype=np.uint8)
    with pytest.raises(ValueError):
        blaze103.Query(db, bad)
    ps = blaze103.PrelimSearch(db)
    p, _ = params_for(10, w.total_residues, w.n_subjects)
    p.gap_extend = 0
    with pytest.raises(blaze103.BlazeError) as e:
        ps.run(w.queries[0][:10], p)
    assert e.value.status == 1
    ps.close()
    db.close()


def test_query_longer_than_shared_copy():
    # queries above 8192 residues are read from global memory by the word finder
    rng = np.random.default_rng(9000)
    q = synth.random_residues(rng, 9000)
    seqs = [synth.random_residues(rng, int(L)) for L in synth.lognormal_lengths(rng, 300, 250, 0.82, 30, 3000)]
    for i in range(0, len(seqs), 6):
        s0 = int(rng.integers(0, len(q) - 300))
        seqs[i] = np.concatenate([seqs[i], synth.mutate(rng, q[s0:s0 + 250], 0.5)])
    res, off = concat(seqs)
    got, _, _ = compare(q, res, off)
    assert len(got) > 10


@pytest.mark.parametrize("cull", [dict(hitlist_size=7), dict(max_hsps=1), dict(hitlist_size=3, max_hsps=2),
                                  dict(hitlist_size=100000), dict(prelim_evalue=1e-3),
                                  dict(prelim_evalue=1e-6, hitlist_size=4, max_hsps=1), dict(hitlist_size=1)])
def test_hitlist_culling(cull):
    rng = np.random.default_rng(77)
    q = synth.random_residues(rng, 400)
    seqs = [synth.random_residues(rng, int(L)) for L in synth.lognormal_lengths(rng, 600, 250, 0.82, 30, 3000)]
    for i in range(0, len(seqs), 3):  # many hits, several HSPs per subject
        for _ in range(2):
            s0 = int(rng.integers(0, len(q) - 120))
            hom = synth.mutate(rng, q[s0:s0 + 120], 0.5)
            pos = int(rng.integers(0, len(seqs[i]) + 1))
            seqs[i] = np.concatenate([seqs[i][:pos], hom, seqs[i][pos:]])
    res, off = concat(seqs)
    got, ref, _ = compare(q, res, off, **cull)
    full, _, _ = compare(q, res, off, **{k: v for k, v in cull.items() if k == "prelim_evalue"})
    assert len(got) > 0
    if "hitlist_size" in cull:
        assert len(set(got["oid"].tolist())) == min(cull["hitlist_size"], len(set(full["oid"].tolist())))
    if "max_hsps" in cull:
        assert np.bincount(got["oid"]).max() <= cull["max_hsps"]


def test_stage_boundary_subjects():
    # subjects around the staging bound (1,024 residues: longer ones are read
    # from global memory) at every 16-byte alignment of their start
    rng = np.random.default_rng(1024)
    q = synth.random_residues(rng, 350)
    seqs = []
    for k, L in enumerate((1008, 1016, 1020, 1023, 1024, 1025, 1040, 2047, 2048, 2049) * 4):
        s = synth.random_residues(rng, L)
        w = int(rng.integers(60, 200))
        s0 = int(rng.integers(0, len(q) - w))
        pos = int(rng.integers(0, L - w))
        hom = synth.mutate(rng, q[s0:s0 + w], 0.6)[:w]  # a homologous stretch, length kept
        s[pos:pos + len(hom)] = hom
        seqs.append(s)
        seqs.append(synth.random_residues(rng, 1 + k % 15))  # shifts the next start's alignment
    res, off = concat(seqs)
    got, _, _ = compare(q, res, off)
    assert len(got) > 5


def test_sharded_search_one_rank_matches_plain(tmp_path):
    # the sharding glue (partition, offsets into the shared residue array,
    # global statistics, gather and merge) on one rank over gloo
    import torch.distributed as dist

    from blaze103 import shard

    w = synth.make_workload("plain-small", scale=0.05)
    store = dist.FileStore(str(tmp_path / "store"), 1)
    dist.init_process_group("gloo", store=store, rank=0, world_size=1)
    try:
        merged = shard.sharded_search(w.residues, w.offsets, w.queries)
    finally:
        dist.destroy_process_group()
    db = blaze103.SeqSrc(w.residues, w.offsets)
    ps = blaze103.PrelimSearch(db)
    for q, got in zip(w.queries, merged):
        want = ps.run(q).hsps
        for f in blaze103.HSP_DTYPE.names:
            assert np.array_equal(got[f], want[f]), f
    ps.close()
    db.close()


def test_homopolymer_query_and_degenerate_databases():
    # a word with more than 255 query positions takes the overflow path of the
    # packed cells; runs in the subjects flood the seed and deferral queues
    rng = np.random.default_rng(255)
    q = np.full(600, 11, dtype=np.uint8)  # L x 600
    seqs = [synth.random_residues(rng, int(rng.integers(50, 900))) for _ in range(60)]
    for i in range(0, 60, 3):
        seqs[i] = np.concatenate([seqs[i], np.full(int(rng.integers(20, 300)), 11, dtype=np.uint8)])
    res, off = concat(seqs)
    got, _, stats = compare(q, res, off)
    assert len(got) > 0 and stats["ungapped_extensions"] > 100
    # databases with no word at all: empty, and only subjects shorter than a word
    for seqs in ([], [q[:0], q[:1], q[:2]]):
        res, off = concat(seqs) if seqs else (np.zeros(0, np.uint8), np.zeros(1, np.uint64))
        got, ref, _ = compare(synth.random_residues(rng, 50), res, off)
        assert len(got) == 0 and len(ref) == 0
