"""Multi-GPU sharding logic, run on the CPU: residue-balanced partition of the
database into contiguous OID ranges, and the host-side gather and merge of
per-rank HSP lists, with two gloo ranks. Each rank searches its shard with
the oracle (standing in for a GPU) under the whole database's statistics; the
merged result must equal one search over the whole database."""
import multiprocessing as mp
import os
import socket

import numpy as np
import pytest

import blaze103
from blaze103 import shard, synth


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _as_blaze(hsps):
    out = np.zeros(len(hsps), dtype=blaze103.HSP_DTYPE)
    out["oid"] = hsps["subject"]
    for f in ("score", "q_start", "q_end", "s_start", "s_end", "evalue"):
        out[f] = hsps[f]
    out["q_gapped_start"] = hsps["q_gstart"]
    out["s_gapped_start"] = hsps["s_gstart"]
    return out


def _rank_main(rank, world, port, residues, offsets, query, outq, hitlist_size=0):
    import torch.distributed as dist

    import oracle

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        lo, hi = shard.partition(offsets, world)[rank]
        total, n = int(offsets[-1] - offsets[0]), len(offsets) - 1
        pd = oracle.default_params(len(query), total, n)
        off = shard.shard_offsets(offsets, lo, hi)
        local_res = residues[int(off[0]):int(off[-1])]
        hs, _ = oracle.search_db(query, local_res, off - off[0], pd, threads=2)
        # with hitlist_size, each rank culls its own shard first, as its
        # device selection would
        local = oracle.cull(oracle.finish(hs, pd), hitlist_size=hitlist_size)
        merged = shard.gather_merge(_as_blaze(local), lo, hitlist_size=hitlist_size)
        if rank == 0:
            outq.put(merged)
    finally:
        dist.destroy_process_group()


def _workload(seed=3, n=600):
    rng = np.random.default_rng(seed)
    q = synth.random_residues(rng, 260)
    seqs = [synth.random_residues(rng, int(L)) for L in synth.lognormal_lengths(rng, n, 250, 0.82, 30, 3000)]
    for i in range(0, n, 4):
        s0 = int(rng.integers(0, 160))
        seqs[i] = np.concatenate([seqs[i], synth.mutate(rng, q[s0:s0 + 100], 0.45)])
    off = np.zeros(n + 1, dtype=np.uint64)
    np.cumsum([len(s) for s in seqs], out=off[1:])
    return q, np.concatenate(seqs).astype(np.uint8), off


@pytest.mark.parametrize("world,hitlist_size", [(2, 0), (3, 0), (2, 20)])
def test_sharded_merge_equals_whole_database(oracle_mod, world, hitlist_size):
    q, res, off = _workload()
    pd = oracle_mod.default_params(len(q), int(off[-1]), len(off) - 1)
    hs, _ = oracle_mod.search_db(q, res, off, pd, threads=4)
    want = _as_blaze(oracle_mod.cull(oracle_mod.finish(hs, pd), hitlist_size=hitlist_size))
    if hitlist_size:
        assert len(np.unique(want["oid"])) == hitlist_size
    ctx = mp.get_context("spawn")
    outq = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, res, off, q, outq, hitlist_size))
             for r in range(world)]
    for p in procs:
        p.start()
    got = outq.get(timeout=240)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert len(want) > (19 if hitlist_size else 50)
    for f in blaze103.HSP_DTYPE.names:
        assert np.array_equal(got[f], want[f]), f


def test_partition_balances_residues():
    rng = np.random.default_rng(1)
    lengths = np.sort(synth.lognormal_lengths(rng, 10_000, 250, 0.82, 30, 5000))
    off = np.zeros(len(lengths) + 1, dtype=np.uint64)
    np.cumsum(lengths, out=off[1:])
    for world in (1, 2, 4, 8):
        parts = shard.partition(off, world)
        assert parts[0][0] == 0 and parts[-1][1] == len(lengths)
        assert all(a[1] == b[0] for a, b in zip(parts, parts[1:]))
        per = [int(off[hi] - off[lo]) for lo, hi in parts]
        assert max(per) - min(per) <= 2 * int(lengths.max())


def test_partition_edge_cases():
    off = np.array([0, 5, 10], dtype=np.uint64)
    parts = shard.partition(off, 4)  # more ranks than subjects: some ranges empty
    assert parts[0][0] == 0 and parts[-1][1] == 2
    assert sum(hi - lo for lo, hi in parts) == 2
    assert shard.partition(np.array([7], dtype=np.uint64), 2) == [(0, 0), (0, 0)]
    with pytest.raises(ValueError):
        shard.partition(off, 0)
    # non-zero first offset: the shard's offsets index the same residue array
    assert np.array_equal(shard.shard_offsets(off, 1, 2), [5, 10])


def test_merge_orders_batch_records():
    a = np.zeros(3, dtype=blaze103.BATCH_HSP_DTYPE)
    a["query"], a["oid"], a["score"] = [0, 0, 1], [0, 1, 0], [5, 6, 7]
    b = np.zeros(2, dtype=blaze103.BATCH_HSP_DTYPE)
    b["query"], b["oid"], b["score"] = [0, 1], [0, 0], [8, 9]
    m = shard.merge([a, b], [0, 10])
    assert m["query"].tolist() == [0, 0, 0, 1, 1]
    assert m["oid"].tolist() == [0, 1, 10, 0, 10]
    assert m["score"].tolist() == [5, 6, 8, 7, 9]


def test_keep_best_subjects_per_query():
    a = np.zeros(7, dtype=blaze103.BATCH_HSP_DTYPE)
    a["query"] = [0, 0, 0, 0, 1, 1, 1]
    a["oid"] = [1, 1, 4, 9, 2, 3, 8]
    a["score"] = [50, 20, 60, 50, 5, 7, 7]
    k = shard.keep_best_subjects(a, 2)
    assert k["query"].tolist() == [0, 0, 0, 1, 1]
    assert k["oid"].tolist() == [1, 1, 4, 3, 8]  # query 0: 60 (oid 4), then 50 by smaller OID
    assert len(shard.keep_best_subjects(a, 0)) == 7
    single = np.zeros(3, dtype=blaze103.HSP_DTYPE)
    single["oid"], single["score"] = [0, 5, 6], [9, 9, 10]
    assert shard.keep_best_subjects(single, 2)["oid"].tolist() == [0, 6]
