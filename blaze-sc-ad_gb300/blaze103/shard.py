"""Database sharding across GPUs (one process per GPU).

Subjects are independent, so a database splits into contiguous OID ranges of
about equal residue count, one per rank; each rank searches its range with the
E-value statistics of the WHOLE database (its length and subject count, passed
in through the search parameters), and the per-subject HSP lists are gathered
to one rank on the host and concatenated in OID order. No device collective is
involved. The merged lists are then exactly those of one search over the whole
database: HSP lists are per subject, and every cutoff and E-value depends only
on the subject and the global statistics.

The reference runs one database per process and splits work between its GPU
threads by byte-balanced chunks (BLAZE_ncbi/blast_seqsrc.c:541-570,
find_balanced_indices); the split here is by residues, over contiguous OIDs.
"""
from __future__ import annotations

import numpy as np


def partition(offsets, world: int) -> list[tuple[int, int]]:
    """Contiguous OID ranges [lo, hi), one per rank, of about total/world
    residues each (a range may be empty when subjects are few)."""
    off = np.asarray(offsets, dtype=np.uint64)
    if off.ndim != 1 or off.size < 1 or world < 1:
        raise ValueError("offsets must be n_subjects + 1 entries and world >= 1")
    n = off.size - 1
    base, total = int(off[0]), int(off[-1] - off[0])
    cuts = [0]
    for r in range(1, world):
        target = base + (total * r) // world
        cuts.append(max(cuts[-1], min(int(np.searchsorted(off, target, side="left")), n)))
    cuts.append(n)
    return [(cuts[r], cuts[r + 1]) for r in range(world)]


def shard_offsets(offsets, lo: int, hi: int) -> np.ndarray:
    """Offsets of OIDs [lo, hi) into the same residue array (the database
    source takes a non-zero first offset), so no residues are copied."""
    return np.ascontiguousarray(np.asarray(offsets, dtype=np.uint64)[lo:hi + 1])


def merge(parts, bases) -> np.ndarray:
    """Concatenates per-rank HSP records (local OIDs) into one array with
    global OIDs, grouped by OID (by query, then OID, for batch records), each
    subject's HSPs in the order its rank gave them."""
    parts = [np.asarray(p) for p in parts]
    if not parts:
        raise ValueError("nothing to merge")
    out = []
    for p, b in zip(parts, bases):
        q = p.copy()
        q["oid"] = q["oid"] + np.uint32(b)
        out.append(q)
    cat = np.concatenate(out)
    keys = (cat["oid"],) if "query" not in cat.dtype.names else (cat["oid"], cat["query"])
    return cat[np.lexsort(keys)]  # lexsort is stable: per-subject order is kept


def keep_best_subjects(hsps: np.ndarray, hitlist_size: int) -> np.ndarray:
    """hitlist_size (NCBI max_target_seqs) over merged records: per query,
    the hitlist_size subjects whose lists start with the best score (E-values
    of one query fall with the score), ties by smaller OID -- the rule each
    rank's device selection applies to its own shard. Every subject of the
    global top k is in its own rank's top k, so culling each shard and then
    the merge gives exactly the lists of one search over the whole database.
    Records must be grouped by (query,) OID with each list best first, as
    merge() returns them."""
    if hitlist_size <= 0 or len(hsps) == 0:
        return hsps
    batched = "query" in hsps.dtype.names
    qcol = hsps["query"].astype(np.int64) if batched else np.zeros(len(hsps), dtype=np.int64)
    oid = hsps["oid"].astype(np.int64)
    # first record of each (query, OID) list carries its best score
    start = np.ones(len(hsps), dtype=bool)
    start[1:] = (qcol[1:] != qcol[:-1]) | (oid[1:] != oid[:-1])
    heads = np.flatnonzero(start)
    hq, ho, hs = qcol[heads], oid[heads], hsps["score"][heads].astype(np.int64)
    order = np.lexsort((ho, -hs, hq))  # by query, then best score descending, then OID
    rank_in_query = np.empty(len(order), dtype=np.int64)
    sq = hq[order]
    first_of_query = np.ones(len(order), dtype=bool)
    first_of_query[1:] = sq[1:] != sq[:-1]
    group_start = np.maximum.accumulate(np.where(first_of_query, np.arange(len(order)), 0))
    rank_in_query[order] = np.arange(len(order)) - group_start
    keep_head = rank_in_query < hitlist_size
    list_id = np.cumsum(start) - 1
    return hsps[keep_head[list_id]]


def gather_merge(local_hsps: np.ndarray, base: int, group=None, dst: int = 0, hitlist_size: int = 0):
    """torch.distributed gather of every rank's records to rank `dst`, which
    returns the merged array (with hitlist_size > 0: culled to the best
    hitlist_size subjects per query over the whole database); other ranks
    return None."""
    import torch.distributed as dist

    rank = dist.get_rank(group)
    world = dist.get_world_size(group)
    payload = (int(base), np.ascontiguousarray(local_hsps))
    got = [None] * world if rank == dst else None
    dist.gather_object(payload, got, dst=dst, group=group)
    if rank != dst:
        return None
    return keep_best_subjects(merge([g[1] for g in got], [g[0] for g in got]), hitlist_size)


def sharded_search(residues, offsets, queries, evalue: float = 10.0, group=None, device: int | None = None,
                   hitlist_size: int = 0, max_hsps: int = 0):
    """Searches each query against this rank's shard of the database on its
    GPU and gathers the merged per-subject HSP lists to rank 0 (None
    elsewhere). Every rank passes the same residues/offsets. hitlist_size and
    max_hsps cull as one search over the whole database would: max_hsps is
    per subject, so each rank applies it; hitlist_size is applied on each
    rank's device and again over the merge."""
    import torch.distributed as dist

    import blaze103

    rank, world = dist.get_rank(group), dist.get_world_size(group)
    off = np.asarray(offsets, dtype=np.uint64)
    lo, hi = partition(off, world)[rank]
    total, n = int(off[-1] - off[0]), off.size - 1
    src = blaze103.SeqSrc(residues, shard_offsets(off, lo, hi), device=rank if device is None else device)
    ps = blaze103.PrelimSearch(src)
    results = []
    try:
        for q in queries:
            p = blaze103.default_params(len(q), evalue=evalue, db_residues=total, db_subjects=n)
            p.hitlist_size, p.max_hsps = int(hitlist_size), int(max_hsps)
            local = ps.run(q, p).hsps if hi > lo else np.empty(0, dtype=blaze103.HSP_DTYPE)
            results.append(gather_merge(local, lo, group, hitlist_size=hitlist_size))
    finally:
        ps.close()
        src.close()
    return results if rank == 0 else None
