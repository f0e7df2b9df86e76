"""Helpers shared by the GPU parity tests: run one query through the C ABI
(libblaze103 on cuda:0) and through the oracle, and compare bit for bit."""
import os

import numpy as np

import blaze103
import oracle

HSP_FIELDS = ["score", "q_start", "q_end", "s_start", "s_end"]
GAPPED_START_FIELDS = [("q_gapped_start", "q_gstart"), ("s_gapped_start", "s_gstart")]
INIT_FIELDS = [("q_start", "q_start"), ("s_start", "s_start"), ("length", "len"),
               ("score", "score"), ("q_trigger", "q_trig"), ("s_trigger", "s_trig")]
EVALUE_RTOL = 1e-12  # E-values are double arithmetic of identical integer scores


def params_for(qlen, residues_total, n_subjects, **override):
    d = oracle.default_params(qlen, residues_total, n_subjects)
    d.update(override)
    p = blaze103.BlazeParams()
    for name, _ in p._fields_:
        key = "lam" if name == "lambda_" else name
        setattr(p, name, d[key])
    return p, d


def oracle_run(query, residues, offsets, pdict):
    hsps, inits = oracle.search_db(query, residues, offsets, pdict,
                                   threads=os.cpu_count() or 1, want_inits=True)
    return oracle.finish(hsps, pdict), inits


def compare(query, residues, offsets, seq_src=None, search=None, **override):
    """Returns (gpu_hsps, oracle_hsps, stats) after asserting equality."""
    residues = np.ascontiguousarray(residues, dtype=np.uint8)
    offsets = np.ascontiguousarray(offsets, dtype=np.uint64)
    n = len(offsets) - 1
    total = int(offsets[-1] - offsets[0])
    p, pdict = params_for(len(query), max(total, 1), max(n, 1), **override)
    own_db = seq_src is None
    db = seq_src or blaze103.SeqSrc(residues, offsets, device=0)
    ps = search or blaze103.PrelimSearch(db)
    q = blaze103.Query(db, query, p.word_threshold)
    try:
        ps.run_query(q, p)
        got = ps.results()
        got_init = ps.init_hits()
        stats = ps.stats()
    finally:
        q.close()
        if search is None:
            ps.close()
        if own_db:
            db.close()
    ref, ref_init = oracle_run(query, residues, offsets, pdict)
    # stage 1: ungapped HSPs that reached the gapped stage
    assert len(got_init) == len(ref_init), f"init hits: gpu {len(got_init)} oracle {len(ref_init)}"
    assert np.array_equal(got_init["oid"], ref_init["subject"]), "init hits: subjects differ"
    for g, r in INIT_FIELDS:
        assert np.array_equal(got_init[g], ref_init[r]), f"init hits: field {g} differs"
    # stage 2: final HSP lists
    assert len(got) == len(ref), f"HSPs: gpu {len(got)} oracle {len(ref)}"
    assert np.array_equal(got["oid"], ref["subject"]), "HSPs: subjects differ"
    for f in HSP_FIELDS:
        assert np.array_equal(got[f], ref[f]), f"HSPs: field {f} differs"
    for g, r in GAPPED_START_FIELDS:
        assert np.array_equal(got[g], ref[r]), f"HSPs: field {g} differs"
    assert np.allclose(got["evalue"], ref["evalue"], rtol=EVALUE_RTOL, atol=0.0)
    return got, ref, stats


def concat(seqs):
    seqs = [np.asarray(s, dtype=np.uint8) for s in seqs]
    off = np.zeros(len(seqs) + 1, dtype=np.uint64)
    off[1:] = np.cumsum([len(s) for s in seqs])
    res = np.concatenate(seqs) if seqs else np.zeros(0, np.uint8)
    return res, off
