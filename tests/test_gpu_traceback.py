"""GPU traceback stage against the oracle: every HSP of a preliminary run
traced again from its gapped start point with the final X-drop; scores,
ranges, alignment length, identities, positives, mismatches, gap openings
and gap letters bit-exact after the per-subject purge and order; E-values
within a relative 1e-12."""
import numpy as np
import pytest

import blaze103
from blaze103 import synth

from _parity import EVALUE_RTOL, concat, oracle_run, params_for

pytestmark = pytest.mark.gpu

TB_FIELDS = ["score", "q_start", "q_end", "s_start", "s_end", "length", "identities", "positives", "mismatches",
             "gap_opens", "gaps"]


def _check(q, res, off, final_xdrop=64, evalue=None):
    import oracle

    res = np.ascontiguousarray(res, dtype=np.uint8)
    off = np.ascontiguousarray(off, dtype=np.uint64)
    p, pd = params_for(len(q), int(off[-1]), len(off) - 1)
    db = blaze103.SeqSrc(res, off)
    ps = blaze103.PrelimSearch(db)
    try:
        prelim = ps.run(q, p).hsps
        got = ps.traceback(q, p, evalue=evalue, final_xdrop=final_xdrop)
    finally:
        ps.close()
        db.close()
    ref_prelim, _ = oracle_run(q, res, off, pd)
    assert len(prelim) == len(ref_prelim)
    ref = oracle.traceback_hsps(q, res, off, ref_prelim, pd, xdrop=final_xdrop, evalue=evalue)
    assert len(got) == len(ref)
    assert got["oid"].tolist() == [r["subject"] for r in ref]
    for f in TB_FIELDS:
        assert got[f].tolist() == [r[f] for r in ref], f
    assert np.allclose(got["evalue"], [r["evalue"] for r in ref], rtol=EVALUE_RTOL, atol=0.0)
    bits = (pd["lam"] * got["score"] - np.log(pd["K"])) / np.log(2.0)
    assert np.allclose(got["bit_score"], bits, rtol=1e-12)
    return got


def _db_with_homologs(seed, q, n=800, ident=0.45, indel_heavy=False):
    rng = np.random.default_rng(seed)
    seqs = [synth.random_residues(rng, int(L)) for L in synth.lognormal_lengths(rng, n, 250, 0.82, 30, 3000)]
    for i in range(0, len(seqs), 4):
        w = min(len(q), int(rng.integers(40, 400)))
        s0 = int(rng.integers(0, len(q) - w + 1))
        hom = synth.mutate(rng, q[s0:s0 + w], ident)
        if indel_heavy:  # extra deletions and insertions
            cut = int(rng.integers(1, max(len(hom) - 8, 2)))
            hom = np.concatenate([hom[:cut], synth.random_residues(rng, int(rng.integers(1, 9))), hom[cut + 4:]])
        pos = int(rng.integers(0, len(seqs[i]) + 1))
        seqs[i] = np.concatenate([seqs[i][:pos], hom, seqs[i][pos:]])
    return concat(seqs)


@pytest.mark.parametrize("qlen", [60, 300, 1200])
def test_traceback_matches_oracle(qlen):
    rng = np.random.default_rng(qlen)
    q = synth.random_residues(rng, qlen)
    res, off = _db_with_homologs(qlen + 1, q)
    got = _check(q, res, off)
    assert len(got) > 20 and got["gaps"].sum() > 0


@pytest.mark.parametrize("xdrop", [38, 200])
def test_traceback_final_xdrop(xdrop):
    rng = np.random.default_rng(11)
    q = synth.random_residues(rng, 500)
    res, off = _db_with_homologs(12, q, indel_heavy=True)
    _check(q, res, off, final_xdrop=xdrop, evalue=1.0)


def test_traceback_identical_and_long():
    rng = np.random.default_rng(13)
    q = synth.random_residues(rng, 2500)
    seqs = [q.copy(), np.concatenate([q[:1000], q[1010:]]), synth.mutate(rng, q, 0.7)]
    seqs += [synth.random_residues(rng, 400) for _ in range(50)]
    res, off = concat(seqs)
    got = _check(q, res, off)
    top = got[got["oid"] == 0][0]
    assert top["identities"] == 2500 and top["length"] == 2500 and top["gaps"] == 0


def test_traceback_buffer_regrowth(monkeypatch):
    monkeypatch.setenv("BLAZE_INITIAL_TRACEBACK_CAP", "128")
    rng = np.random.default_rng(14)
    q = synth.random_residues(rng, 700)
    res, off = _db_with_homologs(15, q, n=300)
    _check(q, res, off)


def test_traceback_to_tabular():
    from blaze103 import tabular

    w = synth.make_workload("plain-small", scale=0.1)
    db = blaze103.SeqSrc(w.residues, w.offsets)
    ps = blaze103.PrelimSearch(db)
    q = w.queries[0]
    p = blaze103.default_params(len(q), db)
    ps.run(q, p)
    tb = ps.traceback(q, p)
    text = tabular.format_tabular(tb, "query1", lambda oid: f"subject{oid}", outfmt=7)
    lines = [ln for ln in text.splitlines() if not ln.startswith("#")]
    assert len(lines) == len(tb) > 0
    cols = lines[0].split("\t")
    assert len(cols) == 12 and float(cols[2]) > 30.0
    assert ps.stats()["traceback_ms"] > 0
    ps.close()
    db.close()


def test_traceback_batch_equals_single():
    rng = np.random.default_rng(21)
    qs = [synth.random_residues(rng, L) for L in (80, 300, 700, 1500)]
    seqs = [synth.random_residues(rng, int(L)) for L in synth.lognormal_lengths(rng, 900, 250, 0.82, 30, 3000)]
    for i in range(0, len(seqs), 4):
        q = qs[i % len(qs)]
        w = min(len(q), int(rng.integers(40, 300)))
        s0 = int(rng.integers(0, len(q) - w + 1))
        seqs[i] = np.concatenate([seqs[i], synth.mutate(rng, q[s0:s0 + w], 0.45)])
    res, off = concat(seqs)
    db = blaze103.SeqSrc(res, off)
    ps = blaze103.PrelimSearch(db)
    params = [blaze103.default_params(len(q), db) for q in qs]
    singles = []
    for q, p in zip(qs, params):
        ps.run(q, p)
        singles.append(ps.traceback(q, p))
    batch = blaze103.QueryBatch(db, qs)
    ps.run_batch(batch, params)
    got = ps.traceback_batch(batch, params)
    for i, want in enumerate(singles):
        g = got[got["query"] == i]
        for f in TB_FIELDS + ["oid"]:
            assert np.array_equal(g[f], want[f]), (i, f)
        assert np.allclose(g["evalue"], want["evalue"], rtol=1e-12)
    assert len(got) == sum(len(w) for w in singles) > 20
    batch.close()
    ps.close()
    db.close()
