"""The oracle's traceback (CPU): its score and end points equal the
score-only semi-gapped DP's, and the alignment it walks back re-scores to
that score, covers exactly the reported ranges and gives the reported
identity, mismatch and gap counts."""
import numpy as np
import pytest

from blaze103 import synth

BLOSUM = None


def _blosum():
    global BLOSUM
    if BLOSUM is None:
        from blaze103._blosum import BLOSUM62
        BLOSUM = np.array(BLOSUM62, dtype=np.int64)
    return BLOSUM


def _rescore(q, s, q0, s0, ops, gap_open=11, gap_extend=1):
    M = _blosum()
    i, j, score, ident, pos, mism, gaps, runs, prev = q0, s0, 0, 0, 0, 0, 0, 0, None
    for op in ops:
        if op == "M":
            v = int(M[q[i], s[j]])
            score += v
            ident += int(q[i] == s[j])
            pos += int(v > 0)
            mism += int(q[i] != s[j])
            i += 1
            j += 1
        else:
            gaps += 1
            if op != prev:
                runs += 1
                score -= gap_open + gap_extend
            else:
                score -= gap_extend
            if op == "I":
                i += 1
            else:
                j += 1
        prev = op
    return dict(score=score, q_end=i, s_end=j, identities=ident, positives=pos, mismatches=mism, gaps=gaps,
                gap_opens=runs, length=len(ops))


def _pairs(seed, n):
    rng = np.random.default_rng(seed)
    for _ in range(n):
        L = int(rng.integers(5, 400))
        q = synth.random_residues(rng, L)
        kind = int(rng.integers(0, 3))
        if kind == 0:
            s = synth.mutate(rng, q, float(rng.uniform(0.3, 0.9)))
        elif kind == 1:
            w = int(rng.integers(1, L + 1))
            a = int(rng.integers(0, L - w + 1))
            s = np.concatenate([synth.random_residues(rng, int(rng.integers(0, 50))),
                                synth.mutate(rng, q[a:a + w], 0.5), synth.random_residues(rng, int(rng.integers(0, 50)))])
        else:
            s = synth.random_residues(rng, int(rng.integers(1, 400)))
        if len(s) == 0:
            s = synth.random_residues(rng, 3)
        q_off = int(rng.integers(0, len(q)))
        s_off = int(rng.integers(0, len(s)))
        yield q, s, q_off, s_off


@pytest.mark.parametrize("xdrop", [38, 64, 10_000])
def test_traceback_consistent(oracle_mod, xdrop):
    for q, s, q_off, s_off in _pairs(xdrop, 120):
        tb, ops = oracle_mod.traceback_ops(q, s, q_off, s_off, xdrop=xdrop)
        # score and ends equal the score-only DP's (left part + right part)
        left, al, bl = oracle_mod.semi_gapped(q, s, q_off + 1, s_off + 1, 1, xdrop=xdrop)
        right, ar, br = 0, 0, 0
        if q_off < len(q) - 1 and s_off < len(s) - 1:
            right, ar, br = oracle_mod.semi_gapped(q[q_off:], s[s_off:], len(q) - q_off - 1, len(s) - s_off - 1, 0,
                                                   xdrop=xdrop)
        assert tb["score"] == left + right
        assert (tb["q_start"], tb["s_start"]) == (q_off + 1 - al, s_off + 1 - bl)
        assert (tb["q_end"], tb["s_end"]) == (q_off + ar + 1, s_off + br + 1)
        # the walked alignment covers the ranges and re-scores to the score
        # (a gap run across the start point is charged one opening, where the
        # two halves each charged one)
        r = _rescore(q, s, tb["q_start"], tb["s_start"], ops)
        assert (r["q_end"], r["s_end"]) == (tb["q_end"], tb["s_end"])
        assert r["score"] in (tb["score"], tb["score"] + 11)
        for k in ("identities", "positives", "mismatches", "gaps", "gap_opens", "length"):
            assert r[k] == tb[k], k


def test_traceback_known_answers(oracle_mod):
    q = np.array(list(range(1, 21)) * 3, dtype=np.uint8)
    tb, ops = oracle_mod.traceback_ops(q, q, 30, 30)
    assert ops == "M" * 60 and tb["identities"] == 60 and tb["gaps"] == 0
    s = np.concatenate([q[:25], q[28:]])  # three residues deleted from the subject
    tb, ops = oracle_mod.traceback_ops(q, s, 10, 10)
    assert ops == "M" * 25 + "I" * 3 + "M" * 32
    assert tb["gap_opens"] == 1 and tb["gaps"] == 3 and tb["length"] == 60
