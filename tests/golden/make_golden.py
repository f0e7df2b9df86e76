"""Regenerate the oracle regression fixtures in this directory.

    python tests/golden/make_golden.py [fixture name ...]

Each fixture holds a seeded synthetic case (query, residues, offsets), the
search parameters, the oracle's init hits and final HSPs for it, and the
oracle's traceback of those HSPs (final X-drop 64, before the E-value reap).
The
reference ships no golden vectors for this path, so these pin the oracle
against its own past output (regressions), while tests/test_oracle.py pins it
against brute force and known answers.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "blaze-sc-ad_gb300")]

import oracle  # noqa: E402
from blaze103 import synth  # noqa: E402

PARAM_KEYS = ["word_threshold", "window", "ungapped_xdrop", "ungapped_cutoff", "gap_open",
              "gap_extend", "gapped_xdrop", "gapped_cutoff"]


def cases():
    w = synth.make_workload("plain-small", scale=0.02)
    yield "plain_small_scale002", w.queries[0], w.residues, w.offsets, (7_000_000, 20_000)
    rng = np.random.default_rng(77)
    alpha = np.array([1, 11, 17], dtype=np.uint8)
    q = np.concatenate([alpha[rng.integers(0, 3, 120)], synth.random_residues(rng, 180)])
    seqs = []
    for i in range(120):
        s = synth.random_residues(rng, int(rng.integers(40, 900)))
        if i % 3 == 0:
            s = np.concatenate([s, alpha[rng.integers(0, 3, int(rng.integers(40, 200)))]])
        if i % 5 == 0:
            s = np.concatenate([synth.mutate(rng, q[50:250], 0.5), s])
        seqs.append(s)
    off = np.zeros(len(seqs) + 1, dtype=np.uint64)
    off[1:] = np.cumsum([len(s) for s in seqs])
    yield "lowcomplexity_homologs", q, np.concatenate(seqs), off, (50_000_000, 150_000)
    # the overflow-stress shape, small: a 2,257-residue query, 80 subjects
    # with low-complexity runs and 30-60 % homologs, plus two long subjects
    # (12,000 and 33,000 residues) holding homologs and a low-complexity run
    w = synth.make_workload("overflow-stress", scale=0.00016)
    q = w.queries[1]
    rng = np.random.default_rng(33)
    seqs = [w.residues[int(w.offsets[i]):int(w.offsets[i + 1])] for i in range(w.n_subjects)]
    for L in (12_000, 33_000):
        s = synth.random_residues(rng, L)
        for _ in range(3):
            s0 = int(rng.integers(0, len(q) - 300))
            hom = synth.mutate(rng, q[s0:s0 + 300], float(rng.uniform(0.3, 0.6)))
            p = int(rng.integers(0, len(s) - len(hom)))
            s[p:p + len(hom)] = hom
        run = alpha[rng.integers(0, 3, 150)]
        p = int(rng.integers(0, len(s) - 150))
        s[p:p + 150] = run
        seqs.append(s)
    off = np.zeros(len(seqs) + 1, dtype=np.uint64)
    off[1:] = np.cumsum([len(s) for s in seqs])
    yield "overflow_stress_small", q, np.concatenate(seqs), off, (60_000_000, 100_000)


def main(only=()):
    for name, q, res, off, (dblen, dbn) in cases():
        if only and name not in only:
            continue
        p = oracle.default_params(len(q), dblen, dbn)
        hsps, inits = oracle.search_db(q, res, off, p, threads=4, want_inits=True)
        traced = traced_records(q, res, off, hsps, p)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), query=np.asarray(q, np.uint8),
                            residues=np.asarray(res, np.uint8), offsets=off,
                            params=np.array([p[k] for k in PARAM_KEYS], np.int32),
                            db_len=np.int64(dblen), db_n=np.int64(dbn), hsps=hsps, inits=inits, traced=traced)
        print(name, len(res), "residues", len(inits), "init hits", len(hsps), "HSPs", len(traced), "traced")


TRACED_DTYPE = np.dtype([("subject", "<u4")] + [(f, "<i4") for f in (
    "score", "q_start", "q_end", "s_start", "s_end", "length", "identities", "positives", "mismatches",
    "gap_opens", "gaps")])


def traced_records(q, res, off, hsps, p):
    """The oracle's traceback stage over the preliminary HSPs, no E-value reap."""
    fin = oracle.finish(hsps, dict(p, prelim_evalue=1e300))
    rows = oracle.traceback_hsps(q, res, off, fin, p, evalue=1e300)
    out = np.zeros(len(rows), dtype=TRACED_DTYPE)
    for i, r in enumerate(rows):
        for f in TRACED_DTYPE.names:
            out[i][f] = r[f]
    return out


if __name__ == "__main__":
    main(tuple(sys.argv[1:]))  # fixture names to regenerate (default: all)
