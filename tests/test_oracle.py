"""CPU tests of the oracle: known answers and independent brute-force checks.

The reference ships no golden vectors for this path (parity with NCBI BLAST+
2.13.0 is unpinned), so the oracle is pinned here against (a) hand-checkable
known answers, (b) brute-force re-derivations written independently in
Python, and (c) committed fixtures in tests/golden/.
"""
import itertools

import numpy as np
import pytest

from blaze103 import synth
from blaze103._blosum import BLOSUM62

NEG = -(1 << 30)


def codes(s: str) -> np.ndarray:
    alpha = "-ABCDEFGHIKLMNPQRSTVWXYZU*OJ"
    return np.array([alpha.index(c) for c in s], dtype=np.uint8)


# ---------------------------------------------------------------- lookup

def test_blosum_matches_published_values():
    m = BLOSUM62
    assert (m == m.T).all()
    assert m[codes("W")[0], codes("W")[0]] == 11
    assert m[codes("C")[0], codes("C")[0]] == 9
    assert m[codes("A")[0], codes("A")[0]] == 4
    assert m[codes("I")[0], codes("V")[0]] == 3
    # U scores as C, row 0 is the sentinel
    assert (m[24] == m[3]).all()
    assert (m[0] == -32768).all()


def test_lookup_matches_brute_force(oracle_mod):
    rng = np.random.default_rng(1)
    q = synth.random_residues(rng, 23)
    cs, offs = oracle_mod.lookup(q, 11)
    words = [(int(q[i]), int(q[i + 1]), int(q[i + 2])) for i in range(len(q) - 2)]
    rng2 = np.random.default_rng(2)
    for v in list(rng2.integers(0, 21952, size=400)) + [w[0] * 784 + w[1] * 28 + w[2] for w in words]:
        v = int(v)
        x, y, z = v // 784, (v // 28) % 28, v % 28
        want = [i for i, (a, b, c) in enumerate(words)
                if (a, b, c) == (x, y, z) or BLOSUM62[a, x] + BLOSUM62[b, y] + BLOSUM62[c, z] >= 11]
        assert list(offs[cs[v]:cs[v + 1]]) == want


def test_exact_word_always_in_lookup(oracle_mod):
    # "XXX" scores -3 against itself, far below T=11: it must still hit itself
    q = codes("XXXAW")
    cs, offs = oracle_mod.lookup(q, 11)
    v = 21 * 784 + 21 * 28 + 21
    assert list(offs[cs[v]:cs[v + 1]]) == [0]


# ---------------------------------------------------------- gapped DP

def brute_xdrop(A, B, M, N, reverse, go=11, ge=1, X=38):
    """Row-major X-drop DP over the full matrix, written from the definition:
    a cell is live when its score is within X of the best live score seen
    before it in row-major order; dead cells are -inf for their successors."""
    goe = go + ge
    X = max(X, goe)
    if M <= 0 or N <= 0:
        return 0, 0, 0
    row_letter = (lambda a: A[M - a]) if reverse else (lambda a: A[a])
    col_letter = (lambda b: B[N - b]) if reverse else (lambda b: B[b])
    H = np.full((M + 1, N + 1), NEG, dtype=np.int64)
    E = np.full((M + 1, N + 1), NEG, dtype=np.int64)
    live = np.zeros((M + 1, N + 1), dtype=bool)
    best, ab, bb = 0, 0, 0
    for b in range(N + 1):
        h = 0 if b == 0 else -(goe + (b - 1) * ge)
        if h >= -X:
            H[0, b], E[0, b], live[0, b] = h, h - goe, True
    for a in range(1, M + 1):
        f = NEG
        for b in range(N + 1):
            e = max(H[a - 1, b] - goe if live[a - 1, b] else NEG, E[a - 1, b] - ge)
            d = H[a - 1, b - 1] + BLOSUM62[row_letter(a), col_letter(b)] if b >= 1 and live[a - 1, b - 1] else NEG
            h = max(d, e, f)
            if best - h <= X:
                live[a, b] = True
                H[a, b], E[a, b] = h, e
                if h > best:
                    best, ab, bb = h, a, b
                f = max(h - goe, f - ge)
            else:
                f = f - ge
                E[a, b] = e
    return int(best), ab, bb


@pytest.mark.parametrize("seed", range(40))
def test_semi_gapped_matches_brute_force(oracle_mod, seed):
    rng = np.random.default_rng(100 + seed)
    M, N = int(rng.integers(1, 45)), int(rng.integers(1, 45))
    if seed % 3 == 0:  # related sequences give long alignments with gaps
        base = synth.random_residues(rng, max(M, N) + 5)
        A = base[:M + 1].copy()
        B = synth.mutate(rng, base, 0.6)[:N + 1]
        N = len(B) - 1
    else:
        A = synth.random_residues(rng, M + 1)
        B = synth.random_residues(rng, N + 1)
    for reverse in (0, 1):
        a_in = A[1:] if reverse else A
        b_in = B[1:] if reverse else B
        got = oracle_mod.semi_gapped(a_in, b_in, M, N, reverse)
        want = brute_xdrop(a_in, b_in, M, N, reverse)
        assert got == want, (seed, reverse, M, N)


def test_semi_gapped_identity_kat(oracle_mod):
    s = codes("MKTAYIAKQRQISFVKSHFSRQ")
    L = len(s)
    # right extension of a sequence against itself from its first residue
    score, a, b = oracle_mod.semi_gapped(s, s, L - 1, L - 1, 0)
    assert (a, b) == (L - 1, L - 1)
    assert score == sum(int(BLOSUM62[c, c]) for c in s[1:])
    # left extension includes the anchor residue
    score, a, b = oracle_mod.semi_gapped(s, s, L, L, 1)
    assert (a, b) == (L, L) and score == sum(int(BLOSUM62[c, c]) for c in s)


def test_gapped_start_kat(oracle_mod):
    q = codes("WWWWWWWWWWWWAAAAAAAAAAAAAAAA")
    # short HSP: centre
    assert oracle_mod.gapped_start(q, q, 3, 3, 9) == 3 + 4
    # best 11-window is the W run: window ending at offset 10 wins first
    assert oracle_mod.gapped_start(q, q, 0, 0, len(q)) == 10 - 5
    # nothing positive: start of the HSP
    s = codes("PPPPPPPPPPPPPPPP")
    w = codes("WWWWWWWWWWWWWWWW")
    assert oracle_mod.gapped_start(w, s, 2, 2, 14) == 2


# ----------------------------------------------------- whole pipeline

def _params(qlen, dblen, n):
    import oracle
    return oracle.default_params(qlen, dblen, n)


def test_identical_subject_gives_full_alignment(oracle_mod):
    rng = np.random.default_rng(7)
    q = synth.random_residues(rng, 120)
    res = np.concatenate([synth.random_residues(rng, 200), q, synth.random_residues(rng, 50)])
    off = np.array([0, 200, 320, 370], dtype=np.uint64)
    p = _params(len(q), 1_000_000, 3000)
    h, _ = oracle_mod.search_db(q, res, off, p, threads=1)
    hits = h[h["subject"] == 1]
    assert len(hits) >= 1
    top = hits[0]
    assert (top["q_start"], top["q_end"], top["s_start"], top["s_end"]) == (0, 120, 0, 120)
    assert top["score"] == sum(int(BLOSUM62[c, c]) for c in q)


def test_short_and_empty_subjects(oracle_mod):
    q = codes("MKTAYIAKQRQISFVKSHFSRQLEERLGLIEVQ")
    subj = [codes(""), codes("M"), codes("MK"), codes("MKT"), codes("MKTA")]
    res = np.concatenate(subj)
    off = np.zeros(len(subj) + 1, dtype=np.uint64)
    off[1:] = np.cumsum([len(s) for s in subj])
    h, ini = oracle_mod.search_db(q, res, off, _params(len(q), 10_000, 100), want_inits=True)
    assert len(h) == 0 and len(ini) == 0


def test_multithreaded_equals_single_thread(oracle_mod):
    w = synth.make_workload("plain-small", scale=0.05)
    p = _params(len(w.queries[0]), w.total_residues, w.n_subjects)
    a = oracle_mod.search_db(w.queries[0], w.residues, w.offsets, p, threads=1, want_inits=True)
    b = oracle_mod.search_db(w.queries[0], w.residues, w.offsets, p, threads=7, want_inits=True)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_planted_homologs_are_found(oracle_mod):
    w = synth.make_workload("plain-small", scale=0.1)
    p = _params(len(w.queries[0]), w.total_residues, w.n_subjects)
    h, _ = oracle_mod.search_db(w.queries[0], w.residues, w.offsets, p, threads=4)
    found = np.isin(w.planted, h["subject"]).mean()
    assert found > 0.9


def test_length_adjustment_fixed_point(oracle_mod):
    import math
    K, lam, alpha, beta = 0.041, 0.267, 1.9, -30.0
    for m, n, N in [(300, 7_000_000, 20_000), (1000, 700_000_000, 2_000_000), (50, 10_000, 40)]:
        ell = oracle_mod.length_adjustment(K, math.log(K), alpha / lam, beta, m, n, N)
        f = lambda x: beta + alpha / lam * (math.log(K) + math.log((m - x) * (n - N * x)))
        assert f(ell) > ell
        nxt = ell + 1
        assert not (f(nxt) > nxt and K * (m - nxt) * (n - N * nxt) > max(m, n))


# ------------------------------------------- word finder, two-hit, ungapped

def _py_init_hits(q, sub, threshold, window, xdrop, cutoff):
    """Independent restatement of the preliminary stage's word finder for one
    subject, from the published two-hit method: neighbourhood words by brute
    force; per diagonal the last hit and a flag set after a right extension
    (hits before its end are skipped, the first one past it starts over); a
    hit 3 to window-1 positions after the last one triggers the ungapped X-drop
    extension (left from the end of the word's best prefix; right only when the
    left walk reached the first hit, stopping at score <= 0)."""
    m = BLOSUM62.astype(np.int64)
    alpha = np.arange(28)
    X, Y, Z = np.meshgrid(alpha, alpha, alpha, indexing="ij")
    X, Y, Z = X.ravel(), Y.ravel(), Z.ravel()
    look = {}
    for i in range(len(q) - 2):
        a, b, c = int(q[i]), int(q[i + 1]), int(q[i + 2])
        sc = m[a][X] + m[b][Y] + m[c][Z]
        for v in np.flatnonzero((sc >= threshold) | ((X == a) & (Y == b) & (Z == c))):
            look.setdefault(int(v), []).append(i)

    def score(qi, si):
        return int(m[q[qi], sub[si]])

    def extend(s_left, s_off, q_off):
        sc = best = rd = 0
        for i in range(3):
            sc += score(q_off + i, s_off + i)
            if sc > best:
                best, rd = sc, i + 1
        qr, sr = q_off + rd, s_off + rd
        left = run = 0
        best_k = -1
        for k in range(min(sr - 1, qr - 1) + 1):  # left walk from (qr - 1, sr - 1)
            run += score(qr - 1 - k, sr - 1 - k)
            if run > left:
                left, best_k = run, k
            if left - run >= xdrop:
                break
        ld = best_k + 1
        right, rlen, rext, slast = 0, 0, False, sr
        if ld >= sr - s_left:
            rext = True
            n = min(len(sub) - sr, len(q) - qr)
            run = right = left
            best_i, i = -1, 0
            while i < n:
                run += score(qr + i, sr + i)
                if run > right:
                    right, best_i = run, i
                if run <= 0 or right - run >= xdrop:
                    break
                i += 1
            rlen, slast = best_i + 1, sr + i
        return max(left, right), qr - ld, sr - ld, ld + rlen, rext, slast

    hits, state = [], {}
    for s in range(len(sub) - 2):
        w = int(sub[s]) * 784 + int(sub[s + 1]) * 28 + int(sub[s + 2])
        for qo in look.get(w, []):
            d = s - qo
            last, flag = state.get(d, (None, False))
            if flag:
                if s >= last:
                    state[d] = (s, False)
                continue
            if last is None or s - last >= window:
                state[d] = (s, False)
                continue
            if s - last < 3:
                continue
            sc, hq, hs, hl, rext, slast = extend(last + 3, s, qo)
            if sc >= cutoff:
                hits.append((hq, hs, hl, sc, qo, s))
            state[d] = (slast - 2, True) if rext else (s, False)
    return hits


@pytest.mark.parametrize("seed", range(30))
def test_init_hits_match_independent_restatement(oracle_mod, seed):
    rng = np.random.default_rng(900 + seed)
    q = synth.random_residues(rng, int(rng.integers(50, 160)))
    if seed % 3 == 0:  # a low-complexity stretch: dense same-diagonal hits
        q[10:40] = np.array([1, 11, 17], dtype=np.uint8)[rng.integers(0, 3, 30)]
    seqs = []
    for i in range(12):
        s = synth.random_residues(rng, int(rng.integers(20, 400)))
        if i % 3 == 0 and len(q) > 30:
            w = int(rng.integers(20, len(q)))
            s0 = int(rng.integers(0, len(q) - w + 1))
            hom = synth.mutate(rng, q[s0:s0 + w], float(rng.uniform(0.4, 0.9)))
            p = int(rng.integers(0, len(s) + 1))
            s = np.concatenate([s[:p], hom, s[p:]])
        seqs.append(s)
    off = np.zeros(len(seqs) + 1, dtype=np.uint64)
    off[1:] = np.cumsum([len(s) for s in seqs])
    res = np.concatenate(seqs)
    p = oracle_mod.default_params(len(q), 50_000_000, 100_000)
    _, ini = oracle_mod.search_db(q, res, off, p, threads=1, want_inits=True)
    total = 0
    for k, s in enumerate(seqs):
        want = sorted(_py_init_hits(q, s, p["word_threshold"], p["window"], p["ungapped_xdrop"],
                                    p["ungapped_cutoff"]))
        mine = ini[ini["subject"] == k]
        got = sorted(zip(*(mine[f].tolist() for f in ("q_start", "s_start", "len", "score", "q_trig", "s_trig"))))
        assert got == want, (seed, k)
        total += len(want)
    if seed % 3 == 0:
        assert total > 0


# ------------------------------------------------ gapped stage per subject

def _py_gapped_subject(oracle_mod, q, s, inits, p):
    """Independent restatement of the per-subject gapped pipeline over the
    subject's init hits: order by ungapped score (ties in discovery order),
    skip an init hit inside a kept HSP at least as good, X-drop DP left and
    right of the gapped start point (the DP itself is checked by brute force
    above), keep what reaches the gapped cutoff, then drop HSPs sharing a
    start and then an end with a better one, and order by score."""
    order = sorted(inits, key=lambda u: (-u["score"], u["s_trig"], u["q_trig"]))
    kept = []
    for u in order:
        if any(u["score"] <= g["score"] and g["q_start"] <= u["q_start"] and u["q_start"] + u["len"] <= g["q_end"]
               and g["s_start"] <= u["s_start"] and u["s_start"] + u["len"] <= g["s_end"] for g in kept):
            continue
        qo = oracle_mod.gapped_start(q, s, u["q_start"], u["s_start"], u["len"])
        so = qo + u["s_start"] - u["q_start"]
        gx = dict(gap_open=p["gap_open"], gap_extend=p["gap_extend"], xdrop=p["gapped_xdrop"])
        left, al, bl = oracle_mod.semi_gapped(q, s, qo + 1, so + 1, True, **gx)
        right, ar, br = 0, 0, 0
        if qo < len(q) - 1 and so < len(s) - 1:
            right, ar, br = oracle_mod.semi_gapped(q[qo:], s[so:], len(q) - qo - 1, len(s) - so - 1, False, **gx)
        if left + right >= p["gapped_cutoff"]:
            kept.append(dict(score=left + right, q_start=qo + 1 - al, q_end=qo + ar + 1, s_start=so + 1 - bl,
                             s_end=so + br + 1, q_gstart=qo, s_gstart=so))
    by_start = sorted(kept, key=lambda h: (h["q_start"], h["s_start"], -h["score"], -h["q_end"], -h["s_end"]))
    m = [h for i, h in enumerate(by_start)
         if i == 0 or (h["q_start"], h["s_start"]) != (by_start[i - 1]["q_start"], by_start[i - 1]["s_start"])]
    by_end = sorted(m, key=lambda h: (h["q_end"], h["s_end"], -h["score"], h["q_start"], h["s_start"]))
    m = [h for i, h in enumerate(by_end)
         if i == 0 or (h["q_end"], h["s_end"]) != (by_end[i - 1]["q_end"], by_end[i - 1]["s_end"])]
    return sorted(m, key=lambda h: (-h["score"], h["s_start"], -h["s_end"], h["q_start"], -h["q_end"]))


@pytest.mark.parametrize("seed", range(10))
def test_gapped_hsps_match_independent_restatement(oracle_mod, seed):
    rng = np.random.default_rng(1300 + seed)
    q = synth.random_residues(rng, int(rng.integers(80, 300)))
    seqs = []
    for i in range(10):
        s = synth.random_residues(rng, int(rng.integers(30, 500)))
        for _ in range(int(rng.integers(0, 3))):  # several homologous stretches, some overlapping
            w = int(rng.integers(20, len(q)))
            s0 = int(rng.integers(0, len(q) - w + 1))
            hom = synth.mutate(rng, q[s0:s0 + w], float(rng.uniform(0.4, 0.95)))
            p0 = int(rng.integers(0, len(s) + 1))
            s = np.concatenate([s[:p0], hom, s[p0:]])
        seqs.append(s)
    off = np.zeros(len(seqs) + 1, dtype=np.uint64)
    off[1:] = np.cumsum([len(s) for s in seqs])
    res = np.concatenate(seqs)
    p = oracle_mod.default_params(len(q), 20_000_000, 50_000)
    hsps, ini = oracle_mod.search_db(q, res, off, p, threads=1, want_inits=True)
    total = 0
    for k, s in enumerate(seqs):
        want = _py_gapped_subject(oracle_mod, q, s, [dict(zip(ini.dtype.names, r.tolist()))
                                                     for r in ini[ini["subject"] == k]], p)
        got = hsps[hsps["subject"] == k]
        fields = ["score", "q_start", "q_end", "s_start", "s_end", "q_gstart", "s_gstart"]
        assert [tuple(int(g[f]) for f in fields) for g in got] == [tuple(h[f] for f in fields) for h in want], (seed, k)
        total += len(want)
    assert total > 0
