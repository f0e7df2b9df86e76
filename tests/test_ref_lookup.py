"""The oracle's word lookup against golden vectors made by the REFERENCE's
own code (tests/golden/ref_lookup.npz, written by
tests/golden/make_ref_lookup.py from oracle/_ref/libblaze_ref.so, which is
compiled from the reference's BLAZE_gpu sources):

* the BLOSUM62 scores of the reference (util.hpp:30-57, and the engine's
  copy in prelim_stage.cpp:69-96) equal this repository's tables on every
  pair of residue codes 1..27;
* the neighbourhood of every one of the 21,952 words (util.hpp:64-85) equals
  the one this repository's tables give (count and checksum for all words,
  full lists for a sample);
* for each fixture query, the words' lists of query offsets built as in
  prelim_stage.cpp:360-386 hold exactly the offsets of the oracle's lookup
  (the reference appends each source word's offsets in turn; the oracle
  keeps each list in ascending order, as NCBI's lookup does -- the sets are
  compared).
CPU only."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
A = 28


@pytest.fixture(scope="module")
def ref():
    return np.load(os.path.join(HERE, "golden", "ref_lookup.npz"))


def _checksum(words) -> int:
    return int(((np.asarray(words, dtype=np.uint64) + 1) * np.uint64(2654435761)).sum() % (1 << 32))


def test_blosum62_equals_the_reference_tables(ref):
    from blaze103 import _blosum

    m = np.asarray(_blosum.BLOSUM62, dtype=np.int64)
    assert np.array_equal(m[1:, 1:], ref["matrix"][1:, 1:])
    assert bool(ref["engine_matrix_same"])


def _neighbourhoods():
    """Every word's neighbours under this repository's BLOSUM62: the other
    words scoring >= 11 against it."""
    from blaze103 import _blosum

    m = np.asarray(_blosum.BLOSUM62, dtype=np.int64)
    m[0, :] = m[:, 0] = -10**6  # code 0 never reaches the threshold
    w = np.arange(A ** 3)
    a, b, c = w // (A * A), (w // A) % A, w % A
    out = []
    for x in range(A ** 3):
        s = m[a[x], a] + m[b[x], b] + m[c[x], c]
        nb = np.flatnonzero(s >= 11)
        out.append(nb[nb != x])
    return out


def test_every_word_neighbourhood_equals_the_reference(ref):
    nbr = _neighbourhoods()
    counts = np.array([len(x) for x in nbr])
    assert np.array_equal(counts, ref["counts"].astype(np.int64))
    sums = np.array([_checksum(x) for x in nbr], dtype=np.uint32)
    assert np.array_equal(sums, ref["checksums"])
    so = ref["std_offsets"]
    for k, w in enumerate(ref["std_words"].tolist()):
        got = nbr[w]
        want = np.sort(ref["std_neighbours"][so[k]:so[k + 1]].astype(np.int64))
        assert np.array_equal(got, want), w


def test_oracle_lookup_holds_the_reference_offsets(ref):
    import oracle

    qo, pb = ref["query_offsets"], ref["pair_bounds"]
    for i in range(len(qo) - 1):
        q = ref["queries"][qo[i]:qo[i + 1]]
        cs, offs = oracle.lookup(q, 11)
        words = ref["pair_words"][pb[i]:pb[i + 1]].astype(np.int64)
        poss = ref["pair_offsets"][pb[i]:pb[i + 1]].astype(np.int64)
        # every word the reference lists, with the same offsets
        want = {}
        for w, p in zip(words.tolist(), poss.tolist()):
            want.setdefault(w, []).append(p)
        present = np.flatnonzero(np.diff(cs.astype(np.int64)))
        assert sorted(want) == present.tolist(), f"query {i}: words with hits differ"
        for w, lst in want.items():
            got = offs[cs[w]:cs[w + 1]].astype(np.int64)
            assert np.all(np.diff(got) > 0)
            assert got.tolist() == sorted(lst), (i, w)
        assert int(cs[-1]) == len(words)
