"""Golden vectors of the word lookup made by the REFERENCE's own code.

    python tests/golden/make_ref_lookup.py

Builds oracle/_ref/libblaze_ref.so from the reference checkout (its
BLAZE_gpu sources, compiled where they lie by `make -C oracle ref`), then
writes ref_lookup.npz here:

* the reference's neighbourhood of every one of the 28^3 words
  (neighbouring_words, BLAZE_gpu/util.hpp:64-85: every other word scoring
  >= 11 under its BLOSUM62 copy, util.hpp:30-57) -- the full lists for
  600 seeded words over the 20 standard residues, and per word its count
  and an order-free checksum for all 21,952;
* for a few seeded queries (3 to 1,000 residues, including rare codes), the
  per-word lists of query offsets that BLAZE_ncbi/prelim_stage.cpp:360-386
  builds from those neighbourhoods (kmerIndex: each query word's offsets;
  kmerNeighbours: a word's own offsets, then its offsets appended to each of
  its neighbours), as (word, offset) pairs in the reference's order;
* its BLOSUM62 copy, and whether the copy the engine uses
  (BLAZE_ncbi/prelim_stage.cpp:69-96, read from that file's text) has the
  same scores for every pair of residue codes 1..27 (the two differ only in
  the sentinel row and column 0).

The kmerIndex/kmerNeighbours loops are restated here in Python from
prelim_stage.cpp:360-386 (that file needs the whole NCBI tree to compile);
the neighbourhoods, which hold all the arithmetic, come from the compiled
reference. tests/test_ref_lookup.py compares the oracle's lookup with these.
"""
import ctypes
import os
import re
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("BLAZE_REF", "/root/reference")
sys.path[:0] = [ROOT, os.path.join(ROOT, "blaze-sc-ad_gb300")]

from blaze103 import synth  # noqa: E402

A = 28
WORDS = A ** 3


def load_ref():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={REF}"], check=True)
    L = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libblaze_ref.so"))
    L.ref_neighbouring_words.argtypes = [ctypes.c_int] * 3 + [ctypes.POINTER(ctypes.c_int), ctypes.c_int]
    L.ref_neighbouring_words.restype = ctypes.c_int
    L.ref_score.argtypes = [ctypes.c_int, ctypes.c_int]
    L.ref_score.restype = ctypes.c_int
    return L


def neighbours(L):
    buf = (ctypes.c_int * WORDS)()
    out = []
    for w in range(WORDS):
        n = L.ref_neighbouring_words(w // (A * A), (w // A) % A, w % A, buf, WORDS)
        out.append(np.array(buf[:n], dtype=np.int64))
    return out


def engine_matrix_text():
    """BLAZE_ncbi/prelim_stage.cpp's score_matrix initializer, as numbers."""
    src = open(os.path.join(REF, "BLAZE_ncbi", "prelim_stage.cpp")).read()
    m = re.search(r"int\s+score_matrix\s*\[\s*28\s*\]\s*\[\s*28\s*\]\s*=\s*\{(.*?)\};", src, re.S)
    vals = [int(x) for x in re.findall(r"-?\d+", m.group(1))]
    return np.array(vals, dtype=np.int64).reshape(A, A)


def checksum(words) -> int:
    """Order-free 32-bit checksum of a list of word indices."""
    return int(((np.asarray(words, dtype=np.uint64) + 1) * np.uint64(2654435761)).sum() % (1 << 32))


def ref_query_lists(query, nbr):
    """(word, offset) pairs of kmerNeighbours, in the reference's order."""
    kmer_index = {}
    for i in range(2, len(query)):
        w = int(query[i - 2]) * A * A + int(query[i - 1]) * A + int(query[i])
        kmer_index.setdefault(w, []).append(i - 2)
    lists = {}
    for w in sorted(kmer_index):
        lists.setdefault(w, []).extend(kmer_index[w])
        for nb in nbr[w].tolist():
            lists.setdefault(nb, []).extend(kmer_index[w])
    words, offs = [], []
    for w in sorted(lists):
        words += [w] * len(lists[w])
        offs += lists[w]
    return np.array(words, dtype=np.int32), np.array(offs, dtype=np.int32)


def main():
    L = load_ref()
    nbr = neighbours(L)
    mat = np.array([[L.ref_score(a, b) for b in range(A)] for a in range(A)], dtype=np.int64)
    eng = engine_matrix_text()
    same = bool(np.array_equal(mat[1:, 1:], eng[1:, 1:]))
    counts = np.array([len(x) for x in nbr], dtype=np.uint16)
    csum = np.array([checksum(x) for x in nbr], dtype=np.uint32)
    std = synth.STD_CODES.astype(np.int64)
    all_std = np.array(sorted(int(a) * A * A + int(b) * A + int(c) for a in std for b in std for c in std))
    std_words = np.sort(np.random.default_rng(7).choice(all_std, size=600, replace=False)).astype(np.int32)
    std_lists = [nbr[w] for w in std_words]
    std_off = np.zeros(len(std_words) + 1, dtype=np.int64)
    np.cumsum([len(x) for x in std_lists], out=std_off[1:])
    rng = np.random.default_rng(2024)
    queries = [synth.random_residues(rng, L_) for L_ in (3, 40, 300, 1000)]
    # rare codes: B(2) Z(23) X(21) U(24) O(26) J(27) * (25) in a short query
    rare = synth.random_residues(rng, 200)
    rare[::9] = np.array([2, 23, 21, 24, 26, 27, 25], dtype=np.uint8)[np.arange(len(rare[::9])) % 7]
    queries.append(rare)
    q_off = np.zeros(len(queries) + 1, dtype=np.int64)
    np.cumsum([len(q) for q in queries], out=q_off[1:])
    pairs = [ref_query_lists(q, nbr) for q in queries]
    p_off = np.zeros(len(queries) + 1, dtype=np.int64)
    np.cumsum([len(w) for w, _ in pairs], out=p_off[1:])
    np.savez_compressed(
        os.path.join(HERE, "ref_lookup.npz"),
        matrix=mat, engine_matrix_same=np.array(same), counts=counts, checksums=csum,
        std_words=std_words, std_offsets=std_off, std_neighbours=np.concatenate(std_lists).astype(np.uint16),
        queries=np.concatenate(queries).astype(np.uint8), query_offsets=q_off,
        pair_words=np.concatenate([w for w, _ in pairs]).astype(np.uint16),
        pair_offsets=np.concatenate([o for _, o in pairs]).astype(np.uint16),
        pair_bounds=p_off)
    print(f"ref_lookup.npz: {counts.sum()} neighbours over {WORDS} words; engine matrix same: {same}; "
          f"{p_off[-1]} (word, offset) pairs over {len(queries)} queries")


if __name__ == "__main__":
    main()
