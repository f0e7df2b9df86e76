"""Seeded synthetic protein databases and queries for the five workload shapes
of the preliminary-search benchmarks (there is no network for real data, and
makeblastdb is not available: databases are written directly as residue
arrays plus offsets).

Residues are NCBIstdaa codes of the 20 standard amino acids drawn i.i.d. from
the Robinson-Robinson background frequencies. Subject lengths are log-normal
(median 250, sigma 0.82 so the mean is ~350), clipped, sorted ascending; the
overflow-stress workload's longest 0.1% are drawn uniformly up to its clip
(35,000), which the log-normal alone would not reach.
Planted homologs copy a 100-300 residue window of a query, substitute
residues toward a target identity using BLOSUM62 target frequencies
(q_ab ~ p_a p_b exp(lambda s_ab)), and insert/delete at 2% per residue with
geometric lengths of mean 3.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

# NCBIstdaa codes of A R N D C Q E G H I L K M F P S T W Y V
STD_CODES = np.array([1, 16, 13, 4, 3, 15, 5, 7, 8, 9, 11, 10, 12, 6, 14, 17, 18, 20, 22, 19],
                     dtype=np.uint8)
# Robinson & Robinson (1991) background frequencies, same residue order.
RR_FREQS = np.array([0.07805, 0.05129, 0.04487, 0.05364, 0.01925, 0.04264, 0.06295, 0.07377,
                     0.02199, 0.05142, 0.09019, 0.05744, 0.02243, 0.03856, 0.05203, 0.07120,
                     0.05841, 0.01330, 0.03216, 0.06441])
RR_FREQS = RR_FREQS / RR_FREQS.sum()
UNGAPPED_LAMBDA = 0.3176

_TABLE_BITS = 16
HOMOLOG_POOL = 100_000  # distinct mutants at most per database (see make_workload)


def _sampling_table() -> np.ndarray:
    """65536-entry table mapping a uniform uint16 to a residue code."""
    n = 1 << _TABLE_BITS
    counts = np.floor(RR_FREQS * n).astype(np.int64)
    counts[np.argmax(RR_FREQS)] += n - counts.sum()
    return np.repeat(STD_CODES, counts)


_TABLE = _sampling_table()


def random_residues(rng: np.random.Generator, n: int) -> np.ndarray:
    return _TABLE[rng.integers(0, 1 << _TABLE_BITS, size=int(n), dtype=np.uint16)]


def _blosum62() -> np.ndarray:
    from . import _blosum
    return _blosum.BLOSUM62


def _substitution_tables() -> np.ndarray:
    """cdf[a_code] over STD_CODES for a substituted residue (never a itself)."""
    m = _blosum62()
    cdf = np.zeros((28, len(STD_CODES)))
    for i, a in enumerate(STD_CODES):
        w = RR_FREQS * np.exp(UNGAPPED_LAMBDA * m[a, STD_CODES].astype(float))
        w[i] = 0.0
        cdf[a] = np.cumsum(w / w.sum())
    return cdf


_CDF = _substitution_tables()


def mutate(rng: np.random.Generator, seq: np.ndarray, identity: float, indel_rate: float = 0.02,
           indel_mean: float = 3.0) -> np.ndarray:
    seq = np.array(seq, dtype=np.uint8)
    cdf = _CDF
    sub = np.flatnonzero(rng.random(len(seq)) >= identity)
    u = rng.random(len(sub))
    j = (cdf[seq[sub]] <= u[:, None]).sum(axis=1)
    seq[sub] = STD_CODES[np.minimum(j, len(STD_CODES) - 1)]
    out = []
    i = 0
    events = np.flatnonzero(rng.random(len(seq)) < indel_rate)
    for e in events:
        if e < i:
            continue
        out.append(seq[i:e])
        glen = int(rng.geometric(1.0 / indel_mean))
        if rng.random() < 0.5:
            out.append(random_residues(rng, glen))
            i = e
        else:
            i = e + glen
    out.append(seq[i:])
    return np.concatenate(out) if out else seq[:0]


def lognormal_lengths(rng, n: int, median: float, sigma: float, lo: int, hi: int) -> np.ndarray:
    x = rng.lognormal(np.log(median), sigma, size=int(n))
    return np.clip(np.rint(x), lo, hi).astype(np.int64)


@dataclass
class Workload:
    name: str
    queries: list
    residues: np.ndarray
    offsets: np.ndarray
    planted: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int64))
    meta: dict = field(default_factory=dict)

    @property
    def n_subjects(self) -> int:
        return len(self.offsets) - 1

    @property
    def total_residues(self) -> int:
        return int(self.offsets[-1])


# The workloads the benchmark and tests draw (sizes at scale 1.0). Each has a
# fixed index, which is also its default random seed.
WORKLOADS = {
    "plain-small": dict(index=0, query_lengths=[300], n_subjects=20_000, clip=(30, 5000),
                        homolog_frac=0.01, identity=(0.40, 0.40), lowcomplex_frac=0.0),
    "plain-db-scale": dict(index=1, query_lengths=[100, 200, 300, 500, 700, 800, 900, 1000],
                           n_subjects=2_000_000, clip=(30, 5000), homolog_frac=0.01, identity=(0.40, 0.40),
                           lowcomplex_frac=0.0),
    "batched": dict(index=2, query_lengths=("lognormal", 512, 350, 50, 2000), n_subjects=5_000_000,
                    clip=(30, 5000), homolog_frac=0.10, identity=(0.40, 0.40), lowcomplex_frac=0.0),
    "overflow-stress": dict(index=3, query_lengths=("uniform", 64, 2000, 5000), n_subjects=500_000,
                            clip=(30, 35000), homolog_frac=0.25, identity=(0.30, 0.60), lowcomplex_frac=0.20,
                            long_tail=(0.001, 15_000, 35_000)),
    "serving": dict(index=4, query_lengths=("lognormal", 256, 350, 30, 5000), n_subjects=10_000_000,
                    clip=(30, 5000), homolog_frac=0.01, identity=(0.40, 0.40), lowcomplex_frac=0.0),
}
_BY_INDEX = {w["index"]: name for name, w in WORKLOADS.items()}


def _query_lengths(rng, spec) -> list:
    if isinstance(spec, (list, tuple)) and spec and spec[0] == "lognormal":
        _, n, med, lo, hi = spec
        return [int(x) for x in lognormal_lengths(rng, n, med, 0.82, lo, hi)]
    if isinstance(spec, (list, tuple)) and spec and spec[0] == "uniform":
        _, n, lo, hi = spec
        return [int(x) for x in rng.integers(lo, hi + 1, size=n)]
    return [int(x) for x in spec]


def make_workload(workload, scale: float = 1.0, seed: int | None = None,
                  n_queries: int | None = None, median: float = 250.0,
                  sigma: float = 0.82) -> Workload:
    """Build a workload (its name, or its index) with n_subjects scaled by `scale`."""
    name = _BY_INDEX[workload] if isinstance(workload, int) else workload
    c = dict(WORKLOADS[name])
    rng = np.random.default_rng(c["index"] if seed is None else seed)
    qlens = _query_lengths(rng, c["query_lengths"])
    if n_queries is not None:
        qlens = qlens[:n_queries]
    queries = [random_residues(rng, L) for L in qlens]
    n = max(int(round(c["n_subjects"] * scale)), 1)
    lo, hi = c["clip"]
    lengths = np.sort(lognormal_lengths(rng, n, median, sigma, lo, hi))
    if c.get("long_tail"):  # the longest subjects reach the clip: lengths uniform in [a, b]
        frac, a, b = c["long_tail"]
        n_long = int(round(frac * n))
        if n_long:
            lengths[n - n_long:] = np.sort(rng.integers(a, b + 1, size=n_long))
    offsets = np.zeros(n + 1, dtype=np.uint64)
    np.cumsum(lengths, out=offsets[1:])
    residues = random_residues(rng, int(offsets[-1]))
    # low-complexity runs: 50-200 residues over a 3-letter alphabet
    n_lc = int(round(c["lowcomplex_frac"] * n))
    for i in rng.choice(n, size=n_lc, replace=False) if n_lc else []:
        L = int(lengths[i])
        run = int(min(rng.integers(50, 201), L))
        letters = rng.choice(STD_CODES, size=3, replace=False)
        pos = int(offsets[i]) + int(rng.integers(0, L - run + 1))
        residues[pos:pos + run] = letters[rng.integers(0, 3, size=run)]
    # planted homologs; above kHomologPool of them (full-size databases with
    # many homologs), each planted subject takes a mutant drawn from a pool
    # of kHomologPool independently made ones, so building a 500,000-homolog
    # database stays a matter of seconds
    n_h = int(round(c["homolog_frac"] * n))
    planted = np.sort(rng.choice(n, size=n_h, replace=False)) if n_h else np.zeros(0, np.int64)
    id_lo, id_hi = c["identity"]

    def one_mutant():
        q = queries[int(rng.integers(0, len(queries)))]
        w = int(min(rng.integers(100, 301), len(q)))
        qs = int(rng.integers(0, len(q) - w + 1))
        return mutate(rng, q[qs:qs + w], float(rng.uniform(id_lo, id_hi)))

    pool = [one_mutant() for _ in range(HOMOLOG_POOL)] if n_h > HOMOLOG_POOL else None
    for i in planted:
        hom = pool[int(rng.integers(0, HOMOLOG_POOL))] if pool is not None else one_mutant()
        L = int(lengths[i])
        hom = hom[:L]
        pos = int(offsets[i]) + int(rng.integers(0, L - len(hom) + 1))
        residues[pos:pos + len(hom)] = hom
    return Workload(name=name, queries=queries, residues=residues, offsets=offsets,
                    planted=planted, meta=dict(workload=name, scale=scale, n_subjects=n,
                                              total_residues=int(offsets[-1])))
