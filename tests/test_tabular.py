"""Tabular output (-outfmt 6/7) from traced HSP records (CPU): columns,
1-based ranges, percent identity, hit order by best E-value, and the E-value
and bit-score text rules."""
import numpy as np

from blaze103 import tabular
from blaze103._lib import ALIGNED_DTYPE


def _rec(rows):
    out = np.zeros(len(rows), dtype=ALIGNED_DTYPE)
    for i, r in enumerate(rows):
        for k, v in r.items():
            out[i][k] = v
    return out


def test_number_text():
    assert tabular.evalue_text(0.0) == "0.0"
    assert tabular.evalue_text(1e-200) == "0.0"
    assert tabular.evalue_text(3.2e-120) == "3e-120"
    assert tabular.evalue_text(4.6e-12) == "5e-12"
    assert tabular.evalue_text(0.0123) == "0.012"
    assert tabular.evalue_text(0.5) == "0.50"
    assert tabular.evalue_text(3.14) == "3.1"
    assert tabular.evalue_text(12.6) == "   13"
    assert tabular.bitscore_text(1234.5) == "1234"
    assert tabular.bitscore_text(55.27) == "55.3"
    assert tabular.bitscore_text(12346.0) == "1.235e+04"


def test_outfmt6_rows_and_order():
    a = _rec([
        dict(oid=2, score=60, q_start=0, q_end=50, s_start=10, s_end=58, length=52, identities=26, mismatches=24,
             gap_opens=1, gaps=2, evalue=1e-5, bit_score=27.5),
        dict(oid=5, score=200, q_start=4, q_end=104, s_start=0, s_end=100, length=100, identities=100,
             mismatches=0, gap_opens=0, gaps=0, evalue=1e-50, bit_score=181.2),
        dict(oid=5, score=40, q_start=200, q_end=230, s_start=300, s_end=330, length=30, identities=12,
             mismatches=18, gap_opens=0, gaps=0, evalue=0.3, bit_score=20.0),
    ])
    text = tabular.format_tabular(a, "q1", lambda oid: f"sub{oid}")
    lines = text.splitlines()
    assert lines[0].split("\t") == ["q1", "sub5", "100.000", "100", "0", "0", "5", "104", "1", "100", "1e-50",
                                    "181"]
    assert lines[1].split("\t")[1] == "sub5" and lines[1].split("\t")[10] == "0.30"
    assert lines[2].split("\t") == ["q1", "sub2", "50.000", "52", "24", "1", "1", "50", "11", "58", "1e-05",
                                    "27.5"]


def test_outfmt7_header():
    text = tabular.format_tabular(_rec([]), "q9", ["a"], outfmt=7, database="db")
    assert text.splitlines() == ["# BLASTP", "# Query: q9", "# Database: db", "# 0 hits found"]
