"""BLAST tabular output (-outfmt 6, and 7 with comment lines) from traced
HSPs (ALIGNED_DTYPE records of PrelimSearch.traceback).

Columns (the default outfmt 6 set): qseqid sseqid pident length mismatch
gapopen qstart qend sstart send evalue bitscore -- 1-based inclusive ranges,
percent identity over the aligned columns. Hits are listed by their best
E-value (ties: higher score, then smaller OID), a subject's HSPs in the
traceback order. The E-value and bit-score text follows the conventions of
BLAST's tabular formatter (fewer digits for smaller E-values, "0.0" below
1e-180, integer bit scores above 99.9); the reference formats through NCBI's
own formatter, which is absent here, so this layout is unpinned.
"""
from __future__ import annotations

import numpy as np

FIELDS_LINE = ("# Fields: query acc.ver, subject acc.ver, % identity, alignment length, mismatches, gap opens, "
               "q. start, q. end, s. start, s. end, evalue, bit score")


def evalue_text(e: float) -> str:
    if e < 1.0e-180:
        return "0.0"
    if e < 1.0e-99:
        return f"{e:2.0e}"
    if e < 0.0009:
        return f"{e:3.0e}"
    if e < 0.1:
        return f"{e:4.3f}"
    if e < 1.0:
        return f"{e:3.2f}"
    if e < 10.0:
        return f"{e:2.1f}"
    return f"{e:5.0f}"


def bitscore_text(b: float) -> str:
    if b > 9999:
        return f"{b:4.3e}"
    if b > 99.9:
        return f"{int(b):3d}"
    return f"{b:4.1f}"


def ordered(aligned: np.ndarray) -> np.ndarray:
    """Subjects by best E-value (ties: higher score, then smaller OID); each
    subject's HSPs in the order given."""
    if len(aligned) == 0:
        return aligned
    oids = aligned["oid"]
    starts = np.flatnonzero(np.r_[True, oids[1:] != oids[:-1]])
    ends = np.r_[starts[1:], len(aligned)]
    keys = [(float(aligned["evalue"][s:e].min()), -int(aligned["score"][s:e].max()), int(oids[s]), s, e)
            for s, e in zip(starts, ends)]
    keys.sort()
    return np.concatenate([aligned[s:e] for *_, s, e in keys])


def format_tabular(aligned: np.ndarray, query_id: str, subject_id, outfmt: int = 6,
                   database: str | None = None, program: str = "BLASTP") -> str:
    """Text of -outfmt 6 (or 7). subject_id maps an OID to its identifier
    (a callable, or a sequence indexed by OID)."""
    sid = subject_id if callable(subject_id) else (lambda oid: subject_id[oid])
    rows = ordered(aligned)
    lines = []
    if outfmt == 7:
        lines.append(f"# {program}")
        lines.append(f"# Query: {query_id}")
        if database:
            lines.append(f"# Database: {database}")
        if len(rows):
            lines.append(FIELDS_LINE)
        lines.append(f"# {len(rows)} hits found")
    elif outfmt != 6:
        raise ValueError("outfmt must be 6 or 7")
    for r in rows:
        length = int(r["length"])
        pident = 100.0 * int(r["identities"]) / length if length else 0.0
        lines.append("\t".join([
            query_id, str(sid(int(r["oid"]))), f"{pident:.3f}", str(length), str(int(r["mismatches"])),
            str(int(r["gap_opens"])), str(int(r["q_start"]) + 1), str(int(r["q_end"])), str(int(r["s_start"]) + 1),
            str(int(r["s_end"])), evalue_text(float(r["evalue"])), bitscore_text(float(r["bit_score"]))]))
    return "\n".join(lines) + ("\n" if lines else "")
