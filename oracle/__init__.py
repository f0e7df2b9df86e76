"""ctypes binding of the CPU oracle (oracle/blaze_oracle.c).

Test infrastructure only: tests/, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of bench.py may call it, as the
checker. The product library never imports it.

Parity against NCBI BLAST+ 2.13.0 is unpinned (its sources are not vendored in
the reference and no golden vectors exist); see blaze_oracle.h.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")

HSP_DTYPE = np.dtype([
    ("subject", "<u4"), ("score", "<i4"), ("q_start", "<i4"), ("q_end", "<i4"),
    ("s_start", "<i4"), ("s_end", "<i4"), ("q_gstart", "<i4"), ("s_gstart", "<i4"),
])
INIT_DTYPE = np.dtype([
    ("subject", "<u4"), ("q_start", "<i4"), ("s_start", "<i4"), ("len", "<i4"),
    ("score", "<i4"), ("q_trig", "<i4"), ("s_trig", "<i4"),
])


class OrcParams(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in (
        "word_threshold", "window", "ungapped_xdrop", "ungapped_cutoff",
        "gap_open", "gap_extend", "gapped_xdrop", "gapped_cutoff")]


class OrcLookup(ctypes.Structure):
    _fields_ = [("cell_start", ctypes.POINTER(ctypes.c_uint32)),
                ("offsets", ctypes.POINTER(ctypes.c_uint32)),
                ("n_offsets", ctypes.c_uint32)]


_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, no GPU needed)."""
    if force or not os.path.exists(_LIB_PATH):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        u8p = ctypes.POINTER(ctypes.c_uint8)
        i32p = ctypes.POINTER(ctypes.c_int32)
        L.orc_lookup_build.argtypes = [u8p, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(OrcLookup)]
        L.orc_lookup_build.restype = ctypes.c_int
        L.orc_lookup_free.argtypes = [ctypes.POINTER(OrcLookup)]
        L.orc_search_db.argtypes = [u8p, ctypes.c_int32, u8p, ctypes.POINTER(ctypes.c_uint64),
                                    ctypes.c_uint32, ctypes.POINTER(OrcParams), ctypes.c_int32,
                                    ctypes.c_int32]
        L.orc_search_db.restype = ctypes.c_void_p
        L.orc_result_n_hsps.argtypes = [ctypes.c_void_p]
        L.orc_result_n_hsps.restype = ctypes.c_uint64
        L.orc_result_n_inits.argtypes = [ctypes.c_void_p]
        L.orc_result_n_inits.restype = ctypes.c_uint64
        L.orc_result_copy_hsps.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.orc_result_copy_inits.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.orc_result_free.argtypes = [ctypes.c_void_p]
        L.orc_semi_gapped.argtypes = [u8p, u8p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                      ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, i32p, i32p]
        L.orc_semi_gapped.restype = ctypes.c_int32
        L.orc_traceback.argtypes = [u8p, ctypes.c_int32, u8p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                    ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(OrcTb)]
        L.orc_traceback.restype = ctypes.c_int
        L.orc_traceback_ops.argtypes = L.orc_traceback.argtypes + [ctypes.c_char_p, ctypes.c_int32,
                                                                   ctypes.POINTER(ctypes.c_int32)]
        L.orc_traceback_ops.restype = ctypes.c_int
        L.orc_gapped_start.argtypes = [u8p, u8p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]
        L.orc_gapped_start.restype = ctypes.c_int32
        L.orc_evalue.argtypes = [ctypes.c_int32, ctypes.c_double, ctypes.c_double, ctypes.c_double]
        L.orc_evalue.restype = ctypes.c_double
        L.orc_length_adjustment.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                            ctypes.c_double, ctypes.c_int32, ctypes.c_int64,
                                            ctypes.c_int64]
        L.orc_length_adjustment.restype = ctypes.c_int32
        _lib = L
    return _lib


def _u8(a):
    a = np.ascontiguousarray(a, dtype=np.uint8)
    return a, a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))


def make_params(p) -> OrcParams:
    """p: mapping or object with the eight search parameters."""
    get = (lambda k: p[k]) if isinstance(p, dict) else (lambda k: getattr(p, k))
    return OrcParams(*[int(get(n)) for n, _ in OrcParams._fields_])


def lookup(query, threshold: int = 11):
    """Return (cell_start[21953], offsets) of the oracle's word lookup."""
    q, qp = _u8(query)
    lk = OrcLookup()
    if lib().orc_lookup_build(qp, len(q), threshold, ctypes.byref(lk)) != 0:
        raise MemoryError("oracle lookup build failed")
    try:
        cs = np.ctypeslib.as_array(lk.cell_start, shape=(21953,)).copy()
        n = lk.n_offsets
        offs = np.ctypeslib.as_array(lk.offsets, shape=(max(n, 1),))[:n].copy()
    finally:
        lib().orc_lookup_free(ctypes.byref(lk))
    return cs, offs


def search_db(query, residues, offsets, params, threads: int = 1, want_inits: bool = False):
    """Run the oracle over a whole database; returns (hsps, inits) record arrays
    ordered by subject index."""
    q, qp = _u8(query)
    r, rp = _u8(residues)
    o = np.ascontiguousarray(offsets, dtype=np.uint64)
    prm = make_params(params)
    L = lib()
    h = L.orc_search_db(qp, len(q), rp, o.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                        len(o) - 1, ctypes.byref(prm), int(threads), int(bool(want_inits)))
    if not h:
        raise MemoryError("oracle search failed")
    try:
        hs = np.zeros(L.orc_result_n_hsps(h), dtype=HSP_DTYPE)
        L.orc_result_copy_hsps(h, hs.ctypes.data)
        ini = np.zeros(L.orc_result_n_inits(h), dtype=INIT_DTYPE)
        L.orc_result_copy_inits(h, ini.ctypes.data)
    finally:
        L.orc_result_free(h)
    return hs, ini


def semi_gapped(A, B, M, N, reverse, gap_open=11, gap_extend=1, xdrop=38):
    a, ap = _u8(A if len(A) else [0])
    b, bp = _u8(B if len(B) else [0])
    ab, bb = ctypes.c_int32(), ctypes.c_int32()
    s = lib().orc_semi_gapped(ap, bp, M, N, int(reverse), gap_open, gap_extend, xdrop,
                              ctypes.byref(ab), ctypes.byref(bb))
    return s, ab.value, bb.value


class OrcTb(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in (
        "score", "q_start", "q_end", "s_start", "s_end", "length", "identities", "positives", "mismatches",
        "gap_opens", "gaps")]


TB_FIELDS = [n for n, _ in OrcTb._fields_]
FINAL_XDROP = 64  # NCBI blastp gap_x_dropoff_final: 25 bits at lambda 0.267


def traceback(query, subject, q_off, s_off, gap_open=11, gap_extend=1, xdrop=FINAL_XDROP) -> dict:
    """Traceback of one HSP from its gapped start point (orc_traceback)."""
    q, qp = _u8(query if len(query) else [0])
    t, tp = _u8(subject if len(subject) else [0])
    out = OrcTb()
    rc = lib().orc_traceback(qp, len(query), tp, len(subject), int(q_off), int(s_off), gap_open, gap_extend,
                             xdrop, ctypes.byref(out))
    if rc != 0:
        raise RuntimeError("oracle traceback failed")
    return {n: getattr(out, n) for n in TB_FIELDS}


def traceback_ops(query, subject, q_off, s_off, gap_open=11, gap_extend=1, xdrop=FINAL_XDROP):
    """(stats, moves) of one traceback; moves in query order as 'M'/'I'/'D'."""
    q, qp = _u8(query if len(query) else [0])
    t, tp = _u8(subject if len(subject) else [0])
    out = OrcTb()
    cap = 2 * (len(query) + len(subject)) + 8
    buf = ctypes.create_string_buffer(cap)
    n = ctypes.c_int32()
    rc = lib().orc_traceback_ops(qp, len(query), tp, len(subject), int(q_off), int(s_off), gap_open, gap_extend,
                                 xdrop, ctypes.byref(out), buf, cap, ctypes.byref(n))
    if rc != 0:
        raise RuntimeError("oracle traceback failed")
    return {n_: getattr(out, n_) for n_ in TB_FIELDS}, buf.raw[: n.value].decode()


def traceback_hsps(query, residues, offsets, hsps, params, xdrop=FINAL_XDROP, evalue=None) -> list:
    """The traceback stage over a preliminary result (records with
    'subject', 'q_gstart', 's_gstart'): every HSP traced from its start
    point, then per subject duplicates purged and the list sorted as in the
    preliminary stage, E-values from the final scores and the reap at
    `evalue` (default: the parameters' preliminary E-value). Returns dicts
    with 'subject' and 'evalue' added, by subject then final order."""
    get = (lambda k: params[k]) if isinstance(params, dict) else (lambda k: getattr(params, k))
    lam = get("lam") if isinstance(params, dict) else params.lambda_
    K, ss = get("K"), get("eff_searchsp")
    cut = get("prelim_evalue") if evalue is None else evalue
    out = []
    subs = hsps["subject"].tolist()
    i = 0
    while i < len(subs):
        j = i
        while j < len(subs) and subs[j] == subs[i]:
            j += 1
        sub = subs[i]
        S = residues[int(offsets[sub]):int(offsets[sub + 1])]
        traced = []
        for k in range(i, j):
            r = traceback(query, S, int(hsps["q_gstart"][k]), int(hsps["s_gstart"][k]), get("gap_open"),
                          get("gap_extend"), xdrop)
            r["subject"] = sub
            traced.append(r)
        kept = _purge_and_sort(traced)
        for r in kept:
            r["evalue"] = ss * K * float(np.exp(-lam * r["score"]))
            if r["evalue"] <= cut:
                out.append(r)
        i = j
    return out


def _purge_and_sort(hs: list) -> list:
    """Same rules as the preliminary stage's purge and final order."""
    by_start = sorted(hs, key=lambda h: (h["q_start"], h["s_start"], -h["score"], -h["q_end"], -h["s_end"]))
    m = []
    for h in by_start:
        if not m or h["q_start"] != m[-1]["q_start"] or h["s_start"] != m[-1]["s_start"]:
            m.append(h)
    by_end = sorted(m, key=lambda h: (h["q_end"], h["s_end"], -h["score"], h["q_start"], h["s_start"]))
    m = []
    for h in by_end:
        if not m or h["q_end"] != m[-1]["q_end"] or h["s_end"] != m[-1]["s_end"]:
            m.append(h)
    return sorted(m, key=lambda h: (-h["score"], h["s_start"], -h["s_end"], h["q_start"], -h["q_end"]))


def gapped_start(q, s, q_start, s_start, length):
    a, ap = _u8(q)
    b, bp = _u8(s)
    return lib().orc_gapped_start(ap, bp, q_start, s_start, length)


def evalue(score, lam, K, searchsp):
    return lib().orc_evalue(int(score), float(lam), float(K), float(searchsp))


def length_adjustment(K, logK, alpha_d_lambda, beta, qlen, db_len, db_n):
    return lib().orc_length_adjustment(K, logK, alpha_d_lambda, beta, int(qlen), int(db_len), int(db_n))


# BLOSUM62 / gap 11,1 Karlin-Altschul constants (published NCBI table values)
KA_UNGAPPED = dict(lam=0.3176, K=0.134)
KA_GAPPED = dict(lam=0.267, K=0.041, alpha=1.9, beta=-30.0)


def default_params(qlen: int, db_len: int, db_n: int, evalue: float = 10.0) -> dict:
    """NCBI blastp default parameters restated in Python for the oracle."""
    import math
    ln2 = math.log(2.0)
    g, u = KA_GAPPED, KA_UNGAPPED
    ell = length_adjustment(g["K"], math.log(g["K"]), g["alpha"] / g["lam"], g["beta"], qlen,
                            db_len, db_n)
    searchsp = max(qlen - ell, 1) * max(db_len - db_n * ell, 1)
    gapped_cutoff = max(int(math.ceil(math.log(g["K"] * searchsp / evalue) / g["lam"])), 1)
    gap_trigger = int((22.0 * ln2 + math.log(u["K"])) / u["lam"])
    return dict(word_threshold=11, window=40,
                ungapped_xdrop=int(math.ceil(7.0 * ln2 / u["lam"])),
                ungapped_cutoff=min(gap_trigger, gapped_cutoff), gap_open=11, gap_extend=1,
                gapped_xdrop=int(15.0 * ln2 / g["lam"]), gapped_cutoff=gapped_cutoff,
                lam=g["lam"], K=g["K"], eff_searchsp=float(searchsp), prelim_evalue=evalue,
                hitlist_size=0, max_hsps=0, length_adjustment=ell)


def finish(hsps: np.ndarray, params) -> np.ndarray:
    """E-values and the preliminary E-value reap of the oracle's HSPs
    (blast_engine.c:1441 and :1457 call sites). Returns a structured array with
    an extra 'evalue' field, keeping per-subject order."""
    get = (lambda k: params[k]) if isinstance(params, dict) else (lambda k: getattr(params, k))
    lam = get("lam") if isinstance(params, dict) else params.lambda_
    K, ss, cut = get("K"), get("eff_searchsp"), get("prelim_evalue")
    ev = ss * K * np.exp(-lam * hsps["score"].astype(np.float64))
    out = np.zeros(len(hsps), dtype=HSP_DTYPE.descr + [("evalue", "<f8")])
    for n in HSP_DTYPE.names:
        out[n] = hsps[n]
    out["evalue"] = ev
    out = out[ev <= cut]
    return cull(out, get("hitlist_size") if _has(params, "hitlist_size") else 0,
                get("max_hsps") if _has(params, "max_hsps") else 0)


def _has(params, key) -> bool:
    return key in params if isinstance(params, dict) else hasattr(params, key)


def cull(hsps: np.ndarray, hitlist_size: int = 0, max_hsps: int = 0) -> np.ndarray:
    """max_hsps: the first HSPs of each subject's list; hitlist_size: the
    subjects with the best E-values (their first HSP), ties by smaller
    subject index. Plain loops: test sizes only."""
    if max_hsps > 0:
        keep, seen = [], {}
        for i, sub in enumerate(hsps["subject"].tolist()):
            seen[sub] = seen.get(sub, 0) + 1
            if seen[sub] <= max_hsps:
                keep.append(i)
        hsps = hsps[np.array(keep, dtype=np.int64)]
    if hitlist_size > 0:
        best = {}
        for sub, sc in zip(hsps["subject"].tolist(), hsps["score"].tolist()):
            best.setdefault(sub, sc)  # first HSP of each subject
        ranked = sorted(best, key=lambda sub: (-best[sub], sub))[:hitlist_size]
        hsps = hsps[np.isin(hsps["subject"], np.array(ranked, dtype=hsps["subject"].dtype))]
    return hsps
