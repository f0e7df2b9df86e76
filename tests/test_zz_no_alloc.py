"""GPU test of blaze_gapped_noalloc, the gapped stage that allocates nothing.

It is for callers that cannot call cudaMalloc (an application whose allocator
owns the device heap, or code that must not risk the device-wide
synchronization of cudaMalloc/cudaFree). Here the test itself plays that
caller: it holds every input and output in its own device buffers (torch
tensors) and passes the pointers through the C ABI. The init hits come from
the regular entry point's diagnostics on the same database, and the HSPs must
equal the regular entry point's, bit for bit, on two calls in a row.

The second test hands the entry point input that breaks its stated limits --
a subject longer than the declared maximum, duplicated init hits, an init hit
reaching past its subject -- and checks that the device skips exactly those
(with their status bits) and leaves every other subject's HSPs unchanged.
Every out-of-range coordinate used here still points inside the test's own
buffers, so the checks are exercised without any access outside them.

This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_SUBJECT = 4096  # BLAZE_NOALLOC_MAX_SUBJECT_LENGTH
MAX_INIT = 128      # BLAZE_NOALLOC_MAX_INIT_HITS
OUTPUT_CUT, TOO_MANY_INIT, SUBJECT_TOO_LONG, BAD_INIT_HIT = 4, 16, 32, 64
COLS = ["oid", "score", "q_start", "q_end", "s_start", "s_end", "q_gapped_start", "s_gapped_start"]


def _workload(long_subject: int = 0):
    """Query and a length-sorted database; with long_subject > 0 one more
    subject of that length (carrying a planted homolog) is appended last."""
    from blaze103 import synth

    rng = np.random.default_rng(31)
    q = synth.random_residues(rng, 320)
    lengths = np.sort(synth.lognormal_lengths(rng, 6000, 250, 0.82, 30, MAX_SUBJECT))
    seqs = [synth.random_residues(rng, int(L)) for L in lengths]
    if long_subject:
        seqs.append(synth.random_residues(rng, long_subject))
        planted = list(rng.choice(len(seqs) - 1, size=300, replace=False)) + [len(seqs) - 1]
    else:
        planted = rng.choice(len(seqs), size=300, replace=False)
    for i in planted:
        w = int(rng.integers(60, 300))
        s0 = int(rng.integers(0, len(q) - w + 1))
        hom = synth.mutate(rng, q[s0:s0 + w], float(rng.uniform(0.35, 0.7)))[: len(seqs[i])]
        p = int(rng.integers(0, len(seqs[i]) - len(hom) + 1))
        seqs[i] = seqs[i].copy()
        seqs[i][p:p + len(hom)] = hom
    off = np.zeros(len(seqs) + 1, dtype=np.uint64)
    off[1:] = np.cumsum([len(s) for s in seqs])
    return q, np.concatenate(seqs), off


def _regular(q, res, off):
    """The regular entry point's HSPs and init hits (every HSP kept)."""
    import blaze103

    db = blaze103.SeqSrc(res, off)
    ps = blaze103.PrelimSearch(db)
    p = blaze103.default_params(len(q), db)
    p.prelim_evalue = 1e300  # keep every HSP: the no-alloc stage reports raw HSPs
    query = blaze103.Query(db, q)
    ps.run_query(query, p)
    want = ps.results()
    init = ps.init_hits()
    query.close()
    ps.close()
    db.close()
    return p, want, init


def _groups(init):
    """Init hits as the entry point takes them, grouped by subject (the
    database is length-sorted, so subject index == OID)."""
    oids, first, counts = np.unique(init["oid"], return_index=True, return_counts=True)
    hits = np.stack([init["q_start"], init["s_start"], init["length"], init["score"],
                     init["q_trigger"], init["s_trigger"]], axis=1).astype(np.int32)
    groups = np.zeros(len(oids), dtype=[("subject", "<u4"), ("n", "<u4"), ("first", "<u8")])
    groups["subject"], groups["n"], groups["first"] = oids, counts, first
    return hits, groups


class _Caller:
    """A caller holding everything in its own device buffers."""

    def __init__(self, q, res, off, cap):
        import torch

        import blaze103

        self.torch = torch
        dev = torch.device("cuda", 0)
        self.dev = dev
        self.d_res = torch.from_numpy(res.copy()).to(dev)
        self.d_off = torch.from_numpy(off.view(np.int64).copy()).to(dev)
        self.d_q = torch.from_numpy(np.asarray(q, dtype=np.uint8).copy()).to(dev)
        self.qlen = len(q)
        self.cap = cap
        self.d_out = torch.zeros((cap, 8), dtype=torch.int32, device=dev)
        self.d_result = torch.zeros(2, dtype=torch.int64, device=dev)
        L = blaze103.load()
        fn = L.blaze_gapped_noalloc
        vp = ctypes.c_void_p
        fn.argtypes = [vp, vp, ctypes.c_uint32, vp, ctypes.c_int32, vp, vp, ctypes.c_uint32,
                       ctypes.c_uint32, ctypes.POINTER(blaze103.BlazeParams), vp, ctypes.c_uint64,
                       vp, vp]
        fn.restype = ctypes.c_int
        self.fn = fn
        self.stream = torch.cuda.current_stream(dev)

    def call(self, hits, groups, max_len, max_init, p):
        """Returns (status, HSP rows ordered by subject, flags)."""
        import blaze103

        torch = self.torch
        d_hits = torch.from_numpy(np.ascontiguousarray(hits)).to(self.dev)
        d_groups = torch.from_numpy(np.ascontiguousarray(groups).view(np.uint8).copy()).to(self.dev)
        self.d_out.fill_(-1)
        st = self.fn(self.d_res.data_ptr(), self.d_off.data_ptr(), max_len, self.d_q.data_ptr(), self.qlen,
                     d_hits.data_ptr(), d_groups.data_ptr(), len(groups), max_init, ctypes.byref(p),
                     self.d_out.data_ptr(), self.cap, self.d_result.data_ptr(),
                     ctypes.c_void_p(self.stream.cuda_stream))
        if st != 0:
            return st, None, None
        self.stream.synchronize()
        n, flags = (int(x) for x in self.d_result.cpu())
        assert n <= self.cap, blaze103.status_string(st)
        got = self.d_out[:n].cpu().numpy()
        # subjects come out in any order; each subject's list is in final order
        return st, got[np.argsort(got[:, 0], kind="stable")], flags


def _assert_equal(got, want, what):
    assert len(got) == len(want), (what, len(got), len(want))
    for j, c in enumerate(COLS):
        assert np.array_equal(got[:, j].astype(np.int64), want[c].astype(np.int64)), (what, c)


def test_gapped_noalloc_matches_regular_entry_point():
    pytest.importorskip("torch")
    q, res, off = _workload()
    p, want, init = _regular(q, res, off)
    assert len(want) > 50 and len(init) > len(want)
    hits, groups = _groups(init)
    assert groups["n"].max() <= MAX_INIT
    caller = _Caller(q, res, off, len(want) + 64)
    max_len = int((off[1:] - off[:-1]).max())
    for call in range(2):
        st, got, flags = caller.call(hits, groups, max_len, int(groups["n"].max()), p)
        assert st == 0
        assert flags == 0, (call, flags)
        _assert_equal(got, want, f"call {call}")

    # sizes beyond the stated maxima are refused before any work is queued
    st, _, _ = caller.call(hits, groups, MAX_SUBJECT + 1, int(groups["n"].max()), p)
    assert st == 6  # BLAZE_ERR_LIMIT
    st, _, _ = caller.call(hits, groups, max_len, MAX_INIT + 1, p)
    assert st == 6


def test_gapped_noalloc_skips_input_beyond_its_limits():
    pytest.importorskip("torch")
    # one subject of 4,100 residues: the regular path searches it, the
    # allocation-free stage must skip it (declared maximum 4,096)
    q, res, off = _workload(long_subject=MAX_SUBJECT + 4)
    long_oid = len(off) - 2
    p, want, init = _regular(q, res, off)
    hits, groups = _groups(init)
    assert long_oid in set(groups["subject"].tolist()), "the long subject has init hits"
    assert long_oid in set(want["oid"].tolist()), "the long subject has HSPs on the regular path"
    want_short = want[want["oid"] != long_oid]
    caller = _Caller(q, res, off, len(want) + 64)
    max_init = int(groups["n"].max())

    # 1. the long subject is skipped and reported; nothing else changes
    for call in range(2):
        st, got, flags = caller.call(hits, groups, MAX_SUBJECT, max_init, p)
        assert st == 0
        assert flags == SUBJECT_TOO_LONG, (call, flags)
        _assert_equal(got, want_short, f"long subject, call {call}")

    short = groups[groups["subject"] != long_oid]

    # 2. every init hit given twice (equal records): the ordering must stay
    # total, and a repeated hit is contained in its twin's HSP, so the output
    # equals the regular one, on two calls in a row
    dup = np.concatenate([hits, hits])
    gdup = short.copy()
    gdup["n"] = 2 * short["n"]
    # group i now takes its records twice: rebuild a layout where a subject's
    # original and repeated records are contiguous
    order, firsts, pos = [], [], 0
    for g in short:
        idx = list(range(int(g["first"]), int(g["first"] + g["n"])))
        order += idx + [i + len(hits) for i in idx]
        firsts.append(pos)
        pos += 2 * int(g["n"])
    dup = dup[np.array(order)]
    gdup["first"] = firsts
    assert int(gdup["n"].max()) <= MAX_INIT
    for call in range(2):
        st, got, flags = caller.call(dup, gdup, MAX_SUBJECT, int(gdup["n"].max()), p)
        assert st == 0
        assert flags == 0, (call, flags)
        _assert_equal(got, want_short, f"duplicated init hits, call {call}")

    # 3. one init hit reaching two residues past the end of its subject (a
    # subject in the middle of the database, so the bytes past it are the
    # next subject's): that hit is skipped and reported
    g0 = short[len(short) // 2]
    bad = hits.copy()
    k = int(g0["first"])
    slen = int(off[g0["subject"] + 1] - off[g0["subject"]])
    bad[k, 2] = slen - int(bad[k, 1]) + 2  # length so that s_start + length = slen + 2
    st, got, flags = caller.call(bad, short, MAX_SUBJECT, max_init, p)
    assert st == 0
    assert flags == BAD_INIT_HIT, flags
    others = got[got[:, 0] != int(g0["subject"])]
    _assert_equal(others, want_short[want_short["oid"] != int(g0["subject"])], "bad init hit")
