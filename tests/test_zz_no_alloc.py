"""GPU test of blaze_gapped_noalloc, the gapped stage that allocates nothing.

It is for callers that cannot call cudaMalloc (an application whose allocator
owns the device heap, or code that must not risk the device-wide
synchronization of cudaMalloc/cudaFree). Here the test itself plays that
caller: it holds every input and output in its own device buffers (torch
tensors) and passes the pointers through the C ABI. The init hits come from
the regular entry point's diagnostics on the same database, and the HSPs must
equal the regular entry point's, bit for bit, on two calls in a row.

This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_SUBJECT = 4096  # BLAZE_NOALLOC_MAX_SUBJECT_LENGTH
MAX_INIT = 128      # BLAZE_NOALLOC_MAX_INIT_HITS


def _workload():
    from blaze103 import synth

    rng = np.random.default_rng(31)
    q = synth.random_residues(rng, 320)
    lengths = np.sort(synth.lognormal_lengths(rng, 6000, 250, 0.82, 30, MAX_SUBJECT))
    seqs = [synth.random_residues(rng, int(L)) for L in lengths]
    for i in rng.choice(len(seqs), size=300, replace=False):
        w = int(rng.integers(60, 300))
        s0 = int(rng.integers(0, len(q) - w + 1))
        hom = synth.mutate(rng, q[s0:s0 + w], float(rng.uniform(0.35, 0.7)))[: len(seqs[i])]
        p = int(rng.integers(0, len(seqs[i]) - len(hom) + 1))
        seqs[i] = seqs[i].copy()
        seqs[i][p:p + len(hom)] = hom
    off = np.zeros(len(seqs) + 1, dtype=np.uint64)
    off[1:] = np.cumsum([len(s) for s in seqs])
    return q, np.concatenate(seqs), off


def test_gapped_noalloc_matches_regular_entry_point():
    torch = pytest.importorskip("torch")
    import blaze103

    q, res, off = _workload()
    db = blaze103.SeqSrc(res, off)
    ps = blaze103.PrelimSearch(db)
    p = blaze103.default_params(len(q), db)
    p.prelim_evalue = 1e300  # keep every HSP: the no-alloc stage reports raw HSPs
    query = blaze103.Query(db, q)
    ps.run_query(query, p)
    want = ps.results()
    init = ps.init_hits()
    query.close()
    assert len(want) > 50 and len(init) > len(want)

    # init hits grouped by subject (the database is length-sorted, so subject
    # index == OID)
    oids, first, counts = np.unique(init["oid"], return_index=True, return_counts=True)
    assert counts.max() <= MAX_INIT
    hits = np.stack([init["q_start"], init["s_start"], init["length"], init["score"],
                     init["q_trigger"], init["s_trigger"]], axis=1).astype(np.int32)
    groups = np.zeros(len(oids), dtype=[("subject", "<u4"), ("n", "<u4"), ("first", "<u8")])
    groups["subject"], groups["n"], groups["first"] = oids, counts, first

    dev = torch.device("cuda", 0)
    d_res = torch.from_numpy(res.copy()).to(dev)
    d_off = torch.from_numpy(off.view(np.int64).copy()).to(dev)
    d_q = torch.from_numpy(np.asarray(q, dtype=np.uint8).copy()).to(dev)
    d_hits = torch.from_numpy(hits.copy()).to(dev)
    d_groups = torch.from_numpy(groups.view(np.uint8).copy()).to(dev)
    cap = len(want) + 64
    d_out = torch.zeros((cap, 8), dtype=torch.int32, device=dev)
    d_result = torch.zeros(2, dtype=torch.int64, device=dev)

    L = blaze103.load()
    fn = L.blaze_gapped_noalloc
    vp = ctypes.c_void_p
    fn.argtypes = [vp, vp, ctypes.c_uint32, vp, ctypes.c_int32, vp, vp, ctypes.c_uint32,
                   ctypes.c_uint32, ctypes.POINTER(blaze103.BlazeParams), vp, ctypes.c_uint64,
                   vp, vp]
    fn.restype = ctypes.c_int
    stream = torch.cuda.current_stream(dev)
    max_len = int((off[1:] - off[:-1]).max())

    for call in range(2):
        d_out.fill_(-1)
        st = fn(d_res.data_ptr(), d_off.data_ptr(), max_len, d_q.data_ptr(), len(q),
                d_hits.data_ptr(), d_groups.data_ptr(), len(oids), int(counts.max()),
                ctypes.byref(p), d_out.data_ptr(), cap, d_result.data_ptr(),
                ctypes.c_void_p(stream.cuda_stream))
        assert st == 0, blaze103.status_string(st)
        stream.synchronize()
        n, flags = (int(x) for x in d_result.cpu())
        assert flags == 0 and n == len(want), (call, n, flags, len(want))
        got = d_out[:n].cpu().numpy()
        # subjects come out in any order; each subject's list is in final order
        order = np.argsort(got[:, 0], kind="stable")
        got = got[order]
        cols = ["oid", "score", "q_start", "q_end", "s_start", "s_end", "q_gapped_start",
                "s_gapped_start"]
        for j, c in enumerate(cols):
            assert np.array_equal(got[:, j].astype(np.int64), want[c].astype(np.int64)), (call, c)

    # sizes beyond the stated maxima are refused before any work is queued
    st = fn(d_res.data_ptr(), d_off.data_ptr(), MAX_SUBJECT + 1, d_q.data_ptr(), len(q),
            d_hits.data_ptr(), d_groups.data_ptr(), len(oids), int(counts.max()),
            ctypes.byref(p), d_out.data_ptr(), cap, d_result.data_ptr(),
            ctypes.c_void_p(stream.cuda_stream))
    assert st == 6  # BLAZE_ERR_LIMIT
    ps.close()
    db.close()
