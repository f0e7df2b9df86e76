"""GPU tests of the BlastSeqSrc-shaped database source
(blaze_db_create_from_source): a database read through the source's
callbacks searches exactly like the same residues passed as flat arrays."""
import subprocess

import numpy as np
import pytest

from test_abi import build_c_client

pytestmark = pytest.mark.gpu


def test_c_client_source_equals_flat_arrays(tmp_path):
    exe = build_c_client("seqsrc_client", tmp_path)
    r = subprocess.run([exe, "gpu"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("same ")


class ListSource:
    """An in-memory source with NCBI BlastSeqSrc's accessors."""

    def __init__(self, seqs, iter_oids=None):
        self.seqs = seqs
        self.iter_oids = iter_oids
        self.pos = 0
        self.fetched = self.released = 0

    def num_seqs(self):
        return len(self.seqs)

    def get_sequence(self, oid):
        self.fetched += 1
        return self.seqs[oid]

    def release_sequence(self, oid):
        self.released += 1

    def tot_len(self):
        return sum(len(s) for s in self.seqs)

    def max_seq_len(self):
        return max(len(s) for s in self.seqs)


class IterSource(ListSource):
    def iter_next(self):
        if self.pos >= len(self.iter_oids):
            return -1
        self.pos += 1
        return self.iter_oids[self.pos - 1]


def test_python_source_equals_flat_arrays():
    import blaze103
    from blaze103 import synth

    w = synth.make_workload("plain-small", scale=0.1)
    seqs = [w.residues[int(w.offsets[i]):int(w.offsets[i + 1])] for i in range(w.n_subjects)]
    rng = np.random.default_rng(5)
    order = rng.permutation(len(seqs))  # unsorted OIDs: the library sorts
    seqs = [seqs[i] for i in order]
    off = np.zeros(len(seqs) + 1, dtype=np.uint64)
    np.cumsum([len(s) for s in seqs], out=off[1:])
    res = np.concatenate(seqs)
    q = w.queries[0]
    flat = blaze103.SeqSrc(res, off)
    src = ListSource(seqs)
    from_src = blaze103.SeqSrc.from_source(src)
    # no seq_len accessor: one fetch pass for the lengths, one for the residues
    assert src.fetched == 2 * len(seqs) and src.released == src.fetched
    assert (from_src.tot_len, from_src.num_seqs, from_src.max_seq_len) == (flat.tot_len, flat.num_seqs,
                                                                            flat.max_seq_len)
    p = blaze103.default_params(len(q), flat)
    a = blaze103.PrelimSearch(flat).run(q, p).hsps
    b = blaze103.PrelimSearch(from_src).run(q, p).hsps
    assert len(a) > 20
    assert a.tobytes() == b.tobytes()

    # an iterator over a subset: those OIDs search as before, the rest are empty
    keep = sorted(rng.choice(len(seqs), size=len(seqs) // 3, replace=False).tolist())
    sub = blaze103.SeqSrc.from_source(IterSource(seqs, keep))
    c = blaze103.PrelimSearch(sub).run(q, p).hsps
    want = a[np.isin(a["oid"], np.array(keep, dtype=np.uint32))]
    assert c.tobytes() == want.tobytes()

    # malformed sources create nothing
    bad = [s.copy() for s in seqs]
    bad[7][0] = 0
    with pytest.raises(blaze103.BlazeError):
        blaze103.SeqSrc.from_source(ListSource(bad))
    with pytest.raises(blaze103.BlazeError):
        blaze103.SeqSrc.from_source(IterSource(seqs, [3, 5, 3]))
    flat.close()
    from_src.close()
    sub.close()
