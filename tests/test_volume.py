"""NCBI BLAST protein volume (.pin/.psq) reading: the library's reader gives
back exactly what was written (versions 4 and 5, empty and edge-length
sequences), rejects malformed volumes, and (GPU) a database opened from a
volume searches exactly like the same residues passed as arrays."""
import os
import struct

import numpy as np
import pytest

import blaze103
from blaze103 import synth, volume


def _seqs(seed=4, n=300):
    rng = np.random.default_rng(seed)
    seqs = [synth.random_residues(rng, int(L)) for L in synth.lognormal_lengths(rng, n, 250, 0.82, 30, 3000)]
    seqs[5] = seqs[5][:0]  # an empty sequence
    seqs[6] = seqs[6][:1]
    seqs.append(np.array([25, 26, 27, 21, 1], dtype=np.uint8))  # rare codes
    off = np.zeros(len(seqs) + 1, dtype=np.uint64)
    np.cumsum([len(s) for s in seqs], out=off[1:])
    return np.concatenate(seqs).astype(np.uint8), off


@pytest.mark.parametrize("version", [4, 5])
def test_volume_round_trip(tmp_path, version):
    res, off = _seqs()
    path = os.path.join(tmp_path, "db")
    volume.write_volume(path, res, off, version=version)
    info = volume.volume_info(path)
    assert info == {"n_subjects": len(off) - 1, "total_residues": int(off[-1]),
                    "max_length": int(np.diff(off.astype(np.int64)).max())}
    r2, o2 = volume.read_volume(path)
    assert np.array_equal(o2, off) and np.array_equal(r2, res)


def test_volume_rejects_malformed(tmp_path):
    res, off = _seqs(n=20)
    path = os.path.join(tmp_path, "db")
    volume.write_volume(path, res, off)
    pin = open(path + ".pin", "rb").read()
    bad = os.path.join(tmp_path, "bad")
    cases = {
        "truncated": pin[: len(pin) // 2],
        "nucleotide": pin[:4] + struct.pack(">I", 0) + pin[8:],
        "version": struct.pack(">I", 3) + pin[4:],
    }
    for name, data in cases.items():
        with open(bad + ".pin", "wb") as f:
            f.write(data)
        with open(bad + ".psq", "wb") as f:
            f.write(open(path + ".psq", "rb").read())
        with pytest.raises(blaze103.BlazeError) as e:
            volume.read_volume(bad)
        assert e.value.status == 1, name
    # sequence file shorter than the index says
    with open(bad + ".pin", "wb") as f:
        f.write(pin)
    with open(bad + ".psq", "wb") as f:
        f.write(open(path + ".psq", "rb").read()[:-10])
    with pytest.raises(blaze103.BlazeError):
        volume.read_volume(bad)
    with pytest.raises(blaze103.BlazeError):
        volume.volume_info(os.path.join(tmp_path, "missing"))
    # a header whose total length disagrees with its own offsets (a huge
    # claim must be refused before anything is sized by it)
    pos = 12 + struct.unpack(">I", pin[8:12])[0]
    pos += 4 + struct.unpack(">I", pin[pos:pos + 4])[0] + 4  # past the date and N
    with open(bad + ".pin", "wb") as f:
        f.write(pin[:pos] + struct.pack("<Q", 1 << 50) + pin[pos + 8:])
    with open(bad + ".psq", "wb") as f:
        f.write(open(path + ".psq", "rb").read())
    for call in (volume.volume_info, volume.read_volume, blaze103.SeqSrc.open):
        with pytest.raises(blaze103.BlazeError) as e:
            call(bad)
        assert e.value.status == 1
    # a sequence file too short for the index: refused before any copy
    with open(bad + ".pin", "wb") as f:
        f.write(pin)
    with open(bad + ".psq", "wb") as f:
        f.write(b"\0")
    with pytest.raises(blaze103.BlazeError) as e:
        blaze103.SeqSrc.open(bad)
    assert e.value.status == 1


@pytest.mark.gpu
def test_opened_volume_searches_like_arrays(tmp_path):
    w = synth.make_workload("plain-small", scale=0.05)
    path = os.path.join(tmp_path, "cfg0")
    volume.write_volume(path, w.residues, w.offsets, version=5)
    a = blaze103.SeqSrc(w.residues, w.offsets)
    b = blaze103.SeqSrc.open(path)
    assert (b.tot_len, b.num_seqs, b.max_seq_len) == (a.tot_len, a.num_seqs, a.max_seq_len)
    pa, pb = blaze103.PrelimSearch(a), blaze103.PrelimSearch(b)
    for q in w.queries:
        ra, rb = pa.run(q).hsps, pb.run(q).hsps
        assert len(ra) > 0 and np.array_equal(ra, rb)
    for x in (pa, pb, a, b):
        x.close()
