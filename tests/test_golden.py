"""The oracle against its committed regression fixtures (tests/golden/), and,
on a GPU, libblaze103 against the same fixtures."""
import glob
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
# the oracle's regression fixtures (ref_lookup.npz holds vectors made by the
# reference's own code: tests/test_ref_lookup.py)
FIXTURES = sorted(p for p in glob.glob(os.path.join(HERE, "golden", "*.npz"))
                  if os.path.basename(p) != "ref_lookup.npz")
PARAM_KEYS = ["word_threshold", "window", "ungapped_xdrop", "ungapped_cutoff", "gap_open",
              "gap_extend", "gapped_xdrop", "gapped_cutoff"]


def load(path):
    z = np.load(path)
    return z, dict(zip(PARAM_KEYS, (int(x) for x in z["params"])))


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p) for p in FIXTURES])
def test_oracle_matches_fixture(oracle_mod, path):
    z, p = load(path)
    hsps, inits = oracle_mod.search_db(z["query"], z["residues"], z["offsets"], p, threads=3,
                                       want_inits=True)
    assert np.array_equal(hsps, z["hsps"])
    assert np.array_equal(inits, z["inits"])
    assert len(z["hsps"]) > 0


@pytest.mark.gpu
@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p) for p in FIXTURES])
def test_gpu_matches_fixture(path):
    import blaze103

    z, p = load(path)
    db = blaze103.SeqSrc(z["residues"], z["offsets"])
    ps = blaze103.PrelimSearch(db)
    prm = blaze103.default_params(len(z["query"]), db_residues=int(z["db_len"]),
                                  db_subjects=int(z["db_n"]))
    for k, v in p.items():
        setattr(prm, k, v)
    prm.prelim_evalue = 1e300  # the fixtures hold HSPs before the E-value reap
    q = blaze103.Query(db, z["query"])
    ps.run_query(q, prm)
    got, ini = ps.results(), ps.init_hits()
    want, wini = z["hsps"], z["inits"]
    assert np.array_equal(got["oid"], want["subject"])
    for f in ("score", "q_start", "q_end", "s_start", "s_end"):
        assert np.array_equal(got[f], want[f]), f
    assert np.array_equal(got["q_gapped_start"], want["q_gstart"])
    assert np.array_equal(ini["oid"], wini["subject"])
    for g, r in (("q_start", "q_start"), ("s_start", "s_start"), ("length", "len"),
                 ("score", "score"), ("q_trigger", "q_trig"), ("s_trigger", "s_trig")):
        assert np.array_equal(ini[g], wini[r]), g
    q.close()
    ps.close()
    db.close()


TRACED_FIELDS = ["score", "q_start", "q_end", "s_start", "s_end", "length", "identities", "positives",
                 "mismatches", "gap_opens", "gaps"]


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p) for p in FIXTURES])
def test_oracle_traceback_matches_fixture(oracle_mod, path):
    z, p = load(path)
    pd = oracle_mod.default_params(len(z["query"]), int(z["db_len"]), int(z["db_n"]))
    pd.update(p)
    fin = oracle_mod.finish(z["hsps"], dict(pd, prelim_evalue=1e300))
    rows = oracle_mod.traceback_hsps(z["query"], z["residues"], z["offsets"], fin, pd, evalue=1e300)
    want = z["traced"]
    assert len(rows) == len(want) > 0
    assert [r["subject"] for r in rows] == want["subject"].tolist()
    for f in TRACED_FIELDS:
        assert [r[f] for r in rows] == want[f].tolist(), f


@pytest.mark.gpu
@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p) for p in FIXTURES])
def test_gpu_traceback_matches_fixture(path):
    import blaze103

    z, p = load(path)
    db = blaze103.SeqSrc(z["residues"], z["offsets"])
    ps = blaze103.PrelimSearch(db)
    prm = blaze103.default_params(len(z["query"]), db_residues=int(z["db_len"]), db_subjects=int(z["db_n"]))
    for k, v in p.items():
        setattr(prm, k, v)
    prm.prelim_evalue = 1e300
    ps.run(z["query"], prm)
    got = ps.traceback(z["query"], prm, evalue=1e300)
    want = z["traced"]
    assert got["oid"].tolist() == want["subject"].tolist()
    for f in TRACED_FIELDS:
        assert got[f].tolist() == want[f].tolist(), f
    ps.close()
    db.close()
