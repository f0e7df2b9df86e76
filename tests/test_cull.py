"""The oracle's hit-list culling on hand-made lists (CPU): max_hsps keeps
the first HSPs of each subject, hitlist_size the subjects with the best
first HSP, ties by smaller subject index."""
import numpy as np

import oracle


def _hsps(rows):
    out = np.zeros(len(rows), dtype=oracle.HSP_DTYPE)
    out["subject"] = [r[0] for r in rows]
    out["score"] = [r[1] for r in rows]
    return out


def test_cull_rules():
    h = _hsps([(0, 50), (0, 40), (0, 30), (2, 90), (3, 50), (3, 45), (7, 50), (9, 10)])
    assert oracle.cull(h).tolist() == h.tolist()
    m = oracle.cull(h, max_hsps=1)
    assert m["subject"].tolist() == [0, 2, 3, 7, 9]
    top = oracle.cull(h, hitlist_size=3)
    assert sorted(set(top["subject"].tolist())) == [0, 2, 3]  # 90, then 50s by subject
    assert top["score"].tolist() == [50, 40, 30, 90, 50, 45]
    both = oracle.cull(h, hitlist_size=2, max_hsps=2)
    assert both["subject"].tolist() == [0, 0, 2]
    assert len(oracle.cull(h, hitlist_size=100)) == len(h)
