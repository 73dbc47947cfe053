"""The independent manifold check (tests/_support.py manifold_report) against
the oracle on small noise grids: it recomputes edge valences, the quads with
non-manifold edges and the face fans from the halfedges alone, and must agree
with the oracle's statistics and multi-fan flags, with and without the
non-manifold split.  The GPU workload tests apply the same check at full size."""
import numpy as np
import pytest

from _support import manifold_report, oracle_run


@pytest.mark.parametrize("n,seed", [(16, 3), (28, 5), (48, 7)])
@pytest.mark.parametrize("split", [0, 1])
def test_manifold_report_agrees_with_the_oracle(n, seed, split):
    v = np.random.default_rng(seed).random((n, n, n), dtype=np.float32)
    r = oracle_run(v.reshape(-1), [n, n, n], np.zeros(3, np.float32), np.ones(3, np.float32), 0.5,
                   split_non_manifold=split)
    st = r["stats"]
    rep = manifold_report(r["halfedges"], len(r["positions"]), r["vertex_flags"])
    assert rep["num_edges"] == st["edges"]
    assert rep["edges_by_valence"].get(3, 0) == st["edges3"]
    assert rep["edges_by_valence"].get(4, 0) == st["edges4"]
    assert max(rep["edges_by_valence"]) <= 4
    assert rep["quads_with_non_manifold_edges"] == [st["quads_nm%d" % k] for k in range(1, 5)]
    assert rep["num_flagged"] == st["nm_vertices"]
    assert rep["clean_mismatch"] == 0 and rep["clean_multi_fan"] > 0
    assert rep["twins_not_opposite_at_valence2"] == 0 and rep["twins_not_involutive_at_valence2"] == 0
    if split:
        assert st["edges4"] == 0


def test_manifold_report_sees_a_planted_second_fan():
    """Cutting one interior edge's twins splits a closed fan: the check must
    count the extra fan at both ends (mistake planted in the oracle's output)."""
    n = 16
    v = np.random.default_rng(9).random((n, n, n), dtype=np.float32)
    r = oracle_run(v.reshape(-1), [n, n, n], np.zeros(3, np.float32), np.ones(3, np.float32), 0.5)
    he = r["halfedges"].copy()
    base = manifold_report(he, len(r["positions"]), r["vertex_flags"])
    # two interior valence-2 edges of one vertex with a single closed fan
    rep_fans = None
    H = len(he)
    origin, nxt, twin = he[:, 0], he[:, 2], he[:, 3]
    flags = r["vertex_flags"]
    for h in range(H):
        t = twin[h]
        if t < 0 or twin[t] != h or flags[origin[h]] & 8:
            continue
        # the fan of origin[h] must be closed (every outgoing halfedge has a twin)
        outs = np.nonzero(origin == origin[h])[0]
        if np.all(twin[outs] >= 0) and len(outs) >= 4:
            g = nxt[t]  # next outgoing halfedge of the same vertex around the fan
            # cut the fan twice: between h and g, and between g and the one after it
            t2 = twin[g]
            if t2 < 0 or twin[t2] != g:
                continue
            he[h, 3] = -1
            he[t, 3] = -1
            he[g, 3] = -1
            he[t2, 3] = -1
            rep_fans = manifold_report(he, len(r["positions"]), r["vertex_flags"])
            break
    assert rep_fans is not None
    # the vertex now has two open fans, but its flag still says one
    assert rep_fans["clean_mismatch"] >= 1 and base["clean_mismatch"] == 0
