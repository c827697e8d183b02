"""Undirected graphs (EEG_VG_SYMMETRIC): the forward graph doubles as the transposed one. Every CC
variant still gives the oracle's labels bit-exactly, PageRank matches the FP64 oracle as on a
separately built transposed graph, and the personalised PageRank (which needs the edge indices of a
real transposed build) refuses such a graph."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

VARIANTS = ["async_push_td", "async_push_dd", "sync_push_td", "sync_push_dd"]


def _sym_graphs(E):
    out = []
    s, d, w = E.gen_rmat(12, 8, seed=41, wmin=1, wmax=63)
    ss, ds, ws = E.symmetrize(s, d, w)
    out.append(("rmat12", 1 << 12, ss, ds, ws))
    side = 40
    s, d, w = E.gen_grid(side, 0.1, 0.01, seed=3, wmin=1, wmax=1000)  # already both arcs
    out.append(("grid40", side * side, s, d, w))
    s, d, w = E.gen_rmat(8, 4, seed=42, wmin=1, wmax=5)
    ss, ds, ws = E.symmetrize(s, d, w)
    out.append(("rmat8", 1 << 8, ss, ds, ws))
    return out


@pytest.mark.parametrize("K", [4, 8, 16])
def test_cc_on_symmetric_graph_all_variants(gpu, K):
    E = gpu
    for name, n, s, d, w in _sym_graphs(E):
        src = int(np.bincount(s, minlength=n).argmax())
        with E.VirtualGraph.build(n, s, d, w, K=K, symmetric=True) as vg:
            assert vg.info()["num_rparts"] == vg.info()["num_parts"]
            for variant in VARIANTS:
                got, res = vg.run("cc", variant, src)
                want = oracle.expected("cc", variant, n, s, d, w, src)
                assert np.array_equal(got, want), (name, variant, K)
            got, _ = vg.run("cc", "async_push_dd", src, host_loop=True)
            assert np.array_equal(got, oracle.cc_labels(n, s, d, w))
            # the traversals still use the forward graph
            got, _ = vg.run("sssp", "sync_push_dd", src)
            assert np.array_equal(got, oracle.dijkstra(n, s, d, w, src))


def test_pagerank_on_symmetric_graph_equals_transposed_build(gpu):
    E = gpu
    s, d, w = E.gen_rmat(12, 8, seed=43, wmin=1, wmax=63)
    ss, ds, ws = E.symmetrize(s, d, w)
    n = 1 << 12
    with E.VirtualGraph.build(n, ss, ds, ws, K=8, symmetric=True) as a, \
            E.VirtualGraph.build(n, ss, ds, None, K=8, reverse=True) as b:
        xa, _ = a.run("pr", "sync_push_td")
        xb, _ = b.run("pr", "sync_push_td")
        # same vertex sums in a different neighbour order (FP32 rounding differs): compare to FP64
        xr, _ = oracle.pagerank(n, ss, ds)
        for x in (xa, xb):
            assert np.abs(x.astype(np.float64) - xr).sum() / np.abs(xr).sum() <= 1e-6
    with E.VirtualGraph.build(n, ss, ds, ws, K=8, symmetric=True, edge_ids=True) as c:
        with pytest.raises(E.EEGError):
            E.PPR(c, 4)
