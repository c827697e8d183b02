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


@pytest.mark.parametrize("K", [4, 8, 16])
def test_symmetrize_on_device_equals_host_symmetrised_build(gpu, K):
    """EEG_VG_SYMMETRIZE builds, from the directed list, the virtual graph of symmetrize()'s output
    (same parts, slots and weights), from host or device arrays, with m a multiple of 4 (128-bit
    first pass) or not; CC on it gives the oracle's labels."""
    import torch

    E = gpu
    for m_extra in (0, 3):
        s, d, w = E.gen_rmat(12, 8, seed=44 + K, wmin=1, wmax=63)
        s, d, w = s[: s.size - m_extra], d[: d.size - m_extra], w[: w.size - m_extra]
        n = 1 << 12
        ss, ds, ws = E.symmetrize(s, d, w)
        for weighted in (True, False):
            wi, wsi = (w, ws) if weighted else (None, None)
            with E.VirtualGraph.build(n, ss, ds, wsi, K=K, symmetric=True) as ref, \
                    E.VirtualGraph.build(n, s, d, wi, K=K, symmetrize=True) as got:
                a, b = ref.download(), got.download()
                for key in a:
                    assert np.array_equal(a[key], b[key]), (K, m_extra, weighted, key)
                assert got.info()["num_edges"] == ss.size
                assert got.info()["num_rparts"] == got.info()["num_parts"]
                src = int(np.bincount(ss, minlength=n).argmax())
                lab, _ = got.run("cc", "async_push_dd", src)
                assert np.array_equal(lab, oracle.cc_labels(n, ss, ds, wsi if weighted else np.ones_like(ss)))
        dev = torch.device("cuda")
        ts, td, tw = (torch.from_numpy(np.ascontiguousarray(x).astype(np.int32)).to(dev) for x in (s, d, w))
        with E.VirtualGraph.build_device(n, s.size, ts.data_ptr(), td.data_ptr(), tw.data_ptr(), K=K,
                                         symmetrize=True) as gd, \
                E.VirtualGraph.build(n, ss, ds, ws, K=K, symmetric=True) as ref:
            a, b = ref.download(), gd.download()
            for key in a:
                assert np.array_equal(a[key], b[key]), (K, m_extra, "device", key)


def _component_minima(n, s, d):
    """Smallest vertex id of each vertex's connected component (scipy, an independent check)."""
    sp = pytest.importorskip("scipy.sparse")
    csgraph = pytest.importorskip("scipy.sparse.csgraph")
    g = sp.coo_matrix((np.ones(s.size), (s.astype(np.int64), d.astype(np.int64))), shape=(n, n))
    _, comp = csgraph.connected_components(g, directed=False)
    first = np.full(comp.max() + 1, n, np.int64)
    np.minimum.at(first, comp, np.arange(n))
    return first[comp].astype(np.uint32)


@pytest.mark.parametrize("K", [4, 8, 16])
def test_cc_components_mode(gpu, K):
    """eeg_options.cc_components: CC relaxes with weight 0, so every all-seeded variant labels each vertex
    with the smallest id of its component (scipy's components); SYNC_PUSH_DD keeps its source-seeded
    fixed point (the oracle with zero weights). Weights are neither needed nor read."""
    E = gpu
    rng = np.random.default_rng(K)
    n = 6000
    s = rng.integers(0, n, 2500).astype(np.uint32)  # sparse: many components, many isolated vertices
    d = rng.integers(0, n, 2500).astype(np.uint32)
    graphs = [("sparse", n, *E.symmetrize(s, d, None)[:2])]
    for name, gn, gs, gd, gw in _sym_graphs(E):
        graphs.append((name, gn, gs, gd))
    for name, gn, gs, gd in graphs:
        want = _component_minima(gn, gs, gd)
        zeros = np.zeros(gs.size, np.uint32)
        src = int(np.bincount(gs, minlength=gn).argmax())
        with E.VirtualGraph.build(gn, gs, gd, None, K=K, symmetric=True) as vg:
            for variant in VARIANTS:
                got, _ = vg.run("cc", variant, src, cc_components=True)
                if variant == "sync_push_dd":
                    assert np.array_equal(got, oracle.expected("cc", variant, gn, gs, gd, zeros, src)), (name, K)
                else:
                    assert np.array_equal(got, want), (name, variant, K)


def test_reverse_only_build(gpu):
    """EEG_VG_REVERSE_ONLY: the transposed graph and out-degrees only. PageRank on it equals PageRank on a
    full two-direction build bit for bit (same transposed parts, same degrees), for plain and symmetrised
    input; everything that needs the forward parts refuses the graph."""
    import torch

    E = gpu
    s, d, w = E.gen_rmat(12, 8, seed=47, wmin=1, wmax=63)
    n = 1 << 12
    for sym in (False, True):
        with E.VirtualGraph.build(n, s, d, None, K=8, reverse=True, symmetrize=sym) as full, \
                E.VirtualGraph.build(n, s, d, None, K=8, reverse_only=True, symmetrize=sym) as ro:
            fi, ri = full.info(), ro.info()
            assert ri["num_parts"] == 0 and ri["num_rparts"] == fi["num_rparts"]
            assert ri["max_out_degree"] == fi["max_out_degree"]
            assert ri["max_degree_vertex"] == fi["max_degree_vertex"]
            for variant in ("sync_push_td", "async_push_td"):
                xa, _ = full.run("pr", variant)
                xb, _ = ro.run("pr", variant)
                assert np.array_equal(xa.view(np.uint32), xb.view(np.uint32)), (sym, variant)
            with pytest.raises(E.EEGError):
                ro.run("bfs", "sync_push_dd", 0)
            with pytest.raises(E.EEGError):
                ro.download()
            with pytest.raises(E.EEGError):
                E.Batch([ro])
    dev = torch.device("cuda")
    ts, td = (torch.from_numpy(np.ascontiguousarray(x).astype(np.int32)).to(dev) for x in (s, d))
    with E.VirtualGraph.build_device(n, s.size, ts.data_ptr(), td.data_ptr(), None, K=16, reverse_only=True) as gd, \
            E.VirtualGraph.build(n, s, d, None, K=16, reverse=True) as ref:
        xa, _ = gd.run("pr", "sync_push_td")
        xb, _ = ref.run("pr", "sync_push_td")
        assert np.array_equal(xa.view(np.uint32), xb.view(np.uint32))
