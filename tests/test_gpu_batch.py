"""Batched queries (eeg_batch_*) on the GPU: every query's values equal a single eeg_run of the same
(graph, algorithm, source); several cluster sizes; repeated replays of the captured launch; autotuners."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _graphs(E, specs):
    out = []
    for scale, ef, seed in specs:
        n = 1 << scale
        s, d, w = E.gen_rmat(scale, ef, seed=seed, wmin=1, wmax=63)
        out.append((n, s, d, w, E.VirtualGraph.build(n, s, d, w, K=[4, 8, 16][seed % 3])))
    return out


@pytest.mark.parametrize("cluster", [1, 2, 4, 8])
def test_batch_equals_single_runs(gpu, cluster):
    torch = pytest.importorskip("torch")
    E = gpu
    gs = _graphs(E, [(8, 8, 1), (13, 16, 2), (10, 32, 3), (14, 8, 4), (6, 4, 5), (12, 24, 6)])
    rng = np.random.default_rng(cluster)
    queries = []
    for gi, (n, *_rest) in enumerate(gs):
        for _ in range(int(rng.integers(1, 5))):
            queries.append((gi, ["bfs", "sssp", "sswp"][int(rng.integers(0, 3))], int(rng.integers(0, n))))
    with E.Batch([g[4] for g in gs]) as b:
        words = b.set_queries(queries, cluster_size=cluster)
        out = torch.full((words,), 7, dtype=torch.int32, device="cuda")
        offs = b.offsets()
        for rep in range(2):  # the captured launch is replayed
            ms = b.run(out.data_ptr())
            assert ms > 0
            host = out.cpu().numpy().view(np.uint32)
            for qi, (gi, algo, src) in enumerate(queries):
                n, s, d, w, vg = gs[gi]
                want, _ = vg.run(algo, "sync_push_dd", src)
                assert np.array_equal(host[offs[qi]:offs[qi] + n], want), (qi, algo)
        assert (b.rounds() > 0).all() or True
    for g in gs:
        g[4].close()


def test_batch_matches_oracle_and_autotune(gpu):
    torch = pytest.importorskip("torch")
    E = gpu
    gs = _graphs(E, [(11, 16, 7), (9, 8, 8)])
    queries = [(0, "sssp", 0), (1, "bfs", 3), (0, "sswp", 5), (1, "sssp", 1)]
    with E.Batch([g[4] for g in gs]) as b:
        words = b.set_queries(queries)
        out = torch.zeros(words, dtype=torch.int32, device="cuda")
        c, ms = b.autotune(out.data_ptr())
        assert c in (1, 2, 4, 8) and ms > 0
        b.run(out.data_ptr())
        host = out.cpu().numpy().view(np.uint32)
        for qi, (gi, algo, src) in enumerate(queries):
            n, s, d, w, _ = gs[gi]
            o = b.offsets()[qi]
            assert np.array_equal(host[o:o + n], oracle.expected(algo, "sync_push_dd", n, s, d, w, src))
    for g in gs:
        g[4].close()


def test_batch_rejects_bad_queries(gpu):
    E = gpu
    gs = _graphs(E, [(8, 8, 1)])
    with E.Batch([gs[0][4]]) as b:
        for bad in ([(1, "bfs", 0)], [(0, "pr", 0)], [(0, "bfs", 256)]):
            with pytest.raises(E.EEGError) as ei:
                b.set_queries(bad)
            assert ei.value.status == E.ERR_INVALID
    gs[0][4].close()


def test_autotune_k(gpu):
    E = gpu
    s, d, w = E.gen_rmat(14, 16, seed=2)
    k, ms = E.autotune_k(1 << 14, s, d, w, reps=2)
    assert k in (4, 8, 16) and all(v > 0 for v in ms.values())
    k2, _ = E.autotune_k(1 << 14, s, d, w, reps=2)  # cached
    assert k2 == k


@pytest.mark.parametrize("algo", ["bfs", "sssp", "sswp", "cc", "pr"])
def test_autotune_k_and_variant(gpu, algo):
    """eeg_autotune: a (K, variant) from the grid it times, every tried entry positive, CC never on
    SYNC_PUSH_DD (another fixed point); the chosen configuration gives the oracle's answer."""
    E = gpu
    n = 1 << 12
    s, d, w = E.gen_rmat(12, 8, seed=31, wmin=1, wmax=63)
    if algo == "cc":
        s, d, w = E.symmetrize(s, d, w)
    t = E.autotune(n, s, d, w, algo=algo, reps=1)
    assert t["K"] in (4, 8, 16) and t["ms"] > 0
    assert (t["K"], t["variant"]) in t["table"] and all(v > 0 for v in t["table"].values())
    tried_variants = {v for _, v in t["table"]}
    # resident CTAs per SM for the chosen configuration: 1 and 2 timed (1 only for the pull PageRank)
    assert t["blocks_per_sm"] in t["ms_per_blocks"] and all(v > 0 for v in t["ms_per_blocks"].values())
    assert set(t["ms_per_blocks"]) == ({1} if algo == "pr" and t["variant"].endswith("_td") else {1, 2})
    if algo == "cc":
        assert "sync_push_dd" not in tried_variants and len(t["table"]) == 9
    else:
        assert len(t["table"]) == 12
    src = int(np.bincount(s, minlength=n).argmax())
    if algo == "pr":
        with E.VirtualGraph.build(n, s, d, None, K=t["K"], reverse=True) as vg:
            x, _ = vg.run("pr", t["variant"])
        xr, _ = oracle.pagerank(n, s, d)
        assert np.abs(x / x.sum() - xr / xr.sum()).sum() <= 1e-6
    else:
        with E.VirtualGraph.build(n, s, d, w, K=t["K"]) as vg:
            got, _ = vg.run(algo, t["variant"], src, blocks_per_sm=t["blocks_per_sm"])
        assert np.array_equal(got, oracle.expected(algo, t["variant"], n, s, d, w, src))


@pytest.mark.parametrize("grid_queries", [1, 3, 100])
def test_batch_whole_grid_queries(gpu, grid_queries):
    """The largest queries run one after another on the whole grid (bounded grid barrier), the rest on
    clusters; every query still equals a single eeg_run, and the timeline marks the whole-grid ones."""
    torch = pytest.importorskip("torch")
    E = gpu
    gs = _graphs(E, [(15, 16, 9), (12, 8, 10), (9, 32, 11), (14, 4, 12)])
    queries = [(0, "bfs", 1), (0, "sssp", 2), (1, "sswp", 3), (2, "bfs", 4), (3, "sssp", 0), (1, "bfs", 0),
               (3, "sswp", 5)]
    with E.Batch([g[4] for g in gs]) as b:
        words = b.set_queries(queries, cluster_size=2)
        b.set_grid_queries(grid_queries)
        assert b.config() == (2, min(grid_queries, len(queries)))
        out = torch.zeros(words, dtype=torch.int32, device="cuda")
        offs = b.offsets()
        for _ in range(2):
            b.run(out.data_ptr())
            host = out.cpu().numpy().view(np.uint32)
            for qi, (gi, algo, src) in enumerate(queries):
                n = gs[gi][0]
                want, _ = gs[gi][4].run(algo, "sync_push_dd", src)
                assert np.array_equal(host[offs[qi]:offs[qi] + n], want), (qi, algo)
        t = b.query_times()
        whole = t[:, 2] == np.uint64(2**64 - 1)
        assert int(whole.sum()) == min(grid_queries, len(queries))
        assert (t[:, 1] >= t[:, 0]).all()
        # the whole-grid queries are the largest graphs (graph 0 first)
        sizes = np.array([gs[gi][4].info()["num_parts"] for gi, _, _ in queries])
        assert sizes[whole].min() >= sizes[~whole].max() if (~whole).any() else True
    for g in gs:
        g[4].close()
