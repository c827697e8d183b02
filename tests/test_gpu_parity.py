"""GPU parity: every algorithm x variant x K against the oracle, through the C ABI (needs a GB300).

Integer algorithms are bit-exact; PageRank is within 1e-6 normalised L1 of the FP64 oracle:
    || x/||x||_1 - x*/||x*||_1 ||_1 <= 1e-6.
"""
from pathlib import Path

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden"
VARIANTS = ["async_push_td", "async_push_dd", "sync_push_td", "sync_push_dd"]
ALGOS = ["bfs", "sssp", "sswp", "cc"]
PR_L1 = 1e-6


def _cases():
    z = np.load(GOLD / "seq_cpu.npz")
    out = []
    for name in z["names"]:
        name = str(name)
        out.append((name, {k.split(".", 1)[1]: z[k] for k in z.files if k.startswith(name + ".")}))
    return out


CASES = _cases()


def pr_l1(x, xr):
    x = np.asarray(x, np.float64)
    return float(np.abs(x / x.sum() - xr / xr.sum()).sum())


@pytest.mark.parametrize("name,c", CASES, ids=[n for n, _ in CASES])
@pytest.mark.parametrize("K", [4, 8, 16])
def test_golden_graphs_all_variants(gpu, name, c, K):
    n, s = int(c["n"][0]), int(c["source"][0])
    with gpu.VirtualGraph.build(n, c["src"], c["dst"], c["w"], K=K, reverse=True) as vg:
        for algo in ALGOS:
            for variant in VARIANTS:
                got, res = vg.run(algo, variant, s, timeout_ms=5000)
                want = oracle.expected(algo, variant, n, c["src"], c["dst"], c["w"], s)
                assert np.array_equal(got, want), (algo, variant, int((got != want).sum()))
                if algo != "sssp" and not (algo == "cc" and variant == "sync_push_dd"):
                    # identical to what the reference's own seq_cpu returned
                    assert np.array_equal(got, c[f"ref_{algo}"]), (algo, variant)
        if c["src"].size:
            xr, _ = oracle.pagerank(n, c["src"], c["dst"])
            for variant in VARIANTS:
                x, res = vg.run("pr", variant)
                assert pr_l1(x, xr) <= PR_L1, (variant, pr_l1(x, xr))


@pytest.mark.parametrize("variant", VARIANTS)
def test_rmat16_sssp_config(gpu, variant):
    """R-MAT scale 16, edge factor 16, a/b/c/d = .57/.19/.19/.05, seed 1, weights [1,63], source =
    highest out-degree vertex, K = 8: distances bit-exact vs Dijkstra."""
    n = 1 << 16
    s, d, w = gpu.gen_rmat(16, 16, seed=1, wmin=1, wmax=63)
    with gpu.VirtualGraph.build(n, s, d, w, K=8) as vg:
        src = vg.info()["max_degree_vertex"]
        assert src == int(np.bincount(s, minlength=n).argmax())
        got, res = vg.run("sssp", variant, src)
        assert np.array_equal(got, oracle.dijkstra(n, s, d, w, src))
        assert res["reached_edges"] > 0 and res["gteps"] > 0


@pytest.mark.parametrize("K", [4, 8, 16])
def test_rmat16_all_algorithms(gpu, K):
    n = 1 << 16
    s, d, w = gpu.gen_rmat(16, 16, seed=1, wmin=1, wmax=63)
    src = int(np.bincount(s, minlength=n).argmax())
    with gpu.VirtualGraph.build(n, s, d, w, K=K, reverse=True) as vg:
        for algo in ALGOS:
            want = oracle.expected(algo, "sync_push_dd", n, s, d, w, src)
            got, _ = vg.run(algo, "sync_push_dd", src)
            assert np.array_equal(got, want), algo
        x, res = vg.run("pr", "sync_push_td")
        xr, _ = oracle.pagerank(n, s, d)
        assert pr_l1(x, xr) <= PR_L1
        assert res["pr_residual"] * 0.85 / 0.15 <= 1e-7 * res["pr_l1_norm"] * 1.0001


def test_cc_symmetrised(gpu):
    n = 1 << 14
    s, d, w = gpu.gen_rmat(14, 16, seed=3, wmin=1, wmax=63)
    s2, d2, w2 = gpu.symmetrize(s, d, w)
    with gpu.VirtualGraph.build(n, s2, d2, w2, K=8) as vg:
        for variant in VARIANTS:
            got, _ = vg.run("cc", variant, 5)
            assert np.array_equal(got, oracle.expected("cc", variant, n, s2, d2, w2, 5)), variant


def test_grid_high_diameter(gpu):
    side = 128
    n = side * side
    s, d, w = gpu.gen_grid(side, 0.1, 0.001, seed=7, wmin=1, wmax=1000)
    with gpu.VirtualGraph.build(n, s, d, w, K=4) as vg:
        for algo in ("bfs", "sssp", "sswp"):
            got, res = vg.run(algo, "sync_push_dd", 0)
            assert np.array_equal(got, oracle.expected(algo, "sync_push_dd", n, s, d, w, 0)), algo
        assert res["iterations"] > side  # many rounds, one launch


@pytest.mark.parametrize("K", [4, 8, 16])
@pytest.mark.parametrize("variant", VARIANTS)
def test_pagerank_variants(gpu, variant, K):
    """Topology-driven variants: Jacobi pull sweeps; data-driven variants: the residual frontier
    (pushes along out-edges, activation threshold derived from the tolerance)."""
    n = 1 << 14
    s, d, _ = gpu.gen_rmat(14, 16, seed=9)
    with gpu.VirtualGraph.build(n, s, d, None, K=K, reverse=True) as vg:
        x, res = vg.run("pr", variant)
    xr, _ = oracle.pagerank(n, s, d)
    assert pr_l1(x, xr) <= PR_L1, (variant, pr_l1(x, xr))
    assert res["iterations"] > 5
    if variant.endswith("_dd"):
        # every residual left is below the threshold tol*(1-d)^2: the bound ||x*-x||_1 <= resid/(1-d)
        assert res["pr_residual"] / 0.15 <= 1e-7 * res["pr_l1_norm"] * 1.0001
        assert res["edges_scanned"] > s.size  # round 0 pushes along every edge, later rounds some


@pytest.mark.parametrize("variant", ["sync_push_dd", "async_push_dd"])
def test_pagerank_dd_accuracy_threshold(gpu, variant):
    """An explicit activation threshold (the reference's --accuracy): fewer rounds and pushes the larger
    it is, every residual left below it, and the error within the bound it implies,
    ||x* - x||_1 <= (sum of residuals) / (1-d)."""
    n = 1 << 14
    s, d, _ = gpu.gen_rmat(14, 16, seed=9)
    xr, _ = oracle.pagerank(n, s, d)
    prev = None
    with gpu.VirtualGraph.build(n, s, d, None, K=8, reverse=True) as vg:
        for acc in (1e-2, 1e-4, 1e-6):
            x, res = vg.run("pr", variant, pr_accuracy=acc)
            err = float(np.abs(np.asarray(x, np.float64) - xr).sum())
            assert err <= res["pr_residual"] / 0.15 * 1.001 + 1e-5 * np.abs(xr).sum(), (acc, err)
            assert res["pr_residual"] <= n * acc
            if prev is not None:
                assert res["edges_scanned"] > prev["edges_scanned"] and res["iterations"] >= prev["iterations"]
            prev = res
        x0, res0 = vg.run("pr", variant, pr_accuracy=0.2)  # above the initial residual 1-d: nothing moves
        assert res0["edges_scanned"] == 0 and not np.any(x0)


def test_pagerank_dd_needs_the_forward_parts(gpu):
    n = 1 << 10
    s, d, _ = gpu.gen_rmat(10, 8, seed=2)
    with gpu.VirtualGraph.build(n, s, d, None, K=8, reverse_only=True) as vg:
        _, res = vg.run("pr", "sync_push_dd", check=False)
        assert res["status"] == gpu.ERR_INVALID
        x, res = vg.run("pr", "sync_push_td")  # the pull still runs on it
    xr, _ = oracle.pagerank(n, s, d)
    assert pr_l1(x, xr) <= PR_L1


def test_builder_layout(gpu):
    n = 1 << 12
    s, d, w = gpu.gen_rmat(12, 16, seed=6, wmin=1, wmax=63)
    for K in (4, 8, 16):
        with gpu.VirtualGraph.build(n, s, d, w, K=K) as vg:
            lay = vg.download()
            deg = np.bincount(s, minlength=n).astype(np.uint32)
            assert np.array_equal(lay["outdeg"], deg)
            np_ = (deg + K - 1) // K
            assert np.array_equal(lay["vstart"], np.concatenate([[0], np.cumsum(np_)]).astype(np.uint32))
            assert np.array_equal(lay["vowner"], np.repeat(np.arange(n, dtype=np.uint32), np_))
            # each vertex's slots hold exactly its out-edges (any order), padding = 0xFFFFFFFF
            vcol, vw = lay["vcol"].reshape(-1), lay["vw"].reshape(-1)
            order = np.argsort(s, kind="stable")
            starts = np.concatenate([[0], np.cumsum(deg, dtype=np.int64)])
            for v in np.flatnonzero(deg)[:500]:
                a = int(lay["vstart"][v]) * K
                b = a + int(deg[v])
                got = sorted(zip(vcol[a:b].tolist(), vw[a:b].tolist()))
                idx = order[starts[v]:starts[v + 1]]
                assert got == sorted(zip(d[idx].tolist(), w[idx].tolist()))
                assert np.all(vcol[b:int(lay["vstart"][v + 1]) * K] == 0xFFFFFFFF)
            # the build is a stable sort by owner: each vertex keeps its edges in input order, so the
            # exported reference layout equals the oracle's (itself pinned to the reference's MakeGraph)
            npn, el, pnp = vg.reference_layout()
            onp, oel, opnp = oracle.virtual_graph(n, s, d, w, K)
            assert np.array_equal(npn, onp) and np.array_equal(pnp, opnp) and np.array_equal(el, oel)
            # and it is deterministic
            with gpu.VirtualGraph.build(n, s, d, w, K=K) as vg2:
                lay2 = vg2.download()
                assert all(np.array_equal(lay[k], lay2[k]) for k in ("vstart", "vowner", "vcol", "vw"))


def test_builder_matches_reference_makegraph_golden(gpu):
    z = np.load(GOLD / "layout.npz")
    cases = dict(CASES)
    for name in ("hub", "rmat8"):
        c = cases[name]
        with gpu.VirtualGraph.build(int(c["n"][0]), c["src"], c["dst"], c["w"], K=8) as vg:
            npn, el, pnp = vg.reference_layout()
        assert np.array_equal(npn, z[f"{name}.nodePointer"])
        assert np.array_equal(el, z[f"{name}.edgeList"])
        assert np.array_equal(pnp, z[f"{name}.partNodePointer"])


def test_edge_cases(gpu):
    # no edges at all
    with gpu.VirtualGraph.build(3, np.array([], np.uint32), np.array([], np.uint32), np.array([], np.uint32)) as vg:
        got, res = vg.run("sssp", "sync_push_dd", 1)
        assert got.tolist() == [gpu.DIST_INFINITY, 0, gpu.DIST_INFINITY]
        got, _ = vg.run("cc", "async_push_td", 0)
        assert got.tolist() == [0, 1, 2]
    # source out of range -> invalid, no launch
    s, d, w = gpu.gen_rmat(8, 4, seed=1)
    with gpu.VirtualGraph.build(256, s, d, w) as vg:
        with pytest.raises(gpu.EEGError) as ei:
            vg.run("bfs", "sync_push_dd", 256)
        assert ei.value.status == gpu.ERR_INVALID
        # iteration cap (host-injected limit): reported, device stays usable
        _, res = vg.run("sssp", "sync_push_td", 0, max_iterations=1, check=False)
        assert res["status"] == gpu.ERR_ITER_CAP
        got, _ = vg.run("sssp", "sync_push_dd", 0)
        assert np.array_equal(got, oracle.dijkstra(256, s, d, w, 0))
    # PageRank needs the transposed graph
    with gpu.VirtualGraph.build(256, s, d, w) as vg:
        with pytest.raises(gpu.EEGError):
            vg.run("pr", "sync_push_td")
    # edge endpoint out of range is rejected by the builder
    with pytest.raises(gpu.EEGError) as ei:
        gpu.VirtualGraph.build(4, np.array([0, 5], np.uint32), np.array([1, 2], np.uint32))
    assert ei.value.status == gpu.ERR_INVALID


def test_activity_vector(gpu):
    n = 1 << 12
    s, d, w = gpu.gen_rmat(12, 16, seed=2)
    with gpu.VirtualGraph.build(n, s, d, w) as vg:
        got, res, act = vg.run("bfs", "sync_push_dd", 0, activity_cap=64)
        assert act.size == res["iterations"] and act.size > 0
        # BFS: each vertex is activated exactly once (when first reached), the source excluded
        assert int(act.sum()) == int((got != gpu.DIST_INFINITY).sum()) - 1


def test_managed_memory_and_graph_handle(gpu):
    s, d, w = gpu.gen_rmat(10, 8, seed=8)
    g = gpu.Graph.from_arrays(1024, s, d, w)
    with gpu.VirtualGraph.from_graph(g, K=8, reverse=True) as vg:
        got, _ = vg.run("sssp", "sync_push_dd", 0)
        assert np.array_equal(got, oracle.dijkstra(1024, s, d, w, 0))
    with gpu.VirtualGraph.build(1024, s, d, w, K=8, managed=True) as vg:
        got, _ = vg.run("sswp", "async_push_dd", 0)
        assert np.array_equal(got, oracle.widest(1024, s, d, w, 0))


def test_one_based_file(gpu):
    g = gpu.Graph.load(GOLD / "loader" / "one_based.wel")
    with gpu.VirtualGraph.from_graph(g) as vg:
        got, _ = vg.run("sssp", "sync_push_dd", 0)
    # edges after the shift: 0->1 (5), 1->2 (7), 2->0 (2), 2->2 (1)
    assert got.tolist() == [0, 5, 12]


def test_repeated_runs_reuse_workspace(gpu):
    n = 1 << 12
    s, d, w = gpu.gen_rmat(12, 16, seed=12)
    with gpu.VirtualGraph.build(n, s, d, w, reverse=True) as vg:
        for src in (0, 1, 7, 100):
            got, _ = vg.run("sssp", "sync_push_dd", src)
            assert np.array_equal(got, oracle.dijkstra(n, s, d, w, src))
            got, _ = vg.run("bfs", "async_push_dd", src)
            assert np.array_equal(got, oracle.bfs(n, s, d, src))


def test_build_from_page_locked_host_arrays(gpu):
    """Page-locked inputs are read in place by the builder; the result equals the copied-input build."""
    torch = pytest.importorskip("torch")
    n = 1 << 12
    s, d, w = gpu.gen_rmat(12, 16, seed=13, wmin=1, wmax=63)
    pin = [torch.from_numpy(a.view(np.int32)).pin_memory().numpy().view(np.uint32) for a in (s, d, w)]
    with gpu.VirtualGraph.build(n, *pin, K=8, reverse=True) as vg_pin, gpu.VirtualGraph.build(n, s, d, w, K=8,
                                                                                              reverse=True) as vg:
        a, b = vg_pin.download(), vg.download()
        assert all(np.array_equal(a[k], b[k]) for k in ("vstart", "vowner", "vcol", "vw", "outdeg"))
        got, _ = vg_pin.run("sssp", "sync_push_dd", 0)
        assert np.array_equal(got, oracle.dijkstra(n, s, d, w, 0))
        x, _ = vg_pin.run("pr", "sync_push_td")
        xr, _ = oracle.pagerank(n, s, d)
        assert pr_l1(x, xr) <= PR_L1


@pytest.mark.parametrize("algo,variant", [("bfs", "sync_push_dd"), ("sssp", "async_push_dd"), ("cc", "sync_push_td"),
                                          ("sswp", "async_push_td")])
def test_host_loop_mode_equals_persistent(gpu, algo, variant):
    """One launch per round with a host round trip (the reference's loop shape) gives the same values
    and the same number of rounds as the single persistent launch."""
    side = 48
    n = side * side
    s, d, w = gpu.gen_grid(side, 0.1, 0.01, seed=7, wmin=1, wmax=1000)
    with gpu.VirtualGraph.build(n, s, d, w, K=4) as vg:
        a, ra = vg.run(algo, variant, 0)
        b, rb = vg.run(algo, variant, 0, host_loop=True)
    assert np.array_equal(a, b)
    assert np.array_equal(a, oracle.expected(algo, variant, n, s, d, w, 0))
    if algo == "bfs":  # level-synchronous: the round count is the source's eccentricity + 1 either way
        assert ra["iterations"] == rb["iterations"]
    assert rb["launches"] == rb["iterations"] + 2  # one per round, the final check, the statistics kernel
    assert ra["launches"] == 2


@pytest.mark.parametrize("K", [4, 8, 16])
def test_bfs_pull_rounds(gpu, K):
    """Source-seeded BFS on a graph built with its transposed parts pulls in its large rounds (every
    unreached vertex looks for a parent at the current level among its in-neighbours) and pushes in the
    others. Levels bit-exact against the oracle and against push rounds only, from the hub (rounds that
    pull, the second one over the list of vertices the first one left unreached), from a vertex with
    one out-edge and from a vertex with no out-edges; far fewer edges read than pushing."""
    n = 1 << 16
    s, d, w = gpu.gen_rmat(16, 16, seed=1, wmin=1, wmax=63)
    deg = np.bincount(s, minlength=n)
    hub = int(deg.argmax())
    srcs = [hub, int(np.flatnonzero(deg == 1)[0]), int(np.flatnonzero(deg == 0)[0])]
    with gpu.VirtualGraph.build(n, s, d, w, K=K, reverse=True) as vg:
        for src in srcs:
            want = oracle.bfs(n, s, d, src)
            got, res = vg.run("bfs", "sync_push_dd", src)
            push, rp = vg.run("bfs", "sync_push_dd", src, bfs_push_only=True)
            assert np.array_equal(got, want), (src, int((got != want).sum()))
            assert np.array_equal(push, want) and rp["pull_rounds"] == 0
            assert res["iterations"] == rp["iterations"]  # one round per level either way
            assert res["reached_vertices"] == rp["reached_vertices"]
            if src == hub:
                assert res["pull_rounds"] >= 2, res["pull_rounds"]
                assert res["edges_scanned"] * 3 < rp["edges_scanned"], (res["edges_scanned"], rp["edges_scanned"])
    with gpu.VirtualGraph.build(n, s, d, w, K=K) as vg:  # no transposed parts: push rounds only
        got, res = vg.run("bfs", "sync_push_dd", hub)
        assert np.array_equal(got, oracle.bfs(n, s, d, hub)) and res["pull_rounds"] == 0


def test_bfs_pull_rounds_symmetric_and_sparse(gpu):
    """An undirected graph (its in-edges are its out-edges: the forward parts serve both directions)
    and a sparse graph whose vertices mostly have no in-edges (edge factor 2)."""
    n = 1 << 15
    s, d, w = gpu.gen_rmat(15, 16, seed=5, wmin=1, wmax=63)
    ss, ds, ws = gpu.symmetrize(s, d, w)
    hub = int(np.bincount(ss, minlength=n).argmax())
    with gpu.VirtualGraph.build(n, ss, ds, ws, K=8, symmetric=True) as vg:
        got, res = vg.run("bfs", "sync_push_dd", hub)
    assert np.array_equal(got, oracle.bfs(n, ss, ds, hub)) and res["pull_rounds"] >= 1
    with gpu.VirtualGraph.build(n, s, d, w, K=8, symmetrize=True) as vg:  # symmetrised on the device
        got, res = vg.run("bfs", "sync_push_dd", hub)
    assert np.array_equal(got, oracle.bfs(n, ss, ds, hub)) and res["pull_rounds"] >= 1
    s, d, w = gpu.gen_rmat(15, 2, seed=9, wmin=1, wmax=63)
    hub = int(np.bincount(s, minlength=n).argmax())
    with gpu.VirtualGraph.build(n, s, d, w, K=8, reverse=True) as vg:
        for src in (hub, 0):
            got, _ = vg.run("bfs", "sync_push_dd", src)
            assert np.array_equal(got, oracle.bfs(n, s, d, src)), src
