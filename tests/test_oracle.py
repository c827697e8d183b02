"""The oracle is pinned before it is trusted (CPU only).

* against the golden vectors produced by the reference's own code (tests/golden/make_golden.py);
* against the reference library itself on fresh seeded graphs, when oracle/_ref is built here;
* the no-wrap restatement against independent textbook oracles (BFS, Dijkstra, widest path,
  multi-source Dijkstra for the min-plus labels), which is the parity contract for the GPU.
"""
from pathlib import Path

import numpy as np
import pytest

import oracle

GOLD = Path(__file__).resolve().parent / "golden"


def _cases():
    z = np.load(GOLD / "seq_cpu.npz")
    for name in z["names"]:
        name = str(name)
        yield name, {k.split(".", 1)[1]: z[k] for k in z.files if k.startswith(name + ".")}


CASES = list(_cases())


@pytest.mark.parametrize("name,c", CASES, ids=[n for n, _ in CASES])
@pytest.mark.parametrize("algo", ["bfs", "sssp", "sswp", "cc"])
def test_restatement_matches_reference_golden(name, c, algo):
    n, s = int(c["n"][0]), int(c["source"][0])
    got, _ = oracle.seq_sweep(algo, n, c["src"], c["dst"], c["w"], s, K=8, wrap=True)
    assert np.array_equal(got, c[f"ref_{algo}"])


@pytest.mark.parametrize("name,c", CASES, ids=[n for n, _ in CASES])
def test_unit_weight_sssp_reference_equals_dijkstra(name, c):
    n, s = int(c["n"][0]), int(c["source"][0])
    want = oracle.dijkstra(n, c["src"], c["dst"], np.ones_like(c["w"]), s)
    assert np.array_equal(c["ref_sssp_unit"], want)


@pytest.mark.parametrize("name,c", CASES, ids=[n for n, _ in CASES])
@pytest.mark.parametrize("algo", ["bfs", "sssp", "sswp", "cc"])
def test_contract_equals_independent_oracles(name, c, algo):
    n, s = int(c["n"][0]), int(c["source"][0])
    got, _ = oracle.seq_sweep(algo, n, c["src"], c["dst"], c["w"], s, K=8, wrap=False)
    want = oracle.expected(algo, "async_push_td", n, c["src"], c["dst"], c["w"], s)
    assert np.array_equal(got, want)
    if algo != "sssp":  # only SSSP differs from the reference (its INF+w wrap)
        assert np.array_equal(got, c[f"ref_{algo}"])


@pytest.mark.parametrize("name,c", CASES, ids=[n for n, _ in CASES])
@pytest.mark.parametrize("K", [4, 8, 16])
def test_frontier_rounds_reach_same_fixed_point(name, c, K):
    n, s = int(c["n"][0]), int(c["source"][0])
    for algo in ("bfs", "sssp", "sswp"):
        got, _ = oracle.frontier_sweep(algo, n, c["src"], c["dst"], c["w"], s, K=K, seed_all=False)
        assert np.array_equal(got, oracle.expected(algo, "sync_push_dd", n, c["src"], c["dst"], c["w"], s))
    all_seeded, _ = oracle.frontier_sweep("cc", n, c["src"], c["dst"], c["w"], s, K=K, seed_all=True)
    assert np.array_equal(all_seeded, oracle.cc_labels(n, c["src"], c["dst"], c["w"]))


def test_layout_matches_reference_golden():
    z = np.load(GOLD / "layout.npz")
    cases = dict(CASES)
    for name in ("hub", "rmat8"):
        c = cases[name]
        npn, el, pnp = oracle.virtual_graph(int(c["n"][0]), c["src"], c["dst"], c["w"], 8)
        assert np.array_equal(npn, z[f"{name}.nodePointer"])
        assert np.array_equal(el, z[f"{name}.edgeList"])
        assert np.array_equal(pnp, z[f"{name}.partNodePointer"])


def test_cc_source_seeded_differs_from_all_seeded():
    # src/eegraph.cu:548-553: SYNC_PUSH_DD seeds only the source, so its CC fixed point differs
    c = dict(CASES)["rmat10"]
    n, s = int(c["n"][0]), int(c["source"][0])
    a = oracle.expected("cc", "sync_push_dd", n, c["src"], c["dst"], c["w"], s)
    b = oracle.expected("cc", "async_push_td", n, c["src"], c["dst"], c["w"], s)
    assert not np.array_equal(a, b)
    assert np.all(a >= b)


def test_pagerank_oracle_fixed_point():
    c = dict(CASES)["rmat10"]
    n = int(c["n"][0])
    x, it = oracle.pagerank(n, c["src"], c["dst"], 0.85, 1e-15)
    deg = np.bincount(c["src"], minlength=n).astype(np.float64)
    contrib = np.where(deg > 0, x / np.maximum(deg, 1), 0.0)
    y = np.zeros(n)
    np.add.at(y, c["dst"], contrib[c["src"]])
    assert np.abs(0.15 + 0.85 * y - x).sum() <= 1e-12 * x.sum()
    assert it > 10


@pytest.mark.skipif(not oracle.ref_available(), reason="reference library not built here")
@pytest.mark.parametrize("seed", [21, 22, 23])
def test_restatement_matches_reference_library(seed):
    import eegraph_gb300 as E

    s, d, w = E.gen_rmat(9, 8, seed=seed, wmin=1, wmax=63)
    n = 512
    src = int(np.bincount(s, minlength=n).argmax())
    for algo in ("bfs", "sssp", "sswp", "cc"):
        got, _ = oracle.seq_sweep(algo, n, s, d, w, src, K=8, wrap=True)
        assert np.array_equal(got, oracle.ref_seq_cpu(algo, n, s, d, w, src))


def test_ppr_oracle_adjoint_against_finite_differences():
    """FP64 personalised PageRank oracle: adjoint gradients equal central differences; duality
    c^T x = (1-d) t^T lambda; sum_v w_uv dL/dw_uv = 0 per source (row normalisation is scale-free)."""
    rng = np.random.default_rng(3)
    n, m, C = 60, 400, 3
    src = rng.integers(0, n, m).astype(np.uint32)
    dst = rng.integers(0, n, m).astype(np.uint32)
    src[:5] = 7  # a few parallel edges and a vertex with several out-edges
    dst[:5] = 9
    w = rng.uniform(0.01, 1.0, m)
    T = np.zeros((n, C))
    for k in range(C):
        T[rng.choice(n, 6, replace=False), k] = 1 / 6
    G = rng.standard_normal((n, C))
    r = oracle.ppr(n, src, dst, w, T, G)
    assert abs((G * r["X"]).sum() - 0.15 * (T * r["L"]).sum()) <= 1e-12 * np.abs(G * r["X"]).sum()

    def loss(wv, Tv):
        return (G * oracle.ppr_solve(n, src, dst, wv, Tv)[0]).sum()

    eps = 1e-6
    for e in (0, 3, 100, 399):
        wp, wm = w.copy(), w.copy()
        wp[e] += eps
        wm[e] -= eps
        fd = (loss(wp, T) - loss(wm, T)) / (2 * eps)
        assert abs(fd - r["gw"][e]) <= 1e-7 + 1e-6 * abs(r["gw"][e])
    for i, k in ((0, 0), (13, 2), (59, 1)):
        Tp, Tm = T.copy(), T.copy()
        Tp[i, k] += eps
        Tm[i, k] -= eps
        fd = (loss(w, Tp) - loss(w, Tm)) / (2 * eps)
        assert abs(fd - r["gT"][i, k]) <= 1e-7 + 1e-6 * abs(r["gT"][i, k])
    tot = np.zeros(n)
    np.add.at(tot, src, w * r["gw"])
    assert np.abs(tot).max() <= 1e-12
    # normalised-weight gradient: d <x_u, lambda_v>
    assert np.allclose(r["gWn"], 0.85 * (r["X"][src] * r["L"][dst]).sum(1), rtol=1e-12, atol=1e-15)


@pytest.mark.parametrize("seed", range(4))
def test_cc_labels_with_zero_weights_are_component_minima(seed):
    """The CC oracle relaxed with weight 0 (what eeg_options.cc_components computes) labels each vertex
    with the smallest id of its connected component: checked against scipy's components."""
    sp = pytest.importorskip("scipy.sparse")
    csgraph = pytest.importorskip("scipy.sparse.csgraph")
    rng = np.random.default_rng(seed)
    n, m = 3000, int(rng.integers(500, 4000))
    s = rng.integers(0, n, m).astype(np.uint32)
    d = rng.integers(0, n, m).astype(np.uint32)
    ss, ds = np.concatenate([s, d]), np.concatenate([d, s])
    got = oracle.cc_labels(n, ss, ds, np.zeros(ss.size, np.uint32))
    g = sp.coo_matrix((np.ones(ss.size), (ss.astype(np.int64), ds.astype(np.int64))), shape=(n, n))
    _, comp = csgraph.connected_components(g, directed=False)
    first = np.full(comp.max() + 1, n, np.int64)
    np.minimum.at(first, comp, np.arange(n))
    assert np.array_equal(got, first[comp].astype(np.uint32))


@pytest.mark.parametrize("scale,ef,seed", [(8, 16, 1), (13, 8, 3), (16, 16, 1)])
def test_oracle_rmat_generator_equals_the_library(E, scale, ef, seed):
    """The oracle makes the benchmark's inputs without the product library (the reference arm of the
    benchmark must not load it); both generators give identical arrays."""
    a = E.gen_rmat(scale, ef, seed=seed, wmin=1, wmax=63)
    b = oracle.gen_rmat(scale, ef, seed=seed, wmin=1, wmax=63, threads=3)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    sa, sb = E.symmetrize(*a), oracle.symmetrize(*b)
    for x, y in zip(sa, sb):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("side", [2, 37, 512])
def test_oracle_grid_generator_equals_the_library(E, side):
    a = E.gen_grid(side, 0.1, 0.001, seed=7, wmin=1, wmax=1000)
    b = oracle.gen_grid(side, 0.1, 0.001, seed=7, wmin=1, wmax=1000, threads=4)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_threaded_fp64_solvers_equal_single_threaded():
    """The threaded PageRank and PPR solves sum in fixed orders: identical results for any thread count."""
    n = 1 << 12
    s, d, _ = oracle.gen_rmat(12, 16, seed=5)
    x1, i1 = oracle.pagerank(n, s, d, threads=1)
    x4, i4 = oracle.pagerank(n, s, d, threads=4)
    assert i1 == i4 and np.array_equal(x1, x4)
    xp, ip = oracle.pagerank_pull(oracle.in_csr(n, s, d), threads=3)
    assert ip == i1 and np.array_equal(xp, x1)
    rng = np.random.default_rng(0)
    w = 1.0 - rng.random(s.size)
    b = rng.random((n, 3))
    for tr in (False, True):
        y1, k1 = oracle.ppr_solve(n, s, d, w, b, transpose=tr, threads=1)
        y5, k5 = oracle.ppr_solve(n, s, d, w, b, transpose=tr, threads=5)
        assert k1 == k5 and np.array_equal(y1, y5)
