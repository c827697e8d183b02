"""Graphs larger than device memory: active-subgraph streaming (eeg_stream_*), on the GPU.

The model of the Subway code in the reference (Subway/shared/subgraph_generator.cu, partitioner.cu and
the subway/*-sync / *-async programs): the CSR stays in host memory and every round's active edges are
gathered into partition buffers of a fixed device budget. Budgets far below the graph's size force
many partitions per round; the results must equal the oracle bit for bit (the fixed points of the
in-memory path) for every budget, part size and variant.
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _budget(K, parts):
    """Device bytes for two partition buffers of `parts` parts each."""
    return 2 * (8 * K + 4) * parts


@pytest.fixture(scope="module")
def rmat14(gpu):
    n = 1 << 14
    s, d, w = gpu.gen_rmat(14, 16, seed=11, wmin=1, wmax=63)
    src = int(np.bincount(s, minlength=n).argmax())
    ss, ds, ws = gpu.symmetrize(s, d, w)
    return n, (s, d, w), (ss, ds, ws), src


@pytest.mark.parametrize("K", [4, 8, 16])
@pytest.mark.parametrize("parts", [37, 1000, 0])  # tiny and medium budgets; 0 = a quarter of free memory
@pytest.mark.parametrize("variant", ["sync_push_dd", "async_push_dd"])
def test_stream_equals_oracle(gpu, rmat14, K, parts, variant):
    n, (s, d, w), (ss, ds, ws), src = rmat14
    budget = _budget(K, parts) if parts else 0
    with gpu.StreamGraph.from_arrays(n, s, d, w, K=K, budget_bytes=budget) as sg:
        info = sg.info()
        if parts:
            assert info["partition_parts"] == parts and info["device_budget_bytes"] == budget
        for algo in ("bfs", "sssp", "sswp"):
            got, res = sg.run(algo, variant, src)
            want = oracle.expected(algo, "sync_push_dd", n, s, d, w, src)
            assert np.array_equal(got, want), (algo, variant, K, parts, int((got != want).sum()))
            if parts == 37:
                assert res["partitions"] > res["iterations"]  # several partitions per round
            assert res["reached_edges"] > 0 and res["edges_scanned"] >= res["reached_edges"]
    with gpu.StreamGraph.from_arrays(n, ss, ds, ws, K=K, budget_bytes=budget) as sg:
        got, _ = sg.run("cc", variant, 0)
    assert np.array_equal(got, oracle.cc_labels(n, ss, ds, ws)), (variant, K, parts)


def test_stream_equals_in_memory_run_at_scale(gpu):
    """R-MAT scale 20 (16.8 M edges) through buffers holding about a tenth of a round's parts."""
    n = 1 << 20
    s, d, w = gpu.gen_rmat(20, 16, seed=2, wmin=1, wmax=63)
    src = int(np.bincount(s, minlength=n).argmax())
    with gpu.VirtualGraph.build(n, s, d, w, K=8) as vg:
        want = {a: vg.run(a, "sync_push_dd", src)[0] for a in ("bfs", "sssp", "sswp")}
    with gpu.StreamGraph.from_arrays(n, s, d, w, K=8, budget_bytes=_budget(8, 200_000)) as sg:
        for algo in ("bfs", "sssp", "sswp"):
            for variant in ("sync_push_dd", "async_push_dd"):
                got, res = sg.run(algo, variant, src)
                assert np.array_equal(got, want[algo]), (algo, variant)
                assert res["partitions"] > res["iterations"]
    assert np.array_equal(want["sssp"], oracle.dijkstra(n, s, d, w, src))


def test_stream_high_diameter_grid(gpu):
    side = 96
    n = side * side
    s, d, w = gpu.gen_grid(side, 0.1, 0.001, seed=7, wmin=1, wmax=1000)
    with gpu.StreamGraph.from_arrays(n, s, d, w, K=4, budget_bytes=_budget(4, 64)) as sg:
        for algo in ("bfs", "sssp", "sswp"):
            got, res = sg.run(algo, "sync_push_dd", 0)
            assert np.array_equal(got, oracle.expected(algo, "sync_push_dd", n, s, d, w, 0)), algo
            assert res["iterations"] > 10  # many rounds (partitions relaxed in place shorten them)


def test_stream_from_one_based_file(gpu, tmp_path):
    s, d, w = gpu.gen_rmat(10, 8, seed=4, wmin=1, wmax=63)
    p = tmp_path / "g.wel"
    with open(p, "w") as f:
        for a, b, c in zip(s.tolist(), d.tolist(), w.tolist()):
            f.write(f"{a + 1} {b + 1} {c}\n")  # no id 0: shifted down by one when loaded
    g = gpu.Graph.load(p)
    n = g.view()["num_nodes"]
    with gpu.StreamGraph(g, K=8, budget_bytes=_budget(8, 50)) as sg, gpu.VirtualGraph.from_graph(g, K=8) as vg:
        for algo in ("bfs", "sssp"):
            got, _ = sg.run(algo, "sync_push_dd", 0)
            want, _ = vg.run(algo, "sync_push_dd", 0)
            assert got.size == n and np.array_equal(got, want), algo


def test_stream_cc_components_and_round_cap(gpu):
    n = 1 << 12
    s, d, w = gpu.gen_rmat(12, 4, seed=6, wmin=1, wmax=63)
    ss, ds, ws = gpu.symmetrize(s, d, w)
    with gpu.StreamGraph.from_arrays(n, ss, ds, ws, K=8, budget_bytes=_budget(8, 100)) as sg:
        got, _ = sg.run("cc", "sync_push_dd", cc_components=True)
        assert np.array_equal(got, oracle.cc_labels(n, ss, ds, np.zeros_like(ws)))
        _, res = sg.run("sssp", "sync_push_dd", 0, max_iterations=1, check=False)
        assert res["status"] == gpu.ERR_ITER_CAP


def test_stream_rejections(gpu):
    n = 1 << 8
    s, d, w = gpu.gen_rmat(8, 4, seed=1)
    with pytest.raises(gpu.EEGError) as e:
        gpu.StreamGraph.from_arrays(n, s, d, w, K=8, budget_bytes=_budget(8, 1) - 1)
    assert e.value.status == gpu.ERR_INVALID and "budget" in str(e.value)
    with gpu.StreamGraph.from_arrays(n, s, d, w, K=8, budget_bytes=_budget(8, 1)) as sg:
        _, res = sg.run("pr", "sync_push_td", check=False)
        assert res["status"] == gpu.ERR_UNSUPPORTED
        _, res = sg.run("bfs", "sync_push_dd", n, check=False)
        assert res["status"] == gpu.ERR_INVALID
        got, res = sg.run("bfs", "sync_push_dd", 0)  # one part per partition still works
    assert np.array_equal(got, oracle.bfs(n, s, d, 0))
