"""Bucketed SSSP/SSWP rounds (eeg_options.delta > 0, SYNC_PUSH_DD) on the GPU: far piles, moving
thresholds, three rotating piles. Every bucket width must give the oracle's fixed point (Dijkstra
distances, max-min widest-path values) bit-exactly, in the persistent kernel and in host-loop mode,
for every part size, on low- and high-diameter graphs; other variants ignore the option."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _graphs(E):
    out = []
    s, d, w = E.gen_rmat(12, 8, seed=31, wmin=1, wmax=63)
    out.append(("rmat12", 1 << 12, s, d, w))
    side = 48
    s, d, w = E.gen_grid(side, 0.1, 0.01, seed=7, wmin=1, wmax=1000)
    out.append(("grid48", side * side, s, d, w))
    # a path with a few long shortcuts: many buckets, many far rounds
    n = 300
    ps = np.arange(n - 1, dtype=np.uint32)
    s = np.concatenate([ps, np.array([0, 10, 50], np.uint32)])
    d = np.concatenate([ps + 1, np.array([200, 250, 299], np.uint32)])
    w = np.concatenate([np.full(n - 1, 3, np.uint32), np.array([900, 5, 2000], np.uint32)])
    out.append(("path300", n, s, d, w))
    return out


@pytest.mark.parametrize("delta", [1, 7, 64, 1000, 1 << 30])
@pytest.mark.parametrize("K", [4, 8, 16])
def test_bucketed_rounds_equal_oracle(gpu, delta, K):
    E = gpu
    for name, n, s, d, w in _graphs(E):
        with E.VirtualGraph.build(n, s, d, w, K=K) as vg:
            for src in (0, int(np.bincount(s, minlength=n).argmax())):
                want = {"sssp": oracle.dijkstra(n, s, d, w, src), "sswp": oracle.widest(n, s, d, w, src)}
                for algo in ("sssp", "sswp"):
                    got, res = vg.run(algo, "sync_push_dd", src, delta=delta)
                    assert np.array_equal(got, want[algo]), (name, algo, src, delta, K)
                    assert res["iterations"] > 0


@pytest.mark.parametrize("delta", [1, 100])
def test_bucketed_host_loop_and_repeats(gpu, delta):
    E = gpu
    side = 40
    s, d, w = E.gen_grid(side, 0.1, 0.01, seed=9, wmin=1, wmax=1000)
    n = side * side
    with E.VirtualGraph.build(n, s, d, w, K=8) as vg:
        want = oracle.dijkstra(n, s, d, w, 5)
        for _ in range(2):  # the far flags of one run must not leak into the next
            got, _ = vg.run("sssp", "sync_push_dd", 5, delta=delta)
            assert np.array_equal(got, want)
        got, _ = vg.run("sssp", "sync_push_dd", 5, delta=delta, host_loop=True)
        assert np.array_equal(got, want)
        # other variants ignore the option
        got, _ = vg.run("sssp", "async_push_dd", 5, delta=delta)
        assert np.array_equal(got, want)
        wide, _ = vg.run("sswp", "sync_push_dd", 5, delta=delta)
        assert np.array_equal(wide, oracle.widest(n, s, d, w, 5))
