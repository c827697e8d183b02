"""Failure detection on the GPU without a GPU fault: a device-side wait that runs out.

Every wait of the persistent kernels (the grid barrier between rounds and sweeps) is bounded. With a
limit of one microsecond (eeg_options.timeout_us) on graphs whose rounds take far longer, a CTA that
reaches a barrier first gives up, raises the abort flag, every CTA leaves at its next barrier and the
call returns EEG_ERR_TIMEOUT; the context and the handle stay usable, and the next run with the default
limit is bit-exact. Nothing faults, traps or hangs.
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rmat20(gpu):
    n = 1 << 20
    s, d, w = gpu.gen_rmat(20, 16, seed=1, wmin=1, wmax=63)
    src = int(np.bincount(s, minlength=n).argmax())
    return n, s, d, w, src


def test_traversal_wait_runs_out_then_recovers(gpu, rmat20):
    n, s, d, w, src = rmat20
    want = {"sssp": oracle.dijkstra(n, s, d, w, src), "bfs": oracle.bfs(n, s, d, src)}
    timed_out = []
    with gpu.VirtualGraph.build(n, s, d, w, K=8) as vg:
        # topology-driven rounds scan every part: each takes far longer than a microsecond
        for algo, variant in (("sssp", "async_push_td"), ("sssp", "sync_push_td"), ("bfs", "async_push_td")):
            _, res = vg.run(algo, variant, src, timeout_us=1, check=False)
            assert res["status"] in (gpu.OK, gpu.ERR_TIMEOUT), res["status"]
            if res["status"] == gpu.ERR_TIMEOUT:
                timed_out.append((algo, variant))
                assert "timeout" in gpu.lib().eeg_last_error().decode()
            got, res2 = vg.run(algo, variant, src)  # default limit, same handle
            assert res2["status"] == gpu.OK
            assert np.array_equal(got, want[algo]), (algo, variant)
    assert timed_out, "no wait ran out under a 1 us limit"


def test_pagerank_wait_runs_out_then_recovers(gpu, rmat20):
    n, s, d, _, _ = rmat20
    xr, _ = oracle.pagerank(n, s, d, threads=oracle.default_threads())
    with gpu.VirtualGraph.build(n, s, d, None, K=16, reverse=True) as vg:
        statuses = []
        for _ in range(3):
            _, res = vg.run("pr", "sync_push_td", timeout_us=1, check=False)
            assert res["status"] in (gpu.OK, gpu.ERR_TIMEOUT)
            statuses.append(res["status"])
        assert gpu.ERR_TIMEOUT in statuses
        x, res = vg.run("pr", "sync_push_td")
    assert res["status"] == gpu.OK
    assert float(np.abs(x / x.sum() - xr / xr.sum()).sum()) <= 1e-6
