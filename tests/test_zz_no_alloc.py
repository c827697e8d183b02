"""The allocation-free entry point eeg_run_noalloc, called through the C ABI (needs a GB300).

It serves callers that cannot allocate device memory when they run a query (a plugin whose host
application owns all GPU memory, a framework that pools every allocation, a loop where cudaMalloc's
possible device synchronisation is not allowed): they pass the virtual graph and the output in memory
they own, and the working memory comes from a fixed device array inside the library. The results must
equal those of eeg_run (integer results: bit-exact), on two calls in a row that share that array.

This file is collected last so that a run stopping at its first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _round256(x):
    return (x + 255) // 256 * 256


def _device_graph(E, torch, vg):
    """Copy a built virtual graph into device buffers owned by the test (torch allocates, not the library)."""
    lay = vg.download()
    info = vg.info()
    dev = {k: torch.from_numpy(np.ascontiguousarray(lay[k]).reshape(-1).view(np.int32)).cuda()
           for k in ("vstart", "vowner", "vcol", "vw")}
    return dev, info


def _noalloc(E, algo, variant, info, dev, source, out):
    its = C.c_uint32(0)
    st = E.lib().eeg_run_noalloc(E.ALGOS[algo], E.VARIANTS[variant], info["num_nodes"], info["num_parts"], info["K"],
                                 C.c_void_p(dev["vstart"].data_ptr()), C.c_void_p(dev["vowner"].data_ptr()),
                                 C.c_void_p(dev["vcol"].data_ptr()), C.c_void_p(dev["vw"].data_ptr()), source,
                                 C.c_void_p(out.data_ptr()), None, C.byref(its))
    return st, its.value


@pytest.mark.parametrize("algo,variant", [("sssp", "sync_push_dd"), ("bfs", "async_push_dd"),
                                          ("sswp", "sync_push_dd"), ("cc", "async_push_td")])
def test_noalloc_matches_eeg_run_twice(gpu, algo, variant):
    torch = pytest.importorskip("torch")
    E = gpu
    scale, n = 14, 1 << 14
    s, d, w = E.gen_rmat(scale, 16, seed=5, wmin=1, wmax=63)
    with E.VirtualGraph.build(n, s, d, w, K=8) as vg:
        dev, info = _device_graph(E, torch, vg)
        out = torch.full((n,), -1, dtype=torch.int32, device="cuda")
        for call, source in enumerate((int(info["max_degree_vertex"]), 3)):  # two calls in a row, one array
            want, _ = vg.run(algo, variant, source)
            torch.cuda.synchronize()
            free_before = torch.cuda.mem_get_info()[0]
            st, its = _noalloc(E, algo, variant, info, dev, source, out)
            torch.cuda.synchronize()
            assert st == E.OK, E.lib().eeg_last_error().decode()
            if call == 1:  # the array's address is known after the first call: nothing is allocated now
                assert torch.cuda.mem_get_info()[0] == free_before
            got = out.cpu().numpy().view(np.uint32)
            assert np.array_equal(got, want)
            assert its > 0


def test_noalloc_rejects_graphs_beyond_the_fixed_array(gpu):
    torch = pytest.importorskip("torch")
    E = gpu
    n = 1 << 10
    s, d, w = E.gen_rmat(10, 8, seed=2)
    with E.VirtualGraph.build(n, s, d, w, K=8) as vg:
        dev, info = _device_graph(E, torch, vg)
        out = torch.zeros(n, dtype=torch.int32, device="cuda")
        too_many_parts = E.NOALLOC_SCRATCH_BYTES // 8 + 1  # 2 queues of 4-byte part ids no longer fit
        info_big = dict(info, num_parts=too_many_parts)
        st, _ = _noalloc(E, "sssp", "sync_push_dd", info_big, dev, 0, out)
        assert st == E.ERR_INVALID
        msg = E.lib().eeg_last_error().decode()
        # 256-byte blocks: the control block, two queues of 4-byte part ids, 4-byte round stamps
        queues = 2 * _round256(4 * too_many_parts) + _round256(4 * n)
        need = int(msg.split("graph needs ")[1].split()[0])
        assert 0 < need - queues <= 1024  # the control block's share
        assert f"graph needs {need} bytes of working memory, more than the 33554432-byte fixed array" in msg
        # the array is still usable afterwards
        st, _ = _noalloc(E, "sssp", "sync_push_dd", info, dev, 0, out)
        assert st == E.OK
        want, _ = vg.run("sssp", "sync_push_dd", 0)
        assert np.array_equal(out.cpu().numpy().view(np.uint32), want)


def test_noalloc_accepts_the_largest_graph_that_fits(gpu):
    """A graph whose working memory is exactly at the limit runs; one 256-byte block more is refused.
    65,536 vertices of 504 or 512 out-edges at K = 8: the largest part count whose queues, stamps and
    control block fit the 32 MiB array."""
    torch = pytest.importorskip("torch")
    E = gpu
    n = 1 << 16
    out = torch.zeros(n, dtype=torch.int32, device="cuda")
    # the control block's share, read from the refusal of a graph that is too large
    dummy = {k: torch.zeros(4, dtype=torch.int32, device="cuda") for k in ("vstart", "vowner", "vcol", "vw")}
    big = E.NOALLOC_SCRATCH_BYTES // 8 + 1
    st, _ = _noalloc(E, "bfs", "sync_push_dd", {"num_nodes": n, "num_parts": big, "K": 8}, dummy, 0, out)
    assert st == E.ERR_INVALID
    ctrl = int(E.lib().eeg_last_error().decode().split("graph needs ")[1].split()[0]) - 2 * _round256(4 * big) \
        - _round256(4 * n)
    p_fit = (E.NOALLOC_SCRATCH_BYTES - ctrl - _round256(4 * n)) // 2 // 256 * 256 // 4
    assert ctrl + 2 * _round256(4 * p_fit) + _round256(4 * n) <= E.NOALLOC_SCRATCH_BYTES
    assert ctrl + 2 * _round256(4 * (p_fit + 1)) + _round256(4 * n) > E.NOALLOC_SCRATCH_BYTES
    # out-degrees: 8 * parts, parts 63 or 64 per vertex, summing to p_fit
    parts = np.full(n, p_fit // n, np.int64)
    parts[: p_fit - int(parts.sum())] += 1
    deg = 8 * parts
    rng = np.random.default_rng(3)
    s = np.repeat(np.arange(n, dtype=np.uint32), deg)
    d = rng.integers(0, n, s.size, dtype=np.uint32)
    w = rng.integers(1, 64, s.size, dtype=np.uint32)
    with E.VirtualGraph.build(n, s, d, w, K=8) as vg:
        dev, info = _device_graph(E, torch, vg)
        assert info["num_parts"] == p_fit
        want, _ = vg.run("sssp", "sync_push_dd", 0)
        st, _ = _noalloc(E, "sssp", "sync_push_dd", info, dev, 0, out)
        torch.cuda.synchronize()
        assert st == E.OK, E.lib().eeg_last_error().decode()
        assert np.array_equal(out.cpu().numpy().view(np.uint32), want)
        # the same vertices with one more part's worth of queue space: refused before any launch
        st, _ = _noalloc(E, "sssp", "sync_push_dd", dict(info, num_parts=p_fit + 64), dev, 0, out)
        assert st == E.ERR_INVALID
