"""CPU oracle for the EEGraph push-kernel path -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import this module, as the
checker. It wraps two native libraries:

* ``_build/liboracle.so`` -- the C restatement in oracle.c (always built, no GPU needed);
* ``_ref/libref.so``      -- the reference's own host code (Graph::ReadGraph, VirtualGraph::MakeGraph,
  ``{bfs,sssp,sswp,cc}::seq_cpu``) compiled from its sources by ``make ref``; present only where the
  reference source tree is (used to pin the restatement and to make tests/golden/).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_LIB = HERE / "_build" / "liboracle.so"
REF_LIB = HERE / "_ref" / "libref.so"
INF = 4294967294
ALGO = {"bfs": 0, "sssp": 1, "sswp": 2, "cc": 3}


def reference_dir() -> Path | None:
    """The reference source tree: $EEG_REFERENCE_DIR, else a checkout named `reference` beside this
    repository; None where neither holds the sources (the reference is then not built)."""
    for cand in (os.environ.get("EEG_REFERENCE_DIR"), HERE.parent.parent / "reference"):
        if cand and Path(cand, "src", "sssp.cu").exists():
            return Path(cand)
    return None


def build(ref_dir: str | None = None) -> None:
    """Compile the restatement and, when the reference sources are present, the reference library."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    ref = Path(ref_dir) if ref_dir else reference_dir()
    if ref is not None and Path(ref, "src", "sssp.cu").exists():
        subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REF={ref}"], check=True)


def default_threads() -> int:
    return max(1, min(64, os.cpu_count() or 1))


_o = None
_r = None


def _vp(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def _u32(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


def lib():
    global _o
    if _o is None:
        if not ORACLE_LIB.exists():
            build()
        _o = C.CDLL(str(ORACLE_LIB))
        vp, u64, u32 = C.c_void_p, C.c_uint64, C.c_uint32
        _o.orc_parse_count.argtypes = [C.c_char_p, C.POINTER(u64), C.POINTER(u32), C.POINTER(C.c_int)]
        _o.orc_parse_fill.argtypes = [C.c_char_p, C.c_int, vp, vp, vp]
        _o.orc_num_parts.restype = u64
        _o.orc_num_parts.argtypes = [u32, u64, vp, u32]
        _o.orc_virtual_graph.argtypes = [u32, u64, vp, vp, vp, u32, vp, vp, vp]
        _o.orc_init_values.argtypes = [C.c_int, u32, u32, vp]
        _o.orc_seq_sweep.restype = C.c_int64
        _o.orc_seq_sweep.argtypes = [C.c_int, u32, u64, vp, vp, vp, u32, C.c_int, u64, vp]
        _o.orc_frontier_sweep.restype = C.c_int64
        _o.orc_frontier_sweep.argtypes = [C.c_int, u32, u64, vp, vp, vp, u32, C.c_int, u32, vp]
        _o.orc_bfs.argtypes = [u32, u64, vp, vp, u32, vp]
        _o.orc_dijkstra.argtypes = [u32, u64, vp, vp, vp, u32, vp]
        _o.orc_widest.argtypes = [u32, u64, vp, vp, vp, u32, vp]
        _o.orc_cc_labels.argtypes = [u32, u64, vp, vp, vp, vp]
        _o.orc_pagerank.restype = C.c_int64
        _o.orc_pagerank.argtypes = [u32, u64, vp, vp, C.c_double, C.c_double, u64, vp]
        _o.orc_ppr_solve.restype = C.c_int64
        _o.orc_ppr_solve.argtypes = [u32, u64, vp, vp, vp, u32, vp, C.c_double, C.c_int, C.c_double, C.c_double,
                                     u64, vp]
        _o.orc_ppr_grads.argtypes = [u32, u64, vp, vp, vp, u32, vp, vp, C.c_double, vp, vp, vp]
        _o.orc_pagerank_mt.restype = C.c_int64
        _o.orc_pagerank_mt.argtypes = [u32, u64, vp, vp, C.c_double, C.c_double, u64, C.c_int, vp]
        _o.orc_ppr_solve_mt.restype = C.c_int64
        _o.orc_ppr_solve_mt.argtypes = [u32, u64, vp, vp, vp, u32, vp, C.c_double, C.c_int, C.c_double,
                                        C.c_double, u64, C.c_int, vp]
        _o.orc_in_csr.argtypes = [u32, u64, vp, vp, vp, vp, vp]
        _o.orc_pagerank_pull.restype = C.c_int64
        _o.orc_pagerank_pull.argtypes = [u32, vp, vp, vp, C.c_double, C.c_double, u64, C.c_int, vp]
        _o.orc_gen_rmat.restype = C.c_int
        _o.orc_gen_rmat.argtypes = [u32, u32, C.c_double, C.c_double, C.c_double, u64, u32, u32, C.c_int, vp, vp, vp]
        _o.orc_gen_grid.restype = C.c_int
        _o.orc_gen_grid.argtypes = [u32, C.c_double, C.c_double, u64, u32, u32, C.c_int, C.POINTER(u64), vp, vp, vp]
        _o.orc_symmetrize.argtypes = [u64, vp, vp, vp, vp, vp, vp]
    return _o


def ref_available() -> bool:
    return REF_LIB.exists()


def ref():
    global _r
    if _r is None:
        _r = C.CDLL(str(REF_LIB))
        vp, u64, u32 = C.c_void_p, C.c_uint64, C.c_uint32
        _r.ref_graph_read.restype = vp
        _r.ref_graph_read.argtypes = [C.c_char_p, C.c_int]
        _r.ref_graph_info.argtypes = [vp, C.POINTER(u32), C.POINTER(u64), C.POINTER(C.c_int), C.POINTER(u64)]
        _r.ref_graph_copy.argtypes = [vp, vp, vp, vp]
        _r.ref_graph_free.argtypes = [vp]
        _r.ref_num_parts.restype = u64
        _r.ref_num_parts.argtypes = [u32, u64, vp, vp, vp]
        _r.ref_virtual_graph.argtypes = [u32, u64, vp, vp, vp, vp, vp, vp]
        _r.ref_seq_cpu.restype = C.c_int
        _r.ref_seq_cpu.argtypes = [C.c_int, u32, u64, vp, vp, vp, u32, vp, C.POINTER(C.c_double)]
        _r.ref_part_size.restype = u32
    return _r


# ---------------------------------------------------------------- restatement wrappers
def parse(path, weighted=True):
    m, n, z = C.c_uint64(), C.c_uint32(), C.c_int()
    if lib().orc_parse_count(str(path).encode(), C.byref(m), C.byref(n), C.byref(z)) != 0:
        raise FileNotFoundError(path)
    s, d = np.empty(m.value, np.uint32), np.empty(m.value, np.uint32)
    w = np.empty(m.value, np.uint32) if weighted else None
    lib().orc_parse_fill(str(path).encode(), int(weighted), _vp(s), _vp(d), _vp(w))
    return {"num_nodes": n.value, "num_edges": m.value, "has_zero_id": bool(z.value), "src": s, "dst": d, "weight": w}


def virtual_graph(n, src, dst, w, K=8):
    src, dst = _u32(src), _u32(dst)
    w = _u32(w) if w is not None else None
    P = lib().orc_num_parts(n, src.size, _vp(src), K)
    npn = np.empty(n, np.uint32)
    el = np.empty(2 * src.size + n, np.uint32)
    pnp = np.empty(2 * P, np.uint32)
    lib().orc_virtual_graph(n, src.size, _vp(src), _vp(dst), _vp(w), K, _vp(npn), _vp(el), _vp(pnp))
    return npn, el, pnp


def init_values(algo, n, source):
    d = np.empty(n, np.uint32)
    lib().orc_init_values(ALGO[algo], n, source, _vp(d))
    return d


def seq_sweep(algo, n, src, dst, w, source=0, K=8, wrap=False, max_sweeps=0, timed=False):
    """Restatement of the reference's seq_cpu(VirtualGraph) on the lossless layout. With timed=True
    also returns the seconds of the sweeps alone (layout construction excluded)."""
    import time

    npn, el, pnp = virtual_graph(n, src, dst, w, K)
    d = init_values(algo, n, source)
    t0 = time.perf_counter()
    sweeps = lib().orc_seq_sweep(ALGO[algo], n, pnp.size // 2, _vp(npn), _vp(el), _vp(pnp), K, int(wrap),
                                 max_sweeps, _vp(d))
    secs = time.perf_counter() - t0
    return (d, sweeps, secs) if timed else (d, sweeps)


def seq_sweep_layout(algo, n, layout, source=0, K=8, wrap=False, max_sweeps=0):
    """seq_sweep on a layout virtual_graph() already built: (values, sweeps, seconds of the sweeps)."""
    import time

    npn, el, pnp = layout
    d = init_values(algo, n, source)
    t0 = time.perf_counter()
    sweeps = lib().orc_seq_sweep(ALGO[algo], n, pnp.size // 2, _vp(npn), _vp(el), _vp(pnp), K, int(wrap),
                                 max_sweeps, _vp(d))
    return d, sweeps, time.perf_counter() - t0


def frontier_sweep(algo, n, src, dst, w, source=0, K=8, seed_all=False):
    npn, el, pnp = virtual_graph(n, src, dst, w, K)
    d = init_values(algo, n, source)
    rounds = lib().orc_frontier_sweep(ALGO[algo], n, pnp.size // 2, _vp(npn), _vp(el), _vp(pnp), K, int(seed_all),
                                      source, _vp(d))
    return d, rounds


def bfs(n, src, dst, source):
    d = np.empty(n, np.uint32)
    src, dst = _u32(src), _u32(dst)
    lib().orc_bfs(n, src.size, _vp(src), _vp(dst), source, _vp(d))
    return d


def dijkstra(n, src, dst, w, source):
    d = np.empty(n, np.uint32)
    src, dst, w = _u32(src), _u32(dst), _u32(w)
    lib().orc_dijkstra(n, src.size, _vp(src), _vp(dst), _vp(w), source, _vp(d))
    return d


def widest(n, src, dst, w, source):
    d = np.empty(n, np.uint32)
    src, dst, w = _u32(src), _u32(dst), _u32(w)
    lib().orc_widest(n, src.size, _vp(src), _vp(dst), _vp(w), source, _vp(d))
    return d


def cc_labels(n, src, dst, w):
    d = np.empty(n, np.uint32)
    src, dst, w = _u32(src), _u32(dst), _u32(w)
    lib().orc_cc_labels(n, src.size, _vp(src), _vp(dst), _vp(w), _vp(d))
    return d


def pagerank(n, src, dst, damping=0.85, tol=1e-15, max_iter=100000, threads=1):
    """FP64 PageRank fixed point (power iteration; same result for any thread count)."""
    x = np.empty(n, np.float64)
    src, dst = _u32(src), _u32(dst)
    it = lib().orc_pagerank_mt(n, src.size, _vp(src), _vp(dst), damping, tol, max_iter, threads, _vp(x))
    return x, it


def in_csr(n, src, dst):
    """(off[n+1], in-edge sources grouped by target, out-degrees) for pagerank_pull."""
    src, dst = _u32(src), _u32(dst)
    off, isrc, deg = np.empty(n + 1, np.uint64), np.empty(src.size, np.uint32), np.empty(n, np.uint32)
    lib().orc_in_csr(n, src.size, _vp(src), _vp(dst), _vp(off), _vp(isrc), _vp(deg))
    return off, isrc, deg


def pagerank_pull(csr_in, damping=0.85, tol=1e-15, max_iter=100000, threads=1):
    """pagerank() on a prepared in_csr(): the sweeps alone."""
    off, isrc, deg = csr_in
    n = deg.size
    x = np.empty(n, np.float64)
    it = lib().orc_pagerank_pull(n, _vp(off), _vp(isrc), _vp(deg), damping, tol, max_iter, threads, _vp(x))
    return x, it


def _f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a if shape is None else a.reshape(shape)


def ppr_solve(n, src, dst, w, b, transpose=False, damping=0.85, tol=1e-14, max_iter=100000, threads=1):
    """FP64 personalised PageRank (transpose=False: X = (1-d)B + d W^T X) or its adjoint
    (transpose=True: L = B + d W L) on row-normalised weights; b is n x C. Returns (Y, sweeps)."""
    src, dst, w = _u32(src), _u32(dst), _f64(w)
    b = _f64(b)
    if b.ndim == 1:
        b = b.reshape(n, 1)
    C_ = b.shape[1]
    y = np.empty((n, C_), np.float64)
    scale = 1.0 if transpose else 1.0 - damping
    it = lib().orc_ppr_solve_mt(n, src.size, _vp(src), _vp(dst), _vp(w), C_, _vp(b), scale, int(transpose), damping,
                                tol, max_iter, threads, _vp(y))
    if it < 0:
        raise RuntimeError("oracle PPR solve did not converge")
    return y, it


def ppr_grads(n, src, dst, w, X, L, damping=0.85):
    """(dLoss/dW_normalised per edge, dLoss/dw_raw per edge, dLoss/dT) from X and the adjoint L."""
    src, dst, w = _u32(src), _u32(dst), _f64(w)
    X, L = _f64(X), _f64(L)
    C_ = X.shape[1]
    m = src.size
    gWn = np.empty(m, np.float64)
    gw = np.empty(m, np.float64)
    gT = np.empty_like(L)
    lib().orc_ppr_grads(n, m, _vp(src), _vp(dst), _vp(w), C_, _vp(X), _vp(L), damping, _vp(gWn), _vp(gw), _vp(gT))
    return gWn, gw, gT


def ppr(n, src, dst, w, T, G, damping=0.85, tol=1e-14, threads=1):
    """Forward, adjoint and gradients in FP64. T: teleport (n x C), G: dLoss/dX (n x C)."""
    X, itf = ppr_solve(n, src, dst, w, T, False, damping, tol, threads=threads)
    L, ita = ppr_solve(n, src, dst, w, G, True, damping, tol, threads=threads)
    gWn, gw, gT = ppr_grads(n, src, dst, w, X, L, damping)
    return {"X": X, "L": L, "gWn": gWn, "gw": gw, "gT": gT, "sweeps": (itf, ita)}


# ---------------------------------------------------------------- synthetic inputs (no product library)
def gen_rmat(scale, edge_factor=16, a=0.57, b=0.19, c=0.19, seed=1, wmin=1, wmax=63, weights=True, threads=0):
    """The benchmark's seeded R-MAT edge list (identical to the product library's generator)."""
    m = edge_factor << scale
    src, dst = np.empty(m, np.uint32), np.empty(m, np.uint32)
    w = np.empty(m, np.uint32) if weights else None
    if lib().orc_gen_rmat(scale, edge_factor, a, b, c, seed, wmin, wmax, threads or default_threads(), _vp(src),
                          _vp(dst), _vp(w)) != 0:
        raise ValueError("invalid R-MAT parameters")
    return src, dst, w


def gen_grid(side, p_delete=0.1, shortcut_frac=0.001, seed=7, wmin=1, wmax=1000, threads=0):
    """The benchmark's road-like grid: both arcs of every kept undirected edge, weights shared."""
    cnt = C.c_uint64(0)
    t = threads or default_threads()
    if lib().orc_gen_grid(side, p_delete, shortcut_frac, seed, wmin, wmax, t, C.byref(cnt), None, None, None) != 0:
        raise ValueError("invalid grid parameters")
    m = cnt.value
    src, dst, w = np.empty(m, np.uint32), np.empty(m, np.uint32), np.empty(m, np.uint32)
    lib().orc_gen_grid(side, p_delete, shortcut_frac, seed, wmin, wmax, t, C.byref(cnt), _vp(src), _vp(dst), _vp(w))
    return src, dst, w


def symmetrize(src, dst, w=None):
    src, dst = _u32(src), _u32(dst)
    m = src.size
    so, do = np.empty(2 * m, np.uint32), np.empty(2 * m, np.uint32)
    wo = np.empty(2 * m, np.uint32) if w is not None else None
    lib().orc_symmetrize(m, _vp(src), _vp(dst), _vp(_u32(w)) if w is not None else None, _vp(so), _vp(do), _vp(wo))
    return so, do, wo


def expected(algo, variant, n, src, dst, w, source):
    """Fixed point every GPU variant must reproduce (integer algorithms) -- by the independent oracles,
    except CC/SYNC_PUSH_DD whose source-seeded fixed point is the frontier restatement's."""
    if algo == "bfs":
        return bfs(n, src, dst, source)
    if algo == "sssp":
        return dijkstra(n, src, dst, w, source)
    if algo == "sswp":
        return widest(n, src, dst, w, source)
    if algo == "cc":
        if variant == "sync_push_dd":
            return frontier_sweep("cc", n, src, dst, w, source, seed_all=False)[0]
        return cc_labels(n, src, dst, w)
    raise ValueError(algo)


# ---------------------------------------------------------------- the reference itself (oracle/_ref)
def ref_read_graph(path, weighted=True):
    r = ref()
    h = r.ref_graph_read(str(path).encode(), int(weighted))
    n, m, z, nw = C.c_uint32(), C.c_uint64(), C.c_int(), C.c_uint64()
    r.ref_graph_info(h, C.byref(n), C.byref(m), C.byref(z), C.byref(nw))
    s, d = np.empty(m.value, np.uint32), np.empty(m.value, np.uint32)
    w = np.empty(nw.value, np.uint32)
    r.ref_graph_copy(h, _vp(s), _vp(d), _vp(w) if nw.value else None)
    r.ref_graph_free(h)
    return {"num_nodes": n.value, "num_edges": m.value, "has_zero_id": bool(z.value), "src": s, "dst": d,
            "weight": w if weighted else None}


def ref_virtual_graph(n, src, dst, w):
    src, dst = _u32(src), _u32(dst)
    w = _u32(w) if w is not None else None
    r = ref()
    P = r.ref_num_parts(n, src.size, _vp(src), _vp(dst), _vp(w))
    npn, el, pnp = np.empty(n, np.uint32), np.empty(2 * src.size + n, np.uint32), np.empty(2 * P, np.uint32)
    r.ref_virtual_graph(n, src.size, _vp(src), _vp(dst), _vp(w), _vp(npn), _vp(el), _vp(pnp))
    return npn, el, pnp


def ref_seq_cpu(algo, n, src, dst, w, source=0, timed=False):
    """The reference's seq_cpu; with timed=True also returns the seconds spent in seq_cpu alone."""
    src, dst = _u32(src), _u32(dst)
    w = _u32(w) if w is not None else None
    d = np.empty(n, np.uint32)
    secs = C.c_double(0.0)
    if ref().ref_seq_cpu(ALGO[algo], n, src.size, _vp(src), _vp(dst), _vp(w), source, _vp(d), C.byref(secs)) != 0:
        raise ValueError("ref_seq_cpu rejected its arguments")
    return (d, secs.value) if timed else d
