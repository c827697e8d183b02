"""eegraph_gb300 -- GB300-native EEGraph push kernels (BFS, SSSP, SSWP, CC, PageRank).

Python binding of the C ABI in ``include/eegraph_c.h`` (ctypes; numpy arrays in and out). The
compute path is ``_lib/libeegraph.so`` (hand-written sm_103a kernels); there is no Python or CPU
fallback: if the library is missing, importing this package raises.

Names follow the reference (rwatling/EEGraph): ``Graph`` (src/graph.cpp), ``VirtualGraph``
(src/virtual_graph.cpp), the variants of include/globals.hpp:36-41 and one ``run`` per
``eegraph_<algo>`` entry point (include/eegraph.cuh:21-39).
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_lib" / "libeegraph.so"
BIN_DIR = _PKG / "_bin"

# ---------------------------------------------------------------- constants (mirror eegraph_c.h)
OK, ERR_INVALID, ERR_IO, ERR_CUDA, ERR_NOMEM, ERR_TIMEOUT, ERR_ITER_CAP, ERR_UNSUPPORTED, ERR_NO_DEVICE, ERR_ENERGY = range(10)
BFS, SSSP, SSWP, CC, PR = range(5)
ASYNC_PUSH_TD, ASYNC_PUSH_DD, SYNC_PUSH_TD, SYNC_PUSH_DD = range(4)
VARIANTS = {"async_push_td": ASYNC_PUSH_TD, "async_push_dd": ASYNC_PUSH_DD,
            "sync_push_td": SYNC_PUSH_TD, "sync_push_dd": SYNC_PUSH_DD}
ALGOS = {"bfs": BFS, "sssp": SSSP, "sswp": SSWP, "cc": CC, "pr": PR}
DIST_INFINITY = 4294967294
VG_REVERSE, VG_MANAGED, VG_INPUT_DEVICE, VG_SHIFT_ONE, VG_EDGE_IDS, VG_SYMMETRIC = 1, 2, 4, 8, 16, 32
VG_SYMMETRIZE, VG_REVERSE_ONLY = 64, 128

# every function the C header declares (checked by the CPU test suite)
EXPORTED = [
    "eeg_status_string", "eeg_last_error", "eeg_version", "eeg_device_count", "eeg_set_device",
    "eeg_managed_alloc", "eeg_managed_free",
    "eeg_graph_load", "eeg_graph_from_arrays", "eeg_graph_view_get", "eeg_graph_normalized_ids",
    "eeg_graph_destroy", "eeg_graph_save_bcsr", "eeg_gen_rmat", "eeg_gen_grid", "eeg_symmetrize",
    "eeg_vgraph_build", "eeg_vgraph_build_arrays", "eeg_vgraph_get_info", "eeg_vgraph_download",
    "eeg_vgraph_export_reference_layout", "eeg_vgraph_destroy", "eeg_options_init", "eeg_run",
    "eeg_run_noalloc", "eeg_energy_begin", "eeg_energy_mark", "eeg_energy_end", "eeg_energy_destroy",
    "eeg_batch_create", "eeg_batch_set_queries", "eeg_batch_query_offset", "eeg_batch_run", "eeg_batch_rounds",
    "eeg_batch_autotune", "eeg_batch_destroy", "eeg_autotune_k", "eeg_autotune", "eeg_batch_query_times",
    "eeg_ppr_create", "eeg_ppr_set_weights", "eeg_ppr_forward", "eeg_ppr_adjoint", "eeg_ppr_destroy",
    "eeg_batch_set_grid_queries", "eeg_batch_get_config",
    "eeg_stream_create", "eeg_stream_get_info", "eeg_stream_run", "eeg_stream_destroy",
]
NOALLOC_SCRATCH_BYTES = 32 << 20


class GraphView(C.Structure):
    _fields_ = [("num_nodes", C.c_uint32), ("num_edges", C.c_uint64), ("has_zero_id", C.c_int),
                ("is_weighted", C.c_int), ("src", C.POINTER(C.c_uint32)), ("dst", C.POINTER(C.c_uint32)),
                ("weight", C.POINTER(C.c_uint32))]


class VGraphInfo(C.Structure):
    _fields_ = [("num_nodes", C.c_uint32), ("num_edges", C.c_uint64), ("K", C.c_uint32),
                ("num_parts", C.c_uint64), ("num_rparts", C.c_uint64), ("max_out_degree", C.c_uint32),
                ("max_degree_vertex", C.c_uint32), ("device_bytes", C.c_uint64), ("build_ms", C.c_float)]


class Options(C.Structure):
    _fields_ = [("max_iterations", C.c_uint32), ("pr_tolerance", C.c_float), ("pr_damping", C.c_float),
                ("pr_accuracy", C.c_float), ("block_size", C.c_uint32), ("blocks_per_sm", C.c_uint32),
                ("record_activity", C.c_uint32), ("timeout_ms", C.c_uint32), ("host_loop", C.c_uint32),
                ("pr_hot_limit", C.c_uint32), ("delta", C.c_uint32), ("cc_components", C.c_uint32),
                ("timeout_us", C.c_uint32), ("bfs_push_only", C.c_uint32), ("reserved", C.c_uint32 * 2)]


class StreamInfo(C.Structure):
    _fields_ = [("num_nodes", C.c_uint32), ("num_edges", C.c_uint64), ("K", C.c_uint32),
                ("partition_parts", C.c_uint32), ("device_budget_bytes", C.c_uint64), ("host_bytes", C.c_uint64)]


class Tuning(C.Structure):
    _fields_ = [("K", C.c_uint32), ("variant", C.c_int), ("ms", C.c_float), ("ms_table", C.c_float * 12),
                ("blocks_per_sm", C.c_uint32), ("ms_per_blocks", C.c_float * 2)]


class Result(C.Structure):
    _fields_ = [("kernel_ms", C.c_float), ("iterations", C.c_uint32), ("reached_vertices", C.c_uint64),
                ("reached_edges", C.c_uint64), ("parts_processed", C.c_uint64), ("edges_scanned", C.c_uint64),
                ("updates", C.c_uint64), ("algorithmic_bytes", C.c_double), ("gteps", C.c_double),
                ("pr_residual", C.c_double), ("pr_l1_norm", C.c_double), ("num_activity", C.c_uint32),
                ("launches", C.c_uint32), ("partitions", C.c_uint32), ("pull_rounds", C.c_uint32),
                ("reserved", C.c_uint32 * 4)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


class EEGError(RuntimeError):
    def __init__(self, status: int, where: str):
        self.status = status
        super().__init__(f"{where}: {_lib.eeg_status_string(status).decode()} -- {_lib.eeg_last_error().decode()}")


def _load() -> C.CDLL:
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is missing: build it first (python -c 'import __graft_entry__ as g; g.build()')")
    lib = C.CDLL(str(LIB_PATH))
    u32p = C.POINTER(C.c_uint32)
    vp = C.c_void_p
    sig = {
        "eeg_status_string": (C.c_char_p, [C.c_int]),
        "eeg_last_error": (C.c_char_p, []),
        "eeg_version": (C.c_char_p, []),
        "eeg_device_count": (C.c_int, []),
        "eeg_set_device": (C.c_int, [C.c_int]),
        "eeg_managed_alloc": (C.c_int, [C.c_size_t, C.POINTER(vp)]),
        "eeg_managed_free": (None, [vp]),
        "eeg_graph_load": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.POINTER(vp)]),
        "eeg_graph_from_arrays": (C.c_int, [C.c_uint32, C.c_uint64, vp, vp, vp, C.POINTER(vp)]),
        "eeg_graph_view_get": (C.c_int, [vp, C.POINTER(GraphView)]),
        "eeg_graph_normalized_ids": (C.c_int, [vp, vp, vp]),
        "eeg_graph_destroy": (None, [vp]),
        "eeg_graph_save_bcsr": (C.c_int, [vp, C.c_char_p]),
        "eeg_gen_rmat": (C.c_int, [C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_double, C.c_uint64,
                                   C.c_uint32, C.c_uint32, vp, vp, vp]),
        "eeg_gen_grid": (C.c_int, [C.c_uint32, C.c_double, C.c_double, C.c_uint64, C.c_uint32, C.c_uint32,
                                   C.POINTER(C.c_uint64), vp, vp, vp]),
        "eeg_symmetrize": (C.c_int, [C.c_uint64, vp, vp, vp, vp, vp, vp]),
        "eeg_vgraph_build": (C.c_int, [vp, C.c_uint32, C.c_uint32, vp, C.POINTER(vp)]),
        "eeg_vgraph_build_arrays": (C.c_int, [C.c_uint32, C.c_uint64, vp, vp, vp, C.c_uint32, C.c_uint32, vp,
                                              C.POINTER(vp)]),
        "eeg_vgraph_get_info": (C.c_int, [vp, C.POINTER(VGraphInfo)]),
        "eeg_vgraph_download": (C.c_int, [vp, vp, vp, vp, vp, vp]),
        "eeg_vgraph_export_reference_layout": (C.c_int, [vp, vp, vp, vp]),
        "eeg_vgraph_destroy": (None, [vp]),
        "eeg_options_init": (None, [C.POINTER(Options)]),
        "eeg_run": (C.c_int, [vp, C.c_int, C.c_int, C.c_uint32, C.POINTER(Options), vp, C.c_int, u32p, C.c_uint32,
                              vp, C.POINTER(Result)]),
        "eeg_run_noalloc": (C.c_int, [C.c_int, C.c_int, C.c_uint32, C.c_uint64, C.c_uint32, vp, vp, vp, vp,
                                      C.c_uint32, vp, vp, C.POINTER(C.c_uint32)]),
        "eeg_batch_create": (C.c_int, [C.POINTER(vp), C.c_uint32, C.POINTER(vp)]),
        "eeg_batch_set_queries": (C.c_int, [vp, vp, C.c_uint32, C.c_uint32, C.POINTER(C.c_ulonglong)]),
        "eeg_batch_query_offset": (C.c_int, [vp, C.c_uint32, C.POINTER(C.c_ulonglong)]),
        "eeg_batch_run": (C.c_int, [vp, vp, vp, C.POINTER(C.c_float)]),
        "eeg_batch_rounds": (C.c_int, [vp, vp]),
        "eeg_batch_query_times": (C.c_int, [vp, vp]),
        "eeg_batch_autotune": (C.c_int, [vp, vp, C.POINTER(C.c_uint32), C.POINTER(C.c_float)]),
        "eeg_batch_destroy": (None, [vp]),
        "eeg_batch_set_grid_queries": (C.c_int, [vp, C.c_uint32]),
        "eeg_batch_get_config": (C.c_int, [vp, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
        "eeg_autotune_k": (C.c_int, [C.c_uint32, C.c_uint64, vp, vp, vp, C.c_uint32, C.POINTER(C.c_uint32),
                                     C.POINTER(C.c_float)]),
        "eeg_autotune": (C.c_int, [C.c_uint32, C.c_uint64, vp, vp, vp, C.c_int, C.c_uint32, C.POINTER(Tuning)]),
        "eeg_ppr_create": (C.c_int, [vp, C.c_uint32, C.POINTER(vp)]),
        "eeg_ppr_set_weights": (C.c_int, [vp, vp, C.c_int]),
        "eeg_ppr_forward": (C.c_int, [vp, vp, C.c_int, vp, C.c_int, C.POINTER(Options), vp, C.POINTER(Result)]),
        "eeg_ppr_adjoint": (C.c_int, [vp, vp, C.c_int, vp, vp, vp, C.c_int, C.c_int, C.POINTER(Options), vp,
                                      C.POINTER(Result)]),
        "eeg_ppr_destroy": (None, [vp]),
        "eeg_stream_create": (C.c_int, [vp, C.c_uint32, C.c_uint64, C.POINTER(vp)]),
        "eeg_stream_get_info": (C.c_int, [vp, C.POINTER(StreamInfo)]),
        "eeg_stream_run": (C.c_int, [vp, C.c_int, C.c_int, C.c_uint32, C.POINTER(Options), vp, C.c_int, vp,
                                     C.POINTER(Result)]),
        "eeg_stream_destroy": (None, [vp]),
        "eeg_energy_begin": (C.c_int, [C.c_int, C.c_char_p, C.c_uint32, C.POINTER(vp)]),
        "eeg_energy_mark": (C.c_int, [vp]),
        "eeg_energy_end": (C.c_int, [vp, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double)]),
        "eeg_energy_destroy": (None, [vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


_lib = _load()


def lib() -> C.CDLL:
    return _lib


def _check(status: int, where: str) -> None:
    if status != OK:
        raise EEGError(status, where)


def _ptr(a: np.ndarray | None):
    return None if a is None else C.c_void_p(a.ctypes.data)


def _u32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.uint32)


def version() -> str:
    return _lib.eeg_version().decode()


def device_count() -> int:
    return _lib.eeg_device_count()


# ---------------------------------------------------------------- synthetic inputs
def gen_rmat(scale: int, edge_factor: int = 16, a: float = 0.57, b: float = 0.19, c: float = 0.19,
             seed: int = 1, wmin: int = 1, wmax: int = 63, weights: bool = True):
    m = edge_factor << scale
    src = np.empty(m, np.uint32)
    dst = np.empty(m, np.uint32)
    w = np.empty(m, np.uint32) if weights else None
    _check(_lib.eeg_gen_rmat(scale, edge_factor, a, b, c, seed, wmin, wmax, _ptr(src), _ptr(dst), _ptr(w)), "gen_rmat")
    return src, dst, w


def gen_grid(side: int, p_delete: float = 0.1, shortcut_frac: float = 0.001, seed: int = 7, wmin: int = 1,
             wmax: int = 1000):
    cnt = C.c_uint64(0)
    _check(_lib.eeg_gen_grid(side, p_delete, shortcut_frac, seed, wmin, wmax, C.byref(cnt), None, None, None), "gen_grid")
    m = cnt.value
    src, dst, w = np.empty(m, np.uint32), np.empty(m, np.uint32), np.empty(m, np.uint32)
    _check(_lib.eeg_gen_grid(side, p_delete, shortcut_frac, seed, wmin, wmax, C.byref(cnt), _ptr(src), _ptr(dst),
                             _ptr(w)), "gen_grid")
    return src, dst, w


def symmetrize(src, dst, w=None):
    src, dst = _u32(src), _u32(dst)
    m = src.size
    so, do = np.empty(2 * m, np.uint32), np.empty(2 * m, np.uint32)
    wo = np.empty(2 * m, np.uint32) if w is not None else None
    wi = _u32(w) if w is not None else None
    _check(_lib.eeg_symmetrize(m, _ptr(src), _ptr(dst), _ptr(wi), _ptr(so), _ptr(do), _ptr(wo)), "symmetrize")
    return so, do, wo


# ---------------------------------------------------------------- host edge list
class Graph:
    """Host edge list (reference ``Graph``). ``Graph.load(path)`` parses like Graph::ReadGraph."""

    def __init__(self, handle: int):
        self._h = C.c_void_p(handle)

    @classmethod
    def load(cls, path: str | os.PathLike, weighted: bool = True, threads: int = 0) -> "Graph":
        h = C.c_void_p()
        _check(_lib.eeg_graph_load(str(path).encode(), int(weighted), threads, C.byref(h)), f"load {path}")
        return cls(h.value)

    @classmethod
    def from_arrays(cls, num_nodes: int, src, dst, w=None) -> "Graph":
        src, dst = _u32(src), _u32(dst)
        wi = _u32(w) if w is not None else None
        h = C.c_void_p()
        _check(_lib.eeg_graph_from_arrays(num_nodes, src.size, _ptr(src), _ptr(dst), _ptr(wi), C.byref(h)), "from_arrays")
        return cls(h.value)

    def view(self) -> dict:
        v = GraphView()
        _check(_lib.eeg_graph_view_get(self._h, C.byref(v)), "view")
        m = v.num_edges

        def arr(p):
            if not p or m == 0:
                return np.empty(0, np.uint32) if p else None
            return np.ctypeslib.as_array(p, shape=(m,)).copy()

        return {"num_nodes": v.num_nodes, "num_edges": m, "has_zero_id": bool(v.has_zero_id),
                "is_weighted": bool(v.is_weighted), "src": arr(v.src), "dst": arr(v.dst), "weight": arr(v.weight)}

    def normalized_ids(self):
        m = self.view()["num_edges"]
        s, d = np.empty(m, np.uint32), np.empty(m, np.uint32)
        _check(_lib.eeg_graph_normalized_ids(self._h, _ptr(s), _ptr(d)), "normalized_ids")
        return s, d

    def save_bcsr(self, path) -> None:
        _check(_lib.eeg_graph_save_bcsr(self._h, str(path).encode()), "save_bcsr")

    def close(self) -> None:
        if self._h:
            _lib.eeg_graph_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------- device virtual graph
class VirtualGraph:
    """K-bounded virtual graph resident on the GPU (reference ``VirtualGraph`` after MakeGraph)."""

    def __init__(self, handle: int):
        self._h = C.c_void_p(handle)

    @classmethod
    def build(cls, num_nodes: int, src, dst, w=None, K: int = 8, reverse: bool = False, managed: bool = False,
              stream: int | None = None, shift_one: bool = False, edge_ids: bool = False,
              symmetric: bool = False, symmetrize: bool = False, reverse_only: bool = False) -> "VirtualGraph":
        """Build from host arrays (copied to the device inside the call). symmetric=True declares an
        undirected edge list (every arc's reverse present with the same weight); symmetrize=True inserts
        every edge in both directions on the device (the graph of symmetrize(src, dst, w)); reverse_only=True
        builds only what PageRank reads (the transposed graph and the out-degrees)."""
        flags = (VG_REVERSE if reverse else 0) | (VG_MANAGED if managed else 0) | (VG_SHIFT_ONE if shift_one else 0)
        flags |= (VG_EDGE_IDS if edge_ids else 0) | (VG_SYMMETRIC if symmetric else 0)
        flags |= (VG_SYMMETRIZE if symmetrize else 0) | (VG_REVERSE_ONLY if reverse_only else 0)
        h = C.c_void_p()
        src, dst = _u32(src), _u32(dst)
        wi = _u32(w) if w is not None else None
        _check(_lib.eeg_vgraph_build_arrays(num_nodes, src.size, _ptr(src), _ptr(dst), _ptr(wi), K, flags,
                                            C.c_void_p(stream) if stream else None, C.byref(h)), "vgraph_build")
        return cls(h.value)

    @classmethod
    def build_device(cls, num_nodes: int, num_edges: int, src_ptr: int, dst_ptr: int, w_ptr: int | None, K: int = 8,
                     reverse: bool = False, stream: int | None = None, edge_ids: bool = False,
                     symmetrize: bool = False, reverse_only: bool = False) -> "VirtualGraph":
        """Build from device arrays of num_edges input edges (symmetrize: both directions of each;
        reverse_only: only the transposed graph and the out-degrees, for PageRank)."""
        flags = VG_INPUT_DEVICE | (VG_REVERSE if reverse else 0) | (VG_EDGE_IDS if edge_ids else 0)
        flags |= (VG_SYMMETRIZE if symmetrize else 0) | (VG_REVERSE_ONLY if reverse_only else 0)
        h = C.c_void_p()
        _check(_lib.eeg_vgraph_build_arrays(num_nodes, num_edges, C.c_void_p(src_ptr), C.c_void_p(dst_ptr),
                                            C.c_void_p(w_ptr) if w_ptr else None, K, flags,
                                            C.c_void_p(stream) if stream else None, C.byref(h)), "vgraph_build")
        return cls(h.value)

    @classmethod
    def from_graph(cls, g: Graph, K: int = 8, reverse: bool = False, stream: int | None = None) -> "VirtualGraph":
        h = C.c_void_p()
        _check(_lib.eeg_vgraph_build(g._h, K, VG_REVERSE if reverse else 0, C.c_void_p(stream) if stream else None,
                                     C.byref(h)), "vgraph_build")
        return cls(h.value)

    def info(self) -> dict:
        i = VGraphInfo()
        _check(_lib.eeg_vgraph_get_info(self._h, C.byref(i)), "info")
        return {k: getattr(i, k) for k, _ in i._fields_}

    def download(self) -> dict:
        inf = self.info()
        n, P, K = inf["num_nodes"], inf["num_parts"], inf["K"]
        vstart, vowner = np.empty(n + 1, np.uint32), np.empty(P, np.uint32)
        vcol, vw, deg = np.empty(P * K, np.uint32), np.empty(P * K, np.uint32), np.empty(n, np.uint32)
        _check(_lib.eeg_vgraph_download(self._h, _ptr(vstart), _ptr(vowner), _ptr(vcol), _ptr(vw), _ptr(deg)), "download")
        return {"vstart": vstart, "vowner": vowner, "vcol": vcol.reshape(P, K), "vw": vw.reshape(P, K), "outdeg": deg}

    def reference_layout(self):
        inf = self.info()
        n, m, P = inf["num_nodes"], inf["num_edges"], inf["num_parts"]
        npn, el, pnp = np.empty(n, np.uint32), np.empty(2 * m + n, np.uint32), np.empty(2 * P, np.uint32)
        _check(_lib.eeg_vgraph_export_reference_layout(self._h, _ptr(npn), _ptr(el), _ptr(pnp)), "export")
        return npn, el, pnp

    def run(self, algo, variant="sync_push_dd", source: int = 0, *, max_iterations: int = 0,
            pr_tolerance: float = 0.0, pr_damping: float = 0.0, blocks_per_sm: int = 0, timeout_ms: int = 0,
            activity_cap: int = 0, out: np.ndarray | None = None, out_device_ptr: int | None = None,
            stream: int | None = None, check: bool = True, host_loop: bool = False, pr_hot_limit: int = 0,
            delta: int = 0, cc_components: bool = False, timeout_us: int = 0, pr_accuracy: float = 0.0,
            bfs_push_only: bool = False):
        """Run one algorithm; returns (values, result-dict[, activity]). host_loop=True runs one launch
        per round with a host round trip in between (the reference's loop shape), for comparison.
        cc_components=True (CC only) relaxes with weight 0: connected components, not the reference's
        min-plus labels. pr_accuracy: the data-driven PageRank variants' activation threshold (the
        reference's --accuracy; 0 = derived from pr_tolerance)."""
        a = ALGOS[algo] if isinstance(algo, str) else int(algo)
        v = VARIANTS[variant] if isinstance(variant, str) else int(variant)
        o = Options()
        _lib.eeg_options_init(C.byref(o))
        o.max_iterations = max_iterations
        o.pr_tolerance = pr_tolerance
        o.pr_damping = pr_damping
        o.blocks_per_sm = blocks_per_sm
        o.timeout_ms = timeout_ms
        o.host_loop = 1 if host_loop else 0
        o.pr_hot_limit = pr_hot_limit
        o.delta = delta
        o.cc_components = 1 if cc_components else 0
        o.timeout_us = timeout_us
        o.pr_accuracy = pr_accuracy
        o.bfs_push_only = 1 if bfs_push_only else 0
        n = self.info()["num_nodes"]
        if out_device_ptr is not None:
            outp, on_dev, vals = C.c_void_p(out_device_ptr), 1, None
        else:
            vals = out if out is not None else np.empty(n, np.float32 if a == PR else np.uint32)
            outp, on_dev = _ptr(vals), 0
        act = np.zeros(activity_cap, np.uint32) if activity_cap else None
        r = Result()
        st = _lib.eeg_run(self._h, a, v, source, C.byref(o), outp, on_dev,
                          act.ctypes.data_as(C.POINTER(C.c_uint32)) if act is not None else None, activity_cap,
                          C.c_void_p(stream) if stream else None, C.byref(r))
        if check:
            _check(st, f"run {algo}/{variant}")
        res = r.as_dict()
        res["status"] = st
        if act is not None:
            return vals, res, act[: r.num_activity].copy()
        return vals, res

    def close(self) -> None:
        if self._h:
            _lib.eeg_vgraph_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------- graphs larger than device memory
class StreamGraph:
    """Active-subgraph streaming (eeg_stream_*): the graph's CSR stays in page-locked host memory and each
    round's active edges are gathered by the GPU into partition buffers of `budget_bytes` (0 = a quarter of
    the free device memory). Same results as VirtualGraph.run for BFS, SSSP, SSWP and CC."""

    def __init__(self, graph: Graph, K: int = 8, budget_bytes: int = 0):
        self.graph = graph
        h = C.c_void_p()
        _check(_lib.eeg_stream_create(graph._h, K, budget_bytes, C.byref(h)), "stream_create")
        self._h = h

    @classmethod
    def from_arrays(cls, num_nodes: int, src, dst, w=None, K: int = 8, budget_bytes: int = 0) -> "StreamGraph":
        return cls(Graph.from_arrays(num_nodes, src, dst, w), K, budget_bytes)

    def info(self) -> dict:
        i = StreamInfo()
        _check(_lib.eeg_stream_get_info(self._h, C.byref(i)), "stream_info")
        return {k: getattr(i, k) for k, _ in i._fields_}

    def run(self, algo, variant="sync_push_dd", source: int = 0, *, max_iterations: int = 0,
            cc_components: bool = False, out_device_ptr: int | None = None, stream: int | None = None,
            check: bool = True):
        a = ALGOS[algo] if isinstance(algo, str) else int(algo)
        v = VARIANTS[variant] if isinstance(variant, str) else int(variant)
        o = Options()
        _lib.eeg_options_init(C.byref(o))
        o.max_iterations = max_iterations
        o.cc_components = 1 if cc_components else 0
        n = self.info()["num_nodes"]
        if out_device_ptr is not None:
            outp, on_dev, vals = C.c_void_p(out_device_ptr), 1, None
        else:
            vals = np.empty(n, np.uint32)
            outp, on_dev = _ptr(vals), 0
        r = Result()
        st = _lib.eeg_stream_run(self._h, a, v, source, C.byref(o), outp, on_dev, C.c_void_p(stream) if stream else None,
                                 C.byref(r))
        if check:
            _check(st, f"stream_run {algo}/{variant}")
        res = r.as_dict()
        res["status"] = st
        return vals, res

    def close(self) -> None:
        if self._h:
            _lib.eeg_stream_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------- batched queries
class Query(C.Structure):
    _fields_ = [("graph", C.c_uint32), ("algo", C.c_uint32), ("source", C.c_uint32), ("reserved", C.c_uint32)]


class Batch:
    """Many BFS/SSSP/SSWP queries over many device graphs in one launch (eeg_batch_*)."""

    def __init__(self, graphs):
        self.graphs = list(graphs)  # keep them alive
        arr = (C.c_void_p * len(self.graphs))(*[g._h.value for g in self.graphs])
        h = C.c_void_p()
        _check(_lib.eeg_batch_create(arr, len(self.graphs), C.byref(h)), "batch_create")
        self._h = h
        self.nq = 0

    def set_queries(self, queries, cluster_size: int = 0) -> int:
        """queries: iterable of (graph_index, algo, source); returns the output size in uint32 words."""
        qs = [(g, ALGOS[a] if isinstance(a, str) else int(a), s) for g, a, s in queries]
        arr = (Query * max(len(qs), 1))(*[Query(g, a, s, 0) for g, a, s in qs])
        words = C.c_ulonglong()
        _check(_lib.eeg_batch_set_queries(self._h, arr, len(qs), cluster_size, C.byref(words)), "batch_set_queries")
        self.nq = len(qs)
        self.out_words = words.value
        return words.value

    def offsets(self):
        out = []
        for i in range(self.nq):
            o = C.c_ulonglong()
            _check(_lib.eeg_batch_query_offset(self._h, i, C.byref(o)), "batch_query_offset")
            out.append(o.value)
        return out

    def run(self, out_device_ptr: int, stream: int | None = None) -> float:
        ms = C.c_float()
        _check(_lib.eeg_batch_run(self._h, C.c_void_p(out_device_ptr), C.c_void_p(stream) if stream else None,
                                  C.byref(ms)), "batch_run")
        return ms.value

    def rounds(self) -> np.ndarray:
        r = np.zeros(max(self.nq, 1), np.uint32)
        _check(_lib.eeg_batch_rounds(self._h, _ptr(r)), "batch_rounds")
        return r[: self.nq]

    def query_times(self) -> np.ndarray:
        """(num_queries, 3): start ns, end ns, cluster index of each query in the last run."""
        t = np.zeros(3 * max(self.nq, 1), np.uint64)
        _check(_lib.eeg_batch_query_times(self._h, _ptr(t)), "batch_query_times")
        return t[: 3 * self.nq].reshape(-1, 3)

    def autotune(self, out_device_ptr: int):
        c, ms = C.c_uint32(), C.c_float()
        _check(_lib.eeg_batch_autotune(self._h, C.c_void_p(out_device_ptr), C.byref(c), C.byref(ms)), "batch_autotune")
        return c.value, ms.value

    def set_grid_queries(self, count: int) -> None:
        """Run the `count` largest queries one after another on the whole grid before the clusters."""
        _check(_lib.eeg_batch_set_grid_queries(self._h, count), "batch_set_grid_queries")

    def config(self) -> tuple[int, int]:
        """(cluster size, whole-grid queries) of the current configuration."""
        c, g = C.c_uint32(), C.c_uint32()
        _check(_lib.eeg_batch_get_config(self._h, C.byref(c), C.byref(g)), "batch_get_config")
        return c.value, g.value

    def close(self):
        if self._h:
            _lib.eeg_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PPR:
    """Differentiable personalised PageRank on a virtual graph built with reverse=True, edge_ids=True
    (C ABI eeg_ppr_*). columns=1 runs the single-column kernels, 2..64 the batched row kernels.
    Array arguments are numpy arrays (host) or device pointers given as ints."""

    def __init__(self, vg: VirtualGraph, columns: int):
        self._h = C.c_void_p()
        self.vg = vg
        self.columns = columns
        inf = vg.info()
        self.n, self.m = inf["num_nodes"], inf["num_edges"]
        _check(_lib.eeg_ppr_create(vg._h, columns, C.byref(self._h)), "ppr_create")

    @staticmethod
    def _opts(tol, damping, max_iterations, timeout_ms):
        o = Options()
        _lib.eeg_options_init(C.byref(o))
        o.pr_tolerance = tol
        o.pr_damping = damping
        o.max_iterations = max_iterations
        o.timeout_ms = timeout_ms
        return o

    @staticmethod
    def _arg(a, dtype=np.float32):
        if a is None:
            return None, 0, None
        if isinstance(a, int):
            return C.c_void_p(a), 1, None
        arr = np.ascontiguousarray(a, dtype=dtype)
        return C.c_void_p(arr.ctypes.data), 0, arr

    def set_weights(self, w) -> None:
        p, dev, keep = self._arg(w)
        _check(_lib.eeg_ppr_set_weights(self._h, p, dev), "ppr_set_weights")

    def forward(self, teleport, x_out=None, *, tol=0.0, damping=0.0, max_iterations=0, timeout_ms=0, stream=None,
                check=True):
        """teleport: n x columns (host array or device pointer). Returns (X or None, result dict).
        x_out: device pointer (int) to write X to; with a host teleport and no x_out, X is returned."""
        tp, tdev, keep = self._arg(teleport)
        o = self._opts(tol, damping, max_iterations, timeout_ms)
        r = Result()
        if isinstance(x_out, int):
            xp, xdev, xh = C.c_void_p(x_out), 1, None
        elif x_out is False:
            xp, xdev, xh = None, 0, None
        else:
            xh = np.empty((self.n, self.columns), np.float32)
            xp, xdev = C.c_void_p(xh.ctypes.data), 0
        st = _lib.eeg_ppr_forward(self._h, tp, tdev, xp, xdev, C.byref(o), C.c_void_p(stream) if stream else None,
                                  C.byref(r))
        if check:
            _check(st, "ppr_forward")
        res = r.as_dict()
        res["status"] = st
        return xh, res

    def adjoint(self, dl_dx, *, outputs=("dw", "dwn", "dt"), out_ptrs=None, out_host=None, accumulate=False,
                tol=0.0, damping=0.0, max_iterations=0, timeout_ms=0, stream=None, check=True):
        """dl_dx: n x columns. Host mode returns dict of numpy arrays for the requested outputs
        (dw: raw-weight gradient, dwn: normalised-weight gradient, dt: teleport gradient), written into
        out_host's arrays when given; device mode writes to out_ptrs = {"dw": ptr, ...}."""
        gp, gdev, keep = self._arg(dl_dx)
        o = self._opts(tol, damping, max_iterations, timeout_ms)
        r = Result()
        out = {}
        if out_ptrs is not None:
            ptr = {k: C.c_void_p(v) for k, v in out_ptrs.items()}
            on_dev = 1
        elif out_host is not None:
            out = dict(out_host)
            for k, v in out.items():
                if not (v.flags.c_contiguous and v.dtype == np.float32):
                    raise ValueError(f"out_host[{k!r}] must be a C-contiguous float32 array")
            ptr = {k: C.c_void_p(v.ctypes.data) for k, v in out.items()}
            on_dev = 0
        else:
            if "dw" in outputs:
                out["dw"] = np.empty(self.m, np.float32)
            if "dwn" in outputs:
                out["dwn"] = np.empty(self.m, np.float32)
            if "dt" in outputs:
                out["dt"] = np.empty((self.n, self.columns), np.float32)
            ptr = {k: C.c_void_p(v.ctypes.data) for k, v in out.items()}
            on_dev = 0
        st = _lib.eeg_ppr_adjoint(self._h, gp, gdev, ptr.get("dt"), ptr.get("dw"), ptr.get("dwn"), on_dev,
                                  1 if accumulate else 0, C.byref(o), C.c_void_p(stream) if stream else None,
                                  C.byref(r))
        if check:
            _check(st, "ppr_adjoint")
        res = r.as_dict()
        res["status"] = st
        return out, res

    def close(self):
        if self._h:
            _lib.eeg_ppr_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def shard_columns(columns: int, world: int) -> list[list[int]]:
    """Contiguous split of a personalised-PageRank column batch over `world` GPUs (sizes differ by at
    most one). Each GPU solves its columns on the whole graph; the batch's edge gradients are the sum
    of the GPUs' (one reduction of m floats), its X and dLoss/dT the concatenation."""
    if world < 1 or columns < 1:
        raise ValueError("columns and world must be >= 1")
    base, extra = divmod(columns, world)
    out, c = [], 0
    for r in range(world):
        k = base + (1 if r < extra else 0)
        out.append(list(range(c, c + k)))
        c += k
    return out


def shard_queries(costs, world: int) -> list[list[int]]:
    """Static partition of independent queries over `world` GPUs by estimated work (largest first onto the
    least-loaded GPU; ties to the lower rank). Every rank computes the same partition from the same costs,
    so no exchange is needed; each shard keeps its queries in input order."""
    if world < 1:
        raise ValueError("world must be >= 1")
    costs = [float(c) for c in costs]
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    load = [0.0] * world
    shards: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        shards[r].append(i)
        load[r] += costs[i]
    return [sorted(sh) for sh in shards]


def autotune_k(num_nodes: int, src, dst, w=None, reps: int = 3):
    """Fastest part size K for this graph (BFS + SSSP from the max-degree vertex); (K, ms per K)."""
    src, dst = _u32(src), _u32(dst)
    wi = _u32(w) if w is not None else None
    k = C.c_uint32()
    ms = (C.c_float * 3)()
    _check(_lib.eeg_autotune_k(num_nodes, src.size, _ptr(src), _ptr(dst), _ptr(wi), reps, C.byref(k), ms), "autotune_k")
    return k.value, {4: ms[0], 8: ms[1], 16: ms[2]}


def autotune(num_nodes: int, src, dst, w=None, algo="sssp", reps: int = 3) -> dict:
    """Fastest (K, variant) for this graph and algorithm among K in {4, 8, 16} and the variants with the
    default's fixed point, then the number of resident CTAs per SM for it; returns {"K", "variant", "ms",
    "table": {(K, variant): ms}, "blocks_per_sm", "ms_per_blocks": {b: ms}}."""
    src, dst = _u32(src), _u32(dst)
    wi = _u32(w) if w is not None else None
    a = ALGOS[algo] if isinstance(algo, str) else int(algo)
    t = Tuning()
    _check(_lib.eeg_autotune(num_nodes, src.size, _ptr(src), _ptr(dst), _ptr(wi), a, reps, C.byref(t)), "autotune")
    names = {v: k for k, v in VARIANTS.items()}
    table = {((4, 8, 16)[i // 4], names[i % 4]): t.ms_table[i] for i in range(12) if t.ms_table[i] >= 0}
    per_blocks = {b + 1: t.ms_per_blocks[b] for b in range(2) if t.ms_per_blocks[b] >= 0}
    return {"K": t.K, "variant": names[t.variant], "ms": t.ms, "table": table, "blocks_per_sm": t.blocks_per_sm,
            "ms_per_blocks": per_blocks}


# ---------------------------------------------------------------- energy
class EnergySession:
    """GPU energy of a region (NVML energy counter; reference nvmlClass)."""

    def __init__(self, device: int = 0, csv_path: str | None = None, period_us: int = 1000):
        h = C.c_void_p()
        st = _lib.eeg_energy_begin(device, csv_path.encode() if csv_path else None, period_us, C.byref(h))
        self.available = st == OK
        self.reason = "" if self.available else _lib.eeg_last_error().decode()
        self._h = h if self.available else None

    def end(self):
        if not self._h:
            return None
        j, s, w = C.c_double(), C.c_double(), C.c_double()
        st = _lib.eeg_energy_end(self._h, C.byref(j), C.byref(s), C.byref(w))
        _lib.eeg_energy_destroy(self._h)
        self._h = None
        if st != OK:
            self.reason = _lib.eeg_last_error().decode()
            return None
        return {"joules": j.value, "seconds": s.value, "avg_watts": w.value}
