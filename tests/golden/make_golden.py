"""Generate the golden vectors in this directory from the REFERENCE ITSELF.

Runs the reference's own host code, compiled from its sources by ``make -C oracle ref`` into
oracle/_ref/libref.so (Graph::ReadGraph, VirtualGraph::MakeGraph, {bfs,sssp,sswp,cc}::seq_cpu), on
small seeded graphs and loader files, and stores inputs and outputs:

* ``seq_cpu.npz``  -- per case: n, src, dst, w, source and ref_<algo> = seq_cpu(VirtualGraph) with the
  reference drivers' initial values (K = Part_Size = 8); SSSP outputs keep the reference's uint32
  wrap of INF + w (the oracle reproduces it with wrap=True).
* ``layout.npz``   -- nodePointer / edgeList / partNodePointer from MakeGraph (lossless, see
  oracle/ref_shim.cpp) for two graphs.
* ``loader/*``     -- text edge lists exercising the parsing rules, and ``loader.npz`` with what
  Graph::ReadGraph returned for each.

Usage (needs the reference sources and nvcc; run from the repository root):
    make -C oracle ref && python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

import eegraph_gb300 as E  # noqa: E402  (host-side generators only; no GPU needed)
import oracle  # noqa: E402


def hand_graphs():
    g = {}
    # path 0->1->2->3->4
    g["path"] = (5, [0, 1, 2, 3], [1, 2, 3, 4], [3, 1, 4, 1], 0)
    # hub with degree 40 (> 4K for K=8), spokes back to the hub, weights varied
    s = [0] * 40 + list(range(1, 41))
    d = list(range(1, 41)) + [0] * 40
    w = [(7 * i) % 63 + 1 for i in range(80)]
    g["hub"] = (41, s, d, w, 0)
    # disconnected pieces, isolated vertices 7..9, self loops and duplicate edges
    g["pieces"] = (10, [0, 0, 1, 1, 2, 4, 5, 6, 6, 3], [1, 1, 2, 2, 2, 5, 6, 4, 4, 3],
                   [5, 2, 9, 9, 1, 3, 3, 1, 7, 2], 4)
    # single vertex, no edges
    g["single"] = (1, [], [], [], 0)
    # source without out-edges
    g["sink_source"] = (4, [0, 1, 2], [1, 2, 3], [1, 1, 1], 3)
    # heavy weights near the uint32 range on a cycle
    g["heavy"] = (3, [0, 1, 2], [1, 2, 0], [2000000000, 2000000000, 5], 0)
    return g


def synthetic():
    out = {}
    s, d, w = E.gen_rmat(8, 8, seed=11, wmin=1, wmax=63)
    out["rmat8"] = (256, s, d, w, int(np.bincount(s, minlength=256).argmax()))
    s, d, w = E.gen_rmat(10, 16, seed=1, wmin=1, wmax=63)
    out["rmat10"] = (1024, s, d, w, int(np.bincount(s, minlength=1024).argmax()))
    s, d, w = E.gen_rmat(9, 8, seed=5, wmin=1, wmax=63)
    s2, d2, w2 = E.symmetrize(s, d, w)
    out["rmat9_sym"] = (512, s2, d2, w2, int(np.bincount(s2, minlength=512).argmax()))
    s, d, w = E.gen_grid(16, 0.1, 0.01, seed=7, wmin=1, wmax=1000)
    out["grid16"] = (256, s, d, w, 0)
    return out


LOADER_FILES = {
    "comments.el": "# comment line\n% another\n\n0 1\n1 2\n 2 3\n2\t0\n",
    "one_based.wel": "1 2 5\n2 3 7\n3 1 2\n3 3 1\n",
    "missing_weight.wel": "0 1 4\n1 2\n2 0 9 99\n",
    "crlf.txt": "0 1 3\r\n1 2 4\r\n2 0 5\r\n",
    "float_weight.edges": "0 1 3.7\n1 0 abc\n",
    "no_newline.edgelist": "0 1 2\n1 2 3",
    "big_ids.el": "4000000000 7\n7 4000000000\n",
}


def main() -> None:
    if not oracle.ref_available():
        raise SystemExit("oracle/_ref/libref.so missing: run `make -C oracle ref` first")
    cases = {**hand_graphs(), **synthetic()}
    arrays = {}
    for name, (n, s, d, w, source) in cases.items():
        s = np.asarray(s, np.uint32)
        d = np.asarray(d, np.uint32)
        w = np.asarray(w, np.uint32)
        arrays[f"{name}.n"] = np.array([n], np.uint32)
        arrays[f"{name}.src"] = s
        arrays[f"{name}.dst"] = d
        arrays[f"{name}.w"] = w
        arrays[f"{name}.source"] = np.array([source], np.uint32)
        for algo in ("bfs", "sssp", "sswp", "cc"):
            arrays[f"{name}.ref_{algo}"] = oracle.ref_seq_cpu(algo, n, s, d, w, source)
        arrays[f"{name}.ref_sssp_unit"] = oracle.ref_seq_cpu("sssp", n, s, d, np.ones_like(w), source)
    np.savez_compressed(HERE / "seq_cpu.npz", names=np.array(sorted(cases)), **arrays)

    lay = {}
    for name in ("hub", "rmat8"):
        n, s, d, w, _ = cases[name]
        npn, el, pnp = oracle.ref_virtual_graph(n, np.asarray(s, np.uint32), np.asarray(d, np.uint32),
                                                np.asarray(w, np.uint32))
        lay[f"{name}.nodePointer"], lay[f"{name}.edgeList"], lay[f"{name}.partNodePointer"] = npn, el, pnp
    np.savez_compressed(HERE / "layout.npz", **lay)

    ldir = HERE / "loader"
    ldir.mkdir(exist_ok=True)
    lg = {}
    for fname, text in LOADER_FILES.items():
        p = ldir / fname
        p.write_bytes(text.encode())
        r = oracle.ref_read_graph(p, weighted=True)
        lg[f"{fname}.meta"] = np.array([r["num_nodes"], r["num_edges"], int(r["has_zero_id"])], np.uint64)
        lg[f"{fname}.src"], lg[f"{fname}.dst"], lg[f"{fname}.weight"] = r["src"], r["dst"], r["weight"]
    np.savez_compressed(HERE / "loader.npz", files=np.array(sorted(LOADER_FILES)), **lg)
    print("golden vectors written:", len(cases), "graphs,", len(LOADER_FILES), "loader files")


if __name__ == "__main__":
    main()
