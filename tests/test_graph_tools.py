"""Experiment tools of the reference on the C++ facade (CPU only): graph-info-main (src/graph_info.cpp),
VertexSubgraph::MakeSubgraph (src/graph.cpp:122-203) and Subway's converter (Subway/tools/converter.cpp)."""
import ctypes
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
BIN = ROOT / "eegraph_gb300" / "_bin"
LIB = ROOT / "eegraph_gb300" / "_lib"


def _graph(tmp_path, n=400, m=3000, seed=5):
    rng = np.random.default_rng(seed)
    s = rng.integers(0, n, m)
    d = rng.integers(0, n, m)
    s[:20] = 0  # a hub at id 0 (the file is 0-based)
    w = rng.integers(1, 64, m)
    p = tmp_path / "g.wel"
    with open(p, "w") as f:
        f.write("# test graph\n")
        for a, b, c in zip(s, d, w):
            f.write(f"{a} {b} {c}\n")
    return p, s, d, w


def test_graph_info_numbers(tmp_path):
    p, s, d, w = _graph(tmp_path)
    r = subprocess.run([str(BIN / "graph-info-main"), "--input", str(p)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    n = int(max(s.max(), d.max())) + 1
    deg = np.bincount(s, minlength=n)
    cut = int(0.2 * n)
    vals = {line.split(":")[0]: float(line.split(":")[1]) for line in r.stdout.splitlines() if ":" in line
            and line.split(":")[0] in ("Max degree", "Avg Degree First 20 percent of Vertices",
                                       "Avg Degree Remaining 80 percent of Vertices")}
    assert vals["Max degree"] == deg.max()
    assert abs(vals["Avg Degree First 20 percent of Vertices"] - deg[:cut].mean()) < 1e-3
    assert abs(vals["Avg Degree Remaining 80 percent of Vertices"] - deg[cut:].mean()) < 1e-3


DRIVER = r'''
#include <iostream>
#include "eegraph.hpp"
int main(int argc, char** argv) {
    Graph g(argv[1], true);
    g.ReadGraph();
    VertexSubgraph sub(g, argv[1], true);
    sub.MakeSubgraph(std::stof(argv[2]), std::stoi(argv[3]), (time_t)std::stol(argv[4]));
    std::cout << "SEL";
    for (uint v = 0; v < sub.num_nodes; ++v) if (sub.selected[v]) std::cout << " " << v;
    std::cout << "\nEDGES " << sub.num_edges << "\n";
    for (uint e = 0; e < sub.num_edges; ++e)
        std::cout << sub.edges[e].source << " " << sub.edges[e].end << " " << sub.weights[e] << "\n";
}
'''


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs a C++ compiler")
def test_vertex_subgraph_selection_and_induced_edges(tmp_path):
    p, s, d, w = _graph(tmp_path)
    src = tmp_path / "drv.cpp"
    src.write_text(DRIVER)
    exe = tmp_path / "drv"
    subprocess.run(["g++", "-std=c++17", "-O1", "-o", str(exe), str(src), "-I", str(ROOT / "include"),
                    "-L", str(LIB), "-leegraph_facade", "-leegraph", f"-Wl,-rpath,{LIB}", "-pthread"],
                   check=True, timeout=120)
    pct, source, seed = 0.3, 7, 12345
    r = subprocess.run([str(exe), str(p), str(pct), str(source), str(seed)], capture_output=True, text=True,
                       timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = r.stdout.splitlines()
    sel_line = next(l for l in lines if l.startswith("SEL"))
    got_sel = set(int(x) for x in sel_line.split()[1:])
    k = next(i for i, l in enumerate(lines) if l.startswith("EDGES "))
    got_edges = [tuple(map(int, l.split())) for l in lines[k + 1:k + 1 + int(lines[k].split()[1])]]
    # the selection restated with the same C library's generator
    n = int(max(s.max(), d.max())) + 1
    sel = _selection(n, pct, source, seed)
    assert got_sel == sel
    want_edges = [(a, b, c) for a, b, c in zip(s.tolist(), d.tolist(), w.tolist()) if a in sel and b in sel]
    assert got_edges == want_edges
    assert "Subgraph number of edges = %d" % len(want_edges) in r.stdout


def _selection(n, pct, source, seed):
    """The reference's draw order (src/graph.cpp:148-164): the source, then rand() % (n/5) for the first
    half, rand() % n after; once the lowest fifth is used up its draws move to the whole range (where
    the reference's loop would not end)."""
    libc = ctypes.CDLL(None)
    want_n = int(np.float32(pct) * np.float32(n))  # the reference's float product
    low = n // 5
    sel = {source}
    libc.srand(ctypes.c_uint(seed))
    while len(sel) < want_n:
        rnd = libc.rand()
        from_low = len(sel) < want_n // 2 and sum(1 for v in sel if v < low) < low
        sel.add(rnd % low if from_low else rnd % n)
    return sel


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs a C++ compiler")
@pytest.mark.parametrize("pct", [0.5, 0.9, 1.0])
def test_vertex_subgraph_large_fractions_end(tmp_path, pct):
    """Percentages above 40 % need more distinct ids in the first half than the lowest fifth holds:
    the selection still ends, keeps exactly pct of the vertices, and matches the restated draws."""
    p, s, d, w = _graph(tmp_path, n=300, m=2000, seed=8)
    src = tmp_path / "drv.cpp"
    src.write_text(DRIVER)
    exe = tmp_path / "drv"
    subprocess.run(["g++", "-std=c++17", "-O1", "-o", str(exe), str(src), "-I", str(ROOT / "include"),
                    "-L", str(LIB), "-leegraph_facade", "-leegraph", f"-Wl,-rpath,{LIB}", "-pthread"],
                   check=True, timeout=120)
    r = subprocess.run([str(exe), str(p), str(pct), "250", "77"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    got = set(int(x) for x in next(l for l in r.stdout.splitlines() if l.startswith("SEL")).split()[1:])
    n = int(max(s.max(), d.max())) + 1
    assert len(got) == int(np.float32(pct) * np.float32(n))
    assert got == _selection(n, pct, 250, 77)


def _subway_csr(src, dst, w):
    """Subway/tools/converter.cpp:38-94 (.el) and :95-165 (.wel), restated: num_nodes = largest id + 1,
    offsets by counting, edges of a source in input order."""
    n = int(max(src.max(), dst.max())) + 1 if src.size else 1
    deg = np.bincount(src, minlength=n)
    ptr = np.concatenate([[0], np.cumsum(deg)[:-1]]).astype(np.uint32)
    order = np.argsort(src, kind="stable")
    rec = dst[order] if w is None else np.stack([dst[order], w[order]], 1).reshape(-1)
    return np.concatenate([[n, src.size], ptr, rec]).astype(np.uint32)


@pytest.mark.parametrize("weighted", [False, True])
@pytest.mark.parametrize("one_based", [False, True])
def test_converter_matches_subway_layout(tmp_path, weighted, one_based):
    rng = np.random.default_rng(11)
    n, m = 300, 4000
    s = rng.integers(1 if one_based else 0, n, m)
    d = rng.integers(1 if one_based else 0, n, m)
    w = rng.integers(1, 1000, m)
    p = tmp_path / ("g.wel" if weighted else "g.el")
    with open(p, "w") as f:
        for i in range(m):
            f.write(f"{s[i]} {d[i]} {w[i]}\n" if weighted else f"{s[i]} {d[i]}\n")
    r = subprocess.run([str(BIN / "converter"), str(p)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    out = tmp_path / ("g.bwcsr" if weighted else "g.bcsr")
    got = np.fromfile(out, np.uint32)
    want = _subway_csr(s.astype(np.uint32), d.astype(np.uint32), w.astype(np.uint32) if weighted else None)
    assert np.array_equal(got, want)


def test_converter_messages(tmp_path):
    (tmp_path / "g.txt").write_text("0 1\n")
    r = subprocess.run([str(BIN / "converter"), str(tmp_path / "g.txt")], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "Input file format is not supported." in r.stdout
    assert not (tmp_path / "g.bcsr").exists()
    r = subprocess.run([str(BIN / "converter")], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "There was an error parsing command line arguments" in r.stdout
