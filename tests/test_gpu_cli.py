"""The per-algorithm executables and the C++ facade behind them, on the GPU.

They are the reference's `{bfs,sssp,sswp,cc,pr}-main` (src/*_main.cu): same flags, same console lines
("Number of iterations = ", "Processing finished in X (ms).", "Total GPU activity finished in X (ms)."),
`--output` as "i value" lines, `--debug` comparing against a sequential host recomputation.
"""
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]
BIN = ROOT / "eegraph_gb300" / "_bin"


def _write_wel(path, s, d, w, one_based=False):
    off = 1 if one_based else 0
    with open(path, "w") as f:
        f.write("# generated R-MAT\n")
        for a, b, c in zip(s.tolist(), d.tolist(), w.tolist()):
            f.write(f"{a + off} {b + off} {c}\n")


def _run(exe, *args):
    r = subprocess.run([str(BIN / exe), *map(str, args)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def _read_out(path, dtype):
    vals = np.loadtxt(path, dtype=np.float64)
    assert np.array_equal(vals[:, 0], np.arange(vals.shape[0]))
    return vals[:, 1].astype(dtype)


@pytest.fixture(scope="module")
def graph(tmp_path_factory, gpu):
    s, d, w = gpu.gen_rmat(12, 8, seed=4, wmin=1, wmax=63)
    n = int(max(s.max(), d.max())) + 1  # what the loader derives from the file (largest id + 1)
    p = tmp_path_factory.mktemp("g") / "g.wel"
    _write_wel(p, s, d, w)
    return p, n, s, d, w


@pytest.mark.parametrize("exe,algo", [("bfs-main", "bfs"), ("sssp-main", "sssp"), ("sswp-main", "sswp"),
                                      ("cc-main", "cc")])
@pytest.mark.parametrize("variant", ["async_push_td", "sync_push_dd"])
def test_cli_output_and_lines(graph, tmp_path, exe, algo, variant):
    p, n, s, d, w = graph
    out = tmp_path / "out.txt"
    src = int(np.bincount(s, minlength=n).argmax())
    stdout = _run(exe, "--input", p, "--source", src, "--variant", variant, "--output", out, "--debug", "true")
    assert re.search(r"Number of iterations = \d+", stdout)
    assert re.search(r"Processing finished in [\d.]+ \(ms\)\.", stdout)
    assert re.search(r"Total GPU activity finished in [\d.]+ \(ms\)\.", stdout)
    assert "Arrays begin to differ" not in stdout  # --debug host check agrees
    got = _read_out(out, np.uint64)
    want = oracle.expected(algo, variant, n, s, d, w, src).astype(np.uint64)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("weighted", [True, False])
def test_cli_binary_csr_input(graph, tmp_path, weighted):
    """Subway's binary CSR files: `converter` turns the text list into .bwcsr (weighted) or .bcsr, and the
    executables read them (Subway/tools/converter.cpp, Subway/shared/subway_graph.cu) with the same
    results as the text file."""
    p, n, s, d, w = graph
    txt = tmp_path / ("g.wel" if weighted else "g.el")
    with open(txt, "w") as f:
        for a, b, c in zip(s.tolist(), d.tolist(), w.tolist()):
            f.write(f"{a} {b} {c}\n" if weighted else f"{a} {b}\n")
    _run("converter", txt)
    binf = tmp_path / ("g.bwcsr" if weighted else "g.bcsr")
    assert binf.exists()
    src = int(np.bincount(s, minlength=n).argmax())
    for exe, algo in ([("sssp-main", "sssp"), ("sswp-main", "sswp")] if weighted else [("bfs-main", "bfs")]):
        for variant in ("sync_push_dd", "async_push_td"):
            out = tmp_path / f"{algo}-{variant}.txt"
            _run(exe, "--input", binf, "--source", src, "--variant", variant, "--output", out)
            got = _read_out(out, np.uint64)
            want = oracle.expected(algo, variant, n, s, d, w, src).astype(np.uint64)
            assert np.array_equal(got, want), (exe, variant)


@pytest.mark.parametrize("exe,algo", [("bfs-main", "bfs"), ("sssp-main", "sssp"), ("cc-main", "cc")])
def test_cli_stream_budget(graph, tmp_path, exe, algo):
    """--stream-budget keeps the graph in host memory and streams each round's active subgraph through
    1 MiB of device buffers (Subway's model): the same output as the device-resident run."""
    p, n, s, d, w = graph
    src = int(np.bincount(s, minlength=n).argmax())
    out = tmp_path / "out.txt"
    stdout = _run(exe, "--input", p, "--source", src, "--variant", "sync_push_dd", "--output", out,
                  "--stream-budget", 1, "--debug", "true")
    assert re.search(r"Processing finished in [\d.]+ \(ms\)\.", stdout)
    assert "Arrays begin to differ" not in stdout
    got = _read_out(out, np.uint64)
    want = oracle.cc_labels(n, s, d, w) if algo == "cc" else oracle.expected(algo, "sync_push_dd", n, s, d, w, src)
    assert np.array_equal(got, want.astype(np.uint64))


def test_cli_pagerank_um_activity_energy(graph, tmp_path):
    p, n, s, d, w = graph
    out, ef, es = tmp_path / "pr.txt", tmp_path / "energy.csv", tmp_path / "stats.csv"
    stdout = _run("pr-main", "--input", p, "--variant", "sync_push_td", "--output", out, "--um", "true",
                  "--energy", "true", "--efile", ef, "--estats", es, "--k", "16")
    assert "Unified memory version" in stdout
    x = _read_out(out, np.float64)
    xr, _ = oracle.pagerank(n, s, d)
    assert np.abs(x / x.sum() - xr / xr.sum()).sum() <= 1e-5  # printed with 6 significant digits
    # energy: reported in joules when NVML works, "Energy unavailable" otherwise -- never a failure
    assert ("Energy consumed" in stdout and es.exists()) or "Energy unavailable" in stdout


@pytest.mark.parametrize("variant", ["sync_push_dd", "async_push_dd"])
def test_cli_pagerank_data_driven_accuracy(graph, tmp_path, variant):
    """pr-main's data-driven variants take the reference's --accuracy as their activation threshold: a
    coarse threshold stops early with a larger error, a fine one meets the oracle."""
    p, n, s, d, w = graph
    xr, _ = oracle.pagerank(n, s, d)
    errs = []
    for acc in ("0.01", "1e-9"):
        out = tmp_path / f"pr-{acc}.txt"
        _run("pr-main", "--input", p, "--variant", variant, "--output", out, "--accuracy", acc)
        x = _read_out(out, np.float64)
        errs.append(np.abs(x / x.sum() - xr / xr.sum()).sum())
    assert errs[1] <= 1e-5 < errs[0]


def test_cli_one_based_file_and_activity(tmp_path, gpu):
    s, d, w = gpu.gen_rmat(10, 8, seed=9, wmin=1, wmax=63)
    p = tmp_path / "one.wel"
    _write_wel(p, s, d, w, one_based=True)  # no id 0: ids are shifted down by one when loaded
    out = tmp_path / "o.txt"
    stdout = _run("bfs-main", "--input", p, "--source", 0, "--variant", "sync_push_dd", "--output", out,
                  "--activity", "true")
    n = int(max(s.max(), d.max())) + 1
    got = _read_out(out, np.uint64)
    assert np.array_equal(got, oracle.bfs(n, s, d, 0).astype(np.uint64)[: got.size])


def test_sweep_writes_the_reference_layout(tmp_path):
    """sweep-main runs every (framework, energy, algorithm, trial, variant) and writes the reference's
    files: <algo>/<bench>[-energy]/[um-]<variant><trial> holding the program's timing lines, plus the
    energy readings/stats files (or the 'Energy unavailable' line where NVML is missing)."""
    import eegraph_gb300 as E

    s, d, w = E.gen_rmat(9, 8, seed=51, wmin=1, wmax=63)
    g = tmp_path / "tiny.wel"
    _write_wel(g, s, d, w)
    out = tmp_path / "sweep"
    r = subprocess.run([str(BIN / "sweep-main"), "--graphs", str(g), "--names", "tiny", "--trials", "2",
                        "--algos", "bfs,sssp,pr", "--frameworks", "classic,um", "--energy", "both", "--out", str(out)],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    for algo in ("bfs", "sssp", "pr"):
        for sub in ("tiny", "tiny-energy"):
            for prefix in ("", "um-"):
                for v in ("async-push-td", "async-push-dd", "sync-push-td", "sync-push-dd"):
                    for t in (0, 1):
                        f = out / algo / sub / f"{prefix}{v}{t}"
                        text = f.read_text()
                        assert "Processing finished in" in text, (f, text)
                        if sub.endswith("energy"):
                            assert ("Energy consumed" in text) or ("Energy unavailable" in text), text
                            if "Energy consumed" in text:
                                assert (out / algo / sub / f"{prefix}{v}-stats{t}").exists()


UM_SUB_DRIVER = r'''
#include <iostream>
#include "eegraph.hpp"
int main(int argc, char** argv) {
    Graph g(argv[1], true);
    g.ReadGraph();
    VertexSubgraph a(g, argv[1], true);
    a.MakeSubgraph(0.4f, 3, (time_t)99);
    UMGraph ug(argv[1], true);
    ug.ReadGraph();
    UMVertexSubgraph b(ug, argv[1], true);
    b.MakeSubgraph(0.4f, 3, (time_t)99);
    bool same = a.num_edges == b.num_edges && a.subgraph_num_nodes == b.subgraph_num_nodes;
    for (uint v = 0; same && v < a.num_nodes; ++v) same = a.selected[v] == b.selected[v];
    for (uint e = 0; same && e < a.num_edges; ++e)
        same = a.edges[e].source == b.edges[e].source && a.edges[e].end == b.edges[e].end &&
               a.weights[e] == b.weights[e];
    std::cout << (same ? "SAME" : "DIFFERENT") << " " << a.num_edges << std::endl;
    UMVirtualGraph vg(b);
    vg.MakeGraph();
    std::cout << "PARTS " << vg.numParts << std::endl;
    return same ? 0 : 1;
}
'''


def test_um_vertex_subgraph_equals_vertex_subgraph(tmp_path):
    """UMVertexSubgraph (managed-memory twin) keeps the same vertices and edges as VertexSubgraph for the
    same seed, and its result builds a UMVirtualGraph."""
    import shutil

    import eegraph_gb300 as E

    if shutil.which("g++") is None:
        pytest.skip("needs a C++ compiler")
    s, d, w = E.gen_rmat(10, 8, seed=61, wmin=1, wmax=63)
    g = tmp_path / "g.wel"
    _write_wel(g, s, d, w)
    src = tmp_path / "drv.cpp"
    src.write_text(UM_SUB_DRIVER)
    exe = tmp_path / "drv"
    lib = ROOT / "eegraph_gb300" / "_lib"
    subprocess.run(["g++", "-std=c++17", "-O1", "-o", str(exe), str(src), "-I", str(ROOT / "include"),
                    "-L", str(lib), "-leegraph_facade", "-leegraph", f"-Wl,-rpath,{lib}", "-pthread"],
                   check=True, timeout=180)
    r = subprocess.run([str(exe), str(g)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "SAME" in r.stdout and "PARTS " in r.stdout


def test_cli_extension_flags(graph, tmp_path, gpu):
    """--delta gives sssp-main the same distances; --cc-components gives cc-main the component minima of
    the (undirected) input, by scipy."""
    p, n, s, d, w = graph
    src = int(np.bincount(s, minlength=n).argmax())
    plain, bucketed = tmp_path / "plain.txt", tmp_path / "bucketed.txt"
    _run("sssp-main", "--input", p, "--source", src, "--variant", "sync_push_dd", "--output", plain)
    _run("sssp-main", "--input", p, "--source", src, "--variant", "sync_push_dd", "--output", bucketed,
         "--delta", 16)
    assert np.array_equal(_read_out(plain, np.uint64), _read_out(bucketed, np.uint64))
    ss, ds, ws = gpu.symmetrize(s, d, w)
    psym = tmp_path / "sym.wel"
    _write_wel(psym, ss, ds, ws)
    out = tmp_path / "cc.txt"
    _run("cc-main", "--input", psym, "--output", out, "--cc-components", "true")
    sp = pytest.importorskip("scipy.sparse")
    csgraph = pytest.importorskip("scipy.sparse.csgraph")
    g = sp.coo_matrix((np.ones(ss.size), (ss.astype(np.int64), ds.astype(np.int64))), shape=(n, n))
    _, comp = csgraph.connected_components(g, directed=False)
    first = np.full(comp.max() + 1, n, np.int64)
    np.minimum.at(first, comp, np.arange(n))
    assert np.array_equal(_read_out(out, np.uint64), first[comp].astype(np.uint64))
