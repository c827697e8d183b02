"""Edge-list loader parity with Graph::ReadGraph (CPU only).

The product loader (eeg_graph_load, multi-threaded) and the oracle's sequential restatement are both
checked against what the reference's own ReadGraph returned for the same files (tests/golden/loader.npz).
"""
from pathlib import Path

import numpy as np
import pytest

import oracle

GOLD = Path(__file__).resolve().parent / "golden"
Z = np.load(GOLD / "loader.npz")
FILES = [str(f) for f in Z["files"]]


@pytest.mark.parametrize("fname", FILES)
def test_loader_matches_reference(E, fname):
    g = E.Graph.load(GOLD / "loader" / fname, weighted=True)
    v = g.view()
    n, m, z = (int(x) for x in Z[f"{fname}.meta"])
    assert (v["num_nodes"], v["num_edges"], int(v["has_zero_id"])) == (n, m, z)
    assert np.array_equal(v["src"], Z[f"{fname}.src"])
    assert np.array_equal(v["dst"], Z[f"{fname}.dst"])
    assert np.array_equal(v["weight"], Z[f"{fname}.weight"])


@pytest.mark.parametrize("fname", FILES)
def test_oracle_parser_matches_reference(fname):
    r = oracle.parse(GOLD / "loader" / fname)
    n, m, z = (int(x) for x in Z[f"{fname}.meta"])
    assert (r["num_nodes"], r["num_edges"], int(r["has_zero_id"])) == (n, m, z)
    assert np.array_equal(r["src"], Z[f"{fname}.src"])
    assert np.array_equal(r["weight"], Z[f"{fname}.weight"])


def test_one_based_ids_are_shifted(E):
    g = E.Graph.load(GOLD / "loader" / "one_based.wel")
    s, d = g.normalized_ids()
    assert s.tolist() == [0, 1, 2, 2] and d.tolist() == [1, 2, 0, 2]


def test_unknown_extension_is_an_io_error(E, tmp_path):
    p = tmp_path / "graph.csv"
    p.write_text("0 1\n")
    with pytest.raises(E.EEGError) as ei:
        E.Graph.load(p)
    assert ei.value.status == E.ERR_IO


def test_missing_file(E, tmp_path):
    with pytest.raises(E.EEGError) as ei:
        E.Graph.load(tmp_path / "nope.el")
    assert ei.value.status == E.ERR_IO


def test_multithreaded_parse_equals_single_thread(E, tmp_path):
    s, d, w = E.gen_rmat(14, 16, seed=4)
    p = tmp_path / "big.wel"
    with open(p, "w") as f:
        f.write("# generated\n")
        for a, b, c in zip(s.tolist(), d.tolist(), w.tolist()):
            f.write(f"{a} {b} {c}\n")
    g1 = E.Graph.load(p, threads=1).view()
    g8 = E.Graph.load(p, threads=8).view()
    for k in ("src", "dst", "weight"):
        assert np.array_equal(g1[k], g8[k])
    assert np.array_equal(g8["src"], s) and np.array_equal(g8["weight"], w)
    r = oracle.parse(p)
    assert np.array_equal(r["dst"], d) and r["num_nodes"] == g8["num_nodes"]


def test_bcsr_roundtrip(E, tmp_path):
    s, d, w = E.gen_rmat(10, 8, seed=2)
    g = E.Graph.from_arrays(1024, s, d, w)
    for ext, weighted in (("bwcsr", True), ("bcsr", False)):
        p = tmp_path / f"g.{ext}"
        g.save_bcsr(p)
        v = E.Graph.load(p).view()
        assert v["num_nodes"] == 1024 and v["num_edges"] == s.size and v["has_zero_id"]
        # CSR order: by source, input order within a source
        order = np.argsort(s, kind="stable")
        assert np.array_equal(v["src"], s[order]) and np.array_equal(v["dst"], d[order])
        assert np.array_equal(v["weight"], w[order] if weighted else np.ones_like(w))


@pytest.mark.parametrize("seed", range(12))
def test_loader_fuzz_matches_oracle_parser(E, tmp_path, seed):
    """Seeded random files mixing the golden files' quirks (comment and blank lines, tabs and runs of
    spaces, CRLF, missing or float weights, extra columns, no final newline, 0- or 1-based ids), parsed
    by the multi-threaded product loader and by the oracle's sequential restatement of ReadGraph (pinned
    to the reference's own ReadGraph on the golden files): the same edge lists."""
    rng = np.random.default_rng(seed)
    n_lines = int(rng.integers(1, 3000))
    base = int(rng.integers(0, 2))  # 1-based files have no id 0
    eol = "\r\n" if rng.random() < 0.3 else "\n"
    lines = []
    for _ in range(n_lines):
        r = rng.random()
        if r < 0.05:
            lines.append(rng.choice(["# comment", "% konect header", "", "   ", "c another"]))
            continue
        a, b = (int(x) for x in rng.integers(base, 5000, 2))
        sep = rng.choice([" ", "\t", "  ", " \t "])
        cols = [str(a), str(b)]
        k = rng.random()
        if k < 0.6:
            cols.append(str(int(rng.integers(1, 100))))
        elif k < 0.7:
            cols.append(f"{rng.uniform(1, 50):.3f}")
        elif k < 0.8:
            cols += [str(int(rng.integers(1, 100))), "extra", "9"]
        line = sep.join(cols)
        if rng.random() < 0.1:
            line += " "
        lines.append(line)
    text = eol.join(lines) + ("" if rng.random() < 0.2 else eol)
    p = tmp_path / f"fuzz{seed}.wel"
    p.write_bytes(text.encode())
    want = oracle.parse(p)
    for threads in (1, 4):
        v = E.Graph.load(p, weighted=True, threads=threads).view()
        assert (v["num_nodes"], v["num_edges"], int(v["has_zero_id"])) == \
               (want["num_nodes"], want["src"].size, int(want["has_zero_id"])), (seed, threads)
        assert np.array_equal(v["src"], want["src"]) and np.array_equal(v["dst"], want["dst"])
        assert np.array_equal(v["weight"], want["weight"]), (seed, threads)
