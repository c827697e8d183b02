"""Command-line handling of the per-algorithm executables (CPU only: no graph is processed).

Same reactions as the reference's ArgumentParser (src/argument_parsing.cpp): help text on a missing
or malformed command line, exit code 0, the same messages.
"""
import subprocess
from pathlib import Path

import pytest

BIN = Path(__file__).resolve().parents[1] / "eegraph_gb300" / "_bin"


def _run(*args):
    return subprocess.run([str(BIN / "sssp-main"), *args], capture_output=True, text=True, timeout=60)


def test_executables_exist():
    for exe in ("bfs-main", "sssp-main", "sswp-main", "cc-main", "pr-main"):
        assert (BIN / exe).exists(), exe


def test_help_and_missing_input():
    r = _run()
    assert r.returncode == 0 and "Required arguments" in r.stdout
    r = _run("--help")
    assert r.returncode == 0 and "--input" in r.stdout


def test_odd_pairing():
    r = _run("--input")
    assert r.returncode == 0 and "error parsing command line arguments" in r.stdout


def test_unknown_flag_and_variant():
    r = _run("--input", "x.el", "--bogus", "1")
    assert r.returncode == 0 and "<--bogus>" in r.stdout
    r = _run("--input", "x.el", "--variant", "nope")
    assert r.returncode == 0 and "Variant not recognized" in r.stdout


def test_energy_requires_files():
    r = _run("--input", "x.el", "--energy", "true")
    assert r.returncode == 0 and "energy file" in r.stdout


def test_bad_k_rejected():
    r = _run("--input", "x.el", "--k", "5")
    assert r.returncode == 0 and "--k must be 4, 8 or 16" in r.stdout


def test_unreadable_graph_reports():
    r = _run("--input", "/nonexistent/graph.el")
    assert "Error reading graph" in r.stdout or "Graph file not read correctly" in r.stdout


def test_extension_flags_parse():
    """--delta and --cc-components are accepted (the run then stops at the missing graph file)."""
    r = subprocess.run([str(BIN / "cc-main"), "--input", "/nonexistent/graph.el", "--cc-components", "true"],
                       capture_output=True, text=True, timeout=60)
    assert "<--cc-components>" not in r.stdout
    assert "Error reading graph" in r.stdout or "Graph file not read correctly" in r.stdout
    r = _run("--input", "/nonexistent/graph.el", "--delta", "16")
    assert "<--delta>" not in r.stdout
    assert "Error reading graph" in r.stdout or "Graph file not read correctly" in r.stdout
    assert "--delta" in _run("--help").stdout and "--cc-components" in _run("--help").stdout


def test_sweep_command_line():
    """sweep-main (the reference's src/main.cu measurement sweep): usage, bad options, bad variant."""
    exe = str(BIN / "sweep-main")
    r = subprocess.run([exe, "--help"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "--graphs" in r.stdout
    assert subprocess.run([exe], capture_output=True, text=True, timeout=60).returncode == 2
    assert subprocess.run([exe, "--graphs", "x.el", "--bogus"], capture_output=True, text=True,
                          timeout=60).returncode == 2
    r = subprocess.run([exe, "--graphs", "x.el", "--variants", "sync-push-xx"], capture_output=True, text=True,
                       timeout=60)
    assert r.returncode == 2 and "unknown variant" in r.stderr
