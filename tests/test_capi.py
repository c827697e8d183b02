"""C ABI surface and host logic (CPU only: no compute call needs a GPU here)."""
import ctypes
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def _declared(header: Path) -> list[str]:
    text = header.read_text()
    return sorted(set(re.findall(r"EEG_API\s+[\w\s\*]+?\b(eeg_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol(E):
    declared = _declared(ROOT / "include" / "eegraph_c.h")
    assert len(declared) >= 25
    lib = ctypes.CDLL(str(E.LIB_PATH))
    missing = [s for s in declared if not hasattr(lib, s)]
    assert not missing, missing
    assert sorted(E.EXPORTED) == declared


def test_library_exports_only_the_c_abi(E):
    out = subprocess.run(["nm", "-D", "--defined-only", str(E.LIB_PATH)], capture_output=True, text=True).stdout
    text_syms = [l.split()[-1] for l in out.splitlines() if " T " in l]
    assert text_syms and all(s.startswith("eeg_") for s in text_syms), [s for s in text_syms if not s.startswith("eeg_")][:5]


def test_status_strings(E):
    for code in range(10):
        assert E.lib().eeg_status_string(code)
    assert E.version().startswith("eegraph-gb300")


def test_rmat_is_deterministic_and_in_range(E):
    a = E.gen_rmat(12, 16, seed=1)
    b = E.gen_rmat(12, 16, seed=1)
    c = E.gen_rmat(12, 16, seed=2)
    assert all(np.array_equal(x, y) for x, y in zip(a, b))
    assert not np.array_equal(a[0], c[0])
    s, d, w = a
    assert s.max() < 4096 and d.max() < 4096 and w.min() >= 1 and w.max() <= 63
    # skew: quadrant a=0.57 -> vertex 0 is the largest hub
    deg = np.bincount(s, minlength=4096)
    assert deg.argmax() == 0 and deg[0] > 20 * deg.mean()


def test_grid_generator(E):
    s, d, w = E.gen_grid(32, p_delete=0.1, shortcut_frac=0.01, seed=7)
    E_grid = 2 * 32 * 31
    assert s.size % 2 == 0
    und = s.size // 2
    assert 0.85 * E_grid < und < E_grid + 0.02 * E_grid
    # arcs come in reversed pairs with equal weights
    assert np.array_equal(s[0::2], d[1::2]) and np.array_equal(w[0::2], w[1::2])
    assert w.min() >= 1 and w.max() <= 1000
    s2, d2, w2 = E.gen_grid(32, p_delete=0.1, shortcut_frac=0.01, seed=7)
    assert np.array_equal(s, s2) and np.array_equal(w, w2)


def test_symmetrize(E):
    s, d, w = E.gen_rmat(8, 4, seed=3)
    so, do, wo = E.symmetrize(s, d, w)
    m = s.size
    assert np.array_equal(so[:m], s) and np.array_equal(so[m:], d) and np.array_equal(do[m:], s)
    assert np.array_equal(wo[:m], wo[m:])


def test_build_without_device_reports_no_device(E):
    if E.device_count() > 0:
        pytest.skip("a GPU is present")
    s, d, w = E.gen_rmat(6, 4)
    with pytest.raises(E.EEGError) as ei:
        E.VirtualGraph.build(64, s, d, w)
    assert ei.value.status == E.ERR_NO_DEVICE


def test_invalid_K_rejected(E):
    s, d, w = E.gen_rmat(6, 4)
    with pytest.raises(E.EEGError) as ei:
        E.VirtualGraph.build(64, s, d, w, K=5)
    assert ei.value.status == E.ERR_UNSUPPORTED


def test_graph_from_arrays_view(E):
    g = E.Graph.from_arrays(5, [0, 1, 2], [1, 2, 4], [3, 4, 5])
    v = g.view()
    assert v["num_nodes"] == 5 and v["num_edges"] == 3 and v["has_zero_id"]
    assert v["weight"].tolist() == [3, 4, 5]


def test_energy_without_nvml_is_reported_not_fatal(E, monkeypatch, tmp_path):
    # no libnvidia-ml on this machine (or a fake path): the session reports "unavailable"
    monkeypatch.setenv("EEG_NVML_LIBRARY", str(tmp_path / "libnvidia-ml-missing.so"))
    s = E.EnergySession(0)
    if s.available:  # a real NVML on a GPU machine already loaded by an earlier test
        s.end()
        pytest.skip("NVML already initialised in this process")
    assert "unavailable" in s.reason
    assert s.end() is None
