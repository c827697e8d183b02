"""bench.py's JSON line, checked on CPU through the reference arm (`--impl reference` runs the
reference's CPU path on a bounded sample and needs no GPU): every key the contract names, with the
reference arm's own additions (`impl`, a `cpu_baseline` describing the run, an `e2e` that moves no
bytes)."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def _reference_line(*extra):
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "0",
                        "--cpu-threads", "2", *extra], capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    return json.loads(lines[0])


def test_reference_arm_line_has_the_contract_keys():
    d = _reference_line()
    for key, typ in [("metric", str), ("value", float), ("unit", str), ("n_gpus", int), ("steps", int),
                     ("warmup", int), ("ms_per_step", float), ("higher_is_better", bool), ("scaling", str),
                     ("dtype", str), ("data", str), ("config", dict), ("cpu_baseline", dict), ("e2e", dict)]:
        assert isinstance(d[key], typ), key
    assert d["impl"] == "reference"
    assert "vs_baseline" in d and d["vs_baseline"] is None  # no published number for this metric
    assert d["unit"] == "GTEPS" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["n_gpus"] == 1 and d["steps"] == 1 and d["warmup"] == 0
    assert d["scaling"] in ("weak", "strong")
    assert "workload" in d["config"]
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["unit"] == d["unit"] and cb["cores"] == 2
    assert cb["kind"] in ("reference", "port") and cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["unit"] == d["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0


def test_bench_help_names_every_workload():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--help"], capture_output=True, text=True,
                       timeout=120, cwd=ROOT)
    assert r.returncode == 0
    for w in ("rmat", "grid", "batch", "ppr"):
        assert w in r.stdout
    for flag in ("--gpus", "--steps", "--warmup", "--impl", "--workload", "--ppr-columns"):
        assert flag in r.stdout
