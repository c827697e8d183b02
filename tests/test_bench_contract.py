"""bench.py's JSON line, checked on CPU through the reference arm (`--impl reference` runs the
reference's CPU path and needs no GPU; here on R-MAT scale 16 to stay quick): every key the contract
names, with the reference arm's own additions (`impl`, a `cpu_baseline` describing the run, an `e2e`
that moves no bytes); the arm maps no product library."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


# runs bench.py's main in this interpreter, then reports whether the product library was mapped
_RUNNER = """
import runpy, sys
sys.argv = ["bench.py"] + sys.argv[1:]
runpy.run_path("bench.py", run_name="__main__")
maps = open("/proc/self/maps").read()
print("PRODUCT_MAPPED", "libeegraph" in maps or "eegraph_gb300" in sys.modules)
"""


def _reference_line(*extra, product_mapped=False):
    r = subprocess.run([sys.executable, "-c", _RUNNER, "--impl", "reference", "--steps", "1", "--warmup", "0",
                        "--cpu-threads", "2", "--scale", "16", *extra], capture_output=True, text=True, timeout=300,
                       cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    assert f"PRODUCT_MAPPED {product_mapped}" in r.stdout, r.stdout[-500:]
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
    sys.path.insert(0, str(ROOT))
    import bench

    c = d["config"]  # the GPU arm's config object for the same workload
    assert c == bench.headline_config(16, 8, 16, 1 << 16, 16 << 16, 32 << 16, c["source"], 1)
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


def test_clock_sampler_keeps_the_timed_window():
    """ClockSampler.summary(): samples stamped inside the start()/stop() window only; every sample when no
    window was marked or a stamp cannot be read; throttle reasons reported by name."""
    import datetime
    import time

    sys.path.insert(0, str(ROOT))
    import bench

    def line(t, sm, reasons=("Not Active",) * 4):
        stamp = datetime.datetime.fromtimestamp(t).strftime("%Y/%m/%d %H:%M:%S.%f")[:-3]
        return ", ".join([stamp, str(sm), "2070", "0x0", *reasons])

    now = time.time()
    c = bench.ClockSampler(0)
    c.lines = [line(now - 5, 1000), line(now + 0.1, 2070), line(now + 0.2, 2070),
               line(now + 0.3, 2070, ("Not Active", "Not Active", "Not Active", "Active")), line(now + 9, 500)]
    whole = c.summary()
    assert whole["samples"] == 5 and whole["window"] == "whole run"
    c.t0, c.t1 = now, now + 0.35
    timed = c.summary()
    assert timed["samples"] == 3 and timed["window"] == "timed region"
    assert timed["sm_mhz"] == 2070 and timed["sm_max_mhz"] == 2070 and timed["reasons"] == ["sw_power_cap"]
    c.lines = ["garbled, 2070, 2070, 0x0, Not Active, Not Active, Not Active, Not Active"]
    assert c.summary()["samples"] == 1 and c.summary()["window"] == "whole run"
    c.lines = []
    assert c.summary()["reasons"] == ["unavailable"]


def test_traffic_figures_follow_the_kernel_code_not_its_comments(tmp_path, monkeypatch):
    """A measured DRAM figure (profiles/traffic.json) stays in use across a comment edit of the kernel's
    sources and is retired by any code change; every committed figure matches the sources here."""
    sys.path.insert(0, str(ROOT))
    import bench

    t = json.loads((ROOT / "profiles" / "traffic.json").read_text())
    for wl, d in t.items():
        if isinstance(d, dict):
            for k, e in d.items():
                if isinstance(e, dict):
                    assert bench.load_traffic(k, wl) == float(e["dram_bytes_per_launch"]), (wl, k)
    csrc = tmp_path / "eegraph_gb300" / "csrc"
    csrc.mkdir(parents=True)
    for f in bench.KERNEL_SOURCES["k_traverse"]:
        (csrc / f).write_text((ROOT / "eegraph_gb300" / "csrc" / f).read_text())
    monkeypatch.setattr(bench, "ROOT", tmp_path)
    base = bench.kernel_source_sha("k_traverse<OP_BFS>")
    assert base == t["s22_k8"]["k_traverse<OP_BFS>"]["source_sha"]
    p = csrc / "traverse.cuh"
    p.write_text(p.read_text() + "\n// a note\n/* another\n   note */\n\n")
    assert bench.kernel_source_sha("k_traverse<OP_BFS>") == base
    p.write_text(p.read_text().replace("constexpr int WCAP = 256;", "constexpr int WCAP = 128;"))
    assert bench.kernel_source_sha("k_traverse<OP_BFS>") != base
