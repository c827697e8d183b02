"""Build recipe for the in-tree native library and executables (no cmake).

Compiles every CUDA translation unit for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a -lineinfo``), the host C++ units with g++, links
``eegraph_gb300/_lib/libeegraph.so`` (static cudart, so the only runtime dependency is the driver)
and the executables in ``eegraph_gb300/_bin/``: the per-algorithm programs ``{bfs,sssp,sswp,cc,pr}-main``,
``sweep-main``, ``graph-info-main`` and ``converter``.
Objects are rebuilt only when a source or header is newer. Sources compile in parallel.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OBJ = PKG / "_obj"
LIB = PKG / "_lib"
BIN = PKG / "_bin"
INCLUDE = ROOT / "include"

CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc")
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["builder.cu", "traverse_bfs.cu", "traverse_sssp.cu", "traverse_sswp.cu", "traverse_cc.cu",
              "traverse_host.cu", "pagerank.cu", "pagerank_dd.cu", "capi.cu", "noalloc.cu", "batch.cu", "ppr.cu",
              "stream.cu"]
CPP_SOURCES = ["host_graph.cpp", "energy.cpp"]
FACADE_SOURCES = ["facade/graph.cpp", "facade/virtual_graph.cpp", "facade/argument_parsing.cpp",
                  "facade/utilities.cpp", "facade/eegraph.cpp"]
CLI = {"bfs-main": "bfs", "sssp-main": "sssp", "sswp-main": "sswp", "cc-main": "cc", "pr-main": "pr"}

LIBNAME = "libeegraph.so"


def _headers() -> list[Path]:
    hs = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.hpp")) + list(INCLUDE.glob("*.h")) + list(INCLUDE.glob("*.hpp"))
    return hs


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.exists() and d.stat().st_mtime > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _compile(src: Path, obj: Path, hdrs: list[Path], verbose_ptxas: bool) -> str:
    if not _stale(obj, [src] + hdrs):
        return f"up-to-date {obj.name}"
    obj.parent.mkdir(parents=True, exist_ok=True)
    if src.suffix == ".cu":
        cmd = [NVCC, "-c", str(src), "-o", str(obj), "-O3", "-std=c++17", "-lineinfo", *GENCODE,
               "-Xcompiler", "-fPIC,-O3,-fvisibility=hidden", "-I", str(INCLUDE), "-I", str(CSRC)]
        if verbose_ptxas:
            cmd += ["-Xptxas", "-v"]
    else:
        # the facade's C++ classes are its public API; the core library exports only the C ABI
        vis = [] if src.parent.name in ("facade", "cli") else ["-fvisibility=hidden"]
        cmd = ["g++", "-c", str(src), "-o", str(obj), "-O3", "-std=c++17", "-fPIC", "-pthread", *vis,
               "-I", str(INCLUDE), "-I", str(CSRC), "-I", str(CUDA_HOME / "include")]
    _run(cmd)
    return f"compiled {src.name}"


def build(verbose: bool = False, jobs: int | None = None, verbose_ptxas: bool = False) -> Path:
    """Compile and link; returns the path of the shared library."""
    if not Path(NVCC).exists() and shutil.which("nvcc") is None:
        raise RuntimeError("nvcc not found (set CUDA_HOME)")
    hdrs = _headers()
    units = [(CSRC / s, OBJ / (Path(s).stem + ".o")) for s in CU_SOURCES + CPP_SOURCES]
    fac = [(CSRC / s, OBJ / ("facade_" + Path(s).stem + ".o")) for s in FACADE_SOURCES]
    cli = [(CSRC / "cli" / "main.cpp", OBJ / "cli_main.o"), (CSRC / "cli" / "sweep.cpp", OBJ / "cli_sweep.o"),
           (CSRC / "cli" / "graph_info.cpp", OBJ / "cli_graph_info.o"),
           (CSRC / "cli" / "converter.cpp", OBJ / "cli_converter.o")]
    jobs = jobs or max(2, min(16, os.cpu_count() or 2))
    with cf.ThreadPoolExecutor(jobs) as ex:
        futs = [ex.submit(_compile, s, o, hdrs, verbose_ptxas) for s, o in units + fac + cli]
        for f in futs:
            msg = f.result()
            if verbose:
                print(msg)
    LIB.mkdir(parents=True, exist_ok=True)
    lib = LIB / LIBNAME
    objs = [o for _, o in units]
    if _stale(lib, objs):
        _run([NVCC, "-shared", "-o", str(lib), *[str(o) for o in objs], *GENCODE, "-cudart", "static",
              "-Xlinker", "-rpath,$ORIGIN", "-ldl", "-lpthread", "-lrt"])
    # C++ facade: a second shared library on top of the C ABI (reference class names and entry points)
    fac_lib = LIB / "libeegraph_facade.so"
    fac_objs = [o for _, o in fac]
    if _stale(fac_lib, fac_objs + [lib]):
        _run(["g++", "-shared", "-o", str(fac_lib), *[str(o) for o in fac_objs], "-L", str(LIB), "-leegraph",
              "-Wl,-rpath,$ORIGIN", "-pthread"])
    BIN.mkdir(parents=True, exist_ok=True)
    # the per-algorithm programs (one program; it picks the algorithm from the name it is started
    # under) and the measurement sweep
    for exe, obj in [(e, cli[0][1]) for e in CLI] + [("sweep-main", cli[1][1]), ("graph-info-main", cli[2][1])]:
        target = BIN / exe
        if _stale(target, [obj, fac_lib, lib]):
            _run(["g++", "-o", str(target), str(obj), "-L", str(LIB),
                  "-leegraph_facade", "-leegraph", "-Wl,-rpath,$ORIGIN/../_lib", "-pthread"])
    # Subway's text-to-binary CSR converter (C ABI only)
    target = BIN / "converter"
    if _stale(target, [cli[3][1], lib]):
        _run(["g++", "-o", str(target), str(cli[3][1]), "-L", str(LIB), "-leegraph", "-Wl,-rpath,$ORIGIN/../_lib",
              "-pthread"])
    return lib


if __name__ == "__main__":
    build(verbose=True, verbose_ptxas="-v" in sys.argv)
    print(LIB / LIBNAME)
