"""The Python binding's ctypes mirrors of the C ABI's structs match include/eegraph_c.h field by field.

A small C program built with gcc against the header prints every field's offset and every struct's
size; each ctypes Structure in eegraph_gb300 must agree, or a field added on one side only would shift
the others silently (no GPU needed).
"""
import shutil
import subprocess
from pathlib import Path

import pytest

import eegraph_gb300 as E

ROOT = Path(__file__).resolve().parents[1]

# ctypes class -> C struct name
PAIRS = [(E.GraphView, "eeg_graph_view"), (E.VGraphInfo, "eeg_vgraph_info"), (E.Options, "eeg_options"),
         (E.Result, "eeg_result"), (E.Query, "eeg_query"), (E.Tuning, "eeg_tuning"),
         (E.StreamInfo, "eeg_stream_info")]


def _c_layout(tmp_path):
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "eegraph_c.h"', "int main(void) {"]
    for cls, cname in PAIRS:
        lines.append(f'    printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            lines.append(f'    printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True,
                   capture_output=True, text=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    layout = {}
    for line in out.splitlines():
        cname, field, val = line.split()
        layout[(cname, field)] = int(val)
    return layout


@pytest.mark.parametrize("cls,cname", PAIRS, ids=[c for _, c in PAIRS])
def test_ctypes_mirror_matches_header(tmp_path, cls, cname):
    layout = _c_layout(tmp_path)
    import ctypes

    assert ctypes.sizeof(cls) == layout[(cname, "sizeof")], cname
    for fname, _ in cls._fields_:
        assert getattr(cls, fname).offset == layout[(cname, fname)], (cname, fname)
