"""The ctypes structures of gdp.py have the layout of the C structures in
include/gdp_ext.h: a C program compiled against the header prints every
field's offset and every structure's size, and they must equal ctypes'."""
import ctypes as C
import shutil
import subprocess
from pathlib import Path

import pytest

import gdp

ROOT = Path(__file__).resolve().parents[1]
STRUCTS = {"gdp_options": gdp.Options, "gdp_stats": gdp.Stats, "gdp_tune_trial": gdp.TuneTrial,
           "gdp_mps_problem": gdp.MpsProblem}


def test_ctypes_structures_match_the_header(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "gdp_ext.h"', "int main(void) {"]
    for cname, py in STRUCTS.items():
        lines.append(f'    printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'    printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c99", f"-I{ROOT / 'include'}", str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    seen = 0
    for line in filter(None, out):
        cname, what, value = line.split()
        py = STRUCTS[cname]
        expect = C.sizeof(py) if what == "size" else getattr(py, what).offset
        assert int(value) == expect, (cname, what, int(value), expect)
        seen += 1
    assert seen == sum(len(py._fields_) + 1 for py in STRUCTS.values())
