"""The ctypes mirrors of the C ABI's structs match include/pps.h byte for byte.

A C program compiled here against the header prints sizeof and the offset of every
field the Python binding declares; each must equal the ctypes layout, so a field
added to (or moved in) one side and not the other fails here instead of corrupting a
caller's stats or tuning at run time."""
import ctypes as C
import os
import shutil
import subprocess

import pytest

import parallelpoissonsolver_gb300 as pps

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PAIRS = [
    ("pps_grid", pps.PpsGrid),
    ("pps_config", pps.PpsConfig),
    ("pps_stats", pps.PpsStats),
    ("pps_tuning", pps.PpsTuning),
    ("pps_batch_stats", pps.PpsBatchStats),
]


def test_struct_layouts_match_the_header(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "pps.h"', "int main(void) {"]
    for cname, cls in PAIRS:
        lines.append(f'    printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for field, _ in cls._fields_:
            lines.append(f'    printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = str(tmp_path / "layout")
    r = subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), "-o", exe, str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr   # a field the binding names that the header lacks
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {}
    for line in out:
        if line:
            cname, what, value = line.split()
            got[(cname, what)] = int(value)
    for cname, cls in PAIRS:
        assert got[(cname, "sizeof")] == C.sizeof(cls), cname
        for field, _ in cls._fields_:
            assert got[(cname, field)] == getattr(cls, field).offset, (cname, field)


def test_tuning_from_dict_fills_the_optional_keys():
    t = pps.PpsTuning.from_dict({"cheb_ty": 8, "cheb_cx": 4, "cheb_waves": 4, "other_ty": 8, "other_waves": 2,
                                 "cheb_us": 1.0, "other_us": 2.0})
    assert t.cheb_fused == 0 and t.fcg_staged == 0
    d = t.as_dict()
    assert pps.PpsTuning.from_dict(d).as_dict() == d
