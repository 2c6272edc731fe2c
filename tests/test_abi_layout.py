"""The ctypes mirrors in turner_gb300 have the C header's struct layouts:
a C program built against include/turner_gpu.h prints sizeof and offsetof
of every field the mirrors declare (gcc, no GPU)."""
import ctypes as C
import shutil
import subprocess

import pytest

import turner_gb300 as tg
from turner_gb300.build import ROOT

MIRRORS = {"turner_camera": tg.Camera, "turner_light": tg.Light, "turner_job": tg.Job,
           "turner_tuning": tg.Tuning, "turner_stats": tg.Stats}


def _c_layout(tmp_path) -> dict:
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "turner_gpu.h"', "int main(void) {"]
    for cname, mirror in MIRRORS.items():
        lines.append(f'    printf("{cname} size %zu\\n", sizeof({cname}));')
        for field, _ in mirror._fields_:
            lines.append(f'    printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    layout = {}
    for line in out.splitlines():
        cname, key, value = line.split()
        layout[(cname, key)] = int(value)
    return layout


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_ctypes_mirrors_match_the_header(tmp_path):
    layout = _c_layout(tmp_path)
    for cname, mirror in MIRRORS.items():
        assert C.sizeof(mirror) == layout[(cname, "size")], cname
        for field, _ in mirror._fields_:
            assert getattr(mirror, field).offset == layout[(cname, field)], (cname, field)
