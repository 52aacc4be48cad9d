"""The Python binding's ctypes structures match include/nr.h: every field at the same offset
and every structure the same size, checked by a C program compiled from the header."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_ctypes_structures_match_the_header(tmp_path):
    import ctypes as C
    from relaibilitygpu_gb300 import engine as E
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    structs = {"nr_graph": E.NrGraph, "nr_options": E.NrOptions, "nr_result": E.NrResult}
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "nr.h"', 'int main(void) {']
    for cname, cls in structs.items():
        lines.append(f'    printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for f, _ in cls._fields_:
            lines.append(f'    printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ['    return 0;', '}']
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    r = subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for cname, cls in structs.items():
        assert got[(cname, "sizeof")] == C.sizeof(cls), cname
        for f, _ in cls._fields_:
            assert got[(cname, f)] == getattr(cls, f).offset, (cname, f)
