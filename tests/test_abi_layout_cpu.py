"""The Python ctypes mirrors of the C-ABI structs have the layout the C
compiler gives the declarations in include/: a small C program built with
gcc prints sizeof and offsetof of every field, compared with ctypes."""
import ctypes as C
import os
import shutil
import subprocess

import pytest

from gpu_accelsearch_gb300 import compat as CP
from gpu_accelsearch_gb300 import native as N

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# (C type name, ctypes class); every field of the ctypes class is checked
STRUCTS = [("accel_config", N.Config), ("accel_harmonic", N.Harmonic),
           ("accel_candidate", N.Candidate), ("accel_stats", N.Stats),
           ("accel_tuning", N.Tuning), ("accel_optimized", N.Optimized),
           ("accel_server_config", N.ServerConfig), ("accel_server_stats", N.ServerStats),
           ("accel_filterbank_info", N.FilterbankInfo),
           ("SubharmonicInfo", CP.SubharmonicInfo), ("ffdotInfo", CP.FfdotInfo),
           ("Candidates", CP.Candidates)]


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    gcc = shutil.which("gcc") or shutil.which("cc")
    if gcc is None:
        pytest.skip("no C compiler")
    d = tmp_path_factory.mktemp("abi")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "bpd_compat.h"', 'int main(void) {']
    for cname, cls in STRUCTS:
        lines.append(f'printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for f in cls._fields_:
            lines.append(f'printf("{cname} {f[0]} %zu\\n", offsetof({cname}, {f[0]}));')
    lines.append("return 0; }")
    src = d / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = d / "layout"
    subprocess.run([gcc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    res = {}
    for line in out.splitlines():
        cname, field, v = line.split()
        res[(cname, field)] = int(v)
    return res


@pytest.mark.parametrize("cname,cls", STRUCTS, ids=[s[0] for s in STRUCTS])
def test_ctypes_mirror_matches_c(c_layout, cname, cls):
    assert C.sizeof(cls) == c_layout[(cname, "sizeof")], cname
    for f in cls._fields_:
        assert getattr(cls, f[0]).offset == c_layout[(cname, f[0])], (cname, f[0])
