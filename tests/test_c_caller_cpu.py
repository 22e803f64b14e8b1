"""The C ABI from C: tests/c/abi_from_c.c includes include/accelsearch.h
and include/bpd_compat.h, is compiled as C11 by gcc, links
libaccelsearch.so and calls host-only entry points (no GPU needed); its
answers are checked against the Python binding and the oracle."""
import os
import shutil
import subprocess

import pytest

import __graft_entry__
from gpu_accelsearch_gb300 import native as N
from gpu_accelsearch_gb300.dedisperse import dm_delays
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def out(tmp_path_factory):
    gcc = shutil.which("gcc") or shutil.which("cc")
    if gcc is None:
        pytest.skip("no C compiler")
    lib = __graft_entry__.build_library()
    d = tmp_path_factory.mktemp("c")
    exe = str(d / "abi_from_c")
    libdir = os.path.dirname(lib)
    subprocess.run([gcc, "-std=c11", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "c", "abi_from_c.c"), "-o", exe, "-L", libdir,
                    "-laccelsearch", "-Wl,-rpath," + libdir], check=True)
    r = subprocess.run([exe], check=True, capture_output=True, text=True)
    return {line.split()[0]: line.split()[1:] for line in r.stdout.splitlines()}


def test_c_caller(out):
    L = N.lib()
    assert out["version"][0] == "gpu_accelsearch_gb300"
    assert out["config"] == ["200", "8", "8192", "6", "200"]
    assert int(out["first_bin"][0]) == 268
    cut = L.accel_power_cut(6.0, 8, 1.0)
    assert abs(float(out["power_cut"][0]) - cut) < 1e-5
    assert abs(float(out["sigma"][0]) - 6.0) < 1e-4
    assert int(out["required_z"][0]) == 150  # 3/4 harmonic of zmax 200 (bank geometry)
    assert int(out["total_harmonics"][0]) == 8
    assert out["step_harmonic"][0] == "0"
    dl, mx = dm_delays(4, 1500.0, -75.0, 64e-6, [0.0, 100.0])
    want = O.dm_delays(4, 1500.0, -75.0, 64e-6, [0.0, 100.0])
    assert out["delays"][0] == "0"
    assert [int(v) for v in out["delays"][1:5]] == [int(v) for v in want[1]] == [int(v) for v in dl[1]]
    assert int(out["delays"][5]) == mx
    assert out["create_bad"][:2] == ["-1", "null"]
