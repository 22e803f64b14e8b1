"""Link-level drop-in under the reference's C++ linkage (no GPU needed).

The reference compiles its pipeline as CUDA C++ and its driver includes the
pipeline headers outside extern "C", so an object built against those
headers refers to C++-mangled names.  Checked here:
  * tests/c/cxx_caller.cpp, compiled against include/bpd_compat_cxx.h, takes
    the address of every function the reference's headers declare, links
    libaccelsearch.so, and its host-only answers equal the C ABI's;
  * with the reference checkout present: the same caller compiled against
    the reference's own headers links and answers the same, and the
    reference's own driver (AccelSearch.cu, unmodified) compiles against its
    headers and links against libaccelsearch.so with no other object.
"""
import os
import shutil
import subprocess

import pytest

import __graft_entry__
from gpu_accelsearch_gb300 import build as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = __graft_entry__.REFERENCE


def nvcc():
    try:
        return B.nvcc()
    except RuntimeError:
        pytest.skip("nvcc not found")


def compile_run(tmp_path, name, includes, defines=()):
    lib = __graft_entry__.build_library()
    libdir = os.path.dirname(lib)
    exe = str(tmp_path / name)
    cmd = [nvcc(), "-std=c++17", "-x", "cu", os.path.join(ROOT, "tests", "c", "cxx_caller.cpp"),
           "-o", exe, "-L", libdir, "-laccelsearch", "-Xlinker", "-rpath=" + libdir]
    for inc in includes:
        cmd += ["-I", inc]
    cmd += ["-D" + d for d in defines]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    r = subprocess.run([exe], check=True, capture_output=True, text=True)
    return {line.split()[0]: line.split()[1:] for line in r.stdout.splitlines()}


def check_answers(out):
    assert out["functions"] == ["36"]
    assert out["required_z"] == ["150", "-26", "112"]
    assert out["required_r"] == ["463.000", "87499.500"]
    assert out["index"] == ["21", "95"]
    assert out["total_harmonics"] == ["8", "16"]
    assert out["log2"] == ["3", "9"]
    assert out["median"] == ["4.0"]
    assert abs(float(out["rsqrt"][0]) - 2 ** -0.5) < 2e-3
    assert out["amps"] == ["0", "0", "1", "2", "3", "4", "5", "6", "0", "0"]
    assert out["spread"] == ["-1", "1", "0", "2", "0", "3", "0", "4", "0", "5", "0", "-1"]


def test_cxx_caller_against_own_header(tmp_path):
    check_answers(compile_run(tmp_path, "cxx_own", [os.path.join(ROOT, "include")]))


def test_symbols_mangled_as_the_reference_headers_declare():
    lib = __graft_entry__.build_library()
    nm = shutil.which("nm")
    if nm is None:
        pytest.skip("no nm")
    syms = set(subprocess.run([nm, "-D", "--defined-only", lib], check=True, capture_output=True,
                              text=True).stdout.split())
    for s in ("_Z21createSubharmonicInfoii", "_Z16realToComplexFFTPflPP6float2i", "_Z8dereddenP6float2j",
              "_Z10spreadDataP6float2iijS0_", "_Z21initialize_cuda_planstP15SubharmonicInfo",
              "_Z19search_ffdot_powersP9ffdotInfoifxP10Candidates", "_Z17__checkCudaErrorsPKcS0_i",
              "deredden", "createSubharmonicInfo", "logMessage", "fast_log2", "readData"):
        assert s in syms, s


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "headers")), reason="reference checkout absent")
def test_cxx_caller_against_reference_headers(tmp_path):
    check_answers(compile_run(tmp_path, "cxx_ref", [os.path.join(REF, "headers")],
                              defines=["WITH_REFERENCE_HEADERS"]))


@pytest.mark.skipif(not os.path.isfile(os.path.join(REF, "AccelSearch.cu")), reason="reference checkout absent")
def test_reference_driver_links_against_the_library(tmp_path):
    # the reference's own main(), compiled unmodified against its own
    # headers, resolves every pipeline call in libaccelsearch.so
    lib = __graft_entry__.build_library()
    libdir = os.path.dirname(lib)
    obj = str(tmp_path / "AccelSearch.o")
    exe = str(tmp_path / "accelsearch_ref_driver")
    subprocess.run([nvcc(), "-c", "-w", "-O2", *B.ARCH, "-I", os.path.join(REF, "headers"),
                    os.path.join(REF, "AccelSearch.cu"), "-o", obj], check=True, capture_output=True, text=True)
    r = subprocess.run([nvcc(), *B.ARCH, obj, "-o", exe, "-L", libdir, "-laccelsearch",
                        "-Xlinker", "-rpath=" + libdir, "-Xlinker", "--no-undefined"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert os.path.isfile(exe)
