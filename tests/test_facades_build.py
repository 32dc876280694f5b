"""The C++ facades compile as their callers would use them (CPU, no device needed):
tests/facade/facade_check.cpp against include/ekgsim.hpp and include/ekgsim_amsdemo.hpp, linked
with the engine's library; and, when the reference sources are present, the same program with
AMS-DEMO's own GeneralOptimizationAlgorithm.h supplying VirtualOptimizationFunction (compiled with
the reference build's flags, oracle/build_ref.sh)."""
import os
import shutil
import subprocess

import pytest

from oracle.refpath import reference_dir

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "facade", "facade_check.cpp")
LIBDIR = os.path.join(ROOT, "ekgsim_gb300")


def test_facade_check_builds_and_links(tmp_path):
    if not os.path.exists(os.path.join(LIBDIR, "libekgsim_gb300.so")):
        pytest.skip("engine library not built")
    out = str(tmp_path / "facade_check")
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), SRC,
                        "-o", out, "-L", LIBDIR, "-lekgsim_gb300", f"-Wl,-rpath,{LIBDIR}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert os.path.exists(out)


@pytest.mark.skipif(reference_dir() is None, reason="the reference sources are not present")
def test_plugin_compiles_against_amsdemo_header():
    ref = reference_dir()
    r = subprocess.run(["g++", "-std=c++11", "-fsyntax-only", "-w", "-DNO_MPI", "-DEKGSIM_WITH_AMSDEMO",
                        "-include", "vector", "-include", "iostream", "-include",
                        os.path.join(ref, "AMS-DEMO", "VectorArithmetics.h"), "-I", os.path.join(ref, "AMS-DEMO"),
                        "-I", os.path.join(ref, "copyOfLibs"), "-I", ref, "-I", os.path.join(ROOT, "include"), SRC],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_headers_compile_as_c_and_cpp(tmp_path):
    """include/ekgsim.h is plain C; the C++ headers need nothing but the standard library."""
    c = tmp_path / "t.c"
    c.write_text('#include "ekgsim.h"\nint main(void) { return ekg_last_error() == 0; }\n')
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-fsyntax-only", "-I", os.path.join(ROOT, "include"),
                        str(c)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    if shutil.which("g++"):
        cc = tmp_path / "t.cpp"
        cc.write_text('#include "ekgsim_amsdemo.hpp"\nint main() { return 0; }\n')
        r = subprocess.run(["g++", "-std=c++11", "-Wall", "-Werror", "-fsyntax-only", "-I",
                            os.path.join(ROOT, "include"), str(cc)], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
