"""The C++ facade (include/lf_gb300.hpp) compiled into a driver program that
checks itself against the oracle library (tests/cpp/facade_test.cc)."""
import os
import subprocess

import pytest

from parity import L, O, ROOT

pytestmark = pytest.mark.gpu


def test_cpp_facade_driver(tmp_path):
    L.load()
    O.lib()
    lib_dir = os.path.dirname(L.LIB_PATH)
    orc_dir = os.path.dirname(O._LIB_PATH)
    exe = str(tmp_path / "facade_test")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "facade_test.cc"), "-L", lib_dir, "-llfg", "-L", orc_dir,
                    "-loracle", "-Wl,-rpath," + lib_dir + ":" + orc_dir, "-o", exe], check=True)
    p = subprocess.run([exe, os.path.join(ROOT, "tests", "golden", "msh")], capture_output=True, text=True,
                       timeout=600)
    print(p.stdout)
    assert p.returncode == 0, p.stdout + p.stderr
    assert "facade_test OK" in p.stdout
