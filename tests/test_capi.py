"""The C-ABI library: builds, loads and exports every declared symbol (CPU only)."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return set(re.findall(r"\b(lfg_[a-z0-9_]+)\s*\(", text))


def test_library_exports_every_declared_symbol():
    import lehrfempp_gb300 as L
    L.load()
    out = subprocess.run(["nm", "-D", "--defined-only", L.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (lfg_[a-z0-9_]+)", out))
    declared = _declared("lfg.h")
    assert declared, "no declarations found"
    missing = declared - exported
    assert not missing, missing


def test_python_binding_covers_the_header():
    from lehrfempp_gb300 import _capi
    assert _declared("lfg.h") == set(_capi.SIGNATURES)


def test_no_cpu_fallback():
    """Without a GPU the library refuses to create a context instead of computing on the CPU."""
    import lehrfempp_gb300 as L
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is visible")
    except ImportError:
        pass
    with pytest.raises(L.LfgError) as e:
        L.Context(0)
    assert e.value.code == L.CUDA_ERROR


def test_workload_generators():
    from lehrfempp_gb300 import workloads as W
    import numpy as np
    xy, cells = W.hybrid_mesh(32, seed=2)
    nq = int((cells[:, 3] >= 0).sum())
    assert len(cells) == nq + 2 * (32 * 32 - nq)
    # interior jitter only; boundary nodes stay on the unit square
    assert xy.min() == 0.0 and xy.max() == 1.0
    wl = W.config2(32)
    assert len(wl["alpha"][1]) == len(wl["mesh"]["cells"])
    ns, degs = W.batch_sizes()
    assert ns.min() >= 24 and ns.max() <= 320 and set(degs) == {1, 2}


def test_cpp_facade_compiles_and_links(tmp_path):
    """The C++ facade header compiles as C++17 and its driver links against
    liblfg.so and the oracle library (no GPU call is made)."""
    from parity import L, O
    L.load()
    O.lib()
    lib_dir, orc_dir = os.path.dirname(L.LIB_PATH), os.path.dirname(O._LIB_PATH)
    exe = str(tmp_path / "facade_test")
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "facade_test.cc"), "-L", lib_dir, "-llfg", "-L", orc_dir,
                    "-loracle", "-Wl,-rpath," + lib_dir + ":" + orc_dir, "-o", exe], check=True)
    assert os.path.exists(exe)
