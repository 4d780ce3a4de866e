"""Precision of the df32 element arithmetic the GPU kernels execute (CPU).

tests/df32_harness.cc compiles the same header code the kernels use
(lehrfempp_gb300/csrc/lfg_elem.h, lfg_df32.h) with g++ and compares element
matrices of random jittered triangles / quadrilaterals, O1-O3, three mesh
scales, with and without the mass term, against a long-double evaluation of
the reference's quadrature sum.  The parity bar is 1e-12 of max|A_K|; the
arithmetic must stay well inside it.
"""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("df32") / "df32_harness")
    src = os.path.join(ROOT, "tests", "df32_harness.cc")
    csrc = os.path.join(ROOT, "lehrfempp_gb300", "csrc")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", csrc, "-o", exe, src, os.path.join(csrc, "lfg_tables.cc")],
                   check=True)
    return exe


def test_df32_element_matrices_within_tolerance(harness):
    out = subprocess.run([harness, "2000"], check=True, capture_output=True, text=True).stdout
    rows = [ln.split() for ln in out.strip().splitlines()]
    assert len(rows) == 58
    assert all(float(r[-1]) >= 0.0 for r in rows), out  # every case ran (sum-factorised tables exist)
    worst = max(float(r[-1]) for r in rows)
    assert worst < 2e-13, out
