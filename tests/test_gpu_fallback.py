"""Cells outside the df32 range take the FP64 formulas inside the df32
kernels (GPU): tiny geometry (coordinate differences below 2^-40) and huge
coefficients.  Results must match the oracle like every other cell, and the
fallback counter must show that the FP64 route ran."""
import numpy as np
import pytest

from parity import O, L, W, Run, block_sizes, compare_triplets

pytestmark = pytest.mark.gpu


def _scaled_hybrid(n, scale, seed=5):
    xy, cells = W.hybrid_mesh(n, seed=seed)
    return {"kind": "factory", "xy": xy * scale, "cells": cells, "edges": None}


def _scaled_tptriag(n, scale):
    xy, cells, pe = O.factory_input("tptriag", n, n, 0.0, 0.0, scale, scale)
    return {"kind": "factory", "xy": xy, "cells": cells, "edges": pe}


def _fallbacks(ctx):
    return ctx.profile_read("fp64_fallback_cells")[1]


def _check(ctx, wl):
    before = _fallbacks(ctx)
    run = Run(ctx, wl)
    coo = run.gpu_matrix()
    t = coo.triplets()
    r, c, v = run.oracle_matrix().arrays()
    compare_triplets(t, r, c, v, block_sizes(run.cells(), run.ospace.n_tria, run.ospace.n_quad))
    return _fallbacks(ctx) - before


@pytest.mark.parametrize("degree", [1, 2, 3])
def test_tiny_hybrid_geometry_takes_fp64_route(ctx, degree):
    rng = np.random.default_rng(degree)
    mesh = _scaled_hybrid(6, 1e-13)
    ncell = len(mesh["cells"])
    wl = {"mesh": mesh, "degree": degree, "alpha": ("cell", np.exp(rng.standard_normal(ncell))),
          "gamma": ("const", 2.5), "qr_tria": 0, "qr_quad": 0}
    assert _check(ctx, wl) == ncell


def test_tiny_triangles_varying_alpha_take_fp64_route(ctx):
    mesh = _scaled_tptriag(5, 1e-13)
    wl = {"mesh": mesh, "degree": 3, "alpha": ("sincos", 1.0, 0.5, 4.0, 4.0), "gamma": ("const", 1.0),
          "qr_tria": 6, "qr_quad": 6}
    assert _check(ctx, wl) == len(mesh["cells"])


def test_huge_coefficient_takes_fp64_route(ctx):
    rng = np.random.default_rng(3)
    mesh = _scaled_hybrid(6, 1.0)
    ncell = len(mesh["cells"])
    alpha = np.exp(rng.standard_normal(ncell))
    alpha[::5] = 1e15  # beyond 2^40: these cells leave the df32 range
    wl = {"mesh": mesh, "degree": 2, "alpha": ("cell", alpha), "gamma": ("zero",), "qr_tria": 0, "qr_quad": 0}
    assert _check(ctx, wl) == len(alpha[::5])


def test_normal_cells_stay_on_df32(ctx):
    rng = np.random.default_rng(4)
    mesh = _scaled_hybrid(6, 1.0)
    wl = {"mesh": mesh, "degree": 2, "alpha": ("cell", np.exp(rng.standard_normal(len(mesh["cells"])))),
          "gamma": ("const", 1.0), "qr_tria": 0, "qr_quad": 0}
    assert _check(ctx, wl) == 0
