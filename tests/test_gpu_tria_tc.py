"""O3 triangles with point-varying alpha on the tcgen05 tensor cores
(RDTriaTcKernel: the 12-point degree-6 rule, exact digit splitting of the
FP64 contraction) against the oracle and against the df32 kernel it replaces:
analytic (sin/cos, polynomial) and O1-nodal alpha, gamma zero / constant /
per cell, jittered meshes, cells on the FP64 route, several tiles per CTA."""
import numpy as np
import pytest

from parity import L, W, Run, block_sizes, compare_triplets

pytestmark = pytest.mark.gpu


def _tria_mesh(n, jitter, seed):
    xs = np.linspace(0.0, 1.0, n + 1)
    X, Y = np.meshgrid(xs, xs, indexing="xy")
    xy = np.stack([X.ravel(), Y.ravel()], 1)
    rng = np.random.default_rng(seed)
    inner = (xy[:, 0] > 0) & (xy[:, 0] < 1) & (xy[:, 1] > 0) & (xy[:, 1] < 1)
    xy[inner] += rng.uniform(-jitter, jitter, (inner.sum(), 2)) / n
    cells = []
    for j in range(n):
        for i in range(n):
            v0 = j * (n + 1) + i
            cells.append([v0, v0 + 1, v0 + n + 2, -1])
            cells.append([v0, v0 + n + 2, v0 + n + 1, -1])
    return {"kind": "factory", "xy": xy, "cells": np.array(cells, np.int32), "edges": None}


def _run(ctx, wl, tc):
    ctx.set_tensor_cores(tc)
    try:
        ctx.profile(True)
        ctx.profile_reset()
        run = Run(ctx, wl)
        t = run.gpu_matrix().triplets()
        n_tc = ctx.profile_read("rd_tria_vary_tc")[1]
        ctx.profile(False)
    finally:
        ctx.set_tensor_cores(True)
    r, c, v = run.oracle_matrix().arrays()
    err = compare_triplets(t, r, c, v, block_sizes(run.cells(), run.ospace.n_tria, run.ospace.n_quad))
    return t, n_tc, err


def _alpha(kind, nv, rng):
    if kind == "sincos":
        return ("sincos", 1.0, 0.5, 4.0, 4.0)
    if kind == "poly":
        return ("poly", [1.0, 0.3, 0.0, 0.0, 0.2, 0.1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0])
    return ("nodal", 1.0 + rng.random(nv))


@pytest.mark.parametrize("alpha", ["sincos", "poly", "nodal"])
@pytest.mark.parametrize("gamma", ["zero", "const"])
def test_tria_tc_matches_oracle(ctx, alpha, gamma):
    m = _tria_mesh(10, 0.3, 1)
    rng = np.random.default_rng(7)
    wl = {"mesh": m, "degree": 3, "alpha": _alpha(alpha, len(m["xy"]), rng),
          "gamma": ("zero",) if gamma == "zero" else ("const", 2.5), "qr_tria": 6, "qr_quad": 6}
    t_tc, n_tc, err_tc = _run(ctx, wl, True)
    t_df, n_df, _ = _run(ctx, wl, False)
    assert n_tc == 1 and n_df == 0
    assert np.array_equal(t_tc["row"], t_df["row"]) and np.array_equal(t_tc["col"], t_df["col"])
    assert err_tc < 1e-13, err_tc
    assert ctx.profile_read("tc_timeouts")[1] == 0


def test_tria_tc_per_cell_gamma_and_fp64_cells(ctx):
    """Per-cell gamma over eight decades; every 9th cell has gamma = 1e15 and
    takes the FP64 formula in the epilogue.  Rows dominated by the mass term
    share their scale with the (much larger) gradient-table columns, which
    costs a few bits: about 2.5e-13 of the block maximum, inside the 1e-12 bar."""
    m = _tria_mesh(12, 0.25, 2)
    nc = len(m["cells"])
    rng = np.random.default_rng(3)
    gam = np.exp(rng.uniform(-9, 9, nc))
    gam[::9] = 1e15
    wl = {"mesh": m, "degree": 3, "alpha": ("sincos", 1.0, 0.5, 4.0, 4.0), "gamma": ("cell", gam),
          "qr_tria": 6, "qr_quad": 6}
    before = ctx.profile_read("fp64_fallback_cells")[1]
    _, n_tc, err = _run(ctx, wl, True)
    assert n_tc == 1 and err < 5e-13
    assert ctx.profile_read("fp64_fallback_cells")[1] - before == len(gam[::9])


def test_tria_tc_many_tiles(ctx):
    """2 x 200 x 200 = 80,000 triangles: 625 tiles, several per CTA, the last partial."""
    m = _tria_mesh(200, 0.3, 4)
    wl = {"mesh": m, "degree": 3, "alpha": ("sincos", 1.0, 0.5, 4.0, 4.0), "gamma": ("const", 1.0),
          "qr_tria": 6, "qr_quad": 6}
    _, n_tc, err = _run(ctx, wl, True)
    assert n_tc == 1 and err < 1e-13
    ctx.synchronize()
