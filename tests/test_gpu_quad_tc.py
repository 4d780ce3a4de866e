"""Q2 quadrilaterals on the tcgen05 tensor cores (RDQuadTcKernel: exact
integer-digit splitting of the FP64 contraction) against the oracle, next to
the df32 CUDA-core kernel it replaces: jittered and strongly distorted
bilinear quads, 3x3 and 2x2 Gauss rules, per-cell alpha over twelve decades,
tiles with cells on the FP64 route, and more tiles than resident CTAs."""
import numpy as np
import pytest

from parity import O, L, W, Run, block_sizes, compare_triplets

pytestmark = pytest.mark.gpu


def _quads(n, jitter, seed, stretch=1.0):
    """n x n quadrilaterals on [0, stretch] x [0, 1], interior nodes jittered."""
    xs = np.linspace(0.0, 1.0, n + 1)
    X, Y = np.meshgrid(xs, xs, indexing="xy")
    xy = np.stack([X.ravel(), Y.ravel()], 1)
    rng = np.random.default_rng(seed)
    inner = (xy[:, 0] > 0) & (xy[:, 0] < 1) & (xy[:, 1] > 0) & (xy[:, 1] < 1)
    xy[inner] += rng.uniform(-jitter, jitter, (inner.sum(), 2)) / n
    xy[:, 0] *= stretch
    cells = []
    for j in range(n):
        for i in range(n):
            v0 = j * (n + 1) + i
            cells.append([v0, v0 + 1, v0 + n + 2, v0 + n + 1])
    return {"kind": "factory", "xy": xy, "cells": np.array(cells, np.int32), "edges": None}


def _hybrid(n, seed):
    xy, cells = W.hybrid_mesh(n, seed=seed)
    return {"kind": "factory", "xy": xy, "cells": cells, "edges": None}


def _run(ctx, wl, tc):
    ctx.set_tensor_cores(tc)
    try:
        ctx.profile(True)
        ctx.profile_reset()
        run = Run(ctx, wl)
        t = run.gpu_matrix().triplets()
        n_tc = ctx.profile_read("rd_quad_tc")[1]
        ctx.profile(False)
    finally:
        ctx.set_tensor_cores(True)
    r, c, v = run.oracle_matrix().arrays()
    err = compare_triplets(t, r, c, v, block_sizes(run.cells(), run.ospace.n_tria, run.ospace.n_quad))
    return t, n_tc, err


CASES = [
    ("jittered", lambda: _quads(12, 0.3, 1), 0),
    ("distorted", lambda: _quads(9, 0.35, 2), 0),
    ("stretched", lambda: _quads(8, 0.3, 3, stretch=300.0), 0),
    ("hybrid", lambda: _hybrid(10, 4), 0),
    ("rule2x2", lambda: _quads(10, 0.3, 5), 3),
]


@pytest.mark.parametrize("mode", [1, 2, 3], ids=["specialised", "two_cta", "producer_writes"])
@pytest.mark.parametrize("name,mesh,qr", CASES, ids=[c[0] for c in CASES])
def test_tensor_core_quads_match_oracle(ctx, name, mesh, qr, mode):
    m = mesh()
    ncell = len(m["cells"])
    rng = np.random.default_rng(len(name))
    alpha = np.exp(rng.uniform(-14, 14, ncell))  # twelve decades inside the df32 range
    wl = {"mesh": m, "degree": 2, "alpha": ("cell", alpha), "gamma": ("zero",), "qr_tria": 0, "qr_quad": qr}
    t_tc, n_tc, err_tc = _run(ctx, wl, mode)
    t_df, n_df, err_df = _run(ctx, wl, False)
    assert n_tc == 1 and n_df == 0  # the tensor-core kernel ran (once), and only when enabled
    assert np.array_equal(t_tc["row"], t_df["row"]) and np.array_equal(t_tc["col"], t_df["col"])
    assert err_tc < 1e-13, err_tc
    assert ctx.profile_read("tc_timeouts")[1] == 0


def test_tensor_core_mode_checked(ctx):
    for bad in (-1, 4):
        with pytest.raises(L.LfgError) as e:
            ctx.set_tensor_cores(bad)
        assert e.value.code == L.INVALID_ARG


@pytest.mark.parametrize("mode", [1, 2, 3], ids=["specialised", "two_cta", "producer_writes"])
def test_tensor_core_constant_alpha_and_fp64_cells(ctx, mode):
    """Constant alpha, and one tile mixing df32-range cells with cells whose
    alpha (1e15) sends them to the FP64 formula in the epilogue."""
    m = _quads(16, 0.25, 7)
    ncell = len(m["cells"])
    wl = {"mesh": m, "degree": 2, "alpha": ("const", 2.75), "gamma": ("zero",), "qr_tria": 0, "qr_quad": 0}
    _run(ctx, wl, mode)
    alpha = np.ones(ncell)
    alpha[::7] = 1e15
    before = ctx.profile_read("fp64_fallback_cells")[1]
    wl["alpha"] = ("cell", alpha)
    _run(ctx, wl, mode)
    assert ctx.profile_read("fp64_fallback_cells")[1] - before == len(alpha[::7])


@pytest.mark.parametrize("mode", [1, 2, 3], ids=["specialised", "two_cta", "producer_writes"])
def test_tensor_core_many_tiles(ctx, mode):
    """90,000 quadrilaterals: 704 tiles of 128 cells, several per CTA of the
    persistent grid (both producer groups and buffers cycle), the last one
    partial."""
    m = _quads(300, 0.3, 8)
    rng = np.random.default_rng(9)
    wl = {"mesh": m, "degree": 2, "alpha": ("cell", np.exp(rng.standard_normal(len(m["cells"])))),
          "gamma": ("zero",), "qr_tria": 0, "qr_quad": 0}
    _, n_tc, err = _run(ctx, wl, mode)
    assert n_tc == 1 and err < 1e-13
    ctx.synchronize()  # raises if a tensor-core wait had timed out
