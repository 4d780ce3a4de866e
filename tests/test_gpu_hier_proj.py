"""Post-processing on hierarchic spaces on the GPU against the oracle.

NodalProjection (fe/fe_tools.h:198-259): uniform degrees 1..12 and per-entity
degrees on four mesh kinds, every coefficient kind, with and without a cell
predicate; the per-entity path with all degrees equal to p gives the uniform
space's result value for value; a mid-size hybrid mesh (about 75k cells).

IntegrateMeshFunction (fe/fe_tools.h:110-165) of u_h + u, (u_h - u)^2 and
|grad u_h - grad u|^2 with u_h on a hierarchic space (uniform degrees 1..10,
per-entity degrees), with and without a cell predicate."""
import numpy as np
import pytest

from parity import O, L, W, oracle_mesh
from test_gpu_hier import MESHES, _hybrid
from test_gpu_post import _coeff, _flags

pytestmark = pytest.mark.gpu

UKINDS = ("cell", "nodal", "const", "poly", "sinsin", "sincos", "exp", "trig")


def _tol(p):
    # the dual's rows grow with the degree (segment duals carry (2i - 1) P'_{i-1}
    # factors); FP64 sums of about n x ne products in another order
    return 1e-12 if p <= 5 else 1e-11


def _check(ctx, sp, osp, p_oracle, tol, mesh, rng, ukinds=UKINDS):
    out = ctx.zeros(sp.num_dofs)
    for ukind in ukinds:
        for fkind in (None, "random"):
            keep = []
            gu, ou = _coeff(ctx, ukind, mesh.num_cells, mesh.num_nodes, rng, keep)
            fl = _flags(fkind, mesh.num_cells, rng)
            L.nodal_projection(sp, gu, out, ctx.to_device(fl) if fl is not None else None)
            got = out.download()
            ref = O.nodal_projection_hier(osp, p_oracle, ou, fl)
            assert np.abs(got - ref).max() <= tol * max(np.abs(ref).max(), 1.0), (ukind, fkind)


@pytest.mark.parametrize("mname,spec", MESHES, ids=[m[0] for m in MESHES])
@pytest.mark.parametrize("p", [1, 2, 3, 5, 8, 12])
def test_hier_projection_matches_oracle(ctx, mname, spec, p):
    mesh = W.build_mesh(ctx, spec)
    sp = L.Space.hierarchic(mesh, p)
    osp = O.hier_space(oracle_mesh(spec), p)
    _check(ctx, sp, osp, p, _tol(p), mesh, np.random.default_rng(31 * p + len(mname)))


@pytest.mark.parametrize("mname,spec", MESHES, ids=[m[0] for m in MESHES])
def test_hier_var_projection_matches_oracle(ctx, mname, spec):
    om = oracle_mesh(spec)
    rng = np.random.default_rng(3 + len(mname))
    ed = rng.integers(1, 7, om.num_edges).astype(np.int32)
    cd = rng.integers(1, 7, om.num_cells).astype(np.int32)
    mesh = W.build_mesh(ctx, spec)
    sp = L.Space.hierarchic_var(mesh, ed, cd)
    osp = O.hier_var_space(om, ed, cd)
    _check(ctx, sp, osp, 0, _tol(6), mesh, rng)


def test_hier_var_projection_larger_mesh(ctx):
    """Per-entity degrees 1..5 on a 24 x 24 hybrid mesh (about 900 cells, many
    distinct dual tables) against the oracle."""
    spec = _hybrid(24, seed=6)
    om = oracle_mesh(spec)
    rng = np.random.default_rng(77)
    ed = rng.integers(1, 6, om.num_edges).astype(np.int32)
    cd = rng.integers(1, 6, om.num_cells).astype(np.int32)
    mesh = W.build_mesh(ctx, spec)
    sp = L.Space.hierarchic_var(mesh, ed, cd)
    osp = O.hier_var_space(om, ed, cd)
    _check(ctx, sp, osp, 0, _tol(5), mesh, rng, ukinds=("nodal", "sincos"))


@pytest.mark.parametrize("p", [2, 4])
def test_hier_var_projection_with_equal_degrees_is_the_uniform_one(ctx, p):
    spec = _hybrid(6, seed=2)
    mesh = W.build_mesh(ctx, spec)
    su = L.Space.hierarchic(mesh, p)
    sv = L.Space.hierarchic_var(mesh, np.full(mesh.num_edges, p), np.full(mesh.num_cells, p))
    u = L.coeff(L.ANALYTIC, func=L.FN_SINCOS, params=[0.2, 1.0, 1.5, 0.5])
    a, b = ctx.zeros(su.num_dofs), ctx.zeros(sv.num_dofs)
    L.nodal_projection(su, u, a)
    L.nodal_projection(sv, u, b)
    assert np.array_equal(a.download(), b.download())


def test_hier_projection_mid_size(ctx):
    """A 224 x 224 hybrid mesh (about 75k cells), degree 4, against the oracle."""
    spec = _hybrid(224, seed=8)
    mesh = W.build_mesh(ctx, spec)
    sp = L.Space.hierarchic(mesh, 4)
    osp = O.hier_space(oracle_mesh(spec), 4)
    _check(ctx, sp, osp, 4, _tol(4), mesh, np.random.default_rng(4), ukinds=("nodal", "trig"))


@pytest.mark.parametrize("mname,spec", MESHES, ids=[m[0] for m in MESHES])
@pytest.mark.parametrize("p", [1, 2, 4, 7, 10])
def test_hier_integrate_matches_oracle(ctx, mname, spec, p):
    mesh = W.build_mesh(ctx, spec)
    sp = L.Space.hierarchic(mesh, p)
    osp = O.hier_space(oracle_mesh(spec), p)
    rng = np.random.default_rng(5 * p + len(mname))
    dofs = rng.standard_normal(sp.num_dofs)
    dd = ctx.to_device(dofs)
    for kind in (L.INT_VALUE, L.INT_SQ_DIFF, L.INT_GRAD_SQ_DIFF):
        for ukind in ("sinsin", "nodal", "cell"):
            for fkind in (None, "random"):
                keep = []
                gu, ou = _coeff(ctx, ukind, mesh.num_cells, mesh.num_nodes, rng, keep)
                fl = _flags(fkind, mesh.num_cells, rng)
                fld = ctx.to_device(fl) if fl is not None else None
                got = L.integrate_mesh_function(mesh, kind, gu, sp, dd, 2 * p + 2, fld)
                ref = O.integrate_hier(osp, p, kind, ou, dofs, 2 * p + 2, fl)
                sq = O.integrate_hier(osp, p, O.INT_SQ_DIFF, ou, -dofs, 2 * p + 2, fl)
                assert abs(got - ref) <= 1e-12 * (abs(ref) + abs(sq) + 1.0), (kind, ukind, fkind, got, ref)


def test_hier_var_integrate_matches_oracle(ctx):
    spec = _hybrid(12, seed=9)
    om = oracle_mesh(spec)
    rng = np.random.default_rng(19)
    ed = rng.integers(1, 7, om.num_edges).astype(np.int32)
    cd = rng.integers(1, 7, om.num_cells).astype(np.int32)
    mesh = W.build_mesh(ctx, spec)
    sp = L.Space.hierarchic_var(mesh, ed, cd)
    osp = O.hier_var_space(om, ed, cd)
    dofs = rng.standard_normal(sp.num_dofs)
    dd = ctx.to_device(dofs)
    for kind in (L.INT_VALUE, L.INT_SQ_DIFF, L.INT_GRAD_SQ_DIFF):
        keep = []
        gu, ou = _coeff(ctx, "sincos", mesh.num_cells, mesh.num_nodes, rng, keep)
        got = L.integrate_mesh_function(mesh, kind, gu, sp, dd, 14)
        ref = O.integrate_hier(osp, 0, kind, ou, dofs, 14)
        assert abs(got - ref) <= 1e-12 * (abs(ref) + 1.0), (kind, got, ref)
    with pytest.raises(L.LfgError) as e:
        L.integrate_mesh_function(mesh, L.INT_SQ_DIFF, gu, sp, dd, 6, None, 1)
    assert e.value.code == L.UNSUPPORTED


@pytest.mark.parametrize("mname,spec", MESHES, ids=[m[0] for m in MESHES])
@pytest.mark.parametrize("p", [1, 3, 6, 9])
def test_hier_fe_eval_matches_oracle(ctx, mname, spec, p):
    """MeshFunctionFE / MeshFunctionGradFE of a hierarchic u_h at shared
    reference points of every cell."""
    mesh = W.build_mesh(ctx, spec)
    sp = L.Space.hierarchic(mesh, p)
    osp = O.hier_space(oracle_mesh(spec), p)
    rng = np.random.default_rng(p + 3 * len(mname))
    dofs = rng.standard_normal(sp.num_dofs)
    pts = np.array([[0.1, 0.2], [0.25, 0.25], [0.6, 0.3], [0.05, 0.9], [0.0, 0.0], [0.5, 0.5]])
    v, g = L.fe_eval(sp, ctx.to_device(dofs), pts, values=True, grads=True)
    vals, grads = v.download(), g.download()
    ov, og = O.eval_fe_hier(osp, p, dofs, pts)
    assert np.abs(vals - ov).max() <= 1e-12 * max(1.0, np.abs(ov).max())
    assert np.abs(grads - og).max() <= 1e-12 * max(1.0, np.abs(og).max())


def test_hier_var_fe_eval_matches_oracle(ctx):
    spec = _hybrid(10, seed=3)
    om = oracle_mesh(spec)
    rng = np.random.default_rng(23)
    ed = rng.integers(1, 7, om.num_edges).astype(np.int32)
    cd = rng.integers(1, 7, om.num_cells).astype(np.int32)
    mesh = W.build_mesh(ctx, spec)
    sp = L.Space.hierarchic_var(mesh, ed, cd)
    osp = O.hier_var_space(om, ed, cd)
    dofs = rng.standard_normal(sp.num_dofs)
    pts = np.array([[0.2, 0.1], [0.3, 0.6], [0.45, 0.45]])
    v, g = L.fe_eval(sp, ctx.to_device(dofs), pts, values=True, grads=True)
    vals, grads = v.download(), g.download()
    ov, og = O.eval_fe_hier(osp, 0, dofs, pts)
    assert np.abs(vals - ov).max() <= 1e-12 * max(1.0, np.abs(ov).max())
    assert np.abs(grads - og).max() <= 1e-12 * max(1.0, np.abs(og).max())
