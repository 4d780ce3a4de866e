"""Hierarchic FE with per-entity degrees on the GPU against the oracle:
HierarchicScalarFESpace(mesh, degree_functor) (fe/hierarchic_scalar_fe_space.h:
93-116) numbered like DynamicFEDofHandler, element matrices of
fe::DiffusionElementMatrixProvider + fe::MassElementMatrixProvider and vectors
of fe::ScalarLoadElementVectorProvider with each cell's own rule 2 Degree()
(indices and order bit-exact, values within 1e-12 of each element block's
largest entry).  Degrees 1..8 drawn per edge and per cell on triangle,
quadrilateral and hybrid meshes, both kernels (folded affine path and the
per-point path), boundary flags, dof entities, the uniform special case and a
known answer (the L2 projection of a quadratic)."""
import numpy as np
import pytest
import scipy.sparse as sps
import scipy.sparse.linalg as spla

from parity import O, L, W, compare_triplets, oracle_mesh
from test_gpu_hier import MESHES, _coeffs, _hybrid

pytestmark = pytest.mark.gpu


def _degrees(n_edges, n_cells, lo, hi, seed):
    rng = np.random.default_rng(seed)
    return rng.integers(lo, hi + 1, n_edges).astype(np.int32), rng.integers(lo, hi + 1, n_cells).astype(np.int32)


def _spaces(ctx, spec, ed, cd):
    mesh = W.build_mesh(ctx, spec)
    om = oracle_mesh(spec)
    assert mesh.num_edges == om.num_edges
    return mesh, L.Space.hierarchic_var(mesh, ed, cd), om, O.hier_var_space(om, ed, cd)


@pytest.mark.parametrize("mname,spec", MESHES, ids=[m[0] for m in MESHES])
@pytest.mark.parametrize("seed", [0, 1])
def test_hier_var_matches_oracle(ctx, mname, spec, seed):
    om0 = oracle_mesh(spec)
    ed, cd = _degrees(om0.num_edges, om0.num_cells, 1, 6, seed + 7 * len(mname))
    mesh, sp, om, osp = _spaces(ctx, spec, ed, cd)
    rng = np.random.default_rng(seed)
    assert sp.num_dofs == osp.num_dofs
    nl = sp.local_counts()
    assert np.array_equal(nl, osp.local_counts())
    gd, od = sp.cell_dofs(), osp.cell_dofs()
    for c in range(mesh.num_cells):
        assert np.array_equal(gd[c, :nl[c]], od[c, :nl[c]]), c
    gc, gi = sp.dof_entities()
    oc, oi = osp.dof_entities()
    assert np.array_equal(gc, oc) and np.array_equal(gi, oi)
    assert np.array_equal(sp.boundary_dof_flags().download(), osp.boundary_dof_flags())
    blocks = nl.astype(np.int64) ** 2
    for ak, gk in (("const", "zero"), ("zero", "const"), ("cell", "cell"), ("nodal", "const"), ("analytic", "zero")):
        keep = []
        ga, oa = _coeffs(ctx, ak, mesh.num_cells, mesh.num_nodes, rng, keep)
        gg, og = _coeffs(ctx, gk, mesh.num_cells, mesh.num_nodes, rng, keep)
        coo = L.COOMatrix(ctx, sp.num_dofs, sp.num_dofs, sp.num_triplets)
        L.assemble_matrix_rd(sp, L.rd_provider(ga, gg), coo)
        r, c, v = O.assemble_hier(osp, 0, oa, og).arrays()
        compare_triplets(coo.triplets(), r, c, v, blocks)
    keep = []
    gf, of = _coeffs(ctx, "analytic", mesh.num_cells, mesh.num_nodes, rng, keep)
    b0 = rng.standard_normal(sp.num_dofs)
    b = ctx.to_device(b0)
    L.assemble_vector_load(sp, L.load_provider(gf), b)
    bo = O.assemble_hier_load(osp, 0, of, b=b0)
    assert np.abs(b.download() - bo).max() <= 1e-12 * np.abs(bo).max()


def test_hier_var_many_groups_and_tiles(ctx):
    """A 12x12 hybrid mesh with degrees 1..8: up to eight degree groups per
    cell type, several tiles per CTA in the folded kernel."""
    spec = _hybrid(12, seed=9)
    om0 = oracle_mesh(spec)
    ed, cd = _degrees(om0.num_edges, om0.num_cells, 1, 8, 21)
    mesh, sp, om, osp = _spaces(ctx, spec, ed, cd)
    blocks = sp.local_counts().astype(np.int64) ** 2
    for ga, oa, gg, og in ((L.coeff(L.CONSTANT, 1.3), O.coeff(O.CONSTANT, 1.3), L.coeff(L.CONSTANT, 0.4),
                            O.coeff(O.CONSTANT, 0.4)),
                           (L.coeff(L.ANALYTIC, func=L.FN_POLY, params=[1, 0.5, 0, 0, 0.25]),
                            O.coeff(O.ANALYTIC, func=O.FN_POLY, params=[1, 0.5, 0, 0, 0.25]), L.coeff(L.ZERO),
                            O.coeff(O.ZERO))):
        coo = L.COOMatrix(ctx, sp.num_dofs, sp.num_dofs, sp.num_triplets)
        L.assemble_matrix_rd(sp, L.rd_provider(ga, gg), coo)
        r, c, v = O.assemble_hier(osp, 0, oa, og).arrays()
        compare_triplets(coo.triplets(), r, c, v, blocks)


@pytest.mark.parametrize("p", [2, 5])
def test_hier_var_uniform_degrees_equal_the_uniform_space(ctx, p):
    spec = _hybrid(5, seed=2)
    mesh = W.build_mesh(ctx, spec)
    su = L.Space.hierarchic(mesh, p)
    sv = L.Space.hierarchic_var(mesh, np.full(mesh.num_edges, p), np.full(mesh.num_cells, p))
    assert sv.num_dofs == su.num_dofs and sv.num_triplets == su.num_triplets
    for ga, gg in ((L.coeff(L.CONSTANT, 2.0), L.coeff(L.CONSTANT, 0.5)),
                   (L.coeff(L.ANALYTIC, func=L.FN_SINSIN, params=[1.5, 0.5, 1.0, 2.0]), L.coeff(L.ZERO))):
        tu, tv = [], []
        for sp, out in ((su, tu), (sv, tv)):
            coo = L.COOMatrix(ctx, sp.num_dofs, sp.num_dofs, sp.num_triplets)
            L.assemble_matrix_rd(sp, L.rd_provider(ga, gg), coo)
            out.append(coo.triplets())
        assert np.array_equal(tu[0]["row"], tv[0]["row"]) and np.array_equal(tu[0]["col"], tv[0]["col"])
        scale = np.abs(tu[0]["value"]).max()
        assert np.abs(tu[0]["value"] - tv[0]["value"]).max() <= 1e-14 * scale


def test_hier_var_projection_of_a_quadratic(ctx):
    """Degrees 2..5 everywhere: the space holds every quadratic, so the L2
    projection (device mass matrix and load vector, direct solve) reproduces
    u = 0.3 + 1.1 x - 0.7 y + 0.9 xy - 0.4 x^2 at the dofs' vertex values."""
    spec = _hybrid(6, seed=4)
    om0 = oracle_mesh(spec)
    ed, cd = _degrees(om0.num_edges, om0.num_cells, 2, 5, 5)
    mesh, sp, om, osp = _spaces(ctx, spec, ed, cd)
    coo = L.COOMatrix(ctx, sp.num_dofs, sp.num_dofs, sp.num_triplets)
    L.assemble_matrix_rd(sp, L.rd_provider(L.coeff(L.ZERO), L.coeff(L.CONSTANT, 1.0), 14, 14), coo)
    prm = np.zeros(16)
    prm[0], prm[1], prm[4], prm[5], prm[8] = 0.3, -0.7, 1.1, 0.9, -0.4
    b = ctx.zeros(sp.num_dofs)
    L.assemble_vector_load(sp, L.load_provider(L.coeff(L.ANALYTIC, func=L.FN_POLY, params=list(prm)), 14, 14), b)
    t = coo.triplets()
    M = sps.csr_matrix((t["value"], (t["row"], t["col"])), shape=(sp.num_dofs, sp.num_dofs))
    x = spla.spsolve(M.tocsc(), b.download())
    X, Y = om.xy[:, 0], om.xy[:, 1]
    u = 0.3 - 0.7 * Y + 1.1 * X + 0.9 * X * Y - 0.4 * X * X
    assert np.abs(x[:mesh.num_nodes] - u).max() < 1e-10  # node dofs are the vertex values


def test_hier_var_errors(ctx):
    mesh = L.Mesh.tp_triag(ctx, 2, 2)
    ne, nc = mesh.num_edges, mesh.num_cells
    for ed, cd in ((np.zeros(ne), np.ones(nc)), (np.ones(ne), np.zeros(nc)), (np.full(ne, 21), np.ones(nc))):
        with pytest.raises(L.LfgError) as e:
            L.Space.hierarchic_var(mesh, ed, cd)
        assert e.value.code == L.UNSUPPORTED
    with pytest.raises(ValueError):
        L.Space.hierarchic_var(mesh, np.ones(ne - 1), np.ones(nc))
