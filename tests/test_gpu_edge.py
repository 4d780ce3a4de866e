"""Boundary-edge providers (GPU): MassEdgeMatrixProvider /
ScalarLoadEdgeVectorProvider with codim-1 AssembleMatrixLocally /
AssembleVectorLocally, against the oracle (indices and order bit-exact,
values within 1e-12 of each edge block's largest entry)."""
import numpy as np
import pytest

from parity import O, L, W, compare_triplets, oracle_mesh

pytestmark = pytest.mark.gpu


def _hybrid(n, seed=3):
    xy, cells = W.hybrid_mesh(n, seed=seed)
    return {"kind": "factory", "xy": xy, "cells": cells, "edges": None}


MESHES = [("tptriag", {"kind": "tptriag", "nx": 6, "ny": 4}), ("tpquad", {"kind": "tpquad", "nx": 4, "ny": 5}),
          ("hybrid", _hybrid(5))]


def _coeffs(ctx, kind, ne, nv, rng, keep):
    """(gpu coeff, oracle coeff) of one kind; per-cell data is per edge here."""
    if kind == "const":
        return L.coeff(L.CONSTANT, 2.5), O.coeff(O.CONSTANT, 2.5)
    if kind == "edge":
        d = np.exp(rng.standard_normal(ne))
        dd = ctx.to_device(d)
        keep.append(dd)
        return L.coeff(L.PER_CELL, data=dd), O.coeff(O.PER_CELL, data=d)
    if kind == "exp":
        d = 0.5 * rng.standard_normal(ne)
        dd = ctx.to_device(d)
        keep.append(dd)
        return L.coeff(L.PER_CELL_EXP, data=dd), O.coeff(O.PER_CELL_EXP, data=d)
    if kind == "nodal":
        d = rng.standard_normal(nv)
        dd = ctx.to_device(d)
        keep.append(dd)
        return L.coeff(L.NODAL_O1, data=dd), O.coeff(O.NODAL_O1, data=d)
    p = [1.0, 0.5, 2.0, 3.0]
    return L.coeff(L.ANALYTIC, func=L.FN_SINSIN, params=p), O.coeff(O.ANALYTIC, func=O.FN_SINSIN, params=p)


def _flags(kind, mesh, rng):
    if kind == "all":
        return None
    if kind == "boundary":
        return mesh.boundary_flags()[1].astype(np.uint8)
    return (rng.random(mesh.num_edges) < 0.4).astype(np.uint8)


@pytest.mark.parametrize("mname,spec", MESHES, ids=[m[0] for m in MESHES])
@pytest.mark.parametrize("degree", [1, 2, 3])
@pytest.mark.parametrize("ckind,fkind", [("const", "all"), ("edge", "boundary"), ("exp", "random"),
                                         ("nodal", "boundary"), ("analytic", "random")])
def test_edge_providers_match_oracle(ctx, mname, spec, degree, ckind, fkind):
    rng = np.random.default_rng(degree * 7 + len(ckind))
    mesh = W.build_mesh(ctx, spec)
    sp = L.Space.lagrange(mesh, degree)
    omesh = oracle_mesh(spec)
    osp = O.Space(omesh, degree)
    keep = []
    gc, oc = _coeffs(ctx, ckind, mesh.num_edges, mesh.num_nodes, rng, keep)
    fl = _flags(fkind, mesh, rng)
    fl_d = ctx.to_device(fl) if fl is not None else None
    n = degree + 1
    active = mesh.num_edges if fl is None else int(fl.sum())
    # matrix
    coo = L.COOMatrix(ctx, sp.num_dofs, sp.num_dofs, active * n * n)
    L.assemble_matrix_edge_mass(sp, L.edge_mass_provider(gc, fl_d), coo)
    r, c, v = O.assemble_edge_mass(osp, oc, fl).arrays()
    compare_triplets(coo.triplets(), r, c, v, np.full(active, n * n))
    # vector, added to a nonzero start
    b0 = rng.standard_normal(sp.num_dofs)
    b = ctx.to_device(b0)
    L.assemble_vector_edge_load(sp, L.edge_load_provider(gc, fl_d), b)
    bo = O.assemble_edge_load(osp, oc, fl, b=b0)
    assert np.abs(b.download() - bo).max() <= 1e-12 * np.abs(bo).max()


def test_edge_mass_known_answer_mesh0(ctx):
    """lagr_fe_tests.cc:571-601, 696-722: O1, gamma = g = 1, every edge of the
    hybrid test mesh: A_e = |e| [[1/3, 1/6], [1/6, 1/3]], phi_e = |e| [1/2, 1/2]."""
    xy, cells, pe = O.factory_input("test0")
    mesh = L.Mesh.from_factory(ctx, xy, cells, pe)
    sp = L.Space.lagrange(mesh, 1)
    coo = L.COOMatrix(ctx, sp.num_dofs, sp.num_dofs, 4 * mesh.num_edges)
    L.assemble_matrix_edge_mass(sp, L.edge_mass_provider(L.coeff(L.CONSTANT, 1.0)), coo)
    en = mesh.topology()[0]
    xyd, _ = mesh.geometry()
    le = np.hypot(*(xyd[en[:, 1]] - xyd[en[:, 0]]).T)
    t = coo.triplets()
    assert np.abs(t["value"] - (le[:, None] * np.array([1 / 3, 1 / 6, 1 / 6, 1 / 3])).ravel()).max() < 1e-15
    assert np.array_equal(t["row"].reshape(-1, 4)[:, [0, 1, 2, 3]], np.stack([en[:, 0], en[:, 0], en[:, 1], en[:, 1]], 1))
    b = ctx.zeros(sp.num_dofs)
    L.assemble_vector_edge_load(sp, L.edge_load_provider(L.coeff(L.CONSTANT, 1.0)), b)
    ref = np.zeros(sp.num_dofs)
    np.add.at(ref, en[:, 0], 0.5 * le)
    np.add.at(ref, en[:, 1], 0.5 * le)
    assert np.abs(b.download() - ref).max() < 1e-14


def test_edge_mass_capacity_and_kinds(ctx):
    mesh = L.Mesh.tp_triag(ctx, 3, 3)
    sp = L.Space.lagrange(mesh, 2)
    small = L.COOMatrix(ctx, sp.num_dofs, sp.num_dofs, 8)
    with pytest.raises(L.LfgError) as e:
        L.assemble_matrix_edge_mass(sp, L.edge_mass_provider(L.coeff(L.CONSTANT, 1.0)), small)
    assert e.value.code == L.CAPACITY
    assert len(small) == 0
