"""Post-processing on the GPU against the oracle: IntegrateMeshFunction
(cells and edges, the three closed integrands, every coefficient kind),
MeshFunctionFE / MeshFunctionGradFE, NodalProjection and
InitEssentialConditionFromFunction (lib/lf/fe/fe_tools.h:110-329), plus the
reference's own known answers computed on the device and size-independent
properties at larger sizes (polynomial reproduction, convergence rates)."""
import math

import numpy as np
import pytest

from parity import O, L, W, oracle_mesh
from helpers import poly

pytestmark = pytest.mark.gpu

F32_EQ = 4 * 2.0 ** -23
F64_EQ = 4 * 2.0 ** -52
RTOL = 1e-12


def _hybrid(n, seed=3):
    xy, cells = W.hybrid_mesh(n, seed=seed)
    return {"kind": "factory", "xy": xy, "cells": cells, "edges": None}


def _test0(scale=1.0):
    xy, cells, pe = O.factory_input("test0", x0=scale)
    return {"kind": "factory", "xy": xy, "cells": cells, "edges": None}


def _test3(goldens):
    t = goldens["test_mesh_3"]
    cells = np.full((len(t["triangles"]), 4), -1, np.int64)
    cells[:, :3] = t["triangles"]
    return {"kind": "factory", "xy": np.array(t["nodes"], float), "cells": cells, "edges": None}


MESHES = [("tptriag", {"kind": "tptriag", "nx": 6, "ny": 4}), ("tpquad", {"kind": "tpquad", "nx": 4, "ny": 5}),
          ("hybrid", _hybrid(5)), ("test0", _test0())]

ANALYTIC = {
    "poly": (1, poly(x2=1.0, x1y1=-0.5, y3=0.25, c=0.3)),
    "sinsin": (2, [0.5, 2.0, 1.0, 2.0]),
    "sincos": (3, [0.0, 1.0, 1.5, 0.5]),
    "exp": (4, [0.1, 0.7, 0.2, 0.3, -0.4, 0.5]),
    "trig": (5, [0.2, 1.0, 0.5, -0.3, 0.2, 1.0, 0.25, 0.5, 0.1]),
}


def _coeff(ctx, kind, n_ent, nv, rng, keep):
    """(gpu coeff, oracle coeff); per-cell data has n_ent entries."""
    if kind == "zero":
        return L.coeff(L.ZERO), O.coeff(O.ZERO)
    if kind == "const":
        return L.coeff(L.CONSTANT, 1.75), O.coeff(O.CONSTANT, 1.75)
    if kind in ("cell", "cellexp"):
        d = rng.standard_normal(n_ent)
        dd = ctx.to_device(d)
        keep.append(dd)
        k = (L.PER_CELL, O.PER_CELL) if kind == "cell" else (L.PER_CELL_EXP, O.PER_CELL_EXP)
        return L.coeff(k[0], data=dd), O.coeff(k[1], data=d)
    if kind == "nodal":
        d = rng.standard_normal(nv)
        dd = ctx.to_device(d)
        keep.append(dd)
        return L.coeff(L.NODAL_O1, data=dd), O.coeff(O.NODAL_O1, data=d)
    fn, p = ANALYTIC[kind]
    return L.coeff(L.ANALYTIC, func=fn, params=list(p)), O.coeff(O.ANALYTIC, func=fn, params=list(p))


class Case:
    def __init__(self, ctx, spec, degree):
        self.ctx = ctx
        self.mesh = W.build_mesh(ctx, spec)
        self.sp = L.Space.lagrange(self.mesh, degree)
        self.omesh = oracle_mesh(spec)
        self.osp = O.Space(self.omesh, degree)
        assert self.sp.num_dofs == self.osp.num_dofs


COMBOS = [  # (integrand, u kind, with u_h, flags)
    (L.INT_VALUE, "const", False, None), (L.INT_VALUE, "trig", True, "random"),
    (L.INT_SQ_DIFF, "cell", True, None), (L.INT_SQ_DIFF, "cellexp", False, "random"),
    (L.INT_SQ_DIFF, "nodal", True, None), (L.INT_SQ_DIFF, "sinsin", True, None),
    (L.INT_GRAD_SQ_DIFF, "poly", True, None), (L.INT_GRAD_SQ_DIFF, "sincos", True, "random"),
    (L.INT_GRAD_SQ_DIFF, "exp", True, None), (L.INT_GRAD_SQ_DIFF, "nodal", True, "none"),
    (L.INT_GRAD_SQ_DIFF, "zero", True, None), (L.INT_VALUE, "exp", False, None),
]


def _flags(kind, n, rng):
    if kind is None:
        return None
    if kind == "none":
        return np.zeros(n, np.uint8)
    return (rng.random(n) < 0.5).astype(np.uint8)


@pytest.mark.parametrize("mname,spec", MESHES, ids=[m[0] for m in MESHES])
@pytest.mark.parametrize("degree", [1, 2, 3])
def test_integrate_cells_matches_oracle(ctx, mname, spec, degree):
    c = Case(ctx, spec, degree)
    rng = np.random.default_rng(11 * degree + len(mname))
    for qdeg in (2 * degree, 5):
        for kind, ukind, fe, fkind in COMBOS:
            keep = []
            gu, ou = _coeff(ctx, ukind, c.mesh.num_cells, c.mesh.num_nodes, rng, keep)
            dofs = rng.standard_normal(c.sp.num_dofs) if fe else None
            dd = ctx.to_device(dofs) if fe else None
            fl = _flags(fkind, c.mesh.num_cells, rng)
            fld = ctx.to_device(fl) if fl is not None else None
            got = L.integrate_mesh_function(c.mesh, kind, gu, c.sp, dd, qdeg, fld)
            ref = O.integrate(c.osp, kind, ou, dofs=dofs, qdeg=qdeg, flags=fl)
            # scale: the integral of |integrand| bounded through the squares
            sq = O.integrate(c.osp, O.INT_SQ_DIFF, ou, dofs=(-dofs if fe else None), qdeg=qdeg, flags=fl)
            scale = abs(ref) + math.sqrt(max(sq, 0.0) * 10.0) + 1e-300
            assert abs(got - ref) <= RTOL * scale, (mname, degree, qdeg, kind, ukind, got, ref)


@pytest.mark.parametrize("mname,spec", MESHES[:3], ids=[m[0] for m in MESHES[:3]])
@pytest.mark.parametrize("degree", [1, 2, 3])
def test_integrate_edges_matches_oracle(ctx, mname, spec, degree):
    c = Case(ctx, spec, degree)
    rng = np.random.default_rng(5 * degree)
    _, ef = c.mesh.boundary_flags()
    for kind, ukind, fe, fl in [(L.INT_VALUE, "const", False, ef), (L.INT_VALUE, "trig", True, None),
                                (L.INT_SQ_DIFF, "cell", True, ef), (L.INT_SQ_DIFF, "nodal", True, "random"),
                                (L.INT_SQ_DIFF, "exp", False, None)]:
        keep = []
        gu, ou = _coeff(ctx, ukind, c.mesh.num_edges, c.mesh.num_nodes, rng, keep)
        dofs = rng.standard_normal(c.sp.num_dofs) if fe else None
        dd = ctx.to_device(dofs) if fe else None
        if isinstance(fl, str):
            fl = _flags(fl, c.mesh.num_edges, rng)
        fld = ctx.to_device(np.ascontiguousarray(fl, np.uint8)) if fl is not None else None
        got = L.integrate_mesh_function(c.mesh, kind, gu, c.sp, dd, 2 * degree + 1, fld, codim=1)
        ref = O.integrate(c.osp, kind, ou, dofs=dofs, qdeg=2 * degree + 1, flags=fl, codim=1)
        assert abs(got - ref) <= RTOL * (abs(ref) + 1.0), (mname, degree, kind, ukind, got, ref)


def test_integrate_known_answers(ctx, goldens):
    """fe_tools_tests.cc:44-85 and gfe_tests.cc:27-45, 141-160 on the device."""
    kat = goldens["integrate_mesh_function_kat"]["integrals"]
    m0 = W.build_mesh(ctx, _test0())

    def val(u, deg):
        return L.integrate_mesh_function(m0, L.INT_VALUE, u, quad_degree=deg)

    def an(fn, p):
        return L.coeff(L.ANALYTIC, func=fn, params=list(p))

    cases = [("intScalar", an(L.FN_TRIG, [0, 0, 0, 1, 0, 1, 0, 0, 0.5]), 20),
             ("intVec[0]", an(L.FN_POLY, poly(x1=1.0)), 20), ("intVec[1]", an(L.FN_POLY, poly(x1y1=1.0)), 20),
             ("intMatrixDyn(0, 0)", an(L.FN_POLY, poly(c=1.0)), 10),
             ("intMatrixDyn(0, 1)", an(L.FN_POLY, poly(x1=1.0)), 10),
             ("intMatrixDyn(0, 2)", an(L.FN_POLY, poly(y1=1.0)), 10),
             ("intMatrixDyn(1, 0)", an(L.FN_POLY, poly(x1y1=1.0)), 10),
             ("intMatrixDyn(1, 1)", an(L.FN_POLY, poly(x2=1.0)), 10),
             ("intMatrixDyn(1, 2)", an(L.FN_POLY, poly(y2=1.0)), 10)]
    for key, u, deg in cases:
        want = kat[key]["value"]
        assert abs(val(u, deg) - want) <= F32_EQ * abs(want), key
    assert val(an(L.FN_TRIG, [0, 1, 0, 0, 0, 1, 0.5, 0, 0.5]), 20) < 1e-10  # cos(pi x)
    g = goldens["gfe_norm_kat"]
    m3 = W.build_mesh(ctx, _test3(goldens))
    n1 = math.sqrt(L.integrate_mesh_function(m3, L.INT_SQ_DIFF, an(L.FN_POLY, poly(x1=1.0, x1y1=-1.0)), quad_degree=4))
    assert abs(n1 - g["l2norm_x_1my"]["value"]) < g["l2norm_x_1my"]["tolerance"]
    n2 = math.sqrt(L.integrate_mesh_function(m3, L.INT_GRAD_SQ_DIFF, an(L.FN_POLY, poly(x1y1=1.0)), quad_degree=4))
    assert abs(n2 - g["l2norm_vf_y_mx"]["value"]) < g["l2norm_vf_y_mx"]["tolerance"]


@pytest.mark.parametrize("degree", [1, 2, 3])
def test_norms_two_ways(ctx, goldens, degree):
    """gfe_tests.cc:47-139 on the device: c^T M c = int u_h^2, c^T A c = int |grad u_h|^2."""
    for spec in (_test3(goldens), _test0(), _hybrid(6)):
        mesh = W.build_mesh(ctx, spec)
        sp = L.Space.lagrange(mesh, degree)
        c = np.random.default_rng(3 + degree).uniform(-1, 1, sp.num_dofs)
        cd = ctx.to_device(c)
        for alpha, gamma, kind in ((0.0, 1.0, L.INT_SQ_DIFF), (1.0, 0.0, L.INT_GRAD_SQ_DIFF)):
            coo = L.COOMatrix(ctx, sp.num_dofs, sp.num_dofs, sp.num_triplets)
            L.assemble_matrix_rd(sp, L.rd_provider(L.coeff(L.CONSTANT, alpha), L.coeff(L.CONSTANT, gamma),
                                                   2 * degree, 2 * degree), coo)
            A = coo.make_sparse()
            y = ctx.zeros(sp.num_dofs)
            A.spmv(cd, y)
            from_a = float(c @ y.download())
            direct = L.integrate_mesh_function(mesh, kind, None, sp, cd, 2 * degree)
            assert abs(from_a - direct) <= 1e-12 * abs(from_a)


@pytest.mark.parametrize("mname,spec", MESHES, ids=[m[0] for m in MESHES])
@pytest.mark.parametrize("degree", [1, 2, 3])
def test_fe_eval_matches_oracle(ctx, mname, spec, degree):
    c = Case(ctx, spec, degree)
    rng = np.random.default_rng(degree)
    pts = np.array([[0.1, 0.2], [0.5, 0.25], [0.0, 0.0], [1 / 3, 1 / 3], [0.7, 0.1]])
    dofs = rng.standard_normal(c.sp.num_dofs)
    v, g = L.fe_eval(c.sp, c.ctx.to_device(dofs), pts, grads=True)
    ov, og = O.eval_fe(c.osp, dofs, pts, grads=True)
    sv = np.abs(ov).max()
    sg = np.abs(og).max()
    assert np.abs(v.download() - ov).max() <= 1e-13 * sv
    assert np.abs(g.download() - og).max() <= 1e-13 * sg


@pytest.mark.parametrize("mname,spec", MESHES, ids=[m[0] for m in MESHES])
@pytest.mark.parametrize("degree", [1, 2, 3])
def test_nodal_projection_matches_oracle(ctx, mname, spec, degree):
    c = Case(ctx, spec, degree)
    rng = np.random.default_rng(17 + degree)
    out = ctx.zeros(c.sp.num_dofs)
    for ukind in ("cell", "cellexp", "nodal", "const", "poly", "sinsin", "sincos", "exp", "trig"):
        for fkind in (None, "random"):
            keep = []
            gu, ou = _coeff(ctx, ukind, c.mesh.num_cells, c.mesh.num_nodes, rng, keep)
            fl = _flags(fkind, c.mesh.num_cells, rng)
            L.nodal_projection(c.sp, gu, out, ctx.to_device(fl) if fl is not None else None)
            got = out.download()
            ref = O.nodal_projection_mf(c.osp, ou, fl)
            if ukind in ("cell", "const"):
                assert np.array_equal(got, ref), (ukind, fkind)  # copies: bit-exact owner choice
            else:
                assert np.abs(got - ref).max() <= 1e-14 * max(np.abs(ref).max(), 1.0), (ukind, fkind)


@pytest.mark.parametrize("mname,spec", MESHES, ids=[m[0] for m in MESHES])
@pytest.mark.parametrize("degree", [1, 2, 3])
def test_essential_condition_matches_oracle(ctx, mname, spec, degree):
    c = Case(ctx, spec, degree)
    rng = np.random.default_rng(23 + degree)
    _, ef = c.mesh.boundary_flags()
    fd = ctx.zeros(c.sp.num_dofs, np.uint8)
    vd = ctx.zeros(c.sp.num_dofs)
    for ukind, fl in (("poly", ef), ("cell", ef), ("nodal", "random"), ("trig", "random")):
        if isinstance(fl, str):
            fl = _flags(fl, c.mesh.num_edges, rng)
        keep = []
        gu, ou = _coeff(ctx, ukind, c.mesh.num_edges, c.mesh.num_nodes, rng, keep)
        L.init_essential_condition(c.sp, ctx.to_device(np.ascontiguousarray(fl, np.uint8)), gu, fd, vd)
        of, ov = O.init_essential_condition(c.osp, fl, ou)
        assert np.array_equal(fd.download(), of)
        if ukind == "cell":
            assert np.array_equal(vd.download(), ov)
        else:
            assert np.abs(vd.download() - ov).max() <= 1e-14 * max(np.abs(ov).max(), 1.0)


def test_projection_known_answers(ctx):
    """gfe_tests.cc:162-236 and fe_tools_tests.cc:87-128 on the device."""
    for scale, p, tol in ((1.0, [0, 1, 0, 1, 0, -1], F64_EQ), (1.0 / 3.0, [0, 1, 0, 0, 0, 1], F32_EQ)):
        spec = _test0(scale)
        mesh = W.build_mesh(ctx, spec)
        sp = L.Space.lagrange(mesh, 1)
        out = ctx.zeros(sp.num_dofs)
        L.nodal_projection(sp, L.coeff(L.ANALYTIC, func=L.FN_EXP, params=p), out)
        v = out.download()
        xy = np.asarray(spec["xy"])[: sp.num_dofs]  # O1: dof = node index
        want = np.exp(p[3] * xy[:, 0] + p[5] * xy[:, 0] * xy[:, 1])
        assert np.all(np.abs(v - want) <= tol * np.abs(want))
    # set_dirbdc: g = x^2 + y^2 on the boundary nodes
    spec = _test0()
    mesh = W.build_mesh(ctx, spec)
    sp = L.Space.lagrange(mesh, 1)
    nf, ef = mesh.boundary_flags()
    fd = L.DeviceArray(ctx, sp.num_dofs, np.uint8)
    vd = ctx.zeros(sp.num_dofs)
    L.init_essential_condition(sp, ctx.to_device(ef.astype(np.uint8)), L.coeff(
        L.ANALYTIC, func=L.FN_POLY, params=list(poly(x2=1.0, y2=1.0))), fd, vd)
    xy = np.asarray(spec["xy"])
    r2 = (xy ** 2).sum(1)
    f, v = fd.download(), vd.download()
    assert np.array_equal(f.astype(bool), nf.astype(bool))
    assert np.all(np.abs(v[f == 1] - r2[f == 1]) <= F64_EQ * r2[f == 1])
    assert np.all(v[f == 0] == 0.0)


def test_first_entity_quirk_and_errors(ctx):
    mesh = W.build_mesh(ctx, _test0())
    sp = L.Space.lagrange(mesh, 2)
    one = L.coeff(L.CONSTANT, 1.0)
    none = ctx.to_device(np.zeros(mesh.num_cells, np.uint8))
    area0 = L.integrate_mesh_function(mesh, L.INT_VALUE, one, quad_degree=1, flags=none)
    osp = O.Space(oracle_mesh(_test0()), 2)
    assert abs(area0 - O.integrate(osp, O.INT_VALUE, O.coeff(O.CONSTANT, 1.0), qdeg=1,
                                   flags=np.zeros(mesh.num_cells, np.uint8))) < 1e-15
    assert abs(L.integrate_mesh_function(mesh, L.INT_VALUE, one, quad_degree=1) - 9.0) < 1e-13
    dd = ctx.zeros(sp.num_dofs)
    with pytest.raises(L.LfgError) as e:
        L.integrate_mesh_function(mesh, L.INT_GRAD_SQ_DIFF, one, sp, dd, 2, codim=1)
    assert e.value.code == L.UNSUPPORTED
    with pytest.raises(L.LfgError) as e:
        L.integrate_mesh_function(mesh, L.INT_VALUE, one, None, dd, 2)
    assert e.value.code == L.INVALID_ARG
    with pytest.raises(L.LfgError) as e:
        L.integrate_mesh_function(mesh, L.INT_VALUE, one, quad_degree=2, codim=2)
    assert e.value.code == L.UNSUPPORTED
    with pytest.raises(L.LfgError) as e:
        L.integrate_mesh_function(mesh, L.INT_VALUE, L.coeff(L.ANALYTIC, func=99), quad_degree=2)
    assert e.value.code == L.UNSUPPORTED
    other = L.Space.lagrange(L.Mesh.tp_triag(ctx, 2, 2), 1)
    with pytest.raises(L.LfgError) as e:
        L.integrate_mesh_function(mesh, L.INT_VALUE, one, other, ctx.zeros(other.num_dofs), 2)
    assert e.value.code == L.INVALID_ARG


@pytest.mark.parametrize("degree", [1, 2, 3])
def test_large_interpolation_reproduces_polynomials(ctx, degree):
    """Size-independent property at 512 x 512 cells: O_p interpolation of a
    degree-p polynomial is exact, so both error integrals vanish."""
    p = {1: poly(x1=1.0, y1=-2.0, c=0.5), 2: poly(x2=1.0, x1y1=-0.5, y1=1.0),
         3: poly(x3=0.1, y3=-0.2, x1y2=0.3, x1=1.0)}[degree]
    u = L.coeff(L.ANALYTIC, func=L.FN_POLY, params=list(p))
    for mesh in (L.Mesh.tp_triag(ctx, 512, 512), L.Mesh.tp_quad(ctx, 512, 512)):
        sp = L.Space.lagrange(mesh, degree)
        c = ctx.zeros(sp.num_dofs)
        L.nodal_projection(sp, u, c)
        assert L.integrate_mesh_function(mesh, L.INT_SQ_DIFF, u, sp, c, 2 * degree + 2) < 1e-26
        assert L.integrate_mesh_function(mesh, L.INT_GRAD_SQ_DIFF, u, sp, c, 2 * degree + 2) < 1e-22


def test_demo_error_norms_converge(ctx):
    """homDir_linfe_demo.cc:150-188 pipeline on the device: -lap u = f with
    u = x(1-x)y(1-y), O1 and O2, solve, L2 / H1-seminorm errors; rates
    h^{p+1} and h^p between successive meshes (O1: 64^2 -> 128^2, O2: 16^2 -> 32^2)."""
    u = L.coeff(L.ANALYTIC, func=L.FN_POLY, params=list(poly(x1y1=1.0, x2y1=-1.0, x1y2=-1.0, x2y2=1.0)))
    f = L.coeff(L.ANALYTIC, func=L.FN_POLY, params=list(poly(y1=2.0, y2=-2.0, x1=2.0, x2=-2.0)))
    for degree, sizes in ((1, (64, 128)), (2, (16, 32))):
        errs = []
        for n in sizes:
            mesh = L.Mesh.tp_triag(ctx, n, n)
            sp = L.Space.lagrange(mesh, degree)
            coo = L.COOMatrix(ctx, sp.num_dofs, sp.num_dofs, sp.num_triplets + sp.num_dofs)
            L.assemble_matrix_rd(sp, L.rd_provider(L.coeff(L.CONSTANT, 1.0), L.coeff(L.ZERO)), coo)
            b = ctx.zeros(sp.num_dofs)
            L.assemble_vector_load(sp, L.load_provider(f), b)
            fd = L.DeviceArray(ctx, sp.num_dofs, np.uint8)
            gd = ctx.zeros(sp.num_dofs)
            _, ef = mesh.boundary_flags()
            L.init_essential_condition(sp, ctx.to_device(ef.astype(np.uint8)), u, fd, gd)
            coo.fix_flagged_solution_components(fd, gd, b)
            x = ctx.zeros(sp.num_dofs)
            coo.make_sparse().solve_pcg(b, x, rtol=1e-12)
            l2 = math.sqrt(L.integrate_mesh_function(mesh, L.INT_SQ_DIFF, u, sp, x, 2 * degree + 2))
            h1 = math.sqrt(L.integrate_mesh_function(mesh, L.INT_GRAD_SQ_DIFF, u, sp, x, 2 * degree + 2))
            errs.append((l2, h1))
        rl2 = math.log2(errs[0][0] / errs[1][0])
        rh1 = math.log2(errs[0][1] / errs[1][1])
        assert abs(rl2 - (degree + 1)) < 0.25, (degree, errs)
        assert abs(rh1 - degree) < 0.2, (degree, errs)
