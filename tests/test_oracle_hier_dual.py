"""Evaluation nodes, dual bases and NodalProjection of hierarchic elements
(CPU): the oracle's restatement of FeHierarchicTria / FeHierarchicQuad::
NodalValuesToDofs (lib/lf/fe/hierarchic_fe.h:820-1083, 1445-1680) against the
reference's own dual tests (fe/test/fe_space_hierarchic_tests.cc:476-582: the
dual of every basis function is its unit vector, all edge orientations), the
library's tables (lfg_hier_dual, built independently in matrix form) against
the oracle, and fe::NodalProjection (fe/fe_tools.h:198-259) on uniform and
per-entity degree spaces: exact reproduction of the polynomials the space
holds, convergence for a smooth function, and the cell predicate; and
IntegrateMeshFunction with u_h on hierarchic spaces against NumPy."""
import itertools
import math
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
import oracle as O  # noqa: E402


def _ori(pat, nv):
    return [-1 if (pat >> j) & 1 else 1 for j in range(nv)]


def _dual_identity_error(is_quad, pc, pe, pat):
    nv = 4 if is_quad else 3
    xy, M = O.hier_dual(is_quad, pc, list(pe), _ori(pat, nv))
    phi, _ = O.hier_shape_var(is_quad, pc, list(pe), _ori(pat, nv), xy)
    return np.abs(M @ phi - np.eye(M.shape[0])).max()


def test_tria_dual_is_the_inverse_of_the_basis():
    """fe_space_hierarchic_tests.cc:476-524 with max_p = 4 (the reference's
    debug-build range): every combination of interior and edge degrees and
    all 8 orientation patterns."""
    worst = 0.0
    for pc, p0, p1, p2 in itertools.product(range(1, 5), repeat=4):
        for pat in range(8):
            worst = max(worst, _dual_identity_error(False, pc, (p0, p1, p2), pat))
    assert worst < 1e-8, worst


def test_quad_dual_is_the_inverse_of_the_basis():
    """fe_space_hierarchic_tests.cc:526-582: all 16 orientation patterns for
    every uniform degree 1..6 and a seeded sample of mixed interior and edge
    degrees up to 6."""
    rng = np.random.default_rng(11)
    combos = [(p, (p,) * 4) for p in range(1, 7)]
    combos += [(int(r[0]), tuple(int(v) for v in r[1:])) for r in rng.integers(1, 7, (40, 5))]
    worst = 0.0
    for pc, pe in combos:
        for pat in range(16):
            worst = max(worst, _dual_identity_error(True, pc, pe, pat))
    assert worst < 1e-8, worst


def test_library_dual_tables_match_the_oracle():
    """lfg_hier_dual builds the nodes and the dual matrix in its own way
    (vertex and edge rows from the segment dual, the quadrilateral interior as
    an outer product of two segment duals, the triangle's face rows
    orthogonalised as F - (F Phi_b^T) M_b); nodes and matrices agree with the
    oracle's functional NodalValuesToDofs applied to unit vectors."""
    L = pytest.importorskip("lehrfempp_gb300")
    try:
        L.lib()
    except Exception as e:  # pragma: no cover - the library is built by build()
        pytest.skip("library not built: %s" % e)
    rng = np.random.default_rng(5)
    cases = []
    for is_quad in (False, True):
        nv = 4 if is_quad else 3
        for p in (1, 2, 3, 4, 6, 9):
            cases += [(is_quad, p, (p,) * nv, pat) for pat in range(1 << nv)]
        for r in rng.integers(1, 9, (24, 1 + nv)):
            cases.append((is_quad, int(r[0]), tuple(int(v) for v in r[1:]), int(rng.integers(0, 1 << nv))))
    for is_quad, pc, pe, pat in cases:
        nv = 4 if is_quad else 3
        xo, Mo = O.hier_dual(is_quad, pc, list(pe), _ori(pat, nv))
        xl, Ml = L.hier_dual(is_quad, pc, list(pe), pat)
        assert xl.shape == xo.shape and Ml.shape == Mo.shape, (is_quad, pc, pe, pat)
        assert np.abs(xl - xo).max() <= 1e-15, (is_quad, pc, pe, pat)
        assert np.abs(Ml - Mo).max() <= 1e-13 * max(1.0, np.abs(Mo).max()), (is_quad, pc, pe, pat)


@pytest.mark.parametrize("is_quad", [False, True])
@pytest.mark.parametrize("p", [12, 16, 20])
def test_library_dual_at_high_degree(is_quad, p):
    """Degrees up to the library's limit of 20 (a triangle of 231 and a
    quadrilateral of 441 local dofs): nodes and dual matrix agree with the
    oracle, and the library's dual inverts the basis evaluated by the oracle
    at its nodes (M phi = I within 1e-10)."""
    L = pytest.importorskip("lehrfempp_gb300")
    try:
        L.lib()
    except Exception as e:  # pragma: no cover
        pytest.skip("library not built: %s" % e)
    nv = 4 if is_quad else 3
    for pat in (0, (1 << nv) - 1, 5):
        xo, Mo = O.hier_dual(is_quad, p, [p] * nv, _ori(pat, nv))
        xl, Ml = L.hier_dual(is_quad, p, [p] * nv, pat)
        assert np.abs(xl - xo).max() <= 1e-15
        assert np.abs(Ml - Mo).max() <= 1e-13 * max(1.0, np.abs(Mo).max())
        phi, _ = O.hier_shape_var(is_quad, p, [p] * nv, _ori(pat, nv), xl)
        assert np.abs(Ml @ phi - np.eye(Ml.shape[0])).max() < 1e-10, (p, pat)


def test_library_dual_rejects_bad_arguments():
    L = pytest.importorskip("lehrfempp_gb300")
    try:
        L.lib()
    except Exception as e:  # pragma: no cover
        pytest.skip("library not built: %s" % e)
    for is_quad, pc, pe, pat in ((False, 0, (1, 1, 1), 0), (False, 21, (2, 2, 2), 0), (False, 2, (2, 0, 2), 0),
                                 (False, 2, (2, 2, 2), 8), (True, 2, (2, 2, 2, 21), 0), (True, 2, (2, 2, 2, 2), 16)):
        with pytest.raises(L.LfgError) as e:
            L.hier_dual(is_quad, pc, pe, pat)
        assert e.value.code == L.INVALID_ARG


# ------------------------------------------------------------ NodalProjection

def _mesh(kind):
    if kind == "hybrid":
        sys.path.insert(0, os.path.dirname(HERE))
        from lehrfempp_gb300 import workloads as W
        xy, cells = W.hybrid_mesh(4, seed=3)
        return O.Mesh(xy, cells, None)
    if kind == "test0":
        xy, cells, pe = O.factory_input("test0", x0=1.0)
    else:
        xy, cells, pe = O.factory_input(kind, 4, 3)
    return O.Mesh(xy, cells, pe)


def _cell_degrees(m, c, quad, p, ed, cd, ce):
    nv = 4 if quad else 3
    if ed is None:
        return p, [p] * nv
    return int(cd[c]), [int(ed[ce[c, j]]) for j in range(nv)]


def _l2_error(m, s, uh, u, qdeg, p=0, ed=None, cd=None):
    """sqrt(int (u - u_h)^2) over the mesh (straight-sided cells), u_h from
    the hierarchic shape functions of each cell's own degrees."""
    dofs = s.cell_dofs()
    _, ce, co, _ = m.topology()
    err = 0.0
    for c in range(m.num_cells):
        quad = m.cells[c, 3] >= 0
        pc, pe = _cell_degrees(m, c, quad, p, ed, cd, ce)
        x, y, w = O.quad_rule(quad, qdeg)
        phi, _ = O.hier_shape_var(quad, pc, pe, list(co[c]), np.stack([x, y], 1))
        v = m.xy[m.cells[c, :4 if quad else 3]]
        if quad:
            b = np.stack([(1 - x) * (1 - y), x * (1 - y), x * y, (1 - x) * y], 1)
            j00 = (v[1, 0] - v[0, 0]) * (1 - y) + (v[2, 0] - v[3, 0]) * y
            j10 = (v[1, 1] - v[0, 1]) * (1 - y) + (v[2, 1] - v[3, 1]) * y
            j01 = (v[3, 0] - v[0, 0]) * (1 - x) + (v[2, 0] - v[1, 0]) * x
            j11 = (v[3, 1] - v[0, 1]) * (1 - x) + (v[2, 1] - v[1, 1]) * x
            det = np.abs(j00 * j11 - j10 * j01)
        else:
            b = np.stack([1 - x - y, x, y], 1)
            det = abs((v[1, 0] - v[0, 0]) * (v[2, 1] - v[0, 1]) - (v[1, 1] - v[0, 1]) * (v[2, 0] - v[0, 0]))
        X = b @ v
        d = phi @ uh[dofs[c, :phi.shape[1]]] - u(X[:, 0], X[:, 1])
        err += float((w * det * d * d).sum())
    return math.sqrt(err)


def _poly(total_degree, seed):
    """Random global polynomial of the given total degree (<= 3), as the
    analytic POLY family sum p[4i+j] x^i y^j and as a Python function."""
    rng = np.random.default_rng(seed)
    prm = np.zeros(16)
    for i in range(4):
        for j in range(4):
            if i + j <= total_degree:
                prm[4 * i + j] = rng.uniform(-1, 1)
    return prm, (lambda X, Y: sum(prm[4 * i + j] * X ** i * Y ** j for i in range(4) for j in range(4)))


@pytest.mark.parametrize("kind", ["tptriag", "tpquad", "hybrid", "test0"])
@pytest.mark.parametrize("p", [1, 2, 3, 4, 6])
def test_projection_reproduces_the_polynomials_of_the_space(kind, p):
    """Every global polynomial of total degree <= p lies in the hierarchic
    space of degree p on straight-sided cells, so NodalProjection returns it."""
    m = _mesh(kind)
    s = O.hier_space(m, p)
    prm, u = _poly(min(p, 3), 17 * p + len(kind))
    uh = O.nodal_projection_hier(s, p, O.coeff(O.ANALYTIC, func=O.FN_POLY, params=list(prm)))
    ref = _l2_error(m, s, np.zeros_like(uh), u, 2 * p + 2, p=p)
    assert _l2_error(m, s, uh, u, 2 * p + 2, p=p) <= 1e-12 * ref


def test_projection_converges_for_a_smooth_function():
    m = _mesh("hybrid")
    errs = []
    for p in (2, 4, 6, 8):
        s = O.hier_space(m, p)
        prm = [0.0, 1.0, 1.0, 1.0]
        uh = O.nodal_projection_hier(s, p, O.coeff(O.ANALYTIC, func=O.FN_SINSIN, params=prm))
        errs.append(_l2_error(m, s, uh, lambda X, Y: np.sin(np.pi * X) * np.sin(np.pi * Y), 2 * p + 2, p=p))
    assert all(b < a / 8 for a, b in zip(errs, errs[1:])), errs
    assert errs[-1] < 1e-6, errs


def test_projection_with_a_cell_predicate():
    """Dofs of no selected cell stay 0; every other dof has the value of the
    full projection (a shared dof is set by the last selected cell)."""
    m = _mesh("test0")
    p = 4
    s = O.hier_space(m, p)
    u = O.coeff(O.ANALYTIC, func=O.FN_SINCOS, params=[0.5, 1.0, 1.0, 0.5])
    full = O.nodal_projection_hier(s, p, u)
    flags = (np.arange(m.num_cells) % 2).astype(np.uint8)
    part = O.nodal_projection_hier(s, p, u, flags)
    dofs = s.cell_dofs()
    touched = np.zeros(s.num_dofs, bool)
    for c in np.nonzero(flags)[0]:
        n = s.n_quad if m.cells[c, 3] >= 0 else s.n_tria
        touched[dofs[c, :n]] = True
    assert np.all(part[~touched] == 0.0)
    assert np.abs(part[touched] - full[touched]).max() <= 1e-13 * np.abs(full).max()


def test_var_degree_projection():
    """Per-entity degrees (2..5 drawn per edge and cell): quadratics are
    reproduced; with every degree equal to p the projection is the uniform
    space's, value for value."""
    m = _mesh("hybrid")
    rng = np.random.default_rng(9)
    ed = rng.integers(2, 6, m.num_edges).astype(np.int32)
    cd = rng.integers(2, 6, m.num_cells).astype(np.int32)
    s = O.hier_var_space(m, ed, cd)
    prm, u = _poly(2, 3)
    uh = O.nodal_projection_hier(s, 0, O.coeff(O.ANALYTIC, func=O.FN_POLY, params=list(prm)))
    ref = _l2_error(m, s, np.zeros_like(uh), u, 12, ed=ed, cd=cd)
    assert _l2_error(m, s, uh, u, 12, ed=ed, cd=cd) <= 1e-12 * ref
    p = 3
    sv = O.hier_var_space(m, np.full(m.num_edges, p, np.int32), np.full(m.num_cells, p, np.int32))
    su = O.hier_space(m, p)
    f = O.coeff(O.ANALYTIC, func=O.FN_SINSIN, params=[0.0, 1.0, 1.0, 2.0])
    assert np.array_equal(O.nodal_projection_hier(sv, 0, f), O.nodal_projection_hier(su, p, f))


# ------------------------------------------------- IntegrateMeshFunction

def _integrals(m, s, uh, u, gu, qdeg, p=0, ed=None, cd=None):
    """(int u_h + u, int (u_h - u)^2, int |grad u_h - grad u|^2) over the
    mesh by NumPy: the cell's hierarchic shape functions at the rule points,
    the element map and its inverse transpose."""
    dofs = s.cell_dofs()
    _, ce, co, _ = m.topology()
    r = np.zeros(3)
    for c in range(m.num_cells):
        quad = m.cells[c, 3] >= 0
        pc, pe = _cell_degrees(m, c, quad, p, ed, cd, ce)
        x, y, w = O.quad_rule(quad, qdeg)
        phi, dphi = O.hier_shape_var(quad, pc, pe, list(co[c]), np.stack([x, y], 1))
        v = m.xy[m.cells[c, :4 if quad else 3]]
        if quad:
            b = np.stack([(1 - x) * (1 - y), x * (1 - y), x * y, (1 - x) * y], 1)
            j00 = (v[1, 0] - v[0, 0]) * (1 - y) + (v[2, 0] - v[3, 0]) * y
            j10 = (v[1, 1] - v[0, 1]) * (1 - y) + (v[2, 1] - v[3, 1]) * y
            j01 = (v[3, 0] - v[0, 0]) * (1 - x) + (v[2, 0] - v[1, 0]) * x
            j11 = (v[3, 1] - v[0, 1]) * (1 - x) + (v[2, 1] - v[1, 1]) * x
        else:
            b = np.stack([1 - x - y, x, y], 1)
            one = np.ones_like(x)
            j00, j01 = (v[1, 0] - v[0, 0]) * one, (v[2, 0] - v[0, 0]) * one
            j10, j11 = (v[1, 1] - v[0, 1]) * one, (v[2, 1] - v[0, 1]) * one
        det = j00 * j11 - j10 * j01
        X = b @ v
        d = uh[dofs[c, :phi.shape[1]]]
        hv = phi @ d
        ghx, ghy = dphi[:, :, 0] @ d, dphi[:, :, 1] @ d
        gx = (j11 * ghx - j10 * ghy) / det  # J^-T grad_hat
        gy = (-j01 * ghx + j00 * ghy) / det
        uv = u(X[:, 0], X[:, 1])
        ux, uy = gu(X[:, 0], X[:, 1])
        wd = w * np.abs(det)
        r += [np.sum(wd * (hv + uv)), np.sum(wd * (hv - uv) ** 2), np.sum(wd * ((gx - ux) ** 2 + (gy - uy) ** 2))]
    return r


def _sinsin():
    prm = [0.3, 1.0, 1.0, 2.0]
    u = lambda X, Y: 0.3 + np.sin(np.pi * X) * np.sin(2 * np.pi * Y)
    gu = lambda X, Y: (np.pi * np.cos(np.pi * X) * np.sin(2 * np.pi * Y),
                       2 * np.pi * np.sin(np.pi * X) * np.cos(2 * np.pi * Y))
    return O.coeff(O.ANALYTIC, func=O.FN_SINSIN, params=prm), u, gu


@pytest.mark.parametrize("kind", ["tptriag", "tpquad", "hybrid", "test0"])
@pytest.mark.parametrize("p", [1, 3, 5])
def test_integrate_with_hierarchic_uh(kind, p):
    """IntegrateMeshFunction (fe/fe_tools.h:110-165) of u_h + u, (u_h - u)^2
    and |grad u_h - grad u|^2 with u_h a random dof vector of the hierarchic
    space (MeshFunctionFE / MeshFunctionGradFE of it), against NumPy."""
    m = _mesh(kind)
    s = O.hier_space(m, p)
    uh = np.random.default_rng(p + len(kind)).standard_normal(s.num_dofs)
    cf, u, gu = _sinsin()
    qdeg = 2 * p + 2
    ref = _integrals(m, s, uh, u, gu, qdeg, p=p)
    for k in range(3):
        got = O.integrate_hier(s, p, k, cf, uh, qdeg)
        assert abs(got - ref[k]) <= 1e-12 * max(1.0, abs(ref[k])), (k, got, ref[k])


def test_integrate_with_hierarchic_uh_var_degrees():
    m = _mesh("hybrid")
    rng = np.random.default_rng(12)
    ed = rng.integers(1, 6, m.num_edges).astype(np.int32)
    cd = rng.integers(1, 6, m.num_cells).astype(np.int32)
    s = O.hier_var_space(m, ed, cd)
    uh = rng.standard_normal(s.num_dofs)
    cf, u, gu = _sinsin()
    ref = _integrals(m, s, uh, u, gu, 12, ed=ed, cd=cd)
    for k in range(3):
        got = O.integrate_hier(s, 0, k, cf, uh, 12)
        assert abs(got - ref[k]) <= 1e-12 * max(1.0, abs(ref[k])), (k, got, ref[k])
