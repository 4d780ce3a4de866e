"""Pin the oracle against the reference's own golden values (CPU only).

Each test restates a LehrFEM++ unit test for this path and checks the oracle
(the CPU restatement in oracle/) against the numbers that test holds.
"""
import math
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import oracle as O  # noqa: E402

from helpers import dense, edge_dof_assembler_matrices, poly, cell_index_matrices  # noqa: E402


def test_mesh0_numbering():
    # assembly_tests.cc:159-161: 9 cells, 18 edges, 10 nodes
    xy, cells, _ = O.factory_input("test0", x0=1.0)
    m = O.Mesh(xy, cells)
    assert (m.num_nodes, m.num_edges, m.num_cells) == (10, 18, 9)
    en, ce, co, nc = m.topology()
    # every cell edge really joins the cell's local vertices j, j+1
    for c in range(9):
        nv = 3 if cells[c, 3] < 0 else 4
        for j in range(nv):
            a, b = cells[c, j], cells[c, (j + 1) % nv]
            e = ce[c, j]
            assert sorted(en[e]) == sorted([a, b])
            assert co[c, j] == (1 if en[e][0] == a else -1)
    # no preset edges: numbered in (min, max) lexicographic order
    keys = [tuple(sorted(e)) for e in en]
    assert keys == sorted(keys)


def test_mat_assembly_ref10(goldens):
    """lf_assembly.mat_assembly_test (assembly_tests.cc:219-300)."""
    ref = np.array(goldens["mat_assembly_test_ref10"]["matrix"])
    xy, cells, _ = O.factory_input("test0", x0=1.0)
    m = O.Mesh(xy, cells)
    s = O.Space(m, 0, (1, 0, 0, 0))
    assert s.num_dofs == 10
    cod, ent = s.dof_entities()
    assert (cod == 2).all()
    e, v = cell_index_matrices(m.num_cells)
    A, b = O.assemble_tabulated(s, e, v)
    D = dense(10, 10, *A.arrays())
    assert np.array_equal(D, ref[np.ix_(ent, ent)])
    assert np.array_equal(b, np.diag(ref)[ent])
    # makeSparse path gives the same matrix
    assert np.array_equal(A.to_scipy().toarray(), D)


def test_edge_dof_ref36(goldens):
    """lf_assembly.edge_dof_static (assembly_tests.cc:302-488)."""
    ref = np.array(goldens["edge_dof_static_ref36"]["matrix"])
    xy, cells, _ = O.factory_input("test0", x0=1.0)
    m = O.Mesh(xy, cells)
    s = O.Space(m, 0, (0, 2, 0, 0))
    assert s.num_dofs == 36
    cod, _ = s.dof_entities()
    assert (cod == 1).all()
    A, _ = O.assemble_tabulated(s, edge_dof_assembler_matrices(m.num_cells))
    assert np.array_equal(dense(36, 36, *A.arrays()), ref)


def _tridiag_coo():
    N = 10
    r, c, v = [], [], []
    for k in range(N):
        if k > 0:
            r.append(k); c.append(k - 1); v.append(-1.0)
        if k < N - 1:
            r.append(k); c.append(k + 1); v.append(-1.0)
        r.append(k); c.append(k); v.append(2.0)
    return O.COO.from_arrays(N, N, r, c, v), np.arange(1, N + 1, dtype=np.float64)


@pytest.mark.parametrize("alt", [False, True])
def test_fix_dof_exact_solution(goldens, alt):
    """fix_dof_flags / fix_dof_flags_alt (coomatrix_tests.cc:126-239)."""
    import scipy.sparse.linalg as spla
    g = goldens["fix_dof_exact"]
    A, b = _tridiag_coo()
    flags = np.zeros(10, np.uint8)
    vals = np.ones(10)
    for k, val in g["fixed"]:
        flags[k] = 1
        vals[k] = val
    A.fix_flagged(flags, vals, b, alt=alt)
    x = spla.splu(A.to_scipy().tocsc()).solve(b)
    assert np.linalg.norm(x - np.array(g["solution"])) < g["tolerance"]


def test_fix_lse_exact_solution(goldens):
    """fix_dof_test (coomatrix_tests.cc:77-121): FixSolutionComponentsLse with
    {2: -1}, {4: -2}, {8: -3}, then a direct solve, meets the exact solution."""
    import scipy.sparse.linalg as spla
    g = goldens["fix_dof_exact"]
    A, b = _tridiag_coo()
    dofs, vals = zip(*g["fixed"])
    A.fix_lse(list(dofs), list(vals), b)
    x = spla.splu(A.to_scipy().tocsc()).solve(b)
    assert np.linalg.norm(x - np.array(g["solution"])) < g["tolerance"]


def test_fix_lse_accumulates_repeated_dofs():
    """fix_dof.h:266-272: `fixed_vec[idx] += value` -- a dof listed twice is
    fixed to the sum of its values, and only fixed rows are removed (CompAlt)."""
    A1, b1 = _tridiag_coo()
    A1.fix_lse([8, 2, 4, 8], [-1.0, -1.0, -2.0, -2.0], b1)
    A2, b2 = _tridiag_coo()
    flags = np.zeros(10, np.uint8)
    flags[[2, 4, 8]] = 1
    vals = np.zeros(10)
    vals[[2, 4, 8]] = [-1.0, -2.0, -3.0]
    A2.fix_flagged(flags, vals, b2, alt=True)
    assert np.array_equal(b1, b2)
    for u, v in zip(A1.arrays(), A2.arrays()):
        assert np.array_equal(u, v)
    with pytest.raises(RuntimeError):
        A1.fix_lse([10], [1.0], b1)


def test_fix_preserves_order_and_appends_diagonal():
    A, b = _tridiag_coo()
    r0, c0, v0 = A.arrays()
    flags = np.zeros(10, np.uint8)
    flags[[2, 4, 8]] = 1
    A.fix_flagged(flags, np.zeros(10), b)
    r, c, v = A.arrays()
    keep = ~(flags[r0].astype(bool) | flags[c0].astype(bool))
    n = keep.sum()
    assert np.array_equal(r[:n], r0[keep]) and np.array_equal(c[:n], c0[keep]) and np.array_equal(v[:n], v0[keep])
    assert list(r[n:]) == [2, 4, 8] and list(c[n:]) == [2, 4, 8] and list(v[n:]) == [1.0, 1.0, 1.0]


def test_kat_tensor_o1(goldens):
    """lf_fe_linear.ReactionDiffusion (lagr_fe_tests.cc:807-832)."""
    k = goldens["reaction_diffusion_kat"]
    assert abs(O.kat_tensor_rd() - k["O1_tensor_deg4"]["value"]) < k["tolerance"]


def test_tensor_coefficient_kinds():
    """The oracle's matrix-valued coefficient kinds: the bilinear-entry kind
    reproduces the tensor known answer exactly, and constant / per-cell kinds
    agree with it where the tensor is the same everywhere."""
    xy, cells, _ = O.factory_input("test0", x0=1.0)
    s = O.Space(O.Mesh(xy, cells), 1)
    tensor = [1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1]  # [[1, x], [y, x y]]
    A = O.assemble_rd(s, O.coeff(O.TENSOR_BILINEAR, params=tensor),
                      O.coeff(O.ANALYTIC, func=O.FN_POLY, params=list(poly(x1y1=1))), 4, 4).to_scipy()
    av = O.nodal_projection(s, O.FN_POLY, poly(c=1, x1=1, y1=2))
    bv = O.nodal_projection(s, O.FN_POLY, poly(x1=3))
    assert abs(av @ (A @ bv) - O.kat_tensor_rd()) <= 1e-13 * O.kat_tensor_rd()
    c = [2.0, 0.3, -0.2, 1.5]
    A1 = O.assemble_rd(s, O.coeff(O.TENSOR_CONSTANT, params=c), O.coeff(O.ZERO)).to_scipy()
    A2 = O.assemble_rd(s, O.coeff(O.TENSOR_PER_CELL, data=np.tile(c, s.mesh.num_cells)), O.coeff(O.ZERO)).to_scipy()
    p = [c[0], 0, 0, 0, c[1], 0, 0, 0, c[2], 0, 0, 0, c[3], 0, 0, 0]
    A3 = O.assemble_rd(s, O.coeff(O.TENSOR_BILINEAR, params=p), O.coeff(O.ZERO)).to_scipy()
    assert (A1 != A2).nnz == 0 and (A1 != A3).nnz == 0
    # a symmetric tensor alpha I gives the scalar coefficient's matrix
    As = O.assemble_rd(s, O.coeff(O.CONSTANT, 1.7), O.coeff(O.ZERO)).to_scipy()
    At = O.assemble_rd(s, O.coeff(O.TENSOR_CONSTANT, params=[1.7, 0, 0, 1.7]), O.coeff(O.ZERO)).to_scipy()
    assert abs(As - At).max() <= 1e-14 * abs(As).max()


@pytest.mark.parametrize("degree,alpha,gamma,a,b,qdeg,key", [
    (2, poly(x1=1), poly(x1y1=1), poly(x2=1, y2=1), poly(x2=1, y2=-1), 6, "O2_deg6"),
    (3, poly(y1=1), poly(x1y1=1), poly(x3=1, y3=1), poly(x1y2=1), 8, "O3_deg8"),
])
def test_kat_reaction_diffusion(goldens, degree, alpha, gamma, a, b, qdeg, key):
    """lf_fe_quadratic/cubic.ReactionDiffusion (lagr_fe_tests.cc:834-883)."""
    k = goldens["reaction_diffusion_kat"]
    xy, cells, _ = O.factory_input("test0", x0=1.0)
    m = O.Mesh(xy, cells)
    s = O.Space(m, degree)
    A = O.assemble_rd(s, O.coeff(O.ANALYTIC, func=O.FN_POLY, params=alpha),
                      O.coeff(O.ANALYTIC, func=O.FN_POLY, params=gamma), qdeg, qdeg)
    av = O.nodal_projection(s, O.FN_POLY, a)
    bv = O.nodal_projection(s, O.FN_POLY, b)
    val = av @ (A.to_scipy() @ bv)
    assert abs(val - k[key]["value"]) < k["tolerance"]


@pytest.mark.parametrize("degree", [1, 2, 3])
@pytest.mark.parametrize("quad", [False, True])
def test_volume_row_sums(degree, quad):
    """loc_comp_products_test (lagr_fe_tests.cc:892-992): mass matrix sums to
    the cell volume, stiffness rows sum to zero."""
    kind = "tpquad" if quad else "tptriag"
    xy, cells, pe = O.factory_input(kind, 3, 2, 0.0, 0.0, 1.5, 1.0)
    m = O.Mesh(xy, cells, pe)
    s = O.Space(m, degree)
    M = O.assemble_rd(s, O.coeff(O.ZERO), O.coeff(O.CONSTANT, 1.0)).to_scipy()
    assert abs(M.sum() - 1.5) < 1e-12
    K = O.assemble_rd(s, O.coeff(O.CONSTANT, 1.0), O.coeff(O.ZERO)).to_scipy()
    assert np.abs(np.asarray(K.sum(axis=1))).max() < 1e-12
    f = O.assemble_load(s, O.coeff(O.CONSTANT, 1.0))
    assert abs(f.sum() - 1.5) < 1e-12


@pytest.mark.parametrize("degree", list(range(0, 51)) + [51, 60])
def test_tria_rule_exactness(degree):
    """make_quad_rule_tests.cc:107-136: monomials up to the degree exactly
    (the reference's tables up to 50, the conical rule beyond)."""
    x, y, w = O.quad_rule(False, degree)
    for a in range(degree + 1):
        for b in range(degree + 1 - a):
            exact = math.factorial(a) * math.factorial(b) / math.factorial(a + b + 2)
            assert abs(math.fsum(w * x ** a * y ** b) - exact) < 2e-15, (a, b)


def _rule_digest(x, y, w):
    import hashlib
    return hashlib.sha256(np.stack([x, y, w], 1).astype("<f8").tobytes()).hexdigest()


@pytest.mark.parametrize("degree", [d for d in range(1, 51) if d != 3])
def test_tria_rules_equal_reference_tables(goldens, degree):
    """Every tabulated triangle rule of quad_rules_tria.cc (degrees 1..50),
    point for point and bit for bit, in the oracle and in the library (host
    query, no GPU)."""
    import lehrfempp_gb300 as L
    ref = goldens["tria_rules"]["degrees"][str(degree)]
    for name, (x, y, w) in (("oracle", O.quad_rule(False, degree)), ("library", L.quad_rule(False, degree))):
        assert len(w) == ref["points"], name
        assert [x[0], y[0], w[0]] == [float(v) for v in ref["first"]], name
        assert _rule_digest(x, y, w) == ref["sha256_xyw_le"], name
    # degree 3 is served by the degree-4 table (make_quad_rule.cc:44-46)
    if degree == 4:
        assert _rule_digest(*O.quad_rule(False, 3)) == ref["sha256_xyw_le"]
        assert _rule_digest(*L.quad_rule(False, 3)) == ref["sha256_xyw_le"]


@pytest.mark.parametrize("degree", [0, 1, 7, 20, 51, 64, 100])
def test_library_rules_equal_oracle_rules(degree):
    """Quadrilateral rules and the conical triangle rule beyond the tables:
    the library's host rules and the oracle's agree to the last bits."""
    import lehrfempp_gb300 as L
    for quad in (False, True):
        xo, yo, wo = O.quad_rule(quad, degree)
        xl, yl, wl = L.quad_rule(quad, degree)
        assert len(wo) == len(wl)
        for a, b in ((xo, xl), (yo, yl), (wo, wl)):
            assert np.abs(a - b).max() <= 4e-16 * max(1.0, np.abs(a).max()), (quad, degree)


@pytest.mark.parametrize("degree", range(1, 12))
def test_quad_rule_exactness(degree):
    x, y, w = O.quad_rule(True, degree)
    assert len(w) == (degree // 2 + 1) ** 2
    for a in range(degree + 1):
        for b in range(degree + 1):
            assert abs((w * x ** a * y ** b).sum() - 1.0 / ((a + 1) * (b + 1))) < 1e-14


def test_gauss_legendre_closed_form():
    x, _, w = O.quad_rule(True, 4)  # n = 3 per direction
    xs = x[::3]
    r = math.sqrt(3.0 / 5.0) / 2
    assert np.allclose(xs, [0.5 - r, 0.5, 0.5 + r], rtol=0, atol=1e-16)
    assert np.allclose(w[:3], np.array([5, 8, 5]) / 18 * 5 / 18, rtol=0, atol=1e-16)


def test_tptriag_numbering():
    """TPTriagMeshBuilder pre-registers every edge: edge index = registration order."""
    xy, cells, pe = O.factory_input("tptriag", 3, 2)
    m = O.Mesh(xy, cells, pe)
    en, _, _, nc = m.topology()
    assert np.array_equal(en, pe)
    assert m.num_edges == 3 * 3 * 2 + 2 * 3 + 2 * 2 - 3 - 2 + 1 or m.num_edges == len(pe)
    assert m.num_cells == 12 and m.num_nodes == 12
    nf, ef = m.boundary_flags()
    assert nf.sum() == 10 and ef.sum() == 10


def test_missing_rule_raises():
    """lf_uscalfe.missingQuadRule (loc_comp_test.cc:154-183): Eval throws."""
    xy, cells, _ = O.factory_input("test0", x0=1.0)
    m = O.Mesh(xy, cells)
    s = O.Space(m, 1)
    with pytest.raises(RuntimeError, match="No local shape function"):
        O.assemble_rd(s, O.coeff(O.CONSTANT, 1.0), O.coeff(O.ZERO), 2, -1)


def test_incomplete_mesh_rejected():
    xy = np.array([[0, 0], [1, 0], [0, 1], [5, 5]], float)
    with pytest.raises(RuntimeError, match="incomplete"):
        O.Mesh(xy, np.array([[0, 1, 2, -1]]))


def test_edge_providers_known_answers():
    """lagr_fe_tests.cc:571-601 and 696-722 (lf_fe_edgemass, lf_fe_edgeload):
    O1 on the hybrid test mesh, gamma = g = 1, every edge:
    A_e = |e| [[1/3, 1/6], [1/6, 1/3]] and phi_e = |e| [1/2, 1/2]."""
    xy, cells, pe = O.factory_input("test0")
    m = O.Mesh(xy, cells, pe)
    sp = O.Space(m, 1)
    r, c, v = O.assemble_edge_mass(sp, O.coeff(O.CONSTANT, 1.0)).arrays()
    en = m.topology()[0]
    le = np.hypot(*(m.xy[en[:, 1]] - m.xy[en[:, 0]]).T)
    assert np.abs(v - (le[:, None] * np.array([1 / 3, 1 / 6, 1 / 6, 1 / 3])).ravel()).max() < 1e-15
    b = O.assemble_edge_load(sp, O.coeff(O.CONSTANT, 1.0))
    ref = np.zeros(sp.num_dofs)
    np.add.at(ref, en[:, 0], 0.5 * le)
    np.add.at(ref, en[:, 1], 0.5 * le)
    assert np.abs(b - ref).max() < 1e-14
    # flags select edges; the load accumulates onto the given vector
    fl = (np.arange(m.num_edges) % 2).astype(np.uint8)
    r2, c2, v2 = O.assemble_edge_mass(sp, O.coeff(O.CONSTANT, 1.0), fl).arrays()
    assert len(v2) == 4 * int(fl.sum())
    b2 = O.assemble_edge_load(sp, O.coeff(O.CONSTANT, 1.0), fl, b=np.ones(sp.num_dofs))
    assert b2.min() >= 1.0
