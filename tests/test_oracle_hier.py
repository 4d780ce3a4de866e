"""Hierarchic (hp) FE in the oracle (CPU): the reference's own tests of
lib/lf/fe/test/fe_space_hierarchic_tests.cc (Legendre orthogonality, derivative
identities by central differences, gradients of the shape functions,
continuity across edges) and the degree-15 Poisson / L2-projection solves of
lib/lf/fe/test/loc_comp_tests.cc:47-204 (L2 error below 1e-5 on test mesh 0)."""
import math
import os
import sys

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
import oracle as O  # noqa: E402

EPS = math.sqrt(np.finfo(float).eps)


def _fd_close(approx, exact):
    return abs(approx - exact) < 1e-5 if abs(exact) < 100 else abs(approx / exact - 1) < 1e-5


def test_legendre_orthogonality():
    """fe_space_hierarchic_tests.cc:21-44."""
    for n in range(20):
        for m in range(20):
            t, w = np.polynomial.legendre.leggauss((n + m) // 2 + 1)
            x, w = 0.5 * (t + 1), 0.5 * w
            r = sum(wi * O.hier_fn(0, n, 1.0, 0, xi) * O.hier_fn(0, m, 1.0, 0, xi) for xi, wi in zip(x, w))
            assert abs(r - (1.0 / (2 * n + 1) if n == m else 0.0)) < 1e-8


def test_integrated_legendre_and_jacobi_derivatives():
    """fe_space_hierarchic_tests.cc:46-162 (central differences, 101 points)."""
    xs = np.linspace(0, 1, 101)
    for p in range(20):
        for x in xs:
            exact = O.hier_fn(0, p, 1.0, 0, x)
            approx = (O.hier_fn(1, p + 1, 1.0, 0, x + EPS / 2) - O.hier_fn(1, p + 1, 1.0, 0, x - EPS / 2)) / EPS
            assert _fd_close(approx, exact), (p, x)
        for alpha in (1, 4, 9):
            for x in xs[::5]:
                exact = O.hier_fn(4, p, alpha, 0.0, x)
                approx = (O.hier_fn(5, p + 1, alpha, 0, x + EPS / 2) - O.hier_fn(5, p + 1, alpha, 0, x - EPS / 2)) / EPS
                assert _fd_close(approx, exact), (p, alpha, x)


def test_integrated_jacobi_is_the_integral_from_zero():
    """IJacobi(n, a, x) = int_0^x Jacobi(n-1, a, s) ds, the definition the
    library's own construction uses."""
    for n in range(1, 14):
        for alpha in (4.0, 8.0, 12.0):
            for x in (0.0, 0.25, 0.6, 1.0):
                t, w = np.polynomial.legendre.leggauss(16)
                s, ws = 0.5 * x * (t + 1), 0.5 * x * w
                integral = sum(wi * O.hier_fn(4, n - 1, alpha, 0.0, si) for si, wi in zip(s, ws))
                val = O.hier_fn(5, n, alpha, 0, x)
                assert abs(val - integral) <= 1e-12 * max(1.0, abs(integral)), (n, alpha, x)


@pytest.mark.parametrize("quad", [False, True])
def test_shape_gradients_central_differences(quad):
    """grad_tria / grad_quad (fe_space_hierarchic_tests.cc:612-800), every
    orientation pattern, degrees 1..8."""
    rng = np.random.default_rng(3)
    pts = rng.uniform(0.05, 0.45, (4, 2))
    for p in range(1, 9):
        for pat in range(16 if quad else 8):
            ori = [-1 if (pat >> j) & 1 else 1 for j in range(4)]
            phi, dphi = O.hier_shape(quad, p, ori, pts)
            px, _ = O.hier_shape(quad, p, ori, pts + [EPS / 2, 0])
            mx, _ = O.hier_shape(quad, p, ori, pts - [EPS / 2, 0])
            py, _ = O.hier_shape(quad, p, ori, pts + [0, EPS / 2])
            my, _ = O.hier_shape(quad, p, ori, pts - [0, EPS / 2])
            assert np.abs((px - mx) / EPS - dphi[:, :, 0]).max() < 1e-5 * max(1, np.abs(dphi).max())
            assert np.abs((py - my) / EPS - dphi[:, :, 1]).max() < 1e-5 * max(1, np.abs(dphi).max())


def _ref_edge_points(quad, j, t):
    """Reference coordinates of the points at parameters t along local edge j (v_j -> v_{j+1})."""
    V = np.array([[0, 0], [1, 0], [1, 1], [0, 1]] if quad else [[0, 0], [1, 0], [0, 1]], float)
    a, b = V[j], V[(j + 1) % len(V)]
    return a[None, :] + t[:, None] * (b - a)[None, :]


def mesh0():
    xy, cells, _ = O.factory_input("test0", x0=1.0)
    return O.Mesh(xy, cells)


@pytest.mark.parametrize("p", [1, 2, 3, 4, 6])
def test_continuity_across_edges(p):
    """continuity (fe_space_hierarchic_tests.cc:166-423): a random FE
    function takes the same values on an interior edge from both sides."""
    m = mesh0()
    s = O.hier_space(m, p)
    dofs = s.cell_dofs()
    en, ce, co, nc = m.topology()
    u = np.random.default_rng(p).standard_normal(s.num_dofs)
    t = np.array([0.1, 0.35, 0.8])
    for e in range(m.num_edges):
        if nc[e] != 2:
            continue
        vals = []
        for c in range(m.num_cells):
            quad = m.cells[c, 3] >= 0
            nloc = (p + 1) ** 2 if quad else (p + 1) * (p + 2) // 2
            for j in range(4 if quad else 3):
                if ce[c, j] != e:
                    continue
                # parameter along the edge's own direction
                tt = t if co[c, j] > 0 else 1 - t
                phi, _ = O.hier_shape(quad, p, list(co[c]), _ref_edge_points(quad, j, tt))
                vals.append(phi @ u[dofs[c, :nloc]])
        assert len(vals) == 2
        assert np.abs(vals[0] - vals[1]).max() < 1e-10, e


def fe_l2_error(m, s, p, uh, u, qdeg):
    """sqrt(int (u - u_h)^2) with hierarchic u_h (Python loop over cells)."""
    dofs = s.cell_dofs()
    _, _, co, _ = m.topology()
    err = 0.0
    for c in range(m.num_cells):
        quad = m.cells[c, 3] >= 0
        x, y, w = O.quad_rule(quad, qdeg)
        phi, _ = O.hier_shape(quad, p, list(co[c]), np.stack([x, y], 1))
        nloc = phi.shape[1]
        v = m.xy[m.cells[c, :4 if quad else 3]]
        if quad:
            b = np.stack([(1 - x) * (1 - y), x * (1 - y), x * y, (1 - x) * y], 1)
            X = b @ v
            j00 = (v[1, 0] - v[0, 0]) * (1 - y) + (v[2, 0] - v[3, 0]) * y
            j10 = (v[1, 1] - v[0, 1]) * (1 - y) + (v[2, 1] - v[3, 1]) * y
            j01 = (v[3, 0] - v[0, 0]) * (1 - x) + (v[2, 0] - v[1, 0]) * x
            j11 = (v[3, 1] - v[0, 1]) * (1 - x) + (v[2, 1] - v[1, 1]) * x
            det = np.abs(j00 * j11 - j10 * j01)
        else:
            b = np.stack([1 - x - y, x, y], 1)
            X = b @ v
            det = abs((v[1, 0] - v[0, 0]) * (v[2, 1] - v[0, 1]) - (v[1, 1] - v[0, 1]) * (v[2, 0] - v[0, 0]))
        d = phi @ uh[dofs[c, :nloc]] - u(X[:, 0], X[:, 1])
        err += float((w * det * d * d).sum())
    return math.sqrt(err)


def _solve_fixed(s, A, b, m):
    nf, ef = m.boundary_flags()
    cod, idx = s.dof_entities()
    flags = np.zeros(s.num_dofs, np.uint8)
    flags[cod == 2] = nf[idx[cod == 2]]
    flags[cod == 1] = ef[idx[cod == 1]]
    A.fix_flagged(flags, np.zeros(s.num_dofs), b)
    r, c, v = A.arrays()
    M = sp.csr_matrix((v, (r, c)), shape=(s.num_dofs, s.num_dofs))
    return spla.spsolve(M.tocsc(), b)


@pytest.mark.parametrize("mass", [False, True])
def test_degree15_solves_on_test_mesh0(mass):
    """lf_fe.diffusion_mat_test / mass_mat_test (loc_comp_tests.cc:47-204):
    degree 15, u = sin(pi x) sin(pi y), L2 error < 1e-5."""
    p = 15
    m = mesh0()
    s = O.hier_space(m, p)
    alpha, gamma = (O.coeff(O.ZERO), O.coeff(O.CONSTANT, 1.0)) if mass else (O.coeff(O.CONSTANT, 1.0),
                                                                             O.coeff(O.ZERO))
    A = O.assemble_hier(s, p, alpha, gamma)
    f = O.coeff(O.ANALYTIC, func=O.FN_SINSIN, params=[0.0, 2 * math.pi ** 2, 1.0, 1.0])
    b = O.assemble_hier_load(s, p, f)
    x = _solve_fixed(s, A, b, m)
    scale = 2 * math.pi ** 2 if mass else 1.0
    err = fe_l2_error(m, s, p, x, lambda X, Y: scale * np.sin(np.pi * X) * np.sin(np.pi * Y), 2 * p - 1)
    assert err < 1e-5, err


@pytest.mark.parametrize("p", [2, 3, 4, 5])
def test_mass_projection_reproduces_polynomials(p):
    """The hierarchic space of degree p contains P_p on triangles and Q_p-mapped
    polynomials on the bilinear quads: the L2 projection of x^a y^b with
    a + b = p is exact (no boundary conditions)."""
    m = mesh0()
    s = O.hier_space(m, p)
    A = O.assemble_hier(s, p, O.coeff(O.ZERO), O.coeff(O.CONSTANT, 1.0), qdeg=2 * p + 2)
    prm = np.zeros(16)
    prm[4 * min(p, 3) + (p - min(p, 3))] = 1.0  # x^min(p,3) y^(p - min(p,3))
    f = O.coeff(O.ANALYTIC, func=O.FN_POLY, params=list(prm))
    b = O.assemble_hier_load(s, p, f, qdeg=2 * p + 2)
    r, c, v = A.arrays()
    M = sp.csr_matrix((v, (r, c)), shape=(s.num_dofs, s.num_dofs))
    x = spla.spsolve(M.tocsc(), b)
    a = min(p, 3)
    err = fe_l2_error(m, s, p, x, lambda X, Y: X ** a * Y ** (p - a), 2 * p + 2)
    assert err < 1e-10, err
