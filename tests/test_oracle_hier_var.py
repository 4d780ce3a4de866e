"""Variable-degree hierarchic FE in the oracle (CPU):
HierarchicScalarFESpace(mesh, degree_functor) (fe/hierarchic_scalar_fe_space.h:
93-116, 178-220) with degrees per edge and per cell, numbered like
DynamicFEDofHandler (assemble/dofhandler.h:550-680).

- uniform degrees given per entity reproduce the uniform space exactly;
- the shape functions of a cell with interior degree pc and edge degrees pe
  are the uniform degree-D functions (D = max(pc, pe, 1)) at the slots of
  `sel_map` (the selection the device kernels use), bit for bit;
- a random FE function is continuous across interior edges (the variable
  counterpart of fe_space_hierarchic_tests.cc:166-423);
- the reference's own varying-degree continuity test (its degree pattern,
  edge traces against the segment functions, fe_space_hierarchic_tests.cc:
  166-247);
- the L2 projection onto a space whose degrees are all >= 2 reproduces a
  quadratic exactly (a known answer pinning numbering, functions and rules);
- constants are in the kernel of the stiffness matrix and the vertex block of
  the mass matrix sums to the area."""
import os
import sys

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
import oracle as O  # noqa: E402
from test_oracle_hier import _ref_edge_points, mesh0  # noqa: E402


def sel_map(quad, D, pc, pe, ori):
    """Uniform degree-D slot of every local slot of a cell with interior degree
    pc, edge degrees pe and relative edge orientations ori (+1 / -1)."""
    nv = 4 if quad else 3
    out = list(range(nv))
    for j in range(nv):
        k = pe[j] - 1
        ub = nv + j * (D - 1)
        for s in range(k):
            out.append(ub + s if ori[j] > 0 else ub + (D - 1 - k) + s)
    ib = nv + nv * (D - 1)
    if quad:
        for i in range(pc - 1):
            for j in range(pc - 1):
                out.append(ib + i * (D - 1) + j)
    else:
        for i in range(pc - 2):
            for j in range(pc - 2 - i):
                out.append(ib + i * (D - 2) - i * (i - 1) // 2 + j)
    return np.array(out, np.int64)


def var_degrees(m, lo, hi, seed):
    rng = np.random.default_rng(seed)
    return rng.integers(lo, hi + 1, m.num_edges), rng.integers(lo, hi + 1, m.num_cells)


def cell_degrees(m, c, ed, cd):
    _, ce, co, _ = m.topology()
    nv = 4 if m.cells[c, 3] >= 0 else 3
    pe = [int(ed[ce[c, j]]) for j in range(nv)]
    return int(cd[c]), pe, list(co[c])


@pytest.mark.parametrize("p", [1, 2, 3, 5])
def test_uniform_degrees_reproduce_the_uniform_space(p):
    m = mesh0()
    su = O.hier_space(m, p)
    sv = O.hier_var_space(m, np.full(m.num_edges, p), np.full(m.num_cells, p))
    assert sv.num_dofs == su.num_dofs
    nl = sv.local_counts()
    du, dv = su.cell_dofs(), sv.cell_dofs()
    for c in range(m.num_cells):
        assert np.array_equal(du[c, :nl[c]], dv[c, :nl[c]])
    assert np.array_equal(su.dof_entities()[0], sv.dof_entities()[0])
    a = O.coeff(O.ANALYTIC, func=O.FN_POLY, params=[1, 0.5, 0, 0, 0.25])
    g = O.coeff(O.CONSTANT, 0.7)
    ru, cu, vu = O.assemble_hier(su, p, a, g).arrays()
    rv, cv, vv = O.assemble_hier(sv, 0, a, g).arrays()
    assert np.array_equal(ru, rv) and np.array_equal(cu, cv) and np.array_equal(vu, vv)
    f = O.coeff(O.ANALYTIC, func=O.FN_SINSIN, params=[1.5, 0.5, 1.0, 2.0])
    assert np.array_equal(O.assemble_hier_load(su, p, f), O.assemble_hier_load(sv, 0, f))


@pytest.mark.parametrize("quad", [False, True])
def test_variable_shapes_are_a_selection_of_the_uniform_ones(quad):
    rng = np.random.default_rng(5 + quad)
    pts = rng.random((7, 2))
    if not quad:
        pts = pts[pts.sum(1) < 1]
    nv = 4 if quad else 3
    for _ in range(60):
        pc = int(rng.integers(1, 8))
        pe = [int(v) for v in rng.integers(1, 8, nv)]
        ori = [int(v) for v in rng.choice([-1, 1], nv)]
        D = max([pc, 1] + pe)
        phi_v, dphi_v = O.hier_shape_var(quad, pc, pe, ori, pts)
        phi_u, dphi_u = O.hier_shape(quad, D, ori, pts)
        s = sel_map(quad, D, pc, pe, ori)
        assert phi_v.shape[1] == len(s)
        assert np.array_equal(phi_v, phi_u[:, s]) and np.array_equal(dphi_v, dphi_u[:, s, :])


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_variable_space_is_continuous_across_edges(seed):
    m = mesh0()
    ed, cd = var_degrees(m, 1, 6, seed)
    s = O.hier_var_space(m, ed, cd)
    dofs, nl = s.cell_dofs(), s.local_counts()
    _, ce, co, nc = m.topology()
    u = np.random.default_rng(seed).standard_normal(s.num_dofs)
    t = np.array([0.1, 0.35, 0.8])
    for e in range(m.num_edges):
        if nc[e] != 2:
            continue
        vals = []
        for c in range(m.num_cells):
            quad = m.cells[c, 3] >= 0
            for j in range(4 if quad else 3):
                if ce[c, j] != e:
                    continue
                tt = t if co[c, j] > 0 else 1 - t
                pc, pe, ori = cell_degrees(m, c, ed, cd)
                phi, _ = O.hier_shape_var(quad, pc, pe, ori, _ref_edge_points(quad, j, tt))
                vals.append(phi @ u[dofs[c, :nl[c]]])
        assert len(vals) == 2
        assert np.abs(vals[0] - vals[1]).max() < 1e-10, e


def test_edge_traces_with_the_reference_degree_pattern():
    """fe_space_hierarchic_tests.cc:166-247 with its own degree assignment: one
    counter runs over the cells and then over the edges, and entity k gets
    degree k % 2 + 2 (nodes degree 1).  For every local edge i of every cell,
    at p + 1 equispaced points (p = 1..10) along the edge in the edge's own
    direction, the cell's shape functions of that edge equal the segment's
    interior functions ILegendre(r + 2, t) (FeHierarchicSegment,
    hierarchic_fe.h:297-310); on a negatively oriented edge the cell's slots
    run backwards.  Tolerance 1e-10, as in the reference test."""
    m = mesh0()
    k = np.arange(m.num_cells + m.num_edges) % 2 + 2
    cd, ed = k[: m.num_cells], k[m.num_cells:]
    s = O.hier_var_space(m, ed, cd)
    nl = s.local_counts()
    checked = 0
    for p in range(1, 11):
        t = np.linspace(0.0, 1.0, p + 1)
        seg = np.array([[O.hier_fn(1, r + 2, 1.0, 0.0, x) for x in t] for r in range(int(ed.max()) - 1)])
        for c in range(m.num_cells):
            quad = m.cells[c, 3] >= 0
            nv = 4 if quad else 3
            pc, pe, ori = cell_degrees(m, c, ed, cd)
            nint = (pc - 1) ** 2 if quad else max(0, (pc - 2) * (pc - 1) // 2)
            assert nl[c] == nv + sum(d - 1 for d in pe) + nint
            off = nv
            for i in range(nv):
                tt = t if ori[i] > 0 else 1.0 - t
                phi, _ = O.hier_shape_var(quad, pc, pe, ori, _ref_edge_points(quad, i, tt))
                ke = pe[i] - 1
                for r in range(ke):
                    slot = off + r if ori[i] > 0 else off + ke - 1 - r
                    assert np.abs(phi[:, slot] - seg[r]).max() < 1e-10, (p, c, i, r)
                    checked += 1
                off += ke
    assert checked > 0


def test_dof_numbering_follows_dynamic_dof_handler():
    """Node dofs, then edge_deg[e] - 1 dofs per edge in edge order, then the
    cell interiors in cell order; a cell lists its vertices, its edges' dofs
    (reversed on a negatively oriented edge) and its interior."""
    m = mesh0()
    ed, cd = var_degrees(m, 1, 5, 11)
    s = O.hier_var_space(m, ed, cd)
    nv, ne = m.num_nodes, m.num_edges
    _, ce, co, _ = m.topology()
    efirst = nv + np.concatenate([[0], np.cumsum(ed - 1)])
    nint = [(cd[c] - 1) ** 2 if m.cells[c, 3] >= 0 else max(0, (cd[c] - 2) * (cd[c] - 1) // 2)
            for c in range(m.num_cells)]
    cfirst = efirst[ne] + np.concatenate([[0], np.cumsum(nint)])
    assert s.num_dofs == cfirst[-1]
    dofs, nl = s.cell_dofs(), s.local_counts()
    for c in range(m.num_cells):
        k = 4 if m.cells[c, 3] >= 0 else 3
        row = list(m.cells[c, :k])
        for j in range(k):
            e = ce[c, j]
            ids = list(range(efirst[e], efirst[e + 1]))
            row += ids if co[c, j] > 0 else ids[::-1]
        row += list(range(cfirst[c], cfirst[c + 1]))
        assert nl[c] == len(row) and list(dofs[c, :nl[c]]) == row, c
    cod, idx = s.dof_entities()
    assert (cod[:nv] == 2).all() and (cod[nv:efirst[ne]] == 1).all() and (cod[efirst[ne]:] == 0).all()


@pytest.mark.parametrize("seed", [3, 4])
def test_mass_projection_of_a_quadratic_is_exact(seed):
    m = mesh0()
    ed, cd = var_degrees(m, 2, 5, seed)
    s = O.hier_var_space(m, ed, cd)
    A = O.assemble_hier(s, 0, O.coeff(O.ZERO), O.coeff(O.CONSTANT, 1.0), qdeg=14)
    prm = np.zeros(16)
    prm[0], prm[1], prm[4], prm[5], prm[8] = 0.3, -0.7, 1.1, 0.9, -0.4  # 0.3 - 0.7 y + 1.1 x + 0.9 xy - 0.4 x^2
    f = O.coeff(O.ANALYTIC, func=O.FN_POLY, params=list(prm))
    b = O.assemble_hier_load(s, 0, f, qdeg=14)
    r, c, v = A.arrays()
    M = sp.csr_matrix((v, (r, c)), shape=(s.num_dofs, s.num_dofs))
    x = spla.spsolve(M.tocsc(), b)
    u = lambda X, Y: 0.3 - 0.7 * Y + 1.1 * X + 0.9 * X * Y - 0.4 * X * X  # noqa: E731
    dofs, nl = s.cell_dofs(), s.local_counts()
    err = 0.0
    for cc in range(m.num_cells):
        quad = m.cells[cc, 3] >= 0
        xq, yq, w = O.quad_rule(quad, 10)
        pc, pe, ori = cell_degrees(m, cc, ed, cd)
        phi, _ = O.hier_shape_var(quad, pc, pe, ori, np.stack([xq, yq], 1))
        vv = m.xy[m.cells[cc, :4 if quad else 3]]
        bb = np.stack([(1 - xq) * (1 - yq), xq * (1 - yq), xq * yq, (1 - xq) * yq], 1) if quad else \
            np.stack([1 - xq - yq, xq, yq], 1)
        X = bb @ vv
        err = max(err, float(np.abs(phi @ x[dofs[cc, :nl[cc]]] - u(X[:, 0], X[:, 1])).max()))
    assert err < 1e-10, err


def test_constants_and_area():
    m = mesh0()
    ed, cd = var_degrees(m, 1, 6, 9)
    s = O.hier_var_space(m, ed, cd)
    K = O.assemble_hier(s, 0, O.coeff(O.CONSTANT, 1.0), O.coeff(O.ZERO))
    r, c, v = K.arrays()
    Ks = sp.csr_matrix((v, (r, c)), shape=(s.num_dofs, s.num_dofs))
    one = np.zeros(s.num_dofs)
    one[:m.num_nodes] = 1.0  # the vertex functions sum to 1
    assert np.abs(Ks @ one).max() < 1e-11
    M = O.assemble_hier(s, 0, O.coeff(O.ZERO), O.coeff(O.CONSTANT, 1.0))
    r, c, v = M.arrays()
    Ms = sp.csr_matrix((v, (r, c)), shape=(s.num_dofs, s.num_dofs))
    area = 0.0
    for cc in range(m.num_cells):
        quad = m.cells[cc, 3] >= 0
        P = m.xy[m.cells[cc, :4 if quad else 3]]
        area += 0.5 * abs(np.dot(P[:, 0], np.roll(P[:, 1], -1)) - np.dot(P[:, 1], np.roll(P[:, 0], -1)))
    assert abs(one @ (Ms @ one) - area) < 1e-12 * area


def test_degree_checks():
    m = mesh0()
    with pytest.raises(RuntimeError):
        O.hier_var_space(m, np.zeros(m.num_edges, np.int32), np.ones(m.num_cells, np.int32))
    with pytest.raises(RuntimeError):
        O.hier_var_space(m, np.ones(m.num_edges, np.int32), np.zeros(m.num_cells, np.int32))
