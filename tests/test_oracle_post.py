"""Pin the oracle's post-processing restatement (CPU only).

IntegrateMeshFunction, MeshFunctionFE / MeshFunctionGradFE, NodalProjection and
InitEssentialConditionFromFunction (lib/lf/fe/fe_tools.h:110-329) against the
values the reference's own tests hold: lib/lf/fe/test/fe_tools_tests.cc and
lib/lf/uscalfe/test/gfe_tests.cc (values in tests/golden/reference_goldens.json).
"""
import math
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
import oracle as O  # noqa: E402

from helpers import poly  # noqa: E402

F32_EQ = 4 * 2.0 ** -23   # EXPECT_FLOAT_EQ: 4 ulp in binary32 (relative)
F64_EQ = 4 * 2.0 ** -52   # EXPECT_DOUBLE_EQ


def mesh0(scale=1.0):
    xy, cells, _ = O.factory_input("test0", x0=scale)
    return O.Mesh(xy, cells)


def mesh3(goldens):
    t = goldens["test_mesh_3"]
    cells = np.full((len(t["triangles"]), 4), -1, np.int64)
    cells[:, :3] = t["triangles"]
    return O.Mesh(np.array(t["nodes"], float), cells)


def analytic(fn, params):
    return O.coeff(O.ANALYTIC, func=fn, params=list(params))


def trig(lin=(1.0, 0.0, 0.0, 0.0), ax=(1.0, 0.0), ay=(0.0, 0.5)):
    """(l0 + l1 x + l2 y + l3 xy) sin(pi (ax0 x + ax1)) sin(pi (ay0 y + ay1))."""
    return analytic(O.FN_TRIG, [0.0, *lin, *ax, *ay])


def test_conical_rule_exactness():
    """make_quad_rule.cc:139-152 rule (degree 0 and beyond the tables, which
    end at 50): monomials up to the degree exactly."""
    for degree in (0, 51, 56, 64):
        x, y, w = O.quad_rule(False, degree)
        assert len(w) == (degree // 2 + 1) ** 2
        for a in range(degree + 1):
            for b in range(degree + 1 - a):
                exact = math.factorial(a) * math.factorial(b) / math.factorial(a + b + 2)
                assert abs((w * x ** a * y ** b).sum() - exact) <= 2e-15 * max(exact, 1e-3)


def test_integrate_mesh_function_kat(goldens):
    """fe_tools_tests.cc:44-85 on test mesh 0 ([0,3]^2, hybrid)."""
    kat = goldens["integrate_mesh_function_kat"]["integrals"]
    m = mesh0()
    s = O.Space(m, 1)

    def integral(u, deg):
        return O.integrate(s, O.INT_VALUE, u, qdeg=deg)

    cases = [
        ("intScalar", trig(lin=(0, 0, 1, 0)), 20),                        # sin(pi x) y
        ("intVec[0]", analytic(O.FN_POLY, poly(x1=1.0)), 20),
        ("intVec[1]", analytic(O.FN_POLY, poly(x1y1=1.0)), 20),
        ("intMatrixDyn(0, 0)", analytic(O.FN_POLY, poly(c=1.0)), 10),
        ("intMatrixDyn(0, 1)", analytic(O.FN_POLY, poly(x1=1.0)), 10),
        ("intMatrixDyn(0, 2)", analytic(O.FN_POLY, poly(y1=1.0)), 10),
        ("intMatrixDyn(1, 0)", analytic(O.FN_POLY, poly(x1y1=1.0)), 10),
        ("intMatrixDyn(1, 1)", analytic(O.FN_POLY, poly(x2=1.0)), 10),
        ("intMatrixDyn(1, 2)", analytic(O.FN_POLY, poly(y2=1.0)), 10),
    ]
    for key, u, deg in cases:
        want = kat[key]["value"]
        got = integral(u, deg)
        assert abs(got - want) <= F32_EQ * abs(want), (key, got, want)
    # intVec[2]: cos(pi x) integrates to < 1e-10
    assert integral(trig(ax=(1.0, 0.5)), 20) < 1e-10


def test_gfe_l2_norms(goldens):
    """gfe_tests.cc:27-45 and 141-160 on test mesh 3 with degree-4 rules."""
    kat = goldens["gfe_norm_kat"]
    m = mesh3(goldens)
    s = O.Space(m, 1)
    u = analytic(O.FN_POLY, poly(x1=1.0, x1y1=-1.0))  # x (1 - y)
    n1 = math.sqrt(O.integrate(s, O.INT_SQ_DIFF, u, qdeg=4))
    assert abs(n1 - kat["l2norm_x_1my"]["value"]) < kat["l2norm_x_1my"]["tolerance"]
    # |(y, -x)|^2 = |grad(x y)|^2
    n2 = math.sqrt(O.integrate(s, O.INT_GRAD_SQ_DIFF, analytic(O.FN_POLY, poly(x1y1=1.0)), qdeg=4))
    assert abs(n2 - kat["l2norm_vf_y_mx"]["value"]) < kat["l2norm_vf_y_mx"]["tolerance"]


@pytest.mark.parametrize("degree", [1, 2, 3])
def test_gfe_norms_two_ways(goldens, degree):
    """gfe_tests.cc:47-139: c^T M c = int u_h^2 and c^T A c = int |grad u_h|^2."""
    for m in (mesh3(goldens), mesh0()):
        s = O.Space(m, degree)
        c = np.random.default_rng(7 + degree).uniform(-1, 1, s.num_dofs)
        for alpha, gamma, kind in ((0.0, 1.0, O.INT_SQ_DIFF), (1.0, 0.0, O.INT_GRAD_SQ_DIFF)):
            A = O.assemble_rd(s, O.coeff(O.CONSTANT, alpha), O.coeff(O.CONSTANT, gamma), 2 * degree, 2 * degree)
            r, cc, v = A.arrays()
            quad = np.zeros(s.num_dofs)
            np.add.at(quad, r, v * c[cc])
            from_a = float(c @ quad)
            direct = O.integrate(s, kind, None, dofs=c, qdeg=2 * degree)
            assert abs(from_a - direct) <= 1e-12 * abs(from_a), (degree, kind, from_a, direct)


def test_lintp_values():
    """gfe_tests.cc:162-188: NodalProjection of exp(x (1 - y)) equals u at the nodes."""
    m = mesh0()
    s = O.Space(m, 1)
    u = analytic(O.FN_EXP, [0.0, 1.0, 0.0, 1.0, 0.0, -1.0])
    v = O.nodal_projection_mf(s, u)
    cod, idx = s.dof_entities()
    xy = m.xy
    for j in range(s.num_dofs):
        assert cod[j] == 2
        x, y = xy[idx[j]]
        want = math.exp(x * (1.0 - y))
        assert abs(v[j] - want) <= F64_EQ * abs(want)


def test_nodal_projection_kat():
    """fe_tools_tests.cc:87-128: exp(x y) on test mesh 0 scaled by 1/3."""
    m = mesh0(1.0 / 3.0)
    s = O.Space(m, 1)
    v = O.nodal_projection_mf(s, analytic(O.FN_EXP, [0.0, 1.0, 0.0, 0.0, 0.0, 1.0]))
    cod, idx = s.dof_entities()
    for j in range(s.num_dofs):
        x, y = m.xy[idx[j]]
        assert abs(v[j] - math.exp(x * y)) <= F32_EQ * math.exp(x * y)


def test_set_dirbdc():
    """gfe_tests.cc:190-236: InitEssentialConditionFromFunction with g = x^2 + y^2."""
    m = mesh0()
    s = O.Space(m, 1)
    _, ef = m.boundary_flags()
    nf, _ = m.boundary_flags()
    fl, val = O.init_essential_condition(s, ef, analytic(O.FN_POLY, poly(x2=1.0, y2=1.0)))
    cod, idx = s.dof_entities()
    for j in range(s.num_dofs):
        x, y = m.xy[idx[j]]
        assert bool(fl[j]) == bool(nf[idx[j]])
        if fl[j]:
            assert abs(val[j] - (x * x + y * y)) <= F64_EQ * (x * x + y * y)
        else:
            assert val[j] == 0.0


@pytest.mark.parametrize("degree", [1, 2, 3])
def test_interpolation_exact(degree):
    """gfe_tests.cc:238-262 (linear, O1) widened: O_p reproduces degree-p polynomials."""
    m = mesh0()
    s = O.Space(m, degree)
    p = {1: poly(x1=1.0, y1=-2.0), 2: poly(x2=1.0, x1y1=-0.5, y1=1.0, c=0.25),
         3: poly(x3=0.1, y3=-0.2, x1y2=0.3, x1=1.0)}[degree]
    # on a bilinear quadrilateral a physical P_p polynomial is in Q_p of the
    # reference coordinates, so the quads of test mesh 0 reproduce it too
    u = analytic(O.FN_POLY, p)
    c = O.nodal_projection_mf(s, u)
    assert O.integrate(s, O.INT_SQ_DIFF, u, dofs=c, qdeg=8) < 1e-24
    assert O.integrate(s, O.INT_GRAD_SQ_DIFF, u, dofs=c, qdeg=8) < 1e-22


def test_first_entity_always_counted():
    """fe_tools.h:117-124 starts the sum with entity 0 whatever the predicate says."""
    m = mesh0()
    s = O.Space(m, 1)
    one = O.coeff(O.CONSTANT, 1.0)
    none = np.zeros(m.num_cells, np.uint8)
    area0 = O.integrate(s, O.INT_VALUE, one, qdeg=1, flags=none)
    assert area0 > 0
    only0 = none.copy()
    only0[0] = 1
    assert O.integrate(s, O.INT_VALUE, one, qdeg=1, flags=only0) == area0
    assert abs(O.integrate(s, O.INT_VALUE, one, qdeg=1) - 9.0) < 1e-14
    # edges: the boundary of [0,3]^2 has length 12; edge 0 is interior and
    # still counted
    _, ef = m.boundary_flags()
    en, _, _, _ = m.topology()
    assert ef[0] == 0
    len0 = float(np.hypot(*(m.xy[en[0, 1]] - m.xy[en[0, 0]])))
    assert abs(O.integrate(s, O.INT_VALUE, one, qdeg=1, flags=ef, codim=1) - (12.0 + len0)) < 1e-14


def test_per_cell_projection_last_cell_wins():
    """NodalProjection sets (not adds): a shared dof keeps the last cell's value."""
    m = mesh0()
    s = O.Space(m, 2)
    vals = np.arange(1.0, m.num_cells + 1.0)
    v = O.nodal_projection_mf(s, O.coeff(O.PER_CELL, data=vals))
    last = np.zeros(s.num_dofs)
    for c, dofs in enumerate(s.cell_dofs()):
        n = s.n_quad if m.cells[c, 3] >= 0 else s.n_tria
        last[dofs[:n]] = vals[c]
    assert np.array_equal(v, last)


def test_analytic_gradients_converge():
    """The hand-written gradients of the analytic families: the H1-seminorm
    interpolation error of O2 falls like h^2 (a wrong gradient would stall)."""
    fams = [(O.FN_POLY, poly(x3=0.5, x1y2=-1.0, y1=2.0, c=1.0)), (O.FN_SINSIN, [0.5, 2.0, 1.0, 2.0]),
            (O.FN_SINCOS, [0.0, 1.0, 1.5, 0.5]), (O.FN_EXP, [0.1, 0.7, 0.2, 0.3, -0.4, 0.5]),
            (O.FN_TRIG, [0.2, 1.0, 0.5, -0.3, 0.2, 1.0, 0.25, 0.5, 0.1])]
    spaces = []
    for n in (6, 12):
        xy, cells, pe = O.factory_input("tptriag", n, n)
        m = O.Mesh(xy, cells, pe)
        spaces.append((m, O.Space(m, 2)))
    for fn, prm in fams:
        u = analytic(fn, prm)
        errs = []
        for m, s in spaces:
            c = O.nodal_projection_mf(s, u)
            errs.append(math.sqrt(O.integrate(s, O.INT_GRAD_SQ_DIFF, u, dofs=c, qdeg=6)))
        assert errs[0] > 0 and 3.2 < errs[0] / errs[1] < 4.8, (fn, errs)
