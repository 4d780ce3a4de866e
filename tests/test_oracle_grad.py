"""The oracle's FP64 reference gradient (no GPU): central differences of J
through exact SparseLU solves, with zero and nonzero Dirichlet data."""
import numpy as np
import pytest

from parity import O, W


def _fd_check(space, theta, u_obs, flags, g, cells, h=1e-6):
    f = O.coeff(O.CONSTANT, 1.0)
    _, _, _, grad = O.adjoint_gradient(space, theta, f, u_obs, flags, g)
    worst = 0.0
    for c in cells:
        tp, tm = theta.copy(), theta.copy()
        tp[c] += h
        tm[c] -= h
        fd = (O.adjoint_gradient(space, tp, f, u_obs, flags, g)[0] -
              O.adjoint_gradient(space, tm, f, u_obs, flags, g)[0]) / (2 * h)
        worst = max(worst, abs(fd - grad[c]))
    return worst / np.abs(grad).max()


def test_oracle_gradient_central_differences_tptriag_o1():
    xy, cells, pe = O.factory_input("tptriag", 8, 8)
    sp = O.Space(O.Mesh(xy, cells, pe), 1)
    rng = np.random.default_rng(1)
    theta = 0.5 * rng.standard_normal(len(cells))
    u_obs = 0.05 * rng.standard_normal(sp.num_dofs)
    err = _fd_check(sp, theta, u_obs, sp.boundary_dof_flags(), None, rng.choice(len(cells), 16, replace=False))
    assert err <= 1e-6, err


@pytest.mark.parametrize("degree", [1, 2, 3])
def test_oracle_gradient_central_differences_hybrid_dirichlet(degree):
    xy, cells = W.hybrid_mesh(4, seed=3)
    sp = O.Space(O.Mesh(xy, cells), degree)
    rng = np.random.default_rng(2)
    theta = 0.5 * rng.standard_normal(len(cells))
    flags = sp.boundary_dof_flags()
    g = np.where(flags != 0, 0.1 * rng.standard_normal(sp.num_dofs), 0.0)
    u_obs = 0.05 * rng.standard_normal(sp.num_dofs)
    err = _fd_check(sp, theta, u_obs, flags, g, rng.choice(len(cells), 8, replace=False))
    assert err <= 1e-6, err


def test_oracle_gradient_is_bilinear_form_of_element_matrices():
    """dJ/dtheta_c sums to -lambda^T A u over free rows (A unfixed)."""
    xy, cells, pe = O.factory_input("tptriag", 6, 5)
    sp = O.Space(O.Mesh(xy, cells, pe), 2)
    rng = np.random.default_rng(4)
    theta = 0.4 * rng.standard_normal(len(cells))
    flags = sp.boundary_dof_flags()
    u_obs = rng.standard_normal(sp.num_dofs) * 0.01
    J, u, lam, grad = O.adjoint_gradient(sp, theta, O.coeff(O.CONSTANT, 1.0), u_obs, flags)
    A = O.assemble_rd(sp, O.coeff(O.PER_CELL_EXP, data=theta), O.coeff(O.ZERO)).to_scipy()
    lm = np.where(flags != 0, 0.0, lam)
    assert abs(grad.sum() + lm @ (A @ u)) <= 1e-12 * np.abs(grad).sum()
