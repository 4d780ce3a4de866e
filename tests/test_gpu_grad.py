"""Differentiation form (GPU): cellwise adjoint gradient, misfit loss and the
forward/backward Function object, against the oracle's FP64 reference
gradient (element matrices + two SparseLU solves) and central differences."""
import ctypes as C

import numpy as np
import pytest

from parity import O, L, W, oracle_mesh

pytestmark = pytest.mark.gpu

GRAD_RTOL = 1e-12  # kernel vs oracle on the same u, lambda: per cell, of sum |lam_i A_ij u_j|


def _spaces(ctx, spec, degree):
    mesh = W.build_mesh(ctx, spec)
    return mesh, L.Space.lagrange(mesh, degree), O.Space(oracle_mesh(spec), degree)


def _hybrid(n, seed=3):
    xy, cells = W.hybrid_mesh(n, seed=seed)
    return {"kind": "factory", "xy": xy, "cells": cells, "edges": None}


CASES = [
    ("tptriag_o1", {"kind": "tptriag", "nx": 9, "ny": 7}, 1),
    ("tptriag_o2", {"kind": "tptriag", "nx": 6, "ny": 5}, 2),
    ("tptriag_o3", {"kind": "tptriag", "nx": 5, "ny": 4}, 3),
    ("tpquad_o2", {"kind": "tpquad", "nx": 5, "ny": 6}, 2),
    ("hybrid_o1", _hybrid(8), 1),
    ("hybrid_o2", _hybrid(6), 2),
    ("hybrid_o3", _hybrid(4), 3),
]


@pytest.mark.parametrize("name,spec,degree", CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize("kind", ["exp", "plain"])
def test_grad_kernel_matches_oracle_formula(ctx, name, spec, degree, kind):
    """Same (u, lambda) on both sides: the kernel's per-point form against
    -lambda^T (dA_K/dtheta) u from the oracle's assembled element matrices."""
    mesh, sp, osp = _spaces(ctx, spec, degree)
    rng = np.random.default_rng(11)
    nc, nd = mesh.num_cells, sp.num_dofs
    theta = 0.5 * rng.standard_normal(nc) if kind == "exp" else np.exp(0.5 * rng.standard_normal(nc))
    u = rng.standard_normal(nd)
    lam = rng.standard_normal(nd)
    flags = osp.boundary_dof_flags()
    okind = O.PER_CELL_EXP if kind == "exp" else O.PER_CELL
    A = O.assemble_rd(osp, O.coeff(okind, data=theta), O.coeff(O.ZERO))
    lam_m = np.where(flags != 0, 0.0, lam)
    ref = -O.cellwise_bilinear(osp, A, lam_m, u)
    if kind == "plain":
        ref = ref / theta  # dA_K/dalpha_c = A_K / alpha_c
    r, c, v = A.arrays()
    scale = np.add.reduceat(np.abs(lam_m[r] * v * u[c]), O.element_blocks(osp)[:-1])
    if kind == "plain":
        scale = scale / theta
    th_d, u_d, l_d = ctx.to_device(theta), ctx.to_device(u), ctx.to_device(lam)
    fl_d = sp.boundary_dof_flags()
    assert np.array_equal(fl_d.download(), flags)
    grad = ctx.zeros(nc)
    gkind = L.PER_CELL_EXP if kind == "exp" else L.PER_CELL
    L.grad_rd_cellwise(sp, L.rd_provider(L.coeff(gkind, data=th_d), L.coeff(L.ZERO)), u_d, l_d, fl_d, grad)
    g = grad.download()
    err = np.abs(g - ref)
    assert (err <= GRAD_RTOL * scale + 1e-300).all(), float((err / np.maximum(scale, 1e-300)).max())


def test_grad_without_flags_and_rules(ctx):
    """NULL flags = no flagged dofs; explicit rule degrees are honoured."""
    spec = _hybrid(5, seed=8)
    mesh, sp, osp = _spaces(ctx, spec, 2)
    rng = np.random.default_rng(5)
    theta = 0.3 * rng.standard_normal(mesh.num_cells)
    u, lam = rng.standard_normal(sp.num_dofs), rng.standard_normal(sp.num_dofs)
    A = O.assemble_rd(osp, O.coeff(O.PER_CELL_EXP, data=theta), O.coeff(O.ZERO), 6, 5)
    ref = -O.cellwise_bilinear(osp, A, lam, u)
    grad = ctx.zeros(mesh.num_cells)
    prov = L.rd_provider(L.coeff(L.PER_CELL_EXP, data=ctx.to_device(theta)), L.coeff(L.ZERO), 6, 5)
    L.grad_rd_cellwise(sp, prov, ctx.to_device(u), ctx.to_device(lam), None, grad)
    g = grad.download()
    assert np.abs(g - ref).max() <= 1e-12 * np.abs(ref).max()


def test_grad_rejects_non_cellwise_alpha(ctx):
    mesh, sp, _ = _spaces(ctx, {"kind": "tptriag", "nx": 3, "ny": 3}, 1)
    z = ctx.zeros(sp.num_dofs)
    with pytest.raises(L.LfgError) as e:
        L.grad_rd_cellwise(sp, L.rd_provider(L.coeff(L.CONSTANT, 1.0), L.coeff(L.ZERO)), z, z, None,
                           ctx.zeros(mesh.num_cells))
    assert e.value.code == L.UNSUPPORTED


def test_misfit_loss(ctx):
    rng = np.random.default_rng(3)
    for n in (1, 8191, 8192, 8193, 100003):
        u, uo = rng.standard_normal(n), rng.standard_normal(n)
        r = ctx.zeros(n)
        J = L.loss_l2_misfit(ctx, ctx.to_device(u), ctx.to_device(uo), r)
        ref = 0.5 * float(np.dot(u - uo, u - uo))
        assert abs(J - ref) <= 1e-13 * ref, (n, J, ref)
        assert np.array_equal(r.download(), u - uo)
    # deterministic: the same inputs give the same bits
    u, uo = ctx.to_device(rng.standard_normal(50000)), ctx.to_device(rng.standard_normal(50000))
    assert L.loss_l2_misfit(ctx, u, uo) == L.loss_l2_misfit(ctx, u, uo)
    # empty vectors: J = 0
    e = ctx.zeros(1)
    out = C.c_double(-1.0)
    ctx.check(L.lib().lfg_loss_l2_misfit(ctx.h, 0, e.ptr, e.ptr, C.byref(out), None))
    assert out.value == 0.0


# ---------------------------------------------------------- Function object

def _problem(ctx, n, degree=1, spec=None, seed=5, dirichlet=False):
    """Config-5 shape at small n: theta ~ N(0, 0.5^2); u_obs from theta_true
    (Gaussian bumps) + N(0, 1e-3^2) noise."""
    spec = spec or {"kind": "tptriag", "nx": n, "ny": n}
    mesh, sp, osp = _spaces(ctx, spec, degree)
    xy, cells = mesh.geometry()
    rng = np.random.default_rng(seed)
    theta = 0.5 * rng.standard_normal(mesh.num_cells)
    tt = W.theta_true(W.cell_centroids(xy, cells))
    flags = osp.boundary_dof_flags()
    g = np.where(flags != 0, 0.1 * np.random.default_rng(seed + 1).standard_normal(sp.num_dofs), 0.0) \
        if dirichlet else np.zeros(sp.num_dofs)
    f = O.coeff(O.CONSTANT, 1.0)
    _, u_true, _, _ = O.adjoint_gradient(osp, tt, f, np.zeros(sp.num_dofs), flags, g)
    u_obs = u_true + W.observation_noise(sp.num_dofs)
    return mesh, sp, osp, theta, u_obs, flags, g


def _function(ctx, sp, u_obs, g=None, recompute=False, rtol=1e-13):
    return L.RDAdjoint(sp, ctx.to_device(u_obs), L.load_provider(L.coeff(L.CONSTANT, 1.0)),
                       dirichlet=ctx.to_device(g) if g is not None else None, rtol=rtol, recompute=recompute)


@pytest.mark.parametrize("degree", [1, 2])
def test_function_gradient_matches_oracle(ctx, degree):
    mesh, sp, osp, theta, u_obs, flags, g = _problem(ctx, 16, degree)
    fn = _function(ctx, sp, u_obs)
    th_d = ctx.to_device(theta)
    u_d = ctx.zeros(sp.num_dofs)
    J = fn.forward(th_d, u_d)
    grad = ctx.zeros(mesh.num_cells)
    fn.backward(grad, 1.0)
    Jr, ur, lr, gr = O.adjoint_gradient(osp, theta, O.coeff(O.CONSTANT, 1.0), u_obs, flags)
    assert abs(J - Jr) <= 1e-10 * Jr
    assert np.abs(u_d.download() - ur).max() <= 1e-10 * np.abs(ur).max()
    gd = grad.download()
    assert np.abs(gd - gr).max() <= 1e-9 * np.abs(gr).max(), np.abs(gd - gr).max() / np.abs(gr).max()
    st = fn.stats()
    assert st["forward"]["converged"] and st["adjoint"]["converged"]
    # dL/dJ scales the gradient
    fn.backward(grad, -2.5)
    assert np.allclose(grad.download(), -2.5 * gd, rtol=1e-12, atol=0.0)


def test_function_gradient_matches_oracle_mid_size(ctx):
    """The inverse-conductivity workload's shape at 256 x 256 (131,072 cells,
    66,049 dofs): GPU forward + adjoint PCG + gradient kernel against the
    oracle's FP64 gradient (element matrices and two SparseLU solves)."""
    mesh, sp, osp, theta, u_obs, flags, g = _problem(ctx, 256, 1, seed=21)
    fn = _function(ctx, sp, u_obs, rtol=1e-11)
    J = fn.forward(ctx.to_device(theta))
    grad = ctx.zeros(mesh.num_cells)
    fn.backward(grad)
    Jr, _, _, gr = O.adjoint_gradient(osp, theta, O.coeff(O.CONSTANT, 1.0), u_obs, flags)
    assert abs(J - Jr) <= 1e-9 * Jr
    gd = grad.download()
    err = np.abs(gd - gr).max() / np.abs(gr).max()
    assert err <= 1e-8, err


def test_function_central_differences(ctx):
    """64 random cells, central differences with step 1e-6 through the GPU
    forward (8 x 8 mesh: the PCG solves reach rounding level)."""
    mesh, sp, osp, theta, u_obs, flags, g = _problem(ctx, 8, 1, seed=7)
    fn = _function(ctx, sp, u_obs, rtol=1e-14)
    J0 = fn.forward(ctx.to_device(theta))
    grad = ctx.zeros(mesh.num_cells)
    fn.backward(grad)
    gd = grad.download()
    h = 1e-6
    cells = np.random.default_rng(8).choice(mesh.num_cells, 64, replace=False)
    fd = []
    for c in cells:
        tp, tm = theta.copy(), theta.copy()
        tp[c] += h
        tm[c] -= h
        fd.append((fn.forward(ctx.to_device(tp)) - fn.forward(ctx.to_device(tm))) / (2 * h))
    fd = np.array(fd)
    err = np.abs(fd - gd[cells]).max() / np.abs(gd).max()
    assert J0 > 0 and err <= 1e-6, err


def test_function_dirichlet_data_central_differences(ctx):
    """Nonzero Dirichlet values on a hybrid O2 mesh: u keeps g on flagged dofs."""
    mesh, sp, osp, theta, u_obs, flags, g = _problem(ctx, 0, 2, spec=_hybrid(5, seed=4), seed=9, dirichlet=True)
    fn = _function(ctx, sp, u_obs, g=g, rtol=1e-14)
    fn.forward(ctx.to_device(theta))
    grad = ctx.zeros(mesh.num_cells)
    fn.backward(grad)
    gd = grad.download()
    _, _, _, gr = O.adjoint_gradient(osp, theta, O.coeff(O.CONSTANT, 1.0), u_obs, flags, g)
    assert np.abs(gd - gr).max() <= 1e-9 * np.abs(gr).max()
    h = 1e-6
    for c in np.random.default_rng(1).choice(mesh.num_cells, 12, replace=False):
        tp, tm = theta.copy(), theta.copy()
        tp[c] += h
        tm[c] -= h
        fd = (fn.forward(ctx.to_device(tp)) - fn.forward(ctx.to_device(tm))) / (2 * h)
        assert abs(fd - gd[c]) <= 1e-6 * np.abs(gd).max(), (c, fd, gd[c])


def test_function_recompute_mode(ctx):
    """Recompute mode keeps only theta between forward and backward and gives
    the same bits (the forward pipeline is deterministic)."""
    mesh, sp, osp, theta, u_obs, flags, g = _problem(ctx, 12, 1, seed=3)
    th_d = ctx.to_device(theta)
    out = []
    for rec in (False, True):
        fn = _function(ctx, sp, u_obs, recompute=rec)
        J = fn.forward(th_d)
        saved = fn.stats()["saved_bytes"]
        grad = ctx.zeros(mesh.num_cells)
        fn.backward(grad)
        out.append((J, saved, grad.download()))
    (J0, s0, g0), (J1, s1, g1) = out
    assert J0 == J1 and np.array_equal(g0, g1)
    assert s1 == mesh.num_cells * 8 and s0 > s1


def test_function_backward_before_forward(ctx):
    mesh, sp, _ = _spaces(ctx, {"kind": "tptriag", "nx": 3, "ny": 3}, 1)
    fn = _function(ctx, sp, np.zeros(sp.num_dofs))
    with pytest.raises(L.LfgError) as e:
        fn.backward(ctx.zeros(mesh.num_cells))
    assert e.value.code == L.INVALID_ARG
