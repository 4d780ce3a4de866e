"""Parity of the sm_103a path with the oracle, through the C-ABI (GPU only).

Indices and triplet order must be bit-exact; values within 1e-12 of the
element matrix scale (max |A_K|); solutions within 1e-8 relative of the FP64
direct solve.
"""
import numpy as np
import pytest

from helpers import cell_index_matrices, dense, edge_dof_assembler_matrices
from parity import VALUE_RTOL, O, L, W, Run, block_sizes, compare_triplets, oracle_mesh

pytestmark = pytest.mark.gpu


def _topology_equal(gm, om):
    en, ce, co, nc = gm.topology()
    oen, oce, oco, onc = om.topology()
    assert (gm.num_nodes, gm.num_edges, gm.num_cells) == (om.num_nodes, om.num_edges, om.num_cells)
    assert np.array_equal(en, oen)
    assert np.array_equal(ce, oce)
    assert np.array_equal(co, oco)
    assert np.array_equal(nc, onc)


@pytest.mark.parametrize("spec", [
    {"kind": "tptriag", "nx": 5, "ny": 3},
    {"kind": "tpquad", "nx": 4, "ny": 6},
    "test0", "hybrid",
])
def test_mesh_numbering(ctx, spec):
    if spec == "test0":
        xy, cells, _ = O.factory_input("test0", x0=1.0)
        spec = {"kind": "factory", "xy": xy, "cells": cells, "edges": None}
    elif spec == "hybrid":
        xy, cells = W.hybrid_mesh(12, seed=7)
        spec = {"kind": "factory", "xy": xy, "cells": cells, "edges": None}
    gm = W.build_mesh(ctx, spec)
    om = oracle_mesh(spec)
    _topology_equal(gm, om)
    nf, ef = gm.boundary_flags()
    onf, oef = om.boundary_flags()
    assert np.array_equal(nf, onf) and np.array_equal(ef, oef)


def test_factory_with_preset_edges(ctx):
    """Preset edges keep their registration index; the rest follow in (min,max) order."""
    xy, cells, pe = O.factory_input("tptriag", 4, 3)
    sel = pe[::3]  # register a third of the edges, in reversed direction
    sel = sel[:, ::-1].copy()
    om = O.Mesh(xy, cells, sel)
    gm = L.Mesh.from_factory(ctx, xy, cells, sel)
    _topology_equal(gm, om)


@pytest.mark.parametrize("degree", [1, 2, 3])
@pytest.mark.parametrize("which", ["tptriag", "tpquad", "hybrid"])
def test_dof_numbering(ctx, degree, which):
    if which == "hybrid":
        xy, cells = W.hybrid_mesh(9, seed=11)
        spec = {"kind": "factory", "xy": xy, "cells": cells, "edges": None}
    else:
        spec = {"kind": which, "nx": 4, "ny": 3}
    gs = L.Space.lagrange(W.build_mesh(ctx, spec), degree)
    os_ = O.Space(oracle_mesh(spec), degree)
    assert gs.num_dofs == os_.num_dofs
    assert np.array_equal(gs.cell_dofs(), os_.cell_dofs())
    cod, idx = gs.dof_entities()
    ocod, oidx = os_.dof_entities()
    assert np.array_equal(cod, ocod) and np.array_equal(idx, oidx)
    assert np.array_equal(gs.boundary_dof_flags().download(), os_.boundary_dof_flags())


def test_golden_ref10(ctx, goldens):
    """The 10x10 golden of lf_assembly.mat_assembly_test through the GPU path."""
    ref = np.array(goldens["mat_assembly_test_ref10"]["matrix"])
    xy, cells, _ = O.factory_input("test0", x0=1.0)
    m = L.Mesh.from_factory(ctx, xy, cells)
    s = L.Space.layout(m, 1, 0, 0, 0)
    e, v = cell_index_matrices(m.num_cells)
    coo = L.COOMatrix(ctx, s.num_dofs, s.num_dofs, s.num_triplets)
    L.assemble_matrix_tabulated(s, ctx.to_device(e), 4, coo)
    t = coo.triplets()
    cod, ent = s.dof_entities()
    assert np.array_equal(dense(10, 10, t["row"], t["col"], t["value"]), ref[np.ix_(ent, ent)])
    b = ctx.zeros(s.num_dofs)
    L.assemble_vector_tabulated(s, ctx.to_device(v), 4, b)
    assert np.array_equal(b.download(), np.diag(ref)[ent])
    # makeSparse on the device gives the same matrix
    assert np.array_equal(coo.make_sparse().to_scipy().toarray(), ref[np.ix_(ent, ent)])


def test_golden_ref36(ctx, goldens):
    """The 36x36 golden of lf_assembly.edge_dof_static (two dofs per edge)."""
    ref = np.array(goldens["edge_dof_static_ref36"]["matrix"])
    xy, cells, _ = O.factory_input("test0", x0=1.0)
    m = L.Mesh.from_factory(ctx, xy, cells)
    s = L.Space.layout(m, 0, 2, 0, 0)
    coo = L.COOMatrix(ctx, s.num_dofs, s.num_dofs, s.num_triplets)
    L.assemble_matrix_tabulated(s, ctx.to_device(edge_dof_assembler_matrices(m.num_cells)), 8, coo)
    t = coo.triplets()
    assert np.array_equal(dense(36, 36, t["row"], t["col"], t["value"]), ref)


WORKLOADS = {
    "c1": lambda: W.config1(64),
    "c2": lambda: W.config2(24),
    "c3": lambda: W.config3(12),
    "c5": lambda: W.config5(16),
}


@pytest.mark.parametrize("name", sorted(WORKLOADS))
def test_matrix_parity(ctx, name):
    r = Run(ctx, WORKLOADS[name]())
    coo = r.gpu_matrix()
    ro, co, vo = r.oracle_matrix().arrays()
    compare_triplets(coo.triplets(), ro, co, vo, block_sizes(r.cells(), r.space.n_tria, r.space.n_quad))


@pytest.mark.parametrize("name", sorted(WORKLOADS))
def test_vector_parity(ctx, name):
    r = Run(ctx, WORKLOADS[name]())
    b = r.gpu_vector().download()
    bo = r.oracle_vector()
    scale = np.abs(bo).max()
    assert np.abs(b - bo).max() <= 1e-12 * scale


@pytest.mark.parametrize("degree,quad", [(1, True), (2, False), (3, True), (3, False), (2, True)])
@pytest.mark.parametrize("coef", ["uniform", "varying"])
def test_matrix_parity_all_elements(ctx, degree, quad, coef):
    spec = {"kind": "tpquad" if quad else "tptriag", "nx": 5, "ny": 4}
    if coef == "uniform":
        alpha, gamma = ("const", 1.7), ("const", 0.3)
    else:
        alpha, gamma = ("poly", W.poly(c=1.0, x1y1=2.0, y2=1.0)), ("sincos", 1.0, 0.25, 2.0, 1.0)
    wl = {"mesh": spec, "degree": degree, "alpha": alpha, "gamma": gamma, "f": ("poly", W.poly(c=1.0, x1=1.0)),
          "qr_tria": 0, "qr_quad": 0}
    r = Run(ctx, wl)
    ro, co, vo = r.oracle_matrix().arrays()
    compare_triplets(r.gpu_matrix().triplets(), ro, co, vo, block_sizes(r.cells(), r.space.n_tria, r.space.n_quad))
    b = r.gpu_vector().download()
    bo = r.oracle_vector()
    assert np.abs(b - bo).max() <= 1e-12 * np.abs(bo).max()


@pytest.mark.parametrize("qdeg", [5, 9, 10])
@pytest.mark.parametrize("degree", [1, 2, 3])
def test_explicit_high_degree_tria_rules(ctx, degree, qdeg):
    """Explicit triangle rules (qr_collection, loc_comp_ellbvp.h:237-263) of
    degree 9 and 10 come from the reference's tables (19 and 25 points) for
    both the matrix and the load vector, with point-varying coefficients."""
    xy, cells = W.hybrid_mesh(6, seed=5)
    wl = {"mesh": {"kind": "factory", "xy": xy, "cells": cells, "edges": None}, "degree": degree,
          "alpha": ("sincos", 1.0, 0.5, 3.0, 2.0), "gamma": ("poly", W.poly(c=0.5, x1y1=1.0)),
          "f": ("sinsin", 0.0, 1.0, 2.0, 1.0), "qr_tria": qdeg, "qr_quad": 4}
    r = Run(ctx, wl)
    ro, co, vo = r.oracle_matrix().arrays()
    compare_triplets(r.gpu_matrix().triplets(), ro, co, vo, block_sizes(r.cells(), r.space.n_tria, r.space.n_quad))
    b = r.gpu_vector().download()
    bo = r.oracle_vector()
    assert np.abs(b - bo).max() <= 1e-12 * np.abs(bo).max()


@pytest.mark.parametrize("degree", [1, 2, 3])
def test_fp64_route_for_out_of_range_cells(ctx, degree):
    """Cells whose coefficients fall outside the df32 range (|alpha| > 2^40 or
    < 2^-40) are computed by the FP64 formula inside the same kernels."""
    xy, cells = W.hybrid_mesh(10, seed=3)
    rng = np.random.default_rng(1)
    alpha = np.exp(rng.standard_normal(len(cells)))
    alpha[::3] *= 1e14
    alpha[1::5] *= 1e-14
    gamma = np.exp(rng.standard_normal(len(cells)))
    gamma[::4] *= 1e15
    wl = {"mesh": {"kind": "factory", "xy": xy, "cells": cells, "edges": None}, "degree": degree,
          "alpha": ("cell", alpha), "gamma": ("cell", gamma), "f": ("const", 1.0), "qr_tria": 0, "qr_quad": 0}
    r = Run(ctx, wl)
    ro, co, vo = r.oracle_matrix().arrays()
    compare_triplets(r.gpu_matrix().triplets(), ro, co, vo, block_sizes(r.cells(), r.space.n_tria, r.space.n_quad))


@pytest.mark.parametrize("cfg", ["c2", "c3"])
@pytest.mark.parametrize("chunk", [0, 1000, 77777])
def test_assemble_to_host(ctx, chunk, cfg):
    """AssembleMatrixLocally into host memory: the same triplets, bit for bit,
    as the device COO -- written by the kernels straight into page-locked
    memory from lfg_host_alloc (also at an offset inside it), and through the
    ring of device buffers with overlapped downloads into pageable memory."""
    r = Run(ctx, W.config2(40) if cfg == "c2" else W.config3(24))
    ref = r.gpu_matrix().triplets()
    p = L.rd_provider(W.to_coeff(ctx, r.wl["alpha"], r.keep), W.to_coeff(ctx, r.wl["gamma"], r.keep))
    pinned = ctx.pinned((r.space.num_triplets,), L.TRIPLET_DTYPE)
    assert L.assemble_matrix_rd_to_host(r.space, p, pinned, chunk) == len(ref)
    bad = np.flatnonzero(pinned.array != ref)
    assert bad.size == 0, (bad.size, bad[:5], pinned.array[bad[:3]], ref[bad[:3]])
    wide = ctx.pinned((r.space.num_triplets + 8,), L.TRIPLET_DTYPE)
    wide.array[:] = np.zeros(1, L.TRIPLET_DTYPE)
    view = wide.array[5:]
    assert L.assemble_matrix_rd_to_host(r.space, p, view, chunk) == len(ref)
    assert np.array_equal(view[:len(ref)], ref) and not wide.array[:5]["row"].any() and not view[len(ref):]["row"].any()
    host = np.zeros(r.space.num_triplets + 5, L.TRIPLET_DTYPE)
    assert L.assemble_matrix_rd_to_host(r.space, p, host, chunk) == len(ref)
    assert np.array_equal(host[:len(ref)], ref) and not host[len(ref):]["row"].any()
    small = np.zeros(r.space.num_triplets - 1, L.TRIPLET_DTYPE)
    with pytest.raises(L.LfgError) as e:
        L.assemble_matrix_rd_to_host(r.space, p, small, chunk)
    assert e.value.code == L.CAPACITY
    with pytest.raises(L.LfgError) as e:
        L.assemble_matrix_rd_to_host(r.space, p, wide.array[10:], chunk)
    assert e.value.code == L.CAPACITY


def test_append_semantics(ctx):
    """AssembleMatrixLocally appends to the triplets already in the matrix."""
    r = Run(ctx, W.config1(8))
    coo = L.COOMatrix(ctx, r.space.num_dofs, r.space.num_dofs, 2 * r.space.num_triplets)
    p = L.rd_provider(W.to_coeff(ctx, r.wl["alpha"], r.keep), W.to_coeff(ctx, r.wl["gamma"], r.keep), 4, 4)
    L.assemble_matrix_rd(r.space, p, coo)
    L.assemble_matrix_rd(r.space, p, coo)
    t = coo.triplets()
    n = r.space.num_triplets
    assert len(t) == 2 * n and np.array_equal(t[:n], t[n:])


def test_fix_lse_parity(ctx, goldens):
    """FixSolutionComponentsLse on the device: the reference's fix_dof_test
    system, and an assembled system with repeated (dof, value) pairs against
    the oracle (b bit-exact, triplets in order)."""
    g = goldens["fix_dof_exact"]
    N = 10
    coo = L.COOMatrix(ctx, N, N, 64)
    r, c, v = [], [], []
    for k in range(N):
        if k > 0:
            r.append(k); c.append(k - 1); v.append(-1.0)
        if k < N - 1:
            r.append(k); c.append(k + 1); v.append(-1.0)
        r.append(k); c.append(k); v.append(2.0)
    coo.append(r, c, v)
    b = ctx.to_device(np.arange(1, N + 1, dtype=np.float64))
    dofs, vals = zip(*g["fixed"])
    coo.fix_solution_components_lse(list(dofs), list(vals), b)
    A = coo.make_sparse().to_scipy().toarray()
    x = np.linalg.solve(A, b.download())
    assert np.linalg.norm(x - np.array(g["solution"])) < g["tolerance"]
    # assembled system, repeated dofs
    run = Run(ctx, W.config2(12))
    gc = run.gpu_matrix()
    gb = run.gpu_vector()
    rng = np.random.default_rng(8)
    nd = run.space.num_dofs
    dofs = rng.integers(0, nd, 300)
    dofs = np.concatenate([dofs, dofs[:50]])  # repeats accumulate
    vals = rng.standard_normal(len(dofs))
    gc.fix_solution_components_lse(dofs, vals, gb)
    oA = run.oracle_matrix()
    ob = run.oracle_vector()
    oA.fix_lse(dofs, vals, ob)
    gbh = gb.download()
    fixed = np.unique(dofs)
    assert np.array_equal(gbh[fixed], ob[fixed])  # the accumulated values, bit for bit
    assert np.abs(gbh - ob).max() <= 1e-12 * np.abs(ob).max()
    ro, co, vo = oA.arrays()
    t = gc.triplets()
    assert np.array_equal(t["row"], ro) and np.array_equal(t["col"], co)
    assert np.abs(t["value"] - vo).max() <= VALUE_RTOL * np.abs(vo).max()
    with pytest.raises(L.LfgError) as e:
        gc.fix_solution_components_lse([nd], [1.0], gb)
    assert e.value.code == L.INVALID_ARG


def test_fix_and_csr_parity(ctx):
    r = Run(ctx, W.config2(16))
    coo = r.gpu_matrix()
    b = r.gpu_vector()
    flags = r.space.boundary_dof_flags()
    vals_h = np.linspace(-1, 1, r.space.num_dofs)  # non-homogeneous to exercise b -= A xhat
    vals = ctx.to_device(vals_h)
    coo.fix_flagged_solution_components(flags, vals, b)
    A = r.oracle_matrix()
    bo = r.oracle_vector()
    oflags = r.ospace.boundary_dof_flags()
    assert np.array_equal(flags.download(), oflags)
    A.fix_flagged(oflags, vals_h, bo)
    ro, co, vo = A.arrays()
    t = coo.triplets()
    assert np.array_equal(t["row"], ro) and np.array_equal(t["col"], co)
    assert np.abs(t["value"] - vo).max() <= VALUE_RTOL * np.abs(vo).max()
    bg = b.download()
    assert np.abs(bg - bo).max() <= 1e-12 * np.abs(bo).max()
    # makeSparse
    csr = coo.make_sparse()
    rp, col, val = csr.download()
    orp, ocol, oval = A.to_csr()
    assert np.array_equal(rp, orp) and np.array_equal(col, ocol)
    assert np.abs(val - oval).max() <= VALUE_RTOL * np.abs(oval).max()


def test_fix_alt_parity(ctx):
    r = Run(ctx, W.config1(6))
    coo = r.gpu_matrix()
    b = r.gpu_vector()
    flags = r.space.boundary_dof_flags()
    vals_h = np.full(r.space.num_dofs, 0.5)
    coo.fix_flagged_solution_comp_alt(flags, ctx.to_device(vals_h), b)
    A = r.oracle_matrix()
    bo = r.oracle_vector()
    A.fix_flagged(r.ospace.boundary_dof_flags(), vals_h, bo, alt=True)
    ro, co, vo = A.arrays()
    t = coo.triplets()
    assert np.array_equal(t["row"], ro) and np.array_equal(t["col"], co)
    assert np.abs(b.download() - bo).max() <= 1e-12 * np.abs(bo).max()


def test_fix_dof_exact_solution_gpu(ctx, goldens):
    """fix_dof_flags (coomatrix_tests.cc:181-239) through the device COO, fix, CSR and PCG."""
    g = goldens["fix_dof_exact"]
    N = 10
    r, c, v = [], [], []
    for k in range(N):
        if k > 0:
            r.append(k); c.append(k - 1); v.append(-1.0)
        if k < N - 1:
            r.append(k); c.append(k + 1); v.append(-1.0)
        r.append(k); c.append(k); v.append(2.0)
    coo = L.COOMatrix(ctx, N, N, 64)
    coo.append(r, c, v)
    b = ctx.to_device(np.arange(1, N + 1, dtype=np.float64))
    flags = np.zeros(N, np.uint8)
    vals = np.ones(N)
    for k, val in g["fixed"]:
        flags[k] = 1
        vals[k] = val
    coo.fix_flagged_solution_components(ctx.to_device(flags), ctx.to_device(vals), b)
    x = ctx.zeros(N)
    st = coo.make_sparse().solve_pcg(b, x, rtol=1e-14)
    assert st["converged"]
    assert np.linalg.norm(x.download() - np.array(g["solution"])) < g["tolerance"]


@pytest.mark.parametrize("name", ["c1", "c2"])
@pytest.mark.parametrize("precision", [L.SOLVE_FP64, L.SOLVE_MIXED])
def test_solve_parity(ctx, name, precision):
    """GPU PCG vs an FP64 sparse direct solve of the oracle's system (the
    reference solves with Eigen SparseLU; SuperLU is the same algorithm)."""
    import scipy.sparse.linalg as spla
    r = Run(ctx, WORKLOADS[name]())
    coo = r.gpu_matrix()
    b = r.gpu_vector()
    flags = r.space.boundary_dof_flags()
    coo.fix_flagged_solution_components(flags, ctx.zeros(r.space.num_dofs), b)
    x = ctx.zeros(r.space.num_dofs)
    st = coo.make_sparse().solve_pcg(b, x, precision=precision, rtol=1e-12)
    assert st["converged"], st
    A = r.oracle_matrix()
    bo = r.oracle_vector()
    A.fix_flagged(r.ospace.boundary_dof_flags(), np.zeros(r.space.num_dofs), bo)
    xo = spla.splu(A.to_scipy().tocsc()).solve(bo)
    err = np.linalg.norm(x.download() - xo) / np.linalg.norm(xo)
    assert err <= 1e-8, err


def test_kat_tensor_coefficient_gpu(ctx, goldens):
    """lf_fe_linear.ReactionDiffusion (lagr_fe_tests.cc:804-831): O1 on test
    mesh 0 with the matrix-valued diffusion coefficient [[1, x], [y, x y]] and
    gamma = x y, degree-4 rules, assembled on the GPU; the bilinear form of the
    projections of 1 + x + 2y and 3x is 7911/8 (to the reference's 1e-2) and
    equals the oracle's value to 1e-12."""
    k = goldens["reaction_diffusion_kat"]
    xy, cells, _ = O.factory_input("test0", x0=1.0)
    m = L.Mesh.from_factory(ctx, xy, cells)
    s = L.Space.lagrange(m, 1)
    coo = L.COOMatrix(ctx, s.num_dofs, s.num_dofs, s.num_triplets)
    tensor = [1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1]  # [[1, x], [y, x y]]
    L.assemble_matrix_rd(s, L.rd_provider(L.coeff(L.TENSOR_BILINEAR, params=tensor),
                                          L.coeff(L.ANALYTIC, func=L.FN_POLY, params=list(W.poly(x1y1=1))), 4, 4), coo)
    os_ = O.Space(O.Mesh(xy, cells), 1)
    av = O.nodal_projection(os_, O.FN_POLY, W.poly(c=1, x1=1, y1=2))
    bv = O.nodal_projection(os_, O.FN_POLY, W.poly(x1=3))
    val = av @ (coo.make_sparse().to_scipy() @ bv)
    assert abs(val - k["O1_tensor_deg4"]["value"]) < k["tolerance"]
    assert abs(val - O.kat_tensor_rd()) <= 1e-12 * abs(val)


@pytest.mark.parametrize("kind", ["constant", "per_cell", "bilinear"])
@pytest.mark.parametrize("degree,mesh", [(1, "hybrid"), (2, "tptriag"), (2, "hybrid"), (3, "tpquad"), (3, "hybrid")])
def test_tensor_coefficient_parity(ctx, kind, degree, mesh):
    """Matrix-valued (non-symmetric) diffusion coefficients against the oracle:
    every element block, full n x n (the block is not symmetric), with and
    without a reaction term."""
    if mesh == "hybrid":
        xy, cells = W.hybrid_mesh(7, seed=4)
        spec = {"kind": "factory", "xy": xy, "cells": cells, "edges": None}
    else:
        spec = {"kind": mesh, "nx": 5, "ny": 4}
    gm = W.build_mesh(ctx, spec)
    om = oracle_mesh(spec)
    gs, os_ = L.Space.lagrange(gm, degree), O.Space(om, degree)
    rng = np.random.default_rng(degree)
    keep = None
    if kind == "constant":
        ga, oa = L.coeff(L.TENSOR_CONSTANT, params=[2.0, 0.3, -0.2, 1.5]), \
            O.coeff(O.TENSOR_CONSTANT, params=[2.0, 0.3, -0.2, 1.5])
    elif kind == "per_cell":
        d = np.tile([1.0, 0.0, 0.0, 1.0], gm.num_cells) + 0.3 * rng.standard_normal(4 * gm.num_cells)
        keep = ctx.to_device(d)
        ga, oa = L.coeff(L.TENSOR_PER_CELL, data=keep), O.coeff(O.TENSOR_PER_CELL, data=d)
    else:
        p = [1, 0.5, 0, 0.2, 0, 0.3, 0.1, 0, 0, 0, -0.4, 0.1, 2, 0, 0.5, 1]
        ga, oa = L.coeff(L.TENSOR_BILINEAR, params=p), O.coeff(O.TENSOR_BILINEAR, params=p)
    for gamma in (0.0, 0.7):
        gg = L.coeff(L.CONSTANT, gamma) if gamma else L.coeff(L.ZERO)
        og = O.coeff(O.CONSTANT, gamma) if gamma else O.coeff(O.ZERO)
        coo = L.COOMatrix(ctx, gs.num_dofs, gs.num_dofs, gs.num_triplets)
        L.assemble_matrix_rd(gs, L.rd_provider(ga, gg), coo)
        ro, co, vo = O.assemble_rd(os_, oa, og).arrays()
        compare_triplets(coo.triplets(), ro, co, vo, block_sizes(om.cells, os_.n_tria, os_.n_quad))
    # matrix-valued coefficients are accepted only as the diffusion coefficient
    coo = L.COOMatrix(ctx, gs.num_dofs, gs.num_dofs, gs.num_triplets)
    with pytest.raises(L.LfgError) as e:
        L.assemble_matrix_rd(gs, L.rd_provider(L.coeff(L.CONSTANT, 1.0), ga), coo)
    assert e.value.code == L.UNSUPPORTED


@pytest.mark.parametrize("degree,alpha,gamma,a,b,qdeg,key", [
    (2, W.poly(x1=1), W.poly(x1y1=1), W.poly(x2=1, y2=1), W.poly(x2=1, y2=-1), 6, "O2_deg6"),
    (3, W.poly(y1=1), W.poly(x1y1=1), W.poly(x3=1, y3=1), W.poly(x1y2=1), 8, "O3_deg8"),
])
def test_kat_reaction_diffusion_gpu(ctx, goldens, degree, alpha, gamma, a, b, qdeg, key):
    """lf_fe_quadratic/cubic.ReactionDiffusion with the matrix assembled on the GPU."""
    k = goldens["reaction_diffusion_kat"]
    xy, cells, _ = O.factory_input("test0", x0=1.0)
    m = L.Mesh.from_factory(ctx, xy, cells)
    s = L.Space.lagrange(m, degree)
    coo = L.COOMatrix(ctx, s.num_dofs, s.num_dofs, s.num_triplets)
    L.assemble_matrix_rd(s, L.rd_provider(L.coeff(L.ANALYTIC, func=L.FN_POLY, params=list(alpha)),
                                          L.coeff(L.ANALYTIC, func=L.FN_POLY, params=list(gamma)), qdeg, qdeg), coo)
    os_ = O.Space(O.Mesh(xy, cells), degree)
    av = O.nodal_projection(os_, O.FN_POLY, a)
    bv = O.nodal_projection(os_, O.FN_POLY, b)
    val = av @ (coo.make_sparse().to_scipy() @ bv)
    assert abs(val - k[key]["value"]) < k["tolerance"]


def test_errors(ctx):
    xy, cells, _ = O.factory_input("test0", x0=1.0)
    m = L.Mesh.from_factory(ctx, xy, cells)
    s = L.Space.lagrange(m, 1)
    coo = L.COOMatrix(ctx, s.num_dofs, s.num_dofs, s.num_triplets)
    # missing quadrature rule for quads (loc_comp_ellbvp.h:278-287)
    with pytest.raises(L.LfgError) as e:
        L.assemble_matrix_rd(s, L.rd_provider(L.coeff(L.CONSTANT, 1.0), L.coeff(L.ZERO), 2, -1), coo)
    assert e.value.code == L.MISSING_RULE and len(coo) == 0
    # capacity
    small = L.COOMatrix(ctx, s.num_dofs, s.num_dofs, 10)
    with pytest.raises(L.LfgError) as e:
        L.assemble_matrix_rd(s, L.rd_provider(L.coeff(L.CONSTANT, 1.0), L.coeff(L.ZERO)), small)
    assert e.value.code == L.CAPACITY and len(small) == 0
    # unsupported coefficient kind
    bad = L.coeff(L.CONSTANT, 1.0)
    bad.kind = 9
    with pytest.raises(L.LfgError) as e:
        L.assemble_matrix_rd(s, L.rd_provider(bad, L.coeff(L.ZERO)), coo)
    assert e.value.code == L.UNSUPPORTED
    # degenerate cell (collapsed triangle)
    xy2 = np.array([[0, 0], [1, 0], [2, 0], [0, 1]], float)
    with pytest.raises(L.LfgError) as e:
        L.Mesh.from_factory(ctx, xy2, np.array([[0, 1, 2, -1], [0, 2, 3, -1]]))
    assert e.value.code == L.DEGENERATE_CELL
    # incomplete mesh (node 3 unused)
    with pytest.raises(L.LfgError) as e:
        L.Mesh.from_factory(ctx, np.array([[0, 0], [1, 0], [0, 1], [4, 4]], float), np.array([[0, 1, 2, -1]]))
    assert e.value.code == L.INCOMPLETE_MESH
    # bad node index
    with pytest.raises(L.LfgError) as e:
        L.Mesh.from_factory(ctx, np.array([[0, 0], [1, 0], [0, 1]], float), np.array([[0, 1, 7, -1]]))
    assert e.value.code == L.INVALID_ARG
    # the context is still usable afterwards
    L.assemble_matrix_rd(s, L.rd_provider(L.coeff(L.CONSTANT, 1.0), L.coeff(L.ZERO)), coo)
    assert len(coo) == s.num_triplets


def test_handles_outlive_context():
    """Destroying the context before its meshes / matrices is safe: the
    context is freed when the last handle is released."""
    c = L.Context(0)
    mesh = L.Mesh.tp_triag(c, 4, 4)
    space = L.Space.lagrange(mesh, 2)
    coo = L.COOMatrix(c, space.num_dofs, space.num_dofs, space.num_triplets)
    L.assemble_matrix_rd(space, L.rd_provider(L.coeff(L.CONSTANT, 1.0), L.coeff(L.ZERO)), coo)
    csr = coo.make_sparse()
    c.close()
    del csr, coo, space, mesh
    import gc
    gc.collect()


def test_not_converged_status(ctx):
    r = Run(ctx, W.config1(16))
    coo = r.gpu_matrix()
    b = r.gpu_vector()
    coo.fix_flagged_solution_components(r.space.boundary_dof_flags(), ctx.zeros(r.space.num_dofs), b)
    x = ctx.zeros(r.space.num_dofs)
    with pytest.raises(L.LfgError) as e:
        coo.make_sparse().solve_pcg(b, x, rtol=1e-14, max_iterations=2, check_every=2)
    assert e.value.code == L.NOT_CONVERGED


@pytest.mark.parametrize("degree", [1, 2, 3])
def test_folded_load_vectors(ctx, degree):
    """Load vectors through the folded rules: bilinear quadrilaterals (jittered,
    |det J| affine in the reference coordinates) with a per-cell f, and
    triangles with an O1-nodal f."""
    rng = np.random.default_rng(degree)
    xy, cells = W.hybrid_mesh(12, seed=degree)
    mesh = {"kind": "factory", "xy": xy, "cells": cells, "edges": None}
    for f in (("cell", np.exp(rng.standard_normal(len(cells)))), ("nodal", 1.0 + rng.random(len(xy)))):
        wl = {"mesh": mesh, "degree": degree, "alpha": ("const", 1.0), "gamma": ("zero",), "f": f,
              "qr_tria": 0, "qr_quad": 0}
        r = Run(ctx, wl)
        b = r.gpu_vector().download()
        bo = r.oracle_vector()
        assert np.abs(b - bo).max() <= 1e-12 * np.abs(bo).max(), f[0]
