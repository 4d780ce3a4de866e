"""Batched form (GPU): persistent multi-mesh assembly and batched PCG.

Each mesh's segment of the batch COO must equal that mesh's own assembly
(indices shifted by the mesh's dof offset, identical order and values), and
each block of the batched solve must match a direct FP64 solve of the oracle's
system for that mesh."""
import numpy as np
import pytest

from parity import O, L, W, block_sizes, compare_triplets, oracle_coeff

pytestmark = pytest.mark.gpu


def _batch(ctx, ns, degs, seed=9):
    rng = np.random.default_rng(seed)
    meshes = [L.Mesh.tp_triag(ctx, int(n), int(n)) for n in ns]
    spaces = [L.Space.lagrange(m, int(d)) for m, d in zip(meshes, degs)]
    batch = L.Batch(ctx, spaces)
    alpha = np.exp(0.5 * rng.standard_normal(batch.num_cells))
    return meshes, spaces, batch, alpha


def _assemble(ctx, batch, alpha_d, gamma=1.0):
    coo = L.COOMatrix(ctx, batch.num_dofs, batch.num_dofs, batch.num_triplets + batch.num_dofs)
    batch.assemble_matrix_rd(L.rd_provider(L.coeff(L.PER_CELL, data=alpha_d), L.coeff(L.CONSTANT, gamma)), coo)
    return coo


def test_batch_assembly_matches_single_meshes(ctx):
    ns, degs = [3, 5, 7, 4, 6, 8, 2, 9], [1, 2, 1, 2, 2, 1, 3, 2]
    meshes, spaces, batch, alpha = _batch(ctx, ns, degs)
    alpha_d = ctx.to_device(alpha)
    coo = _assemble(ctx, batch, alpha_d)
    th, ct, ms = batch.tuning()
    assert th in (64, 128, 256) and ct >= 1 and ms > 0
    t = coo.triplets()
    dof, cell, trip = batch.offsets()
    assert len(t) == trip[-1]
    for b, (sp, n, d) in enumerate(zip(spaces, ns, degs)):
        seg = t[trip[b]:trip[b + 1]]
        a_b = ctx.to_device(alpha[cell[b]:cell[b + 1]])
        single = L.COOMatrix(ctx, sp.num_dofs, sp.num_dofs, sp.num_triplets)
        L.assemble_matrix_rd(sp, L.rd_provider(L.coeff(L.PER_CELL, data=a_b), L.coeff(L.CONSTANT, 1.0)), single)
        st = single.triplets()
        assert np.array_equal(seg["row"] - dof[b], st["row"]) and np.array_equal(seg["col"] - dof[b], st["col"])
        assert np.array_equal(seg["value"], st["value"])
        xy, cells, pe = O.factory_input("tptriag", n, n)
        os_ = O.Space(O.Mesh(xy, cells, pe), d)
        A = O.assemble_rd(os_, O.coeff(O.PER_CELL, data=alpha[cell[b]:cell[b + 1]]), O.coeff(O.CONSTANT, 1.0))
        ro, co, vo = A.arrays()
        seg2 = seg.copy()
        seg2["row"] -= dof[b]
        seg2["col"] -= dof[b]
        compare_triplets(seg2, ro, co, vo, block_sizes(cells, os_.n_tria, os_.n_quad))


@pytest.mark.parametrize("precision", [L.SOLVE_FP64, L.SOLVE_MIXED])
def test_batch_solve_matches_direct_solves(ctx, precision):
    import scipy.sparse.linalg as spla
    ns, degs = [6, 11, 4, 9, 14, 7], [1, 2, 2, 1, 2, 1]
    meshes, spaces, batch, alpha = _batch(ctx, ns, degs, seed=3)
    alpha_d = ctx.to_device(alpha)
    coo = _assemble(ctx, batch, alpha_d)
    b = ctx.zeros(batch.num_dofs)
    batch.assemble_vector_load(L.load_provider(L.coeff(L.CONSTANT, 1.0)), b)
    coo.fix_flagged_solution_components(batch.boundary_dof_flags(), ctx.zeros(batch.num_dofs), b)
    csr = coo.make_sparse()
    x = ctx.zeros(batch.num_dofs)
    st = batch.solve_pcg(csr, b, x, precision=precision, rtol=1e-12, check_every=8)
    assert st["converged"] and all(blk["converged"] for blk in st["blocks"])
    xs = x.download()
    dof, cell, _ = batch.offsets()
    for k, (n, d) in enumerate(zip(ns, degs)):
        xy, cells, pe = O.factory_input("tptriag", n, n)
        os_ = O.Space(O.Mesh(xy, cells, pe), d)
        A = O.assemble_rd(os_, O.coeff(O.PER_CELL, data=alpha[cell[k]:cell[k + 1]]), O.coeff(O.CONSTANT, 1.0))
        bo = O.assemble_load(os_, O.coeff(O.CONSTANT, 1.0))
        A.fix_flagged(os_.boundary_dof_flags(), np.zeros(os_.num_dofs), bo)
        xo = spla.splu(A.to_scipy().tocsc()).solve(bo)
        err = np.linalg.norm(xs[dof[k]:dof[k + 1]] - xo) / np.linalg.norm(xo)
        assert err <= 1e-8, (k, err)
    # blocks of different size take different iteration counts
    its = [blk["iterations"] for blk in st["blocks"]]
    assert max(its) > min(its)


@pytest.mark.parametrize("check_every", [32, 128])
def test_batch_mixed_long_replays_terminate(ctx, check_every):
    """Mixed batched solve with long graph replays: every block converges to
    the FP64 solution within a few times the FP64 iteration count.  With 128
    iterations per replay a small block's FP32 recursion runs far past what
    FP32 resolves before its residual is replaced; the replacement then
    restarts its direction instead of keeping one that no longer belongs to
    the replaced residual (the 512-mesh batch used to run such blocks to the
    iteration cap)."""
    ns, degs = [90, 120, 64, 150], [2, 2, 1, 2]
    meshes, spaces, batch, alpha = _batch(ctx, ns, degs, seed=11)
    alpha_d = ctx.to_device(alpha)
    coo = _assemble(ctx, batch, alpha_d)
    b = ctx.zeros(batch.num_dofs)
    batch.assemble_vector_load(L.load_provider(L.coeff(L.CONSTANT, 1.0)), b)
    coo.fix_flagged_solution_components(batch.boundary_dof_flags(), ctx.zeros(batch.num_dofs), b)
    csr = coo.make_sparse()
    x64, x32 = ctx.zeros(batch.num_dofs), ctx.zeros(batch.num_dofs)
    s64 = batch.solve_pcg(csr, b, x64, precision=L.SOLVE_FP64, rtol=1e-10, check_every=check_every)
    s32 = batch.solve_pcg(csr, b, x32, precision=L.SOLVE_MIXED, rtol=1e-10, check_every=check_every,
                          max_iterations=50000)
    assert s32["converged"] and all(blk["converged"] for blk in s32["blocks"])
    it64 = max(blk["iterations"] for blk in s64["blocks"])
    it32 = max(blk["iterations"] for blk in s32["blocks"])
    assert it32 <= 4 * it64 + 4 * check_every, (it32, it64)
    a, r = x32.download(), x64.download()
    dof, _, _ = batch.offsets()
    for k in range(len(ns)):
        seg, ref = a[dof[k]:dof[k + 1]], r[dof[k]:dof[k + 1]]
        assert np.linalg.norm(seg - ref) <= 1e-8 * np.linalg.norm(ref), k


@pytest.mark.parametrize("precision", [L.SOLVE_FP64, L.SOLVE_MIXED])
def test_batch_solver_chunk_autotuner(ctx, precision):
    """The first solve in a precision times the chunk sizes and keeps one; any
    chunk size gives the same solution up to the order of the partial sums."""
    ns, degs = [40, 24, 56, 33, 47, 29, 61, 38], [2, 1, 2, 2, 1, 2, 1, 2]
    meshes, spaces, batch, alpha = _batch(ctx, ns, degs, seed=12)
    alpha_d = ctx.to_device(alpha)
    coo = _assemble(ctx, batch, alpha_d)
    b = ctx.zeros(batch.num_dofs)
    batch.assemble_vector_load(L.load_provider(L.coeff(L.CONSTANT, 1.0)), b)
    coo.fix_flagged_solution_components(batch.boundary_dof_flags(), ctx.zeros(batch.num_dofs), b)
    csr = coo.make_sparse()
    assert batch.solve_tuning(precision) == (0, 0.0)
    x0 = ctx.zeros(batch.num_dofs)
    assert batch.solve_pcg(csr, b, x0, precision=precision, rtol=1e-11)["converged"]
    rows, rate = batch.solve_tuning(precision)
    assert rows in (512, 1024, 2048, 4096) and rate > 0
    ref = x0.download()
    for rows in (96, 4096):
        batch.set_solve_chunk_rows(precision, rows)
        x = ctx.zeros(batch.num_dofs)
        assert batch.solve_pcg(csr, b, x, precision=precision, rtol=1e-11)["converged"]
        assert np.linalg.norm(x.download() - ref) <= 1e-8 * np.linalg.norm(ref)
    with pytest.raises(L.LfgError):
        batch.set_solve_chunk_rows(precision, 8)


@pytest.mark.parametrize("precision", [L.SOLVE_FP64, L.SOLVE_MIXED])
def test_batch_grouped_solver(ctx, precision):
    """The grouped solver (L2-sized groups, persistent cooperative kernel with
    grid barriers, Chronopoulos-Gear iteration) gives every block the solution
    of the lock-step sweep: one group holding every mesh (a block of 161k rows
    spreads over every block of the grid), one group per mesh, and a middle
    budget; each block also against a direct solve of the oracle's system."""
    import scipy.sparse.linalg as spla
    ns, degs = [40, 24, 200, 33, 47, 6, 61, 38], [2, 1, 2, 2, 1, 2, 1, 2]
    meshes, spaces, batch, alpha = _batch(ctx, ns, degs, seed=21)
    alpha_d = ctx.to_device(alpha)
    coo = _assemble(ctx, batch, alpha_d)
    b = ctx.zeros(batch.num_dofs)
    batch.assemble_vector_load(L.load_provider(L.coeff(L.CONSTANT, 1.0)), b)
    coo.fix_flagged_solution_components(batch.boundary_dof_flags(), ctx.zeros(batch.num_dofs), b)
    csr = coo.make_sparse()
    assert batch.solve_groups() == 0.0
    x0 = ctx.zeros(batch.num_dofs)
    assert batch.solve_pcg(csr, b, x0, precision=precision, rtol=1e-10)["converged"]
    ref = x0.download()
    dof, cell, _ = batch.offsets()
    for budget in (1e12, 1.0, 4e6):
        batch.set_solve_groups(budget)
        assert batch.solve_groups() == budget
        x = ctx.zeros(batch.num_dofs)
        st = batch.solve_pcg(csr, b, x, precision=precision, rtol=1e-10)
        assert st["converged"] and all(blk["converged"] for blk in st["blocks"]), budget
        xs = x.download()
        for k in range(len(ns)):
            seg, r = xs[dof[k]:dof[k + 1]], ref[dof[k]:dof[k + 1]]
            assert np.linalg.norm(seg - r) <= 1e-8 * np.linalg.norm(r), (budget, k)
    for k in (0, 2, 5):
        n, d = ns[k], degs[k]
        xy, cells, pe = O.factory_input("tptriag", n, n)
        os_ = O.Space(O.Mesh(xy, cells, pe), d)
        A = O.assemble_rd(os_, O.coeff(O.PER_CELL, data=alpha[cell[k]:cell[k + 1]]), O.coeff(O.CONSTANT, 1.0))
        bo = O.assemble_load(os_, O.coeff(O.CONSTANT, 1.0))
        A.fix_flagged(os_.boundary_dof_flags(), np.zeros(os_.num_dofs), bo)
        xo = spla.splu(A.to_scipy().tocsc()).solve(bo)
        assert np.linalg.norm(xs[dof[k]:dof[k + 1]] - xo) <= 1e-8 * np.linalg.norm(xo), k
    with pytest.raises(L.LfgError):
        batch.set_solve_groups(-1.0)
    batch.set_solve_groups(0.0)
