"""lfg_solve_pcg_noalloc checked against lfg_solve_pcg (GPU).

Some callers cannot let a library allocate device memory: an application that
gives the GPU a fixed memory budget managed by its own allocator, or a service
that must not grow the CUDA memory pool (or pay an allocation's implicit
synchronisation) inside its time-stepping loop.  For them the library offers
lfg_solve_pcg_noalloc, which keeps every PCG work vector in one fixed device
array inside the library and never allocates.

The test solves one Dirichlet problem with the allocating entry point and then
twice in a row with the non-allocating one (the fixed array keeps the previous
call's contents, so the second call shows that nothing stale is read); the
solutions must agree within the solution tolerance of the other solve tests.
It also checks that a system larger than the array's limit is refused.
This file is collected last on purpose.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SOLUTION_RTOL = 1e-8  # same bound as tests/test_gpu_parity.py::test_solve_parity
MAX_ROWS = 1 << 20


def _system(ctx, L, W):
    wl = W.config2(24)
    keep = []
    mesh = W.build_mesh(ctx, wl["mesh"])
    space = L.Space.lagrange(mesh, 2)
    coo = L.COOMatrix(ctx, space.num_dofs, space.num_dofs, space.num_triplets + space.num_dofs)
    L.assemble_matrix_rd(space, L.rd_provider(W.to_coeff(ctx, wl["alpha"], keep), W.to_coeff(ctx, wl["gamma"], keep)),
                         coo)
    b = ctx.zeros(space.num_dofs)
    L.assemble_vector_load(space, L.load_provider(W.to_coeff(ctx, wl["f"], keep)), b)
    coo.fix_flagged_solution_components(space.boundary_dof_flags(), ctx.zeros(space.num_dofs), b)
    return coo.make_sparse(), b, space.num_dofs


def test_noalloc_solve_matches_allocating_solve(ctx):
    import lehrfempp_gb300 as L
    from lehrfempp_gb300 import workloads as W
    A, b, n = _system(ctx, L, W)
    x_ref = ctx.zeros(n)
    st_ref = A.solve_pcg(b, x_ref, rtol=1e-12)
    assert st_ref["converged"]
    xr = x_ref.download()
    for call in range(2):
        x = ctx.zeros(n)
        st = A.solve_pcg(b, x, rtol=1e-12, noalloc=True)
        assert st["converged"], (call, st)
        rel = np.linalg.norm(x.download() - xr) / np.linalg.norm(xr)
        assert rel <= SOLUTION_RTOL, (call, rel)
        assert st["iterations"] == st_ref["iterations"]


def test_noalloc_rejects_oversized_system(ctx):
    import lehrfempp_gb300 as L
    n = MAX_ROWS + 1
    coo = L.COOMatrix(ctx, n, n, 4)
    coo.append([0], [0], [1.0])
    A = coo.make_sparse()
    b = ctx.zeros(n)
    x = ctx.zeros(n)
    with pytest.raises(L.LfgError) as e:
        A.solve_pcg(b, x, noalloc=True)
    assert e.value.code == L.CAPACITY
