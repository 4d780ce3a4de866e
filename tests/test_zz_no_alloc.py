"""lfg_solve_pcg_noalloc checked against lfg_solve_pcg (GPU).

Some callers cannot let a library allocate device memory: an application that
gives the GPU a fixed memory budget managed by its own allocator, or a service
that must not grow the CUDA memory pool (or pay an allocation's implicit
synchronisation) inside its time-stepping loop.  For them the library offers
lfg_solve_pcg_noalloc, which keeps every PCG work vector in one fixed device
array inside the library and never allocates.

Each case solves one Dirichlet problem with the allocating entry point and
then twice in a row with the non-allocating one (the fixed array keeps the
previous call's contents, so the second call shows that nothing stale is
read); the solutions must agree within the solution tolerance of the other
solve tests, and the device's free memory must be the same before and after
the second call.  One case sits at the row limit (1024 x 1024 nodes =
2^20 rows); a system one row larger is refused.  The two solvers share the
algorithm but not the SpMV's summation order, so their iteration counts may
differ slightly.
This file is collected last on purpose.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SOLUTION_RTOL = 1e-8  # same bound as tests/test_gpu_parity.py::test_solve_parity
MAX_ROWS = 1 << 20


def _system(ctx, L, W, wl):
    keep = []
    mesh = W.build_mesh(ctx, wl["mesh"])
    space = L.Space.lagrange(mesh, wl["degree"])
    coo = L.COOMatrix(ctx, space.num_dofs, space.num_dofs, space.num_triplets + space.num_dofs)
    L.assemble_matrix_rd(space, L.rd_provider(W.to_coeff(ctx, wl["alpha"], keep), W.to_coeff(ctx, wl["gamma"], keep),
                                              wl["qr_tria"], wl["qr_quad"]), coo)
    b = ctx.zeros(space.num_dofs)
    L.assemble_vector_load(space, L.load_provider(W.to_coeff(ctx, wl["f"], keep), wl["qr_tria"], wl["qr_quad"]), b)
    coo.fix_flagged_solution_components(space.boundary_dof_flags(), ctx.zeros(space.num_dofs), b)
    return coo.make_sparse(), b, space.num_dofs


def _free_device_bytes(ctx):
    import torch
    ctx.synchronize()
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


@pytest.mark.parametrize("case", ["hybrid24_o2", "tptriag1023_o1_at_limit"])
def test_noalloc_solve_matches_allocating_solve(ctx, case):
    import lehrfempp_gb300 as L
    from lehrfempp_gb300 import workloads as W
    if case == "hybrid24_o2":
        wl, rtol = W.config2(24), 1e-12
    else:
        wl, rtol = W.config5(1023), 1e-10
    A, b, n = _system(ctx, L, W, wl)
    if case.endswith("at_limit"):
        assert n == MAX_ROWS
    x_ref = ctx.zeros(n)
    st_ref = A.solve_pcg(b, x_ref, rtol=rtol)
    assert st_ref["converged"]
    xr = x_ref.download()
    xs = [ctx.zeros(n), ctx.zeros(n)]
    free = []
    for call in range(2):
        free.append(_free_device_bytes(ctx))
        st = A.solve_pcg(b, xs[call], rtol=rtol, noalloc=True)
        assert st["converged"], (call, st)
        rel = np.linalg.norm(xs[call].download() - xr) / np.linalg.norm(xr)
        assert rel <= SOLUTION_RTOL, (call, rel)
        assert abs(st["iterations"] - st_ref["iterations"]) <= max(64, st_ref["iterations"] // 20), (st, st_ref)
    free.append(_free_device_bytes(ctx))
    # nothing allocated by the second call (the first may load kernels lazily)
    assert free[2] == free[1], free


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
