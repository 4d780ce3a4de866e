"""Time the PCG on the inverse-conductivity system (profiling driver).

    python -m lehrfempp_gb300.pcg_timing [n] [iterations]

Assembles TPTriag n x n, LagrangeO1, alpha = exp(theta) per cell (theta from
the seeded workload generator), gamma = 0, f = 1, Dirichlet 0, converts to
CSR and runs `iterations` PCG iterations (rtol 0: the iteration cap ends the
solve) twice in FP64 and twice in mixed precision, printing microseconds per
iteration.  Used for the ncu captures of the solver kernels.
"""
import sys
import time

import lehrfempp_gb300 as L
from lehrfempp_gb300 import workloads as W


def main(argv):
    n = int(argv[1]) if len(argv) > 1 else 1024
    iters = int(argv[2]) if len(argv) > 2 else 256
    ctx = L.Context(0)
    mesh = L.Mesh.tp_triag(ctx, n, n)
    sp = L.Space.lagrange(mesh, 1)
    theta = ctx.to_device(W.config5(n)["theta"])
    coo = L.COOMatrix(ctx, sp.num_dofs, sp.num_dofs, sp.num_triplets + sp.num_dofs)
    ctx.synchronize()
    t0 = time.perf_counter()
    L.assemble_matrix_rd(sp, L.rd_provider(L.coeff(L.PER_CELL_EXP, data=theta), L.coeff(L.ZERO)), coo)
    b = ctx.zeros(sp.num_dofs)
    L.assemble_vector_load(sp, L.load_provider(L.coeff(L.CONSTANT, 1.0)), b)
    coo.fix_flagged_solution_components(sp.boundary_dof_flags(), ctx.zeros(sp.num_dofs), b)
    ctx.synchronize()
    t1 = time.perf_counter()
    A = coo.make_sparse()
    ctx.synchronize()
    t2 = time.perf_counter()
    print("assemble+fix %.2f ms, csr %.2f ms" % ((t1 - t0) * 1e3, (t2 - t1) * 1e3))
    for prec, name in ((L.SOLVE_FP64, "fp64"), (L.SOLVE_MIXED, "mixed")):
        for _ in range(2):
            x = ctx.zeros(sp.num_dofs)
            ctx.synchronize()
            t0 = time.perf_counter()
            st = A.solve_pcg(b, x, precision=prec, rtol=1e-30, max_iterations=iters, raise_on_failure=False)
            ctx.synchronize()
            dt = time.perf_counter() - t0
            print("%s: %d iterations in %.2f ms = %.1f us/iteration" %
                  (name, st["iterations"], dt * 1e3, dt * 1e6 / max(st["iterations"], 1)))
    ctx.close()


if __name__ == "__main__":
    main(sys.argv)
