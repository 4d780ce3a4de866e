"""Assemble a hierarchic (hp) stiffness matrix repeatedly (profiling driver).

    python -m lehrfempp_gb300.hier_timing [n] [degree] [tria|quad] [repeats]

TPTriag (or TPQuad) n x n, HierarchicScalarFESpace of the given degree,
DiffusionElementMatrixProvider with alpha = 1, `repeats` assemblies into one
COO matrix (cleared in between); prints the triplet count and the time per
assembly.  Used for the ncu captures of the hierarchic element kernels.
"""
import sys
import time

import lehrfempp_gb300 as L


def main(argv):
    n = int(argv[1]) if len(argv) > 1 else 512
    p = int(argv[2]) if len(argv) > 2 else 4
    kind = argv[3] if len(argv) > 3 else "tria"
    reps = int(argv[4]) if len(argv) > 4 else 3
    ctx = L.Context(0)
    mesh = L.Mesh.tp_triag(ctx, n, n) if kind == "tria" else L.Mesh.tp_quad(ctx, n, n)
    sp = L.Space.hierarchic(mesh, p)
    coo = L.COOMatrix(ctx, sp.num_dofs, sp.num_dofs, sp.num_triplets)
    prov = L.rd_provider(L.coeff(L.CONSTANT, 1.0), L.coeff(L.ZERO))
    ctx.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        coo.set_zero()
        L.assemble_matrix_rd(sp, prov, coo)
    ctx.synchronize()
    dt = (time.perf_counter() - t0) / reps
    print("%s %dx%d degree %d: %d triplets, %.3f ms per assembly (first includes table set-up)" %
          (kind, n, n, p, sp.num_triplets, dt * 1e3))
    ctx.close()


if __name__ == "__main__":
    main(sys.argv)
