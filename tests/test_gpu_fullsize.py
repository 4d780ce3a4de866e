"""Parity at the sizes that are benchmarked (GPU).

- The large hybrid configuration at full size (2048 x 2048 squares, 6.29M
  cells, 321M triplets, O2): every triplet of the device assembly against the
  oracle, cell range by cell range (indices and order bit-exact, values within
  1e-12 of each element block's largest entry), plus the whole load vector.
  This runs every tile of the persistent tensor-core quadrilateral kernel and
  of the triangle kernel that the benchmark times.
- The high-order configuration at full size (TPTriag 1024 x 1024, O3,
  2.1M cells, 210M triplets, degree-6 rules, analytic alpha): every triplet
  and the load vector against the oracle.
- The batching configuration at full size (512 meshes): the batched assembly,
  fix, COO->CSR and the batched FP64 and mixed-precision solves of all 512
  meshes, with 32 of them (seeded choice plus the largest mesh) compared with
  the oracle: their triplet segments bit-exact in indices, and their solution
  blocks against a sparse direct FP64 solve (SuperLU) of the oracle's system.

The oracle assembles cell ranges on host threads while the main thread copies
the matching slice of device triplets (one context, one caller).
"""
import concurrent.futures as cf
import os

import numpy as np
import pytest

from parity import O, L, W, Run, block_sizes, compare_triplets, oracle_coeff

pytestmark = pytest.mark.gpu

CHUNK_CELLS = 131072
WORKERS = max(2, min(8, (os.cpu_count() or 4)))


def _compare_all_cells(r, coo, qdeg_tria, qdeg_quad):
    cells = r.cells()
    nc = len(cells)
    bs = block_sizes(cells, r.space.n_tria, r.space.n_quad)
    off = np.concatenate([[0], np.cumsum(bs)])
    assert len(coo) == off[-1]
    alpha, gamma = oracle_coeff(r.wl["alpha"]), oracle_coeff(r.wl["gamma"])

    def work(g, lo, hi):
        ro, co, vo = O.assemble_rd(r.ospace, alpha, gamma, qdeg_tria, qdeg_quad, (lo, hi)).arrays()
        return compare_triplets(g, ro, co, vo, bs[lo:hi])

    worst = 0.0
    pending = []
    with cf.ThreadPoolExecutor(WORKERS) as ex:
        for lo in range(0, nc, CHUNK_CELLS):
            hi = min(nc, lo + CHUNK_CELLS)
            pending.append(ex.submit(work, coo.triplets_range(int(off[lo]), int(off[hi])), lo, hi))
            if len(pending) >= WORKERS:
                worst = max(worst, pending.pop(0).result())
        for f in pending:
            worst = max(worst, f.result())
    return worst


def _check_vector(r):
    b = r.gpu_vector().download()
    bo = r.oracle_vector()
    assert np.abs(b - bo).max() <= 1e-12 * np.abs(bo).max()


def test_config2_full_size_every_triplet(ctx):
    r = Run(ctx, W.config2(2048))
    assert r.mesh.num_cells == 6292364 and r.space.num_dofs == 16785409
    ctx.profile(True)
    ctx.profile_reset()
    fp64_cells = ctx.profile_read("fp64_fallback_cells")[1]  # a running count on the context
    coo = r.gpu_matrix()
    tc_launches = ctx.profile_read("rd_quad_tc")[1]
    ctx.profile(False)
    assert tc_launches == 1  # the quadrilaterals went through the tensor-core kernel
    assert ctx.profile_read("fp64_fallback_cells")[1] == fp64_cells  # no cell left the df32 / digit path
    worst = _compare_all_cells(r, coo, r.wl["qr_tria"], r.wl["qr_quad"])
    assert worst <= 1e-12
    del coo
    _check_vector(r)


def test_config3_full_size_every_triplet(ctx):
    r = Run(ctx, W.config3(1024))
    assert r.space.num_dofs == 9443329 and r.space.num_triplets == 2097152 * 100
    coo = r.gpu_matrix()
    worst = _compare_all_cells(r, coo, r.wl["qr_tria"], r.wl["qr_quad"])
    assert worst <= 1e-12
    del coo
    _check_vector(r)


def test_config4_full_batch_subset_vs_direct_solves(ctx):
    import scipy.sparse.linalg as spla
    wl = W.config4(512)
    ns, degs = wl["ns"], wl["degrees"]
    meshes = [L.Mesh.tp_triag(ctx, int(n), int(n)) for n in ns]
    spaces = [L.Space.lagrange(m, int(d)) for m, d in zip(meshes, degs)]
    batch = L.Batch(ctx, spaces)
    nd = batch.num_dofs
    alpha = wl["alpha"]
    alpha_d = ctx.to_device(alpha)
    coo = L.COOMatrix(ctx, nd, nd, batch.num_triplets + nd)
    batch.assemble_matrix_rd(L.rd_provider(L.coeff(L.PER_CELL, data=alpha_d), L.coeff(L.CONSTANT, wl["gamma"])), coo)
    dof, cell, trip = batch.offsets()
    rng = np.random.default_rng(2024)
    largest = int(np.argmax(np.where(degs == 2, 2 * ns + 1, ns + 1)))
    subset = sorted(set(rng.choice(len(ns), 31, replace=False).tolist()) | {largest})
    assert len(subset) >= 32
    segs = {k: coo.triplets_range(int(trip[k]), int(trip[k + 1])) for k in subset}
    b = ctx.zeros(nd)
    batch.assemble_vector_load(L.load_provider(L.coeff(L.CONSTANT, wl["f"])), b)
    coo.fix_flagged_solution_components(batch.boundary_dof_flags(), ctx.zeros(nd), b)
    csr = coo.make_sparse()
    del coo
    sols = {}
    for name, prec in (("fp64", L.SOLVE_FP64), ("mixed", L.SOLVE_MIXED)):
        x = ctx.zeros(nd)
        st = batch.solve_pcg(csr, b, x, precision=prec, rtol=1e-10)
        assert st["converged"], name
        sols[name] = x.download()
    errs = {"fp64": [], "mixed": []}
    for k in subset:
        n, d = int(ns[k]), int(degs[k])
        xy, cells, pe = O.factory_input("tptriag", n, n)
        os_ = O.Space(O.Mesh(xy, cells, pe), d)
        A = O.assemble_rd(os_, O.coeff(O.PER_CELL, data=alpha[cell[k]:cell[k + 1]]), O.coeff(O.CONSTANT, wl["gamma"]))
        ro, co, vo = A.arrays()
        seg = segs[k]
        seg["row"] -= dof[k]
        seg["col"] -= dof[k]
        compare_triplets(seg, ro, co, vo, block_sizes(cells, os_.n_tria, os_.n_quad))
        bo = O.assemble_load(os_, O.coeff(O.CONSTANT, wl["f"]))
        A.fix_flagged(os_.boundary_dof_flags(), np.zeros(os_.num_dofs), bo)
        xo = spla.splu(A.to_scipy().tocsc()).solve(bo)
        for name, xs in sols.items():
            errs[name].append(float(np.linalg.norm(xs[dof[k]:dof[k + 1]] - xo) / np.linalg.norm(xo)))
    for name, e in errs.items():
        assert max(e) <= 1e-8, (name, max(e), subset[int(np.argmax(e))])
