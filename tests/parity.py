"""Helpers that run one workload through the GPU library and through the oracle."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as O  # noqa: E402

import lehrfempp_gb300 as L  # noqa: E402
from lehrfempp_gb300 import workloads as W  # noqa: E402

VALUE_RTOL = 1e-12  # |gpu - oracle| <= 1e-12 * max |A_K| per element matrix


def oracle_coeff(spec):
    k = spec[0]
    if k == "zero":
        return O.coeff(O.ZERO)
    if k == "const":
        return O.coeff(O.CONSTANT, spec[1])
    if k == "cell":
        return O.coeff(O.PER_CELL, data=spec[1])
    if k == "nodal":
        return O.coeff(O.NODAL_O1, data=spec[1])
    if k == "poly":
        return O.coeff(O.ANALYTIC, func=O.FN_POLY, params=list(spec[1]))
    if k == "sinsin":
        return O.coeff(O.ANALYTIC, func=O.FN_SINSIN, params=list(spec[1:]))
    if k == "sincos":
        return O.coeff(O.ANALYTIC, func=O.FN_SINCOS, params=list(spec[1:]))
    raise ValueError(spec)


def oracle_mesh(spec):
    if spec["kind"] in ("tptriag", "tpquad"):
        xy, cells, pe = O.factory_input(spec["kind"], spec["nx"], spec["ny"])
        return O.Mesh(xy, cells, pe)
    return O.Mesh(spec["xy"], spec["cells"], spec.get("edges"))


def compare_triplets(gpu, rows, cols, vals, block_sizes):
    """Indices and order bit-exact; values per element block within VALUE_RTOL."""
    assert len(gpu) == len(vals), (len(gpu), len(vals))
    assert np.array_equal(gpu["row"], rows), "row indices differ"
    assert np.array_equal(gpu["col"], cols), "column indices differ"
    gv = gpu["value"]
    offs = np.concatenate([[0], np.cumsum(block_sizes)])
    bidx = np.repeat(np.arange(len(block_sizes)), block_sizes)
    scale = np.maximum.reduceat(np.abs(vals), offs[:-1]) if len(vals) else np.zeros(0)
    err = np.abs(gv - vals)
    ok = err <= VALUE_RTOL * scale[bidx] + 1e-300
    if not ok.all():
        i = int(np.argmax(~ok))
        raise AssertionError("value mismatch at triplet %d: gpu %.17g oracle %.17g (scale %.3g)" %
                             (i, gv[i], vals[i], scale[bidx[i]]))
    return float((err / np.maximum(scale[bidx], 1e-300)).max()) if len(vals) else 0.0


def block_sizes(cells, n_tria, n_quad):
    return np.where(np.asarray(cells)[:, 3] >= 0, n_quad * n_quad, n_tria * n_tria)


class Run:
    """One workload assembled on both sides."""

    def __init__(self, ctx, wl):
        self.ctx = ctx
        self.wl = wl
        self.keep = []
        self.mesh = W.build_mesh(ctx, wl["mesh"])
        self.space = L.Space.lagrange(self.mesh, wl["degree"])
        self.omesh = oracle_mesh(wl["mesh"])
        self.ospace = O.Space(self.omesh, wl["degree"])

    def gpu_matrix(self):
        p = L.rd_provider(W.to_coeff(self.ctx, self.wl["alpha"], self.keep),
                          W.to_coeff(self.ctx, self.wl["gamma"], self.keep), self.wl["qr_tria"], self.wl["qr_quad"])
        coo = L.COOMatrix(self.ctx, self.space.num_dofs, self.space.num_dofs, self.space.num_triplets + self.space.num_dofs)
        L.assemble_matrix_rd(self.space, p, coo)
        return coo

    def gpu_vector(self):
        b = self.ctx.zeros(self.space.num_dofs)
        p = L.load_provider(W.to_coeff(self.ctx, self.wl["f"], self.keep), self.wl["qr_tria"], self.wl["qr_quad"])
        L.assemble_vector_load(self.space, p, b)
        return b

    def oracle_matrix(self, cells=(0, -1)):
        return O.assemble_rd(self.ospace, oracle_coeff(self.wl["alpha"]), oracle_coeff(self.wl["gamma"]),
                             self.wl["qr_tria"], self.wl["qr_quad"], cells)

    def oracle_vector(self):
        return O.assemble_load(self.ospace, oracle_coeff(self.wl["f"]), self.wl["qr_tria"], self.wl["qr_quad"])

    def cells(self):
        return self.omesh.cells
