"""Shared test inputs: the reference's test providers and seeded workloads."""
import numpy as np


def cell_index_matrices(num_cells, ld=4):
    """TestAssembler of lib/lf/assemble/test/assembly_tests.cc:61-82: cell index
    on the diagonal, minus the cell index elsewhere (4x4, trias use 3x3)."""
    e = np.zeros((num_cells, ld, ld))
    for c in range(num_cells):
        e[c] = -float(c)
        np.fill_diagonal(e[c], float(c))
    v = np.repeat(np.arange(num_cells, dtype=np.float64)[:, None], ld, axis=1)
    return e, v


def edge_dof_assembler_matrices(num_cells, ld=8):
    """EdgeDofAssembler of assembly_tests.cc:320-345 (8x8)."""
    e = np.zeros((num_cells, ld, ld))
    for c in range(num_cells):
        e[c] = -float(c)
        e[c][0::2, 0::2] = float(c)
        np.fill_diagonal(e[c], float(c))
    return e


def dense(rows, cols, r, c, v):
    A = np.zeros((rows, cols))
    np.add.at(A, (r, c), v)
    return A


def poly(**terms):
    """Coefficients p[4i+j] of sum c_ij x^i y^j; keys like x2y1=1.0, c=1.0."""
    p = np.zeros(16)
    for k, val in terms.items():
        if k == "c":
            p[0] += val
            continue
        i = int(k[1]) if k.startswith("x") else 0
        j = int(k[k.index("y") + 1]) if "y" in k else 0
        p[4 * i + j] += val
    return p


def splitmix64(x):
    x = (x + np.uint64(0x9E3779B97F4A7C15)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    z = x
    z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    return z ^ (z >> np.uint64(31))
