"""ctypes front end of the oracle (test infrastructure only).

The oracle is a CPU restatement of LehrFEM++'s assembly path (see lfo.h).  Only
tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs may import this
module; the library in lehrfempp_gb300/ never does.
"""
import ctypes as C
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None
_lock = threading.Lock()

ZERO, CONSTANT, PER_CELL, NODAL_O1, ANALYTIC, PER_CELL_EXP = 0, 1, 2, 3, 4, 5
# matrix-valued diffusion coefficients (row-major 2x2): constant p[0..3], per cell
# data[4 cell + e], bilinear entries p[4e] + p[4e+1] x + p[4e+2] y + p[4e+3] x y
TENSOR_CONSTANT, TENSOR_PER_CELL, TENSOR_BILINEAR = 6, 7, 8
FN_POLY, FN_SINSIN, FN_SINCOS, FN_EXP, FN_TRIG = 1, 2, 3, 4, 5
INT_VALUE, INT_SQ_DIFF, INT_GRAD_SQ_DIFF = 0, 1, 2


def build(force=False):
    """Compile the oracle with its Makefile (g++, a few seconds)."""
    srcs = [os.path.join(_HERE, f) for f in ("lfo_core.cc", "lfo_capi.cc", "lfo.h", "tria_rules.inc")]
    if not force and os.path.exists(_LIB_PATH):
        if os.path.getmtime(_LIB_PATH) >= max(os.path.getmtime(s) for s in srcs):
            return _LIB_PATH
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


class lfo_coeff(C.Structure):
    _fields_ = [("kind", C.c_int32), ("func", C.c_int32), ("value", C.c_double),
                ("data", C.POINTER(C.c_double)), ("p", C.c_double * 16)]


def coeff(kind=ZERO, value=0.0, data=None, func=0, params=()):
    c = lfo_coeff()
    c.kind = kind
    c.value = value
    c.func = func
    keep = None
    if data is not None:
        keep = np.ascontiguousarray(data, dtype=np.float64)
        c.data = keep.ctypes.data_as(C.POINTER(C.c_double))
    for i, v in enumerate(params):
        c.p[i] = v
    c._keep = keep  # keep the array alive with the struct
    return c


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(_LIB_PATH)
            vp, i64, i32, dp = C.c_void_p, C.c_int64, C.c_int32, C.c_double
            P = C.POINTER
            L.lfo_input_create.argtypes = [C.c_int, i64, i64, dp, dp, dp, dp, P(vp), P(i64), C.c_char_p, C.c_int]
            L.lfo_input_copy.argtypes = [vp, P(dp), P(i64), P(i64)]
            L.lfo_input_destroy.argtypes = [vp]
            L.lfo_mesh_create.argtypes = [i64, P(dp), i64, P(i64), i64, P(i64), P(vp), C.c_char_p, C.c_int]
            L.lfo_mesh_destroy.argtypes = [vp]
            L.lfo_mesh_sizes.argtypes = [vp, P(i64)]
            L.lfo_mesh_topology.argtypes = [vp, P(i64), P(i64), P(C.c_int8), P(i32)]
            L.lfo_boundary_flags.argtypes = [vp, P(C.c_uint8), P(C.c_uint8)]
            L.lfo_mesh_degenerate_cells.argtypes = [vp, P(i64)]
            L.lfo_space_create.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, P(vp), C.c_char_p, C.c_int]
            L.lfo_space_destroy.argtypes = [vp]
            L.lfo_space_info.argtypes = [vp, P(i64)]
            L.lfo_space_cell_dofs.argtypes = [vp, P(i64)]
            L.lfo_space_dof_entity.argtypes = [vp, P(i32), P(i64)]
            L.lfo_quad_rule.argtypes = [C.c_int, C.c_int, P(dp), P(dp), P(dp), P(C.c_int), C.c_char_p, C.c_int]
            L.lfo_assemble_rd.argtypes = [vp, P(lfo_coeff), P(lfo_coeff), C.c_int, C.c_int, i64, i64, P(vp), C.c_char_p, C.c_int]
            L.lfo_assemble_load.argtypes = [vp, P(lfo_coeff), C.c_int, C.c_int, P(dp), C.c_char_p, C.c_int]
            L.lfo_assemble_edge_mass.argtypes = [vp, P(lfo_coeff), P(C.c_uint8), C.c_int, P(vp), C.c_char_p, C.c_int]
            L.lfo_assemble_edge_load.argtypes = [vp, P(lfo_coeff), P(C.c_uint8), C.c_int, P(dp), C.c_char_p, C.c_int]
            L.lfo_assemble_tabulated.argtypes = [vp, P(dp), C.c_int, P(dp), P(dp), P(vp), C.c_char_p, C.c_int]
            L.lfo_coo_create.argtypes = [i64, i64, i64, P(i32), P(i32), P(dp)]
            L.lfo_coo_create.restype = vp
            L.lfo_coo_destroy.argtypes = [vp]
            L.lfo_coo_size.argtypes = [vp]
            L.lfo_coo_size.restype = i64
            L.lfo_coo_copy.argtypes = [vp, P(i32), P(i32), P(dp)]
            L.lfo_fix_flagged.argtypes = [vp, P(C.c_uint8), P(dp), P(dp), C.c_int, C.c_char_p, C.c_int]
            L.lfo_fix_lse.argtypes = [vp, C.c_int64, P(C.c_int64), P(dp), P(dp), C.c_char_p, C.c_int]
            L.lfo_csr_create.argtypes = [vp, P(i64)]
            L.lfo_csr_create.restype = vp
            L.lfo_csr_copy.argtypes = [vp, P(i64), P(i32), P(dp)]
            L.lfo_csr_destroy.argtypes = [vp]
            L.lfo_nodal_projection.argtypes = [vp, C.c_int, P(dp), P(dp), C.c_char_p, C.c_int]
            L.lfo_kat_tensor_rd.argtypes = [P(dp), C.c_char_p, C.c_int]
            L.lfo_assemble_hier.argtypes = [vp, C.c_int, P(lfo_coeff), P(lfo_coeff), C.c_int, P(vp), C.c_char_p,
                                            C.c_int]
            L.lfo_assemble_hier_load.argtypes = [vp, C.c_int, P(lfo_coeff), C.c_int, P(dp), C.c_char_p, C.c_int]
            L.lfo_hier_shape.argtypes = [C.c_int, C.c_int, P(C.c_int8), C.c_int, P(dp), P(dp), P(dp), C.c_char_p,
                                         C.c_int]
            L.lfo_space_create_hier_var.argtypes = [vp, P(i32), P(i32), P(vp), C.c_char_p, C.c_int]
            L.lfo_space_local_counts.argtypes = [vp, P(i32)]
            L.lfo_hier_shape_var.argtypes = [C.c_int, C.c_int, P(i32), P(C.c_int8), C.c_int, P(dp), P(dp), P(dp),
                                             C.c_char_p, C.c_int]
            L.lfo_hier_dual.argtypes = [C.c_int, C.c_int, P(i32), P(C.c_int8), P(dp), P(dp), P(C.c_int), P(C.c_int),
                                        C.c_char_p, C.c_int]
            L.lfo_nodal_projection_hier.argtypes = [vp, C.c_int, P(lfo_coeff), P(C.c_uint8), P(dp), C.c_char_p,
                                                    C.c_int]
            L.lfo_integrate_hier.argtypes = [vp, C.c_int, C.c_int, P(lfo_coeff), P(dp), C.c_int, P(C.c_uint8),
                                             P(dp), C.c_char_p, C.c_int]
            L.lfo_eval_fe_hier.argtypes = [vp, C.c_int, P(dp), C.c_int, P(dp), P(dp), P(dp), C.c_char_p, C.c_int]
            L.lfo_hier_fn.argtypes = [C.c_int, C.c_int, dp, dp, dp]
            L.lfo_hier_fn.restype = dp
            L.lfo_integrate.argtypes = [vp, C.c_int, P(lfo_coeff), P(dp), C.c_int, P(C.c_uint8), C.c_int, P(dp),
                                        C.c_char_p, C.c_int]
            L.lfo_eval_fe.argtypes = [vp, P(dp), C.c_int, P(dp), P(dp), P(dp), C.c_char_p, C.c_int]
            L.lfo_nodal_projection_mf.argtypes = [vp, P(lfo_coeff), P(C.c_uint8), P(dp), C.c_char_p, C.c_int]
            L.lfo_init_essential.argtypes = [vp, P(C.c_uint8), P(lfo_coeff), P(C.c_uint8), P(dp), C.c_char_p,
                                             C.c_int]
            _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def _check(rc, err):
    if rc != 0:
        raise RuntimeError("oracle: " + err.value.decode(errors="replace"))


def _err():
    return C.create_string_buffer(512)


def factory_input(kind, nx=0, ny=0, x0=0.0, y0=0.0, x1=1.0, y1=1.0):
    """Factory arrays (xy, cells[4], preset edges[2]) of a reference builder.

    kind: "tptriag" (TPTriagMeshBuilder), "tpquad" (TPQuadMeshBuilder) or
    "test0" (GenerateHybrid2DTestMesh(0), x0 = scale)."""
    L = lib()
    k = {"tptriag": 0, "tpquad": 1, "test0": 2}[kind]
    h = C.c_void_p()
    sizes = np.zeros(3, np.int64)
    err = _err()
    _check(L.lfo_input_create(k, nx, ny, x0, y0, x1, y1, C.byref(h), _p(sizes, C.c_int64), err, 512), err)
    xy = np.zeros((sizes[0], 2))
    cells = np.zeros((sizes[1], 4), np.int64)
    edges = np.zeros((max(sizes[2], 1), 2), np.int64)
    L.lfo_input_copy(h, _p(xy, C.c_double), _p(cells, C.c_int64), _p(edges, C.c_int64))
    L.lfo_input_destroy(h)
    return xy, cells, edges[: sizes[2]]


class Mesh:
    """hybrid2d::Mesh numbering restated (mesh.cc:178-810)."""

    def __init__(self, xy, cells, preset_edges=None):
        L = lib()
        self.xy = np.ascontiguousarray(xy, np.float64).reshape(-1, 2)
        self.cells = np.ascontiguousarray(cells, np.int64).reshape(-1, 4)
        pe = np.zeros((0, 2), np.int64) if preset_edges is None else np.ascontiguousarray(preset_edges, np.int64).reshape(-1, 2)
        self._pe = pe
        self.h = C.c_void_p()
        err = _err()
        _check(L.lfo_mesh_create(len(self.xy), _p(self.xy, C.c_double), len(self.cells), _p(self.cells, C.c_int64),
                                 len(pe), _p(pe, C.c_int64) if len(pe) else None, C.byref(self.h), err, 512), err)
        s = np.zeros(3, np.int64)
        L.lfo_mesh_sizes(self.h, _p(s, C.c_int64))
        self.num_nodes, self.num_edges, self.num_cells = (int(v) for v in s)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.lfo_mesh_destroy(self.h)
            self.h = None

    def topology(self):
        en = np.zeros((self.num_edges, 2), np.int64)
        ce = np.zeros((self.num_cells, 4), np.int64)
        co = np.zeros((self.num_cells, 4), np.int8)
        nc = np.zeros(self.num_edges, np.int32)
        lib().lfo_mesh_topology(self.h, _p(en, C.c_int64), _p(ce, C.c_int64), _p(co, C.c_int8), _p(nc, C.c_int32))
        return en, ce, co, nc

    def boundary_flags(self):
        nf = np.zeros(self.num_nodes, np.uint8)
        ef = np.zeros(self.num_edges, np.uint8)
        lib().lfo_boundary_flags(self.h, _p(nf, C.c_uint8), _p(ef, C.c_uint8))
        return nf, ef

    def num_degenerate(self):
        n = C.c_int64()
        lib().lfo_mesh_degenerate_cells(self.h, C.byref(n))
        return n.value


class Space:
    """UniformFEDofHandler (dofhandler.cc:86-338); degree>0 = FeSpaceLagrangeO<degree>."""

    def __init__(self, mesh, degree=0, layout=(0, 0, 0, 0)):
        self.mesh = mesh
        self.degree = degree
        self.h = C.c_void_p()
        err = _err()
        _check(lib().lfo_space_create(mesh.h, degree, *layout, C.byref(self.h), err, 512), err)
        info = np.zeros(4, np.int64)
        lib().lfo_space_info(self.h, _p(info, C.c_int64))
        self.num_dofs, self.n_cell, self.n_tria, self.n_quad = (int(v) for v in info)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.lfo_space_destroy(self.h)
            self.h = None

    def cell_dofs(self):
        out = np.zeros((self.mesh.num_cells, self.n_cell), np.int64)
        lib().lfo_space_cell_dofs(self.h, _p(out, C.c_int64))
        return out

    def dof_entities(self):
        cod = np.zeros(self.num_dofs, np.int32)
        idx = np.zeros(self.num_dofs, np.int64)
        lib().lfo_space_dof_entity(self.h, _p(cod, C.c_int32), _p(idx, C.c_int64))
        return cod, idx

    def local_counts(self):
        """Local dof count of every cell (NumLocalDofs)."""
        out = np.zeros(self.mesh.num_cells, np.int32)
        lib().lfo_space_local_counts(self.h, _p(out, C.c_int32))
        return out

    def boundary_dof_flags(self):
        """Selector of the reference drivers: dof flagged iff its entity is on the boundary."""
        nf, ef = self.mesh.boundary_flags()
        cod, idx = self.dof_entities()
        fl = np.zeros(self.num_dofs, np.uint8)
        fl[cod == 2] = nf[idx[cod == 2]]
        fl[cod == 1] = ef[idx[cod == 1]]
        return fl


class COO:
    def __init__(self, h, rows, cols):
        self.h = h
        self.rows = rows
        self.cols = cols

    @classmethod
    def from_arrays(cls, rows, cols, r, c, v):
        r = np.ascontiguousarray(r, np.int32)
        c = np.ascontiguousarray(c, np.int32)
        v = np.ascontiguousarray(v, np.float64)
        h = lib().lfo_coo_create(rows, cols, len(v), _p(r, C.c_int32), _p(c, C.c_int32), _p(v, C.c_double))
        return cls(C.c_void_p(h), rows, cols)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.lfo_coo_destroy(self.h)
            self.h = None

    def __len__(self):
        return int(lib().lfo_coo_size(self.h))

    def arrays(self):
        n = len(self)
        r = np.zeros(n, np.int32)
        c = np.zeros(n, np.int32)
        v = np.zeros(n, np.float64)
        if n:
            lib().lfo_coo_copy(self.h, _p(r, C.c_int32), _p(c, C.c_int32), _p(v, C.c_double))
        return r, c, v

    def fix_flagged(self, flags, values, b, alt=False):
        flags = np.ascontiguousarray(flags, np.uint8)
        values = np.ascontiguousarray(values, np.float64)
        assert b.dtype == np.float64 and b.flags.c_contiguous
        err = _err()
        _check(lib().lfo_fix_flagged(self.h, _p(flags, C.c_uint8), _p(values, C.c_double), _p(b, C.c_double),
                                     int(alt), err, 512), err)

    def fix_lse(self, dofs, values, b):
        """FixSolutionComponentsLse with the (dof, value) pairs in list order."""
        dofs = np.ascontiguousarray(dofs, np.int64)
        values = np.ascontiguousarray(values, np.float64)
        assert b.dtype == np.float64 and b.flags.c_contiguous and len(dofs) == len(values)
        err = _err()
        _check(lib().lfo_fix_lse(self.h, len(dofs), _p(dofs, C.c_int64), _p(values, C.c_double),
                                 _p(b, C.c_double), err, 512), err)

    def to_csr(self):
        sizes = np.zeros(2, np.int64)
        h = lib().lfo_csr_create(self.h, _p(sizes, C.c_int64))
        rowptr = np.zeros(sizes[0] + 1, np.int64)
        col = np.zeros(sizes[1], np.int32)
        val = np.zeros(sizes[1], np.float64)
        lib().lfo_csr_copy(h, _p(rowptr, C.c_int64), _p(col, C.c_int32), _p(val, C.c_double))
        lib().lfo_csr_destroy(h)
        return rowptr, col, val

    def to_scipy(self):
        import scipy.sparse as sp
        rowptr, col, val = self.to_csr()
        return sp.csr_matrix((val, col, rowptr), shape=(self.rows, self.cols))


def assemble_rd(space, alpha, gamma, qdeg_tria=0, qdeg_quad=0, cells=(0, -1)):
    """AssembleMatrixLocally with ReactionDiffusionElementMatrixProvider.

    qdeg = 0 selects the default 2p rule; -1 leaves the cell type without a rule."""
    h = C.c_void_p()
    err = _err()
    _check(lib().lfo_assemble_rd(space.h, C.byref(alpha), C.byref(gamma), qdeg_tria, qdeg_quad, cells[0], cells[1],
                                 C.byref(h), err, 512), err)
    return COO(h, space.num_dofs, space.num_dofs)


def assemble_edge_mass(space, gamma, flags=None, qdeg=0):
    """AssembleMatrixLocally(1, ...) with MassEdgeMatrixProvider on the edges
    with flags[e] != 0 (all edges when flags is None); per-cell coefficient
    data is indexed by edge."""
    h = C.c_void_p()
    err = _err()
    fl = None if flags is None else np.ascontiguousarray(flags, np.uint8)
    _check(lib().lfo_assemble_edge_mass(space.h, C.byref(gamma), _p(fl, C.c_uint8) if fl is not None else None,
                                        qdeg, C.byref(h), err, 512), err)
    return COO(h, space.num_dofs, space.num_dofs)


def assemble_edge_load(space, g, flags=None, qdeg=0, b=None):
    """AssembleVectorLocally(1, ...) with ScalarLoadEdgeVectorProvider."""
    b = np.zeros(space.num_dofs) if b is None else np.ascontiguousarray(b, np.float64).copy()
    err = _err()
    fl = None if flags is None else np.ascontiguousarray(flags, np.uint8)
    _check(lib().lfo_assemble_edge_load(space.h, C.byref(g), _p(fl, C.c_uint8) if fl is not None else None, qdeg,
                                        _p(b, C.c_double), err, 512), err)
    return b


def assemble_load(space, f, qdeg_tria=0, qdeg_quad=0, b=None):
    b = np.zeros(space.num_dofs) if b is None else np.ascontiguousarray(b, np.float64).copy()
    err = _err()
    _check(lib().lfo_assemble_load(space.h, C.byref(f), qdeg_tria, qdeg_quad, _p(b, C.c_double), err, 512), err)
    return b


def assemble_tabulated(space, elem, vec_elem=None):
    """AssembleMatrixLocally/AssembleVectorLocally with a provider that returns
    the given element matrices elem[cell] (ld x ld, row major)."""
    elem = np.ascontiguousarray(elem, np.float64)
    ld = elem.shape[1]
    h = C.c_void_p()
    err = _err()
    b = None
    if vec_elem is not None:
        vec_elem = np.ascontiguousarray(vec_elem, np.float64)
        b = np.zeros(space.num_dofs)
    _check(lib().lfo_assemble_tabulated(space.h, _p(elem, C.c_double), ld,
                                        _p(vec_elem, C.c_double) if vec_elem is not None else None,
                                        _p(b, C.c_double) if b is not None else None, C.byref(h), err, 512), err)
    return COO(h, space.num_dofs, space.num_dofs), b


def nodal_projection(space, func, params):
    out = np.zeros(space.num_dofs)
    p = np.zeros(16)
    p[: len(params)] = params
    err = _err()
    _check(lib().lfo_nodal_projection(space.h, func, _p(p, C.c_double), _p(out, C.c_double), err, 512), err)
    return out


def quad_rule(is_quad, degree):
    n = C.c_int()
    err = _err()
    _check(lib().lfo_quad_rule(int(is_quad), degree, None, None, None, C.byref(n), err, 512), err)
    x, y, w = np.zeros(n.value), np.zeros(n.value), np.zeros(n.value)
    _check(lib().lfo_quad_rule(int(is_quad), degree, _p(x, C.c_double), _p(y, C.c_double), _p(w, C.c_double),
                               C.byref(n), err, 512), err)
    return x, y, w


def kat_tensor_rd():
    v = C.c_double()
    err = _err()
    _check(lib().lfo_kat_tensor_rd(C.byref(v), err, 512), err)
    return v.value


def assemble_rd_parallel(space, alpha, gamma, qdeg_tria=0, qdeg_quad=0, cells=(0, -1), threads=1):
    """Threaded cell-range assembly (same triplets as assemble_rd); returns
    (wall seconds, number of triplets)."""
    L = lib()
    if not hasattr(L, "_par_declared"):
        L.lfo_assemble_rd_parallel.argtypes = [C.c_void_p, C.POINTER(lfo_coeff), C.POINTER(lfo_coeff), C.c_int,
                                               C.c_int, C.c_int64, C.c_int64, C.c_int, C.POINTER(C.c_double),
                                               C.POINTER(C.c_int64), C.c_char_p, C.c_int]
        L._par_declared = True
    sec = C.c_double()
    n = C.c_int64()
    err = _err()
    _check(L.lfo_assemble_rd_parallel(space.h, C.byref(alpha), C.byref(gamma), qdeg_tria, qdeg_quad, cells[0],
                                      cells[1], threads, C.byref(sec), C.byref(n), err, 512), err)
    return sec.value, n.value


# ------------------------------------------------------------ differentiation
# CPU FP64 reference gradient of J(theta) = 1/2 ||u - u_obs||^2 with
# alpha = exp(theta) per cell and gamma = 0 (no reference counterpart; built
# from the restated ReactionDiffusionElementMatrixProvider, which gives A_K,
# and two sparse LU solves of the fixed system).

def element_blocks(space):
    """Start offsets of the per-cell n_K^2 triplet blocks of assemble_rd."""
    cells = space.mesh.cells
    sizes = np.where(cells[:, 3] >= 0, space.n_quad ** 2, space.n_tria ** 2)
    return np.concatenate([[0], np.cumsum(sizes)])


def cellwise_bilinear(space, A, lam, u):
    """Per cell sum_{ij} lam[dof_i] A_K(i,j) u[dof_j] over the cell-ordered
    triplet blocks of an (unfixed) assemble_rd matrix."""
    r, c, v = A.arrays()
    offs = element_blocks(space)
    return np.add.reduceat(lam[r] * v * u[c], offs[:-1])


def adjoint_gradient(space, theta, f, u_obs, flags, g=None, qdeg_tria=0, qdeg_quad=0):
    """J, u, lambda and dJ/dtheta in FP64: assemble, fix, SparseLU for u and
    for the adjoint A lambda = (u - u_obs) on free dofs, then
    dJ/dtheta_c = -sum_{i free, j} lambda_i A_K(i,j) u_j."""
    import scipy.sparse.linalg as spla
    nd = space.num_dofs
    g = np.zeros(nd) if g is None else np.asarray(g, np.float64)
    A = assemble_rd(space, coeff(PER_CELL_EXP, data=theta), coeff(ZERO), qdeg_tria, qdeg_quad)
    Af = assemble_rd(space, coeff(PER_CELL_EXP, data=theta), coeff(ZERO), qdeg_tria, qdeg_quad)
    b = assemble_load(space, f)
    Af.fix_flagged(flags, g, b)
    lu = spla.splu(Af.to_scipy().tocsc())
    u = lu.solve(b)
    r = u - u_obs
    J = 0.5 * float(r @ r)
    rhs = np.where(flags != 0, 0.0, r)
    lam = lu.solve(rhs)
    lam_m = np.where(flags != 0, 0.0, lam)
    grad = -cellwise_bilinear(space, A, lam_m, u)
    return J, u, lam, grad


def _u8(a):
    if a is None:
        return None, None
    a = np.ascontiguousarray(a, np.uint8)
    return a, _p(a, C.c_uint8)


def integrate(space, kind, u=None, dofs=None, qdeg=2, flags=None, codim=0):
    """IntegrateMeshFunction of the closed integrands (INT_*); u a coeff (None: zero)."""
    u = coeff(ZERO) if u is None else u
    d = None if dofs is None else np.ascontiguousarray(dofs, np.float64)
    fl, flp = _u8(flags)
    out = C.c_double()
    err = _err()
    _check(lib().lfo_integrate(space.h, kind, C.byref(u), _p(d, C.c_double) if d is not None else None, qdeg, flp,
                               codim, C.byref(out), err, 512), err)
    return out.value


def eval_fe(space, dofs, ref_points, grads=False):
    """MeshFunctionFE (and MeshFunctionGradFE) on every cell at reference points [k][2]."""
    pts = np.ascontiguousarray(ref_points, np.float64).reshape(-1, 2)
    d = np.ascontiguousarray(dofs, np.float64)
    nc = space.mesh.num_cells
    vals = np.zeros((nc, len(pts)))
    g = np.zeros((nc, len(pts), 2)) if grads else None
    err = _err()
    _check(lib().lfo_eval_fe(space.h, _p(d, C.c_double), len(pts), _p(pts, C.c_double), _p(vals, C.c_double),
                             _p(g, C.c_double) if grads else None, err, 512), err)
    return (vals, g) if grads else vals


def nodal_projection_mf(space, u, cell_flags=None):
    """NodalProjection of a mesh function (coeff) onto a Lagrangian space."""
    out = np.zeros(space.num_dofs)
    fl, flp = _u8(cell_flags)
    err = _err()
    _check(lib().lfo_nodal_projection_mf(space.h, C.byref(u), flp, _p(out, C.c_double), err, 512), err)
    return out


def init_essential_condition(space, edge_flags, g):
    """InitEssentialConditionFromFunction: (flags uint8, values) per dof."""
    fl, flp = _u8(edge_flags)
    f = np.zeros(space.num_dofs, np.uint8)
    v = np.zeros(space.num_dofs)
    err = _err()
    _check(lib().lfo_init_essential(space.h, flp, C.byref(g), _p(f, C.c_uint8), _p(v, C.c_double), err, 512), err)
    return f, v


# ----------------------------------------------------------- hierarchic FE

def hier_space(mesh, p):
    """HierarchicScalarFESpace(mesh, p): the uniform dof layout (1, p-1, tria, quad interior)."""
    return Space(mesh, 0, (1, p - 1, max(0, (p - 1) * (p - 2) // 2), (p - 1) * (p - 1)))


def hier_var_space(mesh, edge_deg, cell_deg):
    """HierarchicScalarFESpace(mesh, degree_functor) with the functor's values
    per edge (edge order) and per cell (cell order), numbered like
    DynamicFEDofHandler.  Assemble on it with p = 0."""
    sp = Space.__new__(Space)
    sp.mesh = mesh
    sp.degree = 0
    sp.h = C.c_void_p()
    ed = np.ascontiguousarray(edge_deg, np.int32)
    cd = np.ascontiguousarray(cell_deg, np.int32)
    err = _err()
    _check(lib().lfo_space_create_hier_var(mesh.h, _p(ed, C.c_int32), _p(cd, C.c_int32), C.byref(sp.h), err, 512),
           err)
    info = np.zeros(4, np.int64)
    lib().lfo_space_info(sp.h, _p(info, C.c_int64))
    sp.num_dofs, sp.n_cell, sp.n_tria, sp.n_quad = (int(v) for v in info)
    return sp


def assemble_hier(space, p, alpha, gamma, qdeg=0):
    h = C.c_void_p()
    err = _err()
    _check(lib().lfo_assemble_hier(space.h, p, C.byref(alpha), C.byref(gamma), qdeg, C.byref(h), err, 512), err)
    return COO(h, space.num_dofs, space.num_dofs)


def assemble_hier_load(space, p, f, qdeg=0, b=None):
    b = np.zeros(space.num_dofs) if b is None else np.ascontiguousarray(b, np.float64).copy()
    err = _err()
    _check(lib().lfo_assemble_hier_load(space.h, p, C.byref(f), qdeg, _p(b, C.c_double), err, 512), err)
    return b


def hier_shape(is_quad, p, ori, pts):
    """Shape values (k, n) and reference gradients (k, n, 2) of FeHierarchicTria/Quad."""
    pts = np.ascontiguousarray(pts, np.float64).reshape(-1, 2)
    n = (p + 1) ** 2 if is_quad else (p + 1) * (p + 2) // 2
    o = np.ascontiguousarray(list(ori) + [1] * (4 - len(ori)), np.int8)
    phi = np.zeros((len(pts), n))
    dphi = np.zeros((len(pts), n, 2))
    err = _err()
    _check(lib().lfo_hier_shape(int(is_quad), p, _p(o, C.c_int8), len(pts), _p(pts, C.c_double),
                                _p(phi, C.c_double), _p(dphi, C.c_double), err, 512), err)
    return phi, dphi


def hier_shape_var(is_quad, pc, pe, ori, pts):
    """Shapes of FeHierarchicTria/Quad with interior degree pc and edge degrees pe."""
    pts = np.ascontiguousarray(pts, np.float64).reshape(-1, 2)
    nv = 4 if is_quad else 3
    pe4 = np.ascontiguousarray(list(pe) + [1] * (4 - len(pe)), np.int32)
    n = nv + sum(int(d) - 1 for d in pe[:nv])
    n += (pc - 1) ** 2 if is_quad else (0 if pc <= 2 else (pc - 2) * (pc - 1) // 2)
    o = np.ascontiguousarray(list(ori) + [1] * (4 - len(ori)), np.int8)
    phi = np.zeros((len(pts), n))
    dphi = np.zeros((len(pts), n, 2))
    err = _err()
    _check(lib().lfo_hier_shape_var(int(is_quad), pc, _p(pe4, C.c_int32), _p(o, C.c_int8), len(pts),
                                    _p(pts, C.c_double), _p(phi, C.c_double), _p(dphi, C.c_double), err, 512), err)
    return phi, dphi


def hier_dual(is_quad, pc, pe, ori):
    """EvaluationNodes (ne, 2) and the NodalValuesToDofs matrix M (n, ne) of
    FeHierarchicTria/Quad(pc, pe, ori): dofs = M @ values at the nodes."""
    pe4 = np.ascontiguousarray(list(pe) + [1] * (4 - len(pe)), np.int32)
    o = np.ascontiguousarray(list(ori) + [1] * (4 - len(ori)), np.int8)
    ne, n = C.c_int(), C.c_int()
    err = _err()
    _check(lib().lfo_hier_dual(int(is_quad), pc, _p(pe4, C.c_int32), _p(o, C.c_int8), None, None, C.byref(ne),
                               C.byref(n), err, 512), err)
    xy = np.zeros((ne.value, 2))
    M = np.zeros((n.value, ne.value))
    _check(lib().lfo_hier_dual(int(is_quad), pc, _p(pe4, C.c_int32), _p(o, C.c_int8), _p(xy, C.c_double),
                               _p(M, C.c_double), C.byref(ne), C.byref(n), err, 512), err)
    return xy, M


def nodal_projection_hier(space, p, u, cell_flags=None):
    """NodalProjection of a mesh function (coeff) onto a hierarchic space of
    uniform degree p (p = 0: a hier_var_space)."""
    out = np.zeros(space.num_dofs)
    fl, flp = _u8(cell_flags)
    err = _err()
    _check(lib().lfo_nodal_projection_hier(space.h, p, C.byref(u), flp, _p(out, C.c_double), err, 512), err)
    return out


def integrate_hier(space, p, kind, u, dofs=None, qdeg=4, flags=None):
    """IntegrateMeshFunction over the cells with u_h (dofs) on a hierarchic
    space of uniform degree p (p = 0: a hier_var_space)."""
    out = C.c_double()
    d = None if dofs is None else np.ascontiguousarray(dofs, np.float64)
    fl, flp = _u8(flags)
    err = _err()
    _check(lib().lfo_integrate_hier(space.h, p, kind, C.byref(u), _p(d, C.c_double) if d is not None else None, qdeg,
                                    flp, C.byref(out), err, 512), err)
    return out.value


def eval_fe_hier(space, p, dofs, pts):
    """MeshFunctionFE / GradFE of u_h on a hierarchic space (uniform degree p,
    0: per entity) at reference points pts (k, 2) of every cell: values
    (cells, k) and gradients (cells, k, 2)."""
    pts = np.ascontiguousarray(pts, np.float64).reshape(-1, 2)
    d = np.ascontiguousarray(dofs, np.float64)
    nc = space.mesh.num_cells
    vals = np.zeros((nc, len(pts)))
    grads = np.zeros((nc, len(pts), 2))
    err = _err()
    _check(lib().lfo_eval_fe_hier(space.h, p, _p(d, C.c_double), len(pts), _p(pts, C.c_double), _p(vals, C.c_double),
                                  _p(grads, C.c_double), err, 512), err)
    return vals, grads


def hier_fn(which, n, a, b, x):
    """0 Legendre(n,x,t=a) 1 ILegendre 2 ILegendreDx 3 ILegendreDt 4 Jacobi(n,a,b,x) 5 IJacobi(n,a,x)."""
    return lib().lfo_hier_fn(which, n, a, b, x)
