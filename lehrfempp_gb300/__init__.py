"""GB300-native LehrFEM++ assembly-and-solve path (Python binding of the C-ABI).

The compute path is the CUDA library lehrfempp_gb300/_build/liblfg.so built
from csrc/ for sm_103a; this module only marshals arguments through ctypes.
There is no CPU fallback: without the library or a GPU every call raises.

Names follow the reference (lf::mesh / lf::assemble / lf::uscalfe):
  Mesh              hybrid2d::MeshFactory + Build, TPTriag/TPQuadMeshBuilder
  Space             UniformFEDofHandler / FeSpaceLagrangeO{1,2,3}
  COOMatrix         assemble::COOMatrix<double> on the device
  assemble_matrix_rd   AssembleMatrixLocally + ReactionDiffusionElementMatrixProvider
  assemble_vector_load AssembleVectorLocally + ScalarLoadElementVectorProvider
  COOMatrix.fix_flagged_solution_components   FixFlaggedSolutionComponents
  COOMatrix.make_sparse                        COOMatrix::makeSparse (CSR)
  CSRMatrix.solve_pcg                          Jacobi-PCG, FP64 or mixed precision
"""
import ctypes as C
import os
import threading

import numpy as np

from . import _capi
from ._capi import (lfg_edge_load_provider, lfg_edge_mass_provider, lfg_rd_adjoint_opts, lfg_coeff, lfg_load_provider, lfg_rd_provider, lfg_solve_opts, lfg_solve_stats,
                    lfg_triplet)

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "liblfg.so")
_lib = None
_lock = threading.Lock()

# status codes (include/lfg.h)
OK, INVALID_ARG, DEGENERATE_CELL, CAPACITY, UNSUPPORTED, NOT_CONVERGED, CUDA_ERROR, MISSING_RULE, \
    INCOMPLETE_MESH, OUT_OF_MEMORY, IO_ERROR, NOT_FOUND = range(12)
STATUS_NAMES = ["OK", "INVALID_ARG", "DEGENERATE_CELL", "CAPACITY", "UNSUPPORTED", "NOT_CONVERGED",
                "CUDA_ERROR", "MISSING_RULE", "INCOMPLETE_MESH", "OUT_OF_MEMORY", "IO_ERROR", "NOT_FOUND"]

# coefficient kinds and analytic families
ZERO, CONSTANT, PER_CELL, NODAL_O1, ANALYTIC, PER_CELL_EXP = 0, 1, 2, 3, 4, 5
# matrix-valued diffusion coefficients (row-major 2x2): constant p[0..3], per cell
# data[4 cell + e], bilinear entries p[4e] + p[4e+1] x + p[4e+2] y + p[4e+3] x y
TENSOR_CONSTANT, TENSOR_PER_CELL, TENSOR_BILINEAR = 6, 7, 8
FN_POLY, FN_SINSIN, FN_SINCOS, FN_EXP, FN_TRIG = 1, 2, 3, 4, 5
# integrands of integrate_mesh_function
INT_VALUE, INT_SQ_DIFF, INT_GRAD_SQ_DIFF = 0, 1, 2
SOLVE_FP64, SOLVE_MIXED = 0, 1

TRIPLET_DTYPE = np.dtype([("row", np.int32), ("col", np.int32), ("value", np.float64)])


class LfgError(RuntimeError):
    def __init__(self, code, msg):
        self.code = code
        super().__init__("%s: %s" % (STATUS_NAMES[code] if 0 <= code < len(STATUS_NAMES) else code, msg))


def build(force=False, verbose=False):
    from . import builder
    return builder.build(force=force, verbose=verbose)


def load(build_if_missing=True):
    """Load liblfg.so (building it with nvcc first if it is missing)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                if not build_if_missing:
                    raise RuntimeError("GPU library %s is missing: run lehrfempp_gb300.build()" % LIB_PATH)
                build()
            _lib = _capi.declare(C.CDLL(LIB_PATH))
    return _lib


def lib():
    return load()


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


class Context:
    """lfg_ctx: one device, one CUDA stream."""

    def __init__(self, device=0):
        L = lib()
        self.h = C.c_void_p()
        rc = L.lfg_ctx_create(device, C.byref(self.h))
        if rc != OK:
            raise LfgError(rc, "could not create a CUDA context on device %d (is a GPU visible?)" % device)
        self._children = []

    def check(self, rc):
        if rc != OK:
            msg = lib().lfg_ctx_last_error(self.h)
            raise LfgError(rc, msg.decode(errors="replace") if msg else "")

    def close(self):
        if self.h:
            lib().lfg_ctx_synchronize(self.h)
            lib().lfg_ctx_destroy(self.h)
            self.h = None

    def synchronize(self):
        self.check(lib().lfg_ctx_synchronize(self.h))

    def launches(self):
        n = C.c_int64()
        self.check(lib().lfg_ctx_launch_count(self.h, C.byref(n)))
        return n.value

    # memory
    def empty(self, shape, dtype):
        return DeviceArray(self, shape, dtype)

    def to_device(self, a):
        a = np.ascontiguousarray(a)
        d = DeviceArray(self, a.shape, a.dtype)
        d.upload(a)
        return d

    def zeros(self, shape, dtype=np.float64):
        d = DeviceArray(self, shape, dtype)
        d.fill_zero()
        return d

    # timing on the context stream
    def timer_begin(self):
        self.check(lib().lfg_timer_begin(self.h))

    def timer_end(self):
        ms = C.c_float()
        self.check(lib().lfg_timer_end(self.h, C.byref(ms)))
        return ms.value

    def l2_flush(self):
        self.check(lib().lfg_l2_flush(self.h))

    def pinned(self, shape, dtype):
        return PinnedArray(self, shape, dtype)

    # per-kernel-family event timing
    def profile(self, enable=True):
        self.check(lib().lfg_profile_enable(self.h, int(enable)))

    def profile_read(self, family):
        ms, n = C.c_double(), C.c_int64()
        self.check(lib().lfg_profile_read(self.h, family.encode(), C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def profile_reset(self):
        self.check(lib().lfg_profile_reset(self.h))

    def set_tensor_cores(self, enable):
        """Q2 quadrilateral element matrices on the tcgen05 tensor cores
        (True / 3: warp-specialised with the triplet writes in the producer
        warps, the default; 1: warp-specialised with the consumer warps
        writing; 2: the two-CTA variant) or on the df32 CUDA-core kernel
        (False / 0)."""
        mode = int(enable) if not isinstance(enable, bool) else (3 if enable else 0)
        self.check(lib().lfg_ctx_set_tensor_cores(self.h, mode))

    def fp64_peak_tflops(self):
        t = C.c_double()
        self.check(lib().lfg_measure_fp64_peak(self.h, C.byref(t)))
        return t.value


class DeviceArray:
    """A device allocation made through lfg_malloc (stream ordered)."""

    def __init__(self, ctx, shape, dtype):
        self.ctx = ctx
        self.shape = tuple(np.atleast_1d(shape)) if not isinstance(shape, tuple) else shape
        self.dtype = np.dtype(dtype)
        self.nbytes = int(np.prod(self.shape)) * self.dtype.itemsize
        self.ptr = C.c_void_p()
        ctx.check(lib().lfg_malloc(ctx.h, self.nbytes, C.byref(self.ptr)))

    @property
    def size(self):
        return int(np.prod(self.shape))

    def __del__(self):
        try:
            if self.ptr and self.ctx.h:
                lib().lfg_free(self.ctx.h, self.ptr)
        except Exception:
            pass
        self.ptr = None

    def upload(self, a):
        a = np.ascontiguousarray(a, dtype=self.dtype)
        assert a.nbytes == self.nbytes, (a.nbytes, self.nbytes)
        self.ctx.check(lib().lfg_memcpy_h2d(self.ctx.h, self.ptr, a.ctypes.data, self.nbytes))
        self.ctx.synchronize()  # the host buffer may be temporary

    def upload_async(self, host):
        """Copy from a PinnedArray without synchronizing."""
        self.ctx.check(lib().lfg_memcpy_h2d(self.ctx.h, self.ptr, host.ptr, self.nbytes))

    def download(self):
        out = np.empty(self.shape, self.dtype)
        self.ctx.check(lib().lfg_memcpy_d2h(self.ctx.h, out.ctypes.data, self.ptr, self.nbytes))
        return out

    def download_into(self, host):
        self.ctx.check(lib().lfg_memcpy_d2h(self.ctx.h, host.ptr, self.ptr, self.nbytes))

    def fill_zero(self):
        self.ctx.check(lib().lfg_memset(self.ctx.h, self.ptr, 0, self.nbytes))

    def copy_from(self, other):
        self.ctx.check(lib().lfg_memcpy_d2d(self.ctx.h, self.ptr, other.ptr, self.nbytes))


class PinnedArray:
    """Page-locked host memory (cudaMallocHost) viewed as a numpy array."""

    def __init__(self, ctx, shape, dtype):
        self.ctx = ctx
        self.dtype = np.dtype(dtype)
        self.shape = shape if isinstance(shape, tuple) else (int(shape),)
        self.nbytes = int(np.prod(self.shape)) * self.dtype.itemsize
        self.ptr = C.c_void_p()
        ctx.check(lib().lfg_host_alloc(ctx.h, max(self.nbytes, 1), C.byref(self.ptr)))
        buf = (C.c_char * max(self.nbytes, 1)).from_address(self.ptr.value)
        self.array = np.frombuffer(buf, dtype=self.dtype, count=int(np.prod(self.shape))).reshape(self.shape)

    def __del__(self):
        try:
            if self.ptr and self.ctx.h:
                lib().lfg_host_free(self.ctx.h, self.ptr)
        except Exception:
            pass
        self.ptr = None


def coeff(kind=ZERO, value=0.0, data=None, func=0, params=()):
    """lfg_coeff: data is a DeviceArray (per cell / per node) or None."""
    c = lfg_coeff()
    c.kind = kind
    c.value = value
    c.func = func
    c.data_dev = data.ptr.value if data is not None else None
    for i, v in enumerate(params):
        c.p[i] = v
    return c


class Mesh:
    """A 2D hybrid mesh on the device (hybrid2d::Mesh numbering)."""

    def __init__(self, ctx, h):
        self.ctx = ctx
        self.h = h
        nv, ne, nc, nt, nq = (C.c_int64() for _ in range(5))
        ctx.check(lib().lfg_mesh_sizes(h, C.byref(nv), C.byref(ne), C.byref(nc), C.byref(nt), C.byref(nq)))
        self.num_nodes, self.num_edges, self.num_cells = nv.value, ne.value, nc.value
        self.num_trias, self.num_quads = nt.value, nq.value

    @classmethod
    def from_factory(cls, ctx, xy, cells, preset_edges=None):
        """MeshFactory::AddPoint / AddEntity / Build from arrays (cells: 4 per cell, -1 pad)."""
        xy = np.ascontiguousarray(xy, np.float64).reshape(-1, 2)
        cells = np.ascontiguousarray(cells, np.int32).reshape(-1, 4)
        pe = None if preset_edges is None or len(preset_edges) == 0 else \
            np.ascontiguousarray(preset_edges, np.int32).reshape(-1, 2)
        h = C.c_void_p()
        ctx.check(lib().lfg_mesh_create(ctx.h, len(xy), _p(xy, C.c_double), len(cells), _p(cells, C.c_int32),
                                        0 if pe is None else len(pe), None if pe is None else _p(pe, C.c_int32),
                                        C.byref(h)))
        return cls(ctx, h)

    @classmethod
    def tp_triag(cls, ctx, nx, ny, x0=0.0, y0=0.0, x1=1.0, y1=1.0):
        h = C.c_void_p()
        ctx.check(lib().lfg_mesh_create_tp_triag(ctx.h, nx, ny, x0, y0, x1, y1, C.byref(h)))
        return cls(ctx, h)

    @classmethod
    def tp_quad(cls, ctx, nx, ny, x0=0.0, y0=0.0, x1=1.0, y1=1.0):
        h = C.c_void_p()
        ctx.check(lib().lfg_mesh_create_tp_quad(ctx.h, nx, ny, x0, y0, x1, y1, C.byref(h)))
        return cls(ctx, h)

    def __del__(self):
        try:
            if self.h:
                lib().lfg_mesh_destroy(self.h)
        except Exception:
            pass
        self.h = None

    def topology(self):
        en = np.zeros((self.num_edges, 2), np.int32)
        ce = np.zeros((self.num_cells, 4), np.int32)
        co = np.zeros((self.num_cells, 4), np.int8)
        nc = np.zeros(self.num_edges, np.int32)
        self.ctx.check(lib().lfg_mesh_download_topology(self.h, _p(en, C.c_int32), _p(ce, C.c_int32),
                                                        _p(co, C.c_int8), _p(nc, C.c_int32)))
        return en, ce, co, nc

    def boundary_flags(self):
        nf = self.ctx.empty(self.num_nodes, np.uint8)
        ef = self.ctx.empty(max(self.num_edges, 1), np.uint8)
        self.ctx.check(lib().lfg_mesh_boundary_flags(self.h, nf.ptr, ef.ptr))
        return nf.download(), ef.download()[: self.num_edges]

    def set_coords(self, xy):
        if isinstance(xy, DeviceArray):
            self.ctx.check(lib().lfg_mesh_set_coords(self.h, xy.ptr, 1))
        else:
            xy = np.ascontiguousarray(xy, np.float64)
            self.ctx.check(lib().lfg_mesh_set_coords(self.h, xy.ctypes.data_as(C.c_void_p), 0))
            self.ctx.synchronize()

    def device_arrays(self):
        xy, cells = C.c_void_p(), C.c_void_p()
        self.ctx.check(lib().lfg_mesh_device_arrays(self.h, C.byref(xy), C.byref(cells)))
        return xy, cells

    def geometry(self):
        """(xy[num_nodes, 2] float64, cells[num_cells, 4] int32; -1 pads triangles)."""
        dxy, dcells = self.device_arrays()
        xy = np.zeros((self.num_nodes, 2), np.float64)
        cells = np.zeros((self.num_cells, 4), np.int32)
        self.ctx.check(lib().lfg_memcpy_d2h(self.ctx.h, xy.ctypes.data_as(C.c_void_p), dxy, xy.nbytes))
        self.ctx.check(lib().lfg_memcpy_d2h(self.ctx.h, cells.ctypes.data_as(C.c_void_p), dcells, cells.nbytes))
        self.ctx.synchronize()
        return xy, cells


class Space:
    """UniformFEDofHandler; Space.lagrange(mesh, p) = FeSpaceLagrangeO<p>."""

    def __init__(self, mesh, h, degree):
        self.mesh = mesh
        self.ctx = mesh.ctx
        self.h = h
        self.degree = degree
        nd, nt, nq, ncs, ntr = C.c_int64(), C.c_int32(), C.c_int32(), C.c_int32(), C.c_int64()
        self.ctx.check(lib().lfg_space_info(h, C.byref(nd), C.byref(nt), C.byref(nq), C.byref(ncs), C.byref(ntr)))
        self.num_dofs, self.n_tria, self.n_quad, self.n_cell = nd.value, nt.value, nq.value, ncs.value
        self.num_triplets = ntr.value

    @classmethod
    def lagrange(cls, mesh, degree):
        h = C.c_void_p()
        mesh.ctx.check(lib().lfg_space_create_lagrange(mesh.h, degree, C.byref(h)))
        return cls(mesh, h, degree)

    @classmethod
    def hierarchic(cls, mesh, degree):
        """fe::HierarchicScalarFESpace(mesh, degree) (uniform degree 1..20)."""
        h = C.c_void_p()
        mesh.ctx.check(lib().lfg_space_create_hierarchic(mesh.h, degree, C.byref(h)))
        sp = cls(mesh, h, 0)
        sp.hier_degree = degree
        return sp

    @classmethod
    def hierarchic_var(cls, mesh, edge_degree, cell_degree):
        """fe::HierarchicScalarFESpace(mesh, degree_functor): the functor's value
        per edge (edge order) and per cell (cell order), each 1..20."""
        ed = np.ascontiguousarray(edge_degree, np.int32)
        cd = np.ascontiguousarray(cell_degree, np.int32)
        if len(ed) != mesh.num_edges or len(cd) != mesh.num_cells:
            raise ValueError("one degree per edge and per cell expected")
        h = C.c_void_p()
        mesh.ctx.check(lib().lfg_space_create_hierarchic_var(mesh.h, _p(ed, C.c_int32), _p(cd, C.c_int32),
                                                             C.byref(h)))
        sp = cls(mesh, h, 0)
        sp.hier_degree = int(max(ed.max(initial=1), cd.max(initial=1)))
        return sp

    def local_counts(self):
        """NumLocalDofs of every cell."""
        out = np.zeros(self.mesh.num_cells, np.int32)
        self.ctx.check(lib().lfg_space_download_local_counts(self.h, _p(out, C.c_int32)))
        return out

    @classmethod
    def layout(cls, mesh, np_, ns, nt, nq):
        h = C.c_void_p()
        mesh.ctx.check(lib().lfg_space_create(mesh.h, np_, ns, nt, nq, C.byref(h)))
        return cls(mesh, h, 0)

    def __del__(self):
        try:
            if self.h:
                lib().lfg_space_destroy(self.h)
        except Exception:
            pass
        self.h = None

    def cell_dofs(self):
        out = np.zeros((self.mesh.num_cells, self.n_cell), np.int32)
        self.ctx.check(lib().lfg_space_download_cell_dofs(self.h, _p(out, C.c_int32)))
        return out

    def dof_entities(self):
        cod = np.zeros(self.num_dofs, np.int8)
        idx = np.zeros(self.num_dofs, np.int32)
        self.ctx.check(lib().lfg_space_download_dof_entities(self.h, _p(cod, C.c_int8), _p(idx, C.c_int32)))
        return cod, idx

    def boundary_dof_flags(self):
        f = self.ctx.empty(self.num_dofs, np.uint8)
        self.ctx.check(lib().lfg_space_boundary_dof_flags(self.h, f.ptr))
        return f


class COOMatrix:
    """assemble::COOMatrix<double> held in device memory."""

    def __init__(self, ctx, rows, cols, capacity):
        self.ctx = ctx
        self.h = C.c_void_p()
        ctx.check(lib().lfg_coo_create(ctx.h, rows, cols, capacity, C.byref(self.h)))
        self.rows, self.cols, self.capacity = rows, cols, capacity

    def __del__(self):
        try:
            if self.h:
                lib().lfg_coo_destroy(self.h)
        except Exception:
            pass
        self.h = None

    def __len__(self):
        n = C.c_int64()
        self.ctx.check(lib().lfg_coo_size(self.h, C.byref(n)))
        return n.value

    def set_zero(self):
        self.ctx.check(lib().lfg_coo_set_zero(self.h))

    def triplets(self):
        n = len(self)
        out = np.zeros(n, TRIPLET_DTYPE)
        if n:
            self.ctx.check(lib().lfg_coo_download(self.h, out.ctypes.data, n))
        return out

    def download_into(self, pinned, count=None):
        n = len(self) if count is None else count
        self.ctx.check(lib().lfg_coo_download(self.h, pinned.ptr, n))

    def triplets_range(self, lo, hi):
        """Triplets [lo, hi) of the matrix (host copy of one slice)."""
        n = len(self)
        if not 0 <= lo <= hi <= n:
            raise ValueError("triplet range [%d, %d) outside [0, %d)" % (lo, hi, n))
        out = np.zeros(hi - lo, TRIPLET_DTYPE)
        if hi > lo:
            d = C.c_void_p()
            self.ctx.check(lib().lfg_coo_triplets(self.h, C.byref(d)))
            self.ctx.check(lib().lfg_memcpy_d2h(self.ctx.h, out.ctypes.data, C.c_void_p(d.value + 16 * lo),
                                                16 * (hi - lo)))
        return out

    def append(self, rows, cols, vals):
        t = np.zeros(len(vals), TRIPLET_DTYPE)
        t["row"], t["col"], t["value"] = rows, cols, vals
        self.ctx.check(lib().lfg_coo_append_host(self.h, t.ctypes.data, len(t)))
        self.ctx.synchronize()

    def fix_flagged_solution_components(self, flags, values, b):
        self.ctx.check(lib().lfg_fix_flagged_solution_components(self.h, flags.ptr, values.ptr, b.ptr))

    def fix_flagged_solution_comp_alt(self, flags, values, b):
        self.ctx.check(lib().lfg_fix_flagged_solution_comp_alt(self.h, flags.ptr, values.ptr, b.ptr))

    def fix_solution_components_lse(self, dofs, values, b):
        """FixSolutionComponentsLse: `dofs` / `values` are the (dof, value)
        pairs in list order (device arrays of int64 / float64, or host
        arrays, which are copied to the device)."""
        if not isinstance(dofs, DeviceArray):
            dofs = self.ctx.to_device(np.ascontiguousarray(dofs, np.int64))
        if not isinstance(values, DeviceArray):
            values = self.ctx.to_device(np.ascontiguousarray(values, np.float64))
        n = dofs.size
        self.ctx.check(lib().lfg_fix_solution_components_lse(self.h, n, dofs.ptr if n else None,
                                                             values.ptr if n else None, b.ptr))

    def make_sparse(self):
        h = C.c_void_p()
        self.ctx.check(lib().lfg_csr_from_coo(self.h, C.byref(h)))
        return CSRMatrix(self.ctx, h)


class CSRMatrix:
    def __init__(self, ctx, h):
        self.ctx = ctx
        self.h = h
        r, c, n = C.c_int64(), C.c_int64(), C.c_int64()
        ctx.check(lib().lfg_csr_info(h, C.byref(r), C.byref(c), C.byref(n)))
        self.rows, self.cols, self.nnz = r.value, c.value, n.value

    def __del__(self):
        try:
            if self.h:
                lib().lfg_csr_destroy(self.h)
        except Exception:
            pass
        self.h = None

    def download(self):
        rp = np.zeros(self.rows + 1, np.int64)
        col = np.zeros(self.nnz, np.int32)
        val = np.zeros(self.nnz, np.float64)
        self.ctx.check(lib().lfg_csr_download(self.h, _p(rp, C.c_int64), _p(col, C.c_int32), _p(val, C.c_double)))
        return rp, col, val

    def to_scipy(self):
        import scipy.sparse as sp
        rp, col, val = self.download()
        return sp.csr_matrix((val, col, rp), shape=(self.rows, self.cols))

    def spmv(self, x, y):
        self.ctx.check(lib().lfg_csr_spmv(self.h, x.ptr, y.ptr))

    def solve_pcg(self, b, x, precision=SOLVE_FP64, rtol=1e-10, max_iterations=200000, inner_rtol=0.0,
                  check_every=32, raise_on_failure=True, noalloc=False):
        """Jacobi-PCG; noalloc=True uses lfg_solve_pcg_noalloc (FP64, <= 2^20 rows,
        work vectors in the library's fixed device array, no allocation)."""
        o = lfg_solve_opts()
        o.precision, o.rtol, o.max_iterations, o.inner_rtol, o.check_every = (precision, rtol, max_iterations,
                                                                             inner_rtol, check_every)
        st = lfg_solve_stats()
        fn = lib().lfg_solve_pcg_noalloc if noalloc else lib().lfg_solve_pcg
        rc = fn(self.h, b.ptr, x.ptr, C.byref(o), C.byref(st))
        if rc != OK and (raise_on_failure or rc != NOT_CONVERGED):
            self.ctx.check(rc)
        return {"iterations": st.iterations, "refinements": st.refinements, "rel_residual": st.rel_residual,
                "converged": bool(st.converged)}


class Batch:
    """Many independent spaces viewed as one block-diagonal system (lfg_batch)."""

    def __init__(self, ctx, spaces):
        self.ctx = ctx
        self.spaces = list(spaces)  # keep the spaces (and meshes) alive
        arr = (C.c_void_p * len(self.spaces))(*[s.h.value for s in self.spaces])
        self.h = C.c_void_p()
        ctx.check(lib().lfg_batch_create(ctx.h, len(self.spaces), arr, C.byref(self.h)))
        n, d, c, t = C.c_int32(), C.c_int64(), C.c_int64(), C.c_int64()
        ctx.check(lib().lfg_batch_info(self.h, C.byref(n), C.byref(d), C.byref(c), C.byref(t)))
        self.num_spaces, self.num_dofs, self.num_cells, self.num_triplets = n.value, d.value, c.value, t.value

    def __del__(self):
        try:
            if self.h:
                lib().lfg_batch_destroy(self.h)
        except Exception:
            pass
        self.h = None

    def offsets(self):
        n = self.num_spaces + 1
        d, c, t = np.zeros(n, np.int64), np.zeros(n, np.int64), np.zeros(n, np.int64)
        self.ctx.check(lib().lfg_batch_offsets(self.h, _p(d, C.c_int64), _p(c, C.c_int64), _p(t, C.c_int64)))
        return d, c, t

    def assemble_matrix_rd(self, provider, coo):
        self.ctx.check(lib().lfg_batch_assemble_matrix_rd(self.h, C.byref(provider), coo.h))

    def tuning(self):
        th, ct, ms = C.c_int32(), C.c_int32(), C.c_double()
        self.ctx.check(lib().lfg_batch_tuning(self.h, C.byref(th), C.byref(ct), C.byref(ms)))
        return th.value, ct.value, ms.value

    def solve_tuning(self, precision=SOLVE_MIXED):
        """(rows per chunk, row-iterations/s) chosen by the solver autotuner for
        `precision` (zeros before the first solve in that precision)."""
        cr, rate = C.c_int32(), C.c_double()
        self.ctx.check(lib().lfg_batch_solve_tuning(self.h, precision, C.byref(cr), C.byref(rate)))
        return cr.value, rate.value

    def set_solve_chunk_rows(self, precision, chunk_rows):
        self.ctx.check(lib().lfg_batch_set_solve_chunk_rows(self.h, precision, int(chunk_rows)))

    def set_solve_groups(self, group_bytes):
        """0: lock-step sweep over the whole batch; > 0: L2-sized groups of
        blocks solved one at a time by the persistent cooperative kernel."""
        self.ctx.check(lib().lfg_batch_set_solve_groups(self.h, float(group_bytes)))

    def solve_groups(self):
        v = C.c_double(0.0)
        self.ctx.check(lib().lfg_batch_solve_groups(self.h, C.byref(v)))
        return v.value

    def assemble_vector_load(self, provider, b):
        self.ctx.check(lib().lfg_batch_assemble_vector_load(self.h, C.byref(provider), b.ptr))

    def boundary_dof_flags(self):
        f = self.ctx.empty(self.num_dofs, np.uint8)
        self.ctx.check(lib().lfg_batch_boundary_dof_flags(self.h, f.ptr))
        return f

    def solve_pcg(self, csr, b, x, precision=SOLVE_FP64, rtol=1e-10, max_iterations=200000, inner_rtol=0.0,
                  check_every=32, raise_on_failure=True):
        o = lfg_solve_opts()
        o.precision, o.rtol, o.max_iterations, o.inner_rtol, o.check_every = (precision, rtol, max_iterations,
                                                                             inner_rtol, check_every)
        st = lfg_solve_stats()
        per = (lfg_solve_stats * self.num_spaces)()
        rc = lib().lfg_batch_solve_pcg(self.h, csr.h, b.ptr, x.ptr, C.byref(o), C.byref(st), per)
        if rc != OK and (raise_on_failure or rc != NOT_CONVERGED):
            self.ctx.check(rc)
        blocks = [{"iterations": p.iterations, "refinements": p.refinements, "rel_residual": p.rel_residual,
                   "converged": bool(p.converged)} for p in per]
        return {"iterations": st.iterations, "refinements": st.refinements, "rel_residual": st.rel_residual,
                "converged": bool(st.converged), "blocks": blocks}


def quad_rule(is_quad, degree):
    """make_QuadRule (lib/lf/quad/make_quad_rule.cc:21-157) as the library
    builds it: (x, y, w) arrays of the rule of `degree` on the reference
    triangle or square.  Host-only; no device needed."""
    n = C.c_int32(0)
    rc = lib().lfg_quad_rule(int(is_quad), int(degree), None, None, None, C.byref(n))
    if rc != OK:
        raise LfgError(rc, "lfg_quad_rule(%d, %d) failed" % (int(is_quad), int(degree)))
    x, y, w = np.zeros(n.value), np.zeros(n.value), np.zeros(n.value)
    rc = lib().lfg_quad_rule(int(is_quad), int(degree), _p(x, C.c_double), _p(y, C.c_double), _p(w, C.c_double),
                             C.byref(n))
    if rc != OK:
        raise LfgError(rc, "lfg_quad_rule(%d, %d) failed" % (int(is_quad), int(degree)))
    return x, y, w


def hier_dual(is_quad, interior_degree, edge_degrees, pattern):
    """EvaluationNodes and NodalValuesToDofs of FeHierarchicTria / Quad
    (lib/lf/fe/hierarchic_fe.h:820-1083, 1445-1680) as the library tabulates
    them: nodes (ne, 2) and M (n, ne) with dofs = M @ values.  `pattern` bit j
    set: local edge j negatively oriented.  Host-only; no device needed."""
    pe = np.ascontiguousarray(list(edge_degrees) + [1] * (4 - len(edge_degrees)), np.int32)
    ne, n = C.c_int32(0), C.c_int32(0)
    args = (int(is_quad), int(interior_degree), _p(pe, C.c_int32), int(pattern))
    rc = lib().lfg_hier_dual(*args, None, None, C.byref(ne), C.byref(n))
    if rc != OK:
        raise LfgError(rc, "lfg_hier_dual(%d, %d, %s, %d) failed" % (int(is_quad), interior_degree, list(pe), pattern))
    xy, M = np.zeros((ne.value, 2)), np.zeros((n.value, ne.value))
    rc = lib().lfg_hier_dual(*args, _p(xy, C.c_double), _p(M, C.c_double), C.byref(ne), C.byref(n))
    if rc != OK:
        raise LfgError(rc, "lfg_hier_dual failed")
    return xy, M


def rd_provider(alpha, gamma, qr_degree_tria=0, qr_degree_quad=0):
    p = lfg_rd_provider()
    p.alpha, p.gamma = alpha, gamma
    p.qr_degree_tria, p.qr_degree_quad = qr_degree_tria, qr_degree_quad
    return p


def load_provider(f, qr_degree_tria=0, qr_degree_quad=0):
    p = lfg_load_provider()
    p.f = f
    p.qr_degree_tria, p.qr_degree_quad = qr_degree_tria, qr_degree_quad
    return p


def edge_mass_provider(gamma, flags=None, qr_degree=0):
    """MassEdgeMatrixProvider: gamma on the edges with flags[e] != 0 (a device
    uint8 array; None = every edge).  Per-cell coefficient data is per edge."""
    p = lfg_edge_mass_provider()
    p.gamma = gamma
    p.edge_flags_dev = flags.ptr if flags is not None else None
    p.qr_degree = qr_degree
    p._keep = flags
    return p


def edge_load_provider(g, flags=None, qr_degree=0):
    """ScalarLoadEdgeVectorProvider on the edges with flags[e] != 0."""
    p = lfg_edge_load_provider()
    p.g = g
    p.edge_flags_dev = flags.ptr if flags is not None else None
    p.qr_degree = qr_degree
    p._keep = flags
    return p


def assemble_matrix_edge_mass(space, provider, coo):
    """AssembleMatrixLocally(1, dofh, dofh, MassEdgeMatrixProvider, A)."""
    space.ctx.check(lib().lfg_assemble_matrix_edge_mass(space.h, C.byref(provider), coo.h))


def assemble_vector_edge_load(space, provider, b):
    """AssembleVectorLocally(1, dofh, ScalarLoadEdgeVectorProvider, b)."""
    space.ctx.check(lib().lfg_assemble_vector_edge_load(space.h, C.byref(provider), b.ptr))


def assemble_matrix_rd(space, provider, coo):
    space.ctx.check(lib().lfg_assemble_matrix_rd(space.h, C.byref(provider), coo.h))


def assemble_matrix_rd_to_host(space, provider, out, chunk_triplets=0):
    """AssembleMatrixLocally into host memory: `out` is a PinnedArray (or a
    numpy array) of TRIPLET_DTYPE with at least space.num_triplets entries.
    Pinned memory from ctx.pinned is written by the kernels directly; other
    host memory through a device ring whose downloads overlap the assembly of
    later cell ranges.  Returns the number of triplets written."""
    arr = out.array if isinstance(out, PinnedArray) else out
    assert arr.dtype == TRIPLET_DTYPE and arr.flags.c_contiguous
    n = C.c_int64()
    space.ctx.check(lib().lfg_assemble_matrix_rd_to_host(space.h, C.byref(provider), arr.ctypes.data, len(arr),
                                                         int(chunk_triplets), C.byref(n)))
    return n.value


def assemble_vector_load(space, provider, b):
    space.ctx.check(lib().lfg_assemble_vector_load(space.h, C.byref(provider), b.ptr))


def assemble_matrix_tabulated(space, elem_dev, ld, coo):
    space.ctx.check(lib().lfg_assemble_matrix_tabulated(space.h, elem_dev.ptr, ld, coo.h))


def assemble_vector_tabulated(space, vec_dev, ld, b):
    space.ctx.check(lib().lfg_assemble_vector_tabulated(space.h, vec_dev.ptr, ld, b.ptr))


def loss_l2_misfit(ctx, u, u_obs, misfit=None):
    """J = 1/2 ||u - u_obs||^2 (returned) and, if given, misfit = u - u_obs."""
    out = C.c_double()
    ctx.check(lib().lfg_loss_l2_misfit(ctx.h, u.size, u.ptr, u_obs.ptr, C.byref(out),
                                       misfit.ptr if misfit is not None else None))
    return out.value


def grad_rd_cellwise(space, provider, u, lam, flags, grad):
    """grad[c] = -lambda_K^T (dA_K/dtheta_c) u_K, lambda zero at flagged dofs."""
    space.ctx.check(lib().lfg_grad_rd_cellwise(space.h, C.byref(provider), u.ptr, lam.ptr,
                                               flags.ptr if flags is not None else None, grad.ptr))


# ---------------------------------------------------------------- Gmsh reader

class GmshReader:
    """lf::io::GmshReader (io/gmsh_reader.h) for 2D first-order meshes: MSH
    2.2 / 4.1, ASCII / binary.  The file is parsed on the host (no device
    needed); `mesh` is built on `ctx` when one is given.

        r = GmshReader(ctx, "domain.msh")
        r.mesh                                   # Mesh (device)
        r.physical_entity_nr(1)                  # per edge: physical numbers
        r.is_physical_entity(1, r.physical_entity_name2nr("arc"))  # uint8 flags
    """

    def __init__(self, ctx=None, filename=None, data=None):
        L = lib()
        self.h = C.c_void_p()
        if data is not None:
            buf = bytes(data)
            st = L.lfg_gmsh_open_buffer(buf, len(buf), C.byref(self.h))
        else:
            st = L.lfg_gmsh_open(os.fsencode(filename), C.byref(self.h))
        if st != OK:
            raise LfgError(st, L.lfg_gmsh_last_error().decode(errors="replace"))
        nv, nc, ne = C.c_int64(), C.c_int64(), C.c_int64()
        L.lfg_gmsh_sizes(self.h, C.byref(nv), C.byref(nc), C.byref(ne))
        self.num_nodes, self.num_cells, self.num_preset_edges = nv.value, nc.value, ne.value
        self.mesh = None
        if ctx is not None:
            mh = C.c_void_p()
            ctx.check(L.lfg_gmsh_build_mesh(ctx.h, self.h, C.byref(mh)))
            self.mesh = Mesh(ctx, mh)

    def __del__(self):
        try:
            if self.h:
                lib().lfg_gmsh_destroy(self.h)
        except Exception:
            pass
        self.h = None

    def _check(self, st):
        if st != OK:
            raise LfgError(st, lib().lfg_gmsh_last_error().decode(errors="replace"))

    def factory_input(self):
        """(xy (N, 2), cells (C, 4) int32, preset edges (E, 2) int32): the MeshFactory input."""
        xy = np.zeros((self.num_nodes, 2))
        cells = np.zeros((self.num_cells, 4), np.int32)
        edges = np.zeros((max(self.num_preset_edges, 1), 2), np.int32)
        self._check(lib().lfg_gmsh_factory_input(self.h, _p(xy, C.c_double), _p(cells, C.c_int32),
                                                 _p(edges, C.c_int32)))
        return xy, cells, edges[: self.num_preset_edges]

    def _count(self, codim, num_entities):
        if num_entities is not None:
            return num_entities
        if self.mesh is not None:
            return {0: self.mesh.num_cells, 1: self.mesh.num_edges, 2: self.mesh.num_nodes}[codim]
        return {0: self.num_cells, 1: self.num_preset_edges, 2: self.num_nodes}[codim]

    def physical_entity_nr(self, codim, num_entities=None):
        """PhysicalEntityNr(e) for every entity of `codim`: a list of lists."""
        n = self._count(codim, num_entities)
        off = np.zeros(n + 1, np.int64)
        self._check(lib().lfg_gmsh_physical_entity_nrs(self.h, codim, n, _p(off, C.c_int64), None))
        nrs = np.zeros(max(int(off[-1]), 1), np.int32)
        self._check(lib().lfg_gmsh_physical_entity_nrs(self.h, codim, n, _p(off, C.c_int64), _p(nrs, C.c_int32)))
        return [list(map(int, nrs[off[i]:off[i + 1]])) for i in range(n)]

    def is_physical_entity(self, codim, nr, num_entities=None):
        """IsPhysicalEntity(e, nr) for every entity of `codim` (host uint8 flags)."""
        n = self._count(codim, num_entities)
        fl = np.zeros(max(n, 1), np.uint8)
        self._check(lib().lfg_gmsh_is_physical_entity(self.h, codim, nr, n, _p(fl, C.c_uint8)))
        return fl[:n]

    def physical_entity_name2nr(self, name, codim=-1):
        nr = C.c_int32()
        self._check(lib().lfg_gmsh_name_to_nr(self.h, name.encode(), codim, C.byref(nr)))
        return nr.value

    def physical_entity_nr2name(self, nr, codim=-1):
        buf = C.create_string_buffer(4096)
        self._check(lib().lfg_gmsh_nr_to_name(self.h, nr, codim, buf, len(buf)))
        return buf.value.decode()

    def physical_entities(self, codim):
        """PhysicalEntities(codim): [(nr, name)] in ascending number order."""
        cnt = C.c_int32()
        self._check(lib().lfg_gmsh_physical_entities(self.h, codim, C.byref(cnt), None))
        nrs = np.zeros(max(cnt.value, 1), np.int32)
        self._check(lib().lfg_gmsh_physical_entities(self.h, codim, C.byref(cnt), _p(nrs, C.c_int32)))
        return [(int(n), self.physical_entity_nr2name(int(n), codim)) for n in nrs[: cnt.value]]


# ----------------------------------------------------------- post-processing

def integrate_mesh_function(mesh, kind, u=None, space=None, dofs=None, quad_degree=2, flags=None, codim=0):
    """IntegrateMeshFunction (fe/fe_tools.h:110-165) of the integrand `kind`
    (INT_VALUE: u_h + u, INT_SQ_DIFF: (u_h - u)^2, INT_GRAD_SQ_DIFF:
    |grad u_h - grad u|^2) with u a coeff (None: zero) and u_h given by `space`
    and the DeviceArray `dofs` (None: zero).  flags: device uint8 per entity of
    the codim (None: all; entity 0 always counts, as in the reference)."""
    g = _capi.lfg_integrand()
    g.kind = kind
    g.u = u if u is not None else coeff(ZERO)
    g.space = space.h if space is not None else None
    g.dofs_dev = dofs.ptr if dofs is not None else None
    out = C.c_double()
    mesh.ctx.check(lib().lfg_integrate_mesh_function(mesh.h, C.byref(g), quad_degree,
                                                      flags.ptr if flags is not None else None, codim,
                                                      C.byref(out)))
    return out.value


def fe_eval(space, dofs, ref_points, values=True, grads=False):
    """MeshFunctionFE / MeshFunctionGradFE on every cell at reference points
    [k][2]: DeviceArrays (num_cells, k) and (num_cells, k, 2)."""
    pts = np.ascontiguousarray(ref_points, np.float64).reshape(-1, 2)
    nc = space.mesh.num_cells
    v = DeviceArray(space.ctx, (nc, len(pts)), np.float64) if values else None
    g = DeviceArray(space.ctx, (nc, len(pts), 2), np.float64) if grads else None
    space.ctx.check(lib().lfg_fe_eval(space.h, dofs.ptr, len(pts), _p(pts, C.c_double),
                                      v.ptr if v is not None else None, g.ptr if g is not None else None))
    return v, g


def nodal_projection(space, u, out, cell_flags=None):
    """NodalProjection (fe/fe_tools.h:198-259) of the coeff u into the
    DeviceArray out (num_dofs)."""
    space.ctx.check(lib().lfg_nodal_projection(space.h, C.byref(u), cell_flags.ptr if cell_flags is not None else None,
                                               out.ptr))


def init_essential_condition(space, edge_flags, g, dof_flags, dof_values):
    """InitEssentialConditionFromFunction (fe/fe_tools.h:263-329) into the
    DeviceArrays dof_flags (uint8) and dof_values (double)."""
    space.ctx.check(lib().lfg_init_essential_condition(space.h, edge_flags.ptr, C.byref(g), dof_flags.ptr,
                                                       dof_values.ptr))


class RDAdjoint:
    """theta -> J = 1/2 ||u(theta) - u_obs||^2 as a forward/backward Function
    object (lfg_rd_adjoint_*): alpha = exp(theta) per cell, gamma = 0."""

    def __init__(self, space, u_obs, load, qr_degree_tria=0, qr_degree_quad=0, flags=None, dirichlet=None,
                 precision=SOLVE_FP64, rtol=1e-12, max_iterations=200000, inner_rtol=0.0, check_every=32,
                 recompute=False):
        self.ctx = space.ctx
        self.space = space  # must outlive the object
        o = lfg_rd_adjoint_opts()
        o.load = load
        o.qr_degree_tria, o.qr_degree_quad = qr_degree_tria, qr_degree_quad
        o.flags_dev = flags.ptr if flags is not None else None
        o.dirichlet_dev = dirichlet.ptr if dirichlet is not None else None
        o.solve.precision, o.solve.rtol, o.solve.max_iterations = precision, rtol, max_iterations
        o.solve.inner_rtol, o.solve.check_every = inner_rtol, check_every
        o.recompute = 1 if recompute else 0
        self.h = C.c_void_p()
        self.ctx.check(lib().lfg_rd_adjoint_create(space.h, C.byref(o), u_obs.ptr, C.byref(self.h)))

    def __del__(self):
        try:
            if self.h:
                lib().lfg_rd_adjoint_destroy(self.h)
        except Exception:
            pass
        self.h = None

    def forward(self, theta, u_out=None):
        loss = C.c_double()
        self.ctx.check(lib().lfg_rd_adjoint_forward(self.h, theta.ptr, C.byref(loss),
                                                    u_out.ptr if u_out is not None else None))
        return loss.value

    def backward(self, grad_theta, grad_loss=1.0):
        self.ctx.check(lib().lfg_rd_adjoint_backward(self.h, float(grad_loss), grad_theta.ptr))

    def stats(self):
        f, a, n = lfg_solve_stats(), lfg_solve_stats(), C.c_int64()
        self.ctx.check(lib().lfg_rd_adjoint_stats(self.h, C.byref(f), C.byref(a), C.byref(n)))
        cv = lambda st: {"iterations": st.iterations, "refinements": st.refinements,
                         "rel_residual": st.rel_residual, "converged": bool(st.converged)}
        return {"forward": cv(f), "adjoint": cv(a), "saved_bytes": n.value}
