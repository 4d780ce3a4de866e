/*
 * lfg.h -- C-ABI of the GB300-native LehrFEM++ assembly-and-solve path.
 *
 * This is the drop-in boundary.  LehrFEM++ has no FFI of its own: its API for
 * this path is a set of C++20 templates and concepts.  Each entry point below
 * replaces one of them and is bound by the header-only C++ facade
 * include/lf_gb300.hpp (the reference's class and function names) or, from
 * Python, by lehrfempp_gb300/_capi.py (ctypes).  Citations are file:line in the
 * LehrFEM++ source tree.
 *
 * Conventions
 *   - Every function returns an lfg_status; LFG_OK == 0.  Nothing aborts; the
 *     message of the last failure on a context is lfg_ctx_last_error().
 *   - Arrays named *_dev are device pointers (allocated with lfg_malloc or by
 *     any CUDA allocator on the context's device); arrays named *_host are host
 *     pointers (pageable or pinned).  Sizes are element counts.
 *   - All work of a context is ordered on the context's CUDA stream
 *     (lfg_ctx_stream).  Calls on one context are not re-entrant; distinct
 *     contexts are independent (reference: single-threaded library).
 *   - Index types: DOF / node / edge / cell indices are int32 on the device;
 *     a triplet is {int32 row, int32 col, double value} = 16 bytes, the memory
 *     layout of Eigen::Triplet<double> (assemble/coomatrix.h:55).
 */
#ifndef LFG_H_
#define LFG_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  LFG_OK = 0,
  LFG_INVALID_ARG = 1,      /* bad handle, size or index (LF_ASSERT_MSG in the reference)   */
  LFG_DEGENERATE_CELL = 2,  /* geometry/tria_o1.cc:10-48, quad_o1.cc:12-58 (LF_VERIFY_MSG)   */
  LFG_CAPACITY = 3,         /* output buffer too small; nothing was written                   */
  LFG_UNSUPPORTED = 4,      /* coefficient kind / degree outside the supported set           */
  LFG_NOT_CONVERGED = 5,    /* iterative solve hit its iteration cap                           */
  LFG_CUDA_ERROR = 6,       /* a CUDA runtime call failed                                      */
  LFG_MISSING_RULE = 7,     /* no quadrature rule for a cell type (loc_comp_ellbvp.h:278-287)  */
  LFG_INCOMPLETE_MESH = 8,  /* hybrid2d/mesh.cc:566-600 check_completeness                     */
  LFG_OUT_OF_MEMORY = 9,
  LFG_IO_ERROR = 10,        /* file missing or not parseable (io/gmsh_reader.cc:622-660, LF_VERIFY_MSG) */
  LFG_NOT_FOUND = 11        /* name or number lookup failed (gmsh_reader.cc:32-99, LfException) */
} lfg_status;

typedef struct lfg_ctx lfg_ctx;
typedef struct lfg_mesh lfg_mesh;
typedef struct lfg_space lfg_space;
typedef struct lfg_coo lfg_coo;
typedef struct lfg_csr lfg_csr;

/* Eigen::Triplet<double> (StorageIndex int) layout. */
typedef struct {
  int32_t row;
  int32_t col;
  double value;
} lfg_triplet;

/* ------------------------------------------------------------------ context
 * Library plumbing, no counterpart in the reference (a single-threaded CPU
 * library with no device or stream): one context per device and stream. */
lfg_status lfg_ctx_create(int device, lfg_ctx** out);
lfg_status lfg_ctx_destroy(lfg_ctx* ctx);
const char* lfg_ctx_last_error(const lfg_ctx* ctx);
void* lfg_ctx_stream(lfg_ctx* ctx); /* the cudaStream_t all work is ordered on */
lfg_status lfg_ctx_synchronize(lfg_ctx* ctx);
/* Kernel launches issued by the library on this context since creation. */
lfg_status lfg_ctx_launch_count(const lfg_ctx* ctx, int64_t* launches);

/* make_QuadRule (lib/lf/quad/make_quad_rule.cc:21-157): the quadrature rule
 * of `degree` on the reference triangle (is_quad = 0: the tables of
 * quad/quad_rules_tria.cc for degrees 1..50, degree 3 served by the degree-4
 * table, the conical Gauss rule for degree 0 and above 50) or on the
 * reference square (is_quad = 1: tensor Gauss-Legendre, degree/2 + 1 points
 * per direction, x slow).  These are the rules every provider of this
 * library integrates with.  Host query, no device or context needed.  With
 * x, y and w null only *n is written; otherwise each must hold *n entries
 * (call once with nulls to get the count).  LFG_INVALID_ARG for a degree
 * outside [0, 100] or a null n. */
lfg_status lfg_quad_rule(int32_t is_quad, int32_t degree, double* x, double* y, double* w, int32_t* n);
/* EvaluationNodes and NodalValuesToDofs of FeHierarchicTria / FeHierarchicQuad
 * (fe/hierarchic_fe.h:820-1083, 1445-1680) with interior degree
 * interior_degree, edge degrees edge_degrees[0..3) (triangle) or [0..4)
 * (quadrilateral), each 1..20, and relative orientations `pattern` (bit j set:
 * local edge j negative).  The dual is linear: the dofs of a function with
 * values v at the nodes are M v, M row-major (*n_dofs x *n_nodes); node k is
 * (xy[2 k], xy[2 k + 1]).  These are the tables lfg_nodal_projection applies
 * on hierarchic spaces.  Host query, same null/count protocol as
 * lfg_quad_rule (xy and M both null: only the counts are written). */
lfg_status lfg_hier_dual(int32_t is_quad, int32_t interior_degree, const int32_t* edge_degrees, int32_t pattern,
                         double* xy, double* M, int32_t* n_nodes, int32_t* n_dofs);

/* Device memory and copies on the context's stream (no torch needed); no
 * counterpart in the reference, whose data lives in host memory.
 * lfg_host_alloc returns page-locked memory that the library also maps into
 * the device: a device-to-host copy of 1 MB or more into it (lfg_memcpy_d2h,
 * lfg_coo_download) with 16-byte aligned ends is done by a kernel storing
 * through the mapping, and lfg_assemble_matrix_rd_to_host writes into it
 * directly; lfg_memcpy_d2h synchronizes, h2d and d2d are stream-ordered.
 * Memory from lfg_host_alloc must be released with lfg_host_free (on the same
 * context), which also drops it from the context's list of mapped ranges. */
lfg_status lfg_malloc(lfg_ctx* ctx, size_t bytes, void** dev);
lfg_status lfg_free(lfg_ctx* ctx, void* dev);
lfg_status lfg_host_alloc(lfg_ctx* ctx, size_t bytes, void** pinned_host);
lfg_status lfg_host_free(lfg_ctx* ctx, void* pinned_host);
lfg_status lfg_memcpy_h2d(lfg_ctx* ctx, void* dst_dev, const void* src_host, size_t bytes);
lfg_status lfg_memcpy_d2h(lfg_ctx* ctx, void* dst_host, const void* src_dev, size_t bytes);
lfg_status lfg_memcpy_d2d(lfg_ctx* ctx, void* dst_dev, const void* src_dev, size_t bytes);
lfg_status lfg_memset(lfg_ctx* ctx, void* dev, int value, size_t bytes);

/* CUDA-event timing on the context stream, and an L2 flush (writes a buffer
 * larger than L2) for cold-cache measurements; measurement plumbing with no
 * counterpart in the reference. */
lfg_status lfg_timer_begin(lfg_ctx* ctx);
lfg_status lfg_timer_end(lfg_ctx* ctx, float* elapsed_ms);
lfg_status lfg_l2_flush(lfg_ctx* ctx);
/* Per-kernel timing (no reference counterpart; replaces lf::base::Timer,
 * base/timer.h:64-278, for device work): while enabled, every element-kernel
 * launch is bracketed by CUDA events on the context stream and accumulated
 * under its kernel family name ("rd_tria_df", "rd_quad_df", "rd_general_tria",
 * "rd_general_quad", "load_tria", "load_quad", "grad_rd", "misfit",
 * "batch_assemble", "rd_quad_tc"); "fp64_fallback_cells" counts cells that left the
 * df32 range, "tc_timeouts" tensor-core pipeline waits that gave up (always 0
 * on a healthy device; lfg_ctx_synchronize then fails with LFG_CUDA_ERROR). */
lfg_status lfg_profile_enable(lfg_ctx* ctx, int enable);
lfg_status lfg_profile_read(lfg_ctx* ctx, const char* family, double* total_ms, int64_t* launches);
lfg_status lfg_profile_reset(lfg_ctx* ctx);
/* Measured FP64 FMA throughput of this device (independent FMA chains on all
 * SMs), the denominator of the FP64 roofline fraction. */
lfg_status lfg_measure_fp64_peak(lfg_ctx* ctx, double* tflops);
/* Element matrices of Q2 quadrilaterals (cell-constant alpha, gamma = 0, tensor
 * Gauss rules of 2x2 or 3x3 points) run on the tcgen05 tensor cores with an
 * exact integer-digit splitting of the FP64 operands (kernel family
 * "rd_quad_tc"): enable = 3 (default) the warp-specialised kernel whose
 * producer warps write the triplets, 1 the warp-specialised kernel whose
 * consumer warps write them, 2 the two-CTA-per-SM variant, 0 the df32
 * CUDA-core kernel ("rd_quad_df"); all tensor-core modes give the same bits.
 * LFG_INVALID_ARG for other values.  No reference counterpart (a device choice). */
lfg_status lfg_ctx_set_tensor_cores(lfg_ctx* ctx, int enable);

/* --------------------------------------------------------------------- mesh
 * Replaces lf::mesh::hybrid2d::MeshFactory::AddPoint/AddEntity/Build
 * (mesh/hybrid2d/mesh_factory.cc:18-125, mesh.cc:178-810).
 *   node_xy_host        2 doubles per node, in AddPoint order
 *   cell_nodes_host     4 int32 per cell in AddEntity order; -1 in slot 3 = triangle
 *   preset_edges_host   2 int32 per edge registered before the cells (may be NULL)
 * Numbering (bit-exact with the reference): nodes and cells keep their order;
 * preset edges keep their registration index, edges created by cells follow
 * in lexicographic (min, max) node order; an edge points the way its first
 * creator lists it; relative orientation of local edge j (v_j -> v_{j+1}) is
 * positive iff the edge starts at v_j.  Degenerate cells (tol 1e-8) and
 * incomplete meshes are rejected. */
lfg_status lfg_mesh_create(lfg_ctx* ctx, int64_t num_nodes, const double* node_xy_host,
                           int64_t num_cells, const int32_t* cell_nodes_host,
                           int64_t num_preset_edges, const int32_t* preset_edges_host,
                           lfg_mesh** out);
/* lf::mesh::utils::TPTriagMeshBuilder::Build (mesh/utils/tp_triag_mesh_builder.cc:18-178)
 * and TPQuadMeshBuilder::Build (tp_quad_mesh_builder.cc:18-94), generated on the device. */
lfg_status lfg_mesh_create_tp_triag(lfg_ctx* ctx, int64_t nx, int64_t ny, double x0, double y0,
                                    double x1, double y1, lfg_mesh** out);
lfg_status lfg_mesh_create_tp_quad(lfg_ctx* ctx, int64_t nx, int64_t ny, double x0, double y0,
                                   double x1, double y1, lfg_mesh** out);
lfg_status lfg_mesh_destroy(lfg_mesh* mesh);
/* Mesh::NumEntities (mesh/mesh_interface.h:92-208); also counts by cell type. */
lfg_status lfg_mesh_sizes(const lfg_mesh* mesh, int64_t* num_nodes, int64_t* num_edges,
                          int64_t* num_cells, int64_t* num_trias, int64_t* num_quads);
/* Topology for inspection: edge endpoints (2/edge, in edge direction), cell
 * edges (4/cell, -1 pad), relative orientations (4/cell, +1/-1, 0 pad),
 * number of cells adjacent to each edge (CountNumSuperEntities). */
lfg_status lfg_mesh_download_topology(lfg_mesh* mesh, int32_t* edge_nodes_host,
                                      int32_t* cell_edges_host, int8_t* cell_ori_host,
                                      int32_t* edge_num_cells_host);
/* Device arrays of the mesh: node_xy (2*N doubles), cell_nodes (4*C int32). */
lfg_status lfg_mesh_device_arrays(lfg_mesh* mesh, const double** node_xy_dev,
                                  const int32_t** cell_nodes_dev);
/* Replace the node coordinates (same topology), from host or device memory. */
lfg_status lfg_mesh_set_coords(lfg_mesh* mesh, const double* node_xy, int from_device);
/* flagEntitiesOnBoundary (mesh/utils/special_entity_sets.cc:64-90): 1 byte per
 * node / edge, device output. */
lfg_status lfg_mesh_boundary_flags(lfg_mesh* mesh, uint8_t* node_flags_dev,
                                   uint8_t* edge_flags_dev);

/* ------------------------------------------------------------ FE space/dofs
 * UniformFEDofHandler (assemble/dofhandler.h:260-503, dofhandler.cc:86-338)
 * with num interior dofs per point / segment / tria / quad, check_edge_orientation
 * = true.  lfg_space_create_lagrange = FeSpaceLagrangeO{1,2,3}
 * (uscalfe/fe_space_lagrange_o1.h:45-51 etc.; layout uniform_scalar_fe_space.h:241-342). */
lfg_status lfg_space_create(lfg_mesh* mesh, int np, int ns, int nt, int nq, lfg_space** out);
lfg_status lfg_space_create_lagrange(lfg_mesh* mesh, int degree, lfg_space** out);
/* fe::HierarchicScalarFESpace(mesh, degree) (fe/hierarchic_scalar_fe_space.h:
 * 36-46) of uniform degree 1..20: hierarchic (integrated Legendre / Jacobi)
 * shape functions (fe/hierarchic_fe.h), dofs numbered like
 * DynamicFEDofHandler (nodes, edge interiors, cell interiors).  With such a
 * space, lfg_assemble_matrix_rd is fe::DiffusionElementMatrixProvider
 * (alpha) + fe::MassElementMatrixProvider (gamma) (fe/loc_comp_ellbvp.h:
 * 169-214, 349-378) and lfg_assemble_vector_load fe::ScalarLoadElementVector-
 * Provider (:642-685), with make_QuadRule(ref_el, 2 * degree) by default. */
lfg_status lfg_space_create_hierarchic(lfg_mesh* mesh, int32_t degree, lfg_space** out);
/* fe::HierarchicScalarFESpace(mesh, degree_functor) (fe/hierarchic_scalar_fe_space.h:
 * 93-116, Init :178-220): the functor's value for every edge (edge_degree[ne],
 * edge index order) and every cell (cell_degree[nc], cell index order), host
 * arrays, each 1..20.  Dofs numbered by DynamicFEDofHandler (assemble/
 * dofhandler.h:550-680): one per node, edge_degree[e] - 1 per edge, the
 * interior count of cell_degree[c] per cell; a cell's shape functions are
 * those of FeHierarchicTria/Quad(cell_degree, edge degrees, orientations)
 * (fe/hierarchic_fe.h:482-501, 1150-1170), and the default rule of a cell is
 * make_QuadRule(ref_el, 2 * max(cell degree, edge degrees)).  NumLocalDofs
 * varies by cell (lfg_space_download_local_counts); lfg_space_info reports
 * the counts of the largest degree as n_tria / n_quad.  Degrees outside 1..20:
 * LFG_UNSUPPORTED. */
lfg_status lfg_space_create_hierarchic_var(lfg_mesh* mesh, const int32_t* edge_degree, const int32_t* cell_degree,
                                           lfg_space** out);
/* DofHandler::NumLocalDofs(cell) (assemble/dofhandler.h:147) of every cell,
 * in cell index order (n_local[nc], host). */
lfg_status lfg_space_download_local_counts(lfg_space* space, int32_t* n_local);
lfg_status lfg_space_destroy(lfg_space* space);
/* NumDofs, NumLocalDofs per tria / quad, row stride of the cell dof table,
 * and the number of triplets one AssembleMatrixLocally call emits. */
lfg_status lfg_space_info(const lfg_space* space, int64_t* num_dofs, int32_t* n_tria,
                          int32_t* n_quad, int32_t* n_cell_stride, int64_t* num_triplets);
/* DofHandler::GlobalDofIndices(cell) (assemble/dofhandler.h:184) of every cell
 * (num_cells x n_cell_stride, -1 pad), host out. */
lfg_status lfg_space_download_cell_dofs(lfg_space* space, int32_t* cell_dofs_host);
/* DofHandler::Entity(dof) (assemble/dofhandler.h:219) for every dof: codim
 * (2 node, 1 edge, 0 cell) and index, host out. */
lfg_status lfg_space_download_dof_entities(lfg_space* space, int8_t* codim_host,
                                           int32_t* index_host);
/* Selector of the reference drivers: dof flagged iff its entity lies on the
 * boundary (flagEntitiesOnBoundary + DofHandler::Entity), device output. */
lfg_status lfg_space_boundary_dof_flags(lfg_space* space, uint8_t* flags_dev);

/* ------------------------------------------------------------- coefficients
 * A scalar MeshFunction (mesh/utils/mesh_function_traits.h:149-155) from a
 * closed set that runs on the device:
 *   LFG_COEFF_ZERO / CONSTANT        MeshFunctionConstant (mesh_function_constant.h:25-45)
 *   LFG_COEFF_PER_CELL               one value per cell, data_dev[num_cells]
 *   LFG_COEFF_NODAL_O1               MeshFunctionFE of an O1 dof vector,
 *                                    data_dev[num_nodes] (fe/mesh_function_fe.h:44-115)
 *   LFG_COEFF_ANALYTIC               MeshFunctionGlobal of a built-in function
 *                                    (mesh_function_global.h:54-94) chosen by func:
 *     LFG_FN_POLY    sum_{i,j<=3} p[4i+j] x^i y^j
 *     LFG_FN_SINSIN  p0 + p1 sin(p2 pi x) sin(p3 pi y)
 *     LFG_FN_SINCOS  p0 + p1 sin(p2 pi x) cos(p3 pi y)
 *     LFG_FN_EXP     p0 + p1 exp(p2 + p3 x + p4 y + p5 x y)
 *     LFG_FN_TRIG    p0 + (p1 + p2 x + p3 y + p4 x y) sin(pi (p5 x + p6)) sin(pi (p7 y + p8))
 *                    (a cosine is the sine shifted by 1/2 in p6 / p8)
 *   The post-processing functions also use the exact gradient of each family.
 * Matrix-valued diffusion coefficients (the 2x2 DIFF_COEFF that
 * ReactionDiffusionElementMatrixProvider accepts, uscalfe/loc_comp_ellbvp.h:
 * 85-127; row-major a00, a01, a10, a11, not necessarily symmetric) are valid
 * only as alpha of lfg_assemble_matrix_rd on Lagrangian spaces:
 *   LFG_COEFF_TENSOR_CONSTANT        p[0..3]
 *   LFG_COEFF_TENSOR_PER_CELL        data_dev[4 * cell + 0..3]
 *   LFG_COEFF_TENSOR_BILINEAR        entry e = p[4e] + p[4e+1] x + p[4e+2] y + p[4e+3] x y
 *                                    at the global point (the reference's
 *                                    tensor test uses [[1, x], [y, x y]])
 * Arbitrary host lambdas cannot run on the GPU: anything else is LFG_UNSUPPORTED. */
enum {
  LFG_COEFF_ZERO = 0,
  LFG_COEFF_CONSTANT = 1,
  LFG_COEFF_PER_CELL = 2,
  LFG_COEFF_NODAL_O1 = 3,
  LFG_COEFF_ANALYTIC = 4,
  LFG_COEFF_PER_CELL_EXP = 5,  /* exp(data_dev[cell]): a per-cell log-coefficient */
  LFG_COEFF_TENSOR_CONSTANT = 6,
  LFG_COEFF_TENSOR_PER_CELL = 7,
  LFG_COEFF_TENSOR_BILINEAR = 8
};
enum { LFG_FN_POLY = 1, LFG_FN_SINSIN = 2, LFG_FN_SINCOS = 3, LFG_FN_EXP = 4, LFG_FN_TRIG = 5 };

typedef struct {
  int32_t kind;
  int32_t func;
  double value;
  const double* data_dev;
  double p[16];
} lfg_coeff;

/* ReactionDiffusionElementMatrixProvider (uscalfe/loc_comp_ellbvp.h:85-339):
 * A_K = sum_k w_k |det J| [ (J^-T grad b_i)^T alpha (J^-T grad b_j) + gamma b_i b_j ].
 * qr_degree_* = 0 selects the default degree 2p (loc_comp_ellbvp.h:227-228);
 * a positive value selects make_QuadRule(type, degree) (the qr_collection
 * constructor, :237-263); -1 leaves that cell type without a rule, and cells
 * of that type then fail with LFG_MISSING_RULE. */
typedef struct {
  lfg_coeff alpha;
  lfg_coeff gamma;
  int32_t qr_degree_tria;
  int32_t qr_degree_quad;
} lfg_rd_provider;

/* Boundary-edge providers (codim-1 assembly).
 * MassEdgeMatrixProvider (uscalfe/loc_comp_ellbvp.h:367-529) with
 * AssembleMatrixLocally(1, dofh, dofh, provider, A) (assembler.h:114-186):
 * edges in index order; an edge is active iff edge_flags_dev[e] != 0 (the
 * EDGESELECTOR; NULL = every edge); per active edge the (p+1)^2 triplets of
 *   A_e(i,j) = sum_k w_k |e| gamma(x_k) phi_i(t_k) phi_j(t_k)
 * in row-major order, rows/cols = the edge's dofs (its two endpoint dofs in
 * edge direction, then its interior dofs), segment basis of the space's
 * degree (FeLagrangeO{1,2,3}Segment), Gauss rule of degree qr_degree (0:
 * 2 * degree).  ScalarLoadEdgeVectorProvider (loc_comp_ellbvp.h:784-921) with
 * AssembleVectorLocally(1, ...) (assembler.h:298-327): b[dof_i] += sum_k
 * w_k |e| g(x_k) phi_i(t_k), contributions added in edge order.  Coefficients:
 * CONSTANT, PER_CELL / PER_CELL_EXP (data indexed by EDGE), NODAL_O1,
 * ANALYTIC.  FP64. */
typedef struct {
  lfg_coeff gamma;
  const uint8_t* edge_flags_dev;
  int32_t qr_degree;
} lfg_edge_mass_provider;
typedef struct {
  lfg_coeff g;
  const uint8_t* edge_flags_dev;
  int32_t qr_degree;
} lfg_edge_load_provider;

/* ScalarLoadElementVectorProvider (loc_comp_ellbvp.h:562-746). */
typedef struct {
  lfg_coeff f;
  int32_t qr_degree_tria;
  int32_t qr_degree_quad;
} lfg_load_provider;

/* ---------------------------------------------------------------- COO matrix
 * lf::assemble::COOMatrix<double> (assemble/coomatrix.h:51-225) on the device. */
lfg_status lfg_coo_create(lfg_ctx* ctx, int64_t rows, int64_t cols, int64_t capacity,
                          lfg_coo** out);
/* Wrap caller-owned device memory of `capacity` triplets holding `size` entries. */
lfg_status lfg_coo_wrap(lfg_ctx* ctx, int64_t rows, int64_t cols, lfg_triplet* triplets_dev,
                        int64_t capacity, int64_t size, lfg_coo** out);
lfg_status lfg_coo_destroy(lfg_coo* coo);
/* COOMatrix::triplets() (coomatrix.h:124-125): its length and its device storage. */
lfg_status lfg_coo_size(const lfg_coo* coo, int64_t* size);
lfg_status lfg_coo_triplets(lfg_coo* coo, lfg_triplet** triplets_dev);
/* COOMatrix::setZero() (coomatrix.h:95-98): drop all triplets. */
lfg_status lfg_coo_set_zero(lfg_coo* coo);
/* Copy the first `count` triplets of COOMatrix::triplets() (coomatrix.h:124)
 * to host memory (count <= size). */
lfg_status lfg_coo_download(lfg_coo* coo, lfg_triplet* host, int64_t count);
/* Append host triplets (COOMatrix::AddToEntry, coomatrix.h:87-91, for each). */
lfg_status lfg_coo_append_host(lfg_coo* coo, const lfg_triplet* host, int64_t count);

/* ------------------------------------------------------------------ assembly
 * AssembleMatrixLocally(0, dofh, dofh, provider, A) (assemble/assembler.h:114-186):
 * appends sum_K n_K^2 triplets to A, cells in index order, (i,j) row-major within
 * a cell, row = GlobalDofIndices(K)[i], col = GlobalDofIndices(K)[j]. */
lfg_status lfg_assemble_matrix_rd(lfg_space* space, const lfg_rd_provider* provider,
                                  lfg_coo* coo);
/* The same assembly with the COOMatrix in host memory, as the reference keeps
 * it (assemble/coomatrix.h:51-225): the sum_K n_K^2 triplets are written to
 * host[0 .. count) in the same order.  When host[0 .. sum_K n_K^2) lies inside
 * one page-locked allocation made by lfg_host_alloc on this context, the
 * element kernels store the triplets straight into it over the host link
 * (one pass; chunk_triplets is not used).  Otherwise the cells are assembled
 * in ranges of about chunk_triplets triplets (<= 0: 2^24) into a ring of three
 * device staging buffers while earlier ranges are copied to the host on a
 * second stream, so the device holds only the ring, not the whole matrix.
 * LFG_CAPACITY if capacity < sum_K n_K^2.  Lagrangian spaces. */
lfg_status lfg_assemble_matrix_rd_to_host(lfg_space* space, const lfg_rd_provider* provider,
                                          lfg_triplet* host, int64_t capacity, int64_t chunk_triplets,
                                          int64_t* count);
/* AssembleVectorLocally(0, dofh, provider, b) (assembler.h:298-327):
 * b_dev[dof] += element vector entries, cells in index order (deterministic). */
lfg_status lfg_assemble_matrix_edge_mass(lfg_space* space, const lfg_edge_mass_provider* provider, lfg_coo* coo);
lfg_status lfg_assemble_vector_edge_load(lfg_space* space, const lfg_edge_load_provider* provider, double* b_dev);
lfg_status lfg_assemble_vector_load(lfg_space* space, const lfg_load_provider* provider,
                                    double* b_dev);
/* Assembly with caller-tabulated element matrices / vectors: elem_dev holds
 * num_cells blocks of ld x ld (row major; the first n_K x n_K entries are used),
 * vec_dev num_cells blocks of ld.  This is the EntityMatrixProvider /
 * EntityVectorProvider concept (assemble/assemble_concepts.h:95-99, 210-214)
 * for providers whose Eval was computed elsewhere. */
lfg_status lfg_assemble_matrix_tabulated(lfg_space* space, const double* elem_dev, int32_t ld,
                                         lfg_coo* coo);
lfg_status lfg_assemble_vector_tabulated(lfg_space* space, const double* vec_dev, int32_t ld,
                                         double* b_dev);

/* -------------------------------------------------------- Dirichlet fixing
 * FixFlaggedSolutionComponents (assemble/fix_dof.h:86-138) with a tabulated
 * selector: flags_dev[k] != 0 <=> dof k fixed to values_dev[k].
 * b -= A xhat; b[k] = value[k] on fixed k; triplets with a fixed row or column
 * are removed keeping the order of the others; (k,k,1.0) appended for fixed k
 * in ascending order.  LFG_CAPACITY (nothing modified) if the appended
 * diagonal does not fit. */
lfg_status lfg_fix_flagged_solution_components(lfg_coo* coo, const uint8_t* flags_dev,
                                               const double* values_dev, double* b_dev);
/* FixFlaggedSolutionCompAlt (fix_dof.h:183-219): only fixed rows are removed. */
lfg_status lfg_fix_flagged_solution_comp_alt(lfg_coo* coo, const uint8_t* flags_dev,
                                             const double* values_dev, double* b_dev);
/* FixSolutionComponentsLse (fix_dof.h:250-280) with fixed_components given
 * as `count` (dof, value) pairs (device arrays, in list order): a dof that
 * appears several times is fixed to the sum of its values, added in list
 * order; then FixFlaggedSolutionCompAlt.  LFG_INVALID_ARG (nothing modified)
 * for a dof outside [0, N). */
lfg_status lfg_fix_solution_components_lse(lfg_coo* coo, int64_t count, const int64_t* dofs_dev,
                                           const double* values_dev, double* b_dev);

/* ------------------------------------------------------------- CSR + solve
 * COOMatrix::makeSparse (coomatrix.h:172-180) -> Eigen::setFromTriplets: the
 * duplicates of each (row, col) are summed in triplet order.  Stored as CSR
 * (int64 row pointers, int32 columns, double values). */
lfg_status lfg_csr_from_coo(lfg_coo* coo, lfg_csr** out);
lfg_status lfg_csr_destroy(lfg_csr* csr);
lfg_status lfg_csr_info(const lfg_csr* csr, int64_t* rows, int64_t* cols, int64_t* nnz);
lfg_status lfg_csr_download(lfg_csr* csr, int64_t* rowptr_host, int32_t* col_host,
                            double* val_host);
/* y = A x (FP64): the product of the Eigen::SparseMatrix that
 * COOMatrix::makeSparse (coomatrix.h:172-180) returns. */
lfg_status lfg_csr_spmv(lfg_csr* csr, const double* x_dev, double* y_dev);

/* Solve A x = b for the (symmetric positive definite, after fixing) Galerkin
 * matrix.  The reference solves with Eigen::SparseLU in its drivers
 * (examples/ellbvp_linfe/homDir_linfe_demo.cc:168-174); on the GPU the solve is
 * a Jacobi-preconditioned CG:
 *   LFG_SOLVE_FP64   FP64 PCG to ||b - A x|| <= rtol ||b|| (restarted from the
 *                    true residual when the recursive one drifts)
 *   LFG_SOLVE_MIXED  FP32 PCG inner solves (FP32 matrix copy and vectors) of
 *                    A d = r / ||r|| to inner_rtol, inside FP64 iterative
 *                    refinement: r = b - A x in FP64, x += ||r|| d in FP64,
 *                    to the same FP64 residual criterion.  The FP32 operator
 *                    is applied in difference form, (A p)_r = sum_k a_rk
 *                    (p_k - p_r) + s_r p_r with the FP64 row sum s_r, so that
 *                    rounding the entries to FP32 keeps it close to A on its
 *                    smooth modes.  An inner solve stops early when its true
 *                    residual departs from the recursive one; when an FP32
 *                    correction does not reduce the FP64 residual norm by 2x
 *                    the solve finishes in FP64 from the better iterate.
 *                    (The batched solver, lfg_batch_solve_pcg, uses residual
 *                    replacement instead, where it needs fewer iterations.)
 * x_dev holds the initial guess on entry. */
enum { LFG_SOLVE_FP64 = 0, LFG_SOLVE_MIXED = 1 };
typedef struct {
  int32_t precision;
  int32_t max_iterations;        /* total inner PCG iterations allowed           */
  double rtol;                   /* relative residual target (FP64)              */
  double inner_rtol;             /* mixed: relative reduction per inner solve (0: 1e-4); batched:
                                    residual-norm drop between replacements (0: 0.1) */
  int32_t check_every;           /* convergence checks every N iterations        */
} lfg_solve_opts;
typedef struct {
  int32_t iterations;            /* PCG iterations (all inner iterations)        */
  int32_t refinements;           /* FP64 refinement steps or residual replacements (mixed) / restarts (FP64) */
  double rel_residual;           /* final ||b - A x|| / ||b|| in FP64            */
  int32_t converged;
} lfg_solve_stats;
lfg_status lfg_solve_pcg(lfg_csr* csr, const double* b_dev, double* x_dev,
                         const lfg_solve_opts* opts, lfg_solve_stats* stats);

/* lfg_solve_pcg for callers that cannot let the library allocate device
 * memory (an application that owns a fixed GPU memory budget through its own
 * allocator, or a service that must not grow the CUDA memory pool or risk an
 * allocation's implicit synchronisation inside its time loop).  This entry
 * point has no counterpart in the reference.  It runs the same algorithm and
 * convergence test as the FP64 PCG of lfg_solve_pcg (restarts from the true
 * residual included), with all work vectors in one fixed, file-scope device
 * array of 40 MiB + 48 KiB that every GPU loading the library holds until
 * exit, and calls no allocator.  Its SpMV reads the CSR arrays directly
 * instead of lfg_solve_pcg's padded copy, so rounding and iteration counts
 * can differ slightly between the two.  Limits: FP64 only (LFG_UNSUPPORTED
 * otherwise) and at most 1,048,576 rows (LFG_CAPACITY otherwise).  All calls
 * share the array and it keeps the last call's contents: calls that overlap
 * on the GPU race.  The first call on a device resolves the array's address;
 * make it before any stream capture. */
lfg_status lfg_solve_pcg_noalloc(lfg_csr* csr, const double* b_dev, double* x_dev,
                                 const lfg_solve_opts* opts, lfg_solve_stats* stats);

/* ------------------------------------------------------ differentiation
 * No reference counterpart (the reference has no derivatives).  For
 * J(theta) = 1/2 ||u - u_obs||^2 and A(theta) u = b after
 * FixFlaggedSolutionComponents (free block A_ff, identity on flagged dofs,
 * b_f -= A_fd g), the adjoint lambda solves A lambda = u - u_obs and
 *   dJ/dtheta_c = - sum_{i free, j} lambda_i (dA_K/dtheta_c)_ij u_j ,
 * the sum over the dofs of cell c; u_j at flagged dofs is the Dirichlet
 * value g_j.  Only the diffusion part of A_K depends on theta:
 *   alpha = exp(theta_c) (LFG_COEFF_PER_CELL_EXP): dA_K/dtheta_c = alpha_c S_K,
 *   alpha = theta_c      (LFG_COEFF_PER_CELL):     dA_K/dtheta_c = S_K,
 * with S_K the element stiffness matrix for alpha = 1 (with gamma = 0 and
 * alpha = exp(theta) this is A_K itself).  Other alpha kinds: LFG_UNSUPPORTED.
 * lfg_loss_l2_misfit: J (host, deterministic reduction) and dJ/du = u - u_obs
 * (device; skipped when misfit_dev is NULL), FP64.
 * lfg_grad_rd_cellwise: grad_dev[c] for every cell, lambda taken as zero at
 * dofs with fixed_flags_dev[i] != 0 (NULL: no flagged dofs); FP64
 * arithmetic and accumulation, one value per cell (no atomics). */
lfg_status lfg_loss_l2_misfit(lfg_ctx* ctx, int64_t n, const double* u_dev, const double* u_obs_dev,
                              double* loss_host, double* misfit_dev);
lfg_status lfg_grad_rd_cellwise(lfg_space* space, const lfg_rd_provider* provider,
                                const double* u_dev, const double* lambda_dev,
                                const uint8_t* fixed_flags_dev, double* grad_dev);

/* Forward/backward Function object of theta -> J (the autograd.Function
 * contract: forward(theta) returns J and saves what backward needs;
 * backward(dL/dJ) returns dL/dtheta = dL/dJ * dJ/dtheta).
 *   forward : A(theta) = AssembleMatrixLocally(ReactionDiffusion(exp(theta), 0)),
 *             b = AssembleVectorLocally(load), FixFlaggedSolutionComponents,
 *             PCG solve A u = b, J = 1/2 ||u - u_obs||^2.
 *   backward: adjoint PCG solve A lambda = (u - u_obs) on free dofs, then
 *             lfg_grad_rd_cellwise scaled by dL/dJ.
 * recompute = 0 keeps the Galerkin matrix, u and u - u_obs between the two
 * calls; recompute = 1 keeps only a copy of theta (8 bytes per cell) and
 * backward re-assembles and re-solves for u first (the memory-saving mode).
 * The space must outlive the object.  Backward before any forward is
 * LFG_INVALID_ARG; backward may run more than once after one forward. */
typedef struct lfg_rd_adjoint lfg_rd_adjoint;
typedef struct {
  lfg_load_provider load;        /* right-hand side f and its rules */
  int32_t qr_degree_tria;        /* rules of the stiffness matrix (0 = 2 * degree) */
  int32_t qr_degree_quad;
  const uint8_t* flags_dev;      /* Dirichlet dofs (NULL: boundary dofs of the space) */
  const double* dirichlet_dev;   /* values at flagged dofs, length num_dofs (NULL: 0) */
  lfg_solve_opts solve;          /* forward and adjoint PCG */
  int32_t recompute;
} lfg_rd_adjoint_opts;
lfg_status lfg_rd_adjoint_create(lfg_space* space, const lfg_rd_adjoint_opts* opts,
                                 const double* u_obs_dev, lfg_rd_adjoint** out);
lfg_status lfg_rd_adjoint_destroy(lfg_rd_adjoint* f);
/* theta_dev: num_cells log-coefficients.  u_out_dev (may be NULL) receives u. */
lfg_status lfg_rd_adjoint_forward(lfg_rd_adjoint* f, const double* theta_dev, double* loss_host,
                                  double* u_out_dev);
lfg_status lfg_rd_adjoint_backward(lfg_rd_adjoint* f, double grad_loss, double* grad_theta_dev);
/* Solver statistics of the last forward (u) and adjoint (lambda) solves;
 * saved_bytes: device memory held between forward and backward. */
lfg_status lfg_rd_adjoint_stats(const lfg_rd_adjoint* f, lfg_solve_stats* forward,
                                lfg_solve_stats* adjoint, int64_t* saved_bytes);

/* ---------------------------------------------------------- batched form
 * Many independent problems (no reference counterpart: the reference loops
 * over problems one at a time, each with AssembleMatrixLocally + SparseLU).
 * A batch is a list of spaces (each on its own mesh) viewed as one
 * block-diagonal system: mesh b's dofs occupy global rows
 * [dof_offset[b], dof_offset[b+1]) and its triplets the range
 * [triplet_offset[b], triplet_offset[b+1]) of a batch COO, in exactly the
 * order AssembleMatrixLocally gives for that mesh alone, with row/col shifted
 * by dof_offset[b].  Batch-wide coefficient arrays are indexed by batch cell
 * (cell_offset[b] + local cell). */
typedef struct lfg_batch lfg_batch;
lfg_status lfg_batch_create(lfg_ctx* ctx, int32_t num_spaces, lfg_space* const* spaces,
                            lfg_batch** out);
lfg_status lfg_batch_destroy(lfg_batch* batch);
lfg_status lfg_batch_info(const lfg_batch* batch, int32_t* num_spaces, int64_t* total_dofs,
                          int64_t* total_cells, int64_t* total_triplets);
/* Host copies of the offset arrays (num_spaces + 1 entries each, any may be NULL). */
lfg_status lfg_batch_offsets(const lfg_batch* batch, int64_t* dof_offset, int64_t* cell_offset,
                             int64_t* triplet_offset);
/* All element matrices of all meshes in one persistent launch (cells with
 * constant / per-cell alpha and gamma; triangles).  Appends total_triplets
 * to coo (global indices).  The first call tunes the launch shape (threads
 * per CTA, CTAs per SM) by timing the candidates on this batch; the choice is
 * kept in the batch (lfg_batch_tuning). */
lfg_status lfg_batch_assemble_matrix_rd(lfg_batch* batch, const lfg_rd_provider* provider,
                                        lfg_coo* coo);
lfg_status lfg_batch_tuning(const lfg_batch* batch, int32_t* threads_per_cta, int32_t* ctas_per_sm,
                            double* best_ms);
/* AssembleVectorLocally of every mesh into b_dev[total_dofs] (global rows). */
lfg_status lfg_batch_assemble_vector_load(lfg_batch* batch, const lfg_load_provider* provider,
                                          double* b_dev);
/* Boundary-dof selector of every mesh, flags_dev[total_dofs]. */
lfg_status lfg_batch_boundary_dof_flags(lfg_batch* batch, uint8_t* flags_dev);
/* Batched PCG: one independent Jacobi-PCG per block of the block-diagonal
 * CSR (each with its own step lengths and stopping test), all advanced
 * together by the same kernels, replayed from a CUDA graph.  precision FP64 or
 * MIXED: per block, FP32 PCG (difference-form operator, see lfg_solve_pcg) on
 * r / ||r_0|| with residual replacement -- once the block's recursive FP32
 * residual norm has dropped by inner_rtol (0: 0.1) since its last replacement
 * or meets the target, its FP32 correction is added to x in FP64, its true
 * residual b - A x is formed in FP64 and replaces the recursive one, and its
 * CG continues along the same direction; a block whose FP32 recursion stops
 * tracking the FP64 residual finishes in FP64.  per_block_stats
 * (num_spaces entries, may be NULL) and the summary stats (iterations = the
 * longest block, converged = all blocks). */
lfg_status lfg_batch_solve_pcg(lfg_batch* batch, lfg_csr* block_diagonal, const double* b_dev,
                               double* x_dev, const lfg_solve_opts* opts, lfg_solve_stats* stats,
                               lfg_solve_stats* per_block_stats);
/* The batched PCG works on chunks of rows that never straddle two blocks;
 * the first solve in each precision times the candidate chunk sizes (512 ..
 * 4096 rows) on this batch and keeps the fastest.  The choice for `precision`
 * (0 before the first solve in that precision) and its measured rate in
 * row-iterations per second; and an override.  The chunk size changes only
 * the order of each block's partial sums.  No reference counterpart. */
lfg_status lfg_batch_solve_tuning(const lfg_batch* batch, int32_t precision, int32_t* chunk_rows,
                                  double* row_iterations_per_s);
lfg_status lfg_batch_set_solve_chunk_rows(lfg_batch* batch, int32_t precision, int32_t chunk_rows);
/* Scheme of the batched PCG.  group_bytes = 0: every block advances in one
 * lock-step sweep over the whole batch per iteration (kernels replayed from a
 * CUDA graph, every iteration streams the batch from HBM).  group_bytes > 0:
 * blocks are packed, largest first, into groups of at most group_bytes of
 * solver data (matrix, diagonal, row sums, work vectors) and solved one
 * group at a time by a persistent cooperative kernel (the Chronopoulos-Gear
 * form of the same Jacobi-PCG: one reduction and two grid barriers per
 * iteration, check_every iterations per launch), so that a group's data
 * stays in the 129 MB L2 across iterations.  The lock-step sweep is the
 * faster scheme on GB300; both give each block its PCG solution to the same
 * tolerance (the iterates differ by rounding).  No reference counterpart. */
lfg_status lfg_batch_set_solve_groups(lfg_batch* batch, double group_bytes);
lfg_status lfg_batch_solve_groups(const lfg_batch* batch, double* group_bytes);

/* ---------------------------------------------------------------- Gmsh reader
 * GmshReader(factory, filename) (io/gmsh_reader.h, io/gmsh_reader.cc:22-30,
 * 116-620) for 2D meshes of first-order cells: MSH 2.2 and 4.1, ASCII and
 * binary.  Parsing runs on the host and needs no device; lfg_gmsh_build_mesh
 * hands the MeshFactory input (main nodes in file order, cells in element
 * order, segment elements as pre-registered edges) to lfg_mesh_create, so the
 * device mesh is numbered exactly as the reference's hybrid2d factory numbers
 * the file.  Element types: 15 point, 1 segment, 2 triangle, 3 quadrilateral;
 * second-order (curved) types 8, 9, 10, 16 and all others: LFG_UNSUPPORTED.
 * The calls below take no context: a failing call stores its message for
 * lfg_gmsh_last_error() (per thread). */
typedef struct lfg_gmsh lfg_gmsh;
const char* lfg_gmsh_last_error(void);
lfg_status lfg_gmsh_open(const char* filename, lfg_gmsh** out);
lfg_status lfg_gmsh_open_buffer(const char* data, int64_t size, lfg_gmsh** out);
lfg_status lfg_gmsh_destroy(lfg_gmsh* g);
/* The MeshFactory input: num_nodes x (x, y); num_cells x 4 node indices (-1
 * in the last slot of a triangle); num_preset_edges x 2 node indices. */
lfg_status lfg_gmsh_sizes(const lfg_gmsh* g, int64_t* num_nodes, int64_t* num_cells, int64_t* num_preset_edges);
lfg_status lfg_gmsh_factory_input(const lfg_gmsh* g, double* xy, int32_t* cells, int32_t* preset_edges);
/* GmshReader::mesh(): the device mesh (destroy with lfg_mesh_destroy). */
lfg_status lfg_gmsh_build_mesh(lfg_ctx* ctx, const lfg_gmsh* g, lfg_mesh** mesh);
/* PhysicalEntityNr(e) for the entities 0..num_entities-1 of a codim (0 cells,
 * 1 edges, 2 nodes), host arrays: offsets[num_entities + 1], nrs[offsets[n]]
 * (NULL: offsets only).  Edges the file does not list have no numbers. */
lfg_status lfg_gmsh_physical_entity_nrs(const lfg_gmsh* g, int32_t codim, int64_t num_entities, int64_t* offsets,
                                        int32_t* nrs);
/* IsPhysicalEntity(e, nr) for every entity of a codim: host flags (the
 * selector the edge providers and lfg_init_essential_condition take, after a
 * copy to the device). */
lfg_status lfg_gmsh_is_physical_entity(const lfg_gmsh* g, int32_t codim, int32_t nr, int64_t num_entities,
                                       uint8_t* flags);
/* PhysicalEntityName2Nr / PhysicalEntityNr2Name (gmsh_reader.cc:32-99),
 * codim -1 = any (an ambiguous lookup fails with LFG_NOT_FOUND, as the
 * reference throws); PhysicalEntities(codim) (gmsh_reader.cc:101-110). */
lfg_status lfg_gmsh_name_to_nr(const lfg_gmsh* g, const char* name, int32_t codim, int32_t* nr);
lfg_status lfg_gmsh_nr_to_name(const lfg_gmsh* g, int32_t nr, int32_t codim, char* name, int64_t capacity);
lfg_status lfg_gmsh_physical_entities(const lfg_gmsh* g, int32_t codim, int32_t* count, int32_t* nrs);

/* ---------------------------------------------------------- post-processing
 * The steps after the solve (and the Dirichlet data before it), FP64 on the
 * device.  An FE function is (space, dof vector) as in MeshFunctionFE
 * (fe/mesh_function_fe.h:44-115); mesh functions are lfg_coeff values.
 *
 * IntegrateMeshFunction(mesh, mf, quad_degree, pred, codim)
 * (fe/fe_tools.h:110-165) for the integrands
 *   LFG_INTEGRAND_VALUE         u_h + u
 *   LFG_INTEGRAND_SQ_DIFF       (u_h - u)^2           squaredNorm(mf_fe - mf_u)
 *   LFG_INTEGRAND_GRAD_SQ_DIFF  |grad u_h - grad u|^2 squaredNorm(mf_grad_fe - mf_grad_u)
 * with u_h = 0 when dofs_dev is NULL and u = 0 for LFG_COEFF_ZERO; grad u is
 * the exact gradient of an analytic u, the gradient of the O1 interpolant for
 * LFG_COEFF_NODAL_O1, 0 for cell-wise constants.  Rules: make_QuadRule(ref_el,
 * quad_degree) per reference element (segments for codim 1).  flags_dev
 * (num_cells or num_edges entries, NULL: all) selects entities; as in the
 * reference, entity 0 always contributes (fe_tools.h:117-124).  Gradients on
 * edges are LFG_UNSUPPORTED.  On codim 1 a PER_CELL u is indexed by edge.
 * u_h may live on a Lagrangian (O1-O3) or a hierarchic space (uniform or
 * per-entity degrees; each cell's own FeHierarchicTria / Quad shape
 * functions; cells only, codim 1 is LFG_UNSUPPORTED there).
 * The sum is deterministic (fixed per-block order).  *result is host memory;
 * the call waits for it. */
enum {
  LFG_INTEGRAND_VALUE = 0,
  LFG_INTEGRAND_SQ_DIFF = 1,
  LFG_INTEGRAND_GRAD_SQ_DIFF = 2
};
typedef struct {
  int32_t kind;             /* LFG_INTEGRAND_* */
  lfg_coeff u;
  lfg_space* space;         /* space of u_h (on the integration mesh), may be NULL without dofs */
  const double* dofs_dev;   /* u_h coefficients, NULL: u_h = 0 */
} lfg_integrand;
lfg_status lfg_integrate_mesh_function(lfg_mesh* mesh, const lfg_integrand* integrand, int32_t quad_degree,
                                       const uint8_t* flags_dev, int32_t codim, double* result);
/* MeshFunctionFE / MeshFunctionGradFE operator()(cell, local)
 * (fe/mesh_function_fe.h:72-91, fe/mesh_function_grad_fe.h:93-118) for every
 * cell at the same npts reference points ref_points[2 k], ref_points[2 k + 1]
 * (host): values_dev[cell * npts + k] and grads_dev[(cell * npts + k) * 2 + d]
 * (either may be NULL).  Lagrangian (O1-O3) or hierarchic spaces (each cell's
 * own FeHierarchicTria / Quad shape functions). */
lfg_status lfg_fe_eval(lfg_space* space, const double* dofs_dev, int32_t npts, const double* ref_points,
                       double* values_dev, double* grads_dev);
/* NodalProjection(fe_space, u, pred) (fe/fe_tools.h:198-259): per selected
 * cell (cell_flags_dev, NULL: all) u at the cell's EvaluationNodes, mapped to
 * dofs by its NodalValuesToDofs.  Lagrangian spaces: the identity, out_dev[dof]
 * = u at the dof's node.  Hierarchic spaces (uniform or per-entity degrees):
 * the dual bases of FeHierarchicTria / FeHierarchicQuad (fe/hierarchic_fe.h:
 * 820-1083, 1445-1680; the tables of lfg_hier_dual), FP64.  Cells are taken in
 * index order; a dof shared by several selected cells takes the value of the
 * last one (the reference sets, it does not add); dofs of no selected cell
 * are 0.  Per-entity degree spaces whose distinct (type, degrees,
 * orientation) combinations need more than 1 GiB of tables: LFG_UNSUPPORTED. */
lfg_status lfg_nodal_projection(lfg_space* space, const lfg_coeff* u, const uint8_t* cell_flags_dev,
                                double* out_dev);
/* InitEssentialConditionFromFunction(fes, esscondflag, g) (fe/fe_tools.h:263-329):
 * for every edge selected by edge_flags_dev (num_edges entries), its dofs get
 * flag 1 and the value of g at their segment evaluation node (the last
 * selected edge wins for a shared node); every other dof gets (0, 0.0).  The
 * two outputs are the (flag, value) pairs FixFlaggedSolutionComponents takes. */
lfg_status lfg_init_essential_condition(lfg_space* space, const uint8_t* edge_flags_dev, const lfg_coeff* g,
                                        uint8_t* dof_flags_dev, double* dof_values_dev);

#ifdef __cplusplus
}
#endif
#endif /* LFG_H_ */
