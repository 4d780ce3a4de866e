// Internal declarations of the GB300 library behind include/lfg.h.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <string>
#include <vector>

#include "../../include/lfg.h"
#include "lfg_tables.h"

namespace lfg {

// Status with message: every entry point converts an exception of this type
// into its return code and stores the message on the context.
struct Failure {
  lfg_status code;
  std::string msg;
};

[[noreturn]] void Fail(lfg_status code, const std::string& msg);
void CudaCheck(cudaError_t e, const char* what);
#define LFG_CUDA(call) ::lfg::CudaCheck((call), #call)

// Owning device buffer (stream-ordered allocation on the context stream).
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaStream_t stream = nullptr;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept { *this = std::move(o); }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) {
      reset();
      p = o.p; bytes = o.bytes; stream = o.stream;
      o.p = nullptr; o.bytes = 0;
    }
    return *this;
  }
  ~DevBuf() { reset(); }
  void alloc(size_t n, cudaStream_t s);
  void reset();
  template <class T> T* as() const { return static_cast<T*>(p); }
};

}  // namespace lfg

namespace lfg {
// Layout of one device table block (reference-element data for one cell type,
// degree and quadrature rule); offsets are in doubles.
struct Tab {
  int n, nq, E;
  int off_w, off_qx, off_qy, off_phi, off_T, off_R, off_L, off_o1, off_G, total;
};
struct TableEntry {
  Tab layout;
  DevBuf buf;
};
struct DfTableEntry {
  DfLayout layout;
  DevBuf buf;
};
}  // namespace lfg

struct lfg_ctx {
  // Meshes, COO and CSR matrices hold a reference; lfg_ctx_destroy only marks
  // the context and the last release frees it, so a handle destroyed after its
  // context is still safe.
  int64_t refs = 0;
  bool destroyed = false;
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  std::string last_error;
  int64_t launches = 0;
  int num_sms = 0;
  lfg::DevBuf flush;   // L2 flush buffer
  lfg::DevBuf status;  // device error word(s)
  // pinned host mirror of small device results
  void* pinned_small = nullptr;
  // reference-element tables keyed by (cell type, degree, rule degree)
  std::map<int, lfg::TableEntry> tables;
  std::map<int, lfg::DfTableEntry> dftables;
  uint32_t sf_const_ready = 0;  // constant-memory slots of the sum-factorised quad tables filled on this context
  // table digits of the tensor-core quad kernel, keyed by the FP64 table block
  std::map<const double*, lfg::DevBuf> tc_images;
  int tensor_cores = 3;  // Q2 quadrilaterals on the tcgen05 path (lfg_ctx_set_tensor_cores; 3 = producer-written triplets)
  // per-kernel-family event timing (lfg_profile_*)
  bool profiling = false;
  struct ProfRec {
    std::string family;
    cudaEvent_t a, b;
  };
  std::vector<ProfRec> prof_pending;
  std::map<std::string, std::pair<double, int64_t>> prof_totals;
  std::vector<cudaEvent_t> event_pool;
  // page-locked host allocations made by lfg_host_alloc (base -> bytes); a
  // host output that lies inside one is written by the kernels directly
  std::map<uintptr_t, size_t> host_allocs;
};

namespace lfg {
void RetainCtx(lfg_ctx* ctx);
void ReleaseCtx(lfg_ctx* ctx);
// First member of every handle: declared first, destroyed last, so the
// handle's device buffers are freed before the context reference is dropped.
struct CtxRef {
  lfg_ctx* c = nullptr;
  CtxRef() = default;
  CtxRef(const CtxRef&) = delete;
  CtxRef& operator=(const CtxRef&) = delete;
  void Set(lfg_ctx* x) {
    c = x;
    RetainCtx(x);
  }
  ~CtxRef() {
    if (c) ReleaseCtx(c);
  }
};

// Brackets the launches inside its lifetime with events on the context stream
// when profiling is enabled.
struct ProfScope {
  lfg_ctx* ctx;
  size_t idx = static_cast<size_t>(-1);
  ProfScope(lfg_ctx* c, const char* family);
  ~ProfScope();
};
}  // namespace lfg

struct lfg_mesh {
  lfg::CtxRef ref;
  lfg_ctx* ctx = nullptr;
  int64_t nv = 0, ne = 0, nc = 0, ntria = 0, nquad = 0;
  lfg::DevBuf xy;          // double2[nv]
  lfg::DevBuf cell_nodes;  // int4[nc]  (w = -1 for a triangle)
  lfg::DevBuf cell_edges;  // int4[nc]
  lfg::DevBuf cell_ori;    // uint8[nc]: bit j set = local edge j negatively oriented
  lfg::DevBuf edge_nodes;  // int2[ne]
  lfg::DevBuf edge_ncell;  // int32[ne]
  int64_t nonaffine_quads = -1;  // quadrilaterals that are not parallelograms (-1: not counted yet)
  lfg::DevBuf tria_list;   // int32[ntria]: cell indices of triangles (ascending)
  lfg::DevBuf quad_list;   // int32[nquad]
  std::vector<int32_t> h_tria_list, h_quad_list;  // host copies (cell-range splits), made when first needed
};

namespace lfg {
constexpr int kMaxLocalDofs = 1024;  // local shape functions per cell ((p+1)^2 <= 1024)
constexpr int kMaxHierDegree = 20;   // hierarchic degree (quadrilateral: 441 local dofs)
}  // namespace lfg

namespace lfg {
// Cells of one type and one hierarchic degree D (max of the cell's and its
// edges' degrees): entries [start, start + count) of lfg_space::hv_sorted.
struct HierGroup {
  bool quad = false;
  int degree = 0;
  int64_t start = 0, count = 0;
};
// Shape values and reference gradients of the uniform degree-p hierarchic
// element at the points of the rule of `rule_degree`, cached on the context
// (lfg_hier.cu): w[nq] | x[nq] | y[nq] at the start, then per orientation
// pattern pat (stride doubles apart, from off_pat) phi[nq][n] and, at o_g
// within the pattern block, grad[nq][n][2].
struct HierTabView {
  int n = 0, nq = 0;
  int64_t off_pat = 0, stride = 0, o_g = 0;
};
const double* HierShapeTable(lfg_ctx* ctx, bool quad, int p, int rule_degree, HierTabView& v);
// The same layout at given reference points (weights 0), on the host.
void HierShapeTableAt(bool quad, int p, const std::vector<double>& x, const std::vector<double>& y,
                      std::vector<double>& h, HierTabView& v);
}  // namespace lfg

struct lfg_space {
  lfg::CtxRef ref;
  lfg_mesh* mesh = nullptr;
  int degree = 0;  // 0 = generic layout
  int hier_degree = 0;  // > 0: HierarchicScalarFESpace of this uniform degree (generic layout)
  // Per-entity hierarchic degrees (HierarchicScalarFESpace with a degree
  // functor, DynamicFEDofHandler numbering); hier_degree is then the largest.
  bool hier_var = false;
  lfg::DevBuf hv_edge_deg;    // int32[ne]
  lfg::DevBuf hv_edge_first;  // int64[ne + 1]: first interior dof of each edge, minus the node count
  lfg::DevBuf hv_sel;         // uint16[nc * n_cell]: degree-D basis slot of every local shape function
  lfg::DevBuf hv_sorted;      // int32[nc]: triangles, then quadrilaterals, each stably grouped by D
  std::vector<lfg::HierGroup> hv_groups;
  std::vector<int32_t> hv_edge_deg_host, hv_cell_deg_host;
  int np = 0, ns = 0, nt = 0, nq = 0;
  int n_tria = 0, n_quad = 0, n_cell = 0, n_edge = 0;
  int64_t num_dofs = 0;
  int64_t num_triplets = 0;   // sum_K n_K^2
  int64_t num_local = 0;      // sum_K n_K
  lfg::DevBuf cell_dofs;      // int32[nc * n_cell]
  lfg::DevBuf tri_offset;     // int64[nc + 1]: prefix of n_K^2 (hybrid meshes)
  lfg::DevBuf loc_offset;     // int64[nc + 1]: prefix of n_K
  // dof -> (cell, local) incidence sorted by (dof, cell): deterministic
  // AssembleVectorLocally as a per-dof ordered gather.
  lfg::DevBuf inc_ptr;        // int64[num_dofs + 1]
  lfg::DevBuf inc_slot;       // int64[sum_K n_K]: loc_offset[cell] + local
  lfg::DevBuf scratch_vec;    // double[sum_K n_K] element vectors
};

struct lfg_coo {
  lfg::CtxRef ref;
  lfg_ctx* ctx = nullptr;
  int64_t rows = 0, cols = 0, capacity = 0, size = 0;
  lfg_triplet* d = nullptr;
  lfg::DevBuf owned;
};

struct lfg_csr {
  lfg::CtxRef ref;
  lfg_ctx* ctx = nullptr;
  int64_t rows = 0, cols = 0, nnz = 0;
  lfg::DevBuf rowptr;  // int64[rows + 1]
  lfg::DevBuf col;     // int32[nnz]
  lfg::DevBuf val;     // double[nnz]
  lfg::DevBuf val32;   // float[nnz] (mixed-precision solve, built lazily)
  lfg::DevBuf rowptr32;  // int32[rows + 1] when nnz < 2^31 (SpMV)
  lfg::DevBuf dinv;    // double[rows] Jacobi
  lfg::DevBuf dinv32;  // float[rows]
  // SELL-32 copy for the PCG SpMV (built with the preconditioner): slice s
  // holds rows 32s..32s+31 column-major, width = longest row of the slice;
  // entry (s, k, lane) at sell_ptr[s] + 32 k + lane; padding has col = row, 0.
  int64_t nslices = 0, sell_nnz = 0;
  lfg::DevBuf sell_ptr;    // int64[nslices + 1]
  lfg::DevBuf sell_col;    // int32[sell_nnz]
  lfg::DevBuf sell_val;    // double[sell_nnz]
  lfg::DevBuf sell_val32;  // float[sell_nnz] (mixed precision, built lazily)
  lfg::DevBuf rowsum32;    // float[rows]: FP64 row sums rounded once (the FP32 SpMV's difference form)
};

namespace lfg {

// Context lifetime: children retain the context; the last release after
// lfg_ctx_destroy frees it.
void RetainCtx(lfg_ctx* ctx);
void ReleaseCtx(lfg_ctx* ctx);

// Grid-size helper: multiples of the SM count for grid-stride kernels.
int GridFor(lfg_ctx* ctx, int64_t n, int block, int per_thread = 1);
void CountLaunch(lfg_ctx* ctx, int n = 1);

// ---- device primitives (lfg_primitives.cu) ----
// Exclusive scan of int64 values (in-place allowed).  Returns the total.
int64_t ExclusiveScanI64(lfg_ctx* ctx, const int64_t* in, int64_t* out, int64_t n);
// Stable LSD radix sort of (uint64 key, uint32 value) pairs on the low `bits`
// bits of the key.  keys/vals are overwritten with the sorted sequence.
void RadixSortPairs(lfg_ctx* ctx, uint64_t* keys, uint32_t* vals, int64_t n, int bits);
// Same with 64-bit payloads.
void RadixSortPairs64(lfg_ctx* ctx, uint64_t* keys, uint64_t* vals, int64_t n, int bits);
// Read a device int32 error word written by kernels (0 = ok); resets it.
int32_t ReadAndClearStatus(lfg_ctx* ctx, int32_t* detail = nullptr);
int32_t* StatusWord(lfg_ctx* ctx);
// Copy a small device value to the host synchronously (stream ordered).
// Stream-ordered device -> host read followed by a stream synchronize; reads
// up to kPinnedSmallBytes go through the context's pinned staging buffer.
constexpr size_t kPinnedSmallBytes = 4096;
void D2HSync(lfg_ctx* ctx, void* host, const void* dev, size_t bytes);
// Device address of host[0 .. bytes) when that range lies inside one
// page-locked allocation made by lfg_host_alloc on this context, else null.
void* MappedHost(lfg_ctx* ctx, const void* host, size_t bytes);
// Device -> host copy on the context stream (not synchronized).  Into a
// mapped allocation (MappedHost) of at least kMappedCopyBytes with 16-byte
// aligned ends, a copy kernel stores through the mapping: it runs at the
// host link's rate, which the copy engines do not reach on every box (they
// moved 54 GB/s on one GB300 machine where kernel stores moved 190 GB/s).
constexpr size_t kMappedCopyBytes = size_t(1) << 20;
void CopyToHost(lfg_ctx* ctx, void* host, const void* dev, size_t bytes);
// Solver data of a CSR matrix (lfg_csr.cu): Jacobi diagonal (FP64 + FP32),
// int32 row pointers and the SELL-32 copy; FP32 values for mixed precision.
void PrepareSolve(lfg_csr* A);
void EnsureFloatValues(lfg_csr* A);
// b[dof] += the element vectors in sp->scratch_vec, cells in ascending order
// (AssembleVectorLocally order), through the space's dof incidence.
void GatherElementVectors(lfg_space* sp, double* b);
void EnsureIncidence(lfg_space* sp);
// Hierarchic (hp) spaces (lfg_hier.cu): fe::DiffusionElementMatrixProvider +
// fe::MassElementMatrixProvider and fe::ScalarLoadElementVectorProvider.
void HierAssembleMatrix(lfg_space* sp, const lfg_rd_provider* pr, lfg_coo* coo);
void HierAssembleVector(lfg_space* sp, const lfg_load_provider* pr, double* b);

}  // namespace lfg
