// UniformFEDofHandler on the device (assemble/dofhandler.cc:86-338).
//
// Global numbering: node dofs first (node order), then interior dofs of the
// edges (edge order), then interior dofs of the cells (cell order).  The
// local dofs of a cell are its vertices' dofs, then per local edge the edge's
// interior dofs (reversed when the edge is negatively oriented relative to
// the cell), then the cell's own interior dofs.  Rows of the cell table have
// the stride max(n_tria, n_quad) like dofs_[kCellOrd] in the reference.
#include <algorithm>
#include <string>

#include "lfg_api.h"
#include "lfg_internal.h"

namespace lfg {
namespace {

__global__ void CellCountsKernel(int64_t nc, const int4* __restrict__ cells, int n_tria,
                                 int n_quad, int nt, int nq, int64_t* __restrict__ nint,
                                 int64_t* __restrict__ nloc, int64_t* __restrict__ nsq) {
  for (int64_t c = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; c < nc;
       c += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const bool q = cells[c].w >= 0;
    const int n = q ? n_quad : n_tria;
    nint[c] = q ? nq : nt;
    nloc[c] = n;
    nsq[c] = static_cast<int64_t>(n) * n;
  }
}

__global__ void CellDofsKernel(int64_t nc, int64_t nv, int64_t ne, const int4* __restrict__ cells,
                               const int4* __restrict__ cell_edges, const uint8_t* __restrict__ ori,
                               const int64_t* __restrict__ int_prefix, int np, int ns, int nt,
                               int nq, int n_cell, int32_t* __restrict__ out) {
  for (int64_t c = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; c < nc;
       c += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int4 cn = cells[c];
    const int4 ce = cell_edges[c];
    const int nvert = cn.w < 0 ? 3 : 4;
    const int v[4] = {cn.x, cn.y, cn.z, cn.w};
    const int e[4] = {ce.x, ce.y, ce.z, ce.w};
    const uint8_t o = ori[c];
    int32_t* row = out + c * n_cell;
    int k = 0;
    for (int j = 0; j < nvert; ++j)
      for (int a = 0; a < np; ++a) row[k++] = static_cast<int32_t>(static_cast<int64_t>(v[j]) * np + a);
    const int64_t edge_base = nv * np;
    for (int j = 0; j < nvert; ++j) {
      const int64_t b = edge_base + static_cast<int64_t>(e[j]) * ns;
      const bool neg = (o >> j) & 1;
      for (int a = 0; a < ns; ++a) row[k++] = static_cast<int32_t>(b + (neg ? ns - 1 - a : a));
    }
    const int nint = nvert == 3 ? nt : nq;
    const int64_t ib = edge_base + ne * ns + int_prefix[c];
    for (int a = 0; a < nint; ++a) row[k++] = static_cast<int32_t>(ib + a);
    for (; k < n_cell; ++k) row[k] = -1;
  }
}

__global__ void IncidenceItemsKernel(int64_t nc, const int32_t* __restrict__ cell_dofs, int n_cell,
                                     const int64_t* __restrict__ loc_offset,
                                     uint64_t* __restrict__ keys, uint64_t* __restrict__ vals) {
  for (int64_t c = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; c < nc;
       c += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t b = loc_offset[c], n = loc_offset[c + 1] - b;
    for (int i = 0; i < n; ++i) {
      keys[b + i] = static_cast<uint64_t>(cell_dofs[c * n_cell + i]);
      vals[b + i] = static_cast<uint64_t>(b + i);
    }
  }
}

__global__ void IncidencePtrKernel(int64_t n, const uint64_t* __restrict__ keys, int64_t ndofs,
                                   int64_t* __restrict__ ptr) {
  // ptr[d] = first position with key >= d (keys sorted)
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t k = static_cast<int64_t>(keys[i]);
    const int64_t prev = i == 0 ? -1 : static_cast<int64_t>(keys[i - 1]);
    for (int64_t d = prev + 1; d <= k; ++d) ptr[d] = i;
    if (i == n - 1)
      for (int64_t d = k + 1; d <= ndofs; ++d) ptr[d] = n;
  }
}

__global__ void BoundaryDofKernel(int64_t nv, int64_t ne, int np, int ns,
                                  const uint8_t* __restrict__ nf, const uint8_t* __restrict__ ef,
                                  uint8_t* __restrict__ flags) {
  const int64_t total = nv * np + ne * ns;
  for (int64_t d = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; d < total;
       d += static_cast<int64_t>(gridDim.x) * blockDim.x)
    flags[d] = d < nv * np ? nf[d / np] : ef[(d - nv * np) / ns];
}

// ---- per-entity hierarchic degrees (DynamicFEDofHandler layout) ----

// Interior dofs of a cell of hierarchic degree p (NumRefShapeFunctions(0),
// fe/hierarchic_fe.h:528-535, 1198-1205).
__device__ __forceinline__ int HierInterior(bool quad, int p) {
  return quad ? (p - 1) * (p - 1) : (p <= 2 ? 0 : (p - 2) * (p - 1) / 2);
}

__global__ void EdgeDofCountKernel(int64_t ne, const int32_t* __restrict__ edeg, int64_t* __restrict__ cnt) {
  for (int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < ne;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x)
    cnt[e] = edeg[e] - 1;
}

// Per cell: interior and local dof counts, the local count squared (triplets)
// and D = max(cell degree, edge degrees, 1), the degree of its basis table.
__global__ void VarCellCountsKernel(int64_t nc, const int4* __restrict__ cells, const int4* __restrict__ cell_edges,
                                    const int32_t* __restrict__ edeg, const int32_t* __restrict__ cdeg,
                                    int64_t* __restrict__ nint, int64_t* __restrict__ nloc,
                                    int64_t* __restrict__ nsq, uint8_t* __restrict__ dcell) {
  for (int64_t c = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; c < nc;
       c += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int4 cn = cells[c], ce = cell_edges[c];
    const bool q = cn.w >= 0;
    const int nvert = q ? 4 : 3;
    const int e[4] = {ce.x, ce.y, ce.z, ce.w};
    const int pc = cdeg[c];
    int d = pc > 1 ? pc : 1, n = nvert;
    for (int j = 0; j < nvert; ++j) {
      const int pe = edeg[e[j]];
      d = pe > d ? pe : d;
      n += pe - 1;
    }
    const int ni = HierInterior(q, pc);
    n += ni;
    nint[c] = ni;
    nloc[c] = n;
    nsq[c] = static_cast<int64_t>(n) * n;
    dcell[c] = static_cast<uint8_t>(d);
  }
}

// Global dofs of every cell (vertices; per local edge its interior dofs,
// reversed on a negative orientation; the cell's interior dofs) and, for each
// local shape function, its slot in the uniform degree-D basis of the cell's
// orientation pattern: the hierarchic functions of an edge of degree pe are
// the first pe - 1 of degree D (stored reversed on a negative edge, so they
// sit at the end of the edge's D - 1 slots), and the interior functions of
// degree pc are the (i, j) pairs of degree D with the tighter bound.
__global__ void VarCellDofsKernel(int64_t nc, int64_t nv, int64_t edge_dofs, const int4* __restrict__ cells,
                                  const int4* __restrict__ cell_edges, const uint8_t* __restrict__ ori,
                                  const int32_t* __restrict__ edeg, const int32_t* __restrict__ cdeg,
                                  const int64_t* __restrict__ efirst, const int64_t* __restrict__ int_prefix,
                                  const uint8_t* __restrict__ dcell, int n_cell, int32_t* __restrict__ out,
                                  uint16_t* __restrict__ sel) {
  for (int64_t c = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; c < nc;
       c += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int4 cn = cells[c], ce = cell_edges[c];
    const bool q = cn.w >= 0;
    const int nvert = q ? 4 : 3;
    const int v[4] = {cn.x, cn.y, cn.z, cn.w};
    const int e[4] = {ce.x, ce.y, ce.z, ce.w};
    const uint8_t o = ori[c];
    const int D = dcell[c];
    int32_t* row = out + c * n_cell;
    uint16_t* srow = sel + c * n_cell;
    int k = 0;
    for (int j = 0; j < nvert; ++j, ++k) {
      row[k] = v[j];
      srow[k] = static_cast<uint16_t>(j);
    }
    for (int j = 0; j < nvert; ++j) {
      const int ns = edeg[e[j]] - 1;
      const int64_t b = nv + efirst[e[j]];
      const bool neg = (o >> j) & 1;
      const int ub = nvert + j * (D - 1);
      for (int a = 0; a < ns; ++a, ++k) {
        row[k] = static_cast<int32_t>(b + (neg ? ns - 1 - a : a));
        srow[k] = static_cast<uint16_t>(ub + (neg ? D - 1 - ns + a : a));
      }
    }
    const int pc = cdeg[c];
    const int64_t ib = nv + edge_dofs + int_prefix[c];
    const int ub = nvert * D;  // nvert + nvert (D - 1)
    int a = 0;
    if (q) {
      for (int i = 0; i < pc - 1; ++i)
        for (int jj = 0; jj < pc - 1; ++jj, ++k, ++a) {
          row[k] = static_cast<int32_t>(ib + a);
          srow[k] = static_cast<uint16_t>(ub + i * (D - 1) + jj);
        }
    } else {
      for (int i = 0; i < pc - 2; ++i)
        for (int jj = 0; jj < pc - 2 - i; ++jj, ++k, ++a) {
          row[k] = static_cast<int32_t>(ib + a);
          srow[k] = static_cast<uint16_t>(ub + i * (D - 2) - i * (i - 1) / 2 + jj);
        }
    }
    for (; k < n_cell; ++k) {
      row[k] = -1;
      srow[k] = 0;
    }
  }
}

// (D, cell) pairs of one cell-type list, and the count of every D.
__global__ void GroupKeysKernel(int64_t n, const int32_t* __restrict__ list, const uint8_t* __restrict__ dcell,
                                uint64_t* __restrict__ keys, uint64_t* __restrict__ vals,
                                unsigned long long* __restrict__ hist) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int c = list[i];
    const int d = dcell[c];
    keys[i] = static_cast<uint64_t>(d);
    vals[i] = static_cast<uint64_t>(c);
    atomicAdd(hist + d, 1ull);
  }
}

__global__ void NarrowKernel(int64_t n, const uint64_t* __restrict__ in, int32_t* __restrict__ out) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    out[i] = static_cast<int32_t>(in[i]);
}

// Boundary flags of a variable-degree space: node dof v = node v, edge e's
// dofs from its first interior dof on.
__global__ void BoundaryDofVarKernel(int64_t nv, int64_t ne, const int32_t* __restrict__ edeg,
                                     const int64_t* __restrict__ efirst, const uint8_t* __restrict__ nf,
                                     const uint8_t* __restrict__ ef, uint8_t* __restrict__ flags) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < nv + ne;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    if (i < nv) {
      flags[i] = nf[i];
    } else {
      const int64_t e = i - nv;
      for (int a = 0; a < edeg[e] - 1; ++a) flags[nv + efirst[e] + a] = ef[e];
    }
  }
}

int BitsFor(int64_t n) {
  int b = 1;
  while ((int64_t(1) << b) < n + 1) ++b;
  return b;
}

}  // namespace

// dof -> (cell, local) incidence in ascending cell order, built on demand.
void EnsureIncidence(lfg_space* sp) {
  if (sp->inc_ptr.p) return;
  lfg_ctx* ctx = sp->mesh->ctx;
  cudaStream_t s = ctx->stream;
  const int64_t nloc = sp->num_local;
  DevBuf keys;
  keys.alloc(std::max<int64_t>(nloc, 1) * sizeof(uint64_t), s);
  sp->inc_slot.alloc(std::max<int64_t>(nloc, 1) * sizeof(uint64_t), s);
  IncidenceItemsKernel<<<GridFor(ctx, sp->mesh->nc, 256), 256, 0, s>>>(
      sp->mesh->nc, sp->cell_dofs.as<int32_t>(), sp->n_cell, sp->loc_offset.as<int64_t>(),
      keys.as<uint64_t>(), sp->inc_slot.as<uint64_t>());
  LFG_LAUNCHED(ctx);
  RadixSortPairs64(ctx, keys.as<uint64_t>(), sp->inc_slot.as<uint64_t>(), nloc, BitsFor(sp->num_dofs));
  sp->inc_ptr.alloc((sp->num_dofs + 1) * sizeof(int64_t), s);
  LFG_CUDA(cudaMemsetAsync(sp->inc_ptr.p, 0, (sp->num_dofs + 1) * sizeof(int64_t), s));
  IncidencePtrKernel<<<GridFor(ctx, nloc, 256), 256, 0, s>>>(nloc, keys.as<uint64_t>(), sp->num_dofs,
                                                             sp->inc_ptr.as<int64_t>());
  LFG_LAUNCHED(ctx);
  sp->scratch_vec.alloc(std::max<int64_t>(nloc, 1) * sizeof(double), s);
}

}  // namespace lfg

using namespace lfg;

extern "C" {

lfg_status lfg_space_create(lfg_mesh* m, int np, int ns, int nt, int nq, lfg_space** out) {
  if (!m) return LFG_INVALID_ARG;
  LFG_API_BEGIN(m->ctx)
  if (!out || np < 0 || ns < 0 || nt < 0 || nq < 0 || np > 1)
    Fail(LFG_INVALID_ARG, "lfg_space_create: layout must have np in {0,1} and non-negative counts");
  *out = nullptr;
  auto* sp = new lfg_space;
  try {
    cudaStream_t s = m->ctx->stream;
    sp->ref.Set(m->ctx);
    sp->mesh = m;
    sp->np = np; sp->ns = ns; sp->nt = nt; sp->nq = nq;
    // InitTotalNumDofs (dofhandler.cc:131-139)
    sp->n_edge = 2 * np + ns;
    sp->n_tria = 3 * np + 3 * ns + nt;
    sp->n_quad = 4 * np + 4 * ns + nq;
    sp->n_cell = std::max(sp->n_tria, sp->n_quad);
    if (sp->n_cell > kMaxLocalDofs || sp->n_cell == 0)
      Fail(LFG_UNSUPPORTED, "at most " + std::to_string(kMaxLocalDofs) + " local dofs per cell are supported");
    const int64_t nc = m->nc;
    DevBuf nint;
    nint.alloc((nc + 1) * sizeof(int64_t), s);
    sp->loc_offset.alloc((nc + 1) * sizeof(int64_t), s);
    sp->tri_offset.alloc((nc + 1) * sizeof(int64_t), s);
    CellCountsKernel<<<GridFor(m->ctx, nc, 256), 256, 0, s>>>(
        nc, m->cell_nodes.as<int4>(), sp->n_tria, sp->n_quad, nt, nq, nint.as<int64_t>(),
        sp->loc_offset.as<int64_t>(), sp->tri_offset.as<int64_t>());
    LFG_LAUNCHED(m->ctx);
    LFG_CUDA(cudaMemsetAsync(nint.as<int64_t>() + nc, 0, sizeof(int64_t), s));
    LFG_CUDA(cudaMemsetAsync(sp->loc_offset.as<int64_t>() + nc, 0, sizeof(int64_t), s));
    LFG_CUDA(cudaMemsetAsync(sp->tri_offset.as<int64_t>() + nc, 0, sizeof(int64_t), s));
    const int64_t n_int = ExclusiveScanI64(m->ctx, nint.as<int64_t>(), nint.as<int64_t>(), nc + 1);
    sp->num_local = ExclusiveScanI64(m->ctx, sp->loc_offset.as<int64_t>(), sp->loc_offset.as<int64_t>(), nc + 1);
    sp->num_triplets = ExclusiveScanI64(m->ctx, sp->tri_offset.as<int64_t>(), sp->tri_offset.as<int64_t>(), nc + 1);
    sp->num_dofs = m->nv * np + m->ne * ns + n_int;
    if (sp->num_dofs >= (int64_t(1) << 31)) Fail(LFG_UNSUPPORTED, "more than 2^31 dofs");
    sp->cell_dofs.alloc(nc * sp->n_cell * sizeof(int32_t), s);
    CellDofsKernel<<<GridFor(m->ctx, nc, 256), 256, 0, s>>>(
        nc, m->nv, m->ne, m->cell_nodes.as<int4>(), m->cell_edges.as<int4>(), m->cell_ori.as<uint8_t>(),
        nint.as<int64_t>(), np, ns, nt, nq, sp->n_cell, sp->cell_dofs.as<int32_t>());
    LFG_LAUNCHED(m->ctx);
    LFG_CUDA(cudaStreamSynchronize(s));
  } catch (...) {
    delete sp;
    throw;
  }
  *out = sp;
  LFG_API_END
}

lfg_status lfg_space_create_lagrange(lfg_mesh* m, int degree, lfg_space** out) {
  if (degree < 1 || degree > 3) {
    if (m) m->ctx->last_error = "Lagrangian spaces of degree 1..3 only";
    return LFG_UNSUPPORTED;
  }
  const int p = degree;
  lfg_status st = lfg_space_create(m, 1, p - 1, (p - 1) * (p - 2) / 2, (p - 1) * (p - 1), out);
  if (st == LFG_OK) (*out)->degree = degree;
  return st;
}

// HierarchicScalarFESpace(mesh, degree) (fe/hierarchic_scalar_fe_space.h:36-46):
// one dof per node, degree-1 per edge, (p-2)(p-1)/2 per triangle and (p-1)^2
// per quadrilateral, numbered like DynamicFEDofHandler (assemble/dofhandler.h:
// 550-650), which for uniform counts is the uniform layout.
lfg_status lfg_space_create_hierarchic(lfg_mesh* m, int32_t degree, lfg_space** out) {
  if (degree < 1 || degree > kMaxHierDegree) {
    if (m) m->ctx->last_error = "hierarchic spaces of degree 1.." + std::to_string(kMaxHierDegree) + " only";
    return LFG_UNSUPPORTED;
  }
  const int p = degree;
  lfg_status st = lfg_space_create(m, 1, p - 1, p <= 2 ? 0 : (p - 2) * (p - 1) / 2, (p - 1) * (p - 1), out);
  if (st == LFG_OK) (*out)->hier_degree = degree;
  return st;
}

// HierarchicScalarFESpace(mesh, degree_functor) (fe/hierarchic_scalar_fe_space.h:
// 93-116, Init :178-220): the functor's values per edge and per cell, numbered
// like DynamicFEDofHandler (assemble/dofhandler.h:550-680): node dofs, then
// edge_degree[e] - 1 per edge in edge order, then the cell interiors in cell
// order.  Cells are grouped by D = max(cell degree, edge degrees, 1) so that
// each group runs the kernels of the uniform degree-D space with a per-cell
// selection of its shape functions.
lfg_status lfg_space_create_hierarchic_var(lfg_mesh* m, const int32_t* edge_degree, const int32_t* cell_degree,
                                           lfg_space** out) {
  if (!m) return LFG_INVALID_ARG;
  LFG_API_BEGIN(m->ctx)
  if (!out || (!edge_degree && m->ne > 0) || (!cell_degree && m->nc > 0))
    Fail(LFG_INVALID_ARG, "lfg_space_create_hierarchic_var: null argument");
  *out = nullptr;
  int dmax = 1;
  for (int64_t e = 0; e < m->ne; ++e) {
    if (edge_degree[e] < 1 || edge_degree[e] > kMaxHierDegree)
      Fail(LFG_UNSUPPORTED, "hierarchic degrees 1.." + std::to_string(kMaxHierDegree) + " only (edge " +
                                std::to_string(e) + ": " + std::to_string(edge_degree[e]) + ")");
    dmax = std::max(dmax, static_cast<int>(edge_degree[e]));
  }
  for (int64_t c = 0; c < m->nc; ++c) {
    if (cell_degree[c] < 1 || cell_degree[c] > kMaxHierDegree)
      Fail(LFG_UNSUPPORTED, "hierarchic degrees 1.." + std::to_string(kMaxHierDegree) + " only (cell " +
                                std::to_string(c) + ": " + std::to_string(cell_degree[c]) + ")");
    dmax = std::max(dmax, static_cast<int>(cell_degree[c]));
  }
  auto* sp = new lfg_space;
  try {
    lfg_ctx* ctx = m->ctx;
    cudaStream_t s = ctx->stream;
    const int64_t nc = m->nc, ne = m->ne;
    sp->ref.Set(ctx);
    sp->mesh = m;
    sp->np = 1;
    sp->hier_var = true;
    sp->hier_degree = dmax;
    // upper bounds of the local counts (the largest degree everywhere)
    sp->n_edge = dmax + 1;
    sp->n_tria = (dmax + 1) * (dmax + 2) / 2;
    sp->n_quad = (dmax + 1) * (dmax + 1);
    sp->n_cell = m->nquad > 0 ? sp->n_quad : sp->n_tria;
    sp->hv_edge_deg_host.assign(edge_degree, edge_degree + ne);
    sp->hv_cell_deg_host.assign(cell_degree, cell_degree + nc);
    DevBuf cdeg, nint, dcell;
    sp->hv_edge_deg.alloc(std::max<int64_t>(ne, 1) * sizeof(int32_t), s);
    cdeg.alloc(std::max<int64_t>(nc, 1) * sizeof(int32_t), s);
    if (ne) LFG_CUDA(cudaMemcpyAsync(sp->hv_edge_deg.p, edge_degree, ne * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    if (nc) LFG_CUDA(cudaMemcpyAsync(cdeg.p, cell_degree, nc * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    // edge interior dofs: exclusive prefix of edge_degree - 1
    sp->hv_edge_first.alloc((ne + 1) * sizeof(int64_t), s);
    if (ne) {
      EdgeDofCountKernel<<<GridFor(ctx, ne, 256), 256, 0, s>>>(ne, sp->hv_edge_deg.as<int32_t>(),
                                                               sp->hv_edge_first.as<int64_t>());
      LFG_LAUNCHED(ctx);
    }
    LFG_CUDA(cudaMemsetAsync(sp->hv_edge_first.as<int64_t>() + ne, 0, sizeof(int64_t), s));
    const int64_t edge_dofs =
        ExclusiveScanI64(ctx, sp->hv_edge_first.as<int64_t>(), sp->hv_edge_first.as<int64_t>(), ne + 1);
    // per-cell counts and degrees
    nint.alloc((nc + 1) * sizeof(int64_t), s);
    sp->loc_offset.alloc((nc + 1) * sizeof(int64_t), s);
    sp->tri_offset.alloc((nc + 1) * sizeof(int64_t), s);
    dcell.alloc(std::max<int64_t>(nc, 1), s);
    if (nc) {
      VarCellCountsKernel<<<GridFor(ctx, nc, 256), 256, 0, s>>>(
          nc, m->cell_nodes.as<int4>(), m->cell_edges.as<int4>(), sp->hv_edge_deg.as<int32_t>(), cdeg.as<int32_t>(),
          nint.as<int64_t>(), sp->loc_offset.as<int64_t>(), sp->tri_offset.as<int64_t>(), dcell.as<uint8_t>());
      LFG_LAUNCHED(ctx);
    }
    LFG_CUDA(cudaMemsetAsync(nint.as<int64_t>() + nc, 0, sizeof(int64_t), s));
    LFG_CUDA(cudaMemsetAsync(sp->loc_offset.as<int64_t>() + nc, 0, sizeof(int64_t), s));
    LFG_CUDA(cudaMemsetAsync(sp->tri_offset.as<int64_t>() + nc, 0, sizeof(int64_t), s));
    const int64_t n_int = ExclusiveScanI64(ctx, nint.as<int64_t>(), nint.as<int64_t>(), nc + 1);
    sp->num_local = ExclusiveScanI64(ctx, sp->loc_offset.as<int64_t>(), sp->loc_offset.as<int64_t>(), nc + 1);
    sp->num_triplets = ExclusiveScanI64(ctx, sp->tri_offset.as<int64_t>(), sp->tri_offset.as<int64_t>(), nc + 1);
    sp->num_dofs = m->nv + edge_dofs + n_int;
    if (sp->num_dofs >= (int64_t(1) << 31)) Fail(LFG_UNSUPPORTED, "more than 2^31 dofs");
    // dof rows and basis slots
    sp->cell_dofs.alloc(std::max<int64_t>(nc * sp->n_cell, 1) * sizeof(int32_t), s);
    sp->hv_sel.alloc(std::max<int64_t>(nc * sp->n_cell, 1) * sizeof(uint16_t), s);
    if (nc) {
      VarCellDofsKernel<<<GridFor(ctx, nc, 256), 256, 0, s>>>(
          nc, m->nv, edge_dofs, m->cell_nodes.as<int4>(), m->cell_edges.as<int4>(), m->cell_ori.as<uint8_t>(),
          sp->hv_edge_deg.as<int32_t>(), cdeg.as<int32_t>(), sp->hv_edge_first.as<int64_t>(), nint.as<int64_t>(),
          dcell.as<uint8_t>(), sp->n_cell, sp->cell_dofs.as<int32_t>(), sp->hv_sel.as<uint16_t>());
      LFG_LAUNCHED(ctx);
    }
    // cells grouped by type, then by D (stable: ascending cell order in a group)
    sp->hv_sorted.alloc(std::max<int64_t>(nc, 1) * sizeof(int32_t), s);
    int64_t pos = 0;
    for (int t = 0; t < 2; ++t) {
      const bool quad = t == 1;
      const int64_t n = quad ? m->nquad : m->ntria;
      if (!n) continue;
      DevBuf keys, vals, hist;
      keys.alloc(n * sizeof(uint64_t), s);
      vals.alloc(n * sizeof(uint64_t), s);
      hist.alloc(32 * sizeof(unsigned long long), s);
      LFG_CUDA(cudaMemsetAsync(hist.p, 0, 32 * sizeof(unsigned long long), s));
      GroupKeysKernel<<<GridFor(ctx, n, 256), 256, 0, s>>>(
          n, quad ? m->quad_list.as<int32_t>() : m->tria_list.as<int32_t>(), dcell.as<uint8_t>(),
          keys.as<uint64_t>(), vals.as<uint64_t>(), hist.as<unsigned long long>());
      LFG_LAUNCHED(ctx);
      RadixSortPairs64(ctx, keys.as<uint64_t>(), vals.as<uint64_t>(), n, 5);
      NarrowKernel<<<GridFor(ctx, n, 256), 256, 0, s>>>(n, vals.as<uint64_t>(), sp->hv_sorted.as<int32_t>() + pos);
      LFG_LAUNCHED(ctx);
      unsigned long long h[32];
      D2HSync(ctx, h, hist.p, sizeof(h));
      for (int d = 1; d <= kMaxHierDegree; ++d)
        if (h[d]) {
          HierGroup g;
          g.quad = quad;
          g.degree = d;
          g.start = pos;
          g.count = static_cast<int64_t>(h[d]);
          sp->hv_groups.push_back(g);
          pos += g.count;
        }
    }
    LFG_CUDA(cudaStreamSynchronize(s));
  } catch (...) {
    delete sp;
    throw;
  }
  *out = sp;
  LFG_API_END
}

lfg_status lfg_space_download_local_counts(lfg_space* sp, int32_t* n_local) {
  if (!sp || !n_local) return LFG_INVALID_ARG;
  LFG_API_BEGIN(sp->mesh->ctx)
  const int64_t nc = sp->mesh->nc;
  std::vector<int64_t> off(nc + 1);
  LFG_CUDA(cudaMemcpyAsync(off.data(), sp->loc_offset.p, (nc + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost,
                           sp->mesh->ctx->stream));
  LFG_CUDA(cudaStreamSynchronize(sp->mesh->ctx->stream));
  for (int64_t c = 0; c < nc; ++c) n_local[c] = static_cast<int32_t>(off[c + 1] - off[c]);
  LFG_API_END
}

lfg_status lfg_space_destroy(lfg_space* sp) {
  if (!sp) return LFG_INVALID_ARG;
  cudaSetDevice(sp->ref.c->device);
  delete sp;
  return LFG_OK;
}

lfg_status lfg_space_info(const lfg_space* sp, int64_t* num_dofs, int32_t* n_tria, int32_t* n_quad,
                          int32_t* n_cell, int64_t* num_triplets) {
  if (!sp) return LFG_INVALID_ARG;
  if (num_dofs) *num_dofs = sp->num_dofs;
  if (n_tria) *n_tria = sp->n_tria;
  if (n_quad) *n_quad = sp->n_quad;
  if (n_cell) *n_cell = sp->n_cell;
  if (num_triplets) *num_triplets = sp->num_triplets;
  return LFG_OK;
}

lfg_status lfg_space_download_cell_dofs(lfg_space* sp, int32_t* host) {
  if (!sp || !host) return LFG_INVALID_ARG;
  LFG_API_BEGIN(sp->mesh->ctx)
  LFG_CUDA(cudaMemcpyAsync(host, sp->cell_dofs.p, sp->mesh->nc * sp->n_cell * sizeof(int32_t),
                           cudaMemcpyDeviceToHost, sp->mesh->ctx->stream));
  LFG_CUDA(cudaStreamSynchronize(sp->mesh->ctx->stream));
  LFG_API_END
}

lfg_status lfg_space_download_dof_entities(lfg_space* sp, int8_t* codim, int32_t* index) {
  if (!sp || !codim || !index) return LFG_INVALID_ARG;
  LFG_API_BEGIN(sp->mesh->ctx)
  const lfg_mesh* m = sp->mesh;
  std::vector<int32_t> cd(m->nc * sp->n_cell);
  std::vector<int32_t> cn(4 * m->nc);
  LFG_CUDA(cudaMemcpyAsync(cd.data(), sp->cell_dofs.p, cd.size() * sizeof(int32_t), cudaMemcpyDeviceToHost, m->ctx->stream));
  LFG_CUDA(cudaMemcpyAsync(cn.data(), m->cell_nodes.p, cn.size() * sizeof(int32_t), cudaMemcpyDeviceToHost, m->ctx->stream));
  LFG_CUDA(cudaStreamSynchronize(m->ctx->stream));
  if (sp->hier_var) {
    // node v -> dof v; each edge's dofs in edge order; the cell interiors in cell order
    int64_t d = 0;
    for (; d < m->nv; ++d) {
      codim[d] = 2;
      index[d] = static_cast<int32_t>(d);
    }
    for (int64_t e = 0; e < m->ne; ++e)
      for (int a = 0; a < sp->hv_edge_deg_host[e] - 1; ++a, ++d) {
        codim[d] = 1;
        index[d] = static_cast<int32_t>(e);
      }
    for (int64_t c = 0; c < m->nc; ++c) {
      const int p = sp->hv_cell_deg_host[c];
      const int nint = cn[4 * c + 3] >= 0 ? (p - 1) * (p - 1) : (p <= 2 ? 0 : (p - 2) * (p - 1) / 2);
      for (int a = 0; a < nint; ++a, ++d) {
        codim[d] = 0;
        index[d] = static_cast<int32_t>(c);
      }
    }
    return LFG_OK;
  }
  const int64_t nnode = m->nv * sp->np, nedge = m->ne * sp->ns;
  for (int64_t d = 0; d < std::min<int64_t>(nnode + nedge, sp->num_dofs); ++d) {
    codim[d] = d < nnode ? 2 : 1;
    index[d] = static_cast<int32_t>(d < nnode ? d / sp->np : (d - nnode) / sp->ns);
  }
  for (int64_t c = 0; c < m->nc; ++c) {
    const bool q = cn[4 * c + 3] >= 0;
    const int n = q ? sp->n_quad : sp->n_tria, nint = q ? sp->nq : sp->nt;
    for (int a = n - nint; a < n; ++a) {
      const int32_t d = cd[c * sp->n_cell + a];
      codim[d] = 0;
      index[d] = static_cast<int32_t>(c);
    }
  }
  LFG_API_END
}

lfg_status lfg_space_boundary_dof_flags(lfg_space* sp, uint8_t* flags) {
  if (!sp || !flags) return LFG_INVALID_ARG;
  LFG_API_BEGIN(sp->mesh->ctx)
  lfg_mesh* m = sp->mesh;
  cudaStream_t s = m->ctx->stream;
  DevBuf nf, ef;
  nf.alloc(m->nv, s);
  ef.alloc(std::max<int64_t>(m->ne, 1), s);
  lfg_status st = lfg_mesh_boundary_flags(m, nf.as<uint8_t>(), ef.as<uint8_t>());
  if (st != LFG_OK) Fail(st, m->ctx->last_error);
  LFG_CUDA(cudaMemsetAsync(flags, 0, sp->num_dofs, s));
  if (sp->hier_var) {
    BoundaryDofVarKernel<<<GridFor(m->ctx, m->nv + m->ne, 256), 256, 0, s>>>(
        m->nv, m->ne, sp->hv_edge_deg.as<int32_t>(), sp->hv_edge_first.as<int64_t>(), nf.as<uint8_t>(),
        ef.as<uint8_t>(), flags);
    LFG_LAUNCHED(m->ctx);
    return LFG_OK;
  }
  BoundaryDofKernel<<<GridFor(m->ctx, m->nv * sp->np + m->ne * sp->ns, 256), 256, 0, s>>>(
      m->nv, m->ne, sp->np, sp->ns, nf.as<uint8_t>(), ef.as<uint8_t>(), flags);
  LFG_LAUNCHED(m->ctx);
  LFG_API_END
}

}  // extern "C"
