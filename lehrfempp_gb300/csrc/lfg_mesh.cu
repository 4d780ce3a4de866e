// Mesh construction on the device: the numbering of lf::mesh::hybrid2d::Mesh
// (mesh/hybrid2d/mesh.cc:178-810) computed by sorting half-edges instead of a
// std::map.
//
// Every preset edge and every (cell, local edge) becomes an item with key
// (min node << b) | max node and value = item index (presets first, then
// cells in (cell, local edge) order).  A stable radix sort groups equal keys
// in key order = the std::map iteration order, and inside a group keeps the
// creation order, so the first item of each group is the edge's creator
// (its direction), a preset in the group supplies the registration index, and
// groups without a preset are numbered after the presets in key order.
#include <algorithm>
#include <cstring>

#include "lfg_api.h"
#include "lfg_internal.h"

namespace lfg {
namespace {

constexpr int kBlock = 256;

// error codes written to the status word
enum : int32_t {
  kErrNone = 0,
  kErrBadNode = 1,
  kErrLoopEdge = 2,
  kErrDupPreset = 3,
  kErrEdgeNoCell = 4,
  kErrNodeNoEdge = 5,
  kErrDegenerate = 6,
};

__device__ void SetStatus(int32_t* st, int32_t code, int32_t detail) {
  if (atomicCAS(st, 0, code) == 0) st[1] = detail;
}

__global__ void ValidateAndItemsKernel(int64_t nv, int64_t nc, const int4* __restrict__ cells,
                                       int64_t npre, const int2* __restrict__ pre, int bits,
                                       uint64_t* __restrict__ keys, uint32_t* __restrict__ vals,
                                       int32_t* __restrict__ is_quad, int32_t* st) {
  const int64_t nitems = npre + 4 * nc;
  const uint64_t sentinel = (bits >= 64) ? ~0ull : ((1ull << bits) - 1ull);
  for (int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; t < nitems;
       t += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    int a, b;
    bool valid = true;
    if (t < npre) {
      const int2 e = pre[t];
      a = e.x;
      b = e.y;
      if (a < 0 || b < 0 || a >= nv || b >= nv) { SetStatus(st, kErrBadNode, static_cast<int32_t>(t)); valid = false; }
      else if (a == b) { SetStatus(st, kErrLoopEdge, static_cast<int32_t>(t)); valid = false; }
    } else {
      const int64_t c = (t - npre) >> 2;
      const int j = static_cast<int>((t - npre) & 3);
      const int4 cn = cells[c];
      const int nvert = cn.w < 0 ? 3 : 4;
      const int v[4] = {cn.x, cn.y, cn.z, cn.w};
      if (j == 0) {
        is_quad[c] = nvert == 4;
        for (int k = 0; k < nvert; ++k)
          if (v[k] < 0 || v[k] >= nv) SetStatus(st, kErrBadNode, static_cast<int32_t>(c));
      }
      if (j >= nvert) {
        valid = false;
        a = b = 0;
      } else {
        a = v[j];
        b = v[(j + 1) % nvert];
        if (a < 0 || b < 0 || a >= nv || b >= nv) valid = false;
        else if (a == b) { SetStatus(st, kErrLoopEdge, static_cast<int32_t>(c)); valid = false; }
      }
    }
    const uint64_t lo = static_cast<uint64_t>(min(a, b)), hi = static_cast<uint64_t>(max(a, b));
    keys[t] = valid ? ((lo << (bits / 2)) | hi) : sentinel;
    vals[t] = static_cast<uint32_t>(t);
  }
}

__global__ void RunHeadsKernel(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ vals,
                               int64_t n, uint64_t sentinel, int64_t npre,
                               int64_t* __restrict__ head, int64_t* __restrict__ head_nopre) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const uint64_t k = keys[i];
    const bool h = k != sentinel && (i == 0 || keys[i - 1] != k);
    head[i] = h;
    head_nopre[i] = h && vals[i] >= npre;
  }
}

__global__ void NumberEdgesKernel(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ vals,
                                  int64_t n, uint64_t sentinel, int64_t npre,
                                  const int64_t* __restrict__ head, const int64_t* __restrict__ rank,
                                  const int2* __restrict__ pre, const int4* __restrict__ cells,
                                  int2* __restrict__ edge_nodes, int32_t* __restrict__ edge_ncell,
                                  int4* __restrict__ cell_edges, int32_t* st) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const uint64_t k = keys[i];
    if (k == sentinel || (i > 0 && keys[i - 1] == k)) continue;  // not a group head
    const uint32_t creator = vals[i];
    int g;
    int2 ends;
    if (creator < npre) {
      g = static_cast<int>(creator);
      ends = pre[creator];
    } else {
      g = static_cast<int>(npre + rank[i]);
      const int64_t c = (creator - npre) >> 2;
      const int j = static_cast<int>((creator - npre) & 3);
      const int4 cn = cells[c];
      const int nvert = cn.w < 0 ? 3 : 4;
      const int v[4] = {cn.x, cn.y, cn.z, cn.w};
      ends = make_int2(v[j], v[(j + 1) % nvert]);
    }
    int ncell = 0;
    for (int64_t m = i; m < n && keys[m] == k; ++m) {
      const uint32_t it = vals[m];
      if (it < npre) {
        if (m != i) SetStatus(st, kErrDupPreset, static_cast<int32_t>(it));
        continue;
      }
      const int64_t c = (it - npre) >> 2;
      const int j = static_cast<int>((it - npre) & 3);
      reinterpret_cast<int*>(&cell_edges[c])[j] = g;
      ++ncell;
    }
    edge_nodes[g] = ends;
    edge_ncell[g] = ncell;
    if (ncell == 0) SetStatus(st, kErrEdgeNoCell, g);
  }
}

__global__ void CellOrientationKernel(int64_t nc, const int4* __restrict__ cells,
                                      const int4* __restrict__ cell_edges,
                                      const int2* __restrict__ edge_nodes,
                                      const double2* __restrict__ xy, uint8_t* __restrict__ ori,
                                      int32_t* st) {
  for (int64_t c = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; c < nc;
       c += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int4 cn = cells[c];
    const int4 ce = cell_edges[c];
    const int nvert = cn.w < 0 ? 3 : 4;
    const int v[4] = {cn.x, cn.y, cn.z, cn.w};
    const int e[4] = {ce.x, ce.y, ce.z, ce.w};
    uint8_t bits = 0;
    for (int j = 0; j < nvert; ++j)
      if (edge_nodes[e[j]].x != v[j]) bits |= static_cast<uint8_t>(1u << j);
    ori[c] = bits;
    // geometry/tria_o1.cc:10-48 and quad_o1.cc:12-58 with tol = 1e-8
    double2 p[4];
    for (int j = 0; j < nvert; ++j) p[j] = xy[v[j]];
    double len[4], circum = 0.0;
    for (int j = 0; j < nvert; ++j) {
      const double2 a = p[j], b = p[(j + 1) % nvert];
      len[j] = (b.x - a.x) * (b.x - a.x) + (b.y - a.y) * (b.y - a.y);
      circum += len[j];
    }
    bool ok = true;
    for (int j = 0; j < nvert; ++j) ok = ok && (len[j] > 1.0e-8 * circum);
    double area = fabs((p[1].x - p[0].x) * (p[2].y - p[0].y) - (p[1].y - p[0].y) * (p[2].x - p[0].x));
    if (nvert == 4)
      area += fabs((p[3].x - p[0].x) * (p[2].y - p[0].y) - (p[3].y - p[0].y) * (p[2].x - p[0].x));
    ok = ok && (area > 1.0e-8 * circum);
    if (!ok) SetStatus(st, kErrDegenerate, static_cast<int32_t>(c));
  }
}

__global__ void NodeUseKernel(int64_t ne, const int2* __restrict__ edge_nodes, int32_t* used) {
  for (int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < ne;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    used[edge_nodes[e].x] = 1;
    used[edge_nodes[e].y] = 1;
  }
}

__global__ void NodeCheckKernel(int64_t nv, const int32_t* __restrict__ used, int32_t* st) {
  for (int64_t v = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; v < nv;
       v += static_cast<int64_t>(gridDim.x) * blockDim.x)
    if (!used[v]) SetStatus(st, kErrNodeNoEdge, static_cast<int32_t>(v));
}

__global__ void TypeFlagsKernel(int64_t nc, const int32_t* __restrict__ is_quad, int64_t* fq,
                                int64_t* ft) {
  for (int64_t c = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; c < nc;
       c += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    fq[c] = is_quad[c];
    ft[c] = 1 - is_quad[c];
  }
}

__global__ void BucketKernel(int64_t nc, const int32_t* __restrict__ is_quad,
                             const int64_t* __restrict__ rq, const int64_t* __restrict__ rt,
                             int32_t* quad_list, int32_t* tria_list) {
  for (int64_t c = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; c < nc;
       c += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    if (is_quad[c]) quad_list[rq[c]] = static_cast<int32_t>(c);
    else tria_list[rt[c]] = static_cast<int32_t>(c);
  }
}

__global__ void BoundaryFlagsKernel(int64_t ne, const int2* __restrict__ edge_nodes,
                                    const int32_t* __restrict__ ncell, uint8_t* nf, uint8_t* ef) {
  for (int64_t e = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; e < ne;
       e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const bool b = ncell[e] == 1;  // special_entity_sets.cc:70
    if (ef) ef[e] = b;
    if (b && nf) {
      nf[edge_nodes[e].x] = 1;
      nf[edge_nodes[e].y] = 1;
    }
  }
}

// tp_triag_mesh_builder.cc:48-176 on the device.
__global__ void TPTriagKernel(int64_t nx, int64_t ny, double x0, double y0, double hx, double hy,
                              double2* xy, int4* cells, int2* pre) {
  const int64_t nv = (nx + 1) * (ny + 1), nc = 2 * nx * ny;
  const int64_t nh = nx * (ny + 1), nvert_e = (nx + 1) * ny, nd = nx * ny;
  const int64_t total = nv + nc / 2 + nh + nvert_e + nd;
  auto vid = [&](int64_t i, int64_t j) { return static_cast<int>(i + j * (nx + 1)); };
  for (int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; t < total;
       t += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    int64_t u = t;
    if (u < nv) {
      const int64_t i = u % (nx + 1), j = u / (nx + 1);
      xy[u] = make_double2(x0 + static_cast<double>(i) * hx, y0 + static_cast<double>(j) * hy);
      continue;
    }
    u -= nv;
    if (u < nc / 2) {
      const int64_t i = u / ny, j = u % ny;
      cells[2 * u] = make_int4(vid(i, j), vid(i + 1, j + 1), vid(i, j + 1), -1);
      cells[2 * u + 1] = make_int4(vid(i, j), vid(i + 1, j), vid(i + 1, j + 1), -1);
      continue;
    }
    u -= nc / 2;
    if (u < nh) {  // horizontal: i outer, j inner (j <= ny)
      const int64_t i = u / (ny + 1), j = u % (ny + 1);
      pre[u] = make_int2(vid(i, j), vid(i + 1, j));
      continue;
    }
    u -= nh;
    if (u < nvert_e) {  // vertical: i <= nx outer, j < ny inner
      const int64_t i = u / ny, j = u % ny;
      pre[nh + u] = make_int2(vid(i, j), vid(i, j + 1));
      continue;
    }
    u -= nvert_e;
    {  // diagonal
      const int64_t i = u / ny, j = u % ny;
      pre[nh + nvert_e + u] = make_int2(vid(i, j), vid(i + 1, j + 1));
    }
  }
}

// tp_quad_mesh_builder.cc:48-93 on the device.
__global__ void TPQuadKernel(int64_t nx, int64_t ny, double x0, double y0, double hx, double hy,
                             double2* xy, int4* cells) {
  const int64_t nv = (nx + 1) * (ny + 1), nc = nx * ny;
  auto vid = [&](int64_t i, int64_t j) { return static_cast<int>(i + j * (nx + 1)); };
  for (int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; t < nv + nc;
       t += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    if (t < nv) {
      const int64_t i = t % (nx + 1), j = t / (nx + 1);
      xy[t] = make_double2(x0 + static_cast<double>(i) * hx, y0 + static_cast<double>(j) * hy);
    } else {
      const int64_t u = t - nv, i = u / ny, j = u % ny;
      cells[u] = make_int4(vid(i, j), vid(i + 1, j), vid(i + 1, j + 1), vid(i, j + 1));
    }
  }
}

const char* ErrText(int32_t code) {
  switch (code) {
    case kErrBadNode: return "invalid node index";
    case kErrLoopEdge: return "edge with identical endpoints";
    case kErrDupPreset: return "duplicate preset edge";
    case kErrEdgeNoCell: return "Mesh is incomplete: edge does not belong to a cell";
    case kErrNodeNoEdge: return "Mesh is incomplete: node is not part of any edge";
    case kErrDegenerate: return "degenerate cell";
  }
  return "mesh error";
}

int BitsFor(int64_t n) {
  int b = 1;
  while ((int64_t(1) << b) < n + 1) ++b;
  return b;
}

// Numbering of a mesh whose xy / cells / preset arrays are already on the device.
void BuildTopology(lfg_mesh* m, DevBuf& pre_buf, int64_t npre) {
  lfg_ctx* ctx = m->ctx;
  cudaStream_t s = ctx->stream;
  const int64_t nv = m->nv, nc = m->nc;
  const int b = BitsFor(nv);
  const int bits = 2 * b;
  if (bits > 62) Fail(LFG_INVALID_ARG, "mesh too large");
  const int64_t nitems = npre + 4 * nc;
  if (nitems >= (int64_t(1) << 32)) Fail(LFG_INVALID_ARG, "mesh too large for 32-bit items");
  DevBuf keys, vals, isq;
  keys.alloc(nitems * sizeof(uint64_t), s);
  vals.alloc(nitems * sizeof(uint32_t), s);
  isq.alloc(std::max<int64_t>(nc, 1) * sizeof(int32_t), s);
  int32_t* st = StatusWord(ctx);
  ReadAndClearStatus(ctx);
  ValidateAndItemsKernel<<<GridFor(ctx, nitems, kBlock), kBlock, 0, s>>>(
      nv, nc, m->cell_nodes.as<int4>(), npre, pre_buf.as<int2>(), bits, keys.as<uint64_t>(),
      vals.as<uint32_t>(), isq.as<int32_t>(), st);
  LFG_LAUNCHED(ctx);
  int32_t detail = 0;
  if (int32_t code = ReadAndClearStatus(ctx, &detail))
    Fail(LFG_INVALID_ARG, std::string(ErrText(code)) + " (item " + std::to_string(detail) + ")");
  RadixSortPairs(ctx, keys.as<uint64_t>(), vals.as<uint32_t>(), nitems, bits);
  const uint64_t sentinel = (1ull << bits) - 1ull;
  DevBuf head, head_nopre, rank;
  head.alloc(nitems * sizeof(int64_t), s);
  head_nopre.alloc(nitems * sizeof(int64_t), s);
  rank.alloc(nitems * sizeof(int64_t), s);
  RunHeadsKernel<<<GridFor(ctx, nitems, kBlock), kBlock, 0, s>>>(
      keys.as<uint64_t>(), vals.as<uint32_t>(), nitems, sentinel, npre, head.as<int64_t>(),
      head_nopre.as<int64_t>());
  LFG_LAUNCHED(ctx);
  const int64_t ne = ExclusiveScanI64(ctx, head.as<int64_t>(), head.as<int64_t>(), nitems);
  const int64_t n_new = ExclusiveScanI64(ctx, head_nopre.as<int64_t>(), rank.as<int64_t>(), nitems);
  if (ne != npre + n_new) {
    // a preset edge duplicated by another preset makes the counts disagree
    Fail(LFG_INVALID_ARG, "duplicate preset edge");
  }
  if (ne >= (int64_t(1) << 31)) Fail(LFG_INVALID_ARG, "too many edges");
  m->ne = ne;
  m->edge_nodes.alloc(std::max<int64_t>(ne, 1) * sizeof(int2), s);
  m->edge_ncell.alloc(std::max<int64_t>(ne, 1) * sizeof(int32_t), s);
  m->cell_edges.alloc(std::max<int64_t>(nc, 1) * sizeof(int4), s);
  m->cell_ori.alloc(std::max<int64_t>(nc, 1), s);
  LFG_CUDA(cudaMemsetAsync(m->cell_edges.p, 0xff, std::max<int64_t>(nc, 1) * sizeof(int4), s));
  NumberEdgesKernel<<<GridFor(ctx, nitems, kBlock), kBlock, 0, s>>>(
      keys.as<uint64_t>(), vals.as<uint32_t>(), nitems, sentinel, npre, head.as<int64_t>(),
      rank.as<int64_t>(), pre_buf.as<int2>(), m->cell_nodes.as<int4>(), m->edge_nodes.as<int2>(),
      m->edge_ncell.as<int32_t>(), m->cell_edges.as<int4>(), st);
  LFG_LAUNCHED(ctx);
  if (int32_t code = ReadAndClearStatus(ctx, &detail))
    Fail(code == kErrEdgeNoCell ? LFG_INCOMPLETE_MESH : LFG_INVALID_ARG,
         std::string(ErrText(code)) + " (" + std::to_string(detail) + ")");
  keys.reset();
  vals.reset();
  head.reset();
  head_nopre.reset();
  rank.reset();
  // every node must lie on an edge (check_completeness)
  {
    DevBuf used;
    used.alloc(std::max<int64_t>(nv, 1) * sizeof(int32_t), s);
    LFG_CUDA(cudaMemsetAsync(used.p, 0, std::max<int64_t>(nv, 1) * sizeof(int32_t), s));
    NodeUseKernel<<<GridFor(ctx, ne, kBlock), kBlock, 0, s>>>(ne, m->edge_nodes.as<int2>(), used.as<int32_t>());
    LFG_LAUNCHED(ctx);
    NodeCheckKernel<<<GridFor(ctx, nv, kBlock), kBlock, 0, s>>>(nv, used.as<int32_t>(), st);
    LFG_LAUNCHED(ctx);
    if (int32_t code = ReadAndClearStatus(ctx, &detail))
      Fail(LFG_INCOMPLETE_MESH, std::string(ErrText(code)) + " (node " + std::to_string(detail) + ")");
  }
  CellOrientationKernel<<<GridFor(ctx, nc, kBlock), kBlock, 0, s>>>(
      nc, m->cell_nodes.as<int4>(), m->cell_edges.as<int4>(), m->edge_nodes.as<int2>(),
      m->xy.as<double2>(), m->cell_ori.as<uint8_t>(), st);
  LFG_LAUNCHED(ctx);
  if (int32_t code = ReadAndClearStatus(ctx, &detail))
    Fail(LFG_DEGENERATE_CELL, std::string(ErrText(code)) + " " + std::to_string(detail));
  // cell-type buckets (ascending cell index)
  DevBuf fq, ft;
  fq.alloc(std::max<int64_t>(nc, 1) * sizeof(int64_t), s);
  ft.alloc(std::max<int64_t>(nc, 1) * sizeof(int64_t), s);
  TypeFlagsKernel<<<GridFor(ctx, nc, kBlock), kBlock, 0, s>>>(nc, isq.as<int32_t>(), fq.as<int64_t>(), ft.as<int64_t>());
  LFG_LAUNCHED(ctx);
  m->nquad = ExclusiveScanI64(ctx, fq.as<int64_t>(), fq.as<int64_t>(), nc);
  m->ntria = ExclusiveScanI64(ctx, ft.as<int64_t>(), ft.as<int64_t>(), nc);
  m->quad_list.alloc(std::max<int64_t>(m->nquad, 1) * sizeof(int32_t), s);
  m->tria_list.alloc(std::max<int64_t>(m->ntria, 1) * sizeof(int32_t), s);
  BucketKernel<<<GridFor(ctx, nc, kBlock), kBlock, 0, s>>>(nc, isq.as<int32_t>(), fq.as<int64_t>(),
                                                          ft.as<int64_t>(), m->quad_list.as<int32_t>(),
                                                          m->tria_list.as<int32_t>());
  LFG_LAUNCHED(ctx);
  LFG_CUDA(cudaStreamSynchronize(s));
}

lfg_mesh* NewMesh(lfg_ctx* ctx, int64_t nv, int64_t nc) {
  if (nv <= 0 || nc <= 0) Fail(LFG_INVALID_ARG, "mesh needs nodes and cells");
  if (nv >= (int64_t(1) << 31) || nc >= (int64_t(1) << 31)) Fail(LFG_INVALID_ARG, "mesh too large");
  auto* m = new lfg_mesh;
  m->ref.Set(ctx);
  m->ctx = ctx;
  m->nv = nv;
  m->nc = nc;
  m->xy.alloc(nv * sizeof(double2), ctx->stream);
  m->cell_nodes.alloc(nc * sizeof(int4), ctx->stream);
  return m;
}

}  // namespace
}  // namespace lfg

using namespace lfg;

extern "C" {

lfg_status lfg_mesh_create(lfg_ctx* ctx, int64_t nv, const double* xy, int64_t nc,
                           const int32_t* cells, int64_t npre, const int32_t* pre, lfg_mesh** out) {
  LFG_API_BEGIN(ctx)
  if (!out || !xy || !cells || (npre > 0 && !pre) || npre < 0)
    Fail(LFG_INVALID_ARG, "lfg_mesh_create: null argument");
  *out = nullptr;
  lfg_mesh* m = NewMesh(ctx, nv, nc);
  try {
    LFG_CUDA(cudaMemcpyAsync(m->xy.p, xy, nv * sizeof(double2), cudaMemcpyHostToDevice, ctx->stream));
    LFG_CUDA(cudaMemcpyAsync(m->cell_nodes.p, cells, nc * sizeof(int4), cudaMemcpyHostToDevice, ctx->stream));
    DevBuf pb;
    pb.alloc(std::max<int64_t>(npre, 1) * sizeof(int2), ctx->stream);
    if (npre) LFG_CUDA(cudaMemcpyAsync(pb.p, pre, npre * sizeof(int2), cudaMemcpyHostToDevice, ctx->stream));
    BuildTopology(m, pb, npre);
  } catch (...) {
    delete m;
    throw;
  }
  *out = m;
  LFG_API_END
}

static lfg_status CreateTP(lfg_ctx* ctx, bool quad, int64_t nx, int64_t ny, double x0, double y0,
                           double x1, double y1, lfg_mesh** out) {
  LFG_API_BEGIN(ctx)
  if (!out || nx <= 0 || ny <= 0 || !(x1 > x0) || !(y1 > y0))
    Fail(LFG_INVALID_ARG, "structured mesh: bad size or box");
  *out = nullptr;
  const int64_t nv = (nx + 1) * (ny + 1);
  const int64_t nc = quad ? nx * ny : 2 * nx * ny;
  const double hx = (x1 - x0) / static_cast<double>(nx), hy = (y1 - y0) / static_cast<double>(ny);
  lfg_mesh* m = NewMesh(ctx, nv, nc);
  try {
    DevBuf pb;
    int64_t npre = 0;
    if (quad) {
      pb.alloc(sizeof(int2), ctx->stream);
      TPQuadKernel<<<GridFor(ctx, nv + nc, 256), 256, 0, ctx->stream>>>(
          nx, ny, x0, y0, hx, hy, m->xy.as<double2>(), m->cell_nodes.as<int4>());
    } else {
      npre = nx * (ny + 1) + (nx + 1) * ny + nx * ny;
      pb.alloc(npre * sizeof(int2), ctx->stream);
      TPTriagKernel<<<GridFor(ctx, nv + nc + npre, 256), 256, 0, ctx->stream>>>(
          nx, ny, x0, y0, hx, hy, m->xy.as<double2>(), m->cell_nodes.as<int4>(), pb.as<int2>());
    }
    LFG_LAUNCHED(ctx);
    BuildTopology(m, pb, npre);
  } catch (...) {
    delete m;
    throw;
  }
  *out = m;
  LFG_API_END
}

lfg_status lfg_mesh_create_tp_triag(lfg_ctx* ctx, int64_t nx, int64_t ny, double x0, double y0,
                                    double x1, double y1, lfg_mesh** out) {
  return CreateTP(ctx, false, nx, ny, x0, y0, x1, y1, out);
}

lfg_status lfg_mesh_create_tp_quad(lfg_ctx* ctx, int64_t nx, int64_t ny, double x0, double y0,
                                   double x1, double y1, lfg_mesh** out) {
  return CreateTP(ctx, true, nx, ny, x0, y0, x1, y1, out);
}

lfg_status lfg_mesh_destroy(lfg_mesh* m) {
  if (!m) return LFG_INVALID_ARG;
  cudaSetDevice(m->ctx->device);
  delete m;
  return LFG_OK;
}

lfg_status lfg_mesh_sizes(const lfg_mesh* m, int64_t* nv, int64_t* ne, int64_t* nc, int64_t* nt,
                          int64_t* nq) {
  if (!m) return LFG_INVALID_ARG;
  if (nv) *nv = m->nv;
  if (ne) *ne = m->ne;
  if (nc) *nc = m->nc;
  if (nt) *nt = m->ntria;
  if (nq) *nq = m->nquad;
  return LFG_OK;
}

lfg_status lfg_mesh_download_topology(lfg_mesh* m, int32_t* edge_nodes, int32_t* cell_edges,
                                      int8_t* cell_ori, int32_t* edge_ncells) {
  if (!m) return LFG_INVALID_ARG;
  LFG_API_BEGIN(m->ctx)
  cudaStream_t s = m->ctx->stream;
  if (edge_nodes)
    LFG_CUDA(cudaMemcpyAsync(edge_nodes, m->edge_nodes.p, m->ne * sizeof(int2), cudaMemcpyDeviceToHost, s));
  if (edge_ncells)
    LFG_CUDA(cudaMemcpyAsync(edge_ncells, m->edge_ncell.p, m->ne * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  std::vector<uint8_t> ori(m->nc);
  std::vector<int32_t> cn(4 * m->nc);
  LFG_CUDA(cudaMemcpyAsync(ori.data(), m->cell_ori.p, m->nc, cudaMemcpyDeviceToHost, s));
  LFG_CUDA(cudaMemcpyAsync(cn.data(), m->cell_nodes.p, m->nc * sizeof(int4), cudaMemcpyDeviceToHost, s));
  if (cell_edges)
    LFG_CUDA(cudaMemcpyAsync(cell_edges, m->cell_edges.p, m->nc * sizeof(int4), cudaMemcpyDeviceToHost, s));
  LFG_CUDA(cudaStreamSynchronize(s));
  if (cell_ori) {
    for (int64_t c = 0; c < m->nc; ++c) {
      const int nvert = cn[4 * c + 3] < 0 ? 3 : 4;
      for (int j = 0; j < 4; ++j)
        cell_ori[4 * c + j] = j < nvert ? ((ori[c] >> j) & 1 ? -1 : 1) : 0;
    }
  }
  LFG_API_END
}

lfg_status lfg_mesh_device_arrays(lfg_mesh* m, const double** xy, const int32_t** cells) {
  if (!m) return LFG_INVALID_ARG;
  if (xy) *xy = m->xy.as<const double>();
  if (cells) *cells = m->cell_nodes.as<const int32_t>();
  return LFG_OK;
}

lfg_status lfg_mesh_set_coords(lfg_mesh* m, const double* xy, int from_device) {
  if (!m || !xy) return LFG_INVALID_ARG;
  LFG_API_BEGIN(m->ctx)
  LFG_CUDA(cudaMemcpyAsync(m->xy.p, xy, m->nv * sizeof(double2),
                           from_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                           m->ctx->stream));
  m->nonaffine_quads = -1;  // the geometry changed: recount parallelograms on next use
  LFG_API_END
}

lfg_status lfg_mesh_boundary_flags(lfg_mesh* m, uint8_t* nf, uint8_t* ef) {
  if (!m) return LFG_INVALID_ARG;
  LFG_API_BEGIN(m->ctx)
  cudaStream_t s = m->ctx->stream;
  if (nf) LFG_CUDA(cudaMemsetAsync(nf, 0, m->nv, s));
  BoundaryFlagsKernel<<<GridFor(m->ctx, m->ne, 256), 256, 0, s>>>(
      m->ne, m->edge_nodes.as<int2>(), m->edge_ncell.as<int32_t>(), nf, ef);
  LFG_LAUNCHED(m->ctx);
  LFG_API_END
}

}  // extern "C"
