// Oracle (test infrastructure only): flat C entry points so that the Python
// test-suite can drive the restatement through ctypes.  Every call returns 0
// on success; on failure it returns -1 and copies the message into err.
#include <array>
#include <cstring>
#include <chrono>
#include <memory>
#include <thread>

#include "lfo.h"

using namespace lfo;

namespace {
struct Space {
  const Mesh* mesh;
  int degree;  // 0 for a generic layout
  DofHandler dh;
};
struct Input {
  FactoryInput in;
};
struct CSR {
  std::vector<int64_t> rowptr;
  std::vector<int32_t> col;
  std::vector<double> val;
};

void SetErr(char* err, int n, const char* msg) {
  if (err && n > 0) {
    std::strncpy(err, msg, n - 1);
    err[n - 1] = 0;
  }
}

}  // namespace

extern "C" {

typedef struct {
  int32_t kind;
  int32_t func;
  double value;
  const double* data;
  double p[16];
} lfo_coeff;

static MeshFunction ToMF(const lfo_coeff* c, size_t n_data) {
  MeshFunction mf;
  if (!c) return mf;
  mf.kind = c->kind;
  mf.value = c->value;
  if (c->kind == MeshFunction::kPerCell || c->kind == MeshFunction::kNodalO1 ||
      c->kind == MeshFunction::kPerCellExp)
    mf.data.assign(c->data, c->data + n_data);
  if (c->kind == MeshFunction::kAnalytic) mf.fn = AnalyticFunction(c->func, c->p);
  // matrix-valued kinds (the library's LFG_COEFF_TENSOR_*)
  if (c->kind == 6) {
    const std::array<double, 4> a{c->p[0], c->p[1], c->p[2], c->p[3]};
    mf.tensor_fn = [a](idx_t, double, double, double* o) { std::copy(a.begin(), a.end(), o); };
  } else if (c->kind == 7) {
    auto d = std::make_shared<std::vector<double>>(c->data, c->data + 4 * n_data);
    mf.tensor_fn = [d](idx_t cell, double, double, double* o) {
      for (int e = 0; e < 4; ++e) o[e] = (*d)[4 * cell + e];
    };
  } else if (c->kind == 8) {
    std::array<double, 16> q;
    std::copy(c->p, c->p + 16, q.begin());
    mf.tensor_fn = [q](idx_t, double x, double y, double* o) {
      for (int e = 0; e < 4; ++e) o[e] = q[4 * e] + q[4 * e + 1] * x + q[4 * e + 2] * y + q[4 * e + 3] * (x * y);
    };
  }
  return mf;
}

#define LFO_TRY try {
#define LFO_CATCH                      \
  }                                    \
  catch (const std::exception& e) {    \
    SetErr(err, errlen, e.what());     \
    return -1;                         \
  }                                    \
  return 0;

int lfo_input_create(int kind, int64_t nx, int64_t ny, double x0, double y0, double x1,
                     double y1, void** out, int64_t* sizes, char* err, int errlen) {
  LFO_TRY
  auto* h = new Input;
  if (kind == 0) h->in = TPTriagInput(nx, ny, x0, y0, x1, y1);
  else if (kind == 1) h->in = TPQuadInput(nx, ny, x0, y0, x1, y1);
  else h->in = TestMesh0Input(x0 == 0.0 ? 1.0 : x0);
  sizes[0] = static_cast<int64_t>(h->in.xy.size() / 2);
  sizes[1] = static_cast<int64_t>(h->in.cells.size() / 4);
  sizes[2] = static_cast<int64_t>(h->in.edges.size() / 2);
  *out = h;
  LFO_CATCH
}

void lfo_input_copy(void* h, double* xy, int64_t* cells, int64_t* edges) {
  auto* in = static_cast<Input*>(h);
  std::memcpy(xy, in->in.xy.data(), in->in.xy.size() * sizeof(double));
  std::memcpy(cells, in->in.cells.data(), in->in.cells.size() * sizeof(int64_t));
  if (!in->in.edges.empty())
    std::memcpy(edges, in->in.edges.data(), in->in.edges.size() * sizeof(int64_t));
}
void lfo_input_destroy(void* h) { delete static_cast<Input*>(h); }

int lfo_mesh_create(int64_t nv, const double* xy, int64_t nc, const int64_t* cells,
                    int64_t npre, const int64_t* pre, void** out, char* err, int errlen) {
  LFO_TRY
  auto m = std::make_unique<Mesh>(BuildMesh(nv, xy, nc, cells, npre, pre));
  // MeshFactory(check_completeness = true): every node on an edge, every edge
  // on a cell (hybrid2d/mesh.cc:566-600)
  std::vector<uint8_t> used(m->num_nodes, 0);
  for (idx_t e = 0; e < m->num_edges; ++e) {
    if (m->edge_num_cells[e] == 0)
      throw Error("Mesh is incomplete: Edge with global index " + std::to_string(e) +
                  " does not belong to a cell.");
    used[m->edge_nodes[e][0]] = used[m->edge_nodes[e][1]] = 1;
  }
  for (idx_t v = 0; v < m->num_nodes; ++v)
    if (!used[v])
      throw Error("Mesh is incomplete: Node with global index " + std::to_string(v) +
                  " is not part of any edge.");
  *out = m.release();
  LFO_CATCH
}
void lfo_mesh_destroy(void* m) { delete static_cast<Mesh*>(m); }
void lfo_mesh_sizes(void* mp, int64_t* s) {
  auto* m = static_cast<Mesh*>(mp);
  s[0] = m->num_nodes;
  s[1] = m->num_edges;
  s[2] = m->num_cells;
}
void lfo_mesh_topology(void* mp, int64_t* edge_nodes, int64_t* cell_edges, int8_t* cell_ori,
                       int32_t* edge_ncells) {
  auto* m = static_cast<Mesh*>(mp);
  for (idx_t e = 0; e < m->num_edges; ++e) {
    edge_nodes[2 * e] = m->edge_nodes[e][0];
    edge_nodes[2 * e + 1] = m->edge_nodes[e][1];
    edge_ncells[e] = m->edge_num_cells[e];
  }
  for (idx_t c = 0; c < m->num_cells; ++c)
    for (int k = 0; k < 4; ++k) {
      cell_edges[4 * c + k] = m->cell_edges[c][k];
      cell_ori[4 * c + k] = m->cell_ori[c][k];
    }
}
void lfo_boundary_flags(void* mp, uint8_t* nf, uint8_t* ef) {
  std::vector<uint8_t> a, b;
  FlagEntitiesOnBoundary(*static_cast<Mesh*>(mp), a, b);
  std::memcpy(nf, a.data(), a.size());
  std::memcpy(ef, b.data(), b.size());
}
int lfo_mesh_degenerate_cells(void* mp, int64_t* count) {
  auto* m = static_cast<Mesh*>(mp);
  int64_t n = 0;
  for (idx_t c = 0; c < m->num_cells; ++c)
    if (!NonDegenerate(m->Geom(c))) ++n;
  *count = n;
  return 0;
}

int lfo_space_create(void* mp, int degree, int np, int ns, int nt, int nq, void** out,
                     char* err, int errlen) {
  LFO_TRY
  auto* m = static_cast<Mesh*>(mp);
  auto s = std::make_unique<Space>();
  s->mesh = m;
  s->degree = degree;
  s->dh = degree > 0 ? MakeLagrangeDofHandler(*m, degree) : MakeDofHandler(*m, np, ns, nt, nq);
  *out = s.release();
  LFO_CATCH
}
void lfo_space_destroy(void* s) { delete static_cast<Space*>(s); }
void lfo_space_info(void* sp, int64_t* info) {
  auto* s = static_cast<Space*>(sp);
  info[0] = s->dh.num_dofs;
  info[1] = s->dh.n_cell;
  info[2] = s->dh.n_tria;
  info[3] = s->dh.n_quad;
}
void lfo_space_cell_dofs(void* sp, int64_t* out) {
  auto* s = static_cast<Space*>(sp);
  std::memcpy(out, s->dh.cell_dofs.data(), s->dh.cell_dofs.size() * sizeof(int64_t));
}
// HierarchicScalarFESpace(mesh, degree_functor): degrees per edge (edge
// order) and per cell (cell order).
int lfo_space_create_hier_var(void* mp, const int32_t* edge_deg, const int32_t* cell_deg, void** out, char* err,
                              int errlen) {
  LFO_TRY
  auto* m = static_cast<Mesh*>(mp);
  auto s = std::make_unique<Space>();
  s->mesh = m;
  s->degree = 0;
  s->dh = MakeHierVarDofHandler(*m, std::vector<int>(edge_deg, edge_deg + m->num_edges),
                                std::vector<int>(cell_deg, cell_deg + m->num_cells));
  *out = s.release();
  LFO_CATCH
}
// Local dof count of every cell.
void lfo_space_local_counts(void* sp, int32_t* out) {
  auto* s = static_cast<Space*>(sp);
  for (idx_t c = 0; c < s->mesh->num_cells; ++c) out[c] = s->dh.NumLocalDofs(c);
}

void lfo_space_dof_entity(void* sp, int32_t* codim, int64_t* idx) {
  auto* s = static_cast<Space*>(sp);
  for (size_t k = 0; k < s->dh.dof_entity.size(); ++k) {
    codim[k] = s->dh.dof_entity[k].first;
    idx[k] = s->dh.dof_entity[k].second;
  }
}

int lfo_quad_rule(int is_quad, int degree, double* x, double* y, double* w, int* n,
                  char* err, int errlen) {
  LFO_TRY
  QuadRule qr = MakeQuadRule(is_quad != 0, degree);
  *n = qr.n();
  if (x) {
    std::memcpy(x, qr.x.data(), qr.n() * sizeof(double));
    std::memcpy(y, qr.y.data(), qr.n() * sizeof(double));
    std::memcpy(w, qr.w.data(), qr.n() * sizeof(double));
  }
  LFO_CATCH
}

int lfo_assemble_rd(void* sp, const lfo_coeff* alpha, const lfo_coeff* gamma, int qdeg_tria,
                    int qdeg_quad, int64_t first_cell, int64_t last_cell, void** out, char* err,
                    int errlen) {
  LFO_TRY
  auto* s = static_cast<Space*>(sp);
  const Mesh& m = *s->mesh;
  RDProvider p;
  p.mesh = &m;
  p.degree = s->degree;
  const size_t nd = alpha && alpha->kind == MeshFunction::kNodalO1 ? m.num_nodes : m.num_cells;
  const size_t nd2 = gamma && gamma->kind == MeshFunction::kNodalO1 ? m.num_nodes : m.num_cells;
  p.alpha = ToMF(alpha, nd);
  p.gamma = ToMF(gamma, nd2);
  const int dt = qdeg_tria > 0 ? qdeg_tria : 2 * s->degree;
  const int dq = qdeg_quad > 0 ? qdeg_quad : 2 * s->degree;
  if (qdeg_tria >= 0) { p.qr_tria = MakeQuadRule(false, dt); p.have_tria = true; }
  if (qdeg_quad >= 0) { p.qr_quad = MakeQuadRule(true, dq); p.have_quad = true; }
  p.Init();
  auto A = std::make_unique<COOMatrix>();
  A->rows = A->cols = s->dh.num_dofs;
  if (last_cell < 0) last_cell = m.num_cells;
  std::vector<double> em;
  for (idx_t c = first_cell; c < last_cell; ++c) {
    const int n = s->dh.NumLocalDofs(c);
    const idx_t* dofs = s->dh.GlobalDofIndices(c);
    p.Eval(c, em);
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) A->AddToEntry(dofs[i], dofs[j], em[i * n + j]);
  }
  *out = A.release();
  LFO_CATCH
}

// The same cell loop split into contiguous cell ranges over `nthreads`
// std::threads, each writing its cells' triplets at their final positions, so
// the result equals the serial COO.  Used to time the CPU path with all host
// cores; returns wall seconds of the assembly (provider set-up excluded).
int lfo_assemble_rd_parallel(void* sp, const lfo_coeff* alpha, const lfo_coeff* gamma,
                             int qdeg_tria, int qdeg_quad, int64_t first_cell, int64_t last_cell,
                             int nthreads, double* seconds, int64_t* ntriplets, char* err,
                             int errlen) {
  LFO_TRY
  auto* s = static_cast<Space*>(sp);
  const Mesh& m = *s->mesh;
  RDProvider p;
  p.mesh = &m;
  p.degree = s->degree;
  p.alpha = ToMF(alpha, alpha && alpha->kind == MeshFunction::kNodalO1 ? m.num_nodes : m.num_cells);
  p.gamma = ToMF(gamma, gamma && gamma->kind == MeshFunction::kNodalO1 ? m.num_nodes : m.num_cells);
  p.qr_tria = MakeQuadRule(false, qdeg_tria > 0 ? qdeg_tria : 2 * s->degree);
  p.qr_quad = MakeQuadRule(true, qdeg_quad > 0 ? qdeg_quad : 2 * s->degree);
  p.have_tria = p.have_quad = true;
  p.Init();
  if (last_cell < 0) last_cell = m.num_cells;
  std::vector<int64_t> off(last_cell - first_cell + 1, 0);
  for (idx_t c = first_cell; c < last_cell; ++c) {
    const int n = s->dh.NumLocalDofs(c);
    off[c - first_cell + 1] = off[c - first_cell] + n * n;
  }
  std::vector<Triplet> out(off.back());
  const auto t0 = std::chrono::steady_clock::now();
  std::vector<std::thread> pool;
  std::vector<std::string> errors(nthreads);
  const idx_t total = last_cell - first_cell;
  for (int t = 0; t < nthreads; ++t) {
    pool.emplace_back([&, t]() {
      try {
        std::vector<double> em;
        const idx_t lo = first_cell + total * t / nthreads, hi = first_cell + total * (t + 1) / nthreads;
        for (idx_t c = lo; c < hi; ++c) {
          const int n = s->dh.NumLocalDofs(c);
          const idx_t* dofs = s->dh.GlobalDofIndices(c);
          p.Eval(c, em);
          Triplet* o = &out[off[c - first_cell]];
          for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j)
              o[i * n + j] = {static_cast<int32_t>(dofs[i]), static_cast<int32_t>(dofs[j]), em[i * n + j]};
        }
      } catch (const std::exception& e) {
        errors[t] = e.what();
      }
    });
  }
  for (auto& th : pool) th.join();
  for (auto& e : errors)
    if (!e.empty()) throw Error(e);
  *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  *ntriplets = static_cast<int64_t>(out.size());
  LFO_CATCH
}

int lfo_assemble_load(void* sp, const lfo_coeff* f, int qdeg_tria, int qdeg_quad, double* b,
                      char* err, int errlen) {
  LFO_TRY
  auto* s = static_cast<Space*>(sp);
  const Mesh& m = *s->mesh;
  LoadProvider p;
  p.mesh = &m;
  p.degree = s->degree;
  p.f = ToMF(f, f && f->kind == MeshFunction::kNodalO1 ? m.num_nodes : m.num_cells);
  p.qr_tria = MakeQuadRule(false, qdeg_tria > 0 ? qdeg_tria : 2 * s->degree);
  p.qr_quad = MakeQuadRule(true, qdeg_quad > 0 ? qdeg_quad : 2 * s->degree);
  p.Init();
  std::vector<double> bv(b, b + s->dh.num_dofs);
  AssembleVectorLocally(s->dh, [&](idx_t c, std::vector<double>& v) { p.Eval(c, v); }, bv);
  std::memcpy(b, bv.data(), bv.size() * sizeof(double));
  LFO_CATCH
}

int lfo_assemble_edge_mass(void* sp, const lfo_coeff* gamma, const uint8_t* flags, int qdeg, void** out,
                           char* err, int errlen) {
  LFO_TRY
  auto* s = static_cast<Space*>(sp);
  const Mesh& m = *s->mesh;
  const MeshFunction mf = ToMF(gamma, gamma && gamma->kind == MeshFunction::kNodalO1 ? m.num_nodes : m.num_edges);
  auto A = std::make_unique<COOMatrix>();
  A->rows = A->cols = s->dh.num_dofs;
  AssembleEdgeMass(s->dh, s->degree, mf, flags, qdeg > 0 ? qdeg : 2 * s->degree, *A);
  *out = A.release();
  LFO_CATCH
}

int lfo_assemble_edge_load(void* sp, const lfo_coeff* g, const uint8_t* flags, int qdeg, double* b, char* err,
                           int errlen) {
  LFO_TRY
  auto* s = static_cast<Space*>(sp);
  const Mesh& m = *s->mesh;
  const MeshFunction mf = ToMF(g, g && g->kind == MeshFunction::kNodalO1 ? m.num_nodes : m.num_edges);
  std::vector<double> bv(b, b + s->dh.num_dofs);
  AssembleEdgeLoad(s->dh, s->degree, mf, flags, qdeg > 0 ? qdeg : 2 * s->degree, bv);
  std::memcpy(b, bv.data(), bv.size() * sizeof(double));
  LFO_CATCH
}

// Post-processing: IntegrateMeshFunction over an integrand of the closed set
// (kind 0: u_h + u, 1: (u_h - u)^2, 2: |grad u_h - grad u|^2; dofs null: u_h
// = 0), over cells (codim 0) or edges (codim 1).
int lfo_integrate(void* sp, int kind, const lfo_coeff* u, const double* dofs, int qdeg, const uint8_t* flags,
                  int codim, double* out, char* err, int errlen) {
  LFO_TRY
  auto* s = static_cast<Space*>(sp);
  const Mesh& m = *s->mesh;
  Integrand g;
  g.kind = kind;
  size_t nd = 0;
  if (u && u->kind == MeshFunction::kNodalO1) nd = m.num_nodes;
  else nd = codim == 0 ? m.num_cells : m.num_edges;
  g.u = ToMF(u, nd);
  if (u && u->kind == MeshFunction::kAnalytic) g.grad_u = AnalyticGradient(u->func, u->p);
  g.dh = &s->dh;
  g.degree = s->degree;
  g.dofs = dofs;
  *out = IntegrateMeshFunction(m, g, qdeg, flags, codim);
  LFO_CATCH
}

// The same over the cells (codim 0) with u_h on a hierarchic space of uniform
// degree p (p = 0: per-entity degrees).
int lfo_integrate_hier(void* sp, int p, int kind, const lfo_coeff* u, const double* dofs, int qdeg,
                       const uint8_t* flags, double* out, char* err, int errlen) {
  LFO_TRY
  auto* s = static_cast<Space*>(sp);
  const Mesh& m = *s->mesh;
  Integrand g;
  g.kind = kind;
  g.u = ToMF(u, u && u->kind == MeshFunction::kNodalO1 ? m.num_nodes : m.num_cells);
  if (u && u->kind == MeshFunction::kAnalytic) g.grad_u = AnalyticGradient(u->func, u->p);
  g.dh = &s->dh;
  g.degree = s->degree;
  g.dofs = dofs;
  g.hier = p;
  *out = IntegrateMeshFunction(m, g, qdeg, flags, 0);
  LFO_CATCH
}

// MeshFunctionFE / MeshFunctionGradFE on every cell at npts reference points:
// vals[cell][k], grads[cell][k][2] (either may be null).
int lfo_eval_fe(void* sp, const double* dofs, int npts, const double* xy, double* vals, double* grads, char* err,
                int errlen) {
  LFO_TRY
  auto* s = static_cast<Space*>(sp);
  const std::vector<double> pts(xy, xy + 2 * npts);
  for (idx_t c = 0; c < s->mesh->num_cells; ++c)
    EvalFE(s->dh, s->degree, dofs, c, pts, vals ? vals + c * npts : nullptr, grads ? grads + 2 * c * npts : nullptr);
  LFO_CATCH
}

int lfo_eval_fe_hier(void* sp, int p, const double* dofs, int npts, const double* xy, double* vals, double* grads,
                     char* err, int errlen) {
  LFO_TRY
  auto* s = static_cast<Space*>(sp);
  const std::vector<double> pts(xy, xy + 2 * npts);
  for (idx_t c = 0; c < s->mesh->num_cells; ++c)
    EvalFEHier(s->dh, p, dofs, c, pts, vals ? vals + c * npts : nullptr, grads ? grads + 2 * c * npts : nullptr);
  LFO_CATCH
}

int lfo_nodal_projection_mf(void* sp, const lfo_coeff* u, const uint8_t* cell_flags, double* out, char* err,
                            int errlen) {
  LFO_TRY
  auto* s = static_cast<Space*>(sp);
  const Mesh& m = *s->mesh;
  const MeshFunction mf = ToMF(u, u && u->kind == MeshFunction::kNodalO1 ? m.num_nodes : m.num_cells);
  std::vector<double> v;
  NodalProjectionMF(s->dh, s->degree, mf, cell_flags, v);
  std::memcpy(out, v.data(), v.size() * sizeof(double));
  LFO_CATCH
}

// FeHierarchicTria / Quad dual: the evaluation nodes (xy[2 k], xy[2 k + 1])
// and M (n x ne, row-major) with M[:, k] = NodalValuesToDofs(e_k).  With xy
// null only the counts are written.
int lfo_hier_dual(int is_quad, int pc, const int32_t* pe, const int8_t* ori, double* xy, double* M, int* ne, int* n,
                  char* err, int errlen) {
  LFO_TRY
  int pv[4] = {pe[0], pe[1], pe[2], is_quad ? pe[3] : 1};
  std::vector<double> nodes;
  HierEvaluationNodes(is_quad != 0, pc, pv, ori, nodes);
  const int nn = static_cast<int>(nodes.size() / 2), nd = HierNumShapeVar(is_quad != 0, pc, pv);
  if (xy) {
    std::memcpy(xy, nodes.data(), nodes.size() * sizeof(double));
    std::vector<double> v(nn, 0.0), d;
    for (int k = 0; k < nn; ++k) {
      v[k] = 1.0;
      HierNodalValuesToDofs(is_quad != 0, pc, pv, ori, v, d);
      for (int r = 0; r < nd; ++r) M[static_cast<size_t>(r) * nn + k] = d[r];
      v[k] = 0.0;
    }
  }
  *ne = nn;
  *n = nd;
  LFO_CATCH
}

// fe::NodalProjection on a hierarchic space (uniform degree p, or p = 0 for a
// space made by lfo_space_create_hier_var).
int lfo_nodal_projection_hier(void* sp, int p, const lfo_coeff* u, const uint8_t* cell_flags, double* out, char* err,
                              int errlen) {
  LFO_TRY
  auto* s = static_cast<Space*>(sp);
  const Mesh& m = *s->mesh;
  const MeshFunction mf = ToMF(u, u && u->kind == MeshFunction::kNodalO1 ? m.num_nodes : m.num_cells);
  std::vector<double> v;
  NodalProjectionHier(s->dh, p, mf, cell_flags, v);
  std::memcpy(out, v.data(), v.size() * sizeof(double));
  LFO_CATCH
}

int lfo_init_essential(void* sp, const uint8_t* edge_flags, const lfo_coeff* g, uint8_t* flags, double* vals,
                       char* err, int errlen) {
  LFO_TRY
  auto* s = static_cast<Space*>(sp);
  const Mesh& m = *s->mesh;
  const MeshFunction mf = ToMF(g, g && g->kind == MeshFunction::kNodalO1 ? m.num_nodes : m.num_edges);
  std::vector<uint8_t> f;
  std::vector<double> v;
  InitEssentialCondition(s->dh, s->degree, edge_flags, mf, f, v);
  std::memcpy(flags, f.data(), f.size());
  std::memcpy(vals, v.data(), v.size() * sizeof(double));
  LFO_CATCH
}

// Hierarchic (hp) FE of uniform degree p on a space created with the layout
// (1, p-1, interior tria, interior quad): fe::Diffusion + fe::Mass element
// matrices (summed) and fe::ScalarLoadElementVectorProvider.
int lfo_assemble_hier(void* sp, int p, const lfo_coeff* alpha, const lfo_coeff* gamma, int qdeg, void** out,
                      char* err, int errlen) {
  LFO_TRY
  auto* s = static_cast<Space*>(sp);
  const Mesh& m = *s->mesh;
  const MeshFunction a = ToMF(alpha, alpha && alpha->kind == MeshFunction::kNodalO1 ? m.num_nodes : m.num_cells);
  const MeshFunction g = ToMF(gamma, gamma && gamma->kind == MeshFunction::kNodalO1 ? m.num_nodes : m.num_cells);
  auto A = std::make_unique<COOMatrix>();
  A->rows = A->cols = s->dh.num_dofs;
  AssembleHierMatrix(s->dh, p, a, g, qdeg, *A);
  *out = A.release();
  LFO_CATCH
}

int lfo_assemble_hier_load(void* sp, int p, const lfo_coeff* f, int qdeg, double* b, char* err, int errlen) {
  LFO_TRY
  auto* s = static_cast<Space*>(sp);
  const Mesh& m = *s->mesh;
  const MeshFunction mf = ToMF(f, f && f->kind == MeshFunction::kNodalO1 ? m.num_nodes : m.num_cells);
  std::vector<double> bv(b, b + s->dh.num_dofs);
  AssembleHierLoad(s->dh, p, mf, qdeg, bv);
  std::memcpy(b, bv.data(), bv.size() * sizeof(double));
  LFO_CATCH
}

// Variable-degree FeHierarchicTria / Quad: interior degree pc, edge degrees pe[4].
int lfo_hier_shape_var(int is_quad, int pc, const int32_t* pe, const int8_t* ori, int npts, const double* xy,
                       double* phi, double* dphi, char* err, int errlen) {
  LFO_TRY
  const int pv[4] = {pe[0], pe[1], pe[2], pe[3]};
  const int n = HierNumShapeVar(is_quad != 0, pc, pv);
  for (int k = 0; k < npts; ++k)
    EvalHierShapeVar(is_quad != 0, pc, pv, ori, xy[2 * k], xy[2 * k + 1], phi + static_cast<size_t>(k) * n,
                     reinterpret_cast<double(*)[2]>(dphi + static_cast<size_t>(k) * n * 2));
  LFO_CATCH
}

// FeHierarchicTria / Quad shape values and reference gradients at npts points.
int lfo_hier_shape(int is_quad, int p, const int8_t* ori, int npts, const double* xy, double* phi, double* dphi,
                   char* err, int errlen) {
  LFO_TRY
  const int n = is_quad ? (p + 1) * (p + 1) : (p + 1) * (p + 2) / 2;
  for (int k = 0; k < npts; ++k)
    EvalHierShape(is_quad != 0, p, ori, xy[2 * k], xy[2 * k + 1], phi + static_cast<size_t>(k) * n,
                  reinterpret_cast<double(*)[2]>(dphi + static_cast<size_t>(k) * n * 2));
  LFO_CATCH
}

double lfo_hier_fn(int which, int n, double a, double b, double x) {
  switch (which) {
    case 0: return HierLegendre(n, x, a);
    case 1: return HierILegendre(n, x, a);
    case 2: return HierILegendreDx(n, x, a);
    case 3: return HierILegendreDt(n, x, a);
    case 4: return HierJacobi(n, a, b, x);
    default: return HierIJacobi(n, a, x);
  }
}

int lfo_assemble_tabulated(void* sp, const double* elem, int ld, double* vec_elem, double* b,
                           void** out, char* err, int errlen) {
  LFO_TRY
  auto* s = static_cast<Space*>(sp);
  auto A = std::make_unique<COOMatrix>();
  A->rows = A->cols = s->dh.num_dofs;
  AssembleMatrixLocally(
      s->dh,
      [&](idx_t c, std::vector<double>& em) {
        em.assign(elem + c * ld * ld, elem + (c + 1) * ld * ld);
      },
      *A);
  if (vec_elem && b) {
    std::vector<double> bv(b, b + s->dh.num_dofs);
    AssembleVectorLocally(
        s->dh,
        [&](idx_t c, std::vector<double>& ev) { ev.assign(vec_elem + c * ld, vec_elem + (c + 1) * ld); },
        bv);
    std::memcpy(b, bv.data(), bv.size() * sizeof(double));
  }
  *out = A.release();
  LFO_CATCH
}

void* lfo_coo_create(int64_t rows, int64_t cols, int64_t n, const int32_t* r, const int32_t* c,
                     const double* v) {
  auto* A = new COOMatrix;
  A->rows = rows;
  A->cols = cols;
  for (int64_t k = 0; k < n; ++k) A->AddToEntry(r[k], c[k], v[k]);
  return A;
}
void lfo_coo_destroy(void* a) { delete static_cast<COOMatrix*>(a); }
int64_t lfo_coo_size(void* a) { return static_cast<int64_t>(static_cast<COOMatrix*>(a)->triplets.size()); }
void lfo_coo_copy(void* a, int32_t* r, int32_t* c, double* v) {
  auto* A = static_cast<COOMatrix*>(a);
  for (size_t k = 0; k < A->triplets.size(); ++k) {
    r[k] = A->triplets[k].row;
    c[k] = A->triplets[k].col;
    v[k] = A->triplets[k].value;
  }
}

int lfo_fix_flagged(void* a, const uint8_t* flags, const double* vals, double* b, int alt,
                    char* err, int errlen) {
  LFO_TRY
  auto* A = static_cast<COOMatrix*>(a);
  std::vector<double> bv(b, b + A->rows);
  if (alt) FixFlaggedSolutionCompAlt(flags, vals, *A, bv);
  else FixFlaggedSolutionComponents(flags, vals, *A, bv);
  std::memcpy(b, bv.data(), bv.size() * sizeof(double));
  LFO_CATCH
}

int lfo_fix_lse(void* a, int64_t count, const int64_t* dofs, const double* vals, double* b, char* err,
                int errlen) {
  LFO_TRY
  auto* A = static_cast<COOMatrix*>(a);
  std::vector<std::pair<idx_t, double>> fixed;
  for (int64_t k = 0; k < count; ++k) fixed.emplace_back(static_cast<idx_t>(dofs[k]), vals[k]);
  std::vector<double> bv(b, b + A->rows);
  FixSolutionComponentsLse(fixed, *A, bv);
  std::memcpy(b, bv.data(), bv.size() * sizeof(double));
  LFO_CATCH
}

void* lfo_csr_create(void* a, int64_t* sizes) {
  auto* A = static_cast<COOMatrix*>(a);
  auto* C = new CSR;
  MakeSparseCSR(*A, C->rowptr, C->col, C->val);
  sizes[0] = A->rows;
  sizes[1] = static_cast<int64_t>(C->col.size());
  return C;
}
void lfo_csr_copy(void* h, int64_t* rowptr, int32_t* col, double* val) {
  auto* C = static_cast<CSR*>(h);
  std::memcpy(rowptr, C->rowptr.data(), C->rowptr.size() * sizeof(int64_t));
  std::memcpy(col, C->col.data(), C->col.size() * sizeof(int32_t));
  std::memcpy(val, C->val.data(), C->val.size() * sizeof(double));
}
void lfo_csr_destroy(void* h) { delete static_cast<CSR*>(h); }

int lfo_nodal_projection(void* sp, int func, const double* p, double* out, char* err,
                         int errlen) {
  LFO_TRY
  auto* s = static_cast<Space*>(sp);
  std::vector<double> v;
  NodalProjection(s->dh, s->degree, AnalyticFunction(func, p), v);
  std::memcpy(out, v.data(), v.size() * sizeof(double));
  LFO_CATCH
}

// Restatement of lf_fe_linear.ReactionDiffusion (uscalfe/test/lagr_fe_tests.cc:
// 807-832): O1 on test mesh 0 with the tensor coefficient [[1, x], [y, xy]],
// gamma = xy, a = 1+x+2y, b = 3x, degree-4 rules; returns a^T A b.
int lfo_kat_tensor_rd(double* value, char* err, int errlen) {
  LFO_TRY
  FactoryInput in = TestMesh0Input(1.0);
  Mesh m = BuildMesh(10, in.xy.data(), 9, in.cells.data(), 0, nullptr);
  DofHandler dh = MakeLagrangeDofHandler(m, 1);
  RDProvider p;
  p.mesh = &m;
  p.degree = 1;
  p.alpha.kind = MeshFunction::kAnalytic;
  p.alpha.tensor_fn = [](idx_t, double x, double y, double* a) {
    a[0] = 1; a[1] = x; a[2] = y; a[3] = x * y;
  };
  p.gamma.kind = MeshFunction::kAnalytic;
  p.gamma.fn = [](double x, double y) { return x * y; };
  p.qr_tria = MakeQuadRule(false, 4);
  p.qr_quad = MakeQuadRule(true, 4);
  p.have_tria = p.have_quad = true;
  p.Init();
  COOMatrix A;
  A.rows = A.cols = dh.num_dofs;
  AssembleMatrixLocally(dh, [&](idx_t c, std::vector<double>& em) { p.Eval(c, em); }, A);
  std::vector<double> a, b;
  NodalProjection(dh, 1, [](double x, double y) { return 1 + x + 2 * y; }, a);
  NodalProjection(dh, 1, [](double x, double) { return 3 * x; }, b);
  double s = 0;
  for (const Triplet& t : A.triplets) s += a[t.row] * t.value * b[t.col];
  *value = s;
  LFO_CATCH
}

}  // extern "C"
