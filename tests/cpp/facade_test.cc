// Drives the C++ facade (lf_gb300.hpp) the way a LehrFEM++ driver drives
// lf::assemble, and checks it against the oracle (the CPU restatement, linked
// from its shared library): triplet indices and order bit-exact, values within
// 1e-12 of each element matrix's largest entry, the load vector within 1e-12,
// a converged PCG solve, and the adjoint Function object against central
// differences of its own forward.  Exit status 0 = all checks passed.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "lf_gb300.hpp"

extern "C" {
typedef struct {
  int32_t kind, func;
  double value;
  const double* data;
  double p[16];
} lfo_coeff;
int lfo_input_create(int kind, int64_t nx, int64_t ny, double x0, double y0, double x1, double y1, void** out,
                     int64_t* sizes, char* err, int errlen);
void lfo_input_copy(void* h, double* xy, int64_t* cells, int64_t* edges);
void lfo_input_destroy(void* h);
int lfo_mesh_create(int64_t nv, const double* xy, int64_t nc, const int64_t* cells, int64_t npre, const int64_t* pre,
                    void** out, char* err, int errlen);
void lfo_mesh_destroy(void* m);
int lfo_space_create(void* mp, int degree, int np, int ns, int nt, int nq, void** out, char* err, int errlen);
void lfo_space_destroy(void* s);
int lfo_assemble_rd(void* sp, const lfo_coeff* alpha, const lfo_coeff* gamma, int qdeg_tria, int qdeg_quad,
                    int64_t first_cell, int64_t last_cell, void** out, char* err, int errlen);
int lfo_assemble_load(void* sp, const lfo_coeff* f, int qdeg_tria, int qdeg_quad, double* b, char* err, int errlen);
int64_t lfo_coo_size(void* a);
void lfo_coo_copy(void* a, int32_t* r, int32_t* c, double* v);
void lfo_coo_destroy(void* a);
}

namespace g = lf::gb300;

static int failures = 0;
#define CHECK(cond, ...)                   \
  do {                                     \
    if (!(cond)) {                         \
      std::printf("FAIL %s:%d: ", __FILE__, __LINE__); \
      std::printf(__VA_ARGS__);            \
      std::printf("\n");                   \
      ++failures;                          \
    }                                      \
  } while (0)

static void CheckAssembly(const g::Context& ctx, int nx, int ny, int degree) {
  auto mesh = g::mesh::TPTriagMeshBuilder(ctx).setBottomLeftCorner(0, 0).setTopRightCorner(1, 1)
                  .setNumXCells(nx).setNumYCells(ny).Build();
  std::shared_ptr<g::uscalfe::FeSpaceLagrange> fes =
      degree == 1 ? g::uscalfe::FeSpaceLagrangeO<1>(mesh)
                  : degree == 2 ? g::uscalfe::FeSpaceLagrangeO<2>(mesh) : g::uscalfe::FeSpaceLagrangeO<3>(mesh);
  const int64_t nd = fes->NumDofs();
  // alpha = 1 + x^2 + y^2, gamma = 1, f = sin(pi x) sin(pi y)
  std::vector<double> pa(16, 0.0);
  pa[0] = 1.0; pa[8] = 1.0; pa[2] = 1.0;
  g::uscalfe::ReactionDiffusionElementMatrixProvider rd(fes, g::uscalfe::MeshFunction::Analytic(LFG_FN_POLY, pa),
                                                        g::uscalfe::MeshFunction::Constant(1.0), 4, 4);
  g::uscalfe::ScalarLoadElementVectorProvider lp(fes, g::uscalfe::MeshFunction::Analytic(LFG_FN_SINSIN, {0, 1, 1, 1}),
                                                 4, 4);
  g::assemble::COOMatrix A(ctx, nd, nd, fes->NumTriplets() + nd);
  g::assemble::AssembleMatrixLocally(0, *fes, *fes, rd, A);
  g::DeviceVector<double> b(ctx, nd);
  b.SetZero();
  g::assemble::AssembleVectorLocally(0, *fes, lp, b);
  const std::vector<lfg_triplet> t = A.Download();

  // the oracle on the same mesh
  char err[512];
  void *in = nullptr, *om = nullptr, *os = nullptr, *oc = nullptr;
  int64_t sz[3];
  lfo_input_create(0, nx, ny, 0, 0, 1, 1, &in, sz, err, 512);
  std::vector<double> xy(sz[0] * 2);
  std::vector<int64_t> cells(sz[1] * 4), edges(sz[2] * 2 + 2);
  lfo_input_copy(in, xy.data(), cells.data(), edges.data());
  CHECK(lfo_mesh_create(sz[0], xy.data(), sz[1], cells.data(), sz[2], edges.data(), &om, err, 512) == 0, "%s", err);
  CHECK(lfo_space_create(om, degree, 0, 0, 0, 0, &os, err, 512) == 0, "%s", err);
  lfo_coeff alpha{}, gamma{}, f{};
  alpha.kind = 4; alpha.func = LFG_FN_POLY;
  for (int i = 0; i < 16; ++i) alpha.p[i] = pa[i];
  gamma.kind = 1; gamma.value = 1.0;
  f.kind = 4; f.func = LFG_FN_SINSIN; f.p[1] = 1; f.p[2] = 1; f.p[3] = 1;
  CHECK(lfo_assemble_rd(os, &alpha, &gamma, 4, 4, 0, -1, &oc, err, 512) == 0, "%s", err);
  const int64_t n = lfo_coo_size(oc);
  std::vector<int32_t> r(n), c(n);
  std::vector<double> v(n);
  lfo_coo_copy(oc, r.data(), c.data(), v.data());
  CHECK(static_cast<int64_t>(t.size()) == n, "triplet count %zu vs %lld", t.size(), static_cast<long long>(n));
  const int nloc = (degree + 1) * (degree + 2) / 2, blk = nloc * nloc;
  for (int64_t k0 = 0; k0 < n && static_cast<size_t>(k0) < t.size(); k0 += blk) {
    double scale = 0.0;
    for (int q = 0; q < blk; ++q) scale = std::fmax(scale, std::fabs(v[k0 + q]));
    for (int q = 0; q < blk; ++q) {
      const int64_t k = k0 + q;
      CHECK(t[k].row == r[k] && t[k].col == c[k], "index mismatch at %lld", static_cast<long long>(k));
      CHECK(std::fabs(t[k].value - v[k]) <= 1e-12 * scale, "value mismatch at %lld: %.17g vs %.17g",
            static_cast<long long>(k), t[k].value, v[k]);
    }
  }
  std::vector<double> bo(nd, 0.0);
  CHECK(lfo_assemble_load(os, &f, 4, 4, bo.data(), err, 512) == 0, "%s", err);
  const std::vector<double> bg = b.Download();
  double bmax = 0.0, berr = 0.0;
  for (int64_t i = 0; i < nd; ++i) {
    bmax = std::fmax(bmax, std::fabs(bo[i]));
    berr = std::fmax(berr, std::fabs(bg[i] - bo[i]));
  }
  CHECK(berr <= 1e-12 * bmax, "load vector error %.3g of %.3g", berr, bmax);
  lfo_coo_destroy(oc);
  lfo_space_destroy(os);
  lfo_mesh_destroy(om);
  lfo_input_destroy(in);

  // Dirichlet 0 on the boundary, solve
  g::DeviceVector<uint8_t> flags = fes->BoundaryDofFlags();
  g::DeviceVector<double> zero(ctx, nd);
  zero.SetZero();
  g::assemble::FixFlaggedSolutionComponents(flags, zero, A, b);
  g::solve::CSRMatrix S = A.makeSparse();
  g::DeviceVector<double> x(ctx, nd);
  x.SetZero();
  g::solve::SolveOptions so;
  so.rtol = 1e-12;
  const lfg_solve_stats st = g::solve::SolvePCG(ctx, S, b, x, so);
  CHECK(st.converged && st.rel_residual <= 1e-12, "PCG: converged %d residual %.3g", st.converged, st.rel_residual);
  std::printf("assembly O%d %dx%d: %lld triplets, %lld dofs, PCG %d iterations\n", degree, nx, ny,
              static_cast<long long>(n), static_cast<long long>(nd), st.iterations);

  // capacity errors surface as lf::gb300::Error
  g::assemble::COOMatrix small(ctx, nd, nd, 4);
  bool threw = false;
  try {
    g::assemble::AssembleMatrixLocally(0, *fes, *fes, rd, small);
  } catch (const g::Error& e) {
    threw = e.code() == LFG_CAPACITY;
  }
  CHECK(threw, "capacity overflow did not throw LFG_CAPACITY");
}

// Robin-type boundary terms on the boundary edges: mass and load of O2 on a
// TPTriag mesh; every boundary edge contributes 9 triplets, the load sums to
// the boundary length (4) times g.
static void CheckEdges(const g::Context& ctx) {
  auto mesh = g::mesh::TPTriagMeshBuilder(ctx).setNumXCells(5).setNumYCells(3).Build();
  auto fes = g::uscalfe::FeSpaceLagrangeO<2>(mesh);
  const int64_t nd = fes->NumDofs(), ne = mesh->NumEntities(1);
  std::vector<uint8_t> nf(mesh->NumEntities(2)), ef(ne);
  g::DeviceVector<uint8_t> nfd(ctx, nf.size()), efd(ctx, ef.size());
  ctx.Check(lfg_mesh_boundary_flags(mesh->get(), nfd.data(), efd.data()));
  ef = efd.Download();
  int64_t nb = 0;
  for (uint8_t f : ef) nb += f != 0;
  g::uscalfe::MassEdgeMatrixProvider mp(fes, g::uscalfe::MeshFunction::Constant(2.0), efd.data());
  g::assemble::COOMatrix A(ctx, nd, nd, 9 * nb);
  g::assemble::AssembleMatrixLocally(1, *fes, *fes, mp, A);
  CHECK(A.size() == 9 * nb, "edge mass: %lld triplets for %lld boundary edges", static_cast<long long>(A.size()),
        static_cast<long long>(nb));
  double msum = 0.0;
  for (const lfg_triplet& t : A.Download()) msum += t.value;
  CHECK(std::fabs(msum - 2.0 * 4.0) < 1e-12, "edge mass sums to %.15g, not 2 x perimeter", msum);
  g::uscalfe::ScalarLoadEdgeVectorProvider lp(fes, g::uscalfe::MeshFunction::Constant(3.0), efd.data());
  g::DeviceVector<double> b(ctx, nd);
  b.SetZero();
  g::assemble::AssembleVectorLocally(1, *fes, lp, b);
  double bsum = 0.0;
  for (double x : b.Download()) bsum += x;
  CHECK(std::fabs(bsum - 3.0 * 4.0) < 1e-12, "edge load sums to %.15g, not 3 x perimeter", bsum);
  std::printf("edges: %lld boundary edges, mass sum %.6f, load sum %.6f\n", static_cast<long long>(nb), msum, bsum);
}

// The demo's post-processing (homDir_linfe_demo.cc:150-188): Dirichlet data
// from InitEssentialConditionFromFunction, solve, then the L2 and H1-seminorm
// errors through the fe:: facade; O2 interpolation of a quadratic is exact.
static void CheckPost(const g::Context& ctx) {
  // u = x(1-x)y(1-y) + 1 + x, -lap u = 2 (x(1-x) + y(1-y))
  const std::vector<double> pu = {1, 0, 0, 0, 1, 1, -1, 0, 0, -1, 1, 0, 0, 0, 0, 0};
  const std::vector<double> pf = {0, 2, -2, 0, 2, 0, 0, 0, -2, 0, 0, 0, 0, 0, 0, 0};
  double err[2][2];
  for (int r = 0; r < 2; ++r) {
    const int n = 16 << r;
    auto mesh = g::mesh::TPTriagMeshBuilder(ctx).setNumXCells(n).setNumYCells(n).Build();
    auto fes = g::uscalfe::FeSpaceLagrangeO<1>(mesh);
    const int64_t nd = fes->NumDofs(), ne = mesh->NumEntities(1);
    g::DeviceVector<uint8_t> nfd(ctx, mesh->NumEntities(2)), efd(ctx, ne);
    ctx.Check(lfg_mesh_boundary_flags(mesh->get(), nfd.data(), efd.data()));
    const auto u = g::uscalfe::MeshFunction::Analytic(LFG_FN_POLY, pu);
    auto ess = g::fe::InitEssentialConditionFromFunction(*fes, efd, u);
    g::uscalfe::ReactionDiffusionElementMatrixProvider ep(fes, g::uscalfe::MeshFunction::Constant(1.0),
                                                          g::uscalfe::MeshFunction::Zero());
    g::uscalfe::ScalarLoadElementVectorProvider lp(fes, g::uscalfe::MeshFunction::Analytic(LFG_FN_POLY, pf));
    g::assemble::COOMatrix A(ctx, nd, nd, fes->NumTriplets() + nd);
    g::assemble::AssembleMatrixLocally(0, *fes, *fes, ep, A);
    g::DeviceVector<double> b(ctx, nd);
    b.SetZero();
    g::assemble::AssembleVectorLocally(0, *fes, lp, b);
    g::assemble::FixFlaggedSolutionComponents(ess.first, ess.second, A, b);
    auto csr = A.makeSparse();
    g::DeviceVector<double> x(ctx, nd);
    x.SetZero();
    g::solve::SolveOptions so;
    so.rtol = 1e-12;
    g::solve::SolvePCG(ctx, csr, b, x, so);
    const g::fe::MeshFunctionFE mf_sol(fes, x);
    const g::fe::MeshFunctionGradFE mf_grad_sol(fes, x);
    err[r][0] = std::sqrt(g::fe::IntegrateMeshFunction(*mesh, g::fe::SquaredNormDiff(mf_sol, u), 4));
    err[r][1] = std::sqrt(g::fe::IntegrateMeshFunction(*mesh, g::fe::SquaredNormDiff(mf_grad_sol, u), 4));
    // the projection of u onto O2 on the same mesh: exact for the quadratic part only
    auto fes2 = g::uscalfe::FeSpaceLagrangeO<2>(mesh);
    const auto lin = g::uscalfe::MeshFunction::Analytic(LFG_FN_POLY, {1, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0});
    auto c2 = g::fe::NodalProjection(*fes2, lin);
    const g::fe::MeshFunctionFE mf2(fes2, c2);
    const double e2 = g::fe::IntegrateMeshFunction(*mesh, g::fe::SquaredNormDiff(mf2, lin), 4);
    CHECK(e2 < 1e-28, "O2 projection of 1 + x is not exact: %.3g", e2);
    const auto vals = mf2({0.25, 0.25});
    CHECK(vals.size() == static_cast<size_t>(mesh->NumEntities(0)), "MeshFunctionFE output size");
  }
  const double rl2 = std::log2(err[0][0] / err[1][0]), rh1 = std::log2(err[0][1] / err[1][1]);
  CHECK(std::fabs(rl2 - 2.0) < 0.2 && std::fabs(rh1 - 1.0) < 0.15, "error rates L2 %.3f H1 %.3f", rl2, rh1);
  std::printf("post: L2 errors %.3e %.3e (rate %.2f), H1 %.3e %.3e (rate %.2f)\n", err[0][0], err[1][0], rl2,
              err[0][1], err[1][1], rh1);
}

// io::GmshReader on the two-element fixture (gmsh_reader_tests.cc:22-140).
static void CheckGmsh(const g::Context& ctx, const char* dir) {
  const std::string path = std::string(dir) + "/two_element_hybrid_2d_v4_binary.msh";
  g::io::GmshReader reader(ctx, path);
  auto mesh = reader.mesh();
  CHECK(mesh->NumEntities(0) == 2 && mesh->NumEntities(1) == 6 && mesh->NumEntities(2) == 5,
        "two-element mesh has %lld cells, %lld edges, %lld nodes", static_cast<long long>(mesh->NumEntities(0)),
        static_cast<long long>(mesh->NumEntities(1)), static_cast<long long>(mesh->NumEntities(2)));
  const int32_t diag = reader.PhysicalEntityName2Nr("diagonal");
  CHECK(diag == 4 && reader.PhysicalEntityNr2Name(4) == "diagonal", "diagonal lookup");
  auto flags = reader.PhysicalEntityFlags(1, diag).Download();
  int64_t nd = 0;
  for (uint8_t f : flags) nd += f;
  CHECK(nd == 1, "%lld edges in the diagonal group", static_cast<long long>(nd));
  CHECK(reader.PhysicalEntities(0).size() == 3, "three cell groups");
  bool threw = false;
  try {
    reader.PhysicalEntityName2Nr("gugus");
  } catch (const g::Error& e) {
    threw = e.code() == LFG_NOT_FOUND;
  }
  CHECK(threw, "unknown name must throw LFG_NOT_FOUND");
  std::printf("gmsh: two-element mesh read, diagonal group = edge set of size %lld\n", static_cast<long long>(nd));
}

// fe::HierarchicScalarFESpace with fe::MassElementMatrixProvider: the mass
// matrix of degree 4 sums (1^T M 1) to the area, the diffusion matrix
// annihilates constants.
static void CheckHierarchic(const g::Context& ctx) {
  auto mesh = g::mesh::TPTriagMeshBuilder(ctx).setNumXCells(6).setNumYCells(5).Build();
  auto fes = g::fe::HierarchicScalarFESpace(mesh, 4);
  const int64_t nd = fes->NumDofs();
  g::fe::MassElementMatrixProvider mp(fes, g::uscalfe::MeshFunction::Constant(1.0));
  g::assemble::COOMatrix M(ctx, nd, nd, fes->NumTriplets());
  g::assemble::AssembleMatrixLocally(0, *fes, *fes, mp, M);
  // the vertex functions sum to one: 1^T M 1 restricted to vertex dofs = area
  const int64_t nv = mesh->NumEntities(2);
  double s = 0.0;
  for (const lfg_triplet& t : M.Download())
    if (t.row < nv && t.col < nv) s += t.value;
  CHECK(std::fabs(s - 1.0) < 1e-12, "hierarchic mass matrix over vertex functions sums to %.15g", s);
  g::fe::DiffusionElementMatrixProvider dp(fes, g::uscalfe::MeshFunction::Constant(2.0));
  g::assemble::COOMatrix A(ctx, nd, nd, fes->NumTriplets());
  g::assemble::AssembleMatrixLocally(0, *fes, *fes, dp, A);
  std::vector<double> row(nv, 0.0);
  for (const lfg_triplet& t : A.Download())
    if (t.row < nv && t.col < nv) row[t.row] += t.value;
  double mx = 0.0;
  for (double r : row) mx = std::max(mx, std::fabs(r));
  CHECK(mx < 1e-11, "diffusion matrix rows over vertex functions sum to %.3g", mx);
  std::printf("hierarchic: degree 4, %lld dofs, mass area %.15f\n", static_cast<long long>(nd), s);
  // a degree functor: edges 2 + index % 3, cells 1 + index % 4; with constant
  // alpha the diffusion matrix still annihilates the constants
  auto vfes = g::fe::HierarchicScalarFESpace(
      mesh, [](const g::mesh::EntityRef& e) { return e.Codim() == 1 ? 2 + e.index % 3 : 1 + e.index % 4; });
  const int64_t vnd = vfes->NumDofs();
  int64_t want = nv;
  for (int64_t e = 0; e < mesh->NumEntities(1); ++e) want += 1 + e % 3;
  for (int64_t c = 0; c < mesh->NumEntities(0); ++c) {
    const int p = 1 + static_cast<int>(c % 4);
    want += p <= 2 ? 0 : (p - 2) * (p - 1) / 2;
  }
  CHECK(vnd == want, "variable-degree hierarchic space has %lld dofs, expected %lld", static_cast<long long>(vnd),
        static_cast<long long>(want));
  g::fe::DiffusionElementMatrixProvider vdp(vfes, g::uscalfe::MeshFunction::Constant(1.0));
  g::assemble::COOMatrix VA(ctx, vnd, vnd, vfes->NumTriplets());
  g::assemble::AssembleMatrixLocally(0, *vfes, *vfes, vdp, VA);
  std::vector<double> vrow(vnd, 0.0);
  for (const lfg_triplet& t : VA.Download())
    if (t.col < nv) vrow[t.row] += t.value;
  double vmx = 0.0;
  for (double r : vrow) vmx = std::max(vmx, std::fabs(r));
  CHECK(vmx < 1e-11, "variable-degree diffusion matrix applied to 1 has entries up to %.3g", vmx);
  std::printf("hierarchic: per-entity degrees, %lld dofs\n", static_cast<long long>(vnd));
}

static double Lcg(uint64_t& s) {
  s = s * 6364136223846793005ull + 1442695040888963407ull;
  return static_cast<double>(s >> 11) * (1.0 / 9007199254740992.0);  // [0, 1)
}

static void CheckAdjoint(const g::Context& ctx) {
  auto mesh = g::mesh::TPTriagMeshBuilder(ctx).setNumXCells(8).setNumYCells(8).Build();
  auto fes = g::uscalfe::FeSpaceLagrangeO<1>(mesh);
  const int64_t nc = mesh->NumEntities(0), nd = fes->NumDofs();
  uint64_t seed = 12345;
  std::vector<double> th(nc), uo(nd);
  for (auto& t : th) t = Lcg(seed) - 0.5;
  for (auto& u : uo) u = 0.02 * Lcg(seed);
  g::DeviceVector<double> theta(ctx, th), u_obs(ctx, uo), grad(ctx, nc);
  g::adjoint::InverseConductivityFunction::Options o;
  o.solve.rtol = 1e-14;
  g::adjoint::InverseConductivityFunction F(fes, u_obs, o);
  const double J = F.Forward(theta);
  F.Backward(1.0, grad);
  const std::vector<double> gr = grad.Download();
  double gmax = 0.0;
  for (double x : gr) gmax = std::fmax(gmax, std::fabs(x));
  const double h = 1e-6;
  double worst = 0.0;
  for (int k = 0; k < 8; ++k) {
    const int64_t cidx = (k * 37 + 5) % nc;
    std::vector<double> tp = th, tm = th;
    tp[cidx] += h;
    tm[cidx] -= h;
    g::DeviceVector<double> dp(ctx, tp), dm(ctx, tm);
    const double fd = (F.Forward(dp) - F.Forward(dm)) / (2 * h);
    worst = std::fmax(worst, std::fabs(fd - gr[cidx]));
  }
  CHECK(worst <= 1e-6 * gmax, "central differences: error %.3g of max |g| %.3g", worst, gmax);
  // recompute mode: the same bits, only theta saved
  o.recompute = true;
  g::adjoint::InverseConductivityFunction R(fes, u_obs, o);
  g::DeviceVector<double> grad2(ctx, nc);
  const double J2 = R.Forward(theta);
  CHECK(R.SavedBytes() == nc * 8, "recompute mode saved %lld bytes", static_cast<long long>(R.SavedBytes()));
  R.Backward(1.0, grad2);
  const std::vector<double> g2 = grad2.Download();
  CHECK(J2 == J && std::memcmp(g2.data(), gr.data(), nc * sizeof(double)) == 0, "recompute mode differs");
  std::printf("adjoint: J %.6g, max |dJ/dtheta| %.3g, FD error %.3g\n", J, gmax, worst);
}

// The reference's fix_dof_test (assemble/test/coomatrix_tests.cc:77-121):
// FixSolutionComponentsLse on the 10 x 10 tridiagonal system; its exact
// solution must satisfy the modified system.  A dof listed twice is fixed to
// the sum of its values.
static void CheckFixLse(const g::Context& ctx) {
  const int N = 10;
  for (int dup = 0; dup < 2; ++dup) {
    g::assemble::COOMatrix A(ctx, N, N, 64);
    std::vector<double> bh(N);
    for (int k = 0; k < N; ++k) {
      if (k > 0) A.AddToEntry(k, k - 1, -1.0);
      if (k < N - 1) A.AddToEntry(k, k + 1, -1.0);
      A.AddToEntry(k, k, 2.0);
      bh[k] = k + 1;
    }
    g::DeviceVector<double> b(ctx, bh);
    g::assemble::fixed_components_t<double> fixed{{2, -1.0}, {4, -2.0}, {8, -3.0}};
    if (dup) fixed = {{8, -1.0}, {2, -1.0}, {4, -2.0}, {8, -2.0}};
    g::assemble::FixSolutionComponentsLse(fixed, A, b);
    const std::vector<double> exact{1, 1, -1, 0.5, -2, 7.75, 11.5, 8.25, -3, 3.5};
    auto S = A.makeSparse();
    g::DeviceVector<double> x(ctx, exact), y(ctx, N);
    ctx.Check(lfg_csr_spmv(S.get(), x.data(), y.data()));
    const std::vector<double> ax = y.Download(), bb = b.Download();
    double res = 0.0;
    for (int k = 0; k < N; ++k) res = std::max(res, std::fabs(ax[k] - bb[k]));
    CHECK(res <= 1e-12, "FixSolutionComponentsLse (dup %d): |A x_exact - b| = %g", dup, res);
    CHECK(A.size() == 3 * N - 2 - 9 + 3, "FixSolutionComponentsLse: %lld triplets", static_cast<long long>(A.size()));
  }
  std::printf("fix: FixSolutionComponentsLse meets the reference's exact solution\n");
}

int main(int argc, char** argv) {
  try {
    g::Context ctx(0);
    if (argc > 1) CheckGmsh(ctx, argv[1]);
    CheckAssembly(ctx, 12, 10, 1);
    CheckAssembly(ctx, 9, 7, 2);
    CheckAssembly(ctx, 6, 5, 3);
    CheckAdjoint(ctx);
    CheckEdges(ctx);
    CheckPost(ctx);
    CheckHierarchic(ctx);
    CheckFixLse(ctx);
  } catch (const g::Error& e) {
    std::printf("FAIL: uncaught lf::gb300::Error %d: %s\n", static_cast<int>(e.code()), e.what());
    return 1;
  }
  if (failures) {
    std::printf("%d check(s) failed\n", failures);
    return 1;
  }
  std::printf("facade_test OK\n");
  return 0;
}
