// Forward/backward Function object of the inverse-conductivity problem
// theta -> J(theta) = 1/2 ||u(theta) - u_obs||^2 (no reference counterpart; it
// drives the reference-shaped pipeline AssembleMatrixLocally ->
// FixFlaggedSolutionComponents -> solve twice, then the cellwise gradient).
//
// Saved state follows the autograd.Function contract: forward keeps what
// backward needs, backward consumes it.  In recompute mode only a copy of
// theta survives the forward; backward re-assembles and re-solves for u,
// trading one forward solve for the Galerkin matrix (about 12 bytes per
// nonzero plus row pointers) and two dof vectors.
#include <cstring>

#include "lfg_api.h"
#include "lfg_internal.h"

namespace lfg {
void GradRDCellwise(lfg_space* sp, const lfg_rd_provider* pr, const double* u, const double* lam,
                    const uint8_t* flags, double gscale, double* grad);
}

struct lfg_rd_adjoint {
  lfg::CtxRef ref;
  lfg_space* sp = nullptr;
  lfg_rd_adjoint_opts o{};
  int64_t nd = 0, nc = 0;
  lfg::DevBuf flags, g, b0, uobs, theta, u, r, lam, rhs, b;
  lfg_coo* coo = nullptr;
  lfg_csr* csr = nullptr;
  bool forward_done = false;
  bool saved = false;  // matrix, u and r valid for backward
  lfg_solve_stats fwd{}, adj{};
};

namespace lfg {
namespace {

void Check(lfg_ctx* ctx, lfg_status st) {
  if (st != LFG_OK) Fail(st, ctx->last_error);
}

// rhs = r with flagged entries set to zero (the adjoint source on free dofs).
__global__ void MaskKernel(int64_t n, const double* __restrict__ r, const uint8_t* __restrict__ flags,
                           double* __restrict__ out) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    out[i] = flags[i] ? 0.0 : r[i];
}

lfg_rd_provider Provider(const lfg_rd_adjoint* f) {
  lfg_rd_provider p{};
  p.alpha.kind = LFG_COEFF_PER_CELL_EXP;
  p.alpha.data_dev = f->theta.as<double>();
  p.gamma.kind = LFG_COEFF_ZERO;
  p.qr_degree_tria = f->o.qr_degree_tria;
  p.qr_degree_quad = f->o.qr_degree_quad;
  return p;
}

void ReleaseMatrix(lfg_rd_adjoint* f) {
  if (f->csr) lfg_csr_destroy(f->csr);
  if (f->coo) lfg_coo_destroy(f->coo);
  f->csr = nullptr;
  f->coo = nullptr;
}

// Assemble A(theta), b, fix, convert to CSR and solve for u (zero start);
// r = u - u_obs and J.
double SolveForward(lfg_rd_adjoint* f) {
  lfg_ctx* ctx = f->ref.c;
  cudaStream_t s = ctx->stream;
  const size_t vb = f->nd * sizeof(double);
  if (!f->u.p) f->u.alloc(vb, s);
  if (!f->r.p) f->r.alloc(vb, s);
  if (!f->b.p) f->b.alloc(vb, s);
  ReleaseMatrix(f);
  Check(ctx, lfg_coo_create(ctx, f->nd, f->nd, f->sp->num_triplets + f->nd, &f->coo));
  const lfg_rd_provider p = Provider(f);
  Check(ctx, lfg_assemble_matrix_rd(f->sp, &p, f->coo));
  LFG_CUDA(cudaMemcpyAsync(f->b.p, f->b0.p, vb, cudaMemcpyDeviceToDevice, s));
  Check(ctx, lfg_fix_flagged_solution_components(f->coo, f->flags.as<uint8_t>(), f->g.as<double>(),
                                                 f->b.as<double>()));
  Check(ctx, lfg_csr_from_coo(f->coo, &f->csr));
  lfg_coo_destroy(f->coo);  // the CSR holds the matrix from here on
  f->coo = nullptr;
  LFG_CUDA(cudaMemsetAsync(f->u.p, 0, vb, s));
  Check(ctx, lfg_solve_pcg(f->csr, f->b.as<double>(), f->u.as<double>(), &f->o.solve, &f->fwd));
  double loss = 0.0;
  Check(ctx, lfg_loss_l2_misfit(ctx, f->nd, f->u.as<double>(), f->uobs.as<double>(), &loss, f->r.as<double>()));
  return loss;
}

void DropSaved(lfg_rd_adjoint* f) {
  ReleaseMatrix(f);
  f->u.reset();
  f->r.reset();
  f->b.reset();
  f->saved = false;
}

}  // namespace
}  // namespace lfg

using namespace lfg;

extern "C" {

lfg_status lfg_rd_adjoint_create(lfg_space* sp, const lfg_rd_adjoint_opts* o, const double* u_obs,
                                 lfg_rd_adjoint** out) {
  if (!sp) return LFG_INVALID_ARG;
  LFG_API_BEGIN(sp->mesh->ctx)
  if (!o || !u_obs || !out) Fail(LFG_INVALID_ARG, "lfg_rd_adjoint_create: null argument");
  if (sp->degree < 1) Fail(LFG_UNSUPPORTED, "adjoint needs a Lagrangian space");
  lfg_ctx* ctx = sp->mesh->ctx;
  cudaStream_t s = ctx->stream;
  auto* f = new lfg_rd_adjoint();
  try {
    f->ref.Set(ctx);
    f->sp = sp;
    f->o = *o;
    f->nd = sp->num_dofs;
    f->nc = sp->mesh->nc;
    const size_t vb = f->nd * sizeof(double);
    f->flags.alloc(f->nd > 0 ? f->nd : 1, s);
    if (o->flags_dev) LFG_CUDA(cudaMemcpyAsync(f->flags.p, o->flags_dev, f->nd, cudaMemcpyDeviceToDevice, s));
    else Check(ctx, lfg_space_boundary_dof_flags(sp, f->flags.as<uint8_t>()));
    f->g.alloc(vb, s);
    if (o->dirichlet_dev) LFG_CUDA(cudaMemcpyAsync(f->g.p, o->dirichlet_dev, vb, cudaMemcpyDeviceToDevice, s));
    else LFG_CUDA(cudaMemsetAsync(f->g.p, 0, vb, s));
    f->uobs.alloc(vb, s);
    LFG_CUDA(cudaMemcpyAsync(f->uobs.p, u_obs, vb, cudaMemcpyDeviceToDevice, s));
    f->b0.alloc(vb, s);
    LFG_CUDA(cudaMemsetAsync(f->b0.p, 0, vb, s));
    Check(ctx, lfg_assemble_vector_load(sp, &o->load, f->b0.as<double>()));
    f->theta.alloc(f->nc * sizeof(double), s);
    LFG_CUDA(cudaStreamSynchronize(s));
  } catch (...) {
    delete f;
    throw;
  }
  *out = f;
  LFG_API_END
}

lfg_status lfg_rd_adjoint_destroy(lfg_rd_adjoint* f) {
  if (!f) return LFG_INVALID_ARG;
  cudaSetDevice(f->ref.c->device);
  ReleaseMatrix(f);
  delete f;  // buffers are freed stream-ordered; the context reference goes last
  return LFG_OK;
}

lfg_status lfg_rd_adjoint_forward(lfg_rd_adjoint* f, const double* theta, double* loss, double* u_out) {
  if (!f) return LFG_INVALID_ARG;
  LFG_API_BEGIN(f->ref.c)
  if (!theta || !loss) Fail(LFG_INVALID_ARG, "lfg_rd_adjoint_forward: null argument");
  lfg_ctx* ctx = f->ref.c;
  cudaStream_t s = ctx->stream;
  LFG_CUDA(cudaMemcpyAsync(f->theta.p, theta, f->nc * sizeof(double), cudaMemcpyDeviceToDevice, s));
  *loss = SolveForward(f);
  if (u_out) LFG_CUDA(cudaMemcpyAsync(u_out, f->u.p, f->nd * sizeof(double), cudaMemcpyDeviceToDevice, s));
  f->forward_done = true;
  f->saved = true;
  if (f->o.recompute) {
    LFG_CUDA(cudaStreamSynchronize(s));
    DropSaved(f);
  }
  LFG_API_END
}

lfg_status lfg_rd_adjoint_backward(lfg_rd_adjoint* f, double grad_loss, double* grad_theta) {
  if (!f) return LFG_INVALID_ARG;
  LFG_API_BEGIN(f->ref.c)
  if (!grad_theta) Fail(LFG_INVALID_ARG, "lfg_rd_adjoint_backward: null argument");
  if (!f->forward_done) Fail(LFG_INVALID_ARG, "lfg_rd_adjoint_backward: no forward call before backward");
  lfg_ctx* ctx = f->ref.c;
  cudaStream_t s = ctx->stream;
  if (!f->saved) SolveForward(f);
  const size_t vb = f->nd * sizeof(double);
  f->rhs.alloc(vb, s);
  f->lam.alloc(vb, s);
  if (f->nd > 0) {
    MaskKernel<<<GridFor(ctx, f->nd, 256), 256, 0, s>>>(f->nd, f->r.as<double>(), f->flags.as<uint8_t>(),
                                                        f->rhs.as<double>());
    LFG_LAUNCHED(ctx);
  }
  LFG_CUDA(cudaMemsetAsync(f->lam.p, 0, vb, s));
  Check(ctx, lfg_solve_pcg(f->csr, f->rhs.as<double>(), f->lam.as<double>(), &f->o.solve, &f->adj));
  const lfg_rd_provider p = Provider(f);
  GradRDCellwise(f->sp, &p, f->u.as<double>(), f->lam.as<double>(), f->flags.as<uint8_t>(), grad_loss, grad_theta);
  LFG_CUDA(cudaStreamSynchronize(s));
  f->rhs.reset();
  f->lam.reset();
  if (f->o.recompute) DropSaved(f);
  LFG_API_END
}

lfg_status lfg_rd_adjoint_stats(const lfg_rd_adjoint* f, lfg_solve_stats* fwd, lfg_solve_stats* adj,
                                int64_t* saved_bytes) {
  if (!f) return LFG_INVALID_ARG;
  if (fwd) *fwd = f->fwd;
  if (adj) *adj = f->adj;
  if (saved_bytes) {
    int64_t n = static_cast<int64_t>(f->u.bytes + f->r.bytes + f->b.bytes + f->theta.bytes);
    if (const lfg_csr* A = f->csr)
      n += static_cast<int64_t>(A->rowptr.bytes + A->col.bytes + A->val.bytes + A->val32.bytes +
                                A->rowptr32.bytes + A->dinv.bytes + A->dinv32.bytes);
    *saved_bytes = n;
  }
  return LFG_OK;
}

}  // extern "C"
