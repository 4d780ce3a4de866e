// Device form of an lfg_coeff (a MeshFunction of the reference:
// mesh/utils/mesh_function_global.h:54-94, mesh_function_constant.h:25-45,
// fe/mesh_function_fe.h:44-115) and the built-in analytic functions with
// their gradients.  Shared by the element kernels and the post-processing
// kernels.
#pragma once

#include <string>

#include "lfg_internal.h"

namespace lfg {

struct CoeffDev {
  int kind;
  int func;
  double value;
  const double* data;
  double p[16];
};

// f(x, y) of a built-in function (LFG_FN_*), FP64.
__device__ inline double EvalAnalytic(const CoeffDev& f, double x, double y) {
  switch (f.func) {
    case LFG_FN_POLY: {
      // Horner in y inside Horner in x: sum_i x^i sum_j p[4i+j] y^j
      double s = 0.0;
      for (int i = 3; i >= 0; --i) {
        const double* q = f.p + 4 * i;
        const double py = ((q[3] * y + q[2]) * y + q[1]) * y + q[0];
        s = s * x + py;
      }
      return s;
    }
    // sinpi / cospi (sin(pi t) with an exact argument reduction) instead of
    // sin(p pi t): the same function up to the rounding of p pi t
    case LFG_FN_SINSIN:
      return f.p[0] + f.p[1] * (sinpi(f.p[2] * x) * sinpi(f.p[3] * y));
    case LFG_FN_SINCOS:
      return f.p[0] + f.p[1] * (sinpi(f.p[2] * x) * cospi(f.p[3] * y));
    case LFG_FN_EXP:
      return f.p[0] + f.p[1] * exp(f.p[2] + f.p[3] * x + f.p[4] * y + f.p[5] * (x * y));
    case LFG_FN_TRIG: {
      const double l = f.p[1] + f.p[2] * x + f.p[3] * y + f.p[4] * (x * y);
      return f.p[0] + l * (sinpi(f.p[5] * x + f.p[6]) * sinpi(f.p[7] * y + f.p[8]));
    }
  }
  return 0.0;
}

// Gradient of EvalAnalytic's function, differentiated by hand per family.
__device__ inline void EvalAnalyticGrad(const CoeffDev& f, double x, double y, double& gx, double& gy) {
  const double pi = 3.141592653589793;
  switch (f.func) {
    case LFG_FN_POLY: {
      // d/dx: sum_{i>=1} i x^{i-1} sum_j p[4i+j] y^j;  d/dy: sum_i x^i sum_{j>=1} j p[4i+j] y^{j-1}
      double sx = 0.0, sy = 0.0;
      for (int i = 3; i >= 0; --i) {
        const double* q = f.p + 4 * i;
        const double py = ((q[3] * y + q[2]) * y + q[1]) * y + q[0];
        const double dpy = (3.0 * q[3] * y + 2.0 * q[2]) * y + q[1];
        if (i >= 1) sx = sx * x + i * py;
        sy = sy * x + dpy;
      }
      gx = sx;
      gy = sy;
      return;
    }
    case LFG_FN_SINSIN:
    case LFG_FN_SINCOS: {
      double sx, cx, sy, cy;
      sincospi(f.p[2] * x, &sx, &cx);
      sincospi(f.p[3] * y, &sy, &cy);
      if (f.func == LFG_FN_SINSIN) {
        gx = f.p[1] * (f.p[2] * pi) * cx * sy;
        gy = f.p[1] * (f.p[3] * pi) * sx * cy;
      } else {
        gx = f.p[1] * (f.p[2] * pi) * cx * cy;
        gy = -f.p[1] * (f.p[3] * pi) * sx * sy;
      }
      return;
    }
    case LFG_FN_EXP: {
      const double e = f.p[1] * exp(f.p[2] + f.p[3] * x + f.p[4] * y + f.p[5] * (x * y));
      gx = e * (f.p[3] + f.p[5] * y);
      gy = e * (f.p[4] + f.p[5] * x);
      return;
    }
    case LFG_FN_TRIG: {
      const double l = f.p[1] + f.p[2] * x + f.p[3] * y + f.p[4] * (x * y);
      double sx, cx, sy, cy;
      sincospi(f.p[5] * x + f.p[6], &sx, &cx);
      sincospi(f.p[7] * y + f.p[8], &sy, &cy);
      gx = (f.p[2] + f.p[4] * y) * sx * sy + l * (pi * f.p[5]) * cx * sy;
      gy = (f.p[3] + f.p[4] * x) * sx * sy + l * sx * (pi * f.p[7]) * cy;
      return;
    }
  }
  gx = gy = 0.0;
}

// Value of a coefficient at reference point (xh, yh) of cell c with global
// coordinates (X, Y): cell-wise constants, the O1 interpolant of nodal data
// (tria_o1 / quad_o1 shape functions), or the analytic function at (X, Y).
__device__ inline double EvalCoeffPoint(const CoeffDev& f, int c, const int4& cn, bool quad, double xh, double yh,
                                        double X, double Y) {
  switch (f.kind) {
    case LFG_COEFF_CONSTANT: return f.value;
    case LFG_COEFF_PER_CELL: return f.data[c];
    case LFG_COEFF_PER_CELL_EXP: return exp(f.data[c]);
    case LFG_COEFF_NODAL_O1:
      if (!quad) return f.data[cn.x] * (1.0 - xh - yh) + f.data[cn.y] * xh + f.data[cn.z] * yh;
      return f.data[cn.x] * ((1 - xh) * (1 - yh)) + f.data[cn.y] * (xh * (1 - yh)) + f.data[cn.z] * (xh * yh) +
             f.data[cn.w] * ((1 - xh) * yh);
    case LFG_COEFF_ANALYTIC: return EvalAnalytic(f, X, Y);
  }
  return 0.0;
}

inline bool KnownAnalytic(int func) { return func >= LFG_FN_POLY && func <= LFG_FN_TRIG; }

inline bool IsTensor(int kind) {
  return kind == LFG_COEFF_TENSOR_CONSTANT || kind == LFG_COEFF_TENSOR_PER_CELL || kind == LFG_COEFF_TENSOR_BILINEAR;
}

// Host conversion with the argument checks every entry point shares.
// Matrix-valued kinds pass only where the caller accepts them (allow_tensor).
inline CoeffDev ToDev(const lfg_coeff& c, const lfg_mesh* m, const char* what, bool allow_tensor = false) {
  (void)m;
  CoeffDev d;
  d.kind = c.kind;
  d.func = c.func;
  d.value = c.value;
  d.data = c.data_dev;
  for (int i = 0; i < 16; ++i) d.p[i] = c.p[i];
  if (IsTensor(c.kind) && !allow_tensor)
    Fail(LFG_UNSUPPORTED, std::string(what) + ": a matrix-valued coefficient is accepted only as the diffusion "
                                              "coefficient of the Lagrangian reaction-diffusion provider");
  if ((c.kind < LFG_COEFF_ZERO || c.kind > LFG_COEFF_PER_CELL_EXP) && !IsTensor(c.kind))
    Fail(LFG_UNSUPPORTED, std::string(what) + ": unsupported coefficient kind");
  if ((c.kind == LFG_COEFF_PER_CELL || c.kind == LFG_COEFF_NODAL_O1 || c.kind == LFG_COEFF_PER_CELL_EXP ||
       c.kind == LFG_COEFF_TENSOR_PER_CELL) &&
      !c.data_dev)
    Fail(LFG_INVALID_ARG, std::string(what) + ": coefficient data pointer is null");
  if (c.kind == LFG_COEFF_ANALYTIC && !KnownAnalytic(c.func))
    Fail(LFG_UNSUPPORTED, std::string(what) + ": unknown analytic function");
  return d;
}

}  // namespace lfg
