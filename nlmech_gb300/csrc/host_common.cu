// host_common.cu -- error text of the C ABI and the deck-level set-up of the
// loading classes restated on the host (region membership, ULoading spatial
// factors, FLoading spatial functions).

#include "fd_handle.h"

namespace nlm {

static thread_local std::string g_err;
void set_error(const std::string &msg) { g_err = msg; }
int cuda_fail(cudaError_t e, const char *what) {
  g_err = std::string(what) + ": " + cudaGetErrorString(e);
  if (e == cudaErrorMemoryAllocation) return NLM_ERR_OOM;
  // the solvers' bounded grid-barrier waits report a wait that ran out so
  if (e == cudaErrorTimeout) return NLM_ERR_TIMEOUT;
  return NLM_ERR_CUDA;
}
int fail(int code, const std::string &msg) {
  g_err = msg;
  return code;
}


const char *last_error() { return g_err.c_str(); }

// ---- host restatement of the deck-level set-up --------------------------

// Displacement_BC / Force_BC region membership (uLoading.cpp:93-160,
// fLoading.cpp:88-111, utilGeom.cpp:43-49,97-115,328-333).
bool in_region(const nlm_bc_set &bc, const double *p, int dim) {
  switch (bc.region) {
    case NLM_REGION_RECTANGLE:
      return !(hLT(p[0], bc.x1 - 1.0E-12) || hLT(p[1], bc.y1 - 1.0E-12) ||
               hGT(p[0], bc.x2 + 1.0E-12) || hGT(p[1], bc.y2 + 1.0E-12));
    case NLM_REGION_LINE:
      return hGT(p[0], bc.x1) && hLT(p[0], bc.x2);
    case NLM_REGION_CIRCLE: {
      const double d[3] = {p[0] - bc.x1, p[1] - bc.y1, p[2] - 0.};
      return std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) <= bc.r1;
    }
    case NLM_REGION_TORUS: {
      const double d[3] = {p[0] - bc.x1, p[1] - bc.y1, p[2] - 0.};
      const double l = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
      return l <= bc.r1 && !(l <= bc.r2);
    }
    case NLM_REGION_CUBOID:
      // isPointInsideCuboid(3, ...) as FLoading calls it (fLoading.cpp:104-107)
      return !(hLT(p[0], bc.x1 - 1.0E-12) || hLT(p[1], bc.y1 - 1.0E-12) ||
               hLT(p[2], bc.z1 - 1.0E-12) || hGT(p[0], bc.x2 + 1.0E-12) ||
               hGT(p[1], bc.y2 + 1.0E-12) || hGT(p[2], bc.z2 + 1.0E-12));
    case NLM_REGION_ANGLED_RECTANGLE: {
      // isPointInsideAngledRectangle with rotateCW2D (transformation.cpp:20-24)
      const double c = std::cos(bc.theta), s = std::sin(bc.theta);
      const double a0 = bc.x2 - bc.x1, a1 = bc.y2 - bc.y1;
      const double lam0 = a0 * c + a1 * s, lam1 = -a0 * s + a1 * c;
      const double b0 = p[0] - bc.x1, b1 = p[1] - bc.y1;
      const double m0 = b0 * c + b1 * s, m1 = -b0 * s + b1 * c;
      return !(hLT(m0, -1.0E-12) || hLT(m1, -1.0E-12) || hGT(m0, lam0 + 1.0E-12) ||
               hGT(m1, lam1 + 1.0E-12));
    }
  }
  return false;
}

// Spatial factor of ULoading::apply times time_params[0] (uLoading.cpp:172-208).
double uload_umax(const nlm_bc_set &bc, const double *x) {
  double umax = bc.time_params[0];
  const double *sp = bc.spatial_params;
  switch (bc.spatial_fn) {
    case NLM_SFN_SIN_X: { const double a = M_PI * sp[0]; umax = umax * std::sin(a * x[0]); } break;
    case NLM_SFN_SIN_Y: { const double a = M_PI * sp[0]; umax = umax * std::sin(a * x[1]); } break;
    case NLM_SFN_SIN_Z: { const double a = M_PI * sp[0]; umax = umax * std::sin(a * x[2]); } break;
    case NLM_SFN_LINEAR_X: { const double a = sp[0]; umax = umax * a * x[0]; } break;
    case NLM_SFN_LINEAR_Y: { const double a = sp[0]; umax = umax * a * x[1]; } break;
    case NLM_SFN_LINEAR_Z: { const double a = sp[0]; umax = umax * a * x[2]; } break;
    case NLM_SFN_CONSTANT: { const double a = sp[0]; umax = umax * a; } break;
    default: break;  // a Force_BC-only function: no spatial factor
  }
  return umax;
}

// util::function::hatFunction (utilFunction.cpp:14-30).
static double hat_function(double x, double x_min, double x_max) {
  if (hGT(x, x_min - 1.0E-12) && hLT(x, x_max + 1.0E-12)) {
    const double x_mid = 0.5 * (x_min + x_max);
    const double l = x_mid - x_min;
    if (l < 1.0E-12) return 1.0;
    return hLT(x, x_mid) ? (x - x_min) / l : (x_max - x) / l;
  }
  return 0.0;
}

// size_t(v) of a non-negative double (truncation); values below zero give 0,
// which is what a truncation of the (-1, 0) values a node inside its region
// can produce gives.
static double trunc_count(double v) {
  return v > 0. ? (v < 1.8e19 ? (double)(uint64_t)v : v) : 0.;
}

// "line_load" (fLoading.cpp:171-232): for each direction d of the set,
// fmax *= pos / nodes with nodes = size_t(|max - min| / h) and
// pos = size_t((x_d - min) / h), or size_t((max - x_d) / h) when p0 == -1.
static double line_load(const nlm_bc_set &bc, const double *x, double h) {
  double fmax = 1.0;
  const double lo[3] = {bc.x1, bc.y1, bc.z1}, hi[3] = {bc.x2, bc.y2, bc.z2};
  for (int d = 0; d < 3; d++) {
    if (!(bc.dir_mask >> d & 1)) continue;
    const double length = std::abs(hi[d] - lo[d]);
    const double nodes = trunc_count(length / h);
    const double scale = 1. / nodes;
    double pos = trunc_count((x[d] - lo[d]) / h);
    if (bc.spatial_params[0] == -1) pos = trunc_count((hi[d] - x[d]) / h);
    fmax *= pos * scale;
  }
  return fmax;
}

// Spatial part of FLoading::apply (fLoading.cpp:124-152).
double fload_spatial(const nlm_bc_set &bc, const double *x, double h) {
  const double *sp = bc.spatial_params;
  switch (bc.spatial_fn) {
    case NLM_SFN_HAT_X: return sp[0] * hat_function(x[0], bc.x1, bc.x2);
    case NLM_SFN_HAT_Y: return sp[0] * hat_function(x[1], bc.y1, bc.y2);
    case NLM_SFN_HAT_Z: return sp[0] * hat_function(x[2], bc.z1, bc.z2);
    case NLM_SFN_LINE_LOAD: return line_load(bc, x, h);
    case NLM_SFN_SIN_X: { const double a = M_PI * sp[0]; return sp[0] * std::sin(a * x[0]); }
    case NLM_SFN_SIN_Y: { const double a = M_PI * sp[0]; return sp[0] * std::sin(a * x[1]); }
    case NLM_SFN_SIN_Z: { const double a = M_PI * sp[0]; return sp[0] * std::sin(a * x[2]); }
    case NLM_SFN_LINEAR_X: { const double a = sp[0]; return sp[0] * a * x[0]; }
    case NLM_SFN_LINEAR_Y: { const double a = sp[0]; return sp[0] * a * x[1]; }
    case NLM_SFN_LINEAR_Z: { const double a = sp[0]; return sp[0] * a * x[2]; }
    default: return sp[0];
  }
}


}  // namespace nlm
