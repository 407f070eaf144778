// fd_host.cu -- C ABI of libnlmgpu: model set-up, time loop, state I/O.
//
// Replaces model::FDModel<T> (src/model/fd/fDModel.cpp) for T = RNPBond and
// ElasticState.  Set-up mirrors FDModel::initHObjects/init (:133-315):
// neighbour lists, pre-cracks, interior flags, loading tables, material
// constants.  The time loop mirrors FDModel::integrate (:317-374).
//
// Phase bookkeeping of the fused step.  One launch K_m does, per node, the
// force evaluation at u^m plus the integrator work on both sides of it:
//   Verlet:  v^m = (v^{m-1} + c f^{m-1}) + c f^m;   u^{m+1} = u^m + dt (v^m + c f^m)
//   CD:      u^{m+1} = u^m + (c' f^m + dt v^m);     v^{m+1} = (u^{m+1} - u^m) / dt
// with c = dt/(2 rho), c' = dt^2/rho.  u is ping-ponged (u^m read, u^{m+1}
// written); v is ping-ponged for CD.  After K_m the buffers hold exactly the
// reference's (u^m, v^m, f^m), and u^{m+1} is already in the other buffer.
// The velocity half-kick v^{m-1} + c f^{m-1} is recomputed from the stored
// f^{m-1}, so every value is produced by the same sequence of roundings as
// integrateVerlet.  K_0 (first = true) does the step-0 force evaluation of
// integrate() (:319-333) and the drift of step 1.

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include <cuda_fp16.h>

#include "fd_internal.h"
#include "neighbor.h"
#include "qs_internal.h"
#include "esqs_internal.h"
#include "fp32_common.cuh"
#include "state_io.cuh"

namespace nlm {

static thread_local std::string g_err;
void set_error(const std::string &msg) { g_err = msg; }
int cuda_fail(cudaError_t e, const char *what) {
  g_err = std::string(what) + ": " + cudaGetErrorString(e);
  if (e == cudaErrorMemoryAllocation) return NLM_ERR_OOM;
  return NLM_ERR_CUDA;
}
static int fail(int code, const std::string &msg) {
  g_err = msg;
  return code;
}

// ---- host restatement of the deck-level set-up --------------------------
static inline bool hGT(double a, double b) { return (a - b) > (amax_d(a, b) * 1e-5); }
static inline bool hLT(double a, double b) { return (b - a) > (amax_d(a, b) * 1e-5); }

// Displacement_BC / Force_BC region membership (uLoading.cpp:93-160,
// fLoading.cpp:88-111, utilGeom.cpp:43-49,97-115,328-333).
static bool in_region(const nlm_bc_set &bc, const double *p, int dim) {
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
static double uload_umax(const nlm_bc_set &bc, const double *x) {
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
static double fload_spatial(const nlm_bc_set &bc, const double *x, double h) {
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

// Time part of FLoading::apply (fLoading.cpp:246-266), applied as
// fmax = (spatial * g(t)) * time_params[0].
__device__ double fload_time(const BCTime &T, double fmax, double time) {
  switch (T.fn) {
    case NLM_TFN_LINEAR: fmax = fmax * time; break;
    case NLM_TFN_LINEAR_STEP: {
      const double x1 = T.p[1], x2 = T.p[2];
      const double period = floor(time / (x1 + x2));
      const double g = dLT(time, period * (x1 + x2) + x1) ? time - period * x2 : (period + 1.) * x1;
      fmax = fmax * g;
    } break;
    case NLM_TFN_LINEAR_SLOW_FAST:
      fmax = dGT(time, T.p[1]) ? fmax * (T.p[3] * time) : fmax * (T.p[2] * time);
      break;
    case NLM_TFN_SIN: fmax = fmax * sin((M_PI * T.p[1]) * time); break;
    default: break;
  }
  return fmax * T.p[0];
}

// ---- small kernels --------------------------------------------------------
struct FBCItem {
  int set;
  int dir_mask;
  double spatial;
};

// time: the load time, or tdev[0] when tdev is set (graph replay).
__global__ void k_fbc_apply(int64_t nf, int S, const int *nodes, const int *iptr,
                            const FBCItem *items, BCTable T, double time, double *fext,
                            const double *tdev = nullptr) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nf) return;
  if (tdev) time = tdev[0];
  double fe[3] = {0., 0., 0.};
  for (int k = iptr[t]; k < iptr[t + 1]; k++) {
    const FBCItem it = items[k];
    const double v = fload_time(T.t[it.set], it.spatial, time);
    for (int d = 0; d < 3; d++)
      if (it.dir_mask >> d & 1) fe[d] = fe[d] + v;
  }
  const int64_t i = nodes[t];
  for (int d = 0; d < S && d < 3; d++) fext[S * i + d] = fe[d];
}

__device__ inline void ld_split_any(const float4 *p, int S, int64_t i, double o[3]) {
  if (S == 2) {
    const float4 a = p[i];
    o[0] = (double)a.x + (double)a.z;
    o[1] = (double)a.y + (double)a.w;
    o[2] = 0.;
  } else {
    const float4 a = p[2 * i], b = p[2 * i + 1];
    o[0] = (double)a.x + (double)b.x;
    o[1] = (double)a.y + (double)b.y;
    o[2] = (double)a.z + (double)b.z;
  }
}
__device__ inline void st_split_any(float4 *p, int S, int64_t i, const double v[3]) {
  float h[3], l[3];
  for (int d = 0; d < 3; d++) {
    h[d] = __double2float_rn(v[d]);
    l[d] = __double2float_rn(v[d] - (double)h[d]);
  }
  if (S == 2)
    p[i] = make_float4(h[0], h[1], l[0], l[1]);
  else {
    p[2 * i] = make_float4(h[0], h[1], h[2], 0.f);
    p[2 * i + 1] = make_float4(l[0], l[1], l[2], 0.f);
  }
}

__global__ void k_bc_apply(int64_t nb, int S, int dim, const int *nodes, const int *bcref,
                           const BCEntry *bce, const uint8_t *flags, BCTable T, double time,
                           double *u64, float4 *u32, double *v, float4 *v32) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nb) return;
  const int64_t i = nodes[t];
  const BCEntry e = bce[bcref[i]];
  const uint8_t fl = flags[i];
  double uo[3], vo[3];
  if (u64) {
    for (int d = 0; d < 3; d++) uo[d] = d < S ? u64[S * i + d] : 0.;
    for (int d = 0; d < 3; d++) vo[d] = d < S ? v[S * i + d] : 0.;
  } else {
    ld_split_any(u32, S, i, uo);
    ld_split_any(v32, S, i, vo);
  }
  for (int d = 0; d < dim; d++)
    if ((fl >> d & 1) && e.set[d] >= 0) {
      double du, dv;
      bc_value(T.t[e.set[d]], e.umax[d], time, du, dv);
      uo[d] = du;
      vo[d] = dv;
    }
  if (u64) {
    for (int d = 0; d < S && d < 3; d++) u64[S * i + d] = uo[d];
    for (int d = 0; d < S && d < 3; d++) v[S * i + d] = vo[d];
  } else {
    st_split_any(u32, S, i, uo);
    st_split_any(v32, S, i, vo);
  }
}

// AoS original order (3 doubles per node) <-> internal layouts.
__global__ void k_scatter_vec(int64_t n, int S, int dim, const int *perm, const double *src,
                              double *dst) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double *p = src + 3 * (int64_t)perm[i];
  for (int d = 0; d < S; d++) dst[S * i + d] = (d < dim && d < 3) ? p[d] : 0.;
}
__global__ void k_invert_perm(int64_t n, const int *perm, int *iperm) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) iperm[perm[i]] = (int)i;
}

// Pinned caller arrays read in place.  The caller's arrays are taken as flat
// sequences of 3n doubles, two per thread with 16-byte loads, so every byte
// crosses the host link once in full lines.  Value k is component k % 3 of
// caller node k / 3; it goes into a staging copy of the state array in the
// internal order (FP32C: its (hi, lo) floats), or, for a component the model
// does not hold (z in 2-D), into zkeep in the caller's order.
template <bool FP32>
__device__ __forceinline__ void stage_value(int S, int dim, int64_t i, int d, double x, void *dst,
                                            double *zkeep, int64_t k) {
  if (d >= dim) {
    if (zkeep) zkeep[k / 3] = x;
    return;
  }
  if (FP32) {
    float *q = static_cast<float *>(dst);
    const float hi = __double2float_rn(x), lo = __double2float_rn(x - (double)hi);
    if (S == 2) {
      q[4 * i + d] = hi;
      q[4 * i + 2 + d] = lo;
    } else {
      q[8 * i + d] = hi;
      q[8 * i + 4 + d] = lo;
    }
  } else {
    static_cast<double *>(dst)[S * i + d] = x;
  }
}

template <bool FP32>
__global__ void k_host_in(int64_t n, int S, int dim, const int *iperm, const double2 *hu,
                          const double2 *hv, const double2 *hf, void *su, void *sv, void *sf,
                          double *zu, double *zv, int *bad) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (2 * t >= 3 * n) return;
  const double2 a = hu[t], b = hv[t], c = hf[t];
  if (!(isfinite(a.x) && isfinite(a.y) && isfinite(b.x) && isfinite(b.y) && isfinite(c.x) &&
        isfinite(c.y)))
    atomicExch(bad, 1);
  for (int h = 0; h < 2; h++) {
    const int64_t k = 2 * t + h;
    const int64_t o = k / 3;
    const int d = (int)(k - 3 * o);
    const int64_t i = iperm[o];
    stage_value<FP32>(S, dim, i, d, h ? a.y : a.x, su, zu, k);
    stage_value<FP32>(S, dim, i, d, h ? b.y : b.x, sv, zv, k);
    if (d < dim) {
      if (FP32)
        static_cast<float *>(sf)[S * i + d] = (float)(h ? c.y : c.x);
      else
        static_cast<double *>(sf)[S * i + d] = h ? c.y : c.x;
    }
  }
}

// The state written into the pinned caller arrays in place, two doubles per
// thread with 16-byte stores: the model's components of u and v, their z in
// 2-D from zkeep (the caller's own values, which the reference's 2-D
// integrator never changes), and f with z = 0 in 2-D (the reference resets f
// every step).
template <bool FP32>
__device__ __forceinline__ double state_value(int S, int64_t i, int d, const void *src) {
  if (FP32) {
    const float *q = static_cast<const float *>(src);
    if (S == 2) return (double)q[4 * i + d] + (double)q[4 * i + 2 + d];
    return (double)q[8 * i + d] + (double)q[8 * i + 4 + d];
  }
  return static_cast<const double *>(src)[S * i + d];
}

template <bool FP32>
__global__ void k_host_out(int64_t n, int S, int dim, const int *iperm, const void *u,
                           const void *v, const void *f, const double *zu, const double *zv,
                           double2 *hu, double2 *hv, double2 *hf) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (2 * t >= 3 * n) return;
  double a[2], b[2], c[2];
  for (int h = 0; h < 2; h++) {
    const int64_t k = 2 * t + h;
    const int64_t o = k / 3;
    const int d = (int)(k - 3 * o);
    const int64_t i = iperm[o];
    if (d < dim) {
      a[h] = state_value<FP32>(S, i, d, u);
      b[h] = state_value<FP32>(S, i, d, v);
      c[h] = FP32 ? (double)static_cast<const float *>(f)[S * i + d]
                  : static_cast<const double *>(f)[S * i + d];
    } else {
      a[h] = zu[o];
      b[h] = zv[o];
      c[h] = 0.;
    }
  }
  hu[t] = make_double2(a[0], a[1]);
  hv[t] = make_double2(b[0], b[1]);
  hf[t] = make_double2(c[0], c[1]);
}

__global__ void k_nonfinite(int64_t m, const double *a, int *flag) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k < m && !isfinite(a[k])) atomicExch(flag, 1);
}
__global__ void k_scatter_split(int64_t n, int S, int dim, const int *perm, const double *src,
                                float4 *dst) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double *p = src + 3 * (int64_t)perm[i];
  float h[3], l[3];
  for (int d = 0; d < 3; d++) {
    const double val = d < dim ? p[d] : 0.;
    h[d] = __double2float_rn(val);
    l[d] = __double2float_rn(val - (double)h[d]);
  }
  if (S == 2)
    dst[i] = make_float4(h[0], h[1], l[0], l[1]);
  else {
    dst[2 * i] = make_float4(h[0], h[1], h[2], 0.f);
    dst[2 * i + 1] = make_float4(l[0], l[1], l[2], 0.f);
  }
}
__global__ void k_scatter_f32(int64_t n, int S, int dim, const int *perm, const double *src,
                              float *dst) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double *p = src + 3 * (int64_t)perm[i];
  for (int d = 0; d < S; d++) dst[S * i + d] = (d < dim && d < 3) ? (float)p[d] : 0.f;
}
// keep_z (2-D): the z entry of dst is left as it is (the caller's own value,
// uploaded into the same slot), as the reference's 2-D integrator never
// writes the z component of u and v.
__global__ void k_gather_vec(int64_t n, int S, const int *perm, const double *src, double *dst,
                             bool keep_z = false) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double *p = dst + 3 * (int64_t)perm[i];
  for (int d = 0; d < 3; d++)
    if (d < S || !keep_z) p[d] = d < S ? src[S * i + d] : 0.;
}
__global__ void k_gather_split(int64_t n, int S, const int *perm, const float4 *src, double *dst,
                               bool keep_z = false) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double *p = dst + 3 * (int64_t)perm[i];
  if (S == 2) {
    const float4 a = src[i];
    p[0] = (double)a.x + (double)a.z;
    p[1] = (double)a.y + (double)a.w;
    if (!keep_z) p[2] = 0.;
  } else {
    const float4 a = src[2 * i], b = src[2 * i + 1];
    p[0] = (double)a.x + (double)b.x;
    p[1] = (double)a.y + (double)b.y;
    p[2] = (double)a.z + (double)b.z;
  }
}
__global__ void k_gather_f32(int64_t n, int S, const int *perm, const float *src, double *dst) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double *p = dst + 3 * (int64_t)perm[i];
  for (int d = 0; d < 3; d++) p[d] = d < S ? (double)src[S * i + d] : 0.;
}
// FP32C position store: hi = (float)x, lo = x - hi packed as half(lo * scale).
__global__ void k_make_pos32(int64_t n, int S, const double *pos, const double *vol, double scale,
                             float4 *pos32, uint2 *pos32lo) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  float h[3];
  __half l[3];
  for (int d = 0; d < 3; d++) {
    const double v = d < S ? pos[S * i + d] : 0.;
    h[d] = __double2float_rn(v);
    l[d] = __float2half_rn((float)((v - (double)h[d]) * scale));
  }
  const __half2 lxy = __halves2half2(l[0], l[1]);
  const __half2 lz = __halves2half2(l[2], __float2half_rn(0.f));
  const float V = (float)vol[i];
  if (S == 2) {
    pos32[i] = make_float4(h[0], h[1], V, *reinterpret_cast<const float *>(&lxy));
  } else {
    pos32[i] = make_float4(h[0], h[1], h[2], V);
    pos32lo[i] = make_uint2(*reinterpret_cast<const unsigned *>(&lxy),
                            *reinterpret_cast<const unsigned *>(&lz));
  }
}
__global__ void k_count_bits(int64_t n, int nwords, int64_t npad, const uint32_t *bits,
                             unsigned long long *out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  int c = 0;
  for (int w = 0; w < nwords; w++) c += __popc(bits[(int64_t)w * npad + i]);
  if (c) atomicAdd(out, (unsigned long long)c);
}

static unsigned nblk(int64_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

}  // namespace nlm

using namespace nlm;

// ---- the handle ----------------------------------------------------------
struct nlm_fd {
  int dim = 2, S = 2;
  int64_t n = 0, nnz = 0;
  int precision = NLM_PREC_FP64, scheme = NLM_VELOCITY_VERLET, decomp = NLM_DECOMP_THREAD;
  int material = NLM_MAT_RNP_BOND;
  double dt = 0., time = 0.;
  int64_t step = 0;
  bool started = false;
  int cur = 0;
  bool rows_by_orig = true;  // device rows ordered by original id
  StepParams P{};
  BCTable T{};
  cudaStream_t stream = nullptr;
  std::vector<void *> allocs;
  DevPtrs D{};
  int64_t nslices = 0, sell_entries = 0;
  bool tile_ok = false;  // tile store built (NLM_DECOMP_TILE available)
  // host copies
  std::vector<int> perm;    // internal -> original
  std::vector<int64_t> rowptr;  // internal CSR offsets (host copy)
  // loads
  int *bc_nodes = nullptr;
  int64_t n_bc_nodes = 0;
  int *fbc_nodes = nullptr, *fbc_iptr = nullptr;
  FBCItem *fbc_items = nullptr;
  int64_t n_fbc_nodes = 0;
  BCTable FT{};
  double bbox_lo[3] = {0., 0., 0.}, bbox_hi[3] = {0., 0., 0.};  // fe::Mesh::computeBBox
  // timed cracks (Fracture::addCrack): cut after a step, bit c of cracks_on set once cut
  std::vector<nlm_crack> timed_cracks;
  uint32_t cracks_on = 0;
  // staging
  double *stage = nullptr;   // 3 slots of 3n doubles (u, v, f in Point3 layout)
  int *bad_input = nullptr;  // set by k_nonfinite
  int *iperm = nullptr;      // original -> internal node id (in-place host I/O)
  char *zstage = nullptr;    // state-layout staging of in-place host input
  int host_io = 0;           // last nlm_fd_step_host: 0 copies, 1 in place, 2 banded
  // banded host step: the caller's arrays move in contiguous bands on the copy
  // engines, each band's arrival releases the tiles whose nodes and halo it
  // completes, and a band goes back out once all tiles owning its nodes ran
  std::vector<int> tile_need;  // per tile: highest caller index its step reads
  int pipe_state = 0;          // 0 not set up, 1 ready, -1 unavailable
  int pipe_nbands = 0;
  std::vector<int64_t> pipe_bounds;  // band b = caller nodes [bounds[b], bounds[b + 1])
  std::vector<int> pipe_toff;  // stage k runs pipe_tiles[toff[k] .. toff[k + 1])
  std::vector<std::vector<int>> pipe_out;  // bands written back after stage k
  int *pipe_tiles = nullptr;
  int *pipe_late = nullptr;    // caller nodes final only after their band went out
  int64_t pipe_nlate = 0;
  double *pipe_in = nullptr, *pipe_back = nullptr;  // staged u, v, f: 9 n doubles each
  float4 *pipe_ua = nullptr, *pipe_ub = nullptr, *pipe_v = nullptr;
  float2 *pipe_f = nullptr;
  uint32_t *pipe_bits = nullptr;
  cudaStream_t pipe_sin = nullptr, pipe_sout = nullptr;
  std::vector<cudaEvent_t> pipe_ev;  // per band: input arrived, output ready
  float *dmg_phi = nullptr, *dmg_Z = nullptr;
  float *en_buf = nullptr;     // nlm_fd_energies: 4 n floats
  double *en_fext = nullptr;   // external force at the current time, S n doubles
  double *rf_buf = nullptr;    // nlm_fd_reaction_force: 2 n doubles
  unsigned long long *counter = nullptr;
  // CUDA-graph replay of the step loop
  int graph_steps = 0;
  cudaGraphExec_t gexec[2] = {nullptr, nullptr};  // by starting ping index
  double *d_times = nullptr, *h_times = nullptr;  // device / pinned host
  cudaEvent_t ev_times = nullptr;
  bool capturing = false;
  // timing
  bool timing = false;
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_used = 0;
  double acc_ms = 0.;
  int64_t launches = 0;
  double bytes_per_launch = 0.;

  int vidx() const { return scheme == NLM_CENTRAL_DIFFERENCE ? cur : 0; }

  // device bytes the handle may still allocate (nlm_fd_set_alloc_limit); < 0: no limit
  int64_t alloc_budget = -1;
  std::vector<size_t> alloc_sizes;  // bytes of allocs[k]

  template <class Tp>
  cudaError_t alloc(Tp **p, size_t count) {
    const size_t bytes = count * sizeof(Tp) + 16;
    if (alloc_budget >= 0 && (int64_t)bytes > alloc_budget) return cudaErrorMemoryAllocation;
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, bytes);
    if (e == cudaSuccess) {
      allocs.push_back(q);
      alloc_sizes.push_back(bytes);
      if (alloc_budget >= 0) alloc_budget -= (int64_t)bytes;
      *p = static_cast<Tp *>(q);
    }
    return e;
  }
  // free one allocation of alloc() (no-op for null) and clear the pointer
  template <class Tp>
  void release(Tp **p) {
    if (!*p) return;
    for (size_t k = 0; k < allocs.size(); k++)
      if (allocs[k] == (void *)*p) {
        cudaFree(allocs[k]);
        if (alloc_budget >= 0) alloc_budget += (int64_t)alloc_sizes[k];
        allocs.erase(allocs.begin() + k);
        alloc_sizes.erase(alloc_sizes.begin() + k);
        break;
      }
    *p = nullptr;
  }
  ~nlm_fd() {
    if (stream) cudaStreamSynchronize(stream);
    for (auto &g : gexec)
      if (g) cudaGraphExecDestroy(g);
    if (h_times) cudaFreeHost(h_times);
    if (ev_times) cudaEventDestroy(ev_times);
    for (void *p : allocs) cudaFree(p);
    for (auto e : ev_pool) cudaEventDestroy(e);
    if (pipe_sin) cudaStreamSynchronize(pipe_sin);
    if (pipe_sout) cudaStreamSynchronize(pipe_sout);
    for (auto e : pipe_ev) cudaEventDestroy(e);
    if (pipe_sin) cudaStreamDestroy(pipe_sin);
    if (pipe_sout) cudaStreamDestroy(pipe_sout);
    if (stream) cudaStreamDestroy(stream);
  }
};

int get_state_impl(nlm_fd *h, double *u, double *v, double *f, bool keep_z);

namespace {

bool finite_all(const double *a, int64_t n) {
  for (int64_t i = 0; i < n; i++)
    if (!std::isfinite(a[i])) return false;
  return true;
}

// No-fail flags (ComputeInterior / DataInterior, interiorFlags.cpp:57-100,
// :146-185): a node is not interior when it lies within tol of the mesh
// bounding box.  fe::Mesh::computeBBox (mesh.cpp:311-324) starts both corners
// at the origin and only widens them, so the box always contains the origin.
void mesh_bbox(const double *x, int64_t n, double lo[3], double hi[3]) {
  for (int dd = 0; dd < 3; dd++) lo[dd] = hi[dd] = 0.;
  for (int64_t i = 0; i < n; i++)
    for (int dd = 0; dd < 3; dd++) {
      if (hLT(x[3 * i + dd], lo[dd])) lo[dd] = x[3 * i + dd];
      if (hLT(hi[dd], x[3 * i + dd])) hi[dd] = x[3 * i + dd];
    }
}

// The No_Fail_Region list (:76-90): circles |x - c| < r and rectangles
// (isPointInsideRectangle, utilGeom.cpp:43-50) are not interior either.
void nofail_flags(const double *x, int64_t n, double tol, int nreg, const nlm_nofail_region *reg,
                  std::vector<uint8_t> &interior) {
  double lo[3], hi[3];
  mesh_bbox(x, n, lo, hi);
  for (int64_t i = 0; i < n; i++) {
    const double *p = x + 3 * i;
    bool in = !(hLT(p[0], lo[0] + tol) || hLT(p[1], lo[1] + tol) ||
                hGT(p[0], hi[0] - tol) || hGT(p[1], hi[1] - tol));
    for (int r = 0; r < nreg && in; r++) {
      const double *q = reg[r].params;
      if (reg[r].kind == NLM_NOFAIL_CIRCLE) {
        const double d0 = p[0] - q[0], d1 = p[1] - q[1], d2 = p[2] - q[2];
        if (hLT(std::sqrt(d0 * d0 + d1 * d1 + d2 * d2), q[3])) in = false;
      } else if (!(hLT(p[0], q[0] - 1.0E-12) || hLT(p[1], q[1] - 1.0E-12) ||
                   hGT(p[0], q[2] + 1.0E-12) || hGT(p[1], q[3] + 1.0E-12))) {
        in = false;
      }
    }
    interior[i] = in;
  }
}

// The function names ULoading and FLoading accept (uLoading.cpp:35-53,
// fLoading.cpp:33-52); the reference exits on any other.
int check_bc_functions(const nlm_fd_desc &d) {
  for (int k = 0; k < d.n_ubc; k++) {
    const nlm_bc_set &b = d.ubc[k];
    if (b.region < NLM_REGION_RECTANGLE || b.region > NLM_REGION_ANGLED_RECTANGLE)
      return fail(NLM_ERR_INVALID, "Displacement_BC region type not recognised");
    if (b.spatial_fn < NLM_SFN_CONSTANT || b.spatial_fn > NLM_SFN_LINEAR_Z)
      return fail(NLM_ERR_INVALID, "Displacement_BC spatial function not recognised");
    if (b.time_fn < NLM_TFN_CONSTANT || b.time_fn > NLM_TFN_LINEAR_SLOW_FAST)
      return fail(NLM_ERR_INVALID, "Displacement_BC time function not recognised");
  }
  for (int k = 0; k < d.n_fbc; k++) {
    const nlm_bc_set &b = d.fbc[k];
    if (b.region != NLM_REGION_RECTANGLE && b.region != NLM_REGION_LINE &&
        b.region != NLM_REGION_ANGLED_RECTANGLE && b.region != NLM_REGION_CUBOID)
      return fail(NLM_ERR_INVALID, "Force_BC region type not recognised (fLoading.cpp:24-31)");
    if (b.spatial_fn < NLM_SFN_CONSTANT || b.spatial_fn > NLM_SFN_LINE_LOAD)
      return fail(NLM_ERR_INVALID, "Force_BC spatial function not recognised");
    if (b.time_fn < NLM_TFN_CONSTANT || b.time_fn > NLM_TFN_LINEAR_SLOW_FAST ||
        b.time_fn == NLM_TFN_QUADRATIC)
      return fail(NLM_ERR_INVALID, "Force_BC time function not recognised");
  }
  return NLM_OK;
}

int check_nofail_regions(const nlm_fd_desc &d) {
  if (d.n_nofail_regions < 0 || (d.n_nofail_regions > 0 && !d.nofail_regions))
    return fail(NLM_ERR_INVALID, "bad no-fail region list");
  for (int r = 0; r < d.n_nofail_regions; r++)
    if (d.nofail_regions[r].kind != NLM_NOFAIL_CIRCLE &&
        d.nofail_regions[r].kind != NLM_NOFAIL_RECTANGLE)
      return fail(NLM_ERR_INVALID, "no-fail region kind must be circle or rectangle");
  return NLM_OK;
}

// RNPBond constants (rnpBond.cpp:23-97, computeParameters :99-189) and the
// influence function (influenceFn.h:85-402).
int rnp_constants(const nlm_material &m, int dim, double delta, StepParams &P) {
  double Kbulk = 0.;
  P.infl_type = m.influence_type;
  const int np = m.n_influence_params;
  double M = 0.;
  if (m.influence_type == 0) {
    P.infl_a0 = np == 0 ? double(dim + 1) : m.influence_params[0];
    M = P.infl_a0 / double(dim + 1);
  } else if (m.influence_type == 1) {
    if (np == 0) {
      P.infl_a0 = dim == 1 ? 6. : (dim == 2 ? 12. : 20.);
      P.infl_a1 = -P.infl_a0;
    } else {
      P.infl_a0 = m.influence_params[0];
      P.infl_a1 = np < 2 ? -P.infl_a0 : m.influence_params[1];
    }
    M = (P.infl_a0 / double(dim + 1)) + (P.infl_a1 / double(dim + 2));
  } else if (m.influence_type == 2) {
    if (np == 0) {
      P.infl_beta = 0.2;
      const double b = P.infl_beta;
      if (dim == 1)
        P.infl_alpha = 2. / (b * (1. - std::exp(-1. / b)));
      else if (dim == 2)
        P.infl_alpha = (4.0 / b) * 1.0 /
                       (std::sqrt(M_PI * b) * std::erf(1.0 / std::sqrt(b)) - 2.0 * std::exp(-1.0 / b));
      else
        P.infl_alpha = (2.0 / b) * 1.0 / (b - (b + 1.) * std::exp(-1.0 / b));
    } else {
      P.infl_alpha = m.influence_params[0];
      P.infl_beta = m.influence_params[1];
    }
    const double a = P.infl_alpha, b = P.infl_beta;
    const double sq1 = std::sqrt(b), sq2 = std::sqrt(M_PI);
    if (dim == 1)
      M = 0.5 * a * b * (1. - std::exp(-1. / b));
    else if (dim == 2)
      M = 0.5 * a * b * sq1 * (0.5 * sq2 * std::erf(1. / sq1) - (1. / sq1) * std::exp(-1. / b));
    else
      M = 0.5 * a * b * b * (1. - (1. + 1. / b) * std::exp(-1. / b));
  } else {
    return fail(NLM_ERR_INVALID, "unknown influence function type");
  }
  P.irrev = m.irreversible ? 1 : 0;
  P.fsc = m.check_sc_factor;
  if (dim == 2)
    P.invF = std::pow(delta, 3) * M_PI;
  else
    P.invF = std::pow(delta, 4) * 4. * M_PI / 3.;
  if (m.compute_from_classical) {
    double E = m.E, K = m.K, Gc = m.Gc, KIc = m.KIc;
    if (hLT(E, 0.) && hLT(K, 0.)) return fail(NLM_ERR_INVALID, "RNPBond needs E or K");
    if (hLT(Gc, 0.) && hLT(KIc, 0.)) return fail(NLM_ERR_INVALID, "RNPBond needs Gc or KIc");
    const double nu = m.plane_strain ? 0.25 : 1. / 3.;
    if (E > 0.) K = E / (3. * (1. - 2. * nu));
    if (K > 0. && E < 0.) E = K * (3. * (1. - 2. * nu));
    if (Gc > 0.) KIc = std::sqrt(Gc * E);
    if (KIc > 0. && Gc < 0.) Gc = KIc * KIc / E;
    const double lambda = E * nu / ((1. + nu) * (1. - 2. * nu));
    if (dim == 2) {
      P.C = M_PI * Gc / (4. * M);
      P.beta = 4. * lambda / (P.C * M);
    } else {
      P.C = 2. * Gc / (3. * M);
      P.beta = 5. * lambda / (P.C * M);
    }
    Kbulk = K;
  } else {
    P.C = m.bond_params[0];
    P.beta = m.bond_params[1];
    // computeMaterialProperties (rnpBond.cpp:190-211): nu = 0.33, lambda
    // from C and beta, then E and K
    const double nu = 0.33;
    const double lambda = dim == 2 ? P.C * M * P.beta / 4. : P.C * M * P.beta / 5.;
    const double E = lambda * (1. + nu) * (1. - 2. * nu) / nu;
    Kbulk = E / (3. * (1. - 2. * nu));
  }
  P.rbar = std::sqrt(0.5 / P.beta);
  // contact between the nodes of broken bonds (RNPBond ctor, rnpBond.cpp:79-88)
  P.contact = m.apply_contact ? 1 : 0;
  P.contact_kn = m.apply_contact ? Kbulk * 18. / (M_PI * std::pow(delta, 5)) : 0.;
  if (!(P.C > 0.) || !(P.beta > 0.)) return fail(NLM_ERR_INVALID, "RNPBond constants not positive");
  return NLM_OK;
}

int launch_step(nlm_fd *h, const StepArgs &a0) {
  StepArgs a = a0;
  if (a.i1 == 0) a.i1 = h->n;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (h->timing && !h->capturing) {
    while (h->ev_used + 2 > h->ev_pool.size()) {
      cudaEvent_t e;
      NLM_CUDA(cudaEventCreate(&e));
      h->ev_pool.push_back(e);
    }
    e0 = h->ev_pool[h->ev_used++];
    e1 = h->ev_pool[h->ev_used++];
    NLM_CUDA(cudaEventRecord(e0, h->stream));
  }
  cudaError_t e;
  const bool fp32 = h->precision == NLM_PREC_FP32C;
  if (h->material == NLM_MAT_RNP_BOND)
    e = fp32 ? launch_rnp_step_fp32(h->P, h->D, h->T, a, h->decomp, h->stream)
             : launch_rnp_step_fp64(h->P, h->D, h->T, a, h->decomp, h->stream);
  else
    e = fp32 ? launch_es_step_fp32(h->P, h->D, h->T, a, h->decomp, h->stream)
             : launch_es_step_fp64(h->P, h->D, h->T, a, h->decomp, h->stream);
  if (e != cudaSuccess) return cuda_fail(e, "step kernel launch");
  if (h->timing && !h->capturing) {
    NLM_CUDA(cudaEventRecord(e1, h->stream));
    h->launches++;
  }
  return NLM_OK;
}

// Tile store of NLM_DECOMP_TILE (FP32C, 2-D): tile t = internal nodes
// [256 t, 256 t + 256); its halo = the nodes outside the tile its rows
// reach, ascending.  Each bond stores its neighbour's index in the tile's
// staged list (tile nodes 0..255, halo from 256), in the sliced layout of
// sell_cols; padding entries point at the row's own node.  If some tile needs
// more than kTileMaxLocal staged nodes the store is not built.  The 2-D
// RNPBond store (max_local == kTileMaxLocal) also gets the byte-offset copy
// tile_boff (16 x index).
// What a tile store is built from (one model or a batch's combined layout).
struct TileInputs {
  int64_t n, nnz, nslices, sell_entries;
  const int *cols_dev;                 // internal column ids, CSR order
  const int64_t *sell_ptr_dev;         // sliced-store offsets
  const std::vector<int64_t> *rowptr;  // host CSR offsets
  const std::vector<int> *perm;        // internal -> caller id (for tile_need), or null
  int max_local;                       // largest staged list allowed
};

template <class H>
int build_tile_store(H *h, const TileInputs &in, bool &ok, std::vector<int> *need_out) {
  const int64_t n = in.n, nt = (n + kTileNodes - 1) / kTileNodes;
  const int max_local = in.max_local;
  ok = false;
  std::vector<int> cols(in.nnz);
  std::vector<int64_t> sptr(in.nslices + 1);
  NLM_CUDA(cudaMemcpyAsync(cols.data(), in.cols_dev, sizeof(int) * in.nnz, cudaMemcpyDeviceToHost,
                           h->stream));
  NLM_CUDA(cudaMemcpyAsync(sptr.data(), in.sell_ptr_dev, sizeof(int64_t) * (in.nslices + 1),
                           cudaMemcpyDeviceToHost, h->stream));
  NLM_CUDA(cudaStreamSynchronize(h->stream));
  const std::vector<int64_t> &rp = *in.rowptr;
  std::vector<std::vector<int>> halo(nt);
  const bool boff_too = max_local == kTileMaxLocal;
  std::vector<uint16_t> lidx(in.sell_entries + 4, 0);
  std::vector<uint16_t> boff(boff_too ? in.sell_entries + 4 : 0, 0);
  std::vector<int> too_big(1, 0);
  std::vector<int> need(nt, -1);
  unsigned nthr = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  auto work = [&](unsigned w) {
    for (int64_t t = w; t < nt; t += nthr) {
      const int64_t a = t * kTileNodes, b = std::min(n, a + kTileNodes);
      std::vector<int> &hl = halo[t];
      for (int64_t q = rp[a]; q < rp[b]; q++)
        if (cols[q] < a || cols[q] >= b) hl.push_back(cols[q]);
      std::sort(hl.begin(), hl.end());
      hl.erase(std::unique(hl.begin(), hl.end()), hl.end());
      if (kTileNodes + (int64_t)hl.size() > max_local) {
        too_big[0] = 1;
        continue;
      }
      if (in.perm) {
        int m = -1;
        for (int64_t i = a; i < b; i++) m = std::max(m, (*in.perm)[i]);
        for (int j : hl) m = std::max(m, (*in.perm)[j]);
        need[t] = m;
      }
      for (int64_t i = a; i < b; i++) {
        const int64_t base = sptr[i >> 5] + 4 * (i & 31);
        const int64_t len = rp[i + 1] - rp[i];
        const int64_t wdt = (sptr[(i >> 5) + 1] - sptr[i >> 5]) / 32;
        for (int64_t k = 0; k < wdt; k++) {
          int loc = (int)(i - a);
          if (k < len) {
            const int j = cols[rp[i] + k];
            loc = (j >= a && j < b) ? (int)(j - a)
                                    : kTileNodes + (int)(std::lower_bound(hl.begin(), hl.end(), j) -
                                                         hl.begin());
          }
          lidx[base + (k >> 2) * 128 + (k & 3)] = (uint16_t)loc;
          if (boff_too) boff[base + (k >> 2) * 128 + (k & 3)] = (uint16_t)(16 * loc);
        }
      }
    }
  };
  std::vector<std::thread> pool;
  for (unsigned w = 0; w < nthr; w++) pool.emplace_back(work, w);
  for (auto &th : pool) th.join();
  if (too_big[0]) return NLM_OK;
  // id block of a tile: its 8 slices, contiguous in the sliced layout
  int64_t ids_max = 0;
  for (int64_t t = 0; t < nt; t++) {
    const int64_t s0 = 8 * t, s1 = std::min<int64_t>(8 * t + 8, in.nslices);
    ids_max = std::max(ids_max, 2 * (sptr[s1] - sptr[s0]));
  }
  if (boff_too && ids_max > kTileIdsMaxBytes) return NLM_OK;
  std::vector<int> hptr(nt + 1, 0);
  size_t nmax = 0;
  for (int64_t t = 0; t < nt; t++) {
    hptr[t + 1] = hptr[t] + (int)halo[t].size();
    nmax = std::max(nmax, halo[t].size());
  }
  std::vector<int> hall(std::max(1, hptr[nt]));
  for (int64_t t = 0; t < nt; t++) std::copy(halo[t].begin(), halo[t].end(), hall.begin() + hptr[t]);
  uint16_t *d_l = nullptr;
  int *d_hp = nullptr, *d_h = nullptr;
  NLM_CUDA(h->alloc(&d_l, lidx.size()));
  NLM_CUDA(h->alloc(&d_hp, hptr.size()));
  NLM_CUDA(h->alloc(&d_h, hall.size()));
  NLM_CUDA(cudaMemcpyAsync(d_l, lidx.data(), sizeof(uint16_t) * lidx.size(), cudaMemcpyHostToDevice, h->stream));
  NLM_CUDA(cudaMemcpyAsync(d_hp, hptr.data(), sizeof(int) * hptr.size(), cudaMemcpyHostToDevice, h->stream));
  NLM_CUDA(cudaMemcpyAsync(d_h, hall.data(), sizeof(int) * hall.size(), cudaMemcpyHostToDevice, h->stream));
  uint16_t *d_b = nullptr;
  if (boff_too) {
    NLM_CUDA(h->alloc(&d_b, boff.size()));
    NLM_CUDA(cudaMemcpyAsync(d_b, boff.data(), sizeof(uint16_t) * boff.size(),
                             cudaMemcpyHostToDevice, h->stream));
  }
  NLM_CUDA(cudaStreamSynchronize(h->stream));
  h->D.tile_lidx = d_l;
  h->D.tile_boff = d_b;
  h->D.tile_ids_bytes = (int)ids_max;
  h->D.tile_hptr = d_hp;
  h->D.tile_halo = d_h;
  h->D.tile_nmax = kTileNodes + (int)nmax;
  ok = true;
  if (need_out) *need_out = std::move(need);
  return NLM_OK;
}

int build_tiles(nlm_fd *h, const int64_t *sell_ptr_dev, int max_local) {
  TileInputs in{h->n, h->nnz, h->nslices, h->sell_entries, h->D.cols, sell_ptr_dev,
                &h->rowptr, &h->perm, max_local};
  return build_tile_store(h, in, h->tile_ok, &h->tile_need);
}

// Work-decomposition autotuner: time each candidate step kernel on scratch
// copies of the arrays a step writes and keep the fastest.
int autotune(nlm_fd *h) {
  const int S = h->S;
  const int64_t n = h->n;
  cudaStream_t s = h->stream;
  DevPtrs D = h->D;
  float4 *sv0 = nullptr, *sv1 = nullptr;
  float *sf = nullptr;
  uint32_t *sb = nullptr;
  const size_t nb = (size_t)h->P.nwords * h->P.npad;
  cudaError_t e = cudaMalloc(&sv0, sizeof(float4) * (S / 2) * n);
  if (e == cudaSuccess) e = cudaMalloc(&sv1, sizeof(float4) * (S / 2) * n);
  if (e == cudaSuccess) e = cudaMalloc(&sf, sizeof(float) * S * n);
  if (e == cudaSuccess) e = cudaMalloc(&sb, sizeof(uint32_t) * nb);
  auto cleanup = [&]() { cudaFree(sv0); cudaFree(sv1); cudaFree(sf); cudaFree(sb); };
  if (e != cudaSuccess) {
    cleanup();
    return cuda_fail(e, "autotune scratch");
  }
  cudaMemcpyAsync(sv0, D.v32[0], sizeof(float4) * (S / 2) * n, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(sv1, D.v32[0], sizeof(float4) * (S / 2) * n, cudaMemcpyDeviceToDevice, s);
  cudaMemsetAsync(sf, 0, sizeof(float) * S * n, s);
  cudaMemcpyAsync(sb, D.bits, sizeof(uint32_t) * nb, cudaMemcpyDeviceToDevice, s);
  D.v32[0] = sv0;
  D.v32[1] = sv1;
  D.f32 = sf;
  D.bits = sb;
  const bool rnp = h->material == NLM_MAT_RNP_BOND;
  std::vector<int> cands = {NLM_DECOMP_THREAD};
  if (rnp) {
    cands.push_back(NLM_DECOMP_THREAD1);
    cands.push_back(NLM_DECOMP_WARP);
  }
  if (h->tile_ok) {
    if (rnp) cands.push_back(NLM_DECOMP_TILE);
    cands.push_back(NLM_DECOMP_TILE_LOCAL);
  }
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  float best = 1e30f;
  int pick = NLM_DECOMP_THREAD;
  StepArgs sa{0, false, h->time, h->time + h->dt, nullptr, 0, h->n};
  for (int c : cands) {
    auto launch = [&]() {
      return rnp ? launch_rnp_step_fp32(h->P, D, h->T, sa, c, s)
                 : launch_es_step_fp32(h->P, D, h->T, sa, c, s);
    };
    for (int w = 0; w < 2; w++) e = launch();
    cudaEventRecord(a, s);
    for (int r = 0; r < 5; r++) e = launch();
    cudaEventRecord(b, s);
    if (e == cudaSuccess) e = cudaEventSynchronize(b);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
    if (e != cudaSuccess) break;
    if (ms < best) {
      best = ms;
      pick = c;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaStreamSynchronize(s);
  cleanup();
  if (e != cudaSuccess) return cuda_fail(e, "autotune");
  h->decomp = pick;
  return NLM_OK;
}

int apply_fbc(nlm_fd *h, double t) {
  if (h->n_fbc_nodes == 0) return NLM_OK;
  k_fbc_apply<<<nblk(h->n_fbc_nodes, 128), 128, 0, h->stream>>>(
      h->n_fbc_nodes, h->S, h->fbc_nodes, h->fbc_iptr, h->fbc_items, h->FT, t,
      const_cast<double *>(h->D.fext));
  NLM_CUDA(cudaGetLastError());
  return NLM_OK;
}

int apply_bc(nlm_fd *h, double t) {
  if (h->n_bc_nodes == 0) return NLM_OK;
  const bool fp32 = h->precision == NLM_PREC_FP32C;
  k_bc_apply<<<nblk(h->n_bc_nodes, 128), 128, 0, h->stream>>>(
      h->n_bc_nodes, h->S, h->dim, h->bc_nodes, h->D.bcref, h->D.bce, h->D.flags, h->T, t,
      fp32 ? nullptr : h->D.u64[h->cur], fp32 ? h->D.u32[h->cur] : nullptr,
      fp32 ? nullptr : h->D.v[h->vidx()], fp32 ? h->D.v32[h->vidx()] : nullptr);
  NLM_CUDA(cudaGetLastError());
  return NLM_OK;
}

// Capture graph_steps consecutive steps starting from ping index c0.
int capture_graph(nlm_fd *h, int c0) {
  cudaGraph_t g = nullptr;
  h->capturing = true;
  cudaError_t e = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) {
    h->capturing = false;
    return cuda_fail(e, "cudaStreamBeginCapture");
  }
  int c = c0, rc = NLM_OK;
  for (int k = 0; k < h->graph_steps && rc == NLM_OK; k++) {
    c = 1 - c;
    if (h->n_fbc_nodes > 0) {
      // FLoading::apply at the step's time, read from the time array
      k_fbc_apply<<<nblk(h->n_fbc_nodes, 128), 128, 0, h->stream>>>(
          h->n_fbc_nodes, h->S, h->fbc_nodes, h->fbc_iptr, h->fbc_items, h->FT, 0.,
          const_cast<double *>(h->D.fext), h->d_times + k);
      const cudaError_t ef = cudaGetLastError();
      if (ef != cudaSuccess) rc = cuda_fail(ef, "force-load kernel");
    }
    StepArgs a{c, false, 0., 0., h->d_times + k, 0, h->n};
    if (rc == NLM_OK) rc = launch_step(h, a);
  }
  e = cudaStreamEndCapture(h->stream, &g);
  h->capturing = false;
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
  e = cudaGraphInstantiate(&h->gexec[c0], g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
  return NLM_OK;
}

// Fracture::addCrack (fracture.cpp:45-70) for the step that ended at h->time:
// the first timed crack not yet cut whose activation time is definitely less
// than that time is cut into the bond state; one crack per call.  The
// reference calls it after the step's output (fDModel.cpp:352-373); here it
// runs just before the next step's launch, which is the same point for the
// dynamics and leaves the state read between run calls equal to the one the
// reference's output of that step sees.
int add_crack(nlm_fd *h) {
  for (size_t c = 0; c < h->timed_cracks.size(); c++) {
    if (h->cracks_on >> c & 1u) continue;
    if (!dLT(h->timed_cracks[c].activation_time, h->time)) continue;
    NLM_CUDA(apply_precrack(h->n, h->S, h->D.pos64, h->D.rowptr, h->D.cols, h->timed_cracks[c],
                            h->P.npad, h->D.bits, h->stream));
    h->cracks_on |= 1u << c;
    return NLM_OK;
  }
  return NLM_OK;
}

// True if a timed crack would be cut before one of the next nsteps steps
// (checked at the times h->time, h->time + dt, ..., accumulated as in do_run).
bool crack_due(const nlm_fd *h, int64_t nsteps) {
  if ((uint64_t)h->cracks_on + 1 == (1ull << h->timed_cracks.size())) return false;
  double t = h->time;
  for (int64_t k = 1; k < nsteps; k++) t = t + h->dt;
  for (size_t c = 0; c < h->timed_cracks.size(); c++)
    if (!(h->cracks_on >> c & 1u) && dLT(h->timed_cracks[c].activation_time, t)) return true;
  return false;
}

int single_steps(nlm_fd *h, int64_t nsteps) {
  for (int64_t s = 0; s < nsteps; s++) {
    int rc;
    if (!h->timed_cracks.empty() && h->step > 0 && (rc = add_crack(h))) return rc;
    const double tm = h->time + h->dt;
    h->cur = 1 - h->cur;
    if ((rc = apply_fbc(h, tm))) return rc;
    StepArgs a{h->cur, false, tm, tm + h->dt, nullptr, 0, h->n};
    if ((rc = launch_step(h, a))) return rc;
    h->time = tm;
    h->step++;
  }
  return NLM_OK;
}

int do_run(nlm_fd *h, int64_t nsteps) {
  if (!h->started) {
    int rc = apply_bc(h, h->time);
    if (rc) return rc;
    if ((rc = apply_fbc(h, h->time))) return rc;
    StepArgs a{h->cur, true, h->time, h->time + h->dt, nullptr, 0, h->n};
    if ((rc = launch_step(h, a))) return rc;
    h->started = true;
  }
  const int G = h->graph_steps;
  while (G > 0 && nsteps >= G) {
    if (!h->timed_cracks.empty() && crack_due(h, G)) {
      // a crack is cut within this chunk: its steps run one by one
      int rc = single_steps(h, G);
      if (rc) return rc;
      nsteps -= G;
      continue;
    }
    if (!h->gexec[h->cur]) {
      int rc = capture_graph(h, h->cur);
      if (rc) return rc;
    }
    // step times of the chunk, accumulated as the reference does
    NLM_CUDA(cudaEventSynchronize(h->ev_times));
    double t = h->time;
    for (int k = 0; k <= G; k++) {
      t = t + h->dt;
      h->h_times[k] = t;
    }
    NLM_CUDA(cudaMemcpyAsync(h->d_times, h->h_times, sizeof(double) * (G + 1),
                             cudaMemcpyHostToDevice, h->stream));
    NLM_CUDA(cudaEventRecord(h->ev_times, h->stream));
    NLM_CUDA(cudaGraphLaunch(h->gexec[h->cur], h->stream));
    h->time = h->h_times[G - 1];
    h->step += G;
    nsteps -= G;
  }
  return single_steps(h, nsteps);
}

}  // namespace

// ---- C ABI ---------------------------------------------------------------
extern "C" {

const char *nlm_last_error(void) { return g_err.c_str(); }
int nlm_abi_version(void) { return NLM_ABI_VERSION; }

int nlm_device_count(int *count) {
  if (!count) return fail(NLM_ERR_INVALID, "null count");
  int c = 0;
  cudaError_t e = cudaGetDeviceCount(&c);
  if (e != cudaSuccess) {
    cudaGetLastError();
    c = 0;
  }
  *count = c;
  return NLM_OK;
}

int nlm_set_device(int device) {
  NLM_CUDA(cudaSetDevice(device));
  return NLM_OK;
}

int nlm_neighbor_search(int dim, int64_t n, const double *x, double horizon, int64_t *rowptr,
                        int32_t *cols) {
  if (n < 0 || (n > 0 && !x) || !rowptr || dim < 1 || dim > 3 || !(horizon > 0.))
    return fail(NLM_ERR_INVALID, "nlm_neighbor_search: bad arguments");
  if (n > INT32_MAX - 1) return fail(NLM_ERR_INVALID, "too many nodes");
  if (!finite_all(x, 3 * n)) return fail(NLM_ERR_NONFINITE, "non-finite coordinate");
  cudaStream_t s;
  NLM_CUDA(cudaStreamCreate(&s));
  double *dx = nullptr;
  NeighborBuild nb;
  std::string why;
  auto cleanup = [&]() {
    cudaFree(dx); cudaFree(nb.perm); cudaFree(nb.pos); cudaFree(nb.rowptr); cudaFree(nb.cols);
    cudaStreamDestroy(s);
  };
  cudaError_t e = cudaMalloc(&dx, sizeof(double) * 3 * (n + 1));
  if (e == cudaSuccess) e = cudaMemcpyAsync(dx, x, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s);
  const Grid g = make_grid(dim, n, x, horizon);
  if (e == cudaSuccess) e = build_neighbors(nb, dim, n, dx, g, 4, s, why);
  if (e != cudaSuccess) {
    int rc = why.empty() ? cuda_fail(e, "neighbour search") : fail(NLM_ERR_INVALID, why);
    cleanup();
    return rc;
  }
  std::vector<int> perm(n);
  std::vector<int64_t> rp(n + 1);
  std::vector<int> cc(nb.nnz);
  e = cudaMemcpy(perm.data(), nb.perm, sizeof(int) * n, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(rp.data(), nb.rowptr, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && nb.nnz) e = cudaMemcpy(cc.data(), nb.cols, sizeof(int) * nb.nnz, cudaMemcpyDeviceToHost);
  cleanup();
  if (e != cudaSuccess) return cuda_fail(e, "neighbour download");
  std::vector<int64_t> inv(n);
  for (int64_t i = 0; i < n; i++) inv[perm[i]] = i;
  rowptr[0] = 0;
  for (int64_t o = 0; o < n; o++) rowptr[o + 1] = rowptr[o] + (rp[inv[o] + 1] - rp[inv[o]]);
  if (cols)
    for (int64_t o = 0; o < n; o++) {
      const int64_t s0 = rp[inv[o]], len = rp[inv[o] + 1] - s0;
      for (int64_t k = 0; k < len; k++) cols[rowptr[o] + k] = perm[cc[s0 + k]];
    }
  return NLM_OK;
}

int nlm_fd_create(const nlm_fd_desc *d, nlm_fd **out) {
  if (!d || !out) return fail(NLM_ERR_INVALID, "null argument");
  *out = nullptr;
  if (d->dim != 2 && d->dim != 3)
    return fail(NLM_ERR_UNSUPPORTED, "explicit model supports dim 2 and 3");
  if (d->n_nodes <= 0 || !d->x || !d->volume) return fail(NLM_ERR_INVALID, "empty mesh");
  if (d->n_nodes > INT32_MAX - 64) return fail(NLM_ERR_INVALID, "too many nodes for one handle");
  if (!(d->horizon > 0.) || !(d->mesh_size > 0.) || !(d->dt > 0.))
    return fail(NLM_ERR_INVALID, "horizon, mesh size and dt must be positive");
  if (!(d->material.density > 0.)) return fail(NLM_ERR_INVALID, "density must be positive");
  if (d->n_ubc < 0 || d->n_ubc > kMaxBCSets || d->n_fbc < 0 || d->n_fbc > kMaxBCSets)
    return fail(NLM_ERR_INVALID, "too many BC sets");
  if ((d->n_ubc && !d->ubc) || (d->n_fbc && !d->fbc) || (d->n_cracks && !d->cracks))
    return fail(NLM_ERR_INVALID, "null BC / crack array");
  if (int rc0 = check_nofail_regions(*d)) return rc0;
  if (int rc0 = check_bc_functions(*d)) return rc0;
  if (d->precision != NLM_PREC_FP64 && d->precision != NLM_PREC_FP32C)
    return fail(NLM_ERR_INVALID, "unknown precision");
  if (d->scheme != NLM_VELOCITY_VERLET && d->scheme != NLM_CENTRAL_DIFFERENCE)
    return fail(NLM_ERR_INVALID, "unknown scheme");
  if (d->material.kind != NLM_MAT_RNP_BOND && d->material.kind != NLM_MAT_ELASTIC_STATE)
    return fail(NLM_ERR_INVALID, "unknown material");
  const int64_t n = d->n_nodes;
  if (!finite_all(d->x, 3 * n) || !finite_all(d->volume, n))
    return fail(NLM_ERR_NONFINITE, "non-finite coordinate or volume");
  if ((d->u0 && !finite_all(d->u0, 3 * n)) || (d->v0 && !finite_all(d->v0, 3 * n)))
    return fail(NLM_ERR_NONFINITE, "non-finite initial state");
  int dev_count = 0;
  if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0) {
    cudaGetLastError();
    return fail(NLM_ERR_CUDA, "no CUDA device");
  }

  nlm_fd *h = new nlm_fd();
  auto bail = [&](int rc) {
    delete h;
    return rc;
  };
  h->dim = d->dim;
  h->S = d->dim == 2 ? 2 : 4;
  h->n = n;
  h->precision = d->precision;
  h->scheme = d->scheme;
  h->material = d->material.kind;
  h->dt = d->dt;
  StepParams &P = h->P;
  P.n = n;
  P.dim = d->dim;
  P.delta = d->horizon;
  P.h = d->mesh_size;
  P.check_up = d->horizon + 0.5 * d->mesh_size;
  P.check_low = d->horizon - 0.5 * d->mesh_size;
  P.dt = d->dt;
  P.rho = d->material.density;
  P.scheme = d->scheme;
  int rc;
  if (h->material == NLM_MAT_RNP_BOND) {
    if ((rc = rnp_constants(d->material, d->dim, d->horizon, P))) return bail(rc);
    P.contact_rc = 0.9 * d->mesh_size;
  } else {
    const nlm_material &m = d->material;
    if (!(m.K > 0.) || !(m.G > 0.)) return bail(fail(NLM_ERR_INVALID, "ElasticState needs K and G"));
    P.es_K = m.K;
    P.es_mu = m.G;
    P.es_nu = (3 * m.K - 2 * m.G) / (2 * (3 * m.K + m.G));
    P.es_E = m.E;
    P.es_plane_strain = m.plane_strain ? 1 : 0;
    P.es_factor2D = (!m.plane_strain && d->dim == 2) ? (2. * P.es_nu - 1.) / (P.es_nu - 1.) : 1.;
    P.es_sc = m.es_sc;
    P.es_ref_compat = m.es_ref_compat ? 1 : 0;
    P.irrev = 1;
  }
  h->decomp = d->decomposition == NLM_DECOMP_AUTO ? NLM_DECOMP_THREAD : d->decomposition;
  if (h->decomp != NLM_DECOMP_THREAD && h->decomp != NLM_DECOMP_WARP &&
      h->decomp != NLM_DECOMP_THREAD1 && h->decomp != NLM_DECOMP_TILE &&
      h->decomp != NLM_DECOMP_TILE_LOCAL)
    return bail(fail(NLM_ERR_INVALID, "unknown decomposition"));
  // tile store: FP32C 2-D RNPBond (both tile kernels) and FP32C 2-D / 3-D
  // ElasticState (the tile-frame kernels only)
  const bool es_model = d->material.kind == NLM_MAT_ELASTIC_STATE;
  const bool tile_able =
      d->precision == NLM_PREC_FP32C &&
      ((d->material.kind == NLM_MAT_RNP_BOND && d->dim == 2) || (es_model && d->dim >= 2));
  if ((h->decomp == NLM_DECOMP_TILE || h->decomp == NLM_DECOMP_TILE_LOCAL) && !tile_able)
    return bail(fail(NLM_ERR_UNSUPPORTED,
                     "the tile decompositions are for FP32C 2-D RNPBond and 2-D / 3-D "
                     "ElasticState"));
  if (h->decomp == NLM_DECOMP_TILE && es_model)
    return bail(fail(NLM_ERR_UNSUPPORTED, "ElasticState takes NLM_DECOMP_TILE_LOCAL"));
  const bool want_tune = d->decomposition == NLM_DECOMP_AUTO && d->precision == NLM_PREC_FP32C &&
                         (d->material.kind == NLM_MAT_RNP_BOND || es_model);

  cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return bail(cuda_fail(e, "cudaStreamCreate"));
  cudaStream_t s = h->stream;
  const int S = h->S;
#define TRY(call)                                     \
  do {                                                \
    cudaError_t _e = (call);                          \
    if (_e != cudaSuccess) return bail(cuda_fail(_e, #call)); \
  } while (0)

  // ---- neighbours (Morton order) ----
  double *dx = nullptr;
  TRY(h->alloc(&dx, 3 * n));
  TRY(cudaMemcpyAsync(dx, d->x, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s));
  const Grid g = make_grid(d->dim, n, d->x, d->horizon);
  NeighborBuild nb;
  std::string why;
  // FP64 plain keeps the reference's row order (its summation order); the
  // FP32C kernels take rows in internal order so that the k-th neighbours of
  // a warp's nodes sit close together in memory.
  h->rows_by_orig = h->precision == NLM_PREC_FP64;
  e = build_neighbors(nb, d->dim, n, dx, g, S, s, why, h->rows_by_orig);
  for (void *p : {(void *)nb.perm, (void *)nb.pos, (void *)nb.rowptr, (void *)nb.cols})
    if (p) {
      h->allocs.push_back(p);
      h->alloc_sizes.push_back(0);
    }
  if (e != cudaSuccess)
    return bail(why.empty() ? cuda_fail(e, "neighbour build") : fail(NLM_ERR_INVALID, why));
  h->nnz = nb.nnz;
  if (h->nnz > INT32_MAX) return bail(fail(NLM_ERR_INVALID, "too many bonds for one handle"));
  SellStore st;
  e = build_sell(n, nb.rowptr, nb.cols, st, s);
  for (void *p : {(void *)st.ptr, (void *)st.width, (void *)st.cols})
    if (p) {
      h->allocs.push_back(p);
      h->alloc_sizes.push_back(0);
    }
  if (e != cudaSuccess) return bail(cuda_fail(e, "bond store build"));
  h->nslices = st.nslices;
  h->sell_entries = st.entries;
  P.nwords = std::max(1, (st.maxw + 31) / 32);
  P.npad = ((n + 31) / 32) * 32;
  h->perm.resize(n);
  h->rowptr.resize(n + 1);
  TRY(cudaMemcpyAsync(h->perm.data(), nb.perm, sizeof(int) * n, cudaMemcpyDeviceToHost, s));
  TRY(cudaMemcpyAsync(h->rowptr.data(), nb.rowptr, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToHost, s));
  TRY(cudaStreamSynchronize(s));

  DevPtrs &D = h->D;
  D.pos64 = nb.pos;
  D.perm_dev = nb.perm;
  D.rowptr = nb.rowptr;
  D.cols = nb.cols;
  D.sell_ptr = st.ptr;
  D.sell_w = st.width;
  D.sell_cols = st.cols;
  uint32_t *bits = nullptr;
  TRY(h->alloc(&bits, (size_t)P.nwords * P.npad));
  TRY(cudaMemsetAsync(bits, 0, sizeof(uint32_t) * P.nwords * P.npad, s));
  D.bits = bits;
  if (tile_able &&
      (h->decomp == NLM_DECOMP_TILE || h->decomp == NLM_DECOMP_TILE_LOCAL || want_tune)) {
    int rc_t = build_tiles(h, st.ptr, es_model ? kTileMaxLocalES : kTileMaxLocal);
    if (rc_t) return bail(rc_t);
    if ((h->decomp == NLM_DECOMP_TILE || h->decomp == NLM_DECOMP_TILE_LOCAL) && !h->tile_ok)
      return bail(fail(NLM_ERR_UNSUPPORTED, "a tile's halo exceeds the tile store limit"));
  }
  for (int c = 0; c < d->n_cracks; c++) {
    if (d->cracks[c].kind == NLM_CRACK_EDGE && d->dim != 2)
      return bail(fail(NLM_ERR_INVALID, "edge pre-cracks are 2-D only (input.cpp:298-307)"));
    if (d->cracks[c].timed) {
      if (h->timed_cracks.size() >= 32) return bail(fail(NLM_ERR_INVALID, "more than 32 timed cracks"));
      h->timed_cracks.push_back(d->cracks[c]);
      continue;
    }
    TRY(apply_precrack(n, S, nb.pos, nb.rowptr, nb.cols, d->cracks[c], P.npad, bits, s));
  }

  // ---- node flags, loads (host, original order then permuted) ----
  std::vector<uint8_t> fix(n, 0), interior(n, 1);
  std::vector<int> wset(3 * n, -1);
  std::vector<double> wumax(3 * n, 0.);
  for (int sidx = 0; sidx < d->n_ubc; sidx++) {
    const nlm_bc_set &bc = d->ubc[sidx];
    if (bc.time_fn < 0 || bc.time_fn > NLM_TFN_LINEAR_SLOW_FAST)
      return bail(fail(NLM_ERR_INVALID, "unknown BC time function"));
    for (int64_t i = 0; i < n; i++) {
      if (!in_region(bc, d->x + 3 * i, d->dim)) continue;
      const double um = uload_umax(bc, d->x + 3 * i);
      for (int dd = 0; dd < 3; dd++)
        if (bc.dir_mask >> dd & 1) {
          fix[i] |= uint8_t(1 << dd);
          wset[3 * i + dd] = sidx;
          wumax[3 * i + dd] = um;
        }
    }
    h->T.t[sidx].fn = bc.time_fn;
    for (int k = 0; k < 4; k++) h->T.t[sidx].p[k] = bc.time_params[k];
  }
  h->T.nsets = d->n_ubc;
  if (d->no_fail != NLM_NOFAIL_OFF)
    nofail_flags(d->x, n, d->no_fail_tol, d->n_nofail_regions, d->nofail_regions, interior);
  mesh_bbox(d->x, n, h->bbox_lo, h->bbox_hi);
  // force BC items per node, in set order
  std::vector<std::vector<FBCItem>> fitems(n);
  for (int sidx = 0; sidx < d->n_fbc; sidx++) {
    const nlm_bc_set &bc = d->fbc[sidx];
    for (int64_t i = 0; i < n; i++)
      if (in_region(bc, d->x + 3 * i, d->dim))
        fitems[i].push_back(FBCItem{sidx, bc.dir_mask & 7, fload_spatial(bc, d->x + 3 * i, d->mesh_size)});
    h->FT.t[sidx].fn = bc.time_fn;
    for (int k = 0; k < 4; k++) h->FT.t[sidx].p[k] = bc.time_params[k];
  }
  h->FT.nsets = d->n_fbc;

  std::vector<uint8_t> flags(n);
  std::vector<int> bcref(n, -1), bcn, fnodes, fptr(1, 0);
  std::vector<BCEntry> bce;
  std::vector<FBCItem> fits;
  std::vector<double> volp(n);
  bool any_nofail = false;
  for (int64_t i = 0; i < n; i++) {
    const int o = h->perm[i];
    uint8_t f = fix[o];
    if (!interior[o]) {
      f |= FLAG_NOFAIL;
      any_nofail = true;
    }
    if (!fitems[o].empty()) {
      f |= FLAG_FBC;
      fnodes.push_back((int)i);
      for (auto &it : fitems[o]) fits.push_back(it);
      fptr.push_back((int)fits.size());
    }
    if (fix[o]) {
      BCEntry be;
      for (int dd = 0; dd < 3; dd++) {
        be.set[dd] = wset[3 * o + dd];
        be.umax[dd] = wumax[3 * o + dd];
      }
      bcref[i] = (int)bce.size();
      bce.push_back(be);
      bcn.push_back((int)i);
    }
    flags[i] = f;
    volp[i] = d->volume[o];
  }
  P.nofail = any_nofail ? 1 : 0;
  uint8_t *dflags;
  int *dbcref;
  BCEntry *dbce;
  TRY(h->alloc(&dflags, n));
  TRY(h->alloc(&dbcref, n));
  TRY(h->alloc(&dbce, bce.size() + 1));
  TRY(cudaMemcpyAsync(dflags, flags.data(), n, cudaMemcpyHostToDevice, s));
  TRY(cudaMemcpyAsync(dbcref, bcref.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
  if (!bce.empty())
    TRY(cudaMemcpyAsync(dbce, bce.data(), sizeof(BCEntry) * bce.size(), cudaMemcpyHostToDevice, s));
  D.flags = dflags;
  D.bcref = dbcref;
  D.bce = dbce;
  h->n_bc_nodes = (int64_t)bcn.size();
  TRY(h->alloc(&h->bc_nodes, bcn.size() + 1));
  if (!bcn.empty())
    TRY(cudaMemcpyAsync(h->bc_nodes, bcn.data(), sizeof(int) * bcn.size(), cudaMemcpyHostToDevice, s));
  h->n_fbc_nodes = (int64_t)fnodes.size();
  double *fext;
  TRY(h->alloc(&fext, (size_t)S * n));
  TRY(cudaMemsetAsync(fext, 0, sizeof(double) * S * n, s));
  D.fext = fext;
  if (!fnodes.empty()) {
    TRY(h->alloc(&h->fbc_nodes, fnodes.size()));
    TRY(h->alloc(&h->fbc_iptr, fptr.size()));
    TRY(h->alloc(&h->fbc_items, fits.size()));
    TRY(cudaMemcpyAsync(h->fbc_nodes, fnodes.data(), sizeof(int) * fnodes.size(), cudaMemcpyHostToDevice, s));
    TRY(cudaMemcpyAsync(h->fbc_iptr, fptr.data(), sizeof(int) * fptr.size(), cudaMemcpyHostToDevice, s));
    TRY(cudaMemcpyAsync(h->fbc_items, fits.data(), sizeof(FBCItem) * fits.size(), cudaMemcpyHostToDevice, s));
  }
  double *vol64;
  TRY(h->alloc(&vol64, n));
  TRY(cudaMemcpyAsync(vol64, volp.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s));
  D.vol64 = vol64;
  {
    // row lengths (the kernels loop k < len)
    std::vector<uint16_t> rl(n);
    for (int64_t i = 0; i < n; i++) rl[i] = (uint16_t)(h->rowptr[i + 1] - h->rowptr[i]);
    uint16_t *drl;
    TRY(h->alloc(&drl, n));
    TRY(cudaMemcpyAsync(drl, rl.data(), sizeof(uint16_t) * n, cudaMemcpyHostToDevice, s));
    TRY(cudaStreamSynchronize(s));
    D.rowlen = drl;
  }
  P.nw1 = P.nwords == 1 ? 1 : 0;
  // a common nodal volume (uniform grids) lets the FP32C tile kernel take
  // K1 V as a constant instead of staging it per node
  P.vol_uniform = n > 0 ? d->volume[0] : 0.;
  for (int64_t i = 1; i < n && P.vol_uniform > 0.; i++)
    if (d->volume[i] != d->volume[0]) P.vol_uniform = 0.;
  if (h->precision == NLM_PREC_FP32C) {
    double xmax = 0.;
    for (int64_t k = 0; k < 3 * n; k++) xmax = std::max(xmax, std::fabs(d->x[k]));
    double X = 1.;
    while (X < xmax) X *= 2.;
    while (X * 0.5 >= xmax && X > 1e-30) X *= 0.5;
    P.lo_scale = std::ldexp(1.0, 24) / X;
    float4 *pos32;
    uint2 *pos32lo = nullptr;
    TRY(h->alloc(&pos32, (size_t)n));
    if (S == 4) TRY(h->alloc(&pos32lo, (size_t)n));
    k_make_pos32<<<nblk(n, 256), 256, 0, s>>>(n, S, nb.pos, vol64, P.lo_scale, pos32, pos32lo);
    TRY(cudaGetLastError());
    D.pos32 = pos32;
    D.pos32lo = pos32lo;
  }

  // ---- state ----
  TRY(h->alloc(&h->stage, 9 * n));
  TRY(h->alloc(&h->bad_input, 1));
  if (h->precision == NLM_PREC_FP64) {
    TRY(h->alloc(&D.u64[0], (size_t)S * n));
    TRY(h->alloc(&D.u64[1], (size_t)S * n));
    TRY(h->alloc(&D.f64, (size_t)S * n));
    TRY(cudaMemsetAsync(D.f64, 0, sizeof(double) * S * n, s));
  } else {
    TRY(h->alloc(&D.u32[0], (size_t)(S / 2) * n));
    TRY(h->alloc(&D.u32[1], (size_t)(S / 2) * n));
    TRY(h->alloc(&D.f32, (size_t)S * n));
    TRY(cudaMemsetAsync(D.f32, 0, sizeof(float) * S * n, s));
  }
  if (h->precision == NLM_PREC_FP64) {
    TRY(h->alloc(&D.v[0], (size_t)S * n));
    TRY(h->alloc(&D.v[1], (size_t)S * n));
  } else {
    TRY(h->alloc(&D.v32[0], (size_t)(S / 2) * n));
    TRY(h->alloc(&D.v32[1], (size_t)(S / 2) * n));
  }
  if (h->material == NLM_MAT_ELASTIC_STATE) {
    double *mw;
    TRY(h->alloc(&mw, n));
    TRY(launch_es_setup(P, D, mw, s));
    D.mw64 = mw;
    if (h->precision == NLM_PREC_FP64) {
      TRY(h->alloc(&D.theta64, n));
      TRY(cudaMemsetAsync(D.theta64, 0, sizeof(double) * n, s));
    } else {
      TRY(h->alloc(&D.es_ab, n));
      TRY(cudaMemsetAsync(D.es_ab, 0, sizeof(float2) * n, s));
    }
  }
  TRY(h->alloc(&D.err, 1));
  TRY(cudaMemsetAsync(D.err, 0, sizeof(int), s));
  TRY(h->alloc(&h->counter, 1));
  TRY(cudaStreamSynchronize(s));
  h->bytes_per_launch = 0.;
  *out = h;
  rc = nlm_fd_set_state(h, d->u0, d->v0);
  if (rc == NLM_OK && (!d->u0 || !d->v0)) {
    // a NULL initial array means zero
    if (!d->u0) {
      if (h->precision == NLM_PREC_FP64)
        TRY(cudaMemsetAsync(D.u64[0], 0, sizeof(double) * S * n, s));
      else
        TRY(cudaMemsetAsync(D.u32[0], 0, sizeof(float4) * (S / 2) * n, s));
    }
    if (!d->v0) {
      if (h->precision == NLM_PREC_FP64)
        TRY(cudaMemsetAsync(D.v[0], 0, sizeof(double) * S * n, s));
      else
        TRY(cudaMemsetAsync(D.v32[0], 0, sizeof(float4) * (S / 2) * n, s));
    }
    TRY(cudaStreamSynchronize(s));
  }
  if (rc != NLM_OK) {
    *out = nullptr;
    return bail(rc);
  }
  if (want_tune && (rc = autotune(h))) {
    *out = nullptr;
    return bail(rc);
  }
  // algorithmic bytes of one step launch (compulsory traffic model)
  {
    const double per_bond = 4.0 + 0.25;  // int32 column + bond bit read/write
    double per_node;
    if (h->precision == NLM_PREC_FP64)
      per_node = 8.0 * S /*x*/ + 8 /*V*/ + 1 /*flags*/ + 8.0 * S * 2 /*u r,w*/ +
                 8.0 * S * 2 /*v r,w*/ + 8.0 * S * 2 /*f r,w*/;
    else
      per_node = (S == 2 ? 16.0 : 24.0) /*x split + V*/ + 1 /*flags*/ + 2 /*row length*/ +
                 8.0 * S * 2 /*u pair r,w*/ + 8.0 * S * 2 /*v pair r,w*/ + 4.0 * S * 2 /*f r,w*/;
    if (h->material == NLM_MAT_ELASTIC_STATE) per_node += 8.0 * 2;  // theta, m
    h->bytes_per_launch = per_bond * (double)h->nnz + per_node * (double)n;
  }
#undef TRY
  return NLM_OK;
}

int nlm_fd_destroy(nlm_fd *h) {
  delete h;
  return NLM_OK;
}

int nlm_fd_num_bonds(const nlm_fd *h, int64_t *nnz) {
  if (!h || !nnz) return fail(NLM_ERR_INVALID, "null argument");
  *nnz = h->nnz;
  return NLM_OK;
}

int nlm_fd_get_neighbors(nlm_fd *h, int64_t *rowptr, int32_t *cols) {
  if (!h || !rowptr) return fail(NLM_ERR_INVALID, "null argument");
  const int64_t n = h->n;
  std::vector<int64_t> inv(n);
  for (int64_t i = 0; i < n; i++) inv[h->perm[i]] = i;
  rowptr[0] = 0;
  for (int64_t o = 0; o < n; o++) rowptr[o + 1] = rowptr[o] + (h->rowptr[inv[o] + 1] - h->rowptr[inv[o]]);
  if (cols) {
    std::vector<int> cc(h->nnz);
    if (h->nnz)
      NLM_CUDA(cudaMemcpyAsync(cc.data(), h->D.cols, sizeof(int) * h->nnz, cudaMemcpyDeviceToHost, h->stream));
    NLM_CUDA(cudaStreamSynchronize(h->stream));
    for (int64_t o = 0; o < n; o++) {
      const int64_t s0 = h->rowptr[inv[o]], len = h->rowptr[inv[o] + 1] - s0;
      for (int64_t k = 0; k < len; k++) cols[rowptr[o] + k] = h->perm[cc[s0 + k]];
      if (!h->rows_by_orig) std::sort(cols + rowptr[o], cols + rowptr[o] + len);
    }
  }
  return NLM_OK;
}

int nlm_fd_run(nlm_fd *h, int64_t nsteps) {
  if (!h || nsteps < 0) return fail(NLM_ERR_INVALID, "bad arguments");
  return do_run(h, nsteps);
}

int nlm_fd_sync(nlm_fd *h) {
  if (!h) return fail(NLM_ERR_INVALID, "null handle");
  NLM_CUDA(cudaStreamSynchronize(h->stream));
  return NLM_OK;
}

}  // extern "C"

// keep_z: the staging slots of u and v hold the caller's arrays as uploaded
// by the call (nlm_fd_step_host), and their z entries go back unchanged in 2-D.
int get_state_impl(nlm_fd *h, double *u, double *v, double *f, bool keep_z) {
  if (!h) return fail(NLM_ERR_INVALID, "null handle");
  const int64_t n = h->n;
  cudaStream_t s = h->stream;
  const int *P = h->D.perm_dev;
  const unsigned g = nblk(n, 256);
  const bool fp32 = h->precision == NLM_PREC_FP32C;
  // gather each requested field into its own staging slot, copy all out,
  // synchronise once
  double *su = h->stage, *sv = h->stage + 3 * n, *sf = h->stage + 6 * n;
  if (u) {
    if (fp32)
      k_gather_split<<<g, 256, 0, s>>>(n, h->S, P, h->D.u32[h->cur], su, keep_z);
    else
      k_gather_vec<<<g, 256, 0, s>>>(n, h->S, P, h->D.u64[h->cur], su, keep_z);
    NLM_CUDA(cudaGetLastError());
    NLM_CUDA(cudaMemcpyAsync(u, su, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, s));
  }
  if (v) {
    if (fp32)
      k_gather_split<<<g, 256, 0, s>>>(n, h->S, P, h->D.v32[h->vidx()], sv, keep_z);
    else
      k_gather_vec<<<g, 256, 0, s>>>(n, h->S, P, h->D.v[h->vidx()], sv, keep_z);
    NLM_CUDA(cudaGetLastError());
    NLM_CUDA(cudaMemcpyAsync(v, sv, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, s));
  }
  if (f) {
    if (fp32)
      k_gather_f32<<<g, 256, 0, s>>>(n, h->S, P, h->D.f32, sf);
    else
      k_gather_vec<<<g, 256, 0, s>>>(n, h->S, P, h->D.f64, sf);
    NLM_CUDA(cudaGetLastError());
    NLM_CUDA(cudaMemcpyAsync(f, sf, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, s));
  }
  NLM_CUDA(cudaStreamSynchronize(s));
  return NLM_OK;
}

extern "C" {

int nlm_fd_get_state(nlm_fd *h, double *u, double *v, double *f) {
  return get_state_impl(h, u, v, f, false);
}

int nlm_fd_set_state(nlm_fd *h, const double *u, const double *v) {
  if (!h) return fail(NLM_ERR_INVALID, "null handle");
  const int64_t n = h->n;
  if ((u && !finite_all(u, 3 * n)) || (v && !finite_all(v, 3 * n)))
    return fail(NLM_ERR_NONFINITE, "non-finite state");
  cudaStream_t s = h->stream;
  const int *P = h->D.perm_dev;
  const unsigned g = nblk(n, 256);
  if (u) {
    NLM_CUDA(cudaMemcpyAsync(h->stage, u, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s));
    if (h->precision == NLM_PREC_FP32C)
      k_scatter_split<<<g, 256, 0, s>>>(n, h->S, h->dim, P, h->stage, h->D.u32[h->cur]);
    else
      k_scatter_vec<<<g, 256, 0, s>>>(n, h->S, h->dim, P, h->stage, h->D.u64[h->cur]);
    NLM_CUDA(cudaGetLastError());
  }
  if (v) {
    double *sv = h->stage + 3 * n;
    NLM_CUDA(cudaMemcpyAsync(sv, v, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s));
    if (h->precision == NLM_PREC_FP32C)
      k_scatter_split<<<g, 256, 0, s>>>(n, h->S, h->dim, P, sv, h->D.v32[h->vidx()]);
    else
      k_scatter_vec<<<g, 256, 0, s>>>(n, h->S, h->dim, P, sv, h->D.v[h->vidx()]);
    NLM_CUDA(cudaGetLastError());
  }
  NLM_CUDA(cudaStreamSynchronize(s));
  if (h->started && (u || v)) {
    // a new state restarts the force history: redo the step-0 evaluation
    h->started = false;
  }
  return NLM_OK;
}

int nlm_fd_get_time(const nlm_fd *h, double *time, int64_t *step) {
  if (!h) return fail(NLM_ERR_INVALID, "null handle");
  if (time) *time = h->time;
  if (step) *step = h->step;
  return NLM_OK;
}

int nlm_fd_get_bond_state(nlm_fd *h, uint8_t *broken) {
  if (!h || !broken) return fail(NLM_ERR_INVALID, "null argument");
  const int64_t n = h->n;
  std::vector<uint32_t> bits((size_t)h->P.nwords * h->P.npad);
  NLM_CUDA(cudaMemcpyAsync(bits.data(), h->D.bits, sizeof(uint32_t) * bits.size(), cudaMemcpyDeviceToHost, h->stream));
  std::vector<int> cc;
  if (!h->rows_by_orig) {
    cc.resize(h->nnz);
    if (h->nnz)
      NLM_CUDA(cudaMemcpyAsync(cc.data(), h->D.cols, sizeof(int) * h->nnz, cudaMemcpyDeviceToHost, h->stream));
  }
  NLM_CUDA(cudaStreamSynchronize(h->stream));
  std::vector<int64_t> inv(n);
  for (int64_t i = 0; i < n; i++) inv[h->perm[i]] = i;
  int64_t o_off = 0;
  std::vector<std::pair<int, uint8_t>> row;
  for (int64_t o = 0; o < n; o++) {
    const int64_t i = inv[o];
    const int64_t r0 = h->rowptr[i], len = h->rowptr[i + 1] - r0;
    if (h->rows_by_orig) {
      for (int64_t k = 0; k < len; k++)
        broken[o_off + k] = (bits[(size_t)(k >> 5) * h->P.npad + i] >> (k & 31)) & 1u;
    } else {
      // device rows are in internal order: re-sort by original id
      row.resize(len);
      for (int64_t k = 0; k < len; k++)
        row[k] = {h->perm[cc[r0 + k]],
                  (uint8_t)((bits[(size_t)(k >> 5) * h->P.npad + i] >> (k & 31)) & 1u)};
      std::sort(row.begin(), row.end());
      for (int64_t k = 0; k < len; k++) broken[o_off + k] = row[k].second;
    }
    o_off += len;
  }
  return NLM_OK;
}

int nlm_fd_set_bond_state(nlm_fd *h, const uint8_t *broken) {
  if (!h || !broken) return fail(NLM_ERR_INVALID, "null argument");
  const int64_t n = h->n;
  std::vector<uint32_t> bits((size_t)h->P.nwords * h->P.npad, 0u);
  std::vector<int> cc;
  if (!h->rows_by_orig) {
    cc.resize(h->nnz);
    if (h->nnz)
      NLM_CUDA(cudaMemcpyAsync(cc.data(), h->D.cols, sizeof(int) * h->nnz, cudaMemcpyDeviceToHost,
                               h->stream));
    NLM_CUDA(cudaStreamSynchronize(h->stream));
  }
  std::vector<int64_t> inv(n);
  for (int64_t i = 0; i < n; i++) inv[h->perm[i]] = i;
  int64_t o_off = 0;
  std::vector<std::pair<int, int>> row;
  for (int64_t o = 0; o < n; o++) {
    const int64_t i = inv[o];
    const int64_t r0 = h->rowptr[i], len = h->rowptr[i + 1] - r0;
    if (h->rows_by_orig) {
      for (int64_t k = 0; k < len; k++)
        if (broken[o_off + k]) bits[(size_t)(k >> 5) * h->P.npad + i] |= 1u << (k & 31);
    } else {
      // external order is ascending original id; device slot k holds cc[r0 + k]
      row.resize(len);
      for (int64_t k = 0; k < len; k++) row[k] = {h->perm[cc[r0 + k]], (int)k};
      std::sort(row.begin(), row.end());
      for (int64_t e = 0; e < len; e++)
        if (broken[o_off + e]) {
          const int k = row[e].second;
          bits[(size_t)(k >> 5) * h->P.npad + i] |= 1u << (k & 31);
        }
    }
    o_off += len;
  }
  NLM_CUDA(cudaMemcpyAsync(h->D.bits, bits.data(), sizeof(uint32_t) * bits.size(),
                           cudaMemcpyHostToDevice, h->stream));
  NLM_CUDA(cudaStreamSynchronize(h->stream));
  return NLM_OK;
}

namespace {
struct CkptHeader {
  char magic[8];
  int32_t version, dim, precision, material, started;
  uint32_t cracks_on;  // timed cracks already cut (bit c = crack c)
  int64_t n, nnz, step;
  double time, dt;
};
const char kCkptMagic[8] = {'N', 'L', 'M', 'C', 'K', 'P', 'T', 0};
}  // namespace

int nlm_fd_save(nlm_fd *h, const char *path) {
  if (!h || !path) return fail(NLM_ERR_INVALID, "null argument");
  const int64_t n = h->n;
  std::vector<double> st((size_t)9 * n);
  std::vector<uint8_t> b((size_t)h->nnz);
  int rc = nlm_fd_get_state(h, st.data(), st.data() + 3 * n, st.data() + 6 * n);
  if (rc) return rc;
  if ((rc = nlm_fd_get_bond_state(h, b.data()))) return rc;
  CkptHeader hd{};
  std::memcpy(hd.magic, kCkptMagic, 8);
  hd.version = 1;
  hd.dim = h->dim;
  hd.precision = h->precision;
  hd.material = h->material;
  hd.started = h->started ? 1 : 0;
  hd.cracks_on = h->cracks_on;
  hd.n = n;
  hd.nnz = h->nnz;
  hd.step = h->step;
  hd.time = h->time;
  hd.dt = h->dt;
  FILE *fp = std::fopen(path, "wb");
  if (!fp) return fail(NLM_ERR_INVALID, std::string("cannot write ") + path);
  bool ok = std::fwrite(&hd, sizeof(hd), 1, fp) == 1 &&
            std::fwrite(st.data(), sizeof(double), st.size(), fp) == st.size() &&
            std::fwrite(b.data(), 1, b.size(), fp) == b.size();
  ok = (std::fclose(fp) == 0) && ok;
  if (!ok) return fail(NLM_ERR_INVALID, std::string("short write to ") + path);
  return NLM_OK;
}

int nlm_fd_load(nlm_fd *h, const char *path) {
  if (!h || !path) return fail(NLM_ERR_INVALID, "null argument");
  FILE *fp = std::fopen(path, "rb");
  if (!fp) return fail(NLM_ERR_INVALID, std::string("cannot read ") + path);
  CkptHeader hd{};
  const int64_t n = h->n;
  std::vector<double> st((size_t)9 * n);
  std::vector<uint8_t> b((size_t)h->nnz);
  bool ok = std::fread(&hd, sizeof(hd), 1, fp) == 1 && std::memcmp(hd.magic, kCkptMagic, 8) == 0;
  if (ok && (hd.version != 1 || hd.n != n || hd.nnz != h->nnz || hd.dim != h->dim ||
             hd.material != h->material || hd.dt != h->dt ||
             (uint64_t)hd.cracks_on >= (1ull << h->timed_cracks.size()))) {
    std::fclose(fp);
    return fail(NLM_ERR_INVALID,
                "checkpoint does not match this model (n, bonds, dim, material, dt, timed cracks)");
  }
  ok = ok && std::fread(st.data(), sizeof(double), st.size(), fp) == st.size() &&
       std::fread(b.data(), 1, b.size(), fp) == b.size();
  std::fclose(fp);
  if (!ok) return fail(NLM_ERR_INVALID, std::string("not a complete checkpoint: ") + path);
  // everything that can be checked is checked before the handle changes
  if (!finite_all(st.data(), (int64_t)st.size()) || !std::isfinite(hd.time) || hd.step < 0)
    return fail(NLM_ERR_NONFINITE, std::string("checkpoint holds a non-finite state or time: ") +
                                       path);
  // what a later failure puts back
  std::vector<uint8_t> bits0((size_t)h->nnz);
  int rc = nlm_fd_get_bond_state(h, bits0.data());
  if (rc) return rc;
  const double time0 = h->time;
  const int64_t step0 = h->step;
  const uint32_t cracks0 = h->cracks_on;
  const bool started0 = h->started;
  rc = nlm_fd_set_bond_state(h, b.data());
  if (rc == NLM_OK) {
    h->time = hd.time;
    h->step = hd.step;
    h->cracks_on = hd.cracks_on;
    if (!hd.started) {
      h->started = false;
      rc = nlm_fd_set_state(h, st.data(), st.data() + 3 * n);
    } else {
      // a started run: u^m, v^m and f^m as step_host takes them, then the
      // drift to u^{m+1} that the interrupted step had done
      h->started = true;
      rc = nlm_fd_step_host(h, st.data(), st.data() + 3 * n, st.data() + 6 * n, 0);
    }
  }
  if (rc != NLM_OK) {
    const std::string msg = nlm_last_error();
    h->time = time0;
    h->step = step0;
    h->cracks_on = cracks0;
    h->started = started0;
    nlm_fd_set_bond_state(h, bits0.data());
    set_error(msg);
  }
  return rc;
}

int nlm_fd_set_time(nlm_fd *h, double time, int64_t step) {
  if (!h || step < 0 || !std::isfinite(time)) return fail(NLM_ERR_INVALID, "bad arguments");
  if (h->started) return fail(NLM_ERR_STATE, "the run has started");
  h->time = time;
  h->step = step;
  return NLM_OK;
}

int nlm_fd_get_fixity(nlm_fd *h, uint8_t *fixity) {
  if (!h || !fixity) return fail(NLM_ERR_INVALID, "null argument");
  std::vector<uint8_t> fl(h->n);
  if (h->n)
    NLM_CUDA(cudaMemcpyAsync(fl.data(), h->D.flags, h->n, cudaMemcpyDeviceToHost, h->stream));
  NLM_CUDA(cudaStreamSynchronize(h->stream));
  for (int64_t i = 0; i < h->n; i++) fixity[h->perm[i]] = fl[i] & 7u;
  return NLM_OK;
}

int nlm_fd_count_broken(nlm_fd *h, int64_t *count) {
  if (!h || !count) return fail(NLM_ERR_INVALID, "null argument");
  NLM_CUDA(cudaMemsetAsync(h->counter, 0, sizeof(unsigned long long), h->stream));
  k_count_bits<<<nblk(h->n, 256), 256, 0, h->stream>>>(h->n, h->P.nwords, h->P.npad, h->D.bits, h->counter);
  NLM_CUDA(cudaGetLastError());
  unsigned long long c = 0;
  NLM_CUDA(cudaMemcpyAsync(&c, h->counter, sizeof(c), cudaMemcpyDeviceToHost, h->stream));
  NLM_CUDA(cudaStreamSynchronize(h->stream));
  *count = (int64_t)c;
  return NLM_OK;
}

int nlm_fd_damage(nlm_fd *h, float *phi, float *Z) {
  if (!h) return fail(NLM_ERR_INVALID, "null handle");
  const int64_t n = h->n;
  cudaStream_t s = h->stream;
  if (!h->dmg_phi) {
    if (h->alloc(&h->dmg_phi, n) != cudaSuccess || h->alloc(&h->dmg_Z, n) != cudaSuccess)
      return fail(NLM_ERR_OOM, "damage buffers");
  }
  cudaError_t e = launch_damage(h->P, h->D, h->cur, h->precision == NLM_PREC_FP32C,
                                h->material == NLM_MAT_ELASTIC_STATE, h->dmg_phi, h->dmg_Z, s);
  if (e != cudaSuccess) return cuda_fail(e, "damage kernel");
  std::vector<float> a(n), b(n);
  NLM_CUDA(cudaMemcpyAsync(a.data(), h->dmg_phi, sizeof(float) * n, cudaMemcpyDeviceToHost, s));
  NLM_CUDA(cudaMemcpyAsync(b.data(), h->dmg_Z, sizeof(float) * n, cudaMemcpyDeviceToHost, s));
  NLM_CUDA(cudaStreamSynchronize(s));
  for (int64_t i = 0; i < n; i++) {
    if (phi) phi[h->perm[i]] = a[i];
    if (Z) Z[h->perm[i]] = b[i];
  }
  return NLM_OK;
}

int nlm_fd_energies(nlm_fd *h, float *strain, float *work, float *kinetic, float *fracture,
                    double *totals) {
  if (!h) return fail(NLM_ERR_INVALID, "null handle");
  if (h->material != NLM_MAT_RNP_BOND) return fail(NLM_ERR_UNSUPPORTED, "energies are for RNPBond");
  const int64_t n = h->n;
  cudaStream_t s = h->stream;
  if (!h->en_buf) {
    if (h->alloc(&h->en_buf, (size_t)4 * n) != cudaSuccess ||
        h->alloc(&h->en_fext, (size_t)h->S * n) != cudaSuccess)
      return fail(NLM_ERR_OOM, "energy buffers");
  }
  // f_ext at the current time, as computePostProcFields evaluates it
  NLM_CUDA(cudaMemsetAsync(h->en_fext, 0, sizeof(double) * h->S * n, s));
  if (h->n_fbc_nodes > 0) {
    k_fbc_apply<<<nblk(h->n_fbc_nodes, 128), 128, 0, s>>>(h->n_fbc_nodes, h->S, h->fbc_nodes,
                                                          h->fbc_iptr, h->fbc_items, h->FT,
                                                          h->time, h->en_fext);
    NLM_CUDA(cudaGetLastError());
  }
  float *e4 = h->en_buf;
  cudaError_t e = launch_energy(h->P, h->D, h->cur, h->vidx(), h->precision == NLM_PREC_FP32C,
                                h->en_fext, e4, e4 + n, e4 + 2 * n, e4 + 3 * n, s);
  if (e != cudaSuccess) return cuda_fail(e, "energy kernel");
  std::vector<float> a((size_t)4 * n);
  NLM_CUDA(cudaMemcpyAsync(a.data(), e4, sizeof(float) * 4 * n, cudaMemcpyDeviceToHost, s));
  NLM_CUDA(cudaStreamSynchronize(s));
  float *out[4] = {strain, work, kinetic, fracture};
  double tot[4] = {0., 0., 0., 0.};
  for (int q = 0; q < 4; q++)
    for (int64_t i = 0; i < n; i++) {
      const float v = a[(size_t)q * n + i];
      tot[q] += v;
      if (out[q]) out[q][h->perm[i]] = v;
    }
  if (totals)
    for (int q = 0; q < 4; q++) totals[q] = tot[q];
  return NLM_OK;
}

int nlm_fd_reaction_force(nlm_fd *h, double *reaction, double *total, double *sum) {
  if (!h) return fail(NLM_ERR_INVALID, "null handle");
  if (h->material != NLM_MAT_RNP_BOND || h->dim != 2)
    return fail(NLM_ERR_UNSUPPORTED, "the reaction force is for 2-D RNPBond");
  const int64_t n = h->n;
  cudaStream_t s = h->stream;
  if (!h->rf_buf && h->alloc(&h->rf_buf, (size_t)2 * n) != cudaSuccess)
    return fail(NLM_ERR_OOM, "reaction-force buffer");
  cudaError_t e = launch_reaction(h->P, h->D, h->cur, h->precision == NLM_PREC_FP32C,
                                  h->bbox_lo[0], h->bbox_hi[0], h->bbox_hi[1], h->rf_buf, s);
  if (e != cudaSuccess) return cuda_fail(e, "reaction-force kernel");
  std::vector<double> a((size_t)2 * n);
  NLM_CUDA(cudaMemcpyAsync(a.data(), h->rf_buf, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost, s));
  NLM_CUDA(cudaStreamSynchronize(s));
  double tot[3] = {0., 0., 0.};
  for (int64_t i = 0; i < n; i++) {
    const double rx = a[2 * i], ry = a[2 * i + 1];
    const int64_t o = h->perm[i];
    if (reaction) {
      reaction[3 * o] = rx;
      reaction[3 * o + 1] = ry;
      reaction[3 * o + 2] = 0.;
    }
    if (total) total[o] = std::sqrt(rx * rx + ry * ry + 0. * 0.);
    tot[0] += rx;
    tot[1] += ry;
  }
  if (sum)
    for (int c = 0; c < 3; c++) sum[c] = tot[c];
  return NLM_OK;
}

int nlm_fd_decomposition(const nlm_fd *h, int *decomp) {
  if (!h || !decomp) return fail(NLM_ERR_INVALID, "null argument");
  *decomp = h->decomp;
  return NLM_OK;
}

int nlm_fd_set_timing(nlm_fd *h, int enable) {
  if (!h) return fail(NLM_ERR_INVALID, "null handle");
  h->timing = enable != 0;
  return NLM_OK;
}

int nlm_fd_kernel_stats(nlm_fd *h, int reset, double *avg_ms, int64_t *launches,
                        double *bytes_per_launch) {
  if (!h) return fail(NLM_ERR_INVALID, "null handle");
  NLM_CUDA(cudaStreamSynchronize(h->stream));
  double acc = 0.;
  for (size_t k = 0; k + 1 < h->ev_used; k += 2) {
    float ms = 0.f;
    NLM_CUDA(cudaEventElapsedTime(&ms, h->ev_pool[k], h->ev_pool[k + 1]));
    acc += ms;
  }
  const int64_t L = h->launches;
  if (avg_ms) *avg_ms = L ? acc / (double)L : 0.;
  if (launches) *launches = L;
  if (bytes_per_launch) *bytes_per_launch = h->bytes_per_launch;
  if (reset) {
    h->ev_used = 0;
    h->launches = 0;
  }
  return NLM_OK;
}

}  // extern "C"

namespace {

typedef int (*PtrAttrFn)(void *, int, unsigned long long);

// The driver's cuPointerGetAttribute, looked up through the runtime (no link
// dependency on the driver library).
PtrAttrFn ptr_attr_fn() {
  static PtrAttrFn fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuPointerGetAttribute", &f, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PtrAttrFn>(f);
    else
      cudaGetLastError();
  }
  return fn;
}

// True when [p, p + bytes) lies inside one page-locked host allocation that
// the device addresses at the same virtual address, so kernels may read and
// write it in place.
bool in_place_ok(const void *p, size_t bytes) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (a.type != cudaMemoryTypeHost || a.devicePointer != p) return false;
  PtrAttrFn fn = ptr_attr_fn();
  if (!fn) return false;
  unsigned long long start = 0;
  size_t size = 0;
  if (fn(&start, 11 /* CU_POINTER_ATTRIBUTE_RANGE_START_ADDR */, (unsigned long long)p) != 0 ||
      fn(&size, 12 /* CU_POINTER_ATTRIBUTE_RANGE_SIZE */, (unsigned long long)p) != 0)
    return false;
  const unsigned long long q = (unsigned long long)p;
  return size > 0 && q >= start && q + bytes <= start + size;
}

// Caller -> internal node ids, built on first use.
int ensure_iperm(nlm_fd *h) {
  if (h->iperm) return NLM_OK;
  if (h->alloc(&h->iperm, h->n) != cudaSuccess) return fail(NLM_ERR_OOM, "host I/O index");
  k_invert_perm<<<nblk(h->n, 256), 256, 0, h->stream>>>(h->n, h->D.perm_dev, h->iperm);
  NLM_CUDA(cudaGetLastError());
  return NLM_OK;
}

// Banded host step: at least kPipeMinNodes nodes.  Band sizes ramp 1, 2, 4
// units up, stay at 8 units (about kPipeMidBand nodes: a few MB per array
// and copy, where a copy's fixed cost is small) and ramp 4, 2, 1 down, so the
// first bands arrive and the last go out quickly.
constexpr int64_t kPipeMinNodes = 1 << 16;
constexpr int64_t kPipeMidBand = 1 << 18;
constexpr int64_t kPipeLateDiv = 32;

// The banded step covers one FP32C velocity-Verlet step of a 2-D RNPBond
// model on a tile decomposition, with no per-launch timing and no timed
// crack to cut first; other calls take the whole-state path.
bool pipe_usable(const nlm_fd *h, int64_t nsteps) {
  return nsteps == 1 && h->pipe_state >= 0 && h->precision == NLM_PREC_FP32C && h->dim == 2 &&
         h->scheme == NLM_VELOCITY_VERLET && h->material == NLM_MAT_RNP_BOND && h->tile_ok &&
         (h->decomp == NLM_DECOMP_TILE || h->decomp == NLM_DECOMP_TILE_LOCAL) && !h->timing &&
         h->n >= kPipeMinNodes && !h->D.qtab &&
         (h->timed_cracks.empty() || !crack_due(h, 1));
}

// Frees what pipe_setup allocated or created, so a failed set-up leaves the
// handle as it was before.
void pipe_teardown(nlm_fd *h) {
  if (h->pipe_sin) cudaStreamSynchronize(h->pipe_sin);
  if (h->pipe_sout) cudaStreamSynchronize(h->pipe_sout);
  for (auto e : h->pipe_ev) cudaEventDestroy(e);
  h->pipe_ev.clear();
  if (h->pipe_sin) cudaStreamDestroy(h->pipe_sin);
  if (h->pipe_sout) cudaStreamDestroy(h->pipe_sout);
  h->pipe_sin = h->pipe_sout = nullptr;
  h->release(&h->pipe_tiles);
  h->release(&h->pipe_in);
  h->release(&h->pipe_back);
  h->release(&h->pipe_ua);
  h->release(&h->pipe_ub);
  h->release(&h->pipe_v);
  h->release(&h->pipe_f);
  h->release(&h->pipe_bits);
  h->release(&h->pipe_late);
  h->pipe_nbands = 0;
}

// Band schedule and buffers of the banded step.  Tile t can run once every
// band up to the one holding caller node tile_need[t] is on the device: its
// stage is that band.  A node is final after the stage of its tile.  Band b
// goes out after the first stage k >= b by which all but at most
// (its size) / kPipeLateDiv of its nodes are final;
// those late nodes (tiles that straddle a jump of the Morton order, mostly)
// are written into the caller's arrays directly once every band is out.
int pipe_setup(nlm_fd *h) {
  const int64_t n = h->n, nt = (n + kTileNodes - 1) / kTileNodes;
  if ((int64_t)h->tile_need.size() != nt) {
    h->pipe_state = -1;
    return NLM_OK;
  }
  const int64_t unit = kPipeMidBand / 8;
  const int64_t mid = std::max<int64_t>(0, (n - 14 * unit + 4 * unit) / (8 * unit));
  std::vector<int64_t> w = {1, 2, 4};
  for (int64_t k = 0; k < mid; k++) w.push_back(8);
  for (int64_t x : {4, 2, 1}) w.push_back(x);
  int64_t wsum = 0;
  for (int64_t x : w) wsum += x;
  const int K = (int)w.size();
  std::vector<int64_t> bounds(K + 1, 0);
  for (int b = 0, acc = 0; b < K; b++) {
    acc += (int)w[b];
    bounds[b + 1] = b + 1 == K ? n : (int64_t)((double)n * acc / wsum);
  }
  auto band_of = [&](int64_t o) {
    return (int)(std::upper_bound(bounds.begin(), bounds.end(), o) - bounds.begin()) - 1;
  };
  std::vector<int> stage(nt);
  std::vector<int> count(K + 1, 0);
  for (int64_t t = 0; t < nt; t++) {
    stage[t] = std::min(K - 1, band_of(std::max(0, h->tile_need[t])));
    count[stage[t] + 1]++;
  }
  for (int k = 0; k < K; k++) count[k + 1] += count[k];
  h->pipe_toff = count;
  std::vector<int> tiles(std::max<int64_t>(1, nt));
  for (int64_t t = 0; t < nt; t++) tiles[count[stage[t]]++] = (int)t;
  // hist[b K + k]: nodes of band b final after stage k
  std::vector<int64_t> hist((size_t)K * K, 0);
  std::vector<int> cband(n);
  for (int64_t i = 0; i < n; i++) {
    cband[i] = band_of(h->perm[i]);
    hist[(size_t)cband[i] * K + stage[i / kTileNodes]]++;
  }
  std::vector<int> release(K, K - 1);
  for (int b = 0; b < K; b++) {
    const int64_t cap = (bounds[b + 1] - bounds[b]) / kPipeLateDiv;
    int64_t later = 0;
    for (int k = K - 1; k >= b; k--) {
      if (later + hist[(size_t)b * K + k] > cap) {
        release[b] = k;
        break;
      }
      later += hist[(size_t)b * K + k];
      release[b] = k - 1;
    }
    release[b] = std::max(release[b], b);
  }
  h->pipe_out.assign(K, {});
  for (int b = 0; b < K; b++) h->pipe_out[release[b]].push_back(b);
  std::vector<int> late;
  for (int64_t i = 0; i < n; i++)
    if (stage[i / kTileNodes] > release[cband[i]]) late.push_back(h->perm[i]);
  std::sort(late.begin(), late.end());
  h->pipe_nlate = (int64_t)late.size();
  if (int rc = ensure_iperm(h)) return rc;
  const size_t nbits = (size_t)h->P.nwords * h->P.npad;
  if (h->alloc(&h->pipe_tiles, tiles.size()) != cudaSuccess ||
      h->alloc(&h->pipe_in, (size_t)9 * n) != cudaSuccess ||
      h->alloc(&h->pipe_back, (size_t)9 * n) != cudaSuccess ||
      h->alloc(&h->pipe_ua, n) != cudaSuccess || h->alloc(&h->pipe_ub, n) != cudaSuccess ||
      h->alloc(&h->pipe_v, n) != cudaSuccess || h->alloc(&h->pipe_f, n) != cudaSuccess ||
      h->alloc(&h->pipe_bits, nbits) != cudaSuccess ||
      h->alloc(&h->pipe_late, std::max<size_t>(1, late.size())) != cudaSuccess)
    return fail(NLM_ERR_OOM, "banded host step buffers");
  NLM_CUDA(cudaMemcpyAsync(h->pipe_tiles, tiles.data(), sizeof(int) * tiles.size(),
                           cudaMemcpyHostToDevice, h->stream));
  if (!late.empty())
    NLM_CUDA(cudaMemcpyAsync(h->pipe_late, late.data(), sizeof(int) * late.size(),
                             cudaMemcpyHostToDevice, h->stream));
  NLM_CUDA(cudaStreamSynchronize(h->stream));
  NLM_CUDA(cudaStreamCreateWithFlags(&h->pipe_sin, cudaStreamNonBlocking));
  NLM_CUDA(cudaStreamCreateWithFlags(&h->pipe_sout, cudaStreamNonBlocking));
  for (int k = 0; k < 2 * K + 1; k++) {
    cudaEvent_t e;
    NLM_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    h->pipe_ev.push_back(e);
  }
  h->pipe_nbands = K;
  h->pipe_bounds = bounds;
  h->pipe_state = 1;
  return NLM_OK;
}

// One step of nlm_fd_step_host on page-locked arrays, banded: the copy-in of
// later bands, the step of the tiles they release and the copy-out of
// finished bands overlap, so both directions of the host link carry traffic
// at once.  The step writes scratch arrays; they become the state only if
// every input value was finite.  Otherwise the bond bits are put back, the
// caller's arrays are restored from the staged input and the call fails with
// the model unchanged.
int step_host_banded(nlm_fd *h, double *u, double *v, double *f) {
  const int64_t n = h->n;
  const int K = h->pipe_nbands;
  const std::vector<int64_t> &bd = h->pipe_bounds;
  cudaStream_t s = h->stream, si = h->pipe_sin, so = h->pipe_sout;
  const double tm = h->time + h->dt;
  const int c = 1 - h->cur;  // ping index of u at the step's time
  DevPtrs Dp = h->D;
  Dp.u32[c] = h->pipe_ua;
  Dp.u32[1 - c] = h->pipe_ub;
  Dp.v32[0] = h->pipe_v;
  Dp.f32 = reinterpret_cast<float *>(h->pipe_f);
  double *in_u = h->pipe_in, *in_v = in_u + 3 * n, *in_f = in_v + 3 * n;
  double *bk_u = h->pipe_back, *bk_v = bk_u + 3 * n, *bk_f = bk_v + 3 * n;
  double *host[3] = {u, v, f}, *in[3] = {in_u, in_v, in_f}, *bk[3] = {bk_u, bk_v, bk_f};
  const size_t nbits = (size_t)h->P.nwords * h->P.npad;
  // the input stream starts once earlier work on the handle's stream is done
  NLM_CUDA(cudaEventRecord(h->pipe_ev[0], s));
  NLM_CUDA(cudaStreamWaitEvent(si, h->pipe_ev[0], 0));
  // copy-in of band b, issued one band ahead of the stage that needs it
  auto copy_in = [&](int b) -> int {
    const int64_t o0 = bd[b], o1 = bd[b + 1];
    for (int a = 0; a < 3; a++)
      NLM_CUDA(cudaMemcpyAsync(in[a] + 3 * o0, host[a] + 3 * o0, sizeof(double) * 3 * (o1 - o0),
                               cudaMemcpyHostToDevice, si));
    NLM_CUDA(cudaEventRecord(h->pipe_ev[2 * b], si));
    return NLM_OK;
  };
  for (int b = 0; b < std::min(K, 2); b++)
    if (int rc = copy_in(b)) return rc;
  NLM_CUDA(cudaMemsetAsync(h->bad_input, 0, sizeof(int), s));
  NLM_CUDA(cudaMemcpyAsync(h->pipe_bits, h->D.bits, sizeof(uint32_t) * nbits,
                           cudaMemcpyDeviceToDevice, s));
  if (int rc = apply_fbc(h, tm)) return rc;
  for (int k = 0; k < K; k++) {
    const int64_t o0 = bd[k], o1 = bd[k + 1];
    if (k + 2 < K)
      if (int rc = copy_in(k + 2)) return rc;
    NLM_CUDA(cudaStreamWaitEvent(s, h->pipe_ev[2 * k], 0));
    NLM_CUDA(launch_pipe_in32(h->P, Dp, h->T, tm, o0, o1, h->iperm, in_u, in_v, in_f, h->pipe_ua,
                              h->pipe_v, h->pipe_f, h->bad_input, s));
    const int nk = h->pipe_toff[k + 1] - h->pipe_toff[k];
    if (nk > 0) {
      StepArgs a{c, false, tm, tm + h->dt, nullptr, 0, n, h->pipe_tiles + h->pipe_toff[k], nk};
      const cudaError_t e = launch_rnp_step_fp32(h->P, Dp, h->T, a, h->decomp, s);
      if (e != cudaSuccess) return cuda_fail(e, "step kernel launch");
    }
    for (int b : h->pipe_out[k]) {
      const int64_t p0 = bd[b], p1 = bd[b + 1];
      NLM_CUDA(launch_pipe_out32(p0, p1, nullptr, h->iperm, h->pipe_ua, h->pipe_v, h->pipe_f,
                                 in_u, in_v, bk_u, bk_v, bk_f, s));
      NLM_CUDA(cudaEventRecord(h->pipe_ev[2 * b + 1], s));
      NLM_CUDA(cudaStreamWaitEvent(so, h->pipe_ev[2 * b + 1], 0));
      for (int a = 0; a < 3; a++)
        NLM_CUDA(cudaMemcpyAsync(host[a] + 3 * p0, bk[a] + 3 * p0, sizeof(double) * 3 * (p1 - p0),
                                 cudaMemcpyDeviceToHost, so));
    }
  }
  // the late nodes, written into the caller's arrays once every band's copy
  // (which carried their values from before their tiles ran) has landed
  if (h->pipe_nlate > 0) {
    NLM_CUDA(cudaEventRecord(h->pipe_ev[2 * K], so));
    NLM_CUDA(cudaStreamWaitEvent(s, h->pipe_ev[2 * K], 0));
    NLM_CUDA(launch_pipe_out32(0, h->pipe_nlate, h->pipe_late, h->iperm, h->pipe_ua, h->pipe_v,
                               h->pipe_f, in_u, in_v, u, v, f, s));
  }
  NLM_CUDA(launch_pipe_commit32(n, (int64_t)nbits, h->bad_input, h->pipe_ua, h->pipe_ub,
                                h->pipe_v, h->pipe_f, h->D.u32[c], h->D.u32[1 - c], h->D.v32[0],
                                reinterpret_cast<float2 *>(h->D.f32), h->D.bits, h->pipe_bits, s));
  int bad = 0;
  NLM_CUDA(cudaMemcpyAsync(&bad, h->bad_input, sizeof(int), cudaMemcpyDeviceToHost, s));
  NLM_CUDA(cudaStreamSynchronize(s));
  NLM_CUDA(cudaStreamSynchronize(so));
  if (bad) {
    for (int a = 0; a < 3; a++)
      NLM_CUDA(cudaMemcpyAsync(host[a], in[a], sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, s));
    NLM_CUDA(cudaStreamSynchronize(s));
    return fail(NLM_ERR_NONFINITE, "non-finite state");
  }
  h->cur = c;
  h->time = tm;
  h->step++;
  h->host_io = 2;
  return NLM_OK;
}

// nlm_fd_step_host with u, v, f read and written in place by kernels (one
// pass each way over the host link), the state replaced only once the input
// is known to be finite.
int step_host_in_place(nlm_fd *h, double *u, double *v, double *f, int64_t nsteps) {
  const int64_t n = h->n;
  const int S = h->S;
  cudaStream_t s = h->stream;
  const bool fp32 = h->precision == NLM_PREC_FP32C;
  if (int rc = ensure_iperm(h)) return rc;
  if (!h->zstage) {
    if (h->alloc(&h->zstage, (size_t)24 * S * n + 16 * n) != cudaSuccess)
      return fail(NLM_ERR_OOM, "in-place host I/O buffers");
    // padding entries of the staged layouts are never written: zero them once
    NLM_CUDA(cudaMemsetAsync(h->zstage, 0, (size_t)24 * S * n + 16 * n, s));
  }
  const size_t bu = fp32 ? sizeof(float4) * (S / 2) * n : sizeof(double) * S * n;
  const size_t bf = fp32 ? sizeof(float) * S * n : sizeof(double) * S * n;
  char *su = h->zstage, *sv = su + bu, *sf = sv + bu;
  double *zu = reinterpret_cast<double *>(h->zstage + (size_t)24 * S * n), *zv = zu + n;
  const int64_t pairs = (3 * n + 1) / 2;
  const double2 *u2 = reinterpret_cast<const double2 *>(u);
  const double2 *v2 = reinterpret_cast<const double2 *>(v);
  const double2 *f2 = reinterpret_cast<const double2 *>(f);
  NLM_CUDA(cudaMemsetAsync(h->bad_input, 0, sizeof(int), s));
  if (fp32)
    k_host_in<true><<<nblk(pairs, 256), 256, 0, s>>>(n, S, h->dim, h->iperm, u2, v2, f2, su, sv,
                                                     sf, zu, zv, h->bad_input);
  else
    k_host_in<false><<<nblk(pairs, 256), 256, 0, s>>>(n, S, h->dim, h->iperm, u2, v2, f2, su, sv,
                                                      sf, zu, zv, h->bad_input);
  NLM_CUDA(cudaGetLastError());
  int bad = 0;
  NLM_CUDA(cudaMemcpyAsync(&bad, h->bad_input, sizeof(int), cudaMemcpyDeviceToHost, s));
  NLM_CUDA(cudaStreamSynchronize(s));
  if (bad) return fail(NLM_ERR_NONFINITE, "non-finite state");
  void *du = fp32 ? (void *)h->D.u32[h->cur] : (void *)h->D.u64[h->cur];
  void *dv = fp32 ? (void *)h->D.v32[h->vidx()] : (void *)h->D.v[h->vidx()];
  void *df_ = fp32 ? (void *)h->D.f32 : (void *)h->D.f64;
  NLM_CUDA(cudaMemcpyAsync(du, su, bu, cudaMemcpyDeviceToDevice, s));
  NLM_CUDA(cudaMemcpyAsync(dv, sv, bu, cudaMemcpyDeviceToDevice, s));
  NLM_CUDA(cudaMemcpyAsync(df_, sf, bf, cudaMemcpyDeviceToDevice, s));
  cudaError_t e = launch_drift(h->P, h->D, h->T, h->cur, h->time + h->dt, fp32, s);
  if (e != cudaSuccess) return cuda_fail(e, "drift kernel");
  int rc = do_run(h, nsteps);
  if (rc) return rc;
  const void *ou = fp32 ? (const void *)h->D.u32[h->cur] : (const void *)h->D.u64[h->cur];
  const void *ov = fp32 ? (const void *)h->D.v32[h->vidx()] : (const void *)h->D.v[h->vidx()];
  const void *of = fp32 ? (const void *)h->D.f32 : (const void *)h->D.f64;
  double2 *u2o = reinterpret_cast<double2 *>(u), *v2o = reinterpret_cast<double2 *>(v);
  double2 *f2o = reinterpret_cast<double2 *>(f);
  if (fp32)
    k_host_out<true><<<nblk(pairs, 256), 256, 0, s>>>(n, S, h->dim, h->iperm, ou, ov, of, zu, zv,
                                                      u2o, v2o, f2o);
  else
    k_host_out<false><<<nblk(pairs, 256), 256, 0, s>>>(n, S, h->dim, h->iperm, ou, ov, of, zu,
                                                       zv, u2o, v2o, f2o);
  NLM_CUDA(cudaGetLastError());
  NLM_CUDA(cudaStreamSynchronize(s));
  h->host_io = 1;
  return NLM_OK;
}

}  // namespace

extern "C" {

int nlm_fd_set_alloc_limit(nlm_fd *h, int64_t bytes) {
  if (!h) return fail(NLM_ERR_INVALID, "null handle");
  h->alloc_budget = bytes < 0 ? -1 : bytes;
  return NLM_OK;
}

int nlm_fd_host_io(const nlm_fd *h, int *mode) {
  if (!h || !mode) return fail(NLM_ERR_INVALID, "null argument");
  *mode = h->host_io;
  return NLM_OK;
}

int nlm_fd_step_host(nlm_fd *h, double *u, double *v, double *f, int64_t nsteps) {
  if (!h || !u || !v || !f || nsteps < 0) return fail(NLM_ERR_INVALID, "null argument");
  if (!h->started) {
    int rc = nlm_fd_set_state(h, u, v);
    if (rc) return rc;
    if ((rc = do_run(h, nsteps))) return rc;
    return get_state_impl(h, u, v, f, true);
  }
  const int64_t n = h->n;
  const size_t bytes = sizeof(double) * 3 * n;
  // in place: page-locked arrays on 16-byte boundaries holding an even
  // number of doubles (whole 16-byte pairs)
  const bool aligned = ((uintptr_t)u | (uintptr_t)v | (uintptr_t)f) % 16 == 0 && n % 2 == 0;
  if (aligned && in_place_ok(u, bytes) && in_place_ok(v, bytes) && in_place_ok(f, bytes)) {
    if (pipe_usable(h, nsteps)) {
      // if the banded path's buffers cannot be allocated, what it had set up
      // is freed and the in-place path below serves this and every later
      // call, with the same results; any other set-up error is returned
      if (h->pipe_state == 0) {
        const int rc = pipe_setup(h);
        if (rc != NLM_OK) {
          pipe_teardown(h);
          cudaGetLastError();
          if (rc != NLM_ERR_OOM) return rc;
          h->pipe_state = -1;
          set_error("");
        }
      }
      if (h->pipe_state == 1) return step_host_banded(h, u, v, f);
    }
    return step_host_in_place(h, u, v, f, nsteps);
  }
  h->host_io = 0;
  cudaStream_t s = h->stream;
  const int *P = h->D.perm_dev;
  const unsigned g = nblk(n, 256);
  const bool fp32 = h->precision == NLM_PREC_FP32C;
  // upload u, v, f into their staging slots, check them for non-finite
  // values on the device, and only then replace the state
  double *su = h->stage, *sv = h->stage + 3 * n, *sf = h->stage + 6 * n;
  NLM_CUDA(cudaMemsetAsync(h->bad_input, 0, sizeof(int), s));
  NLM_CUDA(cudaMemcpyAsync(su, u, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s));
  NLM_CUDA(cudaMemcpyAsync(sv, v, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s));
  NLM_CUDA(cudaMemcpyAsync(sf, f, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s));
  k_nonfinite<<<nblk(9 * n, 256), 256, 0, s>>>(9 * n, h->stage, h->bad_input);
  NLM_CUDA(cudaGetLastError());
  int bad = 0;
  NLM_CUDA(cudaMemcpyAsync(&bad, h->bad_input, sizeof(int), cudaMemcpyDeviceToHost, s));
  NLM_CUDA(cudaStreamSynchronize(s));
  if (bad) return fail(NLM_ERR_NONFINITE, "non-finite state");
  if (fp32) {
    k_scatter_split<<<g, 256, 0, s>>>(n, h->S, h->dim, P, su, h->D.u32[h->cur]);
    k_scatter_split<<<g, 256, 0, s>>>(n, h->S, h->dim, P, sv, h->D.v32[h->vidx()]);
    k_scatter_f32<<<g, 256, 0, s>>>(n, h->S, h->dim, P, sf, h->D.f32);
  } else {
    k_scatter_vec<<<g, 256, 0, s>>>(n, h->S, h->dim, P, su, h->D.u64[h->cur]);
    k_scatter_vec<<<g, 256, 0, s>>>(n, h->S, h->dim, P, sv, h->D.v[h->vidx()]);
    k_scatter_vec<<<g, 256, 0, s>>>(n, h->S, h->dim, P, sf, h->D.f64);
  }
  NLM_CUDA(cudaGetLastError());
  cudaError_t e = launch_drift(h->P, h->D, h->T, h->cur, h->time + h->dt, fp32, s);
  if (e != cudaSuccess) return cuda_fail(e, "drift kernel");
  int rc = do_run(h, nsteps);
  if (rc) return rc;
  return get_state_impl(h, u, v, f, true);
}

int nlm_fd_set_graph(nlm_fd *h, int steps_per_graph) {
  if (!h || steps_per_graph < 0 || (steps_per_graph % 2) || steps_per_graph == 1)
    return fail(NLM_ERR_INVALID, "steps_per_graph must be 0 or an even number >= 2");
  NLM_CUDA(cudaStreamSynchronize(h->stream));
  for (auto &g : h->gexec)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
  if (h->h_times) {
    cudaFreeHost(h->h_times);
    h->h_times = nullptr;
  }
  h->graph_steps = steps_per_graph;
  if (steps_per_graph > 0) {
    NLM_CUDA(cudaMallocHost(&h->h_times, sizeof(double) * (steps_per_graph + 1)));
    if (h->alloc(&h->d_times, (size_t)steps_per_graph + 1) != cudaSuccess)
      return fail(NLM_ERR_OOM, "graph time buffer");
    if (!h->ev_times) NLM_CUDA(cudaEventCreateWithFlags(&h->ev_times, cudaEventDisableTiming));
    NLM_CUDA(cudaEventRecord(h->ev_times, h->stream));
  }
  return NLM_OK;
}

int nlm_fd_run_timed(nlm_fd *h, int64_t nsteps, double *ms) {
  if (!h || !ms || nsteps < 0) return fail(NLM_ERR_INVALID, "bad arguments");
  cudaEvent_t a, b;
  NLM_CUDA(cudaEventCreate(&a));
  NLM_CUDA(cudaEventCreate(&b));
  cudaEventRecord(a, h->stream);
  int rc = do_run(h, nsteps);
  cudaEventRecord(b, h->stream);
  cudaError_t e = cudaEventSynchronize(b);
  float t = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&t, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (rc) return rc;
  if (e != cudaSuccess) return cuda_fail(e, "run timing");
  *ms = t;
  return NLM_OK;
}

}  // extern "C"

// ===========================================================================
// Batched specimens.
//
// Specimen s occupies internal nodes [off_s, off_s + n_s) with off_s a
// multiple of 32, so every 32-node slice of the bond store belongs to one
// specimen; the gaps are ghost nodes (FLAG_GHOST, no bonds) that the kernels
// skip.  Neighbour lists, pre-cracks and loads are built per specimen with the
// single-model code, so they are identical to those of a separate nlm_fd.
// Specimens are laid out by ascending node count and cut into up to three
// node-count buckets; each bucket is one launch per step with its own
// autotuned decomposition.

struct nlm_batch {
  int nspec = 0, dim = 2, S = 2, scheme = NLM_VELOCITY_VERLET;
  int64_t ntot = 0, nnz = 0;
  double dt = 0., time = 0.;
  int64_t step = 0;
  bool started = false;
  int cur = 0;
  StepParams P{};
  BCTable T{};
  DevPtrs D{};
  cudaStream_t stream = nullptr;
  std::vector<void *> allocs;
  std::vector<int64_t> off, n, bond_off, nbond;  // per specimen, by input id
  std::vector<int> order;                          // layout position -> input id
  std::vector<std::vector<int>> perm;              // per specimen: internal -> original
  std::vector<int64_t> rowptr;                     // combined CSR offsets (host)
  struct Bucket {
    int64_t i0, i1;
    int decomp;
  };
  std::vector<Bucket> buckets;
  bool tile_ok = false;  // tile store over the combined layout (2-D)
  int *bc_nodes = nullptr;
  int64_t n_bc_nodes = 0;
  double *stage = nullptr;
  // graphs
  int graph_steps = 0;
  cudaGraphExec_t gexec[2] = {nullptr, nullptr};
  double *d_times = nullptr, *h_times = nullptr;
  cudaEvent_t ev_times = nullptr;

  template <class Tp>
  cudaError_t alloc(Tp **p, size_t count) {
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, count * sizeof(Tp) + 16);
    if (e == cudaSuccess) {
      allocs.push_back(q);
      *p = static_cast<Tp *>(q);
    }
    return e;
  }
  ~nlm_batch() {
    if (stream) cudaStreamSynchronize(stream);
    for (auto &g : gexec)
      if (g) cudaGraphExecDestroy(g);
    if (h_times) cudaFreeHost(h_times);
    if (ev_times) cudaEventDestroy(ev_times);
    for (void *p : allocs) cudaFree(p);
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace {

int batch_launch(nlm_batch *b, StepArgs a) {
  for (const auto &bk : b->buckets) {
    a.i0 = bk.i0;
    a.i1 = bk.i1;
    cudaError_t e = launch_rnp_step_fp32(b->P, b->D, b->T, a, bk.decomp, b->stream);
    if (e != cudaSuccess) return cuda_fail(e, "batched step launch");
  }
  return NLM_OK;
}

int batch_apply_bc(nlm_batch *b, double t) {
  if (b->n_bc_nodes == 0) return NLM_OK;
  k_bc_apply<<<nblk(b->n_bc_nodes, 128), 128, 0, b->stream>>>(
      b->n_bc_nodes, b->S, b->dim, b->bc_nodes, b->D.bcref, b->D.bce, b->D.flags, b->T, t,
      nullptr, b->D.u32[b->cur], nullptr, b->D.v32[b->scheme == NLM_CENTRAL_DIFFERENCE ? b->cur : 0]);
  NLM_CUDA(cudaGetLastError());
  return NLM_OK;
}

// k_bc_apply reads set tables from its BCTable argument; the batch keeps them
// in device memory (D.bct), so the prologue uses this variant.
__global__ void k_bc_apply_tab(int64_t nb, int S, int dim, const int *nodes, const int *bcref,
                               const BCEntry *bce, const uint8_t *flags, const BCTime *tab,
                               double time, float4 *u32, float4 *v32) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nb) return;
  const int64_t i = nodes[t];
  const BCEntry e = bce[bcref[i]];
  const uint8_t fl = flags[i];
  double uo[3], vo[3];
  ld_split_any(u32, S, i, uo);
  ld_split_any(v32, S, i, vo);
  for (int d = 0; d < dim; d++)
    if ((fl >> d & 1) && e.set[d] >= 0) {
      double du, dv;
      bc_value(tab[e.set[d]], e.umax[d], time, du, dv);
      uo[d] = du;
      vo[d] = dv;
    }
  st_split_any(u32, S, i, uo);
  st_split_any(v32, S, i, vo);
}

int batch_capture(nlm_batch *b, int c0) {
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamBeginCapture");
  int c = c0, rc = NLM_OK;
  for (int k = 0; k < b->graph_steps && rc == NLM_OK; k++) {
    c = 1 - c;
    rc = batch_launch(b, StepArgs{c, false, 0., 0., b->d_times + k, 0, 0});
  }
  e = cudaStreamEndCapture(b->stream, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
  e = cudaGraphInstantiate(&b->gexec[c0], g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
  return NLM_OK;
}

int batch_run(nlm_batch *b, int64_t nsteps) {
  if (!b->started) {
    if (b->n_bc_nodes) {
      k_bc_apply_tab<<<nblk(b->n_bc_nodes, 128), 128, 0, b->stream>>>(
          b->n_bc_nodes, b->S, b->dim, b->bc_nodes, b->D.bcref, b->D.bce, b->D.flags, b->D.bct,
          b->time, b->D.u32[b->cur], b->D.v32[b->scheme == NLM_CENTRAL_DIFFERENCE ? b->cur : 0]);
      NLM_CUDA(cudaGetLastError());
    }
    int rc = batch_launch(b, StepArgs{b->cur, true, b->time, b->time + b->dt, nullptr, 0, 0});
    if (rc) return rc;
    b->started = true;
  }
  const int G = b->graph_steps;
  while (G > 0 && nsteps >= G) {
    if (!b->gexec[b->cur]) {
      int rc = batch_capture(b, b->cur);
      if (rc) return rc;
    }
    NLM_CUDA(cudaEventSynchronize(b->ev_times));
    double t = b->time;
    for (int k = 0; k <= G; k++) {
      t = t + b->dt;
      b->h_times[k] = t;
    }
    NLM_CUDA(cudaMemcpyAsync(b->d_times, b->h_times, sizeof(double) * (G + 1),
                             cudaMemcpyHostToDevice, b->stream));
    NLM_CUDA(cudaEventRecord(b->ev_times, b->stream));
    NLM_CUDA(cudaGraphLaunch(b->gexec[b->cur], b->stream));
    b->time = b->h_times[G - 1];
    b->step += G;
    nsteps -= G;
  }
  for (int64_t k = 0; k < nsteps; k++) {
    const double tm = b->time + b->dt;
    b->cur = 1 - b->cur;
    int rc = batch_launch(b, StepArgs{b->cur, false, tm, tm + b->dt, nullptr, 0, 0});
    if (rc) return rc;
    b->time = tm;
    b->step++;
  }
  return NLM_OK;
}

}  // namespace

extern "C" {

int nlm_batch_create(const nlm_fd_desc *descs, int nspec, nlm_batch **out) {
  if (!descs || !out || nspec < 1) return fail(NLM_ERR_INVALID, "bad arguments");
  *out = nullptr;
  const nlm_fd_desc &d0 = descs[0];
  int64_t total_sets = 0;
  for (int s = 0; s < nspec; s++) {
    const nlm_fd_desc &d = descs[s];
    if (d.dim != d0.dim || (d.dim != 2 && d.dim != 3))
      return fail(NLM_ERR_INVALID, "specimens must share dimension 2 or 3");
    if (d.precision != NLM_PREC_FP32C)
      return fail(NLM_ERR_UNSUPPORTED, "batched specimens run in FP32C precision");
    if (d.material.kind != NLM_MAT_RNP_BOND)
      return fail(NLM_ERR_UNSUPPORTED, "batched specimens are RNPBond");
    if (d.dt != d0.dt || d.scheme != d0.scheme)
      return fail(NLM_ERR_INVALID, "specimens must share dt and scheme");
    if (d.n_fbc) return fail(NLM_ERR_UNSUPPORTED, "Force_BC in a batch");
    if (d.n_nodes <= 0 || !d.x || !d.volume) return fail(NLM_ERR_INVALID, "empty specimen");
    if (!(d.horizon > 0.) || !(d.mesh_size > 0.) || !(d.dt > 0.) || !(d.material.density > 0.))
      return fail(NLM_ERR_INVALID, "horizon, mesh size, dt and density must be positive");
    if (d.n_ubc < 0 || d.n_ubc > kMaxBCSets || (d.n_ubc && !d.ubc) || (d.n_cracks && !d.cracks))
      return fail(NLM_ERR_INVALID, "bad BC / crack arrays");
    if (int rc0 = check_nofail_regions(d)) return rc0;
    if (!finite_all(d.x, 3 * d.n_nodes) || !finite_all(d.volume, d.n_nodes))
      return fail(NLM_ERR_NONFINITE, "non-finite coordinate or volume");
    total_sets += d.n_ubc;
  }
  int dev_count = 0;
  if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0) {
    cudaGetLastError();
    return fail(NLM_ERR_CUDA, "no CUDA device");
  }
  nlm_batch *b = new nlm_batch();
  auto bail = [&](int rc) {
    delete b;
    return rc;
  };
#define BTRY(call)                                              \
  do {                                                          \
    cudaError_t _e = (call);                                    \
    if (_e != cudaSuccess) return bail(cuda_fail(_e, #call));   \
  } while (0)
  b->nspec = nspec;
  b->dim = d0.dim;
  b->S = d0.dim == 2 ? 2 : 4;
  b->scheme = d0.scheme;
  b->dt = d0.dt;
  const int S = b->S;
  BTRY(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  cudaStream_t st = b->stream;
  // layout: ascending node count
  b->order.resize(nspec);
  for (int s = 0; s < nspec; s++) b->order[s] = s;
  std::stable_sort(b->order.begin(), b->order.end(),
                   [&](int a, int c) { return descs[a].n_nodes < descs[c].n_nodes; });
  b->off.assign(nspec, 0);
  b->n.assign(nspec, 0);
  int64_t cursor = 0;
  for (int k = 0; k < nspec; k++) {
    const int s = b->order[k];
    b->off[s] = cursor;
    b->n[s] = descs[s].n_nodes;
    cursor += ((descs[s].n_nodes + 31) / 32) * 32;
  }
  const int64_t N = cursor;
  b->ntot = N;
  if (N > INT32_MAX - 64) return bail(fail(NLM_ERR_INVALID, "too many nodes"));
  // per-specimen neighbour builds, merged into one CSR
  double *pos64;
  int64_t *rowptr;
  BTRY(b->alloc(&pos64, (size_t)S * N));
  BTRY(cudaMemsetAsync(pos64, 0, sizeof(double) * S * N, st));
  BTRY(b->alloc(&rowptr, N + 1));
  std::vector<int64_t> hrow(N + 1, 0);
  std::vector<NeighborBuild> nbs(nspec);
  b->perm.resize(nspec);
  b->bond_off.assign(nspec, 0);
  b->nbond.assign(nspec, 0);
  double xmax = 0.;
  int64_t nnz = 0;
  for (int k = 0; k < nspec; k++) {
    const int s = b->order[k];
    const nlm_fd_desc &d = descs[s];
    double *dx = nullptr;
    cudaError_t e = cudaMalloc(&dx, sizeof(double) * 3 * (d.n_nodes + 1));
    if (e == cudaSuccess) e = cudaMemcpyAsync(dx, d.x, sizeof(double) * 3 * d.n_nodes, cudaMemcpyHostToDevice, st);
    std::string why;
    const Grid g = make_grid(d.dim, d.n_nodes, d.x, d.horizon);
    if (e == cudaSuccess) e = build_neighbors(nbs[s], d.dim, d.n_nodes, dx, g, S, st, why, false);
    cudaFree(dx);
    for (void *q : {(void *)nbs[s].perm, (void *)nbs[s].pos, (void *)nbs[s].rowptr, (void *)nbs[s].cols})
      if (q) b->allocs.push_back(q);
    if (e != cudaSuccess)
      return bail(why.empty() ? cuda_fail(e, "neighbour build") : fail(NLM_ERR_INVALID, why));
    b->perm[s].resize(d.n_nodes);
    std::vector<int64_t> rp(d.n_nodes + 1);
    BTRY(cudaMemcpyAsync(b->perm[s].data(), nbs[s].perm, sizeof(int) * d.n_nodes, cudaMemcpyDeviceToHost, st));
    BTRY(cudaMemcpyAsync(rp.data(), nbs[s].rowptr, sizeof(int64_t) * (d.n_nodes + 1), cudaMemcpyDeviceToHost, st));
    BTRY(cudaStreamSynchronize(st));
    b->bond_off[s] = nnz;
    b->nbond[s] = nbs[s].nnz;
    for (int64_t i = 0; i < d.n_nodes; i++) hrow[b->off[s] + i] = nnz + rp[i];
    const int64_t pad_end = (k + 1 < nspec) ? b->off[b->order[k + 1]] : N;
    for (int64_t i = b->off[s] + d.n_nodes; i <= pad_end && i <= N; i++) hrow[i] = nnz + nbs[s].nnz;
    nnz += nbs[s].nnz;
    BTRY(cudaMemcpyAsync(pos64 + (size_t)S * b->off[s], nbs[s].pos, sizeof(double) * S * d.n_nodes,
                         cudaMemcpyDeviceToDevice, st));
    for (int64_t q = 0; q < 3 * d.n_nodes; q++) xmax = std::max(xmax, std::fabs(d.x[q]));
  }
  hrow[N] = nnz;
  if (nnz > INT32_MAX) return bail(fail(NLM_ERR_INVALID, "too many bonds"));
  b->nnz = nnz;
  b->rowptr = hrow;
  BTRY(cudaMemcpyAsync(rowptr, hrow.data(), sizeof(int64_t) * (N + 1), cudaMemcpyHostToDevice, st));
  int *cols;
  BTRY(b->alloc(&cols, nnz + 1));
  for (int s = 0; s < nspec; s++) {
    if (!b->nbond[s]) continue;
    BTRY(cudaMemcpyAsync(cols + b->bond_off[s], nbs[s].cols, sizeof(int) * b->nbond[s],
                         cudaMemcpyDeviceToDevice, st));
    BTRY(offset_cols(b->nbond[s], cols + b->bond_off[s], (int)b->off[s], st));
  }
  BTRY(cudaStreamSynchronize(st));
  // the per-specimen builds are no longer needed
  for (int s = 0; s < nspec; s++) {
    for (void *q : {(void *)nbs[s].perm, (void *)nbs[s].pos, (void *)nbs[s].rowptr, (void *)nbs[s].cols}) {
      auto it = std::find(b->allocs.begin(), b->allocs.end(), q);
      if (it != b->allocs.end()) {
        cudaFree(q);
        b->allocs.erase(it);
      }
    }
  }
  SellStore ss;
  cudaError_t e = build_sell(N, rowptr, cols, ss, st);
  for (void *q : {(void *)ss.ptr, (void *)ss.width, (void *)ss.cols})
    if (q) b->allocs.push_back(q);
  if (e != cudaSuccess) return bail(cuda_fail(e, "bond store build"));
  StepParams &P = b->P;
  P.n = N;
  P.dim = b->dim;
  P.npad = N;
  P.nwords = std::max(1, (ss.maxw + 31) / 32);
  P.nw1 = P.nwords == 1 ? 1 : 0;
  P.dt = b->dt;
  P.scheme = b->scheme;
  P.irrev = 1;
  double X = 1.;
  while (X < xmax) X *= 2.;
  while (X * 0.5 >= xmax && X > 1e-30) X *= 0.5;
  P.lo_scale = std::ldexp(1.0, 24) / X;
  DevPtrs &D = b->D;
  D.pos64 = pos64;
  D.rowptr = rowptr;
  D.cols = cols;
  D.sell_ptr = ss.ptr;
  D.sell_w = ss.width;
  D.sell_cols = ss.cols;
  // explicit decomposition: every specimen names the same one, used for all
  // buckets; NLM_DECOMP_AUTO (any specimen) autotunes per bucket
  int fixed = descs[0].decomposition;
  for (int s = 1; s < nspec; s++)
    if (descs[s].decomposition != fixed) fixed = NLM_DECOMP_AUTO;
  if (fixed == NLM_DECOMP_TILE)
    return bail(fail(NLM_ERR_UNSUPPORTED, "a batch takes NLM_DECOMP_TILE_LOCAL, not TILE"));
  if (fixed != NLM_DECOMP_AUTO && fixed != NLM_DECOMP_THREAD && fixed != NLM_DECOMP_THREAD1 &&
      fixed != NLM_DECOMP_WARP && fixed != NLM_DECOMP_TILE_LOCAL)
    return bail(fail(NLM_ERR_INVALID, "unknown decomposition"));
  if (b->dim == 2 && (fixed == NLM_DECOMP_AUTO || fixed == NLM_DECOMP_TILE_LOCAL)) {
    TileInputs tin{N, nnz, ss.nslices, ss.entries, cols, ss.ptr, &b->rowptr, nullptr,
                   kTileMaxLocal};
    if (int rc_t = build_tile_store(b, tin, b->tile_ok, nullptr)) return bail(rc_t);
  }
  if (fixed == NLM_DECOMP_TILE_LOCAL && !b->tile_ok)
    return bail(fail(NLM_ERR_UNSUPPORTED,
                     "the tile-frame decomposition is for 2-D batches whose tiles fit the store"));
  uint32_t *bits;
  BTRY(b->alloc(&bits, (size_t)P.nwords * N));
  BTRY(cudaMemsetAsync(bits, 0, sizeof(uint32_t) * P.nwords * N, st));
  D.bits = bits;
  // per-specimen constants, loads, cracks
  std::vector<Params32> qtab(nspec);
  std::vector<BCTime> bct;
  std::vector<int> slice_spec(N / 32, -1);
  std::vector<uint8_t> flags(N, FLAG_GHOST);
  std::vector<int> bcref(N, -1), bcn;
  std::vector<BCEntry> bce;
  std::vector<double> volp(N, 0.);
  std::vector<uint16_t> rl(N, 0);
  bool any_nofail = false;
  double span_min = 1e300;
  for (int s = 0; s < nspec; s++) {
    const nlm_fd_desc &d = descs[s];
    StepParams Ps{};
    Ps.n = d.n_nodes;
    Ps.dim = d.dim;
    Ps.delta = d.horizon;
    Ps.h = d.mesh_size;
    Ps.check_up = d.horizon + 0.5 * d.mesh_size;
    Ps.check_low = d.horizon - 0.5 * d.mesh_size;
    Ps.dt = d.dt;
    Ps.rho = d.material.density;
    Ps.scheme = d.scheme;
    Ps.lo_scale = P.lo_scale;
    int rc = rnp_constants(d.material, d.dim, d.horizon, Ps);
    if (rc) return bail(rc);
    if (Ps.contact) return bail(fail(NLM_ERR_UNSUPPORTED, "contact forces are not batched"));
    qtab[s] = make_p32(Ps);
    // the tile kernel decides per tile (specimens may share one): the
    // smallest span limit of all specimens
    span_min = std::min(span_min, (double)qtab[s].span_max);
    for (int64_t q = b->off[s] / 32; q < (b->off[s] + d.n_nodes + 31) / 32; q++) slice_spec[q] = s;
    for (int c = 0; c < d.n_cracks; c++) {
      if (d.cracks[c].kind == NLM_CRACK_EDGE && d.dim != 2)
        return bail(fail(NLM_ERR_INVALID, "edge pre-cracks are 2-D only"));
      if (d.cracks[c].timed)
        return bail(fail(NLM_ERR_UNSUPPORTED, "the batched model takes pre-cracks only"));
      BTRY(apply_precrack(d.n_nodes, S, pos64, rowptr, cols, d.cracks[c], N, bits, st, b->off[s]));
    }
    const int set0 = (int)bct.size();
    for (int k = 0; k < d.n_ubc; k++) {
      BCTime t;
      t.fn = d.ubc[k].time_fn;
      for (int q = 0; q < 4; q++) t.p[q] = d.ubc[k].time_params[q];
      bct.push_back(t);
    }
    // fixity, winning set per dof, no-fail flags (same rules as nlm_fd_create)
    std::vector<uint8_t> fix(d.n_nodes, 0), interior(d.n_nodes, 1);
    std::vector<int> wset(3 * d.n_nodes, -1);
    std::vector<double> wumax(3 * d.n_nodes, 0.);
    for (int k = 0; k < d.n_ubc; k++)
      for (int64_t i = 0; i < d.n_nodes; i++) {
        if (!in_region(d.ubc[k], d.x + 3 * i, d.dim)) continue;
        const double um = uload_umax(d.ubc[k], d.x + 3 * i);
        for (int dd = 0; dd < 3; dd++)
          if (d.ubc[k].dir_mask >> dd & 1) {
            fix[i] |= uint8_t(1 << dd);
            wset[3 * i + dd] = set0 + k;
            wumax[3 * i + dd] = um;
          }
      }
    if (d.no_fail != NLM_NOFAIL_OFF)
      nofail_flags(d.x, d.n_nodes, d.no_fail_tol, d.n_nofail_regions, d.nofail_regions, interior);
    for (int64_t i = 0; i < d.n_nodes; i++) {
      const int64_t g = b->off[s] + i;
      const int o = b->perm[s][i];
      uint8_t f = fix[o];
      if (!interior[o]) {
        f |= FLAG_NOFAIL;
        any_nofail = true;
      }
      flags[g] = f;
      volp[g] = d.volume[o];
      rl[g] = (uint16_t)(hrow[g + 1] - hrow[g]);
      if (fix[o]) {
        BCEntry be;
        for (int dd = 0; dd < 3; dd++) {
          be.set[dd] = wset[3 * o + dd];
          be.umax[dd] = wumax[3 * o + dd];
        }
        bcref[g] = (int)bce.size();
        bce.push_back(be);
        bcn.push_back((int)g);
      }
    }
  }
  (void)total_sets;
  P.nofail = any_nofail ? 1 : 0;
  Params32 *dq;
  BCTime *dbct;
  int *dss;
  uint8_t *dflags;
  int *dbcref;
  BCEntry *dbce;
  double *vol64;
  uint16_t *drl;
  BTRY(b->alloc(&dq, nspec));
  BTRY(b->alloc(&dbct, bct.size() + 1));
  BTRY(b->alloc(&dss, slice_spec.size() + 1));
  BTRY(b->alloc(&dflags, N));
  BTRY(b->alloc(&dbcref, N));
  BTRY(b->alloc(&dbce, bce.size() + 1));
  BTRY(b->alloc(&vol64, N));
  BTRY(b->alloc(&drl, N));
  BTRY(cudaMemcpyAsync(dq, qtab.data(), sizeof(Params32) * nspec, cudaMemcpyHostToDevice, st));
  if (!bct.empty()) BTRY(cudaMemcpyAsync(dbct, bct.data(), sizeof(BCTime) * bct.size(), cudaMemcpyHostToDevice, st));
  BTRY(cudaMemcpyAsync(dss, slice_spec.data(), sizeof(int) * slice_spec.size(), cudaMemcpyHostToDevice, st));
  BTRY(cudaMemcpyAsync(dflags, flags.data(), N, cudaMemcpyHostToDevice, st));
  BTRY(cudaMemcpyAsync(dbcref, bcref.data(), sizeof(int) * N, cudaMemcpyHostToDevice, st));
  if (!bce.empty()) BTRY(cudaMemcpyAsync(dbce, bce.data(), sizeof(BCEntry) * bce.size(), cudaMemcpyHostToDevice, st));
  BTRY(cudaMemcpyAsync(vol64, volp.data(), sizeof(double) * N, cudaMemcpyHostToDevice, st));
  BTRY(cudaMemcpyAsync(drl, rl.data(), sizeof(uint16_t) * N, cudaMemcpyHostToDevice, st));
  D.qtab = dq;
  P.tile_span_max = nspec > 0 ? span_min : 0.;
  D.bct = dbct;
  D.slice_spec = dss;
  D.flags = dflags;
  D.bcref = dbcref;
  D.bce = dbce;
  D.vol64 = vol64;
  D.rowlen = drl;
  b->n_bc_nodes = (int64_t)bcn.size();
  BTRY(b->alloc(&b->bc_nodes, bcn.size() + 1));
  if (!bcn.empty())
    BTRY(cudaMemcpyAsync(b->bc_nodes, bcn.data(), sizeof(int) * bcn.size(), cudaMemcpyHostToDevice, st));
  float4 *pos32;
  uint2 *pos32lo = nullptr;
  BTRY(b->alloc(&pos32, N));
  if (S == 4) BTRY(b->alloc(&pos32lo, N));
  k_make_pos32<<<nblk(N, 256), 256, 0, st>>>(N, S, pos64, vol64, P.lo_scale, pos32, pos32lo);
  BTRY(cudaGetLastError());
  D.pos32 = pos32;
  D.pos32lo = pos32lo;
  BTRY(b->alloc(&D.u32[0], (size_t)(S / 2) * N));
  BTRY(b->alloc(&D.u32[1], (size_t)(S / 2) * N));
  BTRY(b->alloc(&D.v32[0], (size_t)(S / 2) * N));
  BTRY(b->alloc(&D.v32[1], (size_t)(S / 2) * N));
  BTRY(b->alloc(&D.f32, (size_t)S * N));
  BTRY(b->alloc(&b->stage, 3 * (size_t)N));
  double *fx;
  BTRY(b->alloc(&fx, (size_t)S * N));
  D.fext = fx;
  for (float4 *q : {D.u32[0], D.u32[1], D.v32[0], D.v32[1]})
    BTRY(cudaMemsetAsync(q, 0, sizeof(float4) * (S / 2) * N, st));
  BTRY(cudaMemsetAsync(D.f32, 0, sizeof(float) * S * N, st));
  BTRY(cudaMemsetAsync(fx, 0, sizeof(double) * S * N, st));
  // initial states
  int *dperm;
  BTRY(b->alloc(&dperm, N));
  for (int s = 0; s < nspec; s++) {
    const nlm_fd_desc &d = descs[s];
    if (!d.u0 && !d.v0) continue;
    BTRY(cudaMemcpyAsync(dperm, b->perm[s].data(), sizeof(int) * d.n_nodes, cudaMemcpyHostToDevice, st));
    const unsigned g = nblk(d.n_nodes, 256);
    if (d.u0) {
      BTRY(cudaMemcpyAsync(b->stage, d.u0, sizeof(double) * 3 * d.n_nodes, cudaMemcpyHostToDevice, st));
      k_scatter_split<<<g, 256, 0, st>>>(d.n_nodes, S, d.dim, dperm, b->stage, D.u32[0] + (S / 2) * b->off[s]);
    }
    if (d.v0) {
      BTRY(cudaMemcpyAsync(b->stage, d.v0, sizeof(double) * 3 * d.n_nodes, cudaMemcpyHostToDevice, st));
      k_scatter_split<<<g, 256, 0, st>>>(d.n_nodes, S, d.dim, dperm, b->stage, D.v32[0] + (S / 2) * b->off[s]);
    }
    BTRY(cudaGetLastError());
    BTRY(cudaStreamSynchronize(st));
  }
  // node-count buckets (terciles of the specimen list by size) + autotuning
  const int nb = std::min(3, nspec);
  int64_t prev = 0;
  for (int q = 0; q < nb; q++) {
    const int kend = (int)(((int64_t)(q + 1) * nspec) / nb);
    const int64_t end = kend < nspec ? b->off[b->order[kend]] : N;
    if (end > prev)
      b->buckets.push_back({prev, end, fixed == NLM_DECOMP_AUTO ? NLM_DECOMP_THREAD : fixed});
    prev = end;
  }
  BTRY(cudaStreamSynchronize(st));
  if (fixed == NLM_DECOMP_AUTO) {
    // time each candidate per bucket on scratch velocity / force / bit copies
    DevPtrs Dt = D;
    float4 *sv0 = nullptr;
    float *sf = nullptr;
    uint32_t *sb = nullptr;
    cudaError_t e2 = cudaMalloc(&sv0, sizeof(float4) * (S / 2) * N);
    if (e2 == cudaSuccess) e2 = cudaMalloc(&sf, sizeof(float) * S * N);
    if (e2 == cudaSuccess) e2 = cudaMalloc(&sb, sizeof(uint32_t) * P.nwords * N);
    if (e2 == cudaSuccess) {
      cudaMemcpyAsync(sv0, D.v32[0], sizeof(float4) * (S / 2) * N, cudaMemcpyDeviceToDevice, st);
      cudaMemsetAsync(sf, 0, sizeof(float) * S * N, st);
      cudaMemcpyAsync(sb, D.bits, sizeof(uint32_t) * P.nwords * N, cudaMemcpyDeviceToDevice, st);
      Dt.v32[0] = sv0;
      Dt.v32[1] = sv0;
      Dt.f32 = sf;
      Dt.bits = sb;
      cudaEvent_t ea, eb;
      cudaEventCreate(&ea);
      cudaEventCreate(&eb);
      for (auto &bk : b->buckets) {
        float best = 1e30f;
        std::vector<int> cands = {NLM_DECOMP_THREAD, NLM_DECOMP_THREAD1, NLM_DECOMP_WARP};
        if (b->tile_ok) cands.push_back(NLM_DECOMP_TILE_LOCAL);
        for (int c : cands) {
          StepArgs a{0, false, 0., b->dt, nullptr, bk.i0, bk.i1};
          for (int w = 0; w < 2; w++) e2 = launch_rnp_step_fp32(P, Dt, b->T, a, c, st);
          cudaEventRecord(ea, st);
          for (int r = 0; r < 3; r++) e2 = launch_rnp_step_fp32(P, Dt, b->T, a, c, st);
          cudaEventRecord(eb, st);
          if (e2 == cudaSuccess) e2 = cudaEventSynchronize(eb);
          float ms = 0.f;
          if (e2 == cudaSuccess) e2 = cudaEventElapsedTime(&ms, ea, eb);
          if (e2 != cudaSuccess) break;
          if (ms < best) {
            best = ms;
            bk.decomp = c;
          }
        }
        if (e2 != cudaSuccess) break;
      }
      cudaEventDestroy(ea);
      cudaEventDestroy(eb);
    }
    cudaStreamSynchronize(st);
    cudaFree(sv0);
    cudaFree(sf);
    cudaFree(sb);
    if (e2 != cudaSuccess) return bail(cuda_fail(e2, "batch autotune"));
  }
  *out = b;
#undef BTRY
  return NLM_OK;
}

int nlm_batch_destroy(nlm_batch *b) {
  delete b;
  return NLM_OK;
}

int nlm_batch_run(nlm_batch *b, int64_t nsteps) {
  if (!b || nsteps < 0) return fail(NLM_ERR_INVALID, "bad arguments");
  return batch_run(b, nsteps);
}

int nlm_batch_run_timed(nlm_batch *b, int64_t nsteps, double *ms) {
  if (!b || !ms || nsteps < 0) return fail(NLM_ERR_INVALID, "bad arguments");
  cudaEvent_t e0, e1;
  NLM_CUDA(cudaEventCreate(&e0));
  NLM_CUDA(cudaEventCreate(&e1));
  cudaEventRecord(e0, b->stream);
  int rc = batch_run(b, nsteps);
  cudaEventRecord(e1, b->stream);
  cudaError_t e = cudaEventSynchronize(e1);
  float t = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  if (e != cudaSuccess) return cuda_fail(e, "batch timing");
  *ms = t;
  return NLM_OK;
}

int nlm_batch_num_bonds(const nlm_batch *b, int s, int64_t *nnz) {
  if (!b || !nnz || s < -1 || s >= b->nspec) return fail(NLM_ERR_INVALID, "bad arguments");
  *nnz = s < 0 ? b->nnz : b->nbond[s];
  return NLM_OK;
}

int nlm_batch_get_time(const nlm_batch *b, double *time, int64_t *step) {
  if (!b) return fail(NLM_ERR_INVALID, "null handle");
  if (time) *time = b->time;
  if (step) *step = b->step;
  return NLM_OK;
}

int nlm_batch_get_state(nlm_batch *b, int s, double *u, double *v, double *f) {
  if (!b || s < 0 || s >= b->nspec) return fail(NLM_ERR_INVALID, "bad arguments");
  const int64_t n = b->n[s], off = b->off[s];
  const int S = b->S;
  cudaStream_t st = b->stream;
  int *dperm = nullptr;
  NLM_CUDA(cudaMalloc(&dperm, sizeof(int) * (n + 1)));
  cudaError_t e = cudaMemcpyAsync(dperm, b->perm[s].data(), sizeof(int) * n, cudaMemcpyHostToDevice, st);
  const unsigned g = nblk(n, 256);
  const int vi = b->scheme == NLM_CENTRAL_DIFFERENCE ? b->cur : 0;
  if (e == cudaSuccess && u) {
    k_gather_split<<<g, 256, 0, st>>>(n, S, dperm, b->D.u32[b->cur] + (S / 2) * off, b->stage);
    e = cudaMemcpyAsync(u, b->stage, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  }
  if (e == cudaSuccess && v) {
    k_gather_split<<<g, 256, 0, st>>>(n, S, dperm, b->D.v32[vi] + (S / 2) * off, b->stage);
    e = cudaMemcpyAsync(v, b->stage, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  }
  if (e == cudaSuccess && f) {
    k_gather_f32<<<g, 256, 0, st>>>(n, S, dperm, b->D.f32 + (size_t)S * off, b->stage);
    e = cudaMemcpyAsync(f, b->stage, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  }
  cudaStreamSynchronize(st);
  cudaFree(dperm);
  if (e != cudaSuccess) return cuda_fail(e, "batch state download");
  return NLM_OK;
}

int nlm_batch_get_bond_state(nlm_batch *b, int s, uint8_t *broken) {
  if (!b || !broken || s < 0 || s >= b->nspec) return fail(NLM_ERR_INVALID, "bad arguments");
  const int64_t n = b->n[s], off = b->off[s], npad = b->P.npad;
  std::vector<uint32_t> bits((size_t)b->P.nwords * npad);
  std::vector<int> cc(b->nbond[s] + 1);
  NLM_CUDA(cudaMemcpyAsync(bits.data(), b->D.bits, sizeof(uint32_t) * bits.size(), cudaMemcpyDeviceToHost, b->stream));
  if (b->nbond[s])
    NLM_CUDA(cudaMemcpyAsync(cc.data(), b->D.cols + b->bond_off[s], sizeof(int) * b->nbond[s],
                             cudaMemcpyDeviceToHost, b->stream));
  NLM_CUDA(cudaStreamSynchronize(b->stream));
  const std::vector<int> &perm = b->perm[s];
  std::vector<int64_t> inv(n);
  for (int64_t i = 0; i < n; i++) inv[perm[i]] = i;
  int64_t o_off = 0;
  std::vector<std::pair<int, uint8_t>> row;
  for (int64_t o = 0; o < n; o++) {
    const int64_t i = inv[o], g = off + i;
    const int64_t r0 = b->rowptr[g], len = b->rowptr[g + 1] - r0;
    row.resize(len);
    for (int64_t k = 0; k < len; k++)
      row[k] = {perm[cc[r0 - b->bond_off[s] + k] - off],
                (uint8_t)((bits[(size_t)(k >> 5) * npad + g] >> (k & 31)) & 1u)};
    std::sort(row.begin(), row.end());
    for (int64_t k = 0; k < len; k++) broken[o_off + k] = row[k].second;
    o_off += len;
  }
  return NLM_OK;
}

int nlm_batch_set_graph(nlm_batch *b, int steps_per_graph) {
  if (!b || steps_per_graph < 0 || (steps_per_graph % 2) || steps_per_graph == 1)
    return fail(NLM_ERR_INVALID, "steps_per_graph must be 0 or an even number >= 2");
  NLM_CUDA(cudaStreamSynchronize(b->stream));
  for (auto &g : b->gexec)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
  if (b->h_times) {
    cudaFreeHost(b->h_times);
    b->h_times = nullptr;
  }
  b->graph_steps = steps_per_graph;
  if (steps_per_graph > 0) {
    NLM_CUDA(cudaMallocHost(&b->h_times, sizeof(double) * (steps_per_graph + 1)));
    if (b->alloc(&b->d_times, (size_t)steps_per_graph + 1) != cudaSuccess)
      return fail(NLM_ERR_OOM, "graph time buffer");
    if (!b->ev_times) NLM_CUDA(cudaEventCreateWithFlags(&b->ev_times, cudaEventDisableTiming));
    NLM_CUDA(cudaEventRecord(b->ev_times, b->stream));
  }
  return NLM_OK;
}

int nlm_batch_buckets(const nlm_batch *b, int *n_buckets, int64_t *bucket_nodes, int *decomps) {
  if (!b || !n_buckets) return fail(NLM_ERR_INVALID, "null argument");
  *n_buckets = (int)b->buckets.size();
  for (size_t k = 0; k < b->buckets.size() && k < 8; k++) {
    if (bucket_nodes) bucket_nodes[k] = b->buckets[k].i1 - b->buckets[k].i0;
    if (decomps) decomps[k] = b->buckets[k].decomp;
  }
  return NLM_OK;
}

}  // extern "C"

// ===========================================================================
// Quasi-static Newton (RNPBond).  Geometry, bond bits, flags and loads come
// from an FP64 nlm_fd handle; the state is its displacement buffer u64[cur].

struct nlm_qs {
  nlm_fd *fd = nullptr;
  nlm_qs_params prm{};
  QSWork W{};
  unsigned long long *count = nullptr;
  double *saved = nullptr;  // plain start point while a guess is evaluated
  double *cand = nullptr;   // best candidate start so far
  // FP64 Krylov solves from now on, for Newton corrections and for tangent
  // predictors respectively: set once a solve of that kind has not converged
  // in FP32 within its iteration cap (the tangent of this specimen is then
  // too ill-conditioned for FP32 recurrences)
  bool cg64 = false;
  bool cg64_predictor = false;
  std::vector<void *> allocs;
  ~nlm_qs() {
    if (fd) nlm_fd_destroy(fd);  // frees the stream first
    for (void *p : allocs) cudaFree(p);
  }
  template <class Tp>
  cudaError_t alloc(Tp **p, size_t count_) {
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, count_ * sizeof(Tp) + 16);
    if (e == cudaSuccess) {
      allocs.push_back(q);
      *p = static_cast<Tp *>(q);
    }
    return e;
  }
};

namespace {

int qs_norm(nlm_qs *q, const double *u, double *buf, double *norm) {
  nlm_fd *h = q->fd;
  cudaError_t e = qs_residual(h->P, h->D, u, buf, nullptr, nullptr, false, h->stream);
  if (e == cudaSuccess) e = qs_dot(buf, buf, (int64_t)h->dim * h->n, q->W.part, q->W.sc + 4, h->stream);
  double v = 0.;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&v, q->W.sc + 4, sizeof(double), cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return cuda_fail(e, "qs residual");
  *norm = std::sqrt(v);
  return NLM_OK;
}

// Newton iterations from the current u until ||r|| <= target.  Each residual
// evaluation breaks the bonds past the critical strain first.
int qs_newton(nlm_qs *q, double target, nlm_qs_stats *st) {
  nlm_fd *h = q->fd;
  double *u = h->D.u64[h->cur];
  const int64_t m = (int64_t)h->dim * h->n;
  for (int it = 0;; it++) {
    cudaError_t e = cudaMemsetAsync(q->count, 0, sizeof(unsigned long long), h->stream);
    if (e == cudaSuccess)
      e = qs_residual(h->P, h->D, u, q->W.res, q->W.blk, q->W.dblk, true, h->stream,
                      q->prm.break_bonds ? q->count : nullptr);
    if (e == cudaSuccess) e = qs_dot(q->W.res, q->W.res, m, q->W.part, q->W.sc + 4, h->stream);
    double rr = 0.;
    unsigned long long c = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&rr, q->W.sc + 4, sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&c, q->count, sizeof(c), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_fail(e, "qs Newton residual");
    st->broken += (int64_t)c;
    if (c) st->break_rounds++;
    st->res_final = std::sqrt(rr);
    if (!(st->res_final > target) || it >= q->prm.max_newton) return NLM_OK;
    int li = 0;
    e = qs_cg(h->P, h->D, q->W, q->W.res, q->W.dx, q->prm.lin_tol, q->prm.lin_max_iters, 8, &li,
              &q->cg64,
              h->stream);
    if (e == cudaSuccess) e = qs_add(h->P, q->W.dx, u, h->stream);
    if (e != cudaSuccess) return cuda_fail(e, "qs linear solve");
    st->lin_iters += li;
    st->newton_iters++;
  }
}

// ||res0 - (-K) dx|| over free dofs: the linear model of the residual at the
// previous converged state, evaluated at the increment dx.
int qs_linear_norm(nlm_qs *q, double *norm) {
  nlm_fd *h = q->fd;
  const int64_t m = (int64_t)h->dim * h->n;
  cudaStream_t s = h->stream;
  cudaError_t e = qs_spmv(h->P, h->D, q->W.blk, q->W.dblk, q->W.dx, q->W.ap, q->W.part, s);
  if (e == cudaSuccess) e = qs_sub(m, q->W.res0, q->W.ap, q->W.res, s);
  if (e == cudaSuccess) e = qs_dot(q->W.res, q->W.res, m, q->W.part, q->W.sc + 4, s);
  double rr = 0.;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&rr, q->W.sc + 4, sizeof(double), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "qs linear model");
  *norm = std::sqrt(rr);
  return NLM_OK;
}

}  // namespace

extern "C" {

int nlm_qs_create(const nlm_fd_desc *desc, const nlm_qs_params *prm, nlm_qs **out) {
  if (!desc || !prm || !out) return fail(NLM_ERR_INVALID, "null argument");
  *out = nullptr;
  if (desc->material.kind != NLM_MAT_RNP_BOND)
    return fail(NLM_ERR_UNSUPPORTED, "the GPU quasi-static solver is for RNPBond");
  if (desc->material.apply_contact)
    return fail(NLM_ERR_UNSUPPORTED, "the quasi-static solver has no contact term");
  for (int c = 0; c < desc->n_cracks; c++)
    if (desc->cracks && desc->cracks[c].timed)
      return fail(NLM_ERR_UNSUPPORTED, "the quasi-static solver takes pre-cracks only");
  if (prm->max_newton < 1 || !(prm->tol > 0.) || prm->lin_max_iters < 1 || !(prm->lin_tol > 0.))
    return fail(NLM_ERR_INVALID, "bad solver parameters");
  nlm_fd_desc d = *desc;
  d.precision = NLM_PREC_FP64;
  d.scheme = NLM_VELOCITY_VERLET;
  d.decomposition = NLM_DECOMP_THREAD;
  if (!(d.dt > 0.)) return fail(NLM_ERR_INVALID, "load-step increment dt must be positive");
  nlm_qs *q = new nlm_qs();
  int rc = nlm_fd_create(&d, &q->fd);
  if (rc) {
    delete q;
    return rc;
  }
  q->prm = *prm;
  nlm_fd *h = q->fd;
  const int64_t n = h->n, m = (int64_t)h->dim * n, nnz = h->nnz;
  const int NB = h->dim == 2 ? 3 : 6;
  cudaError_t e = cudaSuccess;
  for (double **p : {&q->W.res, &q->W.dx, &q->W.r, &q->W.z, &q->W.p, &q->W.p2, &q->W.ap,
                     &q->W.res0})
    if (e == cudaSuccess) e = q->alloc(p, m);
  if (e == cudaSuccess) e = q->alloc(&q->W.part, std::max<int64_t>((m + 255) / 256 + 1, qs_cg_stride(n)));
  if (e == cudaSuccess) e = q->alloc(&q->W.cgpart, 3 * qs_cg_stride(n));
  if (e == cudaSuccess) e = q->alloc(&q->W.cgs, 8);
  for (float **p : {&q->W.r32, &q->W.z32, &q->W.p32, &q->W.p32b, &q->W.ap32, &q->W.x32})
    if (e == cudaSuccess) e = q->alloc(p, m);
  if (e == cudaSuccess) e = q->alloc(&q->W.blk32, (size_t)(NB == 3 ? 4 : 8) * (nnz + 1));
  if (e == cudaSuccess) e = q->alloc(&q->W.dblk32, (size_t)NB * n);
  q->W.nnz = nnz;
  if (e == cudaSuccess) e = q->alloc(&q->W.ticket, 4);
  if (e == cudaSuccess) e = cudaMemset(q->W.ticket, 0, 4 * sizeof(unsigned));
  if (e == cudaSuccess) e = q->alloc(&q->W.sc, 8);
  if (e == cudaSuccess) e = q->alloc(&q->W.blk, (size_t)NB * (nnz + 1));
  if (e == cudaSuccess) e = q->alloc(&q->W.dblk, (size_t)NB * n);
  if (e == cudaSuccess) e = q->alloc(&q->count, 1);
  if (e == cudaSuccess) e = q->alloc(&q->saved, (size_t)h->S * n);
  if (e == cudaSuccess) e = q->alloc(&q->cand, (size_t)h->S * n);
  if (e != cudaSuccess) {
    delete q;
    return cuda_fail(e, "qs buffers");
  }
  h->started = true;  // no explicit step-0 evaluation
  *out = q;
  return NLM_OK;
}

int nlm_qs_destroy(nlm_qs *q) {
  delete q;
  return NLM_OK;
}

int nlm_qs_load_step(nlm_qs *q, const double *guess, nlm_qs_stats *stats) {
  return nlm_qs_load_step_candidates(q, guess, guess ? 1 : 0, stats);
}

int nlm_qs_load_step_candidates(nlm_qs *q, const double *guesses, int n_cand,
                                nlm_qs_stats *stats) {
  if (!q) return fail(NLM_ERR_INVALID, "null handle");
  if (n_cand < 0 || (n_cand > 0 && !guesses)) return fail(NLM_ERR_INVALID, "bad candidates");
  auto t0 = std::chrono::steady_clock::now();
  nlm_fd *h = q->fd;
  nlm_qs_stats st{};
  cudaStream_t s = h->stream;
  double *u = h->D.u64[h->cur];
  const int64_t m = (int64_t)h->dim * h->n;
  const size_t bytes = sizeof(double) * h->S * h->n;
  // force and tangent at the previous converged state
  NLM_CUDA(cudaMemcpyAsync(q->saved, u, bytes, cudaMemcpyDeviceToDevice, s));
  cudaError_t e = qs_residual(h->P, h->D, u, q->W.res0, q->W.blk, q->W.dblk, true, s);
  if (e != cudaSuccess) return cuda_fail(e, "qs assembly");
  // QuasiStaticModel::solver: time = n * dt, then the displacement loads
  h->step++;
  h->time = (double)h->step * h->dt;
  int rc = apply_bc(h, h->time);
  if (rc) return rc;
  // plain predictor: boundary increment only
  if ((e = qs_bcdiff(h->P, h->D, u, q->saved, q->W.dx, true, s)) != cudaSuccess)
    return cuda_fail(e, "qs predictor");
  if ((rc = qs_linear_norm(q, &st.res_plain))) return rc;
  st.res_start = st.res_plain;
  NLM_CUDA(cudaMemcpyAsync(q->W.r, q->W.res, sizeof(double) * m, cudaMemcpyDeviceToDevice, s));
  bool use_guess = false;
  if (n_cand > 0) {
    // each candidate start is judged by the linear model of the residual at
    // the previous converged state; the best one is kept if it cuts the
    // linearised residual of the plain start clearly (a start no better than
    // the plain one, e.g. the previous state itself, would put the bonds next
    // to the loaded layer past their critical strain in the first residual
    // evaluation, which the tangent predictor of the plain start avoids)
    const double acc = q->prm.guess_accept > 0. ? q->prm.guess_accept : 0.1;
    int best = -1;
    double best_rg = 0.;
    for (int c = 0; c < n_cand; c++) {
      NLM_CUDA(cudaMemcpyAsync(h->stage, guesses + (size_t)3 * h->n * c,
                               sizeof(double) * 3 * h->n, cudaMemcpyHostToDevice, s));
      k_scatter_vec<<<nblk(h->n, 256), 256, 0, s>>>(h->n, h->S, h->dim, h->D.perm_dev, h->stage, u);
      NLM_CUDA(cudaGetLastError());
      if ((rc = apply_bc(h, h->time))) return rc;
      if ((e = qs_bcdiff(h->P, h->D, u, q->saved, q->W.dx, false, s)) != cudaSuccess)
        return cuda_fail(e, "qs guess");
      double rg = 0.;
      if ((rc = qs_linear_norm(q, &rg))) return rc;
      if (best < 0 || rg < best_rg) {
        best = c;
        best_rg = rg;
        if (n_cand > 1) NLM_CUDA(cudaMemcpyAsync(q->cand, u, bytes, cudaMemcpyDeviceToDevice, s));
      }
    }
    if (best >= 0 && best_rg <= acc * st.res_plain) {
      use_guess = true;
      st.used_guess = best + 1;
      st.res_start = best_rg;
      if (n_cand > 1) NLM_CUDA(cudaMemcpyAsync(u, q->cand, bytes, cudaMemcpyDeviceToDevice, s));
    } else {
      NLM_CUDA(cudaMemcpyAsync(u, q->saved, bytes, cudaMemcpyDeviceToDevice, s));
      if ((rc = apply_bc(h, h->time))) return rc;
    }
  }
  const double target = q->prm.tol * st.res_plain;
  if (!use_guess && st.res_plain > 0.) {
    // tangent predictor (first Newton iteration) on the saved right-hand side
    NLM_CUDA(cudaMemcpyAsync(q->W.res, q->W.r, sizeof(double) * m, cudaMemcpyDeviceToDevice, s));
    NLM_CUDA(cudaMemcpyAsync(q->W.ap, q->W.res, sizeof(double) * m, cudaMemcpyDeviceToDevice, s));
    int li = 0;
    e = qs_cg(h->P, h->D, q->W, q->W.ap, q->W.dx, q->prm.lin_tol, q->prm.lin_max_iters, 8, &li,
              &q->cg64_predictor, s);
    if (e == cudaSuccess) e = qs_add(h->P, q->W.dx, u, s);
    if (e != cudaSuccess) return cuda_fail(e, "qs predictor solve");
    st.lin_iters += li;
    st.newton_iters++;
  }
  if ((rc = qs_newton(q, target, &st))) return rc;
  st.ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (stats) *stats = st;
  return NLM_OK;
}

int nlm_qs_get_state(nlm_qs *q, double *u) {
  if (!q || !u) return fail(NLM_ERR_INVALID, "null argument");
  return nlm_fd_get_state(q->fd, u, nullptr, nullptr);
}

int nlm_qs_get_bond_state(nlm_qs *q, uint8_t *broken) {
  if (!q) return fail(NLM_ERR_INVALID, "null handle");
  return nlm_fd_get_bond_state(q->fd, broken);
}

int nlm_qs_damage(nlm_qs *q, float *phi, float *Z) {
  if (!q) return fail(NLM_ERR_INVALID, "null handle");
  return nlm_fd_damage(q->fd, phi, Z);
}

int nlm_qs_num_bonds(const nlm_qs *q, int64_t *nnz) {
  if (!q) return fail(NLM_ERR_INVALID, "null handle");
  return nlm_fd_num_bonds(q->fd, nnz);
}

}  // extern "C"

// ===========================================================================
// Quasi-static ElasticState (QuasiStaticModel<ElasticState>).  Geometry,
// volumes, m_i, flags and loads come from an FP64 nlm_fd handle (a 1-D mesh
// is held as a 2-D one with y = 0; the material law uses the model's own
// dimension); the state is its displacement buffer u64[cur].

struct nlm_esqs {
  nlm_fd *fd = nullptr;
  nlm_esqs_params prm{};
  int mdim = 2;
  int64_t m = 0, nblocks = 0;
  double *theta = nullptr, *f = nullptr, *body = nullptr, *res = nullptr, *rhs = nullptr;
  double *dx = nullptr, *J = nullptr, *r = nullptr, *rhat = nullptr, *p = nullptr;
  double *v = nullptr, *sv = nullptr, *t = nullptr, *part = nullptr, *sc = nullptr;
  std::vector<void *> allocs;
  ~nlm_esqs() {
    if (fd) nlm_fd_destroy(fd);  // synchronises and frees the stream first
    for (void *q : allocs) cudaFree(q);
  }
  template <class Tp>
  cudaError_t alloc(Tp **ptr, size_t count_) {
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, count_ * sizeof(Tp) + 16);
    if (e == cudaSuccess) {
      allocs.push_back(q);
      *ptr = static_cast<Tp *>(q);
    }
    return e;
  }
};

namespace {

int esqs_dot_host(nlm_esqs *q, const double *a, const double *b, double *out) {
  cudaStream_t s = q->fd->stream;
  cudaError_t e = esqs_dot(q->m, a, b, q->part, q->sc, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, q->sc, sizeof(double), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? NLM_OK : cuda_fail(e, "quasi-static dot product");
}

// f and the residual r = f + b at the current u; *norm = ||r||.
int esqs_eval(nlm_esqs *q, double *norm) {
  nlm_fd *h = q->fd;
  cudaError_t e = esqs_force(h->P, h->D, h->S, q->mdim, h->D.u64[h->cur], q->theta, q->f, h->stream);
  if (e == cudaSuccess) e = esqs_residual(h->P, h->D, h->S, q->mdim, q->f, q->body, q->res, h->stream);
  if (e != cudaSuccess) return cuda_fail(e, "quasi-static residual");
  double rr = 0.;
  int rc = esqs_dot_host(q, q->res, q->res, &rr);
  *norm = std::sqrt(rr);
  return rc;
}

// BiCGSTAB (van der Vorst 1992) for J dx = rhs to ||r|| <= tol ||rhs||.
int esqs_bicgstab(nlm_esqs *q, int *iters) {
  nlm_fd *h = q->fd;
  cudaStream_t s = h->stream;
  const int64_t m = q->m;
  const size_t bytes = sizeof(double) * m;
  NLM_CUDA(cudaMemsetAsync(q->dx, 0, bytes, s));
  NLM_CUDA(cudaMemcpyAsync(q->r, q->rhs, bytes, cudaMemcpyDeviceToDevice, s));
  NLM_CUDA(cudaMemcpyAsync(q->rhat, q->rhs, bytes, cudaMemcpyDeviceToDevice, s));
  NLM_CUDA(cudaMemsetAsync(q->p, 0, bytes, s));
  NLM_CUDA(cudaMemsetAsync(q->v, 0, bytes, s));
  double bb = 0.;
  int rc = esqs_dot_host(q, q->rhs, q->rhs, &bb);
  if (rc) return rc;
  *iters = 0;
  const double bnorm = std::sqrt(bb);
  if (bnorm == 0.) return NLM_OK;
  const double stop = q->prm.lin_tol * bnorm;
  double rho = 1., alpha = 1., omega = 1.;
  auto J_times = [&](const double *x, double *y) {
    cudaError_t e = esqs_spmv(h->P, h->D, h->S, q->mdim, q->J, x, y, s);
    return e == cudaSuccess ? NLM_OK : cuda_fail(e, "quasi-static Jacobian product");
  };
  auto lin3 = [&](double a, const double *x, double b, const double *y, double c, const double *z,
                  double *out) {
    cudaError_t e = esqs_lin3(m, a, x, b, y, c, z, out, s);
    return e == cudaSuccess ? NLM_OK : cuda_fail(e, "quasi-static vector update");
  };
  for (int it = 1; it <= q->prm.lin_max_iters; it++) {
    *iters = it;
    double rho_new = 0.;
    if ((rc = esqs_dot_host(q, q->rhat, q->r, &rho_new))) return rc;
    if (rho_new == 0.) break;  // breakdown: keep the iterate
    const double beta = (rho_new / rho) * (alpha / omega);
    if ((rc = lin3(1., q->r, beta, q->p, -beta * omega, q->v, q->p))) return rc;
    if ((rc = J_times(q->p, q->v))) return rc;
    double rv = 0.;
    if ((rc = esqs_dot_host(q, q->rhat, q->v, &rv))) return rc;
    if (rv == 0.) break;
    alpha = rho_new / rv;
    if ((rc = lin3(1., q->r, -alpha, q->v, 0., nullptr, q->sv))) return rc;
    double ss = 0.;
    if ((rc = esqs_dot_host(q, q->sv, q->sv, &ss))) return rc;
    if (std::sqrt(ss) <= stop) {
      if ((rc = lin3(1., q->dx, alpha, q->p, 0., nullptr, q->dx))) return rc;
      break;
    }
    if ((rc = J_times(q->sv, q->t))) return rc;
    double ts = 0., tt = 0.;
    if ((rc = esqs_dot_host(q, q->t, q->sv, &ts))) return rc;
    if ((rc = esqs_dot_host(q, q->t, q->t, &tt))) return rc;
    if (tt == 0.) {
      if ((rc = lin3(1., q->dx, alpha, q->p, 0., nullptr, q->dx))) return rc;
      break;
    }
    omega = ts / tt;
    if ((rc = lin3(1., q->dx, alpha, q->p, omega, q->sv, q->dx))) return rc;
    if ((rc = lin3(1., q->sv, -omega, q->t, 0., nullptr, q->r))) return rc;
    double rr = 0.;
    if ((rc = esqs_dot_host(q, q->r, q->r, &rr))) return rc;
    if (std::sqrt(rr) <= stop || omega == 0.) break;
    rho = rho_new;
  }
  return NLM_OK;
}

}  // namespace

extern "C" {

int nlm_esqs_create(const nlm_fd_desc *desc, const nlm_esqs_params *prm, nlm_esqs **out) {
  if (!desc || !prm || !out) return fail(NLM_ERR_INVALID, "null argument");
  *out = nullptr;
  if (desc->material.kind != NLM_MAT_ELASTIC_STATE)
    return fail(NLM_ERR_UNSUPPORTED, "QuasiStaticModel is instantiated for ElasticState");
  if (desc->dim < 1 || desc->dim > 3) return fail(NLM_ERR_INVALID, "dimension must be 1, 2 or 3");
  if (desc->dim == 1 && !(desc->material.E > 0.))
    return fail(NLM_ERR_INVALID, "1-D ElasticState needs E");
  if (prm->max_iters < 0 || !(prm->tol > 0.) || !(prm->perturbation > 0.) ||
      prm->lin_max_iters < 1 || !(prm->lin_tol > 0.) || !(prm->dt > 0.))
    return fail(NLM_ERR_INVALID, "bad solver parameters");
  for (int c = 0; c < desc->n_cracks; c++)
    if (desc->cracks && desc->cracks[c].timed)
      return fail(NLM_ERR_UNSUPPORTED, "the quasi-static solver takes pre-cracks only");
  nlm_fd_desc d = *desc;
  d.precision = NLM_PREC_FP64;
  d.scheme = NLM_VELOCITY_VERLET;
  d.decomposition = NLM_DECOMP_THREAD;
  d.dt = prm->dt;
  d.material.es_sc = 0.;  // no bond breaks in QuasiStaticModel
  std::vector<double> x1;
  if (desc->dim == 1) {
    // a 1-D mesh as a 2-D one: nodes (x, 0, 0); the 2-D constants are unused
    d.dim = 2;
    x1.assign(3 * (size_t)desc->n_nodes, 0.);
    for (int64_t i = 0; i < desc->n_nodes && desc->x; i++) x1[3 * i] = desc->x[3 * i];
    d.x = x1.data();
    if (!(d.material.K > 0.)) d.material.K = 1.;
    if (!(d.material.G > 0.)) d.material.G = 1.;
  }
  nlm_esqs *q = new nlm_esqs();
  int rc = nlm_fd_create(&d, &q->fd);
  if (rc) {
    delete q;
    return rc;
  }
  q->prm = *prm;
  q->mdim = desc->dim;
  nlm_fd *h = q->fd;
  q->m = (int64_t)h->S * h->n;
  q->nblocks = h->nnz + h->n;
  cudaError_t e = q->alloc(&q->theta, h->n);
  for (double **ptr : {&q->f, &q->body, &q->res, &q->rhs, &q->dx, &q->r, &q->rhat, &q->p, &q->v,
                       &q->sv, &q->t})
    if (e == cudaSuccess) e = q->alloc(ptr, q->m);
  if (e == cudaSuccess) e = q->alloc(&q->J, (size_t)9 * q->nblocks);
  if (e == cudaSuccess) e = q->alloc(&q->part, kEsqsDotParts);
  if (e == cudaSuccess) e = q->alloc(&q->sc, 1);
  if (e == cudaSuccess) e = cudaMemsetAsync(q->body, 0, sizeof(double) * q->m, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) {
    delete q;
    return cuda_fail(e, "quasi-static buffers");
  }
  h->started = true;  // no explicit step-0 evaluation
  *out = q;
  return NLM_OK;
}

int nlm_esqs_destroy(nlm_esqs *q) {
  delete q;
  return NLM_OK;
}

int nlm_esqs_solve(nlm_esqs *q, int nsteps, int *newton_iters, int *lin_iters,
                   double *final_res) {
  if (!q || nsteps < 0) return fail(NLM_ERR_INVALID, "bad arguments");
  nlm_fd *h = q->fd;
  cudaStream_t s = h->stream;
  double *u = h->D.u64[h->cur];
  const double eps = q->prm.perturbation * h->P.h;
  double res = 0.;
  int rc;
  for (int k = 0; k < nsteps; k++) {
    // QuasiStaticModel::solver (:526-594): time = n dt, force loading (added
    // to the body force, fLoading.cpp:268-275), displacement loading
    h->step++;
    h->time = (double)h->step * q->prm.dt;
    if (h->n_fbc_nodes > 0) {
      if ((rc = apply_fbc(h, h->time))) return rc;
      cudaError_t e = esqs_lin3(q->m, 1., q->body, 1., h->D.fext, 0., nullptr, q->body, s);
      if (e != cudaSuccess) return cuda_fail(e, "quasi-static body force");
    }
    if ((rc = apply_bc(h, h->time))) return rc;
    if ((rc = esqs_eval(q, &res))) return rc;
    const double r0 = res;
    int it = 0, li_total = 0;
    auto converged = [&]() {
      return q->prm.tol_relative ? (r0 == 0. || res / r0 < q->prm.tol) : res < q->prm.tol;
    };
    while (!converged() && it < q->prm.max_iters) {
      cudaError_t e = esqs_jacobian(h->P, h->D, h->S, q->mdim, q->prm.jacobian, u, eps, q->J,
                                    q->nblocks, s);
      if (e == cudaSuccess) e = esqs_lin3(q->m, -1., q->res, 0., nullptr, 0., nullptr, q->rhs, s);
      if (e != cudaSuccess) return cuda_fail(e, "quasi-static Jacobian");
      int li = 0;
      if ((rc = esqs_bicgstab(q, &li))) return rc;
      li_total += li;
      e = esqs_lin3(q->m, 1., u, 1., q->dx, 0., nullptr, u, s);
      if (e != cudaSuccess) return cuda_fail(e, "quasi-static update");
      if ((rc = esqs_eval(q, &res))) return rc;
      it++;
    }
    if (newton_iters) newton_iters[k] = it;
    if (lin_iters) lin_iters[k] = li_total;
  }
  if (final_res) *final_res = res;
  return NLM_OK;
}

int nlm_esqs_get_state(nlm_esqs *q, double *u, double *force) {
  if (!q) return fail(NLM_ERR_INVALID, "null handle");
  nlm_fd *h = q->fd;
  if (u) {
    int rc = nlm_fd_get_state(h, u, nullptr, nullptr);
    if (rc) return rc;
  }
  if (force) {
    const int64_t n = h->n;
    std::vector<double> fi((size_t)q->m), vol(n);
    NLM_CUDA(cudaMemcpyAsync(fi.data(), q->f, sizeof(double) * q->m, cudaMemcpyDeviceToHost, h->stream));
    NLM_CUDA(cudaMemcpyAsync(vol.data(), h->D.vol64, sizeof(double) * n, cudaMemcpyDeviceToHost, h->stream));
    NLM_CUDA(cudaStreamSynchronize(h->stream));
    for (int64_t i = 0; i < n; i++) {
      const int64_t o = h->perm[i];
      for (int d = 0; d < 3; d++) {
        const double fd = (d < h->S && d < q->mdim) ? fi[(size_t)h->S * i + d] : 0.;
        force[3 * o + d] = fd * vol[i];
      }
    }
  }
  return NLM_OK;
}

}  // extern "C"
