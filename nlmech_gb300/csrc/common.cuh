// common.cuh -- shared device types and helpers of libnlmgpu.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/nlmgpu.h"

namespace nlm {

// Relative-tolerance comparisons of util::compare (src/util/compare.cpp:25-33,
// COMPARE_EPS 1e-5).  Written with explicit round-to-nearest intrinsics so the
// FP64 path evaluates exactly the reference expression whatever the
// contraction flags of the translation unit.
__host__ __device__ inline double amax_d(double a, double b) {
  return fabs(a) < fabs(b) ? fabs(b) : fabs(a);
}
#ifdef __CUDA_ARCH__
__device__ inline bool dGT(double a, double b) {
  return __dsub_rn(a, b) > __dmul_rn(amax_d(a, b), 1e-5);
}
__device__ inline bool dLT(double a, double b) {
  return __dsub_rn(b, a) > __dmul_rn(amax_d(a, b), 1e-5);
}
#else
inline bool dGT(double a, double b) { return (a - b) > (amax_d(a, b) * 1e-5); }
inline bool dLT(double a, double b) { return (b - a) > (amax_d(a, b) * 1e-5); }
#endif

// Node flag byte.
enum : uint8_t {
  FLAG_FIX_X = 1,
  FLAG_FIX_Y = 2,
  FLAG_FIX_Z = 4,
  FLAG_NOFAIL = 8,  // non-interior node: bonds never break (rnpBond.cpp:235-240)
  FLAG_FBC = 16,    // node carries an external force (Force_BC)
  FLAG_GHOST = 32   // padding node of a batched specimen (never updated)
};

constexpr int kMaxBCSets = 32;
constexpr int kMaxRow = 512;  // longest neighbour row the builder accepts

// Time functions of a displacement BC set, evaluated in the kernel
// (loading/uLoading.cpp:210-236).  umax already carries the spatial factor.
struct BCTime {
  int fn;
  double p[4];
};

struct BCEntry {   // one node with at least one prescribed dof
  int set[3];      // winning BC set per dof (-1: none)
  double umax[3];  // spatial factor times time_params[0]
};

// Kernel parameters shared by the explicit-step kernels.
struct StepParams {
  int64_t n;          // nodes (sorted order)
  int dim;
  int nwords;         // bond-bit words per node
  int64_t npad;       // stride of the word-major bond-bit array
  // geometry / material (FP64 constants)
  double delta, h, check_up, check_low;
  double C, beta, rbar, invF, fsc;
  int irrev;
  int contact;        // normal contact between the nodes of broken bonds
  double contact_kn, contact_rc;  // K 18 / (pi delta^5), 0.9 h (rnpBond.cpp:79-88)
  int nofail;         // 1 when some node is non-interior (no-fail region)
  int infl_type;
  double infl_a0, infl_a1, infl_alpha, infl_beta;
  double lo_scale;    // FP32C position lo parts are stored as half(lo * lo_scale)
  int nw1;            // 1 when every row fits one 32-bit bond-bit word
  double vol_uniform; // the common nodal volume when every node has the same one, else 0
  int uv_specimens;   // batch: every specimen has one nodal volume (K1 V per specimen)
  double tile_span_max;  // > 0: tile-frame displacement span limit (batches: the
                         // smallest of the specimens'); 0: from this model's constants
  // integration
  double dt, rho;
  int scheme;
  // ElasticState constants
  double es_K, es_mu, es_nu, es_E, es_factor2D, es_sc;
  int es_plane_strain, es_ref_compat;
};

__device__ inline double influence_d(const StepParams &P, double r) {
  if (P.infl_type == 0) return P.infl_a0;
  if (P.infl_type == 1) return __dadd_rn(P.infl_a0, __dmul_rn(P.infl_a1, r));
  return __dmul_rn(P.infl_alpha, exp(__ddiv_rn(__dmul_rn(-r, r), P.infl_beta)));
}

// du, dv of ULoading::apply for one dof (uLoading.cpp:166-253).
__device__ inline void bc_value(const BCTime &T, double umax, double time,
                                double &du, double &dv) {
  du = 0.;
  dv = 0.;
  switch (T.fn) {
    case NLM_TFN_CONSTANT:
      du = umax;
      break;
    case NLM_TFN_LINEAR:
      du = __dmul_rn(umax, time);
      dv = umax;
      break;
    case NLM_TFN_QUADRATIC:
      du = __dadd_rn(__dmul_rn(umax, time), __dmul_rn(__dmul_rn(T.p[1], time), time));
      dv = __dadd_rn(umax, __dmul_rn(T.p[1], time));
      break;
    case NLM_TFN_SIN: {
      double a = __dmul_rn(M_PI, T.p[1]);
      du = __dmul_rn(umax, sin(__dmul_rn(a, time)));
      dv = __dmul_rn(__dmul_rn(umax, a), cos(__dmul_rn(a, time)));
    } break;
    case NLM_TFN_LINEAR_STEP: {
      double x1 = T.p[1], x2 = T.p[2];
      double period = floor(__ddiv_rn(time, __dadd_rn(x1, x2)));
      bool up = dLT(time, __dadd_rn(__dmul_rn(period, __dadd_rn(x1, x2)), x1));
      double g = up ? __dsub_rn(time, __dmul_rn(period, x2)) : __dmul_rn(__dadd_rn(period, 1.), x1);
      du = __dmul_rn(umax, g);
      dv = __dmul_rn(umax, up ? 1. : 0.);
    } break;
    case NLM_TFN_LINEAR_SLOW_FAST:
      if (dGT(time, T.p[1])) {
        du = __dmul_rn(__dmul_rn(umax, T.p[3]), time);
        dv = __dmul_rn(umax, T.p[3]);
      } else {
        du = __dmul_rn(__dmul_rn(umax, T.p[2]), time);
        dv = __dmul_rn(umax, T.p[2]);
      }
      break;
  }
}

struct BCTable {
  int nsets;
  BCTime t[kMaxBCSets];
};

// Device error flag written by kernels that detect a bad input.
enum : int {
  DEVERR_NONE = 0,
  DEVERR_ROW_TOO_LONG = 1,
  DEVERR_NONFINITE = 2
};

}  // namespace nlm

// error plumbing (host)
namespace nlm {
void set_error(const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);
}  // namespace nlm

#define NLM_CUDA(call)                                         \
  do {                                                         \
    cudaError_t _e = (call);                                   \
    if (_e != cudaSuccess) return ::nlm::cuda_fail(_e, #call); \
  } while (0)
