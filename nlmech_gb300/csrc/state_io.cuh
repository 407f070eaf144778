// state_io.cuh -- node loads/stores and the per-node integrator epilogue.
#pragma once

#include "fd_internal.h"

namespace nlm {

// Node vectors are S doubles per node: S = 2 in 2-D (x, y), 4 in 3-D
// (x, y, z, pad) so that a node is one or two 16-byte loads.
template <int DIM>
__device__ __forceinline__ void ld_node(const double *p, int64_t i, double o[3]) {
  if (DIM == 2) {
    const double2 a = __ldg(reinterpret_cast<const double2 *>(p) + i);
    o[0] = a.x;
    o[1] = a.y;
    o[2] = 0.;
  } else {
    const double2 *q = reinterpret_cast<const double2 *>(p) + 2 * i;
    const double2 a = __ldg(q), b = __ldg(q + 1);
    o[0] = a.x;
    o[1] = a.y;
    o[2] = b.x;
  }
}

// Same, for arrays the current kernel also writes (no read-only cache).
template <int DIM>
__device__ __forceinline__ void ld_node_rw(const double *p, int64_t i, double o[3]) {
  if (DIM == 2) {
    const double2 a = reinterpret_cast<const double2 *>(p)[i];
    o[0] = a.x;
    o[1] = a.y;
    o[2] = 0.;
  } else {
    const double2 *q = reinterpret_cast<const double2 *>(p) + 2 * i;
    const double2 a = q[0], b = q[1];
    o[0] = a.x;
    o[1] = a.y;
    o[2] = b.x;
  }
}

template <int DIM>
__device__ __forceinline__ void st_node(double *p, int64_t i, const double v[3]) {
  if (DIM == 2) {
    reinterpret_cast<double2 *>(p)[i] = make_double2(v[0], v[1]);
  } else {
    double2 *q = reinterpret_cast<double2 *>(p) + 2 * i;
    q[0] = make_double2(v[0], v[1]);
    q[1] = make_double2(v[2], 0.);
  }
}

// Split (hi, lo) FP32 representation of an FP64 vector: value = hi + lo.
template <int DIM>
__device__ __forceinline__ void ld_split(const float4 *p, int64_t i, double o[3]) {
  if (DIM == 2) {
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

template <int DIM>
__device__ __forceinline__ void st_split(float4 *p, int64_t i, const double v[3]) {
  float h[3], l[3];
  for (int d = 0; d < DIM; d++) {
    h[d] = __double2float_rn(v[d]);
    l[d] = __double2float_rn(v[d] - (double)h[d]);
  }
  if (DIM == 2) {
    p[i] = make_float4(h[0], h[1], l[0], l[1]);
  } else {
    p[2 * i] = make_float4(h[0], h[1], h[2], 0.f);
    p[2 * i + 1] = make_float4(l[0], l[1], l[2], 0.f);
  }
}

template <int DIM>
__device__ __forceinline__ void ld_f32(const float *p, int64_t i, double o[3]) {
  if (DIM == 2) {
    const float2 a = reinterpret_cast<const float2 *>(p)[i];
    o[0] = a.x;
    o[1] = a.y;
    o[2] = 0.;
  } else {
    const float4 a = reinterpret_cast<const float4 *>(p)[i];
    o[0] = a.x;
    o[1] = a.y;
    o[2] = a.z;
  }
}

template <int DIM>
__device__ __forceinline__ void st_f32(float *p, int64_t i, const float v[3]) {
  if (DIM == 2)
    reinterpret_cast<float2 *>(p)[i] = make_float2(v[0], v[1]);
  else
    reinterpret_cast<float4 *>(p)[i] = make_float4(v[0], v[1], v[2], 0.f);
}

// Prescribed value of one dof at time t (ULoading::apply, uLoading.cpp:166).
__device__ __forceinline__ void bc_dof(const DevPtrs &D, const BCTable &T, int ref, int d,
                                       double t, double &du, double &dv) {
  const BCEntry &e = D.bce[ref];
  const int s = e.set[d];
  du = 0.;
  dv = 0.;
  if (s >= 0) bc_value(D.bct ? D.bct[s] : T.t[s], e.umax[d], t, du, dv);
}

// Step times of a launch (from the arguments, or from device memory when the
// launch is replayed from a CUDA graph).
__device__ __forceinline__ double t_now_of(const StepArgs &A) {
  return A.tdev ? __ldg(A.tdev) : A.t_now;
}
__device__ __forceinline__ double t_next_of(const StepArgs &A) {
  return A.tdev ? __ldg(A.tdev + 1) : A.t_next;
}

// Integrator epilogue of the fused step, FP64 state (see fd_host.cu for the
// phase bookkeeping).  f = external + internal force density of node i at
// u^m.  Velocity-Verlet (fDModel.cpp:445-525):
//   v^m     = (v^{m-1} + fact f^{m-1}) + fact f^m      (free dofs)
//   u^{m+1} = u^m + dt (v^m + fact f^m)                (free dofs)
// fixed dofs take the Displacement_BC values at t_m (v) and t_{m+1} (u).
// Central difference (fDModel.cpp:376-443):
//   u^{m+1} = u^m + (fact_cd f^m + dt v^m),  v^{m+1} = (u^{m+1} - u^m) / dt.
template <int DIM, int SCHEME, bool FIRST>
__device__ __forceinline__ void integrate_node64(const StepParams &P, const DevPtrs &D,
                                                 const BCTable &T, const StepArgs &A,
                                                 int64_t i, uint8_t fl, const double ui[3],
                                                 const double fint[3]) {
  double f[3] = {fint[0], fint[1], fint[2]};
  if (fl & FLAG_FBC) {
    double fe[3];
    ld_node<DIM>(D.fext, i, fe);
    for (int d = 0; d < DIM; d++) f[d] = fe[d] + fint[d];
  }
  const int ref = (fl & 7) ? D.bcref[i] : -1;
  double un[3] = {0., 0., 0.};
  if (SCHEME == NLM_VELOCITY_VERLET) {
    const double fact = 0.5 * P.dt / P.rho;
    double v[3], vn[3];
    ld_node_rw<DIM>(D.v[0], i, v);
    if (!FIRST) {
      double fp[3];
      ld_node_rw<DIM>(D.f64, i, fp);
      for (int d = 0; d < DIM; d++) {
        if (!(fl >> d & 1)) {
          const double vh = v[d] + fact * fp[d];
          vn[d] = vh + fact * f[d];
        } else {
          double du, dv;
          bc_dof(D, T, ref, d, t_now_of(A), du, dv);
          vn[d] = dv;
        }
      }
    } else {
      for (int d = 0; d < DIM; d++) vn[d] = v[d];
    }
    for (int d = 0; d < DIM; d++) {
      if (!(fl >> d & 1)) {
        const double vh = vn[d] + fact * f[d];
        un[d] = ui[d] + P.dt * vh;
      } else {
        double du, dv;
        bc_dof(D, T, ref, d, t_next_of(A), du, dv);
        un[d] = du;
      }
    }
    vn[2] = DIM == 3 ? vn[2] : 0.;
    st_node<DIM>(D.v[0], i, vn);
  } else {
    const double fact = P.dt * P.dt / P.rho;
    double v[3], vn[3] = {0., 0., 0.};
    ld_node<DIM>(D.v[A.cur], i, v);
    for (int d = 0; d < DIM; d++) {
      if (!(fl >> d & 1)) {
        un[d] = ui[d] + (fact * f[d] + P.dt * v[d]);
        vn[d] = (un[d] - ui[d]) / P.dt;
      } else {
        double du, dv;
        bc_dof(D, T, ref, d, t_next_of(A), du, dv);
        un[d] = du;
        vn[d] = dv;
      }
    }
    st_node<DIM>(D.v[1 - A.cur], i, vn);
  }
  st_node<DIM>(D.f64, i, f);
  st_node<DIM>(D.u64[1 - A.cur], i, un);
}

}  // namespace nlm
