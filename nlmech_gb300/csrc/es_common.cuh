// es_common.cuh -- ElasticState bond quantities shared by the explicit step
// (es_fp64.cu) and the quasi-static solver (esqs.cu).  Device code compiled
// with --fmad=false in both units.
#pragma once

#include "fd_internal.h"

namespace nlm {

// Volume correction factor omega (volumeCorrection.cpp:25-46).
__device__ __forceinline__ double es_omega(const StepParams &P, double Xl) {
  const double r = P.h * 0.5;
  return dGT(Xl, P.delta - r) ? (P.delta + r - Xl) / P.h : 1.;
}

// Scalar force state t (ElasticState.cpp:191-245); e_d = e - e_s in 3-D unless
// the reference's behaviour (e_d = 0) is requested.
template <int DIM>
__device__ __forceinline__ double es_t64(const StepParams &P, double mi, double theta, double e,
                                         double Xl) {
  if (DIM == 2) {
    double alpha_s;
    if (!P.es_plane_strain) {
      const double q = (P.es_nu + 1.) / (2. * P.es_nu - 1.);
      alpha_s = (9. / mi) * (P.es_K + q * q * P.es_mu / 9.);
    } else {
      alpha_s = (9. / mi) * (P.es_K + P.es_mu / 9.);
    }
    const double alpha_d = (8. / mi) * P.es_mu;
    const double e_s = theta * Xl / 3.;
    const double e_d = e - e_s;
    const double f2 = P.es_factor2D;
    const double t_s = (2. * f2 * alpha_s - (3. - 2. * f2) * alpha_d) * 1. * e_s / 3.;
    const double t_d = alpha_d * 1. * e_d;
    return t_s + t_d;
  }
  const double alpha_s = (9. / mi) * P.es_K;
  const double alpha_d = (15. / mi) * P.es_mu;
  const double e_s = theta * Xl / 3.;
  const double e_d = P.es_ref_compat ? 0. : e - e_s;
  const double t_s = alpha_s * 1. * e_s;
  const double t_d = alpha_d * 1. * e_d;
  return t_s + t_d;
}

template <int DIM>
__device__ __forceinline__ void es_geom64(const double xi[3], const double ui[3],
                                          const double xj[3], const double uj[3], double Y[3],
                                          double &Xl, double &e) {
  double X[3];
  for (int d = 0; d < 3; d++) {
    Y[d] = (xj[d] + uj[d]) - (xi[d] + ui[d]);
    X[d] = xj[d] - xi[d];
  }
  Xl = sqrt(X[0] * X[0] + X[1] * X[1] + X[2] * X[2]);
  e = sqrt(Y[0] * Y[0] + Y[1] * Y[1] + Y[2] * Y[2]) - Xl;
}

}  // namespace nlm
