// es_fp64.cu -- ElasticState explicit step, FP64 plain (two passes).
//
// Pass 1 (k_es_dil64): per node the bond extensions e_ij = |Y_ij| - |X_ij|
// (src/util/stateBasedHelperFunctions.cpp:47), the irreversible break test
// e_ij / |X_ij| > s_c, and the dilatation over intact bonds
//   theta_i = sum_j (c / m_i) f2 |X| e omega_ij V_j   (c = 2 in 2-D, 3 in 3-D;
//   f2 = factor2D in 2-D) as in stateBasedHelperFunctions.cpp:50-79.
// Pass 2 (k_es_force64): the gather form of the reference's half-force
// scatter (QuasiStaticModel.cpp:168-239 with ElasticState::getBondEF,
// ElasticState.cpp:160-271):
//   f_i = sum_j (t_ij + t_ji) M_ij omega_ij V_j,   M = Y / |Y|,
// followed by the integrator epilogue shared with RNPBond.
// Compiled with --fmad=false; sums run in neighbour-list order.

#include "es_common.cuh"
#include "fd_internal.h"
#include "state_io.cuh"

namespace nlm {

// Weighted volume m_i = sum_j |X|^2 omega V_j (volumeCorrection.cpp:48-67).
template <int DIM>
__global__ void k_es_mw(const StepParams P, const DevPtrs D, double *mw) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  double xi[3];
  ld_node<DIM>(D.pos64, i, xi);
  double tmp = 0.;
  for (int64_t k = D.rowptr[i]; k < D.rowptr[i + 1]; k++) {
    const int j = D.cols[k];
    double xj[3];
    ld_node<DIM>(D.pos64, j, xj);
    const double X0 = xj[0] - xi[0], X1 = xj[1] - xi[1], X2 = xj[2] - xi[2];
    const double Xl = sqrt(X0 * X0 + X1 * X1 + X2 * X2);
    tmp += (Xl * Xl * es_omega(P, Xl) * D.vol64[j]);
  }
  mw[i] = tmp;
}

template <int DIM>
__global__ void __launch_bounds__(128)
    k_es_dil64(const StepParams P, const DevPtrs D, const StepArgs A) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  const double *ucur = D.u64[A.cur];
  double xi[3], ui[3];
  ld_node<DIM>(D.pos64, i, xi);
  ld_node<DIM>(ucur, i, ui);
  const int *colp = D.sell_cols + D.sell_ptr[i >> 5] + 4 * (i & 31);
  const int len = D.rowlen[i];
  const double mi = D.mw64[i];
  const double c = DIM == 2 ? 2. : 3.;
  const double fac = DIM == 2 ? P.es_factor2D : 1.;
  double th = 0.;
  uint32_t word = 0;
  bool dirty = false;
  int chunk = 0;
  for (int k = 0; k < len; k++) {
    if ((k & 31) == 0) {
      if (dirty) D.bits[(int64_t)chunk * P.npad + i] = word;
      chunk = k >> 5;
      word = D.bits[(int64_t)chunk * P.npad + i];
      dirty = false;
    }
    const int j = __ldg(colp + (k >> 2) * 128 + (k & 3));
    double xj[3], uj[3], Y[3], Xl, e;
    ld_node<DIM>(D.pos64, j, xj);
    ld_node<DIM>(ucur, j, uj);
    es_geom64<DIM>(xi, ui, xj, uj, Y, Xl, e);
    bool fs = (word >> (k & 31)) & 1u;
    if (P.es_sc > 0. && !fs && dGT(e / Xl, P.es_sc)) {
      fs = true;
      word |= 1u << (k & 31);
      dirty = true;
    }
    if (fs) continue;
    th += (c / mi) * fac * 1. * Xl * e * es_omega(P, Xl) * D.vol64[j];
  }
  if (dirty) D.bits[(int64_t)chunk * P.npad + i] = word;
  D.theta64[i] = th;
}

template <int DIM, int SCHEME>
__global__ void __launch_bounds__(128)
    k_es_force64(const StepParams P, const DevPtrs D, const BCTable T, const StepArgs A) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  const double *ucur = D.u64[A.cur];
  double xi[3], ui[3];
  ld_node<DIM>(D.pos64, i, xi);
  ld_node<DIM>(ucur, i, ui);
  const uint8_t fl = D.flags[i];
  const int *colp = D.sell_cols + D.sell_ptr[i >> 5] + 4 * (i & 31);
  const int len = D.rowlen[i];
  const double mi = D.mw64[i], thi = D.theta64[i];
  double fi[3] = {0., 0., 0.};
  uint32_t word = 0;
  for (int k = 0; k < len; k++) {
    if ((k & 31) == 0) word = D.bits[(int64_t)(k >> 5) * P.npad + i];
    if ((word >> (k & 31)) & 1u) continue;
    const int j = __ldg(colp + (k >> 2) * 128 + (k & 3));
    double xj[3], uj[3], Y[3], Xl, e;
    ld_node<DIM>(D.pos64, j, xj);
    ld_node<DIM>(ucur, j, uj);
    es_geom64<DIM>(xi, ui, xj, uj, Y, Xl, e);
    const double Yl = sqrt(Y[0] * Y[0] + Y[1] * Y[1] + Y[2] * Y[2]);
    const double tsum =
        es_t64<DIM>(P, mi, thi, e, Xl) + es_t64<DIM>(P, D.mw64[j], D.theta64[j], e, Xl);
    const double s = tsum * es_omega(P, Xl) * D.vol64[j];
    fi[0] = fi[0] + (Y[0] / Yl) * s;
    fi[1] = fi[1] + (Y[1] / Yl) * s;
    if (DIM == 3) fi[2] = fi[2] + (Y[2] / Yl) * s;
  }
  if (A.first)
    integrate_node64<DIM, SCHEME, true>(P, D, T, A, i, fl, ui, fi);
  else
    integrate_node64<DIM, SCHEME, false>(P, D, T, A, i, fl, ui, fi);
}

template <int DIM>
static cudaError_t es64(const StepParams &P, const DevPtrs &D, const BCTable &T,
                        const StepArgs &a, cudaStream_t s) {
  const unsigned g = (unsigned)((P.n + 127) / 128);
  k_es_dil64<DIM><<<g, 128, 0, s>>>(P, D, a);
  if (P.scheme == NLM_VELOCITY_VERLET)
    k_es_force64<DIM, NLM_VELOCITY_VERLET><<<g, 128, 0, s>>>(P, D, T, a);
  else
    k_es_force64<DIM, NLM_CENTRAL_DIFFERENCE><<<g, 128, 0, s>>>(P, D, T, a);
  return cudaGetLastError();
}

cudaError_t launch_es_step_fp64(const StepParams &P, const DevPtrs &D, const BCTable &T,
                                const StepArgs &a, int decomp, cudaStream_t s) {
  (void)decomp;
  if (P.n == 0) return cudaSuccess;
  return P.dim == 2 ? es64<2>(P, D, T, a, s) : es64<3>(P, D, T, a, s);
}

cudaError_t launch_es_setup(const StepParams &P, const DevPtrs &D, double *mw, cudaStream_t s) {
  if (P.n == 0) return cudaSuccess;
  const unsigned g = (unsigned)((P.n + 127) / 128);
  if (P.dim == 2)
    k_es_mw<2><<<g, 128, 0, s>>>(P, D, mw);
  else
    k_es_mw<3><<<g, 128, 0, s>>>(P, D, mw);
  return cudaGetLastError();
}

}  // namespace nlm
