// esqs.cu -- the quasi-static ElasticState model (QuasiStaticModel<ElasticState>,
// src/model/quasistatic/QuasiStaticModel.cpp) on the GPU: force density,
// residual, the finite-difference Jacobian of assembly_jacobian_matrix_part
// (:361-454) and a BiCGSTAB solve over it.
//
// Nodes are in the handle's internal order with S doubles per node (S = 2 in
// 2-D and for 1-D meshes, whose y coordinate is zero; S = 4 in 3-D).  The
// material law uses the model dimension mdim (1, 2 or 3); components at or
// above mdim, and the components a Displacement_BC prescribes, are fixed dofs.
// A fixed dof is not an unknown: its residual entry is 0 and its Jacobian row
// and column are the identity's.
//
// Forces follow the gather form f_i = sum_j (t_ij + t_ji) M_ij omega_ij V_j of
// the reference's scatter (QuasiStaticModel.cpp:168-239, ElasticState::getBondEF,
// ElasticState.cpp:160-271); no bond breaks in the quasi-static model.
// Compiled with --fmad=false; sums run in neighbour-list order.

#include <algorithm>

#include "es_common.cuh"
#include "esqs_internal.h"
#include "state_io.cuh"

namespace nlm {

namespace {

__device__ __forceinline__ bool dof_fixed(uint8_t fl, int d, int mdim) {
  return d >= mdim || ((fl >> d) & 1u);
}

// Force state t for the model dimension; 1-D: alpha = E / m_i, t = alpha e
// (ElasticState.cpp:172-189).
__device__ __forceinline__ double esqs_t(const StepParams &P, int mdim, double mi, double th,
                                         double e, double Xl) {
  if (mdim == 1) {
    const double alpha = P.es_E / mi;
    return alpha * 1. * e;
  }
  return mdim == 2 ? es_t64<2>(P, mi, th, e, Xl) : es_t64<3>(P, mi, th, e, Xl);
}

// Node i's displacement with component pc of node pj moved by pe (pj < 0:
// no perturbation).
template <int SD>
__device__ __forceinline__ void ld_u(const double *u, int64_t i, int64_t pj, int pc, double pe,
                                     double o[3]) {
  ld_node_rw<SD>(u, i, o);
  if (i == pj) o[pc] = o[pc] + pe;
}

// Dilatation theta_i (stateBasedHelperFunctions.cpp:26-83, every bond):
// theta_i = sum_j (c / m_i) f2 |X| e omega V_j, c = mdim, f2 = factor2D in 2-D.
template <int SD>
__device__ double theta_node(const StepParams &P, const DevPtrs &D, int mdim, const double *u,
                             int64_t i, int64_t pj, int pc, double pe) {
  double xi[3], ui[3];
  ld_node<SD>(D.pos64, i, xi);
  ld_u<SD>(u, i, pj, pc, pe, ui);
  const double mi = D.mw64[i];
  const double c = (double)mdim;
  double th = 0.;
  for (int64_t k = D.rowptr[i]; k < D.rowptr[i + 1]; k++) {
    const int j = D.cols[k];
    double xj[3], uj[3], Y[3], Xl, e;
    ld_node<SD>(D.pos64, j, xj);
    ld_u<SD>(u, j, pj, pc, pe, uj);
    es_geom64<SD>(xi, ui, xj, uj, Y, Xl, e);
    if (mdim == 2)
      th += (c / mi) * P.es_factor2D * 1. * Xl * e * es_omega(P, Xl) * D.vol64[j];
    else
      th += (c / mi) * 1. * Xl * e * es_omega(P, Xl) * D.vol64[j];
  }
  return th;
}

template <int SD>
__global__ void k_esqs_theta(const StepParams P, const DevPtrs D, int mdim, const double *u,
                             double *theta) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  theta[i] = theta_node<SD>(P, D, mdim, u, i, -1, 0, 0.);
}

template <int SD>
__global__ void k_esqs_force(const StepParams P, const DevPtrs D, int mdim, const double *u,
                             const double *theta, double *f) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  double xi[3], ui[3];
  ld_node<SD>(D.pos64, i, xi);
  ld_node_rw<SD>(u, i, ui);
  const double mi = D.mw64[i], thi = theta[i];
  double fi[3] = {0., 0., 0.};
  for (int64_t k = D.rowptr[i]; k < D.rowptr[i + 1]; k++) {
    const int j = D.cols[k];
    double xj[3], uj[3], Y[3], Xl, e;
    ld_node<SD>(D.pos64, j, xj);
    ld_node_rw<SD>(u, j, uj);
    es_geom64<SD>(xi, ui, xj, uj, Y, Xl, e);
    const double Yl = sqrt(Y[0] * Y[0] + Y[1] * Y[1] + Y[2] * Y[2]);
    const double tsum = esqs_t(P, mdim, mi, thi, e, Xl) + esqs_t(P, mdim, D.mw64[j], theta[j], e, Xl);
    const double s = tsum * es_omega(P, Xl) * D.vol64[j];
    for (int d = 0; d < 3; d++) fi[d] = fi[d] + (Y[d] / Yl) * s;
  }
  st_node<SD>(f, i, fi);
}

// r = f + b on free dofs, 0 on fixed ones (QuasiStaticModel::computeResidual,
// :596-646).
template <int SD>
__global__ void k_esqs_residual(int64_t n, const uint8_t *flags, int mdim, const double *f,
                                const double *b, double *r) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  constexpr int S = SD == 2 ? 2 : 4;
  const uint8_t fl = flags[i];
  for (int d = 0; d < S; d++) {
    const int64_t q = S * i + d;
    r[q] = (d < 3 && !dof_fixed(fl, d, mdim)) ? f[q] + b[q] : 0.;
  }
}

// Force on node i with component pc of node pj moved by pe, every quantity
// recomputed the way k_esqs_theta and k_esqs_force compute it.
template <int SD>
__device__ void force_node(const StepParams &P, const DevPtrs &D, int mdim, const double *u,
                           int64_t i, int64_t pj, int pc, double pe, double fo[3]) {
  double xi[3], ui[3];
  ld_node<SD>(D.pos64, i, xi);
  ld_u<SD>(u, i, pj, pc, pe, ui);
  const double mi = D.mw64[i];
  const double thi = theta_node<SD>(P, D, mdim, u, i, pj, pc, pe);
  double fi[3] = {0., 0., 0.};
  for (int64_t k = D.rowptr[i]; k < D.rowptr[i + 1]; k++) {
    const int j = D.cols[k];
    double xj[3], uj[3], Y[3], Xl, e;
    ld_node<SD>(D.pos64, j, xj);
    ld_u<SD>(u, j, pj, pc, pe, uj);
    es_geom64<SD>(xi, ui, xj, uj, Y, Xl, e);
    const double Yl = sqrt(Y[0] * Y[0] + Y[1] * Y[1] + Y[2] * Y[2]);
    const double thj = theta_node<SD>(P, D, mdim, u, j, pj, pc, pe);
    const double tsum = esqs_t(P, mdim, mi, thi, e, Xl) + esqs_t(P, mdim, D.mw64[j], thj, e, Xl);
    const double s = tsum * es_omega(P, Xl) * D.vol64[j];
    for (int d = 0; d < 3; d++) fi[d] = fi[d] + (Y[d] / Yl) * s;
  }
  for (int d = 0; d < 3; d++) fo[d] = fi[d];
}

// assembly_jacobian_matrix_part (:361-454): for a row node i and each j in
// {i} U N(i), each free component rr of j: central difference of f_i with
// u_j[rr] moved by +-eps.  full = 0 keeps the entries (i, rr; j, rr) only, as
// the reference does; full = 1 keeps the whole 3 x 3 block.  Block b of row i
// (b = 0: the node itself, b = 1 + k: its k-th neighbour) is stored row-major
// at J[9 (rowptr[i] + i + b)].  One CTA per row node.
template <int SD>
__global__ void k_esqs_jacobian(const StepParams P, const DevPtrs D, int mdim, int full,
                                const double *u, double eps, double *J) {
  const int64_t i = blockIdx.x;
  if (i >= P.n) return;
  const uint8_t fli = D.flags[i];
  bool any_free = false;
  for (int d = 0; d < mdim; d++) any_free = any_free || !dof_fixed(fli, d, mdim);
  if (!any_free) return;
  const int64_t r0 = D.rowptr[i];
  const int len = (int)(D.rowptr[i + 1] - r0);
  const int64_t base = r0 + i;
  const int pairs = (len + 1) * mdim;
  for (int t = threadIdx.x; t < pairs; t += blockDim.x) {
    const int b = t / mdim, rr = t % mdim;
    const int64_t j = b == 0 ? i : (int64_t)D.cols[r0 + b - 1];
    if (dof_fixed(D.flags[j], rr, mdim)) continue;
    double fp[3], fm[3];
    force_node<SD>(P, D, mdim, u, i, j, rr, eps, fp);
    force_node<SD>(P, D, mdim, u, i, j, rr, -eps, fm);
    double *blk = J + 9 * (base + b);
    for (int ss = 0; ss < mdim; ss++) {
      if (!full && ss != rr) continue;
      if (dof_fixed(fli, ss, mdim)) continue;
      blk[3 * ss + rr] = (fp[ss] - fm[ss]) / (2. * eps);
    }
  }
}

// y = J x over the dofs (identity on fixed ones).
template <int SD>
__global__ void k_esqs_spmv(int64_t n, const DevPtrs D, int mdim, const double *J,
                            const double *x, double *y) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  constexpr int S = SD == 2 ? 2 : 4;
  const uint8_t fl = D.flags[i];
  const int64_t r0 = D.rowptr[i];
  const int len = (int)(D.rowptr[i + 1] - r0);
  const int64_t base = r0 + i;
  double acc[3] = {0., 0., 0.};
  for (int b = 0; b <= len; b++) {
    const int64_t j = b == 0 ? i : (int64_t)D.cols[r0 + b - 1];
    const double *blk = J + 9 * (base + b);
    for (int rr = 0; rr < mdim; rr++) {
      const double xv = x[S * j + rr];
      for (int ss = 0; ss < mdim; ss++) acc[ss] = acc[ss] + blk[3 * ss + rr] * xv;
    }
  }
  for (int d = 0; d < S; d++) {
    const int64_t q = S * i + d;
    y[q] = (d < 3 && !dof_fixed(fl, d, mdim)) ? acc[d] : x[q];
  }
}

// out = a x + b y + c z (any of y, z may be NULL).
__global__ void k_lin3(int64_t m, double a, const double *x, double b, const double *y, double c,
                       const double *z, double *out) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= m) return;
  double v = a * x[q];
  if (y) v = v + b * y[q];
  if (z) v = v + c * z[q];
  out[q] = v;
}

__global__ void k_esqs_dot(int64_t m, const double *a, const double *b, double *part) {
  __shared__ double sh[256];
  double s = 0.;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < m;
       q += (int64_t)gridDim.x * blockDim.x)
    s += a[q] * b[q];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void k_esqs_sum(const double *part, int nparts, double *out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double s = 0.;
  for (int k = 0; k < nparts; k++) s += part[k];
  *out = s;
}

unsigned blocks_of(int64_t m, int bs) { return (unsigned)((m + bs - 1) / bs); }

}  // namespace

cudaError_t esqs_force(const StepParams &P, const DevPtrs &D, int S, int mdim, const double *u,
                       double *theta, double *f, cudaStream_t s) {
  if (P.n == 0) return cudaSuccess;
  const unsigned g = blocks_of(P.n, 128);
  if (S == 2) {
    k_esqs_theta<2><<<g, 128, 0, s>>>(P, D, mdim, u, theta);
    k_esqs_force<2><<<g, 128, 0, s>>>(P, D, mdim, u, theta, f);
  } else {
    k_esqs_theta<3><<<g, 128, 0, s>>>(P, D, mdim, u, theta);
    k_esqs_force<3><<<g, 128, 0, s>>>(P, D, mdim, u, theta, f);
  }
  return cudaGetLastError();
}

cudaError_t esqs_residual(const StepParams &P, const DevPtrs &D, int S, int mdim,
                          const double *f, const double *b, double *r, cudaStream_t s) {
  if (P.n == 0) return cudaSuccess;
  const unsigned g = blocks_of(P.n, 256);
  if (S == 2)
    k_esqs_residual<2><<<g, 256, 0, s>>>(P.n, D.flags, mdim, f, b, r);
  else
    k_esqs_residual<3><<<g, 256, 0, s>>>(P.n, D.flags, mdim, f, b, r);
  return cudaGetLastError();
}

cudaError_t esqs_jacobian(const StepParams &P, const DevPtrs &D, int S, int mdim, int full,
                          const double *u, double eps, double *J, int64_t nblocks,
                          cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(J, 0, sizeof(double) * 9 * nblocks, s);
  if (e != cudaSuccess || P.n == 0) return e;
  if (S == 2)
    k_esqs_jacobian<2><<<(unsigned)P.n, 128, 0, s>>>(P, D, mdim, full, u, eps, J);
  else
    k_esqs_jacobian<3><<<(unsigned)P.n, 128, 0, s>>>(P, D, mdim, full, u, eps, J);
  return cudaGetLastError();
}

cudaError_t esqs_spmv(const StepParams &P, const DevPtrs &D, int S, int mdim, const double *J,
                      const double *x, double *y, cudaStream_t s) {
  if (P.n == 0) return cudaSuccess;
  const unsigned g = blocks_of(P.n, 128);
  if (S == 2)
    k_esqs_spmv<2><<<g, 128, 0, s>>>(P.n, D, mdim, J, x, y);
  else
    k_esqs_spmv<3><<<g, 128, 0, s>>>(P.n, D, mdim, J, x, y);
  return cudaGetLastError();
}

cudaError_t esqs_lin3(int64_t m, double a, const double *x, double b, const double *y, double c,
                      const double *z, double *out, cudaStream_t s) {
  if (m == 0) return cudaSuccess;
  k_lin3<<<blocks_of(m, 256), 256, 0, s>>>(m, a, x, b, y, c, z, out);
  return cudaGetLastError();
}

cudaError_t esqs_dot(int64_t m, const double *a, const double *b, double *part, double *out,
                     cudaStream_t s) {
  const int nparts = (int)std::min<int64_t>(kEsqsDotParts, std::max<int64_t>(1, (m + 255) / 256));
  k_esqs_dot<<<nparts, 256, 0, s>>>(m, a, b, part);
  k_esqs_sum<<<1, 32, 0, s>>>(part, nparts, out);
  return cudaGetLastError();
}

}  // namespace nlm
