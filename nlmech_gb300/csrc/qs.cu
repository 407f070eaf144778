// qs.cu -- quasi-static Newton solve for RNPBond plates (FP64).
//
// The reference's QuasiStaticModel (src/model/quasistatic/QuasiStaticModel.cpp)
// exists only for ElasticState, with a dense finite-difference Jacobian
// ((N dim)^2 entries, :128-132, :361-454) that does not fit a 40,000-node
// plate.  This solver keeps its load-step / Newton structure (solver :526-594:
// apply loads, residual on free dofs, Newton until the residual norm is below
// tolerance, u += du) with
//   * the residual r = f(u) of FDModel::computeForce (fDModel.cpp:543-582)
//     on free dofs,
//   * the analytic tangent of RNPBond's bond force: for an intact bond with
//     F = k g(S) e, g(S) = S exp(-beta r S^2), S = e.eta / r,
//       dF/du_j = -dF/du_i = A_ij = k g'(S) / r e e^T,
//       g'(S) = (1 - 2 beta r S^2) exp(-beta r S^2),
//     so (-K x)_i = sum_j A_ij (x_i - x_j); 2x2 (or 3x3) symmetric blocks are
//     stored per bond,
//   * block-Jacobi preconditioned conjugate gradients (the reference's
//     default solver tag) on the free dofs, all scalars kept on the device.
// Bonds break as in RNPBond::getBondEF (:263-266): every residual evaluation
// of a Newton iteration marks intact bonds past the critical strain broken and
// leaves them out of that residual.
//
// A load step starts with the displacement-controlled tangent predictor: with
// the tangent K at the previous converged state u and the boundary increment
// du_c, solve K_ff du_f = -(f + K du_c)_f.  (Evaluating f at u + du_c instead
// would put the bonds next to the loaded layer far past the peak of the RNP
// force, where the force, the residual and the stiffness all vanish.)  The
// norm of that right-hand side is the step's residual scale: Newton stops at
// ||f|| <= tol * ||f + K du_c||.  Softening bonds (1 - 2 beta r S^2 < 0)
// are left out of the tangent so the preconditioned CG matrix stays SPD.

#include "fd_internal.h"
#include "qs_internal.h"
#include "state_io.cuh"

namespace nlm {

// Bond quantities shared by the residual and tangent kernels.
template <int DIM>
__device__ __forceinline__ void qs_bond(const StepParams &P, const double xi[3], const double ui[3],
                                        const double xj[3], const double uj[3], double volj,
                                        double e[3], double &r, double &S, double &k,
                                        double &ex) {
  double dx = xj[0] - xi[0], dy = xj[1] - xi[1], dz = DIM == 3 ? xj[2] - xi[2] : 0.;
  double rr = dx * dx + dy * dy;
  if (DIM == 3) rr = rr + dz * dz;
  r = sqrt(rr);
  double dotp = dx * (uj[0] - ui[0]) + dy * (uj[1] - ui[1]);
  if (DIM == 3) dotp = dotp + dz * (uj[2] - ui[2]);
  S = dotp / rr;
  e[0] = dx / r;
  e[1] = dy / r;
  e[2] = dz / r;
  if (dGT(r, P.check_low)) volj = volj * ((P.check_up - r) / P.h);
  const double infl = influence_d(P, r / P.delta);
  k = infl * 4. * P.C * P.beta / P.invF * volj;
  ex = exp(-P.beta * r * S * S);
}

// Residual (force density on free dofs, zero on fixed dofs); with asm, also
// the tangent blocks of every bond (lower triangle, row-major) and the
// diagonal blocks sum_j A_ij.  Broken bonds contribute nothing.
template <int DIM, bool ASM, bool UPD>
__global__ void k_qs_force(const StepParams P, const DevPtrs D, const double *u, double *res,
                           double *blk, double *dblk, unsigned long long *count) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  constexpr int NB = DIM == 2 ? 3 : 6;
  double xi[3], ui[3];
  ld_node<DIM>(D.pos64, i, xi);
  ld_node<DIM>(u, i, ui);
  const uint8_t fl = D.flags[i];
  const int64_t r0 = D.rowptr[i], r1 = D.rowptr[i + 1];
  double fi[3] = {0., 0., 0.};
  double di[6] = {0., 0., 0., 0., 0., 0.};
  int newly = 0;
  for (int64_t q = r0; q < r1; q++) {
    const int kk = (int)(q - r0);
    const int64_t w = (int64_t)(kk >> 5) * P.npad + i;
    const bool fs = (D.bits[w] >> (kk & 31)) & 1u;
    const bool breakable = !(P.nofail && ((fl & FLAG_NOFAIL) || (D.flags[D.cols[q]] & FLAG_NOFAIL)));
    if (fs && breakable) {
      if (ASM)
        for (int c = 0; c < NB; c++) blk[NB * q + c] = 0.;
      continue;
    }
    const int j = D.cols[q];
    double xj[3], uj[3], e[3], r, S, k, ex;
    ld_node<DIM>(D.pos64, j, xj);
    ld_node<DIM>(u, j, uj);
    qs_bond<DIM>(P, xi, ui, xj, uj, D.vol64[j], e, r, S, k, ex);
    if (UPD && breakable && P.irrev && dGT(fabs(S), P.fsc * (P.rbar / sqrt(r)))) {
      D.bits[w] |= 1u << (kk & 31);  // row i is owned by this thread
      newly++;
      if (ASM)
        for (int c = 0; c < NB; c++) blk[NB * q + c] = 0.;
      continue;
    }
    const double s = breakable ? k * S * ex : k * S;
    for (int c = 0; c < DIM; c++) fi[c] += s * e[c];
    if (ASM) {
      const double gp =
          breakable ? k * fmax(1. - 2. * P.beta * r * S * S, 0.) * ex / r : k / r;
      double a[6];
      a[0] = gp * e[0] * e[0];
      a[1] = gp * e[1] * e[0];
      a[2] = gp * e[1] * e[1];
      if (DIM == 3) {
        a[3] = gp * e[2] * e[0];
        a[4] = gp * e[2] * e[1];
        a[5] = gp * e[2] * e[2];
      }
      for (int c = 0; c < NB; c++) {
        blk[NB * q + c] = a[c];
        di[c] += a[c];
      }
    }
  }
  double f[3] = {fi[0], fi[1], fi[2]};
  if (fl & FLAG_FBC) {
    double fe[3];
    ld_node<DIM>(D.fext, i, fe);
    for (int c = 0; c < DIM; c++) f[c] = fe[c] + fi[c];
  }
  for (int c = 0; c < DIM; c++) res[DIM * i + c] = (fl >> c & 1) ? 0. : f[c];
  if (ASM) {
    // relative Levenberg term: keeps blocks of nodes whose remaining bonds
    // are collinear (or gone) invertible
    const double reg = 1e-8 * (DIM == 2 ? 0.5 * (di[0] + di[2]) : (di[0] + di[2] + di[5]) / 3.);
    di[0] += reg;
    di[2] += reg;
    if (DIM == 3) di[5] += reg;
    for (int c = 0; c < NB; c++) dblk[NB * i + c] = di[c];
  }
  if (UPD && newly) atomicAdd(count, (unsigned long long)newly);
}

__device__ __forceinline__ void sym_mul(int dim, const double *a, const double *x, double *y) {
  if (dim == 2) {
    y[0] = a[0] * x[0] + a[1] * x[1];
    y[1] = a[1] * x[0] + a[2] * x[1];
  } else {
    y[0] = a[0] * x[0] + a[1] * x[1] + a[3] * x[2];
    y[1] = a[1] * x[0] + a[2] * x[1] + a[4] * x[2];
    y[2] = a[3] * x[0] + a[4] * x[1] + a[5] * x[2];
  }
}

// Block reduction of one double per thread into part[blockIdx.x].
__device__ __forceinline__ void block_sum(double v, double *part) {
  __shared__ double sh[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  if (w == 0) {
    v = l < (int)(blockDim.x >> 5) ? sh[l] : 0.;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (l == 0) part[blockIdx.x] = v;
  }
}

// y = (-K) x on free dofs (fixed dofs give 0), plus the partial sums of x.y.
template <int DIM>
__global__ void k_qs_spmv(const StepParams P, const DevPtrs D, const double *blk,
                          const double *dblk, const double *x, double *y, double *part) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  constexpr int NB = DIM == 2 ? 3 : 6;
  double dot = 0.;
  if (i < P.n) {
    const uint8_t fl = D.flags[i];
    double xi[3] = {0., 0., 0.}, acc[3] = {0., 0., 0.};
    for (int c = 0; c < DIM; c++) xi[c] = x[DIM * i + c];
    double t[3];
    sym_mul(DIM, dblk + NB * i, xi, acc);
    for (int64_t q = D.rowptr[i]; q < D.rowptr[i + 1]; q++) {
      const int j = D.cols[q];
      double xj[3] = {0., 0., 0.};
      for (int c = 0; c < DIM; c++) xj[c] = x[DIM * j + c];
      sym_mul(DIM, blk + NB * q, xj, t);
      for (int c = 0; c < DIM; c++) acc[c] -= t[c];
    }
    for (int c = 0; c < DIM; c++) {
      const double yc = (fl >> c & 1) ? 0. : acc[c];
      y[DIM * i + c] = yc;
      dot += xi[c] * yc;
    }
  }
  block_sum(dot, part);
}

// Block-Jacobi preconditioner: z_i = (D_i)^-1 r_i on the free dofs of node i
// (fixed dofs removed from the block), plus partial sums of r.z.
template <int DIM>
__global__ void k_qs_precond(const StepParams P, const DevPtrs D, const double *dblk,
                             const double *r, double *z, double *part) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  constexpr int NB = DIM == 2 ? 3 : 6;
  double dot = 0.;
  if (i < P.n) {
    const uint8_t fl = D.flags[i];
    double a[9];  // full block
    const double *b = dblk + NB * i;
    if (DIM == 2) {
      a[0] = b[0]; a[1] = b[1]; a[2] = b[1]; a[3] = b[2];
    } else {
      a[0] = b[0]; a[1] = b[1]; a[2] = b[3];
      a[3] = b[1]; a[4] = b[2]; a[5] = b[4];
      a[6] = b[3]; a[7] = b[4]; a[8] = b[5];
    }
    // remove fixed dofs: identity rows / columns
    for (int c = 0; c < DIM; c++)
      if (fl >> c & 1)
        for (int q = 0; q < DIM; q++) {
          a[c * DIM + q] = (c == q) ? 1. : 0.;
          a[q * DIM + c] = (c == q) ? 1. : 0.;
        }
    double rv[3] = {0., 0., 0.}, zv[3] = {0., 0., 0.};
    for (int c = 0; c < DIM; c++) rv[c] = (fl >> c & 1) ? 0. : r[DIM * i + c];
    if (DIM == 2) {
      const double det = a[0] * a[3] - a[1] * a[2];
      if (fabs(det) > 0.) {
        zv[0] = (a[3] * rv[0] - a[1] * rv[1]) / det;
        zv[1] = (-a[2] * rv[0] + a[0] * rv[1]) / det;
      }
    } else {
      const double c00 = a[4] * a[8] - a[5] * a[7], c01 = a[5] * a[6] - a[3] * a[8],
                   c02 = a[3] * a[7] - a[4] * a[6];
      const double det = a[0] * c00 + a[1] * c01 + a[2] * c02;
      if (fabs(det) > 0.) {
        const double inv[9] = {c00, a[2] * a[7] - a[1] * a[8], a[1] * a[5] - a[2] * a[4],
                               c01, a[0] * a[8] - a[2] * a[6], a[2] * a[3] - a[0] * a[5],
                               c02, a[1] * a[6] - a[0] * a[7], a[0] * a[4] - a[1] * a[3]};
        for (int c = 0; c < 3; c++)
          zv[c] = (inv[3 * c] * rv[0] + inv[3 * c + 1] * rv[1] + inv[3 * c + 2] * rv[2]) / det;
      }
    }
    for (int c = 0; c < DIM; c++) {
      z[DIM * i + c] = zv[c];
      dot += rv[c] * zv[c];
    }
  }
  block_sum(dot, part);
}

// Sum of partials in a fixed order (deterministic): out = sum part[0..n).
__global__ void k_qs_sum(const double *part, int64_t n, double *out) {
  double v = 0.;
  for (int64_t k = threadIdx.x; k < n; k += blockDim.x) v += part[k];
  __shared__ double sh[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  if (w == 0) {
    v = l < (int)(blockDim.x >> 5) ? sh[l] : 0.;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (l == 0) *out = v;
  }
}

// x += alpha p, r -= alpha Ap with alpha = rz / pAp (device scalars).
__global__ void k_qs_axpy(int64_t m, const double *s_rz, const double *s_pap, const double *p,
                          const double *ap, double *x, double *r) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= m) return;
  const double pap = *s_pap;
  const double alpha = pap != 0. ? *s_rz / pap : 0.;
  x[k] += alpha * p[k];
  r[k] -= alpha * ap[k];
}

// p = z + beta p with beta = rz_new / rz_old; then rz_old = rz_new (thread 0).
__global__ void k_qs_pupdate(int64_t m, const double *s_rznew, double *s_rzold, const double *z,
                             double *p) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= m) return;
  const double old = *s_rzold;
  const double beta = old != 0. ? *s_rznew / old : 0.;
  p[k] = z[k] + beta * p[k];
}
__global__ void k_qs_copy_scalar(const double *src, double *dst) { *dst = *src; }

// Bonds of the converged state that exceed the critical strain break.
template <int DIM>
__global__ void k_qs_break(const StepParams P, const DevPtrs D, const double *u,
                           unsigned long long *count) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  double xi[3], ui[3];
  ld_node<DIM>(D.pos64, i, xi);
  ld_node<DIM>(u, i, ui);
  const uint8_t fl = D.flags[i];
  const int64_t r0 = D.rowptr[i], r1 = D.rowptr[i + 1];
  int newly = 0;
  for (int64_t q = r0; q < r1; q++) {
    const int kk = (int)(q - r0);
    const int64_t w = (int64_t)(kk >> 5) * P.npad + i;
    const uint32_t word = D.bits[w];
    if ((word >> (kk & 31)) & 1u) continue;
    const int j = D.cols[q];
    if (P.nofail && ((fl & FLAG_NOFAIL) || (D.flags[j] & FLAG_NOFAIL))) continue;
    double xj[3], uj[3], e[3], r, S, k, ex;
    ld_node<DIM>(D.pos64, j, xj);
    ld_node<DIM>(u, j, uj);
    qs_bond<DIM>(P, xi, ui, xj, uj, D.vol64[j], e, r, S, k, ex);
    if (P.irrev && dGT(fabs(S), P.fsc * (P.rbar / sqrt(r)))) {
      D.bits[w] = word | (1u << (kk & 31));
      newly++;
    }
  }
  if (newly) atomicAdd(count, (unsigned long long)newly);
}

// u_full (S doubles per node) <-> dof vectors (DIM per node).
template <int DIM>
__global__ void k_qs_add(int64_t n, const double *du, double *u) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int c = 0; c < DIM; c++) u[(DIM == 2 ? 2 : 4) * i + c] += du[DIM * i + c];
}

static unsigned qblk(int64_t n) { return (unsigned)((n + 255) / 256); }

template <int DIM>
static void qs_force_dim(const StepParams &P, const DevPtrs &D, const double *u, double *res,
                         double *blk, double *dblk, bool assemble, unsigned long long *count,
                         cudaStream_t s) {
  if (assemble && count)
    k_qs_force<DIM, true, true><<<qblk(P.n), 256, 0, s>>>(P, D, u, res, blk, dblk, count);
  else if (assemble)
    k_qs_force<DIM, true, false><<<qblk(P.n), 256, 0, s>>>(P, D, u, res, blk, dblk, count);
  else if (count)
    k_qs_force<DIM, false, true><<<qblk(P.n), 256, 0, s>>>(P, D, u, res, blk, dblk, count);
  else
    k_qs_force<DIM, false, false><<<qblk(P.n), 256, 0, s>>>(P, D, u, res, blk, dblk, count);
}

cudaError_t qs_residual(const StepParams &P, const DevPtrs &D, const double *u, double *res,
                        double *blk, double *dblk, bool assemble, cudaStream_t s,
                        unsigned long long *count) {
  if (P.n == 0) return cudaSuccess;
  if (P.dim == 2)
    qs_force_dim<2>(P, D, u, res, blk, dblk, assemble, count, s);
  else
    qs_force_dim<3>(P, D, u, res, blk, dblk, assemble, count, s);
  return cudaGetLastError();
}

cudaError_t qs_dot(const double *a, const double *b, int64_t m, double *part, double *out,
                   cudaStream_t s);

__global__ void k_qs_dot(int64_t m, const double *a, const double *b, double *part) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  block_sum(k < m ? a[k] * b[k] : 0., part);
}

cudaError_t qs_dot(const double *a, const double *b, int64_t m, double *part, double *out,
                   cudaStream_t s) {
  const unsigned g = qblk(m);
  k_qs_dot<<<g, 256, 0, s>>>(m, a, b, part);
  k_qs_sum<<<1, 256, 0, s>>>(part, g, out);
  return cudaGetLastError();
}

// Preconditioned CG on (-K) dx = r (free dofs).  Scalars: sc[0] = rz_old,
// sc[1] = pAp, sc[2] = rz_new, sc[3] = r.r (convergence check).
cudaError_t qs_cg(const StepParams &P, const DevPtrs &D, const QSWork &W, const double *rhs,
                  double *dx, double tol, int max_iters, int check_every, int *iters,
                  cudaStream_t s) {
  const int dim = P.dim;
  const int64_t m = (int64_t)dim * P.n;
  const unsigned gn = qblk(P.n), gm = qblk(m);
  cudaError_t e;
  // x = 0, r = rhs, z = M^-1 r, p = z
  if ((e = cudaMemsetAsync(dx, 0, sizeof(double) * m, s))) return e;
  if ((e = cudaMemcpyAsync(W.r, rhs, sizeof(double) * m, cudaMemcpyDeviceToDevice, s))) return e;
  auto precond = [&]() {
    if (dim == 2)
      k_qs_precond<2><<<gn, 256, 0, s>>>(P, D, W.dblk, W.r, W.z, W.part);
    else
      k_qs_precond<3><<<gn, 256, 0, s>>>(P, D, W.dblk, W.r, W.z, W.part);
    k_qs_sum<<<1, 256, 0, s>>>(W.part, gn, W.sc + 2);
  };
  precond();
  k_qs_copy_scalar<<<1, 1, 0, s>>>(W.sc + 2, W.sc + 0);
  if ((e = cudaMemcpyAsync(W.p, W.z, sizeof(double) * m, cudaMemcpyDeviceToDevice, s))) return e;
  double rr0 = 0.;
  if ((e = qs_dot(W.r, W.r, m, W.part, W.sc + 3, s))) return e;
  if ((e = cudaMemcpyAsync(&rr0, W.sc + 3, sizeof(double), cudaMemcpyDeviceToHost, s))) return e;
  if ((e = cudaStreamSynchronize(s))) return e;
  const double target = tol * tol * rr0;
  int it = 0;
  if (rr0 == 0.) {
    *iters = 0;
    return cudaSuccess;
  }
  while (it < max_iters) {
    for (int q = 0; q < check_every && it < max_iters; q++, it++) {
      if (dim == 2)
        k_qs_spmv<2><<<gn, 256, 0, s>>>(P, D, W.blk, W.dblk, W.p, W.ap, W.part);
      else
        k_qs_spmv<3><<<gn, 256, 0, s>>>(P, D, W.blk, W.dblk, W.p, W.ap, W.part);
      k_qs_sum<<<1, 256, 0, s>>>(W.part, gn, W.sc + 1);
      k_qs_axpy<<<gm, 256, 0, s>>>(m, W.sc + 0, W.sc + 1, W.p, W.ap, dx, W.r);
      precond();
      k_qs_pupdate<<<gm, 256, 0, s>>>(m, W.sc + 2, W.sc + 0, W.z, W.p);
      k_qs_copy_scalar<<<1, 1, 0, s>>>(W.sc + 2, W.sc + 0);
    }
    double rr = 0.;
    if ((e = qs_dot(W.r, W.r, m, W.part, W.sc + 3, s))) return e;
    if ((e = cudaMemcpyAsync(&rr, W.sc + 3, sizeof(double), cudaMemcpyDeviceToHost, s))) return e;
    if ((e = cudaStreamSynchronize(s))) return e;
    if (!(rr > target)) break;
  }
  *iters = it;
  return cudaGetLastError();
}

// dx = u - u_prev (DIM per node); with fixed_only, 0 on free dofs
template <int DIM>
__global__ void k_qs_bcdiff(int64_t n, const uint8_t *flags, const double *u,
                            const double *uprev, double *dx, bool fixed_only) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int S = DIM == 2 ? 2 : 4;
  for (int c = 0; c < DIM; c++)
    dx[DIM * i + c] =
        (!fixed_only || (flags[i] >> c & 1)) ? u[S * i + c] - uprev[S * i + c] : 0.;
}
__global__ void k_qs_sub(int64_t m, const double *a, const double *b, double *out) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k < m) out[k] = a[k] - b[k];
}

cudaError_t qs_bcdiff(const StepParams &P, const DevPtrs &D, const double *u,
                      const double *uprev, double *dx, bool fixed_only, cudaStream_t s) {
  if (P.dim == 2)
    k_qs_bcdiff<2><<<qblk(P.n), 256, 0, s>>>(P.n, D.flags, u, uprev, dx, fixed_only);
  else
    k_qs_bcdiff<3><<<qblk(P.n), 256, 0, s>>>(P.n, D.flags, u, uprev, dx, fixed_only);
  return cudaGetLastError();
}

cudaError_t qs_spmv(const StepParams &P, const DevPtrs &D, const double *blk, const double *dblk,
                    const double *x, double *y, double *part, cudaStream_t s) {
  if (P.dim == 2)
    k_qs_spmv<2><<<qblk(P.n), 256, 0, s>>>(P, D, blk, dblk, x, y, part);
  else
    k_qs_spmv<3><<<qblk(P.n), 256, 0, s>>>(P, D, blk, dblk, x, y, part);
  return cudaGetLastError();
}

cudaError_t qs_sub(int64_t m, const double *a, const double *b, double *out, cudaStream_t s) {
  k_qs_sub<<<qblk(m), 256, 0, s>>>(m, a, b, out);
  return cudaGetLastError();
}

cudaError_t qs_add(const StepParams &P, const double *du, double *u, cudaStream_t s) {
  if (P.dim == 2)
    k_qs_add<2><<<qblk(P.n), 256, 0, s>>>(P.n, du, u);
  else
    k_qs_add<3><<<qblk(P.n), 256, 0, s>>>(P.n, du, u);
  return cudaGetLastError();
}

cudaError_t qs_break(const StepParams &P, const DevPtrs &D, const double *u,
                     unsigned long long *count, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(count, 0, sizeof(unsigned long long), s);
  if (e) return e;
  if (P.dim == 2)
    k_qs_break<2><<<qblk(P.n), 256, 0, s>>>(P, D, u, count);
  else
    k_qs_break<3><<<qblk(P.n), 256, 0, s>>>(P, D, u, count);
  return cudaGetLastError();
}

}  // namespace nlm
