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

#include <algorithm>
#include <vector>

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

template <typename T>
__device__ __forceinline__ void sym_mul(int dim, const T *a, const T *x, T *y) {
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

// z = (D_i)^-1 r on the free dofs of node i: the diagonal block b (packed
// symmetric) with the rows and columns of fixed dofs replaced by identity;
// rv is zero on fixed dofs.  A singular block gives z = 0.
template <int DIM, typename T>
__device__ __forceinline__ void block_jacobi(const T *b, uint8_t fl, const T rv[3], T zv[3]) {
  T a[9];
  if (DIM == 2) {
    a[0] = b[0]; a[1] = b[1]; a[2] = b[1]; a[3] = b[2];
  } else {
    a[0] = b[0]; a[1] = b[1]; a[2] = b[3];
    a[3] = b[1]; a[4] = b[2]; a[5] = b[4];
    a[6] = b[3]; a[7] = b[4]; a[8] = b[5];
  }
  for (int c = 0; c < DIM; c++)
    if (fl >> c & 1)
      for (int q = 0; q < DIM; q++) {
        a[c * DIM + q] = (c == q) ? T(1) : T(0);
        a[q * DIM + c] = (c == q) ? T(1) : T(0);
      }
  zv[0] = zv[1] = zv[2] = T(0);
  if (DIM == 2) {
    const T det = a[0] * a[3] - a[1] * a[2];
    if (fabs(det) > T(0)) {
      zv[0] = (a[3] * rv[0] - a[1] * rv[1]) / det;
      zv[1] = (-a[2] * rv[0] + a[0] * rv[1]) / det;
    }
  } else {
    const T c00 = a[4] * a[8] - a[5] * a[7], c01 = a[5] * a[6] - a[3] * a[8],
            c02 = a[3] * a[7] - a[4] * a[6];
    const T det = a[0] * c00 + a[1] * c01 + a[2] * c02;
    if (fabs(det) > T(0)) {
      const T inv[9] = {c00, a[2] * a[7] - a[1] * a[8], a[1] * a[5] - a[2] * a[4],
                             c01, a[0] * a[8] - a[2] * a[6], a[2] * a[3] - a[0] * a[5],
                             c02, a[1] * a[6] - a[0] * a[7], a[0] * a[4] - a[1] * a[3]};
      for (int c = 0; c < 3; c++)
        zv[c] = (inv[3 * c] * rv[0] + inv[3 * c + 1] * rv[1] + inv[3 * c + 2] * rv[2]) / det;
    }
  }
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
    double rv[3] = {0., 0., 0.}, zv[3];
    for (int c = 0; c < DIM; c++) rv[c] = (fl >> c & 1) ? 0. : r[DIM * i + c];
    block_jacobi<DIM, double>(dblk + NB * i, fl, rv, zv);
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

// Final stage of a two-stage sum, done by the last block of a launch to
// finish (atomic ticket after a memory fence; no block waits for another).
// The partials are summed in a fixed order (thread t takes t, t + 256, ...,
// then a fixed tree), so the total does not depend on which block is last.
// The ticket counter is reset for the next launch.
__device__ __forceinline__ bool last_block(unsigned *ticket) {
  __shared__ bool is_last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    is_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  return is_last;
}

__device__ __forceinline__ void finish_sums(int nsum, const double *pa, double *ta,
                                            const double *pb, double *tb, unsigned *ticket) {
  __threadfence();
  const int nb = (int)gridDim.x;
  double va = 0., vb = 0.;
  for (int k = threadIdx.x; k < nb; k += blockDim.x) {
    va += __ldcg(pa + k);
    if (nsum > 1) vb += __ldcg(pb + k);
  }
  __shared__ double sh[2][32];
  for (int o = 16; o > 0; o >>= 1) {
    va += __shfl_xor_sync(0xffffffffu, va, o);
    vb += __shfl_xor_sync(0xffffffffu, vb, o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    sh[0][w] = va;
    sh[1][w] = vb;
  }
  __syncthreads();
  if (w == 0) {
    const bool in = l < (int)(blockDim.x >> 5);
    va = in ? sh[0][l] : 0.;
    vb = in ? sh[1][l] : 0.;
    for (int o = 16; o > 0; o >>= 1) {
      va += __shfl_xor_sync(0xffffffffu, va, o);
      vb += __shfl_xor_sync(0xffffffffu, vb, o);
    }
    if (l == 0) {
      *ta = va;
      if (nsum > 1) *tb = vb;
      *ticket = 0u;
    }
  }
}

// Two block sums at once (partials of block blockIdx.x).
__device__ __forceinline__ void block_sum2(double va, double vb, double *pa, double *pb) {
  __shared__ double sh[2][32];
  for (int o = 16; o > 0; o >>= 1) {
    va += __shfl_xor_sync(0xffffffffu, va, o);
    vb += __shfl_xor_sync(0xffffffffu, vb, o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    sh[0][w] = va;
    sh[1][w] = vb;
  }
  __syncthreads();
  if (w == 0) {
    const bool in = l < (int)(blockDim.x >> 5);
    va = in ? sh[0][l] : 0.;
    vb = in ? sh[1][l] : 0.;
    for (int o = 16; o > 0; o >>= 1) {
      va += __shfl_xor_sync(0xffffffffu, va, o);
      vb += __shfl_xor_sync(0xffffffffu, vb, o);
    }
    if (l == 0) {
      pa[blockIdx.x] = va;
      pb[blockIdx.x] = vb;
    }
  }
}

// Lanes per node in the tangent products: a row (about 26 bonds at
// horizon 3h) is split over kG lanes so that a 40,000-node plate still puts
// enough warps on every SM to hide the latency of the neighbour gathers.
constexpr int kG = 8;

// One PCG iteration k in two launches.  Vectors: p_k lives in pbuf[k & 1],
// rz_k = r_k.z_k as partials in rzp[k & 1].
// First launch (DIR): beta = rz_k / rz_{k-1}, p_k = z_k + beta p_{k-1} (own
// rows stored, neighbour values formed on the fly from z and p_{k-1}), Ap_k =
// (-K) p_k, partials of p_k.Ap_k.  Without DIR: y = (-K) x with x = z.
template <int DIM, bool DIR>
__global__ void __launch_bounds__(256) k_cg_dir_spmv(
    int64_t n, const uint8_t *flags, const int64_t *rowptr, const int *cols, const double *blk,
    const double *dblk, const double *z, const double *pold, double *pnew, double *ap,
    const double *rz_cur, const double *rz_prev, double *pap_part, unsigned *ticket,
    double *pap_total) {
  double beta = 0.;
  if (DIR) {
    const double rzc = *rz_cur, rzo = *rz_prev;
    beta = rzo != 0. ? rzc / rzo : 0.;
  }
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t i = t / kG;
  const int g = (int)(t % kG);
  constexpr int NB = DIM == 2 ? 3 : 6;
  double acc[3] = {0., 0., 0.}, tv[3];
  if (i < n) {
    const int64_t q1 = rowptr[i + 1];
    for (int64_t q = rowptr[i] + g; q < q1; q += kG) {
      const int j = cols[q];
      double pj[3] = {0., 0., 0.};
      for (int c = 0; c < DIM; c++)
        pj[c] = DIR ? z[DIM * j + c] + beta * pold[DIM * j + c] : z[DIM * j + c];
      sym_mul(DIM, blk + NB * q, pj, tv);
      for (int c = 0; c < DIM; c++) acc[c] -= tv[c];
    }
  }
  for (int o = kG / 2; o > 0; o >>= 1)
    for (int c = 0; c < DIM; c++) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
  double dot = 0.;
  if (i < n && g == 0) {
    const uint8_t fl = flags[i];
    double pi[3] = {0., 0., 0.};
    for (int c = 0; c < DIM; c++) {
      pi[c] = DIR ? z[DIM * i + c] + beta * pold[DIM * i + c] : z[DIM * i + c];
      if (DIR) pnew[DIM * i + c] = pi[c];
    }
    sym_mul(DIM, dblk + NB * i, pi, tv);
    for (int c = 0; c < DIM; c++) {
      const double yc = (fl >> c & 1) ? 0. : acc[c] + tv[c];
      ap[DIM * i + c] = yc;
      dot += pi[c] * yc;
    }
  }
  block_sum(dot, pap_part);
  if (DIR && last_block(ticket)) finish_sums(1, pap_part, pap_total, nullptr, nullptr, ticket);
}

static unsigned grp_blocks(int64_t n) { return (unsigned)((n * kG + 255) / 256); }

int64_t qs_cg_stride(int64_t n) { return (int64_t)grp_blocks(n) + 2; }

// Second launch: alpha = rz_k / p_k.Ap_k, x += alpha p_k, r -= alpha Ap_k,
// z = (D_i)^-1 r (block Jacobi, fixed dofs removed), partials of
// rz_{k+1} = r.z and of r.r.
template <int DIM>
__global__ void k_cg_update(int64_t n, const uint8_t *flags, const double *dblk,
                            const double *p, const double *ap, double *x, double *r, double *z,
                            const double *rz_cur, const double *pap_total, double *rz_part,
                            double *rr_part, unsigned *ticket, double *rz_next,
                            double *rr_total) {
  const double rzc = *rz_cur, pap = *pap_total;
  const double alpha = pap != 0. ? rzc / pap : 0.;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  constexpr int NB = DIM == 2 ? 3 : 6;
  double drz = 0., drr = 0.;
  if (i < n) {
    const uint8_t fl = flags[i];
    double rv[3] = {0., 0., 0.}, zv[3] = {0., 0., 0.};
    for (int c = 0; c < DIM; c++) {
      const int64_t k = DIM * i + c;
      x[k] += alpha * p[k];
      const double rk = r[k] - alpha * ap[k];
      r[k] = rk;
      drr += rk * rk;
      rv[c] = (fl >> c & 1) ? 0. : rk;
    }
    block_jacobi<DIM, double>(dblk + NB * i, fl, rv, zv);
    for (int c = 0; c < DIM; c++) {
      z[DIM * i + c] = zv[c];
      drz += rv[c] * zv[c];
    }
  }
  block_sum2(drz, drr, rz_part, rr_part);
  if (last_block(ticket)) finish_sums(2, rz_part, rz_next, rr_part, rr_total, ticket);
}

__global__ void k_cg_seed(double *rz_prev, double *pold, int64_t m) {
  // rz_{-1} = 1 and p_{-1} = 0 so that p_0 = z_0
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k < m) pold[k] = 0.;
  if (k == 0) *rz_prev = 1.;
}

// ---- FP32 Krylov solve ---------------------------------------------------
// The Newton correction only has to cut the residual by lin_tol (1e-4), so
// the tangent blocks, the CG vectors, the SpMV and every per-thread
// operation run in FP32: GB300 issues FP64 at a small fraction of its FP32
// rate, and even a few FP64 operations per thread (a step-length division,
// FP64 partial sums) made these launches FP64-pipe bound.  Block sums are
// formed in FP32 and stored as FP64 partials; the sum over blocks and the
// step lengths alpha, beta are computed in FP64 once per launch, by its last
// block.  The residual, its norm and the Newton update u += dx stay FP64.

__global__ void k_to_f32(int64_t n, const double *a, float *b) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k < n) b[k] = (float)a[k];
}
// Tangent blocks to FP32, padded to nb_out floats per bond (16-byte loads).
__global__ void k_blk_to_f32(int64_t nbonds, int nb_in, int nb_out, const double *a, float *b) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= nbonds) return;
  for (int c = 0; c < nb_out; c++) b[nb_out * q + c] = c < nb_in ? (float)a[nb_in * q + c] : 0.f;
}
__global__ void k_to_f64(int64_t n, const float *a, double *b) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k < n) b[k] = (double)a[k];
}

__device__ __forceinline__ void block_sum_f(float v, double *part) {
  __shared__ float sh[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  if (w == 0) {
    v = l < (int)(blockDim.x >> 5) ? sh[l] : 0.f;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (l == 0) part[blockIdx.x] = (double)v;
  }
}
__device__ __forceinline__ void block_sum2_f(float va, float vb, double *pa, double *pb) {
  __shared__ float sh[2][32];
  for (int o = 16; o > 0; o >>= 1) {
    va += __shfl_xor_sync(0xffffffffu, va, o);
    vb += __shfl_xor_sync(0xffffffffu, vb, o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    sh[0][w] = va;
    sh[1][w] = vb;
  }
  __syncthreads();
  if (w == 0) {
    const bool in = l < (int)(blockDim.x >> 5);
    va = in ? sh[0][l] : 0.f;
    vb = in ? sh[1][l] : 0.f;
    for (int o = 16; o > 0; o >>= 1) {
      va += __shfl_xor_sync(0xffffffffu, va, o);
      vb += __shfl_xor_sync(0xffffffffu, vb, o);
    }
    if (l == 0) {
      pa[blockIdx.x] = (double)va;
      pb[blockIdx.x] = (double)vb;
    }
  }
}

template <int DIM>
__global__ void k_qs_precond32(int64_t n, const uint8_t *flags, const float *dblk,
                               const float *r, float *z, double *part) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  constexpr int NB = DIM == 2 ? 3 : 6;
  float dot = 0.f;
  if (i < n) {
    const uint8_t fl = flags[i];
    float rv[3] = {0.f, 0.f, 0.f}, zv[3];
    for (int c = 0; c < DIM; c++) rv[c] = (fl >> c & 1) ? 0.f : r[DIM * i + c];
    block_jacobi<DIM, float>(dblk + NB * i, fl, rv, zv);
    for (int c = 0; c < DIM; c++) {
      z[DIM * i + c] = zv[c];
      dot = fmaf(rv[c], zv[c], dot);
    }
  }
  block_sum_f(dot, part);
}

// Device scalars of the FP32 CG: tot[0..1] = rz_k by parity, tot[2] = pAp,
// tot[3] = r.r (FP64); fs[0] = alpha, fs[1] = beta (FP32, fs = tot + 4).

// FP32 form of the first CG launch (see k_cg_dir_spmv).  Its last block
// forms alpha_k = rz_k / pAp_k for the second launch.
template <int DIM>
__global__ void __launch_bounds__(256) k_cg32_dir_spmv(
    int64_t n, const uint8_t *flags, const int64_t *rowptr, const int *cols, const float *blk,
    const float *dblk, const float *z, const float *pold, float *pnew, float *ap,
    const double *rz_cur, double *pap_part, unsigned *ticket, double *pap_total, float *fs) {
  const float beta = fs[1];
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t i = t / kG;
  const int g = (int)(t % kG);
  constexpr int NB = DIM == 2 ? 3 : 6;  // diagonal blocks (per node)
  constexpr int NP = DIM == 2 ? 4 : 8;  // bond blocks, padded for 16-byte loads
  float acc[3] = {0.f, 0.f, 0.f}, tv[3];
  if (i < n) {
    const int64_t q1 = rowptr[i + 1];
    // four bonds per pass: all ids, then all gathers, then the products, so
    // that each lane keeps its loads in flight together
    for (int64_t qb = rowptr[i] + g; qb < q1; qb += 4 * kG) {
      int jj[4];
#pragma unroll
      for (int u = 0; u < 4; u++) jj[u] = qb + u * kG < q1 ? cols[qb + u * kG] : -1;
      float bb[4][NP], pj[4][3];
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const int j = jj[u] < 0 ? (int)i : jj[u];
        const int64_t q = jj[u] < 0 ? qb : qb + u * kG;
        const float4 *bp = reinterpret_cast<const float4 *>(blk + NP * q);
        const float4 b0 = bp[0];
        bb[u][0] = b0.x; bb[u][1] = b0.y; bb[u][2] = b0.z; bb[u][3] = b0.w;
        if (DIM == 3) {
          const float4 b1 = bp[1];
          bb[u][4] = b1.x; bb[u][5] = b1.y; bb[u][6] = b1.z; bb[u][7] = b1.w;
        }
        for (int c = 0; c < DIM; c++) pj[u][c] = fmaf(beta, pold[DIM * j + c], z[DIM * j + c]);
        if (DIM == 2) pj[u][2] = 0.f;
      }
#pragma unroll
      for (int u = 0; u < 4; u++) {
        if (jj[u] < 0) continue;
        sym_mul<float>(DIM, bb[u], pj[u], tv);
        for (int c = 0; c < DIM; c++) acc[c] -= tv[c];
      }
    }
  }
  for (int o = kG / 2; o > 0; o >>= 1)
    for (int c = 0; c < DIM; c++) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
  float dot = 0.f;
  if (i < n && g == 0) {
    const uint8_t fl = flags[i];
    float pi[3] = {0.f, 0.f, 0.f};
    for (int c = 0; c < DIM; c++) {
      pi[c] = fmaf(beta, pold[DIM * i + c], z[DIM * i + c]);
      pnew[DIM * i + c] = pi[c];
    }
    sym_mul<float>(DIM, dblk + NB * i, pi, tv);
    for (int c = 0; c < DIM; c++) {
      const float yc = (fl >> c & 1) ? 0.f : acc[c] + tv[c];
      ap[DIM * i + c] = yc;
      dot = fmaf(pi[c], yc, dot);
    }
  }
  block_sum_f(dot, pap_part);
  if (last_block(ticket)) {
    finish_sums(1, pap_part, pap_total, nullptr, nullptr, ticket);
    if (threadIdx.x == 0) {
      const double pap = *pap_total;
      fs[0] = (float)(pap != 0. ? *rz_cur / pap : 0.);
    }
  }
}

// FP32 form of the second CG launch (see k_cg_update).  Its last block forms
// beta_k = rz_{k+1} / rz_k for the next first launch.
template <int DIM>
__global__ void k_cg32_update(int64_t n, const uint8_t *flags, const float *dblk, const float *p,
                              const float *ap, float *x, float *r, float *z,
                              const double *rz_cur, double *rz_part, double *rr_part,
                              unsigned *ticket, double *rz_next, double *rr_total, float *fs) {
  const float alpha = fs[0];
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  constexpr int NB = DIM == 2 ? 3 : 6;
  float drz = 0.f, drr = 0.f;
  if (i < n) {
    const uint8_t fl = flags[i];
    float rv[3] = {0.f, 0.f, 0.f}, zv[3] = {0.f, 0.f, 0.f};
    for (int c = 0; c < DIM; c++) {
      const int64_t k = DIM * i + c;
      x[k] = fmaf(alpha, p[k], x[k]);
      const float rk = fmaf(-alpha, ap[k], r[k]);
      r[k] = rk;
      drr = fmaf(rk, rk, drr);
      rv[c] = (fl >> c & 1) ? 0.f : rk;
    }
    block_jacobi<DIM, float>(dblk + NB * i, fl, rv, zv);
    for (int c = 0; c < DIM; c++) {
      z[DIM * i + c] = zv[c];
      drz = fmaf(rv[c], zv[c], drz);
    }
  }
  block_sum2_f(drz, drr, rz_part, rr_part);
  if (last_block(ticket)) {
    finish_sums(2, rz_part, rz_next, rr_part, rr_total, ticket);
    if (threadIdx.x == 0) {
      const double rzc = *rz_cur;
      fs[1] = (float)(rzc != 0. ? *rz_next / rzc : 0.);
    }
  }
}

// ---- the FP32 PCG in one cooperative launch -------------------------------
// The two-launch iteration above costs two kernel launches per iteration and
// a host round trip every few iterations; at 40,000 nodes that, not the
// work, sets the iteration time.  k_cg32_coop runs the whole solve in one
// launch whose blocks are all resident (cudaLaunchCooperativeKernel): each
// iteration is the same two phases separated by a grid barrier, and every
// block forms alpha, beta and the convergence test itself from the block
// partials, summed in one fixed order (so every block takes the same
// decision and the result does not depend on timing).
//
// Grid barrier: an arrival counter and a generation word.  A waiting block
// polls the generation with a bounded wait (wait_ns of globaltimer); a wait
// that runs out sets status = NLM_ERR_TIMEOUT, and every block leaves at its
// next barrier once status is set, so the launch always ends.  expect is the
// number of arrivals a barrier completes on: gridDim.x in use (more only to
// test the bound).
__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// coop[0] arrivals, coop[1] generation, coop[2] status
__device__ bool coop_barrier(unsigned *coop, unsigned expect, uint64_t wait_ns) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned *gen = coop + 1;
    volatile int *status = reinterpret_cast<volatile int *>(coop + 2);
    const unsigned g = *gen;
    __threadfence();
    int ok = 1;
    if (atomicAdd(coop, 1u) == expect - 1) {
      atomicExch(coop, 0u);
      __threadfence();
      atomicAdd(coop + 1, 1u);
    } else {
      const uint64_t t0 = globaltimer_ns();
      while (*gen == g) {
        if (*status != 0) {
          ok = 0;
          break;
        }
        if (globaltimer_ns() - t0 > wait_ns) {
          atomicExch(reinterpret_cast<int *>(coop + 2), NLM_ERR_TIMEOUT);
          ok = 0;
          break;
        }
        __nanosleep(100);
      }
    }
    __threadfence();
    if (*status != 0) ok = 0;
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// Sum of part[0 .. nb) in a fixed order, the same in every block.
__device__ double coop_sum(const double *part, int nb) {
  __shared__ double sh[32];
  double v = 0.;
  for (int k = threadIdx.x; k < nb; k += blockDim.x) v += __ldcg(part + k);
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  double t = 0.;
  for (int k = 0; k < (int)(blockDim.x >> 5); k++) t += sh[k];
  return t;
}

constexpr int kCoopThreads = 256;

// res[0] = iterations done, res[1] = r.r at the end
template <int DIM>
__global__ void __launch_bounds__(256) k_cg32_coop(
    int64_t n, const uint8_t *flags, const int64_t *rowptr, const int *cols, const float *blk,
    const float *dblk, float *p0, float *p1, float *ap, float *x, float *r, float *z,
    double *part, const double *rz0, double target, int max_iters, unsigned *coop,
    unsigned expect, uint64_t wait_ns, double *res) {
  constexpr int NB = DIM == 2 ? 3 : 6;
  constexpr int NP = DIM == 2 ? 4 : 8;
  const int G = (int)gridDim.x;
  double *pap_p = part, *rz_p = part + G, *rr_p = part + 2 * G;
  double rz = *rz0, rr = 0.;
  float beta = 0.f;
  int it = 0;
  bool ok = true;
  while (it < max_iters) {
    const float *pold = (it & 1) ? p0 : p1;
    float *pnew = (it & 1) ? p1 : p0;
    // phase 1: p_k = z_k + beta p_{k-1}, Ap_k, partials of p_k.Ap_k
    float dot = 0.f;
    const int64_t work = n * kG;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < work;
         base += (int64_t)G * blockDim.x) {
      const int64_t t = base + threadIdx.x;
      const int64_t i = t / kG;
      const int g = (int)(t % kG);
      float acc[3] = {0.f, 0.f, 0.f}, tv[3];
      if (i < n) {
        const int64_t q1 = rowptr[i + 1];
        for (int64_t qb = rowptr[i] + g; qb < q1; qb += 4 * kG) {
          int jj[4];
#pragma unroll
          for (int u = 0; u < 4; u++) jj[u] = qb + u * kG < q1 ? cols[qb + u * kG] : -1;
          float bb[4][NP], pj[4][3];
#pragma unroll
          for (int u = 0; u < 4; u++) {
            const int j = jj[u] < 0 ? (int)i : jj[u];
            const int64_t q = jj[u] < 0 ? qb : qb + u * kG;
            const float4 *bp = reinterpret_cast<const float4 *>(blk + NP * q);
            const float4 b0 = bp[0];
            bb[u][0] = b0.x; bb[u][1] = b0.y; bb[u][2] = b0.z; bb[u][3] = b0.w;
            if (DIM == 3) {
              const float4 b1 = bp[1];
              bb[u][4] = b1.x; bb[u][5] = b1.y; bb[u][6] = b1.z; bb[u][7] = b1.w;
            }
            for (int c = 0; c < DIM; c++) pj[u][c] = fmaf(beta, pold[DIM * j + c], z[DIM * j + c]);
            if (DIM == 2) pj[u][2] = 0.f;
          }
#pragma unroll
          for (int u = 0; u < 4; u++) {
            if (jj[u] < 0) continue;
            sym_mul<float>(DIM, bb[u], pj[u], tv);
            for (int c = 0; c < DIM; c++) acc[c] -= tv[c];
          }
        }
      }
      for (int o = kG / 2; o > 0; o >>= 1)
        for (int c = 0; c < DIM; c++) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
      if (i < n && g == 0) {
        const uint8_t fl = flags[i];
        float pi[3] = {0.f, 0.f, 0.f};
        for (int c = 0; c < DIM; c++) {
          pi[c] = fmaf(beta, pold[DIM * i + c], z[DIM * i + c]);
          pnew[DIM * i + c] = pi[c];
        }
        sym_mul<float>(DIM, dblk + NB * i, pi, tv);
        for (int c = 0; c < DIM; c++) {
          const float yc = (fl >> c & 1) ? 0.f : acc[c] + tv[c];
          ap[DIM * i + c] = yc;
          dot = fmaf(pi[c], yc, dot);
        }
      }
    }
    block_sum_f(dot, pap_p);
    if (!(ok = coop_barrier(coop, expect, wait_ns))) break;
    const double pap = coop_sum(pap_p, G);
    const float alpha = (float)(pap != 0. ? rz / pap : 0.);
    // phase 2: x += alpha p, r -= alpha Ap, z = block-Jacobi(r), partials of
    // r.z and r.r
    float drz = 0.f, drr = 0.f;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)G * blockDim.x) {
      const uint8_t fl = flags[i];
      float rv[3] = {0.f, 0.f, 0.f}, zv[3] = {0.f, 0.f, 0.f};
      for (int c = 0; c < DIM; c++) {
        const int64_t k = DIM * i + c;
        x[k] = fmaf(alpha, pnew[k], x[k]);
        const float rk = fmaf(-alpha, ap[k], r[k]);
        r[k] = rk;
        drr = fmaf(rk, rk, drr);
        rv[c] = (fl >> c & 1) ? 0.f : rk;
      }
      block_jacobi<DIM, float>(dblk + NB * i, fl, rv, zv);
      for (int c = 0; c < DIM; c++) {
        z[DIM * i + c] = zv[c];
        drz = fmaf(rv[c], zv[c], drz);
      }
    }
    block_sum2_f(drz, drr, rz_p, rr_p);
    if (!(ok = coop_barrier(coop, expect, wait_ns))) break;
    const double rz_next = coop_sum(rz_p, G);
    rr = coop_sum(rr_p, G);
    beta = (float)(rz != 0. ? rz_next / rz : 0.);
    rz = rz_next;
    it++;
    if (!(rr > target)) break;
    // the partials are rewritten next iteration only after the next barrier,
    // which every block reaches after reading them
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    res[0] = (double)it;
    res[1] = rr;
  }
  (void)ok;
}

__global__ void k_cg32_seed(float *fs, float *pold, int64_t m) {
  // beta = 0 for the first direction (p_0 = z_0); p_{-1} = 0
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k < m) pold[k] = 0.f;
  if (k == 0) fs[1] = 0.f;
}

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
static cudaError_t qs_cg64(const StepParams &P, const DevPtrs &D, const QSWork &W, const double *rhs,
                  double *dx, double tol, int max_iters, int check_every, int *iters,
                  cudaStream_t s) {
  const int dim = P.dim;
  const int64_t m = (int64_t)dim * P.n;
  const unsigned gn = qblk(P.n), gg = grp_blocks(P.n);
  const int64_t stride = qs_cg_stride(P.n);
  // partials: pAp (K1 blocks), rz and r.r (K2 blocks); totals on the device:
  // rz_k in tot[k & 1], pAp in tot[2], r.r in tot[3]
  double *pap_p = W.cgpart, *rz_p = W.cgpart + stride, *rr_p = W.cgpart + 2 * stride;
  double *tot = W.cgs;
  double *pbuf[2] = {W.p, W.p2};
  cudaError_t e;
  if ((e = cudaMemsetAsync(dx, 0, sizeof(double) * m, s))) return e;
  if ((e = cudaMemcpyAsync(W.r, rhs, sizeof(double) * m, cudaMemcpyDeviceToDevice, s))) return e;
  // z_0 = M^-1 r_0 and rz_0; rz_{-1} = 1, p_{-1} = 0
  if (dim == 2)
    k_qs_precond<2><<<gn, 256, 0, s>>>(P, D, W.dblk, W.r, W.z, rz_p);
  else
    k_qs_precond<3><<<gn, 256, 0, s>>>(P, D, W.dblk, W.r, W.z, rz_p);
  k_qs_sum<<<1, 256, 0, s>>>(rz_p, gn, tot + 0);
  k_cg_seed<<<qblk(m), 256, 0, s>>>(tot + 1, pbuf[1], m);
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
      const int cur = it & 1, prv = cur ^ 1;
      if (dim == 2) {
        k_cg_dir_spmv<2, true><<<gg, 256, 0, s>>>(P.n, D.flags, D.rowptr, D.cols, W.blk,
                                                  W.dblk, W.z, pbuf[prv], pbuf[cur], W.ap,
                                                  tot + cur, tot + prv, pap_p, W.ticket,
                                                  tot + 2);
        k_cg_update<2><<<gn, 256, 0, s>>>(P.n, D.flags, W.dblk, pbuf[cur], W.ap, dx, W.r, W.z,
                                          tot + cur, tot + 2, rz_p, rr_p, W.ticket + 1,
                                          tot + prv, tot + 3);
      } else {
        k_cg_dir_spmv<3, true><<<gg, 256, 0, s>>>(P.n, D.flags, D.rowptr, D.cols, W.blk,
                                                  W.dblk, W.z, pbuf[prv], pbuf[cur], W.ap,
                                                  tot + cur, tot + prv, pap_p, W.ticket,
                                                  tot + 2);
        k_cg_update<3><<<gn, 256, 0, s>>>(P.n, D.flags, W.dblk, pbuf[cur], W.ap, dx, W.r, W.z,
                                          tot + cur, tot + 2, rz_p, rr_p, W.ticket + 1,
                                          tot + prv, tot + 3);
      }
    }
    if ((e = cudaGetLastError())) return e;
    double rr = 0.;
    if ((e = cudaMemcpyAsync(&rr, tot + 3, sizeof(double), cudaMemcpyDeviceToHost, s))) return e;
    if ((e = cudaStreamSynchronize(s))) return e;
    if (!(rr > target)) break;
  }
  *iters = it;
  return cudaGetLastError();
}

static cudaError_t qs_cg32(const StepParams &P, const DevPtrs &D, const QSWork &W,
                           const double *rhs, double *dx, double tol, int max_iters,
                           int check_every, int *iters, bool *converged, cudaStream_t s) {
  *converged = true;
  const int dim = P.dim;
  const int64_t m = (int64_t)dim * P.n;
  const unsigned gn = qblk(P.n), gg = grp_blocks(P.n);
  const int64_t stride = qs_cg_stride(P.n);
  // partials: pAp (K1 blocks), rz and r.r (K2 blocks); totals on the device:
  // rz_k in tot[k & 1], pAp in tot[2], r.r in tot[3]
  double *pap_p = W.cgpart, *rz_p = W.cgpart + stride, *rr_p = W.cgpart + 2 * stride;
  double *tot = W.cgs;
  float *fs = reinterpret_cast<float *>(tot + 4);
  float *pbuf[2] = {W.p32, W.p32b};
  const int NB = dim == 2 ? 3 : 6;
  cudaError_t e;
  // FP32 copies of the tangent and of the right-hand side; x = 0
  k_blk_to_f32<<<qblk(W.nnz + 1), 256, 0, s>>>(W.nnz + 1, NB, dim == 2 ? 4 : 8, W.blk, W.blk32);
  k_to_f32<<<qblk((int64_t)NB * P.n), 256, 0, s>>>((int64_t)NB * P.n, W.dblk, W.dblk32);
  k_to_f32<<<qblk(m), 256, 0, s>>>(m, rhs, W.r32);
  if ((e = cudaMemsetAsync(W.x32, 0, sizeof(float) * m, s))) return e;
  // z_0 = M^-1 r_0 and rz_0; beta_{-1} = 0, p_{-1} = 0
  if (dim == 2)
    k_qs_precond32<2><<<gn, 256, 0, s>>>(P.n, D.flags, W.dblk32, W.r32, W.z32, rz_p);
  else
    k_qs_precond32<3><<<gn, 256, 0, s>>>(P.n, D.flags, W.dblk32, W.r32, W.z32, rz_p);
  k_qs_sum<<<1, 256, 0, s>>>(rz_p, gn, tot + 0);
  k_cg32_seed<<<qblk(m), 256, 0, s>>>(fs, pbuf[1], m);
  double rr0 = 0.;
  if ((e = qs_dot(rhs, rhs, m, W.part, W.sc + 3, s))) return e;
  if ((e = cudaMemcpyAsync(&rr0, W.sc + 3, sizeof(double), cudaMemcpyDeviceToHost, s))) return e;
  if ((e = cudaStreamSynchronize(s))) return e;
  const double target = tol * tol * rr0;
  int it = 0;
  if (rr0 == 0.) {
    *iters = 0;
    return cudaMemsetAsync(dx, 0, sizeof(double) * m, s);
  }
  if (W.coop && W.coop_blocks > 0) {
    // the whole solve in one cooperative launch
    if ((e = cudaMemsetAsync(W.coop, 0, sizeof(unsigned), s))) return e;  // arrivals
    if ((e = cudaMemsetAsync(W.coop + 2, 0, sizeof(unsigned), s))) return e;  // status
    int64_t n = P.n;
    const uint8_t *flags = D.flags;
    const int64_t *rowptr = D.rowptr;
    const int *cols = D.cols;
    const float *blk = W.blk32, *dblk = W.dblk32;
    float *p0 = pbuf[0], *p1 = pbuf[1], *ap = W.ap32, *x = W.x32, *r = W.r32, *z = W.z32;
    double *part = W.cgpart;
    const double *rz0 = tot + 0;
    double tgt = target;
    int mi = max_iters;
    unsigned *coop = W.coop;
    unsigned expect = (unsigned)W.coop_blocks + (unsigned)W.coop_extra;
    uint64_t wait_ns = W.coop_wait_ns;
    double *res = W.cgs + 6;
    void *args[] = {&n, &flags, &rowptr, &cols, &blk, &dblk, &p0, &p1, &ap, &x, &r, &z,
                    &part, &rz0, &tgt, &mi, &coop, &expect, &wait_ns, &res};
    // p_{-1} = 0 lives in pbuf[1] (zeroed by the seed), p_0 goes to pbuf[0]
    e = dim == 2 ? cudaLaunchCooperativeKernel((const void *)k_cg32_coop<2>, W.coop_blocks,
                                               kCoopThreads, args, 0, s)
                 : cudaLaunchCooperativeKernel((const void *)k_cg32_coop<3>, W.coop_blocks,
                                               kCoopThreads, args, 0, s);
    if (e != cudaSuccess) return e;
    double hres[2] = {0., 0.};
    int status = 0;
    if ((e = cudaMemcpyAsync(hres, res, sizeof(hres), cudaMemcpyDeviceToHost, s))) return e;
    if ((e = cudaMemcpyAsync(&status, W.coop + 2, sizeof(int), cudaMemcpyDeviceToHost, s)))
      return e;
    if ((e = cudaStreamSynchronize(s))) return e;
    if (status != 0) return cudaErrorTimeout;
    it = (int)hres[0];
    *converged = !(hres[1] > target) || it < max_iters;
    k_to_f64<<<qblk(m), 256, 0, s>>>(m, W.x32, dx);
    *iters = it;
    return cudaGetLastError();
  }
  while (it < max_iters) {
    for (int q = 0; q < check_every && it < max_iters; q++, it++) {
      const int cur = it & 1, prv = cur ^ 1;
      if (dim == 2) {
        k_cg32_dir_spmv<2><<<gg, 256, 0, s>>>(P.n, D.flags, D.rowptr, D.cols, W.blk32,
                                              W.dblk32, W.z32, pbuf[prv], pbuf[cur], W.ap32,
                                              tot + cur, pap_p, W.ticket, tot + 2, fs);
        k_cg32_update<2><<<gn, 256, 0, s>>>(P.n, D.flags, W.dblk32, pbuf[cur], W.ap32, W.x32,
                                            W.r32, W.z32, tot + cur, rz_p, rr_p, W.ticket + 1,
                                            tot + prv, tot + 3, fs);
      } else {
        k_cg32_dir_spmv<3><<<gg, 256, 0, s>>>(P.n, D.flags, D.rowptr, D.cols, W.blk32,
                                              W.dblk32, W.z32, pbuf[prv], pbuf[cur], W.ap32,
                                              tot + cur, pap_p, W.ticket, tot + 2, fs);
        k_cg32_update<3><<<gn, 256, 0, s>>>(P.n, D.flags, W.dblk32, pbuf[cur], W.ap32, W.x32,
                                            W.r32, W.z32, tot + cur, rz_p, rr_p, W.ticket + 1,
                                            tot + prv, tot + 3, fs);
      }
    }
    if ((e = cudaGetLastError())) return e;
    double rr = 0.;
    if ((e = cudaMemcpyAsync(&rr, tot + 3, sizeof(double), cudaMemcpyDeviceToHost, s))) return e;
    if ((e = cudaStreamSynchronize(s))) return e;
    if (!(rr > target)) break;
  }
  *converged = it < max_iters;
  k_to_f64<<<qblk(m), 256, 0, s>>>(m, W.x32, dx);
  *iters = it;
  return cudaGetLastError();
}

// Blocks of the cooperative solve: up to four blocks of kCoopThreads per SM
// that can be resident together, at most one per kCoopThreads (node, lane)
// items; 0 if the device cannot launch it cooperatively.  (One block of 1024
// threads per SM, fewer arrivals per barrier, measured slower.)
int qs_coop_blocks(int64_t n, int dim) {
  int dev = 0, sms = 0, coop = 0, per = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
  if (!coop || sms <= 0) return 0;
  cudaError_t e =
      dim == 2 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_cg32_coop<2>, kCoopThreads, 0)
               : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_cg32_coop<3>, kCoopThreads, 0);
  if (e != cudaSuccess || per <= 0) {
    cudaGetLastError();
    return 0;
  }
  const int64_t need = std::max<int64_t>(1, (n * kG + kCoopThreads - 1) / kCoopThreads);
  return (int)std::min<int64_t>((int64_t)sms * std::min(per, 4), need);
}

// Newton correction (-K) dx = rhs.  The FP32 solve is tried first; when it
// has not reached the tolerance within kCg32Cap iterations (tangents of
// fractured states are too ill-conditioned for FP32 recurrences), the FP64
// solve takes over from scratch and *use64 is set so that the caller keeps
// FP64 for the rest of the load step.
constexpr int kCg32Cap = 800;

cudaError_t qs_cg(const StepParams &P, const DevPtrs &D, const QSWork &W, const double *rhs,
                  double *dx, double tol, int max_iters, int check_every, int *iters,
                  bool *use64, cudaStream_t s) {
  int it32 = 0;
  if (!*use64) {
    bool conv = false;
    cudaError_t e = qs_cg32(P, D, W, rhs, dx, tol, std::min(max_iters, kCg32Cap), check_every,
                            &it32, &conv, s);
    if (e != cudaSuccess || conv || max_iters <= kCg32Cap) {
      *iters = it32;
      return e;
    }
    *use64 = true;
  }
  int it64 = 0;
  cudaError_t e = qs_cg64(P, D, W, rhs, dx, tol, max_iters, check_every, &it64, s);
  *iters = it32 + it64;
  return e;
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
  // part: grp_blocks(n) partials of x.y
  if (P.dim == 2)
    k_cg_dir_spmv<2, false><<<grp_blocks(P.n), 256, 0, s>>>(
        P.n, D.flags, D.rowptr, D.cols, blk, dblk, x, nullptr, nullptr, y, nullptr, nullptr,
        part, nullptr, nullptr);
  else
    k_cg_dir_spmv<3, false><<<grp_blocks(P.n), 256, 0, s>>>(
        P.n, D.flags, D.rowptr, D.cols, blk, dblk, x, nullptr, nullptr, y, nullptr, nullptr,
        part, nullptr, nullptr);
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
