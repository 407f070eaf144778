// fd_fp64.cu -- FP64 "plain" explicit-step kernels.
//
// Compiled with --fmad=false: every product and sum is rounded separately, in
// the order of the reference expressions, so a bond force differs from the
// reference's only by the last-ulp behaviour of exp().  One thread owns one
// node and sums its bonds in neighbour-list order (ascending original id), as
// FDModel::computeForce does (src/model/fd/fDModel.cpp:557-575).

#include "fd_internal.h"
#include "state_io.cuh"

namespace nlm {

// One RNPBond::getBondEF evaluation (src/material/pd/rnpBond.cpp:216-301),
// contact force off.  Returns the scalar s of F = s * e and the unit vector e.
template <int DIM>
__device__ __forceinline__ double rnp_bond64(const StepParams &P, const double xi[3],
                                             const double ui[3], const double xj[3],
                                             const double uj[3], double &volj,
                                             bool breakable, bool &fs, double e[3]) {
  double dx = xj[0] - xi[0], dy = xj[1] - xi[1];
  double dz = DIM == 3 ? xj[2] - xi[2] : 0.0;
  double rr = dx * dx + dy * dy;
  if (DIM == 3) rr = rr + dz * dz;
  double rji = sqrt(rr);  // xj.dist(xi), also dx.length()
  double dux = uj[0] - ui[0], duy = uj[1] - ui[1];
  double dotp = dx * dux + dy * duy;
  if (DIM == 3) dotp = dotp + dz * (uj[2] - ui[2]);
  double S = dotp / rr;  // getS, :303-306
  e[0] = dx / rji;
  e[1] = dy / rji;
  e[2] = dz / rji;
  if (dGT(rji, P.check_low)) volj = volj * ((P.check_up - rji) / P.h);  // :255-256
  double infl = influence_d(P, rji / P.delta);
  if (breakable) {
    if (P.irrev && !fs && dGT(fabs(S), P.fsc * (P.rbar / sqrt(rji)))) fs = true;  // :263-266
    if (fs) return 0.0;
    return (infl * 4. * S * P.C * P.beta * exp(-P.beta * rji * S * S) / P.invF) * volj;
  }
  return (infl * 4. * S * P.C * P.beta / P.invF) * volj;  // :298
}

// Thread-per-node step over the sliced-ELL bond store.
template <int DIM, int SCHEME, bool FIRST>
__global__ void __launch_bounds__(128)
    k_rnp64_thread(const StepParams P, const DevPtrs D, const BCTable T, const StepArgs A) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  const double *ucur = D.u64[A.cur];
  double xi[3], ui[3];
  ld_node<DIM>(D.pos64, i, xi);
  ld_node<DIM>(ucur, i, ui);
  const uint8_t fl = D.flags[i];
  const bool brk_i = !(fl & FLAG_NOFAIL);
  const double voli = __ldg(D.vol64 + i);
  const int *colp = D.sell_cols + D.sell_ptr[i >> 5] + 4 * (i & 31);
  const int len = D.rowlen[i];
  double fi[3] = {0., 0., 0.};
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
    double xj[3], uj[3], e[3];
    ld_node<DIM>(D.pos64, j, xj);
    ld_node<DIM>(ucur, j, uj);
    bool fs = (word >> (k & 31)) & 1u;
    const bool was = fs;
    bool breakable = brk_i;
    if (P.nofail && breakable) breakable = !(D.flags[j] & FLAG_NOFAIL);
    double volj = __ldg(D.vol64 + j);
    double s = rnp_bond64<DIM>(P, xi, ui, xj, uj, volj, breakable, fs, e);
    if (fs != was) {
      word |= 1u << (k & 31);
      dirty = true;
    }
    if (!fs || !breakable) {
      fi[0] = fi[0] + s * e[0];
      fi[1] = fi[1] + s * e[1];
      if (DIM == 3) fi[2] = fi[2] + s * e[2];
    } else if (P.contact) {
      // normal contact of a broken bond (rnpBond.cpp:281-291):
      // y = (x_j + u_j) - (x_i + u_i), f += -max(0, Kn Vi Vj/(Vi+Vj) (Rc - |y|)/|y|) y
      double y[3];
      for (int c = 0; c < 3; c++) y[c] = (xj[c] + uj[c]) - (xi[c] + ui[c]);
      const double R = sqrt(y[0] * y[0] + y[1] * y[1] + y[2] * y[2]);
      double sf = P.contact_kn * (voli * volj / (voli + volj)) * (P.contact_rc - R) / R;
      if (sf < 0.) sf = 0.;
      fi[0] = fi[0] + (0. + -sf * y[0]);
      fi[1] = fi[1] + (0. + -sf * y[1]);
      if (DIM == 3) fi[2] = fi[2] + (0. + -sf * y[2]);
    }
  }
  if (dirty) D.bits[(int64_t)chunk * P.npad + i] = word;
  integrate_node64<DIM, SCHEME, FIRST>(P, D, T, A, i, fl, ui, fi);
}

template <int DIM, int SCHEME>
static cudaError_t launch_dim(const StepParams &P, const DevPtrs &D, const BCTable &T,
                              const StepArgs &a, cudaStream_t s) {
  const int bs = 128;
  const unsigned grid = (unsigned)((P.n + bs - 1) / bs);
  if (P.n == 0) return cudaSuccess;
  if (a.first)
    k_rnp64_thread<DIM, SCHEME, true><<<grid, bs, 0, s>>>(P, D, T, a);
  else
    k_rnp64_thread<DIM, SCHEME, false><<<grid, bs, 0, s>>>(P, D, T, a);
  return cudaGetLastError();
}

cudaError_t launch_rnp_step_fp64(const StepParams &P, const DevPtrs &D, const BCTable &T,
                                 const StepArgs &a, int decomp, cudaStream_t s) {
  (void)decomp;  // the FP64 path keeps the reference summation order
  if (P.dim == 2)
    return P.scheme == NLM_VELOCITY_VERLET ? launch_dim<2, NLM_VELOCITY_VERLET>(P, D, T, a, s)
                                           : launch_dim<2, NLM_CENTRAL_DIFFERENCE>(P, D, T, a, s);
  return P.scheme == NLM_VELOCITY_VERLET ? launch_dim<3, NLM_VELOCITY_VERLET>(P, D, T, a, s)
                                         : launch_dim<3, NLM_CENTRAL_DIFFERENCE>(P, D, T, a, s);
}

// FDModel::computePostProcFields, damage part (fDModel.cpp:651-778):
// phi_i = 1 - a/b over corrected volumes, Z_i = max |S| / S_c(r).
template <int DIM>
__global__ void k_damage(const StepParams P, const DevPtrs D, int cur, bool fp32, bool es,
                         float *phi, float *Z) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  double xi[3], ui[3];
  ld_node<DIM>(D.pos64, i, xi);
  if (fp32)
    ld_split<DIM>(D.u32[cur], i, ui);
  else
    ld_node<DIM>(D.u64[cur], i, ui);
  double a = 0., b = 0., z = 0.;
  const int64_t r0 = D.rowptr[i], r1 = D.rowptr[i + 1];
  for (int64_t k = r0; k < r1; k++) {
    const int j = D.cols[k];
    const int kk = (int)(k - r0);
    const bool fs = (D.bits[(int64_t)(kk >> 5) * P.npad + i] >> (kk & 31)) & 1u;
    double xj[3], uj[3];
    ld_node<DIM>(D.pos64, j, xj);
    if (fp32)
      ld_split<DIM>(D.u32[cur], j, uj);
    else
      ld_node<DIM>(D.u64[cur], j, uj);
    double dx = xj[0] - xi[0], dy = xj[1] - xi[1], dz = DIM == 3 ? xj[2] - xi[2] : 0.;
    double rr = dx * dx + dy * dy;
    if (DIM == 3) rr = rr + dz * dz;
    double rji = sqrt(rr);
    double volj = D.vol64[j];
    if (dGT(rji, P.check_low)) volj = volj * ((P.check_up - rji) / P.h);
    if (!fs) a += volj;
    b += volj;
    double sr = 0.;
    if (!es) {
      double dotp = dx * (uj[0] - ui[0]) + dy * (uj[1] - ui[1]);
      if (DIM == 3) dotp = dotp + dz * (uj[2] - ui[2]);
      double S = dotp / rr;
      if (dGT(rji, 1.0E-12)) sr = fabs(S) / (P.rbar / sqrt(rji));
    } else if (P.es_sc > 0.) {
      double Y0 = (xj[0] + uj[0]) - (xi[0] + ui[0]);
      double Y1 = (xj[1] + uj[1]) - (xi[1] + ui[1]);
      double Y2 = DIM == 3 ? (xj[2] + uj[2]) - (xi[2] + ui[2]) : 0.;
      double yl = sqrt(Y0 * Y0 + Y1 * Y1 + Y2 * Y2);
      sr = fabs((yl - rji) / rji) / P.es_sc;
    }
    if (dLT(z, sr)) z = sr;
  }
  if (phi) phi[i] = (float)(b > 0. ? 1. - a / b : 0.);
  if (Z) Z[i] = (float)z;
}

// Energies of FDModel::computePostProcFields (fDModel.cpp:651-778), RNPBond:
// strain energy V_i sum_j E_ij with E_ij the energy of getBondEF
// (rnpBond.cpp:267-300; a bond past its critical strain counts as broken, the
// bond state itself is left alone), work done u_i . f_ext_i, kinetic energy
// rho |v_i|^2 V_i / 2, and the strain energy again where Z_i > 1 - 1e-10
// (fracture energy).  FP64 in the reference's operation order.
template <int DIM>
__global__ void k_energy(const StepParams P, const DevPtrs D, int cur, int vcur, bool fp32,
                         const double *fext, float *strain, float *work, float *kinetic, float *fracture) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  double xi[3], ui[3], vi[3];
  ld_node<DIM>(D.pos64, i, xi);
  if (fp32) {
    ld_split<DIM>(D.u32[cur], i, ui);
    ld_split<DIM>(D.v32[vcur], i, vi);
  } else {
    ld_node<DIM>(D.u64[cur], i, ui);
    ld_node<DIM>(D.v[vcur], i, vi);
  }
  const uint8_t fl = D.flags[i];
  const double voli = D.vol64[i];
  double energy = 0., z = 0.;
  const int64_t r0 = D.rowptr[i], r1 = D.rowptr[i + 1];
  for (int64_t k = r0; k < r1; k++) {
    const int j = D.cols[k];
    const int kk = (int)(k - r0);
    bool fs = (D.bits[(int64_t)(kk >> 5) * P.npad + i] >> (kk & 31)) & 1u;
    double xj[3], uj[3];
    ld_node<DIM>(D.pos64, j, xj);
    if (fp32)
      ld_split<DIM>(D.u32[cur], j, uj);
    else
      ld_node<DIM>(D.u64[cur], j, uj);
    double dx = xj[0] - xi[0], dy = xj[1] - xi[1], dz = DIM == 3 ? xj[2] - xi[2] : 0.;
    double rr = dx * dx + dy * dy;
    if (DIM == 3) rr = rr + dz * dz;
    const double rji = sqrt(rr);
    double dotp = dx * (uj[0] - ui[0]) + dy * (uj[1] - ui[1]);
    if (DIM == 3) dotp = dotp + dz * (uj[2] - ui[2]);
    const double S = dotp / rr;
    double volj = D.vol64[j];
    if (dGT(rji, P.check_low)) volj = volj * ((P.check_up - rji) / P.h);
    const double infl = influence_d(P, rji / P.delta);
    const bool breakable = !((fl | D.flags[j]) & FLAG_NOFAIL);
    if (breakable) {
      if (P.irrev && !fs && dGT(fabs(S), P.fsc * (P.rbar / sqrt(rji)))) fs = true;
      if (!fs)
        energy += (infl * P.C * (1. - exp(-P.beta * rji * S * S)) / P.invF) * volj;
      else
        energy += infl * P.C / P.invF * volj;
    } else {
      energy += (infl * P.C * P.beta * rji * S * S / P.invF) * volj;
    }
    double sr = 0.;
    if (dGT(rji, 1.0E-12)) sr = fabs(S) / (P.rbar / sqrt(rji));
    if (dLT(z, sr)) z = sr;
  }
  if (strain) strain[i] = (float)(energy * voli);
  if (work) {
    double fe[3] = {0., 0., 0.};
    if (fl & FLAG_FBC) ld_node<DIM>(fext, i, fe);
    double w = ui[0] * fe[0] + ui[1] * fe[1];
    w = w + ui[2] * fe[2];
    work[i] = (float)w;
  }
  if (kinetic) {
    double vv = vi[0] * vi[0] + vi[1] * vi[1];
    vv = vv + vi[2] * vi[2];
    kinetic[i] = (float)(0.5 * P.rho * vv * voli);
  }
  if (fracture) fracture[i] = dGT(z, 1.0 - 1.0E-10) ? (float)(energy * voli) : 0.f;
}

// util::geometry::direction (utilGeom.cpp:317-326): the orientation of C
// against the line A-B.  The cross product is stored in an int, so it is
// truncated toward zero before its sign is taken.
__device__ int geo_direction(double ax, double ay, double bx, double by, double cx, double cy) {
  const int val = (int)((by - ay) * (cx - bx) - (bx - ax) * (cy - by));
  if (val == 0) return 0;
  return val < 0 ? 2 : 1;
}

// util::geometry::onLine (utilGeom.cpp:308-315), as written there.
__device__ bool geo_on_line(double ax, double ay, double bx, double by, double cx, double cy) {
  return cx <= fmax(ax, bx) && cx <= fmin(ax, bx) && cy <= fmax(ay, by) && cy <= fmin(ay, by);
}

// util::geometry::doLinesIntersect (utilGeom.cpp:281-306) of A-B and C-D.
__device__ bool geo_lines_intersect(double ax, double ay, double bx, double by, double cx,
                                    double cy, double dx, double dy) {
  const int d1 = geo_direction(ax, ay, bx, by, cx, cy);
  const int d2 = geo_direction(ax, ay, bx, by, dx, dy);
  const int d3 = geo_direction(cx, cy, dx, dy, ax, ay);
  const int d4 = geo_direction(cx, cy, dx, dy, bx, by);
  if (d1 != d2 && d3 != d4) return true;
  if (d1 == 0 && geo_on_line(ax, ay, bx, by, cx, cy)) return true;
  if (d2 == 0 && geo_on_line(ax, ay, bx, by, dx, dy)) return true;
  if (d3 == 0 && geo_on_line(cx, cy, dx, dy, ax, ay)) return true;
  if (d4 == 0 && geo_on_line(cx, cy, dx, dy, bx, by)) return true;
  return false;
}

// Reaction force of FDModel::computeForce (fDModel.cpp:543-580) with
// is_reaction_force (:582-605), 2-D RNPBond: for a node i in the layer
// max_y - 1.5 delta < y_i < max_y - delta, R_i = sum of V_i F_ij over the bonds
// i-j that meet the line y = max_y - delta + 1e-6 from min_x to max_x (F_ij
// the getBondEF force, a bond past its critical strain counting as broken);
// R_i = 0 elsewhere.  R: 2 doubles per node.
__global__ void k_reaction(const StepParams P, const DevPtrs D, int cur, bool fp32, double min_x,
                           double max_x, double max_y, double *R) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  double xi[3], ui[3];
  ld_node<2>(D.pos64, i, xi);
  double r0 = 0., r1 = 0.;
  if (xi[1] > max_y - 1.5 * P.delta && xi[1] < max_y - P.delta) {
    if (fp32)
      ld_split<2>(D.u32[cur], i, ui);
    else
      ld_node<2>(D.u64[cur], i, ui);
    const double ay = max_y - P.delta + 1e-6;
    const uint8_t fl = D.flags[i];
    const double voli = D.vol64[i];
    const int64_t k0 = D.rowptr[i], k1 = D.rowptr[i + 1];
    for (int64_t k = k0; k < k1; k++) {
      const int j = D.cols[k];
      double xj[3], uj[3], e[3];
      ld_node<2>(D.pos64, j, xj);
      if (!geo_lines_intersect(min_x, ay, max_x, ay, xi[0], xi[1], xj[0], xj[1])) continue;
      if (fp32)
        ld_split<2>(D.u32[cur], j, uj);
      else
        ld_node<2>(D.u64[cur], j, uj);
      const int kk = (int)(k - k0);
      bool fs = (D.bits[(int64_t)(kk >> 5) * P.npad + i] >> (kk & 31)) & 1u;
      const bool breakable = !((fl | D.flags[j]) & FLAG_NOFAIL);
      double volj = D.vol64[j];
      const double s = rnp_bond64<2>(P, xi, ui, xj, uj, volj, breakable, fs, e);
      double f0, f1;
      if (!fs || !breakable) {
        f0 = s * e[0];
        f1 = s * e[1];
      } else if (P.contact) {
        const double y0 = (xj[0] + uj[0]) - (xi[0] + ui[0]);
        const double y1 = (xj[1] + uj[1]) - (xi[1] + ui[1]);
        const double Rl = sqrt(y0 * y0 + y1 * y1 + 0. * 0.);
        double sf = P.contact_kn * (voli * volj / (voli + volj)) * (P.contact_rc - Rl) / Rl;
        if (sf < 0.) sf = 0.;
        f0 = 0. + -sf * y0;
        f1 = 0. + -sf * y1;
      } else {
        f0 = f1 = 0.;
      }
      r0 = r0 + voli * f0;
      r1 = r1 + voli * f1;
    }
  }
  R[2 * i] = r0;
  R[2 * i + 1] = r1;
}

cudaError_t launch_reaction(const StepParams &P, const DevPtrs &D, int cur, bool fp32,
                            double min_x, double max_x, double max_y, double *R, cudaStream_t s) {
  if (P.n == 0) return cudaSuccess;
  k_reaction<<<(unsigned)((P.n + 127) / 128), 128, 0, s>>>(P, D, cur, fp32, min_x, max_x, max_y, R);
  return cudaGetLastError();
}

cudaError_t launch_energy(const StepParams &P, const DevPtrs &D, int cur, int vcur, bool fp32,
                          const double *fext, float *strain, float *work, float *kinetic,
                          float *fracture, cudaStream_t s) {
  if (P.n == 0) return cudaSuccess;
  const unsigned grid = (unsigned)((P.n + 127) / 128);
  if (P.dim == 2)
    k_energy<2><<<grid, 128, 0, s>>>(P, D, cur, vcur, fp32, fext, strain, work, kinetic, fracture);
  else
    k_energy<3><<<grid, 128, 0, s>>>(P, D, cur, vcur, fp32, fext, strain, work, kinetic, fracture);
  return cudaGetLastError();
}

cudaError_t launch_damage(const StepParams &P, const DevPtrs &D, int cur, bool fp32, bool es,
                          float *phi, float *Z, cudaStream_t s) {
  if (P.n == 0) return cudaSuccess;
  const int bs = 128;
  const unsigned grid = (unsigned)((P.n + bs - 1) / bs);
  if (P.dim == 2)
    k_damage<2><<<grid, bs, 0, s>>>(P, D, cur, fp32, es, phi, Z);
  else
    k_damage<3><<<grid, bs, 0, s>>>(P, D, cur, fp32, es, phi, Z);
  return cudaGetLastError();
}

}  // namespace nlm

namespace nlm {

// Second half of integrate_node64 / integrate_node32 on its own.
template <int DIM>
__global__ void k_drift64(const StepParams P, const DevPtrs D, const BCTable T, int cur,
                          double t_next) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  const uint8_t fl = D.flags[i];
  const int ref = (fl & 7) ? D.bcref[i] : -1;
  double ui[3], v[3], f[3], un[3] = {0., 0., 0.}, vn[3] = {0., 0., 0.};
  ld_node<DIM>(D.u64[cur], i, ui);
  ld_node<DIM>(D.v[P.scheme == NLM_CENTRAL_DIFFERENCE ? cur : 0], i, v);
  ld_node<DIM>(D.f64, i, f);
  for (int d = 0; d < DIM; d++) {
    if (!(fl >> d & 1)) {
      if (P.scheme == NLM_VELOCITY_VERLET) {
        const double fact = 0.5 * P.dt / P.rho;
        const double vh = v[d] + fact * f[d];
        un[d] = ui[d] + P.dt * vh;
      } else {
        const double fact = P.dt * P.dt / P.rho;
        un[d] = ui[d] + (fact * f[d] + P.dt * v[d]);
        vn[d] = (un[d] - ui[d]) / P.dt;
      }
    } else {
      double du, dv;
      bc_dof(D, T, ref, d, t_next, du, dv);
      un[d] = du;
      vn[d] = dv;
    }
  }
  st_node<DIM>(D.u64[1 - cur], i, un);
  if (P.scheme == NLM_CENTRAL_DIFFERENCE) st_node<DIM>(D.v[1 - cur], i, vn);
}

cudaError_t launch_drift(const StepParams &P, const DevPtrs &D, const BCTable &T, int cur,
                         double t_next, bool fp32, cudaStream_t s) {
  if (P.n == 0) return cudaSuccess;
  if (fp32) return launch_drift32(P, D, T, cur, t_next, s);
  const unsigned g = (unsigned)((P.n + 255) / 256);
  if (P.dim == 2)
    k_drift64<2><<<g, 256, 0, s>>>(P, D, T, cur, t_next);
  else
    k_drift64<3><<<g, 256, 0, s>>>(P, D, T, cur, t_next);
  return cudaGetLastError();
}

}  // namespace nlm
