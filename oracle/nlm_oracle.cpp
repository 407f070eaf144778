// nlm_oracle.cpp -- CPU ORACLE (test infrastructure only).
//
// A plain restatement of NLMech's explicit and quasi-static hot path, written
// to follow the reference's arithmetic operation by operation so that the
// FP64 results can be compared to the CUDA library to ~1 ulp per operation.
// Built with -ffp-contract=off so that no multiply-add is fused (the reference
// on x86-64 without -march flags fuses none either).
//
// Only tests/, bench.py's CPU-baseline leg and __graft_entry__.smoke() use this
// file.  The product library never links or loads it.
//
// Reference citations are paths inside the NLMech source tree.

#include "nlm_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

thread_local std::string g_err;

int fail(int code, const std::string &msg) {
  g_err = msg;
  return code;
}

// util::compare::definitelyGreaterThan / definitelyLessThan
// (src/util/compare.cpp:25-33, COMPARE_EPS = 1e-5 in src/util/compare.h:13).
inline double amax(double a, double b) {
  return std::abs(a) < std::abs(b) ? std::abs(b) : std::abs(a);
}
inline bool dGT(double a, double b) { return (a - b) > (amax(a, b) * 1e-5); }
inline bool dLT(double a, double b) { return (b - a) > (amax(a, b) * 1e-5); }

// util::Point3::dist (src/util/point.h:165-169).
inline double dist3(const double *a, const double *b) {
  return std::sqrt((a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]) +
                   (a[2] - b[2]) * (a[2] - b[2]));
}
inline double len3(const double *a) {
  return std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
}
inline double dot3(const double *a, const double *b) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

// ---------------------------------------------------------------------------
// Influence functions (src/material/pd/influenceFn.h:85-402).
struct Influence {
  int type = 0;
  double a0 = 0, a1 = 0, alpha = 0, beta = 0;
  double J(double r) const {
    if (type == 0) return a0;                             // :104-106
    if (type == 1) return a0 + a1 * r;                    // :210-212
    return alpha * std::exp(-r * r / beta);               // :330-332
  }
  double moment(int i) const {
    if (type == 0) return a0 / double(i + 1);             // :117-119
    if (type == 1) return (a0 / double(i + 1)) + (a1 / double(i + 2));
    double sq1 = std::sqrt(beta), sq2 = std::sqrt(M_PI);  // :349-372
    if (i == 0) return 0.5 * alpha * sq1 * sq2 * std::erf(1. / sq1);
    if (i == 1) return 0.5 * alpha * beta * (1. - std::exp(-1. / beta));
    if (i == 2)
      return 0.5 * alpha * beta * sq1 *
             (0.5 * sq2 * std::erf(1. / sq1) - (1. / sq1) * std::exp(-1. / beta));
    return 0.5 * alpha * beta * beta *
           (1. - (1. + 1. / beta) * std::exp(-1. / beta));
  }
};

Influence make_influence(const nlm_material &m, int dim) {
  Influence f;
  f.type = m.influence_type;
  int np = m.n_influence_params;
  if (f.type == 0) {
    f.a0 = np == 0 ? double(dim + 1) : m.influence_params[0];  // :95
  } else if (f.type == 1) {                                    // :177-198
    if (np == 0) {
      f.a0 = dim == 1 ? 6. : (dim == 2 ? 12. : 20.);
      f.a1 = -f.a0;
    } else {
      f.a0 = m.influence_params[0];
      f.a1 = np < 2 ? -f.a0 : m.influence_params[1];
    }
  } else {                                                     // :285-305
    if (np == 0) {
      f.beta = 0.2;
      if (dim == 1)
        f.alpha = 2. / (f.beta * (1. - std::exp(-1. / f.beta)));
      else if (dim == 2)
        f.alpha = (4.0 / f.beta) * 1.0 /
                  (std::sqrt(M_PI * f.beta) * std::erf(1.0 / std::sqrt(f.beta)) -
                   2.0 * std::exp(-1.0 / f.beta));
      else
        f.alpha = (2.0 / f.beta) * 1.0 /
                  (f.beta - (f.beta + 1.) * std::exp(-1.0 / f.beta));
    } else {
      f.alpha = m.influence_params[0];
      f.beta = m.influence_params[1];
    }
  }
  return f;
}

// RNPBond constants (src/material/pd/rnpBond.cpp:23-189).
struct RNP {
  double C = 0, beta = 0, rbar = 0, invF = 0, M = 0, nu = 0, lambda = 0;
  double K = 0;                          // bulk modulus as the deck ends up with it
  bool contact = false;
  double kn = 0, rc = 0;                 // contact constants (ctor :79-88)
  double fsc = 1;
  bool irrev = true;
  Influence J;
};

int make_rnp(const nlm_material &m, int dim, double horizon, RNP &r) {
  r.J = make_influence(m, dim);
  r.M = r.J.moment(dim);                                   // :63
  r.irrev = m.irreversible != 0;
  r.fsc = m.check_sc_factor;
  if (dim == 1)
    r.invF = std::pow(horizon, 2) * 2.;                    // :67-72
  else if (dim == 2)
    r.invF = std::pow(horizon, 3) * M_PI;
  else
    r.invF = std::pow(horizon, 4) * 4. * M_PI / 3.;
  if (m.compute_from_classical) {                          // computeParameters
    double E = m.E, K = m.K, Gc = m.Gc, KIc = m.KIc;
    if (dLT(E, 0.) && dLT(K, 0.))
      return fail(NLM_ERR_INVALID, "RNPBond needs E or K");
    if (dLT(Gc, 0.) && dLT(KIc, 0.))
      return fail(NLM_ERR_INVALID, "RNPBond needs Gc or KIc");
    double nu = m.plane_strain ? 0.25 : 1. / 3.;           // :138-153
    if (E > 0.) K = E / (3. * (1. - 2. * nu));             // toK
    if (K > 0. && E < 0.) E = K * (3. * (1. - 2. * nu));   // toE
    if (Gc > 0.) KIc = std::sqrt(Gc * E);                  // toKIc
    if (KIc > 0. && Gc < 0.) Gc = KIc * KIc / E;           // toGc
    double lambda = E * nu / ((1. + nu) * (1. - 2. * nu)); // toLambdaE
    r.nu = nu;
    r.lambda = lambda;
    r.K = K;
    if (dim == 2) {
      r.C = M_PI * Gc / (4. * r.M);
      r.beta = 4. * lambda / (r.C * r.M);
    } else if (dim == 3) {
      r.C = 2. * Gc / (3. * r.M);
      r.beta = 5. * lambda / (r.C * r.M);
    }
  } else {
    r.C = m.bond_params[0];
    r.beta = m.bond_params[1];
    // computeMaterialProperties (:190-211)
    r.nu = 0.33;
    r.lambda = dim == 2 ? r.C * r.M * r.beta / 4. : r.C * r.M * r.beta / 5.;
    const double E = r.lambda * (1. + r.nu) * (1. - 2. * r.nu) / r.nu;  // toELambda
    r.K = E / (3. * (1. - 2. * r.nu));                                   // toK
  }
  r.rbar = std::sqrt(0.5 / r.beta);
  // contact between the nodes of broken bonds (ctor :79-88); Rc set with h
  r.contact = m.apply_contact != 0;
  if (r.contact) r.kn = r.K * 18. / (M_PI * std::pow(horizon, 5));
  return NLM_OK;
}

// ElasticState constants (src/material/pd/ElasticState.cpp:47-158).
struct ES {
  double K = 0, mu = 0, nu = 0, E = 0, factor2D = 1;
  bool plane_strain = false;
  double sc = 0;
  bool ref_compat = false;
};

int make_es(const nlm_material &m, int dim, ES &e) {
  if (dim == 1 && dLT(m.E, 0.))
    return fail(NLM_ERR_INVALID, "ElasticState 1-D needs E");
  if (dim >= 2 && (m.K <= 0. || m.G <= 0.))
    return fail(NLM_ERR_INVALID, "ElasticState needs K and G");
  e.E = m.E;
  e.K = m.K;
  e.mu = m.G;
  e.nu = (3 * m.K - 2 * m.G) / (2 * (3 * m.K + m.G));     // toNuClassical
  e.plane_strain = m.plane_strain != 0;
  if (!e.plane_strain && dim == 2)
    e.factor2D = (2. * e.nu - 1.) / (e.nu - 1.);
  else
    e.factor2D = 1;
  e.sc = m.es_sc;
  e.ref_compat = m.es_ref_compat != 0;
  return NLM_OK;
}

// ---------------------------------------------------------------------------
// Neighbour lists.
void neighbors_brute(int64_t n, const double *x, double horizon,
                     std::vector<std::vector<int32_t>> &rows) {
  rows.assign(n, {});
  double rad = horizon + 1.0E-10;
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t i = 0; i < n; i++) {  // neighbor.cpp:69-89
    const double *xi = x + 3 * i;
    std::vector<int32_t> nb;
    for (int64_t j = 0; j < n; j++) {
      if (j == i) continue;
      if (dLT(dist3(xi, x + 3 * j), rad)) nb.push_back(int32_t(j));
    }
    rows[i] = std::move(nb);
  }
}

void neighbors_grid(int dim, int64_t n, const double *x, double horizon,
                    std::vector<std::vector<int32_t>> &rows) {
  rows.assign(n, {});
  double rad = horizon + 1.0E-10;
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int64_t i = 0; i < n; i++)
    for (int d = 0; d < 3; d++) {
      lo[d] = std::min(lo[d], x[3 * i + d]);
      hi[d] = std::max(hi[d], x[3 * i + d]);
    }
  double cs = rad * 1.001;
  int64_t nc[3];
  for (int d = 0; d < 3; d++) nc[d] = std::max<int64_t>(1, int64_t((hi[d] - lo[d]) / cs) + 1);
  auto cell_of = [&](const double *p, int64_t c[3]) {
    for (int d = 0; d < 3; d++) {
      int64_t k = int64_t((p[d] - lo[d]) / cs);
      c[d] = std::min<int64_t>(std::max<int64_t>(k, 0), nc[d] - 1);
    }
  };
  int64_t ncell = nc[0] * nc[1] * nc[2];
  std::vector<int64_t> start(ncell + 1, 0);
  std::vector<int64_t> cid(n);
  for (int64_t i = 0; i < n; i++) {
    int64_t c[3];
    cell_of(x + 3 * i, c);
    cid[i] = (c[2] * nc[1] + c[1]) * nc[0] + c[0];
    start[cid[i] + 1]++;
  }
  for (int64_t c = 0; c < ncell; c++) start[c + 1] += start[c];
  std::vector<int64_t> fillp(start.begin(), start.end() - 1), items(n);
  for (int64_t i = 0; i < n; i++) items[fillp[cid[i]]++] = i;
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < n; i++) {
    int64_t c[3];
    cell_of(x + 3 * i, c);
    std::vector<int32_t> nb;
    for (int64_t dz = -1; dz <= 1; dz++)
      for (int64_t dy = -1; dy <= 1; dy++)
        for (int64_t dx = -1; dx <= 1; dx++) {
          int64_t q[3] = {c[0] + dx, c[1] + dy, c[2] + dz};
          bool ok = true;
          for (int d = 0; d < 3; d++) ok = ok && q[d] >= 0 && q[d] < nc[d];
          if (!ok) continue;
          int64_t cc = (q[2] * nc[1] + q[1]) * nc[0] + q[0];
          for (int64_t s = start[cc]; s < start[cc + 1]; s++) {
            int64_t j = items[s];
            if (j == i) continue;
            if (dLT(dist3(x + 3 * i, x + 3 * j), rad)) nb.push_back(int32_t(j));
          }
        }
    std::sort(nb.begin(), nb.end());
    rows[i] = std::move(nb);
  }
  (void)dim;
}

// ---------------------------------------------------------------------------
// Pre-cracks (src/geometry/fracture.cpp:74-160, fractureDeck.h:115-186).
bool crack_pt_outside(const nlm_crack &c, const double *p) {
  if (c.orientation == -1)
    return dLT(p[1], c.pb[1]) || dGT(p[1], c.pt[1]);
  if (c.orientation == 1)
    return dLT(p[0], c.pb[0]) || dGT(p[0], c.pt[0]);
  if (c.orientation == 0) {
    // rotateCW2D(v, theta) = (cos t v.x + sin t v.y, -sin t v.x + cos t v.y)
    double px = p[0] - c.pb[0], py = p[1] - c.pb[1];
    double tx = c.pt[0] - c.pb[0], ty = c.pt[1] - c.pb[1];
    double ct = std::cos(c.theta), st = std::sin(c.theta);
    double pmx = ct * px + st * py;
    double ptx = ct * tx + st * ty;
    return dLT(pmx, 0.0) || dGT(pmx, ptx);
  }
  return true;
}
bool crack_left(const nlm_crack &c, const double *p) {
  double a = 0.5 * ((c.pt[0] - c.pb[0]) * (p[1] - c.pb[1]) -
                    (p[0] - c.pb[0]) * (c.pt[1] - c.pb[1]));
  return !dLT(a, 0.0);
}
// Planar patch (3-D extension): the segment x_i -> x_j crosses z = z0 inside
// the patch.  Sides are "below" (z < z0) and "at or above" (z >= z0).
bool plane_cuts(const nlm_crack &c, const double *a, const double *b) {
  bool sa = a[2] < c.z0, sb = b[2] < c.z0;
  if (sa == sb) return false;
  double t = (c.z0 - a[2]) / (b[2] - a[2]);
  double px = a[0] + t * (b[0] - a[0]);
  double py = a[1] + t * (b[1] - a[1]);
  return px >= c.lo[0] && px <= c.hi[0] && py >= c.lo[1] && py <= c.hi[1];
}

// ---------------------------------------------------------------------------
// Loading (src/loading/uLoading.cpp, fLoading.cpp).
bool in_region(const nlm_bc_set &bc, const double *p, int dim) {
  switch (bc.region) {
    case NLM_REGION_RECTANGLE:  // utilGeom.cpp:43-49
      return !(dLT(p[0], bc.x1 - 1.0E-12) || dLT(p[1], bc.y1 - 1.0E-12) ||
               dGT(p[0], bc.x2 + 1.0E-12) || dGT(p[1], bc.y2 + 1.0E-12));
    case NLM_REGION_LINE:  // uLoading.cpp:137-140
      return dGT(p[0], bc.x1) && dLT(p[0], bc.x2);
    case NLM_REGION_CIRCLE: {  // utilGeom.cpp:328-333
      double c[3] = {bc.x1, bc.y1, 0.};
      double d[3] = {p[0] - c[0], p[1] - c[1], p[2] - c[2]};
      return len3(d) <= bc.r1;
    }
    case NLM_REGION_TORUS: {
      double d[3] = {p[0] - bc.x1, p[1] - bc.y1, p[2]};
      return len3(d) <= bc.r1 && !(len3(d) <= bc.r2);
    }
    case NLM_REGION_CUBOID:  // utilGeom.cpp:97-115 with dim 3 (fLoading.cpp:104-107)
      return !(dLT(p[0], bc.x1 - 1.0E-12) || dLT(p[1], bc.y1 - 1.0E-12) ||
               dLT(p[2], bc.z1 - 1.0E-12) || dGT(p[0], bc.x2 + 1.0E-12) ||
               dGT(p[1], bc.y2 + 1.0E-12) || dGT(p[2], bc.z2 + 1.0E-12));
    case NLM_REGION_ANGLED_RECTANGLE: {  // utilGeom.cpp:60-95, transformation.cpp:20-24
      double lam[2] = {(bc.x2 - bc.x1) * std::cos(bc.theta) + (bc.y2 - bc.y1) * std::sin(bc.theta),
                       -(bc.x2 - bc.x1) * std::sin(bc.theta) + (bc.y2 - bc.y1) * std::cos(bc.theta)};
      double xm[2] = {(p[0] - bc.x1) * std::cos(bc.theta) + (p[1] - bc.y1) * std::sin(bc.theta),
                      -(p[0] - bc.x1) * std::sin(bc.theta) + (p[1] - bc.y1) * std::cos(bc.theta)};
      return !(dLT(xm[0], -1.0E-12) || dLT(xm[1], -1.0E-12) || dGT(xm[0], lam[0] + 1.0E-12) ||
               dGT(xm[1], lam[1] + 1.0E-12));
    }
  }
  return false;
}

double linear_step(double x, double x1, double x2) {  // utilFunction.cpp:46-54
  double period = std::floor(x / (x1 + x2));
  if (dLT(x, period * (x1 + x2) + x1)) return x - period * x2;
  return (period + 1.) * x1;
}
double der_linear_step(double x, double x1, double x2) {
  double period = std::floor(x / (x1 + x2));
  if (dLT(x, period * (x1 + x2) + x1)) return 1.;
  return 0.;
}

// ULoading::apply for one node of one set (uLoading.cpp:166-253).
void uload_value(const nlm_bc_set &bc, const double *x, double time, double &du,
                 double &dv) {
  double umax = bc.time_params[0];
  const double *sp = bc.spatial_params;
  switch (bc.spatial_fn) {
    case NLM_SFN_SIN_X: { double a = M_PI * sp[0]; umax = umax * std::sin(a * x[0]); } break;
    case NLM_SFN_SIN_Y: { double a = M_PI * sp[0]; umax = umax * std::sin(a * x[1]); } break;
    case NLM_SFN_SIN_Z: { double a = M_PI * sp[0]; umax = umax * std::sin(a * x[2]); } break;
    case NLM_SFN_LINEAR_X: { double a = sp[0]; umax = umax * a * x[0]; } break;
    case NLM_SFN_LINEAR_Y: { double a = sp[0]; umax = umax * a * x[1]; } break;
    case NLM_SFN_LINEAR_Z: { double a = sp[0]; umax = umax * a * x[2]; } break;
    case NLM_SFN_CONSTANT: { double a = sp[0]; umax = umax * a; } break;
    default: break;  // ULoading knows no other spatial function
  }
  du = 0.;
  dv = 0.;
  const double *tp = bc.time_params;
  switch (bc.time_fn) {
    case NLM_TFN_CONSTANT: du = umax; break;
    case NLM_TFN_LINEAR: du = umax * time; dv = umax; break;
    case NLM_TFN_QUADRATIC:
      du = umax * time + tp[1] * time * time;
      dv = umax + tp[1] * time;
      break;
    case NLM_TFN_SIN: {
      double a = M_PI * tp[1];
      du = umax * std::sin(a * time);
      dv = umax * a * std::cos(a * time);
    } break;
    case NLM_TFN_LINEAR_STEP:
      du = umax * linear_step(time, tp[1], tp[2]);
      dv = umax * der_linear_step(time, tp[1], tp[2]);
      break;
    case NLM_TFN_LINEAR_SLOW_FAST:
      if (dGT(time, tp[1])) {
        du = umax * tp[3] * time;
        dv = umax * tp[3];
      } else {
        du = umax * tp[2] * time;
        dv = umax * tp[2];
      }
      break;
  }
}

// FLoading::apply value for one node (fLoading.cpp:117-277, no hat/line_load).
// util::function::hatFunction (utilFunction.cpp:14-30).
double hat_function(double x, double x_min, double x_max) {
  if (dGT(x, x_min - 1.0E-12) && dLT(x, x_max + 1.0E-12)) {
    double x_mid = 0.5 * (x_min + x_max);
    double l = x_mid - x_min;
    if (l < 1.0E-12) return 1.0;
    if (dLT(x, x_mid)) return (x - x_min) / l;
    return (x_max - x) / l;
  }
  return 0.0;
}

// size_t conversion (truncation) of a count; negative values give 0.
double to_count(double v) { return v > 0. ? (v < 1.8e19 ? double(uint64_t(v)) : v) : 0.; }

double fload_value(const nlm_bc_set &bc, const double *x, double time, double h) {
  double fmax = 1.0;
  const double *sp = bc.spatial_params;
  switch (bc.spatial_fn) {
    case NLM_SFN_HAT_X: fmax = sp[0] * hat_function(x[0], bc.x1, bc.x2); break;
    case NLM_SFN_HAT_Y: fmax = sp[0] * hat_function(x[1], bc.y1, bc.y2); break;
    case NLM_SFN_HAT_Z: fmax = sp[0] * hat_function(x[2], bc.z1, bc.z2); break;
    case NLM_SFN_LINE_LOAD: {
      // fLoading.cpp:171-232 (the -1 branch's inner min/max are unused there)
      const double lo[3] = {bc.x1, bc.y1, bc.z1}, hi[3] = {bc.x2, bc.y2, bc.z2};
      for (int d = 0; d < 3; d++) {
        if (!(bc.dir_mask >> d & 1)) continue;
        double length = std::abs(hi[d] - lo[d]);
        double nodes = to_count(length / h);
        double scale = 1. / nodes;
        double pos = to_count((x[d] - lo[d]) / h);
        if (sp[0] == -1) pos = to_count((hi[d] - x[d]) / h);
        fmax *= pos * scale;
      }
    } break;
    case NLM_SFN_SIN_X: { double a = M_PI * sp[0]; fmax = sp[0] * std::sin(a * x[0]); } break;
    case NLM_SFN_SIN_Y: { double a = M_PI * sp[0]; fmax = sp[0] * std::sin(a * x[1]); } break;
    case NLM_SFN_SIN_Z: { double a = M_PI * sp[0]; fmax = sp[0] * std::sin(a * x[2]); } break;
    case NLM_SFN_LINEAR_X: { double a = sp[0]; fmax = sp[0] * a * x[0]; } break;
    case NLM_SFN_LINEAR_Y: { double a = sp[0]; fmax = sp[0] * a * x[1]; } break;
    case NLM_SFN_LINEAR_Z: { double a = sp[0]; fmax = sp[0] * a * x[2]; } break;
    default: fmax = sp[0]; break;
  }
  const double *tp = bc.time_params;
  switch (bc.time_fn) {
    case NLM_TFN_LINEAR: fmax *= time; break;
    case NLM_TFN_LINEAR_STEP: fmax *= linear_step(time, tp[1], tp[2]); break;
    case NLM_TFN_LINEAR_SLOW_FAST:
      if (dGT(time, tp[1])) fmax *= tp[3] * time; else fmax *= tp[2] * time;
      break;
    case NLM_TFN_SIN: { double a = M_PI * tp[1]; fmax *= std::sin(a * time); } break;
    default: break;
  }
  fmax *= tp[0];
  return fmax;
}

// ---------------------------------------------------------------------------
// Shared model setup.
struct Model {
  int dim = 2;
  int64_t n = 0;
  std::vector<double> x, vol;
  double delta = 0, h = 0;
  nlm_material mat{};
  RNP rnp;
  ES es;
  std::vector<int64_t> rowptr;
  std::vector<int32_t> cols;
  std::vector<uint8_t> broken;  // one byte per CSR entry
  std::vector<nlm_crack> timed; // timed cracks (Activation_Time >= 0)
  uint32_t cracks_on = 0;       // bit c: timed crack c has been cut
  std::vector<uint8_t> fix;     // bit d = dof d fixed
  std::vector<uint8_t> interior;
  std::vector<nlm_bc_set> ubc, fbc;
  std::vector<std::vector<int64_t>> ubc_nodes, fbc_nodes;
  std::vector<double> u, v, f;
  // ElasticState fields
  std::vector<double> omega, mw, theta;
};

// Fracture::computeFracturedBondFd (fracture.cpp:74-160) over every node:
// bonds that cross the crack are marked broken.
void cut_crack(Model &m, const nlm_crack &ck) {
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < m.n; i++) {
    const double *xi = &m.x[3 * i];
    if (ck.kind == NLM_CRACK_PLANE) {
      for (int64_t k = m.rowptr[i]; k < m.rowptr[i + 1]; k++)
        if (plane_cuts(ck, xi, &m.x[3 * int64_t(m.cols[k])])) m.broken[k] = 1;
      continue;
    }
    if (crack_pt_outside(ck, xi)) continue;
    bool left = crack_left(ck, xi);
    for (int64_t k = m.rowptr[i]; k < m.rowptr[i + 1]; k++) {
      const double *xj = &m.x[3 * int64_t(m.cols[k])];
      bool modify = !crack_pt_outside(ck, xj);
      bool other = left ? !crack_left(ck, xj) : crack_left(ck, xj);
      if (other && modify) m.broken[k] = 1;
    }
  }
}

// Fracture::addCrack (fracture.cpp:45-70) for a step that ended at time: the
// first timed crack not yet cut whose activation time is definitely less than
// time is cut; at most one per call.  Called before the next step rather than
// after the step's output (fDModel.cpp:352-373): the same point for the
// dynamics.
void add_crack(Model &m, double time) {
  for (size_t c = 0; c < m.timed.size(); c++) {
    if (m.cracks_on >> c & 1u) continue;
    if (!dLT(m.timed[c].activation_time, time)) continue;
    cut_crack(m, m.timed[c]);
    m.cracks_on |= 1u << c;
    return;
  }
}

int setup_model(const nlm_fd_desc *d, bool grid, Model &m) {
  if (!d || d->n_nodes < 0 || d->dim < 1 || d->dim > 3 || (d->n_nodes > 0 && (!d->x || !d->volume)))
    return fail(NLM_ERR_INVALID, "bad description");
  m.dim = d->dim;
  m.n = d->n_nodes;
  m.x.assign(d->x, d->x + 3 * m.n);
  m.vol.assign(d->volume, d->volume + m.n);
  m.delta = d->horizon;
  m.h = d->mesh_size;
  m.mat = d->material;
  int rc;
  if (m.mat.kind == NLM_MAT_RNP_BOND) {
    if ((rc = make_rnp(m.mat, m.dim, m.delta, m.rnp))) return rc;
    m.rnp.rc = 0.9 * m.h;
  } else {
    if ((rc = make_es(m.mat, m.dim, m.es))) return rc;
  }
  // neighbours
  std::vector<std::vector<int32_t>> rows;
  if (grid)
    neighbors_grid(m.dim, m.n, m.x.data(), m.delta, rows);
  else
    neighbors_brute(m.n, m.x.data(), m.delta, rows);
  m.rowptr.assign(m.n + 1, 0);
  for (int64_t i = 0; i < m.n; i++) m.rowptr[i + 1] = m.rowptr[i] + int64_t(rows[i].size());
  m.cols.resize(m.rowptr[m.n]);
  for (int64_t i = 0; i < m.n; i++)
    std::copy(rows[i].begin(), rows[i].end(), m.cols.begin() + m.rowptr[i]);
  // pre-cracks (Fracture ctor, fracture.cpp:20-43: every crack with
  // activation time < 0 is applied at construction); timed cracks wait for
  // Fracture::addCrack
  m.broken.assign(m.cols.size(), 0);
  for (int c = 0; c < d->n_cracks; c++) {
    if (d->cracks[c].timed) {
      if (m.timed.size() >= 32) return fail(NLM_ERR_INVALID, "more than 32 timed cracks");
      m.timed.push_back(d->cracks[c]);
    } else
      cut_crack(m, d->cracks[c]);
  }
  // interior flags (interiorFlags.cpp:27-100, 121-191)
  m.interior.assign(m.n, 1);
  if (d->no_fail != NLM_NOFAIL_OFF && m.n > 0) {
    // fe::Mesh::computeBBox (mesh.cpp:311-324): both corners start at the
    // origin; DataInterior (:146-185) stores the same flags ComputeInterior
    // computes
    double lo[3] = {0., 0., 0.}, hi[3] = {0., 0., 0.};
    for (int64_t i = 0; i < m.n; i++)  // fe::Mesh bounding box
      for (int dd = 0; dd < 3; dd++) {
        if (dLT(m.x[3 * i + dd], lo[dd])) lo[dd] = m.x[3 * i + dd];
        if (dLT(hi[dd], m.x[3 * i + dd])) hi[dd] = m.x[3 * i + dd];
      }
    double tol = d->no_fail_tol;
    for (int64_t i = 0; i < m.n; i++) {
      const double *p = &m.x[3 * i];
      bool in = !(dLT(p[0], lo[0] + tol) || dLT(p[1], lo[1] + tol) ||
                  dGT(p[0], hi[0] - tol) || dGT(p[1], hi[1] - tol));
      // No_Fail_Region list (:76-90)
      for (int r = 0; r < d->n_nofail_regions && d->nofail_regions; r++) {
        const double *q = d->nofail_regions[r].params;
        if (d->nofail_regions[r].kind == NLM_NOFAIL_CIRCLE) {
          const double c[3] = {q[0], q[1], q[2]};
          if (dLT(dist3(c, p), q[3])) in = false;
        } else if (!(dLT(p[0], q[0] - 1.0E-12) || dLT(p[1], q[1] - 1.0E-12) ||
                     dGT(p[0], q[2] + 1.0E-12) || dGT(p[1], q[3] + 1.0E-12))) {
          in = false;
        }
      }
      m.interior[i] = in ? 1 : 0;
    }
  }
  // loads (ULoading ctor uLoading.cpp:18-164, FLoading ctor fLoading.cpp:18-116)
  m.fix.assign(m.n, 0);
  m.ubc.assign(d->ubc, d->ubc + d->n_ubc);
  m.fbc.assign(d->fbc, d->fbc + d->n_fbc);
  for (auto &bc : m.ubc) {
    std::vector<int64_t> nodes;
    for (int64_t i = 0; i < m.n; i++)
      if (in_region(bc, &m.x[3 * i], m.dim)) {
        nodes.push_back(i);
        m.fix[i] |= uint8_t(bc.dir_mask & 7);
      }
    m.ubc_nodes.push_back(nodes);
  }
  for (auto &bc : m.fbc) {
    std::vector<int64_t> nodes;
    for (int64_t i = 0; i < m.n; i++)
      if (in_region(bc, &m.x[3 * i], m.dim)) nodes.push_back(i);
    m.fbc_nodes.push_back(nodes);
  }
  m.u.assign(3 * m.n, 0.);
  m.v.assign(3 * m.n, 0.);
  m.f.assign(3 * m.n, 0.);
  if (d->u0) m.u.assign(d->u0, d->u0 + 3 * m.n);
  if (d->v0) m.v.assign(d->v0, d->v0 + 3 * m.n);
  // ElasticState: volume correction and weighted volume
  // (volumeCorrection.cpp:25-67); omega uses h = mesh size.
  if (m.mat.kind == NLM_MAT_ELASTIC_STATE) {
    m.omega.assign(m.cols.size(), 1.);
    m.mw.assign(m.n, 1.);
    m.theta.assign(m.n, 0.);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < m.n; i++) {
      double tmp = 0;
      for (int64_t k = m.rowptr[i]; k < m.rowptr[i + 1]; k++) {
        int64_t j = m.cols[k];
        double X[3] = {m.x[3 * j] - m.x[3 * i], m.x[3 * j + 1] - m.x[3 * i + 1],
                       m.x[3 * j + 2] - m.x[3 * i + 2]};
        double r = m.h * 0.5;
        if (dGT(len3(X), m.delta - r)) m.omega[k] = (m.delta + r - len3(X)) / m.h;
        tmp += (len3(X) * len3(X) * m.omega[k] * m.vol[j]);
      }
      m.mw[i] = tmp;
    }
  }
  return NLM_OK;
}

void apply_uload(Model &m, double time, double *u, double *v) {
  for (size_t s = 0; s < m.ubc.size(); s++) {
    const nlm_bc_set &bc = m.ubc[s];
    for (int64_t i : m.ubc_nodes[s]) {
      double du, dv;
      uload_value(bc, &m.x[3 * i], time, du, dv);
      for (int d = 0; d < 3; d++)
        if (bc.dir_mask & (1 << d)) {
          u[3 * i + d] = du;
          v[3 * i + d] = dv;
        }
    }
  }
}

void apply_fload(Model &m, double time, double *f) {
  for (size_t s = 0; s < m.fbc.size(); s++) {
    const nlm_bc_set &bc = m.fbc[s];
    for (int64_t i : m.fbc_nodes[s]) {
      double fm = fload_value(bc, &m.x[3 * i], time, m.h);
      for (int d = 0; d < 3; d++)
        if (bc.dir_mask & (1 << d)) f[3 * i + d] += fm;
    }
  }
}

// RNPBond::getBondEF (rnpBond.cpp:216-301) for bond k = (i, j_local) with the
// contact term off; updates the bond state, returns force and energy.
inline void rnp_bond(const Model &m, const double *u, int64_t i, int64_t k,
                     uint8_t &fs_io, double force[3], double *energy,
                     bool update_state) {
  const RNP &p = m.rnp;
  int64_t j = m.cols[k];
  bool fs = fs_io != 0;
  const double *xi = &m.x[3 * i], *xj = &m.x[3 * j];
  const double *ui = &u[3 * i], *uj = &u[3 * j];
  bool break_bonds = m.interior[i] && m.interior[j];
  double rji = dist3(xj, xi);
  double dx[3] = {xj[0] - xi[0], xj[1] - xi[1], xj[2] - xi[2]};
  double du[3] = {uj[0] - ui[0], uj[1] - ui[1], uj[2] - ui[2]};
  double Sji = dot3(dx, du) / dot3(dx, dx);  // getS :303-306
  double l = len3(dx);
  double e[3] = {dx[0] / l, dx[1] / l, dx[2] / l};  // direction :330-333
  double h = m.h;
  double check_up = m.delta + 0.5 * h;
  double check_low = m.delta - 0.5 * h;
  double volj = m.vol[j];
  if (dGT(rji, check_low)) volj *= (check_up - rji) / h;
  double influence = p.J.J(rji / m.delta);
  double s = 0, en = 0;
  if (break_bonds) {
    if (p.irrev && !fs && dGT(std::abs(Sji), p.fsc * (p.rbar / std::sqrt(rji))))
      fs = true;
    if (update_state) fs_io = fs ? 1 : 0;
    if (!fs) {
      en = (influence * p.C * (1. - std::exp(-p.beta * rji * Sji * Sji)) / p.invF) * volj;
      s = (influence * 4. * Sji * p.C * p.beta *
           std::exp(-p.beta * rji * Sji * Sji) / p.invF) * volj;
    } else {
      en = influence * p.C / p.invF * volj;
      s = 0.;
      if (p.contact) {
        // normal contact force between the nodes of the broken bond (:281-291)
        const double voli = m.vol[i];
        double y[3];
        for (int c = 0; c < 3; c++) y[c] = (xj[c] + uj[c]) - (xi[c] + ui[c]);
        const double R = std::sqrt(y[0] * y[0] + y[1] * y[1] + y[2] * y[2]);
        double sf = p.kn * (voli * volj / (voli + volj)) * (p.rc - R) / R;
        if (sf < 0.) sf = 0.;
        for (int c = 0; c < 3; c++) force[c] = 0. + -sf * y[c];
        if (energy) *energy = en;
        return;
      }
    }
  } else {
    en = (influence * p.C * p.beta * rji * Sji * Sji / p.invF) * volj;
    s = (influence * 4. * Sji * p.C * p.beta / p.invF) * volj;
  }
  force[0] = s * e[0];
  force[1] = s * e[1];
  force[2] = s * e[2];
  if (energy) *energy = en;
}

// FDModel::computeForces (fDModel.cpp:527-582): f_i += sum_j F_ij.
void rnp_forces(Model &m, const double *u, double *f, bool update_state) {
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < m.n; i++) {
    double fi[3] = {0., 0., 0.};
    for (int64_t k = m.rowptr[i]; k < m.rowptr[i + 1]; k++) {
      double F[3];
      uint8_t fs = m.broken[k];
      rnp_bond(m, u, i, k, fs, F, nullptr, update_state);
      if (update_state) m.broken[k] = fs;
      fi[0] += F[0];
      fi[1] += F[1];
      fi[2] += F[2];
    }
    f[3 * i] += fi[0];
    f[3 * i + 1] += fi[1];
    f[3 * i + 2] += fi[2];
  }
}

// ElasticState explicit two-pass force in gather form (build definition):
// pass 1 = extension, break test (e/|X| > s_c), dilatation over intact bonds
// (stateBasedHelperFunctions.cpp:26-83); pass 2 = f_i = sum_j (t_ij + t_ji)
// M_ij omega_ij V_j (the gather form of the scatter in
// QuasiStaticModel.cpp:168-239 with getBondEF, ElasticState.cpp:160-271).
double es_t(const Model &m, int64_t i, double e, double Xlen) {
  const ES &p = m.es;
  double mi = m.mw[i];
  if (m.dim == 1) {
    double alpha = p.E / mi;
    return alpha * 1. * e;
  }
  if (m.dim == 2) {
    double alpha_s;
    if (!p.plane_strain) {
      // std::pow(q, 2) in the reference; a correctly rounded square either way
      const double q = (p.nu + 1.) / (2. * p.nu - 1.);
      alpha_s = (9. / mi) * (p.K + q * q * p.mu / 9.);
    }
    else {
      alpha_s = (9. / mi) * (p.K + p.mu / 9.);
    }
    double alpha_d = (8. / mi) * p.mu;
    double e_s = m.theta[i] * Xlen / 3.;
    double e_d = e - e_s;
    double t_s = (2. * p.factor2D * alpha_s - (3. - 2. * p.factor2D) * alpha_d) * 1. * e_s / 3.;
    double t_d = alpha_d * 1. * e_d;
    return t_s + t_d;
  }
  double alpha_s = (9. / mi) * p.K;
  double alpha_d = (15. / mi) * p.mu;
  double e_s = m.theta[i] * Xlen / 3.;
  double e_d = p.ref_compat ? 0. : e - e_s;
  double t_s = alpha_s * 1. * e_s;
  double t_d = alpha_d * 1. * e_d;
  return t_s + t_d;
}

void es_bond_geom(const Model &m, const double *u, int64_t i, int64_t j, double Y[3],
                  double &Xlen, double &e) {
  double X[3];
  for (int d = 0; d < 3; d++) {
    Y[d] = (m.x[3 * j + d] + u[3 * j + d]) - (m.x[3 * i + d] + u[3 * i + d]);
    X[d] = m.x[3 * j + d] - m.x[3 * i + d];
  }
  Xlen = len3(X);
  e = len3(Y) - Xlen;  // stateBasedHelperFunctions.cpp:47
}

void es_dilatation(Model &m, const double *u, bool update_state) {
  double c = m.dim == 1 ? 1. : (m.dim == 2 ? 2. : 3.);
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < m.n; i++) {
    double th = 0.;
    for (int64_t k = m.rowptr[i]; k < m.rowptr[i + 1]; k++) {
      int64_t j = m.cols[k];
      double Y[3], Xl, e;
      es_bond_geom(m, u, i, j, Y, Xl, e);
      if (update_state && m.es.sc > 0 && !m.broken[k] && dGT(e / Xl, m.es.sc))
        m.broken[k] = 1;
      if (m.broken[k]) continue;
      double fac = m.dim == 2 ? m.es.factor2D : 1.;
      th += (c / m.mw[i]) * fac * 1. * Xl * e * m.omega[k] * m.vol[j];
    }
    m.theta[i] = th;
  }
}

void es_forces_gather(Model &m, const double *u, double *f, bool update_state) {
  es_dilatation(m, u, update_state);
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < m.n; i++) {
    double fi[3] = {0., 0., 0.};
    for (int64_t k = m.rowptr[i]; k < m.rowptr[i + 1]; k++) {
      if (m.broken[k]) continue;
      int64_t j = m.cols[k];
      double Y[3], Xl, e;
      es_bond_geom(m, u, i, j, Y, Xl, e);
      double Yl = len3(Y);
      double tsum = es_t(m, i, e, Xl) + es_t(m, j, e, Xl);
      double s = tsum * m.omega[k] * m.vol[j];
      for (int d = 0; d < 3; d++) fi[d] += (Y[d] / Yl) * s;
    }
    for (int d = 0; d < 3; d++) f[3 * i + d] += fi[d];
  }
}

void internal_forces(Model &m, const double *u, double *f, bool update_state) {
  if (m.mat.kind == NLM_MAT_RNP_BOND)
    rnp_forces(m, u, f, update_state);
  else
    es_forces_gather(m, u, f, update_state);
}

}  // namespace

// ===========================================================================
extern "C" {

const char *orc_last_error(void) { return g_err.c_str(); }
int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
void orc_set_num_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}
int orc_definitely_less_than(double a, double b) { return dLT(a, b) ? 1 : 0; }
int orc_definitely_greater_than(double a, double b) { return dGT(a, b) ? 1 : 0; }

static int rows_out(const std::vector<std::vector<int32_t>> &rows, int64_t *rowptr,
                    int32_t *cols) {
  int64_t n = int64_t(rows.size());
  rowptr[0] = 0;
  for (int64_t i = 0; i < n; i++) rowptr[i + 1] = rowptr[i] + int64_t(rows[i].size());
  if (cols)
    for (int64_t i = 0; i < n; i++)
      std::copy(rows[i].begin(), rows[i].end(), cols + rowptr[i]);
  return NLM_OK;
}

int orc_neighbors_brute(int64_t n, const double *x, double horizon, int64_t *rowptr,
                        int32_t *cols) {
  if (n < 0 || !rowptr || (n > 0 && !x)) return fail(NLM_ERR_INVALID, "bad args");
  std::vector<std::vector<int32_t>> rows;
  neighbors_brute(n, x, horizon, rows);
  return rows_out(rows, rowptr, cols);
}

int orc_neighbors_grid(int dim, int64_t n, const double *x, double horizon,
                       int64_t *rowptr, int32_t *cols) {
  if (n < 0 || !rowptr || (n > 0 && !x)) return fail(NLM_ERR_INVALID, "bad args");
  std::vector<std::vector<int32_t>> rows;
  neighbors_grid(dim, n, x, horizon, rows);
  return rows_out(rows, rowptr, cols);
}

int orc_rnp_params(const nlm_material *m, int dim, double horizon, double *out) {
  RNP r;
  int rc = make_rnp(*m, dim, horizon, r);
  if (rc) return rc;
  out[0] = r.C;
  out[1] = r.beta;
  out[2] = r.rbar;
  out[3] = r.invF;
  out[4] = r.M;
  out[5] = r.nu;
  out[6] = r.lambda;
  return NLM_OK;
}

struct orc_fd {
  Model m;
  int scheme = NLM_VELOCITY_VERLET;
  double dt = 0, time = 0;
  int64_t step = 0;
  bool started = false;
};

int orc_fd_create(const nlm_fd_desc *d, int use_grid, orc_fd **out) {
  if (!out) return fail(NLM_ERR_INVALID, "null out");
  auto *h = new orc_fd();
  int rc = setup_model(d, use_grid != 0, h->m);
  if (rc) {
    delete h;
    return rc;
  }
  h->scheme = d->scheme;
  h->dt = d->dt;
  *out = h;
  return NLM_OK;
}

int orc_fd_destroy(orc_fd *h) {
  delete h;
  return NLM_OK;
}

int orc_fd_num_bonds(const orc_fd *h, int64_t *nnz) {
  *nnz = int64_t(h->m.cols.size());
  return NLM_OK;
}

int orc_fd_get_neighbors(const orc_fd *h, int64_t *rowptr, int32_t *cols) {
  if (rowptr) std::copy(h->m.rowptr.begin(), h->m.rowptr.end(), rowptr);
  if (cols) std::copy(h->m.cols.begin(), h->m.cols.end(), cols);
  return NLM_OK;
}

// FDModel::integrate (fDModel.cpp:317-374) with integrateVerlet (:445-525)
// or integrateCD (:376-443), after the timed-crack check of the step before.
// Output I/O is not part of it.
int orc_fd_run(orc_fd *h, int64_t nsteps) {
  Model &m = h->m;
  double *u = m.u.data(), *v = m.v.data(), *f = m.f.data();
  if (!h->started) {
    // step 0: IC is the initial state; loads at t = 0; forces (:319-333)
    apply_uload(m, h->time, u, v);
    std::fill(m.f.begin(), m.f.end(), 0.);
    apply_fload(m, h->time, f);
    internal_forces(m, u, f, true);
    h->started = true;
  }
  double rho = m.mat.density;
  for (int64_t s = 0; s < nsteps; s++) {
    if (h->step > 0) add_crack(m, h->time);  // fDModel.cpp:366-373
    if (h->scheme == NLM_VELOCITY_VERLET) {
      double fact = 0.5 * h->dt / rho;
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < m.n; i++) {
        for (int d = 0; d < m.dim; d++)
          if (!(m.fix[i] >> d & 1)) {
            v[3 * i + d] += fact * f[3 * i + d];
            u[3 * i + d] += h->dt * v[3 * i + d];
          }
        f[3 * i] = f[3 * i + 1] = f[3 * i + 2] = 0.;
      }
    } else {
      double fact = h->dt * h->dt / rho;
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < m.n; i++) {
        for (int d = 0; d < m.dim; d++)
          if (!(m.fix[i] >> d & 1)) {
            double u_old = u[3 * i + d];
            u[3 * i + d] += fact * f[3 * i + d] + h->dt * v[3 * i + d];
            v[3 * i + d] = (u[3 * i + d] - u_old) / h->dt;
          }
        f[3 * i] = f[3 * i + 1] = f[3 * i + 2] = 0.;
      }
    }
    h->step++;
    h->time += h->dt;
    apply_uload(m, h->time, u, v);
    apply_fload(m, h->time, f);
    internal_forces(m, u, f, true);
    if (h->scheme == NLM_VELOCITY_VERLET) {
      double fact = 0.5 * h->dt / rho;
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < m.n; i++)
        for (int d = 0; d < m.dim; d++)
          if (!(m.fix[i] >> d & 1)) v[3 * i + d] += fact * f[3 * i + d];
    }
  }
  return NLM_OK;
}

int orc_fd_get_state(const orc_fd *h, double *u, double *v, double *f) {
  size_t n3 = h->m.u.size();
  if (u) std::memcpy(u, h->m.u.data(), n3 * sizeof(double));
  if (v) std::memcpy(v, h->m.v.data(), n3 * sizeof(double));
  if (f) std::memcpy(f, h->m.f.data(), n3 * sizeof(double));
  return NLM_OK;
}

int orc_fd_set_state(orc_fd *h, const double *u, const double *v) {
  size_t n3 = h->m.u.size();
  if (u) std::memcpy(h->m.u.data(), u, n3 * sizeof(double));
  if (v) std::memcpy(h->m.v.data(), v, n3 * sizeof(double));
  return NLM_OK;
}

int orc_fd_get_time(const orc_fd *h, double *t, int64_t *n) {
  if (t) *t = h->time;
  if (n) *n = h->step;
  return NLM_OK;
}

int orc_fd_get_bond_state(const orc_fd *h, uint8_t *broken) {
  std::copy(h->m.broken.begin(), h->m.broken.end(), broken);
  return NLM_OK;
}

int orc_fd_set_bond_state(orc_fd *h, const uint8_t *broken) {
  std::copy(broken, broken + h->m.broken.size(), h->m.broken.begin());
  return NLM_OK;
}

int orc_fd_get_fixity(const orc_fd *h, uint8_t *fix) {
  std::copy(h->m.fix.begin(), h->m.fix.end(), fix);
  return NLM_OK;
}

// FDModel::computePostProcFields damage part (fDModel.cpp:651-778).
int orc_fd_damage(orc_fd *h, float *phi, float *Z) {
  Model &m = h->m;
  if (m.mat.kind != NLM_MAT_RNP_BOND) {
    // ElasticState: phi from the bond state with the same volume weights.
  }
  double check_up = m.delta + 0.5 * m.h, check_low = m.delta - 0.5 * m.h;
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < m.n; i++) {
    double a = 0., b = 0., z = 0.;
    const double *xi = &m.x[3 * i], *ui = &m.u[3 * i];
    for (int64_t k = m.rowptr[i]; k < m.rowptr[i + 1]; k++) {
      int64_t j = m.cols[k];
      bool fs = m.broken[k] != 0;
      const double *xj = &m.x[3 * j], *uj = &m.u[3 * j];
      double rji = dist3(xj, xi);
      double dx[3] = {xj[0] - xi[0], xj[1] - xi[1], xj[2] - xi[2]};
      double du[3] = {uj[0] - ui[0], uj[1] - ui[1], uj[2] - ui[2]};
      double Sji = dot3(dx, du) / dot3(dx, dx);
      double volj = m.vol[j];
      if (dGT(rji, check_low)) volj *= (check_up - rji) / m.h;
      if (!fs) a += volj;
      b += volj;
      double sr = 0.;
      if (m.mat.kind == NLM_MAT_RNP_BOND) {
        if (dGT(rji, 1.0E-12)) sr = std::abs(Sji) / (m.rnp.rbar / std::sqrt(rji));
      } else if (m.es.sc > 0) {
        double Y[3], Xl, e;
        es_bond_geom(m, m.u.data(), i, j, Y, Xl, e);
        sr = std::abs(e / Xl) / m.es.sc;
      }
      if (dLT(z, sr)) z = sr;
    }
    if (phi) phi[i] = float(b > 0 ? 1. - a / b : 0.);
    if (Z) Z[i] = float(z);
  }
  return NLM_OK;
}

// FDModel::computePostProcFields energies (fDModel.cpp:651-778), RNPBond:
// strain energy (sum_j getBondEF energy) V_i with the bond breaking of
// getBondEF applied to a copy of the state, work done u_i . f_ext(t),
// kinetic energy rho |v_i|^2 V_i / 2, fracture energy where Z_i > 1 - 1e-10
// (0 elsewhere).  totals[4]: FP64 sums of the float fields.
int orc_fd_energies(orc_fd *h, float *strain, float *work, float *kinetic, float *fracture,
                    double *totals) {
  Model &m = h->m;
  if (m.mat.kind != NLM_MAT_RNP_BOND) return NLM_ERR_UNSUPPORTED;
  std::vector<double> fext(3 * m.n, 0.);
  apply_fload(m, h->time, fext.data());
  std::vector<float> e(4 * m.n);
  const double rho = m.mat.density;
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < m.n; i++) {
    double energy = 0., z = 0.;
    const double *xi = &m.x[3 * i], *ui = &m.u[3 * i], *vi = &m.v[3 * i];
    for (int64_t k = m.rowptr[i]; k < m.rowptr[i + 1]; k++) {
      uint8_t fs = m.broken[k];
      double F[3], en = 0.;
      rnp_bond(m, m.u.data(), i, k, fs, F, &en, false);
      energy += en;
      const int64_t j = m.cols[k];
      const double *xj = &m.x[3 * j], *uj = &m.u[3 * j];
      double rji = dist3(xj, xi);
      double dx[3] = {xj[0] - xi[0], xj[1] - xi[1], xj[2] - xi[2]};
      double du[3] = {uj[0] - ui[0], uj[1] - ui[1], uj[2] - ui[2]};
      double Sji = dot3(dx, du) / dot3(dx, dx);
      double sr = 0.;
      if (dGT(rji, 1.0E-12)) sr = std::abs(Sji) / (m.rnp.rbar / std::sqrt(rji));
      if (dLT(z, sr)) z = sr;
    }
    const double voli = m.vol[i];
    const double *fe = &fext[3 * i];
    e[i] = float(energy * voli);
    e[m.n + i] = float(ui[0] * fe[0] + ui[1] * fe[1] + ui[2] * fe[2]);
    e[2 * m.n + i] = float(0.5 * rho * (vi[0] * vi[0] + vi[1] * vi[1] + vi[2] * vi[2]) * voli);
    e[3 * m.n + i] = dGT(z, 1.0 - 1.0E-10) ? float(energy * voli) : 0.f;
  }
  float *out[4] = {strain, work, kinetic, fracture};
  for (int q = 0; q < 4; q++) {
    double t = 0.;
    for (int64_t i = 0; i < m.n; i++) {
      t += e[q * m.n + i];
      if (out[q]) out[q][i] = e[q * m.n + i];
    }
    if (totals) totals[q] = t;
  }
  return NLM_OK;
}

// util::geometry::direction / onLine / doLinesIntersect (utilGeom.cpp:281-326)
// as written there: the orientation's cross product is stored in an int.
int geo_direction(const double *A, const double *B, const double *C) {
  int val = (int)((B[1] - A[1]) * (C[0] - B[0]) - (B[0] - A[0]) * (C[1] - B[1]));
  if (val == 0) return 0;
  return val < 0 ? 2 : 1;
}
bool geo_on_line(const double *A, const double *B, const double *C) {
  return C[0] <= std::max(A[0], B[0]) && C[0] <= std::min(A[0], B[0]) &&
         C[1] <= std::max(A[1], B[1]) && C[1] <= std::min(A[1], B[1]);
}
bool geo_lines_intersect(const double *A, const double *B, const double *C, const double *D) {
  int d1 = geo_direction(A, B, C), d2 = geo_direction(A, B, D);
  int d3 = geo_direction(C, D, A), d4 = geo_direction(C, D, B);
  if (d1 != d2 && d3 != d4) return true;
  if (d1 == 0 && geo_on_line(A, B, C)) return true;
  if (d2 == 0 && geo_on_line(A, B, D)) return true;
  if (d3 == 0 && geo_on_line(C, D, A)) return true;
  if (d4 == 0 && geo_on_line(C, D, B)) return true;
  return false;
}

// FDModel::computeForce reaction force (fDModel.cpp:543-605), 2-D RNPBond:
// R[3n] per node, |R| per node, their sum.
int orc_fd_reaction_force(orc_fd *h, double *R, double *total, double *sum) {
  Model &m = h->m;
  if (m.mat.kind != NLM_MAT_RNP_BOND || m.dim != 2) return NLM_ERR_UNSUPPORTED;
  double lo[3] = {0., 0., 0.}, hi[3] = {0., 0., 0.};  // fe::Mesh::computeBBox
  for (int64_t i = 0; i < m.n; i++)
    for (int c = 0; c < 3; c++) {
      if (dLT(m.x[3 * i + c], lo[c])) lo[c] = m.x[3 * i + c];
      if (dLT(hi[c], m.x[3 * i + c])) hi[c] = m.x[3 * i + c];
    }
  const double delta = m.delta, eps = 1e-6;
  const double A[2] = {lo[0], hi[1] - delta + eps}, B[2] = {hi[0], hi[1] - delta + eps};
  std::vector<double> r(3 * m.n, 0.);
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < m.n; i++) {
    const double *xi = &m.x[3 * i];
    if (!(xi[1] > hi[1] - 1.5 * delta && xi[1] < hi[1] - delta)) continue;
    for (int64_t k = m.rowptr[i]; k < m.rowptr[i + 1]; k++) {
      const double *xj = &m.x[3 * int64_t(m.cols[k])];
      if (!geo_lines_intersect(A, B, xi, xj)) continue;
      uint8_t fs = m.broken[k];
      double F[3];
      rnp_bond(m, m.u.data(), i, k, fs, F, nullptr, false);
      for (int c = 0; c < 3; c++) r[3 * i + c] += m.vol[i] * F[c];
    }
  }
  double s[3] = {0., 0., 0.};
  for (int64_t i = 0; i < m.n; i++) {
    const double *q = &r[3 * i];
    if (R)
      for (int c = 0; c < 3; c++) R[3 * i + c] = q[c];
    if (total) total[i] = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
    for (int c = 0; c < 3; c++) s[c] += q[c];
  }
  if (sum)
    for (int c = 0; c < 3; c++) sum[c] = s[c];
  return NLM_OK;
}

int orc_fd_es_fields(orc_fd *h, double *omega, double *mw, double *theta) {
  Model &m = h->m;
  if (m.mat.kind != NLM_MAT_ELASTIC_STATE) return fail(NLM_ERR_INVALID, "not ElasticState");
  es_dilatation(m, m.u.data(), false);
  if (omega) std::copy(m.omega.begin(), m.omega.end(), omega);
  if (mw) std::copy(m.mw.begin(), m.mw.end(), mw);
  if (theta) std::copy(m.theta.begin(), m.theta.end(), theta);
  return NLM_OK;
}

int orc_fd_eval_force(orc_fd *h, double *f) {
  Model &m = h->m;
  std::fill(f, f + 3 * m.n, 0.);
  std::vector<uint8_t> keep = m.broken;
  internal_forces(m, m.u.data(), f, false);
  m.broken = keep;
  return NLM_OK;
}

// ===========================================================================
// Quasi-static ElasticState (QuasiStaticModel.cpp).
struct orc_qs {
  Model m;
  orc_qs_params p{};
  std::vector<double> body;  // body force, accumulated as the reference does
  std::vector<int> free_dof; // dof index map (-1 fixed)
  int64_t nfree = 0;
  int step = 0;
};

namespace {

// Force density with the reference's scatter (QuasiStaticModel.cpp:168-239):
// f_i += T_ij V_j, f_j -= T_ij V_i with T_ij = M t_ij omega_ij.  Sums per node
// are accumulated in a fixed order (the reference's mutex order is not).
void qs_forces(Model &m, const double *u, double *f) {
  // ElasticState::update -> dilatation over every bond (no breaking)
  double c = m.dim == 1 ? 1. : (m.dim == 2 ? 2. : 3.);
  for (int64_t i = 0; i < m.n; i++) {
    double th = 0.;
    for (int64_t k = m.rowptr[i]; k < m.rowptr[i + 1]; k++) {
      int64_t j = m.cols[k];
      double Y[3], Xl, e;
      es_bond_geom(m, u, i, j, Y, Xl, e);
      if (m.dim == 2)
        th += (c / m.mw[i]) * m.es.factor2D * 1. * Xl * e * m.omega[k] * m.vol[j];
      else
        th += (c / m.mw[i]) * 1. * Xl * e * m.omega[k] * m.vol[j];
    }
    m.theta[i] = th;
  }
  std::fill(f, f + 3 * m.n, 0.);
  for (int64_t i = 0; i < m.n; i++) {
    double fi[3] = {0, 0, 0};
    for (int64_t k = m.rowptr[i]; k < m.rowptr[i + 1]; k++) {
      int64_t j = m.cols[k];
      double Y[3], Xl, e;
      es_bond_geom(m, u, i, j, Y, Xl, e);
      double Yl = len3(Y);
      double t = es_t(m, i, e, Xl);
      for (int d = 0; d < 3; d++) {
        double T = (Y[d] / Yl) * t * m.omega[k];
        fi[d] += T * m.vol[j];
        f[3 * j + d] -= T * m.vol[i];
      }
    }
    for (int d = 0; d < 3; d++) f[3 * i + d] += fi[d];
  }
}

// Dense LU with partial pivoting (the oracle's linear solve; the reference
// calls BlazeIterative CG, judged here by the converged Newton state).
bool lu_solve(std::vector<double> &A, std::vector<double> &b, int64_t n) {
  std::vector<int64_t> piv(n);
  for (int64_t k = 0; k < n; k++) {
    int64_t p = k;
    double best = std::abs(A[k * n + k]);
    for (int64_t r = k + 1; r < n; r++)
      if (std::abs(A[r * n + k]) > best) { best = std::abs(A[r * n + k]); p = r; }
    if (best == 0.) return false;
    if (p != k) {
      for (int64_t c = 0; c < n; c++) std::swap(A[k * n + c], A[p * n + c]);
      std::swap(b[k], b[p]);
    }
    double inv = 1. / A[k * n + k];
#pragma omp parallel for schedule(static)
    for (int64_t r = k + 1; r < n; r++) {
      double l = A[r * n + k] * inv;
      if (l == 0.) continue;
      A[r * n + k] = 0.;
      for (int64_t c = k + 1; c < n; c++) A[r * n + c] -= l * A[k * n + c];
      b[r] -= l * b[k];
    }
  }
  for (int64_t k = n - 1; k >= 0; k--) {
    double s = b[k];
    for (int64_t c = k + 1; c < n; c++) s -= A[k * n + c] * b[c];
    b[k] = s / A[k * n + k];
  }
  return true;
}

}  // namespace

int orc_qs_create(const nlm_fd_desc *d, const orc_qs_params *p, orc_qs **out) {
  if (!d || !p || !out) return fail(NLM_ERR_INVALID, "null argument");
  if (d->material.kind != NLM_MAT_ELASTIC_STATE)
    return fail(NLM_ERR_INVALID, "reference QS is ElasticState only");
  auto *h = new orc_qs();
  int rc = setup_model(d, false, h->m);
  if (rc) { delete h; return rc; }
  h->p = *p;
  h->body.assign(3 * h->m.n, 0.);
  int dim = h->m.dim;
  h->free_dof.assign(h->m.n * dim, -1);
  // fixed dofs = every (node, direction) of a displacement BC set
  // (QuasiStaticModel.cpp:466-478)
  std::vector<uint8_t> fixed(h->m.n * dim, 0);
  for (size_t s = 0; s < h->m.ubc.size(); s++)
    for (int64_t i : h->m.ubc_nodes[s])
      for (int dd = 0; dd < dim; dd++)
        if (h->m.ubc[s].dir_mask & (1 << dd)) fixed[i * dim + dd] = 1;
  int64_t c = 0;
  for (int64_t k = 0; k < h->m.n * dim; k++)
    if (!fixed[k]) h->free_dof[k] = int(c++);
  h->nfree = c;
  *out = h;
  return NLM_OK;
}

int orc_qs_destroy(orc_qs *h) { delete h; return NLM_OK; }

// QuasiStaticModel::solver (:526-594): per load step apply loads, residual
// r = f + b on free dofs, Newton until ||r|| < tol.  The Jacobian follows
// assembly_jacobian_matrix_part (:361-454): central differences with
// eps = perturbation * h, rows of free nodes, columns of i and N(i).
int orc_qs_solve(orc_qs *h, int nsteps, int *iters, double *final_res) {
  Model &m = h->m;
  int dim = m.dim;
  int64_t nf = h->nfree;
  double eps = h->p.perturbation * m.h;
  std::vector<double> f(3 * m.n), fp(3 * m.n), fm(3 * m.n), up;
  auto residual = [&](std::vector<double> &r) {
    r.assign(nf, 0.);
    for (int64_t i = 0; i < m.n; i++)
      for (int d = 0; d < dim; d++) {
        int k = h->free_dof[i * dim + d];
        if (k >= 0) r[k] = f[3 * i + d] + h->body[3 * i + d];
      }
  };
  auto norm = [](const std::vector<double> &r) {
    double s = 0;
    for (double a : r) s += a * a;
    return std::sqrt(s);
  };
  for (int s = 0; s < nsteps; s++) {
    h->step++;
    double time = h->step * h->p.dt;
    apply_fload(m, time, h->body.data());  // accumulates (fLoading.cpp:268-275)
    std::vector<double> vdummy(3 * m.n, 0.);
    apply_uload(m, time, m.u.data(), vdummy.data());
    qs_forces(m, m.u.data(), f.data());  // fresh forces at the new BC state
    std::vector<double> r;
    residual(r);
    double r0 = norm(r), res = r0;
    int it = 0;
    auto converged = [&]() {
      return h->p.tol_relative ? (r0 == 0. || res / r0 < h->p.tol) : res < h->p.tol;
    };
    while (!converged() && it < h->p.max_iters) {
      std::vector<double> J(size_t(nf) * size_t(nf), 0.);
      // FD Jacobian.  Each column perturbation re-evaluates the full force.
      up = m.u;
      for (int64_t j = 0; j < m.n; j++)
        for (int rr = 0; rr < dim; rr++) {
          int col = h->free_dof[j * dim + rr];
          if (col < 0) continue;
          up[3 * j + rr] = m.u[3 * j + rr] + eps;
          qs_forces(m, up.data(), fp.data());
          up[3 * j + rr] = m.u[3 * j + rr] - eps;
          qs_forces(m, up.data(), fm.data());
          up[3 * j + rr] = m.u[3 * j + rr];
          // rows i with j in {i} U N(i); reference keeps r == s only
          auto put = [&](int64_t i) {
            for (int ss = 0; ss < dim; ss++) {
              if (h->p.jacobian == 0 && ss != rr) continue;
              int row = h->free_dof[i * dim + ss];
              if (row < 0) continue;
              J[size_t(row) * nf + col] = (fp[3 * i + ss] - fm[3 * i + ss]) / (2. * eps);
            }
          };
          put(j);
          for (int64_t k = m.rowptr[j]; k < m.rowptr[j + 1]; k++) put(m.cols[k]);
        }
      std::vector<double> rhs(nf);
      for (int64_t k = 0; k < nf; k++) rhs[k] = -r[k];
      if (!lu_solve(J, rhs, nf)) return fail(NLM_ERR_INVALID, "singular Jacobian");
      for (int64_t i = 0; i < m.n; i++)
        for (int d = 0; d < dim; d++) {
          int k = h->free_dof[i * dim + d];
          if (k >= 0) m.u[3 * i + d] += rhs[k];
        }
      qs_forces(m, m.u.data(), f.data());
      residual(r);
      res = norm(r);
      it++;
    }
    if (iters) iters[s] = it;
    if (final_res) *final_res = res;
  }
  qs_forces(m, m.u.data(), f.data());
  m.f = f;
  return NLM_OK;
}

int orc_qs_get(const orc_qs *h, double *u, double *fout, int64_t *nnz) {
  const Model &m = h->m;
  if (u) std::copy(m.u.begin(), m.u.end(), u);
  if (fout)
    for (int64_t i = 0; i < m.n; i++)
      for (int d = 0; d < 3; d++) fout[3 * i + d] = m.f[3 * i + d] * m.vol[i];
  if (nnz) *nnz = int64_t(m.cols.size());
  return NLM_OK;
}

// ===========================================================================
// Quasi-static RNPBond (build definition; the reference has QuasiStaticModel
// for ElasticState only, QuasiStaticModel.cpp:648).  Same load-step / Newton
// structure as QuasiStaticModel::solver (:526-594): at load step k the
// Displacement_BC values are applied at time k*dt, the residual is the force
// density of FDModel::computeForce on free dofs, Newton uses the analytic
// tangent of RNPBond's bond force with block-Jacobi preconditioned CG, and
// stops at ||r|| <= tol * ||r(previous-step guess)||.  Bonds over the critical
// strain break after convergence and the step is solved again.

struct orc_qsr {
  Model m;
  int max_newton = 50, lin_max = 10000, break_bonds = 1, max_break_rounds = 50;
  double tol = 1e-8, lin_tol = 1e-4, dt = 1.;
  int step = 0;
  std::vector<uint8_t> fixed;  // dof mask (dim per node)
};

namespace {

inline bool qsr_breakable(const Model &m, int64_t i, int64_t j) {
  return m.interior[i] && m.interior[j];
}

// residual (free dofs) and optionally tangent blocks (3 per bond in 2-D);
// with update, intact bonds past the critical strain break first
// (RNPBond::getBondEF, rnpBond.cpp:263-266) and give no force.
int64_t qsr_residual(orc_qsr *h, const std::vector<double> &u, std::vector<double> &res,
                     std::vector<double> *blk, std::vector<double> *dblk, bool update = false) {
  Model &m = h->m;
  const int dim = m.dim, NB = dim == 2 ? 3 : 6;
  res.assign((size_t)dim * m.n, 0.);
  if (blk) {
    blk->assign((size_t)NB * m.cols.size(), 0.);
    dblk->assign((size_t)NB * m.n, 0.);
  }
  const RNP &p = m.rnp;
  const double check_up = m.delta + 0.5 * m.h, check_low = m.delta - 0.5 * m.h;
  int64_t nbroken = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : nbroken)
  for (int64_t i = 0; i < m.n; i++) {
    double fi[3] = {0, 0, 0}, di[6] = {0, 0, 0, 0, 0, 0};
    for (int64_t k = m.rowptr[i]; k < m.rowptr[i + 1]; k++) {
      const int64_t j = m.cols[k];
      const bool brk = qsr_breakable(m, i, j);
      if (m.broken[k] && brk) continue;
      double dx[3], du[3];
      for (int c = 0; c < 3; c++) {
        dx[c] = m.x[3 * j + c] - m.x[3 * i + c];
        du[c] = u[3 * j + c] - u[3 * i + c];
      }
      const double rr = dot3(dx, dx), r = std::sqrt(rr);
      const double S = dot3(dx, du) / rr;
      double e[3] = {dx[0] / r, dx[1] / r, dx[2] / r};
      if (update && brk && p.irrev && dGT(std::abs(S), p.fsc * (p.rbar / std::sqrt(r)))) {
        m.broken[k] = 1;
        nbroken++;
        continue;
      }
      double volj = m.vol[j];
      if (dGT(r, check_low)) volj = volj * ((check_up - r) / m.h);
      const double k0 = p.J.J(r / m.delta) * 4. * p.C * p.beta / p.invF * volj;
      const double ex = std::exp(-p.beta * r * S * S);
      const double s = brk ? k0 * S * ex : k0 * S;
      for (int c = 0; c < dim; c++) fi[c] += s * e[c];
      if (blk) {
        const double gp = brk ? k0 * std::max(1. - 2. * p.beta * r * S * S, 0.) * ex / r : k0 / r;
        double a[6] = {gp * e[0] * e[0], gp * e[1] * e[0], gp * e[1] * e[1],
                       gp * e[2] * e[0], gp * e[2] * e[1], gp * e[2] * e[2]};
        for (int c = 0; c < NB; c++) {
          (*blk)[(size_t)NB * k + c] = a[c];
          di[c] += a[c];
        }
      }
    }
    for (int c = 0; c < dim; c++) res[(size_t)dim * i + c] = h->fixed[(size_t)dim * i + c] ? 0. : fi[c];
    if (blk) {
      // relative Levenberg term (as the GPU solver)
      const double reg = 1e-8 * (dim == 2 ? 0.5 * (di[0] + di[2]) : (di[0] + di[2] + di[5]) / 3.);
      di[0] += reg;
      di[2] += reg;
      if (dim == 3) di[5] += reg;
      for (int c = 0; c < NB; c++) (*dblk)[(size_t)NB * i + c] = di[c];
    }
  }
  return nbroken;
}

void sym_mul_h(int dim, const double *a, const double *x, double *y) {
  if (dim == 2) {
    y[0] = a[0] * x[0] + a[1] * x[1];
    y[1] = a[1] * x[0] + a[2] * x[1];
  } else {
    y[0] = a[0] * x[0] + a[1] * x[1] + a[3] * x[2];
    y[1] = a[1] * x[0] + a[2] * x[1] + a[4] * x[2];
    y[2] = a[3] * x[0] + a[4] * x[1] + a[5] * x[2];
  }
}

// PCG on (-K) x = b over free dofs, block-Jacobi preconditioner.
int qsr_cg(orc_qsr *h, const std::vector<double> &blk, const std::vector<double> &dblk,
           const std::vector<double> &b, std::vector<double> &x) {
  Model &m = h->m;
  const int dim = m.dim, NB = dim == 2 ? 3 : 6;
  const size_t M = (size_t)dim * m.n;
  auto spmv = [&](const std::vector<double> &v, std::vector<double> &y) {
    y.assign(M, 0.);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < m.n; i++) {
      double acc[3] = {0, 0, 0}, t[3];
      sym_mul_h(dim, &dblk[(size_t)NB * i], &v[(size_t)dim * i], acc);
      for (int64_t k = m.rowptr[i]; k < m.rowptr[i + 1]; k++) {
        sym_mul_h(dim, &blk[(size_t)NB * k], &v[(size_t)dim * m.cols[k]], t);
        for (int c = 0; c < dim; c++) acc[c] -= t[c];
      }
      for (int c = 0; c < dim; c++) y[(size_t)dim * i + c] = h->fixed[(size_t)dim * i + c] ? 0. : acc[c];
    }
  };
  auto precond = [&](const std::vector<double> &r, std::vector<double> &z) {
    z.assign(M, 0.);
    for (int64_t i = 0; i < m.n; i++) {
      const double *bb = &dblk[(size_t)NB * i];
      double a[9];
      if (dim == 2) {
        a[0] = bb[0]; a[1] = bb[1]; a[2] = bb[1]; a[3] = bb[2];
      } else {
        a[0] = bb[0]; a[1] = bb[1]; a[2] = bb[3]; a[3] = bb[1]; a[4] = bb[2];
        a[5] = bb[4]; a[6] = bb[3]; a[7] = bb[4]; a[8] = bb[5];
      }
      for (int c = 0; c < dim; c++)
        if (h->fixed[(size_t)dim * i + c])
          for (int q = 0; q < dim; q++) a[c * dim + q] = a[q * dim + c] = (c == q) ? 1. : 0.;
      double rv[3] = {0, 0, 0};
      for (int c = 0; c < dim; c++) rv[c] = h->fixed[(size_t)dim * i + c] ? 0. : r[(size_t)dim * i + c];
      if (dim == 2) {
        const double det = a[0] * a[3] - a[1] * a[2];
        if (std::abs(det) > 0.) {
          z[(size_t)dim * i] = (a[3] * rv[0] - a[1] * rv[1]) / det;
          z[(size_t)dim * i + 1] = (-a[2] * rv[0] + a[0] * rv[1]) / det;
        }
      } else {
        const double c00 = a[4] * a[8] - a[5] * a[7], c01 = a[5] * a[6] - a[3] * a[8],
                     c02 = a[3] * a[7] - a[4] * a[6];
        const double det = a[0] * c00 + a[1] * c01 + a[2] * c02;
        if (std::abs(det) > 0.) {
          const double inv[9] = {c00, a[2] * a[7] - a[1] * a[8], a[1] * a[5] - a[2] * a[4],
                                 c01, a[0] * a[8] - a[2] * a[6], a[2] * a[3] - a[0] * a[5],
                                 c02, a[1] * a[6] - a[0] * a[7], a[0] * a[4] - a[1] * a[3]};
          for (int c = 0; c < 3; c++)
            z[(size_t)dim * i + c] = (inv[3 * c] * rv[0] + inv[3 * c + 1] * rv[1] + inv[3 * c + 2] * rv[2]) / det;
        }
      }
    }
  };
  auto dotv = [&](const std::vector<double> &a, const std::vector<double> &c) {
    double s = 0;
    for (size_t k = 0; k < M; k++) s += a[k] * c[k];
    return s;
  };
  x.assign(M, 0.);
  std::vector<double> r = b, z, p, ap;
  precond(r, z);
  p = z;
  double rz = dotv(r, z);
  const double rr0 = dotv(r, r);
  if (rr0 == 0.) return 0;
  int it = 0;
  while (it < h->lin_max) {
    spmv(p, ap);
    const double pap = dotv(p, ap);
    const double alpha = pap != 0. ? rz / pap : 0.;
    for (size_t k = 0; k < M; k++) {
      x[k] += alpha * p[k];
      r[k] -= alpha * ap[k];
    }
    precond(r, z);
    const double rzn = dotv(r, z);
    const double beta = rz != 0. ? rzn / rz : 0.;
    for (size_t k = 0; k < M; k++) p[k] = z[k] + beta * p[k];
    rz = rzn;
    it++;
    if (!(dotv(r, r) > h->lin_tol * h->lin_tol * rr0)) break;
  }
  return it;
}

double qsr_norm(const std::vector<double> &r) {
  double s = 0;
  for (double v : r) s += v * v;
  return std::sqrt(s);
}

void qsr_newton(orc_qsr *h, double target, orc_qsr_stats *st) {
  Model &m = h->m;
  std::vector<double> res, blk, dblk, dx;
  for (int it = 0;; it++) {
    const int64_t nb = qsr_residual(h, m.u, res, &blk, &dblk, h->break_bonds != 0);
    st->broken += nb;
    if (nb) st->break_rounds++;
    st->res_final = qsr_norm(res);
    if (!(st->res_final > target) || it >= h->max_newton) return;
    st->lin_iters += qsr_cg(h, blk, dblk, res, dx);
    for (int64_t i = 0; i < m.n; i++)
      for (int c = 0; c < m.dim; c++) m.u[3 * i + c] += dx[(size_t)m.dim * i + c];
    st->newton_iters++;
  }
}

}  // namespace

int orc_qsr_create(const nlm_fd_desc *d, int max_newton, double tol, int lin_max_iters,
                   double lin_tol, int break_bonds, int max_break_rounds, orc_qsr **out) {
  if (!d || !out) return fail(NLM_ERR_INVALID, "null argument");
  if (d->material.kind != NLM_MAT_RNP_BOND) return fail(NLM_ERR_INVALID, "RNPBond only");
  auto *h = new orc_qsr();
  int rc = setup_model(d, true, h->m);
  if (rc) {
    delete h;
    return rc;
  }
  h->max_newton = max_newton;
  h->tol = tol;
  h->lin_max = lin_max_iters;
  h->lin_tol = lin_tol;
  h->break_bonds = break_bonds;
  h->max_break_rounds = max_break_rounds;
  h->dt = d->dt;
  h->fixed.assign((size_t)h->m.dim * h->m.n, 0);
  for (int64_t i = 0; i < h->m.n; i++)
    for (int c = 0; c < h->m.dim; c++) h->fixed[(size_t)h->m.dim * i + c] = (h->m.fix[i] >> c) & 1;
  *out = h;
  return NLM_OK;
}

int orc_qsr_destroy(orc_qsr *h) {
  delete h;
  return NLM_OK;
}

// Load step with the displacement-controlled tangent predictor: with K and f
// at the previous converged state and the boundary increment du_c, the first
// iterate solves (-K) du = f + K du_c on free dofs; ||f + K du_c|| is the
// residual scale of the step.  A caller's guess u_g is used instead when the
// same linear model, ||f + K (u_g - u_prev)||, is not larger.  Newton
// iterations then run with bond breaking in every residual evaluation.
int orc_qsr_load_step(orc_qsr *h, const double *guess, orc_qsr_stats *st_out) {
  Model &m = h->m;
  const int dim = m.dim, NB = dim == 2 ? 3 : 6;
  orc_qsr_stats st{};
  std::vector<double> res0, blk, dblk, dx, vd(3 * m.n, 0.);
  const std::vector<double> uprev = m.u;
  qsr_residual(h, m.u, res0, &blk, &dblk);
  h->step++;
  const double time = h->step * h->dt;
  apply_uload(m, time, m.u.data(), vd.data());
  // f + K d on free dofs, (K d)_i = sum_j A_ij (d_j - d_i)
  auto linear = [&](const std::vector<double> &ucand, bool fixed_only, std::vector<double> &out) {
    out = res0;
    auto d = [&](int64_t a, int c) {
      if (fixed_only && !h->fixed[(size_t)dim * a + c]) return 0.;
      return ucand[3 * a + c] - uprev[3 * a + c];
    };
    for (int64_t i = 0; i < m.n; i++) {
      double acc[3] = {0, 0, 0}, t[3], xi[3] = {0, 0, 0};
      for (int c = 0; c < dim; c++) xi[c] = d(i, c);
      sym_mul_h(dim, &dblk[(size_t)NB * i], xi, acc);
      for (int64_t k = m.rowptr[i]; k < m.rowptr[i + 1]; k++) {
        const int64_t j = m.cols[k];
        double xj[3] = {0, 0, 0};
        for (int c = 0; c < dim; c++) xj[c] = d(j, c);
        sym_mul_h(dim, &blk[(size_t)NB * k], xj, t);
        for (int c = 0; c < dim; c++) acc[c] -= t[c];
      }
      for (int c = 0; c < dim; c++)
        if (!h->fixed[(size_t)dim * i + c]) out[(size_t)dim * i + c] -= acc[c];
    }
  };
  std::vector<double> rhs;
  linear(m.u, true, rhs);
  st.res_plain = st.res_start = qsr_norm(rhs);
  bool use_guess = false;
  if (guess) {
    std::vector<double> saved = m.u, rg;
    for (int64_t k = 0; k < 3 * m.n; k++) m.u[k] = guess[k];
    apply_uload(m, time, m.u.data(), vd.data());
    linear(m.u, false, rg);
    const double ng = qsr_norm(rg);
    if (ng <= 0.1 * st.res_plain) {  // guess_accept = 0.1 (nlm_qs_params default)
      use_guess = true;
      st.used_guess = 1;
      st.res_start = ng;
    } else {
      m.u = saved;
    }
  }
  const double target = h->tol * st.res_plain;
  if (!use_guess && st.res_plain > 0.) {
    st.lin_iters += qsr_cg(h, blk, dblk, rhs, dx);
    for (int64_t i = 0; i < m.n; i++)
      for (int c = 0; c < dim; c++) m.u[3 * i + c] += dx[(size_t)dim * i + c];
    st.newton_iters++;
  }
  qsr_newton(h, target, &st);
  if (st_out) *st_out = st;
  return NLM_OK;
}

int orc_qsr_get_state(const orc_qsr *h, double *u) {
  std::copy(h->m.u.begin(), h->m.u.end(), u);
  return NLM_OK;
}

int orc_qsr_get_bond_state(const orc_qsr *h, uint8_t *broken) {
  std::copy(h->m.broken.begin(), h->m.broken.end(), broken);
  return NLM_OK;
}

}  // extern "C"
