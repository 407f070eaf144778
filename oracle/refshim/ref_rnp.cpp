// ref_rnp.cpp -- runs the reference's own RNPBond explicit dynamics.
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/refshim/Makefile into
// oracle/_ref/libref_rnp.so together with these NLMech sources, compiled
// unmodified from the reference tree (stand-in headers for Blaze and HPX in
// oracle/refshim/shim):
//   geometry/neighbor.cpp      Neighbor(horizon, deck, nodes)   (:24-92)
//   geometry/fracture.cpp      pre-crack bonds, bond-state bits (:20-187)
//   geometry/interiorFlags.cpp no-fail flags                    (:27-191)
//   material/pd/rnpBond.cpp    RNPBond(deck, dm), getBondEF     (:23-321)
//   loading/uLoading.cpp       ULoading ctor (fixity) + apply   (:20-253)
//   loading/fLoading.cpp       FLoading ctor + apply            (:20-277)
//   fe/mesh.cpp                Mesh(dim), setMeshData, setMeshSize
//   data/DataManager.cpp, util/*.cpp, fe/*Elem.cpp, inp/policy.cpp
// The only code of this file on the computed path is the driver loop of
// FDModel::integrate / integrateVerlet / computeForces (fDModel.cpp:317-374,
// :445-541, :543-582), restated because fDModel.cpp itself also needs the
// YAML input, VTK output and restart machinery.  The mesh readers are not
// linked (reader_stub.cpp): nodes and volumes come from the caller.
//
// The description is the nlm_fd_desc of include/nlmgpu.h, so tests feed the
// same inputs to this reference run, the oracle restatement and the GPU.

#include <stdint.h>

#include <cstdio>
#include <exception>
#include <string>
#include <vector>

#include "../../include/nlmgpu.h"
#include "data/DataManager.h"
#include "fe/mesh.h"
#include "geometry/fracture.h"
#include "geometry/interiorFlags.h"
#include "geometry/neighbor.h"
#include "inp/decks/fractureDeck.h"
#include "inp/decks/interiorFlagsDeck.h"
#include "inp/decks/loadingDeck.h"
#include "inp/decks/materialDeck.h"
#include "inp/decks/modelDeck.h"
#include "inp/decks/neighborDeck.h"
#include "loading/fLoading.h"
#include "loading/uLoading.h"
#include "material/pd/rnpBond.h"
#include "util/utilGeom.h"
#include "inp/decks/meshDeck.h"
#include "reader_stub.h"

namespace {

thread_local std::string g_err;

int fail(const std::string &m) {
  g_err = m;
  return 1;
}

const char *region_name(int r) {
  switch (r) {
    case NLM_REGION_RECTANGLE: return "rectangle";
    case NLM_REGION_LINE: return "line";
    case NLM_REGION_CIRCLE: return "circle";
    case NLM_REGION_TORUS: return "torus";
    case NLM_REGION_CUBOID: return "cuboid";
    case NLM_REGION_ANGLED_RECTANGLE: return "angled_rectangle";
  }
  return "";
}
const char *time_name(int t) {
  switch (t) {
    case NLM_TFN_CONSTANT: return "constant";
    case NLM_TFN_LINEAR: return "linear";
    case NLM_TFN_QUADRATIC: return "quadratic";
    case NLM_TFN_SIN: return "sin";
    case NLM_TFN_LINEAR_STEP: return "linear_step";
    case NLM_TFN_LINEAR_SLOW_FAST: return "linear_slow_fast";
  }
  return "";
}
const char *spatial_name(int s) {
  switch (s) {
    case NLM_SFN_CONSTANT: return "constant";
    case NLM_SFN_SIN_X: return "sin_x";
    case NLM_SFN_SIN_Y: return "sin_y";
    case NLM_SFN_SIN_Z: return "sin_z";
    case NLM_SFN_LINEAR_X: return "linear_x";
    case NLM_SFN_LINEAR_Y: return "linear_y";
    case NLM_SFN_LINEAR_Z: return "linear_z";
    case NLM_SFN_HAT_X: return "hat_x";
    case NLM_SFN_HAT_Y: return "hat_y";
    case NLM_SFN_HAT_Z: return "hat_z";
    case NLM_SFN_LINE_LOAD: return "line_load";
  }
  return "";
}

inp::BCData to_bc(const nlm_bc_set &b) {
  inp::BCData d;
  d.d_regionType = region_name(b.region);
  d.d_timeFnType = time_name(b.time_fn);
  d.d_spatialFnType = spatial_name(b.spatial_fn);
  d.d_x1 = b.x1;
  d.d_x2 = b.x2;
  d.d_y1 = b.y1;
  d.d_y2 = b.y2;
  d.d_z1 = b.z1;
  d.d_z2 = b.z2;
  d.d_r1 = b.r1;
  d.d_r2 = b.r2;
  d.d_theta = b.theta;
  for (int k = 0; k < 3; k++)
    if (b.dir_mask >> k & 1) d.d_direction.push_back((size_t)k + 1);
  // the deck parser keeps as many parameters as the function takes; the
  // apply code reads d_timeFnParams[0] always and [1..2] for the step kinds
  const int ntp = (b.time_fn == NLM_TFN_LINEAR_STEP || b.time_fn == NLM_TFN_LINEAR_SLOW_FAST)
                      ? 3
                      : (b.time_fn == NLM_TFN_QUADRATIC || b.time_fn == NLM_TFN_SIN ? 2 : 1);
  for (int k = 0; k < ntp; k++) d.d_timeFnParams.push_back(b.time_params[k]);
  const int nsp = b.spatial_fn == NLM_SFN_CONSTANT ? 1 : 2;
  for (int k = 0; k < nsp; k++) d.d_spatialFnParams.push_back(b.spatial_params[k]);
  return d;
}

}  // namespace

struct ref_rnp {
  size_t dim = 2;
  double dt = 0., time = 0., density = 1.;
  int64_t step = 0;
  bool started = false;
  inp::ModelDeck mdeck;
  inp::MaterialDeck matdeck;
  inp::NeighborDeck ndeck;
  inp::FractureDeck fdeck;
  inp::InteriorFlagsDeck ideck;
  inp::LoadingDeck ldeck;
  fe::Mesh *mesh = nullptr;
  geometry::Neighbor *neigh = nullptr;
  geometry::Fracture *frac = nullptr;
  geometry::InteriorFlags *iflags = nullptr;
  loading::ULoading *uload = nullptr;
  loading::FLoading *fload = nullptr;
  data::DataManager dm;
  material::pd::RNPBond *mat = nullptr;
  std::vector<util::Point3> u, v, f;
  ~ref_rnp() {
    delete mat;
    delete fload;
    delete uload;
    delete iflags;
    delete frac;
    delete neigh;
    delete mesh;
  }

  // FDModel::computeForces / computeForce (fDModel.cpp:527-582): f_i +=
  // sum over the row, in neighbour-list order, of getBondEF(i, j).first
  void compute_forces() {
    const long long n = (long long)u.size();
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < n; i++) {
      auto force_i = util::Point3();
      const auto &row = neigh->getNeighbors((size_t)i);
      for (size_t j = 0; j < row.size(); j++) force_i += mat->getBondEF((size_t)i, j).first;
      f[i] += force_i;
    }
  }

  // FDModel::integrateVerlet (fDModel.cpp:445-525)
  void verlet() {
    const long long n = (long long)u.size();
    // timed cracks of the step before (fDModel.cpp:366-373), after its output
    if (step > 0) frac->addCrack(time, mesh->getNodesP(), neigh->getNeighborsListP());
    const double fact = 0.5 * dt / mat->getDensity();
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < n; i++) {
      if (mesh->isNodeFree(i, 0)) {
        v[i].d_x += fact * f[i].d_x;
        u[i].d_x += dt * v[i].d_x;
      }
      if (dim > 1 && mesh->isNodeFree(i, 1)) {
        v[i].d_y += fact * f[i].d_y;
        u[i].d_y += dt * v[i].d_y;
      }
      if (dim > 2 && mesh->isNodeFree(i, 2)) {
        v[i].d_z += fact * f[i].d_z;
        u[i].d_z += dt * v[i].d_z;
      }
      f[i] = util::Point3();
    }
    step++;
    time += dt;
    uload->apply(time, &u, &v, mesh);
    fload->apply(time, &f, mesh);
    compute_forces();
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < n; i++) {
      if (mesh->isNodeFree(i, 0)) v[i].d_x += fact * f[i].d_x;
      if (dim > 1 && mesh->isNodeFree(i, 1)) v[i].d_y += fact * f[i].d_y;
      if (dim > 2 && mesh->isNodeFree(i, 2)) v[i].d_z += fact * f[i].d_z;
    }
  }

  // FDModel::integrate before the loop (fDModel.cpp:319-333)
  void start() {
    uload->apply(time, &u, &v, mesh);
    fload->apply(time, &f, mesh);
    compute_forces();
    started = true;
  }
};

extern "C" {

const char *ref_rnp_last_error(void) { return g_err.c_str(); }

int ref_rnp_create(const nlm_fd_desc *d, ref_rnp **out) {
  if (!d || !out) return fail("null argument");
  if (d->material.kind != NLM_MAT_RNP_BOND) return fail("RNPBond only");
  if (d->scheme != NLM_VELOCITY_VERLET) return fail("velocity-Verlet only");
  for (int k = 0; k < d->n_cracks; k++)
    if (d->cracks[k].kind != NLM_CRACK_EDGE) return fail("edge cracks only");
  // the reference exits the process on inputs it does not know: refuse them
  for (int k = 0; k < d->n_ubc; k++)
    if (d->ubc[k].region == NLM_REGION_CUBOID)
      return fail("Displacement_BC has no cuboid region in the reference");
  if (d->material.influence_type < 0 || d->material.influence_type > 2)
    return fail("unknown influence function");
  if (d->material.compute_from_classical && !(d->material.E > 0. || d->material.K > 0.))
    return fail("need E or K");
  try {
    ref_rnp *h = new ref_rnp();
    const size_t n = (size_t)d->n_nodes;
    h->dim = (size_t)d->dim;
    h->dt = d->dt;
    h->mdeck.d_dim = h->dim;
    h->mdeck.d_horizon = d->horizon;
    h->mdeck.d_h = d->mesh_size;
    h->mdeck.d_dt = d->dt;
    h->mdeck.d_timeDiscretization = "velocity_verlet";
    h->mdeck.d_spatialDiscretization = "finite_difference";

    std::vector<util::Point3> nodes(n);
    std::vector<double> vols(n);
    for (size_t i = 0; i < n; i++) {
      nodes[i] = util::Point3(d->x[3 * i], d->x[3 * i + 1], d->x[3 * i + 2]);
      vols[i] = d->volume[i];
    }
    h->mesh = new fe::Mesh(h->dim);
    h->mesh->setMeshData(h->dim, nodes, vols);
    h->mesh->setMeshSize(d->mesh_size);

    h->neigh = new geometry::Neighbor(d->horizon, &h->ndeck, h->mesh->getNodesP());

    for (int k = 0; k < d->n_cracks; k++) {
      const nlm_crack &c = d->cracks[k];
      inp::EdgeCrack e;
      e.d_o = c.orientation;
      e.d_pb = util::Point3(c.pb[0], c.pb[1], 0.);
      e.d_pt = util::Point3(c.pt[0], c.pt[1], 0.);
      e.d_l = e.d_pb.dist(e.d_pt);
      e.d_oldPb = e.d_initPb = e.d_pb;
      e.d_oldPt = e.d_initPt = e.d_pt;
      e.d_theta = c.theta;
      if (c.timed) e.d_activationTime = c.activation_time;
      h->fdeck.d_cracks.push_back(e);
    }
    h->frac = new geometry::Fracture(&h->fdeck, h->mesh->getNodesP(),
                                     h->neigh->getNeighborsListP());

    h->ideck.d_noFailActive = d->no_fail != NLM_NOFAIL_OFF;
    h->ideck.d_computeAndNotStoreFlag = d->no_fail == NLM_NOFAIL_COMPUTE;
    h->ideck.d_noFailTol = d->no_fail_tol;
    for (int r = 0; r < d->n_nofail_regions; r++) {
      const nlm_nofail_region &g = d->nofail_regions[r];
      h->ideck.d_noFailRegions.emplace_back(
          g.kind == NLM_NOFAIL_CIRCLE ? "Circle" : "Rectangle",
          std::vector<double>(g.params, g.params + 4));
    }
    h->iflags = new geometry::InteriorFlags(&h->ideck, h->mesh->getNodesP(),
                                            h->mesh->getBoundingBox());

    for (int k = 0; k < d->n_ubc; k++) h->ldeck.d_uBCData.push_back(to_bc(d->ubc[k]));
    for (int k = 0; k < d->n_fbc; k++) h->ldeck.d_fBCData.push_back(to_bc(d->fbc[k]));
    h->uload = new loading::ULoading(&h->ldeck, h->mesh);
    h->fload = new loading::FLoading(&h->ldeck, h->mesh);

    const nlm_material &m = d->material;
    inp::MaterialDeck &md = h->matdeck;
    md.d_materialType = "RNPBond";
    md.d_isPlaneStrain = m.plane_strain != 0;
    md.d_influenceFnType = (size_t)m.influence_type;
    for (int k = 0; k < m.n_influence_params; k++)
      md.d_influenceFnParams.push_back(m.influence_params[k]);
    md.d_irreversibleBondBreak = m.irreversible != 0;
    md.d_checkScFactor = m.check_sc_factor;
    md.d_computeParamsFromElastic = m.compute_from_classical != 0;
    md.d_bondPotentialParams = {m.bond_params[0], m.bond_params[1]};
    md.d_matData.d_E = m.E;
    md.d_matData.d_G = m.G;
    md.d_matData.d_K = m.K;
    md.d_matData.d_Gc = m.Gc;
    md.d_matData.d_KIc = m.KIc;
    md.d_density = m.density;
    md.d_applyContact = m.apply_contact != 0;

    h->u.assign(n, util::Point3());
    h->v.assign(n, util::Point3());
    h->f.assign(n, util::Point3());
    for (size_t i = 0; i < n; i++) {
      if (d->u0) h->u[i] = util::Point3(d->u0[3 * i], d->u0[3 * i + 1], d->u0[3 * i + 2]);
      if (d->v0) h->v[i] = util::Point3(d->v0[3 * i], d->v0[3 * i + 1], d->v0[3 * i + 2]);
    }
    h->dm.setModelDeckP(&h->mdeck);
    h->dm.setMeshP(h->mesh);
    h->dm.setNeighborP(h->neigh);
    h->dm.setFractureP(h->frac);
    h->dm.setInteriorFlagsP(h->iflags);
    h->dm.setDisplacementLoadingP(h->uload);
    h->dm.setForceLoadingP(h->fload);
    h->dm.setDisplacementP(&h->u);
    h->dm.setVelocityP(&h->v);
    h->dm.setForceP(&h->f);
    h->mat = new material::pd::RNPBond(&h->matdeck, &h->dm);
    *out = h;
    return 0;
  } catch (const std::exception &e) {
    return fail(e.what());
  }
}

int ref_rnp_destroy(ref_rnp *h) {
  delete h;
  return 0;
}

int ref_rnp_num_bonds(const ref_rnp *h, int64_t *nnz) {
  int64_t s = 0;
  for (size_t i = 0; i < h->u.size(); i++) s += (int64_t)h->neigh->getNeighbors(i).size();
  *nnz = s;
  return 0;
}

int ref_rnp_get_neighbors(const ref_rnp *h, int64_t *rowptr, int32_t *cols) {
  rowptr[0] = 0;
  for (size_t i = 0; i < h->u.size(); i++) {
    const auto &row = h->neigh->getNeighbors(i);
    for (size_t k = 0; k < row.size(); k++) cols[rowptr[i] + (int64_t)k] = (int32_t)row[k];
    rowptr[i + 1] = rowptr[i] + (int64_t)row.size();
  }
  return 0;
}

int ref_rnp_get_bond_state(const ref_rnp *h, uint8_t *broken) {
  int64_t o = 0;
  for (size_t i = 0; i < h->u.size(); i++) {
    const size_t len = h->neigh->getNeighbors(i).size();
    for (size_t j = 0; j < len; j++) broken[o++] = h->frac->getBondState(i, j) ? 1 : 0;
  }
  return 0;
}

int ref_rnp_get_fixity(const ref_rnp *h, uint8_t *fix) {
  const auto &fx = h->mesh->getFixity();
  for (size_t i = 0; i < fx.size(); i++) fix[i] = fx[i];
  return 0;
}

// Runs nsteps velocity-Verlet steps (the first call also does FDModel's
// step-0 loads and force evaluation).
int ref_rnp_run(ref_rnp *h, int64_t nsteps) {
  try {
    if (!h->started) h->start();
    for (int64_t k = 0; k < nsteps; k++) h->verlet();
  } catch (const std::exception &e) {
    return fail(e.what());
  }
  return 0;
}

int ref_rnp_get_state(const ref_rnp *h, double *u, double *v, double *f) {
  for (size_t i = 0; i < h->u.size(); i++) {
    const util::Point3 *src[3] = {&h->u[i], &h->v[i], &h->f[i]};
    double *dst[3] = {u, v, f};
    for (int a = 0; a < 3; a++)
      if (dst[a]) {
        dst[a][3 * i] = src[a]->d_x;
        dst[a][3 * i + 1] = src[a]->d_y;
        dst[a][3 * i + 2] = src[a]->d_z;
      }
  }
  return 0;
}

int ref_rnp_get_time(const ref_rnp *h, double *t, int64_t *n) {
  *t = h->time;
  *n = h->step;
  return 0;
}

// FDModel::computePostProcFields energies (fDModel.cpp:651-778): strain
// energy (sum of getBondEF energies) V_i, work done u_i . f_ext(t), kinetic
// energy, and the strain energy where Z_i > 1 - 1e-10 (0 elsewhere).
int ref_rnp_energies(ref_rnp *h, float *strain, float *work, float *kinetic, float *fracture) {
  try {
    const long long n = (long long)h->u.size();
    std::vector<util::Point3> f_ext(n, util::Point3());
    h->fload->apply(h->time, &f_ext, h->mesh);
    for (long long i = 0; i < n; i++) {
      double energy_i = 0., z = 0.;
      auto xi = h->mesh->getNode(i);
      auto ui = h->u[i];
      const auto &row = h->neigh->getNeighbors((size_t)i);
      for (size_t j = 0; j < row.size(); j++) {
        energy_i += h->mat->getBondEF((size_t)i, j).second;
        auto xj = h->mesh->getNode(row[j]);
        auto uj = h->u[row[j]];
        auto rji = xj.dist(xi);
        auto Sji = h->mat->getS(xj - xi, uj - ui);
        double sr = 0.;
        if (util::compare::definitelyGreaterThan(rji, 1.0E-12))
          sr = std::abs(Sji) / h->mat->getSc(rji);
        if (util::compare::definitelyLessThan(z, sr)) z = sr;
      }
      const double voli = h->mesh->getNodalVolume(i);
      strain[i] = float(energy_i * voli);
      work[i] = float(ui.dot(f_ext[i]));
      kinetic[i] = float(0.5 * h->mat->getDensity() * h->v[i].dot(h->v[i]) * voli);
      fracture[i] = util::compare::definitelyGreaterThan(z, 1.0 - 1.0E-10)
                        ? float(energy_i * voli) : 0.f;
    }
  } catch (const std::exception &e) {
    return fail(e.what());
  }
  return 0;
}

// Reaction force of FDModel::computeForce (fDModel.cpp:543-580): for the
// bonds FDModel::is_reaction_force (:582-605) selects, V_i times the getBondEF
// force, with the reference's util::geometry::doLinesIntersect and bounding box.
int ref_rnp_reaction_force(ref_rnp *h, double *R) {
  try {
    const size_t n = h->u.size();
    const auto bb = h->mesh->getBoundingBox();
    const double delta = h->mdeck.d_horizon, eps = 1e-6;
    const double min_x = bb.first[0], max_x = bb.second[0];
    const double max_y = bb.second[1];
    for (size_t i = 0; i < n; i++) {
      auto r = util::Point3();
      auto xi = h->mesh->getNode(i);
      const auto &row = h->neigh->getNeighbors(i);
      for (size_t j = 0; j < row.size(); j++) {
        auto fe = h->mat->getBondEF(i, j);
        auto xj = h->mesh->getNode(row[j]);
        if (xi.d_y > max_y - 1.5 * delta && xi.d_y < max_y - delta) {
          util::Point3 A = util::Point3(min_x, max_y - delta + eps, 0.);
          util::Point3 B = util::Point3(max_x, max_y - delta + eps, 0.);
          if (util::geometry::doLinesIntersect(A, B, xi, xj))
            r += (h->mesh->getNodalVolume(i) * fe.first);
        }
      }
      R[3 * i] = r.d_x;
      R[3 * i + 1] = r.d_y;
      R[3 * i + 2] = r.d_z;
    }
  } catch (const std::exception &e) {
    return fail(e.what());
  }
  return 0;
}

// fe::Mesh::computeVol (mesh.cpp:231-309) on a mesh given as nodes and
// element connectivity: the reference's Mesh constructor reads it through the
// stub readMshFile and computes the nodal volumes with its own quadrature.
int ref_mesh_volumes(int dim, int64_t n, const double *x, int etype, int64_t nelem,
                     const int64_t *enc, double *vol) {
  try {
    const size_t nv = etype == 5 ? 3 : (etype == 9 || etype == 10 ? 4 : 0);
    if (!nv) return fail("element type must be triangle (5), quad (9) or tetrahedron (10)");
    InjectedMesh &m = g_injected_mesh;
    m.nodes.clear();
    for (int64_t i = 0; i < n; i++) m.nodes.emplace_back(x[3 * i], x[3 * i + 1], x[3 * i + 2]);
    m.element_type = (size_t)etype;
    m.vertices = nv;
    m.enc.assign(enc, enc + nelem * (int64_t)nv);
    inp::MeshDeck deck;
    deck.d_dim = (size_t)dim;
    deck.d_spatialDiscretization = "finite_difference";
    deck.d_filename = "injected.msh";
    deck.d_h = 0.;  // the constructor's volume floor 0.01 h^dim stays 0
    fe::Mesh mesh(&deck);
    const auto &v = mesh.getNodalVolumes();
    for (int64_t i = 0; i < n; i++) vol[i] = v[i];
    m.nodes.clear();
  } catch (const std::exception &e) {
    g_injected_mesh.nodes.clear();
    return fail(e.what());
  }
  return 0;
}

// RNPBond::getSc(r) = rbar / sqrt(r) (rnpBond.cpp:319-321).
int ref_rnp_sc(ref_rnp *h, double r, double *sc) {
  *sc = h->mat->getSc(r);
  return 0;
}

}  // extern "C"
