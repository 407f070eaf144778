// nlm_fdmodel.hpp -- C++ host classes with the shape of NLMech's
// model::FDModel<T> and material plug-ins, running on libnlmgpu.
//
// The reference runs a whole simulation from the FDModel<T> constructor
// (src/model/fd/fDModel.cpp:47-67) and exposes its state through
// data::DataManager.  These classes keep that shape:
//
//   nlm::FDModel<nlm::material::RNPBond> m(deck);   // initHObjects + init
//   m.integrate(nsteps);                            // integrateVerlet / CD loop
//   const auto& u = m.displacement();               // std::vector<Point3>-like
//
// Material plug-ins are tags that select the force kernel; constants come from
// the deck exactly as RNPBond / ElasticState compute them.  Errors are C++
// exceptions carrying libnlmgpu's message (the reference calls exit(1)).
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/nlmgpu.h"

namespace nlm {

struct Point3 {  // util::Point3 layout: three doubles
  double x = 0., y = 0., z = 0.;
};

class Error : public std::runtime_error {
 public:
  Error(int code, const std::string &msg)
      : std::runtime_error("libnlmgpu error " + std::to_string(code) + ": " + msg), code(code) {}
  int code;
};

inline void check(int rc) {
  if (rc != NLM_OK) throw Error(rc, nlm_last_error());
}

namespace material {
struct RNPBond {  // material::pd::RNPBond (src/material/pd/rnpBond.h)
  static constexpr int kind = NLM_MAT_RNP_BOND;
};
struct ElasticState {  // material::pd::ElasticState (src/material/pd/ElasticState.h)
  static constexpr int kind = NLM_MAT_ELASTIC_STATE;
};
}  // namespace material

// Everything FDModel reads from inp::Input for the explicit step.
struct Deck {
  int dim = 2;
  std::vector<Point3> nodes;     // Mesh nodes
  std::vector<double> volumes;   // Mesh nodal volumes
  double horizon = 0., mesh_size = 0.;
  nlm_material material{};       // MaterialDeck
  std::vector<nlm_bc_set> ubc;   // Displacement_BC sets
  std::vector<nlm_bc_set> fbc;   // Force_BC sets
  std::vector<nlm_crack> cracks; // Fracture.Cracks
  int no_fail = NLM_NOFAIL_OFF;
  double no_fail_tol = 0.;
  double dt = 0.;                // Final_Time / Time_Steps
  int64_t steps = 0;             // Time_Steps
  int scheme = NLM_VELOCITY_VERLET;
  int precision = NLM_PREC_FP64;
  int decomposition = NLM_DECOMP_AUTO;
  std::vector<Point3> u0, v0;    // initial condition (may be empty)

  Deck() {
    material.irreversible = 1;
    material.check_sc_factor = 1.;
    material.compute_from_classical = 1;
    material.E = material.G = material.K = material.Gc = material.KIc = -1.;
  }
};

template <class T>
class FDModel {
 public:
  explicit FDModel(const Deck &deck) : d_deck(deck) {
    nlm_fd_desc d{};
    d.dim = deck.dim;
    d.n_nodes = (int64_t)deck.nodes.size();
    d.x = reinterpret_cast<const double *>(deck.nodes.data());
    d.volume = deck.volumes.data();
    d.horizon = deck.horizon;
    d.mesh_size = deck.mesh_size;
    d.material = deck.material;
    d.material.kind = T::kind;
    d.n_ubc = (int)deck.ubc.size();
    d.ubc = deck.ubc.data();
    d.n_fbc = (int)deck.fbc.size();
    d.fbc = deck.fbc.data();
    d.n_cracks = (int)deck.cracks.size();
    d.cracks = deck.cracks.data();
    d.no_fail = deck.no_fail;
    d.no_fail_tol = deck.no_fail_tol;
    d.dt = deck.dt;
    d.scheme = deck.scheme;
    d.precision = deck.precision;
    d.decomposition = deck.decomposition;
    d.u0 = deck.u0.empty() ? nullptr : reinterpret_cast<const double *>(deck.u0.data());
    d.v0 = deck.v0.empty() ? nullptr : reinterpret_cast<const double *>(deck.v0.data());
    check(nlm_fd_create(&d, &d_h));
    d_u.resize(deck.nodes.size());
    d_v.resize(deck.nodes.size());
    d_f.resize(deck.nodes.size());
  }
  ~FDModel() {
    if (d_h) nlm_fd_destroy(d_h);
  }
  FDModel(const FDModel &) = delete;
  FDModel &operator=(const FDModel &) = delete;

  // FDModel::integrate for n steps (all remaining steps when n < 0).
  void integrate(int64_t n = -1) {
    if (n < 0) n = d_deck.steps - step();
    check(nlm_fd_run(d_h, n));
    sync_state();
  }
  void sync_state() {
    check(nlm_fd_get_state(d_h, reinterpret_cast<double *>(d_u.data()),
                           reinterpret_cast<double *>(d_v.data()),
                           reinterpret_cast<double *>(d_f.data())));
  }
  const std::vector<Point3> &displacement() const { return d_u; }
  const std::vector<Point3> &velocity() const { return d_v; }
  const std::vector<Point3> &force() const { return d_f; }
  double time() const {
    double t;
    int64_t s;
    check(nlm_fd_get_time(d_h, &t, &s));
    return t;
  }
  int64_t step() const {
    double t;
    int64_t s;
    check(nlm_fd_get_time(d_h, &t, &s));
    return s;
  }
  // Neighbor::getNeighborsList in CSR form (rows ascending, original ids).
  void neighbors(std::vector<int64_t> &rowptr, std::vector<int32_t> &cols) const {
    int64_t nnz = 0;
    check(nlm_fd_num_bonds(d_h, &nnz));
    rowptr.resize(d_deck.nodes.size() + 1);
    cols.resize(nnz);
    check(nlm_fd_get_neighbors(d_h, rowptr.data(), cols.data()));
  }
  // Fracture::getBondState for every bond, in the neighbors() order.
  std::vector<uint8_t> bondStates() const {
    int64_t nnz = 0;
    check(nlm_fd_num_bonds(d_h, &nnz));
    std::vector<uint8_t> b(nnz);
    check(nlm_fd_get_bond_state(d_h, b.data()));
    return b;
  }
  // computePostProcFields damage fields (Damage_Phi, Damage_Z).
  void damage(std::vector<float> &phi, std::vector<float> &Z) const {
    phi.resize(d_deck.nodes.size());
    Z.resize(d_deck.nodes.size());
    check(nlm_fd_damage(d_h, phi.data(), Z.data()));
  }
  // computePostProcFields energies: Strain_Energy, Work_Done, kinetic and
  // fracture energy per node; totals = their sums.
  void energies(std::vector<float> &strain, std::vector<float> &work,
                std::vector<float> &kinetic, std::vector<float> &fracture,
                double totals[4]) const {
    const size_t n = d_deck.nodes.size();
    strain.resize(n);
    work.resize(n);
    kinetic.resize(n);
    fracture.resize(n);
    check(nlm_fd_energies(d_h, strain.data(), work.data(), kinetic.data(), fracture.data(),
                          totals));
  }
  // Reaction_Force per node and its sum (computeForce, 2-D RNPBond).
  std::vector<Point3> reactionForce(Point3 *sum = nullptr) const {
    std::vector<Point3> R(d_deck.nodes.size());
    double s[3];
    check(nlm_fd_reaction_force(d_h, reinterpret_cast<double *>(R.data()), nullptr, s));
    if (sum) *sum = {s[0], s[1], s[2]};
    return R;
  }
  // fe::Mesh fixity bits as the displacement loading sets them.
  std::vector<uint8_t> fixity() const {
    std::vector<uint8_t> fx(d_deck.nodes.size());
    check(nlm_fd_get_fixity(d_h, fx.data()));
    return fx;
  }
  // FDModel::restart: start at Restart.Step with the given u and v.
  void restart(int64_t step, const std::vector<Point3> &u, const std::vector<Point3> &v) {
    check(nlm_fd_set_state(d_h, reinterpret_cast<const double *>(u.data()),
                           reinterpret_cast<const double *>(v.data())));
    check(nlm_fd_set_time(d_h, double(step) * d_deck.dt, step));
    sync_state();
  }
  // Checkpoint with the bond state (save) and continue from one (load).
  void save(const std::string &path) const { check(nlm_fd_save(d_h, path.c_str())); }
  void load(const std::string &path) {
    check(nlm_fd_load(d_h, path.c_str()));
    sync_state();
  }
  nlm_fd *handle() const { return d_h; }

 private:
  Deck d_deck;
  nlm_fd *d_h = nullptr;
  std::vector<Point3> d_u, d_v, d_f;
};

// QuasiStaticModel<ElasticState> (src/model/quasistatic/QuasiStaticModel.cpp):
// the Solver block and one solve per load step (solver, :526-594).
struct SolverDeck {
  int max_iters = 100;         // Solver.Max_Iteration
  double tol = 1e-6;           // Solver.Tolerance
  double perturbation = 1e-7;  // Solver.Perturbation
  int full_jacobian = 0;       // 0: the reference's (i, r; j, r) entries
  int lin_max_iters = 5000;
  double lin_tol = 1e-12;
};

template <class T>
class QuasiStaticModel {
 public:
  QuasiStaticModel(const Deck &deck, const SolverDeck &solver) : d_n(deck.nodes.size()) {
    static_assert(T::kind == NLM_MAT_ELASTIC_STATE,
                  "QuasiStaticModel is instantiated for ElasticState");
    nlm_fd_desc d{};
    d.dim = deck.dim;
    d.n_nodes = (int64_t)deck.nodes.size();
    d.x = reinterpret_cast<const double *>(deck.nodes.data());
    d.volume = deck.volumes.data();
    d.horizon = deck.horizon;
    d.mesh_size = deck.mesh_size;
    d.material = deck.material;
    d.material.kind = T::kind;
    d.n_ubc = (int)deck.ubc.size();
    d.ubc = deck.ubc.data();
    d.n_fbc = (int)deck.fbc.size();
    d.fbc = deck.fbc.data();
    d.dt = deck.dt;
    nlm_esqs_params p{};
    p.jacobian = solver.full_jacobian;
    p.max_iters = solver.max_iters;
    p.tol = solver.tol;
    p.perturbation = solver.perturbation;
    p.lin_max_iters = solver.lin_max_iters;
    p.lin_tol = solver.lin_tol;
    p.dt = deck.dt;
    check(nlm_esqs_create(&d, &p, &d_q));
  }
  ~QuasiStaticModel() {
    if (d_q) nlm_esqs_destroy(d_q);
  }
  QuasiStaticModel(const QuasiStaticModel &) = delete;
  QuasiStaticModel &operator=(const QuasiStaticModel &) = delete;

  // n load steps; returns the Newton iterations of the last and its residual.
  int solve(int n, double *residual = nullptr) {
    std::vector<int> it(n > 0 ? n : 1);
    double r = 0.;
    check(nlm_esqs_solve(d_q, n, it.data(), nullptr, &r));
    if (residual) *residual = r;
    return n > 0 ? it[n - 1] : 0;
  }
  std::vector<Point3> displacement() const {
    std::vector<Point3> u(d_n);
    check(nlm_esqs_get_state(d_q, reinterpret_cast<double *>(u.data()), nullptr));
    return u;
  }
  // The output's "Force": force density times nodal volume.
  std::vector<Point3> force() const {
    std::vector<Point3> f(d_n);
    check(nlm_esqs_get_state(d_q, nullptr, reinterpret_cast<double *>(f.data())));
    return f;
  }

 private:
  size_t d_n;
  nlm_esqs *d_q = nullptr;
};

}  // namespace nlm
