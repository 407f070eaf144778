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
  nlm_fd *handle() const { return d_h; }

 private:
  Deck d_deck;
  nlm_fd *d_h = nullptr;
  std::vector<Point3> d_u, d_v, d_f;
};

}  // namespace nlm
