// fd_example.cpp -- the C++ host classes driving a small RNPBond plate:
// 40 x 40 nodes, horizon 3h, centre pre-crack, top and bottom layers pulled
// apart; prints step, time, max |u|, broken bonds and two energy totals as
// one line.  With the argument "qs": QuasiStaticModel<ElasticState> on a
// 14 x 10 plate, clamped on the left, the right edge pulled in y and loaded
// in x, three load steps; prints the Newton iterations, residual and max |u|.
#include <cmath>
#include <cstdio>
#include <cstring>

#include "nlm_fdmodel.hpp"

static nlm_bc_set edge_bc(double x1, double x2, int dir_mask, int time_fn, double rate,
                          double value) {
  nlm_bc_set bc{};
  bc.region = NLM_REGION_RECTANGLE;
  bc.x1 = x1;
  bc.x2 = x2;
  bc.y1 = -0.01;
  bc.y2 = 1.01;
  bc.dir_mask = dir_mask;
  bc.time_fn = time_fn;
  bc.time_params[0] = rate;
  bc.spatial_fn = NLM_SFN_CONSTANT;
  bc.spatial_params[0] = value;
  return bc;
}

static int quasi_static() {
  nlm::Deck deck;
  const double h = 0.1;
  for (int j = 0; j < 10; j++)
    for (int i = 0; i < 14; i++) {
      deck.nodes.push_back({(i + 0.5) * h, (j + 0.5) * h, 0.});
      deck.volumes.push_back(h * h);
    }
  deck.horizon = 3 * h;
  deck.mesh_size = h;
  deck.material.density = 1200.;
  deck.material.K = 4000.;
  deck.material.G = 1500.;
  deck.ubc.push_back(edge_bc(-0.01, 0.12, 3, NLM_TFN_CONSTANT, 0., 1.));
  deck.ubc.push_back(edge_bc(1.28, 1.41, 2, NLM_TFN_LINEAR, 0.01, 1.));
  deck.fbc.push_back(edge_bc(1.28, 1.41, 1, NLM_TFN_LINEAR, 1., -50.));
  deck.dt = 0.25;
  nlm::SolverDeck solver;
  solver.max_iters = 50;
  solver.tol = 1e-9;
  solver.full_jacobian = 1;
  try {
    nlm::QuasiStaticModel<nlm::material::ElasticState> model(deck, solver);
    double res = 0.;
    int it = model.solve(3, &res);
    double umax = 0.;
    for (const auto &p : model.displacement())
      umax = std::fmax(umax, std::sqrt(p.x * p.x + p.y * p.y + p.z * p.z));
    std::printf("qs newton %d residual %.6e umax %.17e\n", it, res, umax);
  } catch (const nlm::Error &e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  return 0;
}

int main(int argc, char **argv) {
  if (argc > 1 && std::strcmp(argv[1], "qs") == 0) return quasi_static();
  nlm::Deck deck;
  const int nx = 40;
  const double h = 1e-3;
  for (int j = 0; j < nx; j++)
    for (int i = 0; i < nx; i++) {
      deck.nodes.push_back({(i + 0.5) * h, (j + 0.5) * h, 0.});
      deck.volumes.push_back(h * h);
    }
  deck.horizon = 3 * h;
  deck.mesh_size = h;
  deck.material.density = 2440.;
  deck.material.E = 72e9;
  deck.material.Gc = 3.8;
  deck.material.influence_type = 0;
  deck.material.n_influence_params = 1;
  deck.material.influence_params[0] = 1.;
  const double W = nx * h;
  for (int s = 0; s < 2; s++) {
    nlm_bc_set bc{};
    bc.region = NLM_REGION_RECTANGLE;
    bc.x1 = -h;
    bc.x2 = W + h;
    bc.y1 = s == 0 ? -h : W - 3 * h;
    bc.y2 = s == 0 ? 3 * h : W + h;
    bc.dir_mask = 2;
    bc.time_fn = NLM_TFN_LINEAR;
    bc.time_params[0] = s == 0 ? -0.1 : 0.1;
    bc.spatial_fn = NLM_SFN_CONSTANT;
    bc.spatial_params[0] = 1.;
    deck.ubc.push_back(bc);
  }
  nlm_crack c{};
  c.kind = NLM_CRACK_EDGE;
  c.orientation = 1;
  c.pb[0] = 0.4 * W;
  c.pb[1] = 0.5 * W;
  c.pt[0] = 0.6 * W;
  c.pt[1] = 0.5 * W;
  deck.cracks.push_back(c);
  deck.dt = 2e-8;
  deck.steps = 200;
  try {
    nlm::FDModel<nlm::material::RNPBond> model(deck);
    model.integrate();
    double umax = 0.;
    for (const auto &p : model.displacement())
      umax = std::fmax(umax, std::sqrt(p.x * p.x + p.y * p.y + p.z * p.z));
    long broken = 0;
    for (auto b : model.bondStates()) broken += b;
    std::vector<float> es, ew, ek, ef;
    double tot[4];
    model.energies(es, ew, ek, ef, tot);
    std::printf("step %lld time %.6e umax %.6e broken %ld strain %.6e kinetic %.6e\n",
                (long long)model.step(), model.time(), umax, broken, tot[0], tot[2]);
  } catch (const nlm::Error &e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  return 0;
}
