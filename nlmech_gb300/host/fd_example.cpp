// fd_example.cpp -- the C++ host classes driving a small RNPBond plate:
// 40 x 40 nodes, horizon 3h, centre pre-crack, top and bottom layers pulled
// apart; prints step, time, max |u| and broken bonds as one line.
#include <cmath>
#include <cstdio>

#include "nlm_fdmodel.hpp"

int main() {
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
    std::printf("step %lld time %.6e umax %.6e broken %ld\n", (long long)model.step(),
                model.time(), umax, broken);
  } catch (const nlm::Error &e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  return 0;
}
