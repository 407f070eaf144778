// fd_host.cu -- C ABI of the model handle: set-up, time loop, state I/O,
// checkpoints and post-processing.
//
// Replaces model::FDModel<T> (src/model/fd/fDModel.cpp) for T = RNPBond and
// ElasticState.  Set-up mirrors FDModel::initHObjects/init (:133-315):
// neighbour lists, pre-cracks, interior flags, loading tables, material
// constants.  The time loop mirrors FDModel::integrate (:317-374).
//
// Phase bookkeeping of the fused step.  One launch K_m does, per node, the
// force evaluation at u^m plus the integrator work on both sides of it:
//   Verlet:  v^m = (v^{m-1} + c f^{m-1}) + c f^m;   u^{m+1} = u^m + dt (v^m + c f^m)
//   CD:      u^{m+1} = u^m + (c' f^m + dt v^m);     v^{m+1} = (u^{m+1} - u^m) / dt
// with c = dt/(2 rho), c' = dt^2/rho.  u is ping-ponged (u^m read, u^{m+1}
// written); v is ping-ponged for CD.  After K_m the buffers hold exactly the
// reference's (u^m, v^m, f^m), and u^{m+1} is already in the other buffer.
// The velocity half-kick v^{m-1} + c f^{m-1} is recomputed from the stored
// f^{m-1}, so every value is produced by the same sequence of roundings as
// integrateVerlet.  K_0 (first = true) does the step-0 force evaluation of
// integrate() (:319-333) and the drift of step 1.

#include <array>

#include "fd_handle.h"
#include "tile_store.h"

namespace nlm {

bool finite_all(const double *a, int64_t n) {
  for (int64_t i = 0; i < n; i++)
    if (!std::isfinite(a[i])) return false;
  return true;
}

// No-fail flags (ComputeInterior / DataInterior, interiorFlags.cpp:57-100,
// :146-185): a node is not interior when it lies within tol of the mesh
// bounding box.  fe::Mesh::computeBBox (mesh.cpp:311-324) starts both corners
// at the origin and only widens them, so the box always contains the origin.
void mesh_bbox(const double *x, int64_t n, double lo[3], double hi[3]) {
  for (int dd = 0; dd < 3; dd++) lo[dd] = hi[dd] = 0.;
  for (int64_t i = 0; i < n; i++)
    for (int dd = 0; dd < 3; dd++) {
      if (hLT(x[3 * i + dd], lo[dd])) lo[dd] = x[3 * i + dd];
      if (hLT(hi[dd], x[3 * i + dd])) hi[dd] = x[3 * i + dd];
    }
}

// The No_Fail_Region list (:76-90): circles |x - c| < r and rectangles
// (isPointInsideRectangle, utilGeom.cpp:43-50) are not interior either.
void nofail_flags(const double *x, int64_t n, double tol, int nreg, const nlm_nofail_region *reg,
                  std::vector<uint8_t> &interior) {
  double lo[3], hi[3];
  mesh_bbox(x, n, lo, hi);
  for (int64_t i = 0; i < n; i++) {
    const double *p = x + 3 * i;
    bool in = !(hLT(p[0], lo[0] + tol) || hLT(p[1], lo[1] + tol) ||
                hGT(p[0], hi[0] - tol) || hGT(p[1], hi[1] - tol));
    for (int r = 0; r < nreg && in; r++) {
      const double *q = reg[r].params;
      if (reg[r].kind == NLM_NOFAIL_CIRCLE) {
        const double d0 = p[0] - q[0], d1 = p[1] - q[1], d2 = p[2] - q[2];
        if (hLT(std::sqrt(d0 * d0 + d1 * d1 + d2 * d2), q[3])) in = false;
      } else if (!(hLT(p[0], q[0] - 1.0E-12) || hLT(p[1], q[1] - 1.0E-12) ||
                   hGT(p[0], q[2] + 1.0E-12) || hGT(p[1], q[3] + 1.0E-12))) {
        in = false;
      }
    }
    interior[i] = in;
  }
}

// The function names ULoading and FLoading accept (uLoading.cpp:35-53,
// fLoading.cpp:33-52); the reference exits on any other.
int check_bc_functions(const nlm_fd_desc &d) {
  for (int k = 0; k < d.n_ubc; k++) {
    const nlm_bc_set &b = d.ubc[k];
    if (b.region < NLM_REGION_RECTANGLE || b.region > NLM_REGION_ANGLED_RECTANGLE)
      return fail(NLM_ERR_INVALID, "Displacement_BC region type not recognised");
    if (b.spatial_fn < NLM_SFN_CONSTANT || b.spatial_fn > NLM_SFN_LINEAR_Z)
      return fail(NLM_ERR_INVALID, "Displacement_BC spatial function not recognised");
    if (b.time_fn < NLM_TFN_CONSTANT || b.time_fn > NLM_TFN_LINEAR_SLOW_FAST)
      return fail(NLM_ERR_INVALID, "Displacement_BC time function not recognised");
  }
  for (int k = 0; k < d.n_fbc; k++) {
    const nlm_bc_set &b = d.fbc[k];
    if (b.region != NLM_REGION_RECTANGLE && b.region != NLM_REGION_LINE &&
        b.region != NLM_REGION_ANGLED_RECTANGLE && b.region != NLM_REGION_CUBOID)
      return fail(NLM_ERR_INVALID, "Force_BC region type not recognised (fLoading.cpp:24-31)");
    if (b.spatial_fn < NLM_SFN_CONSTANT || b.spatial_fn > NLM_SFN_LINE_LOAD)
      return fail(NLM_ERR_INVALID, "Force_BC spatial function not recognised");
    if (b.time_fn < NLM_TFN_CONSTANT || b.time_fn > NLM_TFN_LINEAR_SLOW_FAST ||
        b.time_fn == NLM_TFN_QUADRATIC)
      return fail(NLM_ERR_INVALID, "Force_BC time function not recognised");
  }
  return NLM_OK;
}

int check_nofail_regions(const nlm_fd_desc &d) {
  if (d.n_nofail_regions < 0 || (d.n_nofail_regions > 0 && !d.nofail_regions))
    return fail(NLM_ERR_INVALID, "bad no-fail region list");
  for (int r = 0; r < d.n_nofail_regions; r++)
    if (d.nofail_regions[r].kind != NLM_NOFAIL_CIRCLE &&
        d.nofail_regions[r].kind != NLM_NOFAIL_RECTANGLE)
      return fail(NLM_ERR_INVALID, "no-fail region kind must be circle or rectangle");
  return NLM_OK;
}

// RNPBond constants (rnpBond.cpp:23-97, computeParameters :99-189) and the
// influence function (influenceFn.h:85-402).
int rnp_constants(const nlm_material &m, int dim, double delta, StepParams &P) {
  double Kbulk = 0.;
  P.infl_type = m.influence_type;
  const int np = m.n_influence_params;
  double M = 0.;
  if (m.influence_type == 0) {
    P.infl_a0 = np == 0 ? double(dim + 1) : m.influence_params[0];
    M = P.infl_a0 / double(dim + 1);
  } else if (m.influence_type == 1) {
    if (np == 0) {
      P.infl_a0 = dim == 1 ? 6. : (dim == 2 ? 12. : 20.);
      P.infl_a1 = -P.infl_a0;
    } else {
      P.infl_a0 = m.influence_params[0];
      P.infl_a1 = np < 2 ? -P.infl_a0 : m.influence_params[1];
    }
    M = (P.infl_a0 / double(dim + 1)) + (P.infl_a1 / double(dim + 2));
  } else if (m.influence_type == 2) {
    if (np == 0) {
      P.infl_beta = 0.2;
      const double b = P.infl_beta;
      if (dim == 1)
        P.infl_alpha = 2. / (b * (1. - std::exp(-1. / b)));
      else if (dim == 2)
        P.infl_alpha = (4.0 / b) * 1.0 /
                       (std::sqrt(M_PI * b) * std::erf(1.0 / std::sqrt(b)) - 2.0 * std::exp(-1.0 / b));
      else
        P.infl_alpha = (2.0 / b) * 1.0 / (b - (b + 1.) * std::exp(-1.0 / b));
    } else {
      P.infl_alpha = m.influence_params[0];
      P.infl_beta = m.influence_params[1];
    }
    const double a = P.infl_alpha, b = P.infl_beta;
    const double sq1 = std::sqrt(b), sq2 = std::sqrt(M_PI);
    if (dim == 1)
      M = 0.5 * a * b * (1. - std::exp(-1. / b));
    else if (dim == 2)
      M = 0.5 * a * b * sq1 * (0.5 * sq2 * std::erf(1. / sq1) - (1. / sq1) * std::exp(-1. / b));
    else
      M = 0.5 * a * b * b * (1. - (1. + 1. / b) * std::exp(-1. / b));
  } else {
    return fail(NLM_ERR_INVALID, "unknown influence function type");
  }
  P.irrev = m.irreversible ? 1 : 0;
  P.fsc = m.check_sc_factor;
  if (dim == 2)
    P.invF = std::pow(delta, 3) * M_PI;
  else
    P.invF = std::pow(delta, 4) * 4. * M_PI / 3.;
  if (m.compute_from_classical) {
    double E = m.E, K = m.K, Gc = m.Gc, KIc = m.KIc;
    if (hLT(E, 0.) && hLT(K, 0.)) return fail(NLM_ERR_INVALID, "RNPBond needs E or K");
    if (hLT(Gc, 0.) && hLT(KIc, 0.)) return fail(NLM_ERR_INVALID, "RNPBond needs Gc or KIc");
    const double nu = m.plane_strain ? 0.25 : 1. / 3.;
    if (E > 0.) K = E / (3. * (1. - 2. * nu));
    if (K > 0. && E < 0.) E = K * (3. * (1. - 2. * nu));
    if (Gc > 0.) KIc = std::sqrt(Gc * E);
    if (KIc > 0. && Gc < 0.) Gc = KIc * KIc / E;
    const double lambda = E * nu / ((1. + nu) * (1. - 2. * nu));
    if (dim == 2) {
      P.C = M_PI * Gc / (4. * M);
      P.beta = 4. * lambda / (P.C * M);
    } else {
      P.C = 2. * Gc / (3. * M);
      P.beta = 5. * lambda / (P.C * M);
    }
    Kbulk = K;
  } else {
    P.C = m.bond_params[0];
    P.beta = m.bond_params[1];
    // computeMaterialProperties (rnpBond.cpp:190-211): nu = 0.33, lambda
    // from C and beta, then E and K
    const double nu = 0.33;
    const double lambda = dim == 2 ? P.C * M * P.beta / 4. : P.C * M * P.beta / 5.;
    const double E = lambda * (1. + nu) * (1. - 2. * nu) / nu;
    Kbulk = E / (3. * (1. - 2. * nu));
  }
  P.rbar = std::sqrt(0.5 / P.beta);
  // contact between the nodes of broken bonds (RNPBond ctor, rnpBond.cpp:79-88)
  P.contact = m.apply_contact ? 1 : 0;
  P.contact_kn = m.apply_contact ? Kbulk * 18. / (M_PI * std::pow(delta, 5)) : 0.;
  if (!(P.C > 0.) || !(P.beta > 0.)) return fail(NLM_ERR_INVALID, "RNPBond constants not positive");
  return NLM_OK;
}

// Lattice renumbering of an FP32C model on a tile decomposition (after the
// neighbour build, which orders nodes by the Morton code of their search
// cell, edge >= horizon).  Nodes are renumbered by the Morton code of their
// cell on the mesh lattice (edge h, g = floor((x - lo) / h + 1/2)):
// consecutive nodes then form 4 x 2, 8 x 4, ... 16 x 16 patches of a
// grid-like 2-D mesh (2 x 2 x 2, ... 8 x 8 x 4 blocks in 3-D), and a 256-node
// tile is one such patch.  Each row is ordered by the lattice offset of its
// neighbour (|offset|^2, then the offset's components; ties by node): in the
// interior the k-th neighbours of eight consecutive nodes are then the same
// offset from each of them, a shifted 4 x 2 patch (2 x 2 x 2 block) whose
// lattice residues are all different, which is what the tile kernels'
// shared-memory layout needs to read the eight records of a quarter warp in
// one pass.  Any node set works (the order is only a layout); only the
// results' rounding changes.  lres receives each node's residue (new order):
// (g_x mod 4, g_y mod 2) as a Morton code in 2-D, (g_x, g_y, g_z mod 2) in 3-D.
int lattice_relabel(NeighborBuild &nb, int dim, int S, double mesh_h, double delta,
                    cudaStream_t s, std::vector<uint8_t> &lres) {
  const int64_t n = nb.n, nnz = nb.nnz;
  if (n == 0) return NLM_OK;
  std::vector<int> perm(n), cols(nnz);
  std::vector<double> pos((size_t)S * n);
  std::vector<int64_t> rp(n + 1);
  NLM_CUDA(cudaMemcpyAsync(perm.data(), nb.perm, sizeof(int) * n, cudaMemcpyDeviceToHost, s));
  NLM_CUDA(cudaMemcpyAsync(pos.data(), nb.pos, sizeof(double) * S * n, cudaMemcpyDeviceToHost, s));
  NLM_CUDA(cudaMemcpyAsync(rp.data(), nb.rowptr, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToHost, s));
  if (nnz) NLM_CUDA(cudaMemcpyAsync(cols.data(), nb.cols, sizeof(int) * nnz, cudaMemcpyDeviceToHost, s));
  NLM_CUDA(cudaStreamSynchronize(s));
  const int D3 = dim == 3 ? 3 : 2;
  double lo[3] = {1e300, 1e300, 1e300};
  for (int64_t i = 0; i < n; i++)
    for (int d = 0; d < D3; d++) lo[d] = std::min(lo[d], pos[(size_t)S * i + d]);
  std::vector<int64_t> gc((size_t)3 * n, 0);
  std::vector<std::pair<uint64_t, int64_t>> key(n);
  const int bits = D3 == 3 ? 21 : 32;
  auto spread = [&](uint64_t v) {
    uint64_t r = 0;
    for (int b = 0; b < bits; b++) r |= ((v >> b) & 1ull) << (D3 * b);
    return r;
  };
  const int64_t cmax = (1ll << bits) - 1;
  for (int64_t i = 0; i < n; i++) {
    uint64_t k = 0;
    for (int d = 0; d < D3; d++) {
      const int64_t g = (int64_t)std::floor((pos[(size_t)S * i + d] - lo[d]) / mesh_h + 0.5);
      gc[3 * i + d] = g;
      k |= spread((uint64_t)std::max<int64_t>(0, std::min<int64_t>(g, cmax))) << d;
    }
    key[i] = {k, i};
  }
  std::sort(key.begin(), key.end());  // ties keep the search-cell order
  std::vector<int64_t> order(n), inv(n);
  for (int64_t k = 0; k < n; k++) {
    order[k] = key[k].second;
    inv[key[k].second] = k;
  }
  // rank of a lattice offset: |o|^2, then its components
  const int R = (int)std::ceil(delta / mesh_h) + 2, W = 2 * R + 1, Wz = D3 == 3 ? W : 1;
  std::vector<std::pair<std::array<int, 4>, int>> offs;
  for (int oz = (D3 == 3 ? -R : 0); oz <= (D3 == 3 ? R : 0); oz++)
    for (int oy = -R; oy <= R; oy++)
      for (int ox = -R; ox <= R; ox++)
        offs.push_back({{ox * ox + oy * oy + oz * oz, oz, oy, ox},
                        ((oz + (D3 == 3 ? R : 0)) * W + oy + R) * W + ox + R});
  std::sort(offs.begin(), offs.end());
  std::vector<int> orank((size_t)W * W * Wz);
  for (size_t k = 0; k < offs.size(); k++) orank[offs[k].second] = (int)k;
  std::vector<int> perm2(n), cols2(nnz);
  std::vector<double> pos2((size_t)S * n);
  std::vector<int64_t> rp2(n + 1, 0);
  lres.assign(n, 0);
  for (int64_t k = 0; k < n; k++) {
    const int64_t o = order[k];
    perm2[k] = perm[o];
    for (int d = 0; d < S; d++) pos2[(size_t)S * k + d] = pos[(size_t)S * o + d];
    rp2[k + 1] = rp2[k] + (rp[o + 1] - rp[o]);
    const int64_t *g = &gc[3 * o];
    lres[k] = D3 == 3 ? (uint8_t)((g[0] & 1) | ((g[1] & 1) << 1) | ((g[2] & 1) << 2))
                      : (uint8_t)((g[0] & 1) | ((g[1] & 1) << 1) | ((g[0] & 2) << 1));
  }
  unsigned nthr = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  auto work = [&](unsigned w) {
    std::vector<std::pair<int64_t, int>> row;
    for (int64_t k = w; k < n; k += nthr) {
      const int64_t o = order[k];
      row.clear();
      for (int64_t q = rp[o]; q < rp[o + 1]; q++) {
        const int64_t jo = cols[q];
        int64_t d[3] = {0, 0, 0};
        bool in = true;
        for (int c = 0; c < D3; c++) {
          d[c] = gc[3 * jo + c] - gc[3 * o + c];
          in = in && d[c] >= -R && d[c] <= R;
        }
        const int64_t rk =
            in ? orank[((d[2] + (D3 == 3 ? R : 0)) * W + d[1] + R) * W + d[0] + R]
               : (int64_t)W * W * Wz + d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        row.push_back({rk * (int64_t)n + inv[jo], (int)inv[jo]});
      }
      std::sort(row.begin(), row.end());
      for (size_t q = 0; q < row.size(); q++) cols2[rp2[k] + (int64_t)q] = row[q].second;
    }
  };
  std::vector<std::thread> pool;
  for (unsigned w = 0; w < nthr; w++) pool.emplace_back(work, w);
  for (auto &th : pool) th.join();
  NLM_CUDA(cudaMemcpyAsync(nb.perm, perm2.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
  NLM_CUDA(cudaMemcpyAsync(nb.pos, pos2.data(), sizeof(double) * S * n, cudaMemcpyHostToDevice, s));
  NLM_CUDA(cudaMemcpyAsync(nb.rowptr, rp2.data(), sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice, s));
  if (nnz) NLM_CUDA(cudaMemcpyAsync(nb.cols, cols2.data(), sizeof(int) * nnz, cudaMemcpyHostToDevice, s));
  NLM_CUDA(cudaStreamSynchronize(s));
  return NLM_OK;
}

int launch_step(nlm_fd *h, const StepArgs &a0) {
  StepArgs a = a0;
  if (a.i1 == 0) a.i1 = h->n;
  // after the step-0 evaluation every step launch follows another step or a
  // between-steps kernel that writes only state (u, v, f, bits, loads)
  a.pdl = !a.first;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (h->timing && !h->capturing) {
    while (h->ev_used + 2 > h->ev_pool.size()) {
      cudaEvent_t e;
      NLM_CUDA(cudaEventCreate(&e));
      h->ev_pool.push_back(e);
    }
    e0 = h->ev_pool[h->ev_used++];
    e1 = h->ev_pool[h->ev_used++];
    NLM_CUDA(cudaEventRecord(e0, h->stream));
  }
  cudaError_t e;
  const bool fp32 = h->precision == NLM_PREC_FP32C;
  if (h->material == NLM_MAT_RNP_BOND)
    e = fp32 ? launch_rnp_step_fp32(h->P, h->D, h->T, a, h->decomp, h->stream)
             : launch_rnp_step_fp64(h->P, h->D, h->T, a, h->decomp, h->stream);
  else
    e = fp32 ? launch_es_step_fp32(h->P, h->D, h->T, a, h->decomp, h->stream)
             : launch_es_step_fp64(h->P, h->D, h->T, a, h->decomp, h->stream);
  if (e != cudaSuccess) return cuda_fail(e, "step kernel launch");
  if (h->timing && !h->capturing) {
    NLM_CUDA(cudaEventRecord(e1, h->stream));
    h->launches++;
  }
  return NLM_OK;
}

int build_tiles(nlm_fd *h, const int64_t *sell_ptr_dev, int max_local, const double *x) {
  TileInputs in{h->n, h->nnz, h->nslices, h->sell_entries, h->D.cols, sell_ptr_dev,
                &h->rowptr, &h->perm, max_local,
                h->lattice_res.empty() ? nullptr : &h->lattice_res};
  // Interior prefixes of the rows, for RNPBond with a constant influence
  // function: a bond with r <= check_low - 1e-3 h has volume factor 1 in
  // FP32 too, as long as the tile frame's rounding (2^-24 of the tile's
  // extent per coordinate) and the FP32 forming of r stay far below the
  // 1e-3 h margin: tiles up to 1000 h across.
  if (h->material == NLM_MAT_RNP_BOND && h->P.infl_type == 0 && h->P.h > 0.) {
    in.xc = x;
    in.r_int = h->P.check_low - 1e-3 * h->P.h;
    in.ext_max = 1000. * h->P.h;
  }
  return build_tile_store(h, in, h->tile_ok, &h->tile_need);
}

// Work-decomposition autotuner: time each candidate step kernel on scratch
// copies of the arrays a step writes and keep the fastest.
int autotune(nlm_fd *h) {
  const int S = h->S;
  const int64_t n = h->n;
  cudaStream_t s = h->stream;
  DevPtrs D = h->D;
  float4 *sv0 = nullptr, *sv1 = nullptr;
  float *sf = nullptr;
  uint32_t *sb = nullptr;
  const size_t nb = (size_t)h->P.nwords * h->P.npad;
  cudaError_t e = cudaMalloc(&sv0, sizeof(float4) * (S / 2) * n);
  if (e == cudaSuccess) e = cudaMalloc(&sv1, sizeof(float4) * (S / 2) * n);
  if (e == cudaSuccess) e = cudaMalloc(&sf, sizeof(float) * S * n);
  if (e == cudaSuccess) e = cudaMalloc(&sb, sizeof(uint32_t) * nb);
  auto cleanup = [&]() { cudaFree(sv0); cudaFree(sv1); cudaFree(sf); cudaFree(sb); };
  if (e != cudaSuccess) {
    cleanup();
    return cuda_fail(e, "autotune scratch");
  }
  cudaMemcpyAsync(sv0, D.v32[0], sizeof(float4) * (S / 2) * n, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(sv1, D.v32[0], sizeof(float4) * (S / 2) * n, cudaMemcpyDeviceToDevice, s);
  cudaMemsetAsync(sf, 0, sizeof(float) * S * n, s);
  cudaMemcpyAsync(sb, D.bits, sizeof(uint32_t) * nb, cudaMemcpyDeviceToDevice, s);
  D.v32[0] = sv0;
  D.v32[1] = sv1;
  D.f32 = sf;
  D.bits = sb;
  const bool rnp = h->material == NLM_MAT_RNP_BOND;
  std::vector<int> cands = {NLM_DECOMP_THREAD};
  if (rnp) {
    cands.push_back(NLM_DECOMP_THREAD1);
    cands.push_back(NLM_DECOMP_WARP);
  }
  if (h->tile_ok) {
    if (rnp) cands.push_back(NLM_DECOMP_TILE);
    cands.push_back(NLM_DECOMP_TILE_LOCAL);
  }
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  float best = 1e30f;
  int pick = NLM_DECOMP_THREAD;
  StepArgs sa{0, false, h->time, h->time + h->dt, nullptr, 0, h->n};
  for (int c : cands) {
    auto launch = [&]() {
      return rnp ? launch_rnp_step_fp32(h->P, D, h->T, sa, c, s)
                 : launch_es_step_fp32(h->P, D, h->T, sa, c, s);
    };
    for (int w = 0; w < 2; w++) e = launch();
    cudaEventRecord(a, s);
    for (int r = 0; r < 5; r++) e = launch();
    cudaEventRecord(b, s);
    if (e == cudaSuccess) e = cudaEventSynchronize(b);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
    if (e != cudaSuccess) break;
    if (ms < best) {
      best = ms;
      pick = c;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaStreamSynchronize(s);
  cleanup();
  if (e != cudaSuccess) return cuda_fail(e, "autotune");
  h->decomp = pick;
  return NLM_OK;
}

int apply_fbc(nlm_fd *h, double t) {
  if (h->n_fbc_nodes == 0) return NLM_OK;
  k_fbc_apply<<<nblk(h->n_fbc_nodes, 128), 128, 0, h->stream>>>(
      h->n_fbc_nodes, h->S, h->fbc_nodes, h->fbc_iptr, h->fbc_items, h->FT, t,
      const_cast<double *>(h->D.fext));
  NLM_CUDA(cudaGetLastError());
  return NLM_OK;
}

int apply_bc(nlm_fd *h, double t) {
  if (h->n_bc_nodes == 0) return NLM_OK;
  const bool fp32 = h->precision == NLM_PREC_FP32C;
  k_bc_apply<<<nblk(h->n_bc_nodes, 128), 128, 0, h->stream>>>(
      h->n_bc_nodes, h->S, h->dim, h->bc_nodes, h->D.bcref, h->D.bce, h->D.flags, h->T, t,
      fp32 ? nullptr : h->D.u64[h->cur], fp32 ? h->D.u32[h->cur] : nullptr,
      fp32 ? nullptr : h->D.v[h->vidx()], fp32 ? h->D.v32[h->vidx()] : nullptr);
  NLM_CUDA(cudaGetLastError());
  return NLM_OK;
}

// Capture graph_steps consecutive steps starting from ping index c0.
int capture_graph(nlm_fd *h, int c0) {
  cudaGraph_t g = nullptr;
  h->capturing = true;
  cudaError_t e = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) {
    h->capturing = false;
    return cuda_fail(e, "cudaStreamBeginCapture");
  }
  int c = c0, rc = NLM_OK;
  for (int k = 0; k < h->graph_steps && rc == NLM_OK; k++) {
    c = 1 - c;
    if (h->n_fbc_nodes > 0) {
      // FLoading::apply at the step's time, read from the time array
      k_fbc_apply<<<nblk(h->n_fbc_nodes, 128), 128, 0, h->stream>>>(
          h->n_fbc_nodes, h->S, h->fbc_nodes, h->fbc_iptr, h->fbc_items, h->FT, 0.,
          const_cast<double *>(h->D.fext), h->d_times + k);
      const cudaError_t ef = cudaGetLastError();
      if (ef != cudaSuccess) rc = cuda_fail(ef, "force-load kernel");
    }
    StepArgs a{c, false, 0., 0., h->d_times + k, 0, h->n};
    if (rc == NLM_OK) rc = launch_step(h, a);
  }
  e = cudaStreamEndCapture(h->stream, &g);
  h->capturing = false;
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
  e = cudaGraphInstantiate(&h->gexec[c0], g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
  return NLM_OK;
}

// Fracture::addCrack (fracture.cpp:45-70) for the step that ended at h->time:
// the first timed crack not yet cut whose activation time is definitely less
// than that time is cut into the bond state; one crack per call.  The
// reference calls it after the step's output (fDModel.cpp:352-373); here it
// runs just before the next step's launch, which is the same point for the
// dynamics and leaves the state read between run calls equal to the one the
// reference's output of that step sees.
int add_crack(nlm_fd *h) {
  for (size_t c = 0; c < h->timed_cracks.size(); c++) {
    if (h->cracks_on >> c & 1u) continue;
    if (!dLT(h->timed_cracks[c].activation_time, h->time)) continue;
    NLM_CUDA(apply_precrack(h->n, h->S, h->D.pos64, h->D.rowptr, h->D.cols, h->timed_cracks[c],
                            h->P.npad, h->D.bits, h->stream));
    h->cracks_on |= 1u << c;
    return NLM_OK;
  }
  return NLM_OK;
}

// True if a timed crack would be cut before one of the next nsteps steps
// (checked at the times h->time, h->time + dt, ..., accumulated as in do_run).
bool crack_due(const nlm_fd *h, int64_t nsteps) {
  if ((uint64_t)h->cracks_on + 1 == (1ull << h->timed_cracks.size())) return false;
  double t = h->time;
  for (int64_t k = 1; k < nsteps; k++) t = t + h->dt;
  for (size_t c = 0; c < h->timed_cracks.size(); c++)
    if (!(h->cracks_on >> c & 1u) && dLT(h->timed_cracks[c].activation_time, t)) return true;
  return false;
}

int single_steps(nlm_fd *h, int64_t nsteps) {
  for (int64_t s = 0; s < nsteps; s++) {
    int rc;
    if (!h->timed_cracks.empty() && h->step > 0 && (rc = add_crack(h))) return rc;
    const double tm = h->time + h->dt;
    h->cur = 1 - h->cur;
    if ((rc = apply_fbc(h, tm))) return rc;
    StepArgs a{h->cur, false, tm, tm + h->dt, nullptr, 0, h->n};
    if ((rc = launch_step(h, a))) return rc;
    h->time = tm;
    h->step++;
  }
  return NLM_OK;
}

int do_run(nlm_fd *h, int64_t nsteps) {
  if (!h->started) {
    int rc = apply_bc(h, h->time);
    if (rc) return rc;
    if ((rc = apply_fbc(h, h->time))) return rc;
    StepArgs a{h->cur, true, h->time, h->time + h->dt, nullptr, 0, h->n};
    if ((rc = launch_step(h, a))) return rc;
    h->started = true;
  }
  const int G = h->graph_steps;
  while (G > 0 && nsteps >= G) {
    if (!h->timed_cracks.empty() && crack_due(h, G)) {
      // a crack is cut within this chunk: its steps run one by one
      int rc = single_steps(h, G);
      if (rc) return rc;
      nsteps -= G;
      continue;
    }
    if (!h->gexec[h->cur]) {
      int rc = capture_graph(h, h->cur);
      if (rc) return rc;
    }
    // step times of the chunk, accumulated as the reference does
    NLM_CUDA(cudaEventSynchronize(h->ev_times));
    double t = h->time;
    for (int k = 0; k <= G; k++) {
      t = t + h->dt;
      h->h_times[k] = t;
    }
    NLM_CUDA(cudaMemcpyAsync(h->d_times, h->h_times, sizeof(double) * (G + 1),
                             cudaMemcpyHostToDevice, h->stream));
    NLM_CUDA(cudaEventRecord(h->ev_times, h->stream));
    NLM_CUDA(cudaGraphLaunch(h->gexec[h->cur], h->stream));
    h->time = h->h_times[G - 1];
    h->step += G;
    nsteps -= G;
  }
  return single_steps(h, nsteps);
}

}  // namespace nlm

// ---- C ABI ---------------------------------------------------------------
extern "C" {

const char *nlm_last_error(void) { return last_error(); }
int nlm_abi_version(void) { return NLM_ABI_VERSION; }

int nlm_device_count(int *count) {
  if (!count) return fail(NLM_ERR_INVALID, "null count");
  int c = 0;
  cudaError_t e = cudaGetDeviceCount(&c);
  if (e != cudaSuccess) {
    cudaGetLastError();
    c = 0;
  }
  *count = c;
  return NLM_OK;
}

int nlm_set_device(int device) {
  NLM_CUDA(cudaSetDevice(device));
  return NLM_OK;
}

int nlm_neighbor_search(int dim, int64_t n, const double *x, double horizon, int64_t *rowptr,
                        int32_t *cols) {
  if (n < 0 || (n > 0 && !x) || !rowptr || dim < 1 || dim > 3 || !(horizon > 0.))
    return fail(NLM_ERR_INVALID, "nlm_neighbor_search: bad arguments");
  if (n > INT32_MAX - 1) return fail(NLM_ERR_INVALID, "too many nodes");
  if (!finite_all(x, 3 * n)) return fail(NLM_ERR_NONFINITE, "non-finite coordinate");
  cudaStream_t s;
  NLM_CUDA(cudaStreamCreate(&s));
  double *dx = nullptr;
  NeighborBuild nb;
  std::string why;
  auto cleanup = [&]() {
    cudaFree(dx); cudaFree(nb.perm); cudaFree(nb.pos); cudaFree(nb.rowptr); cudaFree(nb.cols);
    cudaStreamDestroy(s);
  };
  cudaError_t e = cudaMalloc(&dx, sizeof(double) * 3 * (n + 1));
  if (e == cudaSuccess) e = cudaMemcpyAsync(dx, x, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s);
  const Grid g = make_grid(dim, n, x, horizon);
  if (e == cudaSuccess) e = build_neighbors(nb, dim, n, dx, g, 4, s, why);
  if (e != cudaSuccess) {
    int rc = why.empty() ? cuda_fail(e, "neighbour search") : fail(NLM_ERR_INVALID, why);
    cleanup();
    return rc;
  }
  std::vector<int> perm(n);
  std::vector<int64_t> rp(n + 1);
  std::vector<int> cc(nb.nnz);
  e = cudaMemcpy(perm.data(), nb.perm, sizeof(int) * n, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(rp.data(), nb.rowptr, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && nb.nnz) e = cudaMemcpy(cc.data(), nb.cols, sizeof(int) * nb.nnz, cudaMemcpyDeviceToHost);
  cleanup();
  if (e != cudaSuccess) return cuda_fail(e, "neighbour download");
  std::vector<int64_t> inv(n);
  for (int64_t i = 0; i < n; i++) inv[perm[i]] = i;
  rowptr[0] = 0;
  for (int64_t o = 0; o < n; o++) rowptr[o + 1] = rowptr[o] + (rp[inv[o] + 1] - rp[inv[o]]);
  if (cols)
    for (int64_t o = 0; o < n; o++) {
      const int64_t s0 = rp[inv[o]], len = rp[inv[o] + 1] - s0;
      for (int64_t k = 0; k < len; k++) cols[rowptr[o] + k] = perm[cc[s0 + k]];
    }
  return NLM_OK;
}

int nlm_fd_create(const nlm_fd_desc *d, nlm_fd **out) {
  if (!d || !out) return fail(NLM_ERR_INVALID, "null argument");
  *out = nullptr;
  if (d->dim != 2 && d->dim != 3)
    return fail(NLM_ERR_UNSUPPORTED, "explicit model supports dim 2 and 3");
  if (d->n_nodes <= 0 || !d->x || !d->volume) return fail(NLM_ERR_INVALID, "empty mesh");
  if (d->n_nodes > INT32_MAX - 64) return fail(NLM_ERR_INVALID, "too many nodes for one handle");
  if (!(d->horizon > 0.) || !(d->mesh_size > 0.) || !(d->dt > 0.))
    return fail(NLM_ERR_INVALID, "horizon, mesh size and dt must be positive");
  if (!(d->material.density > 0.)) return fail(NLM_ERR_INVALID, "density must be positive");
  if (d->n_ubc < 0 || d->n_ubc > kMaxBCSets || d->n_fbc < 0 || d->n_fbc > kMaxBCSets)
    return fail(NLM_ERR_INVALID, "too many BC sets");
  if ((d->n_ubc && !d->ubc) || (d->n_fbc && !d->fbc) || (d->n_cracks && !d->cracks))
    return fail(NLM_ERR_INVALID, "null BC / crack array");
  if (int rc0 = check_nofail_regions(*d)) return rc0;
  if (int rc0 = check_bc_functions(*d)) return rc0;
  if (d->precision != NLM_PREC_FP64 && d->precision != NLM_PREC_FP32C)
    return fail(NLM_ERR_INVALID, "unknown precision");
  if (d->scheme != NLM_VELOCITY_VERLET && d->scheme != NLM_CENTRAL_DIFFERENCE)
    return fail(NLM_ERR_INVALID, "unknown scheme");
  if (d->material.kind != NLM_MAT_RNP_BOND && d->material.kind != NLM_MAT_ELASTIC_STATE)
    return fail(NLM_ERR_INVALID, "unknown material");
  const int64_t n = d->n_nodes;
  if (!finite_all(d->x, 3 * n) || !finite_all(d->volume, n))
    return fail(NLM_ERR_NONFINITE, "non-finite coordinate or volume");
  if ((d->u0 && !finite_all(d->u0, 3 * n)) || (d->v0 && !finite_all(d->v0, 3 * n)))
    return fail(NLM_ERR_NONFINITE, "non-finite initial state");
  int dev_count = 0;
  if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0) {
    cudaGetLastError();
    return fail(NLM_ERR_CUDA, "no CUDA device");
  }

  nlm_fd *h = new nlm_fd();
  auto bail = [&](int rc) {
    delete h;
    return rc;
  };
  h->dim = d->dim;
  h->S = d->dim == 2 ? 2 : 4;
  h->n = n;
  h->precision = d->precision;
  h->scheme = d->scheme;
  h->material = d->material.kind;
  h->dt = d->dt;
  StepParams &P = h->P;
  P.n = n;
  P.dim = d->dim;
  P.delta = d->horizon;
  P.h = d->mesh_size;
  P.check_up = d->horizon + 0.5 * d->mesh_size;
  P.check_low = d->horizon - 0.5 * d->mesh_size;
  P.dt = d->dt;
  P.rho = d->material.density;
  P.scheme = d->scheme;
  int rc;
  if (h->material == NLM_MAT_RNP_BOND) {
    if ((rc = rnp_constants(d->material, d->dim, d->horizon, P))) return bail(rc);
    P.contact_rc = 0.9 * d->mesh_size;
  } else {
    const nlm_material &m = d->material;
    if (!(m.K > 0.) || !(m.G > 0.)) return bail(fail(NLM_ERR_INVALID, "ElasticState needs K and G"));
    P.es_K = m.K;
    P.es_mu = m.G;
    P.es_nu = (3 * m.K - 2 * m.G) / (2 * (3 * m.K + m.G));
    P.es_E = m.E;
    P.es_plane_strain = m.plane_strain ? 1 : 0;
    P.es_factor2D = (!m.plane_strain && d->dim == 2) ? (2. * P.es_nu - 1.) / (P.es_nu - 1.) : 1.;
    P.es_sc = m.es_sc;
    P.es_ref_compat = m.es_ref_compat ? 1 : 0;
    P.irrev = 1;
  }
  h->decomp = d->decomposition == NLM_DECOMP_AUTO ? NLM_DECOMP_THREAD : d->decomposition;
  if (h->decomp != NLM_DECOMP_THREAD && h->decomp != NLM_DECOMP_WARP &&
      h->decomp != NLM_DECOMP_THREAD1 && h->decomp != NLM_DECOMP_TILE &&
      h->decomp != NLM_DECOMP_TILE_LOCAL)
    return bail(fail(NLM_ERR_INVALID, "unknown decomposition"));
  // tile store: FP32C 2-D RNPBond (both tile kernels) and FP32C 2-D / 3-D
  // ElasticState (the tile-frame kernels only)
  const bool es_model = d->material.kind == NLM_MAT_ELASTIC_STATE;
  const bool tile_able =
      d->precision == NLM_PREC_FP32C &&
      ((d->material.kind == NLM_MAT_RNP_BOND && d->dim == 2) || (es_model && d->dim >= 2));
  if ((h->decomp == NLM_DECOMP_TILE || h->decomp == NLM_DECOMP_TILE_LOCAL) && !tile_able)
    return bail(fail(NLM_ERR_UNSUPPORTED,
                     "the tile decompositions are for FP32C 2-D RNPBond and 2-D / 3-D "
                     "ElasticState"));
  if (h->decomp == NLM_DECOMP_TILE && es_model)
    return bail(fail(NLM_ERR_UNSUPPORTED, "ElasticState takes NLM_DECOMP_TILE_LOCAL"));
  const bool want_tune = d->decomposition == NLM_DECOMP_AUTO && d->precision == NLM_PREC_FP32C &&
                         (d->material.kind == NLM_MAT_RNP_BOND || es_model);

  cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return bail(cuda_fail(e, "cudaStreamCreate"));
  cudaStream_t s = h->stream;
  const int S = h->S;
#define TRY(call)                                     \
  do {                                                \
    cudaError_t _e = (call);                          \
    if (_e != cudaSuccess) return bail(cuda_fail(_e, #call)); \
  } while (0)

  // ---- neighbours (Morton order) ----
  double *dx = nullptr;
  TRY(h->alloc(&dx, 3 * n));
  TRY(cudaMemcpyAsync(dx, d->x, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s));
  const Grid g = make_grid(d->dim, n, d->x, d->horizon);
  NeighborBuild nb;
  std::string why;
  // FP64 plain keeps the reference's row order (its summation order); the
  // FP32C kernels take rows in internal order so that the k-th neighbours of
  // a warp's nodes sit close together in memory.
  h->rows_by_orig = h->precision == NLM_PREC_FP64;
  e = build_neighbors(nb, d->dim, n, dx, g, S, s, why, h->rows_by_orig);
  for (void *p : {(void *)nb.perm, (void *)nb.pos, (void *)nb.rowptr, (void *)nb.cols})
    if (p) {
      h->allocs.push_back(p);
      h->alloc_sizes.push_back(0);
    }
  if (e != cudaSuccess)
    return bail(why.empty() ? cuda_fail(e, "neighbour build") : fail(NLM_ERR_INVALID, why));
  h->nnz = nb.nnz;
  if (h->nnz > INT32_MAX) return bail(fail(NLM_ERR_INVALID, "too many bonds for one handle"));
  if (tile_able && d->mesh_size > 0.) {
    int rc_l = lattice_relabel(nb, d->dim, S, d->mesh_size, d->horizon, s, h->lattice_res);
    if (rc_l) return bail(rc_l);
  }
  SellStore st;
  e = build_sell(n, nb.rowptr, nb.cols, st, s);
  for (void *p : {(void *)st.ptr, (void *)st.width, (void *)st.cols})
    if (p) {
      h->allocs.push_back(p);
      h->alloc_sizes.push_back(0);
    }
  if (e != cudaSuccess) return bail(cuda_fail(e, "bond store build"));
  h->nslices = st.nslices;
  h->sell_entries = st.entries;
  P.nwords = std::max(1, (st.maxw + 31) / 32);
  P.npad = ((n + 31) / 32) * 32;
  h->perm.resize(n);
  h->rowptr.resize(n + 1);
  TRY(cudaMemcpyAsync(h->perm.data(), nb.perm, sizeof(int) * n, cudaMemcpyDeviceToHost, s));
  TRY(cudaMemcpyAsync(h->rowptr.data(), nb.rowptr, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToHost, s));
  TRY(cudaStreamSynchronize(s));

  DevPtrs &D = h->D;
  D.pos64 = nb.pos;
  D.perm_dev = nb.perm;
  D.rowptr = nb.rowptr;
  D.cols = nb.cols;
  D.sell_ptr = st.ptr;
  D.sell_w = st.width;
  D.sell_cols = st.cols;
  uint32_t *bits = nullptr;
  TRY(h->alloc(&bits, (size_t)P.nwords * P.npad));
  TRY(cudaMemsetAsync(bits, 0, sizeof(uint32_t) * P.nwords * P.npad, s));
  D.bits = bits;
  if (tile_able &&
      (h->decomp == NLM_DECOMP_TILE || h->decomp == NLM_DECOMP_TILE_LOCAL || want_tune)) {
    int rc_t = build_tiles(h, st.ptr, es_model ? kTileMaxLocalES : kTileMaxLocal, d->x);
    if (rc_t) return bail(rc_t);
    if ((h->decomp == NLM_DECOMP_TILE || h->decomp == NLM_DECOMP_TILE_LOCAL) && !h->tile_ok)
      return bail(fail(NLM_ERR_UNSUPPORTED, "a tile's halo exceeds the tile store limit"));
  }
  for (int c = 0; c < d->n_cracks; c++) {
    if (d->cracks[c].kind == NLM_CRACK_EDGE && d->dim != 2)
      return bail(fail(NLM_ERR_INVALID, "edge pre-cracks are 2-D only (input.cpp:298-307)"));
    if (d->cracks[c].timed) {
      if (h->timed_cracks.size() >= 32) return bail(fail(NLM_ERR_INVALID, "more than 32 timed cracks"));
      h->timed_cracks.push_back(d->cracks[c]);
      continue;
    }
    TRY(apply_precrack(n, S, nb.pos, nb.rowptr, nb.cols, d->cracks[c], P.npad, bits, s));
  }

  // ---- node flags, loads (host, original order then permuted) ----
  std::vector<uint8_t> fix(n, 0), interior(n, 1);
  std::vector<int> wset(3 * n, -1);
  std::vector<double> wumax(3 * n, 0.);
  for (int sidx = 0; sidx < d->n_ubc; sidx++) {
    const nlm_bc_set &bc = d->ubc[sidx];
    if (bc.time_fn < 0 || bc.time_fn > NLM_TFN_LINEAR_SLOW_FAST)
      return bail(fail(NLM_ERR_INVALID, "unknown BC time function"));
    for (int64_t i = 0; i < n; i++) {
      if (!in_region(bc, d->x + 3 * i, d->dim)) continue;
      const double um = uload_umax(bc, d->x + 3 * i);
      for (int dd = 0; dd < 3; dd++)
        if (bc.dir_mask >> dd & 1) {
          fix[i] |= uint8_t(1 << dd);
          wset[3 * i + dd] = sidx;
          wumax[3 * i + dd] = um;
        }
    }
    h->T.t[sidx].fn = bc.time_fn;
    for (int k = 0; k < 4; k++) h->T.t[sidx].p[k] = bc.time_params[k];
  }
  h->T.nsets = d->n_ubc;
  if (d->no_fail != NLM_NOFAIL_OFF)
    nofail_flags(d->x, n, d->no_fail_tol, d->n_nofail_regions, d->nofail_regions, interior);
  mesh_bbox(d->x, n, h->bbox_lo, h->bbox_hi);
  // force BC items per node, in set order
  std::vector<std::vector<FBCItem>> fitems(n);
  for (int sidx = 0; sidx < d->n_fbc; sidx++) {
    const nlm_bc_set &bc = d->fbc[sidx];
    for (int64_t i = 0; i < n; i++)
      if (in_region(bc, d->x + 3 * i, d->dim))
        fitems[i].push_back(FBCItem{sidx, bc.dir_mask & 7, fload_spatial(bc, d->x + 3 * i, d->mesh_size)});
    h->FT.t[sidx].fn = bc.time_fn;
    for (int k = 0; k < 4; k++) h->FT.t[sidx].p[k] = bc.time_params[k];
  }
  h->FT.nsets = d->n_fbc;

  std::vector<uint8_t> flags(n);
  std::vector<int> bcref(n, -1), bcn, fnodes, fptr(1, 0);
  std::vector<BCEntry> bce;
  std::vector<FBCItem> fits;
  std::vector<double> volp(n);
  bool any_nofail = false;
  for (int64_t i = 0; i < n; i++) {
    const int o = h->perm[i];
    uint8_t f = fix[o];
    if (!interior[o]) {
      f |= FLAG_NOFAIL;
      any_nofail = true;
    }
    if (!fitems[o].empty()) {
      f |= FLAG_FBC;
      fnodes.push_back((int)i);
      for (auto &it : fitems[o]) fits.push_back(it);
      fptr.push_back((int)fits.size());
    }
    if (fix[o]) {
      BCEntry be;
      for (int dd = 0; dd < 3; dd++) {
        be.set[dd] = wset[3 * o + dd];
        be.umax[dd] = wumax[3 * o + dd];
      }
      bcref[i] = (int)bce.size();
      bce.push_back(be);
      bcn.push_back((int)i);
    }
    flags[i] = f;
    volp[i] = d->volume[o];
  }
  P.nofail = any_nofail ? 1 : 0;
  uint8_t *dflags;
  int *dbcref;
  BCEntry *dbce;
  TRY(h->alloc(&dflags, n));
  TRY(h->alloc(&dbcref, n));
  TRY(h->alloc(&dbce, bce.size() + 1));
  TRY(cudaMemcpyAsync(dflags, flags.data(), n, cudaMemcpyHostToDevice, s));
  TRY(cudaMemcpyAsync(dbcref, bcref.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
  if (!bce.empty())
    TRY(cudaMemcpyAsync(dbce, bce.data(), sizeof(BCEntry) * bce.size(), cudaMemcpyHostToDevice, s));
  D.flags = dflags;
  D.bcref = dbcref;
  D.bce = dbce;
  h->n_bc_nodes = (int64_t)bcn.size();
  TRY(h->alloc(&h->bc_nodes, bcn.size() + 1));
  if (!bcn.empty())
    TRY(cudaMemcpyAsync(h->bc_nodes, bcn.data(), sizeof(int) * bcn.size(), cudaMemcpyHostToDevice, s));
  h->n_fbc_nodes = (int64_t)fnodes.size();
  double *fext;
  TRY(h->alloc(&fext, (size_t)S * n));
  TRY(cudaMemsetAsync(fext, 0, sizeof(double) * S * n, s));
  D.fext = fext;
  if (!fnodes.empty()) {
    TRY(h->alloc(&h->fbc_nodes, fnodes.size()));
    TRY(h->alloc(&h->fbc_iptr, fptr.size()));
    TRY(h->alloc(&h->fbc_items, fits.size()));
    TRY(cudaMemcpyAsync(h->fbc_nodes, fnodes.data(), sizeof(int) * fnodes.size(), cudaMemcpyHostToDevice, s));
    TRY(cudaMemcpyAsync(h->fbc_iptr, fptr.data(), sizeof(int) * fptr.size(), cudaMemcpyHostToDevice, s));
    TRY(cudaMemcpyAsync(h->fbc_items, fits.data(), sizeof(FBCItem) * fits.size(), cudaMemcpyHostToDevice, s));
  }
  double *vol64;
  TRY(h->alloc(&vol64, n));
  TRY(cudaMemcpyAsync(vol64, volp.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s));
  D.vol64 = vol64;
  {
    // row lengths (the kernels loop k < len)
    std::vector<uint16_t> rl(n);
    for (int64_t i = 0; i < n; i++) rl[i] = (uint16_t)(h->rowptr[i + 1] - h->rowptr[i]);
    uint16_t *drl;
    TRY(h->alloc(&drl, n));
    TRY(cudaMemcpyAsync(drl, rl.data(), sizeof(uint16_t) * n, cudaMemcpyHostToDevice, s));
    TRY(cudaStreamSynchronize(s));
    D.rowlen = drl;
  }
  P.nw1 = P.nwords == 1 ? 1 : 0;
  // a common nodal volume (uniform grids) lets the FP32C tile kernel take
  // K1 V as a constant instead of staging it per node
  P.vol_uniform = n > 0 ? d->volume[0] : 0.;
  for (int64_t i = 1; i < n && P.vol_uniform > 0.; i++)
    if (d->volume[i] != d->volume[0]) P.vol_uniform = 0.;
  if (h->precision == NLM_PREC_FP32C) {
    double xmax = 0.;
    for (int64_t k = 0; k < 3 * n; k++) xmax = std::max(xmax, std::fabs(d->x[k]));
    double X = 1.;
    while (X < xmax) X *= 2.;
    while (X * 0.5 >= xmax && X > 1e-30) X *= 0.5;
    P.lo_scale = std::ldexp(1.0, 24) / X;
    float4 *pos32;
    uint2 *pos32lo = nullptr;
    TRY(h->alloc(&pos32, (size_t)n));
    if (S == 4) TRY(h->alloc(&pos32lo, (size_t)n));
    k_make_pos32<<<nblk(n, 256), 256, 0, s>>>(n, S, nb.pos, vol64, P.lo_scale, pos32, pos32lo);
    TRY(cudaGetLastError());
    D.pos32 = pos32;
    D.pos32lo = pos32lo;
  }

  // ---- state ----
  TRY(h->alloc(&h->stage, 9 * n));
  TRY(h->alloc(&h->bad_input, 1));
  if (h->precision == NLM_PREC_FP64) {
    TRY(h->alloc(&D.u64[0], (size_t)S * n));
    TRY(h->alloc(&D.u64[1], (size_t)S * n));
    TRY(h->alloc(&D.f64, (size_t)S * n));
    TRY(cudaMemsetAsync(D.f64, 0, sizeof(double) * S * n, s));
  } else {
    TRY(h->alloc(&D.u32[0], (size_t)(S / 2) * n));
    TRY(h->alloc(&D.u32[1], (size_t)(S / 2) * n));
    TRY(h->alloc(&D.f32, (size_t)S * n));
    TRY(cudaMemsetAsync(D.f32, 0, sizeof(float) * S * n, s));
  }
  if (h->precision == NLM_PREC_FP64) {
    TRY(h->alloc(&D.v[0], (size_t)S * n));
    TRY(h->alloc(&D.v[1], (size_t)S * n));
  } else {
    TRY(h->alloc(&D.v32[0], (size_t)(S / 2) * n));
    TRY(h->alloc(&D.v32[1], (size_t)(S / 2) * n));
  }
  if (h->material == NLM_MAT_ELASTIC_STATE) {
    double *mw;
    TRY(h->alloc(&mw, n));
    TRY(launch_es_setup(P, D, mw, s));
    D.mw64 = mw;
    if (h->precision == NLM_PREC_FP64) {
      TRY(h->alloc(&D.theta64, n));
      TRY(cudaMemsetAsync(D.theta64, 0, sizeof(double) * n, s));
    } else {
      TRY(h->alloc(&D.es_ab, n));
      TRY(cudaMemsetAsync(D.es_ab, 0, sizeof(float2) * n, s));
      float *minv;
      TRY(h->alloc(&minv, n));
      TRY(launch_es_minv32(mw, minv, n, s));
      D.minv32 = minv;
    }
  }
  TRY(h->alloc(&D.err, 1));
  TRY(cudaMemsetAsync(D.err, 0, sizeof(int), s));
  TRY(h->alloc(&h->counter, 1));
  TRY(cudaStreamSynchronize(s));
  h->bytes_per_launch = 0.;
  *out = h;
  rc = nlm_fd_set_state(h, d->u0, d->v0);
  if (rc == NLM_OK && (!d->u0 || !d->v0)) {
    // a NULL initial array means zero
    if (!d->u0) {
      if (h->precision == NLM_PREC_FP64)
        TRY(cudaMemsetAsync(D.u64[0], 0, sizeof(double) * S * n, s));
      else
        TRY(cudaMemsetAsync(D.u32[0], 0, sizeof(float4) * (S / 2) * n, s));
    }
    if (!d->v0) {
      if (h->precision == NLM_PREC_FP64)
        TRY(cudaMemsetAsync(D.v[0], 0, sizeof(double) * S * n, s));
      else
        TRY(cudaMemsetAsync(D.v32[0], 0, sizeof(float4) * (S / 2) * n, s));
    }
    TRY(cudaStreamSynchronize(s));
  }
  if (rc != NLM_OK) {
    *out = nullptr;
    return bail(rc);
  }
  if (want_tune && (rc = autotune(h))) {
    *out = nullptr;
    return bail(rc);
  }
  // algorithmic bytes of one step launch (compulsory traffic model)
  {
    const double per_bond = 4.0 + 0.25;  // int32 column + bond bit read/write
    double per_node;
    if (h->precision == NLM_PREC_FP64)
      per_node = 8.0 * S /*x*/ + 8 /*V*/ + 1 /*flags*/ + 8.0 * S * 2 /*u r,w*/ +
                 8.0 * S * 2 /*v r,w*/ + 8.0 * S * 2 /*f r,w*/;
    else
      per_node = (S == 2 ? 16.0 : 24.0) /*x split + V*/ + 1 /*flags*/ + 2 /*row length*/ +
                 8.0 * S * 2 /*u pair r,w*/ + 8.0 * S * 2 /*v pair r,w*/ + 4.0 * S * 2 /*f r,w*/;
    if (h->material == NLM_MAT_ELASTIC_STATE) per_node += 8.0 * 2;  // theta, m
    h->bytes_per_launch = per_bond * (double)h->nnz + per_node * (double)n;
  }
#undef TRY
  return NLM_OK;
}

int nlm_fd_destroy(nlm_fd *h) {
  delete h;
  return NLM_OK;
}

int nlm_fd_num_bonds(const nlm_fd *h, int64_t *nnz) {
  if (!h || !nnz) return fail(NLM_ERR_INVALID, "null argument");
  *nnz = h->nnz;
  return NLM_OK;
}

int nlm_fd_get_neighbors(nlm_fd *h, int64_t *rowptr, int32_t *cols) {
  if (!h || !rowptr) return fail(NLM_ERR_INVALID, "null argument");
  const int64_t n = h->n;
  std::vector<int64_t> inv(n);
  for (int64_t i = 0; i < n; i++) inv[h->perm[i]] = i;
  rowptr[0] = 0;
  for (int64_t o = 0; o < n; o++) rowptr[o + 1] = rowptr[o] + (h->rowptr[inv[o] + 1] - h->rowptr[inv[o]]);
  if (cols) {
    std::vector<int> cc(h->nnz);
    if (h->nnz)
      NLM_CUDA(cudaMemcpyAsync(cc.data(), h->D.cols, sizeof(int) * h->nnz, cudaMemcpyDeviceToHost, h->stream));
    NLM_CUDA(cudaStreamSynchronize(h->stream));
    for (int64_t o = 0; o < n; o++) {
      const int64_t s0 = h->rowptr[inv[o]], len = h->rowptr[inv[o] + 1] - s0;
      for (int64_t k = 0; k < len; k++) cols[rowptr[o] + k] = h->perm[cc[s0 + k]];
      if (!h->rows_by_orig) std::sort(cols + rowptr[o], cols + rowptr[o] + len);
    }
  }
  return NLM_OK;
}

int nlm_fd_run(nlm_fd *h, int64_t nsteps) {
  if (!h || nsteps < 0) return fail(NLM_ERR_INVALID, "bad arguments");
  return do_run(h, nsteps);
}

int nlm_fd_sync(nlm_fd *h) {
  if (!h) return fail(NLM_ERR_INVALID, "null handle");
  NLM_CUDA(cudaStreamSynchronize(h->stream));
  return NLM_OK;
}

}  // extern "C"

// keep_z: the staging slots of u and v hold the caller's arrays as uploaded
// by the call (nlm_fd_step_host), and their z entries go back unchanged in 2-D.
int get_state_impl(nlm_fd *h, double *u, double *v, double *f, bool keep_z) {
  if (!h) return fail(NLM_ERR_INVALID, "null handle");
  const int64_t n = h->n;
  cudaStream_t s = h->stream;
  const int *P = h->D.perm_dev;
  const unsigned g = nblk(n, 256);
  const bool fp32 = h->precision == NLM_PREC_FP32C;
  // gather each requested field into its own staging slot, copy all out,
  // synchronise once
  double *su = h->stage, *sv = h->stage + 3 * n, *sf = h->stage + 6 * n;
  if (u) {
    if (fp32)
      k_gather_split<<<g, 256, 0, s>>>(n, h->S, P, h->D.u32[h->cur], su, keep_z);
    else
      k_gather_vec<<<g, 256, 0, s>>>(n, h->S, P, h->D.u64[h->cur], su, keep_z);
    NLM_CUDA(cudaGetLastError());
    NLM_CUDA(cudaMemcpyAsync(u, su, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, s));
  }
  if (v) {
    if (fp32)
      k_gather_split<<<g, 256, 0, s>>>(n, h->S, P, h->D.v32[h->vidx()], sv, keep_z);
    else
      k_gather_vec<<<g, 256, 0, s>>>(n, h->S, P, h->D.v[h->vidx()], sv, keep_z);
    NLM_CUDA(cudaGetLastError());
    NLM_CUDA(cudaMemcpyAsync(v, sv, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, s));
  }
  if (f) {
    if (fp32)
      k_gather_f32<<<g, 256, 0, s>>>(n, h->S, P, h->D.f32, sf);
    else
      k_gather_vec<<<g, 256, 0, s>>>(n, h->S, P, h->D.f64, sf);
    NLM_CUDA(cudaGetLastError());
    NLM_CUDA(cudaMemcpyAsync(f, sf, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, s));
  }
  NLM_CUDA(cudaStreamSynchronize(s));
  return NLM_OK;
}

extern "C" {

int nlm_fd_get_state(nlm_fd *h, double *u, double *v, double *f) {
  return get_state_impl(h, u, v, f, false);
}

int nlm_fd_set_state(nlm_fd *h, const double *u, const double *v) {
  if (!h) return fail(NLM_ERR_INVALID, "null handle");
  const int64_t n = h->n;
  if ((u && !finite_all(u, 3 * n)) || (v && !finite_all(v, 3 * n)))
    return fail(NLM_ERR_NONFINITE, "non-finite state");
  cudaStream_t s = h->stream;
  const int *P = h->D.perm_dev;
  const unsigned g = nblk(n, 256);
  if (u) {
    NLM_CUDA(cudaMemcpyAsync(h->stage, u, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s));
    if (h->precision == NLM_PREC_FP32C)
      k_scatter_split<<<g, 256, 0, s>>>(n, h->S, h->dim, P, h->stage, h->D.u32[h->cur]);
    else
      k_scatter_vec<<<g, 256, 0, s>>>(n, h->S, h->dim, P, h->stage, h->D.u64[h->cur]);
    NLM_CUDA(cudaGetLastError());
  }
  if (v) {
    double *sv = h->stage + 3 * n;
    NLM_CUDA(cudaMemcpyAsync(sv, v, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s));
    if (h->precision == NLM_PREC_FP32C)
      k_scatter_split<<<g, 256, 0, s>>>(n, h->S, h->dim, P, sv, h->D.v32[h->vidx()]);
    else
      k_scatter_vec<<<g, 256, 0, s>>>(n, h->S, h->dim, P, sv, h->D.v[h->vidx()]);
    NLM_CUDA(cudaGetLastError());
  }
  NLM_CUDA(cudaStreamSynchronize(s));
  if (h->started && (u || v)) {
    // a new state restarts the force history: redo the step-0 evaluation
    h->started = false;
  }
  return NLM_OK;
}

int nlm_fd_get_time(const nlm_fd *h, double *time, int64_t *step) {
  if (!h) return fail(NLM_ERR_INVALID, "null handle");
  if (time) *time = h->time;
  if (step) *step = h->step;
  return NLM_OK;
}

int nlm_fd_get_bond_state(nlm_fd *h, uint8_t *broken) {
  if (!h || !broken) return fail(NLM_ERR_INVALID, "null argument");
  const int64_t n = h->n;
  std::vector<uint32_t> bits((size_t)h->P.nwords * h->P.npad);
  NLM_CUDA(cudaMemcpyAsync(bits.data(), h->D.bits, sizeof(uint32_t) * bits.size(), cudaMemcpyDeviceToHost, h->stream));
  std::vector<int> cc;
  if (!h->rows_by_orig) {
    cc.resize(h->nnz);
    if (h->nnz)
      NLM_CUDA(cudaMemcpyAsync(cc.data(), h->D.cols, sizeof(int) * h->nnz, cudaMemcpyDeviceToHost, h->stream));
  }
  NLM_CUDA(cudaStreamSynchronize(h->stream));
  std::vector<int64_t> inv(n);
  for (int64_t i = 0; i < n; i++) inv[h->perm[i]] = i;
  int64_t o_off = 0;
  std::vector<std::pair<int, uint8_t>> row;
  for (int64_t o = 0; o < n; o++) {
    const int64_t i = inv[o];
    const int64_t r0 = h->rowptr[i], len = h->rowptr[i + 1] - r0;
    if (h->rows_by_orig) {
      for (int64_t k = 0; k < len; k++)
        broken[o_off + k] = (bits[(size_t)(k >> 5) * h->P.npad + i] >> (k & 31)) & 1u;
    } else {
      // device rows are in internal order: re-sort by original id
      row.resize(len);
      for (int64_t k = 0; k < len; k++)
        row[k] = {h->perm[cc[r0 + k]],
                  (uint8_t)((bits[(size_t)(k >> 5) * h->P.npad + i] >> (k & 31)) & 1u)};
      std::sort(row.begin(), row.end());
      for (int64_t k = 0; k < len; k++) broken[o_off + k] = row[k].second;
    }
    o_off += len;
  }
  return NLM_OK;
}

int nlm_fd_set_bond_state(nlm_fd *h, const uint8_t *broken) {
  if (!h || !broken) return fail(NLM_ERR_INVALID, "null argument");
  const int64_t n = h->n;
  std::vector<uint32_t> bits((size_t)h->P.nwords * h->P.npad, 0u);
  std::vector<int> cc;
  if (!h->rows_by_orig) {
    cc.resize(h->nnz);
    if (h->nnz)
      NLM_CUDA(cudaMemcpyAsync(cc.data(), h->D.cols, sizeof(int) * h->nnz, cudaMemcpyDeviceToHost,
                               h->stream));
    NLM_CUDA(cudaStreamSynchronize(h->stream));
  }
  std::vector<int64_t> inv(n);
  for (int64_t i = 0; i < n; i++) inv[h->perm[i]] = i;
  int64_t o_off = 0;
  std::vector<std::pair<int, int>> row;
  for (int64_t o = 0; o < n; o++) {
    const int64_t i = inv[o];
    const int64_t r0 = h->rowptr[i], len = h->rowptr[i + 1] - r0;
    if (h->rows_by_orig) {
      for (int64_t k = 0; k < len; k++)
        if (broken[o_off + k]) bits[(size_t)(k >> 5) * h->P.npad + i] |= 1u << (k & 31);
    } else {
      // external order is ascending original id; device slot k holds cc[r0 + k]
      row.resize(len);
      for (int64_t k = 0; k < len; k++) row[k] = {h->perm[cc[r0 + k]], (int)k};
      std::sort(row.begin(), row.end());
      for (int64_t e = 0; e < len; e++)
        if (broken[o_off + e]) {
          const int k = row[e].second;
          bits[(size_t)(k >> 5) * h->P.npad + i] |= 1u << (k & 31);
        }
    }
    o_off += len;
  }
  NLM_CUDA(cudaMemcpyAsync(h->D.bits, bits.data(), sizeof(uint32_t) * bits.size(),
                           cudaMemcpyHostToDevice, h->stream));
  NLM_CUDA(cudaStreamSynchronize(h->stream));
  return NLM_OK;
}

namespace {
struct CkptHeader {
  char magic[8];
  int32_t version, dim, precision, material, started;
  uint32_t cracks_on;  // timed cracks already cut (bit c = crack c)
  int64_t n, nnz, step;
  double time, dt;
};
const char kCkptMagic[8] = {'N', 'L', 'M', 'C', 'K', 'P', 'T', 0};
}  // namespace

int nlm_fd_save(nlm_fd *h, const char *path) {
  if (!h || !path) return fail(NLM_ERR_INVALID, "null argument");
  const int64_t n = h->n;
  std::vector<double> st((size_t)9 * n);
  std::vector<uint8_t> b((size_t)h->nnz);
  int rc = nlm_fd_get_state(h, st.data(), st.data() + 3 * n, st.data() + 6 * n);
  if (rc) return rc;
  if ((rc = nlm_fd_get_bond_state(h, b.data()))) return rc;
  CkptHeader hd{};
  std::memcpy(hd.magic, kCkptMagic, 8);
  hd.version = 1;
  hd.dim = h->dim;
  hd.precision = h->precision;
  hd.material = h->material;
  hd.started = h->started ? 1 : 0;
  hd.cracks_on = h->cracks_on;
  hd.n = n;
  hd.nnz = h->nnz;
  hd.step = h->step;
  hd.time = h->time;
  hd.dt = h->dt;
  FILE *fp = std::fopen(path, "wb");
  if (!fp) return fail(NLM_ERR_INVALID, std::string("cannot write ") + path);
  bool ok = std::fwrite(&hd, sizeof(hd), 1, fp) == 1 &&
            std::fwrite(st.data(), sizeof(double), st.size(), fp) == st.size() &&
            std::fwrite(b.data(), 1, b.size(), fp) == b.size();
  ok = (std::fclose(fp) == 0) && ok;
  if (!ok) return fail(NLM_ERR_INVALID, std::string("short write to ") + path);
  return NLM_OK;
}

int nlm_fd_load(nlm_fd *h, const char *path) {
  if (!h || !path) return fail(NLM_ERR_INVALID, "null argument");
  FILE *fp = std::fopen(path, "rb");
  if (!fp) return fail(NLM_ERR_INVALID, std::string("cannot read ") + path);
  CkptHeader hd{};
  const int64_t n = h->n;
  std::vector<double> st((size_t)9 * n);
  std::vector<uint8_t> b((size_t)h->nnz);
  bool ok = std::fread(&hd, sizeof(hd), 1, fp) == 1 && std::memcmp(hd.magic, kCkptMagic, 8) == 0;
  if (ok && (hd.version != 1 || hd.n != n || hd.nnz != h->nnz || hd.dim != h->dim ||
             hd.material != h->material || hd.dt != h->dt ||
             (uint64_t)hd.cracks_on >= (1ull << h->timed_cracks.size()))) {
    std::fclose(fp);
    return fail(NLM_ERR_INVALID,
                "checkpoint does not match this model (n, bonds, dim, material, dt, timed cracks)");
  }
  ok = ok && std::fread(st.data(), sizeof(double), st.size(), fp) == st.size() &&
       std::fread(b.data(), 1, b.size(), fp) == b.size();
  std::fclose(fp);
  if (!ok) return fail(NLM_ERR_INVALID, std::string("not a complete checkpoint: ") + path);
  // everything that can be checked is checked before the handle changes
  if (!finite_all(st.data(), (int64_t)st.size()) || !std::isfinite(hd.time) || hd.step < 0)
    return fail(NLM_ERR_NONFINITE, std::string("checkpoint holds a non-finite state or time: ") +
                                       path);
  // what a later failure puts back
  std::vector<uint8_t> bits0((size_t)h->nnz);
  int rc = nlm_fd_get_bond_state(h, bits0.data());
  if (rc) return rc;
  const double time0 = h->time;
  const int64_t step0 = h->step;
  const uint32_t cracks0 = h->cracks_on;
  const bool started0 = h->started;
  rc = nlm_fd_set_bond_state(h, b.data());
  if (rc == NLM_OK) {
    h->time = hd.time;
    h->step = hd.step;
    h->cracks_on = hd.cracks_on;
    if (!hd.started) {
      h->started = false;
      rc = nlm_fd_set_state(h, st.data(), st.data() + 3 * n);
    } else {
      // a started run: u^m, v^m and f^m as step_host takes them, then the
      // drift to u^{m+1} that the interrupted step had done
      h->started = true;
      rc = nlm_fd_step_host(h, st.data(), st.data() + 3 * n, st.data() + 6 * n, 0);
    }
  }
  if (rc != NLM_OK) {
    const std::string msg = nlm_last_error();
    h->time = time0;
    h->step = step0;
    h->cracks_on = cracks0;
    h->started = started0;
    nlm_fd_set_bond_state(h, bits0.data());
    set_error(msg);
  }
  return rc;
}

int nlm_fd_set_time(nlm_fd *h, double time, int64_t step) {
  if (!h || step < 0 || !std::isfinite(time)) return fail(NLM_ERR_INVALID, "bad arguments");
  if (h->started) return fail(NLM_ERR_STATE, "the run has started");
  h->time = time;
  h->step = step;
  return NLM_OK;
}

int nlm_fd_get_fixity(nlm_fd *h, uint8_t *fixity) {
  if (!h || !fixity) return fail(NLM_ERR_INVALID, "null argument");
  std::vector<uint8_t> fl(h->n);
  if (h->n)
    NLM_CUDA(cudaMemcpyAsync(fl.data(), h->D.flags, h->n, cudaMemcpyDeviceToHost, h->stream));
  NLM_CUDA(cudaStreamSynchronize(h->stream));
  for (int64_t i = 0; i < h->n; i++) fixity[h->perm[i]] = fl[i] & 7u;
  return NLM_OK;
}

int nlm_fd_count_broken(nlm_fd *h, int64_t *count) {
  if (!h || !count) return fail(NLM_ERR_INVALID, "null argument");
  NLM_CUDA(cudaMemsetAsync(h->counter, 0, sizeof(unsigned long long), h->stream));
  k_count_bits<<<nblk(h->n, 256), 256, 0, h->stream>>>(h->n, h->P.nwords, h->P.npad, h->D.bits, h->counter);
  NLM_CUDA(cudaGetLastError());
  unsigned long long c = 0;
  NLM_CUDA(cudaMemcpyAsync(&c, h->counter, sizeof(c), cudaMemcpyDeviceToHost, h->stream));
  NLM_CUDA(cudaStreamSynchronize(h->stream));
  *count = (int64_t)c;
  return NLM_OK;
}

int nlm_fd_damage(nlm_fd *h, float *phi, float *Z) {
  if (!h) return fail(NLM_ERR_INVALID, "null handle");
  const int64_t n = h->n;
  cudaStream_t s = h->stream;
  if (!h->dmg_phi) {
    if (h->alloc(&h->dmg_phi, n) != cudaSuccess || h->alloc(&h->dmg_Z, n) != cudaSuccess)
      return fail(NLM_ERR_OOM, "damage buffers");
  }
  cudaError_t e = launch_damage(h->P, h->D, h->cur, h->precision == NLM_PREC_FP32C,
                                h->material == NLM_MAT_ELASTIC_STATE, h->dmg_phi, h->dmg_Z, s);
  if (e != cudaSuccess) return cuda_fail(e, "damage kernel");
  std::vector<float> a(n), b(n);
  NLM_CUDA(cudaMemcpyAsync(a.data(), h->dmg_phi, sizeof(float) * n, cudaMemcpyDeviceToHost, s));
  NLM_CUDA(cudaMemcpyAsync(b.data(), h->dmg_Z, sizeof(float) * n, cudaMemcpyDeviceToHost, s));
  NLM_CUDA(cudaStreamSynchronize(s));
  for (int64_t i = 0; i < n; i++) {
    if (phi) phi[h->perm[i]] = a[i];
    if (Z) Z[h->perm[i]] = b[i];
  }
  return NLM_OK;
}

int nlm_fd_energies(nlm_fd *h, float *strain, float *work, float *kinetic, float *fracture,
                    double *totals) {
  if (!h) return fail(NLM_ERR_INVALID, "null handle");
  if (h->material != NLM_MAT_RNP_BOND) return fail(NLM_ERR_UNSUPPORTED, "energies are for RNPBond");
  const int64_t n = h->n;
  cudaStream_t s = h->stream;
  if (!h->en_buf) {
    if (h->alloc(&h->en_buf, (size_t)4 * n) != cudaSuccess ||
        h->alloc(&h->en_fext, (size_t)h->S * n) != cudaSuccess)
      return fail(NLM_ERR_OOM, "energy buffers");
  }
  // f_ext at the current time, as computePostProcFields evaluates it
  NLM_CUDA(cudaMemsetAsync(h->en_fext, 0, sizeof(double) * h->S * n, s));
  if (h->n_fbc_nodes > 0) {
    k_fbc_apply<<<nblk(h->n_fbc_nodes, 128), 128, 0, s>>>(h->n_fbc_nodes, h->S, h->fbc_nodes,
                                                          h->fbc_iptr, h->fbc_items, h->FT,
                                                          h->time, h->en_fext);
    NLM_CUDA(cudaGetLastError());
  }
  float *e4 = h->en_buf;
  cudaError_t e = launch_energy(h->P, h->D, h->cur, h->vidx(), h->precision == NLM_PREC_FP32C,
                                h->en_fext, e4, e4 + n, e4 + 2 * n, e4 + 3 * n, s);
  if (e != cudaSuccess) return cuda_fail(e, "energy kernel");
  std::vector<float> a((size_t)4 * n);
  NLM_CUDA(cudaMemcpyAsync(a.data(), e4, sizeof(float) * 4 * n, cudaMemcpyDeviceToHost, s));
  NLM_CUDA(cudaStreamSynchronize(s));
  float *out[4] = {strain, work, kinetic, fracture};
  double tot[4] = {0., 0., 0., 0.};
  for (int q = 0; q < 4; q++)
    for (int64_t i = 0; i < n; i++) {
      const float v = a[(size_t)q * n + i];
      tot[q] += v;
      if (out[q]) out[q][h->perm[i]] = v;
    }
  if (totals)
    for (int q = 0; q < 4; q++) totals[q] = tot[q];
  return NLM_OK;
}

int nlm_fd_reaction_force(nlm_fd *h, double *reaction, double *total, double *sum) {
  if (!h) return fail(NLM_ERR_INVALID, "null handle");
  if (h->material != NLM_MAT_RNP_BOND || h->dim != 2)
    return fail(NLM_ERR_UNSUPPORTED, "the reaction force is for 2-D RNPBond");
  const int64_t n = h->n;
  cudaStream_t s = h->stream;
  if (!h->rf_buf && h->alloc(&h->rf_buf, (size_t)2 * n) != cudaSuccess)
    return fail(NLM_ERR_OOM, "reaction-force buffer");
  cudaError_t e = launch_reaction(h->P, h->D, h->cur, h->precision == NLM_PREC_FP32C,
                                  h->bbox_lo[0], h->bbox_hi[0], h->bbox_hi[1], h->rf_buf, s);
  if (e != cudaSuccess) return cuda_fail(e, "reaction-force kernel");
  std::vector<double> a((size_t)2 * n);
  NLM_CUDA(cudaMemcpyAsync(a.data(), h->rf_buf, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost, s));
  NLM_CUDA(cudaStreamSynchronize(s));
  double tot[3] = {0., 0., 0.};
  for (int64_t i = 0; i < n; i++) {
    const double rx = a[2 * i], ry = a[2 * i + 1];
    const int64_t o = h->perm[i];
    if (reaction) {
      reaction[3 * o] = rx;
      reaction[3 * o + 1] = ry;
      reaction[3 * o + 2] = 0.;
    }
    if (total) total[o] = std::sqrt(rx * rx + ry * ry + 0. * 0.);
    tot[0] += rx;
    tot[1] += ry;
  }
  if (sum)
    for (int c = 0; c < 3; c++) sum[c] = tot[c];
  return NLM_OK;
}

int nlm_fd_decomposition(const nlm_fd *h, int *decomp) {
  if (!h || !decomp) return fail(NLM_ERR_INVALID, "null argument");
  *decomp = h->decomp;
  return NLM_OK;
}

int nlm_fd_set_timing(nlm_fd *h, int enable) {
  if (!h) return fail(NLM_ERR_INVALID, "null handle");
  h->timing = enable != 0;
  return NLM_OK;
}

int nlm_fd_kernel_stats(nlm_fd *h, int reset, double *avg_ms, int64_t *launches,
                        double *bytes_per_launch) {
  if (!h) return fail(NLM_ERR_INVALID, "null handle");
  NLM_CUDA(cudaStreamSynchronize(h->stream));
  double acc = 0.;
  for (size_t k = 0; k + 1 < h->ev_used; k += 2) {
    float ms = 0.f;
    NLM_CUDA(cudaEventElapsedTime(&ms, h->ev_pool[k], h->ev_pool[k + 1]));
    acc += ms;
  }
  const int64_t L = h->launches;
  if (avg_ms) *avg_ms = L ? acc / (double)L : 0.;
  if (launches) *launches = L;
  if (bytes_per_launch) *bytes_per_launch = h->bytes_per_launch;
  if (reset) {
    h->ev_used = 0;
    h->launches = 0;
  }
  return NLM_OK;
}

}  // extern "C"

