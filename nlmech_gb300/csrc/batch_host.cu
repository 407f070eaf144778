// batch_host.cu -- nlm_batch_*: many RNPBond specimens stepped together.

#include "fd_handle.h"
#include "tile_store.h"

// ===========================================================================
// Batched specimens.
//
// Specimen s occupies internal nodes [off_s, off_s + n_s) with off_s a
// multiple of 32, so every 32-node slice of the bond store belongs to one
// specimen; the gaps are ghost nodes (FLAG_GHOST, no bonds) that the kernels
// skip.  Neighbour lists, pre-cracks and loads are built per specimen with the
// single-model code, so they are identical to those of a separate nlm_fd.
// Specimens are laid out by ascending node count and cut into up to three
// node-count buckets; each bucket is one launch per step with its own
// autotuned decomposition.

struct nlm_batch {
  int nspec = 0, dim = 2, S = 2, scheme = NLM_VELOCITY_VERLET;
  int64_t ntot = 0, nnz = 0;
  double dt = 0., time = 0.;
  int64_t step = 0;
  bool started = false;
  int cur = 0;
  StepParams P{};
  BCTable T{};
  DevPtrs D{};
  cudaStream_t stream = nullptr;
  std::vector<void *> allocs;
  std::vector<int64_t> off, n, bond_off, nbond;  // per specimen, by input id
  std::vector<int> order;                          // layout position -> input id
  std::vector<std::vector<int>> perm;              // per specimen: internal -> original
  std::vector<int64_t> rowptr;                     // combined CSR offsets (host)
  struct Bucket {
    int64_t i0, i1;
    int decomp;
  };
  std::vector<Bucket> buckets;
  bool tile_ok = false;  // tile store over the combined layout (2-D)
  int *bc_nodes = nullptr;
  int64_t n_bc_nodes = 0;
  double *stage = nullptr;
  // graphs
  int graph_steps = 0;
  cudaGraphExec_t gexec[2] = {nullptr, nullptr};
  double *d_times = nullptr, *h_times = nullptr;
  cudaEvent_t ev_times = nullptr;

  template <class Tp>
  cudaError_t alloc(Tp **p, size_t count) {
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, count * sizeof(Tp) + 16);
    if (e == cudaSuccess) {
      allocs.push_back(q);
      *p = static_cast<Tp *>(q);
    }
    return e;
  }
  ~nlm_batch() {
    if (stream) cudaStreamSynchronize(stream);
    for (auto &g : gexec)
      if (g) cudaGraphExecDestroy(g);
    if (h_times) cudaFreeHost(h_times);
    if (ev_times) cudaEventDestroy(ev_times);
    for (void *p : allocs) cudaFree(p);
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace {

int batch_launch(nlm_batch *b, StepArgs a) {
  // after the step-0 evaluation a step follows another step or a kernel that
  // writes only state: the tile-frame kernel may overlap it
  a.pdl = !a.first;
  // every bucket on the tile-frame kernel: one launch over all of them (its
  // tiles take each node's own specimen constants, and a tile that straddles
  // two buckets is staged once instead of once per bucket)
  bool all_tile = !b->buckets.empty();
  for (const auto &bk : b->buckets) all_tile = all_tile && bk.decomp == NLM_DECOMP_TILE_LOCAL;
  if (all_tile) {
    a.i0 = b->buckets.front().i0;
    a.i1 = b->buckets.back().i1;
    cudaError_t e = launch_rnp_step_fp32(b->P, b->D, b->T, a, NLM_DECOMP_TILE_LOCAL, b->stream);
    return e == cudaSuccess ? NLM_OK : cuda_fail(e, "batched step launch");
  }
  for (const auto &bk : b->buckets) {
    a.i0 = bk.i0;
    a.i1 = bk.i1;
    cudaError_t e = launch_rnp_step_fp32(b->P, b->D, b->T, a, bk.decomp, b->stream);
    if (e != cudaSuccess) return cuda_fail(e, "batched step launch");
  }
  return NLM_OK;
}

int batch_apply_bc(nlm_batch *b, double t) {
  if (b->n_bc_nodes == 0) return NLM_OK;
  k_bc_apply<<<nblk(b->n_bc_nodes, 128), 128, 0, b->stream>>>(
      b->n_bc_nodes, b->S, b->dim, b->bc_nodes, b->D.bcref, b->D.bce, b->D.flags, b->T, t,
      nullptr, b->D.u32[b->cur], nullptr, b->D.v32[b->scheme == NLM_CENTRAL_DIFFERENCE ? b->cur : 0]);
  NLM_CUDA(cudaGetLastError());
  return NLM_OK;
}

// k_bc_apply reads set tables from its BCTable argument; the batch keeps them
// in device memory (D.bct), so the prologue uses this variant.
__global__ void k_bc_apply_tab(int64_t nb, int S, int dim, const int *nodes, const int *bcref,
                               const BCEntry *bce, const uint8_t *flags, const BCTime *tab,
                               double time, float4 *u32, float4 *v32) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nb) return;
  const int64_t i = nodes[t];
  const BCEntry e = bce[bcref[i]];
  const uint8_t fl = flags[i];
  double uo[3], vo[3];
  ld_split_any(u32, S, i, uo);
  ld_split_any(v32, S, i, vo);
  for (int d = 0; d < dim; d++)
    if ((fl >> d & 1) && e.set[d] >= 0) {
      double du, dv;
      bc_value(tab[e.set[d]], e.umax[d], time, du, dv);
      uo[d] = du;
      vo[d] = dv;
    }
  st_split_any(u32, S, i, uo);
  st_split_any(v32, S, i, vo);
}

int batch_capture(nlm_batch *b, int c0) {
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamBeginCapture");
  int c = c0, rc = NLM_OK;
  for (int k = 0; k < b->graph_steps && rc == NLM_OK; k++) {
    c = 1 - c;
    rc = batch_launch(b, StepArgs{c, false, 0., 0., b->d_times + k, 0, 0});
  }
  e = cudaStreamEndCapture(b->stream, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
  e = cudaGraphInstantiate(&b->gexec[c0], g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
  return NLM_OK;
}

int batch_run(nlm_batch *b, int64_t nsteps) {
  if (!b->started) {
    if (b->n_bc_nodes) {
      k_bc_apply_tab<<<nblk(b->n_bc_nodes, 128), 128, 0, b->stream>>>(
          b->n_bc_nodes, b->S, b->dim, b->bc_nodes, b->D.bcref, b->D.bce, b->D.flags, b->D.bct,
          b->time, b->D.u32[b->cur], b->D.v32[b->scheme == NLM_CENTRAL_DIFFERENCE ? b->cur : 0]);
      NLM_CUDA(cudaGetLastError());
    }
    int rc = batch_launch(b, StepArgs{b->cur, true, b->time, b->time + b->dt, nullptr, 0, 0});
    if (rc) return rc;
    b->started = true;
  }
  const int G = b->graph_steps;
  while (G > 0 && nsteps >= G) {
    if (!b->gexec[b->cur]) {
      int rc = batch_capture(b, b->cur);
      if (rc) return rc;
    }
    NLM_CUDA(cudaEventSynchronize(b->ev_times));
    double t = b->time;
    for (int k = 0; k <= G; k++) {
      t = t + b->dt;
      b->h_times[k] = t;
    }
    NLM_CUDA(cudaMemcpyAsync(b->d_times, b->h_times, sizeof(double) * (G + 1),
                             cudaMemcpyHostToDevice, b->stream));
    NLM_CUDA(cudaEventRecord(b->ev_times, b->stream));
    NLM_CUDA(cudaGraphLaunch(b->gexec[b->cur], b->stream));
    b->time = b->h_times[G - 1];
    b->step += G;
    nsteps -= G;
  }
  for (int64_t k = 0; k < nsteps; k++) {
    const double tm = b->time + b->dt;
    b->cur = 1 - b->cur;
    int rc = batch_launch(b, StepArgs{b->cur, false, tm, tm + b->dt, nullptr, 0, 0});
    if (rc) return rc;
    b->time = tm;
    b->step++;
  }
  return NLM_OK;
}

}  // namespace

extern "C" {

int nlm_batch_create(const nlm_fd_desc *descs, int nspec, nlm_batch **out) {
  if (!descs || !out || nspec < 1) return fail(NLM_ERR_INVALID, "bad arguments");
  *out = nullptr;
  const nlm_fd_desc &d0 = descs[0];
  int64_t total_sets = 0;
  for (int s = 0; s < nspec; s++) {
    const nlm_fd_desc &d = descs[s];
    if (d.dim != d0.dim || (d.dim != 2 && d.dim != 3))
      return fail(NLM_ERR_INVALID, "specimens must share dimension 2 or 3");
    if (d.precision != NLM_PREC_FP32C)
      return fail(NLM_ERR_UNSUPPORTED, "batched specimens run in FP32C precision");
    if (d.material.kind != NLM_MAT_RNP_BOND)
      return fail(NLM_ERR_UNSUPPORTED, "batched specimens are RNPBond");
    if (d.dt != d0.dt || d.scheme != d0.scheme)
      return fail(NLM_ERR_INVALID, "specimens must share dt and scheme");
    if (d.n_fbc) return fail(NLM_ERR_UNSUPPORTED, "Force_BC in a batch");
    if (d.n_nodes <= 0 || !d.x || !d.volume) return fail(NLM_ERR_INVALID, "empty specimen");
    if (!(d.horizon > 0.) || !(d.mesh_size > 0.) || !(d.dt > 0.) || !(d.material.density > 0.))
      return fail(NLM_ERR_INVALID, "horizon, mesh size, dt and density must be positive");
    if (d.n_ubc < 0 || d.n_ubc > kMaxBCSets || (d.n_ubc && !d.ubc) || (d.n_cracks && !d.cracks))
      return fail(NLM_ERR_INVALID, "bad BC / crack arrays");
    if (int rc0 = check_nofail_regions(d)) return rc0;
    if (!finite_all(d.x, 3 * d.n_nodes) || !finite_all(d.volume, d.n_nodes))
      return fail(NLM_ERR_NONFINITE, "non-finite coordinate or volume");
    total_sets += d.n_ubc;
  }
  int dev_count = 0;
  if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0) {
    cudaGetLastError();
    return fail(NLM_ERR_CUDA, "no CUDA device");
  }
  nlm_batch *b = new nlm_batch();
  auto bail = [&](int rc) {
    delete b;
    return rc;
  };
#define BTRY(call)                                              \
  do {                                                          \
    cudaError_t _e = (call);                                    \
    if (_e != cudaSuccess) return bail(cuda_fail(_e, #call));   \
  } while (0)
  b->nspec = nspec;
  b->dim = d0.dim;
  b->S = d0.dim == 2 ? 2 : 4;
  b->scheme = d0.scheme;
  b->dt = d0.dt;
  const int S = b->S;
  BTRY(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  cudaStream_t st = b->stream;
  // layout: ascending node count
  b->order.resize(nspec);
  for (int s = 0; s < nspec; s++) b->order[s] = s;
  std::stable_sort(b->order.begin(), b->order.end(),
                   [&](int a, int c) { return descs[a].n_nodes < descs[c].n_nodes; });
  b->off.assign(nspec, 0);
  b->n.assign(nspec, 0);
  // the decomposition (explicit when every specimen names the same one)
  int fixed = descs[0].decomposition;
  for (int s = 1; s < nspec; s++)
    if (descs[s].decomposition != fixed) fixed = NLM_DECOMP_AUTO;
  const bool tiles_possible =
      d0.dim == 2 && (fixed == NLM_DECOMP_AUTO || fixed == NLM_DECOMP_TILE_LOCAL);
  // Specimens start at slice boundaries (32 nodes), or at tile boundaries
  // (256) when the tile-frame kernel may run, so that a specimen's lattice
  // patches are whole tiles.
  const int64_t align = tiles_possible ? kTileNodes : 32;
  int64_t cursor = 0;
  for (int k = 0; k < nspec; k++) {
    const int s = b->order[k];
    b->off[s] = cursor;
    b->n[s] = descs[s].n_nodes;
    cursor += ((descs[s].n_nodes + align - 1) / align) * align;
  }
  const int64_t N = cursor;
  b->ntot = N;
  if (N > INT32_MAX - 64) return bail(fail(NLM_ERR_INVALID, "too many nodes"));
  // per-specimen neighbour builds, merged into one CSR
  double *pos64;
  int64_t *rowptr;
  BTRY(b->alloc(&pos64, (size_t)S * N));
  BTRY(cudaMemsetAsync(pos64, 0, sizeof(double) * S * N, st));
  BTRY(b->alloc(&rowptr, N + 1));
  std::vector<int64_t> hrow(N + 1, 0);
  std::vector<NeighborBuild> nbs(nspec);
  std::vector<uint8_t> lres;  // lattice residues (combined layout), if relabelled
  bool relabel_all = true;    // the residue layout of the halo needs every specimen's
  b->perm.resize(nspec);
  b->bond_off.assign(nspec, 0);
  b->nbond.assign(nspec, 0);
  double xmax = 0.;
  int64_t nnz = 0;
  std::vector<double> posh, rint;
  double hmin = 1e300;
  for (int k = 0; k < nspec; k++) {
    const int s = b->order[k];
    const nlm_fd_desc &d = descs[s];
    double *dx = nullptr;
    cudaError_t e = cudaMalloc(&dx, sizeof(double) * 3 * (d.n_nodes + 1));
    if (e == cudaSuccess) e = cudaMemcpyAsync(dx, d.x, sizeof(double) * 3 * d.n_nodes, cudaMemcpyHostToDevice, st);
    std::string why;
    const Grid g = make_grid(d.dim, d.n_nodes, d.x, d.horizon);
    if (e == cudaSuccess) e = build_neighbors(nbs[s], d.dim, d.n_nodes, dx, g, S, st, why, false);
    cudaFree(dx);
    for (void *q : {(void *)nbs[s].perm, (void *)nbs[s].pos, (void *)nbs[s].rowptr, (void *)nbs[s].cols})
      if (q) b->allocs.push_back(q);
    if (e != cudaSuccess)
      return bail(why.empty() ? cuda_fail(e, "neighbour build") : fail(NLM_ERR_INVALID, why));
    if (tiles_possible && !(d.mesh_size > 0.)) relabel_all = false;
    if (tiles_possible && d.mesh_size > 0.) {
      // each specimen on its own mesh lattice, as a single model's tiles
      std::vector<uint8_t> lr;
      if (int rc_l = lattice_relabel(nbs[s], d.dim, S, d.mesh_size, d.horizon, st, lr))
        return bail(rc_l);
      if (lres.empty()) lres.assign(N, 0);
      std::copy(lr.begin(), lr.end(), lres.begin() + b->off[s]);
    }
    b->perm[s].resize(d.n_nodes);
    std::vector<int64_t> rp(d.n_nodes + 1);
    BTRY(cudaMemcpyAsync(b->perm[s].data(), nbs[s].perm, sizeof(int) * d.n_nodes, cudaMemcpyDeviceToHost, st));
    BTRY(cudaMemcpyAsync(rp.data(), nbs[s].rowptr, sizeof(int64_t) * (d.n_nodes + 1), cudaMemcpyDeviceToHost, st));
    BTRY(cudaStreamSynchronize(st));
    b->bond_off[s] = nnz;
    b->nbond[s] = nbs[s].nnz;
    for (int64_t i = 0; i < d.n_nodes; i++) hrow[b->off[s] + i] = nnz + rp[i];
    const int64_t pad_end = (k + 1 < nspec) ? b->off[b->order[k + 1]] : N;
    for (int64_t i = b->off[s] + d.n_nodes; i <= pad_end && i <= N; i++) hrow[i] = nnz + nbs[s].nnz;
    nnz += nbs[s].nnz;
    BTRY(cudaMemcpyAsync(pos64 + (size_t)S * b->off[s], nbs[s].pos, sizeof(double) * S * d.n_nodes,
                         cudaMemcpyDeviceToDevice, st));
    if (tiles_possible) {
      // internal-order positions and the interior radius per node (constant
      // influence functions only), for the rows' interior prefixes
      if (posh.empty()) {
        posh.assign((size_t)S * N, 0.);
        rint.assign(N, 0.);
      }
      BTRY(cudaMemcpyAsync(posh.data() + (size_t)S * b->off[s], nbs[s].pos,
                           sizeof(double) * S * d.n_nodes, cudaMemcpyDeviceToHost, st));
      if (d.material.influence_type == 0 && d.mesh_size > 0.) {
        const double r = d.horizon - 0.5 * d.mesh_size - 1e-3 * d.mesh_size;
        std::fill(rint.begin() + b->off[s], rint.begin() + b->off[s] + d.n_nodes, r);
        hmin = std::min(hmin, d.mesh_size);
      }
    }
    for (int64_t q = 0; q < 3 * d.n_nodes; q++) xmax = std::max(xmax, std::fabs(d.x[q]));
  }
  hrow[N] = nnz;
  if (nnz > INT32_MAX) return bail(fail(NLM_ERR_INVALID, "too many bonds"));
  b->nnz = nnz;
  b->rowptr = hrow;
  BTRY(cudaMemcpyAsync(rowptr, hrow.data(), sizeof(int64_t) * (N + 1), cudaMemcpyHostToDevice, st));
  int *cols;
  BTRY(b->alloc(&cols, nnz + 1));
  for (int s = 0; s < nspec; s++) {
    if (!b->nbond[s]) continue;
    BTRY(cudaMemcpyAsync(cols + b->bond_off[s], nbs[s].cols, sizeof(int) * b->nbond[s],
                         cudaMemcpyDeviceToDevice, st));
    BTRY(offset_cols(b->nbond[s], cols + b->bond_off[s], (int)b->off[s], st));
  }
  BTRY(cudaStreamSynchronize(st));
  // the per-specimen builds are no longer needed
  for (int s = 0; s < nspec; s++) {
    for (void *q : {(void *)nbs[s].perm, (void *)nbs[s].pos, (void *)nbs[s].rowptr, (void *)nbs[s].cols}) {
      auto it = std::find(b->allocs.begin(), b->allocs.end(), q);
      if (it != b->allocs.end()) {
        cudaFree(q);
        b->allocs.erase(it);
      }
    }
  }
  SellStore ss;
  cudaError_t e = build_sell(N, rowptr, cols, ss, st);
  for (void *q : {(void *)ss.ptr, (void *)ss.width, (void *)ss.cols})
    if (q) b->allocs.push_back(q);
  if (e != cudaSuccess) return bail(cuda_fail(e, "bond store build"));
  StepParams &P = b->P;
  P.n = N;
  P.dim = b->dim;
  P.npad = N;
  P.nwords = std::max(1, (ss.maxw + 31) / 32);
  P.nw1 = P.nwords == 1 ? 1 : 0;
  P.dt = b->dt;
  P.scheme = b->scheme;
  P.irrev = 1;
  double X = 1.;
  while (X < xmax) X *= 2.;
  while (X * 0.5 >= xmax && X > 1e-30) X *= 0.5;
  P.lo_scale = std::ldexp(1.0, 24) / X;
  DevPtrs &D = b->D;
  D.pos64 = pos64;
  D.rowptr = rowptr;
  D.cols = cols;
  D.sell_ptr = ss.ptr;
  D.sell_w = ss.width;
  D.sell_cols = ss.cols;
  // explicit decomposition: every specimen names the same one, used for all
  // buckets; NLM_DECOMP_AUTO (any specimen) autotunes per bucket
  if (fixed == NLM_DECOMP_TILE)
    return bail(fail(NLM_ERR_UNSUPPORTED, "a batch takes NLM_DECOMP_TILE_LOCAL, not TILE"));
  if (fixed != NLM_DECOMP_AUTO && fixed != NLM_DECOMP_THREAD && fixed != NLM_DECOMP_THREAD1 &&
      fixed != NLM_DECOMP_WARP && fixed != NLM_DECOMP_TILE_LOCAL)
    return bail(fail(NLM_ERR_INVALID, "unknown decomposition"));
  if (b->dim == 2 && (fixed == NLM_DECOMP_AUTO || fixed == NLM_DECOMP_TILE_LOCAL)) {
    TileInputs tin{N, nnz, ss.nslices, ss.entries, cols, ss.ptr, &b->rowptr, nullptr,
                   kTileMaxLocal, (lres.empty() || !relabel_all) ? nullptr : &lres};
    BTRY(cudaStreamSynchronize(st));  // posh
    if (hmin < 1e300) {
      tin.xin = posh.data();
      tin.xs = S;
      tin.r_int_node = rint.data();
      tin.ext_max = 1000. * hmin;
    }
    if (int rc_t = build_tile_store(b, tin, b->tile_ok, nullptr)) return bail(rc_t);
  }
  if (fixed == NLM_DECOMP_TILE_LOCAL && !b->tile_ok)
    return bail(fail(NLM_ERR_UNSUPPORTED,
                     "the tile-frame decomposition is for 2-D batches whose tiles fit the store"));
  uint32_t *bits;
  BTRY(b->alloc(&bits, (size_t)P.nwords * N));
  BTRY(cudaMemsetAsync(bits, 0, sizeof(uint32_t) * P.nwords * N, st));
  D.bits = bits;
  // per-specimen constants, loads, cracks
  std::vector<Params32> qtab(nspec);
  std::vector<BCTime> bct;
  std::vector<int> slice_spec(N / 32, -1);
  std::vector<uint8_t> flags(N, FLAG_GHOST);
  std::vector<int> bcref(N, -1), bcn;
  std::vector<BCEntry> bce;
  std::vector<double> volp(N, 0.);
  std::vector<uint16_t> rl(N, 0);
  bool any_nofail = false;
  bool all_uniform = true;
  double span_min = 1e300;
  for (int s = 0; s < nspec; s++) {
    const nlm_fd_desc &d = descs[s];
    StepParams Ps{};
    Ps.n = d.n_nodes;
    Ps.dim = d.dim;
    Ps.delta = d.horizon;
    Ps.h = d.mesh_size;
    Ps.check_up = d.horizon + 0.5 * d.mesh_size;
    Ps.check_low = d.horizon - 0.5 * d.mesh_size;
    Ps.dt = d.dt;
    Ps.rho = d.material.density;
    Ps.scheme = d.scheme;
    Ps.lo_scale = P.lo_scale;
    int rc = rnp_constants(d.material, d.dim, d.horizon, Ps);
    if (rc) return bail(rc);
    if (Ps.contact) return bail(fail(NLM_ERR_UNSUPPORTED, "contact forces are not batched"));
    // one volume for the specimen: its K1 V as a constant in its table
    Ps.vol_uniform = d.n_nodes > 0 ? d.volume[0] : 0.;
    for (int64_t i = 1; i < d.n_nodes && Ps.vol_uniform > 0.; i++)
      if (d.volume[i] != d.volume[0]) Ps.vol_uniform = 0.;
    all_uniform = all_uniform && Ps.vol_uniform > 0.;
    qtab[s] = make_p32(Ps);
    // the tile kernel decides per tile (specimens may share one): the
    // smallest span limit of all specimens
    span_min = std::min(span_min, (double)qtab[s].span_max);
    for (int64_t q = b->off[s] / 32; q < (b->off[s] + d.n_nodes + 31) / 32; q++) slice_spec[q] = s;
    for (int c = 0; c < d.n_cracks; c++) {
      if (d.cracks[c].kind == NLM_CRACK_EDGE && d.dim != 2)
        return bail(fail(NLM_ERR_INVALID, "edge pre-cracks are 2-D only"));
      if (d.cracks[c].timed)
        return bail(fail(NLM_ERR_UNSUPPORTED, "the batched model takes pre-cracks only"));
      BTRY(apply_precrack(d.n_nodes, S, pos64, rowptr, cols, d.cracks[c], N, bits, st, b->off[s]));
    }
    const int set0 = (int)bct.size();
    for (int k = 0; k < d.n_ubc; k++) {
      BCTime t;
      t.fn = d.ubc[k].time_fn;
      for (int q = 0; q < 4; q++) t.p[q] = d.ubc[k].time_params[q];
      bct.push_back(t);
    }
    // fixity, winning set per dof, no-fail flags (same rules as nlm_fd_create)
    std::vector<uint8_t> fix(d.n_nodes, 0), interior(d.n_nodes, 1);
    std::vector<int> wset(3 * d.n_nodes, -1);
    std::vector<double> wumax(3 * d.n_nodes, 0.);
    for (int k = 0; k < d.n_ubc; k++)
      for (int64_t i = 0; i < d.n_nodes; i++) {
        if (!in_region(d.ubc[k], d.x + 3 * i, d.dim)) continue;
        const double um = uload_umax(d.ubc[k], d.x + 3 * i);
        for (int dd = 0; dd < 3; dd++)
          if (d.ubc[k].dir_mask >> dd & 1) {
            fix[i] |= uint8_t(1 << dd);
            wset[3 * i + dd] = set0 + k;
            wumax[3 * i + dd] = um;
          }
      }
    if (d.no_fail != NLM_NOFAIL_OFF)
      nofail_flags(d.x, d.n_nodes, d.no_fail_tol, d.n_nofail_regions, d.nofail_regions, interior);
    for (int64_t i = 0; i < d.n_nodes; i++) {
      const int64_t g = b->off[s] + i;
      const int o = b->perm[s][i];
      uint8_t f = fix[o];
      if (!interior[o]) {
        f |= FLAG_NOFAIL;
        any_nofail = true;
      }
      flags[g] = f;
      volp[g] = d.volume[o];
      rl[g] = (uint16_t)(hrow[g + 1] - hrow[g]);
      if (fix[o]) {
        BCEntry be;
        for (int dd = 0; dd < 3; dd++) {
          be.set[dd] = wset[3 * o + dd];
          be.umax[dd] = wumax[3 * o + dd];
        }
        bcref[g] = (int)bce.size();
        bce.push_back(be);
        bcn.push_back((int)g);
      }
    }
  }
  (void)total_sets;
  P.nofail = any_nofail ? 1 : 0;
  P.uv_specimens = all_uniform ? 1 : 0;
  Params32 *dq;
  BCTime *dbct;
  int *dss;
  uint8_t *dflags;
  int *dbcref;
  BCEntry *dbce;
  double *vol64;
  uint16_t *drl;
  BTRY(b->alloc(&dq, nspec));
  BTRY(b->alloc(&dbct, bct.size() + 1));
  BTRY(b->alloc(&dss, slice_spec.size() + 1));
  BTRY(b->alloc(&dflags, N));
  BTRY(b->alloc(&dbcref, N));
  BTRY(b->alloc(&dbce, bce.size() + 1));
  BTRY(b->alloc(&vol64, N));
  BTRY(b->alloc(&drl, N));
  BTRY(cudaMemcpyAsync(dq, qtab.data(), sizeof(Params32) * nspec, cudaMemcpyHostToDevice, st));
  if (!bct.empty()) BTRY(cudaMemcpyAsync(dbct, bct.data(), sizeof(BCTime) * bct.size(), cudaMemcpyHostToDevice, st));
  BTRY(cudaMemcpyAsync(dss, slice_spec.data(), sizeof(int) * slice_spec.size(), cudaMemcpyHostToDevice, st));
  BTRY(cudaMemcpyAsync(dflags, flags.data(), N, cudaMemcpyHostToDevice, st));
  BTRY(cudaMemcpyAsync(dbcref, bcref.data(), sizeof(int) * N, cudaMemcpyHostToDevice, st));
  if (!bce.empty()) BTRY(cudaMemcpyAsync(dbce, bce.data(), sizeof(BCEntry) * bce.size(), cudaMemcpyHostToDevice, st));
  BTRY(cudaMemcpyAsync(vol64, volp.data(), sizeof(double) * N, cudaMemcpyHostToDevice, st));
  BTRY(cudaMemcpyAsync(drl, rl.data(), sizeof(uint16_t) * N, cudaMemcpyHostToDevice, st));
  D.qtab = dq;
  P.tile_span_max = nspec > 0 ? span_min : 0.;
  D.bct = dbct;
  D.slice_spec = dss;
  D.flags = dflags;
  D.bcref = dbcref;
  D.bce = dbce;
  D.vol64 = vol64;
  D.rowlen = drl;
  b->n_bc_nodes = (int64_t)bcn.size();
  BTRY(b->alloc(&b->bc_nodes, bcn.size() + 1));
  if (!bcn.empty())
    BTRY(cudaMemcpyAsync(b->bc_nodes, bcn.data(), sizeof(int) * bcn.size(), cudaMemcpyHostToDevice, st));
  float4 *pos32;
  uint2 *pos32lo = nullptr;
  BTRY(b->alloc(&pos32, N));
  if (S == 4) BTRY(b->alloc(&pos32lo, N));
  k_make_pos32<<<nblk(N, 256), 256, 0, st>>>(N, S, pos64, vol64, P.lo_scale, pos32, pos32lo);
  BTRY(cudaGetLastError());
  D.pos32 = pos32;
  D.pos32lo = pos32lo;
  BTRY(b->alloc(&D.u32[0], (size_t)(S / 2) * N));
  BTRY(b->alloc(&D.u32[1], (size_t)(S / 2) * N));
  BTRY(b->alloc(&D.v32[0], (size_t)(S / 2) * N));
  BTRY(b->alloc(&D.v32[1], (size_t)(S / 2) * N));
  BTRY(b->alloc(&D.f32, (size_t)S * N));
  BTRY(b->alloc(&b->stage, 3 * (size_t)N));
  double *fx;
  BTRY(b->alloc(&fx, (size_t)S * N));
  D.fext = fx;
  for (float4 *q : {D.u32[0], D.u32[1], D.v32[0], D.v32[1]})
    BTRY(cudaMemsetAsync(q, 0, sizeof(float4) * (S / 2) * N, st));
  BTRY(cudaMemsetAsync(D.f32, 0, sizeof(float) * S * N, st));
  BTRY(cudaMemsetAsync(fx, 0, sizeof(double) * S * N, st));
  // initial states
  int *dperm;
  BTRY(b->alloc(&dperm, N));
  for (int s = 0; s < nspec; s++) {
    const nlm_fd_desc &d = descs[s];
    if (!d.u0 && !d.v0) continue;
    BTRY(cudaMemcpyAsync(dperm, b->perm[s].data(), sizeof(int) * d.n_nodes, cudaMemcpyHostToDevice, st));
    const unsigned g = nblk(d.n_nodes, 256);
    if (d.u0) {
      BTRY(cudaMemcpyAsync(b->stage, d.u0, sizeof(double) * 3 * d.n_nodes, cudaMemcpyHostToDevice, st));
      k_scatter_split<<<g, 256, 0, st>>>(d.n_nodes, S, d.dim, dperm, b->stage, D.u32[0] + (S / 2) * b->off[s]);
    }
    if (d.v0) {
      BTRY(cudaMemcpyAsync(b->stage, d.v0, sizeof(double) * 3 * d.n_nodes, cudaMemcpyHostToDevice, st));
      k_scatter_split<<<g, 256, 0, st>>>(d.n_nodes, S, d.dim, dperm, b->stage, D.v32[0] + (S / 2) * b->off[s]);
    }
    BTRY(cudaGetLastError());
    BTRY(cudaStreamSynchronize(st));
  }
  // node-count buckets (terciles of the specimen list by size) + autotuning
  const int nb = std::min(3, nspec);
  int64_t prev = 0;
  for (int q = 0; q < nb; q++) {
    const int kend = (int)(((int64_t)(q + 1) * nspec) / nb);
    const int64_t end = kend < nspec ? b->off[b->order[kend]] : N;
    if (end > prev)
      b->buckets.push_back({prev, end, fixed == NLM_DECOMP_AUTO ? NLM_DECOMP_THREAD : fixed});
    prev = end;
  }
  BTRY(cudaStreamSynchronize(st));
  if (fixed == NLM_DECOMP_AUTO) {
    // time each candidate per bucket on scratch velocity / force / bit copies
    DevPtrs Dt = D;
    float4 *sv0 = nullptr;
    float *sf = nullptr;
    uint32_t *sb = nullptr;
    cudaError_t e2 = cudaMalloc(&sv0, sizeof(float4) * (S / 2) * N);
    if (e2 == cudaSuccess) e2 = cudaMalloc(&sf, sizeof(float) * S * N);
    if (e2 == cudaSuccess) e2 = cudaMalloc(&sb, sizeof(uint32_t) * P.nwords * N);
    if (e2 == cudaSuccess) {
      cudaMemcpyAsync(sv0, D.v32[0], sizeof(float4) * (S / 2) * N, cudaMemcpyDeviceToDevice, st);
      cudaMemsetAsync(sf, 0, sizeof(float) * S * N, st);
      cudaMemcpyAsync(sb, D.bits, sizeof(uint32_t) * P.nwords * N, cudaMemcpyDeviceToDevice, st);
      Dt.v32[0] = sv0;
      Dt.v32[1] = sv0;
      Dt.f32 = sf;
      Dt.bits = sb;
      cudaEvent_t ea, eb;
      cudaEventCreate(&ea);
      cudaEventCreate(&eb);
      for (auto &bk : b->buckets) {
        float best = 1e30f;
        std::vector<int> cands = {NLM_DECOMP_THREAD, NLM_DECOMP_THREAD1, NLM_DECOMP_WARP};
        if (b->tile_ok) cands.push_back(NLM_DECOMP_TILE_LOCAL);
        for (int c : cands) {
          StepArgs a{0, false, 0., b->dt, nullptr, bk.i0, bk.i1};
          for (int w = 0; w < 2; w++) e2 = launch_rnp_step_fp32(P, Dt, b->T, a, c, st);
          cudaEventRecord(ea, st);
          for (int r = 0; r < 3; r++) e2 = launch_rnp_step_fp32(P, Dt, b->T, a, c, st);
          cudaEventRecord(eb, st);
          if (e2 == cudaSuccess) e2 = cudaEventSynchronize(eb);
          float ms = 0.f;
          if (e2 == cudaSuccess) e2 = cudaEventElapsedTime(&ms, ea, eb);
          if (e2 != cudaSuccess) break;
          if (ms < best) {
            best = ms;
            bk.decomp = c;
          }
        }
        if (e2 != cudaSuccess) break;
      }
      cudaEventDestroy(ea);
      cudaEventDestroy(eb);
    }
    cudaStreamSynchronize(st);
    cudaFree(sv0);
    cudaFree(sf);
    cudaFree(sb);
    if (e2 != cudaSuccess) return bail(cuda_fail(e2, "batch autotune"));
  }
  *out = b;
#undef BTRY
  return NLM_OK;
}

int nlm_batch_destroy(nlm_batch *b) {
  delete b;
  return NLM_OK;
}

int nlm_batch_run(nlm_batch *b, int64_t nsteps) {
  if (!b || nsteps < 0) return fail(NLM_ERR_INVALID, "bad arguments");
  return batch_run(b, nsteps);
}

int nlm_batch_run_timed(nlm_batch *b, int64_t nsteps, double *ms) {
  if (!b || !ms || nsteps < 0) return fail(NLM_ERR_INVALID, "bad arguments");
  cudaEvent_t e0, e1;
  NLM_CUDA(cudaEventCreate(&e0));
  NLM_CUDA(cudaEventCreate(&e1));
  cudaEventRecord(e0, b->stream);
  int rc = batch_run(b, nsteps);
  cudaEventRecord(e1, b->stream);
  cudaError_t e = cudaEventSynchronize(e1);
  float t = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  if (e != cudaSuccess) return cuda_fail(e, "batch timing");
  *ms = t;
  return NLM_OK;
}

int nlm_batch_num_bonds(const nlm_batch *b, int s, int64_t *nnz) {
  if (!b || !nnz || s < -1 || s >= b->nspec) return fail(NLM_ERR_INVALID, "bad arguments");
  *nnz = s < 0 ? b->nnz : b->nbond[s];
  return NLM_OK;
}

int nlm_batch_get_time(const nlm_batch *b, double *time, int64_t *step) {
  if (!b) return fail(NLM_ERR_INVALID, "null handle");
  if (time) *time = b->time;
  if (step) *step = b->step;
  return NLM_OK;
}

int nlm_batch_get_state(nlm_batch *b, int s, double *u, double *v, double *f) {
  if (!b || s < 0 || s >= b->nspec) return fail(NLM_ERR_INVALID, "bad arguments");
  const int64_t n = b->n[s], off = b->off[s];
  const int S = b->S;
  cudaStream_t st = b->stream;
  int *dperm = nullptr;
  NLM_CUDA(cudaMalloc(&dperm, sizeof(int) * (n + 1)));
  cudaError_t e = cudaMemcpyAsync(dperm, b->perm[s].data(), sizeof(int) * n, cudaMemcpyHostToDevice, st);
  const unsigned g = nblk(n, 256);
  const int vi = b->scheme == NLM_CENTRAL_DIFFERENCE ? b->cur : 0;
  if (e == cudaSuccess && u) {
    k_gather_split<<<g, 256, 0, st>>>(n, S, dperm, b->D.u32[b->cur] + (S / 2) * off, b->stage);
    e = cudaMemcpyAsync(u, b->stage, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  }
  if (e == cudaSuccess && v) {
    k_gather_split<<<g, 256, 0, st>>>(n, S, dperm, b->D.v32[vi] + (S / 2) * off, b->stage);
    e = cudaMemcpyAsync(v, b->stage, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  }
  if (e == cudaSuccess && f) {
    k_gather_f32<<<g, 256, 0, st>>>(n, S, dperm, b->D.f32 + (size_t)S * off, b->stage);
    e = cudaMemcpyAsync(f, b->stage, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  }
  cudaStreamSynchronize(st);
  cudaFree(dperm);
  if (e != cudaSuccess) return cuda_fail(e, "batch state download");
  return NLM_OK;
}

int nlm_batch_get_bond_state(nlm_batch *b, int s, uint8_t *broken) {
  if (!b || !broken || s < 0 || s >= b->nspec) return fail(NLM_ERR_INVALID, "bad arguments");
  const int64_t n = b->n[s], off = b->off[s], npad = b->P.npad;
  std::vector<uint32_t> bits((size_t)b->P.nwords * npad);
  std::vector<int> cc(b->nbond[s] + 1);
  NLM_CUDA(cudaMemcpyAsync(bits.data(), b->D.bits, sizeof(uint32_t) * bits.size(), cudaMemcpyDeviceToHost, b->stream));
  if (b->nbond[s])
    NLM_CUDA(cudaMemcpyAsync(cc.data(), b->D.cols + b->bond_off[s], sizeof(int) * b->nbond[s],
                             cudaMemcpyDeviceToHost, b->stream));
  NLM_CUDA(cudaStreamSynchronize(b->stream));
  const std::vector<int> &perm = b->perm[s];
  std::vector<int64_t> inv(n);
  for (int64_t i = 0; i < n; i++) inv[perm[i]] = i;
  int64_t o_off = 0;
  std::vector<std::pair<int, uint8_t>> row;
  for (int64_t o = 0; o < n; o++) {
    const int64_t i = inv[o], g = off + i;
    const int64_t r0 = b->rowptr[g], len = b->rowptr[g + 1] - r0;
    row.resize(len);
    for (int64_t k = 0; k < len; k++)
      row[k] = {perm[cc[r0 - b->bond_off[s] + k] - off],
                (uint8_t)((bits[(size_t)(k >> 5) * npad + g] >> (k & 31)) & 1u)};
    std::sort(row.begin(), row.end());
    for (int64_t k = 0; k < len; k++) broken[o_off + k] = row[k].second;
    o_off += len;
  }
  return NLM_OK;
}

int nlm_batch_set_graph(nlm_batch *b, int steps_per_graph) {
  if (!b || steps_per_graph < 0 || (steps_per_graph % 2) || steps_per_graph == 1)
    return fail(NLM_ERR_INVALID, "steps_per_graph must be 0 or an even number >= 2");
  NLM_CUDA(cudaStreamSynchronize(b->stream));
  for (auto &g : b->gexec)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
  if (b->h_times) {
    cudaFreeHost(b->h_times);
    b->h_times = nullptr;
  }
  b->graph_steps = steps_per_graph;
  if (steps_per_graph > 0) {
    NLM_CUDA(cudaMallocHost(&b->h_times, sizeof(double) * (steps_per_graph + 1)));
    if (b->alloc(&b->d_times, (size_t)steps_per_graph + 1) != cudaSuccess)
      return fail(NLM_ERR_OOM, "graph time buffer");
    if (!b->ev_times) NLM_CUDA(cudaEventCreateWithFlags(&b->ev_times, cudaEventDisableTiming));
    NLM_CUDA(cudaEventRecord(b->ev_times, b->stream));
  }
  return NLM_OK;
}

int nlm_batch_buckets(const nlm_batch *b, int *n_buckets, int64_t *bucket_nodes, int *decomps) {
  if (!b || !n_buckets) return fail(NLM_ERR_INVALID, "null argument");
  *n_buckets = (int)b->buckets.size();
  for (size_t k = 0; k < b->buckets.size() && k < 8; k++) {
    if (bucket_nodes) bucket_nodes[k] = b->buckets[k].i1 - b->buckets[k].i0;
    if (decomps) decomps[k] = b->buckets[k].decomp;
  }
  return NLM_OK;
}

}  // extern "C"

