// qs_host.cu -- nlm_qs_*: quasi-static Newton for RNPBond on the GPU.

#include "fd_handle.h"

// ===========================================================================
// Quasi-static Newton (RNPBond).  Geometry, bond bits, flags and loads come
// from an FP64 nlm_fd handle; the state is its displacement buffer u64[cur].

struct nlm_qs {
  nlm_fd *fd = nullptr;
  nlm_qs_params prm{};
  QSWork W{};
  unsigned long long *count = nullptr;
  double *saved = nullptr;  // plain start point while a guess is evaluated
  double *cand = nullptr;   // best candidate start so far
  // FP64 Krylov solves from now on, for Newton corrections and for tangent
  // predictors respectively: set once a solve of that kind has not converged
  // in FP32 within its iteration cap (the tangent of this specimen is then
  // too ill-conditioned for FP32 recurrences)
  bool cg64 = false;
  bool cg64_predictor = false;
  std::vector<void *> allocs;
  ~nlm_qs() {
    if (fd) nlm_fd_destroy(fd);  // frees the stream first
    for (void *p : allocs) cudaFree(p);
  }
  template <class Tp>
  cudaError_t alloc(Tp **p, size_t count_) {
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, count_ * sizeof(Tp) + 16);
    if (e == cudaSuccess) {
      allocs.push_back(q);
      *p = static_cast<Tp *>(q);
    }
    return e;
  }
};

namespace {

int qs_norm(nlm_qs *q, const double *u, double *buf, double *norm) {
  nlm_fd *h = q->fd;
  cudaError_t e = qs_residual(h->P, h->D, u, buf, nullptr, nullptr, false, h->stream);
  if (e == cudaSuccess) e = qs_dot(buf, buf, (int64_t)h->dim * h->n, q->W.part, q->W.sc + 4, h->stream);
  double v = 0.;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&v, q->W.sc + 4, sizeof(double), cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return cuda_fail(e, "qs residual");
  *norm = std::sqrt(v);
  return NLM_OK;
}

// Newton iterations from the current u until ||r|| <= target.  Each residual
// evaluation breaks the bonds past the critical strain first.
int qs_newton(nlm_qs *q, double target, nlm_qs_stats *st) {
  nlm_fd *h = q->fd;
  double *u = h->D.u64[h->cur];
  const int64_t m = (int64_t)h->dim * h->n;
  for (int it = 0;; it++) {
    cudaError_t e = cudaMemsetAsync(q->count, 0, sizeof(unsigned long long), h->stream);
    if (e == cudaSuccess)
      e = qs_residual(h->P, h->D, u, q->W.res, q->W.blk, q->W.dblk, true, h->stream,
                      q->prm.break_bonds ? q->count : nullptr);
    if (e == cudaSuccess) e = qs_dot(q->W.res, q->W.res, m, q->W.part, q->W.sc + 4, h->stream);
    double rr = 0.;
    unsigned long long c = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&rr, q->W.sc + 4, sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&c, q->count, sizeof(c), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_fail(e, "qs Newton residual");
    st->broken += (int64_t)c;
    if (c) st->break_rounds++;
    st->res_final = std::sqrt(rr);
    if (!(st->res_final > target) || it >= q->prm.max_newton) return NLM_OK;
    // the linear tolerance: lin_tol, or looser when the residual is already
    // near the target (a correction accurate to gamma * target / ||r|| of
    // ||r|| leaves a linear residual of gamma * target)
    double eta = q->prm.lin_tol;
    if (q->prm.lin_tol_gamma > 0. && st->res_final > 0.)
      eta = std::max(eta, std::min(0.1, q->prm.lin_tol_gamma * target / st->res_final));
    int li = 0;
    e = qs_cg(h->P, h->D, q->W, q->W.res, q->W.dx, eta, q->prm.lin_max_iters, 8, &li, &q->cg64,
              h->stream);
    if (e == cudaSuccess) e = qs_add(h->P, q->W.dx, u, h->stream);
    if (e != cudaSuccess) return cuda_fail(e, "qs linear solve");
    st->lin_iters += li;
    st->newton_iters++;
  }
}

// ||res0 - (-K) dx|| over free dofs: the linear model of the residual at the
// previous converged state, evaluated at the increment dx.
int qs_linear_norm(nlm_qs *q, double *norm) {
  nlm_fd *h = q->fd;
  const int64_t m = (int64_t)h->dim * h->n;
  cudaStream_t s = h->stream;
  cudaError_t e = qs_spmv(h->P, h->D, q->W.blk, q->W.dblk, q->W.dx, q->W.ap, q->W.part, s);
  if (e == cudaSuccess) e = qs_sub(m, q->W.res0, q->W.ap, q->W.res, s);
  if (e == cudaSuccess) e = qs_dot(q->W.res, q->W.res, m, q->W.part, q->W.sc + 4, s);
  double rr = 0.;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&rr, q->W.sc + 4, sizeof(double), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "qs linear model");
  *norm = std::sqrt(rr);
  return NLM_OK;
}

}  // namespace

extern "C" {

int nlm_qs_create(const nlm_fd_desc *desc, const nlm_qs_params *prm, nlm_qs **out) {
  if (!desc || !prm || !out) return fail(NLM_ERR_INVALID, "null argument");
  *out = nullptr;
  if (desc->material.kind != NLM_MAT_RNP_BOND)
    return fail(NLM_ERR_UNSUPPORTED, "the GPU quasi-static solver is for RNPBond");
  if (desc->material.apply_contact)
    return fail(NLM_ERR_UNSUPPORTED, "the quasi-static solver has no contact term");
  for (int c = 0; c < desc->n_cracks; c++)
    if (desc->cracks && desc->cracks[c].timed)
      return fail(NLM_ERR_UNSUPPORTED, "the quasi-static solver takes pre-cracks only");
  if (prm->max_newton < 1 || !(prm->tol > 0.) || prm->lin_max_iters < 1 || !(prm->lin_tol > 0.))
    return fail(NLM_ERR_INVALID, "bad solver parameters");
  nlm_fd_desc d = *desc;
  d.precision = NLM_PREC_FP64;
  d.scheme = NLM_VELOCITY_VERLET;
  d.decomposition = NLM_DECOMP_THREAD;
  if (!(d.dt > 0.)) return fail(NLM_ERR_INVALID, "load-step increment dt must be positive");
  nlm_qs *q = new nlm_qs();
  int rc = nlm_fd_create(&d, &q->fd);
  if (rc) {
    delete q;
    return rc;
  }
  q->prm = *prm;
  nlm_fd *h = q->fd;
  const int64_t n = h->n, m = (int64_t)h->dim * n, nnz = h->nnz;
  const int NB = h->dim == 2 ? 3 : 6;
  cudaError_t e = cudaSuccess;
  for (double **p : {&q->W.res, &q->W.dx, &q->W.r, &q->W.z, &q->W.p, &q->W.p2, &q->W.ap,
                     &q->W.res0})
    if (e == cudaSuccess) e = q->alloc(p, m);
  if (e == cudaSuccess) e = q->alloc(&q->W.part, std::max<int64_t>((m + 255) / 256 + 1, qs_cg_stride(n)));
  if (e == cudaSuccess) e = q->alloc(&q->W.cgpart, 3 * qs_cg_stride(n));
  if (e == cudaSuccess) e = q->alloc(&q->W.cgs, 8);
  for (float **p : {&q->W.r32, &q->W.z32, &q->W.p32, &q->W.p32b, &q->W.ap32, &q->W.x32})
    if (e == cudaSuccess) e = q->alloc(p, m);
  if (e == cudaSuccess) e = q->alloc(&q->W.blk32, (size_t)(NB == 3 ? 4 : 8) * (nnz + 1));
  if (e == cudaSuccess) e = q->alloc(&q->W.dblk32, (size_t)NB * n);
  q->W.nnz = nnz;
  if (e == cudaSuccess) e = q->alloc(&q->W.ticket, 4);
  if (e == cudaSuccess) e = cudaMemset(q->W.ticket, 0, 4 * sizeof(unsigned));
  if (e == cudaSuccess && prm->krylov_launch == 1) {
    q->W.coop_blocks = qs_coop_blocks(n, h->dim);
    if (q->W.coop_blocks > 0) {
      e = q->alloc(&q->W.coop, 4);
      if (e == cudaSuccess) e = cudaMemset(q->W.coop, 0, 4 * sizeof(unsigned));
      q->W.coop_extra = std::max(0, prm->barrier_extra);
      const double lim = prm->wait_limit_s > 0. ? prm->wait_limit_s : 1.0;
      q->W.coop_wait_ns = (uint64_t)(std::min(lim, 60.0) * 1e9);
    }
  }
  if (e == cudaSuccess) e = q->alloc(&q->W.sc, 8);
  if (e == cudaSuccess) e = q->alloc(&q->W.blk, (size_t)NB * (nnz + 1));
  if (e == cudaSuccess) e = q->alloc(&q->W.dblk, (size_t)NB * n);
  if (e == cudaSuccess) e = q->alloc(&q->count, 1);
  if (e == cudaSuccess) e = q->alloc(&q->saved, (size_t)h->S * n);
  if (e == cudaSuccess) e = q->alloc(&q->cand, (size_t)h->S * n);
  if (e != cudaSuccess) {
    delete q;
    return cuda_fail(e, "qs buffers");
  }
  h->started = true;  // no explicit step-0 evaluation
  *out = q;
  return NLM_OK;
}

int nlm_qs_destroy(nlm_qs *q) {
  delete q;
  return NLM_OK;
}

int nlm_qs_load_step(nlm_qs *q, const double *guess, nlm_qs_stats *stats) {
  return nlm_qs_load_step_candidates(q, guess, guess ? 1 : 0, stats);
}

int nlm_qs_load_step_candidates(nlm_qs *q, const double *guesses, int n_cand,
                                nlm_qs_stats *stats) {
  if (!q) return fail(NLM_ERR_INVALID, "null handle");
  if (n_cand < 0 || (n_cand > 0 && !guesses)) return fail(NLM_ERR_INVALID, "bad candidates");
  auto t0 = std::chrono::steady_clock::now();
  nlm_fd *h = q->fd;
  nlm_qs_stats st{};
  cudaStream_t s = h->stream;
  double *u = h->D.u64[h->cur];
  const int64_t m = (int64_t)h->dim * h->n;
  const size_t bytes = sizeof(double) * h->S * h->n;
  // force and tangent at the previous converged state
  NLM_CUDA(cudaMemcpyAsync(q->saved, u, bytes, cudaMemcpyDeviceToDevice, s));
  cudaError_t e = qs_residual(h->P, h->D, u, q->W.res0, q->W.blk, q->W.dblk, true, s);
  if (e != cudaSuccess) return cuda_fail(e, "qs assembly");
  // QuasiStaticModel::solver: time = n * dt, then the displacement loads
  h->step++;
  h->time = (double)h->step * h->dt;
  int rc = apply_bc(h, h->time);
  if (rc) return rc;
  // plain predictor: boundary increment only
  if ((e = qs_bcdiff(h->P, h->D, u, q->saved, q->W.dx, true, s)) != cudaSuccess)
    return cuda_fail(e, "qs predictor");
  if ((rc = qs_linear_norm(q, &st.res_plain))) return rc;
  st.res_start = st.res_plain;
  NLM_CUDA(cudaMemcpyAsync(q->W.r, q->W.res, sizeof(double) * m, cudaMemcpyDeviceToDevice, s));
  bool use_guess = false;
  if (n_cand > 0) {
    // each candidate start is judged by the linear model of the residual at
    // the previous converged state; the best one is kept if it cuts the
    // linearised residual of the plain start clearly (a start no better than
    // the plain one, e.g. the previous state itself, would put the bonds next
    // to the loaded layer past their critical strain in the first residual
    // evaluation, which the tangent predictor of the plain start avoids)
    const double acc = q->prm.guess_accept > 0. ? q->prm.guess_accept : 0.1;
    int best = -1;
    double best_rg = 0.;
    for (int c = 0; c < n_cand; c++) {
      NLM_CUDA(cudaMemcpyAsync(h->stage, guesses + (size_t)3 * h->n * c,
                               sizeof(double) * 3 * h->n, cudaMemcpyHostToDevice, s));
      k_scatter_vec<<<nblk(h->n, 256), 256, 0, s>>>(h->n, h->S, h->dim, h->D.perm_dev, h->stage, u);
      NLM_CUDA(cudaGetLastError());
      if ((rc = apply_bc(h, h->time))) return rc;
      if ((e = qs_bcdiff(h->P, h->D, u, q->saved, q->W.dx, false, s)) != cudaSuccess)
        return cuda_fail(e, "qs guess");
      double rg = 0.;
      if ((rc = qs_linear_norm(q, &rg))) return rc;
      if (best < 0 || rg < best_rg) {
        best = c;
        best_rg = rg;
        if (n_cand > 1) NLM_CUDA(cudaMemcpyAsync(q->cand, u, bytes, cudaMemcpyDeviceToDevice, s));
      }
    }
    if (best >= 0 && best_rg <= acc * st.res_plain) {
      use_guess = true;
      st.used_guess = best + 1;
      st.res_start = best_rg;
      if (n_cand > 1) NLM_CUDA(cudaMemcpyAsync(u, q->cand, bytes, cudaMemcpyDeviceToDevice, s));
    } else {
      NLM_CUDA(cudaMemcpyAsync(u, q->saved, bytes, cudaMemcpyDeviceToDevice, s));
      if ((rc = apply_bc(h, h->time))) return rc;
    }
  }
  const double target = q->prm.tol * st.res_plain;
  if (!use_guess && st.res_plain > 0.) {
    // tangent predictor (first Newton iteration) on the saved right-hand side
    NLM_CUDA(cudaMemcpyAsync(q->W.res, q->W.r, sizeof(double) * m, cudaMemcpyDeviceToDevice, s));
    NLM_CUDA(cudaMemcpyAsync(q->W.ap, q->W.res, sizeof(double) * m, cudaMemcpyDeviceToDevice, s));
    int li = 0;
    e = qs_cg(h->P, h->D, q->W, q->W.ap, q->W.dx, q->prm.lin_tol, q->prm.lin_max_iters, 8, &li,
              &q->cg64_predictor, s);
    if (e == cudaSuccess) e = qs_add(h->P, q->W.dx, u, s);
    if (e != cudaSuccess) return cuda_fail(e, "qs predictor solve");
    st.lin_iters += li;
    st.newton_iters++;
  }
  if ((rc = qs_newton(q, target, &st))) return rc;
  st.ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (stats) *stats = st;
  return NLM_OK;
}

int nlm_qs_get_state(nlm_qs *q, double *u) {
  if (!q || !u) return fail(NLM_ERR_INVALID, "null argument");
  return nlm_fd_get_state(q->fd, u, nullptr, nullptr);
}

int nlm_qs_get_bond_state(nlm_qs *q, uint8_t *broken) {
  if (!q) return fail(NLM_ERR_INVALID, "null handle");
  return nlm_fd_get_bond_state(q->fd, broken);
}

int nlm_qs_damage(nlm_qs *q, float *phi, float *Z) {
  if (!q) return fail(NLM_ERR_INVALID, "null handle");
  return nlm_fd_damage(q->fd, phi, Z);
}

int nlm_qs_num_bonds(const nlm_qs *q, int64_t *nnz) {
  if (!q) return fail(NLM_ERR_INVALID, "null handle");
  return nlm_fd_num_bonds(q->fd, nnz);
}

}  // extern "C"

