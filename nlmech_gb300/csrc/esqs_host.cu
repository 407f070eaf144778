// esqs_host.cu -- nlm_esqs_*: quasi-static ElasticState
// (QuasiStaticModel<ElasticState>) on the GPU.

#include "fd_handle.h"

// ===========================================================================
// Quasi-static ElasticState (QuasiStaticModel<ElasticState>).  Geometry,
// volumes, m_i, flags and loads come from an FP64 nlm_fd handle (a 1-D mesh
// is held as a 2-D one with y = 0; the material law uses the model's own
// dimension); the state is its displacement buffer u64[cur].

struct nlm_esqs {
  nlm_fd *fd = nullptr;
  nlm_esqs_params prm{};
  int mdim = 2;
  int64_t m = 0, nblocks = 0;
  double *theta = nullptr, *f = nullptr, *body = nullptr, *res = nullptr, *rhs = nullptr;
  double *dx = nullptr, *J = nullptr, *r = nullptr, *rhat = nullptr, *p = nullptr;
  double *v = nullptr, *sv = nullptr, *t = nullptr, *part = nullptr, *sc = nullptr;
  std::vector<void *> allocs;
  ~nlm_esqs() {
    if (fd) nlm_fd_destroy(fd);  // synchronises and frees the stream first
    for (void *q : allocs) cudaFree(q);
  }
  template <class Tp>
  cudaError_t alloc(Tp **ptr, size_t count_) {
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, count_ * sizeof(Tp) + 16);
    if (e == cudaSuccess) {
      allocs.push_back(q);
      *ptr = static_cast<Tp *>(q);
    }
    return e;
  }
};

namespace {

int esqs_dot_host(nlm_esqs *q, const double *a, const double *b, double *out) {
  cudaStream_t s = q->fd->stream;
  cudaError_t e = esqs_dot(q->m, a, b, q->part, q->sc, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, q->sc, sizeof(double), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? NLM_OK : cuda_fail(e, "quasi-static dot product");
}

// f and the residual r = f + b at the current u; *norm = ||r||.
int esqs_eval(nlm_esqs *q, double *norm) {
  nlm_fd *h = q->fd;
  cudaError_t e = esqs_force(h->P, h->D, h->S, q->mdim, h->D.u64[h->cur], q->theta, q->f, h->stream);
  if (e == cudaSuccess) e = esqs_residual(h->P, h->D, h->S, q->mdim, q->f, q->body, q->res, h->stream);
  if (e != cudaSuccess) return cuda_fail(e, "quasi-static residual");
  double rr = 0.;
  int rc = esqs_dot_host(q, q->res, q->res, &rr);
  *norm = std::sqrt(rr);
  return rc;
}

// BiCGSTAB (van der Vorst 1992) for J dx = rhs to ||r|| <= tol ||rhs||.
int esqs_bicgstab(nlm_esqs *q, int *iters) {
  nlm_fd *h = q->fd;
  cudaStream_t s = h->stream;
  const int64_t m = q->m;
  const size_t bytes = sizeof(double) * m;
  NLM_CUDA(cudaMemsetAsync(q->dx, 0, bytes, s));
  NLM_CUDA(cudaMemcpyAsync(q->r, q->rhs, bytes, cudaMemcpyDeviceToDevice, s));
  NLM_CUDA(cudaMemcpyAsync(q->rhat, q->rhs, bytes, cudaMemcpyDeviceToDevice, s));
  NLM_CUDA(cudaMemsetAsync(q->p, 0, bytes, s));
  NLM_CUDA(cudaMemsetAsync(q->v, 0, bytes, s));
  double bb = 0.;
  int rc = esqs_dot_host(q, q->rhs, q->rhs, &bb);
  if (rc) return rc;
  *iters = 0;
  const double bnorm = std::sqrt(bb);
  if (bnorm == 0.) return NLM_OK;
  const double stop = q->prm.lin_tol * bnorm;
  double rho = 1., alpha = 1., omega = 1.;
  auto J_times = [&](const double *x, double *y) {
    cudaError_t e = esqs_spmv(h->P, h->D, h->S, q->mdim, q->J, x, y, s);
    return e == cudaSuccess ? NLM_OK : cuda_fail(e, "quasi-static Jacobian product");
  };
  auto lin3 = [&](double a, const double *x, double b, const double *y, double c, const double *z,
                  double *out) {
    cudaError_t e = esqs_lin3(m, a, x, b, y, c, z, out, s);
    return e == cudaSuccess ? NLM_OK : cuda_fail(e, "quasi-static vector update");
  };
  for (int it = 1; it <= q->prm.lin_max_iters; it++) {
    *iters = it;
    double rho_new = 0.;
    if ((rc = esqs_dot_host(q, q->rhat, q->r, &rho_new))) return rc;
    if (rho_new == 0.) break;  // breakdown: keep the iterate
    const double beta = (rho_new / rho) * (alpha / omega);
    if ((rc = lin3(1., q->r, beta, q->p, -beta * omega, q->v, q->p))) return rc;
    if ((rc = J_times(q->p, q->v))) return rc;
    double rv = 0.;
    if ((rc = esqs_dot_host(q, q->rhat, q->v, &rv))) return rc;
    if (rv == 0.) break;
    alpha = rho_new / rv;
    if ((rc = lin3(1., q->r, -alpha, q->v, 0., nullptr, q->sv))) return rc;
    double ss = 0.;
    if ((rc = esqs_dot_host(q, q->sv, q->sv, &ss))) return rc;
    if (std::sqrt(ss) <= stop) {
      if ((rc = lin3(1., q->dx, alpha, q->p, 0., nullptr, q->dx))) return rc;
      break;
    }
    if ((rc = J_times(q->sv, q->t))) return rc;
    double ts = 0., tt = 0.;
    if ((rc = esqs_dot_host(q, q->t, q->sv, &ts))) return rc;
    if ((rc = esqs_dot_host(q, q->t, q->t, &tt))) return rc;
    if (tt == 0.) {
      if ((rc = lin3(1., q->dx, alpha, q->p, 0., nullptr, q->dx))) return rc;
      break;
    }
    omega = ts / tt;
    if ((rc = lin3(1., q->dx, alpha, q->p, omega, q->sv, q->dx))) return rc;
    if ((rc = lin3(1., q->sv, -omega, q->t, 0., nullptr, q->r))) return rc;
    double rr = 0.;
    if ((rc = esqs_dot_host(q, q->r, q->r, &rr))) return rc;
    if (std::sqrt(rr) <= stop || omega == 0.) break;
    rho = rho_new;
  }
  return NLM_OK;
}

}  // namespace

extern "C" {

int nlm_esqs_create(const nlm_fd_desc *desc, const nlm_esqs_params *prm, nlm_esqs **out) {
  if (!desc || !prm || !out) return fail(NLM_ERR_INVALID, "null argument");
  *out = nullptr;
  if (desc->material.kind != NLM_MAT_ELASTIC_STATE)
    return fail(NLM_ERR_UNSUPPORTED, "QuasiStaticModel is instantiated for ElasticState");
  if (desc->dim < 1 || desc->dim > 3) return fail(NLM_ERR_INVALID, "dimension must be 1, 2 or 3");
  if (desc->dim == 1 && !(desc->material.E > 0.))
    return fail(NLM_ERR_INVALID, "1-D ElasticState needs E");
  if (prm->max_iters < 0 || !(prm->tol > 0.) || !(prm->perturbation > 0.) ||
      prm->lin_max_iters < 1 || !(prm->lin_tol > 0.) || !(prm->dt > 0.))
    return fail(NLM_ERR_INVALID, "bad solver parameters");
  for (int c = 0; c < desc->n_cracks; c++)
    if (desc->cracks && desc->cracks[c].timed)
      return fail(NLM_ERR_UNSUPPORTED, "the quasi-static solver takes pre-cracks only");
  nlm_fd_desc d = *desc;
  d.precision = NLM_PREC_FP64;
  d.scheme = NLM_VELOCITY_VERLET;
  d.decomposition = NLM_DECOMP_THREAD;
  d.dt = prm->dt;
  d.material.es_sc = 0.;  // no bond breaks in QuasiStaticModel
  std::vector<double> x1;
  if (desc->dim == 1) {
    // a 1-D mesh as a 2-D one: nodes (x, 0, 0); the 2-D constants are unused
    d.dim = 2;
    x1.assign(3 * (size_t)desc->n_nodes, 0.);
    for (int64_t i = 0; i < desc->n_nodes && desc->x; i++) x1[3 * i] = desc->x[3 * i];
    d.x = x1.data();
    if (!(d.material.K > 0.)) d.material.K = 1.;
    if (!(d.material.G > 0.)) d.material.G = 1.;
  }
  nlm_esqs *q = new nlm_esqs();
  int rc = nlm_fd_create(&d, &q->fd);
  if (rc) {
    delete q;
    return rc;
  }
  q->prm = *prm;
  q->mdim = desc->dim;
  nlm_fd *h = q->fd;
  q->m = (int64_t)h->S * h->n;
  q->nblocks = h->nnz + h->n;
  cudaError_t e = q->alloc(&q->theta, h->n);
  for (double **ptr : {&q->f, &q->body, &q->res, &q->rhs, &q->dx, &q->r, &q->rhat, &q->p, &q->v,
                       &q->sv, &q->t})
    if (e == cudaSuccess) e = q->alloc(ptr, q->m);
  if (e == cudaSuccess) e = q->alloc(&q->J, (size_t)9 * q->nblocks);
  if (e == cudaSuccess) e = q->alloc(&q->part, kEsqsDotParts);
  if (e == cudaSuccess) e = q->alloc(&q->sc, 1);
  if (e == cudaSuccess) e = cudaMemsetAsync(q->body, 0, sizeof(double) * q->m, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) {
    delete q;
    return cuda_fail(e, "quasi-static buffers");
  }
  h->started = true;  // no explicit step-0 evaluation
  *out = q;
  return NLM_OK;
}

int nlm_esqs_destroy(nlm_esqs *q) {
  delete q;
  return NLM_OK;
}

int nlm_esqs_solve(nlm_esqs *q, int nsteps, int *newton_iters, int *lin_iters,
                   double *final_res) {
  if (!q || nsteps < 0) return fail(NLM_ERR_INVALID, "bad arguments");
  nlm_fd *h = q->fd;
  cudaStream_t s = h->stream;
  double *u = h->D.u64[h->cur];
  const double eps = q->prm.perturbation * h->P.h;
  double res = 0.;
  int rc;
  for (int k = 0; k < nsteps; k++) {
    // QuasiStaticModel::solver (:526-594): time = n dt, force loading (added
    // to the body force, fLoading.cpp:268-275), displacement loading
    h->step++;
    h->time = (double)h->step * q->prm.dt;
    if (h->n_fbc_nodes > 0) {
      if ((rc = apply_fbc(h, h->time))) return rc;
      cudaError_t e = esqs_lin3(q->m, 1., q->body, 1., h->D.fext, 0., nullptr, q->body, s);
      if (e != cudaSuccess) return cuda_fail(e, "quasi-static body force");
    }
    if ((rc = apply_bc(h, h->time))) return rc;
    if ((rc = esqs_eval(q, &res))) return rc;
    const double r0 = res;
    int it = 0, li_total = 0;
    auto converged = [&]() {
      return q->prm.tol_relative ? (r0 == 0. || res / r0 < q->prm.tol) : res < q->prm.tol;
    };
    while (!converged() && it < q->prm.max_iters) {
      cudaError_t e = esqs_jacobian(h->P, h->D, h->S, q->mdim, q->prm.jacobian, u, eps, q->J,
                                    q->nblocks, s);
      if (e == cudaSuccess) e = esqs_lin3(q->m, -1., q->res, 0., nullptr, 0., nullptr, q->rhs, s);
      if (e != cudaSuccess) return cuda_fail(e, "quasi-static Jacobian");
      int li = 0;
      if ((rc = esqs_bicgstab(q, &li))) return rc;
      li_total += li;
      e = esqs_lin3(q->m, 1., u, 1., q->dx, 0., nullptr, u, s);
      if (e != cudaSuccess) return cuda_fail(e, "quasi-static update");
      if ((rc = esqs_eval(q, &res))) return rc;
      it++;
    }
    if (newton_iters) newton_iters[k] = it;
    if (lin_iters) lin_iters[k] = li_total;
  }
  if (final_res) *final_res = res;
  return NLM_OK;
}

int nlm_esqs_get_state(nlm_esqs *q, double *u, double *force) {
  if (!q) return fail(NLM_ERR_INVALID, "null handle");
  nlm_fd *h = q->fd;
  if (u) {
    int rc = nlm_fd_get_state(h, u, nullptr, nullptr);
    if (rc) return rc;
  }
  if (force) {
    const int64_t n = h->n;
    std::vector<double> fi((size_t)q->m), vol(n);
    NLM_CUDA(cudaMemcpyAsync(fi.data(), q->f, sizeof(double) * q->m, cudaMemcpyDeviceToHost, h->stream));
    NLM_CUDA(cudaMemcpyAsync(vol.data(), h->D.vol64, sizeof(double) * n, cudaMemcpyDeviceToHost, h->stream));
    NLM_CUDA(cudaStreamSynchronize(h->stream));
    for (int64_t i = 0; i < n; i++) {
      const int64_t o = h->perm[i];
      for (int d = 0; d < 3; d++) {
        const double fd = (d < h->S && d < q->mdim) ? fi[(size_t)h->S * i + d] : 0.;
        force[3 * o + d] = fd * vol[i];
      }
    }
  }
  return NLM_OK;
}

}  // extern "C"

