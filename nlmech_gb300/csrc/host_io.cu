// host_io.cu -- nlm_fd_step_host: the drop-in step on the caller's host
// arrays (copies through device staging, in-place reads and writes of
// page-locked arrays, and the banded path whose copies overlap the step).

#include "fd_handle.h"

namespace nlm {

// Pinned caller arrays read in place.  The caller's arrays are taken as flat
// sequences of 3n doubles, two per thread with 16-byte loads, so every byte
// crosses the host link once in full lines.  Value k is component k % 3 of
// caller node k / 3; it goes into a staging copy of the state array in the
// internal order (FP32C: its (hi, lo) floats), or, for a component the model
// does not hold (z in 2-D), into zkeep in the caller's order.
template <bool FP32>
__device__ __forceinline__ void stage_value(int S, int dim, int64_t i, int d, double x, void *dst,
                                            double *zkeep, int64_t k) {
  if (d >= dim) {
    if (zkeep) zkeep[k / 3] = x;
    return;
  }
  if (FP32) {
    float *q = static_cast<float *>(dst);
    const float hi = __double2float_rn(x), lo = __double2float_rn(x - (double)hi);
    if (S == 2) {
      q[4 * i + d] = hi;
      q[4 * i + 2 + d] = lo;
    } else {
      q[8 * i + d] = hi;
      q[8 * i + 4 + d] = lo;
    }
  } else {
    static_cast<double *>(dst)[S * i + d] = x;
  }
}

template <bool FP32>
__global__ void k_host_in(int64_t n, int S, int dim, const int *iperm, const double2 *hu,
                          const double2 *hv, const double2 *hf, void *su, void *sv, void *sf,
                          double *zu, double *zv, int *bad) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (2 * t >= 3 * n) return;
  const double2 a = hu[t], b = hv[t], c = hf[t];
  if (!(isfinite(a.x) && isfinite(a.y) && isfinite(b.x) && isfinite(b.y) && isfinite(c.x) &&
        isfinite(c.y)))
    atomicExch(bad, 1);
  for (int h = 0; h < 2; h++) {
    const int64_t k = 2 * t + h;
    const int64_t o = k / 3;
    const int d = (int)(k - 3 * o);
    const int64_t i = iperm[o];
    stage_value<FP32>(S, dim, i, d, h ? a.y : a.x, su, zu, k);
    stage_value<FP32>(S, dim, i, d, h ? b.y : b.x, sv, zv, k);
    if (d < dim) {
      if (FP32)
        static_cast<float *>(sf)[S * i + d] = (float)(h ? c.y : c.x);
      else
        static_cast<double *>(sf)[S * i + d] = h ? c.y : c.x;
    }
  }
}

// The state written into the pinned caller arrays in place, two doubles per
// thread with 16-byte stores: the model's components of u and v, their z in
// 2-D from zkeep (the caller's own values, which the reference's 2-D
// integrator never changes), and f with z = 0 in 2-D (the reference resets f
// every step).
template <bool FP32>
__device__ __forceinline__ double state_value(int S, int64_t i, int d, const void *src) {
  if (FP32) {
    const float *q = static_cast<const float *>(src);
    if (S == 2) return (double)q[4 * i + d] + (double)q[4 * i + 2 + d];
    return (double)q[8 * i + d] + (double)q[8 * i + 4 + d];
  }
  return static_cast<const double *>(src)[S * i + d];
}

template <bool FP32>
__global__ void k_host_out(int64_t n, int S, int dim, const int *iperm, const void *u,
                           const void *v, const void *f, const double *zu, const double *zv,
                           double2 *hu, double2 *hv, double2 *hf) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (2 * t >= 3 * n) return;
  double a[2], b[2], c[2];
  for (int h = 0; h < 2; h++) {
    const int64_t k = 2 * t + h;
    const int64_t o = k / 3;
    const int d = (int)(k - 3 * o);
    const int64_t i = iperm[o];
    if (d < dim) {
      a[h] = state_value<FP32>(S, i, d, u);
      b[h] = state_value<FP32>(S, i, d, v);
      c[h] = FP32 ? (double)static_cast<const float *>(f)[S * i + d]
                  : static_cast<const double *>(f)[S * i + d];
    } else {
      a[h] = zu[o];
      b[h] = zv[o];
      c[h] = 0.;
    }
  }
  hu[t] = make_double2(a[0], a[1]);
  hv[t] = make_double2(b[0], b[1]);
  hf[t] = make_double2(c[0], c[1]);
}


}  // namespace nlm

namespace {

typedef int (*PtrAttrFn)(void *, int, unsigned long long);

// The driver's cuPointerGetAttribute, looked up through the runtime (no link
// dependency on the driver library).
PtrAttrFn ptr_attr_fn() {
  static PtrAttrFn fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuPointerGetAttribute", &f, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PtrAttrFn>(f);
    else
      cudaGetLastError();
  }
  return fn;
}

// True when [p, p + bytes) lies inside one page-locked host allocation that
// the device addresses at the same virtual address, so kernels may read and
// write it in place.
bool in_place_ok(const void *p, size_t bytes) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (a.type != cudaMemoryTypeHost || a.devicePointer != p) return false;
  PtrAttrFn fn = ptr_attr_fn();
  if (!fn) return false;
  unsigned long long start = 0;
  size_t size = 0;
  if (fn(&start, 11 /* CU_POINTER_ATTRIBUTE_RANGE_START_ADDR */, (unsigned long long)p) != 0 ||
      fn(&size, 12 /* CU_POINTER_ATTRIBUTE_RANGE_SIZE */, (unsigned long long)p) != 0)
    return false;
  const unsigned long long q = (unsigned long long)p;
  return size > 0 && q >= start && q + bytes <= start + size;
}

// Caller -> internal node ids, built on first use.
int ensure_iperm(nlm_fd *h) {
  if (h->iperm) return NLM_OK;
  if (h->alloc(&h->iperm, h->n) != cudaSuccess) return fail(NLM_ERR_OOM, "host I/O index");
  k_invert_perm<<<nblk(h->n, 256), 256, 0, h->stream>>>(h->n, h->D.perm_dev, h->iperm);
  NLM_CUDA(cudaGetLastError());
  return NLM_OK;
}

// Banded host step: at least kPipeMinNodes nodes.  Band sizes ramp 1, 2, 4
// units up, stay at 8 units (about kPipeMidBand nodes: a few MB per array
// and copy, where a copy's fixed cost is small) and ramp 4, 2, 1 down, so the
// first bands arrive and the last go out quickly.
constexpr int64_t kPipeMinNodes = 1 << 16;
constexpr int64_t kPipeMidBand = 1 << 18;
constexpr int64_t kPipeLateDiv = 32;

// The banded step covers one FP32C velocity-Verlet step of a 2-D RNPBond
// model on a tile decomposition, with no per-launch timing and no timed
// crack to cut first; other calls take the whole-state path.
bool pipe_usable(const nlm_fd *h, int64_t nsteps) {
  return nsteps == 1 && h->pipe_state >= 0 && h->precision == NLM_PREC_FP32C && h->dim == 2 &&
         h->scheme == NLM_VELOCITY_VERLET && h->material == NLM_MAT_RNP_BOND && h->tile_ok &&
         (h->decomp == NLM_DECOMP_TILE || h->decomp == NLM_DECOMP_TILE_LOCAL) && !h->timing &&
         h->n >= kPipeMinNodes && !h->D.qtab &&
         (h->timed_cracks.empty() || !crack_due(h, 1));
}

// Frees what pipe_setup allocated or created, so a failed set-up leaves the
// handle as it was before.
void pipe_teardown(nlm_fd *h) {
  if (h->pipe_sin) cudaStreamSynchronize(h->pipe_sin);
  if (h->pipe_sout) cudaStreamSynchronize(h->pipe_sout);
  for (auto e : h->pipe_ev) cudaEventDestroy(e);
  h->pipe_ev.clear();
  if (h->pipe_sin) cudaStreamDestroy(h->pipe_sin);
  if (h->pipe_sout) cudaStreamDestroy(h->pipe_sout);
  h->pipe_sin = h->pipe_sout = nullptr;
  h->release(&h->pipe_tiles);
  h->release(&h->pipe_in);
  h->release(&h->pipe_back);
  h->release(&h->pipe_ua);
  h->release(&h->pipe_ub);
  h->release(&h->pipe_v);
  h->release(&h->pipe_f);
  h->release(&h->pipe_bits);
  h->release(&h->pipe_late);
  h->pipe_nbands = 0;
}

// Band schedule and buffers of the banded step.  Tile t can run once every
// band up to the one holding caller node tile_need[t] is on the device: its
// stage is that band.  A node is final after the stage of its tile.  Band b
// goes out after the first stage k >= b by which all but at most
// (its size) / kPipeLateDiv of its nodes are final;
// those late nodes (tiles that straddle a jump of the Morton order, mostly)
// are written into the caller's arrays directly once every band is out.
int pipe_setup(nlm_fd *h) {
  const int64_t n = h->n, nt = (n + kTileNodes - 1) / kTileNodes;
  if ((int64_t)h->tile_need.size() != nt) {
    h->pipe_state = -1;
    return NLM_OK;
  }
  const int64_t unit = kPipeMidBand / 8;
  const int64_t mid = std::max<int64_t>(0, (n - 14 * unit + 4 * unit) / (8 * unit));
  std::vector<int64_t> w = {1, 2, 4};
  for (int64_t k = 0; k < mid; k++) w.push_back(8);
  for (int64_t x : {4, 2, 1}) w.push_back(x);
  int64_t wsum = 0;
  for (int64_t x : w) wsum += x;
  const int K = (int)w.size();
  std::vector<int64_t> bounds(K + 1, 0);
  for (int b = 0, acc = 0; b < K; b++) {
    acc += (int)w[b];
    bounds[b + 1] = b + 1 == K ? n : (int64_t)((double)n * acc / wsum);
  }
  auto band_of = [&](int64_t o) {
    return (int)(std::upper_bound(bounds.begin(), bounds.end(), o) - bounds.begin()) - 1;
  };
  std::vector<int> stage(nt);
  std::vector<int> count(K + 1, 0);
  for (int64_t t = 0; t < nt; t++) {
    stage[t] = std::min(K - 1, band_of(std::max(0, h->tile_need[t])));
    count[stage[t] + 1]++;
  }
  for (int k = 0; k < K; k++) count[k + 1] += count[k];
  h->pipe_toff = count;
  std::vector<int> tiles(std::max<int64_t>(1, nt));
  for (int64_t t = 0; t < nt; t++) tiles[count[stage[t]]++] = (int)t;
  // hist[b K + k]: nodes of band b final after stage k
  std::vector<int64_t> hist((size_t)K * K, 0);
  std::vector<int> cband(n);
  for (int64_t i = 0; i < n; i++) {
    cband[i] = band_of(h->perm[i]);
    hist[(size_t)cband[i] * K + stage[i / kTileNodes]]++;
  }
  std::vector<int> release(K, K - 1);
  for (int b = 0; b < K; b++) {
    const int64_t cap = (bounds[b + 1] - bounds[b]) / kPipeLateDiv;
    int64_t later = 0;
    for (int k = K - 1; k >= b; k--) {
      if (later + hist[(size_t)b * K + k] > cap) {
        release[b] = k;
        break;
      }
      later += hist[(size_t)b * K + k];
      release[b] = k - 1;
    }
    release[b] = std::max(release[b], b);
  }
  h->pipe_out.assign(K, {});
  for (int b = 0; b < K; b++) h->pipe_out[release[b]].push_back(b);
  std::vector<int> late;
  for (int64_t i = 0; i < n; i++)
    if (stage[i / kTileNodes] > release[cband[i]]) late.push_back(h->perm[i]);
  std::sort(late.begin(), late.end());
  h->pipe_nlate = (int64_t)late.size();
  if (int rc = ensure_iperm(h)) return rc;
  const size_t nbits = (size_t)h->P.nwords * h->P.npad;
  if (h->alloc(&h->pipe_tiles, tiles.size()) != cudaSuccess ||
      h->alloc(&h->pipe_in, (size_t)9 * n) != cudaSuccess ||
      h->alloc(&h->pipe_back, (size_t)9 * n) != cudaSuccess ||
      h->alloc(&h->pipe_ua, n) != cudaSuccess || h->alloc(&h->pipe_ub, n) != cudaSuccess ||
      h->alloc(&h->pipe_v, n) != cudaSuccess || h->alloc(&h->pipe_f, n) != cudaSuccess ||
      h->alloc(&h->pipe_bits, nbits) != cudaSuccess ||
      h->alloc(&h->pipe_late, std::max<size_t>(1, late.size())) != cudaSuccess)
    return fail(NLM_ERR_OOM, "banded host step buffers");
  NLM_CUDA(cudaMemcpyAsync(h->pipe_tiles, tiles.data(), sizeof(int) * tiles.size(),
                           cudaMemcpyHostToDevice, h->stream));
  if (!late.empty())
    NLM_CUDA(cudaMemcpyAsync(h->pipe_late, late.data(), sizeof(int) * late.size(),
                             cudaMemcpyHostToDevice, h->stream));
  NLM_CUDA(cudaStreamSynchronize(h->stream));
  NLM_CUDA(cudaStreamCreateWithFlags(&h->pipe_sin, cudaStreamNonBlocking));
  NLM_CUDA(cudaStreamCreateWithFlags(&h->pipe_sout, cudaStreamNonBlocking));
  for (int k = 0; k < 2 * K + 1; k++) {
    cudaEvent_t e;
    NLM_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    h->pipe_ev.push_back(e);
  }
  h->pipe_nbands = K;
  h->pipe_bounds = bounds;
  h->pipe_state = 1;
  return NLM_OK;
}

// One step of nlm_fd_step_host on page-locked arrays, banded: the copy-in of
// later bands, the step of the tiles they release and the copy-out of
// finished bands overlap, so both directions of the host link carry traffic
// at once.  The step writes scratch arrays; they become the state only if
// every input value was finite.  Otherwise the bond bits are put back, the
// caller's arrays are restored from the staged input and the call fails with
// the model unchanged.
int step_host_banded(nlm_fd *h, double *u, double *v, double *f) {
  const int64_t n = h->n;
  const int K = h->pipe_nbands;
  const std::vector<int64_t> &bd = h->pipe_bounds;
  cudaStream_t s = h->stream, si = h->pipe_sin, so = h->pipe_sout;
  const double tm = h->time + h->dt;
  const int c = 1 - h->cur;  // ping index of u at the step's time
  DevPtrs Dp = h->D;
  Dp.u32[c] = h->pipe_ua;
  Dp.u32[1 - c] = h->pipe_ub;
  Dp.v32[0] = h->pipe_v;
  Dp.f32 = reinterpret_cast<float *>(h->pipe_f);
  double *in_u = h->pipe_in, *in_v = in_u + 3 * n, *in_f = in_v + 3 * n;
  double *bk_u = h->pipe_back, *bk_v = bk_u + 3 * n, *bk_f = bk_v + 3 * n;
  double *host[3] = {u, v, f}, *in[3] = {in_u, in_v, in_f}, *bk[3] = {bk_u, bk_v, bk_f};
  const size_t nbits = (size_t)h->P.nwords * h->P.npad;
  // the input stream starts once earlier work on the handle's stream is done
  NLM_CUDA(cudaEventRecord(h->pipe_ev[0], s));
  NLM_CUDA(cudaStreamWaitEvent(si, h->pipe_ev[0], 0));
  // copy-in of band b, issued one band ahead of the stage that needs it
  auto copy_in = [&](int b) -> int {
    const int64_t o0 = bd[b], o1 = bd[b + 1];
    for (int a = 0; a < 3; a++)
      NLM_CUDA(cudaMemcpyAsync(in[a] + 3 * o0, host[a] + 3 * o0, sizeof(double) * 3 * (o1 - o0),
                               cudaMemcpyHostToDevice, si));
    NLM_CUDA(cudaEventRecord(h->pipe_ev[2 * b], si));
    return NLM_OK;
  };
  for (int b = 0; b < std::min(K, 2); b++)
    if (int rc = copy_in(b)) return rc;
  NLM_CUDA(cudaMemsetAsync(h->bad_input, 0, sizeof(int), s));
  NLM_CUDA(cudaMemcpyAsync(h->pipe_bits, h->D.bits, sizeof(uint32_t) * nbits,
                           cudaMemcpyDeviceToDevice, s));
  if (int rc = apply_fbc(h, tm)) return rc;
  for (int k = 0; k < K; k++) {
    const int64_t o0 = bd[k], o1 = bd[k + 1];
    if (k + 2 < K)
      if (int rc = copy_in(k + 2)) return rc;
    NLM_CUDA(cudaStreamWaitEvent(s, h->pipe_ev[2 * k], 0));
    NLM_CUDA(launch_pipe_in32(h->P, Dp, h->T, tm, o0, o1, h->iperm, in_u, in_v, in_f, h->pipe_ua,
                              h->pipe_v, h->pipe_f, h->bad_input, s));
    const int nk = h->pipe_toff[k + 1] - h->pipe_toff[k];
    if (nk > 0) {
      StepArgs a{c, false, tm, tm + h->dt, nullptr, 0, n, h->pipe_tiles + h->pipe_toff[k], nk};
      const cudaError_t e = launch_rnp_step_fp32(h->P, Dp, h->T, a, h->decomp, s);
      if (e != cudaSuccess) return cuda_fail(e, "step kernel launch");
    }
    for (int b : h->pipe_out[k]) {
      const int64_t p0 = bd[b], p1 = bd[b + 1];
      NLM_CUDA(launch_pipe_out32(p0, p1, nullptr, h->iperm, h->pipe_ua, h->pipe_v, h->pipe_f,
                                 in_u, in_v, bk_u, bk_v, bk_f, s));
      NLM_CUDA(cudaEventRecord(h->pipe_ev[2 * b + 1], s));
      NLM_CUDA(cudaStreamWaitEvent(so, h->pipe_ev[2 * b + 1], 0));
      for (int a = 0; a < 3; a++)
        NLM_CUDA(cudaMemcpyAsync(host[a] + 3 * p0, bk[a] + 3 * p0, sizeof(double) * 3 * (p1 - p0),
                                 cudaMemcpyDeviceToHost, so));
    }
  }
  // the late nodes, written into the caller's arrays once every band's copy
  // (which carried their values from before their tiles ran) has landed
  if (h->pipe_nlate > 0) {
    NLM_CUDA(cudaEventRecord(h->pipe_ev[2 * K], so));
    NLM_CUDA(cudaStreamWaitEvent(s, h->pipe_ev[2 * K], 0));
    NLM_CUDA(launch_pipe_out32(0, h->pipe_nlate, h->pipe_late, h->iperm, h->pipe_ua, h->pipe_v,
                               h->pipe_f, in_u, in_v, u, v, f, s));
  }
  NLM_CUDA(launch_pipe_commit32(n, (int64_t)nbits, h->bad_input, h->pipe_ua, h->pipe_ub,
                                h->pipe_v, h->pipe_f, h->D.u32[c], h->D.u32[1 - c], h->D.v32[0],
                                reinterpret_cast<float2 *>(h->D.f32), h->D.bits, h->pipe_bits, s));
  int bad = 0;
  NLM_CUDA(cudaMemcpyAsync(&bad, h->bad_input, sizeof(int), cudaMemcpyDeviceToHost, s));
  NLM_CUDA(cudaStreamSynchronize(s));
  NLM_CUDA(cudaStreamSynchronize(so));
  if (bad) {
    for (int a = 0; a < 3; a++)
      NLM_CUDA(cudaMemcpyAsync(host[a], in[a], sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, s));
    NLM_CUDA(cudaStreamSynchronize(s));
    return fail(NLM_ERR_NONFINITE, "non-finite state");
  }
  h->cur = c;
  h->time = tm;
  h->step++;
  h->host_io = 2;
  return NLM_OK;
}

// nlm_fd_step_host with u, v, f read and written in place by kernels (one
// pass each way over the host link), the state replaced only once the input
// is known to be finite.
int step_host_in_place(nlm_fd *h, double *u, double *v, double *f, int64_t nsteps) {
  const int64_t n = h->n;
  const int S = h->S;
  cudaStream_t s = h->stream;
  const bool fp32 = h->precision == NLM_PREC_FP32C;
  if (int rc = ensure_iperm(h)) return rc;
  if (!h->zstage) {
    if (h->alloc(&h->zstage, (size_t)24 * S * n + 16 * n) != cudaSuccess)
      return fail(NLM_ERR_OOM, "in-place host I/O buffers");
    // padding entries of the staged layouts are never written: zero them once
    NLM_CUDA(cudaMemsetAsync(h->zstage, 0, (size_t)24 * S * n + 16 * n, s));
  }
  const size_t bu = fp32 ? sizeof(float4) * (S / 2) * n : sizeof(double) * S * n;
  const size_t bf = fp32 ? sizeof(float) * S * n : sizeof(double) * S * n;
  char *su = h->zstage, *sv = su + bu, *sf = sv + bu;
  double *zu = reinterpret_cast<double *>(h->zstage + (size_t)24 * S * n), *zv = zu + n;
  const int64_t pairs = (3 * n + 1) / 2;
  const double2 *u2 = reinterpret_cast<const double2 *>(u);
  const double2 *v2 = reinterpret_cast<const double2 *>(v);
  const double2 *f2 = reinterpret_cast<const double2 *>(f);
  NLM_CUDA(cudaMemsetAsync(h->bad_input, 0, sizeof(int), s));
  if (fp32)
    k_host_in<true><<<nblk(pairs, 256), 256, 0, s>>>(n, S, h->dim, h->iperm, u2, v2, f2, su, sv,
                                                     sf, zu, zv, h->bad_input);
  else
    k_host_in<false><<<nblk(pairs, 256), 256, 0, s>>>(n, S, h->dim, h->iperm, u2, v2, f2, su, sv,
                                                      sf, zu, zv, h->bad_input);
  NLM_CUDA(cudaGetLastError());
  int bad = 0;
  NLM_CUDA(cudaMemcpyAsync(&bad, h->bad_input, sizeof(int), cudaMemcpyDeviceToHost, s));
  NLM_CUDA(cudaStreamSynchronize(s));
  if (bad) return fail(NLM_ERR_NONFINITE, "non-finite state");
  void *du = fp32 ? (void *)h->D.u32[h->cur] : (void *)h->D.u64[h->cur];
  void *dv = fp32 ? (void *)h->D.v32[h->vidx()] : (void *)h->D.v[h->vidx()];
  void *df_ = fp32 ? (void *)h->D.f32 : (void *)h->D.f64;
  NLM_CUDA(cudaMemcpyAsync(du, su, bu, cudaMemcpyDeviceToDevice, s));
  NLM_CUDA(cudaMemcpyAsync(dv, sv, bu, cudaMemcpyDeviceToDevice, s));
  NLM_CUDA(cudaMemcpyAsync(df_, sf, bf, cudaMemcpyDeviceToDevice, s));
  cudaError_t e = launch_drift(h->P, h->D, h->T, h->cur, h->time + h->dt, fp32, s);
  if (e != cudaSuccess) return cuda_fail(e, "drift kernel");
  int rc = do_run(h, nsteps);
  if (rc) return rc;
  const void *ou = fp32 ? (const void *)h->D.u32[h->cur] : (const void *)h->D.u64[h->cur];
  const void *ov = fp32 ? (const void *)h->D.v32[h->vidx()] : (const void *)h->D.v[h->vidx()];
  const void *of = fp32 ? (const void *)h->D.f32 : (const void *)h->D.f64;
  double2 *u2o = reinterpret_cast<double2 *>(u), *v2o = reinterpret_cast<double2 *>(v);
  double2 *f2o = reinterpret_cast<double2 *>(f);
  if (fp32)
    k_host_out<true><<<nblk(pairs, 256), 256, 0, s>>>(n, S, h->dim, h->iperm, ou, ov, of, zu, zv,
                                                      u2o, v2o, f2o);
  else
    k_host_out<false><<<nblk(pairs, 256), 256, 0, s>>>(n, S, h->dim, h->iperm, ou, ov, of, zu,
                                                       zv, u2o, v2o, f2o);
  NLM_CUDA(cudaGetLastError());
  NLM_CUDA(cudaStreamSynchronize(s));
  h->host_io = 1;
  return NLM_OK;
}

}  // namespace

extern "C" {

int nlm_fd_set_alloc_limit(nlm_fd *h, int64_t bytes) {
  if (!h) return fail(NLM_ERR_INVALID, "null handle");
  h->alloc_budget = bytes < 0 ? -1 : bytes;
  return NLM_OK;
}

int nlm_fd_host_io(const nlm_fd *h, int *mode) {
  if (!h || !mode) return fail(NLM_ERR_INVALID, "null argument");
  *mode = h->host_io;
  return NLM_OK;
}

int nlm_fd_step_host(nlm_fd *h, double *u, double *v, double *f, int64_t nsteps) {
  if (!h || !u || !v || !f || nsteps < 0) return fail(NLM_ERR_INVALID, "null argument");
  if (!h->started) {
    int rc = nlm_fd_set_state(h, u, v);
    if (rc) return rc;
    if ((rc = do_run(h, nsteps))) return rc;
    return get_state_impl(h, u, v, f, true);
  }
  const int64_t n = h->n;
  const size_t bytes = sizeof(double) * 3 * n;
  // in place: page-locked arrays on 16-byte boundaries holding an even
  // number of doubles (whole 16-byte pairs)
  const bool aligned = ((uintptr_t)u | (uintptr_t)v | (uintptr_t)f) % 16 == 0 && n % 2 == 0;
  if (aligned && in_place_ok(u, bytes) && in_place_ok(v, bytes) && in_place_ok(f, bytes)) {
    if (pipe_usable(h, nsteps)) {
      // if the banded path's buffers cannot be allocated, what it had set up
      // is freed and the in-place path below serves this and every later
      // call, with the same results; any other set-up error is returned
      if (h->pipe_state == 0) {
        const int rc = pipe_setup(h);
        if (rc != NLM_OK) {
          pipe_teardown(h);
          cudaGetLastError();
          if (rc != NLM_ERR_OOM) return rc;
          h->pipe_state = -1;
          set_error("");
        }
      }
      if (h->pipe_state == 1) return step_host_banded(h, u, v, f);
    }
    return step_host_in_place(h, u, v, f, nsteps);
  }
  h->host_io = 0;
  cudaStream_t s = h->stream;
  const int *P = h->D.perm_dev;
  const unsigned g = nblk(n, 256);
  const bool fp32 = h->precision == NLM_PREC_FP32C;
  // upload u, v, f into their staging slots, check them for non-finite
  // values on the device, and only then replace the state
  double *su = h->stage, *sv = h->stage + 3 * n, *sf = h->stage + 6 * n;
  NLM_CUDA(cudaMemsetAsync(h->bad_input, 0, sizeof(int), s));
  NLM_CUDA(cudaMemcpyAsync(su, u, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s));
  NLM_CUDA(cudaMemcpyAsync(sv, v, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s));
  NLM_CUDA(cudaMemcpyAsync(sf, f, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s));
  k_nonfinite<<<nblk(9 * n, 256), 256, 0, s>>>(9 * n, h->stage, h->bad_input);
  NLM_CUDA(cudaGetLastError());
  int bad = 0;
  NLM_CUDA(cudaMemcpyAsync(&bad, h->bad_input, sizeof(int), cudaMemcpyDeviceToHost, s));
  NLM_CUDA(cudaStreamSynchronize(s));
  if (bad) return fail(NLM_ERR_NONFINITE, "non-finite state");
  if (fp32) {
    k_scatter_split<<<g, 256, 0, s>>>(n, h->S, h->dim, P, su, h->D.u32[h->cur]);
    k_scatter_split<<<g, 256, 0, s>>>(n, h->S, h->dim, P, sv, h->D.v32[h->vidx()]);
    k_scatter_f32<<<g, 256, 0, s>>>(n, h->S, h->dim, P, sf, h->D.f32);
  } else {
    k_scatter_vec<<<g, 256, 0, s>>>(n, h->S, h->dim, P, su, h->D.u64[h->cur]);
    k_scatter_vec<<<g, 256, 0, s>>>(n, h->S, h->dim, P, sv, h->D.v[h->vidx()]);
    k_scatter_vec<<<g, 256, 0, s>>>(n, h->S, h->dim, P, sf, h->D.f64);
  }
  NLM_CUDA(cudaGetLastError());
  cudaError_t e = launch_drift(h->P, h->D, h->T, h->cur, h->time + h->dt, fp32, s);
  if (e != cudaSuccess) return cuda_fail(e, "drift kernel");
  int rc = do_run(h, nsteps);
  if (rc) return rc;
  return get_state_impl(h, u, v, f, true);
}

int nlm_fd_set_graph(nlm_fd *h, int steps_per_graph) {
  if (!h || steps_per_graph < 0 || (steps_per_graph % 2) || steps_per_graph == 1)
    return fail(NLM_ERR_INVALID, "steps_per_graph must be 0 or an even number >= 2");
  NLM_CUDA(cudaStreamSynchronize(h->stream));
  for (auto &g : h->gexec)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
  if (h->h_times) {
    cudaFreeHost(h->h_times);
    h->h_times = nullptr;
  }
  h->graph_steps = steps_per_graph;
  if (steps_per_graph > 0) {
    NLM_CUDA(cudaMallocHost(&h->h_times, sizeof(double) * (steps_per_graph + 1)));
    if (h->alloc(&h->d_times, (size_t)steps_per_graph + 1) != cudaSuccess)
      return fail(NLM_ERR_OOM, "graph time buffer");
    if (!h->ev_times) NLM_CUDA(cudaEventCreateWithFlags(&h->ev_times, cudaEventDisableTiming));
    NLM_CUDA(cudaEventRecord(h->ev_times, h->stream));
  }
  return NLM_OK;
}

int nlm_fd_run_timed(nlm_fd *h, int64_t nsteps, double *ms) {
  if (!h || !ms || nsteps < 0) return fail(NLM_ERR_INVALID, "bad arguments");
  cudaEvent_t a, b;
  NLM_CUDA(cudaEventCreate(&a));
  NLM_CUDA(cudaEventCreate(&b));
  cudaEventRecord(a, h->stream);
  int rc = do_run(h, nsteps);
  cudaEventRecord(b, h->stream);
  cudaError_t e = cudaEventSynchronize(b);
  float t = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&t, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (rc) return rc;
  if (e != cudaSuccess) return cuda_fail(e, "run timing");
  *ms = t;
  return NLM_OK;
}

}  // extern "C"

