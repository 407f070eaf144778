// fd_handle.h -- what the host units of libnlmgpu share: the nlm_fd handle
// (one FDModel<T> and its DataManager), the error helpers, the deck-level
// set-up restated from the reference's loading classes, the small data
// movement kernels and the model functions the other units call.
#pragma once


#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include <cuda_fp16.h>

#include "fd_internal.h"
#include "neighbor.h"
#include "qs_internal.h"
#include "esqs_internal.h"
#include "fp32_common.cuh"
#include "state_io.cuh"

namespace nlm {

// ---- errors (host_common.cu): the thread's last error text --------------
void set_error(const std::string &msg);
const char *last_error();
int cuda_fail(cudaError_t e, const char *what);
int fail(int code, const std::string &msg);

inline unsigned nblk(int64_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

// ---- deck-level set-up (host_common.cu) ------------------------------------
inline bool hGT(double a, double b) { return (a - b) > (amax_d(a, b) * 1e-5); }
inline bool hLT(double a, double b) { return (b - a) > (amax_d(a, b) * 1e-5); }
bool in_region(const nlm_bc_set &bc, const double *p, int dim);
double uload_umax(const nlm_bc_set &bc, const double *x);
double fload_spatial(const nlm_bc_set &bc, const double *x, double h);

// ---- small kernels (fd_kernels.cu) ---------------------------------------
struct FBCItem {
  int set;
  int dir_mask;
  double spatial;
};


__device__ inline void ld_split_any(const float4 *p, int S, int64_t i, double o[3]) {
  if (S == 2) {
    const float4 a = p[i];
    o[0] = (double)a.x + (double)a.z;
    o[1] = (double)a.y + (double)a.w;
    o[2] = 0.;
  } else {
    const float4 a = p[2 * i], b = p[2 * i + 1];
    o[0] = (double)a.x + (double)b.x;
    o[1] = (double)a.y + (double)b.y;
    o[2] = (double)a.z + (double)b.z;
  }
}
__device__ inline void st_split_any(float4 *p, int S, int64_t i, const double v[3]) {
  float h[3], l[3];
  for (int d = 0; d < 3; d++) {
    h[d] = __double2float_rn(v[d]);
    l[d] = __double2float_rn(v[d] - (double)h[d]);
  }
  if (S == 2)
    p[i] = make_float4(h[0], h[1], l[0], l[1]);
  else {
    p[2 * i] = make_float4(h[0], h[1], h[2], 0.f);
    p[2 * i + 1] = make_float4(l[0], l[1], l[2], 0.f);
  }
}

__global__ void k_fbc_apply(int64_t nf, int S, const int *nodes, const int *iptr,
                            const FBCItem *items, BCTable T, double time, double *fext,
                            const double *tdev = nullptr);
__global__ void k_bc_apply(int64_t nb, int S, int dim, const int *nodes, const int *bcref,
                           const BCEntry *bce, const uint8_t *flags, BCTable T, double time,
                           double *u64, float4 *u32, double *v, float4 *v32);
__global__ void k_scatter_vec(int64_t n, int S, int dim, const int *perm, const double *src,
                              double *dst);
__global__ void k_invert_perm(int64_t n, const int *perm, int *iperm);
__global__ void k_nonfinite(int64_t m, const double *a, int *flag);
__global__ void k_scatter_split(int64_t n, int S, int dim, const int *perm, const double *src,
                                float4 *dst);
__global__ void k_scatter_f32(int64_t n, int S, int dim, const int *perm, const double *src,
                              float *dst);
__global__ void k_gather_vec(int64_t n, int S, const int *perm, const double *src, double *dst,
                             bool keep_z = false);
__global__ void k_gather_split(int64_t n, int S, const int *perm, const float4 *src, double *dst,
                               bool keep_z = false);
__global__ void k_gather_f32(int64_t n, int S, const int *perm, const float *src, double *dst);
__global__ void k_make_pos32(int64_t n, int S, const double *pos, const double *vol, double scale,
                             float4 *pos32, uint2 *pos32lo);
__global__ void k_count_bits(int64_t n, int nwords, int64_t npad, const uint32_t *bits,
                             unsigned long long *out);

}  // namespace nlm

using namespace nlm;

// ---- the handle ----------------------------------------------------------
struct nlm_fd {
  int dim = 2, S = 2;
  int64_t n = 0, nnz = 0;
  int precision = NLM_PREC_FP64, scheme = NLM_VELOCITY_VERLET, decomp = NLM_DECOMP_THREAD;
  int material = NLM_MAT_RNP_BOND;
  double dt = 0., time = 0.;
  int64_t step = 0;
  bool started = false;
  int cur = 0;
  bool rows_by_orig = true;  // device rows ordered by original id
  StepParams P{};
  BCTable T{};
  cudaStream_t stream = nullptr;
  std::vector<void *> allocs;
  DevPtrs D{};
  int64_t nslices = 0, sell_entries = 0;
  bool tile_ok = false;  // tile store built (NLM_DECOMP_TILE available)
  // lattice residue (g_x mod 4, g_y mod 2 as a Morton code) of each node of
  // a lattice-renumbered model, for the tile store's halo slots
  std::vector<uint8_t> lattice_res;
  // host copies
  std::vector<int> perm;    // internal -> original
  std::vector<int64_t> rowptr;  // internal CSR offsets (host copy)
  // loads
  int *bc_nodes = nullptr;
  int64_t n_bc_nodes = 0;
  int *fbc_nodes = nullptr, *fbc_iptr = nullptr;
  FBCItem *fbc_items = nullptr;
  int64_t n_fbc_nodes = 0;
  BCTable FT{};
  double bbox_lo[3] = {0., 0., 0.}, bbox_hi[3] = {0., 0., 0.};  // fe::Mesh::computeBBox
  // timed cracks (Fracture::addCrack): cut after a step, bit c of cracks_on set once cut
  std::vector<nlm_crack> timed_cracks;
  uint32_t cracks_on = 0;
  // staging
  double *stage = nullptr;   // 3 slots of 3n doubles (u, v, f in Point3 layout)
  int *bad_input = nullptr;  // set by k_nonfinite
  int *iperm = nullptr;      // original -> internal node id (in-place host I/O)
  char *zstage = nullptr;    // state-layout staging of in-place host input
  int host_io = 0;           // last nlm_fd_step_host: 0 copies, 1 in place, 2 banded
  // banded host step: the caller's arrays move in contiguous bands on the copy
  // engines, each band's arrival releases the tiles whose nodes and halo it
  // completes, and a band goes back out once all tiles owning its nodes ran
  std::vector<int> tile_need;  // per tile: highest caller index its step reads
  int pipe_state = 0;          // 0 not set up, 1 ready, -1 unavailable
  int pipe_nbands = 0;
  std::vector<int64_t> pipe_bounds;  // band b = caller nodes [bounds[b], bounds[b + 1])
  std::vector<int> pipe_toff;  // stage k runs pipe_tiles[toff[k] .. toff[k + 1])
  std::vector<std::vector<int>> pipe_out;  // bands written back after stage k
  int *pipe_tiles = nullptr;
  int *pipe_late = nullptr;    // caller nodes final only after their band went out
  int64_t pipe_nlate = 0;
  double *pipe_in = nullptr, *pipe_back = nullptr;  // staged u, v, f: 9 n doubles each
  float4 *pipe_ua = nullptr, *pipe_ub = nullptr, *pipe_v = nullptr;
  float2 *pipe_f = nullptr;
  uint32_t *pipe_bits = nullptr;
  cudaStream_t pipe_sin = nullptr, pipe_sout = nullptr;
  std::vector<cudaEvent_t> pipe_ev;  // per band: input arrived, output ready
  float *dmg_phi = nullptr, *dmg_Z = nullptr;
  float *en_buf = nullptr;     // nlm_fd_energies: 4 n floats
  double *en_fext = nullptr;   // external force at the current time, S n doubles
  double *rf_buf = nullptr;    // nlm_fd_reaction_force: 2 n doubles
  unsigned long long *counter = nullptr;
  // CUDA-graph replay of the step loop
  int graph_steps = 0;
  cudaGraphExec_t gexec[2] = {nullptr, nullptr};  // by starting ping index
  double *d_times = nullptr, *h_times = nullptr;  // device / pinned host
  cudaEvent_t ev_times = nullptr;
  bool capturing = false;
  // timing
  bool timing = false;
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_used = 0;
  double acc_ms = 0.;
  int64_t launches = 0;
  double bytes_per_launch = 0.;

  int vidx() const { return scheme == NLM_CENTRAL_DIFFERENCE ? cur : 0; }

  // device bytes the handle may still allocate (nlm_fd_set_alloc_limit); < 0: no limit
  int64_t alloc_budget = -1;
  std::vector<size_t> alloc_sizes;  // bytes of allocs[k]

  template <class Tp>
  cudaError_t alloc(Tp **p, size_t count) {
    const size_t bytes = count * sizeof(Tp) + 16;
    if (alloc_budget >= 0 && (int64_t)bytes > alloc_budget) return cudaErrorMemoryAllocation;
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, bytes);
    if (e == cudaSuccess) {
      allocs.push_back(q);
      alloc_sizes.push_back(bytes);
      if (alloc_budget >= 0) alloc_budget -= (int64_t)bytes;
      *p = static_cast<Tp *>(q);
    }
    return e;
  }
  // free one allocation of alloc() (no-op for null) and clear the pointer
  template <class Tp>
  void release(Tp **p) {
    if (!*p) return;
    for (size_t k = 0; k < allocs.size(); k++)
      if (allocs[k] == (void *)*p) {
        cudaFree(allocs[k]);
        if (alloc_budget >= 0) alloc_budget += (int64_t)alloc_sizes[k];
        allocs.erase(allocs.begin() + k);
        alloc_sizes.erase(alloc_sizes.begin() + k);
        break;
      }
    *p = nullptr;
  }
  ~nlm_fd() {
    if (stream) cudaStreamSynchronize(stream);
    for (auto &g : gexec)
      if (g) cudaGraphExecDestroy(g);
    if (h_times) cudaFreeHost(h_times);
    if (ev_times) cudaEventDestroy(ev_times);
    for (void *p : allocs) cudaFree(p);
    for (auto e : ev_pool) cudaEventDestroy(e);
    if (pipe_sin) cudaStreamSynchronize(pipe_sin);
    if (pipe_sout) cudaStreamSynchronize(pipe_sout);
    for (auto e : pipe_ev) cudaEventDestroy(e);
    if (pipe_sin) cudaStreamDestroy(pipe_sin);
    if (pipe_sout) cudaStreamDestroy(pipe_sout);
    if (stream) cudaStreamDestroy(stream);
  }
};


int get_state_impl(nlm_fd *h, double *u, double *v, double *f, bool keep_z);

namespace nlm {

// ---- model functions (fd_host.cu) used by the host I/O, batch and
// quasi-static units ---------------------------------------------------------
bool finite_all(const double *a, int64_t n);
void nofail_flags(const double *x, int64_t n, double tol, int nreg, const nlm_nofail_region *reg,
                  std::vector<uint8_t> &interior);
int check_nofail_regions(const nlm_fd_desc &d);
int rnp_constants(const nlm_material &m, int dim, double delta, StepParams &P);
int lattice_relabel(NeighborBuild &nb, int dim, int S, double mesh_h, double delta,
                    cudaStream_t s, std::vector<uint8_t> &lres);
int launch_step(nlm_fd *h, const StepArgs &a0);
int apply_fbc(nlm_fd *h, double t);
int apply_bc(nlm_fd *h, double t);
bool crack_due(const nlm_fd *h, int64_t nsteps);
int do_run(nlm_fd *h, int64_t nsteps);

}  // namespace nlm
