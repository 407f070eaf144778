// mlp.cu -- per-node MLP of the quasi-static warm start, BF16 tensor-core
// GEMMs with FP32 accumulation, training (backpropagation + Adam) and
// inference.
//
// Network: n_in -> hidden x n_layers (ReLU) -> n_out (linear).  Parameters
// are kept in FP32 (master copy, Adam moments) and rounded to BF16 for every
// GEMM.  All GEMMs go through one tiled kernel built on the warp-level
// mma.sync.m16n8k16 BF16 instruction: a 64 x 64 block tile, four warps of
// 32 x 32, K staged through shared memory in steps of 32.  Operand fragments
// follow the PTX ISA layout of m16n8k16 (A row-major 16x16, B column-major
// 16x8, C 16x8 FP32).

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/nlmgpu.h"
#include "common.cuh"

namespace nlm {
void set_error(const std::string &msg);
}  // namespace nlm

namespace {

using bf16 = __nv_bfloat16;

constexpr int TM = 64, TN = 64, TK = 32, KPAD = 8;

enum Epi : int {
  EPI_STORE = 0,     // C (fp32)
  EPI_BIAS_RELU = 1, // Z = C + b (fp32), A = relu(Z) (bf16)
  EPI_BIAS = 2,      // C + b (fp32)
  EPI_ATOMIC = 3,    // C += (fp32 atomics; split-K weight gradients)
  EPI_RELU_GRAD = 4  // dZ = C * (Z > 0) (bf16), for the layer below
};

struct GemmArgs {
  int M, N, K;
  const bf16 *A;
  int lda;
  const bf16 *B;
  int ldb;
  float *C;
  int ldc;
  const float *bias;
  bf16 *Cb;          // bf16 output (relu activations / masked gradient)
  const float *Zmask;  // EPI_RELU_GRAD: pre-activation of the layer below
  int ksplit;        // K range per blockIdx.z
};

__device__ __forceinline__ void mma_bf16(float c[4], const uint32_t a[4], const uint32_t b[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// C[M x N] = opA[M x K] * opB[K x N] with opA(m,k) = TA ? A[k*lda+m] : A[m*lda+k]
// and opB(k,n) = TB ? B[n*ldb+k] : B[k*ldb+n].
template <bool TA, bool TB, int EPI>
__global__ void __launch_bounds__(128) k_gemm(const GemmArgs g) {
  __shared__ __align__(16) bf16 As[TM][TK + KPAD];
  __shared__ __align__(16) bf16 Bs[TN][TK + KPAD];  // n-major: k contiguous
  const int m0 = blockIdx.y * TM, n0 = blockIdx.x * TN;
  const int kbeg = blockIdx.z * g.ksplit;
  const int kend = min(g.K, kbeg + g.ksplit);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  const int gq = lane >> 2, tq = lane & 3;
  float acc[2][4][4];
#pragma unroll
  for (int a = 0; a < 2; a++)
#pragma unroll
    for (int b = 0; b < 4; b++)
#pragma unroll
      for (int c = 0; c < 4; c++) acc[a][b][c] = 0.f;
  const bf16 zero = __float2bfloat16(0.f);
  for (int k0 = kbeg; k0 < kend; k0 += TK) {
    for (int e = tid; e < TM * TK; e += 128) {
      const int mm = e / TK, kk = e % TK;
      const int m = m0 + mm, k = k0 + kk;
      bf16 v = zero;
      if (m < g.M && k < kend) v = TA ? g.A[(int64_t)k * g.lda + m] : g.A[(int64_t)m * g.lda + k];
      As[mm][kk] = v;
    }
    for (int e = tid; e < TN * TK; e += 128) {
      const int nn = e / TK, kk = e % TK;
      const int n = n0 + nn, k = k0 + kk;
      bf16 v = zero;
      if (n < g.N && k < kend) v = TB ? g.B[(int64_t)n * g.ldb + k] : g.B[(int64_t)k * g.ldb + n];
      Bs[nn][kk] = v;
    }
    __syncthreads();
#pragma unroll
    for (int ks = 0; ks < TK; ks += 16) {
      uint32_t af[2][4], bfr[4][2];
#pragma unroll
      for (int a = 0; a < 2; a++) {
        const int r = wm + 16 * a + gq;
        af[a][0] = *reinterpret_cast<const uint32_t *>(&As[r][ks + 2 * tq]);
        af[a][1] = *reinterpret_cast<const uint32_t *>(&As[r + 8][ks + 2 * tq]);
        af[a][2] = *reinterpret_cast<const uint32_t *>(&As[r][ks + 2 * tq + 8]);
        af[a][3] = *reinterpret_cast<const uint32_t *>(&As[r + 8][ks + 2 * tq + 8]);
      }
#pragma unroll
      for (int b = 0; b < 4; b++) {
        const int c = wn + 8 * b + gq;
        bfr[b][0] = *reinterpret_cast<const uint32_t *>(&Bs[c][ks + 2 * tq]);
        bfr[b][1] = *reinterpret_cast<const uint32_t *>(&Bs[c][ks + 2 * tq + 8]);
      }
#pragma unroll
      for (int a = 0; a < 2; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) mma_bf16(acc[a][b], af[a], bfr[b]);
    }
    __syncthreads();
  }
  // epilogue: c0,c1 at (row gq, cols 2tq, 2tq+1); c2,c3 at row gq+8
#pragma unroll
  for (int a = 0; a < 2; a++)
#pragma unroll
    for (int b = 0; b < 4; b++)
#pragma unroll
      for (int h = 0; h < 2; h++)
#pragma unroll
        for (int q = 0; q < 2; q++) {
          const int m = m0 + wm + 16 * a + gq + 8 * h;
          const int n = n0 + wn + 8 * b + 2 * tq + q;
          if (m >= g.M || n >= g.N) continue;
          float v = acc[a][b][2 * h + q];
          const int64_t o = (int64_t)m * g.ldc + n;
          if (EPI == EPI_STORE) {
            g.C[o] = v;
          } else if (EPI == EPI_BIAS_RELU) {
            v += g.bias[n];
            g.C[o] = v;
            g.Cb[o] = __float2bfloat16(v > 0.f ? v : 0.f);
          } else if (EPI == EPI_BIAS) {
            g.C[o] = v + g.bias[n];
          } else if (EPI == EPI_ATOMIC) {
            atomicAdd(g.C + o, v);
          } else {
            g.Cb[o] = __float2bfloat16(g.Zmask[o] > 0.f ? v : 0.f);
          }
        }
}

template <bool TA, bool TB, int EPI>
cudaError_t gemm(const GemmArgs &a0, int splits, cudaStream_t s) {
  GemmArgs a = a0;
  a.ksplit = ((a.K + splits - 1) / splits + TK - 1) / TK * TK;
  const int gz = (a.K + a.ksplit - 1) / a.ksplit;
  dim3 grid((a.N + TN - 1) / TN, (a.M + TM - 1) / TM, gz);
  k_gemm<TA, TB, EPI><<<grid, 128, 0, s>>>(a);
  return cudaGetLastError();
}

__global__ void k_to_bf16(int64_t n, const float *x, bf16 *y) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) y[i] = __float2bfloat16(x[i]);
}
// rows x cols_in float -> rows x ld bf16 (zero padded columns)
__global__ void k_pack_rows(int64_t rows, int cin, int ld, const float *x, bf16 *y) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= rows * ld) return;
  const int64_t r = t / ld;
  const int c = (int)(t % ld);
  y[t] = __float2bfloat16(c < cin ? x[r * cin + c] : 0.f);
}
// dY = 2 (Y - T) / rows over the first nout columns (ld = padded width);
// per-block squared error partial sums
__global__ void k_loss_grad(int64_t rows, int nout, int ld, const float *Y, const float *T,
                            bf16 *dY, float *part) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  float se = 0.f;
  if (t < rows * ld) {
    const int64_t r = t / ld;
    const int c = (int)(t % ld);
    float d = 0.f;
    if (c < nout) {
      d = Y[t] - T[r * nout + c];
      se = d * d;
    }
    dY[t] = __float2bfloat16(2.f * d / (float)rows);
  }
  __shared__ float sh[32];
  for (int o = 16; o > 0; o >>= 1) se += __shfl_xor_sync(0xffffffffu, se, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = se;
  __syncthreads();
  if (threadIdx.x < 32) {
    se = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.f;
    for (int o = 16; o > 0; o >>= 1) se += __shfl_xor_sync(0xffffffffu, se, o);
    if (threadIdx.x == 0) atomicAdd(part, se);
  }
}
// db[c] += sum over a 256-row chunk of dZ[r, c] (bf16 input); db zeroed
// beforehand.  grid = (column blocks of 128, row chunks of 256).
__global__ void k_bias_grad(int64_t rows, int cols, int ld, const bf16 *dZ, float *db) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  const int64_t r0 = (int64_t)blockIdx.y * 256;
  const int64_t r1 = r0 + 256 < rows ? r0 + 256 : rows;
  float s = 0.f;
#pragma unroll 8
  for (int64_t r = r0; r < r1; r++) s += __bfloat162float(dZ[r * ld + c]);
  atomicAdd(db + c, s);
}
__global__ void k_adam(int64_t n, float *p, const float *g, float *m, float *v, float lr,
                       float b1, float b2, float eps, float c1, float c2) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  m[i] = b1 * m[i] + (1.f - b1) * gi;
  v[i] = b2 * v[i] + (1.f - b2) * gi * gi;
  p[i] -= lr * (m[i] / c1) / (sqrtf(v[i] / c2) + eps);
}
__global__ void k_accum(const float *loss, double *acc, double scale) {
  *acc += (double)*loss * scale;
}
__global__ void k_gather_rows(int64_t nb, const int64_t *idx, int cin, const float *x, float *y,
                              int cout, const float *t, float *ty) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= nb) return;
  const int64_t s = idx[r];
  for (int c = 0; c < cin; c++) y[r * cin + c] = x[s * cin + c];
  for (int c = 0; c < cout; c++) ty[r * cout + c] = t[s * cout + c];
}

unsigned blk(int64_t n) { return (unsigned)((n + 255) / 256); }

}  // namespace

using namespace nlm;

struct nlm_mlp {
  int nin = 0, nh = 0, nl = 0, nout = 0;
  int kin = 16, kout = 8;   // padded widths of the input and output
  std::vector<int> din, dout;   // per layer (padded)
  std::vector<int64_t> woff, boff;  // offsets into params
  int64_t nparams = 0;
  float *params = nullptr, *grads = nullptr, *m1 = nullptr, *m2 = nullptr;
  bf16 *wbf = nullptr;      // bf16 copy of all weights (same layout)
  int64_t adam_t = 0;
  // activations for up to cap rows
  int64_t cap = 0;
  bf16 *xin = nullptr;
  std::vector<float *> Z;   // pre-activations (fp32) per layer
  std::vector<bf16 *> A;    // bf16 activations per layer (A[0] = input)
  std::vector<bf16 *> dZ;   // bf16 gradients per layer
  float *ybuf = nullptr, *tbuf = nullptr, *xbuf = nullptr, *loss = nullptr;
  double *eloss = nullptr;  // epoch loss accumulator
  // dataset
  float *dx = nullptr, *dy = nullptr;
  int64_t drows = 0;
  int64_t *didx = nullptr;
  cudaStream_t s = nullptr;
  std::vector<void *> allocs;
  template <class Tp>
  cudaError_t alloc(Tp **p, size_t count) {
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, count * sizeof(Tp) + 64);
    if (e == cudaSuccess) {
      allocs.push_back(q);
      *p = static_cast<Tp *>(q);
    }
    return e;
  }
  ~nlm_mlp() {
    if (s) cudaStreamSynchronize(s);
    for (void *p : allocs) cudaFree(p);
    if (s) cudaStreamDestroy(s);
  }
};

namespace {

int fail2(int code, const std::string &m) {
  set_error(m);
  return code;
}

cudaError_t ensure_cap(nlm_mlp *h, int64_t rows) {
  if (rows <= h->cap) return cudaSuccess;
  const int64_t cap = std::max<int64_t>(rows, 1024);
  cudaError_t e = cudaSuccess;
  const int L = h->nl + 1;
  h->Z.assign(L, nullptr);
  h->A.assign(L + 1, nullptr);
  h->dZ.assign(L, nullptr);
  e = h->alloc(&h->A[0], (size_t)cap * h->kin);
  for (int l = 0; l < L && e == cudaSuccess; l++) {
    e = h->alloc(&h->Z[l], (size_t)cap * h->dout[l]);
    if (e == cudaSuccess) e = h->alloc(&h->A[l + 1], (size_t)cap * h->dout[l]);
    if (e == cudaSuccess) e = h->alloc(&h->dZ[l], (size_t)cap * h->dout[l]);
  }
  if (e == cudaSuccess) e = h->alloc(&h->xbuf, (size_t)cap * h->nin);
  if (e == cudaSuccess) e = h->alloc(&h->tbuf, (size_t)cap * h->nout);
  if (e == cudaSuccess) e = h->alloc(&h->ybuf, (size_t)cap * h->nout);
  if (e == cudaSuccess) h->cap = cap;
  return e;
}

cudaError_t refresh_bf16(nlm_mlp *h) {
  k_to_bf16<<<blk(h->nparams), 256, 0, h->s>>>(h->nparams, h->params, h->wbf);
  return cudaGetLastError();
}

// forward over rows already packed in A[0]; output pre-activation in Z[L-1]
cudaError_t forward(nlm_mlp *h, int64_t rows) {
  const int L = h->nl + 1;
  cudaError_t e = cudaSuccess;
  for (int l = 0; l < L && e == cudaSuccess; l++) {
    GemmArgs g{};
    g.M = (int)rows;
    g.N = h->dout[l];
    g.K = h->din[l];
    g.A = h->A[l];
    g.lda = h->din[l];
    g.B = h->wbf + h->woff[l];
    g.ldb = h->dout[l];
    g.C = h->Z[l];
    g.ldc = h->dout[l];
    g.bias = h->params + h->boff[l];
    g.Cb = h->A[l + 1];
    if (l < L - 1)
      e = gemm<false, false, EPI_BIAS_RELU>(g, 1, h->s);
    else
      e = gemm<false, false, EPI_BIAS>(g, 1, h->s);
  }
  return e;
}

// gradients of the mean squared error for rows in A[0] with targets tbuf
cudaError_t backward(nlm_mlp *h, int64_t rows) {
  const int L = h->nl + 1;
  cudaError_t e = cudaMemsetAsync(h->loss, 0, sizeof(float), h->s);
  if (e) return e;
  k_loss_grad<<<blk(rows * h->kout), 256, 0, h->s>>>(rows, h->nout, h->kout, h->Z[L - 1],
                                                     h->tbuf, h->dZ[L - 1], h->loss);
  if ((e = cudaMemsetAsync(h->grads, 0, sizeof(float) * h->nparams, h->s))) return e;
  for (int l = L - 1; l >= 0 && e == cudaSuccess; l--) {
    // dW_l = A_l^T dZ_l  (K-dim = rows, split for parallelism)
    GemmArgs g{};
    g.M = h->din[l];
    g.N = h->dout[l];
    g.K = (int)rows;
    g.A = h->A[l];
    g.lda = h->din[l];
    g.B = h->dZ[l];
    g.ldb = h->dout[l];
    g.C = h->grads + h->woff[l];
    g.ldc = h->dout[l];
    const int splits = (int)std::min<int64_t>(64, std::max<int64_t>(1, rows / 512));
    e = gemm<true, false, EPI_ATOMIC>(g, splits, h->s);
    if (e) break;
    k_bias_grad<<<dim3((h->dout[l] + 127) / 128, (unsigned)((rows + 255) / 256)), 128, 0, h->s>>>(
        rows, h->dout[l], h->dout[l], h->dZ[l], h->grads + h->boff[l]);
    if (l == 0) break;
    // dZ_{l-1} = (dZ_l W_l^T) * (Z_{l-1} > 0)
    GemmArgs b{};
    b.M = (int)rows;
    b.N = h->din[l];
    b.K = h->dout[l];
    b.A = h->dZ[l];
    b.lda = h->dout[l];
    b.B = h->wbf + h->woff[l];
    b.ldb = h->dout[l];
    b.Cb = h->dZ[l - 1];
    b.Zmask = h->Z[l - 1];
    b.ldc = h->din[l];
    e = gemm<false, true, EPI_RELU_GRAD>(b, 1, h->s);
  }
  return e ? e : cudaGetLastError();
}

cudaError_t pack_input(nlm_mlp *h, const float *xdev, int64_t rows) {
  k_pack_rows<<<blk(rows * h->kin), 256, 0, h->s>>>(rows, h->nin, h->kin, xdev, h->A[0]);
  return cudaGetLastError();
}

}  // namespace

extern "C" {

int nlm_mlp_create(int n_in, int n_hidden, int n_layers, int n_out, uint64_t seed,
                   nlm_mlp **out) {
  if (!out || n_in < 1 || n_in > 64 || n_hidden < 8 || n_hidden > 512 || n_layers < 1 ||
      n_layers > 8 || n_out < 1 || n_out > 64)
    return fail2(NLM_ERR_INVALID, "nlm_mlp_create: unsupported shape");
  nlm_mlp *h = new nlm_mlp();
  h->nin = n_in;
  h->nh = ((n_hidden + 15) / 16) * 16;
  h->nl = n_layers;
  h->nout = n_out;
  h->kin = ((n_in + 15) / 16) * 16;
  h->kout = ((n_out + 7) / 8) * 8;
  const int L = n_layers + 1;
  int64_t off = 0;
  for (int l = 0; l < L; l++) {
    h->din.push_back(l == 0 ? h->kin : h->nh);
    h->dout.push_back(l == L - 1 ? h->kout : h->nh);
    h->woff.push_back(off);
    off += (int64_t)h->din[l] * h->dout[l];
    h->boff.push_back(off);
    off += h->dout[l];
  }
  h->nparams = off;
  // He initialisation from a seeded generator (splitmix64 + Box-Muller)
  std::vector<float> p(off, 0.f);
  uint64_t st = seed * 0x9E3779B97F4A7C15ull + 1;
  auto next = [&]() {
    st += 0x9E3779B97F4A7C15ull;
    uint64_t z = st;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return ((z >> 11) + 0.5) * (1.0 / 9007199254740992.0);
  };
  for (int l = 0; l < L; l++) {
    const int fan_in = l == 0 ? n_in : h->nh;
    const double sd = std::sqrt(2.0 / fan_in) * (l == L - 1 ? 0.5 : 1.0);
    for (int i = 0; i < h->din[l]; i++)
      for (int j = 0; j < h->dout[l]; j++) {
        const bool live = (l > 0 || i < n_in) && (l < L - 1 || j < n_out);
        const double g = std::sqrt(-2.0 * std::log(next())) * std::cos(6.283185307179586 * next());
        p[h->woff[l] + (int64_t)i * h->dout[l] + j] = live ? (float)(sd * g) : 0.f;
      }
  }
  cudaError_t e = cudaStreamCreateWithFlags(&h->s, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = h->alloc(&h->params, off);
  if (e == cudaSuccess) e = h->alloc(&h->grads, off);
  if (e == cudaSuccess) e = h->alloc(&h->m1, off);
  if (e == cudaSuccess) e = h->alloc(&h->m2, off);
  if (e == cudaSuccess) e = h->alloc(&h->wbf, off);
  if (e == cudaSuccess) e = h->alloc(&h->loss, 1);
  if (e == cudaSuccess) e = h->alloc(&h->eloss, 1);
  if (e == cudaSuccess) e = cudaMemcpyAsync(h->params, p.data(), sizeof(float) * off, cudaMemcpyHostToDevice, h->s);
  if (e == cudaSuccess) e = cudaMemsetAsync(h->m1, 0, sizeof(float) * off, h->s);
  if (e == cudaSuccess) e = cudaMemsetAsync(h->m2, 0, sizeof(float) * off, h->s);
  if (e == cudaSuccess) e = refresh_bf16(h);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->s);
  if (e != cudaSuccess) {
    delete h;
    return cuda_fail(e, "nlm_mlp_create");
  }
  *out = h;
  return NLM_OK;
}

int nlm_mlp_destroy(nlm_mlp *h) {
  delete h;
  return NLM_OK;
}

int nlm_mlp_num_params(const nlm_mlp *h, int64_t *count) {
  if (!h || !count) return fail2(NLM_ERR_INVALID, "null argument");
  *count = h->nparams;
  return NLM_OK;
}

int nlm_mlp_get_params(nlm_mlp *h, float *params) {
  if (!h || !params) return fail2(NLM_ERR_INVALID, "null argument");
  NLM_CUDA(cudaMemcpyAsync(params, h->params, sizeof(float) * h->nparams, cudaMemcpyDeviceToHost, h->s));
  NLM_CUDA(cudaStreamSynchronize(h->s));
  return NLM_OK;
}

int nlm_mlp_set_params(nlm_mlp *h, const float *params) {
  if (!h || !params) return fail2(NLM_ERR_INVALID, "null argument");
  NLM_CUDA(cudaMemcpyAsync(h->params, params, sizeof(float) * h->nparams, cudaMemcpyHostToDevice, h->s));
  NLM_CUDA(refresh_bf16(h));
  NLM_CUDA(cudaStreamSynchronize(h->s));
  return NLM_OK;
}

int nlm_mlp_forward(nlm_mlp *h, const float *x, int64_t rows, float *y) {
  if (!h || !x || !y || rows < 0) return fail2(NLM_ERR_INVALID, "bad arguments");
  if (rows == 0) return NLM_OK;
  NLM_CUDA(ensure_cap(h, rows));
  NLM_CUDA(cudaMemcpyAsync(h->xbuf, x, sizeof(float) * rows * h->nin, cudaMemcpyHostToDevice, h->s));
  NLM_CUDA(pack_input(h, h->xbuf, rows));
  NLM_CUDA(forward(h, rows));
  const int L = h->nl + 1;
  NLM_CUDA(cudaMemcpy2DAsync(y, sizeof(float) * h->nout, h->Z[L - 1], sizeof(float) * h->kout,
                             sizeof(float) * h->nout, rows, cudaMemcpyDeviceToHost, h->s));
  NLM_CUDA(cudaStreamSynchronize(h->s));
  return NLM_OK;
}

int nlm_mlp_grad(nlm_mlp *h, const float *x, const float *t, int64_t rows, float *loss,
                 float *grads) {
  if (!h || !x || !t || rows <= 0) return fail2(NLM_ERR_INVALID, "bad arguments");
  NLM_CUDA(ensure_cap(h, rows));
  NLM_CUDA(cudaMemcpyAsync(h->xbuf, x, sizeof(float) * rows * h->nin, cudaMemcpyHostToDevice, h->s));
  NLM_CUDA(cudaMemcpyAsync(h->tbuf, t, sizeof(float) * rows * h->nout, cudaMemcpyHostToDevice, h->s));
  NLM_CUDA(pack_input(h, h->xbuf, rows));
  NLM_CUDA(forward(h, rows));
  NLM_CUDA(backward(h, rows));
  float l = 0.f;
  NLM_CUDA(cudaMemcpyAsync(&l, h->loss, sizeof(float), cudaMemcpyDeviceToHost, h->s));
  if (grads)
    NLM_CUDA(cudaMemcpyAsync(grads, h->grads, sizeof(float) * h->nparams, cudaMemcpyDeviceToHost, h->s));
  NLM_CUDA(cudaStreamSynchronize(h->s));
  if (loss) *loss = l / (float)rows;
  return NLM_OK;
}

int nlm_mlp_set_data(nlm_mlp *h, const float *x, const float *t, int64_t rows) {
  if (!h || !x || !t || rows <= 0) return fail2(NLM_ERR_INVALID, "bad arguments");
  if (rows > h->drows) {
    NLM_CUDA(h->alloc(&h->dx, (size_t)rows * h->nin));
    NLM_CUDA(h->alloc(&h->dy, (size_t)rows * h->nout));
    NLM_CUDA(h->alloc(&h->didx, (size_t)rows));
  }
  h->drows = rows;
  NLM_CUDA(cudaMemcpyAsync(h->dx, x, sizeof(float) * rows * h->nin, cudaMemcpyHostToDevice, h->s));
  NLM_CUDA(cudaMemcpyAsync(h->dy, t, sizeof(float) * rows * h->nout, cudaMemcpyHostToDevice, h->s));
  NLM_CUDA(cudaStreamSynchronize(h->s));
  return NLM_OK;
}

// Minibatch Adam over the device-resident data set; losses[e] = mean squared
// error over the epoch's batches (may be NULL).
int nlm_mlp_train(nlm_mlp *h, int epochs, int batch, float lr, uint64_t seed, float *losses) {
  if (!h || epochs < 0 || batch < 16 || !(lr > 0.f) || h->drows <= 0)
    return fail2(NLM_ERR_INVALID, "bad training arguments (data set?)");
  NLM_CUDA(ensure_cap(h, batch));
  std::vector<int64_t> idx(h->drows);
  uint64_t st = seed * 0x9E3779B97F4A7C15ull + 7;
  auto rnd = [&]() {
    st ^= st << 13;
    st ^= st >> 7;
    st ^= st << 17;
    return st;
  };
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  for (int ep = 0; ep < epochs; ep++) {
    for (int64_t i = 0; i < h->drows; i++) idx[i] = i;
    for (int64_t i = h->drows - 1; i > 0; i--) std::swap(idx[i], idx[rnd() % (uint64_t)(i + 1)]);
    NLM_CUDA(cudaMemcpyAsync(h->didx, idx.data(), sizeof(int64_t) * h->drows, cudaMemcpyHostToDevice, h->s));
    int64_t nb = 0;
    if (losses) NLM_CUDA(cudaMemsetAsync(h->eloss, 0, sizeof(double), h->s));
    for (int64_t b0 = 0; b0 + batch <= h->drows; b0 += batch) {
      k_gather_rows<<<blk(batch), 256, 0, h->s>>>(batch, h->didx + b0, h->nin, h->dx, h->xbuf,
                                                  h->nout, h->dy, h->tbuf);
      NLM_CUDA(cudaGetLastError());
      NLM_CUDA(pack_input(h, h->xbuf, batch));
      NLM_CUDA(forward(h, batch));
      NLM_CUDA(backward(h, batch));
      h->adam_t++;
      const float c1 = 1.f - std::pow(b1, (float)h->adam_t), c2 = 1.f - std::pow(b2, (float)h->adam_t);
      k_adam<<<blk(h->nparams), 256, 0, h->s>>>(h->nparams, h->params, h->grads, h->m1, h->m2, lr,
                                               b1, b2, eps, c1, c2);
      NLM_CUDA(cudaGetLastError());
      NLM_CUDA(refresh_bf16(h));
      if (losses) {
        k_accum<<<1, 1, 0, h->s>>>(h->loss, h->eloss, 1.0 / batch);
        NLM_CUDA(cudaGetLastError());
      }
      nb++;
    }
    if (losses) {
      double l = 0.;
      NLM_CUDA(cudaMemcpyAsync(&l, h->eloss, sizeof(double), cudaMemcpyDeviceToHost, h->s));
      NLM_CUDA(cudaStreamSynchronize(h->s));
      losses[ep] = nb ? (float)(l / nb) : 0.f;
    }
  }
  NLM_CUDA(cudaStreamSynchronize(h->s));
  return NLM_OK;
}

}  // extern "C"
