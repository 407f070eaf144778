// fd_fp32.cu -- FP32 "compensated" explicit-step kernels (RNPBond).
//
// Bond arithmetic runs in FP32 on split coordinates: every position and
// displacement is stored as an FP32 pair (hi, lo) with value hi + lo, so the
// bond vectors xi = x_j - x_i and eta = u_j - u_i are formed as
// (hi_j - hi_i) + (lo_j - lo_i).  The hi difference of two nearby nodes is
// exact (Sterbenz), so xi and eta keep ~2^-24 relative accuracy however small
// they are compared with the coordinates.  The bond strain is the linearised
// S = xi.eta / |xi|^2 of RNPBond::getS (src/material/pd/rnpBond.cpp:303-306),
// which has no cancellation once eta is accurate.  Forces are summed in FP32;
// velocity and the time update stay FP64 per node.

#include "fd_internal.h"
#include "state_io.cuh"

namespace nlm {

struct Params32 {
  float check_low_eff;  // r > this  <=>  definitelyGreaterThan(r, check_low)
  float check_up, inv_h, inv_delta;
  float K1;             // 4 C beta / invF (times J when J is constant)
  float Ksc;            // (f_sc rbar)^2 / (1 - 1e-5)^2: |S| > S_c  <=>  S^2 r > Ksc
  float beta;
  int infl_type;
  float a0, a1, alpha, ibeta;
};

static Params32 make_p32(const StepParams &P) {
  Params32 q;
  q.check_low_eff = (float)(P.check_low / (1.0 - 1e-5));
  q.check_up = (float)P.check_up;
  q.inv_h = (float)(1.0 / P.h);
  q.inv_delta = (float)(1.0 / P.delta);
  double k1 = 4.0 * P.C * P.beta / P.invF;
  if (P.infl_type == 0) k1 *= P.infl_a0;
  q.K1 = (float)k1;
  double sc = P.fsc * P.rbar / (1.0 - 1e-5);
  q.Ksc = (float)(sc * sc);
  q.beta = (float)P.beta;
  q.infl_type = P.infl_type;
  q.a0 = (float)P.infl_a0;
  q.a1 = (float)P.infl_a1;
  q.alpha = (float)P.infl_alpha;
  q.ibeta = (float)(1.0 / P.infl_beta);
  return q;
}

template <int DIM>
__device__ __forceinline__ void ld_hl(const float4 *p, int64_t j, float h[3], float l[3]) {
  if (DIM == 2) {
    const float4 a = __ldg(p + j);
    h[0] = a.x; h[1] = a.y; h[2] = 0.f;
    l[0] = a.z; l[1] = a.w; l[2] = 0.f;
  } else {
    const float4 a = __ldg(p + 2 * j), b = __ldg(p + 2 * j + 1);
    h[0] = a.x; h[1] = a.y; h[2] = a.z;
    l[0] = b.x; l[1] = b.y; l[2] = b.z;
  }
}

// Bond force of RNPBond in FP32.  Returns s with F = s * xi (xi unnormalised;
// the 1/|xi| of the direction is folded into s).
template <int DIM>
__device__ __forceinline__ float rnp_bond32(const Params32 &Q, const float xih[3],
                                            const float xil[3], const float uih[3],
                                            const float uil[3], const float xjh[3],
                                            const float xjl[3], const float ujh[3],
                                            const float ujl[3], float volj, bool breakable,
                                            bool irrev, bool &fs, float d[3]) {
  float e[3];
  for (int c = 0; c < DIM; c++) {
    d[c] = (xjh[c] - xih[c]) + (xjl[c] - xil[c]);
    e[c] = (ujh[c] - uih[c]) + (ujl[c] - uil[c]);
  }
  float r2 = d[0] * d[0] + d[1] * d[1];
  float de = d[0] * e[0] + d[1] * e[1];
  if (DIM == 3) {
    r2 += d[2] * d[2];
    de += d[2] * e[2];
  }
  const float rinv = rsqrtf(r2);
  const float r = r2 * rinv;
  const float S = de * (rinv * rinv);
  if (r > Q.check_low_eff) volj *= (Q.check_up - r) * Q.inv_h;
  float k = Q.K1;
  if (Q.infl_type == 1)
    k *= Q.a0 + Q.a1 * (r * Q.inv_delta);
  else if (Q.infl_type == 2) {
    const float rr = r * Q.inv_delta;
    k *= Q.alpha * __expf(-rr * rr * Q.ibeta);
  }
  const float s0 = k * S * volj * rinv;
  if (!breakable) return s0;
  const float bs2 = S * S * r;
  if (irrev && !fs && bs2 > Q.Ksc) fs = true;
  if (fs) return 0.f;
  return s0 * __expf(-Q.beta * bs2);
}

// FP32C integrator epilogue: same update as integrate_node64 with the
// displacement kept as an FP32 (hi, lo) pair and f stored in FP32.
template <int DIM, int SCHEME, bool FIRST>
__device__ __forceinline__ void integrate_node32(const StepParams &P, const DevPtrs &D,
                                                 const BCTable &T, const StepArgs &A,
                                                 int64_t i, uint8_t fl, const float uih[3],
                                                 const float uil[3], const float fint[3]) {
  double f[3] = {fint[0], fint[1], fint[2]};
  if (fl & FLAG_FBC) {
    double fe[3];
    ld_node<DIM>(D.fext, i, fe);
    for (int c = 0; c < DIM; c++) f[c] = fe[c] + (double)fint[c];
  }
  float fs_[3] = {(float)f[0], (float)f[1], (float)f[2]};
  double ui[3], un[3] = {0., 0., 0.};
  for (int c = 0; c < DIM; c++) ui[c] = (double)uih[c] + (double)uil[c];
  const int ref = (fl & 7) ? D.bcref[i] : -1;
  if (SCHEME == NLM_VELOCITY_VERLET) {
    const double fact = 0.5 * P.dt / P.rho;
    double v[3], vn[3];
    ld_node_rw<DIM>(D.v[0], i, v);
    if (!FIRST) {
      double fp[3];
      ld_f32<DIM>(D.f32, i, fp);
      for (int c = 0; c < DIM; c++) {
        if (!(fl >> c & 1)) {
          vn[c] = (v[c] + fact * fp[c]) + fact * f[c];
        } else {
          double du, dv;
          bc_dof(D, T, ref, c, A.t_now, du, dv);
          vn[c] = dv;
        }
      }
    } else {
      for (int c = 0; c < DIM; c++) vn[c] = v[c];
    }
    for (int c = 0; c < DIM; c++) {
      if (!(fl >> c & 1)) {
        un[c] = ui[c] + P.dt * (vn[c] + fact * f[c]);
      } else {
        double du, dv;
        bc_dof(D, T, ref, c, A.t_next, du, dv);
        un[c] = du;
      }
    }
    vn[2] = DIM == 3 ? vn[2] : 0.;
    st_node<DIM>(D.v[0], i, vn);
  } else {
    const double fact = P.dt * P.dt / P.rho;
    double v[3], vn[3] = {0., 0., 0.};
    ld_node<DIM>(D.v[A.cur], i, v);
    for (int c = 0; c < DIM; c++) {
      if (!(fl >> c & 1)) {
        un[c] = ui[c] + (fact * f[c] + P.dt * v[c]);
        vn[c] = (un[c] - ui[c]) / P.dt;
      } else {
        double du, dv;
        bc_dof(D, T, ref, c, A.t_next, du, dv);
        un[c] = du;
        vn[c] = dv;
      }
    }
    st_node<DIM>(D.v[1 - A.cur], i, vn);
  }
  st_f32<DIM>(D.f32, i, fs_);
  st_split<DIM>(D.u32[1 - A.cur], i, un);
}

// Thread-per-node, sliced-ELL bond store.
template <int DIM, int SCHEME, bool FIRST>
__global__ void __launch_bounds__(128)
    k_rnp32_thread(const StepParams P, const Params32 Q, const DevPtrs D, const BCTable T,
                   const StepArgs A) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  const float4 *ucur = D.u32[A.cur];
  float xih[3], xil[3], uih[3], uil[3];
  ld_hl<DIM>(D.pos32, i, xih, xil);
  ld_hl<DIM>(ucur, i, uih, uil);
  const uint8_t fl = D.flags[i];
  const bool brk_i = !(fl & FLAG_NOFAIL);
  const int64_t slice = i >> 5;
  const int64_t base = D.sell_ptr[slice] + (i & 31);
  const int w = D.sell_w[slice];
  float fi[3] = {0.f, 0.f, 0.f};
  uint32_t word = 0;
  bool dirty = false;
  int chunk = 0;
  for (int k = 0; k < w; k++) {
    if ((k & 31) == 0) {
      if (dirty) D.bits[(int64_t)chunk * P.npad + i] = word;
      chunk = k >> 5;
      word = D.bits[(int64_t)chunk * P.npad + i];
      dirty = false;
    }
    const int j = __ldg(D.sell_cols + base + (int64_t)k * 32);
    if (j < 0) break;
    float xjh[3], xjl[3], ujh[3], ujl[3], dv[3];
    ld_hl<DIM>(D.pos32, j, xjh, xjl);
    ld_hl<DIM>(ucur, j, ujh, ujl);
    bool fs = (word >> (k & 31)) & 1u;
    const bool was = fs;
    bool breakable = brk_i;
    if (P.nofail && breakable) breakable = !(D.flags[j] & FLAG_NOFAIL);
    const float s = rnp_bond32<DIM>(Q, xih, xil, uih, uil, xjh, xjl, ujh, ujl,
                                    __ldg(D.vol32 + j), breakable, P.irrev, fs, dv);
    if (fs != was) {
      word |= 1u << (k & 31);
      dirty = true;
    }
    fi[0] += s * dv[0];
    fi[1] += s * dv[1];
    if (DIM == 3) fi[2] += s * dv[2];
  }
  if (dirty) D.bits[(int64_t)chunk * P.npad + i] = word;
  integrate_node32<DIM, SCHEME, FIRST>(P, D, T, A, i, fl, uih, uil, fi);
}

// Warp-per-node over CSR rows; lane k of the warp owns bonds k, k+32, ...
template <int DIM, int SCHEME, bool FIRST>
__global__ void __launch_bounds__(256)
    k_rnp32_warp(const StepParams P, const Params32 Q, const DevPtrs D, const BCTable T,
                 const StepArgs A) {
  const int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= P.n) return;
  const float4 *ucur = D.u32[A.cur];
  float xih[3], xil[3], uih[3], uil[3];
  ld_hl<DIM>(D.pos32, i, xih, xil);
  ld_hl<DIM>(ucur, i, uih, uil);
  const uint8_t fl = D.flags[i];
  const bool brk_i = !(fl & FLAG_NOFAIL);
  const int64_t r0 = D.rowptr[i];
  const int len = (int)(D.rowptr[i + 1] - r0);
  float fi[3] = {0.f, 0.f, 0.f};
  for (int b = 0; b < len; b += 32) {
    const int k = b + lane;
    const uint32_t word = D.bits[(int64_t)(b >> 5) * P.npad + i];
    bool newly = false;
    if (k < len) {
      const int j = __ldg(D.cols + r0 + k);
      float xjh[3], xjl[3], ujh[3], ujl[3], dv[3];
      ld_hl<DIM>(D.pos32, j, xjh, xjl);
      ld_hl<DIM>(ucur, j, ujh, ujl);
      bool fs = (word >> lane) & 1u;
      const bool was = fs;
      bool breakable = brk_i;
      if (P.nofail && breakable) breakable = !(D.flags[j] & FLAG_NOFAIL);
      const float s = rnp_bond32<DIM>(Q, xih, xil, uih, uil, xjh, xjl, ujh, ujl,
                                      __ldg(D.vol32 + j), breakable, P.irrev, fs, dv);
      newly = fs != was;
      fi[0] += s * dv[0];
      fi[1] += s * dv[1];
      if (DIM == 3) fi[2] += s * dv[2];
    }
    const uint32_t nb = __ballot_sync(0xffffffffu, newly);
    if (nb && lane == 0) D.bits[(int64_t)(b >> 5) * P.npad + i] = word | nb;
  }
  for (int o = 16; o > 0; o >>= 1) {
    fi[0] += __shfl_xor_sync(0xffffffffu, fi[0], o);
    fi[1] += __shfl_xor_sync(0xffffffffu, fi[1], o);
    if (DIM == 3) fi[2] += __shfl_xor_sync(0xffffffffu, fi[2], o);
  }
  if (lane == 0) integrate_node32<DIM, SCHEME, FIRST>(P, D, T, A, i, fl, uih, uil, fi);
}

template <int DIM, int SCHEME>
static cudaError_t launch32(const StepParams &P, const DevPtrs &D, const BCTable &T,
                            const StepArgs &a, int decomp, cudaStream_t s) {
  if (P.n == 0) return cudaSuccess;
  const Params32 Q = make_p32(P);
  if (decomp == NLM_DECOMP_WARP) {
    const int bs = 256;
    const unsigned grid = (unsigned)((P.n * 32 + bs - 1) / bs);
    if (a.first)
      k_rnp32_warp<DIM, SCHEME, true><<<grid, bs, 0, s>>>(P, Q, D, T, a);
    else
      k_rnp32_warp<DIM, SCHEME, false><<<grid, bs, 0, s>>>(P, Q, D, T, a);
  } else {
    const int bs = 128;
    const unsigned grid = (unsigned)((P.n + bs - 1) / bs);
    if (a.first)
      k_rnp32_thread<DIM, SCHEME, true><<<grid, bs, 0, s>>>(P, Q, D, T, a);
    else
      k_rnp32_thread<DIM, SCHEME, false><<<grid, bs, 0, s>>>(P, Q, D, T, a);
  }
  return cudaGetLastError();
}

cudaError_t launch_rnp_step_fp32(const StepParams &P, const DevPtrs &D, const BCTable &T,
                                 const StepArgs &a, int decomp, cudaStream_t s) {
  if (P.dim == 2)
    return P.scheme == NLM_VELOCITY_VERLET ? launch32<2, NLM_VELOCITY_VERLET>(P, D, T, a, decomp, s)
                                           : launch32<2, NLM_CENTRAL_DIFFERENCE>(P, D, T, a, decomp, s);
  return P.scheme == NLM_VELOCITY_VERLET ? launch32<3, NLM_VELOCITY_VERLET>(P, D, T, a, decomp, s)
                                         : launch32<3, NLM_CENTRAL_DIFFERENCE>(P, D, T, a, decomp, s);
}

}  // namespace nlm
