// es_fp32.cu -- ElasticState explicit step, FP32 compensated (two passes).
//
// Same two-pass scheme as es_fp64.cu.  The bond extension is evaluated in the
// cancellation-free form
//   e = |X + eta| - |X| = (2 X.eta + eta.eta) / (|X + eta| + |X|)
// on split (hi, lo) coordinates, so e keeps FP32 relative accuracy even when
// it is 1e-6 of |X|.  Pass 1 stores, per node, the two coefficients of the
// scalar force state t(e, |X|) = a_i |X| + b_i e (ElasticState.cpp:191-245
// rewritten with e_s = theta |X| / 3), so pass 2 gathers 8 bytes per
// neighbour for t_ji.

#include "fp32_common.cuh"

namespace nlm {

struct ESConst32 {
  float sc_eff;      // e > sc_eff |X|  <=>  definitelyGreaterThan(e / |X|, s_c)
  float check_up, inv_h;
  float cfac;        // c * f2 of the dilatation (2 f2 in 2-D, 3 in 3-D)
  // t = a |X| + b e with a = ka * theta / m, b = kb / m
  float ka, kb;
};

static ESConst32 make_es32(const StepParams &P) {
  ESConst32 c;
  c.sc_eff = P.es_sc > 0. ? (float)(P.es_sc / (1.0 - 1e-5)) : 3.0e38f;
  c.check_up = (float)P.check_up;
  c.inv_h = (float)(1.0 / P.h);
  if (P.dim == 2) {
    const double q = (P.es_nu + 1.) / (2. * P.es_nu - 1.);
    const double as = P.es_plane_strain ? 9. * (P.es_K + P.es_mu / 9.)
                                        : 9. * (P.es_K + q * q * P.es_mu / 9.);
    const double ad = 8. * P.es_mu;
    const double f2 = P.es_factor2D;
    // t = (2 f2 as - (3 - 2 f2) ad) e_s / 3 + ad (e - e_s),  e_s = theta X / 3
    c.ka = (float)(((2. * f2 * as - (3. - 2. * f2) * ad) / 3. - ad) / 3.);
    c.kb = (float)ad;
    c.cfac = (float)(2. * f2);
  } else {
    const double as = 9. * P.es_K, ad = 15. * P.es_mu;
    if (P.es_ref_compat) {
      c.ka = (float)(as / 3.);
      c.kb = 0.f;
    } else {
      c.ka = (float)((as - ad) / 3.);
      c.kb = (float)ad;
    }
    c.cfac = 3.f;
  }
  return c;
}

// Bond vectors in FP32: X from split positions, eta from split displacements.
template <int DIM>
__device__ __forceinline__ void es_vec32(const Params32 &Q, const Node32<DIM> &ni,
                                         const float uih[3], const float uil[3],
                                         const Node32<DIM> &nj, const float ujh[3],
                                         const float ujl[3], float X[3], float et[3]) {
  const float2 dl = __half22float2(__hsub2(nj.lxy, ni.lxy));
  X[0] = fmaf(dl.x, Q.inv_lo, nj.xh[0] - ni.xh[0]);
  X[1] = fmaf(dl.y, Q.inv_lo, nj.xh[1] - ni.xh[1]);
  X[2] = 0.f;
  et[2] = 0.f;
  if (DIM == 3) {
    const float2 dz = __half22float2(__hsub2(nj.lz, ni.lz));
    X[2] = fmaf(dz.x, Q.inv_lo, nj.xh[2] - ni.xh[2]);
  }
  for (int c = 0; c < DIM; c++) et[c] = (ujh[c] - uih[c]) + (ujl[c] - uil[c]);
}

// |X|, the deformed bond Y = X + eta, |Y| and the extension e.
template <int DIM>
__device__ __forceinline__ void es_ext32(const float X[3], const float et[3], float Y[3],
                                         float &Xl, float &Yl, float &e) {
  float x2 = X[0] * X[0] + X[1] * X[1];
  float xe = X[0] * et[0] + X[1] * et[1];
  float ee = et[0] * et[0] + et[1] * et[1];
  if (DIM == 3) {
    x2 = fmaf(X[2], X[2], x2);
    xe = fmaf(X[2], et[2], xe);
    ee = fmaf(et[2], et[2], ee);
  }
  for (int c = 0; c < 3; c++) Y[c] = X[c] + et[c];
  float y2 = Y[0] * Y[0] + Y[1] * Y[1];
  if (DIM == 3) y2 = fmaf(Y[2], Y[2], y2);
  x2 = fmaxf(x2, 1e-30f);
  y2 = fmaxf(y2, 1e-30f);
  Xl = x2 * rsqrt_approx(x2);
  Yl = y2 * rsqrt_approx(y2);
  e = fmaf(2.f, xe, ee) / (Yl + Xl);
}

template <int DIM>
__global__ void __launch_bounds__(128)
    k_es_dil32(const StepParams P, const Params32 Q, const ESConst32 E, const DevPtrs D,
               const StepArgs A) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  const float4 *ucur = D.u32[A.cur];
  Node32<DIM> ni;
  ld_pos<DIM>(D, i, ni);
  float uih[3], uil[3];
  ld_pair<DIM>(ucur, i, uih, uil);
  const int len = D.rowlen[i];
  const int *colp = D.sell_cols + D.sell_ptr[i >> 5] + 4 * (i & 31);
  float th = 0.f;
  uint32_t word = 0, nw = 0;
  for (int k = 0; k < len; k++) {
    if ((k & 31) == 0) {
      if (nw) D.bits[(int64_t)((k >> 5) - 1) * P.npad + i] = word | nw;
      word = D.bits[(int64_t)(k >> 5) * P.npad + i];
      nw = 0;
    }
    const int j = __ldg(colp + (k >> 2) * 128 + (k & 3));
    Node32<DIM> nj;
    ld_pos<DIM>(D, j, nj);
    float ujh[3], ujl[3], X[3], et[3], Y[3], Xl, Yl, e;
    ld_pair<DIM>(ucur, j, ujh, ujl);
    es_vec32<DIM>(Q, ni, uih, uil, nj, ujh, ujl, X, et);
    es_ext32<DIM>(X, et, Y, Xl, Yl, e);
    const bool was = (word >> (k & 31)) & 1u;
    const bool fs = was || e > E.sc_eff * Xl;
    nw |= (uint32_t)(fs && !was) << (k & 31);
    const float om = fminf(1.f, (E.check_up - Xl) * E.inv_h);
    th += fs ? 0.f : Xl * e * om * nj.vol;
  }
  if (nw) D.bits[(int64_t)((len - 1) >> 5) * P.npad + i] = word | nw;
  const float minv = (float)(1.0 / D.mw64[i]);
  const float theta = E.cfac * minv * th;
  D.es_ab[i] = make_float2(E.ka * theta * minv, E.kb * minv);
}

template <int DIM, int SCHEME>
__global__ void __launch_bounds__(128)
    k_es_force32(const StepParams P, const Params32 Q, const ESConst32 E, const DevPtrs D,
                 const BCTable T, const StepArgs A) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  const float4 *ucur = D.u32[A.cur];
  Node32<DIM> ni;
  ld_pos<DIM>(D, i, ni);
  float uih[3], uil[3];
  ld_pair<DIM>(ucur, i, uih, uil);
  const uint8_t fl = D.flags[i];
  const int len = D.rowlen[i];
  const int *colp = D.sell_cols + D.sell_ptr[i >> 5] + 4 * (i & 31);
  const float2 abi = D.es_ab[i];
  float fi[3] = {0.f, 0.f, 0.f};
  uint32_t word = 0;
  for (int k = 0; k < len; k++) {
    if ((k & 31) == 0) word = D.bits[(int64_t)(k >> 5) * P.npad + i];
    if ((word >> (k & 31)) & 1u) continue;
    const int j = __ldg(colp + (k >> 2) * 128 + (k & 3));
    Node32<DIM> nj;
    ld_pos<DIM>(D, j, nj);
    float ujh[3], ujl[3], X[3], et[3], Y[3], Xl, Yl, e;
    ld_pair<DIM>(ucur, j, ujh, ujl);
    const float2 abj = __ldg(D.es_ab + j);
    es_vec32<DIM>(Q, ni, uih, uil, nj, ujh, ujl, X, et);
    es_ext32<DIM>(X, et, Y, Xl, Yl, e);
    const float tsum = (abi.x + abj.x) * Xl + (abi.y + abj.y) * e;
    const float om = fminf(1.f, (E.check_up - Xl) * E.inv_h);
    const float s = tsum * om * nj.vol / Yl;
    fi[0] = fmaf(s, Y[0], fi[0]);
    fi[1] = fmaf(s, Y[1], fi[1]);
    if (DIM == 3) fi[2] = fmaf(s, Y[2], fi[2]);
  }
  integrate_node32<DIM, SCHEME>(P, Q, D, T, A, i, fl, uih, uil, fi);
}

template <int DIM>
static cudaError_t es32(const StepParams &P, const DevPtrs &D, const BCTable &T,
                        const StepArgs &a, cudaStream_t s) {
  const Params32 Q = make_p32(P);
  const ESConst32 E = make_es32(P);
  const unsigned g = (unsigned)((P.n + 127) / 128);
  k_es_dil32<DIM><<<g, 128, 0, s>>>(P, Q, E, D, a);
  if (P.scheme == NLM_VELOCITY_VERLET)
    k_es_force32<DIM, NLM_VELOCITY_VERLET><<<g, 128, 0, s>>>(P, Q, E, D, T, a);
  else
    k_es_force32<DIM, NLM_CENTRAL_DIFFERENCE><<<g, 128, 0, s>>>(P, Q, E, D, T, a);
  return cudaGetLastError();
}

cudaError_t launch_es_step_fp32(const StepParams &P, const DevPtrs &D, const BCTable &T,
                                const StepArgs &a, int decomp, cudaStream_t s) {
  (void)decomp;
  if (P.n == 0) return cudaSuccess;
  return P.dim == 2 ? es32<2>(P, D, T, a, s) : es32<3>(P, D, T, a, s);
}

}  // namespace nlm
