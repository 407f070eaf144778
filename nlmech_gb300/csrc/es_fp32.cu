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

#include <atomic>

#include <type_traits>

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

// es_ext32 for the tile kernels: the same quantities with the division by
// |Y| + |X| done by the hardware reciprocal (relative error ~1 ulp) and 1/|Y|
// returned from the square-root step, so no bond takes an IEEE division.
// Every operation is written out with its rounding, in the order of
// es_ext32_pair, so that the scalar and the pair forms give one bond the same
// e and |X| (and so the same break decision).  The squared lengths carry
// 1e-30 added to the first square: below half an ulp of any bond's squared
// length, it only keeps a zero-length bond (a row's padding entry) away from
// rsqrt(0).
template <int DIM>
__device__ __forceinline__ void es_ext32_fast(const float X[3], const float et[3], float Y[3],
                                              float &Xl, float &iY, float &e) {
  float x2 = __fmaf_rn(X[1], X[1], __fmaf_rn(X[0], X[0], 1e-30f));
  float xe = __fmaf_rn(X[1], et[1], __fmul_rn(X[0], et[0]));
  float ee = __fmaf_rn(et[1], et[1], __fmul_rn(et[0], et[0]));
  if (DIM == 3) {
    x2 = __fmaf_rn(X[2], X[2], x2);
    xe = __fmaf_rn(X[2], et[2], xe);
    ee = __fmaf_rn(et[2], et[2], ee);
  }
  for (int c = 0; c < 3; c++) Y[c] = __fadd_rn(X[c], et[c]);
  float y2 = __fmaf_rn(Y[1], Y[1], __fmaf_rn(Y[0], Y[0], 1e-30f));
  if (DIM == 3) y2 = __fmaf_rn(Y[2], Y[2], y2);
  iY = rsqrt_approx(y2);
  Xl = __fmul_rn(x2, rsqrt_approx(x2));
  e = __fmul_rn(__fmaf_rn(2.f, xe, ee), rcp_approx(__fmaf_rn(y2, iY, Xl)));
}

// es_ext32_fast for two bonds at once (lane x, lane y) by packed FP32 pair
// operations; each lane equals es_ext32_fast of its bond.
template <int DIM>
__device__ __forceinline__ void es_ext32_pair(const float2 X[3], const float2 et[3], float2 Y[3],
                                              float2 &Xl, float2 &iY, float2 &e) {
  const float2 eps = make_float2(1e-30f, 1e-30f);
  float2 x2 = __ffma2_rn(X[1], X[1], __ffma2_rn(X[0], X[0], eps));
  float2 xe = __ffma2_rn(X[1], et[1], __fmul2_rn(X[0], et[0]));
  float2 ee = __ffma2_rn(et[1], et[1], __fmul2_rn(et[0], et[0]));
  if (DIM == 3) {
    x2 = __ffma2_rn(X[2], X[2], x2);
    xe = __ffma2_rn(X[2], et[2], xe);
    ee = __ffma2_rn(et[2], et[2], ee);
  }
  for (int c = 0; c < DIM; c++) Y[c] = __fadd2_rn(X[c], et[c]);
  float2 y2 = __ffma2_rn(Y[1], Y[1], __ffma2_rn(Y[0], Y[0], eps));
  if (DIM == 3) y2 = __ffma2_rn(Y[2], Y[2], y2);
  iY = make_float2(rsqrt_approx(y2.x), rsqrt_approx(y2.y));
  Xl = __fmul2_rn(x2, make_float2(rsqrt_approx(x2.x), rsqrt_approx(x2.y)));
  const float2 den = __ffma2_rn(y2, iY, Xl);
  e = __fmul2_rn(__ffma2_rn(make_float2(2.f, 2.f), xe, ee),
                 make_float2(rcp_approx(den.x), rcp_approx(den.y)));
}

// The staged bond vectors of bonds a (lane x) and b (lane y) of node i.
template <int DIM>
__device__ __forceinline__ void es_pair_vec(const float4 &xi, const float4 &ui, const float4 &xa,
                                            const float4 &ua, const float4 &xb,
                                            const float4 &ub, float2 X[3], float2 et[3]) {
  X[0] = make_float2(__fsub_rn(xa.x, xi.x), __fsub_rn(xb.x, xi.x));
  X[1] = make_float2(__fsub_rn(xa.y, xi.y), __fsub_rn(xb.y, xi.y));
  et[0] = make_float2(__fsub_rn(ua.x, ui.x), __fsub_rn(ub.x, ui.x));
  et[1] = make_float2(__fsub_rn(ua.y, ui.y), __fsub_rn(ub.y, ui.y));
  if (DIM == 3) {
    X[2] = make_float2(__fsub_rn(xa.z, xi.z), __fsub_rn(xb.z, xi.z));
    et[2] = make_float2(__fsub_rn(ua.z, ui.z), __fsub_rn(ub.z, ui.z));
  } else {
    X[2] = et[2] = make_float2(0.f, 0.f);
  }
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
    const bool fs = was || e > __fmul_rn(E.sc_eff, Xl);
    nw |= (uint32_t)(fs && !was) << (k & 31);
    const float om = fminf(1.f, (E.check_up - Xl) * E.inv_h);
    th += fs ? 0.f : Xl * e * om * nj.vol;
  }
  if (nw) D.bits[(int64_t)((len - 1) >> 5) * P.npad + i] = word | nw;
  const float minv = D.minv32[i];
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

// ---- tile-frame variants (NLM_DECOMP_TILE_LOCAL) ---------------------------
// A block takes one tile of kTileNodes consecutive nodes.  It stages the
// tile's nodes and their halo in shared memory, one record per node: the
// reference position and the displacement relative to the tile's first node
// o (each difference formed from the split values, then rounded once to
// FP32), the volume, and in the force pass the node's force-state
// coefficients (a, b).  A bond then reads its neighbour's record through
// the bond's 16-bit index into the staged list (tile_lidx), not by a global
// gather: X = x_j - x_i and eta = u_j - u_i are differences of two staged
// values.  Per bond the arithmetic is that of k_es_dil32 / k_es_force32.
template <int DIM>
__device__ __forceinline__ void es_stage32(const Params32 &Q, const DevPtrs &D,
                                           const float4 *ucur, int64_t g, const Node32<DIM> &no,
                                           const float uoh[3], const float uol[3], float4 &sx,
                                           float4 &su) {
  Node32<DIM> ng;
  ld_pos<DIM>(D, g, ng);
  float uh[3], ul[3], X[3], et[3];
  ld_pair<DIM>(ucur, g, uh, ul);
  es_vec32<DIM>(Q, no, uoh, uol, ng, uh, ul, X, et);
  sx = make_float4(X[0], X[1], X[2], ng.vol);
  su = make_float4(et[0], et[1], et[2], 0.f);
}

template <int DIM, bool FORCE>
__device__ __forceinline__ int es_stage_tile(const Params32 &Q, const DevPtrs &D,
                                             const float4 *ucur, int64_t t0, int nt, float4 *s_x,
                                             float4 *s_u, float *s_b, int tb) {
  const int nh = D.tile_hstride;  // halo lists padded to one stride
  const int64_t h0 = (int64_t)tb * nh;
  Node32<DIM> no;
  ld_pos<DIM>(D, t0, no);
  float uoh[3], uol[3];
  ld_pair<DIM>(ucur, t0, uoh, uol);
  // unrolled so that several staged nodes' loads are in flight at once
#pragma unroll 4
  for (int e = threadIdx.x; e < kTileNodes + nh; e += blockDim.x) {
    if (e < kTileNodes && e >= nt) continue;
    const int64_t g = e < kTileNodes ? t0 + e : (int64_t)D.tile_halo[h0 + e - kTileNodes];
    if (g < 0) continue;  // an empty slot of a lattice-ordered halo
    float4 sx, su;
    es_stage32<DIM>(Q, D, ucur, g, no, uoh, uol, sx, su);
    if (FORCE) {
      const float2 ab = __ldg(D.es_ab + g);
      su.w = ab.x;
      s_b[e] = ab.y;
    }
    s_x[e] = sx;
    s_u[e] = su;
  }
  return nh;
}

// The ids of a warp's 32 rows (one slice of tile_lidx: 256 bytes per group
// of four bonds, contiguous) brought into L2 before the staging, two 128-byte
// lines per group, spread over the lanes; the bond loops then find them in
// L2 instead of waiting on DRAM group by group.
__device__ __forceinline__ void es_prefetch_ids(const DevPtrs &D, int64_t i, int len) {
  const int gmax = __reduce_max_sync(0xffffffffu, (len + 3) >> 2);
  const char *base = reinterpret_cast<const char *>(D.tile_lidx + D.sell_ptr[i >> 5]);
  for (int k = threadIdx.x & 31; k < 2 * gmax; k += 32)
    asm volatile("prefetch.global.L2 [%0];" ::"l"(base + 128 * k));
}

template <int DIM>
__global__ void __launch_bounds__(kTileNodes)
    k_es_dil32_tile(const StepParams P, const Params32 Q, const ESConst32 E, const DevPtrs D,
                    const StepArgs A) {
  extern __shared__ float4 es_sm[];
  float4 *s_x = es_sm, *s_u = es_sm + D.tile_nmax;
  const int tb = blockIdx.x;
  const int64_t t0 = (int64_t)tb * kTileNodes;
  const int nt = (int)min((int64_t)kTileNodes, P.n - t0);
  es_prefetch_ids(D, t0 + threadIdx.x, threadIdx.x < nt ? D.rowlen[t0 + threadIdx.x] : 0);
  es_stage_tile<DIM, false>(Q, D, D.u32[A.cur], t0, nt, s_x, s_u, nullptr, tb);
  __syncthreads();
  const int il = threadIdx.x;
  if (il >= nt) return;
  const int64_t i = t0 + il;
  const float4 xi = s_x[il], ui = s_u[il];
  const int len = D.rowlen[i];
  const uint2 *lp = reinterpret_cast<const uint2 *>(D.tile_lidx + D.sell_ptr[i >> 5]) + (i & 31);
  const int ng = (len + 3) >> 2;
  // fast loop: a row with no broken bond sums theta without bond-state bits
  // and keeps the largest e - s_c |X|; a bond past its critical stretch (or
  // an already broken one) sends the row through the full loop below, which
  // forms e and |X| by the same function and decides with the same test
  uint32_t any_bits = 0;
  for (int w = 0; w * 32 < len; w++) any_bits |= D.bits[(int64_t)w * P.npad + i];
  if (any_bits == 0u) {
    // bonds in pairs (lane x, lane y), each lane summing its share of theta;
    // a row's padding entries (its own node) are masked in the last group
    float mx = -1.f;
    float2 th2 = make_float2(0.f, 0.f);
    const float2 nsc = make_float2(-E.sc_eff, -E.sc_eff);
    const float2 cu2 = make_float2(E.check_up, E.check_up), ih2 = make_float2(E.inv_h, E.inv_h);
    auto fpair = [&](int ja, int jb, bool va, bool vb) {
      const float4 xa = s_x[ja], xb = s_x[jb], ua = s_u[ja], ub = s_u[jb];
      float2 X[3], et[3], Y[3], Xl, iY, e;
      es_pair_vec<DIM>(xi, ui, xa, ua, xb, ub, X, et);
      es_ext32_pair<DIM>(X, et, Y, Xl, iY, e);
      const float2 z = __fadd2_rn(e, __fmul2_rn(nsc, Xl));  // e - s_c |X|
      const float2 t = __fmul2_rn(__ffma2_rn(Xl, make_float2(-1.f, -1.f), cu2), ih2);  // (cu - |X|) / h
      const float2 om = make_float2(fminf(1.f, t.x), fminf(1.f, t.y));
      float2 w = __fmul2_rn(__fmul2_rn(Xl, e), om);
      w = make_float2(va ? w.x : 0.f, vb ? w.y : 0.f);
      mx = fmax3(mx, va ? z.x : -1.f, vb ? z.y : -1.f);
      th2 = __ffma2_rn(w, make_float2(xa.w, xb.w), th2);
    };
    uint2 c = ng > 0 ? __ldg(lp) : make_uint2(0u, 0u);
    const int full = len >> 2;
    for (int g = 0; g < full; g++) {
      const uint2 cur = c;
      if (g + 1 < ng) c = __ldg(lp + 32 * (g + 1));
      fpair((int)(cur.x & 0xffffu), (int)(cur.x >> 16), true, true);
      fpair((int)(cur.y & 0xffffu), (int)(cur.y >> 16), true, true);
    }
    if (const int rem = len & 3) {
      fpair((int)(c.x & 0xffffu), (int)(c.x >> 16), true, rem > 1);
      if (rem > 2) fpair((int)(c.y & 0xffffu), (int)(c.y >> 16), true, false);
    }
    const float thf = __fadd_rn(th2.x, th2.y);
    if (!(mx > 0.f)) {
      const float minv = D.minv32[i];
      const float theta = E.cfac * minv * thf;
      D.es_ab[i] = make_float2(E.ka * theta * minv, E.kb * minv);
      return;
    }
  }
  float th = 0.f;
  uint32_t word = 0, nw = 0;
  auto bond = [&](int k, int jl) {
    const float4 xj = s_x[jl], uj = s_u[jl];
    float X[3] = {xj.x - xi.x, xj.y - xi.y, xj.z - xi.z};
    float et[3] = {uj.x - ui.x, uj.y - ui.y, uj.z - ui.z};
    float Y[3], Xl, iY, e;
    es_ext32_fast<DIM>(X, et, Y, Xl, iY, e);
    const bool was = (word >> (k & 31)) & 1u;
    const bool fs = was || e > __fmul_rn(E.sc_eff, Xl);
    nw |= (uint32_t)(fs && !was) << (k & 31);
    const float om = fminf(1.f, (E.check_up - Xl) * E.inv_h);
    th += fs ? 0.f : Xl * e * om * xj.w;
  };
  // the next group's ids and bit word are loaded one group ahead
  uint2 nxt = ng > 0 ? __ldg(lp) : make_uint2(0u, 0u);
  uint32_t wnext = ng > 0 ? D.bits[i] : 0u;
  auto group = [&](int g) {
    if ((g & 7) == 0) {
      if (nw) D.bits[(int64_t)((g >> 3) - 1) * P.npad + i] = word | nw;
      word = wnext;
      nw = 0;
      if (8 * ((g >> 3) + 1) < ng) wnext = D.bits[(int64_t)((g >> 3) + 1) * P.npad + i];
    }
    const uint2 c = nxt;
    if (g + 1 < ng) nxt = __ldg(lp + 32 * (g + 1));
    return c;
  };
  // whole groups of four bonds, then the row's remainder
  const int full = len >> 2;
  for (int g = 0; g < full; g++) {
    const uint2 c = group(g);
    bond(4 * g, (int)(c.x & 0xffffu));
    bond(4 * g + 1, (int)(c.x >> 16));
    bond(4 * g + 2, (int)(c.y & 0xffffu));
    bond(4 * g + 3, (int)(c.y >> 16));
  }
  if (len & 3) {
    const uint2 c = group(full);
    const int jl[3] = {(int)(c.x & 0xffffu), (int)(c.x >> 16), (int)(c.y & 0xffffu)};
    for (int q = 0; q < (len & 3); q++) bond(4 * full + q, jl[q]);
  }
  if (nw) D.bits[(int64_t)((len - 1) >> 5) * P.npad + i] = word | nw;
  const float minv = D.minv32[i];
  const float theta = E.cfac * minv * th;
  D.es_ab[i] = make_float2(E.ka * theta * minv, E.kb * minv);
}

template <int DIM, int SCHEME>
__global__ void __launch_bounds__(kTileNodes, 4)
    k_es_force32_tile(const StepParams P, const Params32 Q, const ESConst32 E, const DevPtrs D,
                      const BCTable T, const StepArgs A) {
  extern __shared__ float4 es_sm[];
  float4 *s_x = es_sm, *s_u = es_sm + D.tile_nmax;
  float *s_b = reinterpret_cast<float *>(es_sm + 2 * D.tile_nmax);
  const int tb = blockIdx.x;
  const int64_t t0 = (int64_t)tb * kTileNodes;
  const int nt = (int)min((int64_t)kTileNodes, P.n - t0);
  const float4 *ucur = D.u32[A.cur];
  es_prefetch_ids(D, t0 + threadIdx.x, threadIdx.x < nt ? D.rowlen[t0 + threadIdx.x] : 0);
  es_stage_tile<DIM, true>(Q, D, ucur, t0, nt, s_x, s_u, s_b, tb);
  __syncthreads();
  const int il = threadIdx.x;
  if (il >= nt) return;
  const int64_t i = t0 + il;
  const float4 xi = s_x[il], ui = s_u[il];
  const float ai = ui.w, bi = s_b[il];
  float uih[3], uil[3];
  ld_pair<DIM>(ucur, i, uih, uil);
  const uint8_t fl = D.flags[i];
  const int len = D.rowlen[i];
  const uint2 *lp = reinterpret_cast<const uint2 *>(D.tile_lidx + D.sell_ptr[i >> 5]) + (i & 31);
  float fi[3] = {0.f, 0.f, 0.f};
  uint32_t word = 0;
  const int ng = (len + 3) >> 2;
  // a row without broken bonds skips the per-bond state test
  uint32_t any_bits = 0;
  for (int w = 0; w * 32 < len; w++) any_bits |= D.bits[(int64_t)w * P.npad + i];
  // bonds in pairs (lane x: bond k, lane y: bond k + 1), each lane summing
  // its share of the force; padding entries are masked in the last group
  const float2 ai2 = make_float2(ai, ai), bi2 = make_float2(bi, bi);
  const float2 cu2 = make_float2(E.check_up, E.check_up), ih2 = make_float2(E.inv_h, E.inv_h);
  float2 fx = make_float2(0.f, 0.f), fy = fx, fz = fx;
  auto run = [&](auto has_bits) {
    constexpr bool HB = decltype(has_bits)::value;
    auto bond = [&](int k, int ja, int jb, bool va, bool vb) {
      const float4 xa = s_x[ja], xb = s_x[jb], ua = s_u[ja], ub = s_u[jb];
      float2 X[3], et[3], Y[3], Xl, iY, e;
      es_pair_vec<DIM>(xi, ui, xa, ua, xb, ub, X, et);
      es_ext32_pair<DIM>(X, et, Y, Xl, iY, e);
      const float2 tsum = __ffma2_rn(__fadd2_rn(bi2, make_float2(s_b[ja], s_b[jb])), e,
                                     __fmul2_rn(__fadd2_rn(ai2, make_float2(ua.w, ub.w)), Xl));
      const float2 t = __fmul2_rn(__ffma2_rn(Xl, make_float2(-1.f, -1.f), cu2), ih2);  // (cu - |X|) / h
      const float2 om = make_float2(fminf(1.f, t.x), fminf(1.f, t.y));
      float2 s = __fmul2_rn(__fmul2_rn(__fmul2_rn(tsum, om), make_float2(xa.w, xb.w)), iY);
      // a broken bond carries no force
      if (HB) {
        va = va && !((word >> (k & 31)) & 1u);
        vb = vb && !((word >> ((k + 1) & 31)) & 1u);
      }
      s = make_float2(va ? s.x : 0.f, vb ? s.y : 0.f);
      fx = __ffma2_rn(s, Y[0], fx);
      fy = __ffma2_rn(s, Y[1], fy);
      if (DIM == 3) fz = __ffma2_rn(s, Y[2], fz);
    };
    uint2 nxt = ng > 0 ? __ldg(lp) : make_uint2(0u, 0u);
    uint32_t wnext = (HB && ng > 0) ? D.bits[i] : 0u;
    auto group = [&](int g) {
      if (HB && (g & 7) == 0) {
        word = wnext;
        if (8 * ((g >> 3) + 1) < ng) wnext = D.bits[(int64_t)((g >> 3) + 1) * P.npad + i];
      }
      const uint2 c = nxt;
      if (g + 1 < ng) nxt = __ldg(lp + 32 * (g + 1));
      return c;
    };
    const int full = len >> 2;
    for (int g = 0; g < full; g++) {
      const uint2 c = group(g);
      bond(4 * g, (int)(c.x & 0xffffu), (int)(c.x >> 16), true, true);
      bond(4 * g + 2, (int)(c.y & 0xffffu), (int)(c.y >> 16), true, true);
    }
    if (const int rem = len & 3) {
      const uint2 c = group(full);
      bond(4 * full, (int)(c.x & 0xffffu), (int)(c.x >> 16), true, rem > 1);
      if (rem > 2) bond(4 * full + 2, (int)(c.y & 0xffffu), (int)(c.y >> 16), true, false);
    }
  };
  if (any_bits)
    run(std::true_type{});
  else
    run(std::false_type{});
  fi[0] = __fadd_rn(fx.x, fx.y);
  fi[1] = __fadd_rn(fy.x, fy.y);
  if (DIM == 3) fi[2] = __fadd_rn(fz.x, fz.y);
  integrate_node32<DIM, SCHEME>(P, Q, D, T, A, i, fl, uih, uil, fi);
}

// Above 48 KB a kernel's dynamic shared memory must be opted into; each
// kernel is opted in once per device (bit d of done), for the largest staged
// list any tile store holds.
template <class K>
static void es_tile_smem(K kernel, std::atomic<uint64_t> &done) {
  int dev = 0;
  cudaGetDevice(&dev);
  const uint64_t bit = 1ull << (dev & 63);
  if (done.load() & bit) return;
  const size_t most = (2 * sizeof(float4) + sizeof(float)) * kTileMaxLocalES;
  if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)most) ==
      cudaSuccess)
    done.fetch_or(bit);
}

template <int DIM>
static cudaError_t es32_tile(const StepParams &P, const DevPtrs &D, const BCTable &T,
                             const StepArgs &a, cudaStream_t s) {
  const Params32 Q = make_p32(P);
  const ESConst32 E = make_es32(P);
  const unsigned g = (unsigned)((P.n + kTileNodes - 1) / kTileNodes);
  const size_t b1 = sizeof(float4) * 2 * D.tile_nmax;
  const size_t b2 = b1 + sizeof(float) * D.tile_nmax;
  static std::atomic<uint64_t> opt_d{0}, opt_v{0}, opt_c{0};
  es_tile_smem(k_es_dil32_tile<DIM>, opt_d);
  k_es_dil32_tile<DIM><<<g, kTileNodes, b1, s>>>(P, Q, E, D, a);
  if (P.scheme == NLM_VELOCITY_VERLET) {
    es_tile_smem(k_es_force32_tile<DIM, NLM_VELOCITY_VERLET>, opt_v);
    k_es_force32_tile<DIM, NLM_VELOCITY_VERLET><<<g, kTileNodes, b2, s>>>(P, Q, E, D, T, a);
  } else {
    es_tile_smem(k_es_force32_tile<DIM, NLM_CENTRAL_DIFFERENCE>, opt_c);
    k_es_force32_tile<DIM, NLM_CENTRAL_DIFFERENCE><<<g, kTileNodes, b2, s>>>(P, Q, E, D, T, a);
  }
  return cudaGetLastError();
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

// 1 / m_i for the FP32C passes, formed once in FP64 (m_i stays at its
// initial value), so no step takes a per-node FP64 division.
__global__ void k_es_minv32(const double *mw, float *minv, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) minv[i] = (float)(1.0 / mw[i]);
}

cudaError_t launch_es_minv32(const double *mw, float *minv, int64_t n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_es_minv32<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(mw, minv, n);
  return cudaGetLastError();
}

cudaError_t launch_es_step_fp32(const StepParams &P, const DevPtrs &D, const BCTable &T,
                                const StepArgs &a, int decomp, cudaStream_t s) {
  if (P.n == 0) return cudaSuccess;
  if (decomp == NLM_DECOMP_TILE_LOCAL && D.tile_lidx && D.tile_nmax > 0)
    return P.dim == 2 ? es32_tile<2>(P, D, T, a, s) : es32_tile<3>(P, D, T, a, s);
  return P.dim == 2 ? es32<2>(P, D, T, a, s) : es32<3>(P, D, T, a, s);
}

}  // namespace nlm
