// fd_fp32.cu -- FP32 "compensated" explicit-step kernels (RNPBond).
//
// Bond arithmetic runs in FP32 on split coordinates.  A position is stored as
// hi = (float)x plus its remainder lo = x - hi, packed as a half of
// lo * lo_scale (lo_scale = 2^24 / X with X the power of two above max |x|,
// so |lo * lo_scale| <= 1/2).  A displacement is an FP32 pair (hi, lo).  The
// bond vectors are formed as
//   xi  = (xh_j - xh_i) + (xl_j - xl_i),   eta = (uh_j - uh_i) + (ul_j - ul_i)
// The hi difference of two nearby nodes is exact (Sterbenz), so xi and eta
// keep ~2^-24 relative accuracy however small they are compared with the
// coordinates (the half-packed position remainder costs ~2^-36 X absolute).
// The bond strain is the linearised S = xi.eta / |xi|^2 of RNPBond::getS
// (src/material/pd/rnpBond.cpp:303-306), free of cancellation once eta is
// accurate.  Forces are summed in FP32.
//
// Time integration runs on (hi, lo) FP32 pairs ("double-float", ~48-bit
// significand) with error-free transformations (Knuth's TwoSum and the FMA
// TwoProduct): GB300's FP64 rate is a small fraction of its FP32 rate, and the
// per-node FP64 update would otherwise be the slowest part of the step.

#include <algorithm>
#include <atomic>
#include <type_traits>

#include "fp32_common.cuh"

namespace nlm {

// Kernel specialisations.
enum : int {
  OPT_CONSTJ = 1,  // constant influence function (J folded into K1)
  OPT_NOFAIL = 2,  // some nodes are non-interior (per-bond flag test needed)
  OPT_CONTACT = 4  // normal contact force on broken bonds (No_Penetration)
};

// Bond force of RNPBond in FP32 (rnpBond.cpp:242-300 with contact off),
// without branches.  Returns s with F = s * xi (the 1/|xi| of the direction
// is folded into s) and updates the bond state fs.  A padding entry is passed
// as the node itself: xi = eta = 0 gives S = 0, s = 0 and no break.
// The volume correction min(1, (delta + h/2 - r) / h) equals the reference's
// "if r > delta - h/2" factor away from its 1e-5 relative comparison band.
// The bond force from the bond vector d (= xi) and eta's components e (same
// arithmetic for every kernel): returns s with F = s * d and updates fs.
// On a broken bond with contact, d becomes the deformed bond y = xi + eta.
// KVOL: volj is already K1 * V_j (the same product formed here otherwise;
// only without the contact term, which needs V_j itself).
template <int DIM, int OPT, bool KVOL = false>
__device__ __forceinline__ float rnp_bond32_core(const Params32 &Q, float d[3], float e0,
                                                 float e1, float e2, float volj, float voli,
                                                 bool breakable, bool &fs) {
  float r2 = d[0] * d[0] + d[1] * d[1];
  float de = d[0] * e0 + d[1] * e1;
  if (DIM == 3) {
    r2 = fmaf(d[2], d[2], r2);
    de = fmaf(d[2], e2, de);
  }
  r2 = fmaxf(r2, 1e-30f);
  const float rinv = rsqrt_approx(r2);
  const float r = r2 * rinv;
  const float S = de * (rinv * rinv);
  float k = (KVOL ? volj : Q.K1 * volj) * fminf(1.f, (Q.check_up - r) * Q.inv_h);
  if (!(OPT & OPT_CONSTJ) && Q.infl_type != 0) {  // type 0: J folded into K1
    const float rr = r * Q.inv_delta;
    k *= Q.infl_type == 1 ? Q.a0 + Q.a1 * rr
                          : Q.alpha * ex2_approx(-rr * rr * Q.ibeta * 1.4426950408889634f);
  }
  const float s0 = k * S * rinv;
  const float bs2 = S * S * r;
  const bool brk = (OPT & OPT_NOFAIL) ? breakable : true;
  fs = fs || (brk && Q.irrev && bs2 > Q.Ksc);
  if ((OPT & OPT_CONTACT) && brk && fs) {
    // broken bond: normal contact only (rnpBond.cpp:281-291), along the
    // deformed bond y = xi + eta; F = -max(0, Kn Vi Vj/(Vi+Vj) (Rc - |y|)/|y|) y
    const float y0 = d[0] + e0, y1 = d[1] + e1;
    float yy = y0 * y0 + y1 * y1;
    if (DIM == 3) {
      d[2] = d[2] + e2;
      yy = fmaf(d[2], d[2], yy);
    }
    d[0] = y0;
    d[1] = y1;
    const float R = sqrtf(yy);
    const float vj = volj * fminf(1.f, (Q.check_up - r) * Q.inv_h);
    const float sf = Q.kn * (voli * vj / (voli + vj)) * (Q.rc - R) / R;
    return -fmaxf(sf, 0.f);
  }
  const float s1 = fs ? 0.f : s0 * ex2_approx(Q.nbl2e * bs2);
  return brk ? s1 : s0;
}

template <int DIM, int OPT>
__device__ __forceinline__ float rnp_bond32(const Params32 &Q, const Node32<DIM> &ni,
                                            const float uih[3], const float uil[3],
                                            const Node32<DIM> &nj, const float ujh[3],
                                            const float ujl[3], bool breakable, bool &fs,
                                            float d[3]) {
  const float2 dl = __half22float2(__hsub2(nj.lxy, ni.lxy));
  d[0] = fmaf(dl.x, Q.inv_lo, nj.xh[0] - ni.xh[0]);
  d[1] = fmaf(dl.y, Q.inv_lo, nj.xh[1] - ni.xh[1]);
  const float e0 = (ujh[0] - uih[0]) + (ujl[0] - uil[0]);
  const float e1 = (ujh[1] - uih[1]) + (ujl[1] - uil[1]);
  float e2 = 0.f;
  if (DIM == 3) {
    const float2 dz = __half22float2(__hsub2(nj.lz, ni.lz));
    d[2] = fmaf(dz.x, Q.inv_lo, nj.xh[2] - ni.xh[2]);
    e2 = (ujh[2] - uih[2]) + (ujl[2] - uil[2]);
  }
  return rnp_bond32_core<DIM, OPT>(Q, d, e0, e1, e2, nj.vol, ni.vol, breakable, fs);
}

// Thread-per-node, sliced-ELL bond store.  NW1: every row fits one bit word.
// Bonds are taken four at a time: one 16-byte load brings the four neighbour
// ids (the next group's ids are fetched while the current group is gathered
// and evaluated), then the eight node gathers of the group are issued
// together, so each thread keeps several independent loads in flight.
template <int DIM, int SCHEME, bool NW1, int OPT, bool BATCH>
__global__ void __launch_bounds__(128, DIM == 2 ? 7 : 5)
    k_rnp32_thread(const StepParams P, const Params32 Q0, const DevPtrs D, const BCTable T,
                   const StepArgs A) {
  const int64_t i = A.i0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= A.i1) return;
  if (BATCH && (D.flags[i] & FLAG_GHOST)) return;
  const Params32 &Q = BATCH ? static_cast<const Params32 *>(D.qtab)[D.slice_spec[i >> 5]] : Q0;
  const float4 *ucur = D.u32[A.cur];
  Node32<DIM> ni;
  ld_pos<DIM>(D, i, ni);
  float uih[3], uil[3];
  ld_pair<DIM>(ucur, i, uih, uil);
  const uint8_t fl = D.flags[i];
  const bool brk_i = !(fl & FLAG_NOFAIL);
  const int len = D.rowlen[i];
  const int ng = (len + 3) >> 2;
  const int4 *cp = reinterpret_cast<const int4 *>(D.sell_cols + D.sell_ptr[i >> 5]) + (i & 31);
  float fi[3] = {0.f, 0.f, 0.f};
  uint32_t word = NW1 ? D.bits[i] : 0u;
  uint32_t nw = 0;  // newly broken bits of the current word
  int4 nxt = ng > 0 ? __ldg(cp) : make_int4(-1, -1, -1, -1);
  for (int g = 0; g < ng; g++) {
    const int4 cur = nxt;
    if (g + 1 < ng) nxt = __ldg(cp + 32 * (g + 1));
    if (!NW1 && (g & 7) == 0) {
      if (nw) D.bits[(int64_t)((g >> 3) - 1) * P.npad + i] = word | nw;
      word = D.bits[(int64_t)(g >> 3) * P.npad + i];
      nw = 0;
    }
    const int ii = (int)i;
    const int jj[4] = {cur.x < 0 ? ii : cur.x, cur.y < 0 ? ii : cur.y, cur.z < 0 ? ii : cur.z,
                       cur.w < 0 ? ii : cur.w};
    Node32<DIM> nj[4];
    float ujh[4][3], ujl[4][3];
#pragma unroll
    for (int q = 0; q < 4; q++) {
      ld_pos<DIM>(D, jj[q], nj[q]);
      ld_pair<DIM>(ucur, jj[q], ujh[q], ujl[q]);
    }
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int k = 4 * g + q;
      float dv[3];
      const bool was = (word >> (k & 31)) & 1u;
      bool fs = was;
      bool breakable = true;
      if (OPT & OPT_NOFAIL) breakable = brk_i && !(D.flags[jj[q]] & FLAG_NOFAIL);
      const float s =
          rnp_bond32<DIM, OPT>(Q, ni, uih, uil, nj[q], ujh[q], ujl[q], breakable, fs, dv);
      nw |= (uint32_t)(fs && !was) << (k & 31);
      fi[0] = fmaf(s, dv[0], fi[0]);
      fi[1] = fmaf(s, dv[1], fi[1]);
      if (DIM == 3) fi[2] = fmaf(s, dv[2], fi[2]);
    }
  }
  if (nw) D.bits[NW1 ? i : (int64_t)((len - 1) >> 5) * P.npad + i] = word | nw;
  integrate_node32<DIM, SCHEME>(P, Q, D, T, A, i, fl, uih, uil, fi);
}

// Same decomposition without the four-wide grouping (one bond per iteration).
template <int DIM, int SCHEME, bool NW1, int OPT, bool BATCH>
__global__ void __launch_bounds__(128, DIM == 2 ? 12 : 8)
    k_rnp32_thread1(const StepParams P, const Params32 Q0, const DevPtrs D, const BCTable T,
                    const StepArgs A) {
  const int64_t i = A.i0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= A.i1) return;
  if (BATCH && (D.flags[i] & FLAG_GHOST)) return;
  const Params32 &Q = BATCH ? static_cast<const Params32 *>(D.qtab)[D.slice_spec[i >> 5]] : Q0;
  const float4 *ucur = D.u32[A.cur];
  Node32<DIM> ni;
  ld_pos<DIM>(D, i, ni);
  float uih[3], uil[3];
  ld_pair<DIM>(ucur, i, uih, uil);
  const uint8_t fl = D.flags[i];
  const bool brk_i = !(fl & FLAG_NOFAIL);
  const int len = D.rowlen[i];
  const int *colp = D.sell_cols + D.sell_ptr[i >> 5] + 4 * (i & 31);
  float fi[3] = {0.f, 0.f, 0.f};
  uint32_t word = NW1 ? D.bits[i] : 0u;
  uint32_t nw = 0;
  for (int k = 0; k < len; k++) {
    if (!NW1 && (k & 31) == 0) {
      if (nw) D.bits[(int64_t)((k >> 5) - 1) * P.npad + i] = word | nw;
      word = D.bits[(int64_t)(k >> 5) * P.npad + i];
      nw = 0;
    }
    const int j = __ldg(colp + (k >> 2) * 128 + (k & 3));
    Node32<DIM> nj;
    ld_pos<DIM>(D, j, nj);
    float ujh[3], ujl[3], dv[3];
    ld_pair<DIM>(ucur, j, ujh, ujl);
    const bool was = (word >> (k & 31)) & 1u;
    bool fs = was;
    bool breakable = true;
    if (OPT & OPT_NOFAIL) breakable = brk_i && !(D.flags[j] & FLAG_NOFAIL);
    const float s = rnp_bond32<DIM, OPT>(Q, ni, uih, uil, nj, ujh, ujl, breakable, fs, dv);
    nw |= (uint32_t)(fs && !was) << (k & 31);
    fi[0] = fmaf(s, dv[0], fi[0]);
    fi[1] = fmaf(s, dv[1], fi[1]);
    if (DIM == 3) fi[2] = fmaf(s, dv[2], fi[2]);
  }
  if (nw) D.bits[NW1 ? i : (int64_t)((len - 1) >> 5) * P.npad + i] = word | nw;
  integrate_node32<DIM, SCHEME>(P, Q, D, T, A, i, fl, uih, uil, fi);
}

// Warp-per-node over CSR rows; lane k of the warp owns bonds k, k+32, ...
template <int DIM, int SCHEME, int OPT, bool BATCH>
__global__ void __launch_bounds__(256)
    k_rnp32_warp(const StepParams P, const Params32 Q0, const DevPtrs D, const BCTable T,
                 const StepArgs A) {
  const int64_t i = A.i0 + ((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (i >= A.i1) return;
  if (BATCH && (D.flags[i] & FLAG_GHOST)) return;
  const Params32 &Q = BATCH ? static_cast<const Params32 *>(D.qtab)[D.slice_spec[i >> 5]] : Q0;
  const float4 *ucur = D.u32[A.cur];
  Node32<DIM> ni;
  ld_pos<DIM>(D, i, ni);
  float uih[3], uil[3];
  ld_pair<DIM>(ucur, i, uih, uil);
  const uint8_t fl = D.flags[i];
  const bool brk_i = !(fl & FLAG_NOFAIL);
  const int64_t r0 = D.rowptr[i];
  const int len = D.rowlen[i];
  float fi[3] = {0.f, 0.f, 0.f};
  for (int b = 0; b < len; b += 32) {
    const int k = b + lane;
    const uint32_t word = D.bits[(int64_t)(b >> 5) * P.npad + i];
    bool newly = false;
    if (k < len) {
      const int j = __ldg(D.cols + r0 + k);
      Node32<DIM> nj;
      ld_pos<DIM>(D, j, nj);
      float ujh[3], ujl[3], dv[3];
      ld_pair<DIM>(ucur, j, ujh, ujl);
      const bool was = (word >> lane) & 1u;
      bool fs = was;
      bool breakable = true;
      if (OPT & OPT_NOFAIL) breakable = brk_i && !(D.flags[j] & FLAG_NOFAIL);
      const float s = rnp_bond32<DIM, OPT>(Q, ni, uih, uil, nj, ujh, ujl, breakable, fs, dv);
      newly = fs && !was;
      fi[0] = fmaf(s, dv[0], fi[0]);
      fi[1] = fmaf(s, dv[1], fi[1]);
      if (DIM == 3) fi[2] = fmaf(s, dv[2], fi[2]);
    }
    const uint32_t nb = __ballot_sync(0xffffffffu, newly);
    if (nb && lane == 0) D.bits[(int64_t)(b >> 5) * P.npad + i] = word | nb;
  }
  for (int o = 16; o > 0; o >>= 1) {
    fi[0] += __shfl_xor_sync(0xffffffffu, fi[0], o);
    fi[1] += __shfl_xor_sync(0xffffffffu, fi[1], o);
    if (DIM == 3) fi[2] += __shfl_xor_sync(0xffffffffu, fi[2], o);
  }
  if (lane == 0) integrate_node32<DIM, SCHEME>(P, Q, D, T, A, i, fl, uih, uil, fi);
}

// Tile kernel (2-D): a block stages the positions and displacements of its
// kTileNodes nodes and of their halo in shared memory with coalesced loads,
// then runs the thread-per-node bond loop of k_rnp32_thread on the staged
// copies through 16-bit tile-local neighbour ids (half the bytes of the
// global ids).  Bond order and arithmetic are those of k_rnp32_thread, so the
// two decompositions give bit-identical results.
__device__ __forceinline__ void node_from_f4(const float4 a, Node32<2> &n) {
  n.xh[0] = a.x;
  n.xh[1] = a.y;
  n.xh[2] = 0.f;
  n.vol = a.z;
  n.lxy = *reinterpret_cast<const __half2 *>(&a.w);
  n.lz = __floats2half2_rn(0.f, 0.f);
}

template <int SCHEME, bool NW1, int OPT>
__global__ void __launch_bounds__(kTileNodes, 3)
    k_rnp32_tile(const StepParams P, const Params32 Q, const DevPtrs D, const BCTable T,
                 const StepArgs A) {
  __shared__ float4 s_pos[kTileMaxLocal];
  __shared__ float4 s_u[kTileMaxLocal];
  __shared__ uint8_t s_fl[(OPT & OPT_NOFAIL) ? kTileMaxLocal : 1];
  const int tb = A.tiles ? A.tiles[blockIdx.x] : (int)blockIdx.x;
  const int64_t t0 = (int64_t)tb * kTileNodes;
  const int nh = D.tile_hstride;  // halo lists padded to one stride
  const int64_t h0 = (int64_t)tb * nh;
  const int nt = (int)min((int64_t)kTileNodes, P.n - t0);
  const float4 *ucur = D.u32[A.cur];
  for (int e = threadIdx.x; e < kTileNodes + nh; e += blockDim.x) {
    if (e < kTileNodes && e >= nt) continue;
    const int64_t g = e < kTileNodes ? t0 + e : (int64_t)D.tile_halo[h0 + e - kTileNodes];
    if (g < 0) continue;  // an empty slot of a lattice-ordered halo
    s_pos[e] = __ldg(D.pos32 + g);
    s_u[e] = ucur[g];
    if (OPT & OPT_NOFAIL) s_fl[e] = D.flags[g];
  }
  __syncthreads();
  const int il = threadIdx.x;
  if (il >= nt) return;
  const int64_t i = t0 + il;
  Node32<2> ni;
  node_from_f4(s_pos[il], ni);
  float uih[3], uil[3];
  {
    const float4 a = s_u[il];
    uih[0] = a.x; uih[1] = a.y; uih[2] = 0.f;
    uil[0] = a.z; uil[1] = a.w; uil[2] = 0.f;
  }
  const uint8_t fl = D.flags[i];
  const bool brk_i = !(fl & FLAG_NOFAIL);
  const int len = D.rowlen[i];
  const int ng = (len + 3) >> 2;
  const uint2 *lp = reinterpret_cast<const uint2 *>(D.tile_lidx + D.sell_ptr[i >> 5]) + (i & 31);
  float fi[3] = {0.f, 0.f, 0.f};
  uint32_t word = NW1 ? D.bits[i] : 0u;
  uint32_t nw = 0;
  uint2 nxt = ng > 0 ? __ldg(lp) : make_uint2(0u, 0u);
  for (int g = 0; g < ng; g++) {
    const uint2 cur = nxt;
    if (g + 1 < ng) nxt = __ldg(lp + 32 * (g + 1));
    if (!NW1 && (g & 7) == 0) {
      if (nw) D.bits[(int64_t)((g >> 3) - 1) * P.npad + i] = word | nw;
      word = D.bits[(int64_t)(g >> 3) * P.npad + i];
      nw = 0;
    }
    const int jl[4] = {(int)(cur.x & 0xffffu), (int)(cur.x >> 16), (int)(cur.y & 0xffffu),
                       (int)(cur.y >> 16)};
    Node32<2> nj[4];
    float ujh[4][3], ujl[4][3];
#pragma unroll
    for (int q = 0; q < 4; q++) {
      node_from_f4(s_pos[jl[q]], nj[q]);
      const float4 a = s_u[jl[q]];
      ujh[q][0] = a.x; ujh[q][1] = a.y; ujh[q][2] = 0.f;
      ujl[q][0] = a.z; ujl[q][1] = a.w; ujl[q][2] = 0.f;
    }
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int k = 4 * g + q;
      float dv[3];
      const bool was = (word >> (k & 31)) & 1u;
      bool fs = was;
      bool breakable = true;
      if (OPT & OPT_NOFAIL) breakable = brk_i && !(s_fl[jl[q]] & FLAG_NOFAIL);
      const float sc =
          rnp_bond32<2, OPT>(Q, ni, uih, uil, nj[q], ujh[q], ujl[q], breakable, fs, dv);
      nw |= (uint32_t)(fs && !was) << (k & 31);
      fi[0] = fmaf(sc, dv[0], fi[0]);
      fi[1] = fmaf(sc, dv[1], fi[1]);
    }
  }
  if (nw) D.bits[NW1 ? i : (int64_t)((len - 1) >> 5) * P.npad + i] = word | nw;
  integrate_node32<2, SCHEME>(P, Q, D, T, A, i, fl, uih, uil, fi);
}

// Tile kernel with the bond data in the tile's own frame (2-D): staging
// writes, per staged node, x - x_o and u - u_o rounded once to FP32 (x_o, u_o
// of the tile's first node, both differences formed in the split
// representation), so a bond needs one 16-byte shared-memory read and two
// packed subtractions for xi and eta.  xi then carries the FP32 rounding of
// the tile-frame position (~2^-24 of the tile span) instead of ~2^-24 of
// itself, and eta 2^-24 of the largest |u - u_o| of the tile (its
// displacement span).  A tile whose span exceeds Params32::span_max (its
// error in S would exceed 2^-20 of the critical stretch: fragments in free
// flight, loads that throw nodes far) forms eta from the (hi, lo) pairs
// instead, as the thread kernels do: the staged record then holds the hi
// parts of u and a second array their lo parts.  The choice is made per tile
// from a block reduction of the span during staging.  The node's own update
// always stays on the (hi, lo) pairs.
//
// Bonds are read through tile_boff, 16-bit byte offsets into the staged
// arrays (an offset is an address without further arithmetic; padding
// entries address the row's own node, whose bond has xi = eta = 0 and adds
// no force).  The tile's block of tile_boff (its 8 slices, contiguous) is
// brought into shared memory by one bulk copy issued before the node
// staging, so the bond loops read no global memory.  With one nodal volume
// for the whole model (UV) K1 V is a constant and no volume is staged.
//
// Two loops evaluate a row.  The fast loop serves rows with no broken bond
// and no no-fail or contact terms: it keeps no bond-state bits, only the
// largest S^2 r of the row.  If that exceeds the break threshold (a bond
// breaks this step; rare) or the row already has broken bonds, the row is
// evaluated again by the full loop, which keeps the bits and the broken-bond
// terms.  Both loops form S^2 r by the same separately rounded operations
// (tile_bond_core), so they take the same break decisions.
// BATCH: a batch of specimens in one layout.  A launch covers the tiles that
// meet its node range [A.i0, A.i1) (a tile may hold nodes of two ranges and
// of several specimens) and owns only the range's nodes that are not ghosts;
// each node takes its own specimen's constants.  The staged volume is V, not
// K1 V: specimens differ in K1, and a bond's two nodes share a specimen.

// One bond in the tile frame: d = xi, e = eta, vj = K1 V_j (KV) or V_j.
// Returns s0 (the linearised bond's F = s0 d), ex = exp(-beta r S^2) (the
// unbroken bond's F = s0 ex d), bs2 = S^2 r (|S| > S_c <=> bs2 > Ksc) and r.
// A padding bond (d = e = 0) gives s0 = bs2 = 0: r^2 carries 1e-30 added to
// the first square (below half an ulp of any bond's squared length, so it
// only keeps a zero-length bond away from rsqrt(0)).
// UV: one volume for the model, K1 V min(1, cu_ih - r inv_h) formed as
// min(K1 V, K1 V cu_ih - r K1 V inv_h) with the products precomputed.
template <int OPT, bool KV, bool UV = false>
__device__ __forceinline__ void tile_bond_core(const Params32 &Q, float2 d, float2 e, float vj,
                                               float &s0, float &ex, float &bs2, float &r) {
  const float r2 = __fmaf_rn(d.y, d.y, __fmaf_rn(d.x, d.x, 1e-30f));
  const float de = __fmaf_rn(d.y, e.y, __fmul_rn(d.x, e.x));
  const float rinv = rsqrt_approx(r2);
  r = __fmul_rn(r2, rinv);
  float kw = UV ? fminf(Q.kv_uniform, __fmaf_rn(-r, Q.kv_ih, Q.kv_cuih))
                : __fmul_rn(KV ? vj : __fmul_rn(Q.K1, vj),
                            fminf(1.f, __fmaf_rn(-r, Q.inv_h, Q.cu_ih)));
  if (!(OPT & OPT_CONSTJ) && Q.infl_type != 0) {  // type 0: J folded into K1
    const float rr = __fmul_rn(r, Q.inv_delta);
    kw = __fmul_rn(kw, Q.infl_type == 1
                           ? __fmaf_rn(Q.a1, rr, Q.a0)
                           : __fmul_rn(Q.alpha, ex2_approx(__fmul_rn(__fmul_rn(-rr, rr),
                                                                     Q.ibeta * 1.4426950408889634f))));
  }
  const float a = __fmul_rn(de, rinv);  // S r
  const float S = __fmul_rn(a, rinv);
  bs2 = __fmul_rn(a, S);
  s0 = __fmul_rn(kw, __fmul_rn(S, rinv));
  ex = ex2_approx(__fmul_rn(Q.nbl2e, bs2));
}

// Two bonds a, b at once, lane x = a, lane y = b, by packed FP32 pair
// operations: every lane value equals what tile_bond_core gives that bond
// (the same separately rounded operations; rsqrt and exp2 per lane).
// Returns s1 = s0 ex (the unbroken bond's force per unit xi) and bs2.
// INTERIOR: both bonds lie where the volume factor is 1 (a row's interior
// prefix, with a constant influence function): kw is K1 V (or V_j's term)
// itself, the value the general form gives there, without forming r.
template <int OPT, bool KV, bool UV, bool INTERIOR = false>
__device__ __forceinline__ void tile_bond_pair(const Params32 &Q, float2 dx, float2 dy, float2 ex,
                                               float2 ey, float2 vj, float2 &s1, float2 &bs2) {
  const float2 r2 = __ffma2_rn(dy, dy, __ffma2_rn(dx, dx, make_float2(1e-30f, 1e-30f)));
  const float2 de = __ffma2_rn(dy, ey, __fmul2_rn(dx, ex));
  const float2 rinv = make_float2(rsqrt_approx(r2.x), rsqrt_approx(r2.y));
  float2 kw;
  if (INTERIOR) {
    kw = UV ? make_float2(Q.kv_uniform, Q.kv_uniform)
            : (KV ? vj : __fmul2_rn(make_float2(Q.K1, Q.K1), vj));
  } else {
    const float2 r = __fmul2_rn(r2, rinv);
    // fma(-r, a, b) formed as fma(r, -a, b): the same value
    if (UV) {
      const float2 t = __ffma2_rn(r, make_float2(-Q.kv_ih, -Q.kv_ih),
                                  make_float2(Q.kv_cuih, Q.kv_cuih));
      kw = make_float2(fminf(Q.kv_uniform, t.x), fminf(Q.kv_uniform, t.y));
    } else {
      const float2 t = __ffma2_rn(r, make_float2(-Q.inv_h, -Q.inv_h),
                                  make_float2(Q.cu_ih, Q.cu_ih));
      const float2 kv = KV ? vj : __fmul2_rn(make_float2(Q.K1, Q.K1), vj);
      kw = __fmul2_rn(kv, make_float2(fminf(1.f, t.x), fminf(1.f, t.y)));
    }
    if (!(OPT & OPT_CONSTJ) && Q.infl_type != 0) {
      const float2 rr = __fmul2_rn(r, make_float2(Q.inv_delta, Q.inv_delta));
      float2 j;
      if (Q.infl_type == 1) {
        j = __ffma2_rn(make_float2(Q.a1, Q.a1), rr, make_float2(Q.a0, Q.a0));
      } else {
        const float c = Q.ibeta * 1.4426950408889634f;  // (-rr rr) c = (rr rr) (-c)
        const float2 z = __fmul2_rn(__fmul2_rn(rr, rr), make_float2(-c, -c));
        j = __fmul2_rn(make_float2(Q.alpha, Q.alpha), make_float2(ex2_approx(z.x), ex2_approx(z.y)));
      }
      kw = __fmul2_rn(kw, j);
    }
  }
  const float2 a = __fmul2_rn(de, rinv);  // S r
  const float2 S = __fmul2_rn(a, rinv);
  bs2 = __fmul2_rn(a, S);
  const float2 s0 = __fmul2_rn(kw, __fmul2_rn(S, rinv));
  const float2 z = __fmul2_rn(make_float2(Q.nbl2e, Q.nbl2e), bs2);
  s1 = __fmul2_rn(s0, make_float2(ex2_approx(z.x), ex2_approx(z.y)));
}

__device__ __forceinline__ float4 lds_f4(const char *base, uint32_t off) {
  return *reinterpret_cast<const float4 *>(base + off);
}
__device__ __forceinline__ float2 lds_f2(const char *base, uint32_t off) {
  return *reinterpret_cast<const float2 *>(base + off);
}
__device__ __forceinline__ float lds_f(const char *base, uint32_t off) {
  return *reinterpret_cast<const float *>(base + off);
}

// Staged arrays of a tile, as byte addresses for offset arithmetic.
struct TileShared {
  const char *xu;   // float4 per staged node (16 bytes: the offset unit)
  const char *vol;  // float per staged node (offset / 4)
  const char *ul;   // float2 per staged node (offset / 2), exact mode
  const uint8_t *fl;
};

// xi, eta and the volume term of the bond at staged byte offset o.
template <bool UV, bool EXACT>
__device__ __forceinline__ void tile_bond_data(const TileShared &S, uint32_t o, float2 xi_x,
                                               float2 xi_u, float2 uli, float kvu, float2 &d,
                                               float2 &e, float &vj) {
  const float4 xj = lds_f4(S.xu, o);
  d = sub_f32x2(make_float2(xj.x, xj.y), xi_x);
  e = sub_f32x2(make_float2(xj.z, xj.w), xi_u);
  if (EXACT) {
    const float2 ulj = lds_f2(S.ul, o >> 1);
    const float2 dl = sub_f32x2(ulj, uli);
    e = make_float2(e.x + dl.x, e.y + dl.y);
  }
  vj = UV ? kvu : lds_f(S.vol, o >> 2);
}

// The force on node i (row of len bonds at sb) and, in the full loop, its
// bond-state bits; then the integrator epilogue.
template <int SCHEME, bool NW1, int OPT, bool BATCH, bool UV, bool EXACT>
__device__ __forceinline__ void tilel_node(const StepParams &P, const Params32 &Qn,
                                           const DevPtrs &D, const BCTable &T, const StepArgs &A,
                                           const TileShared &S, const uint2 *sb, int64_t i, int il,
                                           uint8_t fl, int len, int nint, uint32_t word,
                                           float4 ui4, const float4 *vpre, const float2 *fpre) {
  constexpr bool KV = !(OPT & OPT_CONTACT) && !BATCH;
  constexpr bool FAST = !(OPT & (OPT_NOFAIL | OPT_CONTACT));
  const int ng = (len + 3) >> 2;
  const float4 xi = reinterpret_cast<const float4 *>(S.xu)[il];
  const float2 xi_x = make_float2(xi.x, xi.y), xi_u = make_float2(xi.z, xi.w);
  const float2 uli = EXACT ? reinterpret_cast<const float2 *>(S.ul)[il] : make_float2(0.f, 0.f);
  const float voli = reinterpret_cast<const float *>(S.vol)[il];  // contact term only (raw V)
  const float kvu = Qn.kv_uniform;
  float uih[3] = {ui4.x, ui4.y, 0.f}, uil[3] = {ui4.z, ui4.w, 0.f};
  const bool brk_i = !(fl & FLAG_NOFAIL);
  float fi[3] = {0.f, 0.f, 0.f};
  bool full = !FAST;
  if (FAST) {
    if (!NW1)
      for (int w = 0; w * 32 < len; w++) word |= D.bits[(int64_t)w * P.npad + i];
    full = word != 0u;
  }
  if (FAST && !full && !EXACT) {
    // bonds in pairs (lane x: bonds 0, 2 of a group; lane y: bonds 1, 3),
    // each lane summing its own share of the force; the row's interior
    // prefix (nint bonds, whole groups) skips the volume factor
    float mx = 0.f;  // largest S^2 r of the row
    float2 fx = make_float2(0.f, 0.f), fy = make_float2(0.f, 0.f);
    auto group = [&](const uint2 cur, auto interior) {
      constexpr bool IN = decltype(interior)::value;
      const uint32_t o[4] = {cur.x & 0xffffu, cur.x >> 16, cur.y & 0xffffu, cur.y >> 16};
      float4 xj[4];
      float vj[4];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        xj[q] = lds_f4(S.xu, o[q]);
        vj[q] = UV ? kvu : lds_f(S.vol, o[q] >> 2);
      }
#pragma unroll
      for (int p = 0; p < 2; p++) {
        const float4 A = xj[2 * p], B = xj[2 * p + 1];
        const float2 dx = make_float2(__fsub_rn(A.x, xi.x), __fsub_rn(B.x, xi.x));
        const float2 dy = make_float2(__fsub_rn(A.y, xi.y), __fsub_rn(B.y, xi.y));
        const float2 ex = make_float2(__fsub_rn(A.z, xi.z), __fsub_rn(B.z, xi.z));
        const float2 ey = make_float2(__fsub_rn(A.w, xi.w), __fsub_rn(B.w, xi.w));
        float2 s1, bs2;
        tile_bond_pair<OPT, KV, UV, IN>(Qn, dx, dy, ex, ey,
                                        make_float2(vj[2 * p], vj[2 * p + 1]), s1, bs2);
        mx = fmax3(mx, bs2.x, bs2.y);
        fx = __ffma2_rn(s1, dx, fx);
        fy = __ffma2_rn(s1, dy, fy);
      }
    };
    const int gi = min(nint >> 2, ng);
    uint2 nxt = ng > 0 ? sb[0] : make_uint2(0u, 0u);  // ids one group ahead
#pragma unroll 1
    for (int g = 0; g < gi; g++) {
      const uint2 cur = nxt;
      if (g + 1 < ng) nxt = sb[32 * (g + 1)];
      group(cur, std::true_type{});
    }
#pragma unroll 1
    for (int g = gi; g < ng; g++) {
      const uint2 cur = nxt;
      if (g + 1 < ng) nxt = sb[32 * (g + 1)];
      group(cur, std::false_type{});
    }
    fi[0] = __fadd_rn(fx.x, fx.y);
    fi[1] = __fadd_rn(fy.x, fy.y);
    full = mx > Qn.ksc_on;
  } else if (FAST && !full) {
    float mx = 0.f;  // largest S^2 r of the row
    uint2 nxt = ng > 0 ? sb[0] : make_uint2(0u, 0u);  // ids one group ahead
#pragma unroll 2
    for (int g = 0; g < ng; g++) {
      const uint2 cur = nxt;
      if (g + 1 < ng) nxt = sb[32 * (g + 1)];
      const uint32_t o[4] = {cur.x & 0xffffu, cur.x >> 16, cur.y & 0xffffu, cur.y >> 16};
      float2 d[4], e[4];
      float vj[4];
#pragma unroll
      for (int q = 0; q < 4; q++)
        tile_bond_data<UV, EXACT>(S, o[q], xi_x, xi_u, uli, kvu, d[q], e[q], vj[q]);
#pragma unroll
      for (int q = 0; q < 4; q++) {
        float s0, ex, bs2, r;
        tile_bond_core<OPT, KV, UV>(Qn, d[q], e[q], vj[q], s0, ex, bs2, r);
        const float s1 = __fmul_rn(s0, ex);
        mx = fmaxf(mx, bs2);
        fi[0] = fmaf(s1, d[q].x, fi[0]);
        fi[1] = fmaf(s1, d[q].y, fi[1]);
      }
    }
    full = mx > Qn.ksc_on;
  }
  if (full) {
    // the rows with broken bonds, bonds breaking now, no-fail or contact
    // terms: bond-state bits kept per bond
    fi[0] = fi[1] = 0.f;
    uint32_t nw = 0;
    word = NW1 ? D.bits[i] : 0u;
    for (int g = 0; g < ng; g++) {
      const uint2 c = sb[32 * g];
      if (!NW1 && (g & 7) == 0) {
        if (nw) D.bits[(int64_t)((g >> 3) - 1) * P.npad + i] = word | nw;
        word = D.bits[(int64_t)(g >> 3) * P.npad + i];
        nw = 0;
      }
      const uint32_t o[4] = {c.x & 0xffffu, c.x >> 16, c.y & 0xffffu, c.y >> 16};
      const int sh = (4 * g) & 31;
      const uint32_t w4 = word >> sh;
      uint32_t n4 = 0;
#pragma unroll
      for (int q = 0; q < 4; q++) {
        float2 d, e;
        float vj;
        tile_bond_data<UV, EXACT>(S, o[q], xi_x, xi_u, uli, kvu, d, e, vj);
        float s0, ex, bs2, r;
        tile_bond_core<OPT, KV, UV>(Qn, d, e, vj, s0, ex, bs2, r);
        bool fs = (w4 >> q) & 1u;
        bool breakable = true;
        if (OPT & OPT_NOFAIL) breakable = brk_i && !(S.fl[o[q] >> 4] & FLAG_NOFAIL);
        if (breakable) fs = fs || bs2 > Qn.ksc_on;
        float sc;
        if (!breakable) {
          // no-fail bond: the linearised force 4 J S C beta / invF V_j^c
          sc = s0;
        } else if ((OPT & OPT_CONTACT) && fs) {
          // broken bond: normal contact only (rnpBond.cpp:281-291), along the
          // deformed bond y = xi + eta
          const float y0 = d.x + e.x, y1 = d.y + e.y;
          const float R = sqrtf(y0 * y0 + y1 * y1);
          const float vjc = vj * fminf(1.f, __fmaf_rn(-r, Qn.inv_h, Qn.cu_ih));
          const float sf = Qn.kn * (voli * vjc / (voli + vjc)) * (Qn.rc - R) / R;
          d = make_float2(y0, y1);
          sc = -fmaxf(sf, 0.f);
        } else {
          sc = fs ? 0.f : __fmul_rn(s0, ex);
        }
        n4 |= fs ? 1u << q : 0u;
        fi[0] = fmaf(sc, d.x, fi[0]);
        fi[1] = fmaf(sc, d.y, fi[1]);
      }
      nw |= n4 << sh;
    }
    // bits past the row's end stay clear
    if (len & 31) nw &= (1u << (len & 31)) - 1u;
    if (nw) D.bits[NW1 ? i : (int64_t)((len - 1) >> 5) * P.npad + i] = word | nw;
  }
  integrate_node32<2, SCHEME>(P, Qn, D, T, A, i, fl, uih, uil, fi, vpre, fpre);
}

template <int SCHEME, bool NW1, int OPT, bool BATCH, bool UV>
__global__ void __launch_bounds__(kTileNodes, 4)
    k_rnp32_tilel(const StepParams P, const Params32 Q, const DevPtrs D, const BCTable T,
                  const StepArgs A) {
  // per staged node: x - x_o, y - y_o, and ux - ux_o, uy - uy_o (frame mode)
  // or the hi parts of ux, uy (exact mode, lo parts in s_ul)
  __shared__ float4 s_xu[kTileMaxLocal];
  __shared__ float s_vol[UV ? 1 : kTileMaxLocal];  // K1 V (V with the contact term or in a batch)
  __shared__ float2 s_ul[kTileMaxLocal];
  constexpr bool KV = !(OPT & OPT_CONTACT) && !BATCH;
  __shared__ uint8_t s_fl[(OPT & OPT_NOFAIL) ? kTileMaxLocal : 1];
  // the tile's own velocity pairs and previous forces, for the epilogue
  __shared__ __align__(16) float4 s_vown[kTileNodes];
  __shared__ __align__(16) float2 s_fown[kTileNodes];
  __shared__ __align__(8) uint64_t s_bar;
  __shared__ __align__(16) float s_wspan[kTileNodes / 32];
  extern __shared__ __align__(128) unsigned char s_ids[];  // the tile's id block
  const int tb = A.tiles ? A.tiles[blockIdx.x]
                         : (int)blockIdx.x + (BATCH ? (int)(A.i0 / kTileNodes) : 0);
  const int64_t t0 = (int64_t)tb * kTileNodes;
  const int64_t sl0 = 8 * (int64_t)tb;
  const int64_t ib0 = D.sell_ptr[sl0];
  const int nt = (int)min((int64_t)kTileNodes, P.n - t0);
  // A whole tile's own v (and f of the previous step) arrive by bulk copies
  // on the same barrier as its id block (contiguous, 16-byte aligned: tiles
  // start at multiples of 256 nodes); a partial last tile reads them directly.
  const bool vpre = nt == kTileNodes;
  const bool fpre = vpre && SCHEME == NLM_VELOCITY_VERLET && !A.first;
  // Launched with programmatic stream serialization: everything up to
  // griddepcontrol.wait reads only what no step writes (ids, positions,
  // flags, row layout), so it overlaps the previous step's last blocks; the
  // state (u, v, f, bond bits) is read after the wait, which returns once
  // the previous step's writes are visible.
  if (threadIdx.x == 0) {
    mbar_init(&s_bar, 1);
    const int64_t sl1 = min(sl0 + 8, (P.n + 31) >> 5);
    const uint32_t bytes = (uint32_t)(2 * (D.sell_ptr[sl1] - ib0));
    const uint32_t vb = vpre ? kTileNodes * sizeof(float4) : 0u;
    const uint32_t fb = fpre ? kTileNodes * sizeof(float2) : 0u;
    mbar_arrive_expect(&s_bar, bytes + vb + fb);
    if (bytes > 0) bulk_copy_g2s(s_ids, D.tile_boff + ib0, bytes, &s_bar);
  }
  const int nh = D.tile_hstride;
  const int64_t h0 = (int64_t)tb * nh;
  const float4 *ucur = D.u32[A.cur];
  const float4 po = __ldg(D.pos32 + t0);
  const float2 plo = __half22float2(*reinterpret_cast<const __half2 *>(&po.w));
  const int il = threadIdx.x;
  const int64_t i = t0 + il;
  bool own = il < nt;
  if (BATCH) own = own && i >= A.i0 && i < A.i1;
  const uint8_t fl = own ? D.flags[i] : 0;
  if (BATCH && (fl & FLAG_GHOST)) own = false;
  const int len = own ? D.rowlen[i] : 0;
  const int nint = (own && D.row_int) ? D.row_int[i] : 0;
  const int64_t rbase = own ? D.sell_ptr[i >> 5] : ib0;
  const float4 pown = il < nt ? __ldg(D.pos32 + i) : make_float4(0.f, 0.f, 0.f, 0.f);
  const uint8_t fown = ((OPT & OPT_NOFAIL) && il < nt) ? D.flags[i] : 0;
  // the first round of halo entries (two per thread): ids and positions
  int g0[2];
  float4 a0[2];
  uint8_t f0[2] = {0, 0};
#pragma unroll
  for (int q = 0; q < 2; q++) {
    const int e = il + q * kTileNodes;
    g0[q] = e < nh ? __ldg(D.tile_halo + h0 + e) : -1;
  }
#pragma unroll
  for (int q = 0; q < 2; q++)
    if (g0[q] >= 0) {
      a0[q] = __ldg(D.pos32 + g0[q]);
      if (OPT & OPT_NOFAIL) f0[q] = D.flags[g0[q]];
    }
  pdl_trigger_and_wait();
  if (threadIdx.x == 0) {
    if (vpre)
      bulk_copy_g2s(s_vown, D.v32[SCHEME == NLM_VELOCITY_VERLET ? 0 : A.cur] + t0,
                    kTileNodes * sizeof(float4), &s_bar);
    if (fpre)
      bulk_copy_g2s(s_fown, reinterpret_cast<const float2 *>(D.f32) + t0,
                    kTileNodes * sizeof(float2), &s_bar);
  }
  const float4 uo = ucur[t0];
  const uint32_t word = (NW1 && own) ? D.bits[i] : 0u;
  const float4 ui4 = il < nt ? __ldg(ucur + i) : make_float4(0.f, 0.f, 0.f, 0.f);
  // Staging: two halo entries per thread per round, the first round's ids
  // and positions already loaded above; then the displacements together,
  // so a thread waits for memory once per round.
  float span = 0.f;  // largest |u - u_o| staged by this thread
  auto stage = [&](int e, const float4 a, const float4 u, uint8_t f) {
    const float2 lo = __half22float2(*reinterpret_cast<const __half2 *>(&a.w));
    const float dux = (u.x - uo.x) + (u.z - uo.z), duy = (u.y - uo.y) + (u.w - uo.w);
    span = fmax3(span, fabsf(dux), fabsf(duy));
    s_xu[e] = make_float4(fmaf(lo.x - plo.x, Q.inv_lo, a.x - po.x),
                          fmaf(lo.y - plo.y, Q.inv_lo, a.y - po.y), dux, duy);
    if (!UV) s_vol[e] = KV ? Q.K1 * a.z : a.z;
    if (OPT & OPT_NOFAIL) s_fl[e] = f;
  };
  for (int base = 0; base < nh; base += 2 * kTileNodes) {
    int g[2] = {g0[0], g0[1]};
    float4 a[2] = {a0[0], a0[1]}, u[2];
    uint8_t f[2] = {f0[0], f0[1]};
    if (base > 0) {
#pragma unroll
      for (int q = 0; q < 2; q++) {
        const int e = base + il + q * kTileNodes;
        g[q] = e < nh ? __ldg(D.tile_halo + h0 + e) : -1;
      }
#pragma unroll
      for (int q = 0; q < 2; q++)
        if (g[q] >= 0) {
          a[q] = __ldg(D.pos32 + g[q]);
          if (OPT & OPT_NOFAIL) f[q] = D.flags[g[q]];
        }
    }
#pragma unroll
    for (int q = 0; q < 2; q++)
      if (g[q] >= 0) u[q] = __ldg(ucur + g[q]);
#pragma unroll
    for (int q = 0; q < 2; q++)
      if (g[q] >= 0) stage(kTileNodes + base + il + q * kTileNodes, a[q], u[q], f[q]);
  }
  if (il < nt) stage(il, pown, ui4, fown);
  // the tile's displacement span (NaN counts as too large): non-negative
  // floats order as their bit patterns, so one warp reduction takes the max
  const float wspan = __uint_as_float(__reduce_max_sync(0xffffffffu, __float_as_uint(span)));
  if ((threadIdx.x & 31) == 0) s_wspan[threadIdx.x >> 5] = wspan != wspan ? 3e38f : wspan;
  __syncthreads();
  static_assert(kTileNodes / 32 == 8, "eight warp spans");
  const float4 w0 = reinterpret_cast<const float4 *>(s_wspan)[0];
  const float4 w1 = reinterpret_cast<const float4 *>(s_wspan)[1];
  const float bspan =
      fmax3(fmax3(w0.x, w0.y, w0.z), fmax3(w0.w, w1.x, w1.y), fmaxf(w1.z, w1.w));
  const bool exact = bspan > Q.span_max;
  if (exact) {
    // block-uniform: restage eta's inputs as (hi, lo) pairs
    for (int e = threadIdx.x; e < kTileNodes + nh; e += blockDim.x) {
      if (e < kTileNodes && e >= nt) continue;
      const int64_t g = e < kTileNodes ? t0 + e : (int64_t)D.tile_halo[h0 + e - kTileNodes];
      if (g < 0) continue;  // an empty slot of a lattice-ordered halo
      const float4 u = ucur[g];
      s_xu[e].z = u.x;
      s_xu[e].w = u.y;
      s_ul[e] = make_float2(u.z, u.w);
    }
    __syncthreads();
  }
  // the id block; a wait that gives up (which only a failing copy would
  // cause) flags the error, waits once more for the copy and leaves
  if (!mbar_wait(&s_bar, 0, 1u << 22)) {
    if (threadIdx.x == 0) atomicExch(D.err, 1);
    mbar_wait(&s_bar, 0, 1u << 22);
    return;
  }
  if (!own) return;
  const Params32 &Qn = BATCH ? static_cast<const Params32 *>(D.qtab)[D.slice_spec[i >> 5]] : Q;
  const uint2 *sb = reinterpret_cast<const uint2 *>(s_ids) + ((rbase - ib0) >> 2) + (i & 31);
  const float4 *vp = vpre ? &s_vown[il] : nullptr;
  const float2 *fp = fpre ? &s_fown[il] : nullptr;
  const TileShared S{reinterpret_cast<const char *>(s_xu), reinterpret_cast<const char *>(s_vol),
                     reinterpret_cast<const char *>(s_ul), s_fl};
  if (exact)
    tilel_node<SCHEME, NW1, OPT, BATCH, UV, true>(P, Qn, D, T, A, S, sb, i, il, fl, len, nint,
                                                  word, ui4, vp, fp);
  else
    tilel_node<SCHEME, NW1, OPT, BATCH, UV, false>(P, Qn, D, T, A, S, sb, i, il, fl, len, nint,
                                                   word, ui4, vp, fp);
}

// Dynamic shared memory above the default 48 KB for the tile-frame kernel's
// id block: opted in once per device and kernel.
template <class K>
static void tile_ids_smem(K kernel, std::atomic<uint64_t> &done) {
  int dev = 0;
  cudaGetDevice(&dev);
  const uint64_t bit = 1ull << (dev & 63);
  if (done.load() & bit) return;
  if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           kTileIdsMaxBytes) == cudaSuccess)
    done.fetch_or(bit);
}

// One launch of the tile-frame kernel; with a.pdl set, with programmatic
// stream serialization (the kernel's griddepcontrol.wait orders its state
// reads after the previous step).
template <class K>
static void tilel_go(K kernel, const StepParams &P, const Params32 &Q, const DevPtrs &D,
                     const BCTable &T, const StepArgs &a, unsigned grid, size_t dyn,
                     cudaStream_t s) {
  launch_pdl(kernel, grid, kTileNodes, dyn, s, a.pdl, P, Q, D, T, a);
}

template <int SCHEME, int OPT, bool BATCH, bool UV>
static void tilel_launch(const StepParams &P, const Params32 &Q, const DevPtrs &D,
                         const BCTable &T, const StepArgs &a, unsigned grid, size_t dyn,
                         cudaStream_t s) {
  if (P.nw1) {
    static std::atomic<uint64_t> opt{0};
    tile_ids_smem(k_rnp32_tilel<SCHEME, true, OPT, BATCH, UV>, opt);
    tilel_go(k_rnp32_tilel<SCHEME, true, OPT, BATCH, UV>, P, Q, D, T, a, grid, dyn, s);
  } else {
    static std::atomic<uint64_t> opt{0};
    tile_ids_smem(k_rnp32_tilel<SCHEME, false, OPT, BATCH, UV>, opt);
    tilel_go(k_rnp32_tilel<SCHEME, false, OPT, BATCH, UV>, P, Q, D, T, a, grid, dyn, s);
  }
}

template <int DIM, int SCHEME, int OPT, bool BATCH>
static void launch_opt(const StepParams &P, const Params32 &Q, const DevPtrs &D,
                       const BCTable &T, const StepArgs &a, int decomp, cudaStream_t s) {
  const int64_t nodes = a.i1 - a.i0;
  if (nodes <= 0) return;
  if (DIM == 2 && !BATCH && decomp == NLM_DECOMP_TILE) {
    // the tile store covers the whole node range [0, n); a tile list picks
    // some of its tiles
    const unsigned grid =
        a.tiles ? (unsigned)a.ntiles : (unsigned)((P.n + kTileNodes - 1) / kTileNodes);
    if (grid == 0) return;
    if (P.nw1)
      k_rnp32_tile<SCHEME, true, OPT><<<grid, kTileNodes, 0, s>>>(P, Q, D, T, a);
    else
      k_rnp32_tile<SCHEME, false, OPT><<<grid, kTileNodes, 0, s>>>(P, Q, D, T, a);
    return;
  }
  if (DIM == 2 && decomp == NLM_DECOMP_TILE_LOCAL && D.tile_boff) {
    // a batch launch covers the tiles that meet its node range
    const unsigned grid =
        a.tiles ? (unsigned)a.ntiles
        : BATCH ? (unsigned)((a.i1 + kTileNodes - 1) / kTileNodes - a.i0 / kTileNodes)
                : (unsigned)((P.n + kTileNodes - 1) / kTileNodes);
    if (grid == 0) return;
    const size_t dyn = (size_t)D.tile_ids_bytes;
    // one nodal volume for the whole model (for a batch: per specimen, the
    // constants in each specimen's table): K1 V as a constant
    constexpr bool UVOK = !(OPT & OPT_CONTACT);
    if (UVOK && (BATCH ? P.uv_specimens != 0 : Q.kv_uniform > 0.f)) {
      tilel_launch<SCHEME, OPT, BATCH, UVOK>(P, Q, D, T, a, grid, dyn, s);
    } else {
      tilel_launch<SCHEME, OPT, BATCH, false>(P, Q, D, T, a, grid, dyn, s);
    }
    return;
  }
  if (decomp == NLM_DECOMP_WARP) {
    const int bs = 256;
    const unsigned grid = (unsigned)((nodes * 32 + bs - 1) / bs);
    k_rnp32_warp<DIM, SCHEME, OPT, BATCH><<<grid, bs, 0, s>>>(P, Q, D, T, a);
    return;
  }
  const int bs = 128;
  const unsigned grid = (unsigned)((nodes + bs - 1) / bs);
  if (decomp == NLM_DECOMP_THREAD1) {
    if (P.nw1)
      k_rnp32_thread1<DIM, SCHEME, true, OPT, BATCH><<<grid, bs, 0, s>>>(P, Q, D, T, a);
    else
      k_rnp32_thread1<DIM, SCHEME, false, OPT, BATCH><<<grid, bs, 0, s>>>(P, Q, D, T, a);
  } else {
    if (P.nw1)
      k_rnp32_thread<DIM, SCHEME, true, OPT, BATCH><<<grid, bs, 0, s>>>(P, Q, D, T, a);
    else
      k_rnp32_thread<DIM, SCHEME, false, OPT, BATCH><<<grid, bs, 0, s>>>(P, Q, D, T, a);
  }
}

template <int DIM, int SCHEME>
static cudaError_t launch32(const StepParams &P, const DevPtrs &D, const BCTable &T,
                            const StepArgs &a, int decomp, cudaStream_t s) {
  if (P.n == 0) return cudaSuccess;
  const Params32 Q = make_p32(P);
  const int opt = (P.infl_type == 0 ? OPT_CONSTJ : 0) | (P.nofail ? OPT_NOFAIL : 0) |
                  (P.contact ? OPT_CONTACT : 0);
  const bool batch = D.qtab != nullptr;
  if (batch) {
    // specimens may mix influence functions: the batch path always takes the
    // general influence evaluation
    if (P.nofail)
      launch_opt<DIM, SCHEME, OPT_NOFAIL, true>(P, Q, D, T, a, decomp, s);
    else
      launch_opt<DIM, SCHEME, 0, true>(P, Q, D, T, a, decomp, s);
    return cudaGetLastError();
  }
  switch (opt) {
    case 0: launch_opt<DIM, SCHEME, 0, false>(P, Q, D, T, a, decomp, s); break;
    case 1: launch_opt<DIM, SCHEME, 1, false>(P, Q, D, T, a, decomp, s); break;
    case 2: launch_opt<DIM, SCHEME, 2, false>(P, Q, D, T, a, decomp, s); break;
    case 3: launch_opt<DIM, SCHEME, 3, false>(P, Q, D, T, a, decomp, s); break;
    case 4: launch_opt<DIM, SCHEME, 4, false>(P, Q, D, T, a, decomp, s); break;
    case 5: launch_opt<DIM, SCHEME, 5, false>(P, Q, D, T, a, decomp, s); break;
    case 6: launch_opt<DIM, SCHEME, 6, false>(P, Q, D, T, a, decomp, s); break;
    default: launch_opt<DIM, SCHEME, 7, false>(P, Q, D, T, a, decomp, s); break;
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

// One node's drift from the state (u, v, f) of the last step: the second
// half of integrate_node32, prescribed dofs from the loading at t_next.
template <int DIM>
__device__ __forceinline__ void drift_node32(const StepParams &P, const Params32 &Q,
                                             const DevPtrs &D, const BCTable &T, uint8_t fl,
                                             int ref, const float uh[3], const float ul[3],
                                             const float vh[3], const float vl[3],
                                             const float f[3], double t_next, df un[3],
                                             df vn[3]) {
  for (int c = 0; c < DIM; c++) {
    if (!(fl >> c & 1)) {
      const df u{uh[c], ul[c]}, v{vh[c], vl[c]};
      if (P.scheme == NLM_VELOCITY_VERLET) {
        un[c] = vv_drift(Q, u, v, f[c]);
        vn[c] = v;
      } else {
        const df inc = df_add(df_cmul(Q.c_hi, Q.c_lo, f[c]), df_mul_c(v, Q.dt_hi, Q.dt_lo));
        un[c] = df_add(u, inc);
        vn[c] = df_mul_c(df_sub(un[c], u), Q.idt_hi, Q.idt_lo);
      }
    } else {
      bc_df(D, T, ref, c, t_next, un[c], vn[c]);
    }
  }
}

// Drift after a host state upload.
template <int DIM>
__global__ void k_drift32(const StepParams P, const Params32 Q, const DevPtrs D,
                          const BCTable T, int cur, double t_next) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  const uint8_t fl = D.flags[i];
  const int ref = (fl & 7) ? D.bcref[i] : -1;
  float uh[3], ul[3], vh[3], vl[3], f[3] = {0.f, 0.f, 0.f};
  ld_pair<DIM>(D.u32[cur], i, uh, ul);
  ld_pair<DIM>(D.v32[P.scheme == NLM_CENTRAL_DIFFERENCE ? cur : 0], i, vh, vl);
  for (int c = 0; c < DIM; c++) f[c] = D.f32[(int64_t)(DIM == 2 ? 2 : 4) * i + c];
  df un[3], vn[3];
  drift_node32<DIM>(P, Q, D, T, fl, ref, uh, ul, vh, vl, f, t_next, un, vn);
  st_pair<DIM>(D.u32[1 - cur], i, un);
  if (P.scheme == NLM_CENTRAL_DIFFERENCE) st_pair<DIM>(D.v32[1 - cur], i, vn);
}

// Banded host step (2-D velocity Verlet, FP32C), input side: caller nodes
// [o0, o1) of the staged caller arrays (caller order, 3 doubles per node)
// into the internal order -- the drifted u into ua, v and f as the step
// kernel reads them -- with the same (hi, lo) splits as a whole-state upload,
// and a flag for any non-finite value.
__global__ void k_pipe_in32(const StepParams P, const Params32 Q, const DevPtrs D,
                            const BCTable T, double t_next, int64_t o0, int64_t o1,
                            const int *iperm, const double *hu, const double *hv,
                            const double *hf, float4 *ua, float4 *sv, float2 *sf, int *bad) {
  const int64_t o = o0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (o >= o1) return;
  double u[3], v[3], f[3];
  bool ok = true;
  for (int d = 0; d < 3; d++) {
    u[d] = hu[3 * o + d];
    v[d] = hv[3 * o + d];
    f[d] = hf[3 * o + d];
    ok = ok && isfinite(u[d]) && isfinite(v[d]) && isfinite(f[d]);
  }
  if (!ok) atomicExch(bad, 1);
  const int64_t i = iperm[o];
  const uint8_t fl = D.flags[i];
  const int ref = (fl & 7) ? D.bcref[i] : -1;
  float uh[3] = {0.f, 0.f, 0.f}, ul[3] = {0.f, 0.f, 0.f}, vh[3] = {0.f, 0.f, 0.f},
        vl[3] = {0.f, 0.f, 0.f}, fs[3] = {0.f, 0.f, 0.f};
  for (int c = 0; c < 2; c++) {
    const df a = df_from_double(u[c]), b = df_from_double(v[c]);
    uh[c] = a.hi;
    ul[c] = a.lo;
    vh[c] = b.hi;
    vl[c] = b.lo;
    fs[c] = __double2float_rn(f[c]);
  }
  df un[3], vn[3];
  drift_node32<2>(P, Q, D, T, fl, ref, uh, ul, vh, vl, fs, t_next, un, vn);
  st_pair<2>(ua, i, un);
  sv[i] = make_float4(vh[0], vh[1], vl[0], vl[1]);
  sf[i] = make_float2(fs[0], fs[1]);
}

// Output side: caller nodes [o0, o1) (or list[o0 .. o1) when a list is
// given) after the step, as doubles in the caller order -- u from ua, v and f
// as the step wrote them -- with the caller's own z of u and v (the 2-D
// integrator never changes it) and f's z = 0.
__global__ void k_pipe_out32(int64_t o0, int64_t o1, const int *list, const int *iperm,
                             const float4 *ua, const float4 *sv, const float2 *sf,
                             const double *hu_in, const double *hv_in, double *ou, double *ov,
                             double *of) {
  const int64_t t = o0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= o1) return;
  const int64_t o = list ? (int64_t)list[t] : t;
  const int64_t i = iperm[o];
  const float4 a = ua[i], b = sv[i];
  const float2 c = sf[i];
  ou[3 * o] = (double)a.x + (double)a.z;
  ou[3 * o + 1] = (double)a.y + (double)a.w;
  ou[3 * o + 2] = hu_in[3 * o + 2];
  ov[3 * o] = (double)b.x + (double)b.z;
  ov[3 * o + 1] = (double)b.y + (double)b.w;
  ov[3 * o + 2] = hv_in[3 * o + 2];
  of[3 * o] = (double)c.x;
  of[3 * o + 1] = (double)c.y;
  of[3 * o + 2] = 0.;
}

// End of a banded step: with a finite input the step's arrays become the
// state (u now, u of the next step, v, f); otherwise the bond bits the step
// may have set are put back and the state is left as it was.
__global__ void k_pipe_commit32(int64_t n, int64_t nbits, const int *bad, const float4 *ua,
                                const float4 *ub, const float4 *sv, const float2 *sf,
                                float4 *u_now, float4 *u_next, float4 *v, float2 *f,
                                uint32_t *bits, const uint32_t *bits_saved) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (*bad) {
    if (k < nbits) bits[k] = bits_saved[k];
    return;
  }
  if (k < n) {
    u_now[k] = ua[k];
    u_next[k] = ub[k];
    v[k] = sv[k];
    f[k] = sf[k];
  }
}

cudaError_t launch_pipe_in32(const StepParams &P, const DevPtrs &D, const BCTable &T,
                             double t_next, int64_t o0, int64_t o1, const int *iperm,
                             const double *hu, const double *hv, const double *hf, float4 *ua,
                             float4 *sv, float2 *sf, int *bad, cudaStream_t s) {
  if (o1 <= o0) return cudaSuccess;
  const Params32 Q = make_p32(P);
  k_pipe_in32<<<(unsigned)((o1 - o0 + 255) / 256), 256, 0, s>>>(P, Q, D, T, t_next, o0, o1,
                                                                 iperm, hu, hv, hf, ua, sv, sf,
                                                                 bad);
  return cudaGetLastError();
}

cudaError_t launch_pipe_out32(int64_t o0, int64_t o1, const int *list, const int *iperm,
                              const float4 *ua, const float4 *sv, const float2 *sf,
                              const double *hu_in, const double *hv_in, double *ou, double *ov,
                              double *of, cudaStream_t s) {
  if (o1 <= o0) return cudaSuccess;
  k_pipe_out32<<<(unsigned)((o1 - o0 + 255) / 256), 256, 0, s>>>(o0, o1, list, iperm, ua, sv,
                                                                  sf, hu_in, hv_in, ou, ov, of);
  return cudaGetLastError();
}

cudaError_t launch_pipe_commit32(int64_t n, int64_t nbits, const int *bad, const float4 *ua,
                                 const float4 *ub, const float4 *sv, const float2 *sf,
                                 float4 *u_now, float4 *u_next, float4 *v, float2 *f,
                                 uint32_t *bits, const uint32_t *bits_saved, cudaStream_t s) {
  const int64_t m = std::max(n, nbits);
  if (m == 0) return cudaSuccess;
  k_pipe_commit32<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(n, nbits, bad, ua, ub, sv, sf,
                                                               u_now, u_next, v, f, bits,
                                                               bits_saved);
  return cudaGetLastError();
}

cudaError_t launch_drift32(const StepParams &P, const DevPtrs &D, const BCTable &T, int cur,
                           double t_next, cudaStream_t s) {
  if (P.n == 0) return cudaSuccess;
  const Params32 Q = make_p32(P);
  const unsigned g = (unsigned)((P.n + 255) / 256);
  if (P.dim == 2)
    k_drift32<2><<<g, 256, 0, s>>>(P, Q, D, T, cur, t_next);
  else
    k_drift32<3><<<g, 256, 0, s>>>(P, Q, D, T, cur, t_next);
  return cudaGetLastError();
}

}  // namespace nlm
