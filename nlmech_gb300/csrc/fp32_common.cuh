// fp32_common.cuh -- shared pieces of the FP32-compensated kernels:
// constants, approximate transcendental instructions, double-float
// arithmetic, split node loads and the double-float integrator epilogue.
#pragma once

#include <cuda_fp16.h>

#include <cmath>

#include "fd_internal.h"
#include "state_io.cuh"

namespace nlm {

struct Params32 {
  float check_low_eff;  // r > this  <=>  definitelyGreaterThan(r, check_low)
  float check_up, inv_h, inv_delta;
  float K1;             // 4 C beta / invF (times J when J is constant)
  float Ksc;            // (f_sc rbar)^2 / (1 - 1e-5)^2: |S| > S_c  <=>  S^2 r > Ksc
  float nbl2e;          // -beta * log2(e)
  float inv_lo;         // 1 / lo_scale
  int irrev;
  int infl_type;
  float a0, a1, alpha, ibeta;
  float kn, rc;         // contact: K 18 / (pi delta^5), 0.9 h
  // integrator constants as (hi, lo) pairs
  float c_hi, c_lo;     // Verlet dt/(2 rho) or CD dt^2/rho
  float dt_hi, dt_lo;
  float idt_hi, idt_lo; // 1/dt
  // tile-frame kernel: volume factor min(1, cu_ih - r inv_h), and the
  // break threshold on S^2 r (+inf when breaking is off)
  float cu_ih;
  float ksc_on;
  // largest |u - u_o| of a tile's staged nodes for which bonds are formed
  // from tile-frame displacements; a tile above it forms them from the
  // (hi, lo) pairs
  float span_max;
  float kv_uniform;  // K1 V when every node has the same volume V, else 0
  float kv_ih, kv_cuih;  // K1 V / h and K1 V (delta + h/2) / h (uniform V)
};

inline void split_const(double v, float &hi, float &lo) {
  hi = (float)v;
  lo = (float)(v - (double)hi);
}

inline Params32 make_p32(const StepParams &P) {
  Params32 q;
  q.check_low_eff = (float)(P.check_low / (1.0 - 1e-5));
  q.check_up = (float)P.check_up;
  q.inv_h = (float)(1.0 / P.h);
  q.inv_delta = (float)(1.0 / P.delta);
  double k1 = 4.0 * P.C * P.beta / P.invF;
  if (P.infl_type == 0) k1 *= P.infl_a0;
  q.K1 = (float)k1;
  const double sc = P.fsc * P.rbar / (1.0 - 1e-5);
  q.Ksc = (float)(sc * sc);
  q.nbl2e = (float)(-P.beta * 1.4426950408889634);
  q.inv_lo = (float)(1.0 / P.lo_scale);
  q.irrev = P.irrev;
  q.infl_type = P.infl_type;
  q.a0 = (float)P.infl_a0;
  q.a1 = (float)P.infl_a1;
  q.alpha = (float)P.infl_alpha;
  q.ibeta = P.infl_type == 2 ? (float)(1.0 / P.infl_beta) : 0.f;
  const double c = P.scheme == NLM_VELOCITY_VERLET ? 0.5 * P.dt / P.rho : P.dt * P.dt / P.rho;
  split_const(c, q.c_hi, q.c_lo);
  split_const(P.dt, q.dt_hi, q.dt_lo);
  split_const(1.0 / P.dt, q.idt_hi, q.idt_lo);
  q.kn = P.contact ? (float)P.contact_kn : 0.f;
  q.rc = (float)P.contact_rc;
  q.cu_ih = (float)(P.check_up / P.h);
  q.ksc_on = P.irrev ? q.Ksc : __builtin_huge_valf();
  // The tile frame rounds u - u_o to FP32: 2^-24 span absolute in eta, so
  // 2^-24 span / |xi| in S.  Up to 16 h S_c(delta) of span that is at most
  // 2^-20 of the critical stretch S_c(r) = f_sc rbar / sqrt(r) of any bond.
  q.span_max = P.tile_span_max > 0.
                   ? (float)P.tile_span_max
                   : (float)(16.0 * P.h * P.fsc * P.rbar / std::sqrt(P.delta));
  q.kv_uniform = P.vol_uniform > 0. ? (float)(k1 * P.vol_uniform) : 0.f;
  q.kv_ih = (float)(k1 * P.vol_uniform / P.h);
  q.kv_cuih = (float)(k1 * P.vol_uniform * P.check_up / P.h);
  return q;
}

// ---- FP32 approximate transcendental instructions -------------------------
__device__ __forceinline__ float rsqrt_approx(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float rcp_approx(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// largest of three (sm_100 and later: one instruction); NaN inputs are
// ignored as by fmaxf
__device__ __forceinline__ float fmax3(float a, float b, float c) {
  float m;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(m) : "f"(a), "f"(b), "f"(c));
  return m;
}

// ---- packed FP32 pairs (sm_100 and later: one instruction for both lanes) --
__device__ __forceinline__ float2 sub_f32x2(float2 a, float2 b) {
  unsigned long long ra, rb, rd;
  asm("mov.b64 %0, {%1,%2};" : "=l"(ra) : "f"(a.x), "f"(a.y));
  asm("mov.b64 %0, {%1,%2};" : "=l"(rb) : "f"(b.x), "f"(b.y));
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(rd) : "l"(ra), "l"(rb));
  float2 d;
  asm("mov.b64 {%0,%1}, %2;" : "=f"(d.x), "=f"(d.y) : "l"(rd));
  return d;
}

// ---- bulk global -> shared copies completed on an mbarrier -----------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
  // make the initialised barrier visible to the copy engine (async proxy)
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// One arrival that also announces `bytes` of copies to complete on the
// barrier (the sum of the copies issued after it).
__device__ __forceinline__ void mbar_arrive_expect(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
// The copy of `bytes` (16-byte aligned addresses, a multiple of 16 bytes)
// completing on the barrier.
__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, uint32_t bytes,
                                              uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
// Wait for phase `parity` of the barrier, giving up after `limit` polls
// (each poll may suspend the thread for a short while); false on give-up.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, uint32_t limit) {
  for (uint32_t it = 0; it < limit; it++) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}" : "=r"(done) : "r"(smem_u32(bar)), "r"(parity) : "memory");
    if (done) return true;
  }
  return false;
}

// ---- launches with programmatic stream serialization ------------------------
// With pdl set the kernel may start while the previous kernel on the stream
// finishes its last blocks; it must read nothing that kernel writes before
// its griddepcontrol.wait, which returns once those writes are visible.
template <class K, class... Args>
static cudaError_t launch_pdl(K kernel, unsigned grid, unsigned block, size_t dyn,
                              cudaStream_t s, bool pdl, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = dyn;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}
__device__ __forceinline__ void pdl_trigger_and_wait() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
}

// ---- double-float arithmetic (error-free transformations) ------------------
struct df {
  float hi, lo;
};
__device__ __forceinline__ df two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ df fast_two_sum(float a, float b) {
  const float s = a + b;
  return {s, b - (s - a)};
}
__device__ __forceinline__ df df_add(df x, df y) {
  const df s = two_sum(x.hi, y.hi);
  return fast_two_sum(s.hi, s.lo + (x.lo + y.lo));
}
__device__ __forceinline__ df df_sub(df x, df y) { return df_add(x, {-y.hi, -y.lo}); }
// (c_hi + c_lo) * y for a float y, as a pair
__device__ __forceinline__ df df_cmul(float c_hi, float c_lo, float y) {
  const float p = c_hi * y;
  const float e = fmaf(c_hi, y, -p);
  return fast_two_sum(p, fmaf(c_lo, y, e));
}
// x * (c_hi + c_lo)
__device__ __forceinline__ df df_mul_c(df x, float c_hi, float c_lo) {
  const float p = x.hi * c_hi;
  float e = fmaf(x.hi, c_hi, -p);
  e = fmaf(x.lo, c_hi, fmaf(x.hi, c_lo, e));
  return fast_two_sum(p, e);
}
// x + y for a pair x and a float y
__device__ __forceinline__ df df_add_f(df x, float y) {
  const df s = two_sum(x.hi, y);
  return fast_two_sum(s.hi, s.lo + x.lo);
}
// Velocity-Verlet drift of one dof, u + dt (v + fact f): the increments fact f
// and dt v^{m+1/2} are formed in FP32 -- f is itself an FP32 sum, so their
// rounding is at the level of its own error -- and added to the (hi, lo)
// pairs without loss.  The fused step and the drift of a host-supplied state
// both use it, so they agree bit for bit.
__device__ __forceinline__ df vv_drift(const Params32 &Q, df u, df v, float f) {
  const df vh2 = df_add_f(v, __fmul_rn(Q.c_hi, f));
  return df_add_f(u, __fmul_rn(Q.dt_hi, vh2.hi));
}
__device__ __forceinline__ df df_from_double(double v) {
  const float h = __double2float_rn(v);
  return {h, __double2float_rn(v - (double)h)};
}

// ---- node access -----------------------------------------------------------
template <int DIM>
struct Node32 {
  float xh[3];
  __half2 lxy;  // lo of (x, y), scaled
  __half2 lz;   // lo of z (3-D), scaled
  float vol;
};

template <int DIM>
__device__ __forceinline__ void ld_pos(const DevPtrs &D, int64_t j, Node32<DIM> &n) {
  if (DIM == 2) {
    const float4 a = __ldg(D.pos32 + j);
    n.xh[0] = a.x;
    n.xh[1] = a.y;
    n.xh[2] = 0.f;
    n.vol = a.z;
    n.lxy = *reinterpret_cast<const __half2 *>(&a.w);
    n.lz = __floats2half2_rn(0.f, 0.f);
  } else {
    const float4 a = __ldg(D.pos32 + j);
    const uint2 b = __ldg(D.pos32lo + j);
    n.xh[0] = a.x;
    n.xh[1] = a.y;
    n.xh[2] = a.z;
    n.vol = a.w;
    n.lxy = *reinterpret_cast<const __half2 *>(&b.x);
    n.lz = *reinterpret_cast<const __half2 *>(&b.y);
  }
}

template <int DIM>
__device__ __forceinline__ void ld_pair(const float4 *p, int64_t j, float h[3], float l[3]) {
  if (DIM == 2) {
    const float4 a = p[j];
    h[0] = a.x; h[1] = a.y; h[2] = 0.f;
    l[0] = a.z; l[1] = a.w; l[2] = 0.f;
  } else {
    const float4 a = p[2 * j], b = p[2 * j + 1];
    h[0] = a.x; h[1] = a.y; h[2] = a.z;
    l[0] = b.x; l[1] = b.y; l[2] = b.z;
  }
}

template <int DIM>
__device__ __forceinline__ void st_pair(float4 *p, int64_t j, const df v[3]) {
  if (DIM == 2) {
    p[j] = make_float4(v[0].hi, v[1].hi, v[0].lo, v[1].lo);
  } else {
    p[2 * j] = make_float4(v[0].hi, v[1].hi, v[2].hi, 0.f);
    p[2 * j + 1] = make_float4(v[0].lo, v[1].lo, v[2].lo, 0.f);
  }
}

// Prescribed (du, dv) of one dof as double-float pairs.  Kept out of line:
// only nodes with prescribed dofs call it, and inlined, its FP64 time
// functions were if-converted into the path of every node.
static __device__ __noinline__ void bc_df(const DevPtrs &D, const BCTable &T, int ref, int c, double t,
                                   df &u, df &v) {
  double du, dv;
  bc_dof(D, T, ref, c, t, du, dv);
  u = df_from_double(du);
  v = df_from_double(dv);
}

// Internal force plus the external force of a Force_BC node, summed in FP64
// and rounded once.  Out of line for the same reason as bc_df: inlined, its
// conversions and FP64 additions were if-converted into every node's path,
// where each FP64 warp instruction holds the SM's FP64 pipe for many cycles
// (GB300: 2 FP64 operations per SM and cycle).
struct F3 {
  float c[3];
};
template <int DIM>
static __device__ __noinline__ F3 fext_add32(const DevPtrs &D, int64_t i, F3 f) {
  double fe[3];
  ld_node<DIM>(D.fext, i, fe);
  for (int c = 0; c < DIM; c++) f.c[c] = (float)(fe[c] + (double)f.c[c]);
  return f;
}

// FP32C integrator epilogue (same phase structure as integrate_node64).
template <int DIM, int SCHEME>
__device__ __forceinline__ void integrate_node32(const StepParams &P, const Params32 &Q,
                                                 const DevPtrs &D, const BCTable &T,
                                                 const StepArgs &A, int64_t i, uint8_t fl,
                                                 const float uih[3], const float uil[3],
                                                 const float fint[3],
                                                 const float4 *vpre = nullptr,
                                                 const float2 *fpre = nullptr) {
  // vpre, fpre (2-D): the node's velocity pair and previous force, already
  // staged in shared memory by the caller
  float f[3] = {fint[0], fint[1], fint[2]};
  if (fl & FLAG_FBC) {
    const F3 r = fext_add32<DIM>(D, i, F3{{fint[0], fint[1], fint[2]}});
    for (int c = 0; c < 3; c++) f[c] = r.c[c];
  }
  const int ref = (fl & 7) ? D.bcref[i] : -1;
  double t_now = 0., t_next = 0.;
  if (fl & 7) {
    t_now = t_now_of(A);
    t_next = t_next_of(A);
  }
  df un[3], vn[3];
  if (SCHEME == NLM_VELOCITY_VERLET) {
    float vh_[3], vl_[3];
    if (DIM == 2 && vpre)
      ld_pair<DIM>(vpre, 0, vh_, vl_);
    else
      ld_pair<DIM>(D.v32[0], i, vh_, vl_);
    const bool FIRST = A.first;
    float fp[3] = {0.f, 0.f, 0.f};
    if (!FIRST) {
      if (DIM == 2) {
        const float2 a = fpre ? *fpre : reinterpret_cast<const float2 *>(D.f32)[i];
        fp[0] = a.x;
        fp[1] = a.y;
      } else {
        const float4 a = reinterpret_cast<const float4 *>(D.f32)[i];
        fp[0] = a.x;
        fp[1] = a.y;
        fp[2] = a.z;
      }
    }
#pragma unroll
    for (int c = 0; c < DIM; c++) {
      const df v{vh_[c], vl_[c]};
      if (!(fl >> c & 1)) {
        // v^m = v^{m-1} + fact (f^{m-1} + f^m), the increment in FP32 (the
        // two forces summed once); then the drift to u^{m+1}
        df vm = v;
        if (!FIRST) vm = df_add_f(v, __fmul_rn(Q.c_hi, __fadd_rn(fp[c], f[c])));
        vn[c] = vm;
        un[c] = vv_drift(Q, {uih[c], uil[c]}, vm, f[c]);
      } else {
        df du, dv;
        if (!FIRST) {
          bc_df(D, T, ref, c, t_now, du, dv);
          vn[c] = dv;
        } else {
          vn[c] = v;
        }
        bc_df(D, T, ref, c, t_next, du, dv);
        un[c] = du;
      }
    }
    st_pair<DIM>(D.v32[0], i, vn);
  } else {
    float vh_[3], vl_[3];
    if (DIM == 2 && vpre)
      ld_pair<DIM>(vpre, 0, vh_, vl_);
    else
      ld_pair<DIM>(D.v32[A.cur], i, vh_, vl_);
#pragma unroll
    for (int c = 0; c < DIM; c++) {
      if (!(fl >> c & 1)) {
        const df u{uih[c], uil[c]};
        const df inc = df_add(df_cmul(Q.c_hi, Q.c_lo, f[c]),
                              df_mul_c({vh_[c], vl_[c]}, Q.dt_hi, Q.dt_lo));
        un[c] = df_add(u, inc);
        vn[c] = df_mul_c(df_sub(un[c], u), Q.idt_hi, Q.idt_lo);
      } else {
        bc_df(D, T, ref, c, t_next, un[c], vn[c]);
      }
    }
    st_pair<DIM>(D.v32[1 - A.cur], i, vn);
  }
  if (DIM == 2)
    reinterpret_cast<float2 *>(D.f32)[i] = make_float2(f[0], f[1]);
  else
    reinterpret_cast<float4 *>(D.f32)[i] = make_float4(f[0], f[1], f[2], 0.f);
  st_pair<DIM>(D.u32[1 - A.cur], i, un);
}

}  // namespace nlm
