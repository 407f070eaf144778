// fd_kernels.cu -- small kernels of the model handle: force-load and
// displacement-load application, scatter / gather between the caller's
// (3 doubles per node, original order) and the internal layouts, the FP32C
// position store and the broken-bond count.

#include "fd_handle.h"

namespace nlm {

// Time part of FLoading::apply (fLoading.cpp:246-266), applied as
// fmax = (spatial * g(t)) * time_params[0].
__device__ double fload_time(const BCTime &T, double fmax, double time) {
  switch (T.fn) {
    case NLM_TFN_LINEAR: fmax = fmax * time; break;
    case NLM_TFN_LINEAR_STEP: {
      const double x1 = T.p[1], x2 = T.p[2];
      const double period = floor(time / (x1 + x2));
      const double g = dLT(time, period * (x1 + x2) + x1) ? time - period * x2 : (period + 1.) * x1;
      fmax = fmax * g;
    } break;
    case NLM_TFN_LINEAR_SLOW_FAST:
      fmax = dGT(time, T.p[1]) ? fmax * (T.p[3] * time) : fmax * (T.p[2] * time);
      break;
    case NLM_TFN_SIN: fmax = fmax * sin((M_PI * T.p[1]) * time); break;
    default: break;
  }
  return fmax * T.p[0];
}


// time: the load time, or tdev[0] when tdev is set (graph replay).
__global__ void k_fbc_apply(int64_t nf, int S, const int *nodes, const int *iptr,
                            const FBCItem *items, BCTable T, double time, double *fext,
                            const double *tdev) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nf) return;
  if (tdev) time = tdev[0];
  double fe[3] = {0., 0., 0.};
  for (int k = iptr[t]; k < iptr[t + 1]; k++) {
    const FBCItem it = items[k];
    const double v = fload_time(T.t[it.set], it.spatial, time);
    for (int d = 0; d < 3; d++)
      if (it.dir_mask >> d & 1) fe[d] = fe[d] + v;
  }
  const int64_t i = nodes[t];
  for (int d = 0; d < S && d < 3; d++) fext[S * i + d] = fe[d];
}

__global__ void k_bc_apply(int64_t nb, int S, int dim, const int *nodes, const int *bcref,
                           const BCEntry *bce, const uint8_t *flags, BCTable T, double time,
                           double *u64, float4 *u32, double *v, float4 *v32) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nb) return;
  const int64_t i = nodes[t];
  const BCEntry e = bce[bcref[i]];
  const uint8_t fl = flags[i];
  double uo[3], vo[3];
  if (u64) {
    for (int d = 0; d < 3; d++) uo[d] = d < S ? u64[S * i + d] : 0.;
    for (int d = 0; d < 3; d++) vo[d] = d < S ? v[S * i + d] : 0.;
  } else {
    ld_split_any(u32, S, i, uo);
    ld_split_any(v32, S, i, vo);
  }
  for (int d = 0; d < dim; d++)
    if ((fl >> d & 1) && e.set[d] >= 0) {
      double du, dv;
      bc_value(T.t[e.set[d]], e.umax[d], time, du, dv);
      uo[d] = du;
      vo[d] = dv;
    }
  if (u64) {
    for (int d = 0; d < S && d < 3; d++) u64[S * i + d] = uo[d];
    for (int d = 0; d < S && d < 3; d++) v[S * i + d] = vo[d];
  } else {
    st_split_any(u32, S, i, uo);
    st_split_any(v32, S, i, vo);
  }
}

// AoS original order (3 doubles per node) <-> internal layouts.
__global__ void k_scatter_vec(int64_t n, int S, int dim, const int *perm, const double *src,
                              double *dst) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double *p = src + 3 * (int64_t)perm[i];
  for (int d = 0; d < S; d++) dst[S * i + d] = (d < dim && d < 3) ? p[d] : 0.;
}
__global__ void k_invert_perm(int64_t n, const int *perm, int *iperm) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) iperm[perm[i]] = (int)i;
}

__global__ void k_nonfinite(int64_t m, const double *a, int *flag) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k < m && !isfinite(a[k])) atomicExch(flag, 1);
}
__global__ void k_scatter_split(int64_t n, int S, int dim, const int *perm, const double *src,
                                float4 *dst) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double *p = src + 3 * (int64_t)perm[i];
  float h[3], l[3];
  for (int d = 0; d < 3; d++) {
    const double val = d < dim ? p[d] : 0.;
    h[d] = __double2float_rn(val);
    l[d] = __double2float_rn(val - (double)h[d]);
  }
  if (S == 2)
    dst[i] = make_float4(h[0], h[1], l[0], l[1]);
  else {
    dst[2 * i] = make_float4(h[0], h[1], h[2], 0.f);
    dst[2 * i + 1] = make_float4(l[0], l[1], l[2], 0.f);
  }
}
__global__ void k_scatter_f32(int64_t n, int S, int dim, const int *perm, const double *src,
                              float *dst) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double *p = src + 3 * (int64_t)perm[i];
  for (int d = 0; d < S; d++) dst[S * i + d] = (d < dim && d < 3) ? (float)p[d] : 0.f;
}
// keep_z (2-D): the z entry of dst is left as it is (the caller's own value,
// uploaded into the same slot), as the reference's 2-D integrator never
// writes the z component of u and v.
__global__ void k_gather_vec(int64_t n, int S, const int *perm, const double *src, double *dst,
                             bool keep_z) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double *p = dst + 3 * (int64_t)perm[i];
  for (int d = 0; d < 3; d++)
    if (d < S || !keep_z) p[d] = d < S ? src[S * i + d] : 0.;
}
__global__ void k_gather_split(int64_t n, int S, const int *perm, const float4 *src, double *dst,
                               bool keep_z) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double *p = dst + 3 * (int64_t)perm[i];
  if (S == 2) {
    const float4 a = src[i];
    p[0] = (double)a.x + (double)a.z;
    p[1] = (double)a.y + (double)a.w;
    if (!keep_z) p[2] = 0.;
  } else {
    const float4 a = src[2 * i], b = src[2 * i + 1];
    p[0] = (double)a.x + (double)b.x;
    p[1] = (double)a.y + (double)b.y;
    p[2] = (double)a.z + (double)b.z;
  }
}
__global__ void k_gather_f32(int64_t n, int S, const int *perm, const float *src, double *dst) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double *p = dst + 3 * (int64_t)perm[i];
  for (int d = 0; d < 3; d++) p[d] = d < S ? (double)src[S * i + d] : 0.;
}
// FP32C position store: hi = (float)x, lo = x - hi packed as half(lo * scale).
__global__ void k_make_pos32(int64_t n, int S, const double *pos, const double *vol, double scale,
                             float4 *pos32, uint2 *pos32lo) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  float h[3];
  __half l[3];
  for (int d = 0; d < 3; d++) {
    const double v = d < S ? pos[S * i + d] : 0.;
    h[d] = __double2float_rn(v);
    l[d] = __float2half_rn((float)((v - (double)h[d]) * scale));
  }
  const __half2 lxy = __halves2half2(l[0], l[1]);
  const __half2 lz = __halves2half2(l[2], __float2half_rn(0.f));
  const float V = (float)vol[i];
  if (S == 2) {
    pos32[i] = make_float4(h[0], h[1], V, *reinterpret_cast<const float *>(&lxy));
  } else {
    pos32[i] = make_float4(h[0], h[1], h[2], V);
    pos32lo[i] = make_uint2(*reinterpret_cast<const unsigned *>(&lxy),
                            *reinterpret_cast<const unsigned *>(&lz));
  }
}
__global__ void k_count_bits(int64_t n, int nwords, int64_t npad, const uint32_t *bits,
                             unsigned long long *out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  int c = 0;
  for (int w = 0; w < nwords; w++) c += __popc(bits[(int64_t)w * npad + i]);
  if (c) atomicAdd(out, (unsigned long long)c);
}

}  // namespace nlm
