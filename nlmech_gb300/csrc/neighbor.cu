// neighbor.cu -- uniform-grid horizon neighbour search and bond-store setup.
//
// Replaces geometry::Neighbor (src/geometry/neighbor.cpp:24-92).  The
// reference tests every pair (O(N^2)); here nodes are binned into cells of
// edge >= horizon + 1e-10, sorted by the Morton code of their cell, and each
// node tests only the 3^dim surrounding cells.  The predicate is the
// reference's, evaluated in FP64 with separately rounded operations:
//   definitelyLessThan(|x_i - x_j|, horizon + 1e-10)   (neighbor.cpp:81-82)
// so the sets are identical.  Rows are then ordered by ascending original id,
// the order the reference's j-loop produces.
//
// Compiled with --fmad=false.

#include <cub/cub.cuh>

#include "fd_internal.h"
#include "neighbor.h"

namespace nlm {

__device__ __forceinline__ uint64_t spread3(uint64_t v) {  // 21 bits -> every 3rd bit
  v &= 0x1fffffull;
  v = (v | v << 32) & 0x1f00000000ffffull;
  v = (v | v << 16) & 0x1f0000ff0000ffull;
  v = (v | v << 8) & 0x100f00f00f00f00full;
  v = (v | v << 4) & 0x10c30c30c30c30c3ull;
  v = (v | v << 2) & 0x1249249249249249ull;
  return v;
}

__device__ __forceinline__ void cell_of(const Grid &g, const double *p, int64_t c[3]) {
  for (int d = 0; d < 3; d++) {
    int64_t k = (int64_t)floor((p[d] - g.lo[d]) / g.cs);
    c[d] = k < 0 ? 0 : (k >= g.nc[d] ? g.nc[d] - 1 : k);
  }
}

// keys: Morton code of the cell (with the specimen id above it); values:
// original node id.
__global__ void k_cell_keys(int64_t n, const double *x, Grid g, const int *specimen,
                            uint64_t *keys, int *vals) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  int64_t c[3];
  cell_of(g, x + 3 * i, c);
  uint64_t m = spread3((uint64_t)c[0]) | (spread3((uint64_t)c[1]) << 1) |
               (spread3((uint64_t)c[2]) << 2);
  (void)specimen;
  keys[i] = m;
  vals[i] = (int)i;
}

// Sorted positions (S doubles per node) and the linear cell id of each node.
__global__ void k_gather_sorted(int64_t n, int S, const double *x, const int *perm, Grid g,
                                double *pos, int64_t *cell) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double *p = x + 3 * (int64_t)perm[i];
  for (int d = 0; d < S; d++) pos[(int64_t)S * i + d] = d < 3 ? p[d] : 0.;
  int64_t c[3];
  cell_of(g, p, c);
  cell[i] = (c[2] * g.nc[1] + c[1]) * g.nc[0] + c[0];
}

__global__ void k_cell_ranges(int64_t n, const int64_t *cell, int64_t *cbeg, int64_t *cend) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t c = cell[i];
  if (i == 0 || cell[i - 1] != c) cbeg[c] = i;
  if (i == n - 1 || cell[i + 1] != c) cend[c] = i + 1;
}

__device__ __forceinline__ bool within(const double *a, const double *b, double rad) {
  // util::Point3::dist (point.h:165-169) with this = x_i, argument = x_j
  const double dx = __dsub_rn(a[0], b[0]), dy = __dsub_rn(a[1], b[1]),
               dz = __dsub_rn(a[2], b[2]);
  const double s = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
  return dLT(__dsqrt_rn(s), rad);
}

// FILL pass: rows are ordered by ascending original id (the reference's order)
// when by_orig, else by ascending internal (Morton) index.
template <bool FILL>
__global__ void k_neighbors(int64_t n, int S, const double *pos, const int64_t *cell, Grid g,
                            const int64_t *cbeg, const int64_t *cend, const int *perm,
                            int64_t *count, const int64_t *rowptr, int *cols, int *err,
                            bool by_orig) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double xi[3] = {pos[S * i], pos[S * i + 1], S > 2 ? pos[S * i + 2] : 0.};
  const int64_t ci = cell[i];
  int64_t c[3] = {ci % g.nc[0], (ci / g.nc[0]) % g.nc[1], ci / (g.nc[0] * g.nc[1])};
  int64_t cnt = 0;
  int64_t out = FILL ? rowptr[i] : 0;
  for (int64_t dz = -1; dz <= 1; dz++) {
    const int64_t z = c[2] + dz;
    if (z < 0 || z >= g.nc[2]) continue;
    for (int64_t dy = -1; dy <= 1; dy++) {
      const int64_t y = c[1] + dy;
      if (y < 0 || y >= g.nc[1]) continue;
      for (int64_t dx = -1; dx <= 1; dx++) {
        const int64_t x = c[0] + dx;
        if (x < 0 || x >= g.nc[0]) continue;
        const int64_t cc = (z * g.nc[1] + y) * g.nc[0] + x;
        const int64_t b = cbeg[cc], e = cend[cc];
        for (int64_t j = b; j < e; j++) {
          if (j == i) continue;
          const double xj[3] = {pos[S * j], pos[S * j + 1], S > 2 ? pos[S * j + 2] : 0.};
          if (within(xi, xj, g.rad)) {
            if (FILL) cols[out + cnt] = (int)j;
            cnt++;
          }
        }
      }
    }
  }
  if (!FILL) {
    count[i] = cnt;
    if (cnt > kMaxRow) atomicExch(err, DEVERR_ROW_TOO_LONG);
    return;
  }
  // order the row (insertion sort, rows <= kMaxRow)
  int *row = cols + out;
  for (int64_t a = 1; a < cnt; a++) {
    const int v = row[a];
    const int key = by_orig ? perm[v] : v;
    int64_t b = a - 1;
    while (b >= 0 && (by_orig ? perm[row[b]] : row[b]) > key) {
      row[b + 1] = row[b];
      b--;
    }
    row[b + 1] = v;
  }
}

__global__ void k_sell_width(int64_t n, const int64_t *rowptr, int *width) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int len = (int)(rowptr[i + 1] - rowptr[i]);
  atomicMax(width + (i >> 5), len);
}

// Sliced ELL, 32 rows per slice, entries interleaved in groups of four: entry
// k of lane l sits at slice_base + (k/4)*128 + 4l + k%4, so a thread fetches
// four neighbour ids with one 16-byte load and a warp's load is 512
// contiguous bytes.  Slice widths are multiples of 4; pads are -1.
__global__ void k_sell_fill(int64_t n, int64_t nslices, const int64_t *rowptr, const int *cols,
                            const int64_t *sell_ptr, const int *width, int *sell_cols) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nslices * 32) return;
  const int64_t s = t >> 5;
  const int lane = (int)(t & 31);
  const int64_t i = t;
  const int w = width[s];
  const int64_t base = sell_ptr[s] + 4 * lane;
  const int64_t r0 = i < n ? rowptr[i] : 0;
  const int len = i < n ? (int)(rowptr[i + 1] - r0) : 0;
  for (int k = 0; k < w; k++)
    sell_cols[base + (int64_t)(k >> 2) * 128 + (k & 3)] = k < len ? cols[r0 + k] : -1;
}

// Pre-crack bits (geometry::Fracture ctor, src/geometry/fracture.cpp:20-160;
// inp::EdgeCrack predicates, src/inp/decks/fractureDeck.h:115-186).
__device__ bool pt_outside(const nlm_crack &c, const double *p) {
  if (c.orientation == -1) return dLT(p[1], c.pb[1]) || dGT(p[1], c.pt[1]);
  if (c.orientation == 1) return dLT(p[0], c.pb[0]) || dGT(p[0], c.pt[0]);
  if (c.orientation == 0) {
    const double px = __dsub_rn(p[0], c.pb[0]), py = __dsub_rn(p[1], c.pb[1]);
    const double tx = __dsub_rn(c.pt[0], c.pb[0]), ty = __dsub_rn(c.pt[1], c.pb[1]);
    const double ct = cos(c.theta), st = sin(c.theta);
    const double pmx = __dadd_rn(__dmul_rn(ct, px), __dmul_rn(st, py));
    const double ptx = __dadd_rn(__dmul_rn(ct, tx), __dmul_rn(st, ty));
    return dLT(pmx, 0.0) || dGT(pmx, ptx);
  }
  return true;
}
__device__ bool pt_left(const nlm_crack &c, const double *p) {
  const double a = __dmul_rn(
      0.5, __dsub_rn(__dmul_rn(__dsub_rn(c.pt[0], c.pb[0]), __dsub_rn(p[1], c.pb[1])),
                     __dmul_rn(__dsub_rn(p[0], c.pb[0]), __dsub_rn(c.pt[1], c.pb[1]))));
  return !dLT(a, 0.0);
}
__device__ bool plane_cuts(const nlm_crack &c, const double *a, const double *b) {
  const bool sa = a[2] < c.z0, sb = b[2] < c.z0;
  if (sa == sb) return false;
  const double t = (c.z0 - a[2]) / (b[2] - a[2]);
  const double px = a[0] + t * (b[0] - a[0]);
  const double py = a[1] + t * (b[1] - a[1]);
  return px >= c.lo[0] && px <= c.hi[0] && py >= c.lo[1] && py <= c.hi[1];
}

__global__ void k_precrack(int64_t n, int64_t off, int S, const double *pos,
                           const int64_t *rowptr, const int *cols, nlm_crack ck, int64_t npad,
                           uint32_t *bits) {
  const int64_t i = off + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= off + n) return;
  const double xi[3] = {pos[S * i], pos[S * i + 1], S > 2 ? pos[S * i + 2] : 0.};
  const int64_t r0 = rowptr[i], r1 = rowptr[i + 1];
  if (ck.kind == NLM_CRACK_PLANE) {
    for (int64_t k = r0; k < r1; k++) {
      const int64_t j = cols[k];
      const double xj[3] = {pos[S * j], pos[S * j + 1], S > 2 ? pos[S * j + 2] : 0.};
      if (plane_cuts(ck, xi, xj)) {
        const int kk = (int)(k - r0);
        bits[(int64_t)(kk >> 5) * npad + i] |= 1u << (kk & 31);
      }
    }
    return;
  }
  if (pt_outside(ck, xi)) return;
  const bool left = pt_left(ck, xi);
  for (int64_t k = r0; k < r1; k++) {
    const int64_t j = cols[k];
    const double xj[3] = {pos[S * j], pos[S * j + 1], S > 2 ? pos[S * j + 2] : 0.};
    const bool modify = !pt_outside(ck, xj);
    const bool other = left ? !pt_left(ck, xj) : pt_left(ck, xj);
    if (other && modify) {
      const int kk = (int)(k - r0);
      bits[(int64_t)(kk >> 5) * npad + i] |= 1u << (kk & 31);
    }
  }
}

// ---------------------------------------------------------------------------
// host driver

#define NB_CHECK(call)                          \
  do {                                          \
    cudaError_t _e = (call);                    \
    if (_e != cudaSuccess) return _e;           \
  } while (0)

static unsigned blocks(int64_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

Grid make_grid(int dim, int64_t n, const double *x, double horizon) {
  Grid g;
  g.rad = horizon + 1.0E-10;
  g.cs = g.rad * (1.0 + 1e-7);
  for (int d = 0; d < 3; d++) {
    g.lo[d] = 1e300;
    double hi = -1e300;
    for (int64_t i = 0; i < n; i++) {
      g.lo[d] = x[3 * i + d] < g.lo[d] ? x[3 * i + d] : g.lo[d];
      hi = x[3 * i + d] > hi ? x[3 * i + d] : hi;
    }
    if (n == 0) g.lo[d] = hi = 0.;
    int64_t k = (int64_t)((hi - g.lo[d]) / g.cs) + 1;
    g.nc[d] = k < 1 ? 1 : k;
  }
  (void)dim;
  return g;
}

cudaError_t build_neighbors(NeighborBuild &nb, int dim, int64_t n, const double *d_x,
                            const Grid &g, int S, cudaStream_t s, std::string &why,
                            bool rows_by_orig) {
  nb.n = n;
  nb.S = S;
  const int bs = 256;
  uint64_t *keys = nullptr, *keys2 = nullptr;
  int *vals = nullptr;
  int *err = nullptr;
  int64_t *cell = nullptr, *cbeg = nullptr, *cend = nullptr, *cnt = nullptr;
  void *tmp = nullptr;
  size_t tmpb = 0;
  const int64_t ncell = g.nc[0] * g.nc[1] * g.nc[2];
  cudaError_t e = cudaSuccess;
  auto cleanup = [&]() {
    cudaFree(keys); cudaFree(keys2); cudaFree(vals); cudaFree(err); cudaFree(cell);
    cudaFree(cbeg); cudaFree(cend); cudaFree(cnt); cudaFree(tmp);
  };
#define NB_TRY(call)             \
  do {                           \
    e = (call);                  \
    if (e != cudaSuccess) {      \
      cleanup();                 \
      return e;                  \
    }                            \
  } while (0)
  NB_TRY(cudaMalloc(&keys, sizeof(uint64_t) * (n + 1)));
  NB_TRY(cudaMalloc(&keys2, sizeof(uint64_t) * (n + 1)));
  NB_TRY(cudaMalloc(&vals, sizeof(int) * (n + 1)));
  NB_TRY(cudaMalloc(&nb.perm, sizeof(int) * (n + 1)));
  NB_TRY(cudaMalloc(&err, sizeof(int)));
  NB_TRY(cudaMemsetAsync(err, 0, sizeof(int), s));
  if (n > 0) {
    k_cell_keys<<<blocks(n, bs), bs, 0, s>>>(n, d_x, g, nullptr, keys, vals);
    NB_TRY(cudaGetLastError());
    NB_TRY(cub::DeviceRadixSort::SortPairs(nullptr, tmpb, keys, keys2, vals, nb.perm, (int)n, 0,
                                           64, s));
    NB_TRY(cudaMalloc(&tmp, tmpb));
    NB_TRY(cub::DeviceRadixSort::SortPairs(tmp, tmpb, keys, keys2, vals, nb.perm, (int)n, 0, 64,
                                           s));
    cudaFree(tmp);
    tmp = nullptr;
  }
  NB_TRY(cudaMalloc(&nb.pos, sizeof(double) * S * (n + 1)));
  NB_TRY(cudaMalloc(&cell, sizeof(int64_t) * (n + 1)));
  NB_TRY(cudaMalloc(&cbeg, sizeof(int64_t) * ncell));
  NB_TRY(cudaMalloc(&cend, sizeof(int64_t) * ncell));
  NB_TRY(cudaMemsetAsync(cbeg, 0, sizeof(int64_t) * ncell, s));
  NB_TRY(cudaMemsetAsync(cend, 0, sizeof(int64_t) * ncell, s));
  NB_TRY(cudaMalloc(&cnt, sizeof(int64_t) * (n + 1)));
  NB_TRY(cudaMalloc(&nb.rowptr, sizeof(int64_t) * (n + 1)));
  if (n > 0) {
    k_gather_sorted<<<blocks(n, bs), bs, 0, s>>>(n, S, d_x, nb.perm, g, nb.pos, cell);
    NB_TRY(cudaGetLastError());
    k_cell_ranges<<<blocks(n, bs), bs, 0, s>>>(n, cell, cbeg, cend);
    NB_TRY(cudaGetLastError());
    k_neighbors<false><<<blocks(n, 128), 128, 0, s>>>(n, S, nb.pos, cell, g, cbeg, cend, nb.perm,
                                                      cnt, nullptr, nullptr, err, true);
    NB_TRY(cudaGetLastError());
    int herr = 0;
    NB_TRY(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s));
    NB_TRY(cudaStreamSynchronize(s));
    if (herr == DEVERR_ROW_TOO_LONG) {
      why = "a neighbour row exceeds the supported maximum";
      cleanup();
      return cudaErrorInvalidValue;
    }
    NB_TRY(cudaMemsetAsync(cnt + n, 0, sizeof(int64_t), s));
    NB_TRY(cub::DeviceScan::ExclusiveSum(nullptr, tmpb, cnt, nb.rowptr, n + 1, s));
    NB_TRY(cudaMalloc(&tmp, tmpb));
    NB_TRY(cub::DeviceScan::ExclusiveSum(tmp, tmpb, cnt, nb.rowptr, n + 1, s));
  } else {
    NB_TRY(cudaMemsetAsync(nb.rowptr, 0, sizeof(int64_t), s));
  }
  NB_TRY(cudaMemcpyAsync(&nb.nnz, nb.rowptr + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  NB_TRY(cudaStreamSynchronize(s));
  NB_TRY(cudaMalloc(&nb.cols, sizeof(int) * (nb.nnz + 1)));
  if (n > 0) {
    k_neighbors<true><<<blocks(n, 128), 128, 0, s>>>(n, S, nb.pos, cell, g, cbeg, cend, nb.perm,
                                                     nullptr, nb.rowptr, nb.cols, err,
                                                     rows_by_orig);
    NB_TRY(cudaGetLastError());
  }
  NB_TRY(cudaStreamSynchronize(s));
  cleanup();
  return cudaSuccess;
#undef NB_TRY
}

cudaError_t build_sell(int64_t n, const int64_t *rowptr, const int *cols, SellStore &st,
                       cudaStream_t s) {
  const int bs = 256;
  st.nslices = (n + 31) / 32;
  NB_CHECK(cudaMalloc(&st.width, sizeof(int) * (st.nslices + 1)));
  NB_CHECK(cudaMemsetAsync(st.width, 0, sizeof(int) * (st.nslices + 1), s));
  if (n > 0) {
    k_sell_width<<<blocks(n, bs), bs, 0, s>>>(n, rowptr, st.width);
    NB_CHECK(cudaGetLastError());
  }
  std::vector<int> w(st.nslices);
  NB_CHECK(cudaMemcpyAsync(w.data(), st.width, sizeof(int) * st.nslices, cudaMemcpyDeviceToHost, s));
  NB_CHECK(cudaStreamSynchronize(s));
  std::vector<int64_t> ptr(st.nslices + 1, 0);
  st.maxw = 0;
  for (int64_t k = 0; k < st.nslices; k++) {
    st.maxw = w[k] > st.maxw ? w[k] : st.maxw;
    w[k] = (w[k] + 3) & ~3;
    ptr[k + 1] = ptr[k] + 32 * (int64_t)w[k];
  }
  NB_CHECK(cudaMemcpyAsync(st.width, w.data(), sizeof(int) * st.nslices, cudaMemcpyHostToDevice, s));
  st.entries = ptr[st.nslices];
  NB_CHECK(cudaMalloc(&st.ptr, sizeof(int64_t) * (st.nslices + 1)));
  NB_CHECK(cudaMemcpyAsync(st.ptr, ptr.data(), sizeof(int64_t) * (st.nslices + 1),
                           cudaMemcpyHostToDevice, s));
  NB_CHECK(cudaMalloc(&st.cols, sizeof(int) * (st.entries + 1)));
  if (n > 0) {
    k_sell_fill<<<blocks(st.nslices * 32, bs), bs, 0, s>>>(n, st.nslices, rowptr, cols, st.ptr,
                                                           st.width, st.cols);
    NB_CHECK(cudaGetLastError());
  }
  NB_CHECK(cudaStreamSynchronize(s));
  return cudaSuccess;
}

cudaError_t apply_precrack(int64_t n, int S, const double *pos, const int64_t *rowptr,
                           const int *cols, const nlm_crack &ck, int64_t npad, uint32_t *bits,
                           cudaStream_t s, int64_t off) {
  if (n == 0) return cudaSuccess;
  k_precrack<<<blocks(n, 128), 128, 0, s>>>(n, off, S, pos, rowptr, cols, ck, npad, bits);
  return cudaGetLastError();
}

__global__ void k_offset_cols(int64_t nnz, int *cols, int off) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k < nnz) cols[k] += off;
}
__global__ void k_offset_rowptr(int64_t n, int64_t *rowptr, int64_t off) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k < n) rowptr[k] += off;
}

cudaError_t offset_cols(int64_t nnz, int *cols, int off, cudaStream_t s) {
  if (nnz == 0) return cudaSuccess;
  k_offset_cols<<<blocks(nnz, 256), 256, 0, s>>>(nnz, cols, off);
  return cudaGetLastError();
}
cudaError_t offset_rowptr(int64_t n, int64_t *rowptr, int64_t off, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  k_offset_rowptr<<<blocks(n, 256), 256, 0, s>>>(n, rowptr, off);
  return cudaGetLastError();
}

}  // namespace nlm
