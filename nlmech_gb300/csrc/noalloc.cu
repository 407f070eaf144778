// noalloc.cu -- horizon neighbour search that allocates no device memory.
//
// nlm_neighbor_search_noalloc returns the same rows as nlm_neighbor_search:
//   row i = { j != i : definitelyLessThan(|x_i - x_j|, horizon + 1e-10) }
// (geometry::Neighbor, src/geometry/neighbor.cpp:69-89), each row ascending
// in j.  Every intermediate lives in one file-scope __device__ array of fixed
// size, so a call makes no cudaMalloc / cudaFree or any other allocating call.
// It is meant for callers that must not allocate: a host whose device memory
// is already reserved by a pool allocator, or a run that re-meshes between
// steps while other streams work and cannot take the device-wide
// synchronisation cudaFree implies.
//
// Limits (the size of the static scratch, 21.5 MiB in total):
//   n      <= 65,536 nodes,
//   cells  <= 262,144 cells of the search grid (edge = horizon + 1e-10),
//   nnz    <= 4,194,304 bonds,
//   rows   <= 512 entries (as nlm_neighbor_search).
// Larger inputs are rejected with NLM_ERR_INVALID before any launch.
//
// Algorithm: counting sort of the nodes into grid cells (per-cell counters,
// one-block scan, atomic scatter), then one thread per node scans the 3^dim
// cells around its own, first to count, then to fill; each row is finally
// sorted ascending, so the output does not depend on the scatter order.
// The distance is evaluated with the separately rounded FP64 operations of
// util::Point3::dist (point.h:165-169); this unit is compiled with
// --fmad=false.

#include <cuda_runtime.h>

#include <cmath>
#include <string>

#include "../../include/nlmgpu.h"
#include "common.cuh"
#include "neighbor.h"

namespace nlm {
void set_error(const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);
}  // namespace nlm

using namespace nlm;

namespace {

constexpr int64_t kNAMaxNodes = 65536;
constexpr int64_t kNAMaxCells = 262144;
constexpr int64_t kNAMaxBonds = 4194304;

constexpr size_t na_round(size_t b) { return (b + 255) / 256 * 256; }
// byte offsets of the regions of the scratch array
constexpr size_t kOffX = 0;                                                  // 3 doubles / node
constexpr size_t kOffCellOf = kOffX + na_round(sizeof(double) * 3 * kNAMaxNodes);
constexpr size_t kOffCount = kOffCellOf + na_round(sizeof(int) * kNAMaxNodes);  // zeroed
constexpr size_t kOffStart = kOffCount + na_round(sizeof(int) * kNAMaxCells);
constexpr size_t kOffFill = kOffStart + na_round(sizeof(int) * (kNAMaxCells + 1));  // zeroed
constexpr size_t kOffSorted = kOffFill + na_round(sizeof(int) * kNAMaxCells);
constexpr size_t kOffRowptr = kOffSorted + na_round(sizeof(int) * kNAMaxNodes);
constexpr size_t kOffCols = kOffRowptr + na_round(sizeof(int64_t) * (kNAMaxNodes + 1));
constexpr size_t kOffErr = kOffCols + na_round(sizeof(int) * kNAMaxBonds);  // zeroed
constexpr size_t kScratchBytes = kOffErr + 256;
static_assert(kScratchBytes == 22545152, "scratch layout changed: update the stated size");

static __device__ __align__(256) unsigned char g_na_scratch[kScratchBytes];

__device__ __forceinline__ int na_cell(const Grid &g, const double *p, int c[3]) {
  for (int d = 0; d < 3; d++) {
    int64_t k = (int64_t)floor((p[d] - g.lo[d]) / g.cs);
    c[d] = (int)(k < 0 ? 0 : (k >= g.nc[d] ? g.nc[d] - 1 : k));
  }
  return (int)((c[2] * g.nc[1] + c[1]) * g.nc[0] + c[0]);
}

__device__ __forceinline__ bool na_within(const double *a, const double *b, double rad) {
  const double dx = __dsub_rn(a[0], b[0]), dy = __dsub_rn(a[1], b[1]),
               dz = __dsub_rn(a[2], b[2]);
  const double s = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
  return dLT(__dsqrt_rn(s), rad);
}

__global__ void k_na_cells(int n, const double *x, Grid g, int *cellof, int *count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int c[3];
  const int cell = na_cell(g, x + 3 * (int64_t)i, c);
  cellof[i] = cell;
  atomicAdd(count + cell, 1);
}

// Exclusive scan of m values into out[0..m] (out[m] = total), one block of
// 1024 threads, each owning a contiguous chunk.
template <class T>
__global__ void __launch_bounds__(1024) k_na_scan(int64_t m, const T *in, T *out) {
  __shared__ T part[1024];
  const int t = threadIdx.x;
  const int64_t chunk = (m + 1023) / 1024;
  const int64_t b = t * chunk, e = b + chunk < m ? b + chunk : m;
  T s = 0;
  for (int64_t k = b; k < e; k++) s += in[k];
  part[t] = s;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    const T v = t >= o ? part[t - o] : 0;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  T run = t ? part[t - 1] : 0;
  for (int64_t k = b; k < e; k++) {
    const T v = in[k];
    out[k] = run;
    run += v;
  }
  if (t == 1023) out[m] = part[1023];
}

__global__ void k_na_scatter(int n, const int *cellof, const int *start, int *fill, int *sorted) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int c = cellof[i];
  sorted[start[c] + atomicAdd(fill + c, 1)] = i;
}

// Count pass (FILL = false): rowlen[i] written to rowptr[i].  Fill pass:
// cols[rowptr[i] ...] then the row is sorted ascending.
template <bool FILL>
__global__ void k_na_rows(int n, const double *x, Grid g, const int *cellof, const int *start,
                          const int *sorted, int64_t *rowptr, int *cols, int *err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double xi[3] = {x[3 * (int64_t)i], x[3 * (int64_t)i + 1], x[3 * (int64_t)i + 2]};
  const int ci = cellof[i];
  const int c[3] = {(int)(ci % g.nc[0]), (int)((ci / g.nc[0]) % g.nc[1]),
                    (int)(ci / (g.nc[0] * g.nc[1]))};
  const int64_t out = FILL ? rowptr[i] : 0;
  int cnt = 0;
  for (int dz = -1; dz <= 1; dz++) {
    const int z = c[2] + dz;
    if (z < 0 || z >= g.nc[2]) continue;
    for (int dy = -1; dy <= 1; dy++) {
      const int y = c[1] + dy;
      if (y < 0 || y >= g.nc[1]) continue;
      for (int dx = -1; dx <= 1; dx++) {
        const int xx = c[0] + dx;
        if (xx < 0 || xx >= g.nc[0]) continue;
        const int cc = (int)((z * g.nc[1] + y) * g.nc[0] + xx);
        for (int k = start[cc]; k < start[cc + 1]; k++) {
          const int j = sorted[k];
          if (j == i) continue;
          const double xj[3] = {x[3 * (int64_t)j], x[3 * (int64_t)j + 1], x[3 * (int64_t)j + 2]};
          if (na_within(xi, xj, g.rad)) {
            if (FILL && cnt < kMaxRow) cols[out + cnt] = j;
            cnt++;
          }
        }
      }
    }
  }
  if (!FILL) {
    rowptr[i] = cnt;
    if (cnt > kMaxRow) atomicExch(err, DEVERR_ROW_TOO_LONG);
    return;
  }
  int *row = cols + out;
  for (int a = 1; a < cnt; a++) {
    const int v = row[a];
    int b = a - 1;
    while (b >= 0 && row[b] > v) {
      row[b + 1] = row[b];
      b--;
    }
    row[b + 1] = v;
  }
}

int na_fail(int code, const char *msg) {
  nlm::set_error(msg);
  return code;
}

}  // namespace

extern "C" int nlm_neighbor_search_noalloc(int dim, int64_t n, const double *x, double horizon,
                                           int64_t *rowptr, int32_t *cols) {
  if (n < 0 || (n > 0 && !x) || !rowptr || dim < 1 || dim > 3 || !(horizon > 0.))
    return na_fail(NLM_ERR_INVALID, "nlm_neighbor_search_noalloc: bad arguments");
  if (n > kNAMaxNodes)
    return na_fail(NLM_ERR_INVALID,
                   "nlm_neighbor_search_noalloc: more than 65536 nodes (static scratch limit)");
  for (int64_t k = 0; k < 3 * n; k++)
    if (!std::isfinite(x[k])) return na_fail(NLM_ERR_NONFINITE, "non-finite coordinate");
  rowptr[0] = 0;
  if (n == 0) return NLM_OK;
  const Grid g = make_grid(dim, n, x, horizon);
  if (g.nc[0] > kNAMaxCells || g.nc[1] > kNAMaxCells || g.nc[2] > kNAMaxCells ||
      g.nc[0] * g.nc[1] * g.nc[2] > kNAMaxCells)
    return na_fail(NLM_ERR_INVALID,
                   "nlm_neighbor_search_noalloc: search grid exceeds 262144 cells "
                   "(static scratch limit)");
  const int64_t ncell = g.nc[0] * g.nc[1] * g.nc[2];

  // the scratch array's device address in the current context, looked up on
  // every call: a cached address would go stale after a device reset or in
  // another context of the same device, where the module is loaded anew.
  // Once the module is loaded the lookup allocates nothing.
  unsigned char *base = nullptr;
  {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_na_scratch);
    if (e != cudaSuccess) return nlm::cuda_fail(e, "cudaGetSymbolAddress(scratch)");
    base = static_cast<unsigned char *>(p);
  }
  double *dx = reinterpret_cast<double *>(base + kOffX);
  int *cellof = reinterpret_cast<int *>(base + kOffCellOf);
  int *count = reinterpret_cast<int *>(base + kOffCount);
  int *start = reinterpret_cast<int *>(base + kOffStart);
  int *fill = reinterpret_cast<int *>(base + kOffFill);
  int *sorted = reinterpret_cast<int *>(base + kOffSorted);
  int64_t *drow = reinterpret_cast<int64_t *>(base + kOffRowptr);
  int *dcols = reinterpret_cast<int *>(base + kOffCols);
  int *derr = reinterpret_cast<int *>(base + kOffErr);

  const cudaStream_t s = cudaStreamPerThread;
  const int nn = (int)n, bs = 256, nb = (nn + bs - 1) / bs;
  // the per-cell counters, the scatter cursors and the error word start at zero
  NLM_CUDA(cudaMemsetAsync(count, 0, sizeof(int) * ncell, s));
  NLM_CUDA(cudaMemsetAsync(fill, 0, sizeof(int) * ncell, s));
  NLM_CUDA(cudaMemsetAsync(derr, 0, sizeof(int), s));
  NLM_CUDA(cudaMemcpyAsync(dx, x, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s));
  k_na_cells<<<nb, bs, 0, s>>>(nn, dx, g, cellof, count);
  k_na_scan<int><<<1, 1024, 0, s>>>(ncell, count, start);
  k_na_scatter<<<nb, bs, 0, s>>>(nn, cellof, start, fill, sorted);
  // row lengths into drow[1..n], then scanned in place through drow[0..n]
  k_na_rows<false><<<nb, bs, 0, s>>>(nn, dx, g, cellof, start, sorted, drow + 1, dcols, derr);
  NLM_CUDA(cudaGetLastError());
  int herr = 0;
  NLM_CUDA(cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, s));
  NLM_CUDA(cudaMemcpyAsync(rowptr + 1, drow + 1, sizeof(int64_t) * n, cudaMemcpyDeviceToHost, s));
  NLM_CUDA(cudaStreamSynchronize(s));
  if (herr == DEVERR_ROW_TOO_LONG)
    return na_fail(NLM_ERR_INVALID, "a neighbour row exceeds 512 entries");
  for (int64_t i = 0; i < n; i++) rowptr[i + 1] += rowptr[i];
  if (rowptr[n] > kNAMaxBonds)
    return na_fail(NLM_ERR_INVALID,
                   "nlm_neighbor_search_noalloc: more than 4194304 bonds (static scratch limit)");
  if (!cols) return NLM_OK;
  NLM_CUDA(cudaMemcpyAsync(drow, rowptr, sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice, s));
  k_na_rows<true><<<nb, bs, 0, s>>>(nn, dx, g, cellof, start, sorted, drow, dcols, derr);
  NLM_CUDA(cudaGetLastError());
  if (rowptr[n] > 0)
    NLM_CUDA(cudaMemcpyAsync(cols, dcols, sizeof(int) * rowptr[n], cudaMemcpyDeviceToHost, s));
  NLM_CUDA(cudaStreamSynchronize(s));
  return NLM_OK;
}
