// neighbor.h -- neighbour search / bond store builders (neighbor.cu).
#pragma once

#include <string>
#include <vector>

#include "common.cuh"

namespace nlm {

struct Grid {
  double lo[3];
  double cs;   // cell edge
  double rad;  // horizon + 1e-10 (neighbor.cpp:82)
  int64_t nc[3];
};

struct NeighborBuild {  // device arrays, owned by the caller after the build
  int64_t n = 0, nnz = 0;
  int S = 2;
  int *perm = nullptr;        // sorted -> original id
  double *pos = nullptr;      // sorted positions, S doubles per node
  int64_t *rowptr = nullptr;  // CSR over sorted nodes
  int *cols = nullptr;        // sorted ids, rows ascending in original id
};

struct SellStore {
  int64_t nslices = 0, entries = 0;
  int maxw = 0;
  int64_t *ptr = nullptr;
  int *width = nullptr;
  int *cols = nullptr;
};

Grid make_grid(int dim, int64_t n, const double *x, double horizon);
// rows_by_orig: order each row by ascending original id (the reference's
// order, needed for its FP64 summation order); otherwise by internal index.
cudaError_t build_neighbors(NeighborBuild &nb, int dim, int64_t n, const double *d_x,
                            const Grid &g, int S, cudaStream_t s, std::string &why,
                            bool rows_by_orig = true);
cudaError_t build_sell(int64_t n, const int64_t *rowptr, const int *cols, SellStore &st,
                       cudaStream_t s);
// Pre-crack bits of rows [off, off + n).
cudaError_t apply_precrack(int64_t n, int S, const double *pos, const int64_t *rowptr,
                           const int *cols, const nlm_crack &ck, int64_t npad, uint32_t *bits,
                           cudaStream_t s, int64_t off = 0);
// cols[k] += off, rowptr[k] += off (batched specimens).
cudaError_t offset_cols(int64_t nnz, int *cols, int off, cudaStream_t s);
cudaError_t offset_rowptr(int64_t n, int64_t *rowptr, int64_t off, cudaStream_t s);

}  // namespace nlm
