// qs_internal.h -- work buffers and launchers of the quasi-static solver.
#pragma once

#include "fd_internal.h"

namespace nlm {

struct QSWork {
  double *res;    // residual, DIM per node
  double *dx;     // Newton correction
  double *r, *z, *p, *ap;  // CG vectors
  double *p2;     // second search-direction buffer (iteration parity)
  double *cgpart; // CG partial sums: 3 arrays of qs_cg_stride(n) entries
  double *cgs;    // CG totals on the device (4) and two FP32 step lengths
  unsigned *ticket;  // last-block tickets of the two CG launches (start at 0)
  double *part;   // block partial sums
  double *sc;     // device scalars
  double *blk;    // tangent blocks per bond (3 or 6 doubles)
  double *dblk;   // diagonal blocks per node
  double *res0;   // force at the previous converged state
  // FP32 Krylov solve: tangent copies and CG vectors
  float *blk32, *dblk32, *r32, *z32, *p32, *p32b, *ap32, *x32;
  int64_t nnz;
  // the FP32 solve in one cooperative launch (coop == null: two launches
  // per iteration): barrier words (arrivals, generation, status), grid
  // size, extra arrivals a barrier waits for (testing the bound only) and
  // the bound of each barrier wait
  unsigned *coop;
  int coop_blocks;
  int coop_extra;
  uint64_t coop_wait_ns;
};

// Grid size of the cooperative FP32 solve for n nodes (0: not available).
int qs_coop_blocks(int64_t n, int dim);

// count != NULL: bonds past the critical strain break during the evaluation
// (RNPBond::getBondEF) and the number broken is added to *count.
cudaError_t qs_residual(const StepParams &P, const DevPtrs &D, const double *u, double *res,
                        double *blk, double *dblk, bool assemble, cudaStream_t s,
                        unsigned long long *count = nullptr);
cudaError_t qs_dot(const double *a, const double *b, int64_t m, double *part, double *out,
                   cudaStream_t s);
// use64: in/out, FP64 Krylov solve (set when the FP32 solve did not converge)
cudaError_t qs_cg(const StepParams &P, const DevPtrs &D, const QSWork &W, const double *rhs,
                  double *dx, double tol, int max_iters, int check_every, int *iters,
                  bool *use64, cudaStream_t s);
// Entries per partial-sum array of the CG (4 arrays live in QSWork::cgpart).
int64_t qs_cg_stride(int64_t n);
cudaError_t qs_add(const StepParams &P, const double *du, double *u, cudaStream_t s);
cudaError_t qs_bcdiff(const StepParams &P, const DevPtrs &D, const double *u,
                      const double *uprev, double *dx, bool fixed_only, cudaStream_t s);
cudaError_t qs_spmv(const StepParams &P, const DevPtrs &D, const double *blk, const double *dblk,
                    const double *x, double *y, double *part, cudaStream_t s);
cudaError_t qs_sub(int64_t m, const double *a, const double *b, double *out, cudaStream_t s);
cudaError_t qs_break(const StepParams &P, const DevPtrs &D, const double *u,
                     unsigned long long *count, cudaStream_t s);

}  // namespace nlm
