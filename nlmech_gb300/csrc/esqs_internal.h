// esqs_internal.h -- launchers of the quasi-static ElasticState solver (esqs.cu).
#pragma once

#include <cstdint>

#include "fd_internal.h"

namespace nlm {

// Partial sums of esqs_dot (the part buffer holds this many doubles).
constexpr int kEsqsDotParts = 512;

// theta (n doubles) and the force density f (S per node) at u.
cudaError_t esqs_force(const StepParams &P, const DevPtrs &D, int S, int mdim, const double *u,
                       double *theta, double *f, cudaStream_t s);
// r = f + b on free dofs, 0 on fixed dofs.
cudaError_t esqs_residual(const StepParams &P, const DevPtrs &D, int S, int mdim,
                          const double *f, const double *b, double *r, cudaStream_t s);
// Finite-difference Jacobian blocks (9 doubles each, nblocks = nnz + n).
cudaError_t esqs_jacobian(const StepParams &P, const DevPtrs &D, int S, int mdim, int full,
                          const double *u, double eps, double *J, int64_t nblocks,
                          cudaStream_t s);
cudaError_t esqs_spmv(const StepParams &P, const DevPtrs &D, int S, int mdim, const double *J,
                      const double *x, double *y, cudaStream_t s);
// out = a x + b y + c z; y or z may be NULL.
cudaError_t esqs_lin3(int64_t m, double a, const double *x, double b, const double *y, double c,
                      const double *z, double *out, cudaStream_t s);
// *out = a . b (device scalar), via kEsqsDotParts partial sums in part.
cudaError_t esqs_dot(int64_t m, const double *a, const double *b, double *part, double *out,
                     cudaStream_t s);

}  // namespace nlm
