// placeholder, replaced by the ElasticState kernels
#include "fd_internal.h"
namespace nlm {
cudaError_t launch_es_step_fp64(const StepParams &, const DevPtrs &, const BCTable &,
                                const StepArgs &, int, cudaStream_t) { return cudaErrorNotSupported; }
cudaError_t launch_es_step_fp32(const StepParams &, const DevPtrs &, const BCTable &,
                                const StepArgs &, int, cudaStream_t) { return cudaErrorNotSupported; }
}
