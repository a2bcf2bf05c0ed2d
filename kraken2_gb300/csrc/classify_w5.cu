// Instantiations of the classify kernels for the default window
// (k = 35, l = 31: five l-mers per k-mer).
#include "classify_kernels.cuh"
#include "pipeline.cuh"

namespace k2g {
template cudaError_t launch_fast<5, false, true>(const ClassifyArgs &, int, int, cudaStream_t);
template cudaError_t launch_fast<5, true, true>(const ClassifyArgs &, int, int, cudaStream_t);
template cudaError_t launch_pipe_step<5, false, true, false>(const StepArgs &, cudaStream_t);
template cudaError_t launch_pipe_step<5, false, true, true>(const StepArgs &, cudaStream_t);
template cudaError_t launch_pipe_step<5, true, true, false>(const StepArgs &, cudaStream_t);
template cudaError_t launch_pipe_step<5, true, true, true>(const StepArgs &, cudaStream_t);
}  // namespace k2g
