// Instantiations of the classify kernels for other windows (k == l, k - l = 6,
// runtime window), the legacy reverse complement, and the slow path.
#include "classify_kernels.cuh"
#include "pipeline.cuh"

namespace k2g {
template cudaError_t launch_fast<1, false, true>(const ClassifyArgs &, int, int, cudaStream_t);
template cudaError_t launch_fast<1, true, true>(const ClassifyArgs &, int, int, cudaStream_t);
template cudaError_t launch_fast<7, false, true>(const ClassifyArgs &, int, int, cudaStream_t);
template cudaError_t launch_fast<7, true, true>(const ClassifyArgs &, int, int, cudaStream_t);
template cudaError_t launch_fast<0, false, true>(const ClassifyArgs &, int, int, cudaStream_t);
template cudaError_t launch_fast<0, true, true>(const ClassifyArgs &, int, int, cudaStream_t);
template cudaError_t launch_fast<0, false, false>(const ClassifyArgs &, int, int, cudaStream_t);
template cudaError_t launch_fast<0, true, false>(const ClassifyArgs &, int, int, cudaStream_t);
template cudaError_t launch_slow<false, true>(const ClassifyArgs &, int, unsigned, unsigned, cudaStream_t);
template cudaError_t launch_slow<true, true>(const ClassifyArgs &, int, unsigned, unsigned, cudaStream_t);
template cudaError_t launch_slow<false, false>(const ClassifyArgs &, int, unsigned, unsigned, cudaStream_t);
template cudaError_t launch_slow<true, false>(const ClassifyArgs &, int, unsigned, unsigned, cudaStream_t);
template cudaError_t launch_pipe_step<1, false, true, false>(const StepArgs &, cudaStream_t);
template cudaError_t launch_pipe_step<1, true, true, false>(const StepArgs &, cudaStream_t);
template cudaError_t launch_pipe_step<7, false, true, false>(const StepArgs &, cudaStream_t);
template cudaError_t launch_pipe_step<7, true, true, false>(const StepArgs &, cudaStream_t);
template cudaError_t launch_pipe_step<0, false, true, false>(const StepArgs &, cudaStream_t);
template cudaError_t launch_pipe_step<0, true, true, false>(const StepArgs &, cudaStream_t);
template cudaError_t launch_pipe_step<0, false, false, false>(const StepArgs &, cudaStream_t);
template cudaError_t launch_pipe_step<0, true, false, false>(const StepArgs &, cudaStream_t);
}  // namespace k2g
