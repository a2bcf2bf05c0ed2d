// Probe and resolve stage launchers of the pipelined classification.
#define K2G_PIPELINE_STAGE_KERNELS
#include "classify_kernels.cuh"
#include "pipeline.cuh"

namespace k2g {

cudaError_t launch_pipe_probe(const PipeArgs &pa, cudaStream_t st) {
  const unsigned blocks = (unsigned)((pa.a.n_frags + kPipeBlock - 1) / kPipeBlock);
  pipe_probe_kernel<<<blocks, kPipeBlock, 0, st>>>(pa);
  return cudaGetLastError();
}

cudaError_t launch_pipe_resolve(const PipeArgs &pa, cudaStream_t st) {
  const unsigned blocks = (unsigned)((pa.a.n_frags + kPipeBlock - 1) / kPipeBlock);
  pipe_resolve_kernel<<<blocks, kPipeBlock, 0, st>>>(pa);
  return cudaGetLastError();
}

}  // namespace k2g
