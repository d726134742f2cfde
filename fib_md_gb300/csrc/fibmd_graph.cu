// fibmd_graph.cu — device-side conditions of the CUDA-graph step loop.
//
// The spec-mode step sequence is captured once into a graph whose WHILE node
// runs pairs of MD steps until a device counter reaches zero, and whose IF
// nodes run the list rebuild only on the steps where the drift found it due
// (the drift sets a flag, the condition kernel after it the IF node).
// These single-thread kernels count the step pairs down (and stop a
// relaxation at its end time) on the device, so no step needs the host.
#include "fibmd_internal.cuh"

namespace fibmd {

__global__ void k_loop_ctl(LoopCtl* loop, const DevScalars* sc, cudaGraphConditionalHandle h) {
  pdl_wait();
  const long long r = loop->pairs - 1;
  loop->pairs = r;
  loop->pairs_run += 1;
  const double t = ((const volatile DevScalars*)sc)->time;
  cudaGraphSetConditional(h, (r > 0 && t < loop->t_stop) ? 1u : 0u);
}

__global__ void k_loop_set(LoopCtl* loop, const DevScalars* sc, long long pairs, double relax) {
  loop->pairs = pairs;
  loop->t_stop = relax > 0.0 ? ((const volatile DevScalars*)sc)->time + relax : 1.0e300;
}

cudaError_t launch_loop_ctl(cudaStream_t s, LoopCtl* loop, const DevScalars* sc,
                            cudaGraphConditionalHandle h, bool pdl) {
  return launch_k(k_loop_ctl, 1, 1, 0, s, pdl, loop, sc, h);
}

cudaError_t launch_loop_set(cudaStream_t s, LoopCtl* loop, const DevScalars* sc, long long pairs,
                            double relax) {
  k_loop_set<<<1, 1, 0, s>>>(loop, sc, pairs, relax);
  return cudaGetLastError();
}

}  // namespace fibmd
