// fibmd_graph.cu — device-side conditions of the CUDA-graph step loop.
//
// The spec-mode step sequence is captured once into a graph whose WHILE node
// runs pairs of MD steps until a device counter reaches zero, and whose IF
// nodes run the list rebuild only on the steps where the drift found an atom
// beyond half the skin (the drift kernel's last block sets that condition).
// This single-thread kernel counts the step pairs down on the device, so no
// step needs the host.
#include "fibmd_internal.cuh"

namespace fibmd {

__global__ void k_loop_ctl(int* remaining, cudaGraphConditionalHandle h) {
  const int r = *remaining - 1;
  *remaining = r;
  cudaGraphSetConditional(h, r > 0 ? 1u : 0u);
}

cudaError_t launch_loop_ctl(cudaStream_t s, int* remaining, cudaGraphConditionalHandle h) {
  k_loop_ctl<<<1, 1, 0, s>>>(remaining, h);
  return cudaGetLastError();
}

}  // namespace fibmd
