// persistent_solo_large.cu — k_persistent with large DCT tiles: one placement on every
// co-resident block of the GPU.
#include "persistent_body.cuh"

namespace tgp {

__global__ void __launch_bounds__(kThreads, kBlocksPerSm)
    k_persistent_large(Dev d, Reduce r, Buffers B, DevRun* run, GridBarrier* bar, int V) {
  run_body<true>(d, r, B, run, bar, (int)blockIdx.x, (int)gridDim.x, V);
}

const void* persistent_kernel_large() { return (const void*)k_persistent_large; }

}  // namespace tgp
