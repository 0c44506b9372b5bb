// persistent_solo_small.cu — k_persistent with small DCT tiles: one placement on every
// co-resident block of the GPU.
#include "persistent_body.cuh"

namespace tgp {

__global__ void __launch_bounds__(kThreads, kBlocksPerSm)
    k_persistent_small(Dev d, Reduce r, Buffers B, DevRun* run, GridBarrier* bar, int V) {
  run_body<false>(d, r, B, run, bar, (int)blockIdx.x, (int)gridDim.x, V);
}

const void* persistent_kernel_small() { return (const void*)k_persistent_small; }

}  // namespace tgp
