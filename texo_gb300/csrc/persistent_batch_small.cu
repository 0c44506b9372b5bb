// persistent_batch_small.cu — k_batch with small DCT tiles: many placements in one launch;
// block b serves instance map[b].x as its physical block map[b].y of map[b].z.
#include "persistent_body.cuh"

namespace tgp {

__global__ void __launch_bounds__(kThreads, kBatchBlocksPerSm) k_batch_small(const InstDesc* descs, const int4* map) {
  __shared__ InstDesc sd;
  const int4 m = map[blockIdx.x];
  copy_words(&sd, descs + m.x);
  __syncthreads();
  run_body<false>(sd.d, sd.r, sd.B, sd.run, sd.bar, m.y, m.z, sd.V);
}

const void* batch_kernel_small() { return (const void*)k_batch_small; }

}  // namespace tgp
