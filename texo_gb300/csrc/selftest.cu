// selftest.cu — exercises the bounded device waits without faulting.
//
// Two blocks meet at a grid barrier sized for three, so the third arrival
// never comes, and one block waits on an mbarrier nothing arrives on. With a
// short poll limit both waits run out, record it and return; the host reads
// the two flags and the context stays usable. The waits are the production
// ones (grid_sync of the persistent loop, tc::try_wait of the tensor-core
// pipeline) with a smaller limit.
#include <string>

#include "engine.h"
#include "persistent_body.cuh"

namespace tgp {
namespace {

__global__ void k_wait_selftest(GridBarrier* bar, unsigned limit, int* barrier_timed_out, int* mbar_timed_out) {
  __shared__ unsigned gen;
  __shared__ int failed;
  __shared__ unsigned long long mbar;
  if (threadIdx.x == 0) gen = 0;
  __syncthreads();
  unsigned long long count = 0;
  const bool ok = grid_sync(bar, gridDim.x + 1u, &gen, &count, nullptr, &failed, limit);
  if (threadIdx.x == 0) atomicOr(barrier_timed_out, ok ? 0 : 1);
  if (blockIdx.x == 0) {
    if (threadIdx.x == 0) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc::saddr(&mbar)) : "memory");
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
      bool done = false;
      for (unsigned i = 0; i < limit && !done; ++i) done = tc::try_wait(tc::saddr(&mbar), 0u);
      *mbar_timed_out = done ? 0 : 1;
    }
    __syncthreads();
  }
}

}  // namespace
}  // namespace tgp

extern "C" int32_t texo_gp_selftest_waits(int32_t device, int32_t* barrier_timed_out, int32_t* mbarrier_timed_out) {
  using namespace tgp;
  if (!barrier_timed_out || !mbarrier_timed_out) return TEXO_GP_ERR_INVALID_ARGUMENT;
  if (cudaSetDevice(device) != cudaSuccess) return TEXO_GP_ERR_CUDA;
  GridBarrier* bar = nullptr;
  int* flags = nullptr;
  int32_t s = TEXO_GP_OK;
  if (cudaMalloc(&bar, sizeof(GridBarrier)) != cudaSuccess || cudaMalloc(&flags, 2 * sizeof(int)) != cudaSuccess) {
    s = TEXO_GP_ERR_OUT_OF_MEMORY;
  } else {
    int h[2] = {-1, -1};
    cudaMemset(bar, 0, sizeof(GridBarrier));
    cudaMemset(flags, 0, 2 * sizeof(int));
    k_wait_selftest<<<2, kThreads>>>(bar, 1u << 12, flags, flags + 1);
    if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess ||
        cudaMemcpy(h, flags, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess) {
      set_last_error(std::string("wait self-test: ") + cudaGetErrorString(cudaGetLastError()));
      s = TEXO_GP_ERR_CUDA;
    }
    *barrier_timed_out = h[0];
    *mbarrier_timed_out = h[1];
  }
  if (bar) cudaFree(bar);
  if (flags) cudaFree(flags);
  return s;
}
