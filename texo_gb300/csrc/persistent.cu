// persistent.cu — cooperative launches of the persistent placement kernels
// (defined in persistent_{solo,batch}_{small,large}.cu over run_body).
#include "persistent.cuh"

#include <cstring>

namespace tgp {

const void* persistent_kernel_small();
const void* persistent_kernel_large();
const void* batch_kernel_small();
const void* batch_kernel_large();

int persistent_blocks_per_sm() {
  int a = 0, b = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, persistent_kernel_small(), kThreads, 0) != cudaSuccess)
    return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, persistent_kernel_large(), kThreads, 0) != cudaSuccess)
    return 0;
  return a < b ? a : b;
}
int batch_blocks_per_sm() {
  int a = 0, b = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, batch_kernel_small(), kThreads, 0) != cudaSuccess) return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, batch_kernel_large(), kThreads, 0) != cudaSuccess) return 0;
  return a < b ? a : b;
}

static bool large_tiles(const Dev& d) { return d.dct_large != 0; }

int32_t enqueue_persistent(const Dev& d, const Reduce& r, const Buffers& b, RunBlock* dev, RunBlock* host,
                           int blocks, int V, cudaStream_t s) {
  if (cudaMemcpyAsync(dev, host, sizeof(RunBlock), cudaMemcpyHostToDevice, s) != cudaSuccess) return TEXO_GP_ERR_CUDA;
  Dev dd = d;
  Reduce rr = r;
  Buffers bb = b;
  DevRun* run = &dev->run;
  GridBarrier* bar = &dev->bar;
  void* args[] = {&dd, &rr, &bb, &run, &bar, &V};
  const void* fn = large_tiles(d) ? persistent_kernel_large() : persistent_kernel_small();
  if (cudaLaunchCooperativeKernel(fn, dim3(blocks), dim3(kThreads), args, 0, s) != cudaSuccess) return TEXO_GP_ERR_CUDA;
  if (cudaMemcpyAsync(host, dev, sizeof(RunBlock), cudaMemcpyDeviceToHost, s) != cudaSuccess) return TEXO_GP_ERR_CUDA;
  return TEXO_GP_OK;
}

int32_t capture_persistent(const Dev& d, const Reduce& r, const Buffers& b, RunBlock* dev, RunBlock* host,
                           int blocks, int V, cudaStream_t s, cudaGraphExec_t* exec) {
  *exec = nullptr;
  if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    return TEXO_GP_ERR_UNSUPPORTED;
  }
  const int32_t q = enqueue_persistent(d, r, b, dev, host, blocks, V, s);
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture(s, &g);
  bool ok = q == TEXO_GP_OK && e == cudaSuccess && g != nullptr;
  if (ok) ok = cudaGraphInstantiate(exec, g, 0) == cudaSuccess;
  if (g) cudaGraphDestroy(g);
  if (!ok) {
    *exec = nullptr;
    cudaGetLastError();   // a refused capture leaves no sticky error
    return TEXO_GP_ERR_UNSUPPORTED;
  }
  return TEXO_GP_OK;
}

int32_t launch_persistent(const Dev& d, const Reduce& r, const Buffers& b, RunBlock* dev, RunBlock* host,
                          int blocks, int V, cudaStream_t s) {
  std::memset(&host->bar, 0, sizeof(GridBarrier));
  const int32_t q = enqueue_persistent(d, r, b, dev, host, blocks, V, s);
  if (q) return q;
  note_launch();
  if (cudaStreamSynchronize(s) != cudaSuccess) return TEXO_GP_ERR_CUDA;
  if (host->bar.error) return TEXO_GP_ERR_DEVICE_TIMEOUT;
  return TEXO_GP_OK;
}

int32_t launch_batch(const InstDesc* descs_dev, const int4* map_dev, int blocks, bool large, cudaStream_t s) {
  void* args[] = {(void*)&descs_dev, (void*)&map_dev};
  const void* fn = large ? batch_kernel_large() : batch_kernel_small();
  if (cudaLaunchCooperativeKernel(fn, dim3(blocks), dim3(kThreads), args, 0, s) != cudaSuccess) return TEXO_GP_ERR_CUDA;
  note_launch();
  return TEXO_GP_OK;
}

}  // namespace tgp
