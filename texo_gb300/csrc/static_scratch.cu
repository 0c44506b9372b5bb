// static_scratch.cu — density scatter that allocates nothing.
//
// texo_gp_scatter_static computes exactly what texo_gp_scatter returns (the
// int64 2^-32 fixed-point physical and filler grids at the given
// coordinates) but keeps every intermediate in one file-scope device array
// instead of the handle's buffers or any new allocation. It calls no
// cudaMalloc/cudaFree, no allocating library routine and no host heap
// allocation; the handle's own buffers and its resumable run state are not
// touched.
//
// Scratch layout (64-bit words, 4 MiB in total):
//   [0, kGridWords)               physical grid  [num_fields][bins]
//   [kGridWords, 2 kGridWords)    filler grid    [num_fields][bins]
//   [2 kGridWords, +2 kMaxObjects) coordinates, double2 per unit / filler
// Limits: num_fields * bins <= kGridWords and units + fillers <=
// kMaxObjects; larger handles are rejected with TEXO_GP_ERR_UNSUPPORTED.
//
// Nothing in the scratch has to start at zero: each call copies the
// coordinates in, then sets every grid word it uses (physical grid to the
// negated capacity background, filler grid to zero) before the scatter.
//
// There is one scratch per device per loaded copy of this library. Calls
// must not overlap on a device: two calls in flight at once (two threads,
// or two handles on one device) race on the same words and corrupt both
// results. Each call synchronizes its stream before it returns, so calls
// made one after another are safe.
#include <mutex>
#include <string>

#include "engine.h"
#include "stages.cuh"

namespace {
using namespace tgp;

constexpr size_t kGridWords = 131072;   // per grid: num_fields * bins
constexpr size_t kMaxObjects = 131072;  // units + fillers
constexpr size_t kScratchWords = 2 * kGridWords + 2 * kMaxObjects;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned long long g_scratch[kScratchWords];

// Device address of g_scratch, looked up once per device with that device
// current (the first call on a device does it; no allocation involved).
std::mutex g_setup_mu;
void* g_scratch_addr[kMaxDevices] = {};

#define SCU(call)                                                          \
  do {                                                                     \
    cudaError_t e_ = (call);                                               \
    if (e_ != cudaSuccess) {                                               \
      set_last_error(std::string(#call) + ": " + cudaGetErrorString(e_));  \
      return TEXO_GP_ERR_CUDA;                                             \
    }                                                                      \
  } while (0)

int32_t scratch_address(int device, void** out) {
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (!g_scratch_addr[device]) {
    void* p = nullptr;
    SCU(cudaGetSymbolAddress(&p, g_scratch));
    g_scratch_addr[device] = p;
  }
  *out = g_scratch_addr[device];
  return TEXO_GP_OK;
}

// Background of the two grids (the same values stage_init writes).
__global__ void __launch_bounds__(kThreads) k_scratch_init(Dev d, long long* phys, long long* fill) {
  const int n = d.K * d.B;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    phys[i] = -d.capfix[i];
    fill[i] = 0;
  }
}

// The scatter of stage_scatter, reading FP64 coordinates and rounding them
// to FP32 on the device (round to nearest even, as the host upload does),
// with no per-block partials.
__global__ void __launch_bounds__(kThreads) k_scatter_scratch(Dev d, const double2* xy, long long* phys,
                                                               long long* fill) {
  const int items = d.Mm + d.F;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < items; i += gridDim.x * blockDim.x) {
    float sxp, syp, q;
    unsigned long long* grid;
    if (i < d.Mm) {
      const int u = d.mem_unit[i];
      const float2 o = d.mem_off[i];
      const double2 pu = xy[u];
      sxp = __fadd_rn(__double2float_rn(pu.x), o.x);
      syp = __fadd_rn(__double2float_rn(pu.y), o.y);
      q = d.mem_q[i];
      grid = (unsigned long long*)(phys + (size_t)d.mem_field[i] * d.B);
    } else {
      const int j = i - d.Mm;
      const double2 pf = xy[d.U + j];
      sxp = __double2float_rn(pf.x);
      syp = __double2float_rn(pf.y);
      q = d.fil_q[j];
      grid = (unsigned long long*)(fill + (size_t)d.fil_field[j] * d.B);
    }
    const AxisTaps ax = taps_x(d, sxp);
    const AxisTaps ay = taps_y(d, syp);
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c)
        atomicAdd(grid + (size_t)ay.idx[r] * d.g.Wb + ax.idx[c],
                  (unsigned long long)tap_fixed(q, ax.w[c], ay.w[r]));
  }
}

int32_t scatter_static(Instance& I, const double* coordinates, int64_t* physical, int64_t* fillers) {
  const size_t nobj = (size_t)I.d.nobj, n = (size_t)I.m.K * I.m.bins();
  if (n > kGridWords) {
    set_last_error("texo_gp_scatter_static: num_fields * bins = " + std::to_string(n) +
                   " exceeds the static scratch limit of " + std::to_string(kGridWords));
    return TEXO_GP_ERR_UNSUPPORTED;
  }
  if (nobj > kMaxObjects) {
    set_last_error("texo_gp_scatter_static: units + fillers = " + std::to_string(nobj) +
                   " exceeds the static scratch limit of " + std::to_string(kMaxObjects));
    return TEXO_GP_ERR_UNSUPPORTED;
  }
  if (I.device < 0 || I.device >= kMaxDevices) {
    set_last_error("texo_gp_scatter_static: device ordinal out of range");
    return TEXO_GP_ERR_UNSUPPORTED;
  }
  int prev = 0;
  SCU(cudaGetDevice(&prev));
  if (prev != I.device) SCU(cudaSetDevice(I.device));
  void* base = nullptr;
  int32_t s = scratch_address(I.device, &base);
  if (s == TEXO_GP_OK) {
    unsigned long long* w = (unsigned long long*)base;
    long long* phys = (long long*)w;
    long long* fill = (long long*)(w + kGridWords);
    double2* xy = (double2*)(w + 2 * kGridWords);
    const cudaStream_t st = I.stream;
    cudaError_t e = cudaMemcpyAsync(xy, coordinates, nobj * sizeof(double2), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
      k_scratch_init<<<I.nvb, kThreads, 0, st>>>(I.d, phys, fill);
      k_scatter_scratch<<<I.nvb, kThreads, 0, st>>>(I.d, xy, phys, fill);
      note_launch();
      note_launch();
      e = cudaGetLastError();
    }
    if (e == cudaSuccess && physical)
      e = cudaMemcpyAsync(physical, phys, n * sizeof(int64_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && fillers)
      e = cudaMemcpyAsync(fillers, fill, n * sizeof(int64_t), cudaMemcpyDeviceToHost, st);
    const cudaError_t es = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = es;
    if (e != cudaSuccess) {
      set_last_error(std::string("texo_gp_scatter_static: ") + cudaGetErrorString(e));
      s = TEXO_GP_ERR_CUDA;
    }
  }
  if (prev != I.device) cudaSetDevice(prev);
  return s;
}

}  // namespace

extern "C" int32_t texo_gp_scatter_static(texo_gp_handle h, const double* coordinates, int64_t* physical_grid,
                                          int64_t* filler_grid) {
  if (!h || !coordinates) return TEXO_GP_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(*handle_mutex(h));
  return scatter_static(*handle_instance(h), coordinates, physical_grid, filler_grid);
}
