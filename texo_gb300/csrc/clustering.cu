// clustering.cu — elfPlace's register-clustering area estimate on the GPU
// (`clustering_areas`, crates/texo-pnr/src/register_clustering.rs:17-80).
//
// For each register, the expected number of registers of its control set
// (clock, LSR) inside its window, split by clock enable, is a sum over the
// other registers of the set of Gaussian window probabilities, x times y:
// all-pairs work within a control set, which the reference spreads over
// rayon threads. Here one thread owns one focal register and walks its
// control set; the registers are sorted stably by (clock, LSR, clock
// enable) on the host, so a clock enable's sum runs in input order and the
// per-enable totals in ascending enable order, as in the reference's
// BTreeMaps. Sums and soft ceilings use explicitly rounded FP64 operations
// (no fused multiply-add, which the reference never uses); erf is CUDA's.
// A pair whose windows lie more than 8 sigma sqrt(2) apart on an axis
// contributes an exact zero (erf saturates), so it is skipped, after a
// conservative FP32 test. Threads take the registers of a control set in
// tile order, so the lanes of a warp agree on which pairs are far (FP64
// runs at a low rate on this part: a warp whose lanes disagree pays for the
// slowest lane's erf work on every pair).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "engine.h"

namespace tgp {
namespace {

constexpr int kClusterThreads = 128;

// soft_division_ceiling (register_clustering.rs:89-97)
__device__ __forceinline__ double soft_ceiling(double value, double divisor) {
  const double quotient = __ddiv_rn(value, divisor);
  const double fl = floor(quotient);
  if (__dsub_rn(quotient, fl) < __ddiv_rn(1.0, divisor)) return __dadd_rn(value, __dmul_rn(1.0 - divisor, fl));
  return ceil(quotient);
}

// gaussian_interval_probability (register_clustering.rs:84-87)
__device__ __forceinline__ double window_probability(double low, double high, double mean, double scale) {
  const double p = __dmul_rn(0.5, __dsub_rn(erf(__ddiv_rn(__dsub_rn(high, mean), scale)),
                                           erf(__ddiv_rn(__dsub_rn(low, mean), scale))));
  return fmin(fmax(p, 0.0), 1.0);
}

struct ClusterDev {
  unsigned n;
  const double *x, *y;                 // sorted by (clock, lsr, ce), stable
  const float2* xy32;                  // the same positions in FP32, for the far-pair test
  const unsigned long long* ce;
  const unsigned* focal;               // thread -> sorted position: near registers share a warp
  const unsigned *group_begin, *group_end;   // per sorted register: its control set's range
  const unsigned* order;               // sorted position -> input index
  double half_window, scale, cutoff;
  float cutoff32;                      // cutoff plus a margin that covers the FP32 rounding
  double* areas;                       // by input index
  int* bad;
};

__global__ void __launch_bounds__(kClusterThreads) k_clustering(ClusterDev d) {
  const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= d.n) return;
  const unsigned p = __ldg(d.focal + t);
  const float2 fi = __ldg(d.xy32 + p);
  const unsigned b = __ldg(d.group_begin + p), e = __ldg(d.group_end + p);
  const double xi = __ldg(d.x + p), yi = __ldg(d.y + p);
  const unsigned long long focal_ce = __ldg(d.ce + p);
  const double xlo = __dsub_rn(xi, d.half_window), xhi = __dadd_rn(xi, d.half_window);
  const double ylo = __dsub_rn(yi, d.half_window), yhi = __dadd_rn(yi, d.half_window);
  double total = 0.0, focal = 0.0, sum = 0.0;
  unsigned long long cur = __ldg(d.ce + b);
  for (unsigned j = b; j < e; ++j) {
    const unsigned long long cj = __ldg(d.ce + j);
    if (cj != cur) {   // one clock enable's expectation is complete
      total = __dadd_rn(total, soft_ceiling(sum, 2.0));
      if (cur == focal_ce) focal = sum;
      sum = 0.0;
      cur = cj;
    }
    // far in FP32 (with margin) implies far in FP64: skip without FP64 work
    const float2 fj = __ldg(d.xy32 + j);
    if (fabsf(fi.x - fj.x) > d.cutoff32 || fabsf(fi.y - fj.y) > d.cutoff32) continue;
    const double xj = __ldg(d.x + j), yj = __ldg(d.y + j);
    if (fabs(__dsub_rn(xi, xj)) > d.cutoff || fabs(__dsub_rn(yi, yj)) > d.cutoff) continue;
    const double px = window_probability(xlo, xhi, xj, d.scale);
    const double py = window_probability(ylo, yhi, yj, d.scale);
    sum = __dadd_rn(sum, __dmul_rn(px, py));
  }
  total = __dadd_rn(total, soft_ceiling(sum, 2.0));
  if (cur == focal_ce) focal = sum;
  const unsigned out = __ldg(d.order + p);
  if (!(isfinite(focal) && focal > 0.0)) {
    atomicExch(d.bad, 1);
    d.areas[out] = 0.0;
    return;
  }
  // 8 / E_focal * ceil2(E_focal) / total * ceil4(total), left to right
  const double area = __dmul_rn(__ddiv_rn(__dmul_rn(__ddiv_rn(8.0, focal), soft_ceiling(focal, 2.0)), total),
                                soft_ceiling(total, 4.0));
  if (!(isfinite(area) && area >= 0.0)) atomicExch(d.bad, 1);
  d.areas[out] = area;
}

}  // namespace
}  // namespace tgp

using namespace tgp;

extern "C" int32_t texo_gp_register_clustering_areas(int32_t device, uint64_t num_registers, const double* xy,
                                                     const uint64_t* clock_lsr, const uint64_t* ce,
                                                     uint64_t movable_instance_count, double* areas,
                                                     double* elapsed_ms) {
  if (elapsed_ms) *elapsed_ms = 0.0;
  const uint64_t n = num_registers;
  if (n == 0) return TEXO_GP_OK;
  if (!xy || !clock_lsr || !ce || !areas) {
    set_last_error("register clustering: null argument");
    return TEXO_GP_ERR_INVALID_ARGUMENT;
  }
  if (movable_instance_count == 0) {   // the reference's empty map: no clustering area
    for (uint64_t r = 0; r < n; ++r) areas[r] = 0.0;
    return TEXO_GP_OK;
  }
  if (movable_instance_count > 0xffffffffull || n > (1ull << 31)) {
    set_last_error("register clustering: count out of range");
    return TEXO_GP_ERR_INVALID_NORMALIZATION;
  }
  const double sigma = std::sqrt(1.0e-5 * (double)(uint32_t)movable_instance_count);
  if (!std::isfinite(sigma) || sigma <= 0.0) return TEXO_GP_ERR_INVALID_NORMALIZATION;
  const double half_window = 2.5 * sigma, scale = sigma * 1.4142135623730951;   // sigma sqrt(2)
  const double cutoff = half_window + 8.0 * scale;

  // sort by (clock, lsr, ce), stable: input order within a clock enable
  std::vector<uint32_t> order(n);
  std::iota(order.begin(), order.end(), 0u);
  std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
    if (clock_lsr[2 * (size_t)a] != clock_lsr[2 * (size_t)b]) return clock_lsr[2 * (size_t)a] < clock_lsr[2 * (size_t)b];
    if (clock_lsr[2 * (size_t)a + 1] != clock_lsr[2 * (size_t)b + 1])
      return clock_lsr[2 * (size_t)a + 1] < clock_lsr[2 * (size_t)b + 1];
    return ce[a] < ce[b];
  });
  std::vector<double> sx(n), sy(n);
  std::vector<float> s32(2 * n);
  std::vector<unsigned long long> sce(n);
  std::vector<uint32_t> gb(n), ge(n), focal(n);
  double extent = 0.0;
  for (uint64_t p = 0; p < n; ++p) {
    sx[p] = xy[2 * (size_t)order[p]];
    sy[p] = xy[2 * (size_t)order[p] + 1];
    s32[2 * p] = (float)sx[p];
    s32[2 * p + 1] = (float)sy[p];
    sce[p] = ce[order[p]];
    if (std::isfinite(sx[p])) extent = std::max(extent, std::fabs(sx[p]));
    if (std::isfinite(sy[p])) extent = std::max(extent, std::fabs(sy[p]));
  }
  for (uint64_t p = 0; p < n;) {
    uint64_t q = p + 1;
    const uint32_t a = order[p];
    while (q < n && clock_lsr[2 * (size_t)order[q]] == clock_lsr[2 * (size_t)a] &&
           clock_lsr[2 * (size_t)order[q] + 1] == clock_lsr[2 * (size_t)a + 1])
      ++q;
    for (uint64_t r = p; r < q; ++r) {
      gb[r] = (uint32_t)p;
      ge[r] = (uint32_t)q;
    }
    // the threads of a control set take its registers in tile order (rows
    // of 8-tile blocks), so a warp's registers are near one another and
    // agree on which pairs are far
    std::iota(focal.begin() + p, focal.begin() + q, (uint32_t)p);
    auto block_of = [&](uint32_t r) -> uint64_t {
      const double bx = std::isfinite(sx[r]) ? std::floor(sx[r] / 8.0) : 0.0;
      const double by = std::isfinite(sy[r]) ? std::floor(sy[r] / 8.0) : 0.0;
      return ((uint64_t)(int64_t)(by + 1.0e6) << 32) | (uint64_t)(uint32_t)(int64_t)(bx + 1.0e6);
    };
    std::stable_sort(focal.begin() + p, focal.begin() + q,
                     [&](uint32_t a, uint32_t b) { return block_of(a) < block_of(b); });
    p = q;
  }
  // FP32 positions are within 2^-24 |coordinate| of the FP64 ones; a margin of
  // 2^-20 (extent + cutoff) keeps the FP32 far test conservative
  const float cutoff32 = (float)(cutoff + std::ldexp(extent + cutoff + 1.0, -20));

  if (cudaSetDevice(device) != cudaSuccess) return TEXO_GP_ERR_CUDA;
  cudaStream_t s = nullptr;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return TEXO_GP_ERR_CUDA;
  auto round = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t s8 = round(n * 8), s4 = round(n * 4);
  char* base = nullptr;
  if (cudaMallocAsync((void**)&base, 5 * s8 + 4 * s4 + 256, s) != cudaSuccess) {
    cudaStreamDestroy(s);
    return TEXO_GP_ERR_OUT_OF_MEMORY;
  }
  ClusterDev d{};
  d.n = (unsigned)n;
  d.half_window = half_window;
  d.scale = scale;
  d.cutoff = cutoff;
  double* dx = (double*)base;
  double* dy = (double*)(base + s8);
  unsigned long long* dce = (unsigned long long*)(base + 2 * s8);
  d.areas = (double*)(base + 3 * s8);
  unsigned* dgb = (unsigned*)(base + 4 * s8);
  unsigned* dge = (unsigned*)(base + 4 * s8 + s4);
  unsigned* dord = (unsigned*)(base + 4 * s8 + 2 * s4);
  float2* d32 = (float2*)(base + 4 * s8 + 3 * s4);
  unsigned* dfoc = (unsigned*)(base + 5 * s8 + 3 * s4);
  d.bad = (int*)(base + 5 * s8 + 4 * s4);
  d.xy32 = d32;
  d.focal = dfoc;
  d.cutoff32 = cutoff32;
  d.x = dx;
  d.y = dy;
  d.ce = dce;
  d.group_begin = dgb;
  d.group_end = dge;
  d.order = dord;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, s);
  bool ok = cudaMemcpyAsync(dx, sx.data(), n * 8, cudaMemcpyHostToDevice, s) == cudaSuccess &&
            cudaMemcpyAsync(dy, sy.data(), n * 8, cudaMemcpyHostToDevice, s) == cudaSuccess &&
            cudaMemcpyAsync(dce, sce.data(), n * 8, cudaMemcpyHostToDevice, s) == cudaSuccess &&
            cudaMemcpyAsync(dgb, gb.data(), n * 4, cudaMemcpyHostToDevice, s) == cudaSuccess &&
            cudaMemcpyAsync(dge, ge.data(), n * 4, cudaMemcpyHostToDevice, s) == cudaSuccess &&
            cudaMemcpyAsync(dord, order.data(), n * 4, cudaMemcpyHostToDevice, s) == cudaSuccess &&
            cudaMemcpyAsync(d32, s32.data(), n * 8, cudaMemcpyHostToDevice, s) == cudaSuccess &&
            cudaMemcpyAsync(dfoc, focal.data(), n * 4, cudaMemcpyHostToDevice, s) == cudaSuccess &&
            cudaMemsetAsync(d.bad, 0, sizeof(int), s) == cudaSuccess;
  if (ok) {
    k_clustering<<<(unsigned)((n + kClusterThreads - 1) / kClusterThreads), kClusterThreads, 0, s>>>(d);
    ok = cudaGetLastError() == cudaSuccess;
    if (ok) note_launch();
  }
  int bad = 0;
  ok = ok && cudaMemcpyAsync(areas, d.areas, n * 8, cudaMemcpyDeviceToHost, s) == cudaSuccess &&
       cudaMemcpyAsync(&bad, d.bad, sizeof(int), cudaMemcpyDeviceToHost, s) == cudaSuccess;
  cudaEventRecord(e1, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) ok = false;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFreeAsync(base, s);
  cudaStreamSynchronize(s);
  cudaStreamDestroy(s);
  if (elapsed_ms) *elapsed_ms = ms;
  if (!ok) {
    set_last_error(std::string("register clustering: ") + cudaGetErrorString(cudaGetLastError()));
    return TEXO_GP_ERR_CUDA;
  }
  if (bad) {
    set_last_error("register clustering: a register's expectation is not positive and finite");
    return TEXO_GP_ERR_INVALID_NORMALIZATION;
  }
  return TEXO_GP_OK;
}
