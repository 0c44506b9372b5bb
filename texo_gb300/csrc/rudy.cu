// rudy.cu — continuous RUDY routing demand on the GPU
// (`continuous_routing_demand`, crates/texo-pnr/src/eplace.rs:856-937).
//
// A net's bounding box (min_x, max_x, min_y, max_y), widened by half a tile on
// every side, spreads the densities dx / area (horizontal) and dy / area
// (vertical), area = (dx + 1)(dy + 1), over the tiles it overlaps, each tile
// weighted by overlap_x * overlap_y. Along one axis the overlap is exactly 1
// for every tile whose unit interval lies inside the widened box and
// fractional for at most one tile on each side, so a box is at most 3 x 3
// rectangles of constant value. Each rectangle goes into a 2-D difference
// array with four int64 2^-40 fixed-point updates (order-independent, so the
// map is deterministic); a row scan and a column scan then give the map.
// The per-rectangle values are the reference's FP64 expressions
// (density * (overlap_x * overlap_y)); the fixed-point rounding (2^-41 per
// rectangle and tile) is the difference from the reference's FP64 sums.
#include <cmath>
#include <cstring>
#include <string>

#include "common.cuh"
#include "engine.h"
#include "kernels.cuh"

namespace tgp {
namespace {

// 2^40: a box adds at most 1 to a tile, so up to 2^22 boxes keep every
// partial sum of the difference array inside int64
constexpr double kRudyFix = 1099511627776.0;
constexpr uint64_t kRudyMaxBoxes = 1ull << 22;

// One axis of a widened box: up to three pieces (first tile, count, overlap).
struct Pieces {
  int a[3], b[3];
  double v[3];
  int n;
};

// The tiles of [0, extent) that the box [lo, hi] widened by 0.5 overlaps,
// grouped as (left edge tile, interior run with overlap 1, right edge tile);
// the overlaps are eplace.rs:885-906's expressions.
__device__ __forceinline__ Pieces axis_pieces(double lo, double hi, int extent) {
  Pieces p;
  p.n = 0;
  const double rlo = lo - 0.5, rhi = hi + 0.5;
  const double ia = ceil(lo), ib = floor(hi);   // tiles whose unit interval lies inside
  auto overlap = [&](double t) { return fmax(fmin(t + 0.5, rhi) - fmax(t - 0.5, rlo), 0.0); };
  const double left = ia - 1.0, right = ib + 1.0;
  if (left >= 0.0 && left < extent) {
    const double o = overlap(left);
    if (o > 0.0) {
      p.a[p.n] = p.b[p.n] = (int)left;
      p.v[p.n++] = o;
    }
  }
  const double s = fmax(ia, 0.0), e = fmin(ib, (double)extent - 1.0);
  if (s <= e) {
    p.a[p.n] = (int)s;
    p.b[p.n] = (int)e;
    p.v[p.n++] = 1.0;
  }
  if (right >= 0.0 && right < extent && right != left) {
    const double o = overlap(right);
    if (o > 0.0) {
      p.a[p.n] = p.b[p.n] = (int)right;
      p.v[p.n++] = o;
    }
  }
  return p;
}

// diff: [2][(H + 1) x (W + 1)] int64, zeroed.
__global__ void k_rudy_boxes(const double* boxes, long long nbox, int W, int H, unsigned long long* diff) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nbox) return;
  const double x0 = boxes[4 * i], x1 = boxes[4 * i + 1], y0 = boxes[4 * i + 2], y1 = boxes[4 * i + 3];
  const double dx = x1 - x0, dy = y1 - y0;
  const double area = (dx + 1.0) * (dy + 1.0);
  const double hd = dx / area, vd = dy / area;
  const Pieces px = axis_pieces(x0, x1, W), py = axis_pieces(y0, y1, H);
  const size_t plane = (size_t)(W + 1) * (H + 1);
  for (int a = 0; a < py.n; ++a)
    for (int b = 0; b < px.n; ++b) {
      const double overlap = px.v[b] * py.v[a];
      const long long h = __double2ll_rn(hd * overlap * kRudyFix), v = __double2ll_rn(vd * overlap * kRudyFix);
      const int xa = px.a[b], xb = px.b[b] + 1, ya = py.a[a], yb = py.b[a] + 1;
      const size_t c00 = (size_t)ya * (W + 1) + xa, c01 = (size_t)ya * (W + 1) + xb;
      const size_t c10 = (size_t)yb * (W + 1) + xa, c11 = (size_t)yb * (W + 1) + xb;
      if (h) {
        atomicAdd(diff + c00, (unsigned long long)h);
        atomicAdd(diff + c01, (unsigned long long)(-h));
        atomicAdd(diff + c10, (unsigned long long)(-h));
        atomicAdd(diff + c11, (unsigned long long)h);
      }
      if (v) {
        atomicAdd(diff + plane + c00, (unsigned long long)v);
        atomicAdd(diff + plane + c01, (unsigned long long)(-v));
        atomicAdd(diff + plane + c10, (unsigned long long)(-v));
        atomicAdd(diff + plane + c11, (unsigned long long)v);
      }
    }
}

// Inclusive scan along each row of both planes: a warp per row, 32 columns
// a step (a shuffle scan plus the carry of the previous step). The sums are
// exact integers, so any order gives the same values.
__global__ void k_rudy_rows(unsigned long long* __restrict__ diff, int W, int H) {
  const int warp = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = (int)(threadIdx.x & 31);
  if (warp >= 2 * H) return;   // uniform across the warp
  const int plane = warp / H, y = warp % H;
  unsigned long long* row = diff + (size_t)plane * (W + 1) * (H + 1) + (size_t)y * (W + 1);
  unsigned long long carry = 0;
  for (int x0 = 0; x0 < W; x0 += 32) {
    const int x = x0 + lane;
    unsigned long long v = x < W ? row[x] : 0ull;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long t = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += t;
    }
    v += carry;
    if (x < W) row[x] = v;
    carry = __shfl_sync(0xffffffffu, v, 31);
  }
}

// Inclusive scan along each column, written out as FP64 demand: a block per
// strip of 32 columns of one plane; its warps take consecutive row segments,
// sum them, add the totals of the segments above and scan their own (the
// loads of a segment do not depend on one another).
constexpr int kColWarps = 8;
__global__ void __launch_bounds__(32 * kColWarps) k_rudy_cols(const unsigned long long* __restrict__ diff, int W,
                                                              int H, double* __restrict__ horizontal,
                                                              double* __restrict__ vertical) {
  __shared__ unsigned long long seg[kColWarps][32];
  const int lane = (int)(threadIdx.x & 31), w = (int)(threadIdx.x >> 5);
  const int strips = (W + 31) / 32;
  const int plane = (int)blockIdx.x / strips, x = ((int)blockIdx.x % strips) * 32 + lane;
  const unsigned long long* col = diff + (size_t)plane * (W + 1) * (H + 1) + x;
  double* out = plane ? vertical : horizontal;
  const int per = (H + kColWarps - 1) / kColWarps, y0 = min(H, w * per), y1 = min(H, y0 + per);
  unsigned long long s = 0;
  if (x < W)
    for (int y = y0; y < y1; ++y) s += col[(size_t)y * (W + 1)];
  seg[w][lane] = s;
  __syncthreads();
  unsigned long long c = 0;
  for (int k = 0; k < w; ++k) c += seg[k][lane];
  if (x < W)
    for (int y = y0; y < y1; ++y) {
      c += col[(size_t)y * (W + 1)];
      out[(size_t)y * W + x] = (double)(long long)c / kRudyFix;
    }
}

}  // namespace
}  // namespace tgp

using namespace tgp;

extern "C" int32_t texo_gp_routing_demand(int32_t device, uint32_t width, uint32_t height, uint64_t num_boxes,
                                          const double* boxes, double* horizontal, double* vertical,
                                          double* elapsed_ms) {
  if (elapsed_ms) *elapsed_ms = 0.0;
  if (!horizontal || !vertical || (num_boxes && !boxes)) return TEXO_GP_ERR_INVALID_ARGUMENT;
  if (width == 0 || height == 0 || (uint64_t)width * height > (1ull << 26)) return TEXO_GP_ERR_INVALID_NORMALIZATION;
  for (uint64_t i = 0; i < num_boxes; ++i) {
    const double* b = boxes + 4 * i;
    if (!(std::isfinite(b[0]) && std::isfinite(b[1]) && std::isfinite(b[2]) && std::isfinite(b[3])) ||
        b[0] > b[1] || b[2] > b[3]) {
      set_last_error("routing demand: box " + std::to_string(i) + " is not finite or not ordered");
      return TEXO_GP_ERR_INVALID_NORMALIZATION;
    }
  }
  if (num_boxes > kRudyMaxBoxes) return TEXO_GP_ERR_FIXED_POINT_RANGE;
  if (cudaSetDevice(device) != cudaSuccess) return TEXO_GP_ERR_CUDA;
  const int W = (int)width, H = (int)height;
  const size_t tiles = (size_t)W * H, plane = (size_t)(W + 1) * (H + 1);
  cudaStream_t s = nullptr;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return TEXO_GP_ERR_CUDA;
  char* base = nullptr;
  const size_t b_bytes = ((std::max<uint64_t>(num_boxes, 1) * 32) + 255) & ~(size_t)255;
  const size_t d_bytes = ((2 * plane * 8) + 255) & ~(size_t)255;
  const size_t o_bytes = ((tiles * 8) + 255) & ~(size_t)255;
  if (cudaMallocAsync((void**)&base, b_bytes + d_bytes + 2 * o_bytes, s) != cudaSuccess) {
    cudaStreamDestroy(s);
    return TEXO_GP_ERR_OUT_OF_MEMORY;
  }
  double* dbox = (double*)base;
  unsigned long long* diff = (unsigned long long*)(base + b_bytes);
  double* dh = (double*)(base + b_bytes + d_bytes);
  double* dv = (double*)(base + b_bytes + d_bytes + o_bytes);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, s);
  bool ok = (!num_boxes || cudaMemcpyAsync(dbox, boxes, num_boxes * 32, cudaMemcpyHostToDevice, s) == cudaSuccess) &&
            cudaMemsetAsync(diff, 0, 2 * plane * 8, s) == cudaSuccess;
  if (ok && num_boxes) {
    k_rudy_boxes<<<(unsigned)((num_boxes + kThreads - 1) / kThreads), kThreads, 0, s>>>(dbox, (long long)num_boxes,
                                                                                       W, H, diff);
    note_launch();
  }
  if (ok) {
    k_rudy_rows<<<(unsigned)((2 * (size_t)H * 32 + kThreads - 1) / kThreads), kThreads, 0, s>>>(diff, W, H);
    k_rudy_cols<<<(unsigned)(2 * ((W + 31) / 32)), 32 * kColWarps, 0, s>>>(diff, W, H, dh, dv);
    note_launch();
    note_launch();
    ok = cudaGetLastError() == cudaSuccess &&
         cudaMemcpyAsync(horizontal, dh, tiles * 8, cudaMemcpyDeviceToHost, s) == cudaSuccess &&
         cudaMemcpyAsync(vertical, dv, tiles * 8, cudaMemcpyDeviceToHost, s) == cudaSuccess;
  }
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
    set_last_error(std::string("routing demand: ") + cudaGetErrorString(cudaGetLastError()));
    return TEXO_GP_ERR_CUDA;
  }
  return TEXO_GP_OK;
}
