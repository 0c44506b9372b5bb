// common.cuh — shared device layout and arithmetic of the placement engine.
//
// Precision plan (GB300 runs FP64 at a small fraction of its FP32 rate):
// every per-object, per-pin and per-bin operation is FP32 or integer; FP64
// appears only in per-block reduction partials and in the scalar controller.
// Positions are FP32. The B-spline offset c - round(c) of an FP32 coordinate
// is exact in FP32, the density is accumulated in int64 2^-32 fixed point,
// and the Poisson GEMMs accumulate with chunked compensation.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace tgp {

constexpr int kThreads = 256;            // every stage runs 256-thread blocks
constexpr int kMaxFields = 4;
constexpr float kFixF = 4294967296.0f;   // density fixed point: 2^32 per unit charge
constexpr double kFix = 4294967296.0;
constexpr double kInvFix = 1.0 / 4294967296.0;
constexpr float kInvFixF = 1.0f / 4294967296.0f;
constexpr int kMaxClasses = 7;           // WA degree classes

// Reduction slots (per-block partials, reduced in a fixed order).
enum Slot {
  SLOT_WA_VALUE = 0,
  SLOT_ENERGY = 1,                       // + field
  SLOT_FORCE = SLOT_ENERGY + kMaxFields, // + field
  SLOT_RAWL1 = SLOT_FORCE + kMaxFields,  // + field
  SLOT_WAL1 = SLOT_RAWL1 + kMaxFields,
  SLOT_DOT,
  SLOT_MSN,
  SLOT_HPWL,
  kSlots
};
constexpr int kMaxPartials = 2048;       // partials per slot

struct Grid {
  int W, H;          // tile grid
  int Wb, Hb;        // density (bin) grid
  float sx, sy;      // bins per tile
  int identity;      // 1 when the bin grid is the tile grid
};

// Device view of one placement instance. All arrays are device pointers.
struct Dev {
  int U, F, nobj, K, Mm, B;
  Grid g;
  const float2* binmap_x;    // [W] bin coordinate of each tile centre as hi+lo floats
  const float2* binmap_y;    // [H]
  // density members (flattened) and fillers
  const int* mem_unit;
  const float2* mem_off;
  const float* mem_q;
  const int* mem_field;
  const int* unit_mem_ptr;   // [U+1]
  const int* fil_field;      // [F]
  const float* fil_q;        // [F]
  // WA nets (timed arcs appended as weighted 2-pin nets), grouped by degree class
  int n_classes;
  int class_begin[kMaxClasses + 1];
  int class_group[kMaxClasses];
  // lanes of a V-virtual-block launch given to each class, warp-aligned
  // prefix offsets: the classes run side by side, not one after another
  int class_lane[kMaxClasses + 1];
  const int* net_ptr;        // [E+1]
  const int* pin_unit;       // [P] -1 for fixed cells
  const float2* pin_base;    // [P] fixed coordinate or cell offset
  const float* net_w;        // [E]
  int n_hpwl_nets;           // the first nets are the baseline hypernets
  // grids
  long long* phys;           // [K][B] members - smoothed capacity
  long long* fill;           // [K][B] fillers
  const long long* capfix;   // [K][B] smoothed capacity (fixed point)
  const long long* capsum;   // [K] sum of capfix
  float* rho;                // [K][B]
  float* t1;                 // [K][B]
  float* t2;                 // [K][B]
  float* phi;                // [K][B]
  const float* Cx;  const float* CxT;   // [Wb][Wb]
  const float* Cy;  const float* CyT;   // [Hb][Hb]
  const float* inv_eig;      // [B]
  // Tensor-core DCT (dct_tc.cuh): every GEMM operand is kept as four bf16
  // integer slices in the tile layout the tensor cores read, with one
  // power-of-two scale per operand row. A operands (rows x K) in 128 x 32
  // blocks, B operands (output columns x K) in 64 x 32 blocks, zero-padded;
  // opA holds rho then t3 (H x W), opB t1 then t2 (W x H); the bases are
  // shared read-only tables.
  int tc;                    // 1: the DCT passes run on tcgen05 tensor cores
  int dct_large;             // FP32 GEMM form: 1 = 64x64 register-blocked tiles, 0 = 16x16 slab tiles
  // FFT form (power-of-two grids): twiddle tables per axis (dct_fft.cuh)
  int fft;                   // 1: the DCT passes run as FFT-based transforms
  int logW, logH;
  const float4 *fx_tw, *fx_post, *fx_pre;   // FFT tables as double-float pairs
  const float2* fx_inv_s;
  const float4 *fy_tw, *fy_post, *fy_pre;
  const float2* fy_inv_s;
  int Hp128, Hp32, Wp64, Wp32;   // padded extents
  uint16_t *opA, *opB;           // dynamic operands (all fields)
  int *eA, *eB;                  // their row exponents [K][Hp128], [K][Wp64]
  float2* tp;                    // [K][B] pass output as double-float pairs (aliases t1)
  unsigned* tmx;                 // [2][K][Wb] column maxima of t1, t2 (float bits of |x|)
  const uint16_t *CxB_t, *CyA_t, *CyTA_t, *CxTB_t;
  const int *eCx, *eCy;          // basis row exponents: [n] rows of C, then [n] rows of C^T
  const float* inv_eig_lo;       // [B] low part of 1 / lambda
  // Tiled scatter (scatter_tiles.cuh, host engine): objects counting-sorted by
  // (grid, 32 x 32-bin tile of their centre bin), then deposited through a
  // shared-memory window per run of the sorted order
  int scatter_tiles;         // 1: the density scatter runs in the tiled form
  int *bin_key, *bin_rank, *bin_order;   // [Mm + F]
  int *bin_cnt, *bin_off;    // [2 K tiles], [2 K tiles + 1]
  // gradients
  unsigned long long* wa_fix;  // [2U] WA gradient, 2^-32 fixed point
  float2* graw;              // [K][nobj] raw per-field density gradient
  // optimizer
  const float2* lo;
  const float2* hi;
  float* P;                  // [nobj] preconditioner
  const float* pre_static;   // [nobj]
  const float* pre_q;        // [K][nobj]
};

// ---- B-spline stencil (bit-exact with the oracle's fixed-point restatement)
struct AxisTaps {
  int idx[3];
  float w[3];
  float o;
};

// quadratic_bspline_axis (electrostatic_placement.rs:950-976) for an FP32
// coordinate: clamp to [0, n-1], centre min(floor(c + 1/2), n-1), offset
// o = c - centre (exact in FP32), weights (1/2(1/2-o)^2, 3/4-o^2,
// 1/2(1/2+o)^2), out-of-range taps folded onto the edge. For a bin grid that
// differs from the tile grid the bin coordinate (s + 1/2) * scale - 1/2 is
// formed from the tile's tabulated FP64 value split into hi + lo floats plus
// the sub-tile fraction times scale, so o keeps ~1e-7 absolute accuracy.
__device__ __forceinline__ AxisTaps axis_taps(int n, float s, const float2* __restrict__ map, float scale,
                                              int identity, int tiles) {
  AxisTaps t;
  const float maximum = (float)(n - 1);
  float hi, lo;
  if (identity) {
    hi = s;
    lo = 0.f;
  } else {
    float ts = rintf(s);
    ts = ts > 0.f ? ts : 0.f;                        // NaN lands on tile 0
    ts = ts < (float)(tiles - 1) ? ts : (float)(tiles - 1);
    const float2 b = map[(int)ts];
    hi = b.x;
    lo = __fadd_rn(b.y, __fmul_rn(__fsub_rn(s, ts), scale));
  }
  const float c = __fadd_rn(hi, lo);
  int center;
  float o;
  if (!(c > 0.f)) {          // also catches NaN
    center = 0;
    o = 0.f;
  } else if (c >= maximum) {
    center = n - 1;
    o = 0.f;
  } else {
    const float cc = fminf(floorf(__fadd_rn(c, 0.5f)), maximum);
    center = (int)cc;
    o = __fadd_rn(__fsub_rn(hi, cc), lo);
  }
  const float a = __fsub_rn(0.5f, o), b = __fadd_rn(0.5f, o);
  t.idx[0] = center == 0 ? 0 : center - 1;
  t.idx[1] = center;
  t.idx[2] = center + 1 < n ? center + 1 : n - 1;
  t.w[0] = __fmul_rn(0.5f, __fmul_rn(a, a));
  t.w[1] = __fsub_rn(0.75f, __fmul_rn(o, o));
  t.w[2] = __fmul_rn(0.5f, __fmul_rn(b, b));
  t.o = o;
  return t;
}

__device__ __forceinline__ long long tap_fixed(float q, float wx, float wy) {
  return __float2ll_rn(__fmul_rn(__fmul_rn(__fmul_rn(q, wx), wy), kFixF));
}

// ---- block reductions (fixed order within a block) --------------------------
template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// FP64 arithmetic issues at a low rate on this part (a warp instruction
// occupies a sub-partition's FP64 pipe for tens of cycles), so block-level
// FP64 folds keep the work in as few warp instructions per sub-partition as
// the tree allows: the values go through shared memory, warps 0-3 (one per
// sub-partition) each fold an interleaved quarter with an xor tree, and
// thread 0 folds the four results. `sh` needs kThreads + 4 slots; the result
// is valid in thread 0. The order is fixed, so every block folds alike.
template <typename Op>
__device__ __forceinline__ double block_fold_fp64(double v, double* sh, Op op) {
  __syncthreads();   // earlier readers of sh are done
  sh[threadIdx.x] = v;
  __syncthreads();
  const int w = threadIdx.x >> 5;
  if (w < 4) {
    double s = sh[threadIdx.x];
    for (int i = threadIdx.x + 128; i < (int)blockDim.x; i += 128) s = op(s, sh[i]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s = op(s, __shfl_xor_sync(0xffffffffu, s, o));
    if ((threadIdx.x & 31) == 0) sh[kThreads + w] = s;
  }
  __syncthreads();
  return threadIdx.x == 0 ? op(op(op(sh[kThreads], sh[kThreads + 1]), sh[kThreads + 2]), sh[kThreads + 3]) : 0.0;
}
struct FoldAdd {
  __device__ double operator()(double a, double b) const { return a + b; }
};
__device__ __forceinline__ double block_sum(double v, double* sh) { return block_fold_fp64(v, sh, FoldAdd()); }

// Sum over the block; result valid in thread 0. `sh` needs kThreads/32 slots.
template <typename T>
__device__ __forceinline__ T block_sum(T v, T* sh) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  T r = 0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) r += sh[i];
  return r;
}

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

}  // namespace tgp
