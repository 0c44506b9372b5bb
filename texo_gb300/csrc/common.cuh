// common.cuh — shared device layout and arithmetic of the placement engine.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace tgp {

constexpr int kThreads = 256;            // every stage runs 256-thread blocks
constexpr int kMaxFields = 4;
constexpr float kFixF = 4294967296.0f;   // density fixed point: 2^32 per unit charge
constexpr double kFix = 4294967296.0;
constexpr double kInvFix = 1.0 / 4294967296.0;
constexpr int kMaxClasses = 6;           // WA degree classes

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

// Integer counters (exact; order-independent atomics).
enum Counter {
  CNT_GRID_SUM = 0,                      // + field: sum of all density taps (int64)
  CNT_OVERFLOW = CNT_GRID_SUM + kMaxFields,   // + field: sum max(phys,0) (int64)
  CNT_OVER_BINS = CNT_OVERFLOW + kMaxFields,  // + field
  CNT_DIFF = CNT_OVER_BINS + kMaxFields,      // coordinates that differ
  CNT_BAD_GRAD,                          // first non-finite gradient coordinate (min)
  CNT_KKT,                               // max KKT component (double bits)
  CNT_CHANGE,                            // max |delta| (double bits)
  CNT_PMIN, CNT_PMAX,                    // preconditioner range (double bits)
  kCounters
};

struct Grid {
  int W, H;          // tile grid
  int Wb, Hb;        // density (bin) grid
  double sx, sy;     // bins per tile
  int identity;      // 1 when the bin grid is the tile grid
};

// Device view of one placement instance. All arrays are device pointers.
struct Dev {
  int U, F, nobj, K, Mm, B;
  Grid g;
  // density members (flattened) and fillers
  const int* mem_unit;
  const double2* mem_off;
  const float* mem_q;
  const int* mem_field;
  const int* unit_mem_ptr;   // [U+1]
  const int* fil_field;      // [F]
  const float* fil_q;        // [F]
  // WA nets (timed arcs appended as weighted 2-pin nets), grouped by degree class
  int n_classes;
  int class_begin[kMaxClasses + 1];
  int class_group[kMaxClasses];
  const int* net_ptr;        // [E+1]
  const int* pin_unit;       // [P] -1 for fixed cells
  const double2* pin_base;   // [P] fixed coordinate or cell offset
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
  // gradients
  unsigned long long* wa_fix;  // [2U] WA gradient, 2^-32 fixed point
  float2* graw;              // [K][nobj] raw per-field density gradient
  // optimizer
  const double2* lo;
  const double2* hi;
  double* P;                 // [nobj] preconditioner
  const double* pre_static;  // [nobj]
  const double* pre_q;       // [K][nobj]
  // reductions
  double* partials;          // [kSlots][kMaxPartials]
  unsigned long long* counters;  // [kCounters]
  double* scal;              // scalars written by finalize kernels
};

// ---- B-spline stencil, device arithmetic (bit-exact with the CPU restatement)
__device__ __forceinline__ double to_bin(double s, double scale, int identity) {
  return identity ? s : __dsub_rn(__dmul_rn(__dadd_rn(s, 0.5), scale), 0.5);
}

struct AxisTaps {
  int idx[3];
  float w[3];
  float o;
};

// quadratic_bspline_axis (electrostatic_placement.rs:950-976) with the offset
// and weights in FP32: c is clamped, the centre is min(floor(c+1/2), n-1) and
// out-of-range taps fold onto the edge.
__device__ __forceinline__ AxisTaps axis_taps(int n, double c) {
  AxisTaps t;
  const double maximum = (double)(n - 1);
  // NaN compares false and lands on 0, so every index stays inside the grid.
  c = c > 0.0 ? c : 0.0;
  c = c < maximum ? c : maximum;
  const double cc = fmin(floor(__dadd_rn(c, 0.5)), maximum);
  int center = (int)cc;
  center = center < 0 ? 0 : (center > n - 1 ? n - 1 : center);
  const float o = __double2float_rn(__dsub_rn(c, cc));
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

__device__ __forceinline__ unsigned long long dbits(double v) {
  return (unsigned long long)__double_as_longlong(v);
}

// ---- block reductions (fixed order within a block) --------------------------
template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

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
