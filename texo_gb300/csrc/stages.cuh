// stages.cuh — the placement engine's stages as block-level device functions.
//
// Every stage takes a virtual block index `vb` out of `nvb` and strides over
// its items, so the same code runs as a standalone kernel (vb = blockIdx.x)
// and inside the persistent cooperative kernel between grid barriers.
// Reductions are written as one partial per virtual block and reduced in a
// fixed order, so every result is bit-for-bit deterministic.
#pragma once
#include "common.cuh"
#include "dct_tc.cuh"

namespace tgp {

// Integer partial slots.
enum ISlot {
  IS_GRID_SUM = 0,                        // + field
  IS_OVERFLOW = IS_GRID_SUM + kMaxFields, // + field
  IS_OVER_BINS = IS_OVERFLOW + kMaxFields,
  IS_DIFF = IS_OVER_BINS + kMaxFields,
  IS_BAD = IS_DIFF + 1,                   // min index of a non-finite gradient
  IS_PBAD,                                // any invalid preconditioner entry
  kISlots
};
// Max/min partial slots (doubles).
enum MSlot { MS_KKT = 0, MS_CHANGE, MS_PMIN, MS_PMAX, kMSlots };

struct Partials {
  double* sum;        // [kSlots][kMaxPartials]
  long long* isum;    // [kISlots][kMaxPartials]
  double* mx;         // [kMSlots][kMaxPartials]
};

__device__ __forceinline__ double* pslot(const Partials& p, int s) { return p.sum + (size_t)s * kMaxPartials; }
__device__ __forceinline__ long long* islot(const Partials& p, int s) { return p.isum + (size_t)s * kMaxPartials; }
__device__ __forceinline__ double* mslot(const Partials& p, int s) { return p.mx + (size_t)s * kMaxPartials; }

// Fixed-order reduction of n partials by the whole block; every thread gets
// the result. Identical in every block that calls it. Warps 0-3 (one per SM
// sub-partition) fold interleaved quarters with an xor tree and thread 0
// folds the four: FP64 folds then cost a few warp instructions per
// sub-partition instead of a tree in every warp. `sh` needs 5 slots.
template <typename T, typename Op>
__device__ __forceinline__ T block_reduce_array(const T* a, int n, T init, Op op, T* sh) {
  const int w = threadIdx.x >> 5;
  if (w < 4) {
    T v = (int)threadIdx.x < n ? a[threadIdx.x] : init;
    for (int i = threadIdx.x + 128; i < n; i += 128) v = op(v, a[i]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = op(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) sh[w] = v;
  }
  __syncthreads();
  if (threadIdx.x == 0) sh[4] = op(op(op(sh[0], sh[1]), sh[2]), sh[3]);
  __syncthreads();
  const T r = sh[4];
  __syncthreads();
  return r;
}
struct OpAdd {
  template <typename T> __device__ T operator()(T a, T b) const { return a + b; }
};
struct OpMax {
  __device__ double operator()(double a, double b) const { return fmax(a, b); }
};
struct OpMin {
  __device__ double operator()(double a, double b) const { return fmin(a, b); }
  __device__ long long operator()(long long a, long long b) const { return a < b ? a : b; }
};

// Block sum of a per-thread value, written as partial vb (thread 0).
template <typename T>
__device__ __forceinline__ void write_partial(T v, T* slot, int vb, T* sh) {
  T r = block_sum(v, sh);
  if (threadIdx.x == 0) slot[vb] = r;
}
struct FoldMax {
  __device__ double operator()(double a, double b) const { return fmax(a, b); }
};
struct FoldMin {
  __device__ double operator()(double a, double b) const { return fmin(a, b); }
};
// Block max (or min) of per-thread FP32 values, written as FP64 partial vb:
// folding in FP32 and widening once gives the same value as widening first.
__device__ __forceinline__ void write_partial_max(float v, double* slot, int vb, float* sh, bool is_min) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float w = __shfl_xor_sync(0xffffffffu, v, o);
    v = is_min ? fminf(v, w) : fmaxf(v, w);
  }
  __syncthreads();   // earlier readers of sh are done
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    float r = sh[0];
    for (int i = 1; i < (int)(blockDim.x >> 5); ++i) r = is_min ? fminf(r, sh[i]) : fmaxf(r, sh[i]);
    slot[vb] = (double)r;
  }
}

struct Shared {
  double d[kThreads + 4];   // block FP64 folds
  long long l[kThreads / 32];
  float f[kThreads / 32];   // block FP32 max / min
};

__device__ __forceinline__ AxisTaps taps_x(const Dev& d, float s) {
  return axis_taps(d.g.Wb, s, d.binmap_x, d.g.sx, d.g.identity, d.g.W);
}
__device__ __forceinline__ AxisTaps taps_y(const Dev& d, float s) {
  return axis_taps(d.g.Hb, s, d.binmap_y, d.g.sy, d.g.identity, d.g.H);
}

// ---------------------------------------------------------------------------
// S1: reset the accumulation grids.
// ---------------------------------------------------------------------------
static __device__ void stage_init(const Dev& d, int vb, int nvb, bool grids, bool wa) {
  const int stride = nvb * blockDim.x;
  const int t0 = vb * blockDim.x + threadIdx.x;
  if (grids) {
    const int n = d.K * d.B;
    for (int i = t0; i < n; i += stride) {
      d.phys[i] = -d.capfix[i];
      d.fill[i] = 0;
    }
  }
  if (wa)
    for (int i = t0; i < 2 * d.U; i += stride) d.wa_fix[i] = 0ull;
}

// ---------------------------------------------------------------------------
// S2: density scatter. Members deposit into phys (after the capacity
// background), fillers into fill; int64 2^-32 fixed point makes the sum
// exact in any order. The per-field tap total is a partial for the mean.
// (deposit_quadratic_bspline + the field loop, electrostatic_placement.rs:296-332)
// ---------------------------------------------------------------------------
static __device__ void stage_scatter(const Dev& d, const float2* pos, Partials p, int vb, int nvb,
                                     Shared& sh) {
  long long tot[kMaxFields];
#pragma unroll
  for (int f = 0; f < kMaxFields; ++f) tot[f] = 0;
  const int stride = nvb * blockDim.x;
  const int items = d.Mm + d.F;
  for (int i = vb * blockDim.x + threadIdx.x; i < items; i += stride) {
    float sxp, syp, q;
    int f;
    unsigned long long* grid;
    if (i < d.Mm) {
      const int u = d.mem_unit[i];
      const float2 o = d.mem_off[i];
      const float2 pu = pos[u];
      sxp = __fadd_rn(pu.x, o.x);
      syp = __fadd_rn(pu.y, o.y);
      q = d.mem_q[i];
      f = d.mem_field[i];
      grid = (unsigned long long*)(d.phys + (size_t)f * d.B);
    } else {
      const int j = i - d.Mm;
      const float2 pf = pos[d.U + j];
      sxp = pf.x;
      syp = pf.y;
      q = d.fil_q[j];
      f = d.fil_field[j];
      grid = (unsigned long long*)(d.fill + (size_t)f * d.B);
    }
    const AxisTaps ax = taps_x(d, sxp);
    const AxisTaps ay = taps_y(d, syp);
    long long s = 0;
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const long long v = tap_fixed(q, ax.w[c], ay.w[r]);
        s += v;
        atomicAdd(grid + (size_t)ay.idx[r] * d.g.Wb + ax.idx[c], (unsigned long long)v);
      }
#pragma unroll
    for (int ff = 0; ff < kMaxFields; ++ff)
      if (ff == f) tot[ff] += s;
  }
  for (int f = 0; f < d.K; ++f) write_partial(tot[f], islot(p, IS_GRID_SUM + f), vb, sh.l);
}

// ---------------------------------------------------------------------------
// S3: weighted-average wirelength (analytical_placement.rs:576-703).
// A group of G lanes takes one net: hard max/min by shuffles, exponential
// weights of the deltas to the extrema, soft means, per-pin derivative.
// Unit gradients accumulate as int64 2^-32 fixed point (order-independent).
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 pin_xy(const Dev& d, const float2* pos, int k) {
  const int u = d.pin_unit[k];
  const float2 b = d.pin_base[k];
  if (u < 0) return b;
  const float2 pu = pos[u];
  return make_float2(pu.x + b.x, pu.y + b.y);
}

// `slot` is this lane's index within the class's lane segment of `seg`
// lanes (both multiples of 32 at the segment start, so a group never
// straddles a warp and every lane of a warp makes the same passes). Lane l
// of a group takes pins p0 + l, p0 + l + G, ...; the first kWaPins of them
// stay in registers across the three passes (their loads are issued
// together), any further ones are read again.
constexpr int kWaPins = 4;
template <int G>
__device__ __forceinline__ void wa_class(const Dev& d, const float2* pos, float inv_gamma, int nb,
                                         int ne, int slot, int seg, double& acc) {
  const int lane = slot & (G - 1);
  const int group = slot / G;
  const int groups = seg / G;
  const unsigned mask = 0xffffffffu;
  const int count = ne - nb;
  float vacc = 0.f;
  for (int base = 0; base < count; base += groups) {
    const int e = nb + base + group;
    const bool active = base + group < count;
    int p0 = 0, p1 = 0;
    float w = 0.f;
    if (active) {
      p0 = d.net_ptr[e];
      p1 = d.net_ptr[e + 1];
      w = d.net_w[e];
    }
    // pass 1: this lane's pins and the hard extrema per axis
    float2 pv[kWaPins];
    int pu[kWaPins];
#pragma unroll
    for (int j = 0; j < kWaPins; ++j) {
      const int k = p0 + lane + j * G;
      pu[j] = k < p1 ? d.pin_unit[k] : -2;   // -2: no pin, -1: fixed pin
      pv[j] = k < p1 ? d.pin_base[k] : make_float2(0.f, 0.f);
    }
    float mx = -INFINITY, mnx = INFINITY, my = -INFINITY, mny = INFINITY;
#pragma unroll
    for (int j = 0; j < kWaPins; ++j) {
      if (pu[j] == -2) continue;
      if (pu[j] >= 0) {
        const float2 q = pos[pu[j]];
        pv[j] = make_float2(q.x + pv[j].x, q.y + pv[j].y);
      }
      mx = fmaxf(mx, pv[j].x);
      mnx = fminf(mnx, pv[j].x);
      my = fmaxf(my, pv[j].y);
      mny = fminf(mny, pv[j].y);
    }
    for (int k = p0 + lane + kWaPins * G; k < p1; k += G) {
      const float2 v = pin_xy(d, pos, k);
      mx = fmaxf(mx, v.x);
      mnx = fminf(mnx, v.x);
      my = fmaxf(my, v.y);
      mny = fminf(mny, v.y);
    }
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) {
      mx = fmaxf(mx, __shfl_xor_sync(mask, mx, o, G));
      mnx = fminf(mnx, __shfl_xor_sync(mask, mnx, o, G));
      my = fmaxf(my, __shfl_xor_sync(mask, my, o, G));
      mny = fminf(mny, __shfl_xor_sync(mask, mny, o, G));
    }
    // pass 2: exponential weights (exactly 1 at the extremum) and their sums
    float sw[4] = {0.f, 0.f, 0.f, 0.f}, sd[4] = {0.f, 0.f, 0.f, 0.f};
    auto weigh = [&](float2 v) {
      const float dxp = v.x - mx, dxn = v.x - mnx, dyp = v.y - my, dyn = v.y - mny;
      const float wxp = expf(dxp * inv_gamma), wxn = expf(-dxn * inv_gamma);
      const float wyp = expf(dyp * inv_gamma), wyn = expf(-dyn * inv_gamma);
      sw[0] += wxp; sd[0] = fmaf(wxp, dxp, sd[0]);
      sw[1] += wxn; sd[1] = fmaf(wxn, dxn, sd[1]);
      sw[2] += wyp; sd[2] = fmaf(wyp, dyp, sd[2]);
      sw[3] += wyn; sd[3] = fmaf(wyn, dyn, sd[3]);
    };
#pragma unroll
    for (int j = 0; j < kWaPins; ++j)
      if (pu[j] != -2) weigh(pv[j]);
    for (int k = p0 + lane + kWaPins * G; k < p1; k += G) weigh(pin_xy(d, pos, k));
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1)
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        sw[a] += __shfl_xor_sync(mask, sw[a], o, G);
        sd[a] += __shfl_xor_sync(mask, sd[a], o, G);
      }
    if (!active) continue;
    float mean[4], inv[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      inv[a] = 1.f / sw[a];
      mean[a] = sd[a] * inv[a];
    }
    // pass 3: per-pin derivative into the fixed-point unit gradient
    auto derive = [&](int u, float2 v) {
      const float dxp = v.x - mx, dxn = v.x - mnx, dyp = v.y - my, dyn = v.y - mny;
      const float wxp = expf(dxp * inv_gamma), wxn = expf(-dxn * inv_gamma);
      const float wyp = expf(dyp * inv_gamma), wyn = expf(-dyn * inv_gamma);
      const float gx = wxp * inv[0] * (1.f + (dxp - mean[0]) * inv_gamma) -
                       wxn * inv[1] * (1.f - (dxn - mean[1]) * inv_gamma);
      const float gy = wyp * inv[2] * (1.f + (dyp - mean[2]) * inv_gamma) -
                       wyn * inv[3] * (1.f - (dyn - mean[3]) * inv_gamma);
      atomicAdd(d.wa_fix + 2 * u, (unsigned long long)__float2ll_rn(w * gx * kFixF));
      atomicAdd(d.wa_fix + 2 * u + 1, (unsigned long long)__float2ll_rn(w * gy * kFixF));
    };
#pragma unroll
    for (int j = 0; j < kWaPins; ++j)
      if (pu[j] >= 0) derive(pu[j], pv[j]);
    for (int k = p0 + lane + kWaPins * G; k < p1; k += G) {
      const int u = d.pin_unit[k];
      if (u >= 0) derive(u, pin_xy(d, pos, k));
    }
    if (lane == 0) vacc += w * (((mx - mnx) + mean[0] - mean[1]) + ((my - mny) + mean[2] - mean[3]));
  }
  acc += (double)vacc;
}

static __device__ void stage_wa(const Dev& d, const float2* pos, double gamma, Partials p, int vb,
                                int nvb, Shared& sh) {
  double acc = 0.0;
  const float ig = (float)(1.0 / gamma);
  const int gl = vb * blockDim.x + threadIdx.x;
  int c = 0;
  while (c < d.n_classes && gl >= d.class_lane[c + 1]) ++c;
  if (c < d.n_classes) {
    const int nb = d.class_begin[c], ne = d.class_begin[c + 1];
    const int slot = gl - d.class_lane[c], seg = d.class_lane[c + 1] - d.class_lane[c];
    if (ne > nb && seg > 0) {
      switch (d.class_group[c]) {
        case 1: wa_class<1>(d, pos, ig, nb, ne, slot, seg, acc); break;
        case 2: wa_class<2>(d, pos, ig, nb, ne, slot, seg, acc); break;
        case 4: wa_class<4>(d, pos, ig, nb, ne, slot, seg, acc); break;
        case 8: wa_class<8>(d, pos, ig, nb, ne, slot, seg, acc); break;
        default: wa_class<32>(d, pos, ig, nb, ne, slot, seg, acc); break;
      }
    }
  }
  write_partial(acc, pslot(p, SLOT_WA_VALUE), vb, sh.d);
}

// ---------------------------------------------------------------------------
// S4: density grid -> FP32 mean-free charge, physical overflow partials
// (the pre-filler positive overflow, electrostatic_placement.rs:317-318).
// ---------------------------------------------------------------------------
static __device__ void stage_prep(const Dev& d, Partials p, int nvb_scatter, int vb, int nvb, Shared& sh) {
  __shared__ long long s_mean[kMaxFields];
  __shared__ long long red[kThreads / 32];
  for (int f = 0; f < d.K; ++f) {
    long long tot = block_reduce_array(islot(p, IS_GRID_SUM + f), nvb_scatter, 0ll, OpAdd(), red);
    if (threadIdx.x == 0) s_mean[f] = (tot - d.capsum[f]) / d.B;   // fixed-point mean (DC mode only)
  }
  __syncthreads();
  long long ov[kMaxFields], cnt[kMaxFields];
#pragma unroll
  for (int f = 0; f < kMaxFields; ++f) ov[f] = cnt[f] = 0;
  const int stride = nvb * blockDim.x;
  for (int f = 0; f < d.K; ++f) {
    const long long mean = s_mean[f];
    const long long* ph = d.phys + (size_t)f * d.B;
    const long long* fl = d.fill + (size_t)f * d.B;
    float* rho = d.rho + (size_t)f * d.B;
    for (int i = vb * blockDim.x + threadIdx.x; i < d.B; i += stride) {
      const long long a = ph[i];
      if (a > 0) {
        ov[f] += a;
        cnt[f] += 1;
      }
      rho[i] = __ll2float_rn(a + fl[i] - mean) * kInvFixF;
    }
  }
  for (int f = 0; f < d.K; ++f) {
    write_partial(ov[f], islot(p, IS_OVERFLOW + f), vb, sh.l);
    write_partial(cnt[f], islot(p, IS_OVER_BINS + f), vb, sh.l);
  }
}

// ---------------------------------------------------------------------------
// S5: FP32 CUDA-core GEMM, C[MxN] = A[MxK] B[KxN], all row-major, for each
// of nf grids (A/B/C advance by their per-grid strides; 0 = shared matrix).
// Epilogue: 0 store; 1 store C * inv_eig; 2 store and accumulate
// <rho, C> into per-field energy partials.
// ---------------------------------------------------------------------------
template <int TM, int TN, int TK, int RM, int RN>
struct GemmSmem {
  float a[TK][TM + 1];
  float b[TK][TN + 4];
};

// Accumulation is compensated: plain FMAs within chunks of kChunk products,
// and each chunk sum enters a (sum, compensation) pair through an
// error-free TwoSum. The potential's low-frequency modes are small sums of
// large cancelling terms that 1/lambda then amplifies; plain FP32
// accumulation leaves ~1e-5 relative error in the field, the chunked
// compensation ~4e-6 (against the FP64 spectral solve).
constexpr int kChunk = 8;

__device__ __forceinline__ void two_sum_acc(float& s, float& c, float part) {
  const float t = __fadd_rn(s, part);
  const float z = __fsub_rn(t, s);
  const float e = __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(part, z));
  s = t;
  c = __fadd_rn(c, e);
}

template <int TM, int TN, int TK, int RM, int RN>
__device__ void gemm_tiles(const float* A, long sa, const float* Bm, long sb, float* Cm, long sc, int M, int N,
                           int Kd, int nf, int epi, const float* inv_eig, const float* rho, double* energy_acc,
                           int vb, int nvb, GemmSmem<TM, TN, TK, RM, RN>& sm) {
  static_assert((TM / RM) * (TN / RN) == kThreads, "tile / thread mismatch");
  static_assert(TK % kChunk == 0, "k slab must hold whole chunks");
  constexpr int TX = TN / RN;
  constexpr int LA = TM * TK / kThreads, LB = TK * TN / kThreads;  // loads per thread per slab
  const int tx = threadIdx.x % TX, ty = threadIdx.x / TX;
  const int tiles_m = (M + TM - 1) / TM, tiles_n = (N + TN - 1) / TN;
  const int tiles = tiles_m * tiles_n * nf;
  for (int t = vb; t < tiles; t += nvb) {
    const int f = t / (tiles_m * tiles_n);
    const int r = t % (tiles_m * tiles_n);
    const int m0 = (r / tiles_n) * TM, n0 = (r % tiles_n) * TN;
    const float* Af = A + f * sa;
    const float* Bf = Bm + f * sb;
    float sum[RM][RN], comp[RM][RN];
#pragma unroll
    for (int i = 0; i < RM; ++i)
#pragma unroll
      for (int j = 0; j < RN; ++j) sum[i][j] = comp[i][j] = 0.f;
    // register prefetch of the next slab overlaps global latency with math
    float ra[LA], rb[LB];
    auto fetch = [&](int k0) {
#pragma unroll
      for (int q = 0; q < LA; ++q) {
        const int e = threadIdx.x + q * kThreads;
        const int mm = e / TK, kk = e % TK;
        const int gm = m0 + mm, gk = k0 + kk;
        ra[q] = (gm < M && gk < Kd) ? Af[(size_t)gm * Kd + gk] : 0.f;
      }
#pragma unroll
      for (int q = 0; q < LB; ++q) {
        const int e = threadIdx.x + q * kThreads;
        const int kk = e / TN, nn = e % TN;
        const int gk = k0 + kk, gn = n0 + nn;
        rb[q] = (gk < Kd && gn < N) ? Bf[(size_t)gk * N + gn] : 0.f;
      }
    };
    fetch(0);
    for (int k0 = 0; k0 < Kd; k0 += TK) {
      __syncthreads();
#pragma unroll
      for (int q = 0; q < LA; ++q) {
        const int e = threadIdx.x + q * kThreads;
        sm.a[e % TK][e / TK] = ra[q];
      }
#pragma unroll
      for (int q = 0; q < LB; ++q) {
        const int e = threadIdx.x + q * kThreads;
        sm.b[e / TN][e % TN] = rb[q];
      }
      __syncthreads();
      if (k0 + TK < Kd) fetch(k0 + TK);
#pragma unroll
      for (int kc = 0; kc < TK; kc += kChunk) {
        float part[RM][RN];
#pragma unroll
        for (int i = 0; i < RM; ++i)
#pragma unroll
          for (int j = 0; j < RN; ++j) part[i][j] = 0.f;
#pragma unroll
        for (int kk = kc; kk < kc + kChunk; ++kk) {
          float av[RM], bv[RN];
#pragma unroll
          for (int i = 0; i < RM; ++i) av[i] = sm.a[kk][ty * RM + i];
#pragma unroll
          for (int j = 0; j < RN; ++j) bv[j] = sm.b[kk][tx * RN + j];
#pragma unroll
          for (int i = 0; i < RM; ++i)
#pragma unroll
            for (int j = 0; j < RN; ++j) part[i][j] = fmaf(av[i], bv[j], part[i][j]);
        }
#pragma unroll
        for (int i = 0; i < RM; ++i)
#pragma unroll
          for (int j = 0; j < RN; ++j) two_sum_acc(sum[i][j], comp[i][j], part[i][j]);
      }
    }
    float* Cf = Cm + f * sc;
    float eacc = 0.f;
#pragma unroll
    for (int i = 0; i < RM; ++i)
#pragma unroll
      for (int j = 0; j < RN; ++j) {
        const int gm = m0 + ty * RM + i, gn = n0 + tx * RN + j;
        if (gm < M && gn < N) {
          const size_t idx = (size_t)gm * N + gn;
          float v = __fadd_rn(sum[i][j], comp[i][j]);
          if (epi == 1) v *= inv_eig[idx];
          Cf[idx] = v;
          if (epi == 2) eacc = fmaf(rho[(size_t)f * M * N + idx], v, eacc);
        }
      }
    if (epi == 2) energy_acc[f] += (double)eacc;
  }
  __syncthreads();
}

// Small grids: 16x16 output tiles, one output per thread, K in slabs of
// 128 staged whole in shared memory. A 256x256 transform then has 256 tiles,
// enough to occupy every SM, where 32x32 tiles left most SMs idle.
constexpr int kT16Slab = 128;
constexpr int kT16Pad = kT16Slab + 4;   // float4-aligned rows; 8-thread phases stay conflict-free
struct Smem16 {
  float a[16][kT16Pad];    // A panel, rows m, k contiguous
  float bt[16][kT16Pad];   // B panel transposed, rows n, k contiguous
};

// Pass 0 of the spectral solve with the density preparation folded in: the
// A operand is formed while it is loaded, rho = (phys + fill - mean) 2^-32
// (the formula of stage_prep), and the tiles of the first column band, which
// load every bin exactly once, also store rho and count the physical
// overflow (per thread, one slot per field).
struct PrepFold {
  const long long* mean;   // [K] fixed-point mean per field
  long long ov[kMaxFields], cnt[kMaxFields];
};

template <bool FOLD = false>
static __device__ void gemm16(const float* A, long sa, const float* Bm, long sb, float* Cm, long sc, int M, int N,
                              int Kd, int nf, int epi, const float* inv_eig, const float* rho, double* energy_acc,
                              int vb, int nvb, Smem16& sm, const Dev* dp = nullptr, PrepFold* pf = nullptr) {
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int tiles_m = (M + 15) / 16, tiles_n = (N + 15) / 16;
  const int tiles = tiles_m * tiles_n * nf;
  // slab-load roles: A element (row ra + 2j, column ca), B element (row rb + 16j, column cb)
  const int ca = threadIdx.x & (kT16Slab - 1), ra = threadIdx.x / kT16Slab;
  const int cb = threadIdx.x & 15, rb = threadIdx.x >> 4;
  for (int t = vb; t < tiles; t += nvb) {
    const int f = t / (tiles_m * tiles_n);
    const int r = t % (tiles_m * tiles_n);
    const int m0 = (r / tiles_n) * 16, n0 = (r % tiles_n) * 16;
    const float* Af = A + f * sa;
    const float* Bf = Bm + f * sb;
    float sum = 0.f, comp = 0.f;
    float va[8], vbv[8];
    // slab k0 -> registers (the next slab's loads are issued before the
    // current slab's products, into the registers its smem copy freed)
    auto fetch = [&](int k0) {
      const int kn = min(kT16Slab, Kd - k0);
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int gm = m0 + ra + 2 * j;
        if (FOLD) {
          float v = 0.f;
          if (gm < M && ca < kn) {
            const size_t i = (size_t)f * dp->B + (size_t)gm * Kd + k0 + ca;
            const long long a = dp->phys[i];
            v = __ll2float_rn(a + dp->fill[i] - pf->mean[f]) * kInvFixF;
            if (n0 == 0) {
              dp->rho[i] = v;
              if (a > 0)
#pragma unroll
                for (int ff = 0; ff < kMaxFields; ++ff)
                  if (ff == f) {
                    pf->ov[ff] += a;
                    pf->cnt[ff] += 1;
                  }
            }
          }
          va[j] = v;
        } else {
          va[j] = (gm < M && ca < kn) ? Af[(size_t)gm * Kd + k0 + ca] : 0.f;
        }
        const int kk = rb + 16 * j, gn = n0 + cb;
        vbv[j] = (kk < kn && gn < N) ? Bf[(size_t)(k0 + kk) * N + gn] : 0.f;
      }
    };
    fetch(0);
    for (int k0 = 0; k0 < Kd; k0 += kT16Slab) {
      __syncthreads();
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        sm.a[ra + 2 * j][ca] = va[j];
        sm.bt[cb][rb + 16 * j] = vbv[j];
      }
      __syncthreads();
      if (k0 + kT16Slab < Kd) fetch(k0 + kT16Slab);
      const float4* a4 = reinterpret_cast<const float4*>(sm.a[ty]);
      const float4* b4 = reinterpret_cast<const float4*>(sm.bt[tx]);
#pragma unroll 4
      for (int kc = 0; kc < kT16Slab / 4; kc += kChunk / 4) {
        float part = 0.f;
#pragma unroll
        for (int q = 0; q < kChunk / 4; ++q) {
          const float4 x = a4[kc + q], y = b4[kc + q];
          part = fmaf(x.x, y.x, part);
          part = fmaf(x.y, y.y, part);
          part = fmaf(x.z, y.z, part);
          part = fmaf(x.w, y.w, part);
        }
        two_sum_acc(sum, comp, part);
      }
    }
    const int gm = m0 + ty, gn = n0 + tx;
    if (gm < M && gn < N) {
      const size_t idx = (size_t)gm * N + gn;
      float v = __fadd_rn(sum, comp);
      if (epi == 1) v *= inv_eig[idx];
      Cm[f * sc + idx] = v;
      if (epi == 2) energy_acc[f] += (double)(rho[(size_t)f * M * N + idx] * v);
    }
  }
  __syncthreads();
}

// Large-grid tile shape (register-blocked) and the small-grid one.
using SmemL = GemmSmem<64, 64, 16, 4, 4>;
union alignas(16) GemmShared {
  Smem16 s;
  SmemL l;
  float4 fft[2048];   // work buffer of the FFT form (fft::Smem: double-float complex)
};

template <bool LARGE>
__device__ __forceinline__ void gemm_any(const float* A, long sa, const float* Bm, long sb, float* Cm, long sc, int M,
                                         int N, int Kd, int nf, int epi, const float* inv_eig, const float* rho,
                                         double* eacc, int vb, int nvb, GemmShared& sm) {
  if (LARGE)
    gemm_tiles<64, 64, 16, 4, 4>(A, sa, Bm, sb, Cm, sc, M, N, Kd, nf, epi, inv_eig, rho, eacc, vb, nvb, sm.l);
  else
    gemm16(A, sa, Bm, sb, Cm, sc, M, N, Kd, nf, epi, inv_eig, rho, eacc, vb, nvb, sm.s);
}

// The four transforms of the spectral solve (Poisson2d::solve,
// electrostatic_placement.rs:725-776) as dense GEMMs:
//   t1 = rho Cx^T ; t2 = (Cy t1) o inv_eig ; t1 = Cy^T t2 ; phi = t1 Cx.
// `step` selects one of the four (a grid barrier separates them).
template <bool LARGE>
static __device__ void stage_dct_t(const Dev& d, int step, Partials p, int vb, int nvb, GemmShared& sm, Shared& sh) {
  const int W = d.g.Wb, H = d.g.Hb;
  const long sg = d.B;
  double eacc[kMaxFields] = {0.0, 0.0, 0.0, 0.0};
  switch (step) {
    case 0: gemm_any<LARGE>(d.rho, sg, d.CxT, 0, d.t1, sg, H, W, W, d.K, 0, nullptr, nullptr, eacc, vb, nvb, sm); break;
    case 1: gemm_any<LARGE>(d.Cy, 0, d.t1, sg, d.t2, sg, H, W, H, d.K, 1, d.inv_eig, nullptr, eacc, vb, nvb, sm); break;
    case 2: gemm_any<LARGE>(d.CyT, 0, d.t2, sg, d.t1, sg, H, W, H, d.K, 0, nullptr, nullptr, eacc, vb, nvb, sm); break;
    default: gemm_any<LARGE>(d.t1, sg, d.Cx, 0, d.phi, sg, H, W, W, d.K, 2, nullptr, d.rho, eacc, vb, nvb, sm); break;
  }
  if (step == 3)
    for (int f = 0; f < d.K; ++f) write_partial(eacc[f], pslot(p, SLOT_ENERGY + f), vb, sh.d);
}
// stage_prep + pass 0 of stage_dct_t<false> in one phase (small tiles only):
// the same rho, overflow sums and t1 as the two phases, bit for bit.
// `mean` holds the fixed-point mean of each field (from the scatter totals).
static __device__ void stage_prep_dct0(const Dev& d, const long long* mean, Partials p, int vb, int nvb,
                                       GemmShared& sm, Shared& sh) {
  const int W = d.g.Wb, H = d.g.Hb;
  const long sg = d.B;
  PrepFold pf;
  pf.mean = mean;
#pragma unroll
  for (int f = 0; f < kMaxFields; ++f) pf.ov[f] = pf.cnt[f] = 0;
  double eacc[kMaxFields] = {0.0, 0.0, 0.0, 0.0};
  gemm16<true>(nullptr, sg, d.CxT, 0, d.t1, sg, H, W, W, d.K, 0, nullptr, nullptr, eacc, vb, nvb, sm.s, &d, &pf);
  for (int f = 0; f < d.K; ++f) {
    write_partial(pf.ov[f], islot(p, IS_OVERFLOW + f), vb, sh.l);
    write_partial(pf.cnt[f], islot(p, IS_OVER_BINS + f), vb, sh.l);
  }
}
__device__ __forceinline__ void stage_dct(const Dev& d, int step, bool large, Partials p, int vb, int nvb,
                                          GemmShared& sm, Shared& sh) {
  if (large)
    stage_dct_t<true>(d, step, p, vb, nvb, sm, sh);
  else
    stage_dct_t<false>(d, step, p, vb, nvb, sm, sh);
}

// ---------------------------------------------------------------------------
// S6: field gather (sample_quadratic_bspline_with_gradient + the member and
// filler loops, electrostatic_placement.rs:338-374, 919-941): raw per-field
// gradient q * dphi per optimizer object, and force_l1 partials.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 sample_grad(const Dev& d, const float* phi, float sxp, float syp) {
  const AxisTaps ax = taps_x(d, sxp);
  const AxisTaps ay = taps_y(d, syp);
  const float dx[3] = {ax.o - 0.5f, -2.f * ax.o, ax.o + 0.5f};
  const float dy[3] = {ay.o - 0.5f, -2.f * ay.o, ay.o + 0.5f};
  // The derivative weights of each axis sum to zero, so the centre tap's
  // potential can be subtracted first: the FP32 sum then rounds relative to
  // the local potential differences, not to the potential itself.
  const float vc = phi[(size_t)ay.idx[1] * d.g.Wb + ax.idx[1]];
  float gx = 0.f, gy = 0.f;
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    const float* row = phi + (size_t)ay.idx[r] * d.g.Wb;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float v = row[ax.idx[c]] - vc;
      gx += dx[c] * ay.w[r] * v;
      gy += ax.w[c] * dy[r] * v;
    }
  }
  if (!d.g.identity) {
    gx *= d.g.sx;
    gy *= d.g.sy;
  }
  return make_float2(gx, gy);
}

static __device__ void stage_gather(const Dev& d, const float2* pos, Partials p, int vb, int nvb,
                                    Shared& sh) {
  float force[kMaxFields] = {0.f, 0.f, 0.f, 0.f};
  const int stride = nvb * blockDim.x;
  for (int o = vb * blockDim.x + threadIdx.x; o < d.nobj; o += stride) {
    if (o < d.U) {
      float2 acc[kMaxFields];
#pragma unroll
      for (int f = 0; f < kMaxFields; ++f) acc[f] = make_float2(0.f, 0.f);
      const int m0 = d.unit_mem_ptr[o], m1 = d.unit_mem_ptr[o + 1];
      const float2 pu = pos[o];
      for (int m = m0; m < m1; ++m) {
        const int f = d.mem_field[m];
        const float2 off = d.mem_off[m];
        const float q = d.mem_q[m];
        const float2 g = sample_grad(d, d.phi + (size_t)f * d.B, __fadd_rn(pu.x, off.x), __fadd_rn(pu.y, off.y));
#pragma unroll
        for (int ff = 0; ff < kMaxFields; ++ff)
          if (ff == f) {
            acc[ff].x += q * g.x;
            acc[ff].y += q * g.y;
            force[ff] += q * (fabsf(g.x) + fabsf(g.y));
          }
      }
      for (int f = 0; f < d.K; ++f) d.graw[(size_t)f * d.nobj + o] = acc[f];
    } else {
      const int j = o - d.U;
      const int f = d.fil_field[j];
      const float q = d.fil_q[j];
      const float2 pf = pos[o];
      const float2 g = sample_grad(d, d.phi + (size_t)f * d.B, pf.x, pf.y);
      d.graw[(size_t)f * d.nobj + o] = make_float2(q * g.x, q * g.y);
#pragma unroll
      for (int ff = 0; ff < kMaxFields; ++ff)
        if (ff == f) force[ff] += q * (fabsf(g.x) + fabsf(g.y));
    }
  }
  for (int f = 0; f < d.K; ++f) write_partial((double)force[f], pslot(p, SLOT_FORCE + f), vb, sh.d);
}

// ---------------------------------------------------------------------------
// S7: combined objective gradient (combined_objective, eplace.rs:1022-1044):
// g = grad WA + sum_f coef_f grad E_f, with the non-finite check and the L1
// norms the initial multiplier needs (eplace.rs:1126-1148).
// ---------------------------------------------------------------------------
__device__ __forceinline__ float kkt_comp(float g, float x, float lo, float hi) {
  if (__float_as_int(lo) == __float_as_int(hi) || (x <= lo && g > 0.f) || (x >= hi && g < 0.f)) return 0.f;
  return fabsf(g);
}

// With kkt_pos, the box-metric KKT residual of the new gradient at kkt_pos is
// reduced in the same pass (box_metric_kkt_residual, global_placement.rs:648-663).
static __device__ void stage_combine(const Dev& d, const double* coef_d, float2* gout, Partials p,
                                     int vb, int nvb, Shared& sh, const float2* kkt_pos = nullptr) {
  float coef[kMaxFields];
#pragma unroll
  for (int f = 0; f < kMaxFields; ++f) coef[f] = f < d.K ? (float)coef_d[f] : 0.f;
  float rawl1[kMaxFields] = {0.f, 0.f, 0.f, 0.f};
  float wal1 = 0.f, kkt = 0.f;
  long long bad = 0x7fffffffffffffffll;
  const int stride = nvb * blockDim.x;
  for (int o = vb * blockDim.x + threadIdx.x; o < d.nobj; o += stride) {
    float gx = 0.f, gy = 0.f;
    if (o < d.U) {
      gx = __ll2float_rn((long long)d.wa_fix[2 * o]) * kInvFixF;
      gy = __ll2float_rn((long long)d.wa_fix[2 * o + 1]) * kInvFixF;
      wal1 += fabsf(gx) + fabsf(gy);
      for (int f = 0; f < d.K; ++f) {
        const float2 r = d.graw[(size_t)f * d.nobj + o];
        gx = fmaf(coef[f], r.x, gx);
        gy = fmaf(coef[f], r.y, gy);
        rawl1[f] += fabsf(r.x) + fabsf(r.y);
      }
    } else {
      const int f = d.fil_field[o - d.U];
      const float2 r = d.graw[(size_t)f * d.nobj + o];
#pragma unroll
      for (int ff = 0; ff < kMaxFields; ++ff)
        if (ff == f) {
          gx = coef[ff] * r.x;
          gy = coef[ff] * r.y;
          rawl1[ff] += fabsf(r.x) + fabsf(r.y);
        }
    }
    if (!isfinite(gx)) bad = min(bad, (long long)(2 * o));
    else if (!isfinite(gy)) bad = min(bad, (long long)(2 * o + 1));
    gout[o] = make_float2(gx, gy);
    if (kkt_pos) {
      const float2 a = kkt_pos[o], lo = d.lo[o], hi = d.hi[o];
      const float s = rsqrtf(d.P[o]);
      kkt = fmaxf(kkt, kkt_comp(gx, a.x, lo.x, hi.x) * s);
      kkt = fmaxf(kkt, kkt_comp(gy, a.y, lo.y, hi.y) * s);
    }
  }
  for (int f = 0; f < d.K; ++f) write_partial((double)rawl1[f], pslot(p, SLOT_RAWL1 + f), vb, sh.d);
  write_partial((double)wal1, pslot(p, SLOT_WAL1), vb, sh.d);
  if (kkt_pos) write_partial_max(kkt, mslot(p, MS_KKT), vb, sh.f, false);
  {
    long long v = bad;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      long long w = __shfl_xor_sync(0xffffffffu, v, o);
      v = w < v ? w : v;
    }
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sh.l[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
      long long r = sh.l[0];
      for (int i = 1; i < (int)(blockDim.x >> 5); ++i) r = sh.l[i] < r ? sh.l[i] : r;
      islot(p, IS_BAD)[vb] = r;
    }
  }
}

// ---------------------------------------------------------------------------
// Nesterov vector stages (global_placement.rs:143-335, 588-712), FP32.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float fclamp(float v, float lo, float hi) { return v < lo ? lo : (v > hi ? hi : v); }

// y = clamp(x + e (x - prev)); counts coordinates where y != x.
static __device__ void stage_extrapolate(const Dev& d, const float2* x, const float2* xp,
                                         float e, float2* y, Partials p, int vb, int nvb, Shared& sh) {
  long long diff = 0;
  const int stride = nvb * blockDim.x;
  for (int o = vb * blockDim.x + threadIdx.x; o < d.nobj; o += stride) {
    const float2 a = x[o], b = xp[o], lo = d.lo[o], hi = d.hi[o];
    float2 r;
    r.x = fclamp(a.x + e * (a.x - b.x), lo.x, hi.x);
    r.y = fclamp(a.y + e * (a.y - b.y), lo.y, hi.y);
    diff += (r.x != a.x) + (r.y != a.y);
    y[o] = r;
  }
  write_partial(diff, islot(p, IS_DIFF), vb, sh.l);
}

// c = clamp(y - g / (L P)); changed count, <g, c - y>, sum P (c - y)^2.
// With origin, also the max coordinate change |c - origin|.
static __device__ void stage_candidate(const Dev& d, const float2* y, const float2* gy,
                                       float invL, float2* c, Partials p, int vb, int nvb, Shared& sh,
                                       const float2* origin = nullptr) {
  long long diff = 0;
  float dot = 0.f, msn = 0.f, ch = 0.f;
  const int stride = nvb * blockDim.x;
  for (int o = vb * blockDim.x + threadIdx.x; o < d.nobj; o += stride) {
    const float2 a = y[o], g = gy[o], lo = d.lo[o], hi = d.hi[o];
    const float m = d.P[o];
    const float s = invL / m;
    float2 r;
    r.x = fclamp(a.x - g.x * s, lo.x, hi.x);
    r.y = fclamp(a.y - g.y * s, lo.y, hi.y);
    diff += (r.x != a.x) + (r.y != a.y);
    const float dx = r.x - a.x, dy = r.y - a.y;
    dot = fmaf(g.x, dx, fmaf(g.y, dy, dot));
    msn = fmaf(m * dx, dx, fmaf(m * dy, dy, msn));
    c[o] = r;
    if (origin) {
      const float2 b = origin[o];
      ch = fmaxf(ch, fmaxf(fabsf(r.x - b.x), fabsf(r.y - b.y)));
    }
  }
  write_partial(diff, islot(p, IS_DIFF), vb, sh.l);
  write_partial((double)dot, pslot(p, SLOT_DOT), vb, sh.d);
  write_partial((double)msn, pslot(p, SLOT_MSN), vb, sh.d);
  if (origin) write_partial_max(ch, mslot(p, MS_CHANGE), vb, sh.f, false);
}

// box_metric_kkt_residual (global_placement.rs:648-663) and, optionally, the
// max coordinate change against `ref`.
static __device__ void stage_kkt(const Dev& d, const float2* x, const float2* g,
                                 const float2* ref, Partials p, int vb, int nvb, Shared& sh) {
  float r = 0.f, ch = 0.f;
  const int stride = nvb * blockDim.x;
  for (int o = vb * blockDim.x + threadIdx.x; o < d.nobj; o += stride) {
    const float2 a = x[o], gg = g[o], lo = d.lo[o], hi = d.hi[o];
    const float s = rsqrtf(d.P[o]);
    r = fmaxf(r, kkt_comp(gg.x, a.x, lo.x, hi.x) * s);
    r = fmaxf(r, kkt_comp(gg.y, a.y, lo.y, hi.y) * s);
    if (ref) {
      const float2 b = ref[o];
      ch = fmaxf(ch, fabsf(a.x - b.x));
      ch = fmaxf(ch, fabsf(a.y - b.y));
    }
  }
  write_partial_max(r, mslot(p, MS_KKT), vb, sh.f, false);
  if (ref) write_partial_max(ch, mslot(p, MS_CHANGE), vb, sh.f, false);
}

// diagonal_preconditioner (eplace.rs:1046-1100).
static __device__ void stage_precond(const Dev& d, const double* lambda_d, Partials p, int vb, int nvb, Shared& sh) {
  float lambda[kMaxFields];
#pragma unroll
  for (int f = 0; f < kMaxFields; ++f) lambda[f] = f < d.K ? (float)lambda_d[f] : 0.f;
  float pmin = INFINITY, pmax = 0.f;
  long long badp = 0;
  const int stride = nvb * blockDim.x;
  for (int o = vb * blockDim.x + threadIdx.x; o < d.nobj; o += stride) {
    float v = d.pre_static[o];
    for (int f = 0; f < d.K; ++f) {
      const float q = d.pre_q[(size_t)f * d.nobj + o];
      if (q == 0.f) continue;
      v = fmaf(lambda[f], q, v);
    }
    if (!isfinite(v) || v < 0.f) badp = 1;
    v = fmaxf(v, 1.f);
    d.P[o] = v;
    pmin = fminf(pmin, v);
    pmax = fmaxf(pmax, v);
  }
  write_partial_max(pmin, mslot(p, MS_PMIN), vb, sh.f, true);
  write_partial_max(pmax, mslot(p, MS_PMAX), vb, sh.f, false);
  write_partial(badp, islot(p, IS_PBAD), vb, sh.l);
}

// HPWL over the baseline hypernets at `pos` (per-net FP32 spans, FP64 sum).
static __device__ void stage_hpwl(const Dev& d, const float2* pos, Partials p, int vb, int nvb,
                                  Shared& sh) {
  double acc = 0.0;
  const int stride = nvb * blockDim.x;
  for (int e = vb * blockDim.x + threadIdx.x; e < d.n_hpwl_nets; e += stride) {
    float mx = -INFINITY, mnx = INFINITY, my = -INFINITY, mny = INFINITY;
    for (int k = d.net_ptr[e]; k < d.net_ptr[e + 1]; ++k) {
      const float2 v = pin_xy(d, pos, k);
      mx = fmaxf(mx, v.x);
      mnx = fminf(mnx, v.x);
      my = fmaxf(my, v.y);
      mny = fminf(mny, v.y);
    }
    acc += (double)((mx - mnx) + (my - mny));
  }
  write_partial(acc, pslot(p, SLOT_HPWL), vb, sh.d);
}

}  // namespace tgp
