// kernels.cu — standalone kernels (one stage each) and their launchers.
#include "dct_fft.cuh"
#include "dct_tc.cuh"
#include "kernels.cuh"
#include "scatter_tiles.cuh"

namespace tgp {

// The FFT form's three passes (dct_fft.cuh).
__global__ void __launch_bounds__(kThreads) k_fft_rows_fwd(Dev d, Partials p) {
  __shared__ fft::Smem sm;
  __shared__ Shared sh;
  fft::pass_rows_fwd(d, p, blockIdx.x, gridDim.x, sm, sh, nullptr);
}
__global__ void __launch_bounds__(kThreads) k_fft_cols(Dev d) {
  __shared__ fft::Smem sm;
  fft::pass_cols(d, blockIdx.x, gridDim.x, sm);
}
__global__ void __launch_bounds__(kThreads) k_fft_rows_inv(Dev d, Partials p) {
  __shared__ fft::Smem sm;
  __shared__ Shared sh;
  fft::pass_rows_inv(d, p, blockIdx.x, gridDim.x, sm, sh);
}

// The slice phase before tensor-core pass `step` (memory-bound, every block).
__global__ void __launch_bounds__(kThreads) k_tc_slice(Dev d, int step) {
  tc::slice_phase(d, step, blockIdx.x, gridDim.x);
}

// One DCT pass on tcgen05 tensor cores, one 128 x 64 tile per block
// iteration; gridDim.x <= the pass's tiles. The energy partials of pass 3 are
// those of the blocks launched; the slice phase before it zeroes the rest.
template <int STEP>
__global__ void __launch_bounds__(kThreads, 1) k_dct_tc(Dev d, Partials p, unsigned long long* err,
                                                       const __grid_constant__ tc::TcMaps maps) {
  extern __shared__ __align__(128) unsigned char tc_dyn[];
  tc::Smem& sm = *reinterpret_cast<tc::Smem*>(tc_dyn);
  double eacc[kMaxFields] = {0.0, 0.0, 0.0, 0.0};
  tc::setup(sm);
  tc::dct_pass<STEP>(d, maps, blockIdx.x, gridDim.x, sm, eacc, err);
  tc::teardown(sm);
  if constexpr (STEP == 3) {
    __shared__ Shared sh;
    for (int f = 0; f < d.K; ++f) write_partial(eacc[f], pslot(p, SLOT_ENERGY + f), (int)blockIdx.x, sh.d);
  }
}
template <int STEP>
void launch_dct_tc(const Dev& d, const Reduce& r, int gb, cudaStream_t s, const tc::TcMaps& maps) {
  static const bool attr = cudaFuncSetAttribute(k_dct_tc<STEP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                (int)sizeof(tc::Smem)) == cudaSuccess;
  (void)attr;
  k_dct_tc<STEP><<<gb, kThreads, sizeof(tc::Smem), s>>>(d, r.p, (unsigned long long*)(r.iscal + SI_TC_FAIL), maps);
}
// Zero energy partials of the virtual blocks [from, nvb) (pass 3 runs fewer).
__global__ void __launch_bounds__(kThreads) k_zero_energy(Dev d, Partials p, int from) {
  __shared__ Shared sh;
  if ((int)blockIdx.x >= from)
    for (int f = 0; f < d.K; ++f) write_partial(0.0, pslot(p, SLOT_ENERGY + f), (int)blockIdx.x, sh.d);
}

__global__ void __launch_bounds__(kThreads) k_init(Dev d, bool grids, bool wa) {
  stage_init(d, blockIdx.x, gridDim.x, grids, wa);
}
__global__ void __launch_bounds__(kThreads) k_scatter(Dev d, Partials p, const float2* pos) {
  __shared__ Shared sh;
  stage_scatter(d, pos, p, blockIdx.x, gridDim.x, sh);
}
// The tiled scatter's four passes (scatter_tiles.cuh).
__global__ void __launch_bounds__(kThreads) k_tile_count(Dev d, const float2* pos) {
  tiles::count(d, pos, blockIdx.x, gridDim.x);
}
__global__ void __launch_bounds__(kThreads) k_tile_scan(Dev d) { tiles::scan(d); }
__global__ void __launch_bounds__(kThreads) k_tile_place(Dev d) { tiles::place(d, blockIdx.x, gridDim.x); }
__global__ void __launch_bounds__(kThreads) k_tile_scatter(Dev d, Partials p, const float2* pos) {
  __shared__ tiles::Smem sm;
  __shared__ Shared sh;
  tiles::scatter(d, pos, p, blockIdx.x, gridDim.x, sm, sh);
}
// Every object uniform in its bounds from a fixed hash (the autotuner's
// stand-in for a spread placement).
__global__ void __launch_bounds__(kThreads) k_spread_positions(Dev d, float2* out) {
  for (int o = blockIdx.x * blockDim.x + threadIdx.x; o < d.nobj; o += gridDim.x * blockDim.x) {
    unsigned h = (unsigned)o * 2654435761u + 12345u;
    h ^= h >> 15;
    h *= 2246822519u;
    h ^= h >> 13;
    const float fx = (float)(h & 0xffffu) * (1.0f / 65536.0f), fy = (float)(h >> 16) * (1.0f / 65536.0f);
    const float2 lo = d.lo[o], hi = d.hi[o];
    out[o] = make_float2(fmaf(hi.x - lo.x, fx, lo.x), fmaf(hi.y - lo.y, fy, lo.y));
  }
}
__global__ void __launch_bounds__(kThreads) k_wa(Dev d, Partials p, const float2* pos, double gamma) {
  __shared__ Shared sh;
  stage_wa(d, pos, gamma, p, blockIdx.x, gridDim.x, sh);
}
__global__ void __launch_bounds__(kThreads) k_prep(Dev d, Partials p) {
  __shared__ Shared sh;
  stage_prep(d, p, gridDim.x, blockIdx.x, gridDim.x, sh);
}
template <bool LARGE>
__global__ void __launch_bounds__(kThreads) k_dct(Dev d, Partials p, int step) {
  __shared__ GemmShared sm;
  __shared__ Shared sh;
  stage_dct_t<LARGE>(d, step, p, blockIdx.x, gridDim.x, sm, sh);
}
__global__ void __launch_bounds__(kThreads) k_gather(Dev d, Partials p, const float2* pos) {
  __shared__ Shared sh;
  stage_gather(d, pos, p, blockIdx.x, gridDim.x, sh);
}
__global__ void __launch_bounds__(kThreads) k_combine(Dev d, Partials p, const double* coef, float2* gout) {
  __shared__ Shared sh;
  stage_combine(d, coef, gout, p, blockIdx.x, gridDim.x, sh);
}
__global__ void __launch_bounds__(kThreads) k_extrapolate(Dev d, Partials p, const float2* x, const float2* xp,
                                                         float e, float2* y) {
  __shared__ Shared sh;
  stage_extrapolate(d, x, xp, e, y, p, blockIdx.x, gridDim.x, sh);
}
__global__ void __launch_bounds__(kThreads) k_candidate(Dev d, Partials p, const float2* y, const float2* gy,
                                                       float invL, float2* c) {
  __shared__ Shared sh;
  stage_candidate(d, y, gy, invL, c, p, blockIdx.x, gridDim.x, sh);
}
__global__ void __launch_bounds__(kThreads) k_kkt(Dev d, Partials p, const float2* x, const float2* g,
                                                 const float2* ref) {
  __shared__ Shared sh;
  stage_kkt(d, x, g, ref, p, blockIdx.x, gridDim.x, sh);
}
__global__ void __launch_bounds__(kThreads) k_precond(Dev d, Partials p, const double* lambda) {
  __shared__ Shared sh;
  stage_precond(d, lambda, p, blockIdx.x, gridDim.x, sh);
}
__global__ void __launch_bounds__(kThreads) k_hpwl(Dev d, Partials p, const float2* pos) {
  __shared__ Shared sh;
  stage_hpwl(d, pos, p, blockIdx.x, gridDim.x, sh);
}

// Reduces the partials selected by `mask` in a fixed order and derives the
// objective scalars (combined_objective / augmented_density_value_and_coefficient,
// eplace.rs:1022-1044, 1111-1124).
__global__ void __launch_bounds__(kThreads) k_finalize(Dev d, Reduce r, int nvb, int mask) {
  __shared__ double shd[kThreads / 32];
  __shared__ long long shl[kThreads / 32];
  const Partials& p = r.p;
  double* sc = r.scal;
  long long* si = r.iscal;
  if (mask & (FIN_ENERGY | FIN_WA)) {
    const double wa = block_reduce_array(pslot(p, SLOT_WA_VALUE), nvb, 0.0, OpAdd(), shd);
    if (threadIdx.x == 0) sc[SC_WA] = wa;
  }
  if (mask & FIN_ENERGY) {
    for (int f = 0; f < d.K; ++f) {
      const double e = block_reduce_array(pslot(p, SLOT_ENERGY + f), nvb, 0.0, OpAdd(), shd);
      const long long ov = block_reduce_array(islot(p, IS_OVERFLOW + f), nvb, 0ll, OpAdd(), shl);
      const long long bins = block_reduce_array(islot(p, IS_OVER_BINS + f), nvb, 0ll, OpAdd(), shl);
      const long long gs = block_reduce_array(islot(p, IS_GRID_SUM + f), nvb, 0ll, OpAdd(), shl);
      if (threadIdx.x == 0) {
        sc[SC_ENERGY + f] = 0.5 * e;
        si[SI_OVERFLOW_FIXED + f] = ov;
        si[SI_OVER_BINS + f] = bins;
        si[SI_GRID_SUM + f] = gs;
        sc[SC_OVERFLOW + f] = ((double)ov * kInvFix) / sc[SC_REAL_AREA + f];
        sc[SC_MEAN + f] = (double)(gs - d.capsum[f]) * kInvFix;
      }
    }
  }
  if (mask & (FIN_ENERGY | FIN_WA)) {
    if (threadIdx.x == 0) {
      double value = sc[SC_WA];
      const double beta = sc[SC_BETA];
      for (int f = 0; f < d.K; ++f) {
        const double e0 = sc[SC_E0 + f], lam = sc[SC_LAMBDA + f];
        const double ne = sc[SC_ENERGY + f] / e0;
        value += lam * e0 * (ne + 0.5 * beta * ne * ne);
        sc[SC_COEF + f] = lam * (1.0 + beta * ne);
      }
      sc[SC_VALUE] = value;
    }
    __syncthreads();
  }
  if (mask & FIN_COMBINE) {
    for (int f = 0; f < d.K; ++f) {
      const double a = block_reduce_array(pslot(p, SLOT_RAWL1 + f), nvb, 0.0, OpAdd(), shd);
      const double b = block_reduce_array(pslot(p, SLOT_FORCE + f), nvb, 0.0, OpAdd(), shd);
      if (threadIdx.x == 0) {
        sc[SC_RAWL1 + f] = a;
        sc[SC_FORCE + f] = b;
      }
    }
    const double w = block_reduce_array(pslot(p, SLOT_WAL1), nvb, 0.0, OpAdd(), shd);
    const long long bad = block_reduce_array(islot(p, IS_BAD), nvb, 0x7fffffffffffffffll, OpMin(), shl);
    if (threadIdx.x == 0) {
      sc[SC_WAL1] = w;
      si[SI_BAD] = bad;
    }
  }
  if (mask & (FIN_CAND | FIN_DIFF)) {
    const long long diff = block_reduce_array(islot(p, IS_DIFF), nvb, 0ll, OpAdd(), shl);
    if (threadIdx.x == 0) si[SI_DIFF] = diff;
  }
  if (mask & FIN_CAND) {
    const double a = block_reduce_array(pslot(p, SLOT_DOT), nvb, 0.0, OpAdd(), shd);
    const double b = block_reduce_array(pslot(p, SLOT_MSN), nvb, 0.0, OpAdd(), shd);
    if (threadIdx.x == 0) {
      sc[SC_DOT] = a;
      sc[SC_MSN] = b;
    }
  }
  if (mask & FIN_KKT) {
    const double a = block_reduce_array(mslot(p, MS_KKT), nvb, 0.0, OpMax(), shd);
    const double b = block_reduce_array(mslot(p, MS_CHANGE), nvb, 0.0, OpMax(), shd);
    if (threadIdx.x == 0) {
      sc[SC_KKT] = a;
      sc[SC_CHANGE] = b;
    }
  }
  if (mask & FIN_PRECOND) {
    const double a = block_reduce_array(mslot(p, MS_PMIN), nvb, (double)INFINITY, OpMin(), shd);
    const double b = block_reduce_array(mslot(p, MS_PMAX), nvb, 0.0, OpMax(), shd);
    const long long c = block_reduce_array(islot(p, IS_PBAD), nvb, 0ll, OpAdd(), shl);
    if (threadIdx.x == 0) {
      sc[SC_PMIN] = a;
      sc[SC_PMAX] = b;
      si[SI_PBAD] = c;
    }
  }
  if (mask & FIN_HPWL) {
    const double a = block_reduce_array(pslot(p, SLOT_HPWL), nvb, 0.0, OpAdd(), shd);
    if (threadIdx.x == 0) sc[SC_HPWL] = a;
  }
}

// rounded_targets_from_coordinates (eplace.rs:954-971) compared with the
// previous stationary targets (stationary_target_is_fixed, :973-985).
__global__ void k_round_compare(Dev d, const float2* x, uint32_t* prev, int W, int H, unsigned long long* mismatch) {
  for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < d.U; u += gridDim.x * blockDim.x) {
    const float2 a = x[u];
    const float rx = fminf(fmaxf(roundf(a.x), 0.f), (float)(W - 1));
    const float ry = fminf(fmaxf(roundf(a.y), 0.f), (float)(H - 1));
    const uint32_t tx = (uint32_t)rx, ty = (uint32_t)ry;
    if (prev[2 * u] != tx || prev[2 * u + 1] != ty) atomicAdd(mismatch, 1ull);
    prev[2 * u] = tx;
    prev[2 * u + 1] = ty;
  }
}

static thread_local unsigned long long t_launches = 0;
unsigned long long launches_issued() { return t_launches; }
void note_launch() { ++t_launches; }
#define COUNT ++t_launches

static inline bool use_large_tiles(const Dev& d) { return d.dct_large != 0; }

void launch_init(const Dev& d, bool grids, bool wa, int nvb, cudaStream_t s) {
  COUNT;
  k_init<<<nvb, kThreads, 0, s>>>(d, grids, wa);
}
void launch_scatter(const Dev& d, const Reduce& r, const float2* pos, int nvb, cudaStream_t s) {
  if (d.scatter_tiles && d.Mm + d.F > 0) {
    t_launches += 4;
    k_tile_count<<<nvb, kThreads, 0, s>>>(d, pos);
    k_tile_scan<<<1, kThreads, 0, s>>>(d);
    k_tile_place<<<nvb, kThreads, 0, s>>>(d);
    k_tile_scatter<<<nvb, kThreads, 0, s>>>(d, r.p, pos);
    return;
  }
  COUNT;
  k_scatter<<<nvb, kThreads, 0, s>>>(d, r.p, pos);
}
void launch_spread_positions(const Dev& d, float2* out, int nvb, cudaStream_t s) {
  COUNT;
  k_spread_positions<<<nvb, kThreads, 0, s>>>(d, out);
}
void launch_wa(const Dev& d, const Reduce& r, const float2* pos, double gamma, int nvb, cudaStream_t s) {
  COUNT;
  k_wa<<<nvb, kThreads, 0, s>>>(d, r.p, pos, gamma);
}
void launch_prep(const Dev& d, const Reduce& r, int nvb, cudaStream_t s) {
  COUNT;
  k_prep<<<nvb, kThreads, 0, s>>>(d, r.p);
}
void launch_dct(const Dev& d, const Reduce& r, int step, int nvb, cudaStream_t s, const tc::TcMaps* maps) {
  if (d.fft) {   // rows, columns (forward, scale, inverse), rows: step 2 has no work
    if (step == 2) return;
    COUNT;
    if (step == 0)
      k_fft_rows_fwd<<<nvb, kThreads, 0, s>>>(d, r.p);
    else if (step == 1)
      k_fft_cols<<<nvb, kThreads, 0, s>>>(d);
    else
      k_fft_rows_inv<<<nvb, kThreads, 0, s>>>(d, r.p);
    return;
  }
  if (d.tc) {
    if (!maps) return;   // the tensor-core form needs the instance's tensor maps
    // one block a tile (at most one resident a multiprocessor: the pipeline
    // holds 192 KB of shared memory and 256 TMEM columns)
    const int gb = std::max(1, std::min(nvb, tc::pass_tiles_host(d)));
    COUNT;
    k_tc_slice<<<nvb, kThreads, 0, s>>>(d, step);
    if (step == 3 && gb < nvb) {
      COUNT;
      k_zero_energy<<<nvb, kThreads, 0, s>>>(d, r.p, gb);
    }
    COUNT;
    switch (step) {
      case 0: launch_dct_tc<0>(d, r, gb, s, *maps); break;
      case 1: launch_dct_tc<1>(d, r, gb, s, *maps); break;
      case 2: launch_dct_tc<2>(d, r, gb, s, *maps); break;
      default: launch_dct_tc<3>(d, r, gb, s, *maps); break;
    }
    return;
  }
  COUNT;
  if (use_large_tiles(d))
    k_dct<true><<<nvb, kThreads, 0, s>>>(d, r.p, step);
  else
    k_dct<false><<<nvb, kThreads, 0, s>>>(d, r.p, step);
}
void launch_gather(const Dev& d, const Reduce& r, const float2* pos, int nvb, cudaStream_t s) {
  COUNT;
  k_gather<<<nvb, kThreads, 0, s>>>(d, r.p, pos);
}
void launch_combine(const Dev& d, const Reduce& r, float2* gout, int nvb, cudaStream_t s) {
  COUNT;
  k_combine<<<nvb, kThreads, 0, s>>>(d, r.p, r.scal + SC_COEF, gout);
}
void launch_extrapolate(const Dev& d, const Reduce& r, const float2* x, const float2* xp, float e, float2* y,
                        int nvb, cudaStream_t s) {
  COUNT;
  k_extrapolate<<<nvb, kThreads, 0, s>>>(d, r.p, x, xp, e, y);
}
void launch_candidate(const Dev& d, const Reduce& r, const float2* y, const float2* gy, float invL, float2* c,
                      int nvb, cudaStream_t s) {
  COUNT;
  k_candidate<<<nvb, kThreads, 0, s>>>(d, r.p, y, gy, invL, c);
}
void launch_kkt(const Dev& d, const Reduce& r, const float2* x, const float2* g, const float2* ref, int nvb,
                cudaStream_t s) {
  COUNT;
  k_kkt<<<nvb, kThreads, 0, s>>>(d, r.p, x, g, ref);
}
void launch_precond(const Dev& d, const Reduce& r, int nvb, cudaStream_t s) {
  COUNT;
  k_precond<<<nvb, kThreads, 0, s>>>(d, r.p, r.scal + SC_LAMBDA);
}
void launch_hpwl(const Dev& d, const Reduce& r, const float2* pos, int nvb, cudaStream_t s) {
  COUNT;
  k_hpwl<<<nvb, kThreads, 0, s>>>(d, r.p, pos);
}
void launch_finalize(const Dev& d, const Reduce& r, int nvb, int mask, cudaStream_t s) {
  COUNT;
  k_finalize<<<1, kThreads, 0, s>>>(d, r, nvb, mask);
}
void launch_round_compare(const Dev& d, const float2* x, uint32_t* prev, int W, int H, unsigned long long* mismatch,
                          int nvb, cudaStream_t s) {
  COUNT;
  k_round_compare<<<nvb, kThreads, 0, s>>>(d, x, prev, W, H, mismatch);
}

}  // namespace tgp
