// persistent_body.cuh — the whole placement loop in one cooperative kernel.
//
// The kernel runs `optimize_density_once` (crates/texo-pnr/src/eplace.rs:439-582)
// with `dynamic_nesterov_step` (crates/texo-pnr/src/global_placement.rs:121-335)
// on the device. Stages are separated by a barrier over the instance's
// blocks; after each barrier every block reduces the partials it needs in the
// same fixed order, so all blocks hold bit-identical scalars and take the same
// branch. Thread 0 of each block keeps the controller state in shared memory;
// the instance's first block writes it back when the kernel returns.
//
// Work is split into a fixed number V of virtual blocks per instance; the
// instance's physical blocks loop over them. Partials are indexed by virtual
// block, so an instance computes bit-identical results whether it runs alone
// on every SM or shares one launch with other instances (batched serving).
//
// Every wait is bounded: a barrier that does not complete within its spin
// budget sets an error word, and the instance's blocks then leave the kernel
// at their next barrier.
//
// run_body is instantiated by four small translation units (one kernel
// each: alone or batched, small or large DCT tiles) so that they compile in
// parallel.
#pragma once
#include <cmath>
#include <cstring>

#include "dct_fft.cuh"
#include "persistent.cuh"

namespace tgp {

constexpr unsigned kSpinLimit = 1u << 25;   // ~seconds of polling before giving up
constexpr unsigned kMaxTrialsPerStep = 8192;

struct ERec {
  double value, wa, wal1, kkt;
  double energy[kMaxFields], overflow[kMaxFields], force[kMaxFields], rawl1[kMaxFields];
  long long ovfix[kMaxFields], bins[kMaxFields];
  long long bad;
};

__device__ __forceinline__ unsigned long long now_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// (generation, error) of a barrier in one acquire load: every write made
// before the releasing arrival is visible once the new generation is seen
__device__ __forceinline__ unsigned long long load_gen_error(const GridBarrier* b) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(&b->gen) : "memory");
  return v;
}

// Barrier over the np physical blocks of one instance. Arrival is an
// acq_rel add on one counter (release publishes this block's writes, acquire
// makes the last arriver see everyone's); the last arriver resets the
// counter and release-increments the generation the others poll with
// acquire loads, which also carry the error word.
__device__ __forceinline__ bool grid_sync(GridBarrier* b, unsigned np, unsigned* gen, unsigned long long* count,
                                          unsigned long long* wait_acc, int* failed, unsigned limit = kSpinLimit) {
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned long long t0 = wait_acc ? now_ns() : 0ull;
    const unsigned g = *gen;
    // One counter: on this two-die part a barrier costs a few L2 round trips
    // whatever the arrival pattern, and a two-level tree only adds one.
    unsigned old;
    asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], 1;" : "=r"(old) : "l"(&b->root.count) : "memory");
    unsigned long long ge;
    if (old + 1u == np) {
      asm volatile("st.relaxed.gpu.global.u32 [%0], 0;" ::"l"(&b->root.count) : "memory");
      asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(&b->gen) : "memory");
      ge = load_gen_error(b);
    } else {
      unsigned spins = 0;
      for (;;) {
        ge = load_gen_error(b);
        if ((unsigned)ge != g || (ge >> 32) != 0ull) break;
        if (++spins > limit) {
          atomicExch(&b->error, 1);
          ge |= 1ull << 32;
          break;
        }
        if (spins > 64) __nanosleep(32);
      }
    }
    *gen = g + 1;
    ++*count;
    if (wait_acc) *wait_acc += now_ns() - t0;
    *failed = (int)(ge >> 32);
  }
  __syncthreads();
  // one read of the error word per block, so all its threads agree
  return *failed == 0;
}

// One reduction of the V partials of a slot, folded by one warp in a fixed
// order (lanes stride the partials, then an xor tree over the lanes).
enum FoldOp { FOLD_DSUM, FOLD_ISUM, FOLD_IMIN, FOLD_DMAX, FOLD_DMIN };
struct FoldJob {
  const void* a;
  int op;
};
union FoldValue {
  double d;
  long long l;
};
constexpr int kMaxFoldJobs = 3 * kMaxFields + 3;
template <typename T, typename Op>
__device__ __forceinline__ T warp_fold(const T* a, int n, T init, Op op) {
  const int lane = threadIdx.x & 31;
  T v = lane < n ? a[lane] : init;
#pragma unroll 4
  for (int i = lane + 32; i < n; i += 32) v = op(v, a[i]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = op(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

template <bool LARGE>
struct Ctx {
  const Dev& d;
  const Reduce& r;
  const Buffers& B;
  DevRun& S;          // shared memory, written by thread 0
  GridBarrier* bar;
  unsigned* gen;
  int* gen_failed;     // shared: the barrier's error word as thread 0 last read it
  GemmShared& gsm;
  Shared& sh;
  double* rd;         // reduction scratch (shared)
  long long* rl;
  double* coef;       // shared [kMaxFields]
  FoldValue* fv;      // shared [kMaxFoldJobs] results of fold()
  long long* fmean;   // shared [kMaxFields] fixed-point density means
  int pb, np;         // physical block of the instance, physical block count
  int V;              // virtual blocks of the instance
  unsigned long long nbar;
  unsigned long long* clock;   // shared [8] phase accumulators, [8] last mark, [9] barrier wait

  unsigned ph = 0;             // barriers passed, counted by every thread

  __device__ bool sync() {
    ++ph;
    return grid_sync(bar, (unsigned)np, gen, &nbar, pb == 0 ? clock + 9 : nullptr, gen_failed);
  }
  // Partials of the loop's back-to-back phases (extrapolate, candidate,
  // stationary check) alternate between two sets: a block that leaves a
  // barrier early and writes the next phase's partials must not overwrite
  // the ones a slower block of the instance is still reducing. wset() is
  // written by the current phase, rset() holds the phase that just ended.
  __device__ Partials wset() const { return (ph & 1u) ? r.q : r.p; }
  __device__ Partials rset() const { return (ph & 1u) ? r.p : r.q; }
  // Charges the time since the previous mark to phase category `cat` (block 0).
  __device__ void mark(int cat) {
    if (pb == 0 && threadIdx.x == 0) {
      const unsigned long long t = now_ns();
      clock[cat] += t - clock[8];
      clock[8] = t;
    }
  }
  // Several reductions of partials at once: job j is folded by warp j (mod
  // the warp count), so the loads of all jobs are in flight together (one
  // L2 round trip for partials that other SMs wrote, often on the other
  // die) and the FP64 folds of different jobs run on different SM
  // sub-partitions. Every thread reads the results in fv after the final
  // block barrier.
  __device__ void fold(const FoldJob* jobs, int n) {
    __syncthreads();   // earlier readers of fv are done
    const int nw = (int)(blockDim.x >> 5);
    for (int j = threadIdx.x >> 5; j < n; j += nw) {
      const FoldJob jb = jobs[j];
      FoldValue out;
      switch (jb.op) {
        case FOLD_DSUM: out.d = warp_fold((const double*)jb.a, V, 0.0, OpAdd()); break;
        case FOLD_ISUM: out.l = warp_fold((const long long*)jb.a, V, 0ll, OpAdd()); break;
        case FOLD_IMIN: out.l = warp_fold((const long long*)jb.a, V, 0x7fffffffffffffffll, OpMin()); break;
        case FOLD_DMAX: out.d = warp_fold((const double*)jb.a, V, 0.0, OpMax()); break;
        default: out.d = warp_fold((const double*)jb.a, V, (double)INFINITY, OpMin()); break;
      }
      if ((threadIdx.x & 31) == 0) fv[j] = out;
    }
    __syncthreads();
  }
  __device__ long long risum_prev(int slot) {
    return block_reduce_array(islot(rset(), slot), V, 0ll, OpAdd(), rl);
  }
  __device__ float2* X() const { return B.pos[S.ix]; }
  __device__ float2* Xp() const { return B.pos[S.ixp]; }
  __device__ float2* Y() const { return B.pos[S.iy]; }
  __device__ float2* C() const { return B.pos[S.ic]; }
  __device__ float2* gX() const { return B.grad[S.igx]; }
  __device__ float2* gY() const { return B.grad[S.igy]; }
  __device__ float2* gC() const { return B.grad[S.igc]; }

  __device__ void copy(float2* dst, const float2* src, int n) {
    for (int i = pb * blockDim.x + threadIdx.x; i < n; i += np * blockDim.x) dst[i] = src[i];
  }

  // fixed-point density mean per field (DC mode), from the scatter's grid sums
  __device__ void fold_means() {
    FoldJob jobs[kMaxFields];
    for (int f = 0; f < d.K; ++f) jobs[f] = FoldJob{islot(r.p, IS_GRID_SUM + f), FOLD_ISUM};
    fold(jobs, d.K);
    if (threadIdx.x == 0)
      for (int f = 0; f < d.K; ++f) fmean[f] = (fv[f].l - d.capsum[f]) / d.B;
    __syncthreads();
  }

  // Objective evaluation at pos after an init phase and its barrier
  // (ContinuousProblem::evaluate + combined_objective, eplace.rs:137-205, 1022-1044).
  __device__ bool eval_tail(const float2* pos, float2* g, double gam, bool full, const float2* kkt_pos, ERec& out) {
    if (full)
      for (int v = pb; v < V; v += np) stage_scatter(d, pos, r.p, v, V, sh);
    for (int v = pb; v < V; v += np) stage_wa(d, pos, gam, r.p, v, V, sh);
    if (!sync()) return false;
    mark(PC_SCATTER_WA);
    if (full) {
      if (d.fft) {
        // FFT form: rows (with the density preparation folded in), columns, rows
        fold_means();
        fft::Smem& fs = *reinterpret_cast<fft::Smem*>(gsm.fft);
        for (int v = pb; v < V; v += np) fft::pass_rows_fwd(d, r.p, v, V, fs, sh, fmean);
        if (!sync()) return false;
        for (int v = pb; v < V; v += np) fft::pass_cols(d, v, V, fs);
        if (!sync()) return false;
        for (int v = pb; v < V; v += np) fft::pass_rows_inv(d, r.p, v, V, fs, sh);
        if (!sync()) return false;
      } else {
        int st0 = 0;
        if (LARGE) {
          for (int v = pb; v < V; v += np) stage_prep(d, r.p, V, v, V, sh);
          if (!sync()) return false;
          mark(PC_PREP);
        } else {
          // density preparation folded into the first transform (one phase less)
          fold_means();
          for (int v = pb; v < V; v += np) stage_prep_dct0(d, fmean, r.p, v, V, gsm, sh);
          if (!sync()) return false;
          st0 = 1;
        }
        for (int st = st0; st < 4; ++st) {
          for (int v = pb; v < V; v += np) stage_dct_t<LARGE>(d, st, r.p, v, V, gsm, sh);
          if (!sync()) return false;
        }
      }
      mark(PC_DCT);
    }
    {
      // energies, overflow and overflowed bins per field (density side
      // rebuilt), and the WA value: one fold
      FoldJob jobs[kMaxFoldJobs];
      int nj = 0;
      if (full)
        for (int f = 0; f < d.K; ++f) {
          jobs[nj++] = FoldJob{pslot(r.p, SLOT_ENERGY + f), FOLD_DSUM};
          jobs[nj++] = FoldJob{islot(r.p, IS_OVERFLOW + f), FOLD_ISUM};
          jobs[nj++] = FoldJob{islot(r.p, IS_OVER_BINS + f), FOLD_ISUM};
        }
      jobs[nj++] = FoldJob{pslot(r.p, SLOT_WA_VALUE), FOLD_DSUM};
      fold(jobs, nj);
    }
    if (threadIdx.x == 0) {
      for (int f = 0; f < d.K; ++f) {
        if (full) {
          const long long ov = fv[3 * f + 1].l;
          out.energy[f] = 0.5 * fv[3 * f].d;
          out.ovfix[f] = ov;
          out.bins[f] = fv[3 * f + 2].l;
          out.overflow[f] = ((double)ov * kInvFix) * S.inv_real_area[f];
        } else {
          out.energy[f] = S.cur_energy[f];
          out.overflow[f] = S.cur_overflow[f];
          out.ovfix[f] = S.cur_overflow_fixed[f];
          out.bins[f] = 0;
        }
      }
      const double wa = fv[full ? 3 * d.K : 0].d;
      out.wa = wa;
      double value = wa;
      for (int f = 0; f < d.K; ++f) {
        const double ne = out.energy[f] * S.inv_e0[f];
        value += S.lambda[f] * S.e0[f] * (ne + 0.5 * S.beta * ne * ne);
        coef[f] = S.lambda[f] * (1.0 + S.beta * ne);
      }
      out.value = value;
    }
    __syncthreads();
    // gather and combine of one virtual block run back to back: the same
    // thread produces and consumes each object's raw field gradient
    for (int v = pb; v < V; v += np) {
      if (full) stage_gather(d, pos, r.p, v, V, sh);
      stage_combine(d, coef, g, r.p, v, V, sh, kkt_pos);
    }
    if (!sync()) return false;
    mark(PC_GATHER);
    {
      FoldJob jobs[kMaxFoldJobs];
      int nj = 0;
      for (int f = 0; f < d.K; ++f) {
        jobs[nj++] = FoldJob{pslot(r.p, SLOT_RAWL1 + f), FOLD_DSUM};
        jobs[nj++] = FoldJob{pslot(r.p, SLOT_FORCE + f), FOLD_DSUM};
      }
      jobs[nj++] = FoldJob{pslot(r.p, SLOT_WAL1), FOLD_DSUM};
      jobs[nj++] = FoldJob{islot(r.p, IS_BAD), FOLD_IMIN};
      if (kkt_pos) jobs[nj++] = FoldJob{mslot(r.p, MS_KKT), FOLD_DMAX};
      fold(jobs, nj);
    }
    if (threadIdx.x == 0) {
      for (int f = 0; f < d.K; ++f) {
        out.rawl1[f] = fv[2 * f].d;
        out.force[f] = fv[2 * f + 1].d;
      }
      out.wal1 = fv[2 * d.K].d;
      out.bad = fv[2 * d.K + 1].l;
      out.kkt = kkt_pos ? fv[2 * d.K + 2].d : 0.0;
      S.evaluations++;
      if (full) S.density_evaluations++;
    }
    __syncthreads();
    return true;
  }
};

// ---- scalar rules (eplace.rs:1300-1415), evaluated by thread 0 ------------
static __device__ int field_gamma_dev(double overflow, double target, double slope, double base, double& g) {
  if (!isfinite(overflow) || overflow < 0.0 || !(target >= 0.0 && target < 1.0) || !(base > 0.0))
    return TEXO_GP_ERR_INVALID_NORMALIZATION;
  const double intercept = 1.0 - slope;   // slope = 2 / (1 - target), from the host
  // 10^t as exp(t ln 10): a fraction of pow's cost on the device, within a
  // few ulps for the exponents this rule produces
  constexpr double kLn10 = 2.302585092994045684;
  g = base * exp(kLn10 * (slope * overflow + intercept));
  return (isfinite(g) && g > 0.0) ? TEXO_GP_OK : TEXO_GP_ERR_INVALID_NORMALIZATION;
}
static __device__ int adaptive_gamma_dev(const DevRun& S, const double* overflow, double& out) {
  double ws = 0.0, wsum = 0.0;
  for (int f = 0; f < S.K; ++f) {
    double g;
    const int st = field_gamma_dev(overflow[f], S.target[f], S.gamma_slope[f], S.gamma_base, g);
    if (st) return st;
    ws += g * S.gamma_weight[f];
    wsum += S.gamma_weight[f];
  }
  out = wsum == 0.0 ? S.gamma_base : ws * S.inv_gamma_weight_sum;
  return (isfinite(out) && out > 0.0) ? TEXO_GP_OK : TEXO_GP_ERR_INVALID_NORMALIZATION;
}
// density_stop_reached (eplace.rs:1397-1415): Final, or AreaAdjustmentReady
// (LUT and register fields at 0.15, AREA_ADJUSTMENT_OVERFLOW_TARGET)
static __device__ bool stop_dev(const DevRun& S, const double* overflow) {
  for (int f = 0; f < S.K; ++f) {
    if (S.stop_mode == 1) {
      if (S.area_field[f] && !(overflow[f] <= 0.15)) return false;
    } else if (!(overflow[f] <= S.target[f])) {
      return false;
    }
  }
  return true;
}
// area_adjusted_density_multipliers and area_adjusted_multiplier_step
// (eplace.rs:1183-1232), elfPlace eqs. (27)-(28)
static __device__ int area_multipliers_dev(DevRun& S, const ERec& e) {
  double sg[kMaxFields], dens = 0.0;
  for (int f = 0; f < S.K; ++f) {
    const double ne = e.energy[f] * S.inv_e0[f];
    sg[f] = ne + 0.5 * S.beta * ne * ne;
    if (!isfinite(sg[f]) || sg[f] < 0.0) return TEXO_GP_ERR_INVALID_NORMALIZATION;
    dens += e.force[f] * sg[f];
  }
  if (!isfinite(e.wal1) || e.wal1 <= 0.0 || !isfinite(dens) || dens <= 0.0) return TEXO_GP_ERR_INVALID_NORMALIZATION;
  const double scale = 0.1 * e.wal1 / dens;
  bool any = false;
  double nn = 0.0;
  for (int f = 0; f < S.K; ++f) {
    S.lambda[f] = scale * sg[f];
    if (!isfinite(S.lambda[f]) || S.lambda[f] < 0.0) return TEXO_GP_ERR_INVALID_NORMALIZATION;
    any = any || S.lambda[f] > 0.0;
    nn += S.lambda[f] * S.lambda[f];
  }
  if (!any) return TEXO_GP_ERR_INVALID_NORMALIZATION;
  S.mstep = (S.alpha_high - 1.0) * sqrt(nn);
  return (isfinite(S.mstep) && S.mstep > 0.0) ? TEXO_GP_OK : TEXO_GP_ERR_INVALID_NORMALIZATION;
}
static __device__ void excess_dev(const DevRun& S, const double* overflow, double& mx, double& tot) {
  mx = 0.0;
  tot = 0.0;
  for (int f = 0; f < S.K; ++f) {
    const double x = fmax(overflow[f] - S.target[f], 0.0);
    mx = fmax(mx, x);
    tot += x;
  }
}
static __device__ int validate_initial_dev(const DevRun& S, const ERec& e) {
  bool ok = isfinite(e.wa) && e.bad == 0x7fffffffffffffffll;
  for (int f = 0; f < S.K && ok; ++f)
    ok = isfinite(e.energy[f]) && e.energy[f] >= 0.0 && isfinite(e.overflow[f]) && isfinite(e.force[f]) &&
         e.force[f] >= 0.0;
  return ok ? TEXO_GP_OK : TEXO_GP_ERR_INVALID_NORMALIZATION;
}
static __device__ int checked_dev(const ERec& e) {
  if (!isfinite(e.value)) return TEXO_GP_ERR_INVALID_OBJECTIVE;
  if (e.bad != 0x7fffffffffffffffll) return TEXO_GP_ERR_NONFINITE_GRADIENT;
  return TEXO_GP_OK;
}
// update_density_multipliers + next_multiplier_step (eplace.rs:1234-1298)
static __device__ int update_multipliers_dev(DevRun& S) {
  for (int f = 0; f < S.K; ++f)
    if (!isfinite(S.cur_energy[f]) || !(S.e0[f] > 0.0)) return TEXO_GP_ERR_DENSITY_FIELD_CHANGED;
  double sg[kMaxFields], nn = 0.0;
  for (int f = 0; f < S.K; ++f) {
    const double ne = S.cur_energy[f] * S.inv_e0[f];
    sg[f] = ne + 0.5 * S.beta * ne * ne;
    if (!isfinite(sg[f]) || sg[f] < 0.0) return TEXO_GP_ERR_INVALID_NORMALIZATION;
    nn += sg[f] * sg[f];
  }
  const double norm = sqrt(nn);
  if (norm != 0.0) {
    if (!isfinite(norm) || !isfinite(S.mstep) || S.mstep <= 0.0) return TEXO_GP_ERR_INVALID_NORMALIZATION;
    for (int f = 0; f < S.K; ++f) {
      S.lambda[f] += S.mstep * sg[f] / norm;
      if (!isfinite(S.lambda[f]) || S.lambda[f] < 0.0) return TEXO_GP_ERR_INVALID_NORMALIZATION;
    }
  }
  double en = 0.0;
  for (int f = 0; f < S.K; ++f) {
    const double ne = S.cur_energy[f] * S.inv_e0[f];
    en += ne * ne;
  }
  const double lg = log(S.beta * sqrt(en) + 1.0);
  if (!isfinite(lg) || lg < 0.0) return TEXO_GP_ERR_INVALID_NORMALIZATION;
  const double growth = S.alpha_low + (1.0 - 1.0 / (1.0 + lg)) * (S.alpha_high - S.alpha_low);
  if (!(growth >= S.alpha_low && growth <= S.alpha_high)) return TEXO_GP_ERR_INVALID_NORMALIZATION;
  S.mstep *= growth;
  return (isfinite(S.mstep) && S.mstep > 0.0) ? TEXO_GP_OK : TEXO_GP_ERR_INVALID_NORMALIZATION;
}
__device__ __forceinline__ double half_nonzero_dev(double v) {
  const double h = v * 0.5;
  return h == 0.0 ? v : h;
}
__device__ __forceinline__ double margin_dev(const DevRun& S, double x, double y) {
  return S.margin_eps * (1.0 + fabs(x) + fabs(y));
}
static __device__ void adopt_density(DevRun& S, const ERec& e) {
  for (int f = 0; f < S.K; ++f) {
    S.cur_overflow[f] = e.overflow[f];
    S.cur_energy[f] = e.energy[f];
    S.cur_force[f] = e.force[f];
    S.cur_overflow_fixed[f] = e.ovfix[f];
  }
}

// Shared-memory step bookkeeping that every thread reads after a barrier.
struct StepVars {
  int restart, y_is_origin, may_reduce, has_wL, action, stationary;
  double wL, tL, f_y, y_stat, next_m, pmin, pmax;
  unsigned trials;
  int pending_best, pending_prev;
};
enum { ACT_NONE = 0, ACT_RESTART, ACT_CONTINUE, ACT_ACCEPT, ACT_STATIONARY };

// Copies *src to *dst one 8-byte word per thread of the block (a struct copy
// by one thread waits for each load in turn). The caller synchronizes.
template <class T>
__device__ __forceinline__ void copy_words(T* dst, const T* src) {
  static_assert(sizeof(T) % 8 == 0 && alignof(T) >= 8, "copied as 8-byte words");
  for (int i = threadIdx.x; i < (int)(sizeof(T) / 8); i += blockDim.x)
    reinterpret_cast<unsigned long long*>(dst)[i] = reinterpret_cast<const unsigned long long*>(src)[i];
}

// The placement loop of one instance, run by its np physical blocks.
template <bool LARGE>
static __device__ void run_body(const Dev& d, const Reduce& r, const Buffers& B, DevRun* run, GridBarrier* bar, int pb,
                         int np, int Vn) {
  __shared__ DevRun S;
  __shared__ ERec eo, ey, ec;
  __shared__ StepVars V;
  __shared__ GemmShared gsm;
  __shared__ Shared sh;
  __shared__ double rd[kThreads / 32];
  __shared__ long long rl[kThreads / 32];
  __shared__ double coef[kMaxFields];
  __shared__ FoldValue fvals[kMaxFoldJobs];
  __shared__ long long fmean[kMaxFields];
  __shared__ unsigned gen;
  __shared__ int bar_failed;
  __shared__ unsigned long long clock[10];
  if (threadIdx.x == 0) {
    for (int i = 0; i < 10; ++i) clock[i] = 0;
    clock[8] = now_ns();
    gen = 0;   // the barrier is cleared with the state copy before every launch
    V.pending_best = 0;
    V.pending_prev = 0;
  }
  copy_words(&S, run);
  __syncthreads();
  Ctx<LARGE> c{d, r, B, S, bar, &gen, &bar_failed, gsm, sh, rd, rl, coef, fvals, fmean, pb, np, Vn, 0ull, clock};
  const int n = d.nobj;
  unsigned done = 0;
  bool ok = true;

// Thread 0 updates the block's shared controller state. The leading
// __syncthreads keeps it from overwriting a field (S, V) that a slower warp
// of the block is still reading from the previous update.
#define T0            \
  __syncthreads();    \
  if (threadIdx.x == 0)
#define VLOOP for (int v = c.pb; v < c.V; v += c.np)
#define SYNC_OR_EXIT(cat) \
  if (!c.sync()) {        \
    ok = false;           \
    goto out;             \
  }                       \
  c.mark(cat);
#define FAIL(code)            \
  {                           \
    T0 {                      \
      S.status = (code);      \
      S.phase = 2;            \
    }                         \
    __syncthreads();          \
    goto out;                 \
  }

  if (S.phase == 2) goto out;
  if (S.phase == 0) {
    // initial probe at the ePlace gamma base, then at the adaptive gamma with
    // the density side reused (same coordinates), eplace.rs:455-471
    VLOOP stage_init(d, v, c.V, true, true);
    SYNC_OR_EXIT(PC_PRECOND)
    if (!c.eval_tail(c.X(), c.gX(), S.gamma_base, true, nullptr, eo)) {
      ok = false;
      goto out;
    }
    {
      T0 {
        double g0 = 0.0;
        int st = validate_initial_dev(S, eo);
        if (!st) st = adaptive_gamma_dev(S, eo.overflow, g0);
        S.status = st;
        S.gamma = g0;
        adopt_density(S, eo);
      }
      __syncthreads();
      if (S.status) FAIL(S.status)
    }
    VLOOP stage_init(d, v, c.V, false, true);
    SYNC_OR_EXIT(PC_PRECOND)
    if (!c.eval_tail(c.X(), c.gX(), S.gamma, false, nullptr, eo)) {
      ok = false;
      goto out;
    }
    T0 {
      int st = validate_initial_dev(S, eo);
      for (int f = 0; f < S.K; ++f) {
        if (!S.fixed_e0) S.e0[f] = fmax(eo.energy[f], 1.0);
        if (!st && !(isfinite(S.e0[f]) && S.e0[f] > 0.0)) st = TEXO_GP_ERR_DENSITY_FIELD_CHANGED;
        S.inv_e0[f] = 1.0 / S.e0[f];
      }
      S.status = st;
      excess_dev(S, eo.overflow, S.best_max, S.best_tot);
      S.density_at_x = 1;
      S.phase = 1;
      S.a = 1.0;
      S.has_L = 0;
      if (!st && stop_dev(S, eo.overflow)) {
        S.phase = 2;
        S.converged = 1;
      } else if (!st && S.reset_mult) {
        S.status = area_multipliers_dev(S, eo);
      } else if (!st) {
        // initial_density_multiplier (eplace.rs:1126-1148)
        double dens = 0.0;
        for (int f = 0; f < S.K; ++f) dens += eo.rawl1[f];
        const double m0 = (eo.wal1 == 0.0 || dens == 0.0) ? 1.0 : S.init_weight * eo.wal1 / dens;
        if (!(isfinite(m0) && m0 > 0.0)) S.status = TEXO_GP_ERR_INVALID_NORMALIZATION;
        for (int f = 0; f < S.K; ++f) S.lambda[f] = m0;
        S.mstep = S.alpha_high - 1.0;
      }
      V.pending_best = 1;
      V.pending_prev = 1;
    }
    __syncthreads();
    if (S.status) FAIL(S.status)
    if (S.phase == 2) goto out;
  }

  // ---- outer loop -------------------------------------------------------
  for (;;) {
    T0 {
      V.action = ACT_NONE;
      if (stop_dev(S, S.cur_overflow)) {
        S.converged = 1;
        S.phase = 2;
      } else if (S.completed >= S.max_iterations) {
        S.exhausted = 1;
        S.phase = 2;
        S.status = S.best_effort ? TEXO_GP_OK : TEXO_GP_ERR_DID_NOT_CONVERGE;
      } else if (S.budget && done >= S.budget) {
        V.action = ACT_CONTINUE;   // leave with the loop still running
      } else {
        double gam = 0.0;
        const int st = adaptive_gamma_dev(S, S.cur_overflow, gam);
        if (st) {
          S.status = st;
          S.phase = 2;
        }
        S.gamma = gam;
        S.completed++;
        if (!isfinite(S.a) || S.a < 1.0) {
          S.status = TEXO_GP_ERR_INVALID_MOMENTUM_PARAMETER;
          S.phase = 2;
        }
        if (S.has_L && (!isfinite(S.L) || S.L <= 0.0)) {
          S.status = TEXO_GP_ERR_INVALID_LIPSCHITZ_ESTIMATE;
          S.phase = 2;
        }
      }
    }
    __syncthreads();
    if (S.phase == 2 || V.action == ACT_CONTINUE) break;
    ++done;

    // Phase 1: preconditioner (eplace.rs:1046-1100), pending copies, and the
    // origin evaluation's init. The origin is re-evaluated (eplace's closure
    // changes with gamma and the multipliers); its density side is reused
    // when the device already holds it for these coordinates.
    {
      const bool full = !S.density_at_x;
      VLOOP {
        stage_precond(d, S.lambda, r.p, v, c.V, sh);
        stage_init(d, v, c.V, full, true);
      }
      if (V.pending_best) c.copy(B.best, c.X(), d.U);
      if (V.pending_prev) c.copy(c.Xp(), c.X(), n);
      SYNC_OR_EXIT(PC_PRECOND)
      {
        const FoldJob jobs[3] = {{mslot(r.p, MS_PMIN), FOLD_DMIN}, {mslot(r.p, MS_PMAX), FOLD_DMAX},
                                 {islot(r.p, IS_PBAD), FOLD_ISUM}};
        c.fold(jobs, 3);
      }
      const double pmin = c.fv[0].d, pmax = c.fv[1].d;
      const long long pbad = c.fv[2].l;
      T0 {
        V.pmin = pmin;
        V.pmax = pmax;
        V.pending_best = 0;
        V.pending_prev = 0;
        if (pbad) S.status = TEXO_GP_ERR_INVALID_NORMALIZATION;
      }
      __syncthreads();
      if (S.status) FAIL(S.status)
      if (!c.eval_tail(c.X(), c.gX(), S.gamma, full, c.X(), eo)) {
        ok = false;
        goto out;
      }
      T0 {
        S.status = checked_dev(eo);
        if (full) adopt_density(S, eo);
        S.density_at_x = 1;
        V.restart = 0;
        V.has_wL = S.has_L;
        V.wL = S.L;
        V.trials = 0;
      }
      __syncthreads();
      if (S.status) FAIL(S.status)
    }

    // Phase 2: the dynamic Nesterov step (global_placement.rs:152-335)
    for (;;) {  // 'step
      T0 {
        const double m = V.restart ? 1.0 : S.a;
        const double s = sqrt(1.0 + 4.0 * m * m);
        V.next_m = fabs(s) <= 8.0e307 ? (1.0 + s) / 2.0 : 0.5 + s / 2.0;   // f64::midpoint(1, s)
        if (!isfinite(V.next_m)) S.status = TEXO_GP_ERR_ITERATION_OVERFLOW;
      }
      __syncthreads();
      if (S.status) FAIL(S.status)
      if (!V.restart) {
        const float e = (float)((S.a - 1.0) / V.next_m);
        VLOOP {
          stage_extrapolate(d, c.X(), c.Xp(), e, c.Y(), c.wset(), v, c.V, sh);
          stage_init(d, v, c.V, true, true);
        }
        SYNC_OR_EXIT(PC_EXTRAP)
        const long long diff = c.risum_prev(IS_DIFF);
        T0 V.y_is_origin = diff == 0;
        __syncthreads();
      } else {
        T0 V.y_is_origin = 1;
        __syncthreads();
      }
      if (V.y_is_origin) {
        T0 {
          V.f_y = eo.value;
          V.y_stat = eo.kkt;
        }
        __syncthreads();
      } else {
        if (!c.eval_tail(c.Y(), c.gY(), S.gamma, true, c.Y(), ey)) {
          ok = false;
          goto out;
        }
        T0 {
          S.density_at_x = 0;
          S.status = checked_dev(ey);
          V.f_y = ey.value;
          V.y_stat = ey.kkt;
        }
        __syncthreads();
        if (S.status) FAIL(S.status)
      }
      T0 {
        V.action = ACT_NONE;
        if (!isfinite(V.y_stat)) {
          S.status = TEXO_GP_ERR_LINE_SEARCH_OVERFLOW;
        } else if (V.y_stat == 0.0) {
          V.action = V.y_is_origin ? ACT_STATIONARY : ACT_RESTART;
          if (!V.y_is_origin) V.restart = 1;
        } else {
          V.tL = half_nonzero_dev(V.has_wL ? V.wL : V.y_stat);
          V.may_reduce = 1;
        }
      }
      __syncthreads();
      if (S.status) FAIL(S.status)
      if (V.action == ACT_RESTART) continue;
      if (V.action == ACT_NONE) {
        const float2* ybuf = V.y_is_origin ? c.X() : c.Y();
        const float2* gy = V.y_is_origin ? c.gX() : c.gY();
        for (;;) {  // line search
          T0 {
            V.action = ACT_NONE;
            V.trials++;
            if (V.trials > kMaxTrialsPerStep) {
              S.status = TEXO_GP_ERR_ITERATION_OVERFLOW;
            } else if (!isfinite(V.tL * V.pmax)) {
              S.status = TEXO_GP_ERR_LINE_SEARCH_OVERFLOW;
            } else if (V.tL * V.pmin == 0.0) {
              V.tL *= 2.0;
              V.may_reduce = 0;
              if (!isfinite(V.tL)) S.status = TEXO_GP_ERR_LINE_SEARCH_OVERFLOW;
              V.action = ACT_CONTINUE;
            }
          }
          __syncthreads();
          if (S.status) FAIL(S.status)
          if (V.action == ACT_CONTINUE) continue;
          // 1/L saturates at FLT_MAX: a huge step clamps to the box as it
          // does in FP64, where an infinite one would turn 0 * inf into NaN
          const float invL = (float)fmin(1.0 / V.tL, 3.0e38);
          VLOOP {
            stage_candidate(d, ybuf, gy, invL, c.C(), c.wset(), v, c.V, sh, c.X());
            stage_init(d, v, c.V, true, true);
          }
          SYNC_OR_EXIT(PC_CANDIDATE)
          {
            const Partials q = c.rset();
            const FoldJob jobs[3] = {{islot(q, IS_DIFF), FOLD_ISUM}, {pslot(q, SLOT_DOT), FOLD_DSUM},
                                     {pslot(q, SLOT_MSN), FOLD_DSUM}};
            c.fold(jobs, 3);
          }
          const long long changed = c.fv[0].l;
          const double dot = c.fv[1].d, msn = c.fv[2].d;
          T0 {
            V.action = ACT_NONE;
            if (changed == 0) {
              const double smaller = half_nonzero_dev(V.tL);
              if (V.may_reduce && smaller < V.tL) {
                V.tL = smaller;
                V.action = ACT_CONTINUE;
              } else if (!V.y_is_origin) {
                V.restart = 1;
                V.has_wL = 1;
                V.wL = V.tL;
                V.action = ACT_RESTART;
              } else {
                V.action = ACT_STATIONARY;
                S.has_L = 1;
                S.L = V.tL;
              }
            }
          }
          __syncthreads();
          if (V.action == ACT_CONTINUE) continue;
          if (V.action != ACT_NONE) break;
          if (!c.eval_tail(c.C(), c.gC(), S.gamma, true, c.C(), ec)) {
            ok = false;
            goto out;
          }
          T0 {
            S.density_at_x = 0;
            S.status = checked_dev(ec);
            const double upper = V.f_y + dot + 0.5 * V.tL * msn;
            if (!S.status && !isfinite(upper)) S.status = TEXO_GP_ERR_LINE_SEARCH_OVERFLOW;
            const bool smooth = ec.value <= upper + margin_dev(S, ec.value, upper);
            const bool mono = ec.value <= eo.value + margin_dev(S, ec.value, eo.value);
            if (smooth && mono) {
              V.action = ACT_ACCEPT;
              if (!isfinite(ec.kkt)) S.status = TEXO_GP_ERR_LINE_SEARCH_OVERFLOW;
              S.last_objective = ec.value;
            } else if (smooth && !V.restart) {
              V.restart = 1;
              V.has_wL = 1;
              V.wL = V.tL;
              V.action = ACT_RESTART;
            } else {
              V.tL *= 2.0;
              V.may_reduce = 0;
              if (!isfinite(V.tL)) S.status = TEXO_GP_ERR_LINE_SEARCH_OVERFLOW;
              V.action = ACT_CONTINUE;
            }
          }
          __syncthreads();
          if (S.status) FAIL(S.status)
          if (V.action != ACT_CONTINUE) break;
        }
      }
      if (V.action == ACT_RESTART) continue;
      // leave the step: accepted or numerically stationary
      T0 {
        S.trials += V.trials;
        if (V.action == ACT_ACCEPT) {
          const int oxp = S.ixp;
          S.ixp = S.ix;
          S.ix = S.ic;
          S.ic = oxp;
          const int og = S.igx;
          S.igx = S.igc;
          S.igc = og;
          S.a = V.next_m;
          S.has_L = 1;
          S.L = V.tL;
          S.density_at_x = 1;
          adopt_density(S, ec);
          V.stationary = 0;
        } else {
          S.a = 1.0;
          S.last_objective = eo.value;
          adopt_density(S, eo);
          V.pending_prev = 1;
          V.stationary = 1;
        }
      }
      __syncthreads();
      break;
    }

    // Phase 3: checkpoint, stop rules, multipliers (eplace.rs:550-573)
    T0 {
      double mx, tot;
      excess_dev(S, S.cur_overflow, mx, tot);
      if (mx < S.best_max || (mx == S.best_max && tot < S.best_tot)) {
        S.best_max = mx;
        S.best_tot = tot;
        V.pending_best = 1;
      }
      if (stop_dev(S, S.cur_overflow)) {
        S.converged = 1;
        S.phase = 2;
      } else if (!V.stationary) {
        S.have_prev_stationary = 0;
      }
    }
    __syncthreads();
    if (S.phase == 2) break;
    if (V.stationary) {
      // stationary_target_is_fixed (eplace.rs:973-985): compare rounded targets
      const float2* x = c.X();
      VLOOP {
        long long mism = 0;
        for (int u = v * blockDim.x + threadIdx.x; u < d.U; u += c.V * blockDim.x) {
          const float2 a = x[u];
          const uint32_t tx = (uint32_t)fminf(fmaxf(roundf(a.x), 0.f), (float)(S.W - 1));
          const uint32_t ty = (uint32_t)fminf(fmaxf(roundf(a.y), 0.f), (float)(S.H - 1));
          mism += (B.prev_targets[2 * u] != tx) + (B.prev_targets[2 * u + 1] != ty);
          B.prev_targets[2 * u] = tx;
          B.prev_targets[2 * u + 1] = ty;
        }
        write_partial(mism, islot(c.wset(), IS_DIFF), v, sh.l);
      }
      SYNC_OR_EXIT(PC_OTHER)
      const long long total = c.risum_prev(IS_DIFF);
      T0 {
        const bool fixed = S.have_prev_stationary && total == 0;
        S.have_prev_stationary = 1;
        if (fixed) {
          S.exhausted = 1;
          S.phase = 2;
          S.status = S.best_effort ? TEXO_GP_OK : TEXO_GP_ERR_DID_NOT_CONVERGE;
        }
      }
      __syncthreads();
      if (S.phase == 2) break;
    }
    T0 {
      const int st = update_multipliers_dev(S);
      if (st) {
        S.status = st;
        S.phase = 2;
      }
    }
    __syncthreads();
    if (S.phase == 2) break;
  }

out:
  // flush pending copies so the host sees the checkpoint and the state
  if (ok && (V.pending_best || V.pending_prev)) {
    if (V.pending_best) c.copy(B.best, c.X(), d.U);
    if (V.pending_prev) c.copy(c.Xp(), c.X(), n);
    ok = c.sync();
  }
  c.mark(PC_OTHER);
  __syncthreads();
  if (pb == 0) {
    if (threadIdx.x == 0) {
      S.barriers += c.nbar;
      for (int i = 0; i < 8; ++i) S.phase_ns[i] += clock[i];
      S.barrier_wait_ns += clock[9];
    }
    __syncthreads();
    copy_words(run, &S);
  }
#undef T0
#undef VLOOP
#undef SYNC_OR_EXIT
#undef FAIL
}

}  // namespace tgp
