// persistent.cu — the whole placement loop in one cooperative kernel.
//
// The kernel runs `optimize_density_once` (crates/texo-pnr/src/eplace.rs:439-582)
// with `dynamic_nesterov_step` (crates/texo-pnr/src/global_placement.rs:121-335)
// on the device. Stages are separated by a grid barrier; after each barrier
// every block reduces the partials it needs in the same fixed order, so all
// blocks hold bit-identical scalars and take the same branch. Thread 0 of each
// block keeps the controller state in shared memory; block 0 writes it back
// when the kernel returns. Every wait is bounded: a barrier that does not
// complete within its spin budget sets an error word, and every block then
// leaves the kernel at its next barrier.
#include <cmath>
#include <cstring>

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

__device__ __forceinline__ bool grid_sync(GridBarrier* b, unsigned nblocks, unsigned* gen, unsigned long long* count) {
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned g = *gen;
    __threadfence();
    const unsigned arrived = atomicAdd(&b->count, 1u) + 1u;
    if (arrived == nblocks) {
      atomicExch(&b->count, 0u);
      __threadfence();
      atomicAdd(&b->gen, 1u);
    } else {
      unsigned spins = 0;
      while (*(volatile unsigned*)&b->gen == g) {
        if (*(volatile int*)&b->error) break;
        if (++spins > kSpinLimit) {
          atomicExch(&b->error, 1);
          break;
        }
        __nanosleep(32);
      }
    }
    *gen = g + 1;
    ++*count;
    __threadfence();
  }
  __syncthreads();
  return *(volatile int*)&b->error == 0;
}

struct Ctx {
  const Dev& d;
  const Reduce& r;
  const Buffers& B;
  DevRun& S;          // shared memory, written by thread 0
  GridBarrier* bar;
  unsigned* gen;
  GemmShared& gsm;
  Shared& sh;
  double* rd;         // reduction scratch (shared)
  long long* rl;
  double* coef;       // shared [kMaxFields]
  int vb, nvb;
  bool large;
  unsigned long long nbar;

  __device__ bool sync() { return grid_sync(bar, (unsigned)nvb, gen, &nbar); }
  __device__ double rsum(int slot) { return block_reduce_array(pslot(r.p, slot), nvb, 0.0, OpAdd(), rd); }
  __device__ long long risum(int slot) { return block_reduce_array(islot(r.p, slot), nvb, 0ll, OpAdd(), rl); }
  __device__ long long rimin(int slot) {
    return block_reduce_array(islot(r.p, slot), nvb, 0x7fffffffffffffffll, OpMin(), rl);
  }
  __device__ double rmax(int slot) { return block_reduce_array(mslot(r.p, slot), nvb, 0.0, OpMax(), rd); }
  __device__ double rmin(int slot) { return block_reduce_array(mslot(r.p, slot), nvb, (double)INFINITY, OpMin(), rd); }
  __device__ float2* X() const { return B.pos[S.ix]; }
  __device__ float2* Xp() const { return B.pos[S.ixp]; }
  __device__ float2* Y() const { return B.pos[S.iy]; }
  __device__ float2* C() const { return B.pos[S.ic]; }
  __device__ float2* gX() const { return B.grad[S.igx]; }
  __device__ float2* gY() const { return B.grad[S.igy]; }
  __device__ float2* gC() const { return B.grad[S.igc]; }

  __device__ void copy(float2* dst, const float2* src, int n) {
    for (int i = vb * blockDim.x + threadIdx.x; i < n; i += nvb * blockDim.x) dst[i] = src[i];
  }

  // Objective evaluation at pos after an init phase and its barrier
  // (ContinuousProblem::evaluate + combined_objective, eplace.rs:137-205, 1022-1044).
  __device__ bool eval_tail(const float2* pos, float2* g, double gam, bool full, const float2* kkt_pos, ERec& out) {
    if (full) stage_scatter(d, pos, r.p, vb, nvb, sh);
    stage_wa(d, pos, gam, r.p, vb, nvb, sh);
    if (!sync()) return false;
    if (full) {
      stage_prep(d, r.p, nvb, vb, nvb, sh);
      if (!sync()) return false;
      for (int st = 0; st < 4; ++st) {
        stage_dct(d, st, large, r.p, vb, nvb, gsm, sh);
        if (!sync()) return false;
      }
      for (int f = 0; f < d.K; ++f) {
        const double e = rsum(SLOT_ENERGY + f);
        const long long ov = risum(IS_OVERFLOW + f);
        const long long nb = risum(IS_OVER_BINS + f);
        if (threadIdx.x == 0) {
          out.energy[f] = 0.5 * e;
          out.ovfix[f] = ov;
          out.bins[f] = nb;
          out.overflow[f] = ((double)ov * kInvFix) / S.real_area[f];
        }
      }
    } else if (threadIdx.x == 0) {
      for (int f = 0; f < d.K; ++f) {
        out.energy[f] = S.cur_energy[f];
        out.overflow[f] = S.cur_overflow[f];
        out.ovfix[f] = S.cur_overflow_fixed[f];
        out.bins[f] = 0;
      }
    }
    const double wa = rsum(SLOT_WA_VALUE);
    if (threadIdx.x == 0) {
      out.wa = wa;
      double value = wa;
      for (int f = 0; f < d.K; ++f) {
        const double ne = out.energy[f] / S.e0[f];
        value += S.lambda[f] * S.e0[f] * (ne + 0.5 * S.beta * ne * ne);
        coef[f] = S.lambda[f] * (1.0 + S.beta * ne);
      }
      out.value = value;
    }
    __syncthreads();
    if (full) stage_gather(d, pos, r.p, vb, nvb, sh);
    stage_combine(d, coef, g, r.p, vb, nvb, sh, kkt_pos);
    if (!sync()) return false;
    for (int f = 0; f < d.K; ++f) {
      const double a = rsum(SLOT_RAWL1 + f);
      const double b = rsum(SLOT_FORCE + f);
      if (threadIdx.x == 0) {
        out.rawl1[f] = a;
        out.force[f] = b;
      }
    }
    const double w = rsum(SLOT_WAL1);
    const long long bad = rimin(IS_BAD);
    const double kkt = kkt_pos ? rmax(MS_KKT) : 0.0;
    if (threadIdx.x == 0) {
      out.wal1 = w;
      out.bad = bad;
      out.kkt = kkt;
      S.evaluations++;
    }
    __syncthreads();
    return true;
  }
};

// ---- scalar rules (eplace.rs:1300-1415), evaluated by thread 0 ------------
__device__ int field_gamma_dev(double overflow, double target, double base, double& g) {
  if (!isfinite(overflow) || overflow < 0.0 || !(target >= 0.0 && target < 1.0) || !(base > 0.0))
    return TEXO_GP_ERR_INVALID_NORMALIZATION;
  const double slope = 2.0 / (1.0 - target), intercept = 1.0 - slope;
  g = base * pow(10.0, slope * overflow + intercept);
  return (isfinite(g) && g > 0.0) ? TEXO_GP_OK : TEXO_GP_ERR_INVALID_NORMALIZATION;
}
__device__ int adaptive_gamma_dev(const DevRun& S, const double* overflow, double& out) {
  double ws = 0.0, wsum = 0.0;
  for (int f = 0; f < S.K; ++f) {
    double g;
    const int st = field_gamma_dev(overflow[f], S.target[f], S.gamma_base, g);
    if (st) return st;
    ws += g * S.gamma_weight[f];
    wsum += S.gamma_weight[f];
  }
  out = wsum == 0.0 ? S.gamma_base : ws / wsum;
  return (isfinite(out) && out > 0.0) ? TEXO_GP_OK : TEXO_GP_ERR_INVALID_NORMALIZATION;
}
__device__ bool stop_dev(const DevRun& S, const double* overflow) {
  for (int f = 0; f < S.K; ++f)
    if (!(overflow[f] <= S.target[f])) return false;
  return true;
}
__device__ void excess_dev(const DevRun& S, const double* overflow, double& mx, double& tot) {
  mx = 0.0;
  tot = 0.0;
  for (int f = 0; f < S.K; ++f) {
    const double x = fmax(overflow[f] - S.target[f], 0.0);
    mx = fmax(mx, x);
    tot += x;
  }
}
__device__ int validate_initial_dev(const DevRun& S, const ERec& e) {
  bool ok = isfinite(e.wa) && e.bad == 0x7fffffffffffffffll;
  for (int f = 0; f < S.K && ok; ++f)
    ok = isfinite(e.energy[f]) && e.energy[f] >= 0.0 && isfinite(e.overflow[f]) && isfinite(e.force[f]) &&
         e.force[f] >= 0.0;
  return ok ? TEXO_GP_OK : TEXO_GP_ERR_INVALID_NORMALIZATION;
}
__device__ int checked_dev(const ERec& e) {
  if (!isfinite(e.value)) return TEXO_GP_ERR_INVALID_OBJECTIVE;
  if (e.bad != 0x7fffffffffffffffll) return TEXO_GP_ERR_NONFINITE_GRADIENT;
  return TEXO_GP_OK;
}
__device__ int update_multipliers_dev(DevRun& S, const ERec& e) {
  for (int f = 0; f < S.K; ++f)
    if (!isfinite(e.energy[f]) || !(S.e0[f] > 0.0)) return TEXO_GP_ERR_DENSITY_FIELD_CHANGED;
  double sg[kMaxFields], nn = 0.0;
  for (int f = 0; f < S.K; ++f) {
    const double ne = e.energy[f] / S.e0[f];
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
    const double ne = e.energy[f] / S.e0[f];
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
__device__ void adopt_density(DevRun& S, const ERec& e) {
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
enum { ACT_NONE = 0, ACT_RESTART, ACT_CONTINUE, ACT_ACCEPT, ACT_STATIONARY, ACT_ERROR };

__global__ void __launch_bounds__(kThreads, 2) k_persistent(Dev d, Reduce r, Buffers B, DevRun* run, GridBarrier* bar) {
  __shared__ DevRun S;
  __shared__ ERec eo, ey, ec;
  __shared__ StepVars V;
  __shared__ GemmShared gsm;
  __shared__ Shared sh;
  __shared__ double rd[kThreads / 32];
  __shared__ long long rl[kThreads / 32];
  __shared__ double coef[kMaxFields];
  __shared__ unsigned gen;
  if (threadIdx.x == 0) {
    S = *run;
    gen = *(volatile unsigned*)&bar->gen;
    V.pending_best = 0;
    V.pending_prev = 0;
  }
  __syncthreads();
  const bool large = (long long)((d.g.Wb + 31) / 32) * ((d.g.Hb + 31) / 32) >= 1024;
  Ctx c{d, r, B, S, bar, &gen, gsm, sh, rd, rl, coef, (int)blockIdx.x, (int)gridDim.x, large, 0ull};
  const int n = d.nobj;
  unsigned done = 0;
  bool ok = true;

#define T0 if (threadIdx.x == 0)
#define SYNC_OR_EXIT \
  if (!c.sync()) {   \
    ok = false;      \
    goto out;        \
  }
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
    stage_init(d, c.vb, c.nvb, true, true);
    SYNC_OR_EXIT
    if (!c.eval_tail(c.X(), c.gX(), S.gamma_base, true, nullptr, eo)) {
      ok = false;
      goto out;
    }
    {
      int st = 0;
      double g0 = 0.0;
      T0 {
        st = validate_initial_dev(S, eo);
        if (!st) st = adaptive_gamma_dev(S, eo.overflow, g0);
        S.status = st;
        S.gamma = g0;
        adopt_density(S, eo);
      }
      __syncthreads();
      if (S.status) FAIL(S.status)
    }
    stage_init(d, c.vb, c.nvb, false, true);
    SYNC_OR_EXIT
    if (!c.eval_tail(c.X(), c.gX(), S.gamma, false, nullptr, eo)) {
      ok = false;
      goto out;
    }
    T0 {
      int st = validate_initial_dev(S, eo);
      for (int f = 0; f < S.K; ++f) S.e0[f] = fmax(eo.energy[f], 1.0);
      S.status = st;
      excess_dev(S, eo.overflow, S.best_max, S.best_tot);
      S.density_at_x = 1;
      S.phase = 1;
      S.a = 1.0;
      S.has_L = 0;
      if (!st && stop_dev(S, eo.overflow)) {
        S.phase = 2;
        S.converged = 1;
      } else if (!st) {
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
        double gam;
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
      stage_precond(d, S.lambda, r.p, c.vb, c.nvb, sh);
      if (V.pending_best) c.copy(B.best, c.X(), d.U);
      if (V.pending_prev) c.copy(c.Xp(), c.X(), n);
      stage_init(d, c.vb, c.nvb, full, true);
      SYNC_OR_EXIT
      const double pmin = c.rmin(MS_PMIN), pmax = c.rmax(MS_PMAX);
      const long long pbad = c.risum(IS_PBAD);
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
        V.next_m = fabs(s) <= 8.0e307 ? (1.0 + s) / 2.0 : 0.5 + s / 2.0;
        if (!isfinite(V.next_m)) S.status = TEXO_GP_ERR_ITERATION_OVERFLOW;
      }
      __syncthreads();
      if (S.status) FAIL(S.status)
      if (!V.restart) {
        const double m = S.a;
        stage_extrapolate(d, c.X(), c.Xp(), (float)((m - 1.0) / V.next_m), c.Y(), r.p, c.vb, c.nvb, sh);
        stage_init(d, c.vb, c.nvb, true, true);
        SYNC_OR_EXIT
        const long long diff = c.risum(IS_DIFF);
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
          stage_candidate(d, ybuf, gy, (float)(1.0 / V.tL), c.C(), r.p, c.vb, c.nvb, sh, c.X());
          stage_init(d, c.vb, c.nvb, true, true);
          SYNC_OR_EXIT
          const long long changed = c.risum(IS_DIFF);
          const double dot = c.rsum(SLOT_DOT), msn = c.rsum(SLOT_MSN), change = c.rmax(MS_CHANGE);
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
              (void)change;
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
      V.action = ACT_NONE;
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
      long long mism = 0;
      const float2* x = c.X();
      for (int u = c.vb * blockDim.x + threadIdx.x; u < d.U; u += c.nvb * blockDim.x) {
        const float2 a = x[u];
        const uint32_t tx = (uint32_t)fminf(fmaxf(roundf(a.x), 0.f), (float)(S.W - 1));
        const uint32_t ty = (uint32_t)fminf(fmaxf(roundf(a.y), 0.f), (float)(S.H - 1));
        mism += (B.prev_targets[2 * u] != tx) + (B.prev_targets[2 * u + 1] != ty);
        B.prev_targets[2 * u] = tx;
        B.prev_targets[2 * u + 1] = ty;
      }
      write_partial(mism, islot(r.p, IS_DIFF), c.vb, sh.l);
      SYNC_OR_EXIT
      const long long total = c.risum(IS_DIFF);
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
      ERec tmp;
      for (int f = 0; f < S.K; ++f) tmp.energy[f] = S.cur_energy[f];
      const int st = update_multipliers_dev(S, tmp);
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
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    S.barriers += c.nbar;
    *run = S;
  }
#undef T0
#undef SYNC_OR_EXIT
#undef FAIL
}

int persistent_blocks_per_sm() {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_persistent, kThreads, 0) != cudaSuccess) return 0;
  return n;
}

int32_t launch_persistent(const Dev& d, const Reduce& r, const Buffers& b, DevRun* run_dev, DevRun* host_run,
                          GridBarrier* bar, int blocks, cudaStream_t s) {
  if (cudaMemcpyAsync(run_dev, host_run, sizeof(DevRun), cudaMemcpyHostToDevice, s) != cudaSuccess)
    return TEXO_GP_ERR_CUDA;
  if (cudaMemsetAsync(bar, 0, sizeof(GridBarrier), s) != cudaSuccess) return TEXO_GP_ERR_CUDA;
  Dev dd = d;
  Reduce rr = r;
  Buffers bb = b;
  void* args[] = {&dd, &rr, &bb, &run_dev, &bar};
  if (cudaLaunchCooperativeKernel((const void*)k_persistent, dim3(blocks), dim3(kThreads), args, 0, s) != cudaSuccess)
    return TEXO_GP_ERR_CUDA;
  note_launch();
  GridBarrier hb;
  if (cudaMemcpyAsync(host_run, run_dev, sizeof(DevRun), cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return TEXO_GP_ERR_CUDA;
  if (cudaMemcpyAsync(&hb, bar, sizeof(GridBarrier), cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return TEXO_GP_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return TEXO_GP_ERR_CUDA;
  if (hb.error) return TEXO_GP_ERR_DEVICE_TIMEOUT;
  return TEXO_GP_OK;
}

}  // namespace tgp
