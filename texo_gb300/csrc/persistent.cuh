// persistent.cuh — state of the device-resident placement loop.
#pragma once
#include "../../include/texo_gp.h"
#include "kernels.cuh"

namespace tgp {

// Co-resident blocks per SM of the persistent kernels. One instance alone
// runs 1 per SM (up to 255 registers per thread; each instance has one
// virtual block per SM, so a single launch covers all of them): at 42k cells
// the loop is bound by its grid barriers and the FFT passes' latency, which
// fewer, larger blocks cut (measured on GB300: 3633 it/s with 1 per SM, 3254
// with 2, 2139 with 4). The batch kernel runs 4 per SM (64 registers): many
// latency-bound instances share the GPU, and more resident warps win over
// registers there (64 mixed jobs: 193 placements/s with 4 per SM against
// 146 with 2).
constexpr int kBlocksPerSm = 1;
constexpr int kBatchBlocksPerSm = 4;

// Grid barrier words (device memory, zeroed before each launch): an arrival
// counter and, on its own 128-byte line, the generation every waiter polls.
struct alignas(128) BarrierLine {
  unsigned int count;
  unsigned int pad[31];
};
struct GridBarrier {
  BarrierLine root;                         // arrivals
  unsigned int gen;                         // generation
  int error;                                // 1 when a bounded wait ran out
  unsigned int pad[30];
};

// Controller state of one placement, shared between the host and the
// persistent kernel: the host fills the inputs and the initial state; the
// kernel advances the loop and writes the state back when it returns.
struct DevRun {
  // inputs
  int K;
  unsigned max_iterations;
  int best_effort;
  int W, H;
  double beta, alpha_low, alpha_high, init_weight, gamma_base, margin_eps;
  double target[kMaxFields], gamma_weight[kMaxFields], real_area[kMaxFields];
  double inv_real_area[kMaxFields];   // 1 / real_area (FP64 division is slow on the device)
  double gamma_slope[kMaxFields];     // 2 / (1 - target) of field_wirelength_gamma
  double inv_gamma_weight_sum;        // 1 / sum of gamma_weight
  // one round of the area-adjustment loop (texo_gp_optimize_round): stop at
  // AreaAdjustmentReady (the area fields at 0.15) instead of the targets;
  // the density scales e0 given (not from the initial energy); the
  // multipliers from the area-reset formula
  int stop_mode, fixed_e0, reset_mult;
  int area_field[kMaxFields];         // LUT and register fields
  // loop state (optimize_density_once, eplace.rs:439-582)
  int phase;                    // 0 fresh, 1 running, 2 finished
  int status;                   // texo_gp_status
  int converged, exhausted;
  unsigned completed;
  double lambda[kMaxFields], e0[kMaxFields], inv_e0[kMaxFields], mstep, gamma;
  double best_max, best_tot;
  int have_prev_stationary, density_at_x;
  double cur_overflow[kMaxFields], cur_energy[kMaxFields], cur_force[kMaxFields];
  long long cur_overflow_fixed[kMaxFields];
  // Nesterov state (global_placement.rs:29-58)
  double a, L;
  int has_L;
  double last_objective;
  // buffer roles: indices into the position / gradient buffer tables
  int ix, ixp, iy, ic;
  int igx, igy, igc;
  // statistics
  unsigned long long evaluations, density_evaluations, trials, barriers;
  // grid-wide phase times seen by block 0 (ns): see PhaseClock
  unsigned long long phase_ns[8];
  unsigned long long barrier_wait_ns;
  // per call
  unsigned budget;
};

// The controller state and the grid barrier of one instance, side by side so
// that one copy each way moves both; the host keeps a pinned mirror of it.
struct RunBlock {
  DevRun run;
  alignas(256) GridBarrier bar;
};

// Phase categories of DevRun::phase_ns.
enum PhaseClock {
  PC_SCATTER_WA = 0,   // scatter + WA (or WA alone) up to its barrier
  PC_PREP = 1,
  PC_DCT = 2,          // the four transform GEMMs
  PC_GATHER = 3,       // gather + combine
  PC_PRECOND = 4,      // preconditioner / init / copies
  PC_EXTRAP = 5,       // extrapolation + init
  PC_CANDIDATE = 6,    // candidate + init
  PC_OTHER = 7
};

struct Buffers {
  float2* pos[4];
  float2* grad[3];
  float2* best;
  uint32_t* prev_targets;
};

// One instance of a batched launch (device memory).
struct InstDesc {
  Dev d;
  Reduce r;
  Buffers B;
  DevRun* run;
  GridBarrier* bar;
  int V;      // virtual blocks
  int pad;
};

// One step of the device engine on stream s: the pinned mirror `host` goes to
// `dev`, the persistent kernel runs up to run.budget iterations on `blocks`
// physical blocks over V virtual blocks, and `dev` comes back to `host`.
// The caller clears host->bar first and reads host->bar.error after a sync.
int32_t enqueue_persistent(const Dev& d, const Reduce& r, const Buffers& b, RunBlock* dev, RunBlock* host,
                           int blocks, int V, cudaStream_t s);
// The same step captured once as a CUDA graph (the kernel arguments are
// fixed for an instance), replayed with cudaGraphLaunch. Returns
// TEXO_GP_ERR_UNSUPPORTED, leaving *exec null, if the capture fails.
int32_t capture_persistent(const Dev& d, const Reduce& r, const Buffers& b, RunBlock* dev, RunBlock* host,
                           int blocks, int V, cudaStream_t s, cudaGraphExec_t* exec);
// enqueue_persistent on a cleared barrier, then a sync and the barrier check.
int32_t launch_persistent(const Dev& d, const Reduce& r, const Buffers& b, RunBlock* dev, RunBlock* host,
                          int blocks, int V, cudaStream_t s);
// Launches every instance of descs_dev at once; map_dev[b] = (instance,
// physical block, physical block count, 0). Asynchronous.
int32_t launch_batch(const InstDesc* descs_dev, const int4* map_dev, int blocks, bool large, cudaStream_t s);
int persistent_blocks_per_sm();
int batch_blocks_per_sm();

}  // namespace tgp
