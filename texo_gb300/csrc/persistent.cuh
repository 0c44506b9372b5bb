// persistent.cuh — state of the device-resident placement loop.
#pragma once
#include "../../include/texo_gp.h"
#include "kernels.cuh"

namespace tgp {

// Grid barrier words (device memory, zeroed before each launch).
struct GridBarrier {
  unsigned int count;
  unsigned int gen;
  int error;          // 1 when a bounded wait ran out
  int pad;
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
  // loop state (optimize_density_once, eplace.rs:439-582)
  int phase;                    // 0 fresh, 1 running, 2 finished
  int status;                   // texo_gp_status
  int converged, exhausted;
  unsigned completed;
  double lambda[kMaxFields], e0[kMaxFields], mstep, gamma;
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
  unsigned long long evaluations, trials, barriers;
  // per call
  unsigned budget;
};

struct Buffers {
  float2* pos[4];
  float2* grad[3];
  float2* best;
  uint32_t* prev_targets;
};

// Launches the persistent kernel for up to `budget` iterations; run lives in
// device memory and is copied to/from host_run around the launch.
int32_t launch_persistent(const Dev& d, const Reduce& r, const Buffers& b, DevRun* run_dev, DevRun* host_run,
                          GridBarrier* bar, int blocks, cudaStream_t s);
int persistent_blocks_per_sm();

}  // namespace tgp
