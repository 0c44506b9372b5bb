/*
 * texo_oracle.h — TEST INFRASTRUCTURE ONLY.
 *
 * C API of the FP64 CPU restatement of Texo's electrostatic global placement
 * (the parity oracle). Only the test suite, the smoke check and the CPU
 * baseline leg of the benchmark load this library, and only as the checker or
 * as the timed CPU baseline; the product path never links or calls it.
 *
 * Every function restates the reference algorithm in the reference's
 * operation order; the citation next to each names the Rust source it
 * follows (paths relative to the texo repository).
 */
#ifndef TEXO_ORACLE_H
#define TEXO_ORACLE_H

#include <stdint.h>
#include "../include/texo_gp.h"

#ifdef __cplusplus
extern "C" {
#endif

/* quadratic_bspline_axis, electrostatic_placement.rs:950-976 */
void orc_bspline_axis(uint64_t length, double coordinate, uint64_t index[3], double weight[3],
                      double derivative[3]);
/* deposit_quadratic_bspline, electrostatic_placement.rs:900-916 */
void orc_deposit(double* density, uint64_t width, uint64_t height, double x, double y,
                 double charge);
/* sample_quadratic_bspline_with_gradient, electrostatic_placement.rs:919-941 */
void orc_sample(const double* potential, uint64_t width, uint64_t height, double x, double y,
                double out[3]);
/* deposit_bilinear / sample_bilinear_with_gradient, electrostatic_placement.rs:979-1027 */
void orc_deposit_bilinear(double* density, uint64_t width, uint64_t height, double x, double y,
                          double charge);
void orc_sample_bilinear(const double* potential, uint64_t width, uint64_t height, double x,
                         double y, double out[3]);

/* Poisson2d::solve (fast, electrostatic_placement.rs:725-776) when matrix == 0;
 * Poisson2d::solve_reference (matrix form, :780-859) when matrix != 0. */
int32_t orc_poisson(uint32_t width, uint32_t height, const double* density, double* potential,
                    double* energy, int32_t matrix);
/* orthonormal_dct2_basis, electrostatic_placement.rs:862-883 ([n][n], row = frequency) */
void orc_dct_basis(uint32_t n, double* basis);

/* ---- problem-level oracle ------------------------------------------------ */
typedef struct orc_handle_s* orc_handle;

typedef struct orc_field_result {
  uint32_t kind, lut_inputs;
  uint64_t available_capacity;
  uint64_t real_charge;
  double real_area, filler_charge, energy, normalized_overflow, net_charge, force_l1;
} orc_field_result;

/* Builds `ContinuousProblem` (eplace.rs:254-346). error_index receives the
 * offending unit/member/filler index for indexed errors. */
int32_t orc_create(const texo_gp_problem* problem, const texo_gp_params* params,
                   orc_handle* out, uint64_t* error_index);
void orc_destroy(orc_handle h);
void orc_sizes(orc_handle h, uint64_t* units, uint64_t* fillers, uint64_t* coordinates,
               uint32_t* bins_x, uint32_t* bins_y, uint32_t* num_fields);
void orc_initial(orc_handle h, double* coordinates, double* lower, double* upper);
void orc_fillers(orc_handle h, uint32_t* field, double* charge, double* xy);
/* Overrides one filler's charge (to reproduce the reference's typed-error tests). */
void orc_set_filler_charge(orc_handle h, uint64_t filler, double charge);
/* Discrete capacity after fixed occupancy, [bins_tile] for one field. */
void orc_capacity(orc_handle h, uint32_t field, uint32_t* out);

/* ContinuousProblem::evaluate at coordinates [2(U+F)] (eplace.rs:137-205).
 * Optional arrays (NULL to skip): wa_gradient [2U]; field_gradient
 * [K][2(U+F)] raw; density [K][B]; potential [K][B]. threads: 1 = serial,
 * >1 = the reference's fork-join shape on std::thread. */
int32_t orc_evaluate(orc_handle h, const double* coordinates, double gamma, int32_t threads,
                     double* wa_value, orc_field_result* fields, double* wa_gradient,
                     double* field_gradient, double* density, double* potential,
                     uint64_t* error_index);
/* The device's fixed-point scatter restated on the CPU: FP32 taps, int64
 * 2^-32 accumulation; grids [K][B]. Also returns per-field positive overflow
 * (fixed point) and overflowed-bin counts. */
int32_t orc_scatter_fixed(orc_handle h, const double* coordinates, int64_t* physical,
                          int64_t* fillers, int64_t* overflow_fixed, uint64_t* overflow_bins);

/* Runs `optimize_density_once` + `place` (Final criterion). threads as above;
 * max_iterations (0 = params) caps this call. Returns the status; targets [2U],
 * coordinates [2(U+F)] optional. */
typedef struct orc_run_stats {
  uint32_t iterations;
  uint64_t evaluations;
  uint64_t line_search_trials;
  uint32_t num_fields;
  double overflow[TEXO_GP_MAX_FIELDS];
  double gamma;
  double objective;
  uint32_t converged;
  uint32_t exhausted;
  int32_t inner_status;
  double hpwl;
} orc_run_stats;
int32_t orc_place(orc_handle h, int32_t threads, uint32_t max_iterations, uint32_t* targets,
                  double* coordinates, orc_run_stats* stats);
/* One round of eplace::place's area-adjustment loop (optimize_density_once,
 * eplace.rs:439-582): stop 0 = final targets, 1 = AreaAdjustmentReady (LUT
 * and register overflow <= 0.15); reset_multipliers = elfPlace eqs. (27)-(28)
 * after an area adjustment; density_scales (NULL = from this round's initial
 * energies); completed_iterations of earlier rounds (the cap counts all). */
typedef struct orc_round {
  int32_t stop;
  int32_t reset_multipliers;
  const double* density_scales;
  uint64_t completed_iterations;
} orc_round;
typedef struct orc_round_result {
  uint64_t completed_iterations;
  uint32_t exhausted;
  double density_scales[TEXO_GP_MAX_FIELDS];
} orc_round_result;
/* Member charges (the problem's member order) and filler charges; either may
 * be NULL. */
int32_t orc_set_charges(orc_handle h, const double* member_charge, const double* filler_charge);
/* Runs one round from coordinates_in [2(U+F)] (NULL: the initial ones). */
int32_t orc_place_round(orc_handle h, int32_t threads, const orc_round* round, const double* coordinates_in,
                        uint32_t* targets, double* coordinates, orc_run_stats* stats, orc_round_result* result);

/* The controller records of the last orc_place (one per completed iteration,
 * the first 4096): copies up to `capacity`, returns how many there are. */
uint32_t orc_trace(orc_handle h, texo_gp_iteration* out, uint32_t capacity);
/* The same loop restarted from the handle's initial state, running exactly
 * `iterations` outer iterations (for timing a bounded sample). */
int32_t orc_hpwl(orc_handle h, const double* coordinates, double* hpwl);

/* Preconditioners (analytical_placement.rs:177-231). */
void orc_wirelength_preconditioner(orc_handle h, double* out_units);
void orc_cell_incidence_weights(orc_handle h, double* out_cells);

/* ---- Nesterov step with a caller-supplied evaluator ----------------------
 * dynamic_nesterov_step, global_placement.rs:121-335. The callback returns 0
 * on success or a nonzero error, which the step reports as
 * TEXO_GP_ERR_EVALUATION with the callback's code in out->inner. */
typedef int32_t (*orc_eval_cb)(void* user, const double* coordinates, uint64_t n, double* value,
                               double* gradient, uint64_t* gradient_len, int64_t* payload);
typedef struct orc_nesterov_state {
  double* coordinates;            /* [n] */
  double* previous;               /* [n] */
  uint64_t n;
  double momentum;
  int32_t has_lipschitz;
  double lipschitz;
} orc_nesterov_state;
typedef struct orc_step_out {
  int32_t stationary;             /* 0 Accepted, 1 NumericallyStationary */
  double objective, stationarity, coordinate_change;
  uint64_t trials;
  int64_t payload;
  int32_t inner;
  uint64_t error_index;
  uint64_t expected, actual;
} orc_step_out;
int32_t orc_nesterov_step(orc_nesterov_state* state, const double* lower, uint64_t lower_len,
                          const double* upper, uint64_t upper_len, const double* metric,
                          uint64_t metric_len, orc_eval_cb cb, void* user, orc_step_out* out);
/* DynamicNesterovState::new (global_placement.rs:38-53): projects when possible. */
void orc_nesterov_init(orc_nesterov_state* state, const double* initial, const double* lower,
                       uint64_t lower_len, const double* upper, uint64_t upper_len);
double orc_box_metric_kkt(const double* gradient, const double* coordinates, const double* lower,
                          const double* upper, const double* metric, uint64_t n);

/* ---- eplace scalar rules (eplace.rs) ------------------------------------ */
void orc_augmented(double energy, double initial_energy, double multiplier, double beta,
                   double* value, double* coefficient);                  /* :1111-1124 */
int32_t orc_multiplier_growth(double logarithm, double low, double high, double* growth); /* :1286-1298 */
int32_t orc_area_adjusted_multiplier_step(const double* multipliers, uint64_t n, double high,
                                          double* step);                 /* :1220-1232 */
int32_t orc_field_gamma(double overflow, double target, double base, double* gamma); /* :1349-1367 */
int32_t orc_weighted_gamma_mean(const double* gammas, const double* weights, uint64_t n,
                                double fallback, double* mean);          /* :1369-1395 */
double orc_overflow_target(uint32_t kind);                              /* :1300-1308 */
int32_t orc_area_adjustment_ready(uint32_t K, const uint32_t* kinds, const double* overflow); /* :1403-1408 */
int32_t orc_area_adjusted_multipliers(uint32_t K, const double* energy, const double* force_l1,
                                      const double* initial_energies, double beta, const double* wa_gradient_xy,
                                      uint64_t units, double* out);      /* :1183-1218 */
int32_t orc_checkpoint_better(double max_excess, double total_excess, double best_max,
                              double best_total);                       /* :106-119 */
int32_t orc_validate_units(const uint32_t* member_ptr, uint64_t units, uint64_t* error_index);

/* continuous_routing_demand (eplace.rs:856-937): returns 0, or 1 for a
 * non-finite / unordered box (InvalidNormalization). */
int32_t orc_routing_demand(uint32_t width, uint32_t height, uint64_t num_boxes, const double* boxes,
                           double* horizontal, double* vertical);

/* ---- coarse quadratic seed (crates/texo-pnr/src/lib.rs:4586-4790) -------- */
typedef struct orc_pcg_stats {
  uint64_t iterations, restarts;
  int32_t stop;                 /* 0 residual, 1 breakdown, 2 dimension */
  int32_t converged;
  double initial_residual_squared, target_squared, final_residual_squared;
} orc_pcg_stats;
/* solve_quadratic: Jacobi-preconditioned CG for (D - W) x = b, W in CSR rows
 * in the reference's adjacency order; `solution` is the initial guess and the
 * result. Returns 0, or 1 when the true final residual misses the target. */
int32_t orc_solve_quadratic(uint64_t n, const double* diagonal, const uint32_t* ptr, const uint32_t* index,
                            const double* weight, const double* rhs, double* solution, orc_pcg_stats* stats);
/* multiply_quadratic (lib.rs:4767-4782) */
void orc_multiply_quadratic(uint64_t n, const double* diagonal, const uint32_t* ptr, const uint32_t* index,
                            const double* weight, const double* values, double* product);

/* ---- legalization: the capacity auction (auction_oracle.cpp) ------------- */
typedef struct orc_auction_stats {
  uint64_t bids, examined, unmatched, total_base_cost;
} orc_auction_stats;
/* assign_implicitly (legalization/auction.rs:131-247) driven by the explicit
 * best-two search of the reference's tests (auction.rs:253-272), base costs
 * multiplied by `cost_scale` (1 in the reference). Returns 0 or a
 * TEXO_GP_ERR_AUCTION_* code; `prices` (may be NULL) gets m prices. With
 * `rounds` NULL the bidders bid one at a time from the FIFO queue (the
 * reference); otherwise all active bidders bid each round (the GPU's rule)
 * and *rounds receives the number of rounds. */
int32_t orc_auction_explicit(uint32_t n, uint32_t m, uint64_t max_base_cost, uint32_t cost_scale,
                             const uint32_t* ptr, const uint32_t* object, const uint64_t* cost,
                             int32_t* assignment, uint64_t* prices, orc_auction_stats* stats,
                             uint64_t* rounds);
/* auction_singletons (legalization/mod.rs:657-677, 733-840) with the ring
 * walk of best_objects_on_cached_rings (mod.rs:876-1021); the layout of
 * texo_gp_auction_singletons. */
int32_t orc_auction_singletons(uint32_t width, uint32_t height, uint32_t num_kinds, const uint32_t* tile_ptr,
                               const uint32_t* tile_object, uint32_t num_objects, const uint8_t* occupied,
                               uint32_t num_bidders, const uint32_t* bidder_kind, const uint32_t* target_xy,
                               uint32_t cost_scale, int32_t* assignment, uint64_t* prices,
                               orc_auction_stats* stats, uint64_t* rounds);
/* The epsilon-complementary-slackness certificate of a singleton result:
 * returns the number of violations (-1 for malformed input); `dual_bound`
 * (may be NULL) the assignment dual at these prices, a lower bound on the
 * least total cost with dummies at n * max_base_cost + n + 1. */
int64_t orc_auction_check_singletons(uint32_t width, uint32_t height, uint32_t num_kinds, const uint32_t* tile_ptr,
                                     const uint32_t* tile_object, uint32_t num_objects, const uint8_t* occupied,
                                     uint32_t num_bidders, const uint32_t* bidder_kind, const uint32_t* target_xy,
                                     uint32_t cost_scale, const int32_t* assignment, const uint32_t* prices,
                                     uint64_t* base_costs,
                                     uint64_t* first_bad, int64_t* dual_bound);

/* ---- routability: register clustering (routability_oracle.cpp) ----------- */
/* clustering_areas (register_clustering.rs:17-80): 0, or
 * TEXO_GP_ERR_INVALID_NORMALIZATION where the reference returns None. */
int32_t orc_register_clustering_areas(uint64_t n, const double* xy, const uint64_t* clock_lsr, const uint64_t* ce,
                                      uint64_t movable_instance_count, double* areas);
/* soft_division_ceiling (register_clustering.rs:89-97) */
double orc_soft_division_ceiling(double value, double divisor);

#ifdef __cplusplus
}
#endif
#endif
