/*
 * texo_gp.h — C ABI of the GB300 electrostatic global-placement engine.
 *
 * This library replaces one stage of the Texo place-and-route flow: the
 * elfPlace/ePlace electrostatic global placement `eplace::place`
 * (crates/texo-pnr/src/eplace.rs:242-421) together with everything it calls on
 * its hot path:
 *   - the dynamic preconditioned Nesterov step
 *     (crates/texo-pnr/src/global_placement.rs:121-335),
 *   - the quadratic-B-spline electrostatic density model and its spectral
 *     Poisson solve (crates/texo-pnr/src/electrostatic_placement.rs:130-441,
 *     602-776, 895-976),
 *   - the weighted-average (WA) hypernet wirelength
 *     (crates/texo-pnr/src/analytical_placement.rs:366-463, 520-703).
 *
 * The reference function is crate-private Rust with no FFI. The entry points
 * below are what a Rust caller (`analytical_place`,
 * crates/texo-pnr/src/lib.rs:4129-4143) would bind through `extern "C"`:
 * plain pointers and sizes, caller-owned host arrays, no allocation visible to
 * the caller except the opaque handles created here.
 *
 * Coordinates are tile (site) coordinates, exactly as in the reference: the
 * optimizer vector is [x0, y0, x1, y1, ...] over all placement units followed
 * by one (x, y) pair per density filler.
 *
 * All functions are synchronous with respect to the caller. A handle owns one
 * CUDA stream; distinct handles are independent and may be driven from
 * different host threads. Results are bit-for-bit deterministic run to run.
 */
#ifndef TEXO_GP_H
#define TEXO_GP_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TEXO_GP_ABI_VERSION 1u

/* ------------------------------------------------------------------------ */
/* Status codes: one per variant of the reference's error enums.            */
/* ------------------------------------------------------------------------ */
typedef enum texo_gp_status {
  TEXO_GP_OK = 0,
  /* ElectrostaticError, crates/texo-pnr/src/electrostatic_placement.rs:15-69 */
  TEXO_GP_ERR_EMPTY_GRID = 1,
  TEXO_GP_ERR_GRID_TOO_LARGE = 2,
  TEXO_GP_ERR_DENSITY_LENGTH = 3,
  TEXO_GP_ERR_NONFINITE_DENSITY = 4,
  TEXO_GP_ERR_EMPTY_UNIT = 5,
  TEXO_GP_ERR_NONFINITE_UNIT_COORDINATE = 6,
  TEXO_GP_ERR_INVALID_MEMBER_CHARGE = 7,
  TEXO_GP_ERR_POINT_OUTSIDE_GRID = 8,
  TEXO_GP_ERR_FIXED_CAPACITY_EXHAUSTED = 9,
  TEXO_GP_ERR_INSUFFICIENT_CAPACITY = 10,
  TEXO_GP_ERR_INSUFFICIENT_AREA = 11,
  TEXO_GP_ERR_NONFINITE_FILLER = 12,
  TEXO_GP_ERR_NEGATIVE_FILLER_CHARGE = 13,
  TEXO_GP_ERR_UNEXPECTED_FILLER_KIND = 14,
  TEXO_GP_ERR_FILLER_CHARGE_MISMATCH = 15,
  /* NesterovError, crates/texo-pnr/src/global_placement.rs:80-109 */
  TEXO_GP_ERR_INVALID_BOUNDS = 32,
  TEXO_GP_ERR_INVALID_METRIC_LENGTH = 33,
  TEXO_GP_ERR_NONPOSITIVE_METRIC = 34,
  TEXO_GP_ERR_INVALID_INITIAL_COORDINATE = 35,
  TEXO_GP_ERR_INVALID_MOMENTUM_PARAMETER = 36,
  TEXO_GP_ERR_INVALID_LIPSCHITZ_ESTIMATE = 37,
  TEXO_GP_ERR_INVALID_OBJECTIVE = 38,
  TEXO_GP_ERR_INVALID_GRADIENT_LENGTH = 39,
  TEXO_GP_ERR_NONFINITE_GRADIENT = 40,
  TEXO_GP_ERR_LINE_SEARCH_OVERFLOW = 41,
  TEXO_GP_ERR_ITERATION_OVERFLOW = 42,
  TEXO_GP_ERR_EVALUATION = 43,
  /* EplaceError, crates/texo-pnr/src/eplace.rs:27-38 */
  TEXO_GP_ERR_DENSITY_FIELD_CHANGED = 64,
  TEXO_GP_ERR_INVALID_NORMALIZATION = 65,
  TEXO_GP_ERR_DID_NOT_CONVERGE = 66,
  /* Errors of this boundary itself (no reference counterpart). */
  TEXO_GP_ERR_INVALID_ARGUMENT = 96,
  TEXO_GP_ERR_CUDA = 97,
  TEXO_GP_ERR_OUT_OF_MEMORY = 98,
  TEXO_GP_ERR_DEVICE_TIMEOUT = 99,   /* a bounded device-side wait ran out */
  TEXO_GP_ERR_FIXED_POINT_RANGE = 100, /* a weight or charge exceeds the int64 accumulator range */
  TEXO_GP_ERR_UNSUPPORTED = 101,
  TEXO_GP_ERR_BUSY = 102,
  /* PnrError::InvalidPlacement of the coarse quadratic seed: "analytical PCG
   * {breakdown|dimension} after i/n iterations" (crates/texo-pnr/src/lib.rs:4702-4752) */
  TEXO_GP_ERR_PCG_NOT_CONVERGED = 110,
  /* AuctionError (crates/texo-pnr/src/legalization/auction.rs:46-54) */
  TEXO_GP_ERR_AUCTION_RANGE = 111,            /* ArithmeticOverflow: the price range does not fit */
  TEXO_GP_ERR_AUCTION_OBJECT_RANGE = 112,     /* ObjectOutOfRange */
  TEXO_GP_ERR_AUCTION_COST_RANGE = 113,       /* BaseCostOutOfRange */
  TEXO_GP_ERR_AUCTION_DUPLICATE_OBJECT = 114, /* DuplicateBestObject: an object twice in one domain */
  /* InstanceAreaError (crates/texo-pnr/src/instance_area.rs:56-62) */
  TEXO_GP_ERR_INSTANCE_AREA_MEMBER = 115,       /* InvalidMemberArea { member } (error_index) */
  TEXO_GP_ERR_INSTANCE_AREA_FILLER = 116,       /* InvalidFillerArea { filler } (error_index) */
  TEXO_GP_ERR_INSTANCE_AREA_POSTCONDITION = 117,/* PostconditionViolation */
  TEXO_GP_ERR_INSTANCE_AREA_OVERFLOW = 118,     /* ArithmeticOverflow */
  /* PnrError::InvalidPlacement of `project` (legalization/mod.rs:391-430,
   * 679-722): fixed units on one BEL, or an auction result on a taken BEL */
  TEXO_GP_ERR_PROJECTION_CONFLICT = 119,
  /* legalization::repair (repair.rs) */
  TEXO_GP_ERR_NO_BEL = 120                    /* PnrError::NoBel { cell }: no legal completion exists */
} texo_gp_status;

/* Resource kinds in the reference's `ResourceKind` order
 * (crates/texo-model/src/lib.rs:69-87). Only LUT, REGISTER and MEMORY are
 * density fields (`density_kind_is_exchangeable`, eplace.rs:1417-1422). */
typedef enum texo_gp_kind {
  TEXO_GP_KIND_LOGIC = 0,
  TEXO_GP_KIND_LUT = 1,
  TEXO_GP_KIND_REGISTER = 2,
  TEXO_GP_KIND_MEMORY = 3,
  TEXO_GP_KIND_CLOCK = 4,
  TEXO_GP_KIND_IO = 5,
  TEXO_GP_KIND_CONSTANT = 6,
  TEXO_GP_KIND_DSP = 7
} texo_gp_kind;

/* One density field (one exchangeable resource kind). Fields must be listed
 * in ascending (kind, lut_inputs) order, which is the reference's BTreeMap
 * order; fields without any member are ignored, as in the reference. */
typedef struct texo_gp_field {
  uint32_t kind;         /* texo_gp_kind */
  uint32_t lut_inputs;   /* ResourceKind::Lut(k) payload; 0 otherwise */
} texo_gp_field;

/* Flattened `eplace::place` inputs (eplace.rs:242-253 and the data it reads
 * from `Device`, `PlacementUnit` and `AnalyticalHypergraph`). All arrays are
 * caller-owned and only read during texo_gp_create / texo_gp_place. */
typedef struct texo_gp_problem {
  uint32_t width, height;            /* Device::width/height: the tile grid */
  uint32_t num_fields;
  const texo_gp_field* fields;       /* [num_fields] */
  const uint32_t* capacity;          /* [num_fields][width*height] BELs per tile */
  uint32_t num_fixed_occupancy;      /* exchangeable BELs held by fixed units */
  const uint32_t* fixed_occupancy;   /* [num_fixed_occupancy][3] = field, x, y */

  uint32_t num_units;                /* all PlacementUnits, movable and fixed */
  const double* initial_xy;          /* [2U] initial_x/initial_y interleaved */
  const double* lower_xy;            /* [2U] choice_bounds (eplace.rs:1470-1481) */
  const double* upper_xy;            /* [2U]; fixed units have lower == upper */
  const uint32_t* member_ptr;        /* [U+1] CSR of density members per unit */
  const uint32_t* member_field;      /* [members] index into fields */
  const double* member_offset_xy;    /* [2*members] offset from the unit origin */
  const double* member_charge;       /* [members] physical area (1.0 by default) */
  const uint32_t* member_cell;       /* [members] logical cell of the member */

  uint32_t num_cells;
  const uint32_t* cell_unit;         /* [cells] unit_by_cell */
  const double* cell_offset_xy;      /* [2*cells] macro_offset_by_cell */
  const uint8_t* cell_fixed;         /* [cells] 1 when fixed_coordinates[cell] is Some */
  const double* cell_fixed_xy;       /* [2*cells] fixed coordinate (read when fixed) */

  uint32_t num_nets;                 /* hypernets with >= 2 pins, driver first */
  const uint32_t* net_ptr;           /* [E+1] */
  const uint32_t* pin_cell;          /* [P] */
  uint32_t num_timed_arcs;
  const uint32_t* arc_driver_cell;   /* [A] */
  const uint32_t* arc_sink_cell;     /* [A] */
  const uint64_t* arc_extra_weight;  /* [A] sink weight - 1 (> 0) */
} texo_gp_problem;

/* DCT forms for the spectral Poisson solve. */
typedef enum texo_gp_dct_mode {
  TEXO_GP_DCT_FP32 = 0,      /* FP32: FFT-based transforms on power-of-two grids, else the GEMM form */
  TEXO_GP_DCT_TENSOR = 1,    /* tcgen05 tensor cores: the BF16x3 split carried to four 8-bit integer
                                slices per value, ten slice products accumulated exactly in FP32 */
  TEXO_GP_DCT_BF16X3 = TEXO_GP_DCT_TENSOR,   /* earlier name of the same mode */
  TEXO_GP_DCT_FP32_GEMM = 2  /* FP32 compensated GEMM against the cosine matrices on every grid */
} texo_gp_dct_mode;

/* Density scatter forms of the host engine (the device engine always runs the
 * direct form). Both give the same int64 fixed-point grids bit for bit. */
typedef enum texo_gp_scatter_mode {
  TEXO_GP_SCATTER_AUTO = 0,     /* the direct form; with autotune = 1 the faster of the two, timed at
                                   creation */
  TEXO_GP_SCATTER_DIRECT = 1,   /* nine global int64 atomics per object */
  TEXO_GP_SCATTER_TILED = 2     /* objects sorted by 32 x 32-bin tile, taps accumulated in a shared-
                                   memory window per run, one global atomic per touched bin */
} texo_gp_scatter_mode;

/* Controller forms. */
typedef enum texo_gp_engine {
  TEXO_GP_ENGINE_HOST = 0,      /* host-driven line search, one sync per evaluation */
  TEXO_GP_ENGINE_DEVICE = 1     /* whole eplace loop in one persistent cooperative kernel */
} texo_gp_engine;

/* Parameters. texo_gp_default_params() returns the reference constants
 * (eplace.rs:125-134), under which the engine reduces to reference
 * semantics. The bin-grid, target-density and gamma-unit fields are
 * extensions for grids that differ from the tile grid. */
typedef struct texo_gp_params {
  double gamma_base;             /* ePlace gamma base in bin widths (8.0) */
  uint32_t max_iterations;       /* MAX_EPLACE_ITERATIONS (3000) */
  double beta;                   /* AUGMENTED_DENSITY_BETA (2000) */
  double initial_density_weight; /* INITIAL_DENSITY_WEIGHT (1e-4) */
  double alpha_low, alpha_high;  /* MULTIPLIER_ALPHA_LOW/HIGH (1.05, 1.06) */
  double overflow_target_override; /* < 0: per-kind targets (0.10 / 0.20) */
  uint32_t bins_x, bins_y;       /* density grid; 0 = the tile grid */
  double target_density;         /* 1.0 = reference semantics */
  int32_t best_effort;           /* keep the best checkpoint instead of DidNotConverge */
  int32_t dct_mode;              /* texo_gp_dct_mode */
  int32_t engine;                /* texo_gp_engine */
  int32_t device;                /* CUDA device ordinal */
  double objective_margin_ulps;  /* line-search rounding margin: max(eps64, ulps * 2^-24) (1 + |a| + |b|) */
  int32_t autotune;              /* 1: time the DCT forms on this instance at creation and keep the
                                    fastest (FP32 GEMM with 16x16 or 64x64 tiles, FP32 FFT on
                                    power-of-two grids; with dct_mode TENSOR also the tensor-core
                                    form, which may give way to the more accurate FP32 forms), and
                                    with the host engine and scatter_mode AUTO also the two scatter
                                    forms, at spread coordinates */
  int32_t scatter_mode;          /* texo_gp_scatter_mode: how the host engine deposits the density */
  uint32_t reserved[6];
} texo_gp_params;

#define TEXO_GP_MAX_FIELDS 4

/* Per-call results; filled by texo_gp_place / texo_gp_run. */
typedef struct texo_gp_stats {
  int32_t status;                /* texo_gp_status of the call */
  uint32_t iterations;           /* completed eplace iterations */
  uint64_t evaluations;          /* objective evaluations */
  uint64_t line_search_trials;
  uint32_t num_fields;
  double overflow[TEXO_GP_MAX_FIELDS];  /* normalized positive overflow per field */
  double energy[TEXO_GP_MAX_FIELDS];
  double gamma;                  /* last global gamma */
  double objective;              /* last accepted combined objective */
  double hpwl;                   /* HPWL of the final continuous coordinates */
  uint64_t error_index;          /* first offending index for indexed errors */
  uint32_t error_field;
  uint32_t converged;            /* 1 when every field reached its target */
  double elapsed_ms;             /* device time of the call (CUDA events on the handle's stream; for
                                    the device engine, around its one step: state in, kernel, state out) */
  uint64_t kernel_launches;      /* kernels this library launched during the call */
  uint64_t density_evaluations;  /* evaluations that rebuilt the density side (scatter, Poisson
                                    solve, field gather); the others reused it for the same
                                    coordinates and ran the wirelength side alone */
} texo_gp_stats;

/* One evaluation of the objective components at given coordinates
 * (`ContinuousProblem::evaluate`, eplace.rs:137-205). */
typedef struct texo_gp_field_eval {
  double energy;                 /* 1/2 <rho - mean, phi> */
  double normalized_overflow;    /* physical positive overflow / real area */
  double net_charge;             /* sum of the density grid */
  double force_l1;               /* sum_members q (|gx| + |gy|) */
  double real_area;
  double filler_charge;
  int64_t overflow_fixed;        /* positive overflow, 2^-32 fixed point (device form) */
  uint64_t overflow_bins;        /* bins with positive physical overflow */
} texo_gp_field_eval;

typedef struct texo_gp_eval {
  double wirelength;             /* WA value, baseline + timing overlays */
  uint32_t num_fields;
  texo_gp_field_eval fields[TEXO_GP_MAX_FIELDS];
} texo_gp_eval;

typedef struct texo_gp_handle_s* texo_gp_handle;

/* ---- version / defaults ------------------------------------------------- */
uint32_t texo_gp_abi_version(void);
void texo_gp_default_params(texo_gp_params* out);
const char* texo_gp_status_name(int32_t status);
/* Last CUDA error text seen by this thread (for TEXO_GP_ERR_CUDA). */
const char* texo_gp_last_error(void);

/* ---- one-shot drop-in ----------------------------------------------------
 * Replaces `eplace::place` (eplace.rs:242-421) with routing_capacity = None:
 * builds the density model, fillers and bounds, runs the augmented-Lagrangian
 * Nesterov loop and writes the best checkpoint's rounded unit targets
 * (`rounded_targets_from_coordinates`, eplace.rs:954-971) to out_targets_xy
 * [2U]. out_coordinates [2(U+F)] (optional, may be NULL) receives the final
 * continuous coordinates. */
int32_t texo_gp_place(const texo_gp_problem* problem, const texo_gp_params* params,
                      uint32_t* out_targets_xy, double* out_coordinates,
                      texo_gp_stats* stats);

/* ---- device-resident handle ----------------------------------------------
 * create = `DensityModel::new` + `initial_fillers` +
 * `initial_coordinates_and_bounds` (eplace.rs:312-318); device buffers are
 * allocated once here. */
int32_t texo_gp_create(const texo_gp_problem* problem, const texo_gp_params* params,
                       texo_gp_handle* out);
int32_t texo_gp_destroy(texo_gp_handle h);
/* Sizes: units, fillers, optimizer coordinates (2(U+F)), bin grid. */
int32_t texo_gp_sizes(texo_gp_handle h, uint64_t* units, uint64_t* fillers,
                      uint64_t* coordinates, uint32_t* bins_x, uint32_t* bins_y,
                      uint32_t* num_fields);
/* Initial optimizer vector and bounds (each [2(U+F)]); any may be NULL. */
int32_t texo_gp_initial(texo_gp_handle h, double* coordinates, double* lower,
                        double* upper);
/* Filler table (`initial_fillers`, electrostatic_placement.rs:198-240):
 * field index and charge per filler; either may be NULL. */
int32_t texo_gp_fillers(texo_gp_handle h, uint32_t* field, double* charge);

/* Evaluates wirelength and every density field at `coordinates` [2(U+F)]
 * with WA smoothing `gamma` (tile units). Optional outputs (NULL to skip):
 *   wa_gradient [2U], field_gradient [num_fields][2(U+F)] (raw, coefficient 1),
 *   density [num_fields][bins] (after fillers), potential [num_fields][bins]. */
int32_t texo_gp_evaluate(texo_gp_handle h, const double* coordinates, double gamma,
                         texo_gp_eval* out, double* wa_gradient,
                         double* field_gradient, double* density,
                         double* potential);
/* Raw device form of the density scatter at `coordinates`: int64 2^-32
 * fixed-point grids of the physical members (minus the smoothed capacity) and
 * of the fillers, [num_fields][bins] each; either may be NULL. */
int32_t texo_gp_scatter(texo_gp_handle h, const double* coordinates,
                        int64_t* physical_grid, int64_t* filler_grid);
/* Spectral Poisson solve of one grid `density` [bins] on the handle's bin
 * grid with the handle's DCT mode: writes potential [bins], returns energy. */
int32_t texo_gp_poisson(texo_gp_handle h, const double* density, double* potential,
                        double* energy);
/* texo_gp_scatter without allocating: the same grids, bit for bit, computed in
 * one file-scope device scratch array (4 MiB per device) instead of the
 * handle's buffers. It calls no cudaMalloc/cudaFree and allocates no host
 * memory, and it leaves the handle's buffers and resumable run state as they
 * were. For callers that may not allocate: a serving loop whose HBM budget is
 * fully committed to admitted jobs, where a new device allocation could fail
 * or take memory the budget promised to a job, and where cudaFree's implicit
 * device synchronization would stall the jobs running on other streams.
 * Limits: num_fields * bins <= 131072 and units + fillers <= 131072, else
 * TEXO_GP_ERR_UNSUPPORTED (texo_gp_last_error says which). Nothing has to be
 * zero beforehand; the call initializes every scratch word it reads. The
 * first call on a device looks up the scratch address (cudaGetSymbolAddress)
 * with that device current, and because CUDA loads device code lazily, that
 * first call is also when the 4 MiB array itself is reserved on the device:
 * make one call at start-up, before the HBM budget is committed and before
 * any stream capture; later calls reserve nothing. Calls
 * that overlap on one device (two threads, or two handles) race on the shared
 * scratch; calls made one after another are safe (each call synchronizes
 * before returning). No counterpart in the reference. */
int32_t texo_gp_scatter_static(texo_gp_handle h, const double* coordinates,
                               int64_t* physical_grid, int64_t* filler_grid);

/* The DCT form the handle runs: 0 FP32 GEMM with 16x16 slab tiles, 1 FP32
 * GEMM with 64x64 register-blocked tiles, 2 tcgen05 tensor cores (integer slices),
 * 3 FP32 FFT-based transforms (power-of-two grids; the default there). No
 * counterpart in the reference (it has one CPU transform). */
int32_t texo_gp_dct_form(texo_gp_handle h, int32_t* form);

/* Runs the placement loop from the handle's current state (the initial
 * coordinates after create) to convergence, the iteration cap, or
 * `max_iterations` more iterations when nonzero. Writes the best rounded
 * targets [2U] and optionally the current coordinates [2(U+F)]. */
int32_t texo_gp_run(texo_gp_handle h, uint32_t max_iterations, uint32_t* out_targets_xy,
                    double* out_coordinates, texo_gp_stats* stats);
/* Restores the handle to its just-created state (positions, multipliers,
 * optimizer state) without touching the device allocations. */
int32_t texo_gp_reset(texo_gp_handle h);

/* ---- routability-driven area rounds ------------------------------------
 * The pieces of eplace::place's area-adjustment loop (eplace.rs:320-420),
 * on the handle's engine (host or device: the persistent kernel's
 * controller takes the same stop criterion, multipliers and scales).
 * texo_gp_optimize_round runs one `optimize_density_once`
 * (eplace.rs:439-582) from the handle's current coordinates with a fresh
 * optimizer, multipliers and checkpoint: `stop` 0 stops at the final
 * targets (10 / 10 / 20 %), 1 at AreaAdjustmentReady (LUT and register
 * overflow <= 15 %, eplace.rs:130, 1403-1415); `reset_multipliers` sets the
 * multipliers from elfPlace eqs. (27)-(28) (`area_adjusted_density_
 * multipliers` / `_multiplier_step`, eplace.rs:1183-1232) instead of the
 * initial weight; `density_scales` (NULL: this round's initial energies)
 * fixes E0 to the first round's; the iteration cap counts
 * `completed_iterations` of the earlier rounds. The result gives the global
 * iteration count, whether the round was exhausted (cap or stationary) and
 * the scales it used. texo_gp_set_charges installs an area adjustment
 * (`apply_area_adjustment`, eplace.rs:793-818): member charges in the
 * problem's member order and filler charges in texo_gp_fillers' order
 * (either may be NULL); the real areas and the preconditioner follow. The
 * caller composes the loop (the proposal between rounds is
 * texo_gp_routing_demand, texo_gp_register_clustering_areas and
 * texo_gp_adjust_instance_areas; texo_gb300.routability.place_routable is
 * the Python composition). */
typedef struct texo_gp_round {
  int32_t stop;                  /* 0 final, 1 area-adjustment ready */
  int32_t reset_multipliers;
  const double* density_scales;  /* [num_fields] or NULL */
  uint64_t completed_iterations;
  uint32_t reserved[4];
} texo_gp_round;
typedef struct texo_gp_round_result {
  uint64_t completed_iterations;
  uint32_t exhausted;
  uint32_t reserved;
  double density_scales[TEXO_GP_MAX_FIELDS];
} texo_gp_round_result;
int32_t texo_gp_optimize_round(texo_gp_handle h, const texo_gp_round* round, uint32_t* out_targets_xy,
                               double* out_coordinates, texo_gp_stats* stats, texo_gp_round_result* result);
int32_t texo_gp_set_charges(texo_gp_handle h, const double* member_charge, const double* filler_charge);

/* eplace::place with its routing_capacity and register_controls arguments
 * (crates/texo-pnr/src/eplace.rs:242-420) in one call: area rounds that stop
 * at AreaAdjustmentReady, each followed by propose_area_adjustment
 * (eplace.rs:627-740: net bounding boxes at the unit origins, the RUDY map on
 * the capacity grid, each movable member's utilization at its rounded
 * position capped at sqrt(2), eq. 29 for LUT and register members, the
 * register-clustering areas, adjust_instance_areas against the fillers); an
 * adjustment that grows any kind is installed and the optimizer restarts
 * with the area-reset multipliers and the first round's density scales;
 * once the installed increase is below 1 % (or nothing grew) a last round
 * runs to the final targets. The rounds run on params->engine's engine.
 * `capacity` NULL is texo_gp_place (the pure density
 * objective). A register member whose cell has no control set, a cell with
 * two, or more area rounds than area_adjustment_round_limit (eplace.rs:
 * 584-626) return TEXO_GP_ERR_INVALID_NORMALIZATION like the reference.
 * `out_targets_xy` [2U]: the last round's best rounded targets;
 * `out_coordinates` [2(U+F)] (may be NULL): its final coordinates. */
typedef struct texo_gp_routing_capacity {
  uint32_t width, height;            /* RoutingCapacityMap (routing_demand.rs:22-27) */
  const uint32_t* horizontal;        /* [height][width] channel capacities */
  const uint32_t* vertical;          /* [height][width] */
} texo_gp_routing_capacity;
typedef struct texo_gp_register_control {   /* RegisterControlSet (lib.rs:2157-2164) */
  uint32_t cell;
  uint32_t reserved;
  uint64_t clock_lsr[2];
  uint64_t ce;
} texo_gp_register_control;
typedef struct texo_gp_routable_report {
  uint32_t rounds;                   /* density rounds run */
  uint32_t area_rounds;              /* adjustments installed */
  uint64_t iterations;               /* eplace iterations over all rounds */
  double last_relative_increase;     /* of the last proposal: total and largest per kind */
  double last_maximum_relative_increase;
  double max_horizontal_utilization; /* of the last proposal */
  double max_vertical_utilization;
  uint64_t last_members_inflated;
  uint32_t reserved[8];
} texo_gp_routable_report;
int32_t texo_gp_place_routable(const texo_gp_problem* problem, const texo_gp_params* params,
                               const texo_gp_routing_capacity* capacity, uint64_t num_register_controls,
                               const texo_gp_register_control* register_controls, uint32_t* out_targets_xy,
                               double* out_coordinates, texo_gp_stats* stats, texo_gp_routable_report* report);

/* Per-stage device times: runs each stage of one full objective evaluation at
 * the handle's current coordinates `reps` times and writes the mean time of
 * one launch in milliseconds, measured with CUDA events on the handle's
 * stream, to ms[i] for the stages named by texo_gp_stage_name(i). Returns
 * the stage count in *count. */
int32_t texo_gp_stage_times(texo_gp_handle h, uint32_t reps, double* ms, uint32_t capacity,
                            uint32_t* count);
const char* texo_gp_stage_name(uint32_t stage);
/* Cumulative phase profile of the device engine since create/reset, in
 * microseconds, as seen by the persistent kernel's first block: out[0..7] =
 * scatter+WA, prep, transforms, gather+combine, preconditioner/init,
 * extrapolation, candidate, other; out[8] = time block 0 spent waiting in
 * grid barriers; out[9] = number of grid barriers. */
int32_t texo_gp_device_profile(texo_gp_handle h, double out[10]);

/* Per-iteration controller trace of the host engine (diagnostic, for parity
 * with the oracle's controller): one record per completed eplace iteration of
 * `optimize_density_once` (eplace.rs:439-582) since create/reset, the first
 * 4096 kept. The device engine keeps its controller on the GPU and records
 * none (count 0). No counterpart in the reference (it only traces through
 * its `tracing` spans). */
typedef struct texo_gp_iteration {
  uint32_t iteration;            /* 1-based */
  uint32_t trials;               /* line-search trials of this Nesterov step */
  double gamma;                  /* WA gamma of the step (tile units) */
  double objective;              /* accepted combined objective */
  double lipschitz;              /* Lipschitz estimate after the step */
  double momentum;               /* Nesterov momentum parameter after the step */
  double lambda[TEXO_GP_MAX_FIELDS];        /* density multipliers the step used */
  double energy_scale[TEXO_GP_MAX_FIELDS];  /* E0 = max(initial energy, 1) per field */
  double overflow[TEXO_GP_MAX_FIELDS];      /* normalized overflow at the accepted point */
} texo_gp_iteration;
int32_t texo_gp_trace(texo_gp_handle h, texo_gp_iteration* out, uint32_t capacity, uint32_t* count);

/* HPWL = sum over hypernets of the x and y pin spans at `coordinates`
 * (the continuous form of `exact_objective`, analytical_placement.rs:473-511),
 * FP64 reduction. */
int32_t texo_gp_hpwl(texo_gp_handle h, const double* coordinates, double* hpwl);

/* ---- synthetic ECP5-like netlists ----------------------------------------
 * Seeded generator of the benchmark netlists: movable unit-area LUT cells on a
 * side x side site fabric with one LUT per site, fixed IO cells evenly spaced
 * on the perimeter, nets in 2 / 3-5 / 6-32 pin bands with Gaussian index-grid
 * locality. Owned by the returned handle; `problem` points into it. */
typedef struct texo_gp_synth_spec {
  uint32_t side;          /* fabric side in sites */
  uint32_t cells;         /* movable unit-area cells */
  uint32_t io;            /* fixed perimeter IO cells (evenly spaced; may share sites) */
  uint32_t nets;
  double sigma;           /* locality radius in sites */
  double p_local;         /* probability that a sink is local (0.8) */
  double jitter;          /* initial N(0, jitter) sites around the centre */
  uint64_t seed;
} texo_gp_synth_spec;
typedef struct texo_gp_synth_s* texo_gp_synth;
int32_t texo_gp_synth_create(const texo_gp_synth_spec* spec, texo_gp_synth* out,
                             const texo_gp_problem** problem);
int32_t texo_gp_synth_destroy(texo_gp_synth s);

/* ---- batched and served placement ----------------------------------------
 * Many independent placements resident on the device at once; the device
 * engine advances all of them in one persistent kernel per chunk of
 * iterations. A job retires when its stop rule fires. */
typedef struct texo_gp_batch_s* texo_gp_batch;
int32_t texo_gp_batch_create(const texo_gp_params* params, uint64_t hbm_budget_bytes,
                             uint32_t max_slots, texo_gp_batch* out);
int32_t texo_gp_batch_destroy(texo_gp_batch b);
/* Admits one job when its device footprint fits the remaining HBM budget and
 * a slot is free; returns TEXO_GP_ERR_BUSY otherwise. `params` (NULL = the
 * batch's) may set a per-job bin grid, target density and stop rule; the
 * engine is always the device engine and the device the batch's. */
int32_t texo_gp_batch_admit(texo_gp_batch b, const texo_gp_problem* problem,
                            const texo_gp_params* params, uint64_t job_id, uint32_t* out_slot);
/* Advances every resident job by up to `iterations` eplace iterations. */
int32_t texo_gp_batch_advance(texo_gp_batch b, uint32_t iterations);
/* Pops one finished job: its id, rounded targets (caller buffer of 2U) and stats.
 * Returns TEXO_GP_ERR_BUSY when no job has finished. */
int32_t texo_gp_batch_retire(texo_gp_batch b, uint64_t* job_id, uint32_t* out_targets_xy,
                             uint64_t targets_capacity, texo_gp_stats* stats);
int32_t texo_gp_batch_counts(texo_gp_batch b, uint32_t* resident, uint32_t* finished,
                             uint64_t* bytes_in_use);
/* An advance whose resident set (jobs, order and iteration chunk) repeats the
 * previous advance's is captured once as a CUDA graph (state copies in, the
 * persistent launches, state copies out) and replayed while the set stays;
 * counts of captures and replays since create (diagnostic; no counterpart in
 * the reference). */
int32_t texo_gp_batch_graphs(texo_gp_batch b, uint64_t* captures, uint64_t* replays);

/* ---- Serving loop (continuous batching) ----------------------------------
 * Placement requests are submitted at any time from any thread. Admission
 * threads build each job's model and upload it once its device footprint
 * fits the HBM budget; the serving thread adds uploaded jobs to the resident
 * batch at the next launch boundary, advances all resident jobs together
 * (one persistent launch per `chunk_iterations`), and retires each job when
 * it stops (overflow target reached, iteration cap, or an error), freeing
 * its memory for waiting jobs. A job's result does not depend on the other
 * jobs in the batch. No counterpart in the reference (its placement is one
 * synchronous call); the per-job semantics are those of texo_gp_place. */
typedef struct texo_gp_server_s* texo_gp_server;
typedef struct texo_gp_server_options {
  uint64_t hbm_budget_bytes;   /* device bytes uploaded jobs may hold (0: 3/4 of free memory) */
  uint32_t max_resident;       /* jobs advanced together (0: 256) */
  uint32_t chunk_iterations;   /* iterations per launch between admissions (0: 20) */
  uint32_t admission_threads;  /* host threads building and uploading jobs (0: 4) */
  uint32_t reserved[5];
} texo_gp_server_options;
typedef struct texo_gp_job_result {
  uint64_t job_id;
  int32_t status;              /* TEXO_GP_OK, DID_NOT_CONVERGE, or the job's error */
  uint32_t units;              /* targets written: 2 * units */
  texo_gp_stats stats;
  double submit_ms;            /* server clock (ms since texo_gp_server_create) */
  double admit_ms;             /* upload finished, waiting for the next launch */
  double finish_ms;            /* retired */
} texo_gp_job_result;

int32_t texo_gp_server_create(const texo_gp_params* defaults, const texo_gp_server_options* options,
                              texo_gp_server* out);
/* Stops the serving and admission threads (finishing the launch in flight)
 * and frees every job. */
int32_t texo_gp_server_destroy(texo_gp_server s);
/* Queues one request; the problem is copied, so the caller's arrays may be
 * released on return. `params` NULL = the server defaults (engine and device
 * are the server's). */
int32_t texo_gp_server_submit(texo_gp_server s, const texo_gp_problem* problem,
                              const texo_gp_params* params, uint64_t job_id);
/* Pops one finished job, waiting up to `wait_ms` (negative: forever) for
 * one; TEXO_GP_ERR_BUSY when none finished in time. `out_targets_xy` (may be
 * NULL) receives 2U rounded targets when `targets_capacity` >= 2U, else the
 * call returns TEXO_GP_ERR_INVALID_ARGUMENT, sets out->job_id and out->units
 * and keeps the job for a call with a larger buffer. */
int32_t texo_gp_server_poll(texo_gp_server s, int32_t wait_ms, texo_gp_job_result* out,
                            uint32_t* out_targets_xy, uint64_t targets_capacity);
int32_t texo_gp_server_counts(texo_gp_server s, uint32_t* queued, uint32_t* resident,
                              uint32_t* finished, uint64_t* bytes_in_use);
double texo_gp_server_clock_ms(texo_gp_server s);

/* ---- coarse quadratic seed ------------------------------------------------
 * Replaces `solve_quadratic` (crates/texo-pnr/src/lib.rs:4586-4752, called
 * from `solve_analytical_axis`, lib.rs:4531-4560): Jacobi-preconditioned
 * conjugate gradients for (D - W) x = b, D = `diagonal` (finite, > 0), W the
 * symmetric `adjacency` (row i: weights adjacency_weight[k] to columns
 * adjacency_index[k], k in [adjacency_ptr[i], adjacency_ptr[i+1]), in the
 * order of the reference's Vec<(usize, f64)>), all FP64, on one GPU. Stops
 * when |r|^2 <= 1e-8 max(|r0|^2, eps64), re-checking the true residual before
 * accepting (and restarting from it otherwise), on a breakdown, or after n
 * loop passes; `solution` holds the initial guess on entry and the result on
 * return. Returns TEXO_GP_ERR_PCG_NOT_CONVERGED (with the solution anyway)
 * when the true final residual misses the target, like the reference. */
typedef struct texo_gp_pcg_stats {
  int32_t status;
  uint32_t iterations;           /* conjugate-gradient steps taken */
  uint32_t restarts;             /* true-residual restarts */
  int32_t stop;                  /* 0 residual, 1 breakdown, 2 dimension (the reference's labels) */
  double initial_residual_squared;
  double target_squared;
  double final_residual_squared; /* |b - (D - W) x|^2 of the returned solution */
  double elapsed_ms;             /* device time (CUDA events), copies included */
  uint64_t kernel_launches;
} texo_gp_pcg_stats;
int32_t texo_gp_quadratic_solve(int32_t device, uint32_t n, const double* diagonal,
                                const uint32_t* adjacency_ptr, const uint32_t* adjacency_index,
                                const double* adjacency_weight, const double* rhs, double* solution,
                                texo_gp_pcg_stats* stats);

/* ---- routability: continuous RUDY demand ----------------------------------
 * Replaces `continuous_routing_demand` (crates/texo-pnr/src/eplace.rs:856-937):
 * every net bounding box (boxes[i] = min_x, max_x, min_y, max_y, as
 * `external_baseline_net_bounding_boxes` gives them, analytical_placement.rs:
 * 238-276), widened by half a tile, adds dx / area to the horizontal and
 * dy / area to the vertical demand of each tile of the width x height grid it
 * overlaps, weighted by the overlap (area = (dx + 1)(dy + 1)). Outputs are
 * [height][width] FP64. The demand accumulates in int64 2^-40 fixed point
 * (deterministic; within 2^-41 per box and tile of the reference's FP64
 * sums; at most 2^22 boxes, else TEXO_GP_ERR_FIXED_POINT_RANGE). A
 * non-finite or unordered box returns TEXO_GP_ERR_INVALID_NORMALIZATION like
 * the reference. `elapsed_ms` (may be NULL): device time with the copies. */
int32_t texo_gp_routing_demand(int32_t device, uint32_t width, uint32_t height, uint64_t num_boxes,
                               const double* boxes, double* horizontal, double* vertical, double* elapsed_ms);

/* ---- routability: instance-area adjustment (host, FP64) ------------------
 * The arithmetic of elfPlace's charge-conserving instance-area update
 * (crates/texo-pnr/src/instance_area.rs), in the reference's operation order
 * without fused multiply-adds, so results are the reference's bit for bit.
 * A resource kind is an opaque key; keys must sort like the reference's
 * ResourceKind (e.g. kind << 8 | lut_inputs); results per kind come back in
 * ascending key order.
 *
 * adjust_instance_areas (:157-253): each member asks for the largest of its
 * routability, pin, clustering and current areas; per kind the increase is
 * scaled by min(1, filler area / desired increase), the last member of a kind
 * takes the rounding remainder, and the fillers of each kind shrink in
 * proportion (the last one taking the remainder) so every kind's total is
 * conserved. `scale_kind` / `scale` (capacity `max_scales`, count in
 * *num_scales) receive the per-kind scales; `requires_optimizer_reset` is 1
 * when any kind grew. `error_index` (may be NULL): the member or filler of an
 * INSTANCE_AREA_MEMBER / _FILLER error. */
int32_t texo_gp_adjust_instance_areas(uint64_t num_members, const uint32_t* member_kind, const double* current_area,
                                      const double* routability_area, const double* pin_area,
                                      const double* clustering_area, uint64_t num_fillers,
                                      const uint32_t* filler_kind, const double* filler_area,
                                      double* out_member_area, double* out_filler_area,
                                      int32_t* requires_optimizer_reset, uint32_t max_scales,
                                      uint32_t* num_scales, uint32_t* scale_kind, double* scale,
                                      uint64_t* error_index);
/* routability_optimized_area (:64-84), elfPlace eq. (29): current area times
 * min(max(h, v)^2, 2). */
int32_t texo_gp_routability_optimized_area(double current_area, double horizontal_utilization,
                                           double vertical_utilization, double* out);
/* routability_optimized_area_from_bin (:91-127): utilization from one RUDY
 * bin's demand and integer channel capacity; a direction with demand but no
 * capacity is a hotspot (twice the area), with neither it counts zero. */
int32_t texo_gp_routability_optimized_area_from_bin(double current_area, double horizontal_demand,
                                                    uint64_t horizontal_capacity, double vertical_demand,
                                                    uint64_t vertical_capacity, double* out);
/* pin_optimized_area (:130-148), elfPlace eq. (30). */
int32_t texo_gp_pin_optimized_area(uint64_t pin_count, double unit_area_pin_capacity,
                                   double local_pin_utilization, double* out);

/* ---- routability: register-clustering areas (GPU) -----------------------
 * Replaces `clustering_areas` (crates/texo-pnr/src/register_clustering.rs:
 * 17-80), as `propose_register_clustering_areas` (eplace.rs:760-791) calls
 * it: register r at (xy[2r], xy[2r+1]) with control set (clock_lsr[2r],
 * clock_lsr[2r+1]) and clock enable ce[r]; sigma = sqrt(1e-5 * count) for
 * `movable_instance_count`, window half-width 2.5 sigma. For each register
 * the expected registers of its control set in its window, per clock
 * enable, are the sums of the other registers' Gaussian window
 * probabilities (x times y, FP64 erf); areas[r] =
 * 8 / E_focal * ceil2(E_focal) / sum_ce ceil2(E_ce) * ceil4(sum_ce ceil2(E_ce))
 * with the reference's soft ceilings. Sums run in the reference's order
 * (input order within a clock enable, clock enables ascending); pairs whose
 * windows are more than 8 sigma sqrt(2) apart on an axis contribute an exact
 * zero and are skipped. The device erf is CUDA's, not the reference's libm
 * erf, so areas agree to rounding, not bit for bit. Returns
 * TEXO_GP_ERR_INVALID_NORMALIZATION where the reference returns None
 * (count above 2^32 - 1, a non-positive focal expectation, a non-finite
 * area). `elapsed_ms` (may be NULL): device time with the copies. */
int32_t texo_gp_register_clustering_areas(int32_t device, uint64_t num_registers, const double* xy,
                                          const uint64_t* clock_lsr, const uint64_t* ce,
                                          uint64_t movable_instance_count, double* areas, double* elapsed_ms);

/* ---- legalization: the capacity auction ---------------------------------
 * Replaces `assign_implicitly` (crates/texo-pnr/src/legalization/auction.rs:
 * 131-247): the integer-cost assignment of bidders to objects with epsilon
 * one, every bidder owning a private dummy of cost
 * D = n * max_base_cost + n + 1 (n = bidders; at the reference's cost scale
 * 1, `cost_scale` below generalises it), so the result has exactly the
 * maximum cardinality and a total base cost at most n above the minimum
 * among assignments of that cardinality. A bidder's bid raises its best
 * object's price by (second-best reduced cost - best reduced cost + 1), ties
 * broken by the lower object id, the dummy losing equal-cost ties.
 *
 * The reference bids one bidder at a time from a FIFO queue; here all
 * unassigned bidders bid at once each round and each object goes to its
 * highest bid (equal bids: the lower bidder index). The result is
 * deterministic and has the same guarantees, but where several assignments
 * meet them it may be another one than the reference's.
 *
 * `cost_scale` s multiplies every base cost before the auction, epsilon
 * staying one (the reference's `cost_scale`, auction.rs:142, fixed there at
 * 1): the dummy becomes D = n * s * max_base_cost + n + 1 and the total base
 * cost is at most n / s above the least one of the maximum cardinality.
 * s = 1 is the reference's setting. 0 picks the largest of 4, 2, 1 whose
 * price range fits when every bidder is sure to be matched (the BEL grid
 * below with at least as many free BELs of each kind as bidders of that
 * kind, no BEL under two kinds) and every kind with bidders holds at most
 * two BELs a tile on average, else 1: bidders left over leave only once prices pass D, about
 * one price step a round, and D grows with s; with many BELs a tile a
 * displaced bidder moves a ring out only after s price steps on each of
 * them. On placement targets the scaled
 * auction lands within a fraction of a percent of the optimum for about a
 * quarter more bids; the reference's setting lands about 12 % above it.
 * Explicit domains take 1 for 0 (whether every bidder can be matched is not
 * known up front there).
 *
 * `assignment` receives, per bidder, its object or -1 (its dummy);
 * `prices` (may be NULL) the final object prices (the certificate of the
 * epsilon-optimality). Prices live in 32 bits on the device:
 * D + 1 + s * max_base_cost must stay below 2^32, else
 * TEXO_GP_ERR_AUCTION_RANGE (the reference's ArithmeticOverflow, there at 2^64). */
typedef struct texo_gp_auction_stats {
  int32_t status;
  uint32_t rounds;               /* parallel bidding rounds */
  uint32_t cost_scale;           /* the scale s the auction ran with */
  uint32_t tail_rounds;          /* of the rounds, those one block ran alone (few bidders left) */
  uint64_t bids;                 /* bids placed (each raises one object's price if it wins) */
  uint64_t candidates_examined;  /* candidate objects visited by the searches */
  uint64_t unmatched;            /* bidders left on their dummy */
  uint64_t total_base_cost;      /* sum of the matched bidders' base costs */
  double elapsed_ms;             /* device time (CUDA events), copies included */
  uint64_t kernel_launches;
} texo_gp_auction_stats;

/* Explicit candidate lists, the form the reference's own tests drive the
 * auction with (`explicit_best_two`, auction.rs:253-272): bidder b may take
 * domain_object[k] at base cost domain_cost[k], k in
 * [domain_ptr[b], domain_ptr[b+1]). An object out of range, a cost above
 * max_base_cost or an object twice in one domain is an error. */
int32_t texo_gp_auction_explicit(int32_t device, uint32_t num_bidders, uint32_t num_objects,
                                 uint64_t max_base_cost, uint32_t cost_scale, const uint32_t* domain_ptr,
                                 const uint32_t* domain_object, const uint64_t* domain_cost,
                                 int32_t* assignment, uint32_t* prices, texo_gp_auction_stats* stats);

/* The singleton-BEL auction of `project` (`auction_singletons` and
 * `auction_units`, legalization/mod.rs:657-677, 733-840), candidates found
 * by Manhattan ring walks (`best_objects_on_cached_rings`,
 * `discover_legal_ring`, mod.rs:876-1021): objects are BELs; the BELs of kind
 * q at tile t = y * width + x are tile_object[k], k in
 * [tile_ptr[q * width * height + t], tile_ptr[q * width * height + t + 1]);
 * bidder b of kind bidder_kind[b] with rounded target (target_xy[2b],
 * target_xy[2b+1]) takes an unoccupied BEL of its kind at base cost
 * |x - tx| + |y - ty|; max_base_cost = width - 1 + height - 1. The ring walk
 * stops after ring r once the second-best reduced cost is below s (r + 1).
 * A BEL may be listed under several kinds (once in each; bidders of those
 * kinds then compete for its one price), so kinds can be the distinct
 * candidate tables of SingleCell units.
 * `occupied` (may be NULL): one byte per BEL, nonzero for BELs held by fixed
 * units or earlier cohorts. Legality beyond occupancy (pin wires, shared
 * resources) is the caller's: a BEL that fails it is passed as occupied.
 * Grid sides up to 16384 tiles. */
int32_t texo_gp_auction_singletons(int32_t device, uint32_t width, uint32_t height, uint32_t num_kinds,
                                   const uint32_t* tile_ptr, const uint32_t* tile_object, uint32_t num_objects,
                                   const uint8_t* occupied, uint32_t num_bidders, const uint32_t* bidder_kind,
                                   const uint32_t* target_xy, uint32_t cost_scale, int32_t* assignment,
                                   uint32_t* prices, texo_gp_auction_stats* stats);

/* ---- legalization: `project` up to its repair ---------------------------
 * `project` (crates/texo-pnr/src/legalization/mod.rs:322-389) before
 * `repair_relaxed`: the preferred choice of every unit from its rounded
 * target. BELs are 0..num_bels-1 at tiles bel_xy[2b], bel_xy[2b+1]. Unit u
 * chooses among the rows of tables[unit_table[u]] (one BEL per cell of the
 * unit); unit_first_cell[u] is its first cell id, the reference's order key.
 * A table with one row is a fixed unit's (its BELs are taken first; two
 * fixed units on one BEL is TEXO_GP_ERR_PROJECTION_CONFLICT, the reference's
 * "fixed analytical placement assignments conflict"). Units of one `shared`
 * table form a family: pairwise BEL-disjoint rows are auctioned (families
 * scarcest first: rows x the other family's units, then wider rows, then
 * first cell), other families' units are seeded one at a time (fewest rows,
 * widest, first cell) on the least (point, row) free on the first Manhattan
 * ring around the target that has one. Non-shared tables (SingleCell
 * candidates, width 1, ascending BEL ids) are one auction, a kind per table.
 * A row is free when none of its BELs is taken; occupancy is the only
 * legality rule. Auctions run on the GPU (texo_gp_auction_singletons, cost
 * scale `cost_scale`, 0 automatic). out_choice[u]: the chosen row, or -1
 * when the unit was left unmatched (the repair's). */
typedef struct texo_gp_choice_table {
  uint32_t num_choices;          /* rows */
  uint32_t width;                /* BELs a row: the cells of the units using it */
  const uint32_t* bels;          /* [num_choices][width] */
  int32_t shared;                /* 1: Shared rows; 0: SingleCell candidates (width 1) */
  uint32_t reserved;
} texo_gp_choice_table;
typedef struct texo_gp_projection_stats {
  uint64_t fixed_units;
  uint64_t overlapping_shared_families, overlapping_shared_units;
  uint64_t disjoint_shared_families, disjoint_shared_units;
  uint64_t singleton_units;
  uint64_t relaxed_unmatched_units;
  uint64_t bids, candidates_examined;   /* over the auctions */
  uint64_t auctions;
  double elapsed_ms;                    /* the auctions' device time */
  uint32_t reserved[8];
} texo_gp_projection_stats;
int32_t texo_gp_project(int32_t device, uint32_t width, uint32_t height, uint32_t num_bels, const uint32_t* bel_xy,
                        uint32_t num_tables, const texo_gp_choice_table* tables, uint32_t num_units,
                        const uint32_t* unit_table, const uint32_t* unit_first_cell, const uint32_t* target_xy,
                        uint32_t cost_scale, int32_t* out_choice, texo_gp_projection_stats* stats);

/* ---- legalization: the transactional repair of `project` ----------------
 * `repair_relaxed` (crates/texo-pnr/src/legalization/repair.rs:60-151), the
 * last step of `project`: a relaxed proposal (preferred[u] a row of
 * tables[unit_table[u]], or -1 unmatched; rows may conflict) becomes a legal
 * placement. Unit u's cells are unit_cells[unit_cell_ptr[u] ..
 * unit_cell_ptr[u+1]] (one per row BEL, the first the order key), cells
 * 0..num_cells-1; fixed[u] nonzero marks a fixed unit (never evicted; it must
 * have a choice). Legality: BEL occupancy and, with `legality` (may be
 * NULL), pin wires and shared resources:
 *   - a connected cell pin (cell_pin_cell[k], key cell_pin_key[k], net
 *     cell_pin_net[k]) placed on BEL b takes the wire bel_pin_wire[j] of the
 *     entry with bel_pin_bel[j] = b and bel_pin_key[j] = key; wire w admits
 *     wire_capacity[w] distinct nets (`visit_assignment_pin_resources`,
 *     lib.rs:6989-7005). A candidate BEL without the key is an error;
 *   - under rule r a cell carries a value (cell_value_*) and a BEL belongs
 *     to a resource (bel_resource_*); a (rule, resource) holds one value
 *     (`visit_assignment_shared_resources`, lib.rs:6972-6987).
 * The search (initial pending units, the direct and single-blocker fast
 * paths, the exact search over every blocker set with memoised states;
 * choices from the preferred one outwards ring by ring around target_xy) is
 * the reference's, so the placement and the counters equal its own.
 * out_cell_bel[c]: the BEL of cell c (-1 for cells of no unit). Errors:
 * TEXO_GP_ERR_PROJECTION_CONFLICT for the reference's invalid-placement
 * cases (two fixed units on a BEL, incompatible fixed values or nets, an
 * out-of-range or missing fixed choice), TEXO_GP_ERR_NO_BEL when no legal
 * completion exists (stats->failed_cell: the first unplaced unit's first
 * cell). Host code; no device work. */
typedef struct texo_gp_legality {
  uint32_t num_wires;
  const uint32_t* wire_capacity;
  uint32_t num_cell_pins;
  const uint32_t *cell_pin_cell, *cell_pin_key, *cell_pin_net;
  uint32_t num_bel_pins;
  const uint32_t *bel_pin_bel, *bel_pin_key, *bel_pin_wire;
  uint32_t num_rules;
  uint32_t num_cell_values;
  const uint32_t *cell_value_rule, *cell_value_cell;
  const uint64_t* cell_value;
  uint32_t num_bel_resources;
  const uint32_t *bel_resource_rule, *bel_resource_bel;
  const uint64_t* bel_resource;
} texo_gp_legality;
typedef struct texo_gp_repair_stats {   /* RepairStats (repair.rs:35-49) */
  uint64_t initial_pending;
  uint64_t direct_fast_choices, direct_fast_moves, direct_fast_fallbacks;
  uint64_t augmenting_roots, augmenting_fallbacks;
  uint64_t states_visited, failed_states, max_unplaced, max_blocker_branches;
  uint64_t units_evicted, choices_examined;
  double elapsed_ms;
  uint32_t failed_cell;
  uint32_t reserved[7];
} texo_gp_repair_stats;
int32_t texo_gp_repair(uint32_t width, uint32_t height, uint32_t num_bels, const uint32_t* bel_xy,
                       uint32_t num_tables, const texo_gp_choice_table* tables, uint32_t num_units,
                       const uint32_t* unit_table, const uint32_t* unit_cell_ptr, const uint32_t* unit_cells,
                       uint32_t num_cells, const uint32_t* target_xy, const int32_t* preferred,
                       const uint8_t* fixed, const texo_gp_legality* legality, int32_t* out_cell_bel,
                       texo_gp_repair_stats* stats);

/* Diagnostic: runs the engine's bounded device waits (the grid barrier of
 * the persistent loop and the mbarrier wait of the tensor-core pipeline)
 * against partners that never arrive, with a short limit. Both must run out
 * (flags set to 1) and return without faulting; the device stays usable. No
 * counterpart in the reference. */
int32_t texo_gp_selftest_waits(int32_t device, int32_t* barrier_timed_out, int32_t* mbarrier_timed_out);

#ifdef __cplusplus
}
#endif
#endif /* TEXO_GP_H */
