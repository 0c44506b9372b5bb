// kernels.cuh — standalone-kernel launchers over the stage functions, and the
// scalar block the finalize kernels write (read back by the host controller).
#pragma once
#include "stages.cuh"

namespace tgp {

// Scalar block layout (doubles): outputs of finalize, inputs set by the host.
enum Scalar {
  SC_WA = 0,
  SC_ENERGY = 1,                 // + field
  SC_OVERFLOW = 5,               // + field, normalized
  SC_FORCE = 9,                  // + field
  SC_RAWL1 = 13,                 // + field
  SC_WAL1 = 17,
  SC_COEF = 18,                  // + field
  SC_VALUE = 22,
  SC_DOT = 23,
  SC_MSN = 24,
  SC_KKT = 25,
  SC_CHANGE = 26,
  SC_PMIN = 27,
  SC_PMAX = 28,
  SC_HPWL = 29,
  SC_MEAN = 30,                  // + field
  // inputs
  SC_LAMBDA = 40,                // + field
  SC_E0 = 44,                    // + field
  SC_BETA = 48,
  SC_REAL_AREA = 49,             // + field
  kScalars = 64
};
enum IScalar {
  SI_OVERFLOW_FIXED = 0,         // + field
  SI_OVER_BINS = 4,              // + field
  SI_DIFF = 8,
  SI_BAD = 9,
  SI_PBAD = 10,
  SI_GRID_SUM = 11,              // + field
  SI_TC_FAIL = 15,               // set when a tensor-core DCT wait ran out
  kIScalars = 16
};

enum FinalizeMask {
  FIN_ENERGY = 1,     // WA value, energies, overflow, coefficients, objective value
  FIN_COMBINE = 2,    // raw L1, WA L1, force L1, bad index
  FIN_CAND = 4,       // diff count, dot, msn
  FIN_KKT = 8,        // kkt residual, change
  FIN_PRECOND = 16,   // pmin, pmax, pbad
  FIN_DIFF = 32,      // diff count only
  FIN_HPWL = 64,
  FIN_WA = 128        // WA value + objective value without density refresh
};

// One instance's partial buffers and scalar block (device pointers).
struct Reduce {
  Partials p;
  Partials q;            // second set: the persistent kernel's loop phases alternate p and q
  double* scal;          // [kScalars]
  long long* iscal;      // [kIScalars]
};

unsigned long long launches_issued();
void note_launch();
void launch_init(const Dev& d, bool grids, bool wa, int nvb, cudaStream_t s);
void launch_scatter(const Dev& d, const Reduce& r, const float2* pos, int nvb, cudaStream_t s);
void launch_spread_positions(const Dev& d, float2* out, int nvb, cudaStream_t s);
void launch_wa(const Dev& d, const Reduce& r, const float2* pos, double gamma, int nvb, cudaStream_t s);
void launch_prep(const Dev& d, const Reduce& r, int nvb, cudaStream_t s);
void launch_dct(const Dev& d, const Reduce& r, int step, int nvb, cudaStream_t s,
                const tc::TcMaps* maps = nullptr);
void launch_gather(const Dev& d, const Reduce& r, const float2* pos, int nvb, cudaStream_t s);
void launch_combine(const Dev& d, const Reduce& r, float2* gout, int nvb, cudaStream_t s);
void launch_extrapolate(const Dev& d, const Reduce& r, const float2* x, const float2* xp, float e, float2* y,
                        int nvb, cudaStream_t s);
void launch_candidate(const Dev& d, const Reduce& r, const float2* y, const float2* gy, float invL, float2* c,
                      int nvb, cudaStream_t s);
void launch_kkt(const Dev& d, const Reduce& r, const float2* x, const float2* g, const float2* ref, int nvb,
                cudaStream_t s);
void launch_precond(const Dev& d, const Reduce& r, int nvb, cudaStream_t s);
void launch_hpwl(const Dev& d, const Reduce& r, const float2* pos, int nvb, cudaStream_t s);
void launch_finalize(const Dev& d, const Reduce& r, int nvb, int mask, cudaStream_t s);
void launch_round_compare(const Dev& d, const float2* x, uint32_t* prev_targets, int W, int H,
                          unsigned long long* mismatch, int nvb, cudaStream_t s);

}  // namespace tgp
