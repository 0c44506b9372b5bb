// routability_oracle.cpp — TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of elfPlace's register-clustering area estimate
// (`clustering_areas`, crates/texo-pnr/src/register_clustering.rs:17-97), in
// FP64 with the reference's loops and summation order: registers grouped by
// control set (clock, LSR) in input order, per focal register a BTreeMap of
// expectations by clock enable, every pair computed (no pruning). erf is the
// C library's (the reference links the `libm` crate 0.2.16), so results
// agree with the reference to rounding.
#include <cmath>
#include <cstdint>
#include <map>
#include <utility>
#include <vector>

#include "texo_oracle.h"

namespace {

double soft_ceiling(double value, double divisor) {
  const double quotient = value / divisor;
  const double fl = std::floor(quotient);
  if (quotient - fl < 1.0 / divisor) return value + (1.0 - divisor) * fl;
  return std::ceil(quotient);
}

double window_probability(double low, double high, double mean, double sigma) {
  const double scale = sigma * 1.4142135623730951;   // sigma sqrt(2)
  const double p = 0.5 * (std::erf((high - mean) / scale) - std::erf((low - mean) / scale));
  return p < 0.0 ? 0.0 : (p > 1.0 ? 1.0 : p);
}

}  // namespace

extern "C" double orc_soft_division_ceiling(double value, double divisor) { return soft_ceiling(value, divisor); }

extern "C" int32_t orc_register_clustering_areas(uint64_t n, const double* xy, const uint64_t* clock_lsr,
                                                 const uint64_t* ce, uint64_t movable_instance_count,
                                                 double* areas) {
  if (n == 0) return 0;
  if (movable_instance_count == 0) {
    for (uint64_t r = 0; r < n; ++r) areas[r] = 0.0;
    return 0;
  }
  if (movable_instance_count > 0xffffffffull) return TEXO_GP_ERR_INVALID_NORMALIZATION;
  const double sigma = std::sqrt(1.0e-5 * (double)(uint32_t)movable_instance_count);
  if (!std::isfinite(sigma) || sigma <= 0.0) return TEXO_GP_ERR_INVALID_NORMALIZATION;
  const double half_window = 2.5 * sigma;
  std::map<std::pair<uint64_t, uint64_t>, std::vector<uint64_t>> groups;
  for (uint64_t r = 0; r < n; ++r) groups[{clock_lsr[2 * r], clock_lsr[2 * r + 1]}].push_back(r);
  for (uint64_t r = 0; r < n; ++r) {
    const double x = xy[2 * r], y = xy[2 * r + 1];
    std::map<uint64_t, double> expected_by_ce;
    for (uint64_t o : groups[{clock_lsr[2 * r], clock_lsr[2 * r + 1]}]) {
      const double px = window_probability(x - half_window, x + half_window, xy[2 * o], sigma);
      const double py = window_probability(y - half_window, y + half_window, xy[2 * o + 1], sigma);
      expected_by_ce[ce[o]] += px * py;
    }
    const auto it = expected_by_ce.find(ce[r]);
    const double focal = it == expected_by_ce.end() ? 0.0 : it->second;
    if (!(std::isfinite(focal) && focal > 0.0)) return TEXO_GP_ERR_INVALID_NORMALIZATION;
    double total = 0.0;
    for (const auto& kv : expected_by_ce) total += soft_ceiling(kv.second, 2.0);
    const double area = 8.0 / focal * soft_ceiling(focal, 2.0) / total * soft_ceiling(total, 4.0);
    if (!(std::isfinite(area) && area >= 0.0)) return TEXO_GP_ERR_INVALID_NORMALIZATION;
    areas[r] = area;
  }
  return 0;
}
