// instance_area.cpp — the arithmetic of elfPlace's charge-conserving
// instance-area update (crates/texo-pnr/src/instance_area.rs), host FP64.
//
// Built with -ffp-contract=off and written in the reference's operation
// order, so every result equals the reference's bit for bit: the per-kind
// totals accumulate in member (filler) order, the scales and remainders are
// the same expressions, and kinds are visited in ascending key order like the
// reference's BTreeMap<ResourceKind, f64>.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <vector>

#include "texo_gp.h"

namespace {

// checked_add (:280-291): accumulate, fail on a non-finite total
bool checked_add(std::map<uint32_t, double>& totals, uint32_t kind, double value) {
  double& t = totals[kind];
  t += value;
  return std::isfinite(t);
}

// usize_to_f64 (:369-371): through u32, as the reference converts
bool to_f64(uint64_t v, double* out) {
  if (v > 0xffffffffull) return false;
  *out = (double)(uint32_t)v;
  return true;
}

}  // namespace

extern "C" int32_t texo_gp_routability_optimized_area(double current_area, double horizontal_utilization,
                                                      double vertical_utilization, double* out) {
  if (!out) return TEXO_GP_ERR_INVALID_ARGUMENT;
  if (!std::isfinite(current_area) || current_area < 0.0 || !std::isfinite(horizontal_utilization) ||
      horizontal_utilization < 0.0 || !std::isfinite(vertical_utilization) || vertical_utilization < 0.0)
    return TEXO_GP_ERR_INSTANCE_AREA_OVERFLOW;
  const double utilization = std::max(horizontal_utilization, vertical_utilization);
  const double factor = std::min(utilization * utilization, 2.0);
  const double area = current_area * factor;
  if (!std::isfinite(area)) return TEXO_GP_ERR_INSTANCE_AREA_OVERFLOW;
  *out = area;
  return TEXO_GP_OK;
}

extern "C" int32_t texo_gp_routability_optimized_area_from_bin(double current_area, double horizontal_demand,
                                                               uint64_t horizontal_capacity, double vertical_demand,
                                                               uint64_t vertical_capacity, double* out) {
  if (!out) return TEXO_GP_ERR_INVALID_ARGUMENT;
  // demand over capacity; capacity up to 2^53 converted exactly from its two halves
  auto utilization = [](double demand, uint64_t capacity, double* u) {
    if (!std::isfinite(demand) || demand < 0.0) return false;
    if (capacity == 0) {
      *u = demand == 0.0 ? 0.0 : INFINITY;
      return true;
    }
    if (capacity > (1ull << 53)) return false;
    const double c = (double)(uint32_t)(capacity >> 32) * 4294967296.0 + (double)(uint32_t)(capacity & 0xffffffffu);
    *u = demand / c;
    return true;
  };
  double h = 0.0, v = 0.0;
  if (!utilization(horizontal_demand, horizontal_capacity, &h) || !utilization(vertical_demand, vertical_capacity, &v))
    return TEXO_GP_ERR_INSTANCE_AREA_OVERFLOW;
  if (std::isinf(h) || std::isinf(v)) {
    if (!std::isfinite(current_area) || current_area < 0.0) return TEXO_GP_ERR_INSTANCE_AREA_OVERFLOW;
    const double area = current_area * 2.0;
    if (!std::isfinite(area)) return TEXO_GP_ERR_INSTANCE_AREA_OVERFLOW;
    *out = area;
    return TEXO_GP_OK;
  }
  return texo_gp_routability_optimized_area(current_area, h, v, out);
}

extern "C" int32_t texo_gp_pin_optimized_area(uint64_t pin_count, double unit_area_pin_capacity,
                                              double local_pin_utilization, double* out) {
  if (!out) return TEXO_GP_ERR_INVALID_ARGUMENT;
  if (!std::isfinite(unit_area_pin_capacity) || unit_area_pin_capacity <= 0.0 ||
      !std::isfinite(local_pin_utilization) || local_pin_utilization < 0.0)
    return TEXO_GP_ERR_INSTANCE_AREA_OVERFLOW;
  double pins = 0.0;
  if (!to_f64(pin_count, &pins)) return TEXO_GP_ERR_INSTANCE_AREA_OVERFLOW;
  const double area = pins / unit_area_pin_capacity * std::min(local_pin_utilization, 1.5);
  if (!std::isfinite(area)) return TEXO_GP_ERR_INSTANCE_AREA_OVERFLOW;
  *out = area;
  return TEXO_GP_OK;
}

extern "C" int32_t texo_gp_adjust_instance_areas(uint64_t num_members, const uint32_t* member_kind,
                                                 const double* current_area, const double* routability_area,
                                                 const double* pin_area, const double* clustering_area,
                                                 uint64_t num_fillers, const uint32_t* filler_kind,
                                                 const double* filler_area, double* out_member_area,
                                                 double* out_filler_area, int32_t* requires_optimizer_reset,
                                                 uint32_t max_scales, uint32_t* num_scales, uint32_t* scale_kind,
                                                 double* scale, uint64_t* error_index) {
  const uint64_t n = num_members, nf = num_fillers;
  if ((n && (!member_kind || !current_area || !routability_area || !pin_area || !clustering_area ||
             !out_member_area)) ||
      (nf && (!filler_kind || !filler_area || !out_filler_area)))
    return TEXO_GP_ERR_INVALID_ARGUMENT;
  // validate_inputs (:255-278)
  auto ok_area = [](double a) { return std::isfinite(a) && !(a < 0.0); };
  for (uint64_t i = 0; i < n; ++i)
    if (!ok_area(current_area[i]) || !ok_area(routability_area[i]) || !ok_area(pin_area[i]) ||
        !ok_area(clustering_area[i])) {
      if (error_index) *error_index = i;
      return TEXO_GP_ERR_INSTANCE_AREA_MEMBER;
    }
  for (uint64_t j = 0; j < nf; ++j)
    if (!ok_area(filler_area[j])) {
      if (error_index) *error_index = j;
      return TEXO_GP_ERR_INSTANCE_AREA_FILLER;
    }
  // requested area: the largest of routability, pin, clustering and current (:163-172)
  std::vector<double> requested(n), delta(n);
  for (uint64_t i = 0; i < n; ++i) {
    requested[i] = std::max(std::max(std::max(routability_area[i], pin_area[i]), clustering_area[i]), current_area[i]);
    delta[i] = requested[i] - current_area[i];
  }
  std::map<uint32_t, double> desired, available, scales, target, actual;
  for (uint64_t i = 0; i < n; ++i)
    if (!checked_add(desired, member_kind[i], delta[i])) return TEXO_GP_ERR_INSTANCE_AREA_OVERFLOW;
  for (uint64_t j = 0; j < nf; ++j)
    if (!checked_add(available, filler_kind[j], filler_area[j])) return TEXO_GP_ERR_INSTANCE_AREA_OVERFLOW;
  // elfPlace eq. (24): per-kind scale, bounded by the kind's filler area (:187-203)
  for (const auto& [kind, want] : desired) {
    const auto it = available.find(kind);
    const double have = it == available.end() ? 0.0 : it->second;
    scales[kind] = want == 0.0 ? 1.0 : std::min(have / want, 1.0);
    target[kind] = std::min(want, have);
  }
  std::map<uint32_t, uint64_t> last_member;
  for (uint64_t i = 0; i < n; ++i) last_member[member_kind[i]] = i;
  for (uint64_t i = 0; i < n; ++i) {
    const uint32_t kind = member_kind[i];
    const double s = scales[kind];
    double increase = delta[i] * s;
    if (last_member[kind] == i) {   // the kind's last member takes the remainder
      const auto it = actual.find(kind);
      const double assigned = it == actual.end() ? 0.0 : it->second;
      increase = std::clamp(target[kind] - assigned, 0.0, delta[i]);
    }
    // a full scale installs the requested bits themselves (:228-232)
    const double adjusted = s == 1.0 ? requested[i] : current_area[i] + increase;
    if (!std::isfinite(adjusted)) return TEXO_GP_ERR_INSTANCE_AREA_OVERFLOW;
    if (!checked_add(actual, kind, adjusted - current_area[i])) return TEXO_GP_ERR_INSTANCE_AREA_OVERFLOW;
    out_member_area[i] = adjusted;
  }
  // adjusted_filler_areas (:293-332): fillers shrink in proportion per kind
  bool grew = false;
  for (const auto& kv : actual) grew = grew || kv.second != 0.0;
  if (!grew) {
    for (uint64_t j = 0; j < nf; ++j) out_filler_area[j] = filler_area[j];
  } else {
    std::map<uint32_t, double> remaining, assigned;
    for (const auto& [kind, have] : available) {
      const auto it = actual.find(kind);
      const double inc = it == actual.end() ? 0.0 : it->second;
      remaining[kind] = std::max(have - inc, 0.0);
    }
    std::map<uint32_t, uint64_t> last_filler;
    for (uint64_t j = 0; j < nf; ++j) last_filler[filler_kind[j]] = j;
    for (uint64_t j = 0; j < nf; ++j) {
      const uint32_t kind = filler_kind[j];
      const double total = available[kind], want = remaining[kind];
      double area;
      if (last_filler[kind] == j) {
        const auto it = assigned.find(kind);
        area = std::max(want - (it == assigned.end() ? 0.0 : it->second), 0.0);
      } else if (total == 0.0) {
        area = 0.0;
      } else {
        area = filler_area[j] * want / total;
      }
      const double tolerance = 64.0 * DBL_EPSILON * std::max(std::fabs(filler_area[j]), 1.0);
      if (!std::isfinite(area) || area > filler_area[j] + tolerance) return TEXO_GP_ERR_INSTANCE_AREA_OVERFLOW;
      area = std::min(area, filler_area[j]);
      if (!checked_add(assigned, kind, area)) return TEXO_GP_ERR_INSTANCE_AREA_OVERFLOW;
      out_filler_area[j] = area;
    }
  }
  // validate_postconditions (:334-367): no member shrinks, no filler grows,
  // every kind's total conserved within 64 eps (terms) max(|total|, 1)
  {
    std::map<uint32_t, double> before, after;
    for (uint64_t i = 0; i < n; ++i) {
      if (out_member_area[i] < current_area[i] || !std::isfinite(out_member_area[i]))
        return TEXO_GP_ERR_INSTANCE_AREA_POSTCONDITION;
      if (!checked_add(before, member_kind[i], current_area[i]) || !checked_add(after, member_kind[i], out_member_area[i]))
        return TEXO_GP_ERR_INSTANCE_AREA_OVERFLOW;
    }
    for (uint64_t j = 0; j < nf; ++j) {
      if (out_filler_area[j] < 0.0 || out_filler_area[j] > filler_area[j] || !std::isfinite(out_filler_area[j]))
        return TEXO_GP_ERR_INSTANCE_AREA_POSTCONDITION;
      if (!checked_add(before, filler_kind[j], filler_area[j]) || !checked_add(after, filler_kind[j], out_filler_area[j]))
        return TEXO_GP_ERR_INSTANCE_AREA_OVERFLOW;
    }
    if (n + nf > 0xffffffffull) return TEXO_GP_ERR_INSTANCE_AREA_OVERFLOW;
    const double terms = std::max((double)(uint32_t)(n + nf), 1.0);
    for (const auto& [kind, b] : before) {
      const auto it = after.find(kind);
      const double a = it == after.end() ? 0.0 : it->second;
      const double tolerance = 64.0 * DBL_EPSILON * terms * std::max(std::fabs(b), 1.0);
      if (std::fabs(b - a) > tolerance) return TEXO_GP_ERR_INSTANCE_AREA_POSTCONDITION;
    }
  }
  if (requires_optimizer_reset) {
    bool any = false;
    for (const auto& kv : actual) any = any || kv.second > 0.0;
    *requires_optimizer_reset = any ? 1 : 0;
  }
  if (num_scales) {
    if (scales.size() > max_scales) return TEXO_GP_ERR_INVALID_ARGUMENT;
    uint32_t k = 0;
    for (const auto& [kind, s] : scales) {
      if (scale_kind) scale_kind[k] = kind;
      if (scale) scale[k] = s;
      ++k;
    }
    *num_scales = k;
  }
  return TEXO_GP_OK;
}
