// routable.cpp — eplace::place with a routing-capacity map
// (crates/texo-pnr/src/eplace.rs:242-420) behind one C-ABI call.
//
// The loop is host code over this library's own entry points: density rounds
// on one handle (texo_gp_optimize_round, host or device engine), between them the
// area-adjustment proposal of eplace.rs:627-740 (the nets' bounding boxes,
// the RUDY map on the GPU, every movable member's utilization, elfPlace
// eq. 29 for LUT and register members, the register-clustering areas on the
// GPU, the charge-conserving instance areas) and its installation
// (texo_gp_set_charges). Per-kind totals and the relative increases are
// summed in ascending kind order like the reference's BTreeMaps; the host
// arithmetic is compiled without fused multiply-adds.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "texo_gp.h"

namespace tgp {
void set_last_error(const std::string& s);
}

namespace {

constexpr double kSqrt2 = 1.4142135623730951;

uint32_t kind_key(const texo_gp_field& f) { return f.kind << 8 | f.lut_inputs; }

// rounded_coordinate (lib.rs:4565-4568): round half away from zero, clamp to
// the grid; NaN maps to 0 like Rust's saturating cast.
uint32_t rounded(double v, uint32_t extent) {
  double r = std::round(v);
  if (std::isnan(r)) return 0;
  const double hi = (double)(extent - 1);
  if (r < 0.0) r = 0.0;
  if (r > hi) r = hi;
  return (uint32_t)r;
}

// ContinuousRoutingDemand::utilization (eplace.rs:822-853)
bool utilization(double demand, uint32_t capacity, double* out) {
  if (capacity == 0) {
    *out = demand == 0.0 ? 0.0 : kSqrt2;
    return true;
  }
  const double u = demand / (double)capacity;
  if (!(std::isfinite(u) && u >= 0.0)) return false;
  *out = u;
  return true;
}

bool movable_unit(const texo_gp_problem* p, uint32_t u) {
  return p->lower_xy[2 * u] != p->upper_xy[2 * u] || p->lower_xy[2 * u + 1] != p->upper_xy[2 * u + 1];
}

// area_adjustment_round_limit (eplace.rs:584-626)
int32_t round_limit(const texo_gp_problem* p, uint64_t* limit) {
  double initial = 0.0;
  std::vector<uint8_t> used(p->num_fields, 0);
  for (uint32_t u = 0; u < p->num_units; ++u) {
    if (!movable_unit(p, u)) continue;
    for (uint32_t i = p->member_ptr[u]; i < p->member_ptr[u + 1]; ++i) {
      initial += p->member_charge[i];
      used[p->member_field[i]] = 1;
    }
  }
  const size_t tiles = (size_t)p->width * p->height;
  double available = 0.0;
  for (uint32_t f = 0; f < p->num_fields; ++f) {
    if (!used[f]) continue;
    uint64_t cap = 0;
    for (size_t t = 0; t < tiles; ++t) cap += p->capacity[(size_t)f * tiles + t];
    uint64_t fixed = 0;
    for (uint32_t j = 0; j < p->num_fixed_occupancy; ++j) fixed += p->fixed_occupancy[3 * j] == f;
    const uint64_t free_bels = cap >= fixed ? cap - fixed : 0;
    if (free_bels > 0xffffffffull) return TEXO_GP_ERR_INVALID_NORMALIZATION;
    available += (double)(uint32_t)free_bels;
  }
  if (!(std::isfinite(initial) && initial > 0.0 && available >= initial)) return TEXO_GP_ERR_INVALID_NORMALIZATION;
  double threshold = initial;
  uint64_t rounds = 0;
  while (threshold < available) {
    threshold *= 1.01;
    if (!std::isfinite(threshold)) return TEXO_GP_ERR_INVALID_NORMALIZATION;
    ++rounds;
  }
  *limit = rounds + 1;
  return TEXO_GP_OK;
}

// external_baseline_net_bounding_boxes (analytical_placement.rs:238-276): the
// (min x, max x, min y, max y) of every net not wholly inside one unit, fixed
// cells at their coordinates, others at unit origin + cell offset.
void net_boxes(const texo_gp_problem* p, const double* origin, std::vector<double>& boxes) {
  boxes.clear();
  for (uint32_t e = 0; e < p->num_nets; ++e) {
    const uint32_t a = p->net_ptr[e], b = p->net_ptr[e + 1];
    if (a == b) continue;
    const uint32_t first_unit = p->cell_unit[p->pin_cell[a]];
    bool one_unit = true;
    for (uint32_t k = a + 1; k < b && one_unit; ++k) one_unit = p->cell_unit[p->pin_cell[k]] == first_unit;
    if (one_unit) continue;
    double lx = 0, hx = 0, ly = 0, hy = 0;
    for (uint32_t k = a; k < b; ++k) {
      const uint32_t c = p->pin_cell[k];
      double x, y;
      if (p->cell_fixed[c]) {
        x = p->cell_fixed_xy[2 * c];
        y = p->cell_fixed_xy[2 * c + 1];
      } else {
        const uint32_t u = p->cell_unit[c];
        x = origin[2 * u] + p->cell_offset_xy[2 * c];
        y = origin[2 * u + 1] + p->cell_offset_xy[2 * c + 1];
      }
      if (k == a) {
        lx = hx = x;
        ly = hy = y;
      } else {
        lx = std::min(lx, x);
        hx = std::max(hx, x);
        ly = std::min(ly, y);
        hy = std::max(hy, y);
      }
    }
    boxes.insert(boxes.end(), {lx, hx, ly, hy});
  }
}

struct Control {
  uint64_t clock_lsr[2];
  uint64_t ce;
};

struct Proposal {
  std::vector<uint32_t> members;       // problem member indices of movable units
  std::vector<double> member_area;     // adjusted areas of those members
  std::vector<double> filler_area;
  bool reset = false;
  double total_relative_increase = 0, maximum_relative_increase = 0;
  double max_h = 0, max_v = 0;
  uint64_t inflated = 0;
};

// propose_area_adjustment (eplace.rs:627-740) at unit origins `origin` [2U]
// with the installed member charges `charge` and fillers (`filler_field`,
// `filler_charge`).
int32_t propose(const texo_gp_problem* p, int32_t device, const texo_gp_routing_capacity* cap,
                const std::map<uint32_t, Control>& controls, uint64_t movable_instances, const double* origin,
                const std::vector<double>& charge, const std::vector<uint32_t>& filler_field,
                const std::vector<double>& filler_charge, Proposal* out) {
  const uint32_t W = cap->width, H = cap->height;
  std::vector<double> boxes;
  net_boxes(p, origin, boxes);
  std::vector<double> hd((size_t)W * H), vd((size_t)W * H);
  double ms = 0;
  int32_t s = texo_gp_routing_demand(device, W, H, boxes.size() / 4, boxes.empty() ? nullptr : boxes.data(),
                                     hd.data(), vd.data(), &ms);
  if (s) return s;
  Proposal& P = *out;
  P = Proposal();
  std::vector<uint32_t> keys;
  std::vector<double> cur, routing, clus;
  std::vector<uint32_t> reg_slot;    // member slots that are registers
  std::vector<double> reg_xy;
  std::vector<uint64_t> reg_cl, reg_ce;
  for (uint32_t u = 0; u < p->num_units; ++u) {
    if (!movable_unit(p, u)) continue;
    for (uint32_t i = p->member_ptr[u]; i < p->member_ptr[u + 1]; ++i) {
      const texo_gp_field& fd = p->fields[p->member_field[i]];
      const double mx = origin[2 * u] + p->member_offset_xy[2 * i];
      const double my = origin[2 * u + 1] + p->member_offset_xy[2 * i + 1];
      const size_t t = (size_t)rounded(my, H) * W + rounded(mx, W);
      double hu, vu;
      if (!utilization(hd[t], cap->horizontal[t], &hu) || !utilization(vd[t], cap->vertical[t], &vu))
        return TEXO_GP_ERR_INVALID_NORMALIZATION;
      P.max_h = std::max(P.max_h, hu);
      P.max_v = std::max(P.max_v, vu);
      double area = charge[i];
      s = texo_gp_routability_optimized_area(charge[i], std::min(hu, kSqrt2), std::min(vu, kSqrt2), &area);
      if (s) return s;
      // routability_adjusted_member_area (eplace.rs:741-758): LUT and
      // register members take the inflated area, other kinds keep theirs
      if (fd.kind != TEXO_GP_KIND_LUT && fd.kind != TEXO_GP_KIND_REGISTER) area = charge[i];
      if (fd.kind == TEXO_GP_KIND_REGISTER && !controls.empty()) {
        auto it = controls.find(p->member_cell[i]);
        if (it == controls.end()) {
          tgp::set_last_error("texo_gp_place_routable: register cell " + std::to_string(p->member_cell[i]) +
                              " has no control set");
          return TEXO_GP_ERR_INVALID_NORMALIZATION;
        }
        reg_slot.push_back((uint32_t)P.members.size());
        reg_xy.insert(reg_xy.end(), {mx, my});
        reg_cl.insert(reg_cl.end(), {it->second.clock_lsr[0], it->second.clock_lsr[1]});
        reg_ce.push_back(it->second.ce);
      }
      P.members.push_back(i);
      keys.push_back(kind_key(fd));
      cur.push_back(charge[i]);
      routing.push_back(area);
    }
  }
  const size_t n = P.members.size();
  clus.assign(n, 0.0);
  if (!reg_slot.empty()) {
    std::vector<double> areas(reg_slot.size());
    s = texo_gp_register_clustering_areas(device, reg_slot.size(), reg_xy.data(), reg_cl.data(), reg_ce.data(),
                                          movable_instances, areas.data(), &ms);
    if (s) return s;
    for (size_t r = 0; r < reg_slot.size(); ++r) clus[reg_slot[r]] = areas[r];
  }
  std::vector<uint32_t> fkeys(filler_field.size());
  for (size_t j = 0; j < filler_field.size(); ++j) fkeys[j] = kind_key(p->fields[filler_field[j]]);
  std::vector<double> pin(n, 0.0);
  P.member_area.assign(n, 0.0);
  P.filler_area.assign(filler_charge.size(), 0.0);
  int32_t reset = 0;
  uint32_t nscales = 0;
  uint32_t scale_kind[64];
  double scale[64];
  uint64_t err = 0;
  s = texo_gp_adjust_instance_areas(n, keys.data(), cur.data(), routing.data(), pin.data(), clus.data(),
                                    filler_charge.size(), fkeys.data(), filler_charge.data(), P.member_area.data(),
                                    P.filler_area.data(), &reset, 64, &nscales, scale_kind, scale, &err);
  if (s) return s;
  P.reset = reset != 0;
  std::map<uint32_t, double> before, increase;
  for (size_t k = 0; k < n; ++k) {
    before[keys[k]] += cur[k];
    const double inc = P.member_area[k] - cur[k];
    increase[keys[k]] += inc;
    P.inflated += inc > 0.0;
  }
  double before_total = 0.0, increase_total = 0.0;
  for (const auto& kv : before) before_total += kv.second;
  for (const auto& kv : increase) increase_total += kv.second;
  P.total_relative_increase = increase_total / before_total;
  P.maximum_relative_increase = 0.0;
  for (const auto& kv : before) P.maximum_relative_increase = std::max(P.maximum_relative_increase,
                                                                       increase[kv.first] / kv.second);
  if (!std::isfinite(P.total_relative_increase) || !std::isfinite(P.maximum_relative_increase))
    return TEXO_GP_ERR_INVALID_NORMALIZATION;
  return TEXO_GP_OK;
}

int32_t fail(texo_gp_stats* stats, int32_t s) {
  if (stats && stats->status == 0) stats->status = s;
  return s;
}

}  // namespace

extern "C" int32_t texo_gp_place_routable(const texo_gp_problem* problem, const texo_gp_params* params,
                                          const texo_gp_routing_capacity* capacity, uint64_t num_register_controls,
                                          const texo_gp_register_control* register_controls, uint32_t* out_targets_xy,
                                          double* out_coordinates, texo_gp_stats* stats,
                                          texo_gp_routable_report* report) {
  if (stats) std::memset(stats, 0, sizeof(*stats));
  if (report) std::memset(report, 0, sizeof(*report));
  if (!problem || !out_targets_xy) return fail(stats, TEXO_GP_ERR_INVALID_ARGUMENT);
  if (num_register_controls && !register_controls) return fail(stats, TEXO_GP_ERR_INVALID_ARGUMENT);
  if (!capacity) {
    // no routing capacity: the pure density objective, one final round
    const int32_t s = texo_gp_place(problem, params, out_targets_xy, out_coordinates, stats);
    if (report && s == TEXO_GP_OK) {
      report->rounds = 1;
      if (stats) report->iterations = stats->iterations;
    }
    return s;
  }
  if (capacity->width == 0 || capacity->height == 0 || !capacity->horizontal || !capacity->vertical)
    return fail(stats, TEXO_GP_ERR_INVALID_NORMALIZATION);
  // register controls by cell; a cell listed twice is the reference's
  // InvalidNormalization (eplace.rs:320-326)
  std::map<uint32_t, Control> controls;
  for (uint64_t r = 0; r < num_register_controls; ++r) {
    const texo_gp_register_control& c = register_controls[r];
    if (!controls.emplace(c.cell, Control{{c.clock_lsr[0], c.clock_lsr[1]}, c.ce}).second) {
      tgp::set_last_error("texo_gp_place_routable: cell " + std::to_string(c.cell) + " has two control sets");
      return fail(stats, TEXO_GP_ERR_INVALID_NORMALIZATION);
    }
  }
  texo_gp_params prm;
  if (params)
    prm = *params;
  else
    texo_gp_default_params(&prm);
  texo_gp_handle h = nullptr;
  int32_t s = texo_gp_create(problem, &prm, &h);
  if (s) return fail(stats, s);
  struct Closer {
    texo_gp_handle h;
    ~Closer() { texo_gp_destroy(h); }
  } closer{h};
  uint64_t limit = 0;
  s = round_limit(problem, &limit);
  if (s) return fail(stats, s);
  uint64_t units = 0, fillers = 0, ncoord = 0;
  uint32_t bx = 0, by = 0, nf = 0;
  s = texo_gp_sizes(h, &units, &fillers, &ncoord, &bx, &by, &nf);
  if (s) return fail(stats, s);
  std::vector<uint32_t> filler_field(fillers);
  std::vector<double> filler_charge(fillers);
  s = texo_gp_fillers(h, fillers ? filler_field.data() : nullptr, fillers ? filler_charge.data() : nullptr);
  if (s) return fail(stats, s);
  uint64_t movable_instances = 0;   // cells of movable units
  for (uint32_t c = 0; c < problem->num_cells; ++c) movable_instances += movable_unit(problem, problem->cell_unit[c]);
  const uint32_t members_total = problem->member_ptr[problem->num_units];
  std::vector<double> charge(problem->member_charge, problem->member_charge + members_total);
  std::vector<double> coords(ncoord);
  std::vector<double> scales;
  uint64_t completed = 0, area_round = 0;
  bool have_previous = false, reset = false;
  double previous = 0.0;
  texo_gp_stats st;
  for (;;) {
    const int32_t stop = (have_previous && previous < 0.01) ? 0 : 1;
    texo_gp_round rd;
    std::memset(&rd, 0, sizeof(rd));
    rd.stop = stop;
    rd.reset_multipliers = reset ? 1 : 0;
    rd.density_scales = scales.empty() ? nullptr : scales.data();
    rd.completed_iterations = completed;
    texo_gp_round_result res;
    s = texo_gp_optimize_round(h, &rd, out_targets_xy, coords.data(), &st, &res);
    if (s != TEXO_GP_OK && s != TEXO_GP_ERR_DID_NOT_CONVERGE) {
      if (stats) *stats = st;
      return fail(stats, s);
    }
    if (scales.empty()) scales.assign(res.density_scales, res.density_scales + nf);
    completed = res.completed_iterations;
    if (report) {
      report->rounds += 1;
      report->iterations = completed;
    }
    if (stop == 0 || res.exhausted) {
      if (stats) {
        *stats = st;
        stats->iterations = (uint32_t)completed;
      }
      if (out_coordinates) std::memcpy(out_coordinates, coords.data(), ncoord * sizeof(double));
      return s;
    }
    Proposal P;
    s = propose(problem, prm.device, capacity, controls, movable_instances, coords.data(), charge, filler_field,
                filler_charge, &P);
    if (s) return fail(stats, s);
    if (report) {
      report->last_relative_increase = P.total_relative_increase;
      report->last_maximum_relative_increase = P.maximum_relative_increase;
      report->max_horizontal_utilization = P.max_h;
      report->max_vertical_utilization = P.max_v;
      report->last_members_inflated = P.inflated;
    }
    if (!P.reset) {
      have_previous = true;
      previous = 0.0;
      reset = true;
      continue;
    }
    if (area_round >= limit) {
      tgp::set_last_error("texo_gp_place_routable: area round limit");
      return fail(stats, TEXO_GP_ERR_INVALID_NORMALIZATION);
    }
    for (size_t k = 0; k < P.members.size(); ++k) charge[P.members[k]] = P.member_area[k];
    filler_charge = P.filler_area;
    s = texo_gp_set_charges(h, charge.data(), fillers ? filler_charge.data() : nullptr);
    if (s) return fail(stats, s);
    have_previous = true;
    previous = P.total_relative_increase;
    reset = true;
    ++area_round;
    if (report) report->area_rounds = (uint32_t)area_round;
  }
}
