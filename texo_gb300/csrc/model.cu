// model.cpp — host preprocessing of a texo_gp_problem into the device layout.
//
// The setup mirrors the reference: capacity per kind minus fixed occupancy and
// its B-spline smoothing (DensityModel::new, electrostatic_placement.rs:139-196),
// capacity-proportional fillers (initial_fillers, :198-240), coordinates and
// bounds (initial_coordinates_and_bounds, eplace.rs:1441-1468), the wirelength
// preconditioner and cell incidence (analytical_placement.rs:177-231) and the
// per-kind gamma weights (density_gamma_weights, eplace.rs:1424-1439).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <future>
#include <thread>

#include "engine.h"

namespace tgp {

namespace {
inline double clampd(double v, double lo, double hi) { return v < lo ? lo : (v > hi ? hi : v); }

// quadratic_bspline_axis / deposit_quadratic_bspline in FP64
// (electrostatic_placement.rs:900-916, 950-976), used for the capacity background.
void deposit64(std::vector<double>& g, uint32_t W, uint32_t H, double x, double y, double q) {
  auto axis = [](uint32_t n, double c, size_t idx[3], double w[3]) {
    const double maximum = (double)(n - 1);
    c = clampd(c, 0.0, maximum);
    const double cc = std::fmin(std::floor(c + 0.5), maximum);
    const size_t center = (size_t)cc;
    const double o = c - cc, a = 0.5 - o, b = 0.5 + o;
    idx[0] = center == 0 ? 0 : center - 1;
    idx[1] = center;
    idx[2] = std::min<size_t>(center + 1, n - 1);
    w[0] = 0.5 * (a * a);
    w[1] = 0.75 - o * o;
    w[2] = 0.5 * (b * b);
  };
  size_t ix[3], iy[3];
  double wx[3], wy[3];
  axis(W, x, ix, wx);
  axis(H, y, iy, wy);
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) g[iy[r] * W + ix[c]] += q * wx[c] * wy[r];
}

double u64_to_f64(uint64_t v) {
  return (double)(uint32_t)(v >> 32) * 4294967296.0 + (double)(uint32_t)(v & 0xffffffffu);
}
}  // namespace

double HostModel::overflow_target(uint32_t f) const {
  if (params.overflow_target_override >= 0.0) return params.overflow_target_override;
  switch (kinds[f].kind) {
    case TEXO_GP_KIND_MEMORY:
    case TEXO_GP_KIND_DSP:
      return 0.20;
    case TEXO_GP_KIND_LUT:
    case TEXO_GP_KIND_REGISTER:
      return 0.10;
    default:
      return 0.0;
  }
}

double HostModel::gamma_base_tiles() const {
  return params.gamma_base * (identity ? 1.0 : 1.0 / sx);
}

int32_t build_model(const texo_gp_problem* p, const texo_gp_params* prm, HostModel& m, uint64_t* err) {
  uint64_t dummy;
  if (!err) err = &dummy;
  *err = 0;
  if (!p || !prm) return TEXO_GP_ERR_INVALID_ARGUMENT;
  if (p->width == 0 || p->height == 0) return TEXO_GP_ERR_EMPTY_GRID;
  m.params = *prm;
  m.W = p->width;
  m.H = p->height;
  m.Wb = prm->bins_x ? prm->bins_x : p->width;
  m.Hb = prm->bins_y ? prm->bins_y : p->height;
  if ((uint64_t)m.Wb * m.Hb > (1ull << 26) || (uint64_t)m.W * m.H > (1ull << 30)) return TEXO_GP_ERR_GRID_TOO_LARGE;
  m.identity = (m.Wb == m.W && m.Hb == m.H);
  m.sx = (double)m.Wb / (double)m.W;
  m.sy = (double)m.Hb / (double)m.H;
  m.td = prm->target_density;
  if (!(m.td > 0.0 && m.td <= 1.0)) return TEXO_GP_ERR_INVALID_ARGUMENT;
  const uint32_t U = p->num_units;
  if (U == 0 || !p->member_ptr || !p->initial_xy || !p->lower_xy || !p->upper_xy) return TEXO_GP_ERR_INVALID_ARGUMENT;
  if (p->num_fields && (!p->fields || !p->capacity)) return TEXO_GP_ERR_INVALID_ARGUMENT;
  const uint32_t M = p->member_ptr[U];
  for (uint32_t u = 0; u < U; ++u)
    if (p->member_ptr[u + 1] < p->member_ptr[u]) return TEXO_GP_ERR_INVALID_ARGUMENT;
  const size_t tiles = (size_t)m.W * m.H;
  std::vector<uint64_t> member_count(p->num_fields, 0);
  for (uint32_t i = 0; i < M; ++i) {
    if (p->member_field[i] >= p->num_fields) return TEXO_GP_ERR_INVALID_ARGUMENT;
    member_count[p->member_field[i]]++;
  }
  // hypergraph: pins and nets (AnalyticalHypergraph::new, analytical_placement.rs:116-168).
  // It is validated and its pin layout started first, on a second thread
  // beside the density sections below; its errors are reported after
  // theirs, in the reference's order.
  const uint32_t C = p->num_cells, E = p->num_nets;
  int32_t hyper_status = TEXO_GP_OK;
  uint64_t hyper_err = 0;
  auto hyper_check = [&]() -> int32_t {
    if (E && (!p->net_ptr || !p->pin_cell)) return TEXO_GP_ERR_INVALID_ARGUMENT;
    for (uint32_t c = 0; c < C; ++c)
      if (p->cell_unit[c] >= U) return TEXO_GP_ERR_INVALID_ARGUMENT;
    for (uint32_t i = 0; i < M; ++i)
      if (p->member_cell && p->member_cell[i] >= C) return TEXO_GP_ERR_INVALID_ARGUMENT;
    // nets and timed arcs: the two passes over them read only checked indices
    for (uint32_t e = 0; e < E; ++e) {
      const uint32_t b = p->net_ptr[e], en = p->net_ptr[e + 1];
      if (en < b + 2) {
        hyper_err = e;
        return TEXO_GP_ERR_INVALID_ARGUMENT;
      }
      for (uint32_t k = b; k < en; ++k)
        if (p->pin_cell[k] >= C) return TEXO_GP_ERR_INVALID_ARGUMENT;
    }
    for (uint32_t a = 0; a < p->num_timed_arcs; ++a) {
      if (p->arc_driver_cell[a] >= C || p->arc_sink_cell[a] >= C) return TEXO_GP_ERR_INVALID_ARGUMENT;
      if (u64_to_f64(p->arc_extra_weight[a]) > 16777216.0) return TEXO_GP_ERR_FIXED_POINT_RANGE;
    }
    return TEXO_GP_OK;
  };
  const size_t arcs = p->num_timed_arcs;
  auto pin_of = [&](uint32_t cell, int& unit, double& bx, double& by) {
    if (p->cell_fixed[cell]) {
      unit = -1;
      bx = p->cell_fixed_xy[2 * (size_t)cell];
      by = p->cell_fixed_xy[2 * (size_t)cell + 1];
    } else {
      unit = (int)p->cell_unit[cell];
      bx = p->cell_offset_xy[2 * (size_t)cell];
      by = p->cell_offset_xy[2 * (size_t)cell + 1];
    }
  };

  // Pin layout (second thread): degree classes 2 | 3-4 | 5-8 | 9-16 | 17-32
  // | 33+ laid out class by class (a counting sort over the classes, nets of
  // a class in input order), then the timed arcs as 2-pin nets; every output
  // is sized once and filled by index. pin_count[u] = pins of unit u. The
  // WA kernel gives a net of class c groups[c] lanes, so that a lane holds
  // at most four pins of a net up to 32 pins (33+: one warp per net).
  constexpr int kNetClasses = 6;
  static const int groups[kNetClasses] = {1, 1, 2, 4, 8, 32};
  auto cls = [](uint32_t deg) {
    return deg <= 2 ? 0 : deg <= 4 ? 1 : deg <= 8 ? 2 : deg <= 16 ? 3 : deg <= 32 ? 4 : 5;
  };
  size_t pins = 0;   // set once the hypergraph is validated
  std::vector<double> pin_count(U, 0.0);
  bool layout_ok = true;
  auto layout = [&]() {
    try {
      size_t nets_in[kNetClasses] = {0, 0, 0, 0, 0, 0}, pins_in[kNetClasses] = {0, 0, 0, 0, 0, 0};
      for (uint32_t e = 0; e < E; ++e) {
        const uint32_t deg = p->net_ptr[e + 1] - p->net_ptr[e];
        nets_in[cls(deg)]++;
        pins_in[cls(deg)] += deg;
      }
      size_t net_at[kNetClasses], pin_at[kNetClasses];
      for (int c = 0, n0 = 0, p0 = 0; c < kNetClasses; ++c) {
        net_at[c] = n0;
        pin_at[c] = p0;
        m.class_begin[c] = n0;
        m.class_group[c] = groups[c];
        n0 += (int)nets_in[c];
        p0 += (int)pins_in[c];
      }
      m.net_ptr.resize((size_t)E + arcs + 1);
      m.net_w.assign((size_t)E + arcs, 1.0f);
      m.pin_unit.resize(pins + 2 * arcs);
      m.pin_base.resize(2 * (pins + 2 * arcs));
      m.net_ptr[0] = 0;
      for (uint32_t e = 0; e < E; ++e) {
        const uint32_t b = p->net_ptr[e], en = p->net_ptr[e + 1];
        const int c = cls(en - b);
        const size_t slot = net_at[c]++;
        size_t q = pin_at[c];
        for (uint32_t k = b; k < en; ++k, ++q) {
          int unit;
          pin_of(p->pin_cell[k], unit, m.pin_base[2 * q], m.pin_base[2 * q + 1]);
          m.pin_unit[q] = unit;
          if (unit >= 0) pin_count[unit] += 1.0;
        }
        pin_at[c] = q;
        m.net_ptr[slot + 1] = (int)q;
      }
      m.n_hpwl_nets = (int)E;
      m.class_begin[kNetClasses] = (int)E;   // timed arcs: 2-pin nets, one lane each
      m.class_group[kNetClasses] = 1;
      for (uint32_t a = 0; a < arcs; ++a) {
        size_t q = pins + 2 * (size_t)a;
        for (uint32_t cell : {p->arc_driver_cell[a], p->arc_sink_cell[a]}) {
          int unit;
          pin_of(cell, unit, m.pin_base[2 * q], m.pin_base[2 * q + 1]);
          m.pin_unit[q] = unit;
          ++q;
        }
        m.net_ptr[(size_t)E + a + 1] = (int)q;
        m.net_w[(size_t)E + a] = (float)u64_to_f64(p->arc_extra_weight[a]);
      }
    } catch (...) {
      layout_ok = false;
    }
  };
  // buffers of this thread's pass over the nets (further below)
  std::vector<double> wl(U, 0.0), inc(C, 0.0), pin_weight_sum(U, 0.0);
  std::vector<uint32_t> unit_seen(U, ~0u), cell_seen(C, ~0u);
  // Large hypergraphs are validated and laid out on a second thread while
  // this one builds the density side; small problems are not worth a thread.
  // The guards join the threads on every way out of this function, an early
  // error return included. Every sum keeps its order, so the threading
  // changes no value.
  struct Joiner {
    std::thread t;
    ~Joiner() {
      if (t.joinable()) t.join();
    }
  } layout_thread, smooth_thread;
  const bool threaded = E && p->net_ptr && p->pin_cell && p->net_ptr[E] >= 65536;
  std::promise<void> hyper_checked;
  std::future<void> hyper_ready = hyper_checked.get_future();
  auto check_and_layout = [&]() {
    hyper_status = hyper_check();
    pins = (E && !hyper_status) ? p->net_ptr[E] : 0;
    hyper_checked.set_value();
    if (!hyper_status) layout();
  };
  if (threaded) {
    layout_thread.t = std::thread(check_and_layout);
  } else {
    hyper_status = hyper_check();
    pins = (E && !hyper_status) ? p->net_ptr[E] : 0;
  }
  // capacity minus fixed occupancy (electrostatic_placement.rs:146-172)
  std::vector<std::vector<uint32_t>> caps(p->num_fields);
  for (uint32_t f = 0; f < p->num_fields; ++f)
    caps[f].assign(p->capacity + (size_t)f * tiles, p->capacity + (size_t)(f + 1) * tiles);
  for (uint32_t i = 0; i < p->num_fixed_occupancy; ++i) {
    const uint32_t f = p->fixed_occupancy[3 * (size_t)i], x = p->fixed_occupancy[3 * (size_t)i + 1],
                   y = p->fixed_occupancy[3 * (size_t)i + 2];
    if (x >= m.W || y >= m.H) {
      *err = i;
      return TEXO_GP_ERR_POINT_OUTSIDE_GRID;
    }
    if (f >= p->num_fields || caps[f][(size_t)y * m.W + x] == 0) {
      *err = i;
      return TEXO_GP_ERR_FIXED_CAPACITY_EXHAUSTED;
    }
    caps[f][(size_t)y * m.W + x] -= 1;
  }
  std::vector<int> active(p->num_fields, -1);
  for (uint32_t f = 0; f < p->num_fields; ++f) {
    if (member_count[f] == 0) continue;
    active[f] = (int)m.K++;
    m.kinds.push_back(p->fields[f]);
    m.cap.push_back(caps[f]);
  }
  if (m.K > (uint32_t)kMaxFields) return TEXO_GP_ERR_UNSUPPORTED;
  m.available.assign(m.K, 0);
  m.smoothed.assign(m.K, std::vector<double>());
  for (uint32_t f = 0; f < m.K; ++f)
    for (auto c : m.cap[f]) m.available[f] += c;
  // the smoothed capacity (a third thread on large problems; nothing below
  // reads it)
  auto smooth = [&]() {
    for (uint32_t f = 0; f < m.K; ++f) {
      m.smoothed[f].assign((size_t)m.Wb * m.Hb, 0.0);
      for (size_t i = 0; i < tiles; ++i) {
        const uint32_t c = m.cap[f][i];
        if (!c) continue;
        double bx = (double)(uint32_t)(i % m.W), by = (double)(uint32_t)(i / m.W);
        if (!m.identity) {
          bx = (bx + 0.5) * m.sx - 0.5;
          by = (by + 0.5) * m.sy - 0.5;
        }
        deposit64(m.smoothed[f], m.Wb, m.Hb, bx, by, m.td * (double)c);
      }
    }
  };
  if (threaded)
    smooth_thread.t = std::thread(smooth);
  else
    smooth();
  // density units and members (eplace.rs:261-301)
  m.U = U;
  m.unit_mem_ptr.assign(U + 1, 0);
  m.mem_unit.reserve(M);
  m.mem_field.reserve(M);
  m.mem_off.reserve(2 * (size_t)M);
  m.mem_q.reserve(M);
  m.real_count.assign(m.K, 0);
  m.real_area.assign(m.K, 0.0);
  uint32_t dunit = 0;
  for (uint32_t u = 0; u < U; ++u) {
    const uint32_t b = p->member_ptr[u], e = p->member_ptr[u + 1];
    for (uint32_t i = b; i < e; ++i) {
      const double dx = p->member_offset_xy[2 * (size_t)i], dy = p->member_offset_xy[2 * (size_t)i + 1];
      const double q = p->member_charge[i];
      if (!std::isfinite(dx) || !std::isfinite(dy)) {
        *err = dunit;
        return TEXO_GP_ERR_NONFINITE_UNIT_COORDINATE;
      }
      if (!std::isfinite(q) || q <= 0.0) {
        *err = dunit;
        return TEXO_GP_ERR_INVALID_MEMBER_CHARGE;
      }
      const int f = active[p->member_field[i]];
      m.mem_unit.push_back((int)u);
      m.mem_field.push_back(f);
      m.mem_off.push_back(dx);
      m.mem_off.push_back(dy);
      m.mem_q.push_back((float)q);
      m.real_count[f] += 1;
      m.real_area[f] += q;
    }
    if (e > b) ++dunit;
    m.unit_mem_ptr[u + 1] = (int)m.mem_unit.size();
  }
  m.Mm = (uint32_t)m.mem_unit.size();
  m.has_density = m.Mm > 0;
  // fillers (electrostatic_placement.rs:198-240)
  std::vector<double> fx, fy;
  fx.reserve(tiles * m.K);
  fy.reserve(tiles * m.K);
  m.fil_field.reserve(tiles * m.K);
  m.fil_q.reserve(tiles * m.K);
  std::vector<size_t> occ;
  occ.reserve(tiles);
  for (uint32_t f = 0; f < m.K; ++f) {
    if (m.real_count[f] > m.available[f]) {
      *err = f;
      return TEXO_GP_ERR_INSUFFICIENT_CAPACITY;
    }
    const double avail = m.td * (double)(uint32_t)m.available[f];
    const double ra = m.real_area[f];
    if (!std::isfinite(ra) || ra < 0.0 || (m.td == 1.0 && ra > avail + 1.0e-9)) {
      *err = f;
      return TEXO_GP_ERR_INSUFFICIENT_AREA;
    }
    double total = avail - ra;
    if (m.td != 1.0) total = std::max(total, 0.0);
    if (total == 0.0) continue;
    const double denominator = (double)(uint32_t)m.available[f];
    occ.clear();
    for (size_t i = 0; i < tiles; ++i)
      if (m.cap[f][i]) occ.push_back(i);
    double assigned = 0.0;
    for (size_t o = 0; o < occ.size(); ++o) {
      const size_t i = occ[o];
      const double q = o + 1 == occ.size() ? total - assigned : total * (double)m.cap[f][i] / denominator;
      assigned += q;
      m.fil_field.push_back((int)f);
      m.fil_q.push_back(q);
      fx.push_back((double)(uint32_t)(i % m.W));
      fy.push_back((double)(uint32_t)(i / m.W));
    }
  }
  m.F = (uint32_t)m.fil_field.size();
  const size_t nobj = (size_t)m.U + m.F;
  if (nobj >= (1ull << 30)) return TEXO_GP_ERR_GRID_TOO_LARGE;
  // fixed-point range: every bin's charge stays far inside int64 at 2^32
  for (uint32_t f = 0; f < m.K; ++f) {
    double tot = m.real_area[f] + m.td * (double)m.available[f];
    if (tot * 16.0 > 2147483648.0) return TEXO_GP_ERR_FIXED_POINT_RANGE;
  }
  // coordinates and bounds (eplace.rs:1441-1468, 316-318)
  m.init.resize(2 * nobj);
  m.lo.resize(2 * nobj);
  m.hi.resize(2 * nobj);
  for (uint32_t u = 0; u < U; ++u)
    for (int a = 0; a < 2; ++a) {
      const size_t i = 2 * (size_t)u + a;
      m.init[i] = p->initial_xy[i];
      m.lo[i] = p->lower_xy[i];
      m.hi[i] = p->upper_xy[i];
      if (!std::isfinite(m.lo[i]) || !std::isfinite(m.hi[i]) || m.lo[i] > m.hi[i]) return TEXO_GP_ERR_INVALID_BOUNDS;
      if (!std::isfinite(m.init[i])) {
        *err = i;
        return (p->member_ptr[u + 1] > p->member_ptr[u]) ? TEXO_GP_ERR_NONFINITE_UNIT_COORDINATE
                                                           : TEXO_GP_ERR_INVALID_INITIAL_COORDINATE;
      }
    }
  for (uint32_t j = 0; j < m.F; ++j) {
    const size_t i = 2 * ((size_t)U + j);
    m.init[i] = fx[j];
    m.init[i + 1] = fy[j];
    m.lo[i] = 0.0;
    m.lo[i + 1] = 0.0;
    m.hi[i] = (double)(m.W - 1);
    m.hi[i + 1] = (double)(m.H - 1);
  }
  for (size_t i = 0; i < 2 * nobj; ++i) m.init[i] = clampd(m.init[i], m.lo[i], m.hi[i]);
  // hypergraph (validated and laid out beside): report its errors here, in
  // the reference's order
  if (threaded) hyper_ready.wait();
  if (hyper_status) {
    *err = hyper_err;
    return hyper_status;
  }

  // wirelength preconditioner and cell incidence (this thread): each
  // distinct unit (cell) of a net counts once, found with a per-net stamp
  // instead of a sort
  for (uint32_t e = 0; e < E; ++e) {
    const uint32_t b = p->net_ptr[e], en = p->net_ptr[e + 1];
    const double w = 1.0 / (double)(uint32_t)(en - b - 1);
    uint32_t distinct = 0;
    for (uint32_t k = b; k < en; ++k) {
      const uint32_t u = p->cell_unit[p->pin_cell[k]];
      if (unit_seen[u] != e) {
        unit_seen[u] = e;
        ++distinct;
      }
    }
    if (distinct >= 2)
      for (uint32_t k = b; k < en; ++k) {
        const uint32_t u = p->cell_unit[p->pin_cell[k]];
        if (unit_seen[u] == e) {
          unit_seen[u] = ~0u - 1;   // counted for this net
          wl[u] += w;
        }
      }
    for (uint32_t k = b; k < en; ++k) {
      const uint32_t c = p->pin_cell[k];
      if (cell_seen[c] != e) {
        cell_seen[c] = e;
        inc[c] += w;
      }
    }
  }
  for (uint32_t a = 0; a < arcs; ++a) {
    const uint32_t du = p->cell_unit[p->arc_driver_cell[a]], su = p->cell_unit[p->arc_sink_cell[a]];
    const double w = u64_to_f64(p->arc_extra_weight[a]);
    if (du != su) {
      wl[du] += w;
      wl[su] += w;
    }
    pin_weight_sum[du] += w;
    pin_weight_sum[su] += w;
  }
  if (threaded) {
    layout_thread.t.join();
    smooth_thread.t.join();
  } else {
    layout();
  }
  if (!layout_ok) return TEXO_GP_ERR_INVALID_ARGUMENT;
  for (uint32_t u = 0; u < U; ++u) pin_weight_sum[u] += pin_count[u];
  m.n_classes = kNetClasses + 1;
  m.class_begin[kNetClasses + 1] = (int)m.net_w.size();
  if (m.pin_unit.size() >= (1ull << 31)) return TEXO_GP_ERR_GRID_TOO_LARGE;
  // WA fixed point: |derivative| <= 3 per pin, summed per unit, at 2^32 per unit
  for (uint32_t u = 0; u < U; ++u)
    if (pin_weight_sum[u] * 4.0 > 1073741824.0) return TEXO_GP_ERR_FIXED_POINT_RANGE;
  // static preconditioner and per-field charges per optimizer object
  m.pre_static.assign(nobj, 0.0);
  for (uint32_t u = 0; u < U; ++u) m.pre_static[u] = wl[u];
  m.pre_q.assign((size_t)m.K * nobj, 0.0);
  for (uint32_t u = 0; u < U; ++u)
    for (int i = m.unit_mem_ptr[u]; i < m.unit_mem_ptr[u + 1]; ++i)
      m.pre_q[(size_t)m.mem_field[i] * nobj + u] += (double)p->member_charge[p->member_ptr[u] + (i - m.unit_mem_ptr[u])];
  for (uint32_t j = 0; j < m.F; ++j) m.pre_q[(size_t)m.fil_field[j] * nobj + U + j] = m.fil_q[j];
  // gamma weights (eplace.rs:1424-1439)
  m.gamma_weight.assign(m.K, 0.0);
  if (p->member_cell)
    for (uint32_t i = 0; i < M; ++i) m.gamma_weight[active[p->member_field[i]]] += inc[p->member_cell[i]];
  return TEXO_GP_OK;
}

}  // namespace tgp
