// synth.cpp — seeded generator of ECP5-like placement problems.
//
// Movable unit-area LUT cells on a side x side site fabric with one LUT BEL
// per site; fixed IO cells evenly spaced on the perimeter; nets in three
// degree bands (60% 2-pin, 30% 3-5 pins, 10% 6-32 pins) with a uniform driver
// and sinks drawn, with probability p_local, near the driver's index-grid
// position (Gaussian radius sigma), otherwise uniformly; duplicate sinks are
// rejected. Initial positions: fabric centre plus N(0, jitter^2).
//
// The random source is xoshiro256** seeded through splitmix64; normal draws
// are Irwin-Hall sums of twelve uniforms, so the generator uses integer and
// basic IEEE arithmetic only and yields identical problems on every host.
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "../../include/texo_gp.h"

namespace {

struct Rng {
  uint64_t s[4];
  explicit Rng(uint64_t seed) {
    uint64_t x = seed;
    for (auto& v : s) {
      x += 0x9e3779b97f4a7c15ull;
      uint64_t z = x;
      z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
      z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
      v = z ^ (z >> 31);
    }
  }
  static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  uint64_t next() {
    const uint64_t r = rotl(s[1] * 5, 7) * 9;
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return r;
  }
  double uniform() { return (double)(next() >> 11) * 0x1p-53; }
  uint32_t below(uint32_t n) { return (uint32_t)(((__uint128_t)next() * n) >> 64); }
  double normal() {
    double acc = 0.0;
    for (int i = 0; i < 12; ++i) acc += uniform();
    return acc - 6.0;
  }
};

}  // namespace

struct texo_gp_synth_s {
  texo_gp_problem p{};
  texo_gp_field field{TEXO_GP_KIND_LUT, 4};
  std::vector<uint32_t> capacity, member_ptr, member_field, member_cell, cell_unit, net_ptr, pin_cell;
  std::vector<double> initial, lower, upper, member_off, member_charge, cell_off, cell_fxy;
  std::vector<uint8_t> cell_fixed;
};

extern "C" int32_t texo_gp_synth_create(const texo_gp_synth_spec* spec, texo_gp_synth* out,
                                        const texo_gp_problem** problem) {
  if (!spec || !out || spec->side < 2 || spec->cells == 0 ||
      (uint64_t)spec->cells > (uint64_t)spec->side * spec->side || spec->io > 64u * (spec->side - 1) ||
      !(spec->sigma > 0.0) || !(spec->p_local >= 0.0 && spec->p_local <= 1.0) || !(spec->jitter >= 0.0))
    return TEXO_GP_ERR_INVALID_ARGUMENT;
  auto s = std::make_unique<texo_gp_synth_s>();
  const uint32_t S = spec->side, N = spec->cells, IO = spec->io, C = N + IO, E = spec->nets;
  Rng rng(spec->seed);
  s->capacity.assign((size_t)S * S, 1u);
  const double centre = 0.5 * (double)(S - 1), maxc = (double)(S - 1);
  s->initial.resize(2 * (size_t)C);
  s->lower.resize(2 * (size_t)C);
  s->upper.resize(2 * (size_t)C);
  s->member_ptr.assign(C + 1, 0);
  s->cell_unit.resize(C);
  s->cell_off.assign(2 * (size_t)C, 0.0);
  s->cell_fixed.assign(C, 0);
  s->cell_fxy.assign(2 * (size_t)C, 0.0);
  for (uint32_t i = 0; i < N; ++i) {
    double x = centre + spec->jitter * rng.normal();
    double y = centre + spec->jitter * rng.normal();
    x = x < 0.0 ? 0.0 : (x > maxc ? maxc : x);
    y = y < 0.0 ? 0.0 : (y > maxc ? maxc : y);
    s->initial[2 * (size_t)i] = x;
    s->initial[2 * (size_t)i + 1] = y;
    s->lower[2 * (size_t)i] = 0.0;
    s->lower[2 * (size_t)i + 1] = 0.0;
    s->upper[2 * (size_t)i] = maxc;
    s->upper[2 * (size_t)i + 1] = maxc;
    s->member_field.push_back(0);
    s->member_off.push_back(0.0);
    s->member_off.push_back(0.0);
    s->member_charge.push_back(1.0);
    s->member_cell.push_back(i);
    s->member_ptr[i + 1] = (uint32_t)s->member_field.size();
    s->cell_unit[i] = i;
  }
  // IO evenly spaced along the perimeter walk (x grows on y=0, then up x=S-1, ...);
  // with more IO cells than perimeter sites, neighbours share a site
  const uint64_t perim = 4ull * (S - 1);
  for (uint32_t k = 0; k < IO; ++k) {
    const uint64_t t = (uint64_t)k * perim / (IO ? IO : 1);
    uint32_t px, py;
    if (t < S - 1) {
      px = (uint32_t)t;
      py = 0;
    } else if (t < 2ull * (S - 1)) {
      px = S - 1;
      py = (uint32_t)(t - (S - 1));
    } else if (t < 3ull * (S - 1)) {
      px = (uint32_t)(S - 1 - (t - 2ull * (S - 1)));
      py = S - 1;
    } else {
      px = 0;
      py = (uint32_t)(S - 1 - (t - 3ull * (S - 1)));
    }
    const uint32_t i = N + k;
    s->initial[2 * (size_t)i] = px;
    s->initial[2 * (size_t)i + 1] = py;
    s->lower[2 * (size_t)i] = px;
    s->lower[2 * (size_t)i + 1] = py;
    s->upper[2 * (size_t)i] = px;
    s->upper[2 * (size_t)i + 1] = py;
    s->member_ptr[i + 1] = (uint32_t)s->member_field.size();
    s->cell_unit[i] = i;
    s->cell_fixed[i] = 1;
    s->cell_fxy[2 * (size_t)i] = px;
    s->cell_fxy[2 * (size_t)i + 1] = py;
  }
  // nets
  s->net_ptr.assign(1, 0);
  std::vector<uint32_t> pins;
  for (uint32_t e = 0; e < E; ++e) {
    const double band = rng.uniform();
    uint32_t deg = band < 0.6 ? 2 : (band < 0.9 ? 3 + rng.below(3) : 6 + rng.below(27));
    if (deg > C) deg = C;
    pins.clear();
    const uint32_t driver = rng.below(C);
    pins.push_back(driver);
    const int64_t gx = driver % S, gy = driver / S;
    uint32_t guard = 0;
    while (pins.size() < deg && guard < 64u * deg) {
      ++guard;
      uint32_t cand;
      if (rng.uniform() < spec->p_local) {
        const int64_t x = gx + (int64_t)std::llround(spec->sigma * rng.normal());
        const int64_t y = gy + (int64_t)std::llround(spec->sigma * rng.normal());
        if (x < 0 || y < 0 || x >= (int64_t)S || y >= (int64_t)S) continue;
        const int64_t idx = y * S + x;
        if (idx >= (int64_t)C) continue;
        cand = (uint32_t)idx;
      } else {
        cand = rng.below(C);
      }
      bool dup = false;
      for (uint32_t q : pins) dup |= q == cand;
      if (!dup) pins.push_back(cand);
    }
    if (pins.size() < 2) continue;
    s->pin_cell.insert(s->pin_cell.end(), pins.begin(), pins.end());
    s->net_ptr.push_back((uint32_t)s->pin_cell.size());
  }
  texo_gp_problem& p = s->p;
  std::memset(&p, 0, sizeof(p));
  p.width = S;
  p.height = S;
  p.num_fields = 1;
  p.fields = &s->field;
  p.capacity = s->capacity.data();
  p.num_units = C;
  p.initial_xy = s->initial.data();
  p.lower_xy = s->lower.data();
  p.upper_xy = s->upper.data();
  p.member_ptr = s->member_ptr.data();
  p.member_field = s->member_field.data();
  p.member_offset_xy = s->member_off.data();
  p.member_charge = s->member_charge.data();
  p.member_cell = s->member_cell.data();
  p.num_cells = C;
  p.cell_unit = s->cell_unit.data();
  p.cell_offset_xy = s->cell_off.data();
  p.cell_fixed = s->cell_fixed.data();
  p.cell_fixed_xy = s->cell_fxy.data();
  p.num_nets = (uint32_t)(s->net_ptr.size() - 1);
  p.net_ptr = s->net_ptr.data();
  p.pin_cell = s->pin_cell.data();
  if (problem) *problem = &s->p;
  *out = s.release();
  return TEXO_GP_OK;
}

extern "C" int32_t texo_gp_synth_destroy(texo_gp_synth s) {
  delete s;
  return TEXO_GP_OK;
}
