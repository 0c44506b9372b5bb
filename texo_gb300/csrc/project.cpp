// project.cpp — `project` up to its repair (crates/texo-pnr/src/
// legalization/mod.rs:322-389) behind one C-ABI call.
//
// Host code around this library's GPU auction (texo_gp_auction_singletons):
// fixed units take their BELs (`install_fixed_units`, :391-430); units with
// Shared choice tables form families, a family whose rows are pairwise
// BEL-disjoint is auctioned and the others' units are seeded one at a time on
// the nearest free row (`classify_units`, :432-471; `seed_overlapping_units`
// and `nearest_direct_choice`, :473-575); the disjoint families are auctioned
// scarcest first, each over its free rows at the Manhattan distance of the
// row's first BEL (`auction_disjoint_families`, :577-655); the SingleCell
// units share one auction whose objects are the BELs of each distinct
// candidate table (`auction_singletons`, :657-677). Occupancy is the only
// legality rule; units left unmatched keep -1 (the reference's transactional
// repair places them).
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <map>
#include <numeric>
#include <string>
#include <vector>

#include "texo_gp.h"

namespace tgp {
void set_last_error(const std::string& s);
}

namespace {

struct Ctx {
  uint32_t W, H;
  const uint32_t* bel_xy;
  const texo_gp_choice_table* tables;
  std::vector<uint8_t> occupied;
};

const uint32_t* row(const texo_gp_choice_table& t, uint32_t c) { return t.bels + (size_t)c * t.width; }

bool row_free(const Ctx& x, const texo_gp_choice_table& t, uint32_t c) {
  const uint32_t* r = row(t, c);
  for (uint32_t i = 0; i < t.width; ++i)
    if (x.occupied[r[i]]) return false;
  return true;
}

void take_row(Ctx& x, const texo_gp_choice_table& t, uint32_t c) {
  const uint32_t* r = row(t, c);
  for (uint32_t i = 0; i < t.width; ++i) x.occupied[r[i]] = 1;
}

// SpatialChoiceIndex (lib.rs:3774-3787): choice indices by the tile of the
// choice's first BEL, ascending within a tile (CSR over tiles)
void by_point(const Ctx& x, const texo_gp_choice_table& t, std::vector<uint32_t>& ptr, std::vector<uint32_t>& idx) {
  const size_t tiles = (size_t)x.W * x.H;
  ptr.assign(tiles + 1, 0);
  for (uint32_t c = 0; c < t.num_choices; ++c) {
    const uint32_t b = row(t, c)[0];
    ++ptr[(size_t)x.bel_xy[2 * b + 1] * x.W + x.bel_xy[2 * b] + 1];
  }
  for (size_t i = 0; i < tiles; ++i) ptr[i + 1] += ptr[i];
  idx.assign(t.num_choices, 0);
  std::vector<uint32_t> at(ptr.begin(), ptr.end() - 1);
  for (uint32_t c = 0; c < t.num_choices; ++c) {
    const uint32_t b = row(t, c)[0];
    idx[at[(size_t)x.bel_xy[2 * b + 1] * x.W + x.bel_xy[2 * b]]++] = c;
  }
}

// ring_coordinates (lib.rs:6814-6821)
int ring(uint32_t center, uint32_t offset, uint32_t extent, uint32_t out[2]) {
  int n = 0;
  if (center >= offset && center - offset < extent) out[n++] = center - offset;
  if (offset != 0 && (uint64_t)center + offset < extent) out[n++] = center + offset;
  return n;
}

// nearest_direct_choice (mod.rs:533-575): the least (point, choice) whose row
// is free, on the first ring around the target that has one; -1 when none.
int64_t nearest(const Ctx& x, const texo_gp_choice_table& t, const std::vector<uint32_t>& ptr,
                const std::vector<uint32_t>& idx, uint32_t tx, uint32_t ty) {
  const uint32_t max_r = (x.W - 1) + (x.H - 1);
  for (uint32_t r = 0; r <= max_r; ++r) {
    bool found = false;
    uint32_t bx = 0, by = 0, bc = 0;
    for (uint32_t dy = 0; dy <= r; ++dy) {
      uint32_t ys[2], xs[2];
      const int ny = ring(ty, dy, x.H, ys), nx = ring(tx, r - dy, x.W, xs);
      for (int a = 0; a < ny; ++a)
        for (int b = 0; b < nx; ++b) {
          const size_t tile = (size_t)ys[a] * x.W + xs[b];
          for (uint32_t k = ptr[tile]; k < ptr[tile + 1]; ++k) {
            const uint32_t c = idx[k];
            if (!row_free(x, t, c)) continue;
            // Point orders by (x, y), then the choice index
            if (!found || std::make_tuple(xs[b], ys[a], c) < std::make_tuple(bx, by, bc)) {
              found = true;
              bx = xs[b];
              by = ys[a];
              bc = c;
            }
          }
        }
    }
    if (found) return bc;
  }
  return -1;
}

int32_t fail(const std::string& why, int32_t code) {
  tgp::set_last_error(why);
  return code;
}

}  // namespace

extern "C" int32_t texo_gp_project(int32_t device, uint32_t width, uint32_t height, uint32_t num_bels,
                                   const uint32_t* bel_xy, uint32_t num_tables, const texo_gp_choice_table* tables,
                                   uint32_t num_units, const uint32_t* unit_table, const uint32_t* unit_first_cell,
                                   const uint32_t* target_xy, uint32_t cost_scale, int32_t* out_choice,
                                   texo_gp_projection_stats* stats) {
  if (stats) std::memset(stats, 0, sizeof(*stats));
  if (num_units == 0) return TEXO_GP_OK;
  if (width == 0 || height == 0 || !bel_xy || !tables || !unit_table || !unit_first_cell || !target_xy ||
      !out_choice)
    return fail("texo_gp_project: empty grid or null argument", TEXO_GP_ERR_INVALID_ARGUMENT);
  for (uint32_t b = 0; b < num_bels; ++b)
    if (bel_xy[2 * b] >= width || bel_xy[2 * b + 1] >= height)
      return fail("texo_gp_project: BEL " + std::to_string(b) + " outside the grid", TEXO_GP_ERR_INVALID_ARGUMENT);
  for (uint32_t t = 0; t < num_tables; ++t) {
    const texo_gp_choice_table& tb = tables[t];
    if (tb.num_choices == 0 || tb.width == 0 || !tb.bels || (!tb.shared && tb.width != 1))
      return fail("texo_gp_project: malformed choice table " + std::to_string(t), TEXO_GP_ERR_INVALID_ARGUMENT);
    for (size_t k = 0; k < (size_t)tb.num_choices * tb.width; ++k)
      if (tb.bels[k] >= num_bels)
        return fail("texo_gp_project: table " + std::to_string(t) + " names a BEL out of range",
                    TEXO_GP_ERR_INVALID_ARGUMENT);
  }
  for (uint32_t u = 0; u < num_units; ++u)
    if (unit_table[u] >= num_tables || target_xy[2 * u] >= width || target_xy[2 * u + 1] >= height)
      return fail("texo_gp_project: unit " + std::to_string(u) + " table or target out of range",
                  TEXO_GP_ERR_INVALID_ARGUMENT);
  Ctx x{width, height, bel_xy, tables, std::vector<uint8_t>(num_bels, 0)};
  texo_gp_projection_stats s;
  std::memset(&s, 0, sizeof(s));
  std::fill(out_choice, out_choice + num_units, -1);
  // 1. fixed units
  for (uint32_t u = 0; u < num_units; ++u) {
    const texo_gp_choice_table& t = tables[unit_table[u]];
    if (t.num_choices != 1) continue;
    if (!row_free(x, t, 0))
      return fail("fixed analytical placement assignments conflict", TEXO_GP_ERR_PROJECTION_CONFLICT);
    take_row(x, t, 0);
    out_choice[u] = 0;
    s.fixed_units++;
  }
  // 2. classification: families by table, units by first cell
  std::map<uint32_t, std::vector<uint32_t>> families;
  std::vector<uint32_t> singletons;
  for (uint32_t u = 0; u < num_units; ++u) {
    const texo_gp_choice_table& t = tables[unit_table[u]];
    if (t.num_choices == 1) continue;
    if (t.shared)
      families[unit_table[u]].push_back(u);
    else
      singletons.push_back(u);
  }
  auto by_cell = [&](uint32_t a, uint32_t b) { return unit_first_cell[a] < unit_first_cell[b]; };
  std::vector<uint32_t> overlapping;
  std::vector<std::pair<uint32_t, std::vector<uint32_t>>> disjoint;
  for (auto& kv : families) {
    std::sort(kv.second.begin(), kv.second.end(), by_cell);
    const texo_gp_choice_table& t = tables[kv.first];
    std::vector<uint8_t> seen(num_bels, 0);
    bool disjoint_rows = true;
    for (size_t k = 0; k < (size_t)t.num_choices * t.width && disjoint_rows; ++k) {
      if (seen[t.bels[k]]) disjoint_rows = false;
      seen[t.bels[k]] = 1;
    }
    if (disjoint_rows) {
      s.disjoint_shared_families++;
      s.disjoint_shared_units += kv.second.size();
      disjoint.emplace_back(kv.first, kv.second);
    } else {
      s.overlapping_shared_families++;
      s.overlapping_shared_units += kv.second.size();
      overlapping.insert(overlapping.end(), kv.second.begin(), kv.second.end());
    }
  }
  std::sort(singletons.begin(), singletons.end(), by_cell);
  s.singleton_units = singletons.size();
  // 3. overlapping families, one unit at a time
  std::sort(overlapping.begin(), overlapping.end(), [&](uint32_t a, uint32_t b) {
    const texo_gp_choice_table &ta = tables[unit_table[a]], &tb = tables[unit_table[b]];
    if (ta.num_choices != tb.num_choices) return ta.num_choices < tb.num_choices;
    if (ta.width != tb.width) return ta.width > tb.width;
    return unit_first_cell[a] < unit_first_cell[b];
  });
  std::map<uint32_t, std::pair<std::vector<uint32_t>, std::vector<uint32_t>>> spatial;
  for (uint32_t u : overlapping) {
    const uint32_t ti = unit_table[u];
    const texo_gp_choice_table& t = tables[ti];
    auto it = spatial.find(ti);
    if (it == spatial.end()) {
      it = spatial.emplace(ti, std::make_pair(std::vector<uint32_t>(), std::vector<uint32_t>())).first;
      by_point(x, t, it->second.first, it->second.second);
    }
    const int64_t c = nearest(x, t, it->second.first, it->second.second, target_xy[2 * u], target_xy[2 * u + 1]);
    if (c < 0) continue;
    out_choice[u] = (int32_t)c;
    take_row(x, t, (uint32_t)c);
  }
  // one auction over objects grouped by (kind, tile); record the winners
  auto run_auction = [&](const std::vector<std::vector<uint32_t>>& kind_ptr,
                         const std::vector<std::vector<uint32_t>>& kind_obj, uint32_t num_objects,
                         const std::vector<uint8_t>& occ, const std::vector<uint32_t>& bidders,
                         const std::vector<uint32_t>& bidder_kind, std::vector<int32_t>& assignment) -> int32_t {
    const size_t tiles = (size_t)width * height;
    const uint32_t K = (uint32_t)kind_ptr.size();
    std::vector<uint32_t> tp(K * tiles + 1, 0), to;
    for (uint32_t q = 0; q < K; ++q) {
      for (size_t t = 0; t < tiles; ++t) tp[q * tiles + t + 1] = (uint32_t)(to.size() + kind_ptr[q][t + 1]);
      to.insert(to.end(), kind_obj[q].begin(), kind_obj[q].end());
    }
    std::vector<uint32_t> txy(2 * bidders.size());
    for (size_t i = 0; i < bidders.size(); ++i) {
      txy[2 * i] = target_xy[2 * bidders[i]];
      txy[2 * i + 1] = target_xy[2 * bidders[i] + 1];
    }
    assignment.assign(bidders.size(), -1);
    texo_gp_auction_stats ast;
    const uint32_t zero = 0;
    const int32_t st = texo_gp_auction_singletons(device, width, height, K, tp.data(), to.empty() ? &zero : to.data(),
                                                  num_objects, occ.data(), (uint32_t)bidders.size(),
                                                  bidder_kind.data(), txy.data(), cost_scale, assignment.data(),
                                                  nullptr, &ast);
    s.bids += ast.bids;
    s.candidates_examined += ast.candidates_examined;
    s.elapsed_ms += ast.elapsed_ms;
    s.auctions++;
    return st;
  };
  // 4. disjoint families, scarcest first
  std::stable_sort(disjoint.begin(), disjoint.end(), [&](const auto& a, const auto& b) {
    const texo_gp_choice_table &ta = tables[a.first], &tb = tables[b.first];
    const unsigned __int128 la = (unsigned __int128)ta.num_choices * b.second.size();
    const unsigned __int128 lb = (unsigned __int128)tb.num_choices * a.second.size();
    if (la != lb) return la < lb;
    if (ta.width != tb.width) return ta.width > tb.width;
    return unit_first_cell[a.second[0]] < unit_first_cell[b.second[0]];
  });
  for (const auto& fam : disjoint) {
    const texo_gp_choice_table& t = tables[fam.first];
    std::vector<std::vector<uint32_t>> ptr(1), obj(1);
    by_point(x, t, ptr[0], obj[0]);
    std::vector<uint8_t> occ(t.num_choices);
    for (uint32_t c = 0; c < t.num_choices; ++c) occ[c] = row_free(x, t, c) ? 0 : 1;
    std::vector<uint32_t> kinds(fam.second.size(), 0);
    std::vector<int32_t> a;
    const int32_t st = run_auction(ptr, obj, t.num_choices, occ, fam.second, kinds, a);
    if (st) return st;
    for (size_t i = 0; i < fam.second.size(); ++i) {
      if (a[i] < 0) {
        s.relaxed_unmatched_units++;
        continue;
      }
      if (!row_free(x, t, (uint32_t)a[i]))
        return fail("capacity auction returned an occupied assignment", TEXO_GP_ERR_PROJECTION_CONFLICT);
      out_choice[fam.second[i]] = a[i];
      take_row(x, t, (uint32_t)a[i]);
    }
  }
  // 5. singletons: a kind per distinct candidate table
  if (!singletons.empty()) {
    std::map<uint32_t, uint32_t> kind_of;
    std::vector<uint32_t> kind_table;
    for (uint32_t u : singletons)
      if (kind_of.emplace(unit_table[u], (uint32_t)kind_table.size()).second) kind_table.push_back(unit_table[u]);
    // kinds numbered by first appearance in first-cell order
    std::vector<std::vector<uint32_t>> ptr(kind_table.size()), obj(kind_table.size());
    for (size_t q = 0; q < kind_table.size(); ++q) {
      const texo_gp_choice_table& t = tables[kind_table[q]];
      std::vector<uint32_t> idx;
      by_point(x, t, ptr[q], idx);
      obj[q].resize(idx.size());
      for (size_t k = 0; k < idx.size(); ++k) obj[q][k] = row(t, idx[k])[0];
      // ascending BEL ids within a tile
      for (size_t tl = 0; tl + 1 < ptr[q].size(); ++tl) std::sort(obj[q].begin() + ptr[q][tl], obj[q].begin() + ptr[q][tl + 1]);
    }
    std::vector<uint32_t> kinds(singletons.size());
    for (size_t i = 0; i < singletons.size(); ++i) kinds[i] = kind_of[unit_table[singletons[i]]];
    std::vector<int32_t> a;
    const int32_t st = run_auction(ptr, obj, num_bels, x.occupied, singletons, kinds, a);
    if (st) return st;
    std::map<uint32_t, std::map<uint32_t, uint32_t>> pos;   // table -> BEL -> choice
    for (size_t i = 0; i < singletons.size(); ++i) {
      const uint32_t u = singletons[i];
      if (a[i] < 0) {
        s.relaxed_unmatched_units++;
        continue;
      }
      const uint32_t ti = unit_table[u];
      auto& m = pos[ti];
      if (m.empty())
        for (uint32_t c = 0; c < tables[ti].num_choices; ++c) m.emplace(row(tables[ti], c)[0], c);
      auto it = m.find((uint32_t)a[i]);
      if (it == m.end()) return fail("auction returned a noncandidate BEL", TEXO_GP_ERR_PROJECTION_CONFLICT);
      if (x.occupied[(uint32_t)a[i]])
        return fail("capacity auction returned an occupied assignment", TEXO_GP_ERR_PROJECTION_CONFLICT);
      out_choice[u] = (int32_t)it->second;
      x.occupied[(uint32_t)a[i]] = 1;
    }
  }
  if (stats) *stats = s;
  return TEXO_GP_OK;
}
