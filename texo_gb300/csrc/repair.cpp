// repair.cpp — the transactional repair of `project`
// (crates/texo-pnr/src/legalization/repair.rs, `repair_relaxed` :60-151)
// behind one C-ABI call (texo_gp_repair).
//
// Host code: the relaxed projection (texo_gp_project's choices, which may
// leave units unmatched, or the caller's own, which may conflict) becomes a
// legal placement. A search state is always a legal partial placement;
// trying an assignment evicts every unit blocking it and installs it in one
// journalled transaction. Legality: BEL occupancy, pin wires (a connected
// cell pin placed on a BEL takes the BEL pin's wire; a wire admits
// `capacity` distinct nets) and shared resources (under a rule a cell
// carries a value and a BEL belongs to a resource; a resource holds one
// value). Steps, in the reference's order:
//   initial pending units (:325-414): unmatched units, and of every relaxed
//     conflict all owners but a deterministic survivor;
//   the legal base: fixed units, then the others (:103-124);
//   direct fast path (:853-886): each unplaced unit (fewest choices, most
//     cells, first cell) takes the first installable choice of its cursor;
//   single-blocker fast path (:888-996): alternating paths in which each step
//     evicts at most one unit;
//   exact search (:998-1117): depth-first over every blocker set of every
//     choice, states memoised by their deviation from the proposal.
// Choices are visited by a cursor: the preferred choice, then Manhattan ring
// by ring around the target (x ascending, below before above, a tile's
// choices in index order; `ChoiceCursor`, :641-790). Every search keeps
// explicit frames, so long augmenting chains need no call stack.
#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstring>
#include <map>
#include <set>
#include <string>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "texo_gp.h"

namespace tgp {
void set_last_error(const std::string& s);
}

namespace {

using PinClaim = std::pair<uint32_t, uint32_t>;                     // (wire, net)
using SharedKey = std::pair<uint32_t, uint64_t>;                     // (rule, resource)
using SharedClaim = std::pair<SharedKey, uint64_t>;                  // resource, value
using Key = std::vector<std::pair<uint32_t, int64_t>>;               // deviations from the proposal
constexpr int64_t kUnplaced = -1;

struct SharedKeyHash {
  size_t operator()(const SharedKey& k) const {
    return std::hash<uint64_t>()(k.second * 0x9E3779B97F4A7C15ull ^ (uint64_t)k.first);
  }
};

struct Footprint {
  std::vector<PinClaim> pins;
  std::vector<SharedClaim> shared;
};

struct BadInput {
  std::string why;
  int32_t code;
};

// ---- the problem ------------------------------------------------------------
struct Model {
  uint32_t W = 0, H = 0, B = 0, U = 0, C = 0;
  const uint32_t* bel_xy = nullptr;
  const texo_gp_choice_table* tables = nullptr;
  const uint32_t* unit_table = nullptr;
  const uint32_t* cell_ptr = nullptr;
  const uint32_t* cells = nullptr;
  const uint32_t* target = nullptr;
  // legality, as CSR lists
  std::vector<uint32_t> wire_cap;
  std::vector<uint32_t> cp_ptr;                       // cell -> connected pins
  std::vector<std::pair<uint32_t, uint32_t>> cp;      // (key, net)
  std::vector<uint32_t> bp_ptr;                       // BEL -> pins, by key
  std::vector<std::pair<uint32_t, uint32_t>> bp;      // (key, wire)
  std::vector<uint32_t> cv_ptr;                       // cell -> (rule, value)
  std::vector<std::pair<uint32_t, uint64_t>> cv;
  std::vector<uint32_t> br_ptr;                       // BEL -> (rule, resource)
  std::vector<std::pair<uint32_t, uint64_t>> br;
  // per table: choices by the tile of their first BEL (`SpatialChoiceIndex`)
  std::vector<std::vector<uint32_t>> sp_ptr, sp_idx;

  const texo_gp_choice_table& table(uint32_t u) const { return tables[unit_table[u]]; }
  uint32_t ncells(uint32_t u) const { return cell_ptr[u + 1] - cell_ptr[u]; }
  uint32_t cell(uint32_t u, uint32_t i) const { return cells[cell_ptr[u] + i]; }
  const uint32_t* row(uint32_t u, uint32_t c) const {
    const texo_gp_choice_table& t = table(u);
    return t.bels + (size_t)c * t.width;
  }
  void spatial(uint32_t t) {
    if (!sp_ptr[t].empty()) return;
    const texo_gp_choice_table& tb = tables[t];
    std::vector<uint32_t>& ptr = sp_ptr[t];
    std::vector<uint32_t>& idx = sp_idx[t];
    ptr.assign((size_t)W * H + 1, 0);
    auto tile = [&](uint32_t c) {
      const uint32_t b = tb.bels[(size_t)c * tb.width];
      return (size_t)bel_xy[2 * b + 1] * W + bel_xy[2 * b];
    };
    for (uint32_t c = 0; c < tb.num_choices; ++c) ++ptr[tile(c) + 1];
    for (size_t i = 0; i < (size_t)W * H; ++i) ptr[i + 1] += ptr[i];
    idx.resize(tb.num_choices);
    std::vector<uint32_t> at(ptr.begin(), ptr.end() - 1);
    for (uint32_t c = 0; c < tb.num_choices; ++c) idx[at[tile(c)]++] = c;
  }

  // `assignment_footprint` (repair.rs:161-188): sorted distinct claims
  Footprint footprint(uint32_t u, uint32_t c) const {
    Footprint f;
    footprint_into(u, c, f);
    return f;
  }
  void footprint_into(uint32_t u, uint32_t c, Footprint& f) const {
    f.pins.clear();
    f.shared.clear();
    const uint32_t* r = row(u, c);
    for (uint32_t i = 0; i < ncells(u); ++i) {
      const uint32_t cl = cell(u, i), b = r[i];
      for (uint32_t k = cp_ptr[cl]; k < cp_ptr[cl + 1]; ++k) {
        const uint32_t key = cp[k].first;
        auto lo = bp.begin() + bp_ptr[b], hi = bp.begin() + bp_ptr[b + 1];
        auto it = std::lower_bound(lo, hi, std::make_pair(key, 0u),
                                   [](const std::pair<uint32_t, uint32_t>& a, const std::pair<uint32_t, uint32_t>& v) {
                                     return a.first < v.first;
                                   });
        if (it == hi || it->first != key)
          throw BadInput{"placement candidate lacks a bound physical pin (cell " + std::to_string(cl) + ", BEL " +
                             std::to_string(b) + ")",
                         TEXO_GP_ERR_INVALID_ARGUMENT};
        f.pins.emplace_back(it->second, cp[k].second);
      }
      for (uint32_t k = cv_ptr[cl]; k < cv_ptr[cl + 1]; ++k)
        for (uint32_t j = br_ptr[b]; j < br_ptr[b + 1]; ++j)
          if (br[j].first == cv[k].first) f.shared.push_back({{cv[k].first, br[j].second}, cv[k].second});
    }
    std::sort(f.pins.begin(), f.pins.end());
    f.pins.erase(std::unique(f.pins.begin(), f.pins.end()), f.pins.end());
    std::sort(f.shared.begin(), f.shared.end());
    f.shared.erase(std::unique(f.shared.begin(), f.shared.end()), f.shared.end());
  }
};

// ---- `ChoiceCursor` (repair.rs:641-790) --------------------------------------
struct Cursor {
  const uint32_t* ptr = nullptr;
  const uint32_t* idx = nullptr;
  int64_t W = 0, H = 0, tx = 0, ty = 0, pref = -1;
  bool pref_pending = false;
  int64_t r = 0, max_r = 0, x = 0, x_end = -1, xc = 0;
  int64_t ys[2] = {0, 0};
  int ny = 0, yi = 0;
  uint32_t bk = 0, bend = 0;

  Cursor() = default;
  Cursor(Model& m, uint32_t u, int64_t preferred) {
    const uint32_t t = m.unit_table[u];
    m.spatial(t);   // built on a table's first cursor: most tables never need one
    ptr = m.sp_ptr[t].data();
    idx = m.sp_idx[t].data();
    W = m.W, H = m.H;
    tx = m.target[2 * u], ty = m.target[2 * u + 1];
    pref = preferred;
    pref_pending = preferred >= 0;
    max_r = (W - 1) + (H - 1);
    begin_ring();
  }
  void begin_ring() {
    x = std::max<int64_t>(tx - r, 0);
    x_end = std::min<int64_t>(tx + r, W - 1);
    ny = yi = 0;
    bk = bend = 0;
  }
  // the next choice, or -1 past the last ring
  int64_t next() {
    if (pref_pending) {
      pref_pending = false;
      return pref;
    }
    for (;;) {
      while (bk < bend) {
        const uint32_t c = idx[bk++];
        if ((int64_t)c != pref) return c;
      }
      if (yi < ny) {
        const size_t p = (size_t)ys[yi++] * W + xc;
        bk = ptr[p];
        bend = ptr[p + 1];
        continue;
      }
      if (x <= x_end) {
        xc = x++;
        const int64_t dx = xc > tx ? xc - tx : tx - xc;
        ny = yi = 0;
        if (dx > r) continue;
        const int64_t dy = r - dx;
        if (ty >= dy && ty - dy < H) ys[ny++] = ty - dy;
        if (dy != 0 && ty + dy < H) ys[ny++] = ty + dy;
        continue;
      }
      if (r == max_r) return -1;
      ++r;
      begin_ring();
    }
  }
};

// ---- `RepairState` (repair.rs:418-590) ---------------------------------------
struct State {
  Model& m;
  const std::vector<int64_t>& preferred;
  const std::vector<uint8_t>& fixed;
  std::vector<int64_t> choice;
  std::map<uint32_t, int64_t> dev;
  std::vector<int32_t> placed, bel_owner;
  std::unordered_map<uint32_t, std::map<uint32_t, std::set<uint32_t>>> pin_owner;
  std::unordered_map<SharedKey, std::map<uint64_t, std::set<uint32_t>>, SharedKeyHash> shared_owner;
  struct Entry {
    bool installed;
    uint32_t unit;
    int64_t choice;
  };
  std::vector<Entry> journal;
  std::unordered_map<uint64_t, Footprint> fps;
  // unplaced units ordered as `next_unplaced` picks them
  struct Order {
    const Model* m;
    bool operator()(uint32_t a, uint32_t b) const {
      const uint32_t ca = m->table(a).num_choices, cb = m->table(b).num_choices;
      if (ca != cb) return ca < cb;
      const uint32_t na = m->ncells(a), nb = m->ncells(b);
      if (na != nb) return na > nb;
      const uint32_t fa = m->cell(a, 0), fb = m->cell(b, 0);
      if (fa != fb) return fa < fb;
      return a < b;
    }
  };
  std::set<uint32_t, Order> unplaced;

  bool legality = false;   // any pin or shared claims at all
  const Footprint none{};

  State(Model& mm, const std::vector<int64_t>& pref, const std::vector<uint8_t>& fx)
      : m(mm), preferred(pref), fixed(fx), unplaced(Order{&mm}) {
    choice.assign(m.U, -1);
    placed.assign(m.C, -1);
    bel_owner.assign(m.B, -1);
    legality = !m.cp.empty() || !m.cv.empty();
  }
  // After the legal base is installed: the unplaced units and their
  // deviations (the state the reference reaches by installing from an empty
  // placement, without visiting the installed units twice)
  void seed_unplaced() {
    for (uint32_t u = 0; u < m.U; ++u)
      if (choice[u] < 0) {
        unplaced.insert(u);
        if (preferred[u] >= 0) dev[u] = kUnplaced;
      }
  }
  const Footprint& fp(uint32_t u, int64_t c) {
    if (!legality) return none;
    const uint64_t k = ((uint64_t)u << 32) | (uint64_t)c;
    auto it = fps.find(k);
    if (it == fps.end()) it = fps.emplace(k, m.footprint(u, (uint32_t)c)).first;
    return it->second;
  }
  void record(uint32_t u, int64_t c) {
    if (c == preferred[u])
      dev.erase(u);
    else
      dev[u] = c < 0 ? kUnplaced : c;
  }
  Footprint probe;   // the footprint of a choice only tested (not cached)
  bool can_install(uint32_t u, int64_t c) {
    const uint32_t* r = m.row(u, (uint32_t)c);
    for (uint32_t i = 0; i < m.ncells(u); ++i)
      if (bel_owner[r[i]] >= 0) return false;
    if (!legality) return true;
    const uint64_t k = ((uint64_t)u << 32) | (uint64_t)c;
    auto hit = fps.find(k);
    if (hit == fps.end()) m.footprint_into(u, (uint32_t)c, probe);
    const Footprint& f = hit == fps.end() ? probe : hit->second;
    for (size_t i = 0; i < f.pins.size();) {
      const uint32_t w = f.pins[i].first;
      auto it = pin_owner.find(w);
      size_t have = it == pin_owner.end() ? 0 : it->second.size(), add = 0;
      size_t j = i;
      for (; j < f.pins.size() && f.pins[j].first == w; ++j)
        if (it == pin_owner.end() || !it->second.count(f.pins[j].second)) ++add;
      if (have + add > m.wire_cap[w]) return false;
      i = j;
    }
    for (size_t i = 0; i < f.shared.size();) {
      const SharedKey& res = f.shared[i].first;
      auto it = shared_owner.find(res);
      size_t have = it == shared_owner.end() ? 0 : it->second.size(), add = 0;
      size_t j = i;
      for (; j < f.shared.size() && f.shared[j].first == res; ++j)
        if (it == shared_owner.end() || !it->second.count(f.shared[j].second)) ++add;
      if (have + add > 1) return false;
      i = j;
    }
    return true;
  }
  void raw_install(uint32_t u, int64_t c) {
    const uint32_t* r = m.row(u, (uint32_t)c);
    const Footprint& f = fp(u, c);
    for (uint32_t i = 0; i < m.ncells(u); ++i) {
      bel_owner[r[i]] = (int32_t)u;
      placed[m.cell(u, i)] = (int32_t)r[i];
    }
    for (const PinClaim& p : f.pins) pin_owner[p.first][p.second].insert(u);
    for (const SharedClaim& s : f.shared) shared_owner[s.first][s.second].insert(u);
    choice[u] = c;
    unplaced.erase(u);
    record(u, c);
  }
  void raw_remove(uint32_t u, int64_t c) {
    const uint32_t* r = m.row(u, (uint32_t)c);
    const Footprint& f = fp(u, c);
    for (uint32_t i = 0; i < m.ncells(u); ++i) {
      bel_owner[r[i]] = -1;
      placed[m.cell(u, i)] = -1;
    }
    for (const PinClaim& p : f.pins) {
      auto& nets = pin_owner[p.first];
      auto& owners = nets[p.second];
      owners.erase(u);
      if (owners.empty()) nets.erase(p.second);
      if (nets.empty()) pin_owner.erase(p.first);
    }
    for (const SharedClaim& s : f.shared) {
      auto& vals = shared_owner[s.first];
      auto& owners = vals[s.second];
      owners.erase(u);
      if (owners.empty()) vals.erase(s.second);
      if (vals.empty()) shared_owner.erase(s.first);
    }
    choice[u] = -1;
    unplaced.insert(u);
    record(u, -1);
  }
  void remove_branch(uint32_t u) {
    const int64_t c = choice[u];
    raw_remove(u, c);
    journal.push_back({false, u, c});
  }
  void install_branch(uint32_t u, int64_t c) {
    raw_install(u, c);
    journal.push_back({true, u, c});
  }
  void rollback(size_t mark) {
    while (journal.size() > mark) {
      const Entry e = journal.back();
      journal.pop_back();
      if (e.installed)
        raw_remove(e.unit, e.choice);
      else
        raw_install(e.unit, e.choice);
    }
  }
  int64_t next_unplaced() const { return unplaced.empty() ? -1 : (int64_t)*unplaced.begin(); }
  Key key() const { return Key(dev.begin(), dev.end()); }
};

// `enumerate_combinations` (repair.rs:1232-1257)
std::vector<std::vector<uint32_t>> combinations(uint32_t n, uint32_t k) {
  std::vector<std::vector<uint32_t>> out;
  if (k > n) return out;
  std::vector<uint32_t> cur(k);
  for (uint32_t i = 0; i < k; ++i) cur[i] = i;
  for (;;) {
    out.push_back(cur);
    int64_t piv = -1;
    for (int64_t i = (int64_t)k - 1; i >= 0; --i)
      if (cur[i] < n - k + (uint32_t)i) {
        piv = i;
        break;
      }
    if (piv < 0) return out;
    ++cur[piv];
    for (uint32_t i = (uint32_t)piv + 1; i < k; ++i) cur[i] = cur[i - 1] + 1;
  }
}

using Branch = std::vector<uint32_t>;   // sorted unit ids

// ---- `RepairSearch` (repair.rs:592-1230) -------------------------------------
struct Search {
  State& s;
  texo_gp_repair_stats& st;
  std::set<Key> visiting, failed;

  void frame_seen() {
    st.states_visited++;
    st.max_unplaced = std::max<uint64_t>(st.max_unplaced, s.unplaced.size());
  }
  Cursor cursor(uint32_t u) { return Cursor(s.m, u, s.preferred[u]); }

  // `mandatory_blockers` (:1119-1167); false: the choice is impossible
  bool mandatory(uint32_t u, int64_t c, std::set<uint32_t>& out) {
    out.clear();
    const uint32_t* r = s.m.row(u, (uint32_t)c);
    for (uint32_t i = 0; i < s.m.ncells(u); ++i) {
      const int32_t o = s.bel_owner[r[i]];
      if (o >= 0) {
        if (s.fixed[o]) return false;
        out.insert((uint32_t)o);
      }
    }
    const Footprint& f = s.fp(u, c);
    for (size_t i = 0; i < f.shared.size();) {
      const SharedKey& res = f.shared[i].first;
      size_t j = i + 1;
      while (j < f.shared.size() && f.shared[j].first == res) ++j;
      if (j - i > 1) return false;   // claims are distinct: two values for one resource
      const uint64_t v = f.shared[i].second;
      auto it = s.shared_owner.find(res);
      if (it != s.shared_owner.end())
        for (const auto& kv : it->second) {
          if (kv.first == v) continue;
          for (uint32_t o : kv.second) {
            if (s.fixed[o]) return false;
            out.insert(o);
          }
        }
      i = j;
    }
    return true;
  }

  // `pin_blocker_branches` (:1169-1230)
  std::vector<Branch> pin_branches(uint32_t u, int64_t c, const std::set<uint32_t>& mand) {
    const Footprint& f = s.fp(u, c);
    std::vector<Branch> branches{Branch(mand.begin(), mand.end())};
    for (size_t i = 0; i < f.pins.size();) {
      const uint32_t w = f.pins[i].first;
      std::set<uint32_t> cand;
      size_t j = i;
      for (; j < f.pins.size() && f.pins[j].first == w; ++j) cand.insert(f.pins[j].second);
      i = j;
      const uint32_t cap = s.m.wire_cap[w];
      if (cand.size() > cap) return {};
      std::vector<Branch> next;
      auto wit = s.pin_owner.find(w);
      for (const Branch& bl : branches) {
        std::vector<std::pair<uint32_t, std::vector<uint32_t>>> eff;
        if (wit != s.pin_owner.end())
          for (const auto& kv : wit->second) {
            std::vector<uint32_t> rem;
            for (uint32_t o : kv.second)
              if (!std::binary_search(bl.begin(), bl.end(), o)) rem.push_back(o);
            if (!rem.empty()) eff.emplace_back(kv.first, std::move(rem));
          }
        std::set<uint32_t> distinct(cand);
        for (const auto& e : eff) distinct.insert(e.first);
        const size_t need = distinct.size() > cap ? distinct.size() - cap : 0;
        if (need == 0) {
          next.push_back(bl);
          continue;
        }
        std::vector<const std::vector<uint32_t>*> removable;
        for (const auto& e : eff) {
          if (cand.count(e.first)) continue;
          bool movable = true;
          for (uint32_t o : e.second)
            if (s.fixed[o]) movable = false;
          if (movable) removable.push_back(&e.second);
        }
        if (removable.size() < need) continue;
        for (const auto& comb : combinations((uint32_t)removable.size(), (uint32_t)need)) {
          std::set<uint32_t> nb(bl.begin(), bl.end());
          for (uint32_t k : comb) nb.insert(removable[k]->begin(), removable[k]->end());
          next.emplace_back(nb.begin(), nb.end());
        }
      }
      std::sort(next.begin(), next.end());
      next.erase(std::unique(next.begin(), next.end()), next.end());
      branches.swap(next);
      if (branches.empty()) break;
    }
    return branches;
  }

  // `try_direct_empty_fast_path` (:853-886)
  bool direct() {
    const size_t mark = s.journal.size();
    for (int64_t u; (u = s.next_unplaced()) >= 0;) {
      Cursor cur = cursor((uint32_t)u);
      bool done = false;
      for (int64_t c; (c = cur.next()) >= 0;) {
        st.direct_fast_choices++;
        st.choices_examined++;
        if (s.can_install((uint32_t)u, c)) {
          s.install_branch((uint32_t)u, c);
          st.direct_fast_moves++;
          done = true;
          break;
        }
      }
      if (!done) {
        s.rollback(mark);
        st.direct_fast_fallbacks++;
        return false;
      }
    }
    s.journal.resize(mark);
    return true;
  }

  // `augment_one` (:919-996)
  bool augment(uint32_t root) {
    struct Frame {
      uint32_t unit;
      Cursor cur;
      int64_t resume;
    };
    const size_t root_mark = s.journal.size();
    std::set<uint32_t> seen_units{root};
    std::set<std::pair<uint32_t, int64_t>> seen;
    frame_seen();
    std::vector<Frame> stack;
    stack.push_back({root, cursor(root), -1});
    std::set<uint32_t> mand;
    while (!stack.empty()) {
      Frame fr = std::move(stack.back());
      stack.pop_back();
      if (fr.resume >= 0) {
        s.rollback((size_t)fr.resume);
        fr.resume = -1;
      }
      const int64_t c = fr.cur.next();
      if (c < 0) continue;
      if (!seen.insert({fr.unit, c}).second) {
        stack.push_back(std::move(fr));
        continue;
      }
      st.choices_examined++;
      if (!mandatory(fr.unit, c, mand)) {
        stack.push_back(std::move(fr));
        continue;
      }
      const std::vector<Branch> br = pin_branches(fr.unit, c, mand);
      st.max_blocker_branches = std::max<uint64_t>(st.max_blocker_branches, br.size());
      if (br.size() != 1 || br[0].size() > 1) {
        stack.push_back(std::move(fr));
        continue;
      }
      const int64_t blocker = br[0].empty() ? -1 : (int64_t)br[0][0];
      if (blocker >= 0 && seen_units.count((uint32_t)blocker)) {
        stack.push_back(std::move(fr));
        continue;
      }
      const size_t mark = s.journal.size();
      if (blocker >= 0) {
        s.remove_branch((uint32_t)blocker);
        st.units_evicted++;
      }
      if (!s.can_install(fr.unit, c)) {
        s.rollback(mark);
        stack.push_back(std::move(fr));
        continue;
      }
      s.install_branch(fr.unit, c);
      if (blocker < 0) return true;
      seen_units.insert((uint32_t)blocker);
      frame_seen();
      fr.resume = (int64_t)mark;
      stack.push_back(std::move(fr));
      stack.push_back({(uint32_t)blocker, cursor((uint32_t)blocker), -1});
    }
    s.rollback(root_mark);
    return false;
  }

  // `try_single_blocker_fast_path` (:888-917)
  bool single_blocker() {
    const size_t mark = s.journal.size();
    for (int64_t root; (root = s.next_unplaced()) >= 0;) {
      st.augmenting_roots++;
      if (augment((uint32_t)root)) continue;
      s.rollback(mark);
      st.augmenting_fallbacks++;
      return false;
    }
    s.journal.resize(mark);
    return true;
  }

  struct ExactFrame {
    uint32_t unit;
    Key key;
    Cursor cur;
    int64_t choice = -1;
    std::vector<Branch> branches;
    size_t next_branch = 0;
    int64_t resume = -1;
  };
  bool begin(ExactFrame& fr) {
    const int64_t u = s.next_unplaced();
    if (u < 0) return false;
    Key k = s.key();
    if (failed.count(k) || !visiting.insert(k).second) return false;
    frame_seen();
    fr = ExactFrame{(uint32_t)u, std::move(k), cursor((uint32_t)u)};
    return true;
  }
  // `next_exact_attempt` (:1021-1048)
  bool attempt(ExactFrame& fr, int64_t& c, const Branch*& blockers) {
    std::set<uint32_t> mand;
    for (;;) {
      if (fr.next_branch < fr.branches.size()) {
        c = fr.choice;
        blockers = &fr.branches[fr.next_branch++];
        return true;
      }
      const int64_t ch = fr.cur.next();
      if (ch < 0) return false;
      st.choices_examined++;
      if (!mandatory(fr.unit, ch, mand)) continue;
      fr.branches = pin_branches(fr.unit, ch, mand);
      st.max_blocker_branches = std::max<uint64_t>(st.max_blocker_branches, fr.branches.size());
      fr.choice = ch;
      fr.next_branch = 0;
    }
  }
  // `solve_exact_iterative` (:1050-1117)
  bool exact() {
    ExactFrame root;
    if (!begin(root)) return s.next_unplaced() < 0;
    std::vector<ExactFrame> stack;
    stack.push_back(std::move(root));
    while (!stack.empty()) {
      ExactFrame fr = std::move(stack.back());
      stack.pop_back();
      if (fr.resume >= 0) {
        s.rollback((size_t)fr.resume);
        fr.resume = -1;
      }
      int64_t c = -1;
      const Branch* blockers = nullptr;
      if (!attempt(fr, c, blockers)) {
        visiting.erase(fr.key);
        failed.insert(fr.key);
        if (stack.empty()) return false;
        continue;
      }
      const Branch bl = *blockers;
      const size_t mark = s.journal.size();
      for (uint32_t b : bl)
        if (s.choice[b] >= 0) {
          s.remove_branch(b);
          st.units_evicted++;
        }
      if (s.can_install(fr.unit, c)) {
        s.install_branch(fr.unit, c);
        if (s.next_unplaced() < 0) {
          visiting.clear();
          return true;
        }
        ExactFrame child;
        if (begin(child)) {
          fr.resume = (int64_t)mark;
          stack.push_back(std::move(fr));
          stack.push_back(std::move(child));
          continue;
        }
      }
      s.rollback(mark);
      stack.push_back(std::move(fr));
    }
    return false;
  }

  bool solve() {
    if (s.next_unplaced() < 0) return true;
    if (direct()) return true;
    if (single_blocker()) return true;
    return exact();
  }
};

// `initial_pending_units` (repair.rs:325-414)
std::set<uint32_t> initial_pending(State& s) {
  const Model& m = s.m;
  std::vector<uint32_t> claims(m.B, 0);   // proposals naming each BEL
  std::map<uint32_t, std::map<uint32_t, std::set<uint32_t>>> pins;
  std::map<SharedKey, std::map<uint64_t, std::set<uint32_t>>> shared;
  std::set<uint32_t> pending;
  for (uint32_t u = 0; u < m.U; ++u) {
    const int64_t c = s.preferred[u];
    if (c < 0) {
      pending.insert(u);
      continue;
    }
    const uint32_t* r = m.row(u, (uint32_t)c);
    for (uint32_t i = 0; i < m.ncells(u); ++i) ++claims[r[i]];
    const Footprint& f = s.fp(u, c);
    for (const PinClaim& p : f.pins) pins[p.first][p.second].insert(u);
    for (const SharedClaim& sc : f.shared) shared[sc.first][sc.second].insert(u);
  }
  // owners of the BELs claimed twice or more, in unit order
  std::map<uint32_t, std::vector<uint32_t>> contested;
  for (uint32_t u = 0; u < m.U; ++u) {
    const int64_t c = s.preferred[u];
    if (c < 0) continue;
    const uint32_t* r = m.row(u, (uint32_t)c);
    for (uint32_t i = 0; i < m.ncells(u); ++i)
      if (claims[r[i]] > 1) contested[r[i]].push_back(u);
  }
  for (const auto& bo : contested) {
    const std::vector<uint32_t>& owners = bo.second;
    std::vector<uint32_t> fx;
    for (uint32_t u : owners)
      if (s.fixed[u]) fx.push_back(u);
    if (fx.size() > 1)
      throw BadInput{"multiple fixed units occupy one BEL during repair", TEXO_GP_ERR_PROJECTION_CONFLICT};
    uint32_t keep = fx.empty() ? owners[0] : fx[0];
    if (fx.empty())
      for (uint32_t u : owners) {
        const auto ku = std::make_tuple(m.table(u).num_choices, -(int64_t)m.ncells(u), u);
        const auto kk = std::make_tuple(m.table(keep).num_choices, -(int64_t)m.ncells(keep), keep);
        if (ku < kk) keep = u;
      }
    for (uint32_t u : owners)
      if (u != keep) pending.insert(u);
  }
  for (const auto& kv : shared) {
    const auto& values = kv.second;
    if (values.size() < 2) continue;
    std::vector<uint64_t> fv;
    for (const auto& vo : values)
      for (uint32_t u : vo.second)
        if (s.fixed[u]) {
          fv.push_back(vo.first);
          break;
        }
    if (fv.size() > 1)
      throw BadInput{"fixed units require incompatible shared-resource values", TEXO_GP_ERR_PROJECTION_CONFLICT};
    uint64_t keep = 0;
    if (!fv.empty()) {
      keep = fv[0];
    } else {
      size_t best = 0;
      bool first = true;
      for (const auto& vo : values)   // most owners, then the least value (values ascend)
        if (first || vo.second.size() > best) {
          keep = vo.first;
          best = vo.second.size();
          first = false;
        }
    }
    for (const auto& vo : values)
      if (vo.first != keep) pending.insert(vo.second.begin(), vo.second.end());
  }
  for (const auto& kv : pins) {
    const uint32_t cap = m.wire_cap[kv.first];
    if (kv.second.size() <= cap) continue;
    struct Ranked {
      bool has_fixed;
      size_t owners;
      uint32_t net;
      const std::set<uint32_t>* set;
    };
    std::vector<Ranked> ranked;
    for (const auto& no : kv.second) {
      bool f = false;
      for (uint32_t u : no.second) f = f || s.fixed[u];
      ranked.push_back({f, no.second.size(), no.first, &no.second});
    }
    std::sort(ranked.begin(), ranked.end(), [](const Ranked& a, const Ranked& b) {
      if (a.has_fixed != b.has_fixed) return a.has_fixed;
      if (a.owners != b.owners) return a.owners > b.owners;
      return a.net < b.net;
    });
    size_t fixed_nets = 0;
    for (const Ranked& r : ranked) fixed_nets += r.has_fixed;
    if (fixed_nets > cap)
      throw BadInput{"fixed units exceed a placement pin-wire capacity", TEXO_GP_ERR_PROJECTION_CONFLICT};
    for (size_t i = cap; i < ranked.size(); ++i) pending.insert(ranked[i].set->begin(), ranked[i].set->end());
  }
  return pending;
}

int32_t fail(const std::string& why, int32_t code) {
  tgp::set_last_error(why);
  return code;
}

template <typename T>
void csr(uint32_t n, uint32_t count, const uint32_t* owner, std::vector<uint32_t>& ptr, std::vector<T>& out,
         const std::vector<T>& items) {
  ptr.assign(n + 1, 0);
  for (uint32_t k = 0; k < count; ++k) ++ptr[owner[k] + 1];
  for (uint32_t i = 0; i < n; ++i) ptr[i + 1] += ptr[i];
  out.resize(count);
  std::vector<uint32_t> at(ptr.begin(), ptr.end() - 1);
  for (uint32_t k = 0; k < count; ++k) out[at[owner[k]]++] = items[k];
}

}  // namespace

extern "C" int32_t texo_gp_repair(uint32_t width, uint32_t height, uint32_t num_bels, const uint32_t* bel_xy,
                                  uint32_t num_tables, const texo_gp_choice_table* tables, uint32_t num_units,
                                  const uint32_t* unit_table, const uint32_t* unit_cell_ptr,
                                  const uint32_t* unit_cells, uint32_t num_cells, const uint32_t* target_xy,
                                  const int32_t* preferred, const uint8_t* fixed, const texo_gp_legality* legality,
                                  int32_t* out_cell_bel, texo_gp_repair_stats* stats) {
  const auto t0 = std::chrono::steady_clock::now();
  texo_gp_repair_stats st;
  std::memset(&st, 0, sizeof(st));
  if (stats) std::memset(stats, 0, sizeof(*stats));
  if (num_units == 0) {
    if (out_cell_bel)
      for (uint32_t c = 0; c < num_cells; ++c) out_cell_bel[c] = -1;
    return TEXO_GP_OK;
  }
  if (width == 0 || height == 0 || !bel_xy || !tables || !unit_table || !unit_cell_ptr || !unit_cells ||
      !target_xy || !preferred || !fixed || !out_cell_bel)
    return fail("texo_gp_repair: empty grid or null argument", TEXO_GP_ERR_INVALID_ARGUMENT);
  Model m;
  m.W = width, m.H = height, m.B = num_bels, m.U = num_units, m.C = num_cells;
  m.bel_xy = bel_xy, m.tables = tables, m.unit_table = unit_table;
  m.cell_ptr = unit_cell_ptr, m.cells = unit_cells, m.target = target_xy;
  for (uint32_t b = 0; b < num_bels; ++b)
    if (bel_xy[2 * b] >= width || bel_xy[2 * b + 1] >= height)
      return fail("texo_gp_repair: BEL " + std::to_string(b) + " outside the grid", TEXO_GP_ERR_INVALID_ARGUMENT);
  for (uint32_t t = 0; t < num_tables; ++t) {
    const texo_gp_choice_table& tb = tables[t];
    if (tb.num_choices == 0 || tb.width == 0 || !tb.bels)
      return fail("texo_gp_repair: malformed choice table " + std::to_string(t), TEXO_GP_ERR_INVALID_ARGUMENT);
    for (size_t k = 0; k < (size_t)tb.num_choices * tb.width; ++k)
      if (tb.bels[k] >= num_bels)
        return fail("texo_gp_repair: table " + std::to_string(t) + " names a BEL out of range",
                    TEXO_GP_ERR_INVALID_ARGUMENT);
  }
  if (unit_cell_ptr[0] != 0)
    return fail("texo_gp_repair: unit_cell_ptr[0] must be 0", TEXO_GP_ERR_INVALID_ARGUMENT);
  for (uint32_t u = 0; u < num_units; ++u) {
    if (unit_table[u] >= num_tables || target_xy[2 * u] >= width || target_xy[2 * u + 1] >= height)
      return fail("texo_gp_repair: unit " + std::to_string(u) + " table or target out of range",
                  TEXO_GP_ERR_INVALID_ARGUMENT);
    if (unit_cell_ptr[u + 1] <= unit_cell_ptr[u] || unit_cell_ptr[u + 1] - unit_cell_ptr[u] != tables[unit_table[u]].width)
      return fail("texo_gp_repair: unit " + std::to_string(u) + " has no cells or not one per row BEL",
                  TEXO_GP_ERR_INVALID_ARGUMENT);
    for (uint32_t i = unit_cell_ptr[u]; i < unit_cell_ptr[u + 1]; ++i)
      if (unit_cells[i] >= num_cells)
        return fail("texo_gp_repair: unit " + std::to_string(u) + " names a cell out of range",
                    TEXO_GP_ERR_INVALID_ARGUMENT);
  }
  // legality lists
  if (legality) {
    const texo_gp_legality& L = *legality;
    if ((L.num_wires && !L.wire_capacity) ||
        (L.num_cell_pins && (!L.cell_pin_cell || !L.cell_pin_key || !L.cell_pin_net)) ||
        (L.num_bel_pins && (!L.bel_pin_bel || !L.bel_pin_key || !L.bel_pin_wire)) ||
        (L.num_cell_values && (!L.cell_value_rule || !L.cell_value_cell || !L.cell_value)) ||
        (L.num_bel_resources && (!L.bel_resource_rule || !L.bel_resource_bel || !L.bel_resource)))
      return fail("texo_gp_repair: a legality list without its arrays", TEXO_GP_ERR_INVALID_ARGUMENT);
    m.wire_cap.assign(L.wire_capacity, L.wire_capacity + L.num_wires);
    std::vector<std::pair<uint32_t, uint32_t>> cp(L.num_cell_pins), bp(L.num_bel_pins);
    std::vector<std::pair<uint32_t, uint64_t>> cv(L.num_cell_values), br(L.num_bel_resources);
    for (uint32_t k = 0; k < L.num_cell_pins; ++k) {
      if (L.cell_pin_cell[k] >= num_cells)
        return fail("texo_gp_repair: cell pin " + std::to_string(k) + " names a cell out of range",
                    TEXO_GP_ERR_INVALID_ARGUMENT);
      cp[k] = {L.cell_pin_key[k], L.cell_pin_net[k]};
    }
    for (uint32_t k = 0; k < L.num_bel_pins; ++k) {
      if (L.bel_pin_bel[k] >= num_bels || L.bel_pin_wire[k] >= L.num_wires)
        return fail("texo_gp_repair: BEL pin " + std::to_string(k) + " out of range", TEXO_GP_ERR_INVALID_ARGUMENT);
      bp[k] = {L.bel_pin_key[k], L.bel_pin_wire[k]};
    }
    for (uint32_t k = 0; k < L.num_cell_values; ++k) {
      if (L.cell_value_cell[k] >= num_cells || L.cell_value_rule[k] >= L.num_rules)
        return fail("texo_gp_repair: cell value " + std::to_string(k) + " out of range", TEXO_GP_ERR_INVALID_ARGUMENT);
      cv[k] = {L.cell_value_rule[k], L.cell_value[k]};
    }
    for (uint32_t k = 0; k < L.num_bel_resources; ++k) {
      if (L.bel_resource_bel[k] >= num_bels || L.bel_resource_rule[k] >= L.num_rules)
        return fail("texo_gp_repair: BEL resource " + std::to_string(k) + " out of range",
                    TEXO_GP_ERR_INVALID_ARGUMENT);
      br[k] = {L.bel_resource_rule[k], L.bel_resource[k]};
    }
    csr(num_cells, L.num_cell_pins, L.cell_pin_cell, m.cp_ptr, m.cp, cp);
    csr(num_bels, L.num_bel_pins, L.bel_pin_bel, m.bp_ptr, m.bp, bp);
    for (uint32_t b = 0; b < num_bels; ++b) {
      std::sort(m.bp.begin() + m.bp_ptr[b], m.bp.begin() + m.bp_ptr[b + 1]);
      for (uint32_t k = m.bp_ptr[b] + 1; k < m.bp_ptr[b + 1]; ++k)
        if (m.bp[k].first == m.bp[k - 1].first)
          return fail("texo_gp_repair: BEL " + std::to_string(b) + " binds one pin key twice",
                      TEXO_GP_ERR_INVALID_ARGUMENT);
    }
    csr(num_cells, L.num_cell_values, L.cell_value_cell, m.cv_ptr, m.cv, cv);
    csr(num_bels, L.num_bel_resources, L.bel_resource_bel, m.br_ptr, m.br, br);
  } else {
    m.cp_ptr.assign(num_cells + 1, 0);
    m.bp_ptr.assign(num_bels + 1, 0);
    m.cv_ptr.assign(num_cells + 1, 0);
    m.br_ptr.assign(num_bels + 1, 0);
  }
  m.sp_ptr.resize(num_tables);
  m.sp_idx.resize(num_tables);

  std::vector<int64_t> pref(num_units);
  std::vector<uint8_t> fx(fixed, fixed + num_units);
  for (uint32_t u = 0; u < num_units; ++u) {
    pref[u] = preferred[u] < 0 ? -1 : preferred[u];
    if (pref[u] >= (int64_t)tables[unit_table[u]].num_choices)
      return fail("transactional repair received an out-of-range assignment", TEXO_GP_ERR_PROJECTION_CONFLICT);
    if (fx[u] && pref[u] < 0)
      return fail("transactional repair received an unmatched fixed unit", TEXO_GP_ERR_PROJECTION_CONFLICT);
  }
  try {
    State s(m, pref, fx);
    const std::set<uint32_t> pending = initial_pending(s);
    st.initial_pending = pending.size();
    st.max_unplaced = pending.size();
    for (int pass = 0; pass < 2; ++pass)   // fixed units, then the others
      for (uint32_t u = 0; u < num_units; ++u) {
        if ((fx[u] != 0) != (pass == 0) || pref[u] < 0 || pending.count(u)) continue;
        if (!s.can_install(u, pref[u]))
          return fail("relaxed-conflict removal did not leave a legal repair base", TEXO_GP_ERR_PROJECTION_CONFLICT);
        s.raw_install(u, pref[u]);
      }
    s.seed_unplaced();
    const int64_t first = s.next_unplaced();
    Search search{s, st, {}, {}};
    const bool ok = search.solve();
    st.failed_states = search.failed.size();
    st.elapsed_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (!ok) {
      st.failed_cell = m.cell(first >= 0 ? (uint32_t)first : 0u, 0);
      if (stats) *stats = st;
      return fail("no legal BEL for cell " + std::to_string(st.failed_cell), TEXO_GP_ERR_NO_BEL);
    }
    for (uint32_t c = 0; c < num_cells; ++c) out_cell_bel[c] = s.placed[c];
  } catch (const BadInput& e) {
    return fail(e.why, e.code);
  }
  if (stats) *stats = st;
  return TEXO_GP_OK;
}
