// auction_oracle.cpp — TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of the capacity auction of Texo's legalizer, used by the
// test suite as the checker and by the benchmark as the timed CPU baseline of
// the auction; the product path never links it.
//
//   assign_implicitly            crates/texo-pnr/src/legalization/auction.rs:131-247
//   explicit_best_two            auction.rs:253-272 (the reference tests' search)
//   best_objects_on_cached_rings legalization/mod.rs:876-970 (the ring walk;
//   discover_legal_ring          mod.rs:972-1021  its per-bidder ring cache only
//   insert_best_two              mod.rs:1163-1174 saves legality checks, so the
//   ring_coordinates             lib.rs:6814-6821 walk here is uncached)
//
// The auction is the reference's: one bidder at a time from a FIFO queue,
// epsilon one, a private dummy of cost n * max_base_cost + n + 1 per bidder.
// A second driver, assign_jacobi, restates the parallel rounds the GPU runs
// with the same searches, so the GPU's result can be checked bit for bit.
#include <cstdint>
#include <cstring>
#include <deque>
#include <vector>

#include "texo_oracle.h"

namespace {

struct Priced {
  uint64_t object, base, reduced;
};
struct BestTwo {
  bool has_best = false, has_second = false;
  Priced best{}, second{};
  uint64_t examined = 0;
};

bool key_less(const Priced& a, const Priced& b) {
  return a.reduced < b.reduced || (a.reduced == b.reduced && a.object < b.object);
}

// insert_best_two (mod.rs:1163-1174)
void insert_best_two(BestTwo& r, const Priced& c) {
  if (!r.has_best || key_less(c, r.best)) {
    if (r.has_best) {
      r.second = r.best;
      r.has_second = true;
    }
    r.best = c;
    r.has_best = true;
  } else if (!r.has_second || key_less(c, r.second)) {
    r.second = c;
    r.has_second = true;
  }
}

bool add_overflows(uint64_t a, uint64_t b, uint64_t* out) { return __builtin_add_overflow(a, b, out); }
bool mul_overflows(uint64_t a, uint64_t b, uint64_t* out) { return __builtin_mul_overflow(a, b, out); }

// assign_implicitly (auction.rs:131-247). The reference fixes cost_scale at 1
// (:142); with a scale s the reduced costs are s * base + price and the
// dummy n * s * max_base_cost + n + 1, which is the same rule on the scaled
// costs.
template <class Search>
int32_t assign_fifo(uint64_t n, uint64_t m, uint64_t max_base_cost, uint64_t scale, Search&& search,
                    int32_t* assignment, uint64_t* prices_out, orc_auction_stats* st) {
  orc_auction_stats s{};
  if (n == 0) {
    if (st) *st = s;
    return 0;
  }
  uint64_t dummy = 0, tmp = 0, top = 0;
  // D = n * s * max_base_cost + n + 1, and D + 1 + s * max_base_cost must stay representable (:143-162)
  if (scale == 0 || mul_overflows(scale, max_base_cost, &top) || mul_overflows(n, top, &dummy) ||
      add_overflows(dummy, n, &dummy) || add_overflows(dummy, 1, &dummy) || add_overflows(dummy, 1, &tmp) ||
      add_overflows(tmp, top, &tmp))
    return TEXO_GP_ERR_AUCTION_RANGE;
  std::vector<uint64_t> prices(m, 0);
  std::vector<int64_t> owners(m, -1);
  std::vector<int64_t> assign(n, -1);
  std::vector<uint64_t> held_base(n, 0);   // base cost of the object each bidder holds
  std::deque<uint64_t> queue;
  for (uint64_t b = 0; b < n; ++b) queue.push_back(b);
  while (!queue.empty()) {
    const uint64_t bidder = queue.front();
    queue.pop_front();
    BestTwo real = search(bidder, prices);
    s.examined += real.examined;
    const Priced* both[2] = {real.has_best ? &real.best : nullptr, real.has_second ? &real.second : nullptr};
    for (const Priced* c : both) {
      if (!c) continue;
      if (c->object >= m) return TEXO_GP_ERR_AUCTION_OBJECT_RANGE;
      if (c->base > max_base_cost) return TEXO_GP_ERR_AUCTION_COST_RANGE;
    }
    if (real.has_best && real.has_second && real.best.object == real.second.object)
      return TEXO_GP_ERR_AUCTION_DUPLICATE_OBJECT;
    // [best, second, dummy] sorted by (reduced cost, object); the dummy's
    // object sorts last, so a real object wins an equal-cost tie (:207-219)
    const Priced dummy_choice{UINT64_MAX, max_base_cost, dummy};
    Priced choice[3];
    int count = 0;
    if (real.has_best) choice[count++] = real.best;
    if (real.has_second) choice[count++] = real.second;
    choice[count++] = dummy_choice;
    for (int i = 1; i < count; ++i)
      for (int j = i; j > 0 && key_less(choice[j], choice[j - 1]); --j) std::swap(choice[j], choice[j - 1]);
    const Priced best = choice[0];
    if (best.object == UINT64_MAX) {
      assign[bidder] = -1;
      continue;
    }
    const Priced second = choice[1];
    const uint64_t increment = second.reduced - best.reduced + 1;
    prices[best.object] += increment;
    const int64_t displaced = owners[best.object];
    owners[best.object] = (int64_t)bidder;
    if (displaced >= 0) {
      assign[displaced] = -1;
      queue.push_back((uint64_t)displaced);
    }
    assign[bidder] = (int64_t)best.object;
    held_base[bidder] = best.base;
    s.bids++;
  }
  for (uint64_t b = 0; b < n; ++b) {
    assignment[b] = (int32_t)assign[b];
    if (assign[b] < 0)
      s.unmatched++;
    else
      s.total_base_cost += held_base[b];
  }
  if (prices_out)
    for (uint64_t o = 0; o < m; ++o) prices_out[o] = prices[o];
  if (st) *st = s;
  return 0;
}

// The parallel (Jacobi) form of the same auction, the rule the GPU runs:
// every active bidder bids at the prices of the round's start; each object
// bid on goes to its highest offer (equal offers: the lower bidder index) at
// the offered price; its previous holder and the losing bidders form the
// next round's active set. Bidders whose best option is their dummy leave.
// The outcome of a round depends only on the active set, so this sequential
// restatement gives the GPU's assignment, prices, rounds and bids exactly.
template <class Search>
int32_t assign_jacobi(uint64_t n, uint64_t m, uint64_t max_base_cost, uint64_t scale, Search&& search,
                      int32_t* assignment, uint64_t* prices_out, orc_auction_stats* st, uint64_t* rounds_out) {
  orc_auction_stats s{};
  uint64_t rounds = 0;
  if (n == 0) {
    if (st) *st = s;
    if (rounds_out) *rounds_out = 0;
    return 0;
  }
  uint64_t dummy = 0, tmp = 0, top = 0;
  if (scale == 0 || mul_overflows(scale, max_base_cost, &top) || mul_overflows(n, top, &dummy) ||
      add_overflows(dummy, n, &dummy) || add_overflows(dummy, 1, &dummy) || add_overflows(dummy, 1, &tmp) ||
      add_overflows(tmp, top, &tmp))
    return TEXO_GP_ERR_AUCTION_RANGE;
  std::vector<uint64_t> prices(m, 0), best_offer(m, 0);
  std::vector<int64_t> owners(m, -1), winner(m, -1), assign(n, -1);
  std::vector<uint64_t> held_base(n, 0), want_base(n, 0);
  std::vector<int64_t> want(n, -1);
  std::vector<uint64_t> active(n), next, touched;
  for (uint64_t b = 0; b < n; ++b) active[b] = b;
  while (!active.empty()) {
    ++rounds;
    touched.clear();
    for (uint64_t bidder : active) {
      BestTwo real = search(bidder, prices);
      s.examined += real.examined;
      const Priced dummy_choice{UINT64_MAX, max_base_cost, dummy};
      if (!real.has_best || key_less(dummy_choice, real.best)) {
        want[bidder] = -1;
        continue;
      }
      const Priced second = (!real.has_second || key_less(dummy_choice, real.second)) ? dummy_choice : real.second;
      const uint64_t o = real.best.object;
      const uint64_t offer = prices[o] + (second.reduced - real.best.reduced) + 1;
      if (winner[o] < 0) touched.push_back(o);
      if (winner[o] < 0 || offer > best_offer[o] || (offer == best_offer[o] && (int64_t)bidder < winner[o])) {
        best_offer[o] = offer;
        winner[o] = (int64_t)bidder;
      }
      want[bidder] = (int64_t)o;
      want_base[bidder] = real.best.base;
      s.bids++;
    }
    next.clear();
    for (uint64_t o : touched) {
      const int64_t w = winner[o], prev = owners[o];
      owners[o] = w;
      prices[o] = best_offer[o];
      assign[w] = (int64_t)o;
      held_base[w] = want_base[w];
      if (prev >= 0) {
        assign[prev] = -1;
        next.push_back((uint64_t)prev);
      }
    }
    for (uint64_t bidder : active)
      if (want[bidder] >= 0 && winner[want[bidder]] != (int64_t)bidder) next.push_back(bidder);
    for (uint64_t o : touched) {
      winner[o] = -1;
      best_offer[o] = 0;
    }
    active.swap(next);
  }
  for (uint64_t b = 0; b < n; ++b) {
    assignment[b] = (int32_t)assign[b];
    if (assign[b] < 0)
      s.unmatched++;
    else
      s.total_base_cost += held_base[b];
  }
  if (prices_out)
    for (uint64_t o = 0; o < m; ++o) prices_out[o] = prices[o];
  if (st) *st = s;
  if (rounds_out) *rounds_out = rounds;
  return 0;
}

// Up-front checks shared by both searches: objects in range, none listed twice.
int32_t check_objects(const uint32_t* objects, uint64_t count, uint32_t m, std::vector<uint32_t>& stamp,
                      uint32_t mark) {
  for (uint64_t k = 0; k < count; ++k) {
    const uint32_t o = objects[k];
    if (o >= m) return TEXO_GP_ERR_AUCTION_OBJECT_RANGE;
    if (stamp[o] == mark) return TEXO_GP_ERR_AUCTION_DUPLICATE_OBJECT;
    stamp[o] = mark;
  }
  return 0;
}

struct Grid {
  uint32_t W, H, K;
  const uint32_t* tile_ptr;
  const uint32_t* tile_object;
  const uint8_t* occupied;
};

// ring_coordinates (lib.rs:6814-6821): center - offset and center + offset
// (the latter only for a nonzero offset), each kept when inside [0, extent)
int ring_coordinates(uint32_t center, uint32_t offset, uint32_t extent, uint32_t out[2]) {
  int c = 0;
  if (center >= offset && center - offset < extent) out[c++] = center - offset;
  if (offset != 0 && (uint64_t)center + offset < extent) out[c++] = center + offset;
  return c;
}

// Visits ring r around (tx, ty) in the reference's order (dy ascending, minus
// before plus), calling f(object) for each unoccupied candidate; returns the
// candidates visited, occupied ones included.
template <class F>
uint64_t visit_ring(const Grid& g, uint32_t kind, uint32_t tx, uint32_t ty, uint32_t r, F&& f) {
  uint64_t examined = 0;
  const uint64_t base = (uint64_t)kind * g.W * g.H;
  for (uint32_t dy = 0; dy <= r; ++dy) {
    const uint32_t dx = r - dy;
    uint32_t ys[2], xs[2];
    const int ny = ring_coordinates(ty, dy, g.H, ys);
    const int nx = ring_coordinates(tx, dx, g.W, xs);
    for (int a = 0; a < ny; ++a)
      for (int c = 0; c < nx; ++c) {
        const uint64_t t = base + (uint64_t)ys[a] * g.W + xs[c];
        for (uint32_t k = g.tile_ptr[t]; k < g.tile_ptr[t + 1]; ++k) {
          ++examined;
          const uint32_t o = g.tile_object[k];
          if (g.occupied && g.occupied[o]) continue;
          f(o);
        }
      }
  }
  return examined;
}

int32_t check_grid(const Grid& g, uint32_t m, uint32_t n, const uint32_t* kind, const uint32_t* target_xy) {
  if (n == 0) return 0;
  if (g.W == 0 || g.H == 0 || g.K == 0 || !g.tile_ptr || !kind || !target_xy) return TEXO_GP_ERR_INVALID_ARGUMENT;
  const uint64_t slots = (uint64_t)g.K * g.W * g.H;
  if (g.tile_ptr[0] != 0) return TEXO_GP_ERR_INVALID_ARGUMENT;
  for (uint64_t t = 0; t < slots; ++t)
    if (g.tile_ptr[t + 1] < g.tile_ptr[t]) return TEXO_GP_ERR_INVALID_ARGUMENT;
  if (g.tile_ptr[slots] && !g.tile_object) return TEXO_GP_ERR_INVALID_ARGUMENT;
  std::vector<uint32_t> stamp(m, 0);
  const uint64_t per_kind = (uint64_t)g.W * g.H;   // a BEL at most once in each kind's lists
  for (uint32_t q = 0; q < g.K; ++q) {
    const uint32_t k0 = g.tile_ptr[q * per_kind], k1 = g.tile_ptr[(q + 1) * per_kind];
    if (int32_t e = check_objects(g.tile_object + k0, k1 - k0, m, stamp, q + 1)) return e;
  }
  for (uint32_t b = 0; b < n; ++b)
    if (kind[b] >= g.K || target_xy[2 * b] >= g.W || target_xy[2 * b + 1] >= g.H) return TEXO_GP_ERR_INVALID_ARGUMENT;
  return 0;
}

}  // namespace

extern "C" int32_t orc_auction_explicit(uint32_t n, uint32_t m, uint64_t max_base_cost, uint32_t cost_scale,
                                        const uint32_t* ptr, const uint32_t* object, const uint64_t* cost,
                                        int32_t* assignment, uint64_t* prices, orc_auction_stats* st,
                                        uint64_t* rounds) {
  if (st) std::memset(st, 0, sizeof(*st));
  if (n && (!ptr || !assignment || ptr[0] != 0)) return TEXO_GP_ERR_INVALID_ARGUMENT;
  std::vector<uint32_t> stamp(m, 0);
  for (uint32_t b = 0; b < n; ++b) {
    if (ptr[b + 1] < ptr[b]) return TEXO_GP_ERR_INVALID_ARGUMENT;
    if (int32_t e = check_objects(object + ptr[b], ptr[b + 1] - ptr[b], m, stamp, b + 1)) return e;
    for (uint32_t k = ptr[b]; k < ptr[b + 1]; ++k)
      if (cost[k] > max_base_cost) return TEXO_GP_ERR_AUCTION_COST_RANGE;
  }
  // explicit_best_two (auction.rs:253-272): the two least (reduced cost, object)
  auto search = [&](uint64_t b, const std::vector<uint64_t>& price) {
    BestTwo r;
    for (uint32_t k = ptr[b]; k < ptr[b + 1]; ++k) {
      insert_best_two(r, Priced{object[k], cost[k], cost_scale * cost[k] + price[object[k]]});
      ++r.examined;
    }
    return r;
  };
  if (rounds) return assign_jacobi(n, m, max_base_cost, cost_scale, search, assignment, prices, st, rounds);
  return assign_fifo(n, m, max_base_cost, cost_scale, search, assignment, prices, st);
}

extern "C" int32_t orc_auction_singletons(uint32_t width, uint32_t height, uint32_t num_kinds, const uint32_t* tile_ptr,
                                          const uint32_t* tile_object, uint32_t num_objects, const uint8_t* occupied,
                                          uint32_t num_bidders, const uint32_t* bidder_kind,
                                          const uint32_t* target_xy, uint32_t cost_scale, int32_t* assignment,
                                          uint64_t* prices, orc_auction_stats* st, uint64_t* rounds) {
  if (st) std::memset(st, 0, sizeof(*st));
  const Grid g{width, height, num_kinds, tile_ptr, tile_object, occupied};
  if (int32_t e = check_grid(g, num_objects, num_bidders, bidder_kind, target_xy)) return e;
  if (num_bidders == 0) return 0;
  const uint64_t max_base_cost = (uint64_t)(width - 1) + (height - 1);
  const uint32_t max_radius = (width - 1) + (height - 1);
  // best_objects_on_cached_rings (mod.rs:876-970) without the cache
  auto search = [&](uint64_t b, const std::vector<uint64_t>& price) {
    BestTwo r;
    const uint32_t tx = target_xy[2 * b], ty = target_xy[2 * b + 1];
    for (uint32_t radius = 0;; ++radius) {
      const uint64_t ring_cost = (uint64_t)cost_scale * radius;
      r.examined += visit_ring(g, bidder_kind[b], tx, ty, radius,
                               [&](uint32_t o) { insert_best_two(r, Priced{o, radius, ring_cost + price[o]}); });
      if (radius == max_radius) break;
      // strict: an unseen object at the next radius could tie the second best
      if (r.has_second && r.second.reduced < ring_cost + cost_scale) break;
    }
    return r;
  };
  if (rounds)
    return assign_jacobi(num_bidders, num_objects, max_base_cost, cost_scale, search, assignment, prices, st, rounds);
  return assign_fifo(num_bidders, num_objects, max_base_cost, cost_scale, search, assignment, prices, st);
}

// Epsilon-complementary-slackness certificate of a singleton auction result:
// every object held at most once, by a bidder of its kind, unoccupied; every
// matched bidder's reduced cost within one of its best option (real or
// dummy); every unmatched bidder's dummy within one of its best real object;
// every unassigned object at price 0. Together these bound the total base
// cost by the optimum of the same cardinality plus the bidder count.
// `base_costs` (may be NULL) receives each matched bidder's base cost (0 for
// unmatched). `dual_bound` (may be NULL) receives the assignment dual's value
// at these prices, sum over bidders of the least reduced cost (dummy
// included) minus the sum of all prices: a lower bound on the least total
// cost (dummies at D) of any assignment. Returns the number of violations;
// *first_bad the first bidder (or object + num_bidders) that fails.
extern "C" int64_t orc_auction_check_singletons(uint32_t width, uint32_t height, uint32_t num_kinds,
                                                const uint32_t* tile_ptr, const uint32_t* tile_object,
                                                uint32_t num_objects, const uint8_t* occupied, uint32_t num_bidders,
                                                const uint32_t* bidder_kind, const uint32_t* target_xy,
                                                uint32_t cost_scale, const int32_t* assignment, const uint32_t* prices,
                                                uint64_t* base_costs, uint64_t* first_bad, int64_t* dual_bound) {
  const Grid g{width, height, num_kinds, tile_ptr, tile_object, occupied};
  if (check_grid(g, num_objects, num_bidders, bidder_kind, target_xy)) return -1;
  int64_t bad = 0;
  uint64_t first = UINT64_MAX;
  auto fail = [&](uint64_t who) {
    if (first == UINT64_MAX) first = who;
    ++bad;
  };
  // where each BEL sits: (kind, x, y)
  std::vector<int64_t> where(num_objects, -1);
  const uint64_t tiles = (uint64_t)width * height;
  for (uint64_t s = 0; s < (uint64_t)num_kinds * tiles; ++s)
    for (uint32_t k = tile_ptr[s]; k < tile_ptr[s + 1]; ++k) where[tile_object[k]] = (int64_t)s;
  std::vector<int64_t> holder(num_objects, -1);
  const uint64_t n = num_bidders, max_base_cost = (uint64_t)(width - 1) + (height - 1);
  const uint64_t s = cost_scale ? cost_scale : 1;
  const uint64_t dummy = n * s * max_base_cost + n + 1;
  const uint32_t max_radius = (width - 1) + (height - 1);
  __int128 dual = 0;
  for (uint32_t o = 0; o < num_objects; ++o) dual -= prices[o];
  for (uint32_t b = 0; b < num_bidders; ++b) {
    const uint32_t tx = target_xy[2 * b], ty = target_xy[2 * b + 1];
    uint64_t mine = UINT64_MAX;   // reduced cost of the held option
    if (base_costs) base_costs[b] = 0;
    if (assignment[b] >= 0) {
      const uint32_t o = (uint32_t)assignment[b];
      if (o >= num_objects || where[o] < 0 || (uint64_t)where[o] / tiles != bidder_kind[b] ||
          (occupied && occupied[o]) || holder[o] >= 0) {
        fail(b);
        continue;
      }
      holder[o] = b;
      const uint64_t t = (uint64_t)where[o] % tiles;
      const uint32_t x = (uint32_t)(t % width), y = (uint32_t)(t / width);
      const uint64_t base = (uint64_t)(x > tx ? x - tx : tx - x) + (y > ty ? y - ty : ty - y);
      if (base_costs) base_costs[b] = base;
      mine = s * base + prices[o];
    } else {
      mine = dummy;
    }
    // least reduced cost over every real candidate: rings until the radius
    // passes the best found (a ring-r object costs at least r)
    uint64_t least = dummy;
    for (uint32_t r = 0;; ++r) {
      if (s * r > least) break;
      visit_ring(g, bidder_kind[b], tx, ty, r, [&](uint32_t o) {
        const uint64_t c = s * r + (uint64_t)prices[o];
        if (c < least) least = c;
      });
      if (r == max_radius) break;
    }
    dual += least;
    if (mine > least + 1) fail(b);
  }
  if (dual_bound) *dual_bound = (int64_t)dual;
  for (uint32_t o = 0; o < num_objects; ++o)
    if (holder[o] < 0 && prices[o] != 0) fail((uint64_t)num_bidders + o);
  if (first_bad) *first_bad = first;
  return bad;
}
