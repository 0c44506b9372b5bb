// auction.cu — the capacity auction of the legalizer on the GPU
// (`assign_implicitly`, crates/texo-pnr/src/legalization/auction.rs:131-247,
// as `auction_singletons` / `auction_units` call it, legalization/mod.rs:
// 657-677, 733-840).
//
// The reference bids one bidder at a time from a FIFO queue. Here every
// unassigned bidder bids in the same round (a Jacobi auction), which keeps
// the guarantees the reference states for its result: epsilon one, a private
// dummy of cost D = n * s * max_base_cost + n + 1 per bidder, so the assignment
// has exactly the maximum cardinality and a total base cost at most n / s
// above the least one of that cardinality (s the cost scale, 1 in the
// reference). Prices only rise, every bid raises its
// object's price by at least one, and an object priced above D is no better
// than any bidder's dummy, so the rounds end.
//
// One cooperative persistent kernel runs the auction; a round is two phases
// between bounded grid barriers:
//   bid     one warp per active bidder finds its two least (reduced cost,
//           object) candidates - a Manhattan ring walk over the BEL grid
//           (best_objects_on_cached_rings, mod.rs:876-970) or a scan of an
//           explicit domain - sets the price the bid offers,
//           second - best + 1 above the current one, and posts
//           (offered price, ~bidder) with a 64-bit atomicMax on the object;
//           the first poster of an object lists it as touched.
//   resolve each touched object goes to its highest bid (equal offers: the
//           lower bidder index) at the offered price; its previous holder
//           and the round's losing bidders form the next round's active list.
// An object's price and holder are written only in the resolve phase, the
// bids only in the bid phase, so a round's outcome depends on the set of
// active bidders alone, not on the order threads reach the atomics: the
// result is deterministic. The bid slots, touched lists and active lists
// alternate between two buffers and the list counters rotate over four
// slots, so no phase clears what another block may still read.
#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "engine.h"
#include "persistent_body.cuh"

namespace tgp {
namespace {

constexpr int kAucThreads = 256;
constexpr int kAucWarps = kAucThreads / 32;
constexpr int kAucBlocksPerSm = 2;   // resident blocks a multiprocessor runs
constexpr int kTailPerWarp = 2;      // active bidders per warp at which block 0 finishes alone
constexpr unsigned kNone = 0xFFFFFFFFu;
constexpr unsigned long long kNoKey = ~0ull;                      // "no candidate"
constexpr unsigned long long kTimeLimitNs = 20ull * 1000000000ull; // the whole auction

struct AucResult {
  unsigned rounds;
  unsigned tail_rounds;  // rounds run by block 0 alone
  unsigned stop_round;   // nonzero: every block leaves at the top of this round (the time limit ran out)
  unsigned pad;
  unsigned long long bids, examined;
  unsigned long long total_base;   // sum of the holders' base costs (kept as holders change)
  unsigned long long matched;      // objects held
};

struct AucDev {
  int grid;            // 1 ring walks over the BEL grid, 0 explicit domains
  unsigned n, m;
  unsigned scale;      // s: reduced cost = s * base cost + price
  unsigned dummy;      // D = n * s * max_base_cost + n + 1
  // explicit domains
  const unsigned *dptr, *dobj, *dcost;
  // BEL grid
  unsigned W, H, max_radius, slots;
  const unsigned *tptr, *tobj, *kind, *txy;
  const unsigned char* occ;
  // auction state
  unsigned* price;
  int* owner;
  unsigned long long* bid;   // [2][m]
  int* assign;
  unsigned* want;            // object bid on this round, or kNone
  unsigned* want_base;       // base cost of that object
  unsigned* held_base;       // base cost of the object held
  unsigned* act;             // [2][n] active bidders
  unsigned* touched;         // [2][cap] objects bid on
  unsigned cap;
  unsigned* cnt;             // active counts [4], touched counts [4]
  GridBarrier* bar;
  AucResult* out;
};

__device__ __forceinline__ unsigned long long make_key(unsigned reduced, unsigned object) {
  return ((unsigned long long)reduced << 32) | object;
}

// best two of (a1 <= a2) and (b1 <= b2), drawn from disjoint candidate sets
__device__ __forceinline__ void merge2(unsigned long long& a1, unsigned long long& a2, unsigned long long b1,
                                       unsigned long long b2) {
  const unsigned long long lo = a1 < b1 ? a1 : b1, hi = a1 < b1 ? b1 : a1;
  a1 = lo;
  a2 = min(hi, min(a2, b2));
}

__device__ __forceinline__ void insert2(unsigned long long& a1, unsigned long long& a2, unsigned long long k) {
  if (k < a1) {
    a2 = a1;
    a1 = k;
  } else if (k < a2) {
    a2 = k;
  }
}

__device__ __forceinline__ void warp_best2(unsigned long long& a1, unsigned long long& a2) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const unsigned long long b1 = __shfl_xor_sync(0xffffffffu, a1, off);
    const unsigned long long b2 = __shfl_xor_sync(0xffffffffu, a2, off);
    merge2(a1, a2, b1, b2);
  }
}

// Objects of one tile a lane reads per batch in the ring walk.
constexpr int kTileBatch = 8;

// The Manhattan diamond around a target, flattened in ring order: point 0 is
// ring 0, ring r >= 1 holds the points [1 + 2r(r-1), 1 + 2r(r+1)).
__device__ __forceinline__ unsigned ring_of(unsigned p) {
  if (p == 0) return 0;
  unsigned r = (unsigned)((1.0f + sqrtf((float)(2u * p - 1u))) * 0.5f);
  if (r == 0) r = 1;
  while (1u + 2u * r * (r + 1u) <= p) ++r;
  while (r > 1u && 1u + 2u * r * (r - 1u) > p) --r;
  return r;
}

// The two least (reduced cost, object) keys among bidder b's candidates, the
// same in every lane of the warp. Returns the candidates this lane visited.
//
// The ring walk hands the warp 32 consecutive points of the diamond at a
// time and stops once the second best is below the least cost an unseen
// object can have, s times the first ring not fully seen. Visiting rings
// past the reference's stopping ring adds only objects that cannot enter
// the best two, so the result is the reference's exact best two.
__device__ __forceinline__ unsigned long long best_two(const AucDev& d, unsigned b, int lane, unsigned long long& k1,
                                                       unsigned long long& k2) {
  unsigned long long a1 = kNoKey, a2 = kNoKey, seen = 0;
  if (!d.grid) {
    const unsigned e = __ldg(d.dptr + b + 1);
    for (unsigned k = __ldg(d.dptr + b) + lane; k < e; k += 32) {
      const unsigned o = __ldg(d.dobj + k);
      insert2(a1, a2, make_key(d.scale * __ldg(d.dcost + k) + __ldcg(d.price + o), o));
      ++seen;
    }
    warp_best2(a1, a2);
  } else {
    const int tx = (int)__ldg(d.txy + 2 * b), ty = (int)__ldg(d.txy + 2 * b + 1);
    const int W = (int)d.W, H = (int)d.H;
    const unsigned* tp = d.tptr + (size_t)__ldg(d.kind + b) * d.W * d.H;
    const unsigned R = d.max_radius;
    const unsigned total = 1u + 2u * R * (R + 1u);   // points of the whole diamond
    unsigned long long m1 = kNoKey, m2 = kNoKey;
    for (unsigned p0 = 0;; p0 += 32) {
      const unsigned p = p0 + lane;
      if (p < total) {
        const unsigned r = ring_of(p);
        int dx = 0, dy = 0;
        if (r) {
          // ring r as four quarter turns of (r - i, i)
          const unsigned j = p - (1u + 2u * r * (r - 1u)), q = j / r, i = j - q * r;
          const int u = (int)(r - i), v = (int)i;
          dx = q == 0 ? u : q == 1 ? -v : q == 2 ? -u : v;
          dy = q == 0 ? v : q == 1 ? u : q == 2 ? -v : -u;
        }
        const int x = tx + dx, y = ty + dy;
        if (x >= 0 && y >= 0 && x < W && y < H) {
          const int t = y * W + x;
          const unsigned ring_cost = d.scale * r, e = __ldg(tp + t + 1);
          // a tile's objects kTileBatch at a time, their loads issued together
          // (keys are distinct, so the order of insertion does not matter);
          // a tile with one object takes the short path
          const unsigned kb = __ldg(tp + t);
          if (e == kb + 1) {
            const unsigned o = __ldg(d.tobj + kb);
            ++seen;
            if (!(d.occ && __ldg(d.occ + o))) insert2(a1, a2, make_key(ring_cost + __ldcg(d.price + o), o));
          } else
          for (unsigned k0 = kb; k0 < e; k0 += kTileBatch) {
            unsigned o[kTileBatch], pr[kTileBatch];
            bool use[kTileBatch];
#pragma unroll
            for (int i = 0; i < kTileBatch; ++i) o[i] = k0 + i < e ? __ldg(d.tobj + k0 + i) : kNone;
#pragma unroll
            for (int i = 0; i < kTileBatch; ++i) {
              use[i] = o[i] != kNone && !(d.occ && __ldg(d.occ + o[i]));
              pr[i] = o[i] != kNone ? __ldcg(d.price + o[i]) : 0u;
            }
#pragma unroll
            for (int i = 0; i < kTileBatch; ++i) {
              seen += o[i] != kNone;
              if (use[i]) insert2(a1, a2, make_key(ring_cost + pr[i], o[i]));
            }
          }
        }
      }
      // the warp's best two so far, merged from copies: each lane keeps the
      // best two of the points it visited itself, so the merge always joins
      // disjoint candidate sets
      m1 = a1;
      m2 = a2;
      warp_best2(m1, m2);
      const unsigned last = min(p0 + 32u, total) - 1u;
      if (last == total - 1u) break;   // every ring seen
      const unsigned rl = ring_of(last);
      const unsigned unseen = last == 2u * rl * (rl + 1u) ? rl + 1u : rl;   // first ring not fully seen
      // strict: an unseen object could tie the second best
      if (m2 != kNoKey && (unsigned)(m2 >> 32) < d.scale * unseen) break;
    }
    a1 = m1;
    a2 = m2;
  }
  k1 = a1;
  k2 = a2;
  return seen;
}

// Bid phase of round k: warps [w0, w0 + nw) of the launch take the active
// bidders in turn.
__device__ __forceinline__ void bid_phase(const AucDev& d, unsigned k, unsigned nA, unsigned w0, unsigned nw, int lane,
                                          unsigned long long& bids, unsigned long long& seen) {
  const unsigned cur = k & 1u;
  const unsigned* A = d.act + (size_t)cur * d.n;
  unsigned long long* bidc = d.bid + (size_t)cur * d.m;
  unsigned* cntT = d.cnt + 4;
  for (unsigned j = w0; j < nA; j += nw) {
    const unsigned b = __ldcg(A + j);
    unsigned long long k1, k2;
    seen += best_two(d, b, lane, k1, k2);
    if (lane == 0) {
      const unsigned long long dummy = make_key(d.dummy, kNone);
      if (k1 > dummy) {
        d.want[b] = kNone;   // the private dummy is strictly better: unmatched for good
      } else {
        const unsigned o = (unsigned)k1, price = __ldcg(d.price + o);
        const unsigned second = (unsigned)(min(k2, dummy) >> 32), best = (unsigned)(k1 >> 32);
        const unsigned offer = price + (second - best) + 1u;
        const unsigned long long old = atomicMax(bidc + o, make_key(offer, kNone - b));
        if (old == 0) d.touched[(size_t)cur * d.cap + atomicAdd(cntT + (k & 3u), 1u)] = o;
        d.want[b] = o;
        d.want_base[b] = (best - price) / d.scale;
        ++bids;
      }
    }
  }
}

// Resolve phase of round k over threads [t0, t0 + nt): each touched object
// goes to its highest bid; the holders it displaces and the round's losing
// bidders form the next round's active list; the previous round's bid slots
// are cleared. Returns this thread's change of the held base-cost total and
// of the number of held objects.
__device__ __forceinline__ void resolve_phase(const AucDev& d, unsigned k, unsigned nA, unsigned t0, unsigned nt,
                                              long long& dbase, long long& dmatched) {
  const unsigned cur = k & 1u, nxt = cur ^ 1u;
  unsigned* cntA = d.cnt;
  unsigned* cntT = d.cnt + 4;
  const unsigned nT = __ldcg(cntT + (k & 3u));
  const unsigned* T = d.touched + (size_t)cur * d.cap;
  const unsigned* A = d.act + (size_t)cur * d.n;
  const unsigned long long* bidc = d.bid + (size_t)cur * d.m;
  unsigned* N = d.act + (size_t)nxt * d.n;
  for (unsigned t = t0; t < nT; t += nt) {
    const unsigned o = __ldcg(T + t);
    const unsigned long long key = __ldcg(bidc + o);
    const unsigned w = kNone - (unsigned)key;
    const int prev = __ldcg(d.owner + o);
    const unsigned wb = __ldcg(d.want_base + w);
    d.owner[o] = (int)w;
    d.price[o] = (unsigned)(key >> 32);
    d.assign[w] = (int)o;
    d.held_base[w] = wb;
    dbase += wb;
    if (prev >= 0) {
      d.assign[prev] = -1;
      dbase -= __ldcg(d.held_base + prev);
      N[atomicAdd(cntA + ((k + 1) & 3u), 1u)] = (unsigned)prev;
    } else {
      ++dmatched;
    }
  }
  for (unsigned j = t0; j < nA; j += nt) {
    const unsigned b = __ldcg(A + j);
    const unsigned o = __ldcg(d.want + b);
    if (o == kNone) continue;
    if (kNone - (unsigned)__ldcg(bidc + o) != b) N[atomicAdd(cntA + ((k + 1) & 3u), 1u)] = b;
  }
  // the previous round's touched list is stable now: clear its bid slots
  const unsigned nP = __ldcg(cntT + ((k + 3) & 3u));
  const unsigned* P = d.touched + (size_t)nxt * d.cap;
  unsigned long long* bidp = d.bid + (size_t)nxt * d.m;
  for (unsigned t = t0; t < nP; t += nt) bidp[__ldcg(P + t)] = 0;
}

// Adds the block's changes of the held totals to the result (one atomic each
// when nonzero).
__device__ __forceinline__ void publish_totals(const AucDev& d, long long dbase, long long dmatched, long long* sh) {
  if (threadIdx.x == 0) sh[0] = sh[1] = 0;
  __syncthreads();
  if (dbase) atomicAdd((unsigned long long*)&sh[0], (unsigned long long)dbase);
  if (dmatched) atomicAdd((unsigned long long*)&sh[1], (unsigned long long)dmatched);
  __syncthreads();
  if (threadIdx.x == 0) {
    if (sh[0]) atomicAdd(&d.out->total_base, (unsigned long long)sh[0]);
    if (sh[1]) atomicAdd(&d.out->matched, (unsigned long long)sh[1]);
  }
}

__global__ void __launch_bounds__(kAucThreads, kAucBlocksPerSm) k_auction(AucDev d) {
  __shared__ unsigned gen;
  __shared__ int failed, s_stop;
  __shared__ unsigned long long s_bids, s_seen;
  __shared__ long long s_tot[2];
  const int pb = blockIdx.x, np = gridDim.x;
  const int lane = threadIdx.x & 31;
  const unsigned gtid = pb * blockDim.x + threadIdx.x, gstride = np * blockDim.x;
  const unsigned gwarp = pb * kAucWarps + (threadIdx.x >> 5), nwarps = np * kAucWarps;
  unsigned long long nbar = 0, my_bids = 0, my_seen = 0;
  const unsigned long long t_start = now_ns();
  unsigned* cntA = d.cnt;
  unsigned* cntT = d.cnt + 4;
  if (threadIdx.x == 0) {
    gen = 0;
    s_bids = s_seen = 0;
  }
  // initial state: every bidder active in index order, prices zero
  for (unsigned o = gtid; o < d.m; o += gstride) {
    d.price[o] = 0;
    d.owner[o] = -1;
    d.bid[o] = 0;
    d.bid[d.m + o] = 0;
  }
  for (unsigned b = gtid; b < d.n; b += gstride) {
    d.assign[b] = -1;
    d.want[b] = kNone;
    d.act[b] = b;
  }
  if (pb == 0 && threadIdx.x < 8) d.cnt[threadIdx.x] = threadIdx.x == 0 ? d.n : 0u;
  if (!grid_sync(d.bar, (unsigned)np, &gen, &nbar, nullptr, &failed)) return;

  unsigned k = 0;
  bool tail = false;
  for (;; ++k) {
    const unsigned nA = __ldcg(cntA + (k & 3u));
    // block 0 may set the stop round during this round's bid phase; it names
    // the next round, so every block reads the same decision at each top
    const unsigned stop = __ldcg(&d.out->stop_round);
    if (nA == 0 || (stop != 0 && k >= stop)) break;
    // The active set never grows (a bidder wins, displacing at most one
    // holder, loses or leaves), so once it fits one block that block
    // finishes the auction alone, without grid barriers.
    if (nA <= (unsigned)kAucWarps * kTailPerWarp) {
      tail = true;
      break;
    }
    if (pb == 0 && threadIdx.x == 0) {
      cntA[(k + 2) & 3u] = 0;
      cntT[(k + 1) & 3u] = 0;
      if (now_ns() - t_start > kTimeLimitNs) d.out->stop_round = k + 1;
    }
    bid_phase(d, k, nA, gwarp, nwarps, lane, my_bids, my_seen);
    if (!grid_sync(d.bar, (unsigned)np, &gen, &nbar, nullptr, &failed)) return;
    long long dbase = 0, dmatched = 0;
    resolve_phase(d, k, nA, gtid, gstride, dbase, dmatched);
    publish_totals(d, dbase, dmatched, s_tot);
    if (!grid_sync(d.bar, (unsigned)np, &gen, &nbar, nullptr, &failed)) return;
  }
  const unsigned grid_rounds = k;
  if (tail && pb == 0) {
    for (;; ++k) {
      const unsigned nA = __ldcg(cntA + (k & 3u));
      if (threadIdx.x == 0) {
        s_stop = now_ns() - t_start > kTimeLimitNs;
        if (s_stop) d.out->stop_round = k + 1;
        cntA[(k + 2) & 3u] = 0;
        cntT[(k + 1) & 3u] = 0;
      }
      __syncthreads();
      if (nA == 0 || s_stop) break;
      bid_phase(d, k, nA, threadIdx.x >> 5, kAucWarps, lane, my_bids, my_seen);
      __syncthreads();
      long long dbase = 0, dmatched = 0;
      resolve_phase(d, k, nA, threadIdx.x, blockDim.x, dbase, dmatched);
      publish_totals(d, dbase, dmatched, s_tot);   // ends with the block barrier the next round needs
    }
  }
  atomicAdd(&s_bids, my_bids);
  atomicAdd(&s_seen, my_seen);
  __syncthreads();
  if (threadIdx.x == 0) {
    atomicAdd(&d.out->bids, s_bids);
    atomicAdd(&d.out->examined, s_seen);
    if (pb == 0) {
      d.out->rounds = k;
      d.out->tail_rounds = k - grid_rounds;
    }
  }
}

}  // namespace
}  // namespace tgp

using namespace tgp;

namespace {

// Host side shared by both entry points: the checked inputs in device
// layout, then one allocation, the copies, one cooperative launch, the
// copies back.
struct AucHost {
  bool grid = false;
  uint32_t n = 0, m = 0;
  uint64_t max_base_cost = 0;
  uint32_t scale = 1;
  // explicit
  const uint32_t* dptr = nullptr;
  const uint32_t* dobj = nullptr;
  std::vector<uint32_t> dcost;
  // grid
  uint32_t W = 0, H = 0, K = 0;
  const uint32_t *tptr = nullptr, *tobj = nullptr, *kind = nullptr, *txy = nullptr;
  const uint8_t* occ = nullptr;
};

int32_t fail_with(texo_gp_auction_stats* st, int32_t code, const std::string& why) {
  if (!why.empty()) set_last_error(why);
  if (st) st->status = code;
  return code;
}

// The reference's range check (auction.rs:143-162) at the device's 32-bit
// prices and cost scale s: the dummy cost D = n * s * max_base_cost + n + 1,
// plus one, plus s * max_base_cost must stay below 2^32.
bool dummy_cost(uint64_t n, uint64_t max_base_cost, uint64_t scale, uint32_t* out) {
  const unsigned __int128 top = (unsigned __int128)scale * max_base_cost;
  const unsigned __int128 d = (unsigned __int128)n * top + n + 1;
  if (d + 1 + top >= ((unsigned __int128)1 << 32)) return false;
  *out = (uint32_t)d;
  return true;
}

// The scale to run with: the caller's, or (0) the largest of 4, 2, 1 that
// fits; 0 when none does. Rounds grow about in proportion to the scale
// (a displaced bidder moves one ring out only after s price steps), while the
// matched cost gains little past 4: on the 42k workload's targets s = 4 lands
// within 0.03 % of s = 8's total displacement in 84 instead of 181 rounds, on
// a congested ECP5-like fabric within 0.15 % in 903 instead of 2,416.
uint32_t pick_scale(uint64_t n, uint64_t max_base_cost, uint32_t requested) {
  uint32_t d = 0;
  if (requested) return dummy_cost(n, max_base_cost, requested, &d) ? requested : 0u;
  for (uint32_t s : {4u, 2u, 1u})
    if (dummy_cost(n, max_base_cost, s, &d)) return s;
  return 0u;
}

constexpr const char* kRangeText =
    "auction price range: n * s * max_base_cost + n + 2 + s * max_base_cost must stay below 2^32";

// Up-front object checks shared with the oracle: in range, none twice in one list.
int32_t check_objects(const uint32_t* objects, uint64_t count, uint32_t m, std::vector<uint32_t>& stamp, uint32_t mark) {
  for (uint64_t k = 0; k < count; ++k) {
    const uint32_t o = objects[k];
    if (o >= m) return TEXO_GP_ERR_AUCTION_OBJECT_RANGE;
    if (stamp[o] == mark) return TEXO_GP_ERR_AUCTION_DUPLICATE_OBJECT;
    stamp[o] = mark;
  }
  return TEXO_GP_OK;
}

int32_t run_auction(int32_t device, AucHost& h, int32_t* assignment, uint32_t* prices_out, texo_gp_auction_stats* st) {
  uint32_t dummy = 0;
  if (!dummy_cost(h.n, h.max_base_cost, h.scale, &dummy)) return fail_with(st, TEXO_GP_ERR_AUCTION_RANGE, kRangeText);
  if (cudaSetDevice(device) != cudaSuccess) return fail_with(st, TEXO_GP_ERR_CUDA, "cudaSetDevice failed");
  // resident blocks a multiprocessor, computed once per device ordinal with
  // that device current (the cooperative launch must fit the device it runs on)
  static std::mutex occ_mu;
  static std::map<int32_t, int> occupancy;
  int per_sm = 0;
  {
    std::lock_guard<std::mutex> lk(occ_mu);
    auto it = occupancy.find(device);
    if (it == occupancy.end()) {
      int b = 0;
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_auction, kAucThreads, 0) != cudaSuccess) b = 0;
      it = occupancy.emplace(device, b).first;
    }
    per_sm = it->second;
  }
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (per_sm <= 0 || sms <= 0) return fail_with(st, TEXO_GP_ERR_CUDA, "k_auction cannot be resident");
  const uint64_t want_blocks = std::max<uint64_t>(1, ((uint64_t)h.n + kAucWarps - 1) / kAucWarps);
  const int blocks = (int)std::min<uint64_t>((uint64_t)std::min(per_sm, kAucBlocksPerSm) * sms, want_blocks);

  const uint64_t n = h.n, m = h.m;
  const uint64_t cap = std::max<uint64_t>(1, std::min(n, m));
  const uint64_t slots = h.grid ? (uint64_t)h.K * h.W * h.H : 0;
  const uint64_t nnz = h.grid ? h.tptr[slots] : h.dptr[n];
  auto round = [](uint64_t b) { return (size_t)((b + 255) & ~(uint64_t)255); };
  const size_t sz_m4 = round(std::max<uint64_t>(m, 1) * 4), sz_n4 = round(std::max<uint64_t>(n, 1) * 4);
  const size_t sz_bid = round(std::max<uint64_t>(2 * m, 1) * 8), sz_act = round(2 * std::max<uint64_t>(n, 1) * 4);
  const size_t sz_touch = round(2 * cap * 4), sz_nnz = round(std::max<uint64_t>(nnz, 1) * 4);
  const size_t sz_ptr = round(((h.grid ? slots : n) + 1) * 4);
  const size_t sz_occ = round(h.occ ? m : 1), sz_txy = round(2 * std::max<uint64_t>(n, 1) * 4);
  const size_t total = 2 * sz_m4 + sz_bid + 5 * sz_n4 + sz_act + sz_touch + 2 * sz_nnz + sz_ptr + sz_occ + sz_txy +
                       round(32) + round(sizeof(GridBarrier)) + round(sizeof(AucResult));
  cudaStream_t s = nullptr;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess)
    return fail_with(st, TEXO_GP_ERR_CUDA, "cudaStreamCreate failed");
  char* base = nullptr;
  if (cudaMallocAsync((void**)&base, total, s) != cudaSuccess) {
    cudaStreamDestroy(s);
    return fail_with(st, TEXO_GP_ERR_OUT_OF_MEMORY, "cudaMallocAsync failed");
  }
  char* at = base;
  auto take = [&](size_t b) {
    char* r = at;
    at += b;
    return r;
  };
  AucDev d{};
  d.grid = h.grid ? 1 : 0;
  d.n = h.n;
  d.m = h.m;
  d.scale = h.scale;
  d.dummy = dummy;
  d.price = (unsigned*)take(sz_m4);
  d.owner = (int*)take(sz_m4);
  d.bid = (unsigned long long*)take(sz_bid);
  d.assign = (int*)take(sz_n4);
  d.want = (unsigned*)take(sz_n4);
  d.want_base = (unsigned*)take(sz_n4);
  d.held_base = (unsigned*)take(sz_n4);
  unsigned* kind = (unsigned*)take(sz_n4);
  d.act = (unsigned*)take(sz_act);
  d.touched = (unsigned*)take(sz_touch);
  d.cap = (unsigned)cap;
  unsigned* list = (unsigned*)take(sz_nnz);
  unsigned* cost = (unsigned*)take(sz_nnz);
  unsigned* ptr = (unsigned*)take(sz_ptr);
  unsigned char* occ = (unsigned char*)take(sz_occ);
  unsigned* txy = (unsigned*)take(sz_txy);
  d.cnt = (unsigned*)take(round(32));
  d.bar = (GridBarrier*)take(round(sizeof(GridBarrier)));
  d.out = (AucResult*)take(round(sizeof(AucResult)));
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, s);   // timed: the input copies, the launch, the copies back
  const size_t ptr_bytes = ((h.grid ? slots : n) + 1) * 4;
  bool ok = cudaMemcpyAsync(ptr, h.grid ? h.tptr : h.dptr, ptr_bytes, cudaMemcpyHostToDevice, s) == cudaSuccess;
  if (nnz)
    ok = ok && cudaMemcpyAsync(list, h.grid ? h.tobj : h.dobj, nnz * 4, cudaMemcpyHostToDevice, s) == cudaSuccess;
  if (h.grid) {
    d.W = h.W;
    d.H = h.H;
    d.slots = (unsigned)slots;
    d.max_radius = (h.W - 1) + (h.H - 1);
    d.tptr = ptr;
    d.tobj = list;
    d.kind = kind;
    d.txy = txy;
    d.occ = h.occ ? occ : nullptr;
    ok = ok && cudaMemcpyAsync(kind, h.kind, n * 4, cudaMemcpyHostToDevice, s) == cudaSuccess &&
         cudaMemcpyAsync(txy, h.txy, 2 * n * 4, cudaMemcpyHostToDevice, s) == cudaSuccess;
    if (h.occ) ok = ok && cudaMemcpyAsync(occ, h.occ, m, cudaMemcpyHostToDevice, s) == cudaSuccess;
  } else {
    d.dptr = ptr;
    d.dobj = list;
    d.dcost = cost;
    if (nnz) ok = ok && cudaMemcpyAsync(cost, h.dcost.data(), nnz * 4, cudaMemcpyHostToDevice, s) == cudaSuccess;
  }
  ok = ok && cudaMemsetAsync(d.bar, 0, sizeof(GridBarrier), s) == cudaSuccess &&
       cudaMemsetAsync(d.out, 0, sizeof(AucResult), s) == cudaSuccess;

  if (ok) {
    void* args[] = {&d};
    ok = cudaLaunchCooperativeKernel((const void*)k_auction, dim3(blocks), dim3(kAucThreads), args, 0, s) == cudaSuccess;
    if (ok) note_launch();
  }
  AucResult res{};
  GridBarrier hb{};
  ok = ok && cudaMemcpyAsync(assignment, d.assign, n * 4, cudaMemcpyDeviceToHost, s) == cudaSuccess &&
       cudaMemcpyAsync(&res, d.out, sizeof(AucResult), cudaMemcpyDeviceToHost, s) == cudaSuccess &&
       cudaMemcpyAsync(&hb, d.bar, sizeof(GridBarrier), cudaMemcpyDeviceToHost, s) == cudaSuccess;
  if (prices_out && m)
    ok = ok && cudaMemcpyAsync(prices_out, d.price, m * 4, cudaMemcpyDeviceToHost, s) == cudaSuccess;
  cudaEventRecord(e1, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) ok = false;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFreeAsync(base, s);
  cudaStreamSynchronize(s);
  cudaStreamDestroy(s);
  int32_t code = TEXO_GP_OK;
  if (!ok) {
    code = TEXO_GP_ERR_CUDA;
    set_last_error(std::string("auction: ") + cudaGetErrorString(cudaGetLastError()));
  } else if (hb.error) {
    code = TEXO_GP_ERR_DEVICE_TIMEOUT;
    set_last_error("auction: a grid barrier wait ran out");
  } else if (res.stop_round) {
    code = TEXO_GP_ERR_DEVICE_TIMEOUT;
    set_last_error("auction: the rounds ran past the time limit (" + std::to_string(res.rounds) + " rounds)");
  }
  if (st) {
    st->status = code;
    st->rounds = res.rounds;
    st->cost_scale = h.scale;
    st->bids = res.bids;
    st->candidates_examined = res.examined;
    st->tail_rounds = res.tail_rounds;
    st->unmatched = (uint64_t)h.n - res.matched;
    st->total_base_cost = res.total_base;
    st->elapsed_ms = ms;
    st->kernel_launches = 1;
  }
  return code;
}

}  // namespace

extern "C" int32_t texo_gp_auction_explicit(int32_t device, uint32_t num_bidders, uint32_t num_objects,
                                            uint64_t max_base_cost, uint32_t cost_scale, const uint32_t* domain_ptr,
                                            const uint32_t* domain_object, const uint64_t* domain_cost,
                                            int32_t* assignment, uint32_t* prices, texo_gp_auction_stats* stats) {
  if (stats) std::memset(stats, 0, sizeof(*stats));
  if (num_bidders == 0) return fail_with(stats, TEXO_GP_OK, "");   // the empty auction (auction.rs:138-141)
  if (!domain_ptr || !assignment || domain_ptr[0] != 0)
    return fail_with(stats, TEXO_GP_ERR_INVALID_ARGUMENT, "auction: null argument or domain_ptr[0] != 0");
  std::vector<uint32_t> stamp(num_objects, 0);
  for (uint32_t b = 0; b < num_bidders; ++b) {
    if (domain_ptr[b + 1] < domain_ptr[b])
      return fail_with(stats, TEXO_GP_ERR_INVALID_ARGUMENT, "auction: domain_ptr decreases");
    const uint32_t len = domain_ptr[b + 1] - domain_ptr[b];
    if (len && (!domain_object || !domain_cost))
      return fail_with(stats, TEXO_GP_ERR_INVALID_ARGUMENT, "auction: null domain arrays");
    if (int32_t e = check_objects(domain_object + domain_ptr[b], len, num_objects, stamp, b + 1))
      return fail_with(stats, e,
                       e == TEXO_GP_ERR_AUCTION_OBJECT_RANGE ? "auction: object out of range"
                                                             : "auction: an object twice in one domain");
    for (uint32_t k = domain_ptr[b]; k < domain_ptr[b + 1]; ++k)
      if (domain_cost[k] > max_base_cost)
        return fail_with(stats, TEXO_GP_ERR_AUCTION_COST_RANGE, "auction: base cost above max_base_cost");
  }
  AucHost h;
  h.n = num_bidders;
  h.m = num_objects;
  h.max_base_cost = max_base_cost;
  h.dptr = domain_ptr;
  h.dobj = domain_object;
  // whether every bidder can be matched is not known up front for explicit
  // domains, so the automatic scale is the reference's
  h.scale = pick_scale(num_bidders, max_base_cost, cost_scale ? cost_scale : 1u);
  if (!h.scale) return fail_with(stats, TEXO_GP_ERR_AUCTION_RANGE, kRangeText);
  h.dcost.resize(domain_ptr[num_bidders]);
  for (size_t k = 0; k < h.dcost.size(); ++k) h.dcost[k] = (uint32_t)domain_cost[k];   // <= max_base_cost < 2^32
  return run_auction(device, h, assignment, prices, stats);
}

extern "C" int32_t texo_gp_auction_singletons(int32_t device, uint32_t width, uint32_t height, uint32_t num_kinds,
                                              const uint32_t* tile_ptr, const uint32_t* tile_object,
                                              uint32_t num_objects, const uint8_t* occupied, uint32_t num_bidders,
                                              const uint32_t* bidder_kind, const uint32_t* target_xy,
                                              uint32_t cost_scale, int32_t* assignment, uint32_t* prices,
                                              texo_gp_auction_stats* stats) {
  if (stats) std::memset(stats, 0, sizeof(*stats));
  if (num_bidders == 0) return fail_with(stats, TEXO_GP_OK, "");   // auction_units' empty case (mod.rs:744-747)
  if (width == 0 || height == 0 || num_kinds == 0 || !tile_ptr || !bidder_kind || !target_xy || !assignment)
    return fail_with(stats, TEXO_GP_ERR_INVALID_ARGUMENT, "auction: empty grid or null argument");
  if ((uint64_t)width * height > (1ull << 28) || width > 16384 || height > 16384 ||
      (uint64_t)num_kinds * width * height >= (1ull << 32))
    return fail_with(stats, TEXO_GP_ERR_INVALID_ARGUMENT, "auction: BEL grid too large");
  const uint64_t slots = (uint64_t)num_kinds * width * height;
  if (tile_ptr[0] != 0) return fail_with(stats, TEXO_GP_ERR_INVALID_ARGUMENT, "auction: tile_ptr[0] != 0");
  for (uint64_t t = 0; t < slots; ++t)
    if (tile_ptr[t + 1] < tile_ptr[t])
      return fail_with(stats, TEXO_GP_ERR_INVALID_ARGUMENT, "auction: tile_ptr decreases");
  if (tile_ptr[slots] && !tile_object)
    return fail_with(stats, TEXO_GP_ERR_INVALID_ARGUMENT, "auction: null tile_object");
  // a BEL at most once in each kind's lists (kinds may share BELs: bidders of
  // both compete for its one price)
  std::vector<uint32_t> stamp(num_objects, 0);
  std::vector<uint8_t> listed(num_objects, 0);
  bool shared_bels = false;
  const uint64_t tiles_per_kind = (uint64_t)width * height;
  for (uint32_t q = 0; q < num_kinds; ++q) {
    const uint32_t k0 = tile_ptr[q * tiles_per_kind], k1 = tile_ptr[(q + 1) * tiles_per_kind];
    if (int32_t e = check_objects(tile_object + k0, k1 - k0, num_objects, stamp, q + 1))
      return fail_with(stats, e,
                       e == TEXO_GP_ERR_AUCTION_OBJECT_RANGE ? "auction: BEL out of range"
                                                             : "auction: a BEL listed twice in one kind");
    for (uint32_t k = k0; k < k1; ++k) {
      shared_bels |= listed[tile_object[k]] != 0;
      listed[tile_object[k]] = 1;
    }
  }
  for (uint32_t b = 0; b < num_bidders; ++b)
    if (bidder_kind[b] >= num_kinds || target_xy[2 * b] >= width || target_xy[2 * b + 1] >= height)
      return fail_with(stats, TEXO_GP_ERR_INVALID_ARGUMENT, "auction: bidder kind or target outside the grid");
  AucHost h;
  h.grid = true;
  h.n = num_bidders;
  h.m = num_objects;
  h.max_base_cost = (uint64_t)(width - 1) + (height - 1);
  // Surplus bidders leave only once prices pass the dummy cost D, about one
  // price step a round, and D grows with the scale: scale automatically only
  // when every kind has at least as many free BELs as bidders (then every
  // bidder is matched and no price climbs towards D).
  //
  // With several BELs a tile, a displaced bidder looks one ring out only after
  // s price steps on each of its tile's equal-cost BELs, so the rounds of a
  // congested region grow with s times the BELs a tile: scale automatically
  // only where kinds hold at most two BELs a tile on average (measured: an
  // ECP5-like fabric of 8 LUT and 8 FF BELs a tile, 42,000 singletons, runs
  // 937 rounds at s = 1 and 4,419 at s = 4 for 1.4 % less displacement).
  if (cost_scale == 0) {
    std::vector<uint64_t> free_bels(num_kinds, 0), bidders(num_kinds, 0), bels(num_kinds, 0), tiles_used(num_kinds, 0);
    const uint64_t tiles = (uint64_t)width * height;
    for (uint32_t q = 0; q < num_kinds; ++q)
      for (uint64_t t = q * tiles; t < (q + 1) * tiles; ++t) {
        bels[q] += tile_ptr[t + 1] - tile_ptr[t];
        tiles_used[q] += tile_ptr[t + 1] > tile_ptr[t];
        for (uint32_t k = tile_ptr[t]; k < tile_ptr[t + 1]; ++k)
          free_bels[q] += (occupied && occupied[tile_object[k]]) ? 0 : 1;
      }
    for (uint32_t b = 0; b < num_bidders; ++b) bidders[bidder_kind[b]]++;
    for (uint32_t q = 0; q < num_kinds; ++q)
      if (bidders[q] > free_bels[q] || (bidders[q] && bels[q] > 2 * tiles_used[q])) cost_scale = 1;
    // kinds sharing BELs: whether every bidder can be matched is not known
    // from the per-kind counts
    if (shared_bels) cost_scale = 1;
  }
  h.scale = pick_scale(num_bidders, h.max_base_cost, cost_scale);
  if (!h.scale) return fail_with(stats, TEXO_GP_ERR_AUCTION_RANGE, kRangeText);
  h.W = width;
  h.H = height;
  h.K = num_kinds;
  h.tptr = tile_ptr;
  h.tobj = tile_object;
  h.kind = bidder_kind;
  h.txy = target_xy;
  h.occ = occupied;
  return run_auction(device, h, assignment, prices, stats);
}
