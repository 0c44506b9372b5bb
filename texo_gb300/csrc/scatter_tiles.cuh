// scatter_tiles.cuh — the density scatter privatised in shared memory.
//
// The direct scatter (stage_scatter) sends every one of an object's nine
// B-spline taps to a global int64 atomic; at a million objects the grids'
// atomic throughput bounds it. This form first groups the objects by tile:
// the bin grid is cut into 32 x 32-bin tiles, an object's key is its grid
// (members of field f, or fillers of field f) and the tile of its centre bin,
// and a counting sort orders the objects by key (count with a rank per
// object, exclusive scan, place). Each block then takes an equal run of the
// sorted objects, accumulates the taps of the run's main key into a shared
// 34 x 34-bin window (the tile and a one-bin halo, where every tap of an
// object centred in the tile lands), and flushes the window with one global
// atomic per touched bin; objects of other keys in the run deposit directly.
//
// The deposits are int64 2^-32 fixed point, so their sums do not depend on
// the order or the grouping: the grids, the overflow and the per-field tap
// totals are bit-identical to the direct scatter's (and to the oracle's
// fixed-point restatement), and the counting sort's nondeterministic ranks
// change nothing. (deposit_quadratic_bspline and the field loop,
// electrostatic_placement.rs:296-332, 900-916)
#pragma once
#include "stages.cuh"

namespace tgp {
namespace tiles {

constexpr int kTile = 32;              // bins per tile side
constexpr int kWin = kTile + 2;        // window side: the tile and a one-bin halo

__device__ __forceinline__ int ntiles(const Dev& d) {
  return ((d.g.Wb + kTile - 1) / kTile) * ((d.g.Hb + kTile - 1) / kTile);
}

// The object's position, charge and grid (0..K-1 members, K..2K-1 fillers).
struct Item {
  float x, y, q;
  int grid;
};
__device__ __forceinline__ Item item(const Dev& d, const float2* pos, int i) {
  Item it;
  if (i < d.Mm) {
    const int u = d.mem_unit[i];
    const float2 o = d.mem_off[i];
    const float2 pu = pos[u];
    it.x = __fadd_rn(pu.x, o.x);
    it.y = __fadd_rn(pu.y, o.y);
    it.q = d.mem_q[i];
    it.grid = d.mem_field[i];
  } else {
    const int j = i - d.Mm;
    const float2 pf = pos[d.U + j];
    it.x = pf.x;
    it.y = pf.y;
    it.q = d.fil_q[j];
    it.grid = d.K + d.fil_field[j];
  }
  return it;
}
__device__ __forceinline__ unsigned long long* grid_base(const Dev& d, int grid) {
  return (unsigned long long*)(grid < d.K ? d.phys + (size_t)grid * d.B : d.fill + (size_t)(grid - d.K) * d.B);
}

// Pass 1: key and rank of every object (bin_cnt is zero on entry). Lanes of
// a warp with the same key take one atomic between them.
static __device__ void count(const Dev& d, const float2* pos, int vb, int nvb) {
  const int items = d.Mm + d.F, nt = ntiles(d), tx = (d.g.Wb + kTile - 1) / kTile;
  const int lane = threadIdx.x & 31;
  for (int i0 = vb * blockDim.x + (threadIdx.x & ~31); i0 < items; i0 += nvb * blockDim.x) {
    const int i = i0 + lane;
    int key = -1 - lane;   // distinct for lanes past the end
    if (i < items) {
      const Item it = item(d, pos, i);
      const AxisTaps ax = taps_x(d, it.x);
      const AxisTaps ay = taps_y(d, it.y);
      key = it.grid * nt + (ay.idx[1] / kTile) * tx + ax.idx[1] / kTile;
    }
    const unsigned same = __match_any_sync(0xffffffffu, key);
    const int leader = __ffs(same) - 1;
    int base = 0;
    if (lane == leader && key >= 0) base = atomicAdd(d.bin_cnt + key, __popc(same));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (key >= 0) {
      d.bin_key[i] = key;
      d.bin_rank[i] = base + __popc(same & ((1u << lane) - 1u));
    }
  }
}

// Pass 2 (one block): bin_off = exclusive scan of bin_cnt, which is then
// cleared for the next sort.
static __device__ void scan(const Dev& d) {
  __shared__ int part[kThreads];
  const int nk = 2 * d.K * ntiles(d);
  const int per = (nk + blockDim.x - 1) / blockDim.x;
  const int b = threadIdx.x * per, e = min(b + per, nk);
  int s = 0;
  for (int k = b; k < e; ++k) s += d.bin_cnt[k];
  part[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int run = 0;
    for (int t = 0; t < (int)blockDim.x; ++t) {
      const int v = part[t];
      part[t] = run;
      run += v;
    }
    d.bin_off[nk] = run;
  }
  __syncthreads();
  int run = part[threadIdx.x];
  for (int k = b; k < e; ++k) {
    const int c = d.bin_cnt[k];
    d.bin_off[k] = run;
    run += c;
    d.bin_cnt[k] = 0;
  }
}

// Pass 3: the sorted order.
static __device__ void place(const Dev& d, int vb, int nvb) {
  const int items = d.Mm + d.F;
  for (int i = vb * blockDim.x + threadIdx.x; i < items; i += nvb * blockDim.x)
    d.bin_order[d.bin_off[d.bin_key[i]] + d.bin_rank[i]] = i;
}

struct Smem {
  unsigned long long win[kWin * kWin];
  int key, ox, oy;
};

// Pass 4: block vb takes sorted objects [vb R, (vb + 1) R), R = ceil(items / nvb).
static __device__ void scatter(const Dev& d, const float2* pos, Partials p, int vb, int nvb, Smem& sm,
                               Shared& sh) {
  const int items = d.Mm + d.F, nt = ntiles(d), tx = (d.g.Wb + kTile - 1) / kTile;
  const int R = (items + nvb - 1) / nvb;
  const int s0 = min(vb * R, items), s1 = min(s0 + R, items);
  if (threadIdx.x == 0) {
    // the key with the most objects in this run
    int best = -1, most = 0;
    if (s0 < s1) {
      const int k0 = d.bin_key[d.bin_order[s0]], k1 = d.bin_key[d.bin_order[s1 - 1]];
      for (int k = k0; k <= k1; ++k) {
        const int n = min(d.bin_off[k + 1], s1) - max(d.bin_off[k], s0);
        if (n > most) {
          most = n;
          best = k;
        }
      }
    }
    sm.key = best;
    const int t = best >= 0 ? best % nt : 0;
    sm.ox = (t % tx) * kTile - 1;
    sm.oy = (t / tx) * kTile - 1;
  }
  for (int i = threadIdx.x; i < kWin * kWin; i += blockDim.x) sm.win[i] = 0ull;
  __syncthreads();
  const int wkey = sm.key, ox = sm.ox, oy = sm.oy;
  long long tot[kMaxFields];
#pragma unroll
  for (int f = 0; f < kMaxFields; ++f) tot[f] = 0;
  for (int s = s0 + threadIdx.x; s < s1; s += blockDim.x) {
    const int i = d.bin_order[s];
    const Item it = item(d, pos, i);
    const AxisTaps ax = taps_x(d, it.x);
    const AxisTaps ay = taps_y(d, it.y);
    const bool local = d.bin_key[i] == wkey;
    unsigned long long* g = grid_base(d, it.grid);
    long long sum = 0;
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const long long v = tap_fixed(it.q, ax.w[c], ay.w[r]);
        sum += v;
        if (local)
          atomicAdd(&sm.win[(ay.idx[r] - oy) * kWin + (ax.idx[c] - ox)], (unsigned long long)v);
        else
          atomicAdd(g + (size_t)ay.idx[r] * d.g.Wb + ax.idx[c], (unsigned long long)v);
      }
    const int f = it.grid < d.K ? it.grid : it.grid - d.K;
#pragma unroll
    for (int ff = 0; ff < kMaxFields; ++ff)
      if (ff == f) tot[ff] += sum;
  }
  __syncthreads();
  if (wkey >= 0) {
    unsigned long long* g = grid_base(d, wkey / nt);
    for (int i = threadIdx.x; i < kWin * kWin; i += blockDim.x) {
      const unsigned long long v = sm.win[i];
      const int bx = ox + i % kWin, by = oy + i / kWin;
      if (v && bx >= 0 && by >= 0 && bx < d.g.Wb && by < d.g.Hb) atomicAdd(g + (size_t)by * d.g.Wb + bx, v);
    }
  }
  for (int f = 0; f < d.K; ++f) write_partial(tot[f], islot(p, IS_GRID_SUM + f), vb, sh.l);
}

}  // namespace tiles
}  // namespace tgp
