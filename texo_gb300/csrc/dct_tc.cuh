// dct_tc.cuh — the DCT GEMM passes on tcgen05 tensor cores, BF16x3 form.
//
// Each FP32 operand x is split into bfloat16 halves x = hi + lo (+ O(2^-18 x));
// a product is accumulated as lo*hi + hi*lo + hi*hi in FP32 in tensor memory
// (the published bfloat16x3 scheme of Henry, Tang and Heinecke, ARITH 2019).
//
// Operand layout. Every operand lives in global memory already split and in
// the exact byte layout the MMA reads from shared memory: the canonical
// K-major no-swizzle layout of 8-row x 16-byte core matrices (128 B between
// K-adjacent core matrices, 512 B between 8-row groups), cut into blocks of
// 32 K-elements. An A operand (rows x K) is a grid of 128 x 32 blocks, a B
// operand (output columns x K) a grid of 64 x 32 blocks; each block stores
// its hi half then its lo half, blocks ordered K-chunk fastest. The tiles are
// zero-padded to those multiples. The epilogue of each pass writes its result
// in the layout the next pass reads, so no pass converts its inputs.
//
// One 128 x 64 output tile per block iteration. Thread 0 runs a four-stage
// pipeline: TMA tensor copies (cp.async.bulk.tensor through the operands'
// tensor maps, complete_tx on a "full" mbarrier) keep the next three K-chunks
// in flight while the six MMAs of
// chunk c (two K = 16 steps x three split terms) run, and each commit
// arrives on that stage's "empty" mbarrier before the stage is reloaded.
// The accumulator occupies 64 TMEM columns (row i = lane i); the epilogue
// reads it with tcgen05.ld, warp w taking lanes 32 (w mod 4) ... + 31 and
// columns 32 (w / 4) ... + 31.
//
// Every wait is bounded. When one runs out the block records it (shared
// `failed` and the caller's error word), waits once more (bounded) for its
// own copies and MMAs, frees its tensor memory and leaves its tiles undone.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>

#include "common.cuh"

namespace tgp {
namespace tc {

constexpr int kM = 128;                        // accumulator rows (TMEM lanes)
constexpr int kN = 64;                         // accumulator columns per tile
constexpr int kKC = 32;                        // K per block / pipeline stage
constexpr int kStages = 4;                     // chunks in flight (TMA prefetch depth)
constexpr uint32_t kCols = 64;                 // TMEM columns per block
constexpr uint32_t kCore = 128;                // one 8 x 16 B core matrix
constexpr uint32_t kSbo = (kKC / 8) * kCore;   // next 8-row group
constexpr uint32_t kLbo = kCore;               // next 8-element K group
constexpr uint32_t kABlock = 2u * kM * kKC;    // elements of one A block (hi + lo)
constexpr uint32_t kBBlock = 2u * kN * kKC;    // elements of one B block
constexpr uint32_t kTx = (kABlock + kBBlock) * 2u;   // bytes per stage
constexpr unsigned kWaitLimit = 1u << 22;      // mbarrier polls before giving up
// kind::f16 instruction descriptor: D = F32, A = B = BF16, both K-major, N, M.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kN >> 3) << 17) |
                            ((uint32_t)(kM >> 4) << 24);

// TMA descriptors of the tiled operands, each a 2-D view of one operand
// buffer as rows of 128 bytes (64 bf16 halves): an A block is a 64 x 128
// box (16 KB), a B block a 64 x 64 box (8 KB). The data are already in the
// MMA's shared-memory layout, so the copies use no swizzle.
enum TcMap { TM_RHO = 0, TM_T1, TM_T2, TM_T3, TM_CXB, TM_CYA, TM_CYTA, TM_CXTB, TM_COUNT };
struct alignas(64) TcMaps {
  CUtensorMap m[TM_COUNT];
};

// ---- layout (host and device) ------------------------------------------------
__host__ __device__ inline uint32_t kmaj(int r, int k) {
  return (uint32_t)(r >> 3) * kSbo + (uint32_t)(k >> 3) * kCore + (uint32_t)(r & 7) * 16u + (uint32_t)(k & 7) * 2u;
}
__host__ __device__ inline int pad(int n, int m) { return (n + m - 1) / m * m; }
// element index of (row r, k) half `half` in an A operand with K padded to kp
__host__ __device__ inline size_t a_index(int r, int k, int kp, int half) {
  const size_t blk = ((size_t)(r >> 7) * (size_t)(kp >> 5) + (size_t)(k >> 5)) * kABlock;
  return blk + (size_t)half * (kM * kKC) + kmaj(r & 127, k & 31) / 2;
}
// element index of (output column n, k) half `half` in a B operand
__host__ __device__ inline size_t b_index(int n, int k, int kp, int half) {
  const size_t blk = ((size_t)(n >> 6) * (size_t)(kp >> 5) + (size_t)(k >> 5)) * kBBlock;
  return blk + (size_t)half * (kN * kKC) + kmaj(n & 63, k & 31) / 2;
}
__host__ __device__ inline void split(float v, uint16_t& hi, uint16_t& lo) {
  const __nv_bfloat16 h = __float2bfloat16_rn(v);
  hi = __bfloat16_as_ushort(h);
  lo = __bfloat16_as_ushort(__float2bfloat16_rn(v - __bfloat162float(h)));
}

#ifdef __CUDACC__
struct alignas(128) Stage {
  uint16_t a[kABlock];
  uint16_t b[kBBlock];
};
struct alignas(128) Smem {
  Stage st[kStages];
  unsigned long long full[kStages], empty[kStages];
  uint32_t tmem;
  uint32_t full_ph[kStages], empty_ph[kStages];   // completed phases waited on (thread 0)
  int failed;
};

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t sdesc(uint32_t a) {
  return (uint64_t)((a & 0x3FFFFu) >> 4) | ((uint64_t)(kLbo >> 4) << 16) | ((uint64_t)(kSbo >> 4) << 32) |
         (1ull << 46);
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy global writes ordered with later TMA (async-proxy) reads
__device__ __forceinline__ void fence_global_async() { asm volatile("fence.proxy.async.global;" ::: "memory"); }

__device__ __forceinline__ void mma(uint32_t d, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(kIdesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ bool try_wait(uint32_t mbar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred P;\n\tmbarrier.try_wait.parity.shared::cta.b64 P, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, P;\n\t}\n"
      : "=r"(ok)
      : "r"(mbar), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool wait_phase(uint32_t mbar, uint32_t parity) {
  for (unsigned i = 0; i < kWaitLimit; ++i)
    if (try_wait(mbar, parity)) return true;
  return false;
}

// One block of a tiled operand: box of 128-byte rows starting at row y.
__device__ __forceinline__ void tensor_load(uint32_t dst, const CUtensorMap* map, int y, uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"((unsigned long long)map), "r"(0), "r"(y), "r"(mbar)
      : "memory");
}

// Block-wide: tensor memory and the mbarriers (every thread calls it).
__device__ __forceinline__ void setup(Smem& sm) {
  if (threadIdx.x == 0) {
    for (int i = 0; i < kStages; ++i) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(saddr(&sm.full[i])) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(saddr(&sm.empty[i])) : "memory");
      sm.full_ph[i] = 0;
      sm.empty_ph[i] = 0;
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    sm.failed = 0;
  }
  if (threadIdx.x < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(&sm.tmem)),
                 "r"(kCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_before();
  __syncthreads();
  fence_after();
}

// Block-wide: frees the tensor memory (gemm has waited, bounded, for every
// copy and MMA it issued before it returns).
__device__ __forceinline__ void teardown(Smem& sm) {
  fence_before();
  __syncthreads();
  if (threadIdx.x < 32) {
    fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(sm.tmem), "r"(kCols) : "memory");
  }
  __syncthreads();
}

#define TGP_TC_R(i) "=r"(v[i])
__device__ __forceinline__ void ld16(uint32_t taddr, uint32_t* v) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];\n"
      : TGP_TC_R(0), TGP_TC_R(1), TGP_TC_R(2), TGP_TC_R(3), TGP_TC_R(4), TGP_TC_R(5), TGP_TC_R(6), TGP_TC_R(7),
        TGP_TC_R(8), TGP_TC_R(9), TGP_TC_R(10), TGP_TC_R(11), TGP_TC_R(12), TGP_TC_R(13), TGP_TC_R(14), TGP_TC_R(15)
      : "r"(taddr)
      : "memory");
}
#undef TGP_TC_R

// Where a pass puts its result: the next pass's B operand (epi 0, or 1 with
// the inverse-eigenvalue scaling), its A operand (epi 2), or the FP32
// potential with the energy <rho, phi> (epi 3).
struct Out {
  int epi;
  uint16_t* t;         // tiled operand for epi 0..2
  long ts;             // its per-field stride (elements)
  int kp;              // its padded K
  float* phi;          // epi 3
  const float* rho;    // epi 3 (FP32 mean-free density)
  const float* inv_eig;
};

__device__ __forceinline__ void emit(const Out& o, int f, int row, int col, int M, int N, float x, float& e) {
  const size_t idx = (size_t)row * N + col;
  uint16_t h, l;
  switch (o.epi) {
    case 0:
    case 1:
      if (o.epi == 1) x *= o.inv_eig[idx];
      split(x, h, l);
      o.t[(size_t)f * o.ts + b_index(col, row, o.kp, 0)] = h;
      o.t[(size_t)f * o.ts + b_index(col, row, o.kp, 1)] = l;
      break;
    case 2:
      split(x, h, l);
      o.t[(size_t)f * o.ts + a_index(row, col, o.kp, 0)] = h;
      o.t[(size_t)f * o.ts + a_index(row, col, o.kp, 1)] = l;
      break;
    default:
      o.phi[(size_t)f * M * N + idx] = x;
      e = fmaf(o.rho[(size_t)f * M * N + idx], x, e);
      break;
  }
}

// C[f] = A[f] (M x K) * B[f]^T, B given as N x K, both tiled; output tiles
// t = vb, vb + nvb, ... of 128 x 64, written by `out`. kp = K padded to 32.
// The block must have called setup(); blockDim.x must be 256.
static __device__ void gemm(const CUtensorMap* mA, long sa, const CUtensorMap* mB, long sb, int M, int N, int kp,
                            int nf, const Out& out, double* eacc, int vb, int nvb, Smem& sm, unsigned long long* err) {
  const int tiles_m = (M + kM - 1) / kM, tiles_n = (N + kN - 1) / kN;
  const int tiles = tiles_m * tiles_n * nf;
  const int nkc = kp / kKC;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  for (int t = vb; t < tiles; t += nvb) {
    if (sm.failed) break;
    const int f = t / (tiles_m * tiles_n);
    const int rr = t % (tiles_m * tiles_n);
    const int mt = rr / tiles_n, nt = rr % tiles_n;
    if (threadIdx.x == 0) {
      fence_global_async();
      // first 128-byte row of this tile's K-chunk 0 in each operand
      const int a0 = (int)(((size_t)f * sa + (size_t)mt * nkc * kABlock) / 64);
      const int b0 = (int)(((size_t)f * sb + (size_t)nt * nkc * kBBlock) / 64);
      bool bad = false;
      bool busy[kStages], loading[kStages];   // a commit / a copy not yet waited for
      for (int s = 0; s < kStages; ++s) busy[s] = loading[s] = false;
      auto wait_empty = [&](int s) {
        if (!busy[s] || bad) return;
        if (wait_phase(saddr(&sm.empty[s]), sm.empty_ph[s] & 1u)) {
          ++sm.empty_ph[s];
          busy[s] = false;
        } else {
          bad = true;
        }
      };
      auto produce = [&](int c) {
        const int s = c % kStages;
        wait_empty(s);
        if (bad) return;
        const uint32_t fb = saddr(&sm.full[s]);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(fb), "r"(kTx) : "memory");
        tensor_load(saddr(sm.st[s].a), mA, a0 + c * (int)(kABlock / 64), fb);
        tensor_load(saddr(sm.st[s].b), mB, b0 + c * (int)(kBBlock / 64), fb);
        loading[s] = true;
      };
      for (int c = 0; c < kStages - 1 && c < nkc; ++c) produce(c);
      for (int c = 0; c < nkc && !bad; ++c) {
        const int s = c % kStages;
        if (!wait_phase(saddr(&sm.full[s]), sm.full_ph[s] & 1u)) {
          bad = true;
          break;
        }
        ++sm.full_ph[s];
        loading[s] = false;
        fence_after();
        const uint32_t ahi = saddr(sm.st[s].a), alo = ahi + kM * kKC * 2u;
        const uint32_t bhi = saddr(sm.st[s].b), blo = bhi + kN * kKC * 2u;
#pragma unroll
        for (int q = 0; q < kKC / 16; ++q) {
          const uint32_t ko = (uint32_t)q * 2u * kCore;   // two K groups of 8 per MMA
          const uint32_t acc0 = (c > 0 || q > 0) ? 1u : 0u;
          mma(sm.tmem, sdesc(alo + ko), sdesc(bhi + ko), acc0);   // small terms first
          mma(sm.tmem, sdesc(ahi + ko), sdesc(blo + ko), 1u);
          mma(sm.tmem, sdesc(ahi + ko), sdesc(bhi + ko), 1u);
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                         saddr(&sm.empty[s]))
                     : "memory");
        busy[s] = true;
        // with chunk c queued on the tensor pipe, reload the stage of chunk
        // c - 1 (its MMAs finish first) with chunk c + kStages - 1
        if (c + kStages - 1 < nkc) produce(c + kStages - 1);
      }
      for (int s = 0; s < kStages; ++s) wait_empty(s);   // every MMA of the tile has completed
      if (bad) {
        sm.failed = 1;
        if (err) atomicExch(err, 1ull);
        // one more bounded wait for the copies and MMAs still in flight
        for (int s = 0; s < kStages; ++s) {
          if (loading[s]) wait_phase(saddr(&sm.full[s]), sm.full_ph[s] & 1u);
          if (busy[s]) wait_phase(saddr(&sm.empty[s]), sm.empty_ph[s] & 1u);
        }
      }
    }
    __syncthreads();
    if (sm.failed) break;
    fence_after();
    // epilogue: this warp's 32 rows x 32 columns of the tile
    const int q = warp & 3, h = warp >> 2;
    const int row = mt * kM + q * 32 + lane;
    float e = 0.f;
#pragma unroll
    for (int part = 0; part < 2; ++part) {
      uint32_t v[16];
      ld16(sm.tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(h * 32 + part * 16), v);
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (row < M) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int col = nt * kN + h * 32 + part * 16 + j;
          if (col < N) emit(out, f, row, col, M, N, __uint_as_float(v[j]), e);
        }
      }
    }
    if (out.epi == 3) eacc[f] += (double)e;
    fence_global_async();
    fence_before();
    __syncthreads();
  }
  __syncthreads();
}

// Output tiles of one pass (all four passes have the same H x W output).
__device__ __forceinline__ int pass_tiles(const Dev& d) {
  return ((d.g.Hb + kM - 1) / kM) * ((d.g.Wb + kN - 1) / kN) * d.K;
}

// One of the four GEMM passes of the spectral solve (the passes of the FP32
// form): t1 = rho Cx^T, t2 = (Cy t1) / lambda, t3 = Cy^T t2, phi = t3 Cx with
// the energy <rho, phi>.
static __device__ void dct_pass(const Dev& d, const TcMaps& tm, int step, int vb, int nvb, Smem& sm, double* eacc,
                                unsigned long long* err) {
  const int W = d.g.Wb, H = d.g.Hb;
  const long sA = (long)d.Hp128 * d.Wp32 * 2, sB = (long)d.Wp64 * d.Hp32 * 2;
  switch (step) {
    case 0: {
      const Out o{0, d.t1_t, sB, d.Hp32, nullptr, nullptr, nullptr};
      gemm(&tm.m[TM_RHO], sA, &tm.m[TM_CXB], 0, H, W, d.Wp32, d.K, o, eacc, vb, nvb, sm, err);
      break;
    }
    case 1: {
      const Out o{1, d.t2_t, sB, d.Hp32, nullptr, nullptr, d.inv_eig};
      gemm(&tm.m[TM_CYA], 0, &tm.m[TM_T1], sB, H, W, d.Hp32, d.K, o, eacc, vb, nvb, sm, err);
      break;
    }
    case 2: {
      const Out o{2, d.t3_t, sA, d.Wp32, nullptr, nullptr, nullptr};
      gemm(&tm.m[TM_CYTA], 0, &tm.m[TM_T2], sB, H, W, d.Hp32, d.K, o, eacc, vb, nvb, sm, err);
      break;
    }
    default: {
      const Out o{3, nullptr, 0, 0, d.phi, d.rho, nullptr};
      gemm(&tm.m[TM_T3], sA, &tm.m[TM_CXTB], 0, H, W, d.Wp32, d.K, o, eacc, vb, nvb, sm, err);
      break;
    }
  }
}

// The A-operand form of one mean-free density value (pass 0's input).
__device__ __forceinline__ void put_rho(const Dev& d, int f, int i, float v) {
  const int y = i / d.g.Wb, x = i % d.g.Wb;
  uint16_t h, l;
  split(v, h, l);
  const size_t base = (size_t)f * d.Hp128 * d.Wp32 * 2;
  d.rho_t[base + a_index(y, x, d.Wp32, 0)] = h;
  d.rho_t[base + a_index(y, x, d.Wp32, 1)] = l;
}
#endif  // __CUDACC__

}  // namespace tc
}  // namespace tgp
