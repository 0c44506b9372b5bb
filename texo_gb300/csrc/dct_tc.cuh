// dct_tc.cuh — the DCT GEMM passes on tcgen05 tensor cores with exact
// accumulation (bf16 integer slices).
//
// Split form. Every operand row (a row of A over K, or a row of B over K) has
// a power-of-two scale 2^e with |value| <= 2^e over the row, and each value
// is cut into four 8-bit integer slices,
//     value = 2^(e-7) (s0 + 2^-8 s1 + 2^-16 s2 + 2^-24 s3),  s_i in [-128, 128],
// each an exact bfloat16 (31 bits of the row's range in all). A product of
// two slices is an integer of at most 2^14, so a K <= 1024 sum of them is an
// integer of at most 2^24: the tensor cores' FP32 accumulation of one slice
// pair is exact. The products s_i(A) s_j(B) with i + j = L go to accumulator
// L (L = 0..3, ten products per K step; the dropped ones are below 2^-31 of
// the row ranges), and the epilogue joins the four exact accumulators in
// double-float arithmetic and applies the two row scales. This is the
// Ozaki-style generalisation of the bfloat16x3 split (Henry, Tang and
// Heinecke, ARITH 2019): the two-term split keeps about 16 bits and rounds
// in the accumulator, which leaves the field gradient 1e-3 away from FP64 on
// a 1024^2 grid; four integer slices with exact sums keep it at the level of
// the FP32 output.
//
// Passes of one spectral solve (the passes of the FP32 GEMM form):
//   t1 = rho Cx^T ; t2 = (Cy t1) / lambda ; t3 = Cy^T t2 ; phi = t3 Cx.
// The dynamic operands (rho, t1, t2, t3) are sliced by a memory-bound slice
// phase before each pass. The scale of a row needs the whole row's maximum: a
// warp per row finds it for the A operands (rho, t3); for the B operands (t1,
// t2), whose rows are the grid's columns, the previous pass's epilogue
// gathers it with atomicMax on the float bits of |x|, an order-independent
// and so deterministic reduction. Each pass's epilogue writes its result as a
// double-float pair grid. The bases are sliced once on the host from FP64.
//
// Operand layout. Sliced operands live in global memory in the exact byte
// layout the MMA reads from shared memory: the canonical K-major no-swizzle
// layout of 8-row x 16-byte core matrices (128 B between K-adjacent core
// matrices, 512 B between 8-row groups), cut into blocks of 32 K-elements.
// An A operand (rows x K) is a grid of 128 x 32 blocks, a B operand (output
// columns x K) a grid of 64 x 32 blocks; a block stores its four slices one
// after another, blocks ordered K-chunk fastest, zero-padded.
//
// One 128 x 64 output tile per block iteration, on a four-stage pipeline:
// thread 0 issues the TMA tensor copies (cp.async.bulk.tensor through the
// operands' tensor maps, complete_tx on a stage's "full" mbarrier); lane 0
// of warps 1..4 each issues the MMAs of one A slice of each chunk and a
// commit to the stage's "empty" mbarrier (four arrivals), which releases the
// stage to the next copy. The accumulators are zeroed (tcgen05.st) at the
// start of a tile and every MMA accumulates, so the issuers need no order
// among themselves: every level sum is an exact integer. The MMA issue
// limits the main loop: a 1024^2 solve takes 148 us with one issuer, 134
// with two, 124 with four. The four B slices of a block lie one after
// another in the K-major layout, so their
// first 64 (4 - i) rows read as one operand of slices 0 .. 3 - i: one MMA of
// N = 64 (4 - i) multiplies A slice i by all of them, into TMEM columns
// 64 i ..., which puts A_i B_j on accumulator i + j (columns 64 (i + j)).
// Eight MMAs of N = 256, 192, 128, 64 a chunk (two K = 16 steps x four A
// slices) instead of twenty of N = 64: an MMA costs about the same to issue
// whatever its N. The four
// accumulators occupy 4 x 64 TMEM columns (row i = lane i); the epilogue
// reads them with tcgen05.ld, warp w taking lanes 32 (w mod 4) ... + 31 and
// columns 32 (w / 4) ... + 31, and turns them through shared memory for
// row-wise global accesses.
//
// Every wait is bounded. When one runs out the block records it (shared
// `failed` and the caller's error word), waits once more (bounded) for its
// own copies and MMAs, frees its tensor memory and leaves its tiles undone.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>

#include "common.cuh"

namespace tgp {
namespace tc {

constexpr int kM = 128;                        // accumulator rows (TMEM lanes)
constexpr int kN = 64;                         // accumulator columns per tile
constexpr int kKC = 32;                        // K per block / pipeline stage
constexpr int kStages = 4;                     // chunks in flight (TMA prefetch depth)
constexpr int kSlices = 4;                     // 8-bit integer slices per value
constexpr int kLevels = 4;                     // accumulators: slice pairs with i + j = level
constexpr uint32_t kCols = kLevels * kN;       // TMEM columns per block: accumulator L at kN L
static_assert(kSlices == kLevels, "A slice i meets B slices 0 .. kLevels - 1 - i");
constexpr uint32_t kCore = 128;                // one 8 x 16 B core matrix
constexpr uint32_t kSbo = (kKC / 8) * kCore;   // next 8-row group
constexpr uint32_t kLbo = kCore;               // next 8-element K group
constexpr uint32_t kASlice = (uint32_t)kM * kKC;    // elements of one slice of an A block
constexpr uint32_t kBSlice = (uint32_t)kN * kKC;
constexpr uint32_t kABlock = kSlices * kASlice;     // elements of one A block (all slices)
constexpr uint32_t kBBlock = kSlices * kBSlice;
constexpr uint32_t kTx = (kABlock + kBBlock) * 2u;  // bytes per stage
constexpr unsigned kWaitLimit = 1u << 22;      // mbarrier polls before giving up
constexpr int kIssuers = 4;                    // MMA-issuing threads: lane 0 of warps 1 .. kIssuers
// kind::f16 instruction descriptor: D = F32, A = B = BF16, both K-major, N, M.
__host__ __device__ constexpr uint32_t idesc(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kM >> 4) << 24);
}

// TMA descriptors of the sliced operands, each a 2-D view of one operand
// buffer as rows of 128 bytes (64 bf16 values): an A block is a 64 x 256 box
// (32 KB), a B block a 64 x 128 box (16 KB). The data are already in the
// MMA's shared-memory layout, so the copies use no swizzle.
enum TcMap { TM_OPA = 0, TM_OPB, TM_CXB, TM_CYA, TM_CYTA, TM_CXTB, TM_COUNT };
struct TcMaps {   // aligned as CUtensorMap requires
  CUtensorMap m[TM_COUNT];
};

// ---- layout (host and device) ------------------------------------------------
__host__ __device__ inline uint32_t kmaj(int r, int k) {
  return (uint32_t)(r >> 3) * kSbo + (uint32_t)(k >> 3) * kCore + (uint32_t)(r & 7) * 16u + (uint32_t)(k & 7) * 2u;
}
__host__ __device__ inline int pad(int n, int m) { return (n + m - 1) / m * m; }
// element index of (row r, k) slice s in an A operand with K padded to kp
__host__ __device__ inline size_t a_index(int r, int k, int kp, int s) {
  const size_t blk = ((size_t)(r >> 7) * (size_t)(kp >> 5) + (size_t)(k >> 5)) * kABlock;
  return blk + (size_t)s * kASlice + kmaj(r & 127, k & 31) / 2;
}
// element index of (output column n, k) slice s in a B operand
__host__ __device__ inline size_t b_index(int n, int k, int kp, int s) {
  const size_t blk = ((size_t)(n / kN) * (size_t)(kp >> 5) + (size_t)(k >> 5)) * kBBlock;
  return blk + (size_t)s * kBSlice + kmaj(n % kN, k & 31) / 2;
}
// Operand sizes in elements (all fields).
__host__ __device__ inline size_t a_elems(int rows, int k, int fields) {
  return (size_t)pad(rows, kM) * pad(k, kKC) * kSlices * fields;
}
__host__ __device__ inline size_t b_elems(int cols, int k, int fields) {
  return (size_t)pad(cols, kN) * pad(k, kKC) * kSlices * fields;
}

// Row scale: the exponent e with max|row| <= 2^e (0 for an all-zero row).
inline int row_exponent_host(double mx) {
  if (!(mx > 0.0)) return 0;
  int e = 0;
  std::frexp(mx, &e);   // mx = m 2^e, m in [0.5, 1)
  return e;
}
// bfloat16 bits of an integer of magnitude <= 256 (exact: <= 8 significant bits)
inline uint16_t int_bf16_host(double s) {
  const float f = (float)s;
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return (uint16_t)(u >> 16);
}
// The four slices of an FP64 value at row exponent e (host: the bases).
inline void slice_host(double v, int e, uint16_t out[kSlices]) {
  double x = std::ldexp(v, 7 - e);
  for (int i = 0; i < kSlices; ++i) {
    const double s = std::nearbyint(x);
    out[i] = int_bf16_host(s);
    x = (x - s) * 256.0;
  }
}

#ifdef __CUDACC__
__device__ __forceinline__ float pow2f(int e) {
  return (e >= -126 && e <= 127) ? __int_as_float((e + 127) << 23) : ldexpf(1.0f, e);
}
__device__ __forceinline__ int row_exponent(unsigned max_bits) {
  const float m = __uint_as_float(max_bits);
  if (!(m > 0.f)) return 0;
  int e = 0;
  frexpf(m, &e);
  return e;
}
__device__ __forceinline__ uint16_t int_bf16(float s) { return __bfloat16_as_ushort(__float2bfloat16_rn(s)); }
// The four slices of the double-float value hi + lo at row exponent e, as
// bf16 bits: 2^(7-e)(hi + lo) = s0 + 2^-8 s1 + 2^-16 s2 + 2^-24 s3 + O(2^-25).
// x - rint(x) is exact; adding the scaled lo rounds below the last slice.
__device__ __forceinline__ void slice_pair(float hi, float lo, float scale, uint16_t s[kSlices]) {
  const float x = hi * scale;
  const float s0 = rintf(x);
  float r = (x - s0) + lo * scale;
  s[0] = int_bf16(s0);
#pragma unroll
  for (int i = 1; i < kSlices; ++i) {
    r *= 256.f;
    const float si = rintf(r);
    r -= si;
    s[i] = int_bf16(si);
  }
}
// Error-free sum of two floats (Knuth).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

struct alignas(128) Stage {
  uint16_t a[kABlock];
  uint16_t b[kBBlock];
};
struct alignas(128) Smem {
  Stage st[kStages];
  unsigned long long full[kStages], empty[kStages];
  unsigned long long done;   // every MMA of the tile has completed
  uint32_t tmem;
  uint32_t issued, consumed[kIssuers];   // chunks copied / taken by each MMA issuer (cleanup after a failure)
  int failed;
};
// The epilogue stages each warp's 32 rows x kN/2 columns of (hi, lo) pairs
// in the pipeline's shared memory (free once the tile's MMAs completed) to
// write and read global memory a row at a time.
constexpr int kEpiCols = kN / 2;
constexpr int kEpiStride = kEpiCols + 1;   // pairs per staged row (conflict-free both ways)
static_assert(8 * 32 * kEpiStride * 8 <= (int)(kStages * sizeof(Stage)), "epilogue staging fits the stages");

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t sdesc(uint32_t a) {
  return (uint64_t)((a & 0x3FFFFu) >> 4) | ((uint64_t)(kLbo >> 4) << 16) | ((uint64_t)(kSbo >> 4) << 32) |
         (1ull << 46);
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy global writes ordered with later TMA (async-proxy) reads
__device__ __forceinline__ void fence_global_async() { asm volatile("fence.proxy.async.global;" ::: "memory"); }

// One MMA (M = 128, K = 16, N in the descriptor), accumulating into D when acc != 0.
__device__ __forceinline__ void mma(uint32_t d, uint64_t a, uint64_t b, uint32_t id, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(id), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}
// generic-proxy shared-memory accesses ordered with later TMA writes
__device__ __forceinline__ void fence_shared_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

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
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(&sm.empty[i])), "r"(kIssuers) : "memory");
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(&sm.done)), "r"(kIssuers) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    sm.failed = 0;
    sm.issued = 0;
    for (int k = 0; k < kIssuers; ++k) sm.consumed[k] = 0;
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
// Zeroes 16 columns of this warp's 32 TMEM lanes.
__device__ __forceinline__ void st16_zero(uint32_t taddr) {
  const uint32_t z = 0;
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, "
      "%1};\n" ::"r"(taddr),
      "r"(z)
      : "memory");
}

// Where a pass puts its result: the double-float pair grid (epi 0 and 2,
// epi 1 after the inverse-eigenvalue scaling), with the column maxima the
// next slice phase needs for epi 0 and 1 (a B operand's rows are the grid's
// columns), or the FP32 potential with the energy <rho, phi> (epi 3).
struct Out {
  float2* tp;            // [K][M][N] pair grid (epi 0..2)
  unsigned* mx;          // column maxima [K][N] for the next B operand (epi 0, 1)
  float* phi;            // epi 3
  const float* rho;      // epi 3 (FP32 mean-free density)
  const float* ie_hi;    // epi 1: 1 / lambda as a double-float pair
  const float* ie_lo;
  const int* eA;         // row exponents of A and B (per field stride sa_e / sb_e; 0 = shared)
  const int* eB;
  int sa_e, sb_e;
};

// C[f] = A[f] (M x K) * B[f]^T, B given as N x K, both sliced; output tiles
// t = vb, vb + nvb, ... of 128 x 64, written by `out`. kp = K padded to 32.
// The block must have called setup(); blockDim.x must be 256.
//
// Thread 0 copies K-chunks into the stages, each copy waiting for the MMAs
// that last read its stage (the stage's "empty" commits); the issuers issue
// their MMAs of each chunk once its copy landed ("full") and commit them to
// the stage's "empty" barrier without waiting, so the tensor pipe keeps up
// to kStages chunks queued. Chunk counters run on across the block's tiles,
// so the k-th use of a stage waits for the (k-1)-th release. After the last
// chunk each issuer commits to "done" and waits for it; then the block runs
// the epilogue: each warp moves its 32 x 32 accumulator block from tensor
// memory (lane = row) through shared memory (lane = column), so that every
// global load and store of the epilogue covers a row segment.
template <int EPI>
static __device__ void gemm(const CUtensorMap* mA, long sa, const CUtensorMap* mB, long sb, int M, int N, int kp,
                            int nf, const Out& out, double* eacc, int vb, int nvb, Smem& sm, unsigned long long* err) {
  const int tiles_m = (M + kM - 1) / kM, tiles_n = (N + kN - 1) / kN;
  const int tiles = tiles_m * tiles_n * nf;
  const int nkc = kp / kKC;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  volatile int* failed = &sm.failed;
  auto fail = [&]() {
    *failed = 1;
    if (err) atomicExch(err, 1ull);
  };
  uint32_t gp = 0, gm = 0, done_ph = 0;   // thread 0's copies, thread 32's chunks and tiles
  __syncthreads();
  for (int t = vb; t < tiles; t += nvb) {
    if (*failed) break;
    const int f = t / (tiles_m * tiles_n);
    const int rr = t % (tiles_m * tiles_n);
    const int mt = rr / tiles_n, nt = rr % tiles_n;
    {
      // the accumulators start at zero, so that the two issuers' MMAs all
      // accumulate (their order is free: every sum is an exact integer)
      const uint32_t lanes = (uint32_t)((warp & 3) * 32) << 16;
#pragma unroll
      for (int part = 0; part < (int)kCols / 2 / 16; ++part)
        st16_zero(sm.tmem + lanes + (uint32_t)((warp >> 2) * (kCols / 2) + part * 16));
      asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
      fence_before();
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      fence_global_async();
      fence_shared_async();
      // first 128-byte row of this tile's K-chunk 0 in each operand
      const int a0 = (int)(((size_t)f * sa + (size_t)mt * nkc * kABlock) / 64);
      const int b0 = (int)(((size_t)f * sb + (size_t)nt * nkc * kBBlock) / 64);
      for (int c = 0; c < nkc; ++c) {
        if (*failed) break;
        const uint32_t s = gp % kStages;
        if (gp >= (uint32_t)kStages && !wait_phase(saddr(&sm.empty[s]), (gp / kStages - 1) & 1u)) {
          fail();
          break;
        }
        const uint32_t fb = saddr(&sm.full[s]);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(fb), "r"(kTx) : "memory");
        tensor_load(saddr(sm.st[s].a), mA, a0 + c * (int)(kABlock / 64), fb);
        tensor_load(saddr(sm.st[s].b), mB, b0 + c * (int)(kBBlock / 64), fb);
        ++gp;
      }
      sm.issued = gp;
    } else if ((threadIdx.x & 31) == 0 && threadIdx.x >= 32 && threadIdx.x <= 32 * kIssuers) {
      // issuer k takes A slices kSlices / kIssuers * k ... of every K step
      const int k = (int)(threadIdx.x >> 5) - 1;
      for (int c = 0; c < nkc; ++c) {
        if (*failed) break;
        const uint32_t s = gm % kStages;
        if (!wait_phase(saddr(&sm.full[s]), (gm / kStages) & 1u)) {
          fail();
          break;
        }
        ++gm;
        fence_after();
        const uint32_t abase = saddr(sm.st[s].a), bbase = saddr(sm.st[s].b);
#pragma unroll
        for (int q = 0; q < kKC / 16; ++q) {
          const uint32_t ko = (uint32_t)q * 2u * kCore;   // two K groups of 8 per MMA
          const uint64_t bd = sdesc(bbase + ko);          // B slices 0..3 as 4 kN rows
#pragma unroll
          for (int ii = 0; ii < kSlices / kIssuers; ++ii) {
            // A slice i times B slices 0 .. 3 - i (the first kN (4 - i) rows)
            // into columns kN i ...: A_i B_j lands on accumulator i + j
            const int i = kSlices / kIssuers * k + ii;
            mma(sm.tmem + (uint32_t)(i * kN), sdesc(abase + i * kASlice * 2u + ko), bd, idesc(kN * (kLevels - i)),
                1u);
          }
        }
        commit(saddr(&sm.empty[s]));
      }
      // every MMA issued so far (a failure included) completes before the
      // epilogue or the teardown touches tensor memory
      commit(saddr(&sm.done));
      if (!wait_phase(saddr(&sm.done), done_ph & 1u)) fail();
      ++done_ph;
      sm.consumed[k] = gm;
      fence_before();
    }
    __syncthreads();
    if (*failed) {
      // one more bounded wait for the copies still in flight (from the
      // fewest chunks any issuer took)
      if (threadIdx.x == 0)
        for (int k = 1; k < kIssuers; ++k) sm.consumed[0] = min(sm.consumed[0], sm.consumed[k]);
      if (threadIdx.x == 0)
        for (uint32_t g = sm.consumed[0]; g < sm.issued; ++g)
          wait_phase(saddr(&sm.full[g % kStages]), (g / kStages) & 1u);
      break;
    }
    fence_after();
    // epilogue. This warp's block: 32 rows (TMEM lanes 32 q ...) x 32 columns
    // (h). Its global inputs (epi 1: 1 / lambda pairs, epi 3: rho), one row
    // per step with lane = column, are loaded first, so that their latency
    // overlaps the accumulators' staging.
    const int q = warp & 3, h = warp >> 2;
    const int rows = min(32, M - (mt * kM + q * 32));
    const int col = nt * kN + h * kEpiCols + lane;
    const bool col_ok = col < N;
    float in0[32], in1[32];
#pragma unroll
    for (int r = 0; r < 32; ++r) {
      in0[r] = in1[r] = 0.f;
      if (r < rows && col_ok) {
        const size_t idx = (size_t)(mt * kM + q * 32 + r) * N + col;
        if constexpr (EPI == 3) {
          in0[r] = out.rho[(size_t)f * M * N + idx];
        } else if constexpr (EPI == 1) {
          in0[r] = out.ie_hi[idx];
          in1[r] = out.ie_lo[idx];
        }
      }
    }
    // first half: lane = row, the four accumulators joined and scaled by
    // the row, into this warp's staging rows
    float2* stage = reinterpret_cast<float2*>(&sm.st[0]) + (size_t)warp * 32 * kEpiStride;
    {
      const int row = mt * kM + q * 32 + lane;
      const float row_scale = pow2f((row < M ? out.eA[(size_t)f * out.sa_e + row] : 0) - 14);
#pragma unroll
      for (int part = 0; part < kEpiCols / 16; ++part) {
        uint32_t v[kLevels][16];
#pragma unroll
        for (int L = 0; L < kLevels; ++L)
          ld16(sm.tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(L * kN + h * kEpiCols + part * 16), v[L]);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          // join the exact level sums: a0 + 2^-8 a1 + 2^-16 a2 + 2^-24 a3
          float s, r;
          two_sum(__uint_as_float(v[0][j]), __uint_as_float(v[1][j]) * 0x1p-8f, s, r);
          r += __uint_as_float(v[2][j]) * 0x1p-16f;
          r += __uint_as_float(v[3][j]) * 0x1p-24f;
          float hi, lo;
          two_sum(s, r, hi, lo);
          stage[lane * kEpiStride + part * 16 + j] = make_float2(hi * row_scale, lo * row_scale);
        }
      }
    }
    __syncwarp();
    // second half: lane = column, a row of the warp's block per step
    float e = 0.f;
    if (col_ok) {
      const float col_scale = pow2f(out.eB[(size_t)f * out.sb_e + col]);
      unsigned cmax = 0;
#pragma unroll
      for (int r = 0; r < 32; ++r) {
        if (r >= rows) break;
        const size_t idx = (size_t)(mt * kM + q * 32 + r) * N + col;
        const float2 pr = stage[r * kEpiStride + lane];
        float hi = pr.x * col_scale, lo = pr.y * col_scale;
        if constexpr (EPI == 3) {
          const float p = hi + lo;
          out.phi[(size_t)f * M * N + idx] = p;
          e = fmaf(in0[r], p, e);
        } else {
          if constexpr (EPI == 1) {   // (hi + lo)(ie_hi + ie_lo) in double-float
            const float ih = in0[r], il = in1[r];
            const float p = hi * ih;
            float pe = fmaf(hi, ih, -p);
            pe = fmaf(hi, il, fmaf(lo, ih, pe));
            two_sum(p, pe, hi, lo);
          }
          out.tp[(size_t)f * M * N + idx] = make_float2(hi, lo);
          cmax = max(cmax, __float_as_uint(fabsf(hi)));
        }
      }
      // column maxima: one atomic per column and warp
      if constexpr (EPI == 0 || EPI == 1)
        if (cmax) atomicMax(out.mx + (size_t)f * N + col, cmax);
    }
    if constexpr (EPI == 3) eacc[f] += (double)e;
    fence_shared_async();   // the staging writes before the next tile's copies
    fence_before();
    __syncthreads();
  }
  __syncthreads();
}

// Output tiles of one pass (all four passes have the same H x W output).
__host__ __device__ __forceinline__ int pass_tiles_host(const Dev& d) {
  return ((d.g.Hb + kM - 1) / kM) * ((d.g.Wb + kN - 1) / kN) * d.K;
}

// Column-maximum words of t1 (which = 0) and t2 (which = 1): [2][K][Wb].
__device__ __forceinline__ unsigned* tmx_of(const Dev& d, int which) {
  return d.tmx + (size_t)which * d.K * d.g.Wb;
}

// One of the four GEMM passes of the spectral solve.
// Each pass is its own kernel instance (STEP = the pass), so that an
// instance holds only its own epilogue's code.
template <int STEP>
static __device__ void dct_pass(const Dev& d, const TcMaps& tm, int vb, int nvb, Smem& sm, double* eacc,
                                unsigned long long* err) {
  const int W = d.g.Wb, H = d.g.Hb;
  const long sA = (long)a_elems(H, W, 1), sB = (long)b_elems(W, H, 1);
  Out o{};
  o.tp = d.tp;
  o.ie_hi = d.inv_eig;
  o.ie_lo = d.inv_eig_lo;
  if constexpr (STEP == 0) {   // t1 = rho Cx^T: A = rho (rows y), B = rows of Cx (frequency kx)
    o.mx = tmx_of(d, 0);
    o.eA = d.eA, o.sa_e = d.Hp128;
    o.eB = d.eCx, o.sb_e = 0;
    gemm<0>(&tm.m[TM_OPA], sA, &tm.m[TM_CXB], 0, H, W, d.Wp32, d.K, o, eacc, vb, nvb, sm, err);
  } else if constexpr (STEP == 1) {   // t2 = (Cy t1) / lambda: A = rows of Cy (ky), B = t1 columns (kx)
    o.mx = tmx_of(d, 1);
    o.eA = d.eCy, o.sa_e = 0;
    o.eB = d.eB, o.sb_e = d.Wp64;
    gemm<1>(&tm.m[TM_CYA], 0, &tm.m[TM_OPB], sB, H, W, d.Hp32, d.K, o, eacc, vb, nvb, sm, err);
  } else if constexpr (STEP == 2) {   // t3 = Cy^T t2: A = rows of Cy^T (y), B = t2 columns (kx)
    o.eA = d.eCy + d.g.Hb, o.sa_e = 0;
    o.eB = d.eB, o.sb_e = d.Wp64;
    gemm<2>(&tm.m[TM_CYTA], 0, &tm.m[TM_OPB], sB, H, W, d.Hp32, d.K, o, eacc, vb, nvb, sm, err);
  } else {   // phi = t3 Cx: A = t3 (rows y), B = rows of Cx^T (x)
    o.phi = d.phi;
    o.rho = d.rho;
    o.eA = d.eA, o.sa_e = d.Hp128;
    o.eB = d.eCx + d.g.Wb, o.sb_e = 0;
    gemm<3>(&tm.m[TM_OPA], sA, &tm.m[TM_CXTB], 0, H, W, d.Wp32, d.K, o, eacc, vb, nvb, sm, err);
  }
}

// The slice phase before GEMM pass `step`: the dynamic operand of the pass
// from its FP32 / pair grid. An A operand (rho before pass 0, t3 before pass
// 3; rows y over K = x) takes 128 threads per row, which find the row's
// maximum themselves (blockDim.x must be 256); a B operand (t1 before pass 1, t2 before pass 2; rows kx over K =
// y) takes its column maxima from the previous pass's epilogue. Before pass
// 0 it clears the t1 maxima and before pass 1 the t2 maxima (both last read
// one solve ago), so each is empty when its pass gathers into it.
static __device__ void slice_phase(const Dev& d, int step, int vb, int nvb) {
  const int W = d.g.Wb, H = d.g.Hb, K = d.K;
  const int lane = threadIdx.x & 31;
  if (step == 0 || step == 1) {
    unsigned* z = tmx_of(d, step);
    for (int i = vb * blockDim.x + threadIdx.x; i < K * W; i += nvb * blockDim.x) z[i] = 0u;
  }
  if (step == 0 || step == 3) {
    // A operand: a row per 128 threads (two rows a block), each thread one
    // group of 8 consecutive x (more past 1024 columns), read once for the
    // row's maximum and again, from L1, for the slices
    __shared__ unsigned red[2][4];
    const int slot = threadIdx.x >> 7, t = threadIdx.x & 127;
    const int ng = d.Wp32 / 8;
    const size_t fs = a_elems(H, W, 1);
    for (int base = vb * 2; base < K * H; base += nvb * 2) {   // the same trips for the whole block
      const int rw = base + slot;
      const bool ok = rw < K * H;
      const int f = ok ? rw / H : 0, y = ok ? rw % H : 0;
      const float* rrow = d.rho + (size_t)f * d.B + (size_t)y * W;
      const float2* prow = d.tp + (size_t)f * d.B + (size_t)y * W;
      unsigned m = 0;
      if (ok)
        for (int g = t; g < ng; g += 128)
#pragma unroll
          for (int k = 0; k < 8; ++k) {
            const int x = g * 8 + k;
            if (x < W) m = max(m, __float_as_uint(fabsf(step == 0 ? rrow[x] : prow[x].x)));
          }
      m = __reduce_max_sync(0xffffffffu, m);
      if ((t & 31) == 0) red[slot][t >> 5] = m;
      __syncthreads();
      m = max(max(red[slot][0], red[slot][1]), max(red[slot][2], red[slot][3]));
      __syncthreads();   // the next row pair rewrites red
      if (!ok) continue;
      const int e = row_exponent(m);
      if (t == 0) d.eA[(size_t)f * d.Hp128 + y] = e;
      const float sc = pow2f(7 - e);
      uint16_t* dst = d.opA + (size_t)f * fs;
      for (int g = t; g < ng; g += 128) {
        uint16_t sl[kSlices][8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          const int x = g * 8 + k;
          float hi = 0.f, lo = 0.f;
          if (x < W) {
            if (step == 0) {
              hi = rrow[x];
            } else {
              const float2 p = prow[x];
              hi = p.x;
              lo = p.y;
            }
          }
          uint16_t s[kSlices];
          slice_pair(hi, lo, sc, s);
#pragma unroll
          for (int i = 0; i < kSlices; ++i) sl[i][k] = s[i];
        }
#pragma unroll
        for (int i = 0; i < kSlices; ++i) {
          uint4 w;
          w.x = (uint32_t)sl[i][0] | ((uint32_t)sl[i][1] << 16);
          w.y = (uint32_t)sl[i][2] | ((uint32_t)sl[i][3] << 16);
          w.z = (uint32_t)sl[i][4] | ((uint32_t)sl[i][5] << 16);
          w.w = (uint32_t)sl[i][6] | ((uint32_t)sl[i][7] << 16);
          *reinterpret_cast<uint4*>(dst + a_index(y, g * 8, d.Wp32, i)) = w;
        }
      }
    }
  } else {
    // B operand: groups of 8 consecutive y of one column, consecutive
    // threads on consecutive columns (coalesced reads of the pair rows)
    const unsigned* mx = tmx_of(d, step - 1);
    const int ng = d.Hp32 / 8;
    const size_t fs = b_elems(W, H, 1);
    for (int it = vb * blockDim.x + threadIdx.x; it < K * ng * W; it += nvb * blockDim.x) {
      const int f = it / (ng * W), rem = it % (ng * W), g = rem / W, n = rem % W;
      const int e = row_exponent(mx[(size_t)f * W + n]);
      if (g == 0) d.eB[(size_t)f * d.Wp64 + n] = e;
      const float sc = pow2f(7 - e);
      uint16_t sl[kSlices][8];
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const int y = g * 8 + k;
        float2 p = make_float2(0.f, 0.f);
        if (y < H) p = d.tp[(size_t)f * d.B + (size_t)y * W + n];
        uint16_t s[kSlices];
        slice_pair(p.x, p.y, sc, s);
#pragma unroll
        for (int i = 0; i < kSlices; ++i) sl[i][k] = s[i];
      }
      uint16_t* dst = d.opB + (size_t)f * fs;
#pragma unroll
      for (int i = 0; i < kSlices; ++i) {
        uint4 w;
        w.x = (uint32_t)sl[i][0] | ((uint32_t)sl[i][1] << 16);
        w.y = (uint32_t)sl[i][2] | ((uint32_t)sl[i][3] << 16);
        w.z = (uint32_t)sl[i][4] | ((uint32_t)sl[i][5] << 16);
        w.w = (uint32_t)sl[i][6] | ((uint32_t)sl[i][7] << 16);
        *reinterpret_cast<uint4*>(dst + b_index(n, g * 8, d.Hp32, i)) = w;
      }
    }
  }
}
#endif  // __CUDACC__

}  // namespace tc
}  // namespace tgp
