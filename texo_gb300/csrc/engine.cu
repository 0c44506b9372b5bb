// engine.cu — device buffers of one instance, the host-driven controller and
// the C ABI entry points of include/texo_gp.h.
//
// The controller restates, on device buffers, the reference's
//   optimize_density_once          (crates/texo-pnr/src/eplace.rs:439-582)
//   dynamic_nesterov_step          (crates/texo-pnr/src/global_placement.rs:121-335)
// Every vector operation and reduction runs on the GPU; the host reads back a
// small scalar block once per objective evaluation.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <limits>
#include <map>
#include <tuple>

#include <cuda_bf16.h>
#include <memory>
#include <mutex>
#include <string>

#include "engine.h"
#include "dct_tc.cuh"
#include "scatter_tiles.cuh"

namespace tgp {

static thread_local std::string g_last_error;
void set_last_error(const std::string& s) { g_last_error = s; }

#define CU(call)                                                                           \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess) {                                                               \
      set_last_error(std::string(#call) + ": " + cudaGetErrorString(e_));                  \
      return e_ == cudaErrorMemoryAllocation ? TEXO_GP_ERR_OUT_OF_MEMORY : TEXO_GP_ERR_CUDA; \
    }                                                                                      \
  } while (0)
#define TRY(call)                \
  do {                           \
    int32_t s_ = (call);         \
    if (s_ != TEXO_GP_OK) return s_; \
  } while (0)

void release_mirror(RunBlock* run);

Instance::~Instance() {
  if (stream) cudaStreamSynchronize(stream);
  for (void* p : allocations) cudaFreeAsync(p, stream);
  if (stream) {
    cudaStreamSynchronize(stream);
    cudaStreamDestroy(stream);
  }
  release_mirror(h_run);
}

// Device buffers come from the device's stream-ordered pool (kept, not
// trimmed, between instances): admitting and retiring many short-lived
// placements then reuses pooled memory instead of a driver allocation, and
// its implicit synchronization, per buffer.
int32_t Instance::alloc(void** p, size_t n) {
  n = ((n ? n : 16) + 255) & ~(size_t)255;
  CU(cudaMallocAsync(p, n, stream));
  allocations.push_back(*p);
  bytes += n;
  return TEXO_GP_OK;
}

namespace {
// The default pool of a device keeps freed memory for reuse (once per device).
cudaError_t keep_pool(int device) {
  static std::mutex mu;
  static std::vector<int> done;
  std::lock_guard<std::mutex> lk(mu);
  if (std::find(done.begin(), done.end(), device) != done.end()) return cudaSuccess;
  cudaMemPool_t pool;
  cudaError_t e = cudaDeviceGetDefaultMemPool(&pool, device);
  if (e != cudaSuccess) return e;
  uint64_t keep = ~0ull;
  e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  if (e == cudaSuccess) done.push_back(device);
  return e;
}
// Host FP64 coordinates -> device FP32 optimizer buffer.
int32_t upload_coords(Instance& I, float2* dst, const double* src, size_t nobj) {
  std::vector<float> tmp(2 * nobj);
  for (size_t i = 0; i < 2 * nobj; ++i) tmp[i] = (float)src[i];
  CU(cudaMemcpyAsync(dst, tmp.data(), nobj * sizeof(float2), cudaMemcpyHostToDevice, I.stream));
  CU(cudaStreamSynchronize(I.stream));
  return TEXO_GP_OK;
}
std::vector<double> dct_basis(uint32_t n) {
  const double nf = (double)n;
  std::vector<double> b((size_t)n * n);
  for (uint32_t f = 0; f < n; ++f) {
    const double s = f == 0 ? std::sqrt(1.0 / nf) : std::sqrt(2.0 / nf);
    for (uint32_t c = 0; c < n; ++c) b[(size_t)f * n + c] = s * std::cos(3.14159265358979323846 * f * (c + 0.5) / nf);
  }
  return b;
}

// Spectral tables of a bin grid (DCT basis and its transpose per axis, the
// inverse Laplacian eigenvalues), read-only and identical for every
// instance with the same grid: built once per device and size and shared.
struct SpectralTables {
  float *Cx = nullptr, *CxT = nullptr, *Cy = nullptr, *CyT = nullptr, *inv_eig = nullptr;
};
struct BasisTables {
  float *c = nullptr, *ct = nullptr;   // FP32 C and C^T, row-major n x n
  // tensor-core operands (dct_tc.cuh layout, four integer slices of the FP64
  // values): C and C^T as B operands (rows padded to 64) and as A operands
  // (rows padded to 128), K padded to 32; `e` the row exponents, [n] for the
  // rows of C then [n] for the rows of C^T
  uint16_t *cB = nullptr, *ctB = nullptr, *cA = nullptr, *ctA = nullptr;
  int* e = nullptr;
};
cudaError_t shared_basis(int device, uint32_t n, BasisTables* out) {
  static std::mutex mu;
  static std::map<std::pair<int, uint32_t>, BasisTables> cache;
  std::lock_guard<std::mutex> lk(mu);
  auto it = cache.find({device, n});
  if (it == cache.end()) {
    const auto b = dct_basis(n);
    const size_t nn = (size_t)n * n;
    const int N = (int)n, kp = tc::pad(N, tc::kKC);
    std::vector<float> m(nn), mt(nn);
    std::vector<uint16_t> cB(tc::b_elems(N, N, 1), 0), ctB(cB.size(), 0);
    std::vector<uint16_t> cA(tc::a_elems(N, N, 1), 0), ctA(cA.size(), 0);
    std::vector<int> e(2 * (size_t)n, 0);
    std::vector<double> rmax(n, 0.0), cmax(n, 0.0);
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j) {
        const double v = std::fabs(b[(size_t)i * n + j]);
        rmax[i] = std::max(rmax[i], v);
        cmax[j] = std::max(cmax[j], v);
      }
    for (int i = 0; i < N; ++i) {
      e[i] = tc::row_exponent_host(rmax[i]);
      e[n + i] = tc::row_exponent_host(cmax[i]);
    }
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j) {
        const double v = b[(size_t)i * n + j];   // C[i][j] = C^T[j][i]
        m[(size_t)i * n + j] = (float)v;
        mt[(size_t)j * n + i] = (float)v;
        uint16_t sr[tc::kSlices], sc[tc::kSlices];
        tc::slice_host(v, e[i], sr);       // in row i of C
        tc::slice_host(v, e[n + j], sc);   // in row j of C^T
        for (int s = 0; s < tc::kSlices; ++s) {
          cB[tc::b_index(i, j, kp, s)] = sr[s];
          cA[tc::a_index(i, j, kp, s)] = sr[s];
          ctB[tc::b_index(j, i, kp, s)] = sc[s];
          ctA[tc::a_index(j, i, kp, s)] = sc[s];
        }
      }
    BasisTables t;
    cudaError_t err = cudaSuccess;
    auto up = [&](auto** dst, const auto& v) {
      if (err != cudaSuccess) return;
      err = cudaMalloc((void**)dst, v.size() * sizeof(v[0]));
      if (err == cudaSuccess) err = cudaMemcpy(*dst, v.data(), v.size() * sizeof(v[0]), cudaMemcpyHostToDevice);
    };
    up(&t.c, m);
    up(&t.ct, mt);
    up(&t.cB, cB);
    up(&t.ctB, ctB);
    up(&t.cA, cA);
    up(&t.ctA, ctA);
    up(&t.e, e);
    if (err != cudaSuccess) return err;
    it = cache.emplace(std::make_pair(device, n), t).first;
  }
  *out = it->second;
  return cudaSuccess;
}
// Twiddle tables of the FFT form for one power-of-two length n (FP64 values
// rounded to FP32): tw[n/2] = exp(-2 pi i j / n), post[n] = s_k exp(-i pi k /
// 2n), pre[n] = exp(-i pi k / 2n), inv_s[n] = 1 / s_k.
// FFT tables of one length as double-float pairs: an FP64 value x becomes
// hi = (float)x, lo = (float)(x - hi), so hi + lo carries about 48 bits.
struct FftTables {
  float4 *tw = nullptr, *post = nullptr, *pre = nullptr;   // (re.hi, im.hi, re.lo, im.lo)
  float2* inv_s = nullptr;                                  // (hi, lo)
};
static float2 split_df(double x) {
  const float hi = (float)x;
  return make_float2(hi, (float)(x - (double)hi));
}
static float4 split_cdf(double re, double im) {
  const float2 r = split_df(re), i = split_df(im);
  return make_float4(r.x, i.x, r.y, i.y);
}
cudaError_t shared_fft(int device, uint32_t n, FftTables* out) {
  static std::mutex mu;
  static std::map<std::pair<int, uint32_t>, FftTables> cache;
  std::lock_guard<std::mutex> lk(mu);
  auto it = cache.find({device, n});
  if (it == cache.end()) {
    const double pi = 3.14159265358979323846, nf = (double)n;
    std::vector<float4> tw(n / 2), post(n), pre(n);
    std::vector<float2> inv_s(n);
    for (uint32_t j = 0; j < n / 2; ++j) tw[j] = split_cdf(std::cos(-2.0 * pi * j / nf), std::sin(-2.0 * pi * j / nf));
    for (uint32_t k = 0; k < n; ++k) {
      const double sk = k == 0 ? std::sqrt(1.0 / nf) : std::sqrt(2.0 / nf);
      const double c = std::cos(-pi * k / (2.0 * nf)), sn = std::sin(-pi * k / (2.0 * nf));
      post[k] = split_cdf(sk * c, sk * sn);
      pre[k] = split_cdf(c, sn);
      inv_s[k] = split_df(1.0 / sk);
    }
    FftTables t;
    cudaError_t e = cudaSuccess;
    auto up = [&](auto** dst, const auto& v) {
      if (e != cudaSuccess) return;
      e = cudaMalloc((void**)dst, std::max<size_t>(v.size(), 1) * sizeof(v[0]));
      if (e == cudaSuccess && !v.empty())
        e = cudaMemcpy(*dst, v.data(), v.size() * sizeof(v[0]), cudaMemcpyHostToDevice);
    };
    up(&t.tw, tw);
    up(&t.post, post);
    up(&t.pre, pre);
    up(&t.inv_s, inv_s);
    if (e != cudaSuccess) return e;
    it = cache.emplace(std::make_pair(device, n), t).first;
  }
  *out = it->second;
  return cudaSuccess;
}
// lengths the FFT form takes: powers of two whose group data fits its buffer
bool fft_length(uint32_t n) { return n >= 2 && n <= 1024 && (n & (n - 1)) == 0; }
int ilog2(uint32_t n) {
  int l = 0;
  while ((1u << l) < n) ++l;
  return l;
}

cudaError_t shared_inv_eig(int device, uint32_t Wb, uint32_t Hb, float** out) {
  static std::mutex mu;
  static std::map<std::tuple<int, uint32_t, uint32_t>, float*> cache;
  std::lock_guard<std::mutex> lk(mu);
  auto it = cache.find({device, Wb, Hb});
  if (it == cache.end()) {
    // [B] FP32 values of 1 / lambda, then [B] their low parts (1/lambda - hi)
    const size_t nb = (size_t)Wb * Hb;
    std::vector<float> ie(2 * nb, 0.0f);
    for (uint32_t ky = 0; ky < Hb; ++ky) {
      const double sy = std::sin(3.14159265358979323846 * ky / (2.0 * Hb));
      const double ly = 4.0 * (sy * sy);
      for (uint32_t kx = 0; kx < Wb; ++kx) {
        const double sx = std::sin(3.14159265358979323846 * kx / (2.0 * Wb));
        const double l = 4.0 * (sx * sx) + ly;
        const double v = (kx == 0 && ky == 0) ? 0.0 : 1.0 / l;
        const float hi = (float)v;
        ie[(size_t)ky * Wb + kx] = hi;
        ie[nb + (size_t)ky * Wb + kx] = (float)(v - (double)hi);
      }
    }
    float* d = nullptr;
    cudaError_t e = cudaMalloc(&d, ie.size() * 4);
    if (e == cudaSuccess) e = cudaMemcpy(d, ie.data(), ie.size() * 4, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return e;
    it = cache.emplace(std::make_tuple(device, Wb, Hb), d).first;
  }
  *out = it->second;
  return cudaSuccess;
}
}  // namespace

// Pinned host mirrors of the controller state, grid barrier and reduction
// scalars of one instance, carved from shared slabs: page-locking memory per
// instance would dominate admitting small jobs.
namespace {
constexpr size_t kMirrorBytes =
    sizeof(RunBlock) + (((kScalars * sizeof(double) + kIScalars * sizeof(long long)) + 255) & ~(size_t)255);
static_assert(sizeof(RunBlock) % 256 == 0, "RunBlock keeps the scalars 256-byte aligned");
std::mutex g_mirror_mu;
std::vector<char*> g_mirror_free;
}  // namespace
int32_t acquire_mirror(RunBlock** run, double** scal, long long** iscal) {
  std::lock_guard<std::mutex> lk(g_mirror_mu);
  if (g_mirror_free.empty()) {
    constexpr int kPerSlab = 64;
    char* slab = nullptr;
    CU(cudaMallocHost((void**)&slab, kMirrorBytes * kPerSlab));
    for (int i = kPerSlab - 1; i >= 0; --i) g_mirror_free.push_back(slab + i * kMirrorBytes);
  }
  char* b = g_mirror_free.back();
  g_mirror_free.pop_back();
  std::memset(b, 0, kMirrorBytes);
  *run = (RunBlock*)b;
  *scal = (double*)(b + sizeof(RunBlock));
  *iscal = (long long*)(b + sizeof(RunBlock) + kScalars * sizeof(double));
  return TEXO_GP_OK;
}
void release_mirror(RunBlock* run) {
  if (!run) return;
  std::lock_guard<std::mutex> lk(g_mirror_mu);
  g_mirror_free.push_back((char*)run);
}

// A 2-D tensor map over a tiled tensor-core operand: rows of 64 bf16 halves
// (128 B), boxes of `box_rows` rows (one A or B block).
int32_t encode_operand_map(CUtensorMap* m, const uint16_t* base, size_t elems, uint32_t box_rows) {
  using Encode = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                              const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                              CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
  static Encode encode = [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      fn = nullptr;
    return (Encode)fn;
  }();
  if (!encode) {
    set_last_error("cuTensorMapEncodeTiled is not available from the driver");
    return TEXO_GP_ERR_CUDA;
  }
  const cuuint64_t dims[2] = {64, (cuuint64_t)(elems / 64)};
  const cuuint64_t strides[1] = {128};
  const cuuint32_t box[2] = {64, box_rows};
  const cuuint32_t unit[2] = {1, 1};
  if (encode(m, CU_TENSOR_MAP_DATA_TYPE_UINT16, 2, (void*)base, dims, strides, box, unit, CU_TENSOR_MAP_INTERLEAVE_NONE,
             CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS) {
    set_last_error("cuTensorMapEncodeTiled rejected a tensor-core operand map");
    return TEXO_GP_ERR_CUDA;
  }
  return TEXO_GP_OK;
}

// Lanes of the WA stage per degree class: every class gets its own
// warp-aligned segment of the launch's T lanes (one G-lane group per net),
// all nets in one pass when they fit, otherwise segments in proportion to the
// lanes each class needs, so the classes finish together.
void wa_lane_split(const int* begin, const int* group, int n, long long T, int* lane) {
  long long need[kMaxClasses + 1] = {0}, total = 0;
  for (int c = 0; c < n; ++c) {
    need[c] = (long long)(begin[c + 1] - begin[c]) * group[c];
    total += need[c];
  }
  long long give[kMaxClasses + 1] = {0}, sum = 0;
  for (int c = 0; c < n; ++c) {
    if (!need[c]) continue;
    long long g = total <= T ? (need[c] + 31) / 32 * 32 : (long long)((double)T * need[c] / total) / 32 * 32;
    give[c] = std::max<long long>(g, 32);
    sum += give[c];
  }
  while (sum > T) {   // rounding overshoot: trim the largest segment
    int big = 0;
    for (int c = 1; c < n; ++c)
      if (give[c] > give[big]) big = c;
    if (give[big] <= 32) break;
    give[big] -= 32;
    sum -= 32;
  }
  lane[0] = 0;
  for (int c = 0; c < n; ++c) lane[c + 1] = lane[c] + (int)give[c];
  for (int c = n; c < kMaxClasses; ++c) lane[c + 1] = lane[n];
}

// Device layout of one instance: every buffer is a 256-byte aligned slice
// of one pool allocation. The slices with host data come first and are
// filled by one copy from a pinned staging buffer; the rest are zeroed by
// one memset. The same plan sizes the instance before anything is
// allocated (admission by HBM footprint).
namespace {
struct Slicer {
  char* base = nullptr;     // device arena (null while sizing)
  char* stage = nullptr;    // host staging for the uploaded region
  size_t up = 0, zero = 0, zero_at = 0;
  static size_t round(size_t b) { return ((b ? b : 16) + 255) & ~(size_t)255; }
  // a slice with host data: returns the host slot to fill (null while sizing)
  template <typename T>
  T* put(T** dev, size_t count) {
    const size_t at = up;
    up += round(count * sizeof(T));
    if (!base) return nullptr;
    *dev = (T*)(base + at);
    return (T*)(stage + at);
  }
  template <typename T, typename D>
  void put_const(const D** dev, size_t count) {
    T* d = nullptr;
    put(&d, count);
    if (base) *dev = (const D*)d;
  }
  template <typename T>
  void zeroed(T** dev, size_t count) {
    const size_t at = zero;
    zero += round(count * sizeof(T));
    if (base) *dev = (T*)(base + zero_at + at);
  }
};
// per-thread pinned staging buffer, kept for the thread's next upload
struct Staging {
  char* p = nullptr;
  size_t bytes = 0;
  ~Staging() {
    if (p) cudaFreeHost(p);
  }
};
thread_local Staging t_stage;
}  // namespace

void Instance::plan(bool fill, void* slicer_ptr) {
  Slicer& S = *(Slicer*)slicer_ptr;
  const HostModel& h = m;
  const size_t nobj = (size_t)h.U + h.F, B = h.bins(), K = h.K;
  Dev& D = d;
  // bin coordinate of every tile centre, (t + 1/2) * scale - 1/2 in FP64,
  // split into hi + lo floats
  auto binmap = [&](const float2** dst, uint32_t tiles, uint32_t bins) {
    float2* v = nullptr;
    float2* slot = S.put(&v, tiles);
    if (fill) {
      const double scale = (double)bins / (double)tiles;
      for (uint32_t t = 0; t < tiles; ++t) {
        const double b = ((double)t + 0.5) * scale - 0.5;
        const float hi = (float)b;
        slot[t] = make_float2(hi, (float)(b - (double)hi));
      }
    }
    *dst = v;
  };
  auto copy_i = [&](const int** dst, const std::vector<int>& v) {
    int* p = nullptr;
    int* slot = S.put(&p, v.size());
    if (fill && !v.empty()) std::memcpy(slot, v.data(), v.size() * sizeof(int));
    *dst = p;
  };
  auto copy_f = [&](const float** dst, const auto& v) {   // any numeric vector -> float
    float* p = nullptr;
    float* slot = S.put(&p, v.size());
    if (fill)
      for (size_t i = 0; i < v.size(); ++i) slot[i] = (float)v[i];
    *dst = p;
  };
  auto copy_f2 = [&](const float2** dst, const std::vector<double>& v) {   // interleaved pairs
    float2* p = nullptr;
    float2* slot = S.put(&p, v.size() / 2);
    if (fill)
      for (size_t i = 0; i < v.size() / 2; ++i) slot[i] = make_float2((float)v[2 * i], (float)v[2 * i + 1]);
    *dst = p;
  };
  binmap(&D.binmap_x, h.W, h.Wb);
  binmap(&D.binmap_y, h.H, h.Hb);
  copy_i(&D.mem_unit, h.mem_unit);
  copy_f2(&D.mem_off, h.mem_off);
  copy_f(&D.mem_q, h.mem_q);
  copy_i(&D.mem_field, h.mem_field);
  copy_i(&D.unit_mem_ptr, h.unit_mem_ptr);
  copy_i(&D.fil_field, h.fil_field);
  copy_f(&D.fil_q, h.fil_q);
  copy_i(&D.net_ptr, h.net_ptr);
  copy_i(&D.pin_unit, h.pin_unit);
  copy_f2(&D.pin_base, h.pin_base);
  copy_f(&D.net_w, h.net_w);
  {
    long long *cf = nullptr, *cs = nullptr;
    long long* slot = S.put(&cf, K * B);
    long long* sum = S.put(&cs, std::max<size_t>(K, 1));
    if (fill) {
      sum[0] = 0;
      for (size_t f = 0; f < K; ++f) {
        long long acc = 0;
        for (size_t i = 0; i < B; ++i) {
          slot[f * B + i] = (long long)std::nearbyint(h.smoothed[f][i] * kFix);
          acc += slot[f * B + i];
        }
        sum[f] = acc;
      }
    }
    D.capfix = cf;
    D.capsum = cs;
  }
  copy_f2(&D.lo, h.lo);
  copy_f2(&D.hi, h.hi);
  copy_f(&D.pre_static, h.pre_static);
  copy_f(&D.pre_q, h.pre_q);
  {
    float2* slot = S.put(&bufX, nobj);   // the initial coordinates
    if (fill)
      for (size_t i = 0; i < nobj; ++i) slot[i] = make_float2((float)h.init[2 * i], (float)h.init[2 * i + 1]);
    double* sc = S.put(&r.scal, kScalars);
    if (fill) {
      std::memset(sc, 0, kScalars * sizeof(double));
      sc[SC_BETA] = h.params.beta;
      for (uint32_t f = 0; f < K; ++f) {
        sc[SC_REAL_AREA + f] = h.real_area[f];
        sc[SC_E0 + f] = 1.0;
        sc[SC_LAMBDA + f] = 0.0;
      }
    }
  }
  // zero-initialized slices
  S.zeroed(&D.phys, K * B);
  S.zeroed(&D.fill, K * B);
  S.zeroed(&D.rho, K * B);
  // t1 / t2: FP32 grids of the GEMM forms; the FFT form keeps them as
  // double-float pairs (float2 per bin), hence twice the size, and the
  // tensor-core form its pass outputs (tp) in t1
  S.zeroed(&D.t1, 2 * K * B);
  D.tp = reinterpret_cast<float2*>(D.t1);
  S.zeroed(&D.t2, 2 * K * B);
  S.zeroed(&D.phi, K * B);
  S.zeroed(&D.wa_fix, 2 * (size_t)h.U);
  S.zeroed(&D.graw, std::max<size_t>(K, 1) * nobj);
  S.zeroed(&D.P, nobj);
  S.zeroed(&bufXp, nobj);
  S.zeroed(&bufY, nobj);
  S.zeroed(&bufC, nobj);
  S.zeroed(&gX, nobj);
  S.zeroed(&gY, nobj);
  S.zeroed(&gC, nobj);
  S.zeroed(&run_dev, 1);
  S.zeroed(&best, std::max<size_t>(h.U, 1));
  S.zeroed(&prev_targets, 2 * (size_t)h.U);
  S.zeroed(&mismatch, 1);
  S.zeroed(&r.p.sum, (size_t)kSlots * kMaxPartials);
  S.zeroed(&r.p.isum, (size_t)kISlots * kMaxPartials);
  S.zeroed(&r.p.mx, (size_t)kMSlots * kMaxPartials);
  S.zeroed(&r.q.sum, (size_t)kSlots * kMaxPartials);
  S.zeroed(&r.q.isum, (size_t)kISlots * kMaxPartials);
  S.zeroed(&r.q.mx, (size_t)kMSlots * kMaxPartials);
  S.zeroed(&r.iscal, kIScalars);
  if (h.params.engine == TEXO_GP_ENGINE_HOST) {   // the tiled scatter's counting sort
    const size_t items = (size_t)h.Mm + h.F;
    const size_t nk = 2 * K * (size_t)((h.Wb + tiles::kTile - 1) / tiles::kTile) *
                      ((h.Hb + tiles::kTile - 1) / tiles::kTile);
    S.zeroed(&D.bin_key, items);
    S.zeroed(&D.bin_rank, items);
    S.zeroed(&D.bin_order, items);
    S.zeroed(&D.bin_cnt, nk);
    S.zeroed(&D.bin_off, nk + 1);
  }
  if (h.params.dct_mode == TEXO_GP_DCT_TENSOR) {   // tensor-core operands (zero padding)
    S.zeroed(&D.opA, tc::a_elems((int)h.Hb, (int)h.Wb, (int)K));
    S.zeroed(&D.opB, tc::b_elems((int)h.Wb, (int)h.Hb, (int)K));
    S.zeroed(&D.eA, (size_t)tc::pad((int)h.Hb, tc::kM) * K);
    S.zeroed(&D.eB, (size_t)tc::pad((int)h.Wb, tc::kN) * K);
    S.zeroed(&D.tmx, 2 * (size_t)h.Wb * K);
  }
}

uint64_t Instance::device_bytes() {
  Slicer S;
  plan(false, &S);
  return S.up + S.zero;
}

int32_t Instance::upload() {
  HostModel& h = m;
  CU(cudaSetDevice(device));
  CU(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  CU(keep_pool(device));
  CU(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  const size_t nobj = (size_t)h.U + h.F, B = h.bins(), K = h.K;
  // enough blocks to cover the widest stage, up to kBlocksPerSm per SM
  const size_t widest = std::max(std::max(std::max(nobj, (size_t)h.Mm + h.F), std::max(B, h.pin_unit.size() / 2)), (size_t)1);
  // Virtual blocks: the reduction structure of every stage. The standalone
  // kernels of the host engine launch exactly this many blocks, up to
  // kHostBlocksPerSm a SM so that large instances keep enough loads in
  // flight; the persistent engine runs kBlocksPerSm a SM and loops its
  // physical blocks over the virtual ones, which therefore match that grid.
  constexpr size_t kHostBlocksPerSm = 8;
  const size_t per_sm = h.params.engine == TEXO_GP_ENGINE_DEVICE ? (size_t)kBlocksPerSm : kHostBlocksPerSm;
  nvb = (int)std::min(std::min((widest + kThreads - 1) / kThreads, (size_t)sms * per_sm), (size_t)kMaxPartials);
  nvb = std::max(nvb, 1);
  Dev& D = d;
  D.U = (int)h.U;
  D.F = (int)h.F;
  D.nobj = (int)nobj;
  D.K = (int)K;
  D.Mm = (int)h.Mm;
  D.B = (int)B;
  D.g = Grid{(int)h.W, (int)h.H, (int)h.Wb, (int)h.Hb, (float)h.sx, (float)h.sy, h.identity ? 1 : 0};
  D.n_classes = h.n_classes;
  std::memcpy(D.class_begin, h.class_begin, sizeof(D.class_begin));
  std::memcpy(D.class_group, h.class_group, sizeof(D.class_group));
  D.n_hpwl_nets = h.n_hpwl_nets;
  wa_lane_split(h.class_begin, h.class_group, h.n_classes, (long long)nvb * kThreads, D.class_lane);
  {
    BasisTables bx, by;
    float* ie;
    CU(shared_basis(device, h.Wb, &bx));
    CU(shared_basis(device, h.Hb, &by));
    CU(shared_inv_eig(device, h.Wb, h.Hb, &ie));
    D.Cx = bx.c;
    D.CxT = bx.ct;
    D.Cy = by.c;
    D.CyT = by.ct;
    D.inv_eig = ie;
    D.inv_eig_lo = ie + (size_t)h.Wb * h.Hb;
    D.eCx = bx.e;
    D.eCy = by.e;
    D.tc = h.params.dct_mode == TEXO_GP_DCT_TENSOR ? 1 : 0;
    // the tiled scatter (host engine) when asked for; AUTO leaves it to the autotuner
    D.scatter_tiles = h.params.engine == TEXO_GP_ENGINE_HOST && h.params.scatter_mode == TEXO_GP_SCATTER_TILED;
    // fixed rule unless autotuned: large tiles once the grid has >= 1024 32x32 blocks
    D.dct_large = (long long)((h.Wb + 31) / 32) * ((h.Hb + 31) / 32) >= 1024 ? 1 : 0;
    // the FFT form for power-of-two grids (FP32 mode)
    D.fft = 0;
    D.logW = ilog2(h.Wb);
    D.logH = ilog2(h.Hb);
    if (fft_length(h.Wb) && fft_length(h.Hb)) {
      FftTables fx, fy;
      CU(shared_fft(device, h.Wb, &fx));
      CU(shared_fft(device, h.Hb, &fy));
      D.fx_tw = fx.tw;
      D.fx_post = fx.post;
      D.fx_pre = fx.pre;
      D.fx_inv_s = fx.inv_s;
      D.fy_tw = fy.tw;
      D.fy_post = fy.post;
      D.fy_pre = fy.pre;
      D.fy_inv_s = fy.inv_s;
      D.fft = h.params.dct_mode == TEXO_GP_DCT_FP32 ? 1 : 0;
    }
    D.Hp128 = tc::pad((int)h.Hb, tc::kM);
    D.Hp32 = tc::pad((int)h.Hb, tc::kKC);
    D.Wp64 = tc::pad((int)h.Wb, tc::kN);
    D.Wp32 = tc::pad((int)h.Wb, tc::kKC);
    D.CxB_t = bx.cB;      // pass 0: B = rows of Cx
    D.CxTB_t = bx.ctB;    // pass 3: B = rows of Cx^T
    D.CyA_t = by.cA;      // pass 1: A = Cy
    D.CyTA_t = by.ctA;    // pass 2: A = Cy^T
  }
  // size, allocate, pack, copy
  Slicer sizing;
  plan(false, &sizing);
  const size_t up_bytes = sizing.up, zero_bytes = sizing.zero;
  void* base = nullptr;
  TRY(alloc(&base, up_bytes + zero_bytes));
  if (t_stage.bytes < up_bytes) {
    if (t_stage.p) cudaFreeHost(t_stage.p);
    t_stage.p = nullptr;
    t_stage.bytes = 0;
    const size_t want = std::max(up_bytes, (size_t)4 << 20) * 2;
    CU(cudaMallocHost((void**)&t_stage.p, want));
    t_stage.bytes = want;
  }
  Slicer S;
  S.base = (char*)base;
  S.stage = t_stage.p;
  S.zero_at = up_bytes;
  plan(true, &S);
  CU(cudaMemcpyAsync(base, t_stage.p, up_bytes, cudaMemcpyHostToDevice, stream));
  CU(cudaMemsetAsync((char*)base + up_bytes, 0, zero_bytes, stream));
  posb[0] = bufX;
  posb[1] = bufXp;
  posb[2] = bufY;
  posb[3] = bufC;
  gradb[0] = gX;
  gradb[1] = gY;
  gradb[2] = gC;
  {
    static const int per_sm = persistent_blocks_per_sm();
    pblocks = std::min(std::max(per_sm, 1), kBlocksPerSm) * sms;
    pblocks = std::min(pblocks, kMaxPartials);
  }
  TRY(acquire_mirror(&h_run, &h_scal, &h_iscal));
  std::memset(h_scal, 0, kScalars * sizeof(double));
  std::memset(h_iscal, 0, kIScalars * sizeof(long long));
  h_scal[SC_BETA] = h.params.beta;
  for (uint32_t f = 0; f < K; ++f) {
    h_scal[SC_REAL_AREA + f] = h.real_area[f];
    h_scal[SC_E0 + f] = 1.0;
    h_scal[SC_LAMBDA + f] = 0.0;
  }
  if (h.params.dct_mode == TEXO_GP_DCT_TENSOR) {   // tensor maps of the tensor-core operands
    const int W = (int)h.Wb, H = (int)h.Hb;
    const uint32_t ra = tc::kABlock / 64, rb = tc::kBBlock / 64;
    TRY(encode_operand_map(&tmaps.m[tc::TM_OPA], D.opA, tc::a_elems(H, W, (int)K), ra));
    TRY(encode_operand_map(&tmaps.m[tc::TM_OPB], D.opB, tc::b_elems(W, H, (int)K), rb));
    TRY(encode_operand_map(&tmaps.m[tc::TM_CXB], D.CxB_t, tc::b_elems(W, W, 1), rb));
    TRY(encode_operand_map(&tmaps.m[tc::TM_CXTB], D.CxTB_t, tc::b_elems(W, W, 1), rb));
    TRY(encode_operand_map(&tmaps.m[tc::TM_CYA], D.CyA_t, tc::a_elems(H, H, 1), ra));
    TRY(encode_operand_map(&tmaps.m[tc::TM_CYTA], D.CyTA_t, tc::a_elems(H, H, 1), ra));
  }
  // the staging buffer is reused by this thread's next upload
  CU(cudaStreamSynchronize(stream));
  return TEXO_GP_OK;
}

// ---------------------------------------------------------------------------
// Host-driven controller.
// ---------------------------------------------------------------------------
struct EvalRec {
  double value = 0, wa = 0, wal1 = 0;
  double energy[kMaxFields] = {}, overflow[kMaxFields] = {}, force[kMaxFields] = {}, rawl1[kMaxFields] = {};
  double net_charge[kMaxFields] = {};
  long long overflow_fixed[kMaxFields] = {}, overflow_bins[kMaxFields] = {};
  long long bad = std::numeric_limits<long long>::max();
};

static inline double midpoint1(double b) {
  const double hi = std::numeric_limits<double>::max() / 2.0;
  if (std::fabs(b) <= hi) return (1.0 + b) / 2.0;
  return 0.5 + b / 2.0;
}
static inline double half_nonzero(double v) {
  const double h = v * 0.5;
  return h == 0.0 ? v : h;
}

struct Controller {
  Instance& I;
  // eplace state (eplace.rs:439-582)
  int phase = 0;              // 0 fresh, 1 running, 2 finished
  std::vector<double> lambda, e0;
  double mstep = 0.0;
  EvalRec current;
  double gamma = 0.0;
  uint32_t completed = 0;
  double best_max = 0, best_tot = 0;
  bool have_prev_stationary = false;
  bool converged = false, exhausted = false;
  int32_t final_status = TEXO_GP_OK;
  // Nesterov state (global_placement.rs:29-58)
  double a = 1.0;
  bool has_L = false;
  double L = 0.0;
  bool density_at_x = false;  // graw/phi/energies describe bufX
  // statistics
  uint64_t evaluations = 0, device_evaluations = 0, trials = 0;
  uint64_t density_evaluations = 0;   // evaluations that rebuilt the density side
  double last_objective = 0.0;
  double elapsed_ms = 0.0;
  unsigned long long launches = 0;
  static constexpr size_t kTraceMax = 4096;
  std::vector<texo_gp_iteration> trace;   // host engine: one record per completed iteration
  // One round of eplace::place's area-adjustment loop (texo_gp_optimize_round):
  // the stop criterion (0 final, 1 area-adjustment ready), the area-reset
  // multipliers, fixed density scales (E0 of the first round) and the
  // iterations of the earlier rounds.
  int stop_mode = 0;
  bool reset_mult = false;
  std::vector<double> fixed_scales;
  uint64_t iter_offset = 0;

  explicit Controller(Instance& i) : I(i), hr(i.h_run->run) { std::memset(&hr, 0, sizeof(hr)); }
  ~Controller() {
    if (step_exec) cudaGraphExecDestroy(step_exec);
    for (cudaEvent_t e : step_ev)
      if (e) cudaEventDestroy(e);
  }

  static int32_t fail_norm(const char* what) {
    set_last_error(what);
    return TEXO_GP_ERR_INVALID_NORMALIZATION;
  }
  double margin(double x, double y) const {
    const double eps = std::max(std::numeric_limits<double>::epsilon(), I.m.params.objective_margin_ulps * 0x1p-24);
    return eps * (1.0 + std::fabs(x) + std::fabs(y));
  }

  int32_t sync_read() {
    CU(cudaMemcpyAsync(I.h_scal, I.r.scal, kScalars * sizeof(double), cudaMemcpyDeviceToHost, I.stream));
    CU(cudaMemcpyAsync(I.h_iscal, I.r.iscal, kIScalars * sizeof(long long), cudaMemcpyDeviceToHost, I.stream));
    CU(cudaStreamSynchronize(I.stream));
    CU(cudaGetLastError());
    if (I.h_iscal[SI_TC_FAIL]) {
      set_last_error("tensor-core DCT: an mbarrier wait ran out");
      return TEXO_GP_ERR_DEVICE_TIMEOUT;
    }
    return TEXO_GP_OK;
  }
  int32_t push_inputs() {
    for (uint32_t f = 0; f < I.m.K; ++f) {
      I.h_scal[SC_LAMBDA + f] = lambda.empty() ? 0.0 : lambda[f];
      I.h_scal[SC_E0 + f] = e0.empty() ? 1.0 : e0[f];
    }
    CU(cudaMemcpyAsync(I.r.scal + SC_LAMBDA, I.h_scal + SC_LAMBDA, 2 * kMaxFields * sizeof(double),
                       cudaMemcpyHostToDevice, I.stream));
    return TEXO_GP_OK;
  }

  // Enqueues one objective evaluation (ContinuousProblem::evaluate +
  // combined_objective). With reuse, the density side of `pos` is the one
  // already on the device (same coordinates), and only WA and the
  // combination are recomputed.
  void enqueue_eval(const float2* pos, float2* g, double gam, bool reuse) {
    const Dev& D = I.d;
    cudaStream_t s = I.stream;
    const int nvb = I.nvb;
    if (!reuse && I.m.has_density) {
      launch_init(D, true, true, nvb, s);
      launch_scatter(D, I.r, pos, nvb, s);
      launch_prep(D, I.r, nvb, s);
      for (int st = 0; st < 4; ++st) launch_dct(D, I.r, st, nvb, s, &I.tmaps);
      launch_gather(D, I.r, pos, nvb, s);
      density_evaluations++;
    } else {
      launch_init(D, false, true, nvb, s);
    }
    launch_wa(D, I.r, pos, gam, nvb, s);
    launch_finalize(D, I.r, nvb, (reuse || !I.m.has_density) ? FIN_WA : FIN_ENERGY, s);
    launch_combine(D, I.r, g, nvb, s);
    launch_finalize(D, I.r, nvb, FIN_COMBINE, s);
    device_evaluations++;
  }
  void read_eval(EvalRec& e) const {
    const double* sc = I.h_scal;
    const long long* si = I.h_iscal;
    e.value = sc[SC_VALUE];
    e.wa = sc[SC_WA];
    e.wal1 = sc[SC_WAL1];
    for (uint32_t f = 0; f < I.m.K; ++f) {
      e.energy[f] = sc[SC_ENERGY + f];
      e.overflow[f] = sc[SC_OVERFLOW + f];
      e.force[f] = sc[SC_FORCE + f];
      e.rawl1[f] = sc[SC_RAWL1 + f];
      e.net_charge[f] = sc[SC_MEAN + f];
      e.overflow_fixed[f] = si[SI_OVERFLOW_FIXED + f];
      e.overflow_bins[f] = si[SI_OVER_BINS + f];
    }
    e.bad = si[SI_BAD];
  }
  int32_t evaluate(const float2* pos, float2* g, double gam, bool reuse, EvalRec& e) {
    enqueue_eval(pos, g, gam, reuse);
    TRY(sync_read());
    read_eval(e);
    evaluations++;
    return TEXO_GP_OK;
  }
  int32_t checked(const EvalRec& e) const {
    if (!std::isfinite(e.value)) return TEXO_GP_ERR_INVALID_OBJECTIVE;
    if (e.bad != std::numeric_limits<long long>::max()) return TEXO_GP_ERR_NONFINITE_GRADIENT;
    return TEXO_GP_OK;
  }

  // ---- eplace rules (eplace.rs:1111-1415) ----
  int32_t field_gamma(double overflow, double target, double base, double& g) const {
    if (!std::isfinite(overflow) || overflow < 0.0 || !(target >= 0.0 && target < 1.0) || !(base > 0.0))
      return TEXO_GP_ERR_INVALID_NORMALIZATION;
    const double slope = 2.0 / (1.0 - target), intercept = 1.0 - slope;
    g = base * std::pow(10.0, slope * overflow + intercept);
    return (std::isfinite(g) && g > 0.0) ? TEXO_GP_OK : TEXO_GP_ERR_INVALID_NORMALIZATION;
  }
  int32_t adaptive_gamma(const EvalRec& e, double& out) const {
    const double base = I.m.gamma_base_tiles();
    double ws = 0.0, wsum = 0.0;
    for (uint32_t f = 0; f < I.m.K; ++f) {
      double g;
      TRY(field_gamma(e.overflow[f], I.m.overflow_target(f), base, g));
      const double w = I.m.gamma_weight[f];
      ws += g * w;
      wsum += w;
    }
    out = wsum == 0.0 ? base : ws / wsum;
    return (std::isfinite(out) && out > 0.0) ? TEXO_GP_OK : TEXO_GP_ERR_INVALID_NORMALIZATION;
  }
  // density_stop_reached (eplace.rs:1397-1415): Final, or AreaAdjustmentReady
  // (LUT and register fields at 0.15, AREA_ADJUSTMENT_OVERFLOW_TARGET, eplace.rs:130)
  bool stop_reached(const EvalRec& e) const {
    for (uint32_t f = 0; f < I.m.K; ++f) {
      if (stop_mode == 1) {
        const uint32_t k = I.m.kinds[f].kind;
        if (k != TEXO_GP_KIND_LUT && k != TEXO_GP_KIND_REGISTER) continue;
        if (!(e.overflow[f] <= 0.15)) return false;
      } else if (!(e.overflow[f] <= I.m.overflow_target(f))) {
        return false;
      }
    }
    return true;
  }
  // area_adjusted_density_multipliers and area_adjusted_multiplier_step
  // (eplace.rs:1183-1232), elfPlace eqs. (27)-(28)
  int32_t area_multipliers(const EvalRec& e) {
    TRY(validate_fields(e));
    const double beta = I.m.params.beta;
    double sg[kMaxFields], dens = 0.0;
    for (uint32_t f = 0; f < I.m.K; ++f) {
      const double ne = e.energy[f] / e0[f];
      sg[f] = ne + 0.5 * beta * ne * ne;
      if (!std::isfinite(sg[f]) || sg[f] < 0.0) return fail_norm("area-reset multipliers: subgradient");
      dens += e.force[f] * sg[f];
    }
    if (!std::isfinite(e.wal1) || e.wal1 <= 0.0 || !std::isfinite(dens) || dens <= 0.0) {
      set_last_error("area-reset multipliers: wirelength force " + std::to_string(e.wal1) + ", density force " +
                     std::to_string(dens));
      return TEXO_GP_ERR_INVALID_NORMALIZATION;
    }
    const double scale = 0.1 * e.wal1 / dens;
    bool any = false;
    double nn = 0.0;
    for (uint32_t f = 0; f < I.m.K; ++f) {
      lambda[f] = scale * sg[f];
      if (!std::isfinite(lambda[f]) || lambda[f] < 0.0) return fail_norm("area-reset multipliers: multiplier");
      any = any || lambda[f] > 0.0;
      nn += lambda[f] * lambda[f];
    }
    if (!any) return fail_norm("area-reset multipliers: all zero");
    mstep = (I.m.params.alpha_high - 1.0) * std::sqrt(nn);
    return (std::isfinite(mstep) && mstep > 0.0) ? TEXO_GP_OK : TEXO_GP_ERR_INVALID_NORMALIZATION;
  }
  void excess(const EvalRec& e, double& mx, double& tot) const {
    mx = 0.0;
    tot = 0.0;
    for (uint32_t f = 0; f < I.m.K; ++f) {
      const double x = std::fmax(e.overflow[f] - I.m.overflow_target(f), 0.0);
      mx = std::fmax(mx, x);
      tot += x;
    }
  }
  int32_t validate_initial(const EvalRec& e) const {
    bool ok = std::isfinite(e.wa) && e.bad == std::numeric_limits<long long>::max();
    for (uint32_t f = 0; f < I.m.K && ok; ++f)
      ok = std::isfinite(e.energy[f]) && e.energy[f] >= 0.0 && std::isfinite(e.overflow[f]) &&
           std::isfinite(e.force[f]) && e.force[f] >= 0.0;
    return ok ? TEXO_GP_OK : fail_norm("initial evaluation not finite");
  }
  int32_t validate_fields(const EvalRec& e) const {
    for (uint32_t f = 0; f < I.m.K; ++f)
      if (!std::isfinite(e.energy[f]) || !std::isfinite(e0[f]) || e0[f] <= 0.0) return TEXO_GP_ERR_DENSITY_FIELD_CHANGED;
    return TEXO_GP_OK;
  }
  int32_t update_multipliers(const EvalRec& e) {
    TRY(validate_fields(e));
    const double beta = I.m.params.beta;
    double sg[kMaxFields], nn = 0.0;
    for (uint32_t f = 0; f < I.m.K; ++f) {
      const double ne = e.energy[f] / e0[f];
      sg[f] = ne + 0.5 * beta * ne * ne;
      if (!std::isfinite(sg[f]) || sg[f] < 0.0) return TEXO_GP_ERR_INVALID_NORMALIZATION;
      nn += sg[f] * sg[f];
    }
    const double norm = std::sqrt(nn);
    if (norm != 0.0) {
      if (!std::isfinite(norm) || !std::isfinite(mstep) || mstep <= 0.0) return TEXO_GP_ERR_INVALID_NORMALIZATION;
      for (uint32_t f = 0; f < I.m.K; ++f) {
        lambda[f] += mstep * sg[f] / norm;
        if (!std::isfinite(lambda[f]) || lambda[f] < 0.0) return TEXO_GP_ERR_INVALID_NORMALIZATION;
      }
    }
    // next_multiplier_step (eplace.rs:1261-1298)
    double en = 0.0;
    for (uint32_t f = 0; f < I.m.K; ++f) {
      const double ne = e.energy[f] / e0[f];
      en += ne * ne;
    }
    const double lg = std::log(beta * std::sqrt(en) + 1.0);
    if (!std::isfinite(lg) || lg < 0.0) return fail_norm("multiplier growth logarithm");
    const double lo = I.m.params.alpha_low, hi = I.m.params.alpha_high;
    const double growth = lo + (1.0 - 1.0 / (1.0 + lg)) * (hi - lo);
    if (!(growth >= lo && growth <= hi)) return TEXO_GP_ERR_INVALID_NORMALIZATION;
    mstep *= growth;
    return (std::isfinite(mstep) && mstep > 0.0) ? TEXO_GP_OK : TEXO_GP_ERR_INVALID_NORMALIZATION;
  }

  // ---- one dynamic Nesterov step on the device buffers ----
  int32_t nesterov_step(double gam, EvalRec& payload, bool& stationary) {
    const Dev& D = I.d;
    cudaStream_t s = I.stream;
    const int nvb = I.nvb;
    if (!std::isfinite(a) || a < 1.0) return TEXO_GP_ERR_INVALID_MOMENTUM_PARAMETER;
    if (has_L && (!std::isfinite(L) || L <= 0.0)) return TEXO_GP_ERR_INVALID_LIPSCHITZ_ESTIMATE;
    // preconditioner range for the denominator checks
    launch_precond(D, I.r, nvb, s);
    launch_finalize(D, I.r, nvb, FIN_PRECOND, s);
    EvalRec eo;
    TRY(evaluate(I.bufX, I.gX, gam, density_at_x, eo));
    if (I.h_iscal[SI_PBAD]) return fail_norm("preconditioner out of range");
    const double pmin = I.h_scal[SC_PMIN], pmax = I.h_scal[SC_PMAX];
    TRY(checked(eo));
    bool restart = false;
    bool has_wL = has_L;
    double wL = L;
    uint64_t step_trials = 0;
    for (;;) {  // 'step
      const double momentum = restart ? 1.0 : a;
      const double next_m = midpoint1(std::sqrt(1.0 + 4.0 * momentum * momentum));
      if (!std::isfinite(next_m)) return TEXO_GP_ERR_ITERATION_OVERFLOW;
      const double extrap = (momentum - 1.0) / next_m;
      bool y_is_origin = true;
      if (!restart) {
        launch_extrapolate(D, I.r, I.bufX, I.bufXp, extrap, I.bufY, nvb, s);
        launch_finalize(D, I.r, nvb, FIN_DIFF, s);
        TRY(sync_read());
        y_is_origin = I.h_iscal[SI_DIFF] == 0;
      }
      const float2* ybuf = y_is_origin ? I.bufX : I.bufY;
      const float2* gy = y_is_origin ? I.gX : I.gY;
      double f_y = eo.value;
      if (!y_is_origin) {
        enqueue_eval(I.bufY, I.gY, gam, false);
        density_at_x = false;
      }
      launch_kkt(D, I.r, ybuf, gy, nullptr, nvb, s);
      launch_finalize(D, I.r, nvb, FIN_KKT, s);
      TRY(sync_read());
      if (!y_is_origin) {
        EvalRec ey;
        read_eval(ey);
        evaluations++;
        TRY(checked(ey));
        f_y = ey.value;
      }
      const double y_stat = I.h_scal[SC_KKT];
      if (!std::isfinite(y_stat)) return TEXO_GP_ERR_LINE_SEARCH_OVERFLOW;
      if (y_stat == 0.0) {
        if (!y_is_origin) {
          restart = true;
          continue;
        }
        CU(cudaMemcpyAsync(I.bufXp, I.bufX, (size_t)D.nobj * sizeof(float2), cudaMemcpyDeviceToDevice, s));
        a = 1.0;
        stationary = true;
        payload = eo;
        trials += step_trials;
        last_objective = eo.value;
        return TEXO_GP_OK;
      }
      double tL = half_nonzero(has_wL ? wL : y_stat);
      bool may_reduce = true;
      bool restart_step = false;
      EvalRec ec;
      for (;;) {
        step_trials++;
        if (!std::isfinite(tL * pmax)) return TEXO_GP_ERR_LINE_SEARCH_OVERFLOW;
        if (tL * pmin == 0.0) {
          tL *= 2.0;
          may_reduce = false;
          if (!std::isfinite(tL)) return TEXO_GP_ERR_LINE_SEARCH_OVERFLOW;
          continue;
        }
        launch_candidate(D, I.r, ybuf, gy, (float)std::fmin(1.0 / tL, 3.0e38), I.bufC, nvb, s);
        launch_finalize(D, I.r, nvb, FIN_CAND, s);
        // The candidate is evaluated speculatively in the same submission;
        // it is discarded when the candidate equals y.
        enqueue_eval(I.bufC, I.gC, gam, false);
        density_at_x = false;
        TRY(sync_read());
        const long long changed = I.h_iscal[SI_DIFF];
        const double dot = I.h_scal[SC_DOT], msn = I.h_scal[SC_MSN];
        if (changed == 0) {
          if (may_reduce) {
            const double smaller = half_nonzero(tL);
            if (smaller < tL) {
              tL = smaller;
              continue;
            }
          }
          if (!y_is_origin) {
            restart = true;
            has_wL = true;
            wL = tL;
            restart_step = true;
            break;
          }
          CU(cudaMemcpyAsync(I.bufXp, I.bufX, (size_t)D.nobj * sizeof(float2), cudaMemcpyDeviceToDevice, s));
          a = 1.0;
          has_L = true;
          L = tL;
          stationary = true;
          payload = eo;
          trials += step_trials;
          last_objective = eo.value;
          return TEXO_GP_OK;
        }
        read_eval(ec);
        evaluations++;
        TRY(checked(ec));
        const double upper = f_y + dot + 0.5 * tL * msn;
        if (!std::isfinite(upper)) return TEXO_GP_ERR_LINE_SEARCH_OVERFLOW;
        const bool smooth = ec.value <= upper + margin(ec.value, upper);
        const bool mono = ec.value <= eo.value + margin(ec.value, eo.value);
        if (smooth && mono) break;
        if (smooth && !restart) {
          restart = true;
          has_wL = true;
          wL = tL;
          restart_step = true;
          break;
        }
        tL *= 2.0;
        may_reduce = false;
        if (!std::isfinite(tL)) return TEXO_GP_ERR_LINE_SEARCH_OVERFLOW;
      }
      if (restart_step) continue;
      // accept: stationarity at the candidate and the coordinate change
      launch_kkt(D, I.r, I.bufC, I.gC, I.bufX, nvb, s);
      launch_finalize(D, I.r, nvb, FIN_KKT, s);
      TRY(sync_read());
      if (!std::isfinite(I.h_scal[SC_KKT])) return TEXO_GP_ERR_LINE_SEARCH_OVERFLOW;
      std::swap(I.bufXp, I.bufX);   // previous <- origin
      std::swap(I.bufX, I.bufC);    // origin <- candidate
      std::swap(I.gX, I.gC);
      a = next_m;
      has_L = true;
      L = tL;
      density_at_x = true;
      stationary = false;
      payload = ec;
      trials += step_trials;
      last_objective = ec.value;
      return TEXO_GP_OK;
    }
  }

  int32_t save_best() {
    CU(cudaMemcpyAsync(I.best, I.bufX, (size_t)I.m.U * sizeof(float2), cudaMemcpyDeviceToDevice, I.stream));
    return TEXO_GP_OK;
  }

  // The device engine: the same loop inside one persistent cooperative kernel.
  DevRun& hr;                 // the pinned mirror's controller state
  bool dev_ready = false;
  // The device-engine step captured as a CUDA graph once it repeats (the
  // descriptor it was captured with is kept: a different one recaptures; a
  // one-shot placement, a single step to convergence, pays no capture), and
  // the CUDA events that time the step's device work.
  cudaGraphExec_t step_exec = nullptr;
  bool step_graph_off = false;
  unsigned device_steps = 0;
  Dev step_dev{};
  cudaEvent_t step_ev[2] = {nullptr, nullptr};
  double device_ms = -1.0;    // device time of the last device-engine step

  // Initializes the kernel's controller state on first use.
  void prepare_devrun() {
    const HostModel& m = I.m;
    if (!dev_ready) {
      std::memset(&hr, 0, sizeof(hr));
      hr.K = (int)m.K;
      hr.max_iterations = m.params.max_iterations;
      hr.best_effort = m.params.best_effort;
      hr.W = (int)m.W;
      hr.H = (int)m.H;
      hr.beta = m.params.beta;
      hr.alpha_low = m.params.alpha_low;
      hr.alpha_high = m.params.alpha_high;
      hr.init_weight = m.params.initial_density_weight;
      hr.gamma_base = m.gamma_base_tiles();
      hr.margin_eps = std::max(std::numeric_limits<double>::epsilon(), m.params.objective_margin_ulps * 0x1p-24);
      double weight_sum = 0.0;
      for (uint32_t f = 0; f < m.K; ++f) {
        hr.target[f] = m.overflow_target(f);
        hr.gamma_slope[f] = 2.0 / (1.0 - hr.target[f]);
        hr.gamma_weight[f] = m.gamma_weight[f];
        hr.real_area[f] = m.real_area[f];
        hr.inv_real_area[f] = 1.0 / m.real_area[f];
        hr.e0[f] = 1.0;
        hr.inv_e0[f] = 1.0;
        weight_sum += m.gamma_weight[f];
      }
      hr.inv_gamma_weight_sum = weight_sum == 0.0 ? 0.0 : 1.0 / weight_sum;
      // a round of the area-adjustment loop (texo_gp_optimize_round)
      hr.stop_mode = stop_mode;
      hr.reset_mult = reset_mult ? 1 : 0;
      hr.fixed_e0 = fixed_scales.empty() ? 0 : 1;
      for (uint32_t f = 0; f < m.K; ++f) {
        const uint32_t k = m.kinds[f].kind;
        hr.area_field[f] = (k == TEXO_GP_KIND_LUT || k == TEXO_GP_KIND_REGISTER) ? 1 : 0;
        if (!fixed_scales.empty()) hr.e0[f] = fixed_scales[f];
      }
      hr.completed = (unsigned)iter_offset;
      hr.a = 1.0;
      hr.ix = 0;
      hr.ixp = 1;
      hr.iy = 2;
      hr.ic = 3;
      hr.igx = 0;
      hr.igy = 1;
      hr.igc = 2;
      for (int i = 0; i < 4; ++i) I.posb[i] = i == 0 ? I.bufX : (i == 1 ? I.bufXp : (i == 2 ? I.bufY : I.bufC));
      dev_ready = true;
    }
  }

  Buffers buffers() const {
    Buffers b;
    for (int i = 0; i < 4; ++i) b.pos[i] = I.posb[i];
    for (int i = 0; i < 3; ++i) b.grad[i] = I.gradb[i];
    b.best = I.best;
    b.prev_targets = I.prev_targets;
    return b;
  }

  int32_t run_device(uint32_t budget) {
    prepare_devrun();
    hr.budget = budget;
    const int blocks = std::min(I.pblocks, I.nvb);
    if (step_exec && std::memcmp(&step_dev, &I.d, sizeof(Dev)) != 0) {
      cudaGraphExecDestroy(step_exec);
      step_exec = nullptr;
    }
    if (!step_exec && !step_graph_off && device_steps++ > 0) {
      if (capture_persistent(I.d, I.r, buffers(), I.run_dev, I.h_run, blocks, I.nvb, I.stream, &step_exec))
        step_graph_off = true;   // the direct launch below takes over
      else
        step_dev = I.d;
    }
    for (cudaEvent_t& e : step_ev)
      if (!e) CU(cudaEventCreate(&e));
    std::memset(&I.h_run->bar, 0, sizeof(GridBarrier));
    CU(cudaEventRecord(step_ev[0], I.stream));
    int32_t s = step_exec ? (cudaGraphLaunch(step_exec, I.stream) == cudaSuccess ? TEXO_GP_OK : TEXO_GP_ERR_CUDA)
                          : enqueue_persistent(I.d, I.r, buffers(), I.run_dev, I.h_run, blocks, I.nvb, I.stream);
    if (!s) {
      note_launch();
      CU(cudaEventRecord(step_ev[1], I.stream));
      if (cudaStreamSynchronize(I.stream) != cudaSuccess) s = TEXO_GP_ERR_CUDA;
      else if (I.h_run->bar.error) s = TEXO_GP_ERR_DEVICE_TIMEOUT;
    }
    if (!s) {
      float ms = 0.f;
      CU(cudaEventElapsedTime(&ms, step_ev[0], step_ev[1]));
      device_ms = ms;
    }
    if (s) {
      set_last_error(s == TEXO_GP_ERR_DEVICE_TIMEOUT ? "persistent kernel: a grid barrier wait ran out"
                                                     : std::string("persistent kernel: ") +
                                                           cudaGetErrorString(cudaGetLastError()));
      return s;
    }
    return absorb_devrun();
  }

  // Mirrors the kernel's state (hr, already copied back) for the common
  // result path.
  int32_t absorb_devrun() {
    const HostModel& m = I.m;
    I.bufX = I.posb[hr.ix];
    I.bufXp = I.posb[hr.ixp];
    I.bufY = I.posb[hr.iy];
    I.bufC = I.posb[hr.ic];
    I.gX = I.gradb[hr.igx];
    I.gY = I.gradb[hr.igy];
    I.gC = I.gradb[hr.igc];
    completed = hr.completed;
    evaluations = hr.evaluations;
    density_evaluations = hr.density_evaluations;
    trials = hr.trials;
    converged = hr.converged != 0;
    exhausted = hr.exhausted != 0;
    gamma = hr.gamma;
    last_objective = hr.last_objective;
    e0.assign(hr.e0, hr.e0 + m.K);
    lambda.assign(hr.lambda, hr.lambda + m.K);
    for (uint32_t f = 0; f < m.K; ++f) {
      current.overflow[f] = hr.cur_overflow[f];
      current.energy[f] = hr.cur_energy[f];
    }
    phase = hr.phase;
    final_status = hr.status;
    density_at_x = false;   // the host engine's scalar block no longer describes X
    return hr.status;
  }

  // optimize_density_once (eplace.rs:439-582), resumable: runs at most
  // `budget` more iterations when budget > 0.
  int32_t run(uint32_t budget) {
    if (phase == 2) return final_status;
    if (!I.m.has_density) {
      phase = 2;
      converged = true;
      return TEXO_GP_OK;
    }
    if (I.m.params.engine == TEXO_GP_ENGINE_DEVICE) return run_device(budget);
    const uint32_t K = I.m.K;
    if (phase == 0) {
      completed = (uint32_t)iter_offset;
      lambda.assign(K, 0.0);
      e0.assign(K, 1.0);
      TRY(push_inputs());
      EvalRec probe;
      TRY(evaluate(I.bufX, I.gX, I.m.gamma_base_tiles(), false, probe));
      TRY(validate_initial(probe));
      double g0;
      TRY(adaptive_gamma(probe, g0));
      EvalRec initial;
      TRY(evaluate(I.bufX, I.gX, g0, true, initial));
      TRY(validate_initial(initial));
      for (uint32_t f = 0; f < K; ++f) e0[f] = fixed_scales.empty() ? std::fmax(initial.energy[f], 1.0) : fixed_scales[f];
      TRY(validate_fields(initial));
      CU(cudaMemcpyAsync(I.bufXp, I.bufX, (size_t)I.d.nobj * sizeof(float2), cudaMemcpyDeviceToDevice, I.stream));
      TRY(save_best());
      excess(initial, best_max, best_tot);
      density_at_x = true;
      current = initial;
      gamma = g0;
      phase = 1;
      if (stop_reached(initial)) {
        phase = 2;
        converged = true;
        return TEXO_GP_OK;
      }
      if (reset_mult) {
        TRY(area_multipliers(initial));
      } else {
        // initial_density_multiplier (eplace.rs:1126-1148)
        double dens = 0.0;
        for (uint32_t f = 0; f < K; ++f) dens += initial.rawl1[f];
        const double m0 =
            (initial.wal1 == 0.0 || dens == 0.0) ? 1.0 : I.m.params.initial_density_weight * initial.wal1 / dens;
        if (!(std::isfinite(m0) && m0 > 0.0)) return TEXO_GP_ERR_INVALID_NORMALIZATION;
        lambda.assign(K, m0);
        mstep = I.m.params.alpha_high - 1.0;
      }
      TRY(push_inputs());
    }
    uint32_t done_now = 0;
    for (;;) {
      if (stop_reached(current)) {
        converged = true;
        phase = 2;
        break;
      }
      if (completed >= I.m.params.max_iterations) {
        exhausted = true;
        phase = 2;
        final_status = I.m.params.best_effort ? TEXO_GP_OK : TEXO_GP_ERR_DID_NOT_CONVERGE;
        break;
      }
      if (budget && done_now >= budget) break;
      double gam;
      TRY(adaptive_gamma(current, gam));
      completed++;
      done_now++;
      gamma = gam;
      EvalRec payload;
      bool stationary = false;
      const uint64_t trials_before = trials;
      TRY(nesterov_step(gam, payload, stationary));
      TRY(validate_fields(payload));
      current = payload;
      if (trace.size() < kTraceMax) {
        texo_gp_iteration rec{};
        rec.iteration = completed;
        rec.trials = (uint32_t)(trials - trials_before);
        rec.gamma = gam;
        rec.objective = current.value;
        rec.lipschitz = has_L ? L : 0.0;
        rec.momentum = a;
        for (uint32_t f = 0; f < K && f < TEXO_GP_MAX_FIELDS; ++f) {
          rec.lambda[f] = lambda[f];
          rec.energy_scale[f] = e0[f];
          rec.overflow[f] = current.overflow[f];
        }
        trace.push_back(rec);
      }
      double mx, tot;
      excess(current, mx, tot);
      if (mx < best_max || (mx == best_max && tot < best_tot)) {
        TRY(save_best());
        best_max = mx;
        best_tot = tot;
      }
      if (stop_reached(current)) {
        converged = true;
        phase = 2;
        break;
      }
      if (!stationary) {
        have_prev_stationary = false;
      } else {
        CU(cudaMemsetAsync(I.mismatch, 0, sizeof(unsigned long long), I.stream));
        launch_round_compare(I.d, I.bufX, I.prev_targets, (int)I.m.W, (int)I.m.H, I.mismatch, I.nvb, I.stream);
        unsigned long long mm = 0;
        CU(cudaMemcpyAsync(&mm, I.mismatch, sizeof(mm), cudaMemcpyDeviceToHost, I.stream));
        CU(cudaStreamSynchronize(I.stream));
        const bool fixed = have_prev_stationary && mm == 0;
        have_prev_stationary = true;
        if (fixed) {
          exhausted = true;
          phase = 2;
          final_status = I.m.params.best_effort ? TEXO_GP_OK : TEXO_GP_ERR_DID_NOT_CONVERGE;
          break;
        }
      }
      TRY(update_multipliers(current));
      TRY(push_inputs());
    }
    return phase == 2 ? final_status : TEXO_GP_OK;
  }
};

}  // namespace tgp

using namespace tgp;

struct texo_gp_handle_s {
  std::unique_ptr<Instance> inst;
  std::unique_ptr<Controller> ctl;
  std::mutex mu;
};

namespace tgp {
int32_t batch_stage_in(texo_gp_handle_s* h, uint32_t budget, cudaStream_t s, InstDesc* desc, bool* large) {
  Instance& I = *h->inst;
  Controller& C = *h->ctl;
  C.prepare_devrun();
  C.hr.budget = budget;
  std::memset(&I.h_run->bar, 0, sizeof(GridBarrier));
  CU(cudaMemcpyAsync(I.run_dev, I.h_run, sizeof(RunBlock), cudaMemcpyHostToDevice, s));
  desc->d = I.d;
  desc->r = I.r;
  desc->B = C.buffers();
  desc->run = &I.run_dev->run;
  desc->bar = &I.run_dev->bar;
  desc->V = I.nvb;
  desc->pad = 0;
  *large = I.d.dct_large != 0;
  return TEXO_GP_OK;
}
// The host half of batch_stage_in (no copy): the controller state in the
// pinned mirror, and where the mirror and its device copy live.
void batch_stage_host(texo_gp_handle_s* h, uint32_t budget, InstDesc* desc, bool* large, RunBlock** host,
                      RunBlock** dev) {
  Instance& I = *h->inst;
  Controller& C = *h->ctl;
  C.prepare_devrun();
  C.hr.budget = budget;
  std::memset(&I.h_run->bar, 0, sizeof(GridBarrier));
  desc->d = I.d;
  desc->r = I.r;
  desc->B = C.buffers();
  desc->run = &I.run_dev->run;
  desc->bar = &I.run_dev->bar;
  desc->V = I.nvb;
  desc->pad = 0;
  *large = I.d.dct_large != 0;
  *host = I.h_run;
  *dev = I.run_dev;
}
int32_t batch_stage_out(texo_gp_handle_s* h, cudaStream_t s) {
  Instance& I = *h->inst;
  CU(cudaMemcpyAsync(I.h_run, I.run_dev, sizeof(RunBlock), cudaMemcpyDeviceToHost, s));
  return TEXO_GP_OK;
}
bool batch_timed_out(texo_gp_handle_s* h) { return h->inst->h_run->bar.error != 0; }
int32_t batch_absorb(texo_gp_handle_s* h) { return h->ctl->absorb_devrun(); }
bool handle_finished(texo_gp_handle_s* h) { return h->ctl->phase == 2; }
uint64_t handle_bytes(texo_gp_handle_s* h) { return h->inst->bytes; }
int handle_virtual_blocks(texo_gp_handle_s* h) { return h->inst->nvb; }
uint64_t handle_work(texo_gp_handle_s* h) {
  const HostModel& m = h->inst->m;
  return (uint64_t)m.U + m.F + m.Mm + m.pin_unit.size() + 2ull * m.K * m.bins();
}
int handle_sms(texo_gp_handle_s* h) { return h->inst->sms; }
Instance* handle_instance(texo_gp_handle_s* h) { return h->inst.get(); }
int32_t handle_build(const texo_gp_problem* p, const texo_gp_params* prm, texo_gp_handle_s** out,
                     uint64_t* err_index) {
  *out = nullptr;
  texo_gp_params defaults;
  if (!prm) {
    texo_gp_default_params(&defaults);
    prm = &defaults;
  }
  if (!p) return TEXO_GP_ERR_INVALID_ARGUMENT;
  if (prm->dct_mode != TEXO_GP_DCT_FP32 && prm->dct_mode != TEXO_GP_DCT_TENSOR &&
      prm->dct_mode != TEXO_GP_DCT_FP32_GEMM)
    return TEXO_GP_ERR_INVALID_ARGUMENT;
  if (prm->scatter_mode < TEXO_GP_SCATTER_AUTO || prm->scatter_mode > TEXO_GP_SCATTER_TILED)
    return TEXO_GP_ERR_INVALID_ARGUMENT;
  if (prm->dct_mode == TEXO_GP_DCT_TENSOR && prm->engine == TEXO_GP_ENGINE_DEVICE) {
    set_last_error("the tensor-core DCT runs with the host engine only");
    return TEXO_GP_ERR_UNSUPPORTED;
  }
  auto h = std::make_unique<texo_gp_handle_s>();
  h->inst = std::make_unique<Instance>();
  h->inst->device = prm->device;
  uint64_t err = 0;
  const int32_t s = build_model(p, prm, h->inst->m, &err);
  if (err_index) *err_index = err;
  if (s) return s;
  *out = h.release();
  return TEXO_GP_OK;
}
uint64_t handle_device_bytes(texo_gp_handle_s* h) { return h->inst->device_bytes(); }
int32_t handle_upload(texo_gp_handle_s* h) {
  TRY(h->inst->upload());
  h->ctl = std::make_unique<Controller>(*h->inst);
  return TEXO_GP_OK;
}
std::mutex* handle_mutex(texo_gp_handle_s* h) { return &h->mu; }
}  // namespace tgp

namespace {
// The autotuner: times the four DCT passes of every admissible form on this
// instance (5 repetitions after a warm-up, CUDA events on its stream) and
// keeps the fastest. The FP32 tile families are always admissible; the
// tensor-core form only when the caller asked for it (the FP32 forms are
// more accurate, so they may replace it). Choices are cached per device,
// grid, field count, engine and requested mode.
int32_t autotune_dct(Instance& I) {
  struct Form {
    int large, tc, fft;
  };
  const texo_gp_params& prm = I.m.params;
  std::vector<Form> forms = {{0, 0, 0}, {1, 0, 0}};
  if (fft_length(I.m.Wb) && fft_length(I.m.Hb) && prm.dct_mode != TEXO_GP_DCT_FP32_GEMM) forms.push_back({0, 0, 1});
  if (prm.dct_mode == TEXO_GP_DCT_TENSOR && prm.engine == TEXO_GP_ENGINE_HOST) forms.push_back({0, 1, 0});
  static std::mutex mu;
  static std::map<std::tuple<int, uint32_t, uint32_t, uint32_t, int, int>, Form> cache;
  const auto key = std::make_tuple(I.device, I.m.Wb, I.m.Hb, I.m.K, prm.engine, prm.dct_mode);
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(key);
    if (it != cache.end()) {
      I.d.dct_large = it->second.large;
      I.d.tc = it->second.tc;
      I.d.fft = it->second.fft;
      return TEXO_GP_OK;
    }
  }
  cudaEvent_t a, b;
  CU(cudaEventCreate(&a));
  CU(cudaEventCreate(&b));
  float best = 1e30f;
  Form pick = forms[0];
  for (const Form& f : forms) {
    Dev D = I.d;
    D.dct_large = f.large;
    D.tc = f.tc;
    D.fft = f.fft;
    float t = 1e30f;
    for (int rep = 0; rep < 6; ++rep) {
      CU(cudaEventRecord(a, I.stream));
      for (int st = 0; st < 4; ++st) launch_dct(D, I.r, st, I.nvb, I.stream, &I.tmaps);
      CU(cudaEventRecord(b, I.stream));
      CU(cudaEventSynchronize(b));
      float ms = 0.f;
      CU(cudaEventElapsedTime(&ms, a, b));
      if (rep > 0) t = std::min(t, ms);   // the first run is a warm-up
    }
    if (t < best) {
      best = t;
      pick = f;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  CU(cudaMemsetAsync(I.r.iscal + SI_TC_FAIL, 0, sizeof(long long), I.stream));
  CU(cudaStreamSynchronize(I.stream));
  I.d.dct_large = pick.large;
  I.d.tc = pick.tc;
  I.d.fft = pick.fft;
  std::lock_guard<std::mutex> lk(mu);
  cache[key] = pick;
  return TEXO_GP_OK;
}

// The wirelength part of the autotuner: the lanes a net of each degree class
// (2 | 3-4 | 5-8 | 9-16 | 17-32 | 33+ pins) gets in the WA stage. The fixed
// table gives every lane at most four pins of a net (held in registers); the
// candidates trade lanes for pins per lane: two (more lanes, shorter shuffle
// trees) or eight (fewer lanes, pins beyond four read again). Each table is
// timed on the instance (init + WA at its coordinates, both engines run the
// same WA stage) and the fastest kept, cached per (device, class sizes,
// virtual blocks). The per-net sums then run over a different lane count, so
// WA values and gradients change by FP32 rounding (within the 1e-5 bounds)
// with the table; a given table gives bit-identical results run to run.
int32_t autotune_wa(Instance& I) {
  static const int tables[3][6] = {{1, 1, 2, 4, 8, 32}, {1, 2, 4, 8, 32, 32}, {1, 1, 1, 2, 4, 32}};
  HostModel& m = I.m;
  if (m.n_classes < 6) return TEXO_GP_OK;
  static std::mutex mu;
  static std::map<std::vector<long long>, int> cache;
  std::vector<long long> key = {I.device, I.nvb};
  for (int c = 0; c <= m.n_classes; ++c) key.push_back(m.class_begin[c]);
  auto apply = [&](int t) {
    for (int c = 0; c < 6; ++c) {
      m.class_group[c] = tables[t][c];
      I.d.class_group[c] = tables[t][c];
    }
    wa_lane_split(m.class_begin, m.class_group, m.n_classes, (long long)I.nvb * kThreads, I.d.class_lane);
  };
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(key);
    if (it != cache.end()) {
      apply(it->second);
      return TEXO_GP_OK;
    }
  }
  cudaEvent_t a, b;
  CU(cudaEventCreate(&a));
  CU(cudaEventCreate(&b));
  float best = 1e30f;
  int pick = 0;
  const double gamma = m.gamma_base_tiles();
  for (int t = 0; t < 3; ++t) {
    apply(t);
    float tm = 1e30f;
    for (int rep = 0; rep < 6; ++rep) {
      CU(cudaEventRecord(a, I.stream));
      launch_init(I.d, false, true, I.nvb, I.stream);
      launch_wa(I.d, I.r, I.bufX, gamma, I.nvb, I.stream);
      CU(cudaEventRecord(b, I.stream));
      CU(cudaEventSynchronize(b));
      float ms = 0.f;
      CU(cudaEventElapsedTime(&ms, a, b));
      if (rep > 0) tm = std::min(tm, ms);   // the first run is a warm-up
    }
    if (tm < best) {
      best = tm;
      pick = t;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  CU(cudaStreamSynchronize(I.stream));
  apply(pick);
  std::lock_guard<std::mutex> lk(mu);
  cache[key] = pick;
  return TEXO_GP_OK;
}

// The scatter half of the autotuner (host engine, scatter_mode AUTO): times
// the direct and the tiled scatter (init + scatter, and for the tiled form its
// counting sort) at spread coordinates (every object uniform in its bounds,
// as a placement near convergence is, from a fixed hash) and keeps the faster,
// cached per (device, grid, fields, objects). The grids both forms produce
// are identical, so the choice changes the time only.
int32_t autotune_scatter(Instance& I) {
  const texo_gp_params& prm = I.m.params;
  if (prm.engine != TEXO_GP_ENGINE_HOST || prm.scatter_mode != TEXO_GP_SCATTER_AUTO || !I.m.has_density)
    return TEXO_GP_OK;
  static std::mutex mu;
  static std::map<std::tuple<int, uint32_t, uint32_t, uint32_t, uint64_t>, int> cache;
  const auto key = std::make_tuple(I.device, I.m.Wb, I.m.Hb, I.m.K, (uint64_t)I.m.Mm + I.m.F);
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(key);
    if (it != cache.end()) {
      I.d.scatter_tiles = it->second;
      return TEXO_GP_OK;
    }
  }
  launch_spread_positions(I.d, I.bufC, I.nvb, I.stream);
  cudaEvent_t a, b;
  CU(cudaEventCreate(&a));
  CU(cudaEventCreate(&b));
  float best = 1e30f;
  int pick = 0;
  for (int form = 0; form < 2; ++form) {
    Dev D = I.d;
    D.scatter_tiles = form;
    float t = 1e30f;
    for (int rep = 0; rep < 6; ++rep) {
      CU(cudaEventRecord(a, I.stream));
      launch_init(D, true, false, I.nvb, I.stream);
      launch_scatter(D, I.r, I.bufC, I.nvb, I.stream);
      CU(cudaEventRecord(b, I.stream));
      CU(cudaEventSynchronize(b));
      float ms = 0.f;
      CU(cudaEventElapsedTime(&ms, a, b));
      if (rep > 0) t = std::min(t, ms);   // the first run is a warm-up
    }
    if (t < best) {
      best = t;
      pick = form;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  CU(cudaStreamSynchronize(I.stream));
  I.d.scatter_tiles = pick;
  std::lock_guard<std::mutex> lk(mu);
  cache[key] = pick;
  return TEXO_GP_OK;
}

uint32_t round_coord(double v, uint32_t extent) {
  double r = std::round(v);
  r = r < 0.0 ? 0.0 : (r > (double)(extent - 1) ? (double)(extent - 1) : r);
  return (uint32_t)r;
}

int32_t handle_targets(texo_gp_handle h, uint32_t* out, double* coords, texo_gp_stats* st, int32_t status) {
  Instance& I = *h->inst;
  Controller& C = *h->ctl;
  const size_t nobj = (size_t)I.d.nobj;
  std::vector<float> best32(2 * (size_t)I.m.U), cur32(2 * nobj);
  std::vector<double> best(2 * (size_t)I.m.U), cur(2 * nobj);
  if (I.m.has_density)
    CU(cudaMemcpyAsync(best32.data(), I.best, best32.size() * sizeof(float), cudaMemcpyDeviceToHost, I.stream));
  CU(cudaMemcpyAsync(cur32.data(), I.bufX, cur32.size() * sizeof(float), cudaMemcpyDeviceToHost, I.stream));
  launch_hpwl(I.d, I.r, I.bufX, I.nvb, I.stream);
  launch_finalize(I.d, I.r, I.nvb, FIN_HPWL, I.stream);
  CU(cudaMemcpyAsync(I.h_scal + SC_HPWL, I.r.scal + SC_HPWL, sizeof(double), cudaMemcpyDeviceToHost, I.stream));
  CU(cudaStreamSynchronize(I.stream));
  for (size_t i = 0; i < best.size(); ++i) best[i] = I.m.has_density ? (double)best32[i] : I.m.init[i];
  for (size_t i = 0; i < cur.size(); ++i) cur[i] = cur32[i];
  if (out)
    for (uint32_t u = 0; u < I.m.U; ++u) {
      out[2 * (size_t)u] = round_coord(best[2 * (size_t)u], I.m.W);
      out[2 * (size_t)u + 1] = round_coord(best[2 * (size_t)u + 1], I.m.H);
    }
  if (coords) std::memcpy(coords, cur.data(), cur.size() * sizeof(double));
  if (st) {
    st->status = status;
    st->iterations = C.completed;
    st->evaluations = C.evaluations;
    st->density_evaluations = C.density_evaluations;
    st->line_search_trials = C.trials;
    st->num_fields = I.m.K;
    for (uint32_t f = 0; f < I.m.K && f < TEXO_GP_MAX_FIELDS; ++f) {
      st->overflow[f] = C.current.overflow[f];
      st->energy[f] = C.current.energy[f];
    }
    st->gamma = C.gamma;
    st->objective = C.last_objective;
    st->hpwl = I.h_scal[SC_HPWL];
    st->converged = C.converged ? 1 : 0;
    st->elapsed_ms = C.elapsed_ms;
    st->kernel_launches = C.launches;
  }
  return TEXO_GP_OK;
}
}  // namespace

extern "C" {

uint32_t texo_gp_abi_version(void) { return TEXO_GP_ABI_VERSION; }

void texo_gp_default_params(texo_gp_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->gamma_base = 8.0;
  p->max_iterations = 3000;
  p->beta = 2000.0;
  p->initial_density_weight = 1.0e-4;
  p->alpha_low = 1.05;
  p->alpha_high = 1.06;
  p->overflow_target_override = -1.0;
  p->target_density = 1.0;
  p->best_effort = 0;
  p->dct_mode = TEXO_GP_DCT_FP32;
  p->autotune = 0;
  p->engine = TEXO_GP_ENGINE_HOST;
  p->device = 0;
  p->objective_margin_ulps = 64.0;
}

const char* texo_gp_status_name(int32_t s) {
  switch (s) {
    case TEXO_GP_OK: return "OK";
    case TEXO_GP_ERR_EMPTY_GRID: return "EMPTY_GRID";
    case TEXO_GP_ERR_GRID_TOO_LARGE: return "GRID_TOO_LARGE";
    case TEXO_GP_ERR_DENSITY_LENGTH: return "DENSITY_LENGTH";
    case TEXO_GP_ERR_NONFINITE_DENSITY: return "NONFINITE_DENSITY";
    case TEXO_GP_ERR_EMPTY_UNIT: return "EMPTY_UNIT";
    case TEXO_GP_ERR_NONFINITE_UNIT_COORDINATE: return "NONFINITE_UNIT_COORDINATE";
    case TEXO_GP_ERR_INVALID_MEMBER_CHARGE: return "INVALID_MEMBER_CHARGE";
    case TEXO_GP_ERR_POINT_OUTSIDE_GRID: return "POINT_OUTSIDE_GRID";
    case TEXO_GP_ERR_FIXED_CAPACITY_EXHAUSTED: return "FIXED_CAPACITY_EXHAUSTED";
    case TEXO_GP_ERR_INSUFFICIENT_CAPACITY: return "INSUFFICIENT_CAPACITY";
    case TEXO_GP_ERR_INSUFFICIENT_AREA: return "INSUFFICIENT_AREA";
    case TEXO_GP_ERR_NONFINITE_FILLER: return "NONFINITE_FILLER";
    case TEXO_GP_ERR_NEGATIVE_FILLER_CHARGE: return "NEGATIVE_FILLER_CHARGE";
    case TEXO_GP_ERR_UNEXPECTED_FILLER_KIND: return "UNEXPECTED_FILLER_KIND";
    case TEXO_GP_ERR_FILLER_CHARGE_MISMATCH: return "FILLER_CHARGE_MISMATCH";
    case TEXO_GP_ERR_INVALID_BOUNDS: return "INVALID_BOUNDS";
    case TEXO_GP_ERR_INVALID_METRIC_LENGTH: return "INVALID_METRIC_LENGTH";
    case TEXO_GP_ERR_NONPOSITIVE_METRIC: return "NONPOSITIVE_METRIC";
    case TEXO_GP_ERR_INVALID_INITIAL_COORDINATE: return "INVALID_INITIAL_COORDINATE";
    case TEXO_GP_ERR_INVALID_MOMENTUM_PARAMETER: return "INVALID_MOMENTUM_PARAMETER";
    case TEXO_GP_ERR_INVALID_LIPSCHITZ_ESTIMATE: return "INVALID_LIPSCHITZ_ESTIMATE";
    case TEXO_GP_ERR_INVALID_OBJECTIVE: return "INVALID_OBJECTIVE";
    case TEXO_GP_ERR_INVALID_GRADIENT_LENGTH: return "INVALID_GRADIENT_LENGTH";
    case TEXO_GP_ERR_NONFINITE_GRADIENT: return "NONFINITE_GRADIENT";
    case TEXO_GP_ERR_LINE_SEARCH_OVERFLOW: return "LINE_SEARCH_OVERFLOW";
    case TEXO_GP_ERR_ITERATION_OVERFLOW: return "ITERATION_OVERFLOW";
    case TEXO_GP_ERR_EVALUATION: return "EVALUATION";
    case TEXO_GP_ERR_DENSITY_FIELD_CHANGED: return "DENSITY_FIELD_CHANGED";
    case TEXO_GP_ERR_INVALID_NORMALIZATION: return "INVALID_NORMALIZATION";
    case TEXO_GP_ERR_DID_NOT_CONVERGE: return "DID_NOT_CONVERGE";
    case TEXO_GP_ERR_INVALID_ARGUMENT: return "INVALID_ARGUMENT";
    case TEXO_GP_ERR_CUDA: return "CUDA";
    case TEXO_GP_ERR_OUT_OF_MEMORY: return "OUT_OF_MEMORY";
    case TEXO_GP_ERR_DEVICE_TIMEOUT: return "DEVICE_TIMEOUT";
    case TEXO_GP_ERR_FIXED_POINT_RANGE: return "FIXED_POINT_RANGE";
    case TEXO_GP_ERR_UNSUPPORTED: return "UNSUPPORTED";
    case TEXO_GP_ERR_BUSY: return "BUSY";
    case TEXO_GP_ERR_PCG_NOT_CONVERGED: return "PCG_NOT_CONVERGED";
    case TEXO_GP_ERR_AUCTION_RANGE: return "AUCTION_RANGE";
    case TEXO_GP_ERR_AUCTION_OBJECT_RANGE: return "AUCTION_OBJECT_RANGE";
    case TEXO_GP_ERR_AUCTION_COST_RANGE: return "AUCTION_COST_RANGE";
    case TEXO_GP_ERR_AUCTION_DUPLICATE_OBJECT: return "AUCTION_DUPLICATE_OBJECT";
    case TEXO_GP_ERR_INSTANCE_AREA_MEMBER: return "INSTANCE_AREA_MEMBER";
    case TEXO_GP_ERR_INSTANCE_AREA_FILLER: return "INSTANCE_AREA_FILLER";
    case TEXO_GP_ERR_INSTANCE_AREA_POSTCONDITION: return "INSTANCE_AREA_POSTCONDITION";
    case TEXO_GP_ERR_INSTANCE_AREA_OVERFLOW: return "INSTANCE_AREA_OVERFLOW";
    case TEXO_GP_ERR_PROJECTION_CONFLICT: return "PROJECTION_CONFLICT";
    case TEXO_GP_ERR_NO_BEL: return "NO_BEL";
    default: return "UNKNOWN";
  }
}

const char* texo_gp_last_error(void) { return g_last_error.c_str(); }

int32_t texo_gp_create(const texo_gp_problem* p, const texo_gp_params* prm, texo_gp_handle* out) {
  if (!out) return TEXO_GP_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  texo_gp_handle h = nullptr;
  TRY(tgp::handle_build(p, prm, &h, nullptr));
  int32_t s = tgp::handle_upload(h);
  if (!s && h->inst->m.params.autotune) s = autotune_dct(*h->inst);
  if (!s && h->inst->m.params.autotune) s = autotune_scatter(*h->inst);
  if (!s && h->inst->m.params.autotune) s = autotune_wa(*h->inst);
  if (s) {
    delete h;
    return s;
  }
  *out = h;
  return TEXO_GP_OK;
}

int32_t texo_gp_dct_form(texo_gp_handle h, int32_t* form) {
  if (!h || !form) return TEXO_GP_ERR_INVALID_ARGUMENT;
  const Dev& d = h->inst->d;
  *form = d.tc ? 2 : (d.fft ? 3 : (d.dct_large ? 1 : 0));
  return TEXO_GP_OK;
}

int32_t texo_gp_destroy(texo_gp_handle h) {
  if (!h) return TEXO_GP_ERR_INVALID_ARGUMENT;
  delete h;
  return TEXO_GP_OK;
}

int32_t texo_gp_sizes(texo_gp_handle h, uint64_t* units, uint64_t* fillers, uint64_t* coordinates,
                      uint32_t* bins_x, uint32_t* bins_y, uint32_t* num_fields) {
  if (!h) return TEXO_GP_ERR_INVALID_ARGUMENT;
  const HostModel& m = h->inst->m;
  if (units) *units = m.U;
  if (fillers) *fillers = m.F;
  if (coordinates) *coordinates = m.coords();
  if (bins_x) *bins_x = m.Wb;
  if (bins_y) *bins_y = m.Hb;
  if (num_fields) *num_fields = m.K;
  return TEXO_GP_OK;
}

int32_t texo_gp_initial(texo_gp_handle h, double* c, double* lo, double* hi) {
  if (!h) return TEXO_GP_ERR_INVALID_ARGUMENT;
  const HostModel& m = h->inst->m;
  const size_t n = m.coords();
  if (c) std::memcpy(c, m.init.data(), n * 8);
  if (lo) std::memcpy(lo, m.lo.data(), n * 8);
  if (hi) std::memcpy(hi, m.hi.data(), n * 8);
  return TEXO_GP_OK;
}

int32_t texo_gp_fillers(texo_gp_handle h, uint32_t* field, double* charge) {
  if (!h) return TEXO_GP_ERR_INVALID_ARGUMENT;
  const HostModel& m = h->inst->m;
  for (uint32_t j = 0; j < m.F; ++j) {
    if (field) field[j] = (uint32_t)m.fil_field[j];
    if (charge) charge[j] = m.fil_q[j];
  }
  return TEXO_GP_OK;
}

int32_t texo_gp_evaluate(texo_gp_handle h, const double* coordinates, double gamma, texo_gp_eval* out,
                         double* wa_gradient, double* field_gradient, double* density, double* potential) {
  if (!h || !coordinates || !(gamma > 0.0) || !std::isfinite(gamma)) return TEXO_GP_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(h->mu);
  Instance& I = *h->inst;
  Controller& C = *h->ctl;
  const size_t nobj = (size_t)I.d.nobj, B = I.m.bins(), K = I.m.K;
  for (size_t i = 0; i < 2 * nobj; ++i)
    if (!std::isfinite(coordinates[i])) return TEXO_GP_ERR_NONFINITE_UNIT_COORDINATE;
  TRY(upload_coords(I, I.bufY, coordinates, nobj));
  EvalRec e;
  TRY(C.evaluate(I.bufY, I.gY, gamma, false, e));
  C.density_at_x = false;
  if (out) {
    out->wirelength = e.wa;
    out->num_fields = (uint32_t)K;
    for (size_t f = 0; f < K; ++f) {
      out->fields[f].energy = e.energy[f];
      out->fields[f].normalized_overflow = e.overflow[f];
      out->fields[f].net_charge = e.net_charge[f];
      out->fields[f].force_l1 = e.force[f];
      out->fields[f].real_area = I.m.real_area[f];
      out->fields[f].filler_charge =
          I.m.td == 1.0 ? I.m.td * (double)I.m.available[f] - I.m.real_area[f]
                        : std::max(I.m.td * (double)I.m.available[f] - I.m.real_area[f], 0.0);
      out->fields[f].overflow_fixed = e.overflow_fixed[f];
      out->fields[f].overflow_bins = (uint64_t)e.overflow_bins[f];
    }
  }
  if (wa_gradient) {
    std::vector<long long> fix(2 * (size_t)I.m.U);
    CU(cudaMemcpyAsync(fix.data(), I.d.wa_fix, fix.size() * 8, cudaMemcpyDeviceToHost, I.stream));
    CU(cudaStreamSynchronize(I.stream));
    for (size_t i = 0; i < fix.size(); ++i) wa_gradient[i] = (double)fix[i] * kInvFix;
  }
  if (field_gradient) {
    std::vector<float2> g(K * nobj);
    CU(cudaMemcpyAsync(g.data(), I.d.graw, g.size() * sizeof(float2), cudaMemcpyDeviceToHost, I.stream));
    CU(cudaStreamSynchronize(I.stream));
    for (size_t f = 0; f < K; ++f)
      for (size_t o = 0; o < nobj; ++o) {
        bool valid = o < I.m.U || (size_t)I.m.fil_field[o - I.m.U] == f;
        const float2 v = valid ? g[f * nobj + o] : make_float2(0.f, 0.f);
        field_gradient[f * 2 * nobj + 2 * o] = v.x;
        field_gradient[f * 2 * nobj + 2 * o + 1] = v.y;
      }
  }
  if (density) {
    std::vector<long long> a(K * B), b(K * B);
    CU(cudaMemcpyAsync(a.data(), I.d.phys, a.size() * 8, cudaMemcpyDeviceToHost, I.stream));
    CU(cudaMemcpyAsync(b.data(), I.d.fill, b.size() * 8, cudaMemcpyDeviceToHost, I.stream));
    CU(cudaStreamSynchronize(I.stream));
    for (size_t i = 0; i < K * B; ++i) density[i] = (double)(a[i] + b[i]) * kInvFix;
  }
  if (potential) {
    std::vector<float> p(K * B);
    CU(cudaMemcpyAsync(p.data(), I.d.phi, p.size() * 4, cudaMemcpyDeviceToHost, I.stream));
    CU(cudaStreamSynchronize(I.stream));
    for (size_t i = 0; i < K * B; ++i) potential[i] = p[i];
  }
  return TEXO_GP_OK;
}

int32_t texo_gp_scatter(texo_gp_handle h, const double* coordinates, int64_t* physical, int64_t* fillers) {
  if (!h || !coordinates) return TEXO_GP_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(h->mu);
  Instance& I = *h->inst;
  const size_t nobj = (size_t)I.d.nobj, n = (size_t)I.m.K * I.m.bins();
  TRY(upload_coords(I, I.bufY, coordinates, nobj));
  launch_init(I.d, true, false, I.nvb, I.stream);
  launch_scatter(I.d, I.r, I.bufY, I.nvb, I.stream);
  if (physical) CU(cudaMemcpyAsync(physical, I.d.phys, n * 8, cudaMemcpyDeviceToHost, I.stream));
  if (fillers) CU(cudaMemcpyAsync(fillers, I.d.fill, n * 8, cudaMemcpyDeviceToHost, I.stream));
  CU(cudaStreamSynchronize(I.stream));
  CU(cudaGetLastError());
  h->ctl->density_at_x = false;
  return TEXO_GP_OK;
}

int32_t texo_gp_poisson(texo_gp_handle h, const double* density, double* potential, double* energy) {
  if (!h || !density) return TEXO_GP_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(h->mu);
  Instance& I = *h->inst;
  if (I.m.K == 0) return TEXO_GP_ERR_UNSUPPORTED;
  const size_t B = I.m.bins();
  double s = 0.0;
  for (size_t i = 0; i < B; ++i) {
    if (!std::isfinite(density[i])) return TEXO_GP_ERR_NONFINITE_DENSITY;
    s += density[i];
  }
  const double mean = s / (double)B;
  std::vector<float> rho(B);
  for (size_t i = 0; i < B; ++i) rho[i] = (float)(density[i] - mean);
  // Field 0's buffers carry the solve; K is forced to one for the call.
  Dev D = I.d;
  D.K = 1;
  CU(cudaMemcpyAsync(D.rho, rho.data(), B * 4, cudaMemcpyHostToDevice, I.stream));
  for (int st = 0; st < 4; ++st) launch_dct(D, I.r, st, I.nvb, I.stream, &I.tmaps);
  launch_finalize(D, I.r, I.nvb, FIN_ENERGY, I.stream);
  std::vector<float> phi(B);
  CU(cudaMemcpyAsync(phi.data(), D.phi, B * 4, cudaMemcpyDeviceToHost, I.stream));
  CU(cudaMemcpyAsync(I.h_scal, I.r.scal, kScalars * sizeof(double), cudaMemcpyDeviceToHost, I.stream));
  CU(cudaMemcpyAsync(I.h_iscal, I.r.iscal, kIScalars * sizeof(long long), cudaMemcpyDeviceToHost, I.stream));
  CU(cudaStreamSynchronize(I.stream));
  CU(cudaGetLastError());
  if (I.h_iscal[SI_TC_FAIL]) {
    set_last_error("tensor-core DCT: an mbarrier wait ran out");
    return TEXO_GP_ERR_DEVICE_TIMEOUT;
  }
  if (potential)
    for (size_t i = 0; i < B; ++i) potential[i] = phi[i];
  if (energy) *energy = I.h_scal[SC_ENERGY];
  h->ctl->density_at_x = false;
  return TEXO_GP_OK;
}

int32_t texo_gp_run(texo_gp_handle h, uint32_t max_iterations, uint32_t* out_targets, double* out_coords,
                    texo_gp_stats* stats) {
  if (!h) return TEXO_GP_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(h->mu);
  Controller& C = *h->ctl;
  Instance& I = *h->inst;
  cudaEvent_t e0, e1;
  CU(cudaEventCreate(&e0));
  CU(cudaEventCreate(&e1));
  const unsigned long long l0 = launches_issued();
  CU(cudaEventRecord(e0, I.stream));
  C.device_ms = -1.0;
  int32_t s = C.run(max_iterations);
  cudaEventRecord(e1, I.stream);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  // the device engine times its one step (state in, kernel, state out) on
  // the stream itself; the host engine's call is timed whole
  C.elapsed_ms = C.device_ms >= 0.0 ? C.device_ms : ms;
  C.launches = launches_issued() - l0;
  if (s != TEXO_GP_OK && s != TEXO_GP_ERR_DID_NOT_CONVERGE) {
    if (stats) {
      std::memset(stats, 0, sizeof(*stats));
      stats->status = s;
      stats->iterations = C.completed;
    }
    return s;
  }
  int32_t t = handle_targets(h, out_targets, out_coords, stats, s);
  return t ? t : s;
}

int32_t texo_gp_set_charges(texo_gp_handle h, const double* member_charge, const double* filler_charge) {
  if (!h) return TEXO_GP_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(h->mu);
  Instance& I = *h->inst;
  HostModel& m = I.m;
  const size_t nobj = (size_t)m.U + m.F;
  if (member_charge)
    for (uint32_t i = 0; i < m.Mm; ++i)
      if (!std::isfinite(member_charge[i]) || member_charge[i] <= 0.0) {
        set_last_error("texo_gp_set_charges: member " + std::to_string(i));
        return TEXO_GP_ERR_INVALID_MEMBER_CHARGE;
      }
  if (filler_charge)
    for (uint32_t j = 0; j < m.F; ++j) {
      if (!std::isfinite(filler_charge[j])) return TEXO_GP_ERR_NONFINITE_FILLER;
      if (filler_charge[j] < 0.0) return TEXO_GP_ERR_NEGATIVE_FILLER_CHARGE;
    }
  if (member_charge) {
    m.real_area.assign(m.K, 0.0);
    for (uint32_t i = 0; i < m.Mm; ++i) {
      m.mem_q[i] = (float)member_charge[i];
      m.real_area[m.mem_field[i]] += member_charge[i];
    }
  }
  if (filler_charge)
    for (uint32_t j = 0; j < m.F; ++j) m.fil_q[j] = filler_charge[j];
  // per-field charge of every optimizer object (the preconditioner's)
  std::fill(m.pre_q.begin(), m.pre_q.end(), 0.0);
  for (uint32_t u = 0; u < m.U; ++u)
    for (int i = m.unit_mem_ptr[u]; i < m.unit_mem_ptr[u + 1]; ++i)
      m.pre_q[(size_t)m.mem_field[i] * nobj + u] += member_charge ? member_charge[i] : (double)m.mem_q[i];
  for (uint32_t j = 0; j < m.F; ++j) m.pre_q[(size_t)m.fil_field[j] * nobj + m.U + j] = m.fil_q[j];
  std::vector<float> fq(m.F), pq(m.pre_q.size());
  for (uint32_t j = 0; j < m.F; ++j) fq[j] = (float)m.fil_q[j];
  for (size_t i = 0; i < pq.size(); ++i) pq[i] = (float)m.pre_q[i];
  Dev& D = I.d;
  if (m.Mm) CU(cudaMemcpyAsync((void*)D.mem_q, m.mem_q.data(), m.Mm * sizeof(float), cudaMemcpyHostToDevice, I.stream));
  if (m.F) CU(cudaMemcpyAsync((void*)D.fil_q, fq.data(), m.F * sizeof(float), cudaMemcpyHostToDevice, I.stream));
  if (!pq.empty())
    CU(cudaMemcpyAsync((void*)D.pre_q, pq.data(), pq.size() * sizeof(float), cudaMemcpyHostToDevice, I.stream));
  for (uint32_t f = 0; f < m.K; ++f) I.h_scal[SC_REAL_AREA + f] = m.real_area[f];
  CU(cudaMemcpyAsync(I.r.scal + SC_REAL_AREA, I.h_scal + SC_REAL_AREA, m.K * sizeof(double), cudaMemcpyHostToDevice,
                     I.stream));
  CU(cudaStreamSynchronize(I.stream));
  return TEXO_GP_OK;
}

int32_t texo_gp_optimize_round(texo_gp_handle h, const texo_gp_round* round, uint32_t* out_targets,
                               double* out_coords, texo_gp_stats* stats, texo_gp_round_result* result) {
  if (!h || !round) return TEXO_GP_ERR_INVALID_ARGUMENT;
  if (round->stop != 0 && round->stop != 1) return TEXO_GP_ERR_INVALID_ARGUMENT;
  {
    std::lock_guard<std::mutex> lk(h->mu);
    Instance& I = *h->inst;
    // a fresh controller (Nesterov state, multipliers, checkpoint) from the
    // handle's current coordinates
    auto c = std::make_unique<Controller>(I);
    c->stop_mode = round->stop;
    c->reset_mult = round->reset_multipliers != 0;
    c->iter_offset = round->completed_iterations;
    if (round->density_scales) c->fixed_scales.assign(round->density_scales, round->density_scales + I.m.K);
    h->ctl = std::move(c);
    CU(cudaMemsetAsync(I.prev_targets, 0, 2 * (size_t)I.m.U * 4, I.stream));
  }
  const int32_t s = texo_gp_run(h, 0, out_targets, out_coords, stats);
  if (result) {
    std::lock_guard<std::mutex> lk(h->mu);
    const Controller& C = *h->ctl;
    std::memset(result, 0, sizeof(*result));
    result->completed_iterations = C.completed;
    result->exhausted = C.exhausted ? 1u : 0u;
    for (size_t f = 0; f < C.e0.size() && f < TEXO_GP_MAX_FIELDS; ++f) result->density_scales[f] = C.e0[f];
  }
  return s;
}

int32_t texo_gp_reset(texo_gp_handle h) {
  if (!h) return TEXO_GP_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(h->mu);
  Instance& I = *h->inst;
  h->ctl = std::make_unique<Controller>(I);
  TRY(upload_coords(I, I.bufX, I.m.init.data(), (size_t)I.d.nobj));
  CU(cudaMemsetAsync(I.prev_targets, 0, 2 * (size_t)I.m.U * 4, I.stream));
  CU(cudaStreamSynchronize(I.stream));
  return TEXO_GP_OK;
}

int32_t texo_gp_trace(texo_gp_handle h, texo_gp_iteration* out, uint32_t capacity, uint32_t* count) {
  if (!h || !count || (capacity && !out)) return TEXO_GP_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(h->mu);
  const auto& tr = h->ctl->trace;
  const uint32_t n = (uint32_t)std::min<size_t>(tr.size(), capacity);
  if (n) std::memcpy(out, tr.data(), n * sizeof(texo_gp_iteration));
  *count = (uint32_t)tr.size();
  return TEXO_GP_OK;
}

int32_t texo_gp_hpwl(texo_gp_handle h, const double* coordinates, double* hpwl) {
  if (!h || !coordinates || !hpwl) return TEXO_GP_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(h->mu);
  Instance& I = *h->inst;
  TRY(upload_coords(I, I.bufY, coordinates, (size_t)I.d.nobj));
  launch_hpwl(I.d, I.r, I.bufY, I.nvb, I.stream);
  launch_finalize(I.d, I.r, I.nvb, FIN_HPWL, I.stream);
  CU(cudaMemcpyAsync(I.h_scal + SC_HPWL, I.r.scal + SC_HPWL, sizeof(double), cudaMemcpyDeviceToHost, I.stream));
  CU(cudaStreamSynchronize(I.stream));
  *hpwl = I.h_scal[SC_HPWL];
  return TEXO_GP_OK;
}

static const char* kStageNames[] = {"init", "scatter", "wa", "prep", "dct_row_fwd", "dct_col_fwd",
                                     "dct_col_inv", "dct_row_inv", "gather", "combine", "finalize",
                                     "extrapolate", "candidate", "kkt", "precond"};
constexpr uint32_t kNumStages = sizeof(kStageNames) / sizeof(kStageNames[0]);

const char* texo_gp_stage_name(uint32_t i) { return i < kNumStages ? kStageNames[i] : nullptr; }

int32_t texo_gp_stage_times(texo_gp_handle h, uint32_t reps, double* ms, uint32_t capacity, uint32_t* count) {
  if (!h || !ms || reps == 0) return TEXO_GP_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(h->mu);
  Instance& I = *h->inst;
  const Dev& D = I.d;
  cudaStream_t s = I.stream;
  const int nvb = I.nvb;
  if (count) *count = kNumStages;
  cudaEvent_t a, b;
  CU(cudaEventCreate(&a));
  CU(cudaEventCreate(&b));
  const double gam = I.m.gamma_base_tiles();
  // one evaluation first so that every input of every stage is populated
  h->ctl->enqueue_eval(I.bufX, I.gX, gam, false);
  launch_precond(D, I.r, nvb, s);
  for (uint32_t st = 0; st < kNumStages && st < capacity; ++st) {
    CU(cudaStreamSynchronize(s));
    CU(cudaEventRecord(a, s));
    for (uint32_t k = 0; k < reps; ++k) {
      switch (st) {
        case 0: launch_init(D, true, true, nvb, s); break;
        case 1: launch_scatter(D, I.r, I.bufX, nvb, s); break;
        case 2: launch_wa(D, I.r, I.bufX, gam, nvb, s); break;
        case 3: launch_prep(D, I.r, nvb, s); break;
        case 4: case 5: case 6: case 7: launch_dct(D, I.r, (int)st - 4, nvb, s, &I.tmaps); break;
        case 8: launch_gather(D, I.r, I.bufX, nvb, s); break;
        case 9: launch_combine(D, I.r, I.gX, nvb, s); break;
        case 10: launch_finalize(D, I.r, nvb, FIN_ENERGY | FIN_COMBINE, s); break;
        case 11: launch_extrapolate(D, I.r, I.bufX, I.bufXp, 0.5, I.bufY, nvb, s); break;
        case 12: launch_candidate(D, I.r, I.bufX, I.gX, 1.0, I.bufC, nvb, s); break;
        case 13: launch_kkt(D, I.r, I.bufX, I.gX, I.bufXp, nvb, s); break;
        default: launch_precond(D, I.r, nvb, s); break;
      }
    }
    CU(cudaEventRecord(b, s));
    CU(cudaEventSynchronize(b));
    float t = 0.f;
    CU(cudaEventElapsedTime(&t, a, b));
    ms[st] = (double)t / reps;
    // restore the accumulation grids that repeated launches disturbed
    if (st == 1 || st == 2) h->ctl->enqueue_eval(I.bufX, I.gX, gam, false);
  }
  CU(cudaStreamSynchronize(s));
  CU(cudaGetLastError());
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  h->ctl->density_at_x = false;
  return TEXO_GP_OK;
}

int32_t texo_gp_device_profile(texo_gp_handle h, double out[10]) {
  if (!h || !out) return TEXO_GP_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(h->mu);
  const DevRun& hr = h->ctl->hr;
  for (int i = 0; i < 8; ++i) out[i] = hr.phase_ns[i] * 1e-3;
  out[8] = hr.barrier_wait_ns * 1e-3;
  out[9] = (double)hr.barriers;
  return TEXO_GP_OK;
}

int32_t texo_gp_place(const texo_gp_problem* p, const texo_gp_params* prm, uint32_t* out_targets, double* out_coords,
                      texo_gp_stats* stats) {
  texo_gp_handle h = nullptr;
  int32_t s = texo_gp_create(p, prm, &h);
  if (s) {
    if (stats) {
      std::memset(stats, 0, sizeof(*stats));
      stats->status = s;
    }
    return s;
  }
  s = texo_gp_run(h, 0, out_targets, out_coords, stats);
  texo_gp_destroy(h);
  return s;
}

}  // extern "C"
