// dct_fft.cuh — the spectral Poisson solve as FFT-based DCTs (FP32), for
// power-of-two bin grids.
//
// The orthonormal DCT-II of a real vector x of length n is computed with
// Makhoul's reordering (IEEE TASSP 28(1), 1980): v = (x0, x2, x4, ...,
// x5, x3, x1), V = FFT_n(v), X_k = s_k Re(exp(-i pi k / 2n) V_k) with
// s_0 = sqrt(1/n), s_k = sqrt(2/n). The inverse (DCT-III) forms
// W_k = exp(-i pi k / 2n) (X_k / s_k + i X_{n-k} / s_{n-k}) (X_n = 0), takes
// F = FFT_n(W) and reads x_{2j} = Re F_j / n, x_{2j+1} = Re F_{n-1-j} / n.
// The FFT is an in-place radix-2 decimation-in-time transform in shared
// memory over a group of vectors stored back to back, fed in bit-reversed
// order. Twiddles come from FP64 tables rounded to FP32.
//
// The 2-D solve t1 = rows-DCT(rho), t2 = cols-IDCT(cols-DCT(t1) / lambda),
// phi = rows-IDCT(t2) takes three passes: the column pass owns whole
// columns, so the forward transform, the inverse-eigenvalue scaling and the
// inverse transform run back to back in shared memory.
#pragma once
#include "stages.cuh"

namespace tgp {
namespace fft {

constexpr int kBuf = 2048;                       // complex slots of the work buffer (16 KB)
constexpr int kPer = kBuf / kThreads;            // slots per thread

struct Smem {
  float2 buf[kBuf];
};

// Tables of one transform length n (a power of two).
struct Axis {
  const float2* tw;      // [n/2] exp(-2 pi i j / n)
  const float2* post;    // [n]   s_k exp(-i pi k / 2n)
  const float2* pre;     // [n]   exp(-i pi k / 2n)
  const float* inv_s;    // [n]   1 / s_k
  int n, logn;
};

__device__ __forceinline__ Axis axis_x(const Dev& d) {
  return Axis{d.fx_tw, d.fx_post, d.fx_pre, d.fx_inv_s, d.g.Wb, d.logW};
}
__device__ __forceinline__ Axis axis_y(const Dev& d) {
  return Axis{d.fy_tw, d.fy_post, d.fy_pre, d.fy_inv_s, d.g.Hb, d.logH};
}

// Up to 256 points the data of a group takes at most 1024 slots of the work
// buffer, and the tables (n/2 twiddles, n post and n pre factors, n 1/s_k)
// are copied into the other 1024 once per pass: the stages then read their
// twiddles from shared memory instead of making an L2 round trip per stage
// (the persistent kernel's grid barriers leave L1 cold).
constexpr int kTableLog = 8;
__device__ __forceinline__ Axis stage_tables(const Axis& a, float2* buf) {
  if (a.logn > kTableLog) return a;
  float2* tw = buf + kBuf / 2;
  float2* post = tw + (a.n >> 1);
  float2* pre = post + a.n;
  float* inv_s = reinterpret_cast<float*>(pre + a.n);
  __syncthreads();   // earlier readers of the buffer are done
  for (int i = threadIdx.x; i < a.n; i += blockDim.x) {
    if (i < (a.n >> 1)) tw[i] = a.tw[i];
    post[i] = a.post[i];
    pre[i] = a.pre[i];
    inv_s[i] = a.inv_s[i];
  }
  __syncthreads();
  return Axis{tw, post, pre, inv_s, a.n, a.logn};
}

// Vectors transformed together: one butterfly per thread per stage (n/2
// butterflies per vector), at least one vector; many small groups keep every
// SM busy on small grids.
__device__ __forceinline__ int group_size(int logn) { return max(1, (2 * kThreads) >> logn); }

__device__ __forceinline__ int brev(int m, int logn) {
  return logn ? (int)(__brev((unsigned)m) >> (32 - logn)) : 0;
}
// position of sample i in Makhoul's order (and, for the inverse, the FFT
// output index that holds sample i)
__device__ __forceinline__ int mak(int i, int n) { return (i & 1) ? n - 1 - (i >> 1) : (i >> 1); }

// In-place radix-2 DIT over G vectors of length n (bit-reversed input).
__device__ __forceinline__ void stages(float2* buf, int G, const Axis& a) {
  const int half_n = a.n >> 1, total = G * half_n;
  for (int s = 0; s < a.logn; ++s) {
    const int half = 1 << s, step = half_n >> s;
    __syncthreads();
    for (int b = threadIdx.x; b < total; b += blockDim.x) {
      const int g = b >> (a.logn - 1), j = b & (half_n - 1);
      const int jj = j & (half - 1);
      float2* p = buf + (g << a.logn) + ((j >> s) << (s + 1)) + jj;
      const float2 w = a.tw[jj * step];
      const float2 u = p[0], v = p[half];
      const float2 t = make_float2(v.x * w.x - v.y * w.y, v.x * w.y + v.y * w.x);
      p[0] = make_float2(u.x + t.x, u.y + t.y);
      p[half] = make_float2(u.x - t.x, u.y - t.y);
    }
  }
  __syncthreads();
}

// Forward: G real vectors x(g, i) -> buf holds V = FFT(v) in natural order;
// X_k = post_k.x V_k.x - post_k.y V_k.y. With logG >= 0 the loads run with
// the vector index fastest (G = 2^logG neighbouring columns of a row-major
// grid are then read together), else with the sample index fastest.
template <class Load>
__device__ __forceinline__ void dct2(float2* buf, int G, const Axis& a, Load load, int logG = -1) {
  __syncthreads();
  for (int e = threadIdx.x; e < (G << a.logn); e += blockDim.x) {
    int g, i;
    if (logG >= 0) {
      g = e & (G - 1);
      i = e >> logG;
    } else {
      g = e >> a.logn;
      i = e & (a.n - 1);
    }
    buf[(g << a.logn) + brev(mak(i, a.n), a.logn)] = make_float2(load(g, i), 0.f);
  }
  stages(buf, G, a);
}
__device__ __forceinline__ float coef(const Axis& a, const float2* buf, int g, int k) {
  const float2 v = buf[(g << a.logn) + k], p = a.post[k];
  return p.x * v.x - p.y * v.y;
}

// Inverse: coefficients c(g, k) -> buf holds F; sample i of vector g is
// Re buf[g n + mak(i, n)] / n. The coefficients may be read from buf itself:
// every thread reads its W values before any is written.
template <class Coef>
__device__ __forceinline__ void dct3(float2* buf, int G, const Axis& a, Coef c) {
  float2 w[kPer];
  int at[kPer];
  __syncthreads();
#pragma unroll
  for (int q = 0; q < kPer; ++q) {
    const int e = threadIdx.x + q * kThreads;
    at[q] = -1;
    if (e < (G << a.logn)) {
      const int g = e >> a.logn, k = e & (a.n - 1);
      const float ck = c(g, k) * a.inv_s[k];
      const float cn = k ? c(g, a.n - k) * a.inv_s[a.n - k] : 0.f;
      const float2 p = a.pre[k];
      w[q] = make_float2(p.x * ck - p.y * cn, p.x * cn + p.y * ck);
      at[q] = (g << a.logn) + brev(k, a.logn);
    }
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < kPer; ++q)
    if (at[q] >= 0) buf[at[q]] = w[q];
  stages(buf, G, a);
}

// Pass 1: t1 = rows-DCT(rho). With `mean` (fixed-point mean per field) the
// density preparation is folded in: rho = (phys + fill - mean) 2^-32 is
// formed while loading (every bin once), stored, and the physical overflow
// is counted into the IS_OVERFLOW / IS_OVER_BINS partials.
static __device__ void pass_rows_fwd(const Dev& d, Partials p, int vb, int nvb, Smem& sm, Shared& sh,
                                     const long long* mean) {
  const int W = d.g.Wb, H = d.g.Hb, G = min(group_size(d.logW), H);
  const int gpf = (H + G - 1) / G, groups = gpf * d.K;
  const Axis a = vb < groups ? stage_tables(axis_x(d), sm.buf) : axis_x(d);
  long long ov[kMaxFields], cnt[kMaxFields];
#pragma unroll
  for (int f = 0; f < kMaxFields; ++f) ov[f] = cnt[f] = 0;
  for (int t = vb; t < groups; t += nvb) {
    const int f = t / gpf, y0 = (t % gpf) * G;
    const size_t base = (size_t)f * d.B;
    dct2(sm.buf, G, a, [&](int g, int x) -> float {
      const int y = y0 + g;
      if (y >= H) return 0.f;
      const size_t i = base + (size_t)y * W + x;
      if (!mean) return d.rho[i];
      const long long q = d.phys[i];
      const float v = __ll2float_rn(q + d.fill[i] - mean[f]) * kInvFixF;
      d.rho[i] = v;
      if (q > 0)
#pragma unroll
        for (int ff = 0; ff < kMaxFields; ++ff)
          if (ff == f) {
            ov[ff] += q;
            cnt[ff] += 1;
          }
      return v;
    });
    for (int e = threadIdx.x; e < (G << a.logn); e += blockDim.x) {
      const int g = e >> a.logn, k = e & (W - 1), y = y0 + g;
      if (y < H) d.t1[base + (size_t)y * W + k] = coef(a, sm.buf, g, k);
    }
  }
  if (mean)
    for (int f = 0; f < d.K; ++f) {
      write_partial(ov[f], islot(p, IS_OVERFLOW + f), vb, sh.l);
      write_partial(cnt[f], islot(p, IS_OVER_BINS + f), vb, sh.l);
    }
}

// Pass 2: t2 = cols-IDCT(cols-DCT(t1) * inv_eig), whole columns per group.
static __device__ void pass_cols(const Dev& d, int vb, int nvb, Smem& sm) {
  const int W = d.g.Wb, H = d.g.Hb, G = min(group_size(d.logH), W);
  const int gpf = (W + G - 1) / G, groups = gpf * d.K;
  const Axis a = vb < groups ? stage_tables(axis_y(d), sm.buf) : axis_y(d);
  const int logG = 31 - __clz(G);
  const float inv_n = 1.0f / (float)H;
  for (int t = vb; t < groups; t += nvb) {
    const int f = t / gpf, x0 = (t % gpf) * G;
    const size_t base = (size_t)f * d.B;
    dct2(
        sm.buf, G, a,
        [&](int g, int y) -> float {
          const int x = x0 + g;
          return x < W ? d.t1[base + (size_t)y * W + x] : 0.f;
        },
        logG);
    // scaled coefficients, in place (each slot read and written by one thread)
    for (int e = threadIdx.x; e < (G << a.logn); e += blockDim.x) {
      const int g = e & (G - 1), ky = e >> logG, x = x0 + g;
      const int slot = (g << a.logn) + ky;
      const float c = x < W ? coef(a, sm.buf, g, ky) * d.inv_eig[(size_t)ky * W + x] : 0.f;
      sm.buf[slot] = make_float2(c, 0.f);
    }
    dct3(sm.buf, G, a, [&](int g, int k) -> float { return sm.buf[(g << a.logn) + k].x; });
    for (int e = threadIdx.x; e < (G << a.logn); e += blockDim.x) {
      const int g = e & (G - 1), y = e >> logG, x = x0 + g;
      if (x < W) d.t2[base + (size_t)y * W + x] = sm.buf[(g << a.logn) + mak(y, H)].x * inv_n;
    }
  }
}

// Pass 3: phi = rows-IDCT(t2) and the energy partials <rho, phi>.
static __device__ void pass_rows_inv(const Dev& d, Partials p, int vb, int nvb, Smem& sm, Shared& sh) {
  const int W = d.g.Wb, H = d.g.Hb, G = min(group_size(d.logW), H);
  const int gpf = (H + G - 1) / G, groups = gpf * d.K;
  const Axis a = vb < groups ? stage_tables(axis_x(d), sm.buf) : axis_x(d);
  const float inv_n = 1.0f / (float)W;
  double eacc[kMaxFields] = {0.0, 0.0, 0.0, 0.0};
  for (int t = vb; t < groups; t += nvb) {
    const int f = t / gpf, y0 = (t % gpf) * G;
    const size_t base = (size_t)f * d.B;
    dct3(sm.buf, G, a, [&](int g, int k) -> float {
      const int y = y0 + g;
      return y < H ? d.t2[base + (size_t)y * W + k] : 0.f;
    });
    for (int e = threadIdx.x; e < (G << a.logn); e += blockDim.x) {
      const int g = e >> a.logn, x = e & (W - 1), y = y0 + g;
      if (y < H) {
        const size_t i = base + (size_t)y * W + x;
        const float v = sm.buf[(g << a.logn) + mak(x, W)].x * inv_n;
        d.phi[i] = v;
#pragma unroll
        for (int ff = 0; ff < kMaxFields; ++ff)
          if (ff == f) eacc[ff] += (double)(d.rho[i] * v);
      }
    }
  }
  for (int f = 0; f < d.K; ++f) write_partial(eacc[f], pslot(p, SLOT_ENERGY + f), vb, sh.d);
}

}  // namespace fft
}  // namespace tgp
