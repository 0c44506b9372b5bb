// dct_fft.cuh — the spectral Poisson solve as FFT-based DCTs, for
// power-of-two bin grids up to 1024, in double-float arithmetic.
//
// The orthonormal DCT-II of a real vector x of length n is computed with
// Makhoul's reordering (IEEE TASSP 28(1), 1980): v = (x0, x2, x4, ...,
// x5, x3, x1), V = FFT_n(v), X_k = s_k Re(exp(-i pi k / 2n) V_k) with
// s_0 = sqrt(1/n), s_k = sqrt(2/n). The inverse (DCT-III) forms
// W_k = exp(-i pi k / 2n) (X_k / s_k + i X_{n-k} / s_{n-k}) (X_n = 0), takes
// F = FFT_n(W) and reads x_{2j} = Re F_j / n, x_{2j+1} = Re F_{n-1-j} / n.
// The FFT is an in-place radix-2 decimation-in-time transform in shared
// memory over a group of vectors stored back to back, fed in bit-reversed
// order.
//
// Every value inside a transform is a double-float: an unevaluated sum
// hi + lo of two FP32 numbers, added with Knuth's two-sum and multiplied with
// the exact FMA product (the double-double arithmetic of Dekker 1971 and of
// Hida, Li and Bailey 2001, in single precision: about 2^-44 relative). The
// twiddle and scaling tables are FP64 values split into such pairs. Plain
// FP32 butterflies lose about log2(n) roundings of the vector norm, which the
// 1/lambda scaling and the field gather amplify (potential 2.6e-6 and field
// gradient 1.3e-5 normwise at 256 x 256); with double-float butterflies the
// transforms are exact to FP32 and the only roundings left are the FP32
// stores between the passes, as in the compensated GEMM form. The arithmetic
// runs on the FP32 pipes: an FP64 butterfly would occupy this part's FP64
// pipe for hundreds of cycles.
//
// The 2-D solve t1 = rows-DCT(rho), t2 = cols-IDCT(cols-DCT(t1) / lambda),
// phi = rows-IDCT(t2) takes three passes: the column pass owns whole
// columns, so the forward transform, the inverse-eigenvalue scaling and the
// inverse transform run back to back in shared memory. The intermediate
// grids t1 and t2 are stored as double-float pairs (float2 per bin), so the
// only FP32 roundings are the density entering (exact from fixed point when
// the preparation is folded in) and the potential leaving.
#pragma once
#include "stages.cuh"

namespace tgp {
namespace fft {

constexpr int kBuf = 2048;                       // complex double-float slots of the work buffer (32 KB)
constexpr int kData = 1024;                      // slots a group's data takes at most (n <= 1024)
constexpr int kPer = kData / kThreads;           // data slots per thread

struct Smem {
  float4 buf[kBuf];   // (re.hi, im.hi, re.lo, im.lo)
};

// ---- double-float arithmetic ---------------------------------------------
// The _rn intrinsics keep the compiler from contracting a product into a
// following add, which would break the error-free transformations.
struct DF {
  float hi, lo;
};
__device__ __forceinline__ DF two_sum(float a, float b) {
  const float s = __fadd_rn(a, b), bb = __fsub_rn(s, a);
  return DF{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ DF quick_two_sum(float a, float b) {   // |a| >= |b| or a == 0
  const float s = __fadd_rn(a, b);
  return DF{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ DF df_add(DF a, DF b) {
  const DF s = two_sum(a.hi, b.hi);
  return quick_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ DF df_neg(DF a) { return DF{-a.hi, -a.lo}; }
__device__ __forceinline__ DF df_sub(DF a, DF b) { return df_add(a, df_neg(b)); }
__device__ __forceinline__ DF df_mul(DF a, DF b) {
  const float p = __fmul_rn(a.hi, b.hi);
  const float e = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, __fmaf_rn(a.hi, b.hi, -p)));
  return quick_two_sum(p, e);
}
__device__ __forceinline__ DF df_scale(DF a, float s) {   // s a power of two: exact
  return DF{__fmul_rn(a.hi, s), __fmul_rn(a.lo, s)};
}
__device__ __forceinline__ float df_float(DF a) { return __fadd_rn(a.hi, a.lo); }
// an int64 as a double-float (exact for |v| < 2^48)
__device__ __forceinline__ DF df_from_ll(long long v) {
  const float hi = __ll2float_rn(v);
  return DF{hi, __ll2float_rn(v - __float2ll_rn(hi))};
}

struct CDF {
  DF re, im;
};
__device__ __forceinline__ CDF cdf_load(const float4& v) { return CDF{{v.x, v.z}, {v.y, v.w}}; }
__device__ __forceinline__ float4 cdf_store(const CDF& c) { return make_float4(c.re.hi, c.im.hi, c.re.lo, c.im.lo); }
__device__ __forceinline__ CDF cdf_mul(const CDF& a, const CDF& b) {
  return CDF{df_sub(df_mul(a.re, b.re), df_mul(a.im, b.im)), df_add(df_mul(a.re, b.im), df_mul(a.im, b.re))};
}

// Tables of one transform length n (a power of two), FP64 values as
// double-float pairs: complex tables (re.hi, im.hi, re.lo, im.lo), real
// (hi, lo).
struct Axis {
  const float4* tw;      // [n/2] exp(-2 pi i j / n)
  const float4* post;    // [n]   s_k exp(-i pi k / 2n)
  const float4* pre;     // [n]   exp(-i pi k / 2n)
  const float2* inv_s;   // [n]   1 / s_k
  int n, logn;
};

__device__ __forceinline__ Axis axis_x(const Dev& d) {
  return Axis{d.fx_tw, d.fx_post, d.fx_pre, d.fx_inv_s, d.g.Wb, d.logW};
}
__device__ __forceinline__ Axis axis_y(const Dev& d) {
  return Axis{d.fy_tw, d.fy_post, d.fy_pre, d.fy_inv_s, d.g.Hb, d.logH};
}

// Up to 256 points the tables (n/2 twiddles, n post and n pre factors, n
// 1/s_k) fit in the half of the buffer the data leaves free and are copied
// there once per pass: the stages then read their twiddles from shared
// memory instead of making an L2 round trip per stage (the persistent
// kernel's grid barriers leave L1 cold).
constexpr int kTableLog = 8;
__device__ __forceinline__ Axis stage_tables(const Axis& a, float4* buf) {
  if (a.logn > kTableLog) return a;
  float4* tw = buf + kData;
  float4* post = tw + (a.n >> 1);
  float4* pre = post + a.n;
  float2* inv_s = reinterpret_cast<float2*>(pre + a.n);
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
__device__ __forceinline__ void stages(float4* buf, int G, const Axis& a) {
  const int half_n = a.n >> 1, total = G * half_n;
  for (int s = 0; s < a.logn; ++s) {
    const int half = 1 << s, step = half_n >> s;
    __syncthreads();
    for (int b = threadIdx.x; b < total; b += blockDim.x) {
      const int g = b >> (a.logn - 1), j = b & (half_n - 1);
      const int jj = j & (half - 1);
      float4* p = buf + (g << a.logn) + ((j >> s) << (s + 1)) + jj;
      const CDF w = cdf_load(a.tw[jj * step]);
      const CDF u = cdf_load(p[0]);
      const CDF t = cdf_mul(cdf_load(p[half]), w);
      p[0] = cdf_store(CDF{df_add(u.re, t.re), df_add(u.im, t.im)});
      p[half] = cdf_store(CDF{df_sub(u.re, t.re), df_sub(u.im, t.im)});
    }
  }
  __syncthreads();
}

// Forward: G real vectors x(g, i) (double-floats) -> buf holds V = FFT(v) in
// natural order; X_k = Re(post_k V_k). With logG >= 0 the loads run with the
// vector index fastest (G = 2^logG neighbouring columns of a row-major grid
// are then read together), else with the sample index fastest.
template <class Load>
__device__ __forceinline__ void dct2(float4* buf, int G, const Axis& a, Load load, int logG = -1) {
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
    const DF x = load(g, i);
    buf[(g << a.logn) + brev(mak(i, a.n), a.logn)] = make_float4(x.hi, 0.f, x.lo, 0.f);
  }
  stages(buf, G, a);
}
__device__ __forceinline__ DF coef(const Axis& a, const float4* buf, int g, int k) {
  const CDF v = cdf_load(buf[(g << a.logn) + k]), p = cdf_load(a.post[k]);
  return df_sub(df_mul(p.re, v.re), df_mul(p.im, v.im));
}

// Inverse: coefficients c(g, k) (double-floats) -> buf holds F; sample i of
// vector g is Re buf[g n + mak(i, n)] / n. The coefficients may be read from
// buf itself: every thread reads its W values before any is written.
template <class Coef>
__device__ __forceinline__ void dct3(float4* buf, int G, const Axis& a, Coef c) {
  float4 w[kPer];
  int at[kPer];
  __syncthreads();
#pragma unroll
  for (int q = 0; q < kPer; ++q) {
    const int e = threadIdx.x + q * kThreads;
    at[q] = -1;
    if (e < (G << a.logn)) {
      const int g = e >> a.logn, k = e & (a.n - 1);
      const float2 sk = a.inv_s[k];
      const DF ck = df_mul(c(g, k), DF{sk.x, sk.y});
      DF cn = DF{0.f, 0.f};
      if (k) {
        const float2 sn = a.inv_s[a.n - k];
        cn = df_mul(c(g, a.n - k), DF{sn.x, sn.y});
      }
      w[q] = cdf_store(cdf_mul(cdf_load(a.pre[k]), CDF{ck, cn}));
      at[q] = (g << a.logn) + brev(k, a.logn);
    }
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < kPer; ++q)
    if (at[q] >= 0) buf[at[q]] = w[q];
  stages(buf, G, a);
}
// Re of an inverse-transform output slot, times 1/n (a power of two)
__device__ __forceinline__ DF out_sample(const float4& v, float inv_n) { return df_scale(DF{v.x, v.z}, inv_n); }
// t1 / t2 as double-float grids
__device__ __forceinline__ float2* df_grid(float* g) { return reinterpret_cast<float2*>(g); }
__device__ __forceinline__ DF df_at(const float* g, size_t i) {
  const float2 v = reinterpret_cast<const float2*>(g)[i];
  return DF{v.x, v.y};
}

// Pass 1: t1 = rows-DCT(rho). With `mean` (fixed-point mean per field) the
// density preparation is folded in: rho = (phys + fill - mean) 2^-32 enters
// the transform exactly (as a double-float), is stored rounded to FP32, and
// the physical overflow is counted into the IS_OVERFLOW / IS_OVER_BINS
// partials.
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
    dct2(sm.buf, G, a, [&](int g, int x) -> DF {
      const int y = y0 + g;
      if (y >= H) return DF{0.f, 0.f};
      const size_t i = base + (size_t)y * W + x;
      if (!mean) return DF{d.rho[i], 0.f};
      const long long q = d.phys[i];
      const long long v = q + d.fill[i] - mean[f];
      d.rho[i] = __ll2float_rn(v) * kInvFixF;
      if (q > 0)
#pragma unroll
        for (int ff = 0; ff < kMaxFields; ++ff)
          if (ff == f) {
            ov[ff] += q;
            cnt[ff] += 1;
          }
      return df_scale(df_from_ll(v), kInvFixF);
    });
    for (int e = threadIdx.x; e < (G << a.logn); e += blockDim.x) {
      const int g = e >> a.logn, k = e & (W - 1), y = y0 + g;
      if (y < H) {
        const DF c = coef(a, sm.buf, g, k);
        df_grid(d.t1)[base + (size_t)y * W + k] = make_float2(c.hi, c.lo);
      }
    }
  }
  if (mean)
    for (int f = 0; f < d.K; ++f) {
      write_partial(ov[f], islot(p, IS_OVERFLOW + f), vb, sh.l);
      write_partial(cnt[f], islot(p, IS_OVER_BINS + f), vb, sh.l);
    }
}

// Pass 2: t2 = cols-IDCT(cols-DCT(t1) * inv_eig), whole columns per group;
// the scaled coefficients stay double-floats between the two transforms.
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
        [&](int g, int y) -> DF {
          const int x = x0 + g;
          return x < W ? df_at(d.t1, base + (size_t)y * W + x) : DF{0.f, 0.f};
        },
        logG);
    // scaled coefficients, in place (each slot read and written by one thread)
    for (int e = threadIdx.x; e < (G << a.logn); e += blockDim.x) {
      const int g = e & (G - 1), ky = e >> logG, x = x0 + g;
      const int slot = (g << a.logn) + ky;
      DF c = DF{0.f, 0.f};
      if (x < W) c = df_mul(coef(a, sm.buf, g, ky), DF{d.inv_eig[(size_t)ky * W + x], 0.f});
      sm.buf[slot] = make_float4(c.hi, 0.f, c.lo, 0.f);
    }
    dct3(sm.buf, G, a, [&](int g, int k) -> DF {
      const float4 v = sm.buf[(g << a.logn) + k];
      return DF{v.x, v.z};
    });
    for (int e = threadIdx.x; e < (G << a.logn); e += blockDim.x) {
      const int g = e & (G - 1), y = e >> logG, x = x0 + g;
      if (x < W) {
        const DF v = out_sample(sm.buf[(g << a.logn) + mak(y, H)], inv_n);
        df_grid(d.t2)[base + (size_t)y * W + x] = make_float2(v.hi, v.lo);
      }
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
    dct3(sm.buf, G, a, [&](int g, int k) -> DF {
      const int y = y0 + g;
      return y < H ? df_at(d.t2, base + (size_t)y * W + k) : DF{0.f, 0.f};
    });
    for (int e = threadIdx.x; e < (G << a.logn); e += blockDim.x) {
      const int g = e >> a.logn, x = e & (W - 1), y = y0 + g;
      if (y < H) {
        const size_t i = base + (size_t)y * W + x;
        const float v = df_float(out_sample(sm.buf[(g << a.logn) + mak(x, W)], inv_n));
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
