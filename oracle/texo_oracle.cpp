// texo_oracle.cpp — TEST INFRASTRUCTURE ONLY (parity oracle and timed CPU
// baseline; never linked into the product library).
//
// An FP64 C++17 restatement of Texo's electrostatic global placement, written
// from the reference's Rust sources and following their operation order so
// that reductions happen in the same sequence:
//   crates/texo-pnr/src/electrostatic_placement.rs  (density model, Poisson)
//   crates/texo-pnr/src/analytical_placement.rs     (hypergraph, WA wirelength)
//   crates/texo-pnr/src/global_placement.rs         (dynamic Nesterov step)
//   crates/texo-pnr/src/eplace.rs                   (augmented-Lagrangian loop)
// The reference delegates its DCT to the third-party crate rustdct 0.7.1
// (pinned in Cargo.lock), which is not vendored; this file computes the same
// orthonormal DCT-II/III pair with an FFT written here (radix-2 plus Bluestein
// for arbitrary lengths), and the reference's own matrix-form oracle
// (`solve_reference`) pins it. Parity status: pinned by the reference's
// known-answer tests, which the test suite ports; full trajectories have no
// reference golden output (the Rust reference cannot be built here).
//
// Build with -ffp-contract=off so that no multiply-add is fused: Rust never
// contracts, and the known-answer tests compare exact bits.

#include "texo_oracle.h"

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <complex>
#include <cstring>
#include <functional>
#include <limits>
#include <map>
#include <memory>
#include <thread>
#include <vector>

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr double kEps = std::numeric_limits<double>::epsilon();

// ---------------------------------------------------------------------------
// Rust f64 helpers restated.
// ---------------------------------------------------------------------------
inline double rclamp(double v, double lo, double hi) {
  // f64::clamp: NaN passes through.
  if (v < lo) return lo;
  if (v > hi) return hi;
  return v;
}
inline double rmax(double a, double b) { return std::fmax(a, b); }
inline double rmin(double a, double b) { return std::fmin(a, b); }
// f64::total_cmp ordering key.
inline int64_t total_key(double v) {
  int64_t bits;
  std::memcpy(&bits, &v, 8);
  bits ^= (int64_t)(((uint64_t)(bits >> 63)) >> 1);
  return bits;
}
inline int total_cmp(double a, double b) {
  int64_t ka = total_key(a), kb = total_key(b);
  return ka < kb ? -1 : (ka > kb ? 1 : 0);
}
// f64::midpoint (Rust core), restated from its documented behaviour.
inline double midpoint(double a, double b) {
  const double lo = std::numeric_limits<double>::min() * 2.0;
  const double hi = std::numeric_limits<double>::max() / 2.0;
  double aa = std::fabs(a), ab = std::fabs(b);
  if (aa <= hi && ab <= hi) return (a + b) / 2.0;
  if (aa < lo) return a + (b / 2.0);
  if (ab < lo) return (a / 2.0) + b;
  return (a / 2.0) + (b / 2.0);
}
inline double sum(const std::vector<double>& v) {
  double s = -0.0;
  for (double x : v) s += x;
  return s;
}
inline double dotv(const double* a, const double* b, size_t n) {
  double s = -0.0;
  for (size_t i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}

// ---------------------------------------------------------------------------
// B-spline stencil (electrostatic_placement.rs:895-976).
// ---------------------------------------------------------------------------
struct AxisEntry {
  size_t index;
  double weight, derivative;
};
inline std::array<AxisEntry, 3> bspline_axis(size_t length, double coordinate) {
  const double maximum = (double)(uint32_t)(length - 1);
  const double c = rclamp(coordinate, 0.0, maximum);
  const double center_c = rmin(std::floor(c + 0.5), maximum);
  const size_t center = (size_t)center_c;
  const double o = c - center_c;
  std::array<AxisEntry, 3> r;
  const double a = 0.5 - o, b = 0.5 + o;
  r[0] = {center == 0 ? 0 : center - 1, 0.5 * (a * a), o - 0.5};
  r[1] = {center, 0.75 - o * o, -2.0 * o};
  r[2] = {std::min(center + 1, length - 1), 0.5 * (b * b), o + 0.5};
  return r;
}
inline void deposit(double* density, size_t width, size_t height, double x, double y,
                    double charge) {
  auto ax = bspline_axis(width, x);
  auto ay = bspline_axis(height, y);
  for (const auto& row : ay)
    for (const auto& col : ax) density[row.index * width + col.index] += charge * col.weight * row.weight;
}
inline void sample(const double* potential, size_t width, size_t height, double x, double y,
                   double& value, double& gx, double& gy) {
  auto ax = bspline_axis(width, x);
  auto ay = bspline_axis(height, y);
  value = 0.0;
  gx = 0.0;
  gy = 0.0;
  for (const auto& row : ay)
    for (const auto& col : ax) {
      const double p = potential[row.index * width + col.index];
      value += col.weight * row.weight * p;
      gx += col.derivative * row.weight * p;
      gy += col.weight * row.derivative * p;
    }
}

// Cloud-in-cell pair (electrostatic_placement.rs:979-1062).
struct InterpAxis {
  size_t lower, upper;
  double fraction;
};
inline InterpAxis interp_axis(size_t length, double coordinate) {
  if (length == 1) return {0, 0, 0.0};
  const double maximum = (double)(uint32_t)(length - 1);
  const double c = rclamp(coordinate, 0.0, maximum);
  if (c >= maximum) return {length - 2, length - 1, 1.0};
  const size_t lower = (size_t)std::floor(c);
  return {lower, lower + 1, c - (double)(uint32_t)lower};
}

// ---------------------------------------------------------------------------
// DFT (radix-2 + Bluestein) and the orthonormal DCT pair.
// ---------------------------------------------------------------------------
using cd = std::complex<double>;

struct Radix2 {
  size_t n = 0;
  std::vector<cd> tw;     // e^{-2 pi i k / n}, k < n/2
  std::vector<size_t> rev;
  explicit Radix2(size_t n_ = 0) { init(n_); }
  void init(size_t n_) {
    n = n_;
    if (n == 0) return;
    tw.resize(n / 2 > 0 ? n / 2 : 1);
    for (size_t k = 0; k < n / 2; ++k) {
      double ang = -2.0 * kPi * (double)k / (double)n;
      tw[k] = cd(std::cos(ang), std::sin(ang));
    }
    rev.resize(n);
    size_t bits = 0;
    while (((size_t)1 << bits) < n) ++bits;
    for (size_t i = 0; i < n; ++i) {
      size_t r = 0;
      for (size_t b = 0; b < bits; ++b)
        if (i & ((size_t)1 << b)) r |= (size_t)1 << (bits - 1 - b);
      rev[i] = r;
    }
  }
  // In place; inverse = conjugate exponent, unnormalised.
  void run(cd* a, bool inverse) const {
    for (size_t i = 0; i < n; ++i)
      if (i < rev[i]) std::swap(a[i], a[rev[i]]);
    for (size_t len = 2; len <= n; len <<= 1) {
      size_t step = n / len;
      for (size_t i = 0; i < n; i += len)
        for (size_t j = 0; j < len / 2; ++j) {
          cd w = tw[j * step];
          if (inverse) w = std::conj(w);
          cd u = a[i + j], v = a[i + j + len / 2] * w;
          a[i + j] = u + v;
          a[i + j + len / 2] = u - v;
        }
    }
  }
};

struct Dft {
  size_t n = 0;
  bool pow2 = false;
  Radix2 r2;
  // Bluestein
  size_t m = 0;
  Radix2 rm;
  std::vector<cd> chirp;    // e^{-i pi k^2 / n}
  std::vector<cd> bfft;     // FFT of conj chirp kernel
  explicit Dft(size_t n_) : n(n_) {
    pow2 = n && !(n & (n - 1));
    if (pow2) {
      r2.init(n);
      return;
    }
    m = 1;
    while (m < 2 * n - 1) m <<= 1;
    rm.init(m);
    chirp.resize(n);
    for (size_t k = 0; k < n; ++k) {
      uint64_t kk = ((uint64_t)k * (uint64_t)k) % (2 * (uint64_t)n);
      double ang = -kPi * (double)kk / (double)n;
      chirp[k] = cd(std::cos(ang), std::sin(ang));
    }
    bfft.assign(m, cd(0, 0));
    for (size_t k = 0; k < n; ++k) {
      bfft[k] = std::conj(chirp[k]);
      if (k) bfft[m - k] = std::conj(chirp[k]);
    }
    rm.run(bfft.data(), false);
  }
  // Forward (negative exponent) or inverse (positive exponent), unnormalised.
  void run(std::vector<cd>& a, bool inverse) const {
    if (pow2) {
      r2.run(a.data(), inverse);
      return;
    }
    // inverse DFT = conj(DFT(conj(a)))
    std::vector<cd> t(m, cd(0, 0));
    for (size_t k = 0; k < n; ++k) t[k] = (inverse ? std::conj(a[k]) : a[k]) * chirp[k];
    rm.run(t.data(), false);
    for (size_t k = 0; k < m; ++k) t[k] *= bfft[k];
    rm.run(t.data(), true);
    const double inv_m = 1.0 / (double)m;
    for (size_t k = 0; k < n; ++k) {
      cd v = t[k] * inv_m * chirp[k];
      a[k] = inverse ? std::conj(v) : v;
    }
  }
};

// Orthonormal DCT-II / its inverse (the transpose), as the reference's
// OrthonormalDct (electrostatic_placement.rs:616-672): unnormalised sums
// scaled by sqrt(1/n) at DC and sqrt(2/n) elsewhere.
struct OrthoDct {
  size_t n;
  Dft dft;      // length 2n
  std::vector<cd> phase;  // e^{-i pi k / (2n)}
  double dc, other;
  explicit OrthoDct(size_t n_) : n(n_), dft(2 * n_) {
    phase.resize(n);
    for (size_t k = 0; k < n; ++k) {
      double ang = -kPi * (double)k / (2.0 * (double)n);
      phase[k] = cd(std::cos(ang), std::sin(ang));
    }
    const double nf = (double)(uint32_t)n;
    dc = std::sqrt(1.0 / nf);
    other = std::sqrt(2.0 / nf);
  }
  void forward(double* v, std::vector<cd>& buf) const {
    buf.assign(2 * n, cd(0, 0));
    for (size_t i = 0; i < n; ++i) buf[i] = cd(v[i], 0);
    dft.run(buf, false);
    for (size_t k = 0; k < n; ++k) v[k] = (buf[k] * phase[k]).real() * (k == 0 ? dc : other);
  }
  void inverse(double* v, std::vector<cd>& buf) const {
    buf.assign(2 * n, cd(0, 0));
    for (size_t k = 0; k < n; ++k) buf[k] = std::conj(phase[k]) * (v[k] * (k == 0 ? dc : other));
    dft.run(buf, true);
    for (size_t i = 0; i < n; ++i) v[i] = buf[i].real();
  }
};

std::vector<double> dct_basis(size_t length) {
  const double lf = (double)(uint32_t)length;
  std::vector<double> basis;
  basis.reserve(length * length);
  for (size_t f = 0; f < length; ++f) {
    const double ff = (double)(uint32_t)f;
    const double scale = f == 0 ? std::sqrt(1.0 / lf) : std::sqrt(2.0 / lf);
    for (size_t c = 0; c < length; ++c) {
      const double cf = (double)(uint32_t)c;
      basis.push_back(scale * std::cos(kPi * ff * (cf + 0.5) / lf));
    }
  }
  return basis;
}

// Poisson2d (electrostatic_placement.rs:602-776).
struct Poisson2d {
  size_t width, height;
  OrthoDct tx, ty;
  std::vector<double> inv_eig;
  Poisson2d(size_t w, size_t h) : width(w), height(h), tx(w), ty(h) {
    inv_eig.reserve(w * h);
    const double wf = (double)(uint32_t)w, hf = (double)(uint32_t)h;
    for (size_t ky = 0; ky < h; ++ky) {
      const double sy = std::sin(kPi * (double)(uint32_t)ky / (2.0 * hf));
      const double ly = 4.0 * (sy * sy);
      for (size_t kx = 0; kx < w; ++kx) {
        const double sx = std::sin(kPi * (double)(uint32_t)kx / (2.0 * wf));
        const double lx = 4.0 * (sx * sx);
        const double l = lx + ly;
        inv_eig.push_back(kx == 0 && ky == 0 ? 0.0 : 1.0 / l);
      }
    }
  }
  // Returns a status; potential [w*h]; index of the first non-finite entry.
  int32_t solve(const double* density, double* potential, double& energy, uint64_t* bad) const {
    const size_t expected = width * height;
    for (size_t i = 0; i < expected; ++i)
      if (!std::isfinite(density[i])) {
        if (bad) *bad = i;
        return TEXO_GP_ERR_NONFINITE_DENSITY;
      }
    const double count = (double)(uint32_t)expected;
    double s = -0.0;
    for (size_t i = 0; i < expected; ++i) s += density[i];
    const double mean = s / count;
    std::vector<double> centered(expected), t(expected);
    for (size_t i = 0; i < expected; ++i) centered[i] = density[i] - mean;
    t = centered;
    std::vector<cd> buf;
    for (size_t y = 0; y < height; ++y) tx.forward(&t[y * width], buf);
    std::vector<double> column(height);
    for (size_t kx = 0; kx < width; ++kx) {
      for (size_t y = 0; y < height; ++y) column[y] = t[y * width + kx];
      ty.forward(column.data(), buf);
      for (size_t ky = 0; ky < height; ++ky) column[ky] *= inv_eig[ky * width + kx];
      ty.inverse(column.data(), buf);
      for (size_t y = 0; y < height; ++y) potential[y * width + kx] = column[y];
    }
    for (size_t y = 0; y < height; ++y) tx.inverse(&potential[y * width], buf);
    energy = 0.5 * dotv(centered.data(), potential, expected);
    return TEXO_GP_OK;
  }
  int32_t solve_matrix(const double* density, double* potential, double& energy) const {
    const size_t W = width, H = height, n = W * H;
    for (size_t i = 0; i < n; ++i)
      if (!std::isfinite(density[i])) return TEXO_GP_ERR_NONFINITE_DENSITY;
    auto bx = dct_basis(W), by = dct_basis(H);
    double s = -0.0;
    for (size_t i = 0; i < n; ++i) s += density[i];
    const double mean = s / (double)(uint32_t)n;
    std::vector<double> centered(n);
    for (size_t i = 0; i < n; ++i) centered[i] = density[i] - mean;
    std::vector<double> rs(n), sp(n), ci(n);
    for (size_t y = 0; y < H; ++y)
      for (size_t kx = 0; kx < W; ++kx) rs[y * W + kx] = dotv(&bx[kx * W], &centered[y * W], W);
    for (size_t ky = 0; ky < H; ++ky)
      for (size_t kx = 0; kx < W; ++kx) {
        double c = 0.0;
        for (size_t y = 0; y < H; ++y) c += by[ky * H + y] * rs[y * W + kx];
        sp[ky * W + kx] = c * inv_eig[ky * W + kx];
      }
    for (size_t y = 0; y < H; ++y)
      for (size_t kx = 0; kx < W; ++kx) {
        double v = 0.0;
        for (size_t ky = 0; ky < H; ++ky) v += by[ky * H + y] * sp[ky * W + kx];
        ci[y * W + kx] = v;
      }
    for (size_t y = 0; y < H; ++y)
      for (size_t x = 0; x < W; ++x) {
        double v = 0.0;
        for (size_t kx = 0; kx < W; ++kx) v += bx[kx * W + x] * ci[y * W + kx];
        potential[y * W + x] = v;
      }
    energy = 0.5 * dotv(centered.data(), potential, n);
    return TEXO_GP_OK;
  }
};

// ---------------------------------------------------------------------------
// Problem model.
// ---------------------------------------------------------------------------
struct Member {
  uint32_t field;
  double dx, dy, charge;
  uint32_t cell;
};
struct DUnit {              // DensityUnit (electrostatic_placement.rs:81-87)
  uint32_t unit;            // index into the placement-unit coordinate vector
  std::vector<Member> members;
};
struct Filler {             // DensityFiller (:96-102)
  uint32_t field;
  double x, y, charge;
};
struct Pin {
  uint32_t unit, cell;
};
struct Arc {
  Pin driver, sink;
  uint64_t extra;
};
struct FieldResult {
  double energy = 0, overflow = 0, net_charge = 0, force_l1 = 0;
  uint64_t available = 0, real_charge = 0;
  double real_area = 0, filler_charge = 0;
  std::vector<double> density, potential;
  std::vector<double> unit_gx, unit_gy;      // per density unit
  std::vector<double> filler_gx, filler_gy;  // per filler of this field (index list below)
  std::vector<uint32_t> filler_index;
};
struct Evaluation {         // ContinuousEvaluation (eplace.rs:84-87)
  double wa_value = 0;
  std::vector<double> wa_gx, wa_gy;  // [U]
  std::vector<FieldResult> fields;
};

double u64_to_f64(uint64_t v) {
  // analytical_placement.rs:705-709
  return (double)(uint32_t)(v >> 32) * 4294967296.0 + (double)(uint32_t)(v & 0xffffffffu);
}

struct Oracle {
  // Tile grid and density (bin) grid.
  uint32_t W = 0, H = 0, Wb = 0, Hb = 0;
  double sx = 1, sy = 1;        // bins per tile
  bool identity_map = true;
  double td = 1.0;
  texo_gp_params params{};
  uint32_t K = 0;               // active fields
  std::vector<texo_gp_field> field_kind;     // per active field
  std::vector<uint32_t> field_of_input;      // input field -> active index or ~0
  std::vector<std::vector<uint32_t>> capacity;     // [K][W*H]
  std::vector<std::vector<double>> smoothed;       // [K][Wb*Hb], td scaled
  std::vector<uint64_t> available;                 // [K]
  std::unique_ptr<Poisson2d> solver;

  uint32_t U = 0, C = 0;
  std::vector<DUnit> dunits;
  std::vector<Filler> fillers;
  std::vector<double> init_coords, lower, upper;
  // cells
  std::vector<uint32_t> cell_unit;
  std::vector<double> cell_off;      // [2C]
  std::vector<uint8_t> cell_fixed;
  std::vector<double> cell_fxy;      // [2C]
  // hypergraph
  std::vector<uint32_t> net_ptr;
  std::vector<Pin> pins;
  std::vector<Arc> arcs;
  std::vector<double> gamma_weights;  // [K]
  std::vector<double> wl_precond;     // [U]

  size_t coord_count() const { return 2 * ((size_t)U + fillers.size()); }
  size_t bins() const { return (size_t)Wb * Hb; }

  double to_bin_x(double s) const { return identity_map ? s : (s + 0.5) * sx - 0.5; }
  double to_bin_y(double s) const { return identity_map ? s : (s + 0.5) * sy - 0.5; }

  // ---- hypergraph (analytical_placement.rs) --------------------------------
  void build_preconditioners() {
    wl_precond.assign(U, 0.0);
    for (size_t e = 0; e + 1 < net_ptr.size(); ++e) {
      const size_t b = net_ptr[e], en = net_ptr[e + 1];
      std::vector<uint32_t> units;
      for (size_t p = b; p < en; ++p) units.push_back(pins[p].unit);
      std::sort(units.begin(), units.end());
      units.erase(std::unique(units.begin(), units.end()), units.end());
      if (units.size() < 2) continue;
      const double w = 1.0 / (double)(uint32_t)(en - b - 1);
      for (auto u : units) wl_precond[u] += w;
    }
    for (const auto& a : arcs) {
      if (a.driver.unit == a.sink.unit) continue;
      const double w = u64_to_f64(a.extra);
      wl_precond[a.driver.unit] += w;
      wl_precond[a.sink.unit] += w;
    }
  }
  std::vector<double> cell_incidence() const {
    std::vector<double> w(C, 0.0);
    for (size_t e = 0; e + 1 < net_ptr.size(); ++e) {
      const size_t b = net_ptr[e], en = net_ptr[e + 1];
      std::vector<uint32_t> cells;
      for (size_t p = b; p < en; ++p) cells.push_back(pins[p].cell);
      std::sort(cells.begin(), cells.end());
      cells.erase(std::unique(cells.begin(), cells.end()), cells.end());
      const double wt = 1.0 / (double)(uint32_t)(en - b - 1);
      for (auto c : cells) w[c] += wt;
    }
    return w;
  }

  inline double pin_coord(const Pin& pin, const double* coords, bool y_axis) const {
    if (cell_fixed[pin.cell]) return cell_fxy[2 * (size_t)pin.cell + (y_axis ? 1 : 0)];
    return coords[2 * (size_t)pin.unit + (y_axis ? 1 : 0)] + cell_off[2 * (size_t)pin.cell + (y_axis ? 1 : 0)];
  }

  // weighted_average_axis + add_weighted_average_axis (analytical_placement.rs:576-703)
  double wa_axis(const Pin* p, size_t count, double weight, double gamma, const double* coords,
                 bool y_axis, double* grad, std::vector<double>& sc, std::vector<double>& sp,
                 std::vector<double>& sn) const {
    if (sc.size() < count) {
      sc.resize(count);
      sp.resize(count);
      sn.resize(count);
    }
    const double first = pin_coord(p[0], coords, y_axis);
    sc[0] = first;
    double minimum = first, maximum = first;
    for (size_t i = 1; i < count; ++i) {
      const double v = pin_coord(p[i], coords, y_axis);
      sc[i] = v;
      minimum = rmin(minimum, v);
      maximum = rmax(maximum, v);
    }
    double pws = 0.0, pds = 0.0, nws = 0.0, nds = 0.0;
    for (size_t i = 0; i < count; ++i) {
      const double v = sc[i];
      const double md = v - maximum, nd = v - minimum;
      const double pw = md == 0.0 ? 1.0 : std::exp(md / gamma);
      const double nw = nd == 0.0 ? 1.0 : std::exp(-nd / gamma);
      sp[i] = pw;
      sn[i] = nw;
      pws += pw;
      pds += pw * md;
      nws += nw;
      nds += nw * nd;
    }
    const double pm = pds / pws, nm = nds / nws;
    for (size_t i = 0; i < count; ++i) {
      const double v = sc[i];
      const double md = v - maximum, nd = v - minimum;
      const double pp = sp[i] / pws, np = sn[i] / nws;
      const double d = pp * (1.0 + (md - pm) / gamma) - np * (1.0 - (nd - nm) / gamma);
      if (!cell_fixed[p[i].cell]) grad[p[i].unit] += weight * d;
    }
    return weight * ((maximum - minimum) + pm - nm);
  }
  // weighted_average_hypernets_axis / weighted_average_timed_arcs_axis
  double wa_nets_axis(const double* coords, double gamma, bool y_axis, double* grad) const {
    double value = 0.0;
    std::vector<double> sc, sp, sn;
    for (size_t e = 0; e + 1 < net_ptr.size(); ++e)
      value += wa_axis(&pins[net_ptr[e]], net_ptr[e + 1] - net_ptr[e], 1.0, gamma, coords, y_axis, grad,
                       sc, sp, sn);
    return value;
  }
  double wa_arcs_axis(const double* coords, double gamma, bool y_axis, double* grad) const {
    double value = 0.0;
    std::vector<double> sc, sp, sn;
    for (const auto& a : arcs) {
      Pin pp[2] = {a.driver, a.sink};
      value += wa_axis(pp, 2, u64_to_f64(a.extra), gamma, coords, y_axis, grad, sc, sp, sn);
    }
    return value;
  }
  // weighted_average_objective_with_global_gamma (analytical_placement.rs:366-463)
  void wa_objective(const double* coords, double gamma, int threads, Evaluation& ev) const {
    std::vector<double> bx(U, 0.0), by(U, 0.0), tx(U, 0.0), ty(U, 0.0);
    double vbx = 0, vby = 0, vtx = 0, vty = 0;
    if (threads > 1) {
      std::thread t1([&] { vbx = wa_nets_axis(coords, gamma, false, bx.data()); });
      std::thread t2([&] { vby = wa_nets_axis(coords, gamma, true, by.data()); });
      std::thread t3([&] { vtx = wa_arcs_axis(coords, gamma, false, tx.data()); });
      vty = wa_arcs_axis(coords, gamma, true, ty.data());
      t1.join();
      t2.join();
      t3.join();
    } else {
      vbx = wa_nets_axis(coords, gamma, false, bx.data());
      vby = wa_nets_axis(coords, gamma, true, by.data());
      vtx = wa_arcs_axis(coords, gamma, false, tx.data());
      vty = wa_arcs_axis(coords, gamma, true, ty.data());
    }
    double base = vbx + vby;
    double timing = vtx + vty;
    ev.wa_value = base + timing;
    ev.wa_gx.resize(U);
    ev.wa_gy.resize(U);
    for (uint32_t u = 0; u < U; ++u) {
      ev.wa_gx[u] = bx[u] + tx[u];
      ev.wa_gy[u] = by[u] + ty[u];
    }
  }

  // ---- density model (electrostatic_placement.rs:139-441) -------------------
  int32_t capacity_checks(uint32_t f, uint64_t real_count, double real_area) const {
    if (real_count > available[f]) return TEXO_GP_ERR_INSUFFICIENT_CAPACITY;
    const double avail = td * (double)(uint32_t)available[f];
    if (!std::isfinite(real_area) || real_area < 0.0) return TEXO_GP_ERR_INSUFFICIENT_AREA;
    if (td == 1.0 && real_area > avail + 1.0e-9) return TEXO_GP_ERR_INSUFFICIENT_AREA;
    return TEXO_GP_OK;
  }
  double filler_total(uint32_t f, double real_area) const {
    const double avail = td * (double)(uint32_t)available[f];
    const double t = avail - real_area;
    return td == 1.0 ? t : std::max(t, 0.0);
  }
  void real_counts(std::vector<uint64_t>& counts, std::vector<double>& areas) const {
    counts.assign(K, 0);
    areas.assign(K, 0.0);
    for (const auto& u : dunits)
      for (const auto& m : u.members) {
        counts[m.field] += 1;
        areas[m.field] += m.charge;
      }
  }
  // initial_fillers (electrostatic_placement.rs:198-240)
  int32_t make_fillers(uint64_t* err) {
    for (size_t i = 0; i < dunits.size(); ++i)
      for (size_t j = 0; j < dunits[i].members.size(); ++j) {
        const auto& m = dunits[i].members[j];
        if (!std::isfinite(m.dx) || !std::isfinite(m.dy)) {
          *err = i;
          return TEXO_GP_ERR_NONFINITE_UNIT_COORDINATE;
        }
        if (!std::isfinite(m.charge) || m.charge <= 0.0) {
          *err = i;
          return TEXO_GP_ERR_INVALID_MEMBER_CHARGE;
        }
      }
    std::vector<uint64_t> counts;
    std::vector<double> areas;
    real_counts(counts, areas);
    fillers.clear();
    for (uint32_t f = 0; f < K; ++f) {
      if (counts[f] == 0) continue;
      int32_t st = capacity_checks(f, counts[f], areas[f]);
      if (st) {
        *err = f;
        return st;
      }
      const double avail_area = td * (double)(uint32_t)available[f];
      const double filler_area = filler_total(f, areas[f]);
      if (filler_area == 0.0) continue;
      const double total = filler_area;
      const double denominator = (double)(uint32_t)available[f];
      std::vector<size_t> occupied;
      for (size_t i = 0; i < capacity[f].size(); ++i)
        if (capacity[f][i] != 0) occupied.push_back(i);
      (void)avail_area;
      double assigned = 0.0;
      for (size_t o = 0; o < occupied.size(); ++o) {
        const size_t index = occupied[o];
        const double charge = o + 1 == occupied.size()
                                  ? total - assigned
                                  : total * (double)capacity[f][index] / denominator;
        assigned += charge;
        fillers.push_back({f, (double)(uint32_t)(index % W), (double)(uint32_t)(index / W), charge});
      }
    }
    return TEXO_GP_OK;
  }

  // DensityModel::evaluate_with_positions for one field.
  void eval_field(uint32_t f, const double* coords, FieldResult& r, double real_area) const {
    const size_t B = bins();
    r.density.resize(B);
    for (size_t i = 0; i < B; ++i) r.density[i] = -smoothed[f][i];
    for (const auto& u : dunits) {
      const double ox = coords[2 * (size_t)u.unit], oy = coords[2 * (size_t)u.unit + 1];
      for (const auto& m : u.members)
        if (m.field == f) deposit(r.density.data(), Wb, Hb, to_bin_x(ox + m.dx), to_bin_y(oy + m.dy), m.charge);
    }
    double pos = -0.0;
    for (size_t i = 0; i < B; ++i) pos += rmax(r.density[i], 0.0);
    const size_t nf = fillers.size();
    for (size_t i = 0; i < nf; ++i) {
      if (fillers[i].field != f) continue;
      const size_t base = 2 * ((size_t)U + i);
      deposit(r.density.data(), Wb, Hb, to_bin_x(coords[base]), to_bin_y(coords[base + 1]), fillers[i].charge);
    }
    r.potential.assign(B, 0.0);
    uint64_t bad = 0;
    solver->solve(r.density.data(), r.potential.data(), r.energy, &bad);
    r.unit_gx.assign(dunits.size(), 0.0);
    r.unit_gy.assign(dunits.size(), 0.0);
    double force = 0.0;
    for (size_t ui = 0; ui < dunits.size(); ++ui) {
      const auto& u = dunits[ui];
      const double ox = coords[2 * (size_t)u.unit], oy = coords[2 * (size_t)u.unit + 1];
      for (const auto& m : u.members) {
        if (m.field != f) continue;
        double v, gx, gy;
        sample(r.potential.data(), Wb, Hb, to_bin_x(ox + m.dx), to_bin_y(oy + m.dy), v, gx, gy);
        if (!identity_map) {
          gx *= sx;
          gy *= sy;
        }
        force += m.charge * (std::fabs(gx) + std::fabs(gy));
        r.unit_gx[ui] += m.charge * gx;
        r.unit_gy[ui] += m.charge * gy;
      }
    }
    r.filler_gx.clear();
    r.filler_gy.clear();
    r.filler_index.clear();
    for (size_t i = 0; i < nf; ++i) {
      if (fillers[i].field != f) continue;
      const size_t base = 2 * ((size_t)U + i);
      double v, gx, gy;
      sample(r.potential.data(), Wb, Hb, to_bin_x(coords[base]), to_bin_y(coords[base + 1]), v, gx, gy);
      if (!identity_map) {
        gx *= sx;
        gy *= sy;
      }
      force += fillers[i].charge * (std::fabs(gx) + std::fabs(gy));
      r.filler_index.push_back((uint32_t)i);
      r.filler_gx.push_back(fillers[i].charge * gx);
      r.filler_gy.push_back(fillers[i].charge * gy);
    }
    double nc = -0.0;
    for (size_t i = 0; i < B; ++i) nc += r.density[i];
    r.net_charge = nc;
    r.force_l1 = force;
    r.available = available[f];
    r.real_area = real_area;
    r.filler_charge = filler_total(f, real_area);
    r.overflow = pos / real_area;
  }

  int32_t density_evaluate(const double* coords, int threads, Evaluation& ev, uint64_t* err) const {
    // validate_units_with_positions / validate_fillers_with_positions
    for (size_t i = 0; i < dunits.size(); ++i) {
      const double ox = coords[2 * (size_t)dunits[i].unit], oy = coords[2 * (size_t)dunits[i].unit + 1];
      for (size_t j = 0; j < dunits[i].members.size(); ++j) {
        const auto& m = dunits[i].members[j];
        if (!std::isfinite(ox) || !std::isfinite(oy) || !std::isfinite(m.dx) || !std::isfinite(m.dy)) {
          *err = i;
          return TEXO_GP_ERR_NONFINITE_UNIT_COORDINATE;
        }
        if (!std::isfinite(m.charge) || m.charge <= 0.0) {
          *err = i;
          return TEXO_GP_ERR_INVALID_MEMBER_CHARGE;
        }
      }
    }
    for (size_t i = 0; i < fillers.size(); ++i) {
      const size_t base = 2 * ((size_t)U + i);
      if (!std::isfinite(coords[base]) || !std::isfinite(coords[base + 1]) || !std::isfinite(fillers[i].charge)) {
        *err = i;
        return TEXO_GP_ERR_NONFINITE_FILLER;
      }
      if (fillers[i].charge < 0.0) {
        *err = i;
        return TEXO_GP_ERR_NEGATIVE_FILLER_CHARGE;
      }
    }
    std::vector<uint64_t> counts;
    std::vector<double> areas;
    real_counts(counts, areas);
    // validate_filler_totals
    std::vector<double> supplied(K, 0.0);
    for (size_t i = 0; i < fillers.size(); ++i) {
      if (counts[fillers[i].field] == 0) {
        *err = i;
        return TEXO_GP_ERR_UNEXPECTED_FILLER_KIND;
      }
      supplied[fillers[i].field] += fillers[i].charge;
    }
    for (uint32_t f = 0; f < K; ++f) {
      if (counts[f] == 0) continue;
      int32_t st = capacity_checks(f, counts[f], areas[f]);
      if (st) {
        *err = f;
        return st;
      }
      const double expected = filler_total(f, areas[f]);
      if (std::fabs(supplied[f] - expected) > 1.0e-9 * rmax(expected, 1.0)) {
        *err = f;
        return TEXO_GP_ERR_FILLER_CHARGE_MISMATCH;
      }
    }
    ev.fields.assign(K, FieldResult());
    auto run = [&](uint32_t f) {
      ev.fields[f].real_charge = counts[f];
      eval_field(f, coords, ev.fields[f], areas[f]);
    };
    if (threads > 1 && K > 1) {
      std::vector<std::thread> ts;
      for (uint32_t f = 1; f < K; ++f) ts.emplace_back(run, f);
      run(0);
      for (auto& t : ts) t.join();
    } else {
      for (uint32_t f = 0; f < K; ++f) run(f);
    }
    for (uint32_t f = 0; f < K; ++f)
      for (size_t i = 0; i < bins(); ++i)
        if (!std::isfinite(ev.fields[f].density[i])) {
          *err = i;
          return TEXO_GP_ERR_NONFINITE_DENSITY;
        }
    return TEXO_GP_OK;
  }

  // ContinuousProblem::evaluate (eplace.rs:137-205): WA || density.
  int32_t evaluate(const double* coords, double gamma, int threads, Evaluation& ev, uint64_t* err) const {
    int32_t st = TEXO_GP_OK;
    if (threads > 1) {
      std::thread wa([&] { wa_objective(coords, gamma, threads, ev); });
      Evaluation dens;
      st = density_evaluate(coords, threads, dens, err);
      wa.join();
      ev.fields = std::move(dens.fields);
    } else {
      wa_objective(coords, gamma, 1, ev);
      st = density_evaluate(coords, 1, ev, err);
    }
    return st;
  }

  // add_scaled_field_gradient (eplace.rs:213-231)
  void add_field_gradient(const FieldResult& fr, double coef, double* g) const {
    for (size_t i = 0; i < dunits.size(); ++i) {
      g[2 * (size_t)dunits[i].unit] += coef * fr.unit_gx[i];
      g[2 * (size_t)dunits[i].unit + 1] += coef * fr.unit_gy[i];
    }
    for (size_t j = 0; j < fr.filler_index.size(); ++j) {
      const size_t c = 2 * ((size_t)U + fr.filler_index[j]);
      g[c] += coef * fr.filler_gx[j];
      g[c + 1] += coef * fr.filler_gy[j];
    }
  }

  double hpwl(const double* coords) const {
    double total = 0.0;
    for (size_t e = 0; e + 1 < net_ptr.size(); ++e) {
      for (int axis = 0; axis < 2; ++axis) {
        double lo = pin_coord(pins[net_ptr[e]], coords, axis), hi = lo;
        for (size_t p = net_ptr[e] + 1; p < net_ptr[e + 1]; ++p) {
          const double v = pin_coord(pins[p], coords, axis);
          lo = rmin(lo, v);
          hi = rmax(hi, v);
        }
        total += hi - lo;
      }
    }
    return total;
  }
};

// ---------------------------------------------------------------------------
// Dynamic Nesterov step (global_placement.rs:121-335).
// ---------------------------------------------------------------------------
struct Bounds {
  const double* lo;
  size_t lo_len;
  const double* hi;
  size_t hi_len;
};
struct NState {
  std::vector<double> x, prev;
  double a = 1.0;
  bool has_L = false;
  double L = 0.0;
};
struct StepOut {
  bool stationary = false;
  double objective = 0, stationarity = 0, coordinate_change = 0;
  uint64_t trials = 0;
  int64_t payload = -1;
  int32_t inner = 0;
  uint64_t error_index = 0, expected = 0, actual = 0;
};
// evaluator: returns 0 or an error code; fills value, gradient, payload.
using Evaluator = std::function<int32_t(const std::vector<double>&, double&, std::vector<double>&, int64_t&)>;

int32_t validate_bounds(const std::vector<double>& x, const Bounds& b, uint64_t* idx) {
  if (b.lo_len != x.size() || b.hi_len != x.size()) return TEXO_GP_ERR_INVALID_BOUNDS;
  for (size_t i = 0; i < x.size(); ++i) {
    if (!std::isfinite(b.lo[i]) || !std::isfinite(b.hi[i]) || b.lo[i] > b.hi[i]) return TEXO_GP_ERR_INVALID_BOUNDS;
    if (!std::isfinite(x[i])) {
      *idx = i;
      return TEXO_GP_ERR_INVALID_INITIAL_COORDINATE;
    }
  }
  return TEXO_GP_OK;
}
std::vector<double> project(const std::vector<double>& x, const Bounds& b) {
  std::vector<double> r(x.size());
  for (size_t i = 0; i < x.size(); ++i) r[i] = rclamp(x[i], b.lo[i], b.hi[i]);
  return r;
}
inline double kkt_component(size_t i, double g, const double* x, const double* lo, const double* hi) {
  if (total_cmp(lo[i], hi[i]) == 0 || (x[i] <= lo[i] && g > 0.0) || (x[i] >= hi[i] && g < 0.0)) return 0.0;
  return std::fabs(g);
}
double kkt_residual(const double* g, const double* x, const double* lo, const double* hi, const double* m,
                    size_t n) {
  double r = 0.0;
  for (size_t i = 0; i < n; ++i) r = rmax(r, kkt_component(i, g[i], x, lo, hi) / std::sqrt(m[i]));
  return r;
}
inline double half_nonzero(double v) {
  const double h = v * 0.5;
  return h == 0.0 ? v : h;
}
inline double rounding_margin(double a, double b) { return kEps * (1.0 + std::fabs(a) + std::fabs(b)); }

int32_t checked(const std::vector<double>& x, double value, const std::vector<double>& g, StepOut& out) {
  if (!std::isfinite(value)) return TEXO_GP_ERR_INVALID_OBJECTIVE;
  if (g.size() != x.size()) {
    out.expected = x.size();
    out.actual = g.size();
    return TEXO_GP_ERR_INVALID_GRADIENT_LENGTH;
  }
  for (size_t i = 0; i < g.size(); ++i)
    if (!std::isfinite(g[i])) {
      out.error_index = i;
      return TEXO_GP_ERR_NONFINITE_GRADIENT;
    }
  return TEXO_GP_OK;
}

int32_t dynamic_nesterov_step(NState& st, const Bounds& b, const double* metric, size_t metric_len,
                              const Evaluator& evaluate, StepOut& out) {
  int32_t s;
  if ((s = validate_bounds(st.x, b, &out.error_index))) return s;
  if ((s = validate_bounds(st.prev, b, &out.error_index))) return s;
  if (metric_len != st.x.size()) {
    out.expected = st.x.size();
    out.actual = metric_len;
    return TEXO_GP_ERR_INVALID_METRIC_LENGTH;
  }
  for (size_t i = 0; i < metric_len; ++i)
    if (!std::isfinite(metric[i]) || metric[i] <= 0.0) {
      out.error_index = i;
      return TEXO_GP_ERR_NONPOSITIVE_METRIC;
    }
  if (!std::isfinite(st.a) || st.a < 1.0) return TEXO_GP_ERR_INVALID_MOMENTUM_PARAMETER;
  if (st.has_L && (!std::isfinite(st.L) || st.L <= 0.0)) return TEXO_GP_ERR_INVALID_LIPSCHITZ_ESTIMATE;
  const size_t n = st.x.size();
  const std::vector<double> origin = project(st.x, b);
  const std::vector<double> previous = project(st.prev, b);
  double f_origin;
  std::vector<double> g_origin;
  int64_t origin_payload;
  if ((s = evaluate(origin, f_origin, g_origin, origin_payload))) {
    out.inner = s;
    return TEXO_GP_ERR_EVALUATION;
  }
  if ((s = checked(origin, f_origin, g_origin, out))) return s;
  bool restart = false;
  bool has_wL = st.has_L;
  double wL = st.L;
  uint64_t trials = 0;
  std::vector<double> y(n), cand(n), delta(n), g_y, g_c;
  for (;;) {  // 'step
    const double momentum = restart ? 1.0 : st.a;
    const double next_m = midpoint(1.0, std::sqrt(1.0 + 4.0 * momentum * momentum));
    if (!std::isfinite(next_m)) return TEXO_GP_ERR_ITERATION_OVERFLOW;
    const double extrap = (momentum - 1.0) / next_m;
    if (restart) {
      y = origin;
    } else {
      for (size_t i = 0; i < n; ++i) y[i] = rclamp(origin[i] + extrap * (origin[i] - previous[i]), b.lo[i], b.hi[i]);
    }
    const bool y_is_origin = (y == origin);
    double f_y;
    if (y_is_origin) {
      f_y = f_origin;
      g_y = g_origin;
    } else {
      int64_t pl;
      if ((s = evaluate(y, f_y, g_y, pl))) {
        out.inner = s;
        return TEXO_GP_ERR_EVALUATION;
      }
      if ((s = checked(y, f_y, g_y, out))) return s;
    }
    const double y_stat = kkt_residual(g_y.data(), y.data(), b.lo, b.hi, metric, n);
    if (!std::isfinite(y_stat)) return TEXO_GP_ERR_LINE_SEARCH_OVERFLOW;
    if (y_stat == 0.0) {
      if (!y_is_origin) {
        restart = true;
        continue;
      }
      st.x = origin;
      st.prev = origin;
      st.a = 1.0;
      out.stationary = true;
      out.objective = f_origin;
      out.stationarity = kkt_residual(g_origin.data(), origin.data(), b.lo, b.hi, metric, n);
      out.coordinate_change = 0.0;
      out.trials = trials;
      out.payload = origin_payload;
      return TEXO_GP_OK;
    }
    const double initial_L = has_wL ? wL : y_stat;
    double tL = half_nonzero(initial_L);
    bool may_reduce = true;
    double f_c = 0;
    int64_t cand_payload = -1;
    bool restart_step = false;
    for (;;) {
      trials += 1;
      bool underflow = false;
      for (size_t i = 0; i < n; ++i) {
        const double d = tL * metric[i];
        if (!std::isfinite(d)) return TEXO_GP_ERR_LINE_SEARCH_OVERFLOW;
        underflow |= d == 0.0;
      }
      if (underflow) {
        tL *= 2.0;
        may_reduce = false;
        if (!std::isfinite(tL)) return TEXO_GP_ERR_LINE_SEARCH_OVERFLOW;
        continue;
      }
      for (size_t i = 0; i < n; ++i) cand[i] = rclamp(y[i] - g_y[i] / (tL * metric[i]), b.lo[i], b.hi[i]);
      if (cand == y) {
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
        st.x = origin;
        st.prev = origin;
        st.a = 1.0;
        st.has_L = true;
        st.L = tL;
        out.stationary = true;
        out.objective = f_origin;
        out.stationarity = kkt_residual(g_origin.data(), origin.data(), b.lo, b.hi, metric, n);
        out.coordinate_change = 0.0;
        out.trials = trials;
        out.payload = origin_payload;
        return TEXO_GP_OK;
      }
      if ((s = evaluate(cand, f_c, g_c, cand_payload))) {
        out.inner = s;
        return TEXO_GP_ERR_EVALUATION;
      }
      if ((s = checked(cand, f_c, g_c, out))) return s;
      for (size_t i = 0; i < n; ++i) delta[i] = cand[i] - y[i];
      double msn = -0.0;
      for (size_t i = 0; i < n; ++i) msn += metric[i] * delta[i] * delta[i];
      const double upper = f_y + dotv(g_y.data(), delta.data(), n) + 0.5 * tL * msn;
      if (!std::isfinite(upper)) return TEXO_GP_ERR_LINE_SEARCH_OVERFLOW;
      const bool smooth = f_c <= upper + rounding_margin(f_c, upper);
      const bool mono = f_c <= f_origin + rounding_margin(f_c, f_origin);
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
    double change = 0.0;
    for (size_t i = 0; i < n; ++i) change = rmax(change, std::fabs(cand[i] - origin[i]));
    const double stat = kkt_residual(g_c.data(), cand.data(), b.lo, b.hi, metric, n);
    if (!std::isfinite(stat)) return TEXO_GP_ERR_LINE_SEARCH_OVERFLOW;
    st.prev = origin;
    st.x = cand;
    st.a = next_m;
    st.has_L = true;
    st.L = tL;
    out.stationary = false;
    out.objective = f_c;
    out.stationarity = stat;
    out.coordinate_change = change;
    out.trials = trials;
    out.payload = cand_payload;
    return TEXO_GP_OK;
  }
}

// ---------------------------------------------------------------------------
// eplace rules (eplace.rs:1111-1415).
// ---------------------------------------------------------------------------
double overflow_target(uint32_t kind) {
  switch (kind) {
    case TEXO_GP_KIND_MEMORY:
    case TEXO_GP_KIND_DSP:
      return 0.20;
    case TEXO_GP_KIND_LUT:
    case TEXO_GP_KIND_REGISTER:
      return 0.10;
    default:
      return 0.0;
  }
}
void augmented(double energy, double e0, double lambda, double beta, double& value, double& coef) {
  const double ne = energy / e0;
  value = lambda * e0 * (ne + 0.5 * beta * ne * ne);
  coef = lambda * (1.0 + beta * ne);
}
int32_t growth_from_log(double lg, double lo, double hi, double& g) {
  if (!std::isfinite(lg) || lg < 0.0) return TEXO_GP_ERR_INVALID_NORMALIZATION;
  const double interp = 1.0 - 1.0 / (1.0 + lg);
  g = lo + interp * (hi - lo);
  if (std::isfinite(g) && g >= lo && g <= hi) return TEXO_GP_OK;
  return TEXO_GP_ERR_INVALID_NORMALIZATION;
}
int32_t field_gamma(double overflow, double target, double base, double& g) {
  if (!std::isfinite(overflow) || overflow < 0.0 || !std::isfinite(target) || !(target >= 0.0 && target < 1.0) ||
      !std::isfinite(base) || base <= 0.0)
    return TEXO_GP_ERR_INVALID_NORMALIZATION;
  const double slope = 2.0 / (1.0 - target);
  const double intercept = 1.0 - slope;
  g = base * std::pow(10.0, slope * overflow + intercept);
  if (std::isfinite(g) && g > 0.0) return TEXO_GP_OK;
  return TEXO_GP_ERR_INVALID_NORMALIZATION;
}
int32_t weighted_gamma_mean(const double* gm, const double* w, size_t n, double fallback, double& mean) {
  if (!std::isfinite(fallback) || fallback <= 0.0) return TEXO_GP_ERR_INVALID_NORMALIZATION;
  double ws = 0.0, wsum = 0.0;
  for (size_t i = 0; i < n; ++i) {
    if (!std::isfinite(gm[i]) || gm[i] <= 0.0 || !std::isfinite(w[i]) || w[i] < 0.0)
      return TEXO_GP_ERR_INVALID_NORMALIZATION;
    ws += gm[i] * w[i];
    wsum += w[i];
  }
  mean = wsum == 0.0 ? fallback : ws / wsum;
  if (std::isfinite(mean) && mean > 0.0) return TEXO_GP_OK;
  return TEXO_GP_ERR_INVALID_NORMALIZATION;
}

// area_adjustment_is_ready (eplace.rs:1403-1408): the LUT and register
// fields at AREA_ADJUSTMENT_OVERFLOW_TARGET = 0.15 (eplace.rs:130)
bool area_adjustment_ready(uint32_t K, const uint32_t* kinds, const double* overflow) {
  for (uint32_t f = 0; f < K; ++f) {
    if (kinds[f] != TEXO_GP_KIND_LUT && kinds[f] != TEXO_GP_KIND_REGISTER) continue;
    if (!(overflow[f] <= 0.15)) return false;
  }
  return true;
}
// normalized_density_subgradient (eplace.rs:1154-1175) with validate_fields
int32_t density_subgradient(uint32_t K, const double* energy, const double* scales, double beta,
                            std::vector<double>& sg) {
  for (uint32_t f = 0; f < K; ++f)
    if (!std::isfinite(energy[f]) || !std::isfinite(scales[f]) || scales[f] <= 0.0)
      return TEXO_GP_ERR_DENSITY_FIELD_CHANGED;
  sg.resize(K);
  for (uint32_t f = 0; f < K; ++f) {
    const double ne = energy[f] / scales[f];
    sg[f] = ne + 0.5 * beta * ne * ne;
    if (!std::isfinite(sg[f]) || sg[f] < 0.0) return TEXO_GP_ERR_INVALID_NORMALIZATION;
  }
  return TEXO_GP_OK;
}
// area_adjusted_density_multipliers (eplace.rs:1183-1218), elfPlace eq. (27):
// lambda_f = 0.1 |grad W|_1 / (sum_f force_l1_f sg_f) * sg_f; `wa_l1` is
// |grad W|_1 summed in the reference's order
int32_t area_adjusted_multipliers(uint32_t K, const double* energy, const double* force_l1, const double* scales,
                                  double beta, double wa_l1, std::vector<double>& lambda) {
  std::vector<double> sg;
  int32_t s = density_subgradient(K, energy, scales, beta, sg);
  if (s) return s;
  double dens = 0.0;
  for (uint32_t f = 0; f < K; ++f) dens += force_l1[f] * sg[f];
  if (!std::isfinite(wa_l1) || wa_l1 <= 0.0 || !std::isfinite(dens) || dens <= 0.0)
    return TEXO_GP_ERR_INVALID_NORMALIZATION;
  const double scale = 0.1 * wa_l1 / dens;
  lambda.assign(K, 0.0);
  bool any = false;
  for (uint32_t f = 0; f < K; ++f) {
    lambda[f] = scale * sg[f];
    if (!std::isfinite(lambda[f]) || lambda[f] < 0.0) return TEXO_GP_ERR_INVALID_NORMALIZATION;
    any = any || lambda[f] > 0.0;
  }
  return any ? TEXO_GP_OK : TEXO_GP_ERR_INVALID_NORMALIZATION;
}

struct Eplace {
  Oracle& o;
  int threads;
  double gamma_base_tiles;
  static constexpr size_t kTraceMax = 4096;
  std::vector<texo_gp_iteration>* trace = nullptr;   // per-iteration controller records (optional)
  explicit Eplace(Oracle& oo, int th) : o(oo), threads(th) {
    const double bin_width = o.identity_map ? 1.0 : 1.0 / o.sx;
    gamma_base_tiles = o.params.gamma_base * bin_width;
  }
  double target_of(uint32_t f) const {
    if (o.params.overflow_target_override >= 0.0) return o.params.overflow_target_override;
    return overflow_target(o.field_kind[f].kind);
  }
  int32_t adaptive_gamma(const Evaluation& ev, double& gamma) const {
    std::vector<double> gm(o.K), w(o.K);
    for (uint32_t f = 0; f < o.K; ++f) {
      int32_t s = field_gamma(ev.fields[f].overflow, target_of(f), gamma_base_tiles, gm[f]);
      if (s) return s;
      w[f] = o.gamma_weights[f];
    }
    return weighted_gamma_mean(gm.data(), w.data(), o.K, gamma_base_tiles, gamma);
  }
  // density_stop_reached (eplace.rs:1397-1415): Final (every field at its
  // target) or, before an area adjustment, AreaAdjustmentReady (the LUT and
  // register fields at AREA_ADJUSTMENT_OVERFLOW_TARGET = 0.15, eplace.rs:130).
  int stop_mode = 0;
  bool stop_reached(const Evaluation& ev) const {
    if (stop_mode == 1) {
      std::vector<uint32_t> kinds(o.K);
      std::vector<double> ov(o.K);
      for (uint32_t f = 0; f < o.K; ++f) {
        kinds[f] = o.field_kind[f].kind;
        ov[f] = ev.fields[f].overflow;
      }
      return area_adjustment_ready(o.K, kinds.data(), ov.data());
    }
    for (uint32_t f = 0; f < o.K; ++f)
      if (!(ev.fields[f].overflow <= target_of(f))) return false;
    return true;
  }
  // area_adjusted_density_multipliers (eplace.rs:1183-1218) and
  // area_adjusted_multiplier_step (:1220-1232): elfPlace eqs. (27)-(28).
  int32_t area_multipliers(const Evaluation& ev, const std::vector<double>& scales, std::vector<double>& lambda,
                           double& step) const {
    if (ev.fields.size() != scales.size()) return TEXO_GP_ERR_DENSITY_FIELD_CHANGED;
    double wl = 0.0;
    for (uint32_t u = 0; u < o.U; ++u) {
      wl += std::fabs(ev.wa_gx[u]);
      wl += std::fabs(ev.wa_gy[u]);
    }
    std::vector<double> energy(o.K), force(o.K);
    for (uint32_t f = 0; f < o.K; ++f) {
      energy[f] = ev.fields[f].energy;
      force[f] = ev.fields[f].force_l1;
    }
    int32_t s = area_adjusted_multipliers(o.K, energy.data(), force.data(), scales.data(), o.params.beta, wl, lambda);
    if (s) return s;
    double nn = 0.0;
    for (double m : lambda) nn += m * m;
    step = (o.params.alpha_high - 1.0) * std::sqrt(nn);
    return (std::isfinite(step) && step > 0.0) ? TEXO_GP_OK : TEXO_GP_ERR_INVALID_NORMALIZATION;
  }
  void excess(const Evaluation& ev, double& mx, double& tot) const {
    mx = 0.0;
    tot = 0.0;
    for (uint32_t f = 0; f < o.K; ++f) {
      const double e = rmax(ev.fields[f].overflow - target_of(f), 0.0);
      mx = rmax(mx, e);
      tot = tot + e;
    }
  }
  int32_t validate_initial(const Evaluation& ev) const {
    bool ok = std::isfinite(ev.wa_value);
    for (uint32_t u = 0; u < o.U && ok; ++u) ok = std::isfinite(ev.wa_gx[u]) && std::isfinite(ev.wa_gy[u]);
    for (const auto& fr : ev.fields) {
      if (!ok) break;
      ok = std::isfinite(fr.energy) && fr.energy >= 0.0 && std::isfinite(fr.overflow) && std::isfinite(fr.net_charge) &&
           std::isfinite(fr.force_l1) && fr.force_l1 >= 0.0;
      for (size_t i = 0; ok && i < fr.unit_gx.size(); ++i) ok = std::isfinite(fr.unit_gx[i]) && std::isfinite(fr.unit_gy[i]);
      for (size_t i = 0; ok && i < fr.filler_gx.size(); ++i)
        ok = std::isfinite(fr.filler_gx[i]) && std::isfinite(fr.filler_gy[i]);
    }
    return ok ? TEXO_GP_OK : TEXO_GP_ERR_INVALID_NORMALIZATION;
  }
  int32_t validate_fields(const Evaluation& ev, const std::vector<double>& scales) const {
    if (ev.fields.size() != scales.size()) return TEXO_GP_ERR_DENSITY_FIELD_CHANGED;
    for (size_t f = 0; f < scales.size(); ++f)
      if (!std::isfinite(ev.fields[f].energy) || !std::isfinite(scales[f]) || scales[f] <= 0.0)
        return TEXO_GP_ERR_DENSITY_FIELD_CHANGED;
    return TEXO_GP_OK;
  }
  void combined(const Evaluation& ev, const std::vector<double>& scales, const std::vector<double>& lambda,
                size_t n, double& value, std::vector<double>& g) const {
    value = ev.wa_value;
    g.assign(n, 0.0);
    for (uint32_t u = 0; u < o.U; ++u) {
      g[2 * (size_t)u] = ev.wa_gx[u];
      g[2 * (size_t)u + 1] = ev.wa_gy[u];
    }
    for (uint32_t f = 0; f < o.K; ++f) {
      double fv, coef;
      augmented(ev.fields[f].energy, scales[f], lambda[f], o.params.beta, fv, coef);
      value += fv;
      o.add_field_gradient(ev.fields[f], coef, g.data());
    }
  }
  int32_t preconditioner(const std::vector<double>& lambda, size_t n, std::vector<double>& diag) const {
    diag.assign(n, 0.0);
    for (uint32_t u = 0; u < o.U; ++u) diag[2 * (size_t)u] = diag[2 * (size_t)u + 1] = o.wl_precond[u];
    for (uint32_t f = 0; f < o.K; ++f) {
      const double c = lambda[f];
      if (!std::isfinite(c) || c < 0.0) return TEXO_GP_ERR_INVALID_NORMALIZATION;
      for (const auto& du : o.dunits) {
        double q = -0.0;
        for (const auto& m : du.members)
          if (m.field == f) q += m.charge;
        if (q == 0.0) continue;
        const double curv = c * q;
        diag[2 * (size_t)du.unit] += curv;
        diag[2 * (size_t)du.unit + 1] += curv;
      }
      for (size_t i = 0; i < o.fillers.size(); ++i) {
        if (o.fillers[i].field != f) continue;
        const size_t cc = 2 * ((size_t)o.U + i);
        const double curv = c * o.fillers[i].charge;
        diag[cc] += curv;
        diag[cc + 1] += curv;
      }
    }
    for (auto& d : diag) {
      if (!std::isfinite(d) || d < 0.0) return TEXO_GP_ERR_INVALID_NORMALIZATION;
      d = rmax(d, 1.0);
    }
    return TEXO_GP_OK;
  }
  int32_t initial_multiplier(const Evaluation& ev, size_t n, double& m) const {
    double wl = 0.0;
    for (uint32_t u = 0; u < o.U; ++u) {
      wl += std::fabs(ev.wa_gx[u]);
      wl += std::fabs(ev.wa_gy[u]);
    }
    double dens = 0.0;
    for (uint32_t f = 0; f < o.K; ++f) {
      std::vector<double> g(n, 0.0);
      o.add_field_gradient(ev.fields[f], 1.0, g.data());
      double l1 = 0.0;
      for (double v : g) l1 += std::fabs(v);
      dens += l1;
    }
    m = (wl == 0.0 || dens == 0.0) ? 1.0 : o.params.initial_density_weight * wl / dens;
    return (std::isfinite(m) && m > 0.0) ? TEXO_GP_OK : TEXO_GP_ERR_INVALID_NORMALIZATION;
  }
  int32_t subgradient(const Evaluation& ev, const std::vector<double>& scales, std::vector<double>& sg) const {
    int32_t s = validate_fields(ev, scales);
    if (s) return s;
    sg.resize(o.K);
    for (uint32_t f = 0; f < o.K; ++f) {
      const double ne = ev.fields[f].energy / scales[f];
      sg[f] = ne + 0.5 * o.params.beta * ne * ne;
      if (!std::isfinite(sg[f]) || sg[f] < 0.0) return TEXO_GP_ERR_INVALID_NORMALIZATION;
    }
    return TEXO_GP_OK;
  }
  int32_t update_multipliers(std::vector<double>& lambda, double step, const Evaluation& ev,
                             const std::vector<double>& scales) const {
    std::vector<double> sg;
    int32_t s = subgradient(ev, scales, sg);
    if (s) return s;
    double nn = 0.0;
    for (double v : sg) nn += v * v;
    const double norm = std::sqrt(nn);
    if (norm == 0.0) return TEXO_GP_OK;
    if (!std::isfinite(norm) || !std::isfinite(step) || step <= 0.0) return TEXO_GP_ERR_INVALID_NORMALIZATION;
    for (uint32_t f = 0; f < o.K; ++f) {
      lambda[f] += step * sg[f] / norm;
      if (!std::isfinite(lambda[f]) || lambda[f] < 0.0) return TEXO_GP_ERR_INVALID_NORMALIZATION;
    }
    return TEXO_GP_OK;
  }
  int32_t next_step(double prev, const Evaluation& ev, const std::vector<double>& scales, double& next) const {
    int32_t s = validate_fields(ev, scales);
    if (s) return s;
    double nn = 0.0;
    for (uint32_t f = 0; f < o.K; ++f) {
      const double ne = ev.fields[f].energy / scales[f];
      nn += ne * ne;
    }
    const double lg = std::log(o.params.beta * std::sqrt(nn) + 1.0);
    double g;
    s = growth_from_log(lg, o.params.alpha_low, o.params.alpha_high, g);
    if (s) return s;
    next = prev * g;
    return (std::isfinite(next) && next > 0.0) ? TEXO_GP_OK : TEXO_GP_ERR_INVALID_NORMALIZATION;
  }
  static uint32_t rounded(double v, uint32_t extent) {
    double r = rclamp(std::round(v), 0.0, (double)(extent - 1));
    return (uint32_t)r;
  }
  void targets(const std::vector<double>& x, std::vector<uint32_t>& t) const {
    t.resize(2 * (size_t)o.U);
    for (uint32_t u = 0; u < o.U; ++u) {
      t[2 * (size_t)u] = rounded(x[2 * (size_t)u], o.W);
      t[2 * (size_t)u + 1] = rounded(x[2 * (size_t)u + 1], o.H);
    }
  }

  // optimize_density_once (eplace.rs:439-582) with the Final stop criterion.
  // One round of eplace::place (optimize_density_once): from `start` (the
  // initial coordinates when null), with fixed density scales when given,
  // the area-reset multipliers when `reset`, and the iteration count of the
  // earlier rounds (the cap counts all rounds).
  const double* start = nullptr;
  const double* fixed_scales = nullptr;
  bool reset = false;
  uint64_t offset = 0;
  std::vector<double> scales_used;
  bool exhausted_out = false;
  int32_t run(uint32_t cap_override, std::vector<uint32_t>& best_targets, std::vector<double>& final_coords,
              orc_run_stats& stats) {
    const size_t n = o.coord_count();
    std::vector<double> coords = start ? std::vector<double>(start, start + n) : o.init_coords;
    Bounds b{o.lower.data(), o.lower.size(), o.upper.data(), o.upper.size()};
    uint64_t err = 0;
    stats = orc_run_stats{};
    stats.num_fields = o.K;
    Evaluation probe;
    int32_t s = o.evaluate(coords.data(), gamma_base_tiles, threads, probe, &err);
    stats.evaluations++;
    if (s) return s;
    if ((s = validate_initial(probe))) return s;
    double g0;
    if ((s = adaptive_gamma(probe, g0))) return s;
    Evaluation initial;
    s = o.evaluate(coords.data(), g0, threads, initial, &err);
    stats.evaluations++;
    if (s) return s;
    if ((s = validate_initial(initial))) return s;
    std::vector<double> scales(o.K);
    for (uint32_t f = 0; f < o.K; ++f) scales[f] = fixed_scales ? fixed_scales[f] : rmax(initial.fields[f].energy, 1.0);
    scales_used = scales;
    if ((s = validate_fields(initial, scales))) return s;
    NState st;
    st.x = (b.lo_len == coords.size() && b.hi_len == coords.size()) ? project(coords, b) : coords;
    st.prev = st.x;
    std::vector<uint32_t> rt;
    targets(st.x, best_targets);
    double best_max, best_tot;
    excess(initial, best_max, best_tot);
    auto finish = [&](const Evaluation& cur) {
      final_coords = st.x;
      for (uint32_t f = 0; f < o.K && f < TEXO_GP_MAX_FIELDS; ++f) stats.overflow[f] = cur.fields[f].overflow;
      stats.converged = stop_reached(cur) ? 1u : 0u;
      stats.hpwl = o.hpwl(final_coords.data());
    };
    if (stop_reached(initial)) {
      finish(initial);
      stats.iterations = (uint32_t)offset;
      return TEXO_GP_OK;
    }
    std::vector<double> lambda;
    double mstep = o.params.alpha_high - 1.0;
    if (reset) {
      if ((s = area_multipliers(initial, scales, lambda, mstep))) return s;
    } else {
      double m0;
      if ((s = initial_multiplier(initial, n, m0))) return s;
      lambda.assign(o.K, m0);
    }
    Evaluation current = std::move(initial);
    std::vector<uint32_t> prev_stationary;
    bool have_prev_stationary = false;
    const uint32_t cap = cap_override ? cap_override : o.params.max_iterations;
    uint32_t completed = (uint32_t)offset;
    std::vector<Evaluation> payloads;
    for (;;) {
      if (stop_reached(current)) break;
      if (completed >= cap) {
        stats.exhausted = 1;
        if (!o.params.best_effort) {
          finish(current);
          stats.iterations = completed;
          return TEXO_GP_ERR_DID_NOT_CONVERGE;
        }
        break;
      }
      double gamma;
      if ((s = adaptive_gamma(current, gamma))) return s;
      completed += 1;
      std::vector<double> P;
      if ((s = preconditioner(lambda, n, P))) return s;
      payloads.clear();
      Evaluator ev = [&](const std::vector<double>& c, double& value, std::vector<double>& g, int64_t& pl) -> int32_t {
        Evaluation e;
        uint64_t eerr = 0;
        int32_t es = o.evaluate(c.data(), gamma, threads, e, &eerr);
        stats.evaluations++;
        if (es) return es;
        combined(e, scales, lambda, c.size(), value, g);
        payloads.push_back(std::move(e));
        pl = (int64_t)payloads.size() - 1;
        return TEXO_GP_OK;
      };
      StepOut so;
      s = dynamic_nesterov_step(st, b, P.data(), P.size(), ev, so);
      if (s) {
        stats.inner_status = so.inner;
        stats.iterations = completed;
        return s;
      }
      stats.line_search_trials += so.trials;
      stats.objective = so.objective;
      stats.gamma = gamma;
      current = std::move(payloads[(size_t)so.payload]);
      if ((s = validate_fields(current, scales))) return s;
      if (trace && trace->size() < kTraceMax) {
        texo_gp_iteration rec{};
        rec.iteration = completed;
        rec.trials = (uint32_t)so.trials;
        rec.gamma = gamma;
        rec.objective = so.objective;
        rec.lipschitz = st.has_L ? st.L : 0.0;
        rec.momentum = st.a;
        for (uint32_t f = 0; f < o.K && f < TEXO_GP_MAX_FIELDS; ++f) {
          rec.lambda[f] = lambda[f];
          rec.energy_scale[f] = scales[f];
          rec.overflow[f] = current.fields[f].overflow;
        }
        trace->push_back(rec);
      }
      targets(st.x, rt);
      double mx, tot;
      excess(current, mx, tot);
      int c1 = total_cmp(mx, best_max);
      if (c1 < 0 || (c1 == 0 && total_cmp(tot, best_tot) < 0)) {
        best_targets = rt;
        best_max = mx;
        best_tot = tot;
      }
      if (stop_reached(current)) break;
      // stationary_target_is_fixed (eplace.rs:973-985)
      if (!so.stationary) {
        have_prev_stationary = false;
      } else {
        bool fixed = have_prev_stationary && prev_stationary == rt;
        prev_stationary = rt;
        have_prev_stationary = true;
        if (fixed) {
          stats.exhausted = 1;
          if (!o.params.best_effort) {
            finish(current);
            stats.iterations = completed;
            return TEXO_GP_ERR_DID_NOT_CONVERGE;
          }
          break;
        }
      }
      if ((s = update_multipliers(lambda, mstep, current, scales))) return s;
      double ns;
      if ((s = next_step(mstep, current, scales, ns))) return s;
      mstep = ns;
    }
    stats.iterations = completed;
    finish(current);
    return TEXO_GP_OK;
  }
};

}  // namespace

// ---------------------------------------------------------------------------
// C API
// ---------------------------------------------------------------------------
struct orc_handle_s {
  Oracle o;
  std::vector<texo_gp_iteration> trace;   // of the last orc_place
};

extern "C" {

void orc_bspline_axis(uint64_t length, double coordinate, uint64_t index[3], double weight[3],
                      double derivative[3]) {
  auto a = bspline_axis((size_t)length, coordinate);
  for (int i = 0; i < 3; ++i) {
    index[i] = a[i].index;
    weight[i] = a[i].weight;
    derivative[i] = a[i].derivative;
  }
}
void orc_deposit(double* density, uint64_t width, uint64_t height, double x, double y, double charge) {
  deposit(density, (size_t)width, (size_t)height, x, y, charge);
}
void orc_sample(const double* potential, uint64_t width, uint64_t height, double x, double y, double out[3]) {
  sample(potential, (size_t)width, (size_t)height, x, y, out[0], out[1], out[2]);
}
void orc_deposit_bilinear(double* density, uint64_t width, uint64_t height, double x, double y, double charge) {
  auto ax = interp_axis((size_t)width, x);
  auto ay = interp_axis((size_t)height, y);
  const size_t rows[2] = {ay.lower, ay.upper};
  const double wy[2] = {1.0 - ay.fraction, ay.fraction};
  const size_t cols[2] = {ax.lower, ax.upper};
  const double wx[2] = {1.0 - ax.fraction, ax.fraction};
  for (int r = 0; r < 2; ++r)
    for (int c = 0; c < 2; ++c) density[rows[r] * width + cols[c]] += charge * wx[c] * wy[r];
}
void orc_sample_bilinear(const double* p, uint64_t width, uint64_t height, double x, double y, double out[3]) {
  auto ax = interp_axis((size_t)width, x);
  auto ay = interp_axis((size_t)height, y);
  auto at = [&](size_t r, size_t c) { return p[r * width + c]; };
  const double p00 = at(ay.lower, ax.lower), p10 = at(ay.lower, ax.upper);
  const double p01 = at(ay.upper, ax.lower), p11 = at(ay.upper, ax.upper);
  const double tx = ax.fraction, ty = ay.fraction;
  const double lower = p00 + tx * (p10 - p00);
  const double upper = p01 + tx * (p11 - p01);
  out[0] = lower + ty * (upper - lower);
  out[1] = (1.0 - ty) * (p10 - p00) + ty * (p11 - p01);
  out[2] = (1.0 - tx) * (p01 - p00) + tx * (p11 - p10);
}
int32_t orc_poisson(uint32_t width, uint32_t height, const double* density, double* potential, double* energy,
                    int32_t matrix) {
  if (width == 0 || height == 0) return TEXO_GP_ERR_EMPTY_GRID;
  Poisson2d p(width, height);
  double e = 0;
  int32_t s = matrix ? p.solve_matrix(density, potential, e) : p.solve(density, potential, e, nullptr);
  *energy = e;
  return s;
}
void orc_dct_basis(uint32_t n, double* basis) {
  auto b = dct_basis(n);
  std::memcpy(basis, b.data(), b.size() * sizeof(double));
}

int32_t orc_create(const texo_gp_problem* p, const texo_gp_params* prm, orc_handle* out, uint64_t* error_index) {
  uint64_t dummy = 0;
  if (!error_index) error_index = &dummy;
  *out = nullptr;
  if (!p || !prm) return TEXO_GP_ERR_INVALID_ARGUMENT;
  if (p->width == 0 || p->height == 0) return TEXO_GP_ERR_EMPTY_GRID;
  auto h = std::make_unique<orc_handle_s>();
  Oracle& o = h->o;
  o.params = *prm;
  o.W = p->width;
  o.H = p->height;
  o.Wb = prm->bins_x ? prm->bins_x : p->width;
  o.Hb = prm->bins_y ? prm->bins_y : p->height;
  o.identity_map = (o.Wb == o.W && o.Hb == o.H);
  o.sx = (double)o.Wb / (double)o.W;
  o.sy = (double)o.Hb / (double)o.H;
  o.td = prm->target_density;
  if (!(o.td > 0.0 && o.td <= 1.0)) return TEXO_GP_ERR_INVALID_ARGUMENT;
  const size_t tiles = (size_t)o.W * o.H;
  // Active fields: those with at least one member.
  std::vector<uint64_t> member_count(p->num_fields, 0);
  const uint32_t U = p->num_units;
  const uint32_t M = U ? p->member_ptr[U] : 0;
  for (uint32_t m = 0; m < M; ++m) {
    if (p->member_field[m] >= p->num_fields) return TEXO_GP_ERR_INVALID_ARGUMENT;
    member_count[p->member_field[m]]++;
  }
  o.field_of_input.assign(p->num_fields, ~0u);
  std::vector<std::vector<uint32_t>> caps;
  for (uint32_t f = 0; f < p->num_fields; ++f) {
    std::vector<uint32_t> cap(p->capacity + (size_t)f * tiles, p->capacity + (size_t)(f + 1) * tiles);
    caps.push_back(cap);
  }
  // DensityModel::new fixed occupancy (electrostatic_placement.rs:155-172)
  for (uint32_t i = 0; i < p->num_fixed_occupancy; ++i) {
    const uint32_t f = p->fixed_occupancy[3 * (size_t)i], x = p->fixed_occupancy[3 * (size_t)i + 1],
                   y = p->fixed_occupancy[3 * (size_t)i + 2];
    if (x >= o.W || y >= o.H) {
      *error_index = i;
      return TEXO_GP_ERR_POINT_OUTSIDE_GRID;
    }
    if (f >= p->num_fields || caps[f][(size_t)y * o.W + x] == 0) {
      *error_index = i;
      return TEXO_GP_ERR_FIXED_CAPACITY_EXHAUSTED;
    }
    caps[f][(size_t)y * o.W + x] -= 1;
  }
  for (uint32_t f = 0; f < p->num_fields; ++f) {
    if (member_count[f] == 0) continue;
    o.field_of_input[f] = o.K++;
    o.field_kind.push_back(p->fields[f]);
    o.capacity.push_back(caps[f]);
  }
  if (o.K > TEXO_GP_MAX_FIELDS) return TEXO_GP_ERR_UNSUPPORTED;
  o.available.resize(o.K);
  o.smoothed.resize(o.K);
  for (uint32_t f = 0; f < o.K; ++f) {
    uint64_t tot = 0;
    for (auto c : o.capacity[f]) tot += c;
    o.available[f] = tot;
    o.smoothed[f].assign((size_t)o.Wb * o.Hb, 0.0);
    for (size_t i = 0; i < tiles; ++i) {
      const uint32_t c = o.capacity[f][i];
      if (c == 0) continue;
      deposit(o.smoothed[f].data(), o.Wb, o.Hb, o.to_bin_x((double)(uint32_t)(i % o.W)),
              o.to_bin_y((double)(uint32_t)(i / o.W)), o.td * (double)c);
    }
  }
  o.solver = std::make_unique<Poisson2d>(o.Wb, o.Hb);
  // Units and density members.
  o.U = U;
  o.C = p->num_cells;
  for (uint32_t u = 0; u < U; ++u) {
    const uint32_t b = p->member_ptr[u], e = p->member_ptr[u + 1];
    if (b == e) continue;
    DUnit du;
    du.unit = u;
    for (uint32_t m = b; m < e; ++m)
      du.members.push_back({o.field_of_input[p->member_field[m]], p->member_offset_xy[2 * (size_t)m],
                            p->member_offset_xy[2 * (size_t)m + 1], p->member_charge[m],
                            p->member_cell ? p->member_cell[m] : 0u});
    o.dunits.push_back(std::move(du));
  }
  o.cell_unit.assign(p->cell_unit, p->cell_unit + o.C);
  o.cell_off.assign(p->cell_offset_xy, p->cell_offset_xy + 2 * (size_t)o.C);
  o.cell_fixed.assign(p->cell_fixed, p->cell_fixed + o.C);
  o.cell_fxy.assign(p->cell_fixed_xy, p->cell_fixed_xy + 2 * (size_t)o.C);
  o.net_ptr.assign(p->net_ptr, p->net_ptr + p->num_nets + 1);
  const uint32_t P = p->net_ptr[p->num_nets];
  for (uint32_t e = 0; e < p->num_nets; ++e)
    if (p->net_ptr[e + 1] - p->net_ptr[e] < 2) {
      *error_index = e;
      return TEXO_GP_ERR_INVALID_ARGUMENT;
    }
  o.pins.resize(P);
  for (uint32_t i = 0; i < P; ++i) {
    const uint32_t c = p->pin_cell[i];
    if (c >= o.C) return TEXO_GP_ERR_INVALID_ARGUMENT;
    o.pins[i] = {o.cell_unit[c], c};
  }
  for (uint32_t a = 0; a < p->num_timed_arcs; ++a) {
    const uint32_t dc = p->arc_driver_cell[a], sc = p->arc_sink_cell[a];
    o.arcs.push_back({{o.cell_unit[dc], dc}, {o.cell_unit[sc], sc}, p->arc_extra_weight[a]});
  }
  o.build_preconditioners();
  // density_gamma_weights (eplace.rs:1424-1439)
  auto inc = o.cell_incidence();
  o.gamma_weights.assign(o.K, 0.0);
  for (const auto& du : o.dunits)
    for (const auto& m : du.members) o.gamma_weights[m.field] += inc[m.cell];
  // Fillers and coordinates (eplace.rs:312-318).
  if (!o.dunits.empty()) {
    int32_t s = o.make_fillers(error_index);
    if (s) return s;
  }
  const size_t n = o.coord_count();
  o.init_coords.resize(n);
  o.lower.resize(n);
  o.upper.resize(n);
  for (uint32_t u = 0; u < U; ++u) {
    o.init_coords[2 * (size_t)u] = p->initial_xy[2 * (size_t)u];
    o.init_coords[2 * (size_t)u + 1] = p->initial_xy[2 * (size_t)u + 1];
    o.lower[2 * (size_t)u] = p->lower_xy[2 * (size_t)u];
    o.lower[2 * (size_t)u + 1] = p->lower_xy[2 * (size_t)u + 1];
    o.upper[2 * (size_t)u] = p->upper_xy[2 * (size_t)u];
    o.upper[2 * (size_t)u + 1] = p->upper_xy[2 * (size_t)u + 1];
  }
  for (size_t i = 0; i < o.fillers.size(); ++i) {
    const size_t c = 2 * ((size_t)U + i);
    o.init_coords[c] = o.fillers[i].x;
    o.init_coords[c + 1] = o.fillers[i].y;
    o.lower[c] = 0.0;
    o.lower[c + 1] = 0.0;
    o.upper[c] = (double)(o.W - 1);
    o.upper[c + 1] = (double)(o.H - 1);
  }
  for (size_t i = 0; i < n; ++i) o.init_coords[i] = rclamp(o.init_coords[i], o.lower[i], o.upper[i]);
  *out = h.release();
  return TEXO_GP_OK;
}

void orc_destroy(orc_handle h) { delete h; }

void orc_sizes(orc_handle h, uint64_t* units, uint64_t* fillers, uint64_t* coordinates, uint32_t* bins_x,
               uint32_t* bins_y, uint32_t* num_fields) {
  if (units) *units = h->o.U;
  if (fillers) *fillers = h->o.fillers.size();
  if (coordinates) *coordinates = h->o.coord_count();
  if (bins_x) *bins_x = h->o.Wb;
  if (bins_y) *bins_y = h->o.Hb;
  if (num_fields) *num_fields = h->o.K;
}
void orc_initial(orc_handle h, double* c, double* lo, double* hi) {
  const size_t n = h->o.coord_count();
  if (c) std::memcpy(c, h->o.init_coords.data(), n * 8);
  if (lo) std::memcpy(lo, h->o.lower.data(), n * 8);
  if (hi) std::memcpy(hi, h->o.upper.data(), n * 8);
}
void orc_fillers(orc_handle h, uint32_t* field, double* charge, double* xy) {
  for (size_t i = 0; i < h->o.fillers.size(); ++i) {
    if (field) field[i] = h->o.fillers[i].field;
    if (charge) charge[i] = h->o.fillers[i].charge;
    if (xy) {
      xy[2 * i] = h->o.fillers[i].x;
      xy[2 * i + 1] = h->o.fillers[i].y;
    }
  }
}
void orc_set_filler_charge(orc_handle h, uint64_t i, double charge) {
  if (i < h->o.fillers.size()) h->o.fillers[i].charge = charge;
}
void orc_capacity(orc_handle h, uint32_t f, uint32_t* out) {
  if (f < h->o.K) std::memcpy(out, h->o.capacity[f].data(), h->o.capacity[f].size() * 4);
}

int32_t orc_evaluate(orc_handle h, const double* coords, double gamma, int32_t threads, double* wa_value,
                     orc_field_result* fields, double* wa_gradient, double* field_gradient, double* density,
                     double* potential, uint64_t* error_index) {
  Oracle& o = h->o;
  Evaluation ev;
  uint64_t err = 0;
  if (!(std::isfinite(gamma) && gamma > 0.0)) return TEXO_GP_ERR_INVALID_ARGUMENT;
  int32_t s = o.evaluate(coords, gamma, threads, ev, &err);
  if (error_index) *error_index = err;
  if (s) return s;
  if (wa_value) *wa_value = ev.wa_value;
  const size_t n = o.coord_count(), B = o.bins();
  for (uint32_t f = 0; f < o.K; ++f) {
    const auto& fr = ev.fields[f];
    if (fields) {
      fields[f].kind = o.field_kind[f].kind;
      fields[f].lut_inputs = o.field_kind[f].lut_inputs;
      fields[f].available_capacity = fr.available;
      fields[f].real_charge = fr.real_charge;
      fields[f].real_area = fr.real_area;
      fields[f].filler_charge = fr.filler_charge;
      fields[f].energy = fr.energy;
      fields[f].normalized_overflow = fr.overflow;
      fields[f].net_charge = fr.net_charge;
      fields[f].force_l1 = fr.force_l1;
    }
    if (field_gradient) {
      double* g = field_gradient + (size_t)f * n;
      std::fill(g, g + n, 0.0);
      o.add_field_gradient(fr, 1.0, g);
    }
    if (density) std::memcpy(density + (size_t)f * B, fr.density.data(), B * 8);
    if (potential) std::memcpy(potential + (size_t)f * B, fr.potential.data(), B * 8);
  }
  if (wa_gradient)
    for (uint32_t u = 0; u < o.U; ++u) {
      wa_gradient[2 * (size_t)u] = ev.wa_gx[u];
      wa_gradient[2 * (size_t)u + 1] = ev.wa_gy[u];
    }
  return TEXO_GP_OK;
}

// The device's deposit arithmetic restated: FP32 coordinates; for a bin grid
// that differs from the tile grid, the bin coordinate is the tile centre's
// FP64 value split into hi + lo floats plus the sub-tile fraction times the
// FP32 scale; FP32 offset and weights; FP32 tap rounded to nearest-even into
// int64 at 2^32 per unit charge.
struct FixedMap {
  bool identity;
  uint32_t tiles, bins;
  float scale;
  std::vector<float> hi, lo;
  FixedMap(uint32_t t, uint32_t b, bool id) : identity(id), tiles(t), bins(b) {
    scale = (float)((double)b / (double)t);
    hi.resize(t);
    lo.resize(t);
    const double sc = (double)b / (double)t;
    for (uint32_t i = 0; i < t; ++i) {
      const double v = ((double)i + 0.5) * sc - 0.5;
      hi[i] = (float)v;
      lo[i] = (float)(v - (double)hi[i]);
    }
  }
};
static inline void fixed_axis(const FixedMap& m, float s, uint32_t idx[3], float w[3]) {
  const uint32_t n = m.bins;
  const float maximum = (float)(n - 1);
  float hi, lo;
  if (m.identity) {
    hi = s;
    lo = 0.f;
  } else {
    float ts = std::nearbyint(s);
    ts = ts > 0.f ? ts : 0.f;
    ts = ts < (float)(m.tiles - 1) ? ts : (float)(m.tiles - 1);
    const uint32_t t = (uint32_t)ts;
    hi = m.hi[t];
    const float frac = s - ts;
    const float prod = frac * m.scale;
    lo = m.lo[t] + prod;
  }
  const float c = hi + lo;
  uint32_t center;
  float o;
  if (!(c > 0.f)) {
    center = 0;
    o = 0.f;
  } else if (c >= maximum) {
    center = n - 1;
    o = 0.f;
  } else {
    const float cc = std::fmin(std::floor(c + 0.5f), maximum);
    center = (uint32_t)cc;
    const float d = hi - cc;
    o = d + lo;
  }
  const float a = 0.5f - o, b = 0.5f + o;
  idx[0] = center == 0 ? 0 : center - 1;
  idx[1] = center;
  idx[2] = std::min(center + 1, n - 1);
  const float aa = a * a, bb = b * b, oo = o * o;
  w[0] = 0.5f * aa;
  w[1] = 0.75f - oo;
  w[2] = 0.5f * bb;
}
static inline int64_t to_fixed(float v) {
  const float scaled = v * 4294967296.0f;
  return (int64_t)std::nearbyint((double)scaled);
}
static void deposit_fixed(int64_t* g, const FixedMap& mx, const FixedMap& my, float x, float y, float q) {
  uint32_t ix[3], iy[3];
  float wx[3], wy[3];
  fixed_axis(mx, x, ix, wx);
  fixed_axis(my, y, iy, wy);
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) {
      const float t1 = q * wx[c];
      const float t2 = t1 * wy[r];
      g[(size_t)iy[r] * mx.bins + ix[c]] += to_fixed(t2);
    }
}

int32_t orc_scatter_fixed(orc_handle h, const double* coords, int64_t* physical, int64_t* fill,
                          int64_t* overflow_fixed, uint64_t* overflow_bins) {
  Oracle& o = h->o;
  const size_t B = o.bins();
  const FixedMap mapx(o.W, o.Wb, o.identity_map), mapy(o.H, o.Hb, o.identity_map);
  for (uint32_t f = 0; f < o.K; ++f) {
    int64_t* gp = physical + (size_t)f * B;
    int64_t* gf = fill + (size_t)f * B;
    for (size_t i = 0; i < B; ++i) {
      gp[i] = -(int64_t)std::nearbyint(o.smoothed[f][i] * 4294967296.0);
      gf[i] = 0;
    }
    for (const auto& du : o.dunits) {
      const float ox = (float)coords[2 * (size_t)du.unit], oy = (float)coords[2 * (size_t)du.unit + 1];
      for (const auto& m : du.members)
        if (m.field == f) {
          const float px = ox + (float)m.dx, py = oy + (float)m.dy;
          deposit_fixed(gp, mapx, mapy, px, py, (float)m.charge);
        }
    }
    for (size_t i = 0; i < o.fillers.size(); ++i) {
      if (o.fillers[i].field != f) continue;
      const size_t c = 2 * ((size_t)o.U + i);
      deposit_fixed(gf, mapx, mapy, (float)coords[c], (float)coords[c + 1], (float)o.fillers[i].charge);
    }
    int64_t ov = 0;
    uint64_t cnt = 0;
    for (size_t i = 0; i < B; ++i)
      if (gp[i] > 0) {
        ov += gp[i];
        cnt++;
      }
    if (overflow_fixed) overflow_fixed[f] = ov;
    if (overflow_bins) overflow_bins[f] = cnt;
  }
  return TEXO_GP_OK;
}

int32_t orc_place(orc_handle h, int32_t threads, uint32_t max_iterations, uint32_t* targets, double* coordinates,
                  orc_run_stats* stats) {
  Oracle& o = h->o;
  orc_run_stats local{};
  if (!stats) stats = &local;
  if (o.dunits.empty()) {
    // rounded_unit_targets (eplace.rs:1015-1020) of the unclamped initial vector.
    for (uint32_t u = 0; u < o.U; ++u) {
      if (targets) {
        targets[2 * (size_t)u] = Eplace::rounded(o.init_coords[2 * (size_t)u], o.W);
        targets[2 * (size_t)u + 1] = Eplace::rounded(o.init_coords[2 * (size_t)u + 1], o.H);
      }
    }
    if (coordinates) std::memcpy(coordinates, o.init_coords.data(), o.coord_count() * 8);
    *stats = orc_run_stats{};
    stats->converged = 1;
    return TEXO_GP_OK;
  }
  Eplace ep(o, threads);
  h->trace.clear();
  ep.trace = &h->trace;
  std::vector<uint32_t> best;
  std::vector<double> fc;
  int32_t s = ep.run(max_iterations, best, fc, *stats);
  if (targets && !best.empty()) std::memcpy(targets, best.data(), best.size() * 4);
  if (coordinates && !fc.empty()) std::memcpy(coordinates, fc.data(), fc.size() * 8);
  return s;
}

int32_t orc_set_charges(orc_handle h, const double* member_charge, const double* filler_charge) {
  Oracle& o = h->o;
  if (member_charge) {
    size_t k = 0;
    for (auto& u : o.dunits)
      for (auto& m : u.members) m.charge = member_charge[k++];
  }
  if (filler_charge)
    for (size_t i = 0; i < o.fillers.size(); ++i) o.fillers[i].charge = filler_charge[i];
  return TEXO_GP_OK;
}

int32_t orc_place_round(orc_handle h, int32_t threads, const orc_round* round, const double* coordinates_in,
                        uint32_t* targets, double* coordinates, orc_run_stats* stats, orc_round_result* result) {
  Oracle& o = h->o;
  orc_run_stats local{};
  if (!stats) stats = &local;
  Eplace ep(o, threads);
  h->trace.clear();
  ep.trace = &h->trace;
  ep.stop_mode = round ? round->stop : 0;
  ep.reset = round && round->reset_multipliers;
  ep.fixed_scales = round ? round->density_scales : nullptr;
  ep.offset = round ? round->completed_iterations : 0;
  ep.start = coordinates_in;
  std::vector<uint32_t> best;
  std::vector<double> fc;
  const int32_t s = ep.run(0, best, fc, *stats);
  if (targets && !best.empty()) std::memcpy(targets, best.data(), best.size() * 4);
  if (coordinates && !fc.empty()) std::memcpy(coordinates, fc.data(), fc.size() * 8);
  if (result) {
    *result = orc_round_result{};
    result->completed_iterations = stats->iterations;
    result->exhausted = stats->exhausted;
    for (size_t f = 0; f < ep.scales_used.size() && f < TEXO_GP_MAX_FIELDS; ++f)
      result->density_scales[f] = ep.scales_used[f];
  }
  return s;
}

uint32_t orc_trace(orc_handle h, texo_gp_iteration* out, uint32_t capacity) {
  const uint32_t n = (uint32_t)std::min<size_t>(h->trace.size(), capacity);
  if (n) std::memcpy(out, h->trace.data(), n * sizeof(texo_gp_iteration));
  return (uint32_t)h->trace.size();
}

int32_t orc_hpwl(orc_handle h, const double* coordinates, double* out) {
  *out = h->o.hpwl(coordinates);
  return TEXO_GP_OK;
}
void orc_wirelength_preconditioner(orc_handle h, double* out) {
  std::memcpy(out, h->o.wl_precond.data(), h->o.wl_precond.size() * 8);
}
void orc_cell_incidence_weights(orc_handle h, double* out) {
  auto w = h->o.cell_incidence();
  std::memcpy(out, w.data(), w.size() * 8);
}

void orc_nesterov_init(orc_nesterov_state* s, const double* initial, const double* lower, uint64_t lower_len,
                       const double* upper, uint64_t upper_len) {
  const size_t n = s->n;
  bool projectable = lower_len == n && upper_len == n;
  for (size_t i = 0; projectable && i < n; ++i)
    projectable = std::isfinite(initial[i]) && std::isfinite(lower[i]) && std::isfinite(upper[i]) && lower[i] <= upper[i];
  for (size_t i = 0; i < n; ++i) {
    const double v = projectable ? rclamp(initial[i], lower[i], upper[i]) : initial[i];
    s->coordinates[i] = v;
    s->previous[i] = v;
  }
  s->momentum = 1.0;
  s->has_lipschitz = 0;
  s->lipschitz = 0.0;
}

int32_t orc_nesterov_step(orc_nesterov_state* state, const double* lower, uint64_t lower_len, const double* upper,
                          uint64_t upper_len, const double* metric, uint64_t metric_len, orc_eval_cb cb, void* user,
                          orc_step_out* out) {
  NState st;
  st.x.assign(state->coordinates, state->coordinates + state->n);
  st.prev.assign(state->previous, state->previous + state->n);
  st.a = state->momentum;
  st.has_L = state->has_lipschitz != 0;
  st.L = state->lipschitz;
  Bounds b{lower, (size_t)lower_len, upper, (size_t)upper_len};
  Evaluator ev = [&](const std::vector<double>& c, double& value, std::vector<double>& g, int64_t& pl) -> int32_t {
    std::vector<double> buf(c.size() + 64, 0.0);
    uint64_t glen = c.size();
    int32_t r = cb(user, c.data(), c.size(), &value, buf.data(), &glen, &pl);
    if (r) return r;
    g.assign(buf.begin(), buf.begin() + (ptrdiff_t)std::min<uint64_t>(glen, buf.size()));
    if (glen > buf.size()) g.resize(glen, 0.0);
    return 0;
  };
  StepOut so;
  int32_t s = dynamic_nesterov_step(st, b, metric, (size_t)metric_len, ev, so);
  if (out) {
    out->stationary = so.stationary ? 1 : 0;
    out->objective = so.objective;
    out->stationarity = so.stationarity;
    out->coordinate_change = so.coordinate_change;
    out->trials = so.trials;
    out->payload = so.payload;
    out->inner = so.inner;
    out->error_index = so.error_index;
    out->expected = so.expected;
    out->actual = so.actual;
  }
  if (s == TEXO_GP_OK) {
    std::memcpy(state->coordinates, st.x.data(), st.x.size() * 8);
    std::memcpy(state->previous, st.prev.data(), st.prev.size() * 8);
    state->momentum = st.a;
    state->has_lipschitz = st.has_L ? 1 : 0;
    state->lipschitz = st.L;
  }
  return s;
}

double orc_box_metric_kkt(const double* g, const double* x, const double* lo, const double* hi, const double* m,
                          uint64_t n) {
  return kkt_residual(g, x, lo, hi, m, (size_t)n);
}

void orc_augmented(double energy, double e0, double lambda, double beta, double* value, double* coef) {
  augmented(energy, e0, lambda, beta, *value, *coef);
}
int32_t orc_multiplier_growth(double lg, double lo, double hi, double* g) { return growth_from_log(lg, lo, hi, *g); }
int32_t orc_area_adjusted_multiplier_step(const double* m, uint64_t n, double high, double* step) {
  double s = -0.0;
  for (uint64_t i = 0; i < n; ++i) s += m[i] * m[i];
  *step = (high - 1.0) * std::sqrt(s);
  return (std::isfinite(*step) && *step > 0.0) ? TEXO_GP_OK : TEXO_GP_ERR_INVALID_NORMALIZATION;
}
int32_t orc_field_gamma(double overflow, double target, double base, double* g) {
  return field_gamma(overflow, target, base, *g);
}
int32_t orc_weighted_gamma_mean(const double* g, const double* w, uint64_t n, double fallback, double* mean) {
  return weighted_gamma_mean(g, w, (size_t)n, fallback, *mean);
}
double orc_overflow_target(uint32_t kind) { return overflow_target(kind); }
int32_t orc_area_adjustment_ready(uint32_t K, const uint32_t* kinds, const double* overflow) {
  return area_adjustment_ready(K, kinds, overflow) ? 1 : 0;
}
int32_t orc_area_adjusted_multipliers(uint32_t K, const double* energy, const double* force_l1,
                                      const double* initial_energies, double beta, const double* wa_gradient_xy,
                                      uint64_t units, double* out) {
  // |grad W|_1 in the reference's order: x then y of each unit
  double wl = 0.0;
  for (uint64_t u = 0; u < units; ++u) {
    wl += std::fabs(wa_gradient_xy[2 * u]);
    wl += std::fabs(wa_gradient_xy[2 * u + 1]);
  }
  std::vector<double> lambda;
  const int32_t s = area_adjusted_multipliers(K, energy, force_l1, initial_energies, beta, wl, lambda);
  if (s) return s;
  for (uint32_t f = 0; f < K; ++f) out[f] = lambda[f];
  return TEXO_GP_OK;
}
int32_t orc_checkpoint_better(double mx, double tot, double bmx, double btot) {
  int c = total_cmp(mx, bmx);
  return (c < 0 || (c == 0 && total_cmp(tot, btot) < 0)) ? 1 : 0;
}
int32_t orc_validate_units(const uint32_t* member_ptr, uint64_t units, uint64_t* err) {
  for (uint64_t u = 0; u < units; ++u)
    if (member_ptr[u + 1] == member_ptr[u]) {
      if (err) *err = u;
      return TEXO_GP_ERR_EMPTY_UNIT;
    }
  return TEXO_GP_OK;
}

// ---- continuous RUDY demand (crates/texo-pnr/src/eplace.rs:856-937) -------
int32_t orc_routing_demand(uint32_t width, uint32_t height, uint64_t num_boxes, const double* boxes,
                           double* horizontal, double* vertical) {
  const size_t tiles = (size_t)width * height;
  for (size_t t = 0; t < tiles; ++t) horizontal[t] = vertical[t] = 0.0;
  std::vector<std::pair<uint32_t, double>> xo, yo;
  for (uint64_t i = 0; i < num_boxes; ++i) {
    const double minx = boxes[4 * i], maxx = boxes[4 * i + 1], miny = boxes[4 * i + 2], maxy = boxes[4 * i + 3];
    if (!(std::isfinite(minx) && std::isfinite(maxx) && std::isfinite(miny) && std::isfinite(maxy)) || minx > maxx ||
        miny > maxy)
      return 1;
    const double dx = maxx - minx, dy = maxy - miny;
    const double rminx = minx - 0.5, rmaxx = maxx + 0.5, rminy = miny - 0.5, rmaxy = maxy + 0.5;
    const double area = (dx + 1.0) * (dy + 1.0);
    if (!std::isfinite(area) || area <= 0.0) return 1;
    const double hd = dx / area, vd = dy / area;
    yo.clear();
    for (uint32_t y = 0; y < height; ++y) {
      const double o = std::max(std::min((double)y + 0.5, rmaxy) - std::max((double)y - 0.5, rminy), 0.0);
      if (o > 0.0) yo.emplace_back(y, o);
    }
    xo.clear();
    for (uint32_t x = 0; x < width; ++x) {
      const double o = std::max(std::min((double)x + 0.5, rmaxx) - std::max((double)x - 0.5, rminx), 0.0);
      if (o > 0.0) xo.emplace_back(x, o);
    }
    for (const auto& [y, oy] : yo)
      for (const auto& [x, ox] : xo) {
        const double overlap = ox * oy;
        const size_t index = (size_t)y * width + x;
        horizontal[index] += hd * overlap;
        vertical[index] += vd * overlap;
      }
  }
  for (size_t t = 0; t < tiles; ++t)
    if (!(std::isfinite(horizontal[t]) && horizontal[t] >= 0.0 && std::isfinite(vertical[t]) && vertical[t] >= 0.0))
      return 1;
  return 0;
}

// ---- coarse quadratic seed (crates/texo-pnr/src/lib.rs:4586-4790) --------
// multiply_quadratic (lib.rs:4767-4782): diagonal * v[i], then minus
// weight * v[j] per adjacency entry, in order.
void orc_multiply_quadratic(uint64_t n, const double* diagonal, const uint32_t* ptr, const uint32_t* index,
                            const double* weight, const double* values, double* product) {
  for (uint64_t i = 0; i < n; ++i) {
    double s = diagonal[i] * values[i];
    for (uint32_t k = ptr[i]; k < ptr[i + 1]; ++k) s = s - weight[k] * values[index[k]];
    product[i] = s;
  }
}
static double pcg_dot(const std::vector<double>& a, const std::vector<double>& b) {   // lib.rs:4784-4789
  double s = 0.0;
  for (size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
  return s;
}
// apply_jacobi_preconditioner (lib.rs:4754-4765)
static double pcg_jacobi(const std::vector<double>& r, const double* diagonal, std::vector<double>& z) {
  for (size_t i = 0; i < r.size(); ++i) z[i] = r[i] / diagonal[i];
  return pcg_dot(r, z);
}
// solve_quadratic + finish_quadratic_solve (lib.rs:4586-4752)
int32_t orc_solve_quadratic(uint64_t n, const double* diagonal, const uint32_t* ptr, const uint32_t* index,
                            const double* weight, const double* rhs, double* solution, orc_pcg_stats* st) {
  const double kTol = 1e-8;
  std::vector<double> x(solution, solution + n), product(n, 0.0), residual(n), pre(n, 0.0);
  orc_multiply_quadratic(n, diagonal, ptr, index, weight, x.data(), product.data());
  for (uint64_t i = 0; i < n; ++i) residual[i] = rhs[i] - product[i];
  double rr = pcg_dot(residual, residual);
  const double initial = rr;
  const double target = std::max(initial, std::numeric_limits<double>::epsilon()) * kTol;
  double rho = pcg_jacobi(residual, diagonal, pre);
  std::vector<double> direction = pre;
  uint64_t iterations = 0, restarts = 0;
  bool breakdown = false;
  for (uint64_t loop = 0; loop < n; ++loop) {
    if (rr <= target) break;
    orc_multiply_quadratic(n, diagonal, ptr, index, weight, direction.data(), product.data());
    const double den = pcg_dot(direction, product);
    if (!std::isfinite(den) || den <= 0.0 || !std::isfinite(rho) || rho <= 0.0) {
      breakdown = true;
      break;
    }
    const double alpha = rho / den;
    if (!std::isfinite(alpha)) {
      breakdown = true;
      break;
    }
    for (uint64_t i = 0; i < n; ++i) {
      x[i] += alpha * direction[i];
      residual[i] -= alpha * product[i];
    }
    ++iterations;
    rr = pcg_dot(residual, residual);
    if (rr <= target) {
      orc_multiply_quadratic(n, diagonal, ptr, index, weight, x.data(), product.data());
      for (uint64_t i = 0; i < n; ++i) residual[i] = rhs[i] - product[i];
      rr = pcg_dot(residual, residual);
      if (rr <= target) break;
      ++restarts;
      rho = pcg_jacobi(residual, diagonal, pre);
      if (!std::isfinite(rho) || rho <= 0.0) {
        breakdown = true;
        break;
      }
      direction = pre;
      continue;
    }
    const double next = pcg_jacobi(residual, diagonal, pre);
    if (!std::isfinite(next) || next <= 0.0) {
      breakdown = true;
      break;
    }
    const double beta = next / rho;
    for (uint64_t i = 0; i < n; ++i) direction[i] = pre[i] + beta * direction[i];
    rho = next;
  }
  orc_multiply_quadratic(n, diagonal, ptr, index, weight, x.data(), product.data());
  double fin = 0.0;
  for (uint64_t i = 0; i < n; ++i) {
    const double r = rhs[i] - product[i];
    fin += r * r;
  }
  const bool converged = fin <= target;
  for (uint64_t i = 0; i < n; ++i) solution[i] = x[i];
  if (st) {
    st->iterations = iterations;
    st->restarts = restarts;
    st->converged = converged ? 1 : 0;
    st->stop = converged ? 0 : (breakdown ? 1 : 2);
    st->initial_residual_squared = initial;
    st->target_squared = target;
    st->final_residual_squared = fin;
  }
  return converged ? 0 : 1;
}

}  // extern "C"
