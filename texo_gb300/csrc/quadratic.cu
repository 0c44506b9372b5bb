// quadratic.cu — the coarse quadratic seed's linear solve on the GPU:
// Jacobi-preconditioned conjugate gradients for (D - W) x = b
// (`solve_quadratic`, crates/texo-pnr/src/lib.rs:4586-4752), FP64.
//
// One cooperative persistent kernel runs the whole solve. Each block owns
// rows strided over the grid; the products of a row (`multiply_quadratic`,
// lib.rs:4767-4782: diagonal * v[i], then minus weight * v[j] in adjacency
// order) and the vector updates use the reference's operations in its order
// without contraction into FMAs, so a row's value is the reference's bit for
// bit given the same inputs. The dot products fold per-block partials in a
// fixed order (one warp per reduction), so the solve is deterministic, but
// their rounding differs from the reference's left-to-right sums: the
// iterates agree to rounding, not bit for bit.
//
// A CG step takes three grid barriers: the product q = A p with the partial
// <p, q>; the updates of x and r with <r, r>, z = r / D and <r, z>; the new
// direction p = z + beta p. Partials alternate between two sets so a block
// that leaves a barrier early never overwrites a set another block still
// reads. Every wait is the bounded grid barrier of the placement engine.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>

#include "engine.h"
#include "persistent_body.cuh"

namespace tgp {
namespace {

enum PcgSlot { PS_A = 0, PS_B, kPcgSlots };   // two dot products a phase at most
constexpr int kMaxPcgBlocks = 2048;
constexpr double kPcgTolerance = 1e-8;      // on squared residuals: 1e-4 on the norm (lib.rs:4592-4594)

struct PcgResult {
  unsigned iterations, restarts;
  int stop;             // 0 residual, 1 breakdown, 2 dimension
  int converged;
  double initial_rr, target, final_rr;
};

struct PcgDev {
  int n;
  const double *diag, *w, *b;
  const unsigned *ptr, *idx;
  double *x, *r, *z, *p, *q;
  double* part;          // [2 sets][kPcgSlots][kMaxPcgBlocks]
  GridBarrier* bar;
  PcgResult* out;
};

__device__ __forceinline__ double row_product(const PcgDev& d, const double* v, int i) {
  double s = __dmul_rn(d.diag[i], v[i]);
  for (unsigned k = d.ptr[i]; k < d.ptr[i + 1]; ++k) s = __dsub_rn(s, __dmul_rn(d.w[k], v[d.idx[k]]));
  return s;
}

__global__ void __launch_bounds__(kThreads, 2) k_pcg(PcgDev d) {
  __shared__ double sh[kThreads + 4];
  __shared__ FoldValue fv[kPcgSlots];
  __shared__ unsigned gen;
  __shared__ int failed;
  // controller state, identical in every block (thread 0 writes it)
  __shared__ double rr, rho, alpha, beta, target;
  __shared__ unsigned iterations, restarts;
  __shared__ int stop, action;
  const int pb = blockIdx.x, np = gridDim.x, n = d.n;
  const int stride = np * blockDim.x;
  unsigned long long nbar = 0;
  unsigned phase = 0;
  if (threadIdx.x == 0) {
    gen = 0;   // the barrier is cleared before the launch
    iterations = restarts = 0;
    stop = 2;
  }
  __syncthreads();
  auto slot = [&](int s) { return d.part + ((size_t)(phase & 1u) * kPcgSlots + s) * kMaxPcgBlocks; };
  auto put = [&](int s, double v) {
    const double t = block_fold_fp64(v, sh, FoldAdd());
    if (threadIdx.x == 0) slot(s)[pb] = t;
  };
  // barrier, then fold the slots of the phase that just ended
  auto sync_fold = [&](int nslots) -> bool {
    if (!grid_sync(d.bar, (unsigned)np, &gen, &nbar, nullptr, &failed)) return false;
    const int w = threadIdx.x >> 5;
    if (w < nslots) {
      const double* a = slot(w);
      const double v = warp_fold(a, np, 0.0, OpAdd());
      if ((threadIdx.x & 31) == 0) fv[w].d = v;
    }
    __syncthreads();
    ++phase;
    return true;
  };
  auto sync_only = [&]() -> bool {
    if (!grid_sync(d.bar, (unsigned)np, &gen, &nbar, nullptr, &failed)) return false;
    ++phase;
    return true;
  };

  // r = b - A x, z = r / D, p = z; |r|^2 and <r, z>
  {
    double a = 0.0, c = 0.0;
    for (int i = pb * blockDim.x + threadIdx.x; i < n; i += stride) {
      const double ri = __dsub_rn(d.b[i], row_product(d, d.x, i));
      const double zi = __ddiv_rn(ri, d.diag[i]);
      d.r[i] = ri;
      d.z[i] = zi;
      d.p[i] = zi;
      a = __dadd_rn(a, __dmul_rn(ri, ri));
      c = __dadd_rn(c, __dmul_rn(ri, zi));
    }
    put(PS_A, a);
    put(PS_B, c);
  }
  if (!sync_fold(2)) return;
  if (threadIdx.x == 0) {
    rr = fv[PS_A].d;
    if (pb == 0) d.out->initial_rr = rr;
    target = fmax(rr, 2.220446049250313e-16) * kPcgTolerance;
    rho = fv[PS_B].d;
  }
  __syncthreads();

  for (int loop = 0; loop < n; ++loop) {
    if (rr <= target) break;
    // q = A p and <p, q>
    {
      double a = 0.0;
      for (int i = pb * blockDim.x + threadIdx.x; i < n; i += stride) {
        const double qi = row_product(d, d.p, i);
        d.q[i] = qi;
        a = __dadd_rn(a, __dmul_rn(d.p[i], qi));
      }
      put(PS_A, a);
    }
    if (!sync_fold(1)) return;
    if (threadIdx.x == 0) {
      const double den = fv[PS_A].d;
      action = 0;
      if (!isfinite(den) || den <= 0.0 || !isfinite(rho) || rho <= 0.0) {
        action = 1;
      } else {
        alpha = __ddiv_rn(rho, den);
        if (!isfinite(alpha)) action = 1;
      }
      if (action) stop = 1;
    }
    __syncthreads();
    if (action) break;
    // x += alpha p, r -= alpha q; |r|^2, z = r / D, <r, z>
    {
      double a = 0.0, c = 0.0;
      for (int i = pb * blockDim.x + threadIdx.x; i < n; i += stride) {
        d.x[i] = __dadd_rn(d.x[i], __dmul_rn(alpha, d.p[i]));
        const double ri = __dsub_rn(d.r[i], __dmul_rn(alpha, d.q[i]));
        const double zi = __ddiv_rn(ri, d.diag[i]);
        d.r[i] = ri;
        d.z[i] = zi;
        a = __dadd_rn(a, __dmul_rn(ri, ri));
        c = __dadd_rn(c, __dmul_rn(ri, zi));
      }
      put(PS_A, a);
      put(PS_B, c);
    }
    if (!sync_fold(2)) return;
    if (threadIdx.x == 0) {
      iterations++;
      rr = fv[PS_A].d;
      action = rr <= target ? 2 : 0;
      if (!action) {
        const double next = fv[PS_B].d;
        if (!isfinite(next) || next <= 0.0) {
          stop = 1;
          action = 1;
        } else {
          beta = __ddiv_rn(next, rho);
          rho = next;
        }
      }
    }
    __syncthreads();
    if (action == 1) break;
    if (action == 2) {
      // the recursive residual says converged: recompute the true one
      // (lib.rs:4656-4677) and restart from it when it is not small enough
      {
        double a = 0.0, c = 0.0;
        for (int i = pb * blockDim.x + threadIdx.x; i < n; i += stride) {
          const double ri = __dsub_rn(d.b[i], row_product(d, d.x, i));
          const double zi = __ddiv_rn(ri, d.diag[i]);
          d.r[i] = ri;
          d.z[i] = zi;
          d.p[i] = zi;   // the restart direction, used only if the check fails
          a = __dadd_rn(a, __dmul_rn(ri, ri));
          c = __dadd_rn(c, __dmul_rn(ri, zi));
        }
        put(PS_A, a);
        put(PS_B, c);
      }
      if (!sync_fold(2)) return;
      if (threadIdx.x == 0) {
        rr = fv[PS_A].d;
        action = 0;
        if (rr > target) {
          const double next = fv[PS_B].d;
          restarts++;
          if (!isfinite(next) || next <= 0.0) {
            stop = 1;
            action = 1;
          } else {
            rho = next;
          }
        }
      }
      __syncthreads();
      if (action == 1) break;
      continue;   // p = z is already in place (or the loop test ends the solve)
    }
    // p = z + beta p
    for (int i = pb * blockDim.x + threadIdx.x; i < n; i += stride)
      d.p[i] = __dadd_rn(d.z[i], __dmul_rn(beta, d.p[i]));
    if (!sync_only()) return;
  }

  // the true final residual (finish_quadratic_solve, lib.rs:4702-4752)
  {
    double a = 0.0;
    for (int i = pb * blockDim.x + threadIdx.x; i < n; i += stride) {
      const double ri = __dsub_rn(d.b[i], row_product(d, d.x, i));
      a = __dadd_rn(a, __dmul_rn(ri, ri));
    }
    put(PS_A, a);
  }
  if (!sync_fold(1)) return;
  if (pb == 0 && threadIdx.x == 0) {
    PcgResult& o = *d.out;
    o.final_rr = fv[PS_A].d;
    o.target = target;
    o.iterations = iterations;
    o.restarts = restarts;
    o.converged = o.final_rr <= target ? 1 : 0;
    o.stop = o.converged ? 0 : stop;
  }
}

}  // namespace
}  // namespace tgp

using namespace tgp;

extern "C" int32_t texo_gp_quadratic_solve(int32_t device, uint32_t n, const double* diagonal,
                                           const uint32_t* adjacency_ptr, const uint32_t* adjacency_index,
                                           const double* adjacency_weight, const double* rhs, double* solution,
                                           texo_gp_pcg_stats* stats) {
  if (stats) std::memset(stats, 0, sizeof(*stats));
  auto fail = [&](int32_t s, const std::string& why) {
    if (!why.empty()) set_last_error(why);
    if (stats) stats->status = s;
    return s;
  };
  if (!diagonal || !adjacency_ptr || !rhs || !solution) return fail(TEXO_GP_ERR_INVALID_ARGUMENT, "null argument");
  if (n == 0) return fail(TEXO_GP_OK, "");
  if (n > (1u << 30)) return fail(TEXO_GP_ERR_INVALID_ARGUMENT, "system too large");
  const uint64_t nnz = adjacency_ptr[n];
  if (adjacency_ptr[0] != 0 || (nnz && (!adjacency_index || !adjacency_weight)))
    return fail(TEXO_GP_ERR_INVALID_ARGUMENT, "adjacency_ptr must start at 0");
  for (uint32_t i = 0; i < n; ++i) {
    if (adjacency_ptr[i + 1] < adjacency_ptr[i]) return fail(TEXO_GP_ERR_INVALID_ARGUMENT, "adjacency_ptr decreases");
    if (!(std::isfinite(diagonal[i]) && diagonal[i] > 0.0))
      return fail(TEXO_GP_ERR_INVALID_ARGUMENT, "diagonal entries must be finite and positive");
    if (!std::isfinite(rhs[i]) || !std::isfinite(solution[i]))
      return fail(TEXO_GP_ERR_INVALID_ARGUMENT, "non-finite right-hand side or initial solution");
  }
  for (uint64_t k = 0; k < nnz; ++k)
    if (adjacency_index[k] >= n || !std::isfinite(adjacency_weight[k]))
      return fail(TEXO_GP_ERR_INVALID_ARGUMENT, "adjacency index out of range or non-finite weight");

  if (cudaSetDevice(device) != cudaSuccess) return fail(TEXO_GP_ERR_CUDA, "cudaSetDevice failed");
  static const int per_sm = [] {   // thread-safe one-time initialisation
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_pcg, kThreads, 0) != cudaSuccess) b = 0;
    return b;
  }();
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (per_sm <= 0 || sms <= 0) return fail(TEXO_GP_ERR_CUDA, "k_pcg cannot be resident");
  const int blocks = (int)std::min<uint64_t>(std::min<uint64_t>((uint64_t)std::min(per_sm, 2) * sms, kMaxPcgBlocks),
                                             std::max<uint64_t>(1, (n + kThreads - 1) / kThreads));

  // one allocation: vectors, matrix, partials, barrier, result
  auto round = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t vec = round((size_t)n * 8), nz8 = round(std::max<uint64_t>(nnz, 1) * 8),
               nz4 = round(std::max<uint64_t>(nnz, 1) * 4), p4 = round(((size_t)n + 1) * 4);
  const size_t part = round((size_t)2 * kPcgSlots * kMaxPcgBlocks * 8);
  const size_t total = 8 * vec + nz8 + nz4 + p4 + part + round(sizeof(GridBarrier)) + round(sizeof(PcgResult));
  cudaStream_t s = nullptr;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return fail(TEXO_GP_ERR_CUDA, "stream");
  char* base = nullptr;
  if (cudaMallocAsync((void**)&base, total, s) != cudaSuccess) {
    cudaStreamDestroy(s);
    return fail(TEXO_GP_ERR_OUT_OF_MEMORY, "cudaMallocAsync failed");
  }
  char* at = base;
  auto take = [&](size_t b) {
    char* r = at;
    at += b;
    return r;
  };
  PcgDev d{};
  d.n = (int)n;
  double* diag = (double*)take(vec);
  double* b = (double*)take(vec);
  d.x = (double*)take(vec);
  d.r = (double*)take(vec);
  d.z = (double*)take(vec);
  d.p = (double*)take(vec);
  d.q = (double*)take(vec);
  take(vec);   // spare (keeps the layout 256-byte aligned for any n)
  double* w = (double*)take(nz8);
  unsigned* idx = (unsigned*)take(nz4);
  unsigned* ptr = (unsigned*)take(p4);
  d.part = (double*)take(part);
  d.bar = (GridBarrier*)take(round(sizeof(GridBarrier)));
  d.out = (PcgResult*)take(round(sizeof(PcgResult)));
  d.diag = diag;
  d.b = b;
  d.w = w;
  d.idx = idx;
  d.ptr = ptr;

  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int32_t st = TEXO_GP_OK;
  PcgResult res{};
  cudaEventRecord(e0, s);
  bool ok = cudaMemcpyAsync(diag, diagonal, (size_t)n * 8, cudaMemcpyHostToDevice, s) == cudaSuccess &&
            cudaMemcpyAsync(b, rhs, (size_t)n * 8, cudaMemcpyHostToDevice, s) == cudaSuccess &&
            cudaMemcpyAsync(d.x, solution, (size_t)n * 8, cudaMemcpyHostToDevice, s) == cudaSuccess &&
            cudaMemcpyAsync(ptr, adjacency_ptr, ((size_t)n + 1) * 4, cudaMemcpyHostToDevice, s) == cudaSuccess &&
            (!nnz || (cudaMemcpyAsync(idx, adjacency_index, nnz * 4, cudaMemcpyHostToDevice, s) == cudaSuccess &&
                      cudaMemcpyAsync(w, adjacency_weight, nnz * 8, cudaMemcpyHostToDevice, s) == cudaSuccess)) &&
            cudaMemsetAsync(d.bar, 0, sizeof(GridBarrier), s) == cudaSuccess &&
            cudaMemsetAsync(d.out, 0, sizeof(PcgResult), s) == cudaSuccess;
  if (ok) {
    void* args[] = {&d};
    ok = cudaLaunchCooperativeKernel((const void*)k_pcg, dim3(blocks), dim3(kThreads), args, 0, s) == cudaSuccess;
    if (ok) note_launch();
  }
  GridBarrier hb{};
  ok = ok && cudaMemcpyAsync(solution, d.x, (size_t)n * 8, cudaMemcpyDeviceToHost, s) == cudaSuccess &&
       cudaMemcpyAsync(&res, d.out, sizeof(PcgResult), cudaMemcpyDeviceToHost, s) == cudaSuccess &&
       cudaMemcpyAsync(&hb, d.bar, sizeof(GridBarrier), cudaMemcpyDeviceToHost, s) == cudaSuccess;
  cudaEventRecord(e1, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) ok = false;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFreeAsync(base, s);
  cudaStreamSynchronize(s);
  cudaStreamDestroy(s);
  if (!ok) {
    st = TEXO_GP_ERR_CUDA;
    set_last_error(std::string("quadratic solve: ") + cudaGetErrorString(cudaGetLastError()));
  } else if (hb.error) {
    st = TEXO_GP_ERR_DEVICE_TIMEOUT;
    set_last_error("quadratic solve: a grid barrier wait ran out");
  } else if (!res.converged) {
    st = TEXO_GP_ERR_PCG_NOT_CONVERGED;
    set_last_error(std::string("analytical PCG ") + (res.stop == 1 ? "breakdown" : "dimension") + " after " +
                   std::to_string(res.iterations) + "/" + std::to_string(n) + " iterations");
  }
  if (stats) {
    stats->status = st;
    stats->iterations = res.iterations;
    stats->restarts = res.restarts;
    stats->stop = res.stop;
    stats->initial_residual_squared = res.initial_rr;
    stats->target_squared = res.target;
    stats->final_residual_squared = res.final_rr;
    stats->elapsed_ms = ms;
    stats->kernel_launches = 1;
  }
  return st;
}
