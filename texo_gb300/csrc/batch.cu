// batch.cu — many resident placements advanced by one persistent launch.
//
// Each admitted job is a device-engine handle with its own buffers, its own
// controller state and its own barrier. `advance` gives every resident job a
// share of the GPU's co-resident blocks (by its estimated work per iteration,
// up to its virtual block count) and runs all of them in one cooperative
// launch of k_batch; jobs run
// independently inside it, each over its own physical blocks. A job's results
// do not depend on how many physical blocks it got, so they are bit-identical
// to the same job placed alone. When the resident set repeats from one advance
// to the next, the whole advance (state copies in, launches, state copies
// out) is captured once as a CUDA graph and replayed.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <vector>

#include "engine.h"

namespace {
using namespace tgp;

// A job's weight in the share of physical blocks: its estimated work per
// iteration.
inline double share_weight(uint64_t work) { return (double)work; }

struct Job {
  uint64_t id = 0;
  texo_gp_handle h = nullptr;
  uint64_t bytes = 0;
  int V = 1;
  uint64_t W = 1;   // estimated work per iteration
};

}  // namespace

struct texo_gp_batch_s {
  texo_gp_params params{};
  uint64_t budget = 0;
  uint32_t max_slots = 0;
  std::vector<Job> resident;
  std::deque<Job> done;
  uint64_t used = 0;
  cudaStream_t stream = nullptr;
  InstDesc* d_descs = nullptr;
  int4* d_map = nullptr;
  std::vector<InstDesc> h_descs;
  std::vector<int4> h_map;
  int pblocks = 0;
  size_t rr = 0;
  std::mutex mu;
  // The advance of an unchanged resident set as one CUDA graph: the state
  // copies in, the batch launches, the state copies out. Recaptured when the
  // set, its order or the iteration chunk changes.
  int4* d_map1 = nullptr;                 // the second launch family's block map
  cudaGraphExec_t exec = nullptr;
  std::vector<texo_gp_handle> g_jobs;     // with their state mirrors and device copies: a
  std::vector<RunBlock*> g_hosts, g_devs; // handle at a reused address is still a new key
  uint32_t g_iters = 0;
  int g_launches = 0;
  uint64_t captures = 0, replays = 0;
  std::vector<texo_gp_handle> p_jobs;     // the set of the previous advance (captured once it repeats)
  std::vector<RunBlock*> p_hosts;
  uint32_t p_iters = 0;

  ~texo_gp_batch_s() {
    if (stream) cudaStreamSynchronize(stream);
    if (exec) cudaGraphExecDestroy(exec);
    if (d_map1) cudaFree(d_map1);
    for (auto& j : resident) texo_gp_destroy(j.h);
    for (auto& j : done) texo_gp_destroy(j.h);
    if (d_descs) cudaFree(d_descs);
    if (d_map) cudaFree(d_map);
    if (stream) cudaStreamDestroy(stream);
  }
};

#define BCU(call)                                                                 \
  do {                                                                            \
    cudaError_t e_ = (call);                                                      \
    if (e_ != cudaSuccess) {                                                      \
      set_last_error(std::string(#call) + ": " + cudaGetErrorString(e_));         \
      return TEXO_GP_ERR_CUDA;                                                    \
    }                                                                             \
  } while (0)

extern "C" {

int32_t texo_gp_batch_create(const texo_gp_params* params, uint64_t hbm_budget_bytes, uint32_t max_slots,
                             texo_gp_batch* out) {
  if (!out || max_slots == 0) return TEXO_GP_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  auto b = std::make_unique<texo_gp_batch_s>();
  if (params)
    b->params = *params;
  else
    texo_gp_default_params(&b->params);
  b->params.engine = TEXO_GP_ENGINE_DEVICE;
  b->budget = hbm_budget_bytes;
  b->max_slots = max_slots;
  BCU(cudaSetDevice(b->params.device));
  cudaDeviceProp prop;
  BCU(cudaGetDeviceProperties(&prop, b->params.device));
  const int per_sm = std::min(std::max(batch_blocks_per_sm(), 1), kBatchBlocksPerSm);
  b->pblocks = per_sm * prop.multiProcessorCount;
  BCU(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  BCU(cudaMalloc(&b->d_descs, sizeof(InstDesc) * max_slots));
  BCU(cudaMalloc(&b->d_map, sizeof(int4) * b->pblocks));
  BCU(cudaMalloc(&b->d_map1, sizeof(int4) * b->pblocks));
  b->h_descs.resize(max_slots);
  b->h_map.reserve(b->pblocks);
  *out = b.release();
  return TEXO_GP_OK;
}

int32_t texo_gp_batch_destroy(texo_gp_batch b) {
  if (!b) return TEXO_GP_ERR_INVALID_ARGUMENT;
  delete b;
  return TEXO_GP_OK;
}

int32_t texo_gp_batch_admit(texo_gp_batch b, const texo_gp_problem* problem, const texo_gp_params* params,
                            uint64_t job_id, uint32_t* out_slot) {
  if (!b || !problem) return TEXO_GP_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(b->mu);
  if (b->resident.size() + b->done.size() >= b->max_slots) return TEXO_GP_ERR_BUSY;
  texo_gp_params prm = params ? *params : b->params;
  prm.engine = TEXO_GP_ENGINE_DEVICE;
  prm.device = b->params.device;
  texo_gp_handle h = nullptr;
  const int32_t s = texo_gp_create(problem, &prm, &h);
  if (s) return s;
  const uint64_t bytes = handle_bytes(h);
  if (b->used + bytes > b->budget) {
    texo_gp_destroy(h);
    return TEXO_GP_ERR_BUSY;
  }
  Job j;
  j.id = job_id;
  j.h = h;
  j.bytes = bytes;
  j.V = handle_virtual_blocks(h);
  j.W = std::max<uint64_t>(handle_work(h), 1);
  b->used += bytes;
  b->resident.push_back(j);
  if (out_slot) *out_slot = (uint32_t)(b->resident.size() - 1);
  return TEXO_GP_OK;
}

}  // extern "C"

namespace tgp {
// Adds an uploaded handle as a resident job; the caller has accounted its
// device bytes (the serving loop admits by its own HBM budget).
int32_t batch_add_handle(texo_gp_batch b, texo_gp_handle h, uint64_t job_id) {
  if (!b || !h) return TEXO_GP_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(b->mu);
  if (b->resident.size() + b->done.size() >= b->max_slots) return TEXO_GP_ERR_BUSY;
  Job j;
  j.id = job_id;
  j.h = h;
  j.bytes = handle_bytes(h);
  j.V = handle_virtual_blocks(h);
  j.W = std::max<uint64_t>(handle_work(h), 1);
  b->used += j.bytes;
  b->resident.push_back(j);
  return TEXO_GP_OK;
}
}  // namespace tgp

extern "C" {

int32_t texo_gp_batch_advance(texo_gp_batch b, uint32_t iterations) {
  if (!b) return TEXO_GP_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(b->mu);
  if (b->resident.empty()) return TEXO_GP_OK;
  const int P = b->pblocks;
  // jobs of this launch: all of them when they fit, else a rotating window
  const size_t nres = b->resident.size();
  const size_t n = std::min(nres, (size_t)P);
  std::vector<size_t> pick(n);
  for (size_t i = 0; i < n; ++i) pick[i] = (b->rr + i) % nres;
  b->rr = (b->rr + n) % std::max<size_t>(nres, 1);
  std::vector<char> lg(n, 0);
  // Block maps of the (at most two) launches: one per DCT tile family (a job
  // runs the same kernel instantiation as it does alone). Every job gets one
  // physical block, the rest go by estimated work per iteration, so that the
  // jobs' iterations take about as long as one another, and no job gets more
  // than its virtual blocks (blocks a capped job cannot use go to the others).
  auto block_map = [&](int fam, std::vector<int4>& map) {
    std::vector<size_t> jobs;
    for (size_t i = 0; i < n; ++i)
      if (lg[i] == fam) jobs.push_back(i);
    map.clear();
    if (jobs.empty()) return;
    const int nj = (int)jobs.size();
    std::vector<int> give(nj, 1);
    std::vector<char> full(nj, 0);
    int left = std::max(0, P - nj);
    for (int pass = 0; pass < 8 && left > 0; ++pass) {
      double wsum = 0.0;
      for (int k = 0; k < nj; ++k)
        if (!full[k]) wsum += share_weight(b->resident[pick[jobs[k]]].W);
      if (wsum <= 0.0) break;
      int handed = 0;
      for (int k = 0; k < nj; ++k) {
        if (full[k]) continue;
        const Job& jb = b->resident[pick[jobs[k]]];
        int add = (int)((double)left * share_weight(jb.W) / wsum);
        if (pass > 0 && add == 0 && handed < left) add = 1;   // spread what rounding left over
        add = std::min(add, std::min(jb.V - give[k], left - handed));
        give[k] += add;
        handed += add;
        if (give[k] >= jb.V) full[k] = 1;
      }
      left -= handed;
      if (handed == 0) break;
    }
    for (int k = 0; k < nj; ++k)
      for (int q = 0; q < give[k]; ++q) map.push_back(make_int4((int)jobs[k], q, give[k], 0));
  };
  int32_t s = TEXO_GP_OK;
  bool graphed = false;
  if (n == nres) {
    // Every resident job in this launch: replay (or capture) the advance as a graph.
    std::vector<texo_gp_handle> hs(n);
    std::vector<RunBlock*> hosts(n), devs(n);
    for (size_t i = 0; i < n; ++i) {
      bool large = false;
      hs[i] = b->resident[pick[i]].h;
      batch_stage_host(hs[i], iterations, &b->h_descs[i], &large, &hosts[i], &devs[i]);
      lg[i] = large ? 1 : 0;
    }
    const bool same = b->exec && b->g_jobs == hs && b->g_hosts == hosts && b->g_devs == devs &&
                      b->g_iters == iterations;
    // capture a set only once it repeats (a serving loop that changes the
    // set at every launch boundary would pay a capture per launch)
    const bool repeat = b->p_jobs == hs && b->p_hosts == hosts && b->p_iters == iterations;
    if (!same && !repeat) {
      b->p_jobs = hs;
      b->p_hosts = hosts;
      b->p_iters = iterations;
      if (b->exec) cudaGraphExecDestroy(b->exec);
      b->exec = nullptr;
    } else if (!same) {
      if (b->exec) cudaGraphExecDestroy(b->exec);
      b->exec = nullptr;
      b->g_jobs.clear();
      std::vector<int4> m0, m1;
      block_map(0, m0);
      block_map(1, m1);
      BCU(cudaMemcpyAsync(b->d_descs, b->h_descs.data(), sizeof(InstDesc) * n, cudaMemcpyHostToDevice, b->stream));
      if (!m0.empty())
        BCU(cudaMemcpyAsync(b->d_map, m0.data(), sizeof(int4) * m0.size(), cudaMemcpyHostToDevice, b->stream));
      if (!m1.empty())
        BCU(cudaMemcpyAsync(b->d_map1, m1.data(), sizeof(int4) * m1.size(), cudaMemcpyHostToDevice, b->stream));
      BCU(cudaStreamSynchronize(b->stream));
      if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        bool ok = true;
        for (size_t i = 0; i < n && ok; ++i)
          ok = cudaMemcpyAsync(devs[i], hosts[i], sizeof(RunBlock), cudaMemcpyHostToDevice, b->stream) == cudaSuccess;
        int launches = 0;
        if (ok && !m0.empty()) {
          ok = launch_batch(b->d_descs, b->d_map, (int)m0.size(), false, b->stream) == TEXO_GP_OK;
          ++launches;
        }
        if (ok && !m1.empty()) {
          ok = launch_batch(b->d_descs, b->d_map1, (int)m1.size(), true, b->stream) == TEXO_GP_OK;
          ++launches;
        }
        for (size_t i = 0; i < n && ok; ++i)
          ok = cudaMemcpyAsync(hosts[i], devs[i], sizeof(RunBlock), cudaMemcpyDeviceToHost, b->stream) == cudaSuccess;
        cudaGraph_t g = nullptr;
        const bool ended = cudaStreamEndCapture(b->stream, &g) == cudaSuccess && g != nullptr;
        if (ok && ended && cudaGraphInstantiate(&b->exec, g, 0) == cudaSuccess) {
          b->g_jobs = hs;
          b->g_hosts = hosts;
          b->g_devs = devs;
          b->g_iters = iterations;
          b->g_launches = launches;
          ++b->captures;
        } else {
          b->exec = nullptr;
        }
        if (g) cudaGraphDestroy(g);
      }
      cudaGetLastError();   // a refused capture leaves no sticky error; the plain path runs instead
    }
    if (b->exec) {
      BCU(cudaGraphLaunch(b->exec, b->stream));
      ++b->replays;
      for (int k = 0; k < b->g_launches; ++k) note_launch();
      graphed = true;
    }
  }
  if (!graphed) {
    for (size_t i = 0; i < n; ++i) {
      bool large = false;
      const int32_t st = batch_stage_in(b->resident[pick[i]].h, iterations, b->stream, &b->h_descs[i], &large);
      if (st) return st;
      lg[i] = large ? 1 : 0;
    }
    BCU(cudaMemcpyAsync(b->d_descs, b->h_descs.data(), sizeof(InstDesc) * n, cudaMemcpyHostToDevice, b->stream));
    for (int fam = 0; fam < 2; ++fam) {
      block_map(fam, b->h_map);
      if (b->h_map.empty()) continue;
      int4* dm = fam == 0 ? b->d_map : b->d_map1;
      BCU(cudaMemcpyAsync(dm, b->h_map.data(), sizeof(int4) * b->h_map.size(), cudaMemcpyHostToDevice, b->stream));
      s = launch_batch(b->d_descs, dm, (int)b->h_map.size(), fam == 1, b->stream);
      if (s) {
        set_last_error(std::string("batch launch: ") + cudaGetErrorString(cudaGetLastError()));
        return s;
      }
    }
    for (size_t i = 0; i < n; ++i) {
      s = batch_stage_out(b->resident[pick[i]].h, b->stream);
      if (s) return s;
    }
  }
  BCU(cudaStreamSynchronize(b->stream));
  int32_t result = TEXO_GP_OK;
  std::vector<char> finished(nres, 0);
  for (size_t i = 0; i < n; ++i) {
    Job& j = b->resident[pick[i]];
    batch_absorb(j.h);
    if (batch_timed_out(j.h)) {
      result = TEXO_GP_ERR_DEVICE_TIMEOUT;
      set_last_error("batch: a job's barrier wait ran out");
    }
    if (handle_finished(j.h)) finished[pick[i]] = 1;
  }
  std::vector<Job> keep;
  keep.reserve(nres);
  for (size_t i = 0; i < nres; ++i) {
    if (finished[i])
      b->done.push_back(b->resident[i]);
    else
      keep.push_back(b->resident[i]);
  }
  b->resident.swap(keep);
  if (!b->resident.empty()) b->rr %= b->resident.size();
  return result;
}

int32_t texo_gp_batch_retire(texo_gp_batch b, uint64_t* job_id, uint32_t* out_targets, uint64_t targets_capacity,
                             texo_gp_stats* stats) {
  if (!b) return TEXO_GP_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(b->mu);
  if (b->done.empty()) return TEXO_GP_ERR_BUSY;
  Job j = b->done.front();
  uint64_t units = 0;
  texo_gp_sizes(j.h, &units, nullptr, nullptr, nullptr, nullptr, nullptr);
  if (out_targets && targets_capacity < 2 * units) return TEXO_GP_ERR_INVALID_ARGUMENT;
  b->done.pop_front();
  if (job_id) *job_id = j.id;
  const int32_t s = texo_gp_run(j.h, 0, out_targets, nullptr, stats);
  texo_gp_destroy(j.h);
  b->used -= j.bytes;
  return s;
}

int32_t texo_gp_batch_graphs(texo_gp_batch b, uint64_t* captures, uint64_t* replays) {
  if (!b) return TEXO_GP_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(b->mu);
  if (captures) *captures = b->captures;
  if (replays) *replays = b->replays;
  return TEXO_GP_OK;
}

int32_t texo_gp_batch_counts(texo_gp_batch b, uint32_t* resident, uint32_t* finished, uint64_t* bytes_in_use) {
  if (!b) return TEXO_GP_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(b->mu);
  if (resident) *resident = (uint32_t)b->resident.size();
  if (finished) *finished = (uint32_t)b->done.size();
  if (bytes_in_use) *bytes_in_use = b->used;
  return TEXO_GP_OK;
}

}  // extern "C"
