// batch.cu — many resident placements advanced by one persistent launch.
//
// Each admitted job is a device-engine handle with its own buffers, its own
// controller state and its own barrier. `advance` gives every resident job a
// share of the GPU's co-resident blocks (proportional to its virtual block
// count) and runs all of them in one cooperative launch of k_batch; jobs run
// independently inside it, each over its own physical blocks. A job's results
// do not depend on how many physical blocks it got, so they are bit-identical
// to the same job placed alone.
#include <algorithm>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <vector>

#include "engine.h"

namespace {
using namespace tgp;

struct Job {
  uint64_t id = 0;
  texo_gp_handle h = nullptr;
  uint64_t bytes = 0;
  int V = 1;
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

  ~texo_gp_batch_s() {
    if (stream) cudaStreamSynchronize(stream);
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
  for (size_t i = 0; i < n; ++i) {
    bool large = false;
    const int32_t st = batch_stage_in(b->resident[pick[i]].h, iterations, b->stream, &b->h_descs[i], &large);
    if (st) return st;
    lg[i] = large ? 1 : 0;
  }
  BCU(cudaMemcpyAsync(b->d_descs, b->h_descs.data(), sizeof(InstDesc) * n, cudaMemcpyHostToDevice, b->stream));
  // One launch per DCT tile family (a job runs the same kernel instantiation
  // as it does alone); physical blocks proportional to virtual blocks, at
  // least one each.
  int32_t s = TEXO_GP_OK;
  for (int fam = 0; fam < 2; ++fam) {
    std::vector<size_t> jobs;
    for (size_t i = 0; i < n; ++i)
      if (lg[i] == fam) jobs.push_back(i);
    if (jobs.empty()) continue;
    const int nj = (int)jobs.size();
    long long vsum = 0;
    for (size_t i : jobs) vsum += b->resident[pick[i]].V;
    b->h_map.clear();
    int used = nj;
    for (size_t i : jobs) {
      const int V = b->resident[pick[i]].V;
      const int want = std::max(1, (int)((long long)(P - nj) * V / std::max(vsum, 1ll)) + 1);
      const int add = std::max(0, std::min(std::min(want, V) - 1, P - used));
      used += add;
      for (int k = 0; k < 1 + add; ++k) b->h_map.push_back(make_int4((int)i, k, 1 + add, 0));
    }
    BCU(cudaMemcpyAsync(b->d_map, b->h_map.data(), sizeof(int4) * b->h_map.size(), cudaMemcpyHostToDevice,
                        b->stream));
    s = launch_batch(b->d_descs, b->d_map, (int)b->h_map.size(), fam == 1, b->stream);
    if (s) {
      set_last_error(std::string("batch launch: ") + cudaGetErrorString(cudaGetLastError()));
      return s;
    }
  }
  for (size_t i = 0; i < n; ++i) {
    s = batch_stage_out(b->resident[pick[i]].h, b->stream);
    if (s) return s;
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

int32_t texo_gp_batch_counts(texo_gp_batch b, uint32_t* resident, uint32_t* finished, uint64_t* bytes_in_use) {
  if (!b) return TEXO_GP_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(b->mu);
  if (resident) *resident = (uint32_t)b->resident.size();
  if (finished) *finished = (uint32_t)b->done.size();
  if (bytes_in_use) *bytes_in_use = b->used;
  return TEXO_GP_OK;
}

}  // extern "C"
