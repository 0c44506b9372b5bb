// server.cu — the serving loop: continuous batching of placement requests.
//
// Three kinds of threads share one server:
//  * callers submit requests (the problem is copied) and poll results;
//  * admission threads build each job's host model, wait until its exact
//    device footprint fits the HBM budget, reserve it and upload the job;
//  * the serving thread adds uploaded jobs to the resident batch at each
//    launch boundary, advances all resident jobs by one persistent launch of
//    `chunk_iterations` iterations, and retires the jobs that stopped,
//    returning their memory to the budget.
// Uploads run on the jobs' own streams while the batch kernel runs, so a
// request that arrives while others are on the GPU is prepared in parallel
// and joins them at the next launch.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "engine.h"

namespace {
using namespace tgp;

// A texo_gp_problem whose arrays the server owns.
struct OwnedProblem {
  std::vector<texo_gp_field> fields;
  std::vector<uint32_t> capacity, fixed_occupancy, member_ptr, member_field, member_cell, cell_unit, net_ptr,
      pin_cell, arc_driver, arc_sink;
  std::vector<double> initial_xy, lower_xy, upper_xy, member_offset_xy, member_charge, cell_offset_xy, cell_fixed_xy;
  std::vector<uint8_t> cell_fixed;
  std::vector<uint64_t> arc_weight;
  texo_gp_problem p{};
};

template <typename T>
const T* dup(std::vector<T>& store, const T* src, size_t n) {
  if (!src) return nullptr;
  store.assign(src, src + n);
  return store.data();
}

int32_t copy_problem(const texo_gp_problem* s, OwnedProblem& o) {
  if (!s || !s->member_ptr || (s->num_nets && !s->net_ptr)) return TEXO_GP_ERR_INVALID_ARGUMENT;
  const size_t tiles = (size_t)s->width * s->height, U = s->num_units, C = s->num_cells, E = s->num_nets;
  const size_t M = s->member_ptr[U], P = E ? s->net_ptr[E] : 0, A = s->num_timed_arcs;
  texo_gp_problem& p = o.p;
  p = *s;
  p.fields = dup(o.fields, s->fields, s->num_fields);
  p.capacity = dup(o.capacity, s->capacity, (size_t)s->num_fields * tiles);
  p.fixed_occupancy = dup(o.fixed_occupancy, s->fixed_occupancy, 3 * (size_t)s->num_fixed_occupancy);
  p.initial_xy = dup(o.initial_xy, s->initial_xy, 2 * U);
  p.lower_xy = dup(o.lower_xy, s->lower_xy, 2 * U);
  p.upper_xy = dup(o.upper_xy, s->upper_xy, 2 * U);
  p.member_ptr = dup(o.member_ptr, s->member_ptr, U + 1);
  p.member_field = dup(o.member_field, s->member_field, M);
  p.member_offset_xy = dup(o.member_offset_xy, s->member_offset_xy, 2 * M);
  p.member_charge = dup(o.member_charge, s->member_charge, M);
  p.member_cell = dup(o.member_cell, s->member_cell, M);
  p.cell_unit = dup(o.cell_unit, s->cell_unit, C);
  p.cell_offset_xy = dup(o.cell_offset_xy, s->cell_offset_xy, 2 * C);
  p.cell_fixed = dup(o.cell_fixed, s->cell_fixed, C);
  p.cell_fixed_xy = dup(o.cell_fixed_xy, s->cell_fixed_xy, 2 * C);
  p.net_ptr = dup(o.net_ptr, s->net_ptr, E ? E + 1 : 0);
  p.pin_cell = dup(o.pin_cell, s->pin_cell, P);
  p.arc_driver_cell = dup(o.arc_driver, s->arc_driver_cell, A);
  p.arc_sink_cell = dup(o.arc_sink, s->arc_sink_cell, A);
  p.arc_extra_weight = dup(o.arc_weight, s->arc_extra_weight, A);
  return TEXO_GP_OK;
}

struct Pending {
  uint64_t id = 0;
  std::unique_ptr<OwnedProblem> prob;
  texo_gp_params prm{};
  double submit_ms = 0;
};
struct Uploaded {
  uint64_t id = 0;
  texo_gp_handle h = nullptr;
  uint64_t bytes = 0;
  uint32_t units = 0;
  double submit_ms = 0, admit_ms = 0;
};
struct Finished {
  texo_gp_job_result r{};
  std::vector<uint32_t> targets;
};

}  // namespace

struct texo_gp_server_s {
  texo_gp_params defaults{};
  texo_gp_server_options opt{};
  texo_gp_batch batch = nullptr;
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  std::mutex mu;
  std::condition_variable cv_queue, cv_budget, cv_ready, cv_done;
  std::deque<Pending> queue;
  std::deque<Uploaded> ready;
  std::deque<Finished> done;
  std::unordered_map<uint64_t, Uploaded> resident;   // by job id (handles owned by the batch)
  uint64_t budget = 0, reserved = 0;
  uint32_t building = 0;
  bool stop = false;
  std::vector<std::thread> workers;
  std::thread loop;

  double now_ms() const {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
  // (mu held)
  void finish_error(uint64_t id, int32_t status, double submit_ms) {
    Finished f;
    f.r.job_id = id;
    f.r.status = status;
    f.r.stats.status = status;
    f.r.submit_ms = submit_ms;
    f.r.admit_ms = -1.0;
    f.r.finish_ms = now_ms();
    done.push_back(std::move(f));
    cv_done.notify_all();
  }
  void admission_thread();
  void serving_thread();
};

void texo_gp_server_s::admission_thread() {
  cudaSetDevice(defaults.device);
  for (;;) {
    Pending job;
    {
      std::unique_lock<std::mutex> lk(mu);
      cv_queue.wait(lk, [&] { return stop || !queue.empty(); });
      if (stop) return;
      job = std::move(queue.front());
      queue.pop_front();
      ++building;
    }
    texo_gp_handle h = nullptr;
    int32_t s = handle_build(&job.prob->p, &job.prm, &h, nullptr);
    job.prob.reset();   // the model holds what the device needs
    uint64_t bytes = 0;
    uint32_t units = 0;
    if (s == TEXO_GP_OK) {
      bytes = handle_device_bytes(h);
      uint64_t u = 0;
      texo_gp_sizes(h, &u, nullptr, nullptr, nullptr, nullptr, nullptr);
      units = (uint32_t)u;
      if (bytes > budget) s = TEXO_GP_ERR_OUT_OF_MEMORY;
    }
    if (s != TEXO_GP_OK) {
      if (h) texo_gp_destroy(h);
      std::lock_guard<std::mutex> lk(mu);
      --building;
      finish_error(job.id, s, job.submit_ms);
      continue;
    }
    {
      std::unique_lock<std::mutex> lk(mu);
      cv_budget.wait(lk, [&] { return stop || reserved + bytes <= budget; });
      if (stop) {
        --building;
        lk.unlock();
        texo_gp_destroy(h);
        return;
      }
      reserved += bytes;
    }
    s = handle_upload(h);
    std::lock_guard<std::mutex> lk(mu);
    --building;
    if (s != TEXO_GP_OK) {
      reserved -= bytes;
      cv_budget.notify_all();
      texo_gp_destroy(h);
      finish_error(job.id, s, job.submit_ms);
      continue;
    }
    Uploaded u;
    u.id = job.id;
    u.h = h;
    u.bytes = bytes;
    u.units = units;
    u.submit_ms = job.submit_ms;
    u.admit_ms = now_ms();
    ready.push_back(u);
    cv_ready.notify_one();
  }
}

void texo_gp_server_s::serving_thread() {
  cudaSetDevice(defaults.device);
  std::vector<uint32_t> targets;
  for (;;) {
    uint32_t max_units = 0;
    {
      std::unique_lock<std::mutex> lk(mu);
      cv_ready.wait(lk, [&] { return stop || !ready.empty() || !resident.empty(); });
      if (stop) return;
      while (!ready.empty() && resident.size() < opt.max_resident) {
        Uploaded u = ready.front();
        ready.pop_front();
        const int32_t s = batch_add_handle(batch, u.h, u.id);
        if (s != TEXO_GP_OK) {   // no slot: retry at the next boundary
          ready.push_front(u);
          break;
        }
        resident[u.id] = u;
      }
      for (auto& kv : resident) max_units = std::max(max_units, kv.second.units);
    }
    const int32_t adv = texo_gp_batch_advance(batch, opt.chunk_iterations);
    targets.resize(std::max<size_t>(2 * (size_t)max_units, 2));
    for (;;) {
      uint64_t id = 0;
      texo_gp_stats st{};
      const int32_t s = texo_gp_batch_retire(batch, &id, targets.data(), targets.size(), &st);
      if (s == TEXO_GP_ERR_BUSY) break;
      std::lock_guard<std::mutex> lk(mu);
      auto it = resident.find(id);
      if (it == resident.end()) continue;
      Finished f;
      f.r.job_id = id;
      f.r.status = s;
      f.r.units = it->second.units;
      f.r.stats = st;
      f.r.stats.status = s;
      f.r.submit_ms = it->second.submit_ms;
      f.r.admit_ms = it->second.admit_ms;
      f.r.finish_ms = now_ms();
      if (s == TEXO_GP_OK || s == TEXO_GP_ERR_DID_NOT_CONVERGE)
        f.targets.assign(targets.begin(), targets.begin() + 2 * (size_t)it->second.units);
      reserved -= it->second.bytes;
      resident.erase(it);
      done.push_back(std::move(f));
      cv_done.notify_all();
      cv_budget.notify_all();
    }
    if (adv != TEXO_GP_OK) {
      // a launch failed (CUDA error or a barrier timeout): every job still
      // resident ends with that status and the batch starts over empty
      std::lock_guard<std::mutex> lk(mu);
      texo_gp_batch_destroy(batch);
      batch = nullptr;
      for (auto& kv : resident) {
        reserved -= kv.second.bytes;
        Finished f;
        f.r.job_id = kv.first;
        f.r.status = adv;
        f.r.stats.status = adv;
        f.r.units = kv.second.units;
        f.r.submit_ms = kv.second.submit_ms;
        f.r.admit_ms = kv.second.admit_ms;
        f.r.finish_ms = now_ms();
        done.push_back(std::move(f));
      }
      resident.clear();
      cv_done.notify_all();
      cv_budget.notify_all();
      if (texo_gp_batch_create(&defaults, ~0ull, opt.max_resident, &batch) != TEXO_GP_OK) {
        stop = true;   // the device is unusable; fail what is left
        for (auto& u : ready) {
          texo_gp_destroy(u.h);
          reserved -= u.bytes;
          finish_error(u.id, adv, u.submit_ms);
        }
        ready.clear();
        cv_queue.notify_all();
        return;
      }
    }
  }
}

extern "C" {

int32_t texo_gp_server_create(const texo_gp_params* defaults, const texo_gp_server_options* options,
                              texo_gp_server* out) {
  if (!out) return TEXO_GP_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  auto s = std::make_unique<texo_gp_server_s>();
  if (defaults)
    s->defaults = *defaults;
  else
    texo_gp_default_params(&s->defaults);
  s->defaults.engine = TEXO_GP_ENGINE_DEVICE;
  if (options) s->opt = *options;
  if (!s->opt.max_resident) s->opt.max_resident = 256;
  if (!s->opt.chunk_iterations) s->opt.chunk_iterations = 20;
  if (!s->opt.admission_threads) s->opt.admission_threads = 4;
  if (cudaSetDevice(s->defaults.device) != cudaSuccess) return TEXO_GP_ERR_CUDA;
  s->budget = s->opt.hbm_budget_bytes;
  if (!s->budget) {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return TEXO_GP_ERR_CUDA;
    s->budget = free_b / 4 * 3;
  }
  const int32_t st = texo_gp_batch_create(&s->defaults, ~0ull, s->opt.max_resident, &s->batch);
  if (st) return st;
  texo_gp_server_s* raw = s.get();
  for (uint32_t i = 0; i < s->opt.admission_threads; ++i) s->workers.emplace_back([raw] { raw->admission_thread(); });
  s->loop = std::thread([raw] { raw->serving_thread(); });
  *out = s.release();
  return TEXO_GP_OK;
}

int32_t texo_gp_server_destroy(texo_gp_server s) {
  if (!s) return TEXO_GP_ERR_INVALID_ARGUMENT;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_queue.notify_all();
  s->cv_budget.notify_all();
  s->cv_ready.notify_all();
  s->cv_done.notify_all();
  if (s->loop.joinable()) s->loop.join();
  for (auto& t : s->workers)
    if (t.joinable()) t.join();
  for (auto& u : s->ready) texo_gp_destroy(u.h);
  if (s->batch) texo_gp_batch_destroy(s->batch);
  delete s;
  return TEXO_GP_OK;
}

int32_t texo_gp_server_submit(texo_gp_server s, const texo_gp_problem* problem, const texo_gp_params* params,
                              uint64_t job_id) {
  if (!s || !problem) return TEXO_GP_ERR_INVALID_ARGUMENT;
  Pending p;
  p.id = job_id;
  p.prob = std::make_unique<OwnedProblem>();
  const int32_t st = copy_problem(problem, *p.prob);
  if (st) return st;
  p.prm = params ? *params : s->defaults;
  p.prm.engine = TEXO_GP_ENGINE_DEVICE;
  p.prm.device = s->defaults.device;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return TEXO_GP_ERR_CUDA;
    p.submit_ms = s->now_ms();
    s->queue.push_back(std::move(p));
  }
  s->cv_queue.notify_one();
  return TEXO_GP_OK;
}

int32_t texo_gp_server_poll(texo_gp_server s, int32_t wait_ms, texo_gp_job_result* out, uint32_t* out_targets,
                            uint64_t targets_capacity) {
  if (!s || !out) return TEXO_GP_ERR_INVALID_ARGUMENT;
  std::unique_lock<std::mutex> lk(s->mu);
  auto ready = [&] { return !s->done.empty() || s->stop; };
  if (wait_ms < 0)
    s->cv_done.wait(lk, ready);
  else
    s->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), ready);
  if (s->done.empty()) return TEXO_GP_ERR_BUSY;
  Finished& f = s->done.front();
  if (out_targets && !f.targets.empty()) {
    if (targets_capacity < f.targets.size()) {
      out->job_id = f.r.job_id;   // tells the caller the size it needs
      out->units = f.r.units;
      return TEXO_GP_ERR_INVALID_ARGUMENT;
    }
    std::memcpy(out_targets, f.targets.data(), f.targets.size() * sizeof(uint32_t));
  }
  *out = f.r;
  s->done.pop_front();
  return TEXO_GP_OK;
}

int32_t texo_gp_server_counts(texo_gp_server s, uint32_t* queued, uint32_t* resident, uint32_t* finished,
                              uint64_t* bytes_in_use) {
  if (!s) return TEXO_GP_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lk(s->mu);
  if (queued) *queued = (uint32_t)(s->queue.size() + s->building + s->ready.size());
  if (resident) *resident = (uint32_t)s->resident.size();
  if (finished) *finished = (uint32_t)s->done.size();
  if (bytes_in_use) *bytes_in_use = s->reserved;
  return TEXO_GP_OK;
}

double texo_gp_server_clock_ms(texo_gp_server s) { return s ? s->now_ms() : 0.0; }

}  // extern "C"
