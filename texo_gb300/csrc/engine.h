// engine.h — host-side model of one placement instance and its device state.
#pragma once
#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/texo_gp.h"
#include "kernels.cuh"
#include "persistent.cuh"

namespace tgp {

void set_last_error(const std::string& s);

// Host preprocessing of a texo_gp_problem into the device layout. Mirrors
// `eplace::place` setup (eplace.rs:254-346), `DensityModel::new` and
// `initial_fillers` (electrostatic_placement.rs:139-240) and the hypergraph
// preconditioners (analytical_placement.rs:177-231).
struct HostModel {
  texo_gp_params params{};
  uint32_t W = 0, H = 0, Wb = 0, Hb = 0;
  double sx = 1, sy = 1;
  bool identity = true;
  double td = 1.0;
  uint32_t K = 0;
  std::vector<texo_gp_field> kinds;
  std::vector<std::vector<uint32_t>> cap;        // [K][W*H] after fixed occupancy
  std::vector<uint64_t> available;               // [K]
  std::vector<std::vector<double>> smoothed;     // [K][B] td-scaled smoothed capacity
  std::vector<uint64_t> real_count;              // [K]
  std::vector<double> real_area;                 // [K]
  uint32_t U = 0, F = 0, Mm = 0;
  // members (flattened, density units only)
  std::vector<int> mem_unit, mem_field;
  std::vector<double> mem_off;                   // [2Mm]
  std::vector<float> mem_q;
  std::vector<int> unit_mem_ptr;                 // [U+1]
  // fillers
  std::vector<int> fil_field;
  std::vector<double> fil_q;
  // optimizer vector
  std::vector<double> init, lo, hi;              // [2(U+F)]
  std::vector<double> pre_static;                // [U+F]
  std::vector<double> pre_q;                     // [K][U+F]
  std::vector<double> gamma_weight;              // [K]
  // WA
  std::vector<int> net_ptr, pin_unit;
  std::vector<double> pin_base;                  // [2P]
  std::vector<float> net_w;
  int n_classes = 0;
  int class_begin[kMaxClasses + 1] = {0};
  int class_group[kMaxClasses] = {0};
  int n_hpwl_nets = 0;
  bool has_density = false;

  uint64_t coords() const { return 2ull * (U + F); }
  uint64_t bins() const { return (uint64_t)Wb * Hb; }
  double overflow_target(uint32_t f) const;
  double gamma_base_tiles() const;
};

int32_t build_model(const texo_gp_problem* p, const texo_gp_params* prm, HostModel& m, uint64_t* err_index);

// Device-resident instance: every buffer one placement needs.
struct Instance {
  HostModel m;
  int device = 0;
  int sms = 152;
  int nvb = 1;
  cudaStream_t stream = nullptr;
  std::vector<void*> allocations;
  Dev d{};
  Reduce r{};
  float2 *bufX = nullptr, *bufXp = nullptr, *bufY = nullptr, *bufC = nullptr;
  float2 *gX = nullptr, *gY = nullptr, *gC = nullptr;
  float2* best = nullptr;                        // best checkpoint coordinates [U]
  uint32_t* prev_targets = nullptr;              // [2U]
  unsigned long long* mismatch = nullptr;
  // device engine: fixed buffer tables (roles rotate inside the kernel)
  float2* posb[4] = {nullptr, nullptr, nullptr, nullptr};
  float2* gradb[3] = {nullptr, nullptr, nullptr};
  RunBlock* run_dev = nullptr;                   // controller state + grid barrier
  RunBlock* h_run = nullptr;                     // its pinned host mirror
  int pblocks = 0;                               // persistent grid size
  double* h_scal = nullptr;                      // pinned host mirror
  long long* h_iscal = nullptr;
  uint64_t bytes = 0;
  tc::TcMaps tmaps{};                            // tensor maps of the tensor-core DCT operands

  ~Instance();
  int32_t alloc(void** p, size_t bytes);
  int32_t upload();
  // device layout: sizes every slice (fill = false) or also packs the host
  // data of the uploaded slices into the staging buffer (fill = true)
  void plan(bool fill, void* slicer);
  uint64_t device_bytes();   // the one allocation upload() makes
};

}  // namespace tgp

struct texo_gp_handle_s;

namespace tgp {
// Hooks the batch uses to drive device-engine handles through one launch.
// stage_in queues the controller state and barrier reset on stream s and
// fills the instance descriptor; stage_out queues the copies back; absorb
// mirrors the state once the stream has completed.
int32_t batch_stage_in(texo_gp_handle_s* h, uint32_t budget, cudaStream_t s, InstDesc* desc, bool* large);
int32_t batch_stage_out(texo_gp_handle_s* h, cudaStream_t s);
void batch_stage_host(texo_gp_handle_s* h, uint32_t budget, InstDesc* desc, bool* large, RunBlock** host,
                      RunBlock** dev);
bool batch_timed_out(texo_gp_handle_s* h);     // the last launch's barrier wait ran out
int32_t batch_absorb(texo_gp_handle_s* h);
bool handle_finished(texo_gp_handle_s* h);
uint64_t handle_bytes(texo_gp_handle_s* h);
int handle_virtual_blocks(texo_gp_handle_s* h);
// Elements one iteration of the instance touches (objects, members, pins,
// bins per field, the transform counted twice): its share of a batch.
uint64_t handle_work(texo_gp_handle_s* h);
int handle_sms(texo_gp_handle_s* h);
Instance* handle_instance(texo_gp_handle_s* h);
// texo_gp_create in two steps: the host model (no device work), then the
// device upload; between them handle_device_bytes gives the footprint.
int32_t handle_build(const texo_gp_problem* p, const texo_gp_params* prm, texo_gp_handle_s** out,
                     uint64_t* err_index);
uint64_t handle_device_bytes(texo_gp_handle_s* h);
int32_t handle_upload(texo_gp_handle_s* h);
int32_t batch_add_handle(texo_gp_batch b, texo_gp_handle h, uint64_t job_id);
std::mutex* handle_mutex(texo_gp_handle_s* h);
}  // namespace tgp
