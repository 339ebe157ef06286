// Host-side interface of one simulation, shared by the C-ABI implementation
// (kh_sim.cu) and the request server (kh_serve.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <string>

#include "../../include/khronos_gb300.h"

namespace kh_host {

// Library allocations.  Device memory comes from a per-device stream-ordered
// pool (cudaMallocFromPoolAsync / cudaFreeAsync) that keeps freed memory for
// reuse instead of returning it to the device: freeing never synchronises the
// device, so simulations released while others step (the request server) or
// temporaries of a flux read do not stall the other streams.  Pinned host
// staging buffers are likewise recycled, never freed while the process runs.
cudaError_t dev_alloc(void** p, size_t bytes, cudaStream_t s);
cudaError_t dev_free(void* p, cudaStream_t s);
void* pinned_get(size_t bytes);
void pinned_put(void* p, size_t bytes);

// Device view of one DFT monitor: accumulators F[f·ncell + cell] (cell x
// fastest over the monitor box) and, for FP32 runs, the Kahan compensation
// C (value = F − C); C is null in FP64 runs.
struct MonitorView {
  const void* F = nullptr;
  const void* C = nullptr;
  int dims[3] = {0, 0, 0};
  int nf = 0;
  int dtype = KH_F32;
  long long ncell() const { return (long long)dims[0] * dims[1] * dims[2]; }
};

// Device view of one history monitor: field values of one component over a
// cell box at every step, buf[step·ncell + cell] (cell x fastest), `recorded`
// steps valid (0 ≤ step < recorded).
struct HistoryView {
  const void* buf = nullptr;
  int dims[3] = {0, 0, 0};
  long long ncell = 0;
  int64_t capacity = 0, recorded = 0;
  int dtype = KH_F32;
};

struct SimBase {
  virtual ~SimBase() = default;
  std::string err;
  int64_t launches = 0;
  virtual kh_status set_material(int kind, int comp, const double* v) = 0;
  virtual kh_status attach_material(int kind, int comp, const void* v, int dtype) = 0;
  virtual kh_status add_pole(const kh_pole_coeffs& c, const double* s) = 0;
  virtual kh_status add_source(const kh_source_desc& s) = 0;
  virtual kh_status add_monitor(int comp, const int32_t* st, const int32_t* dm, int nf,
                                const double* f, int dec, int32_t* id) = 0;
  virtual kh_status prepare() = 0;
  virtual bool is_prepared() const = 0;
  virtual kh_status step(int64_t n, cudaStream_t s) = 0;
  virtual int64_t timestep() const = 0;
  virtual int sources_active() const = 0;
  virtual int64_t cells() const = 0;
  // Device bytes prepare() will allocate (before prepare) / has allocated.
  virtual int64_t estimate_bytes() const = 0;
  virtual int64_t device_bytes() const = 0;
  // Block the calling thread until this simulation's queued work is done.
  virtual kh_status wait_idle() = 0;
  virtual kh_status get_field(int comp, double* out) = 0;
  virtual kh_status read_dft(int id, double* out) = 0;
  virtual kh_status monitor_info(int id, int32_t* dims, int32_t* nf) const = 0;
  virtual kh_status flux(const int32_t* ids, int normal, double dA, double* out) = 0;
  virtual kh_status flux_static(const int32_t* ids, int normal, double dA, double* out) = 0;
  virtual kh_status reset() = 0;
  virtual int64_t state_bytes() const = 0;
  virtual kh_status export_state(void* dst, int64_t bytes) = 0;
  virtual kh_status import_state(const void* src, int64_t bytes) = 0;
  virtual double model_bytes_per_step() const = 0;
  virtual kh_status device_error() = 0;
  virtual void model_split(double& h, double& e, double& dft) const = 0;
  virtual kh_status step_timed(int64_t n, cudaStream_t s, double* h_ms, double* e_ms,
                               double* dft_ms) = 0;
  // After prepare: overwrite per-voxel ε⁻¹/μ⁻¹ in a cell box; replace one
  // source's amplitudes (same footprint) and time table.
  virtual kh_status update_material_box(int kind, int comp, const int32_t* st, const int32_t* dm,
                                        const double* v) = 0;
  virtual kh_status update_source(int index, const double* amp, int64_t table_len,
                                  const double* table, double cutoff) = 0;
  // Device arrays of a monitor, valid once this simulation's queued work is done.
  virtual kh_status monitor_view(int id, MonitorView* out) = 0;
  virtual int monitor_count() const = 0;
  virtual int dtype() const = 0;
  // Device arrays of E_x..E_z, H_x..H_z (padded layout, `count` elements each,
  // zero outside the grid), valid once this simulation's queued work is done.
  virtual kh_status field_arrays(const void* out[6], long long* count) = 0;
  virtual kh_status field_view(int comp, kh_field_view* out) = 0;
  virtual kh_status add_history(int comp, const int32_t* st, const int32_t* dm, int64_t capacity,
                                int32_t* id) = 0;
  virtual kh_status history_view(int id, HistoryView* out) = 0;
  // Step counts that keep batch boundaries aligned with the DFT decimation
  // (their multiples replay captured step graphs).
  virtual int step_alignment() const = 0;
  virtual int64_t graph_replays() const = 0;
  virtual kh_status set_geometry(const kh_object* objs, int n, double background, const double* origin,
                                 int smoothing) = 0;
  virtual kh_status read_material(int kind, int comp, double* out) = 0;
};

}  // namespace kh_host

struct kh_sim {
  std::unique_ptr<kh_host::SimBase> impl;
  std::string err;
};
