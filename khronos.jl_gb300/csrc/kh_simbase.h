// Host-side interface of one simulation, shared by the C-ABI implementation
// (kh_sim.cu) and the request server (kh_serve.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <string>

#include "../../include/khronos_gb300.h"

namespace kh_host {

struct SimBase {
  virtual ~SimBase() = default;
  std::string err;
  int64_t launches = 0;
  virtual kh_status set_material(int kind, int comp, const double* v) = 0;
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
};

}  // namespace kh_host

struct kh_sim {
  std::unique_ptr<kh_host::SimBase> impl;
  std::string err;
};
