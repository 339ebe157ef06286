// FP64 reductions on the device: the objective's DFT overlap, the forward ×
// adjoint DFT-field product per design voxel (the adjoint path), and the
// squared norms of the six field arrays (decay checks).
//
// The reference computes both on the host after downloading the DFT arrays:
//   evaluate(::FourierFieldsObjective) + the user objective
//     (src/Adjoint/ObjectiveQuantities.jl:282-288),
//   calculate_gradient! (src/Adjoint/GradientKernel.jl:35-109): a triple loop
//     Σ_f Re[dε⁻¹/dρ · w · D_adj · D_fwd] per design parameter.
// Here both run on the device in FP64 over the FP32 (Kahan) or FP64 DFT
// accumulators, with a fixed reduction order so results are reproducible.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "../../include/khronos_gb300.h"
#include "kh_kernels.cuh"
#include "kh_simbase.h"

using kh::Cplx;
using kh_host::MonitorView;

namespace {

constexpr int kRedThreads = 256;

template <typename T>
__device__ __forceinline__ double2 dft_value(const Cplx<T>* F, const Cplx<T>* C, long long q) {
  double re = double(F[q].re), im = double(F[q].im);
  if (C) {  // Kahan: sum − compensation
    re -= double(C[q].re);
    im -= double(C[q].im);
  }
  return make_double2(re, im);
}

__device__ __forceinline__ double2 block_sum(double re, double im) {
  __shared__ double sr[kRedThreads], si[kRedThreads];
  sr[threadIdx.x] = re;
  si[threadIdx.x] = im;
  __syncthreads();
  for (int w = kRedThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      sr[threadIdx.x] += sr[threadIdx.x + w];
      si[threadIdx.x] += si[threadIdx.x + w];
    }
    __syncthreads();
  }
  return make_double2(sr[0], si[0]);
}

// Stage 1: block (b, f) sums w·F over its contiguous chunk of cells.
template <typename T>
__global__ void __launch_bounds__(kRedThreads) overlap_partial_kernel(
    const Cplx<T>* F, const Cplx<T>* C, const double2* w, long long ncell, long long chunk,
    double2* partial) {
  const int f = blockIdx.y;
  const long long lo = (long long)blockIdx.x * chunk;
  const long long hi = min(ncell, lo + chunk);
  double re = 0.0, im = 0.0;
  for (long long c = lo + threadIdx.x; c < hi; c += kRedThreads) {
    const long long q = (long long)f * ncell + c;
    const double2 v = dft_value(F, C, q);
    const double2 ww = w[q];
    re += v.x * ww.x - v.y * ww.y;
    im += v.x * ww.y + v.y * ww.x;
  }
  const double2 s = block_sum(re, im);
  if (threadIdx.x == 0) partial[(long long)f * gridDim.x + blockIdx.x] = s;
}

// Stage 2: one block per frequency sums the partials in a fixed order.
__global__ void __launch_bounds__(kRedThreads) overlap_final_kernel(const double2* partial, int nblk,
                                                                    double2* out) {
  const int f = blockIdx.x;
  double re = 0.0, im = 0.0;
  for (int b = threadIdx.x; b < nblk; b += kRedThreads) {
    re += partial[(long long)f * nblk + b].x;
    im += partial[(long long)f * nblk + b].y;
  }
  const double2 s = block_sum(re, im);
  if (threadIdx.x == 0) out[f] = s;
}

// Squared norm Σ|F|² of one DFT array (all cells and frequencies): block b
// sums its contiguous chunk.
template <typename T>
__global__ void __launch_bounds__(kRedThreads) dft_sq_partial_kernel(const Cplx<T>* F, const Cplx<T>* C,
                                                                     long long total, long long chunk,
                                                                     double2* partial) {
  const long long lo = (long long)blockIdx.x * chunk;
  const long long hi = min(total, lo + chunk);
  double s = 0.0;
  for (long long q = lo + threadIdx.x; q < hi; q += kRedThreads) {
    const double2 v = dft_value(F, C, q);
    s += v.x * v.x + v.y * v.y;
  }
  const double2 r = block_sum(s, 0.0);
  if (threadIdx.x == 0) partial[blockIdx.x] = r;
}

// Squared L2 norm of one field array: block (b, c) sums x² over its chunk.
template <typename T>
struct FieldArgs {
  const T* f[6];
  long long count, chunk;
};

template <typename T>
__global__ void __launch_bounds__(kRedThreads) sq_norm_partial_kernel(const FieldArgs<T> a, double2* partial) {
  const int c = blockIdx.y;
  const T* x = a.f[c];
  const long long lo = (long long)blockIdx.x * a.chunk;
  const long long hi = min(a.count, lo + a.chunk);
  double s = 0.0;
  for (long long q = lo + threadIdx.x; q < hi; q += kRedThreads) {
    const double v = double(x[q]);
    s += v * v;
  }
  const double2 r = block_sum(s, 0.0);
  if (threadIdx.x == 0) partial[(long long)c * gridDim.x + blockIdx.x] = r;
}

// Per design voxel v: Re(coef · Σ_c F_c(v, f_fwd) · A_c(v, f_adj)).
template <typename T>
struct GradArgs {
  const Cplx<T>* F[3];
  const Cplx<T>* FC[3];
  const Cplx<T>* A[3];
  const Cplx<T>* AC[3];
  long long ncell;
  int ff, fa;
  double coef_re, coef_im;
};

template <typename T>
__global__ void __launch_bounds__(kRedThreads) adjoint_gradient_kernel(const GradArgs<T> a, double* out) {
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < a.ncell;
       v += (long long)gridDim.x * blockDim.x) {
    double re = 0.0, im = 0.0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const double2 f = dft_value(a.F[c], a.FC[c], (long long)a.ff * a.ncell + v);
      const double2 g = dft_value(a.A[c], a.AC[c], (long long)a.fa * a.ncell + v);
      re += f.x * g.x - f.y * g.y;
      im += f.x * g.y + f.y * g.x;
    }
    out[v] = a.coef_re * re - a.coef_im * im;
  }
}

// Time correlation of two histories per voxel v:
//   out[v] = coef · Σ_c Σ_{m<N} F_c[m, v] · A_c[N−1−m, v]
// (forward field at step m times the adjoint field of the time-reversed run
// at step N−1−m), FP64 accumulation, one thread per voxel.
template <typename T>
struct CorrArgs {
  const T* F[3];
  const T* A[3];
  long long ncell;
  int64_t nsteps;
  double coef;
};

template <typename T>
__global__ void __launch_bounds__(kRedThreads) history_correlate_kernel(const CorrArgs<T> a, double* out) {
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < a.ncell;
       v += (long long)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int c = 0; c < 3; ++c) {
      const T* f = a.F[c] + v;
      const T* g = a.A[c] + (a.nsteps - 1) * a.ncell + v;
      for (int64_t m = 0; m < a.nsteps; ++m) s += double(f[m * a.ncell]) * double(g[-m * a.ncell]);
    }
    out[v] = a.coef * s;
  }
}

kh_status fail(kh_sim* s, kh_status st, const std::string& msg) {
  s->impl->err = msg;
  return st;
}

// Temporary device buffer from the library pool, on the legacy stream the
// reduction kernels and their synchronous copies run on.
struct DevBuf {
  void* p = nullptr;
  ~DevBuf() { kh_host::dev_free(p, cudaStreamLegacy); }
};

#define KH_ACUDA(sim, call)                                                              \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return fail(sim, e_ == cudaErrorMemoryAllocation ? KH_ERR_OOM : KH_ERR_CUDA,       \
                  std::string(#call) + ": " + cudaGetErrorString(e_));                   \
  } while (0)

template <typename T>
kh_status overlap_impl(kh_sim* sim, const MonitorView& m, const double* weights, double* out) {
  const long long ncell = m.ncell();
  const long long total = ncell * m.nf;
  const long long chunk = 8LL * kRedThreads;
  const int nblk = int(std::max<long long>(1, (ncell + chunk - 1) / chunk));
  DevBuf w, part, res;
  KH_ACUDA(sim, kh_host::dev_alloc(&w.p, size_t(total) * sizeof(double2), cudaStreamLegacy));
  KH_ACUDA(sim, kh_host::dev_alloc(&part.p, size_t(nblk) * m.nf * sizeof(double2), cudaStreamLegacy));
  KH_ACUDA(sim, kh_host::dev_alloc(&res.p, size_t(m.nf) * sizeof(double2), cudaStreamLegacy));
  KH_ACUDA(sim, cudaMemcpy(w.p, weights, size_t(total) * sizeof(double2), cudaMemcpyHostToDevice));
  overlap_partial_kernel<T><<<dim3(nblk, m.nf), kRedThreads>>>(
      static_cast<const Cplx<T>*>(m.F), static_cast<const Cplx<T>*>(m.C),
      static_cast<const double2*>(w.p), ncell, chunk, static_cast<double2*>(part.p));
  overlap_final_kernel<<<m.nf, kRedThreads>>>(static_cast<const double2*>(part.p), nblk,
                                               static_cast<double2*>(res.p));
  sim->impl->launches += 2;
  KH_ACUDA(sim, cudaGetLastError());
  KH_ACUDA(sim, cudaMemcpy(out, res.p, size_t(m.nf) * sizeof(double2), cudaMemcpyDeviceToHost));
  return KH_OK;
}

template <typename T>
kh_status gradient_impl(kh_sim* fwd, const MonitorView* fv, int ff, const MonitorView* av, int fa,
                        double coef_re, double coef_im, double* grad) {
  GradArgs<T> a;
  for (int c = 0; c < 3; ++c) {
    a.F[c] = static_cast<const Cplx<T>*>(fv[c].F);
    a.FC[c] = static_cast<const Cplx<T>*>(fv[c].C);
    a.A[c] = static_cast<const Cplx<T>*>(av[c].F);
    a.AC[c] = static_cast<const Cplx<T>*>(av[c].C);
  }
  a.ncell = fv[0].ncell();
  a.ff = ff;
  a.fa = fa;
  a.coef_re = coef_re;
  a.coef_im = coef_im;
  DevBuf out;
  KH_ACUDA(fwd, kh_host::dev_alloc(&out.p, size_t(a.ncell) * sizeof(double), cudaStreamLegacy));
  int blocks = int(std::min<long long>((a.ncell + kRedThreads - 1) / kRedThreads, 152LL * 8));
  adjoint_gradient_kernel<T><<<std::max(blocks, 1), kRedThreads>>>(a, static_cast<double*>(out.p));
  fwd->impl->launches += 1;
  KH_ACUDA(fwd, cudaGetLastError());
  std::vector<double> h(size_t(a.ncell));
  KH_ACUDA(fwd, cudaMemcpy(h.data(), out.p, h.size() * sizeof(double), cudaMemcpyDeviceToHost));
  for (size_t v = 0; v < h.size(); ++v) grad[v] += h[v];
  return KH_OK;
}

template <typename T>
kh_status sq_norms_impl(kh_sim* sim, const void* const* arrays, long long count, double* out) {
  FieldArgs<T> a;
  for (int c = 0; c < 6; ++c) a.f[c] = static_cast<const T*>(arrays[c]);
  a.count = count;
  a.chunk = 16LL * kRedThreads;
  const int nblk = int(std::max<long long>(1, (count + a.chunk - 1) / a.chunk));
  DevBuf part, res;
  KH_ACUDA(sim, kh_host::dev_alloc(&part.p, size_t(nblk) * 6 * sizeof(double2), cudaStreamLegacy));
  KH_ACUDA(sim, kh_host::dev_alloc(&res.p, 6 * sizeof(double2), cudaStreamLegacy));
  sq_norm_partial_kernel<T><<<dim3(nblk, 6), kRedThreads>>>(a, static_cast<double2*>(part.p));
  overlap_final_kernel<<<6, kRedThreads>>>(static_cast<const double2*>(part.p), nblk,
                                            static_cast<double2*>(res.p));
  sim->impl->launches += 2;
  KH_ACUDA(sim, cudaGetLastError());
  double2 h[6];
  KH_ACUDA(sim, cudaMemcpy(h, res.p, sizeof(h), cudaMemcpyDeviceToHost));
  for (int c = 0; c < 6; ++c) out[c] = h[c].x;
  return KH_OK;
}

template <typename T>
kh_status correlate_impl(kh_sim* fwd, const kh_host::HistoryView* fv, const kh_host::HistoryView* av,
                         int64_t nsteps, double coef, double* grad) {
  CorrArgs<T> a;
  for (int c = 0; c < 3; ++c) {
    a.F[c] = static_cast<const T*>(fv[c].buf);
    a.A[c] = static_cast<const T*>(av[c].buf);
  }
  a.ncell = fv[0].ncell;
  a.nsteps = nsteps;
  a.coef = coef;
  DevBuf out;
  KH_ACUDA(fwd, kh_host::dev_alloc(&out.p, size_t(a.ncell) * sizeof(double), cudaStreamLegacy));
  int blocks = int(std::min<long long>((a.ncell + kRedThreads - 1) / kRedThreads, 152LL * 16));
  history_correlate_kernel<T><<<std::max(blocks, 1), kRedThreads>>>(a, static_cast<double*>(out.p));
  fwd->impl->launches += 1;
  KH_ACUDA(fwd, cudaGetLastError());
  std::vector<double> h(size_t(a.ncell));
  KH_ACUDA(fwd, cudaMemcpy(h.data(), out.p, h.size() * sizeof(double), cudaMemcpyDeviceToHost));
  for (size_t v = 0; v < h.size(); ++v) grad[v] += h[v];
  return KH_OK;
}

}  // namespace

extern "C" {

kh_status kh_history_correlate(kh_sim* fwd, const int32_t fwd_ids[3], kh_sim* adj, const int32_t adj_ids[3],
                               int64_t nsteps, double coef, double* grad) {
  if (!fwd) return KH_ERR_INVALID;
  if (!adj || !fwd_ids || !adj_ids || !grad) return fail(fwd, KH_ERR_INVALID, "null correlation argument");
  if (fwd->impl->dtype() != adj->impl->dtype())
    return fail(fwd, KH_ERR_INVALID, "forward and adjoint simulations differ in precision");
  if (nsteps <= 0) return fail(fwd, KH_ERR_INVALID, "step count must be positive");
  kh_host::HistoryView fv[3], av[3];
  for (int c = 0; c < 3; ++c) {
    kh_status st = fwd->impl->history_view(fwd_ids[c], &fv[c]);
    if (st != KH_OK) return st;
    if ((st = adj->impl->history_view(adj_ids[c], &av[c])) != KH_OK)
      return fail(fwd, st, "adjoint history: " + adj->impl->err);
    for (int a = 0; a < 3; ++a)
      if (fv[c].dims[a] != fv[0].dims[a] || av[c].dims[a] != fv[0].dims[a])
        return fail(fwd, KH_ERR_INVALID, "history monitors must cover the same cell box");
    if (fv[c].recorded < nsteps || av[c].recorded < nsteps)
      return fail(fwd, KH_ERR_INVALID, "a history holds fewer steps than requested");
  }
  kh_status st = fwd->impl->wait_idle();
  if (st != KH_OK) return st;
  if ((st = adj->impl->wait_idle()) != KH_OK) return fail(fwd, st, "adjoint: " + adj->impl->err);
  return fwd->impl->dtype() == KH_F32 ? correlate_impl<float>(fwd, fv, av, nsteps, coef, grad)
                                      : correlate_impl<double>(fwd, fv, av, nsteps, coef, grad);
}

kh_status kh_sim_read_history(kh_sim* sim, int32_t id, int64_t step, double* out) {
  if (!sim) return KH_ERR_INVALID;
  if (!out) return fail(sim, KH_ERR_INVALID, "null output");
  kh_host::HistoryView h;
  kh_status st = sim->impl->history_view(id, &h);
  if (st != KH_OK) return st;
  if ((st = sim->impl->wait_idle()) != KH_OK) return st;
  if (step < 0 || step >= h.recorded) return fail(sim, KH_ERR_INVALID, "step not recorded");
  const size_t esz = h.dtype == KH_F32 ? 4 : 8;
  std::vector<unsigned char> buf(size_t(h.ncell) * esz);
  KH_ACUDA(sim, cudaMemcpy(buf.data(), static_cast<const unsigned char*>(h.buf) + size_t(step) * h.ncell * esz,
                           buf.size(), cudaMemcpyDeviceToHost));
  for (long long q = 0; q < h.ncell; ++q)
    out[q] = h.dtype == KH_F32 ? double(reinterpret_cast<const float*>(buf.data())[q])
                               : reinterpret_cast<const double*>(buf.data())[q];
  return KH_OK;
}

kh_status kh_sim_check_finite(kh_sim* sim) {
  if (!sim) return KH_ERR_INVALID;
  double n[6];
  kh_status st = kh_sim_field_sq_norms(sim, n);
  if (st != KH_OK) return st;
  static const char* names[6] = {"Ex", "Ey", "Ez", "Hx", "Hy", "Hz"};
  for (int c = 0; c < 6; ++c)
    if (!std::isfinite(n[c]))
      return fail(sim, KH_ERR_NAN, std::string("non-finite values in ") + names[c]);
  return KH_OK;
}

kh_status kh_sim_dft_norms(kh_sim* sim, double* out) {
  if (!sim) return KH_ERR_INVALID;
  if (!out) return fail(sim, KH_ERR_INVALID, "null output");
  std::vector<MonitorView> ms(size_t(sim->impl->monitor_count()));
  for (size_t id = 0; id < ms.size(); ++id) {
    const kh_status st = sim->impl->monitor_view(int(id), &ms[id]);
    if (st != KH_OK) return st;
  }
  if (ms.empty()) return KH_OK;
  kh_status st = sim->impl->wait_idle();
  if (st != KH_OK) return st;
  const long long chunk = 16LL * kRedThreads;
  std::vector<long long> nblk(ms.size());
  long long tot_blk = 0;
  for (size_t i = 0; i < ms.size(); ++i) {
    nblk[i] = std::max<long long>(1, (ms[i].ncell() * ms[i].nf + chunk - 1) / chunk);
    tot_blk += nblk[i];
  }
  DevBuf part, res;
  KH_ACUDA(sim, kh_host::dev_alloc(&part.p, size_t(tot_blk) * sizeof(double2), cudaStreamLegacy));
  KH_ACUDA(sim, kh_host::dev_alloc(&res.p, ms.size() * sizeof(double2), cudaStreamLegacy));
  long long off = 0;
  for (size_t i = 0; i < ms.size(); ++i) {
    const MonitorView& m = ms[i];
    double2* pp = static_cast<double2*>(part.p) + off;
    const long long total = m.ncell() * m.nf;
    if (m.dtype == KH_F32)
      dft_sq_partial_kernel<float><<<unsigned(nblk[i]), kRedThreads>>>(
          static_cast<const Cplx<float>*>(m.F), static_cast<const Cplx<float>*>(m.C), total, chunk, pp);
    else
      dft_sq_partial_kernel<double><<<unsigned(nblk[i]), kRedThreads>>>(
          static_cast<const Cplx<double>*>(m.F), static_cast<const Cplx<double>*>(m.C), total, chunk, pp);
    overlap_final_kernel<<<1, kRedThreads>>>(pp, int(nblk[i]), static_cast<double2*>(res.p) + i);
    off += nblk[i];
  }
  sim->impl->launches += 2 * int64_t(ms.size());
  KH_ACUDA(sim, cudaGetLastError());
  std::vector<double2> h(ms.size());
  KH_ACUDA(sim, cudaMemcpy(h.data(), res.p, h.size() * sizeof(double2), cudaMemcpyDeviceToHost));
  for (size_t i = 0; i < ms.size(); ++i) out[i] = std::sqrt(h[i].x);
  return KH_OK;
}

kh_status kh_sim_field_sq_norms(kh_sim* sim, double out[6]) {
  if (!sim) return KH_ERR_INVALID;
  if (!out) return fail(sim, KH_ERR_INVALID, "null output");
  const void* arrays[6];
  long long count = 0;
  kh_status st = sim->impl->field_arrays(arrays, &count);
  if (st != KH_OK) return st;
  if ((st = sim->impl->wait_idle()) != KH_OK) return st;
  return sim->impl->dtype() == KH_F32 ? sq_norms_impl<float>(sim, arrays, count, out)
                                      : sq_norms_impl<double>(sim, arrays, count, out);
}

kh_status kh_sim_dft_overlap(kh_sim* sim, int32_t monitor_id, const double* weights, double* out) {
  if (!sim) return KH_ERR_INVALID;
  if (!weights || !out) return fail(sim, KH_ERR_INVALID, "null overlap argument");
  MonitorView m;
  kh_status st = sim->impl->monitor_view(monitor_id, &m);
  if (st != KH_OK) return st;
  if ((st = sim->impl->wait_idle()) != KH_OK) return st;
  return m.dtype == KH_F32 ? overlap_impl<float>(sim, m, weights, out)
                           : overlap_impl<double>(sim, m, weights, out);
}

kh_status kh_adjoint_accumulate(kh_sim* fwd, const int32_t fwd_ids[3], int32_t fwd_freq, kh_sim* adj,
                                const int32_t adj_ids[3], int32_t adj_freq, double coef_re,
                                double coef_im, double* grad) {
  if (!fwd) return KH_ERR_INVALID;
  if (!adj || !fwd_ids || !adj_ids || !grad) return fail(fwd, KH_ERR_INVALID, "null adjoint argument");
  if (fwd->impl->dtype() != adj->impl->dtype())
    return fail(fwd, KH_ERR_INVALID, "forward and adjoint simulations differ in precision");
  MonitorView fv[3], av[3];
  for (int c = 0; c < 3; ++c) {
    kh_status st = fwd->impl->monitor_view(fwd_ids[c], &fv[c]);
    if (st != KH_OK) return st;
    if ((st = adj->impl->monitor_view(adj_ids[c], &av[c])) != KH_OK)
      return fail(fwd, st, "adjoint monitor: " + adj->impl->err);
    for (int a = 0; a < 3; ++a)
      if (fv[c].dims[a] != fv[0].dims[a] || av[c].dims[a] != fv[0].dims[a])
        return fail(fwd, KH_ERR_INVALID, "design monitors must cover the same cell box");
    if (fwd_freq < 0 || fwd_freq >= fv[c].nf || adj_freq < 0 || adj_freq >= av[c].nf)
      return fail(fwd, KH_ERR_INVALID, "frequency index outside a monitor's frequencies");
  }
  kh_status st = fwd->impl->wait_idle();
  if (st != KH_OK) return st;
  if ((st = adj->impl->wait_idle()) != KH_OK) return fail(fwd, st, "adjoint: " + adj->impl->err);
  return fwd->impl->dtype() == KH_F32
             ? gradient_impl<float>(fwd, fv, fwd_freq, av, adj_freq, coef_re, coef_im, grad)
             : gradient_impl<double>(fwd, fv, fwd_freq, av, adj_freq, coef_re, coef_im, grad);
}

}  // extern "C"
