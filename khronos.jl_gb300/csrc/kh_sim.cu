// Host side of the C ABI declared in include/khronos_gb300.h.
//
// A kh_sim owns one single-domain grid in device memory.  kh_sim_prepare
// classifies every cell once (CPML region flags, sources, χ3, poles), builds
// the sparse source table and allocates only the auxiliary arrays some cell
// uses.  kh_sim_step then issues, per step, the fused H kernel, the H-side DFT
// launches on decimation steps, the fused E kernel and the E-side DFT
// launches, mirroring step!(sim) (src/Kernels/Kernels.jl:20-88).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/khronos_gb300.h"
#include "kh_kernels.cuh"
#include "kh_simbase.h"

#include <cudaTypedefs.h>

using kh::Cplx;

namespace {

const char* kVersion = "khronos_gb300 1.0 (sm_103a)";
constexpr int kMaxDevices = 64;

// Device scratch of kh_sim_flux_static: the per-frequency flux sums of one
// call followed by the per-block partial sums of the reduction.  Fixed size
// (kFluxStaticMaxFreqs + kFluxStaticPartials doubles = 288 KB per device),
// shared by every simulation in the process on that device; it keeps the
// last call's values.  The flux kernels write every entry they read, so
// nothing has to start at zero.
constexpr int kFluxStaticMaxFreqs = 4096;
constexpr int kFluxStaticPartials = 8 * kFluxStaticMaxFreqs;
static __device__ __align__(256) double g_flux_static_scratch[kFluxStaticMaxFreqs + kFluxStaticPartials];
// Partial sums of kh_sim_flux per frequency (blocks per frequency at most).
constexpr int kFluxMaxBlocks = 64;

// Device address of g_flux_static_scratch, resolved once per device with that
// device current (the first kh_sim_flux_static call on the device).
kh_status flux_static_scratch(double** out, std::string& err) {
  static std::mutex mu;
  static double* addr[kMaxDevices] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    err = std::string("cudaGetDevice: ") + cudaGetErrorString(e);
    return KH_ERR_CUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    err = "device ordinal above the supported range";
    return KH_ERR_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_flux_static_scratch);
    if (e != cudaSuccess || !p) {
      err = std::string("cudaGetSymbolAddress(flux scratch): ") + cudaGetErrorString(e);
      return KH_ERR_CUDA;
    }
    addr[dev] = static_cast<double*>(p);
  }
  *out = addr[dev];
  return KH_OK;
}

using kh_host::SimBase;

}  // namespace

namespace kh_host {

std::atomic<int64_t> g_alloc_count{0};

cudaError_t dev_alloc(void** p, size_t bytes, cudaStream_t s) {
  ++g_alloc_count;
  static std::mutex mu;
  static cudaMemPool_t pools[kMaxDevices] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  cudaMemPool_t pool;
  {
    std::lock_guard<std::mutex> lock(mu);
    if (!pools[dev]) {
      cudaMemPoolProps props;
      std::memset(&props, 0, sizeof(props));
      props.allocType = cudaMemAllocationTypePinned;
      props.location.type = cudaMemLocationTypeDevice;
      props.location.id = dev;
      if ((e = cudaMemPoolCreate(&pools[dev], &props)) != cudaSuccess) return e;
      uint64_t keep = UINT64_MAX;  // keep freed memory in the pool
      if ((e = cudaMemPoolSetAttribute(pools[dev], cudaMemPoolAttrReleaseThreshold, &keep)) != cudaSuccess)
        return e;
    }
    pool = pools[dev];
  }
  return cudaMallocFromPoolAsync(p, bytes, pool, s);
}

cudaError_t dev_free(void* p, cudaStream_t s) { return p ? cudaFreeAsync(p, s) : cudaSuccess; }

namespace {
std::mutex g_pinned_mu;
std::multimap<size_t, void*> g_pinned_free;  // size -> buffer
}  // namespace

void* pinned_get(size_t bytes) {
  {
    std::lock_guard<std::mutex> lock(g_pinned_mu);
    auto it = g_pinned_free.lower_bound(bytes);
    if (it != g_pinned_free.end() && it->first <= 2 * bytes + 4096) {
      void* p = it->second;
      g_pinned_free.erase(it);
      return p;
    }
  }
  void* p = nullptr;
  if (cudaMallocHost(&p, bytes) != cudaSuccess) return nullptr;
  return p;
}

void pinned_put(void* p, size_t bytes) {
  if (!p) return;
  std::lock_guard<std::mutex> lock(g_pinned_mu);
  g_pinned_free.emplace(bytes, p);
}

}  // namespace kh_host

namespace {

#define KH_CUDA(call)                                                          \
  do {                                                                         \
    cudaError_t e_ = (call);                                                   \
    if (e_ != cudaSuccess) {                                                   \
      err = std::string(#call) + ": " + cudaGetErrorString(e_);                \
      return e_ == cudaErrorMemoryAllocation ? KH_ERR_OOM : KH_ERR_CUDA;       \
    }                                                                          \
  } while (0)

// Extra staggered layer per axis of Ex, Ey, Ez, Hx, Hy, Hz: component dims are
// n + kStagger[c] (src/utils.jl:26-37).
constexpr int kStagger[6][3] = {{0, 1, 1}, {1, 0, 1}, {1, 1, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};

template <typename T>
class Sim : public SimBase {
 public:
  static constexpr int VN = kh::Vec<T>::N;

  explicit Sim(const kh_sim_desc& desc) : d_(desc) {
    for (int a = 0; a < 3; ++a) n_[a] = desc.n[a];
    dt_ = T(desc.dt);
    for (int a = 0; a < 3; ++a) delta_[a] = T(desc.delta[a]);
    static_assert(kh::xoff<T>() >= VN && kh::xoff<T>() % VN == 0, "row offset keeps the vector alignment");
    const long long nxp = (n_[0] + VN - 1) / VN * VN;
    const long long align = 128 / sizeof(T);
    const long long xo = kh::xoff<T>();
    pitch_ = (xo + nxp + VN + align - 1) / align * align;
    plane_ = pitch_ * (n_[1] + 2);
    origin_ = plane_ + pitch_ + xo;
    total_ = plane_ * (n_[2] + 2);
    nxb_ = int((n_[0] + 32 * kh::kVN - 1) / (32 * kh::kVN));
    for (int a = 0; a < 3; ++a) {
      sigb_h_[a].assign(n_[a], T(0));
      sigd_h_[a].assign(n_[a], T(0));
      if (desc.sigma_b[a]) for (int i = 0; i < n_[a]; ++i) sigb_h_[a][i] = T(desc.sigma_b[a][i]);
      if (desc.sigma_d[a]) for (int i = 0; i < n_[a]; ++i) sigd_h_[a][i] = T(desc.sigma_d[a][i]);
    }
  }

  ~Sim() override {
    // wait for this simulation's own work only, then hand the memory back to
    // the pools (no device-wide synchronisation)
    if (batch_recorded_) cudaEventSynchronize(batch_done_);
    for (int b = 0; b < 2; ++b)
      if (copy_pending_[b]) cudaEventSynchronize(copy_ev_[b]);
    for (void* p : allocs_) kh_host::dev_free(p, cudaStreamLegacy);
    for (int b = 0; b < 2; ++b) {
      if (pinned_[b]) kh_host::pinned_put(pinned_[b], tab_cap_);
      if (copy_ev_[b]) cudaEventDestroy(copy_ev_[b]);
    }
    if (batch_done_) cudaEventDestroy(batch_done_);
    for (cudaEvent_t ev : events_) cudaEventDestroy(ev);
    for (auto& g : graphs_) cudaGraphExecDestroy(g.exec);
    if (ev_in_) cudaEventDestroy(ev_in_);
    if (ev_out_) cudaEventDestroy(ev_out_);
    if (gstream_) cudaStreamDestroy(gstream_);
  }

  // ---------------- set-up ----------------
  kh_status set_material(int kind, int comp, const double* v) override {
    if (prepared_) return fail(KH_ERR_INVALID, "set_material after prepare");
    if (!v) return fail(KH_ERR_INVALID, "null material array");
    std::vector<T>* dst = nullptr;
    if (kind == KH_MAT_CHI3) dst = &chi3_h_;
    else if (comp < 0 || comp > 2) return fail(KH_ERR_INVALID, "material component must be 0..2");
    else if (kind == KH_MAT_EPS_INV) dst = &eps_h_[comp];
    else if (kind == KH_MAT_MU_INV) dst = &mu_h_[comp];
    else if (kind == KH_MAT_SIGMA_D) dst = &msigd_h_[comp];
    else if (kind == KH_MAT_SIGMA_B) dst = &msigb_h_[comp];
    else return fail(KH_ERR_INVALID, "unknown material kind");
    const size_t cnt = size_t(n_[0]) * n_[1] * n_[2];
    dst->resize(cnt);
    for (size_t q = 0; q < cnt; ++q) (*dst)[q] = T(v[q]);
    if (kind == KH_MAT_EPS_INV) att_eps_[comp] = {};
    if (kind == KH_MAT_MU_INV) att_mu_[comp] = {};
    return KH_OK;
  }

  // kh_sim_attach_material: ε⁻¹ / μ⁻¹ stay in the caller's array until
  // prepare copies them straight to the device (converted there when the
  // precision differs); the other kinds are classified on the host and are
  // copied now.
  kh_status attach_material(int kind, int comp, const void* v, int dtype) override {
    if (prepared_) return fail(KH_ERR_INVALID, "attach_material after prepare");
    if (!v) return fail(KH_ERR_INVALID, "null material array");
    if (dtype != KH_F32 && dtype != KH_F64) return fail(KH_ERR_INVALID, "material dtype must be KH_F32 or KH_F64");
    if (kind != KH_MAT_CHI3 && (comp < 0 || comp > 2)) return fail(KH_ERR_INVALID, "material component must be 0..2");
    if (kind == KH_MAT_EPS_INV || kind == KH_MAT_MU_INV) {
      (kind == KH_MAT_EPS_INV ? att_eps_ : att_mu_)[comp] = {v, dtype};
      std::vector<T>& h = kind == KH_MAT_EPS_INV ? eps_h_[comp] : mu_h_[comp];
      std::vector<T>().swap(h);
      return KH_OK;
    }
    std::vector<T>* dst = nullptr;
    if (kind == KH_MAT_CHI3) dst = &chi3_h_;
    else if (kind == KH_MAT_SIGMA_D) dst = &msigd_h_[comp];
    else if (kind == KH_MAT_SIGMA_B) dst = &msigb_h_[comp];
    else return fail(KH_ERR_INVALID, "unknown material kind");
    const size_t cnt = size_t(n_[0]) * n_[1] * n_[2];
    dst->resize(cnt);
    if (dtype == KH_F32) {
      const float* f = static_cast<const float*>(v);
      for (size_t q = 0; q < cnt; ++q) (*dst)[q] = T(f[q]);
    } else {
      const double* f = static_cast<const double*>(v);
      for (size_t q = 0; q < cnt; ++q) (*dst)[q] = T(f[q]);
    }
    return KH_OK;
  }

  kh_status set_geometry(const kh_object* objs, int n, double background, const double* origin,
                         int smoothing) override {
    if (prepared_) return fail(KH_ERR_INVALID, "set_geometry after prepare");
    if (n < 0 || n > 65536 || (n > 0 && !objs) || !origin) return fail(KH_ERR_INVALID, "bad geometry arguments");
    if (smoothing < KH_SMOOTH_NONE || smoothing > KH_SMOOTH_ANISOTROPIC)
      return fail(KH_ERR_INVALID, "unknown smoothing mode");
    if (!(background > 0)) return fail(KH_ERR_INVALID, "background permittivity must be positive");
    if (has_eps(0) || has_eps(1) || has_eps(2))
      return fail(KH_ERR_INVALID, "per-voxel ε⁻¹ was already set with kh_sim_set_material");
    geo_.clear();
    for (int q = 0; q < n; ++q) {
      const kh_object& o = objs[q];
      kh::GeomObj g;
      g.shape = o.shape;
      g.axis = o.axis;
      for (int a = 0; a < 3; ++a) {
        g.c[a] = o.center[a];
        g.s[a] = o.size[a];
      }
      g.eps = o.eps;
      if (!(o.eps > 0)) return fail(KH_ERR_INVALID, "object permittivity must be positive");
      if (o.shape == KH_SHAPE_BALL) {
        for (int a = 0; a < 3; ++a) { g.lo[a] = o.center[a] - o.size[0]; g.hi[a] = o.center[a] + o.size[0]; }
      } else if (o.shape == KH_SHAPE_CUBOID) {
        for (int a = 0; a < 3; ++a) { g.lo[a] = o.center[a] - 0.5 * o.size[a]; g.hi[a] = o.center[a] + 0.5 * o.size[a]; }
      } else if (o.shape == KH_SHAPE_CYLINDER) {
        if (o.axis < 0 || o.axis > 2) return fail(KH_ERR_INVALID, "cylinder axis must be 0..2");
        for (int a = 0; a < 3; ++a) {
          const double e = a == o.axis ? 0.5 * o.size[1] : o.size[0];
          g.lo[a] = o.center[a] - e;
          g.hi[a] = o.center[a] + e;
        }
      } else {
        return fail(KH_ERR_INVALID, "unknown shape");
      }
      geo_.push_back(g);
    }
    geo_set_ = true;
    geo_bg_ = background;
    geo_smooth_ = smoothing;
    for (int a = 0; a < 3; ++a) geo_origin_[a] = origin[a];
    return KH_OK;
  }

  kh_status read_material(int kind, int comp, double* out) override {
    if (!prepared_) return fail(KH_ERR_INVALID, "read_material before prepare");
    if (!out || comp < 0 || comp > 2) return fail(KH_ERR_INVALID, "bad read_material arguments");
    const T* src = nullptr;
    if (kind == KH_MAT_EPS_INV) src = eps_[comp];
    else if (kind == KH_MAT_MU_INV) src = mu_[comp];
    else if (kind == KH_MAT_SIGMA_D) src = msigd_[comp];
    else if (kind == KH_MAT_SIGMA_B) src = msigb_[comp];
    else if (kind == KH_MAT_CHI3) src = chi3_;
    else return fail(KH_ERR_INVALID, "unknown material kind");
    if (!src) return fail(KH_ERR_INVALID, "no per-voxel array of this kind");
    std::vector<T> h(static_cast<size_t>(total_));
    if (kh_status es = wait_idle(); es != KH_OK) return es;
    KH_CUDA(cudaMemcpy(h.data(), src, total_ * sizeof(T), cudaMemcpyDeviceToHost));
    for (int k = 0; k < n_[2]; ++k)
      for (int j = 0; j < n_[1]; ++j)
        for (int i = 0; i < n_[0]; ++i)
          out[(size_t(k) * n_[1] + j) * n_[0] + i] = double(h[origin_ + (long long)k * plane_ + (long long)j * pitch_ + i]);
    return KH_OK;
  }

  kh_status add_pole(const kh_pole_coeffs& c, const double* s) override {
    if (prepared_) return fail(KH_ERR_INVALID, "add_pole after prepare");
    if (int(poles_.size()) >= kh::kMaxPoles) return fail(KH_ERR_UNSUPPORTED, "too many poles");
    if (!s) return fail(KH_ERR_INVALID, "null pole sigma");
    PoleH p;
    p.c = c;
    const size_t cnt = size_t(n_[0]) * n_[1] * n_[2];
    p.sigma.resize(cnt);
    for (size_t q = 0; q < cnt; ++q) p.sigma[q] = T(s[q]);
    poles_.push_back(std::move(p));
    return KH_OK;
  }

  kh_status add_source(const kh_source_desc& s) override {
    if (prepared_) return fail(KH_ERR_INVALID, "add_source after prepare");
    if (s.component < 0 || s.component > 5) return fail(KH_ERR_INVALID, "bad source component");
    if (s.dims[0] < 0 || s.dims[1] < 0 || s.dims[2] < 0) return fail(KH_ERR_INVALID, "bad source dims");
    if (s.time_kind < KH_TIME_GAUSSIAN || s.time_kind > KH_TIME_TABLE)
      return fail(KH_ERR_INVALID, "bad time profile");
    const size_t cnt = size_t(s.dims[0]) * s.dims[1] * s.dims[2];
    if (cnt && !s.amp) return fail(KH_ERR_INVALID, "null amplitude");
    SrcH h;
    h.d = s;
    h.d.amp = nullptr;
    h.d.table = nullptr;
    h.amp.resize(cnt);
    for (size_t q = 0; q < cnt; ++q) h.amp[q] = std::complex<double>(s.amp[2 * q], s.amp[2 * q + 1]);
    if (s.time_kind == KH_TIME_TABLE) {
      if (s.table_len < 0 || (s.table_len > 0 && !s.table)) return fail(KH_ERR_INVALID, "bad table");
      h.table.resize(size_t(2 * s.table_len));
      for (int64_t q = 0; q < 2 * s.table_len; ++q)
        h.table[q] = std::complex<T>(T(s.table[2 * q]), T(s.table[2 * q + 1]));
    }
    srcs_.push_back(std::move(h));
    return KH_OK;
  }

  kh_status add_monitor(int comp, const int32_t* st, const int32_t* dm, int nf, const double* f,
                        int dec, int32_t* id) override {
    if (prepared_) return fail(KH_ERR_INVALID, "add_dft_monitor after prepare");
    if (comp < 0 || comp > 5 || !st || !dm || nf <= 0 || !f || !id)
      return fail(KH_ERR_INVALID, "bad monitor arguments");
    Mon m;
    m.comp = comp;
    for (int a = 0; a < 3; ++a) {
      m.start[a] = st[a];
      m.dims[a] = dm[a];
      // the read box may reach the staggered wall layer (index n) but no further
      if (dm[a] <= 0 || st[a] < 0 || st[a] + dm[a] > n_[a] + 1)
        return fail(KH_ERR_INVALID, "monitor box outside the grid");
    }
    m.nf = nf;
    m.dec = dec < 1 ? 1 : dec;
    m.freqs.assign(f, f + nf);
    mons_.push_back(std::move(m));
    *id = int32_t(mons_.size() - 1);
    return KH_OK;
  }

  kh_status add_history(int comp, const int32_t* st, const int32_t* dm, int64_t cap,
                        int32_t* id) override {
    if (prepared_) return fail(KH_ERR_INVALID, "add_history_monitor after prepare");
    if (comp < 0 || comp > 5 || !st || !dm || !id || cap <= 0)
      return fail(KH_ERR_INVALID, "bad history monitor arguments");
    Hist h;
    h.comp = comp;
    for (int a = 0; a < 3; ++a) {
      h.start[a] = st[a];
      h.dims[a] = dm[a];
      if (dm[a] <= 0 || st[a] < 0 || st[a] + dm[a] > n_[a] + 1)
        return fail(KH_ERR_INVALID, "history box outside the grid");
    }
    h.cap = cap;
    h.ncell = (long long)dm[0] * dm[1] * dm[2];
    hists_.push_back(h);
    *id = int32_t(hists_.size() - 1);
    return KH_OK;
  }

  kh_status history_view(int id, kh_host::HistoryView* out) override {
    if (!prepared_) return fail(KH_ERR_INVALID, "history read before prepare");
    if (id < 0 || id >= int(hists_.size()) || !out) return fail(KH_ERR_INVALID, "bad history monitor id");
    const Hist& h = hists_[id];
    out->buf = h.buf;
    for (int a = 0; a < 3; ++a) out->dims[a] = h.dims[a];
    out->ncell = h.ncell;
    out->capacity = h.cap;
    out->recorded = std::min<int64_t>(timestep_, h.cap);
    out->dtype = sizeof(T) == 4 ? KH_F32 : KH_F64;
    return KH_OK;
  }

  kh_status prepare() override {
    if (prepared_) return KH_OK;
    for (int a = 0; a < 3; ++a) {
      if (d_.pml_lo[a] < 0 || d_.pml_hi[a] < 0 || d_.pml_lo[a] + d_.pml_hi[a] > n_[a])
        if (!(d_.pml_lo[a] == n_[a] && d_.pml_hi[a] == 0))
          return fail(KH_ERR_INVALID, "PML widths exceed the axis");
      lo_[a] = d_.pml_lo[a];
      hi_[a] = d_.pml_hi[a];
      pml_axis_[a] = lo_[a] > 0 || hi_[a] > 0;
    }
    const bool any_pml = pml_axis_[0] || pml_axis_[1] || pml_axis_[2];

    if (d_.semantics != KH_SEM_REFERENCE_CPU && d_.semantics != KH_SEM_CPML)
      return fail(KH_ERR_INVALID, "unknown CPML semantics");
    if (d_.periodic & ~7)
      return fail(KH_ERR_INVALID, "periodic is a mask of axes 0..2");
    // Regions with material conductivity (PhysicsFlags.has_sigma_{B,D}).
    sigmask_b_ = region_mask(msigb_h_);
    sigmask_d_ = region_mask(msigd_h_);
    const bool any_msig = !msigb_h_[0].empty() || !msigb_h_[1].empty() || !msigb_h_[2].empty() ||
                          !msigd_h_[0].empty() || !msigd_h_[1].empty() || !msigd_h_[2].empty();
    if (d_.semantics == KH_SEM_CPML && any_msig && any_pml)
      return fail(KH_ERR_UNSUPPORTED,
                  "the CUDA-path CPML kernels take no material conductivity (CUDAKernels.jl:122-124)");
    // The reference's generic_curl! has no method for C without U, or for a
    // conductivity array with U but no C (Helpers.jl:39-270): reject.
    for (int r = 0; r < 27; ++r) {
      const int rr[3] = {r % 3, (r / 3) % 3, r / 9};
      if (!region_nonempty(rr)) continue;
      bool f[3];
      for (int a = 0; a < 3; ++a) f[a] = rr[a] != 1;
      if (!(f[0] || f[1] || f[2])) continue;
      for (int c = 0; c < 3; ++c) {
        const int nx = (c + 1) % 3, pv = (c + 2) % 3;
        for (int h = 0; h < 2; ++h) {
          const uint32_t mask = h ? sigmask_b_ : sigmask_d_;
          const bool arr = h ? !msigb_h_[c].empty() : !msigd_h_[c].empty();
          const bool hasC = ((mask >> r) & 1u) && (f[nx] || f[pv]);
          const bool hasU = f[nx];
          if ((hasC && !hasU) || (!hasC && hasU && arr))
            return fail(KH_ERR_UNSUPPORTED,
                        "material conductivity in this CPML region has no generic_curl! method "
                        "in the reference (Helpers.jl:39-270)");
        }
      }
    }

    kh_status st = KH_OK;
#define KH_TRY(x)            \
  do {                       \
    st = (x);                \
    if (st != KH_OK) return st; \
  } while (0)
    for (int c = 0; c < 3; ++c) {
      KH_TRY(alloc_field(&E_[c]));
      KH_TRY(alloc_field(&H_[c]));
    }
    // materials: compact uploads scattered into the padded layout on the device,
    // queued before the host builds the source table so the copies overlap it
    if (geo_set_) KH_TRY(build_geometry());
    const int tdt = sizeof(T) == 4 ? KH_F32 : KH_F64;
    for (int c = 0; c < 3; ++c) {
      if (att_eps_[c].ptr) KH_TRY(upload_center(att_eps_[c].ptr, att_eps_[c].dtype, &eps_[c]));
      else if (!eps_h_[c].empty()) KH_TRY(upload_center(eps_h_[c].data(), tdt, &eps_[c]));
      if (att_mu_[c].ptr) KH_TRY(upload_center(att_mu_[c].ptr, att_mu_[c].dtype, &mu_[c]));
      else if (!mu_h_[c].empty()) KH_TRY(upload_center(mu_h_[c].data(), tdt, &mu_[c]));
      if (!msigd_h_[c].empty()) KH_TRY(upload_center(msigd_h_[c].data(), tdt, &msigd_[c]));
      if (!msigb_h_[c].empty()) KH_TRY(upload_center(msigb_h_[c].data(), tdt, &msigb_[c]));
    }
    if ((eps_[0] != nullptr) != (eps_[2] != nullptr) || (eps_[0] != nullptr) != (eps_[1] != nullptr))
      return fail(KH_ERR_INVALID, "per-voxel ε⁻¹ must be given for all three components");
    if ((mu_[0] != nullptr) != (mu_[2] != nullptr) || (mu_[0] != nullptr) != (mu_[1] != nullptr))
      return fail(KH_ERR_INVALID, "per-voxel μ⁻¹ must be given for all three components");
    if (!chi3_h_.empty()) KH_TRY(upload_center(chi3_h_.data(), tdt, &chi3_));
    std::vector<T*> pole_sigma(poles_.size(), nullptr);
    for (size_t q = 0; q < poles_.size(); ++q) KH_TRY(upload_center(poles_[q].sigma.data(), tdt, &pole_sigma[q]));
    auto cidx = [&](int i, int j, int k) { return origin_ + (long long)k * plane_ + (long long)j * pitch_ + i; };
    auto center = [&](int i, int j, int k) { return (size_t(k) * n_[1] + j) * n_[0] + i; };
    // Sparse source table: entries per cell in injection order
    // (components Ex..Hz, then sources in order; Kernels.jl:455-463, Sources.jl:330-340).
    struct Ent { long long cell; int src, comp; std::complex<double> amp; int i, j, k; long long q; };
    std::vector<Ent> ents;
    {
      size_t cap = 0;
      for (const SrcH& s : srcs_) cap += size_t(s.d.dims[0]) * s.d.dims[1] * s.d.dims[2];
      ents.reserve(cap);
    }
    for (int comp = 0; comp < 6; ++comp)
      for (size_t si = 0; si < srcs_.size(); ++si) {
        const SrcH& s = srcs_[si];
        if (s.d.component != comp) continue;
        for (int k = 0; k < s.d.dims[2]; ++k)
          for (int j = 0; j < s.d.dims[1]; ++j)
            for (int i = 0; i < s.d.dims[0]; ++i) {
              const int gi = s.d.start[0] + i, gj = s.d.start[1] + j, gk = s.d.start[2] + k;
              // cells outside the updated range are never consumed by the reference
              if (gi < 0 || gj < 0 || gk < 0 || gi >= n_[0] || gj >= n_[1] || gk >= n_[2]) continue;
              const long long q = ((long long)k * s.d.dims[1] + j) * s.d.dims[0] + i;
              const std::complex<double> a = s.amp[size_t(q)];
              const std::complex<T> aT(T(a.real()), T(a.imag()));
              if (aT.real() == T(0) && aT.imag() == T(0)) continue;
              ents.push_back({cidx(gi, gj, gk), int(si), comp, std::complex<double>(aT.real(), aT.imag()), gi, gj, gk, q});
            }
      }
    // one source, or sources on disjoint increasing boxes, come out sorted already
    auto by_cell = [](const Ent& a, const Ent& b) { return a.cell < b.cell; };
    if (!std::is_sorted(ents.begin(), ents.end(), by_cell)) std::stable_sort(ents.begin(), ents.end(), by_cell);
    // Special cells keep their B|D state: E sources, χ3 and poles (E half), H
    // sources (H half).  An all-zero χ3 or pole array counts as present.
    bool anySpecialE = !chi3_h_.empty() || !poles_.empty(), anySpecialH = false;
    src_ent_.assign(srcs_.size(), {});
    std::vector<int> slot_off(1, 0), ent_src, ent_comp;
    std::vector<long long> slot_cell;
    std::vector<uint32_t> slot_bits;
    std::vector<Cplx<T>> ent_amp;
    slot_off.reserve(ents.size() + 1);
    ent_src.reserve(ents.size());
    ent_comp.reserve(ents.size());
    ent_amp.reserve(ents.size());
    slot_cell.reserve(ents.size());
    slot_bits.reserve(ents.size());
    for (size_t e = 0; e < ents.size();) {
      size_t e2 = e;
      const int slot = int(slot_off.size() - 1);
      if (slot >= (1 << 24)) return fail(KH_ERR_UNSUPPORTED, "too many source cells");
      uint32_t bits = uint32_t(slot) << kh::kSlotShift;
      while (e2 < ents.size() && ents[e2].cell == ents[e].cell) {
        src_ent_[ents[e2].src].push_back({ents[e2].q, int(ent_src.size())});
        ent_src.push_back(ents[e2].src);
        ent_comp.push_back(ents[e2].comp);
        ent_amp.push_back({T(ents[e2].amp.real()), T(ents[e2].amp.imag())});
        if (ents[e2].comp < 3) { bits |= kh::kSpecialE | kh::kHasSrcE; anySpecialE = true; }
        else { bits |= kh::kSpecialH | kh::kHasSrcH; anySpecialH = true; }
        ++e2;
      }
      slot_off.push_back(int(ent_src.size()));
      slot_cell.push_back(ents[e].cell);
      slot_bits.push_back(bits);
      e = e2;
    }
    // Which cells the LEAN kernels can take (see run_batch): a source cell's
    // term can be added after the kernel when its component has no W stage
    // there and the cell carries no χ3 or pole; CPU-path semantics keep B|D
    // for every component of a special cell inside CPML, which LEAN does not.
    auto flag = [&](int a, int idx) { return idx < lo_[a] || idx >= n_[a] - hi_[a]; };
    has_src_[0] = has_src_[1] = false;
    src_lean_ok_[0] = src_lean_ok_[1] = true;
    src_on_dispersive_ = false;
    for (const Ent& e : ents) {
      const int half = e.comp >= 3 ? 1 : 0;
      has_src_[half] = true;
      const int own = e.comp % 3;
      // own-axis CPML: a W stage, which the source kernel applies for the
      // CUDA-path stages; the CPU-path dispatch keeps such cells FULL
      const bool fown = flag(own, own == 0 ? e.i : (own == 1 ? e.j : e.k));
      if (fown && d_.semantics == KH_SEM_REFERENCE_CPU) src_lean_ok_[half] = false;
      if (!half) {
        const size_t ci = center(e.i, e.j, e.k);
        bool dispersive = !chi3_h_.empty() && chi3_h_[ci] != T(0);
        for (auto& p : poles_) dispersive = dispersive || p.sigma[ci] != T(0);
        if (dispersive) src_on_dispersive_ = true;
      }
    }

    // state arrays that some cell needs
    const bool msb = !msigb_h_[0].empty() || !msigb_h_[1].empty() || !msigb_h_[2].empty();
    const bool msd = !msigd_h_[0].empty() || !msigd_h_[1].empty() || !msigd_h_[2].empty();
    for (int c = 0; c < 3; ++c) {
      const int nx = (c + 1) % 3, pv = (c + 2) % 3;
      if (any_pml || anySpecialH) KH_TRY(alloc_field(&B_[c]));
      if (any_pml || anySpecialE) KH_TRY(alloc_field(&D_[c]));
      if (pml_axis_[nx]) { KH_TRY(alloc_field(&UB_[c])); KH_TRY(alloc_field(&UD_[c])); }
      if (pml_axis_[c]) { KH_TRY(alloc_field(&WB_[c])); KH_TRY(alloc_field(&WD_[c])); }
      if (msb && sigmask_b_ && (pml_axis_[nx] || pml_axis_[pv])) KH_TRY(alloc_field(&CB_[c]));
      if (msd && sigmask_d_ && (pml_axis_[nx] || pml_axis_[pv])) KH_TRY(alloc_field(&CD_[c]));
    }
    for (size_t q = 0; q < poles_.size(); ++q) {
      PoleD pd;
      pd.sigma = pole_sigma[q];
      for (int c = 0; c < 3; ++c) {
        KH_TRY(alloc_field(&pd.P[c]));
        KH_TRY(alloc_field(&pd.Pp[c]));
      }
      pd.c = poles_[q].c;
      poles_d_.push_back(pd);
    }
    // The small tables (CPML coefficients, the source table) go up in one
    // asynchronous copy from a pinned staging buffer into one device block,
    // released after the synchronisation at the end of prepare.
    std::vector<char> stg;
    std::vector<std::pair<void**, size_t>> stg_out;
    auto stage = [&](const void* h, size_t bytes, void** out) {
      const size_t off = (stg.size() + 255) & ~size_t(255);
      stg.resize(off + bytes);
      std::memcpy(stg.data() + off, h, bytes);
      stg_out.push_back({out, off});
    };
    for (int a = 0; a < 3; ++a) {
      // CPML coefficient tables (σ, 1-σ, 1/(1+σ), 1+σ) in the run's precision
      for (int h = 0; h < 2; ++h) {
        const std::vector<T>& sg = h ? sigb_h_[a] : sigd_h_[a];
        std::vector<kh::AxisCoef<T>> tab(sg.size());
        for (size_t i = 0; i < sg.size(); ++i) {
          const T sv = sg[i];
          tab[i] = {sv, T(1) - sv, T(1) / (T(1) + sv), T(1) + sv};
        }
        stage(tab.data(), tab.size() * sizeof(kh::AxisCoef<T>), (void**)(h ? &axb_[a] : &axd_[a]));
      }
    }
    nsrc_ = int(srcs_.size());
    if (!ent_src.empty()) {
      stage(slot_off.data(), slot_off.size() * sizeof(int), (void**)&slot_off_);
      stage(ent_src.data(), ent_src.size() * sizeof(int), (void**)&ent_src_);
      stage(ent_comp.data(), ent_comp.size() * sizeof(int), (void**)&ent_comp_);
      stage(ent_amp.data(), ent_amp.size() * sizeof(Cplx<T>), (void**)&ent_amp_);
      ent_amp_h_ = ent_amp;
      stage(slot_cell.data(), slot_cell.size() * sizeof(long long), (void**)&slot_cell_);
      nslots_ = int(slot_cell.size());
      slot_off_h_ = slot_off;
      ent_src_h_ = ent_src;
      ent_comp_h_ = ent_comp;
      std::vector<kh::SlotPack<T>> pack = pack_slots();
      stage(pack.data(), pack.size() * sizeof(kh::SlotPack<T>), (void**)&slot_pack_);
    }
    void* stg_pinned = nullptr;
    if (!stg.empty()) {
      void* dev = nullptr;
      KH_CUDA(kh_host::dev_alloc(&dev, stg.size(), cudaStreamLegacy));
      allocs_.push_back(dev);
      device_bytes_ += int64_t(stg.size());
      stg_pinned = kh_host::pinned_get(stg.size());
      cudaError_t e = stg_pinned ? cudaSuccess : cudaErrorMemoryAllocation;
      if (e == cudaSuccess) {
        std::memcpy(stg_pinned, stg.data(), stg.size());
        e = cudaMemcpyAsync(dev, stg_pinned, stg.size(), cudaMemcpyHostToDevice, cudaStreamLegacy);
      }
      if (e != cudaSuccess) {
        if (stg_pinned) {
          cudaStreamSynchronize(cudaStreamLegacy);
          kh_host::pinned_put(stg_pinned, stg.size());
        }
        return fail(KH_ERR_CUDA, std::string("table upload: ") + cudaGetErrorString(e));
      }
      for (auto& o : stg_out) *o.first = static_cast<char*>(dev) + o.second;
    }
    // the staging buffer goes back to the pool once the copies queued so far
    // have run (every exit from here on synchronises the legacy stream first)
    struct StgRelease {
      void* p;
      size_t n;
      ~StgRelease() {
        if (p) {
          cudaStreamSynchronize(cudaStreamLegacy);
          kh_host::pinned_put(p, n);
        }
      }
    } stg_release{stg_pinned, stg.size()};
    // Cell classes and the per-row-segment plane bitmasks (word (k/64, j, xb),
    // bit k%64), computed on the device from the material arrays and the
    // source table.
    unsigned int* region_flags = nullptr;
    if (anySpecialE || anySpecialH) {
      KH_TRY(alloc_raw(size_t(total_) * sizeof(uint32_t), (void**)&cls_, false));
      kh::ClassifyArgs<T> ca;
      std::memset(&ca, 0, sizeof(ca));
      for (int a = 0; a < 3; ++a) ca.n[a] = n_[a];
      ca.pitch = pitch_;
      ca.plane = plane_;
      ca.origin = origin_;
      ca.chi3 = chi3_;
      ca.npoles = int(poles_d_.size());
      for (size_t q = 0; q < poles_d_.size(); ++q) ca.pole_sigma[q] = poles_d_[q].sigma;
      ca.cls = cls_;
      if (ca.chi3 || ca.npoles) {
        kh::launch_classify<T>(ca, cudaStreamLegacy);
        ++launches;
      }
      if (nslots_ > 0) {
        uint32_t* dbits = nullptr;
        KH_CUDA(kh_host::dev_alloc((void**)&dbits, slot_bits.size() * sizeof(uint32_t), cudaStreamLegacy));
        cudaError_t e = cudaMemcpyAsync(dbits, slot_bits.data(), slot_bits.size() * sizeof(uint32_t),
                                        cudaMemcpyHostToDevice, cudaStreamLegacy);
        if (e == cudaSuccess) {
          kh::launch_mark_cells(slot_cell_, dbits, nslots_, cls_, cudaStreamLegacy);
          ++launches;
        }
        // the host vector stays alive until the synchronisation at the end of prepare
        kh_host::dev_free(dbits, cudaStreamLegacy);
        if (e != cudaSuccess) return fail(KH_ERR_CUDA, cudaGetErrorString(e));
      }
      const size_t nwords = size_t((n_[2] + 63) / 64) * n_[1] * nxb_;
      KH_TRY(alloc_raw(nwords * sizeof(uint64_t), (void**)&tbits_e_, false));
      KH_TRY(alloc_raw(nwords * sizeof(uint64_t), (void**)&tbits_h_, false));
      KH_TRY(alloc_raw(sizeof(unsigned int), (void**)&region_flags, false));
      kh::TileBitsArgs ta;
      for (int a = 0; a < 3; ++a) {
        ta.n[a] = n_[a];
        ta.lo[a] = lo_[a];
        ta.hi[a] = hi_[a];
      }
      ta.pitch = pitch_;
      ta.plane = plane_;
      ta.origin = origin_;
      ta.nxb = nxb_;
      ta.cls = cls_;
      ta.bits_e = reinterpret_cast<unsigned long long*>(tbits_e_);
      ta.bits_h = reinterpret_cast<unsigned long long*>(tbits_h_);
      ta.region_flags = region_flags;
      kh::launch_tile_bits(ta, cudaStreamLegacy);
      ++launches;
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) return fail(KH_ERR_CUDA, std::string("classification kernels: ") + cudaGetErrorString(e));
    }
    // monitors
    for (auto& m : mons_) {
      m.ncell = (long long)m.dims[0] * m.dims[1] * m.dims[2];
      const size_t bytes = size_t(m.ncell) * m.nf * sizeof(Cplx<T>);
      KH_TRY(alloc_raw(bytes, (void**)&m.F, true));
      if (sizeof(T) == 4) KH_TRY(alloc_raw(bytes, (void**)&m.C, true));
    }
    for (auto& h : hists_)
      KH_TRY(alloc_raw(size_t(h.ncell) * size_t(h.cap) * sizeof(T), (void**)&h.buf, false));
    // Step alignment: lcm of the monitors' decimations (1 if above a batch).
    {
      long long l = 1;
      for (auto& m : mons_)
        if (m.dec > 1) {
          long long a = l, b2 = m.dec;
          while (b2) { const long long t2 = a % b2; a = b2; b2 = t2; }
          l = l / a * m.dec;
          if (l > kBatch) break;
        }
      align_ = l > kBatch ? 1 : int(l);
      batch_len_ = (kBatch / align_) * align_;
    }
    // last_source_time (TimeSources.jl:40-47); a CW source never cuts off.
    has_cw_ = false;
    last_time_ = -INFINITY;
    for (auto& s : srcs_) {
      if (s.d.time_kind == KH_TIME_CW) has_cw_ = true;
      else last_time_ = std::max(last_time_, double(T(s.d.cutoff)));
    }
    // Per-batch time-factor/phase tables: two device buffers and two pinned
    // staging buffers (batch b uses buffer b % 2), sized for the largest batch
    // so stepping never allocates.
    tab_cap_ = table_capacity() * sizeof(Cplx<T>);
    for (int b = 0; b < 2; ++b) {
      KH_TRY(alloc_raw(tab_cap_, &tab_dev_[b], false));
      pinned_[b] = kh_host::pinned_get(tab_cap_);
      if (!pinned_[b]) return fail(KH_ERR_OOM, "pinned staging buffer");
      KH_CUDA(cudaEventCreateWithFlags(&copy_ev_[b], cudaEventDisableTiming));
    }
    KH_CUDA(cudaEventCreateWithFlags(&batch_done_, cudaEventDisableTiming));
    // Step graphs (KHRONOS_GB300_GRAPHS=0 turns them off)
    const char* gv = std::getenv("KHRONOS_GB300_GRAPHS");
    graphs_on_ = !(gv && std::string(gv) == "0");
    if (graphs_on_) {
      KH_CUDA(cudaStreamCreateWithFlags(&gstream_, cudaStreamNonBlocking));
      KH_CUDA(cudaEventCreateWithFlags(&ev_in_, cudaEventDisableTiming));
      KH_CUDA(cudaEventCreateWithFlags(&ev_out_, cudaEventDisableTiming));
    }
    KH_TRY(alloc_raw(sizeof(int), (void**)&err_dev_, false));
    // Half-step kernel: TMA-staged unless KHRONOS_GB300_KERNEL=simt selects the
    // register-pipelined one.
    const char* kv = std::getenv("KHRONOS_GB300_KERNEL");
    use_tma_ = !(kv && std::string(kv) == "simt");
    const char* bv = std::getenv("KHRONOS_GB300_DFT_BATCH");
    dft_batch_ = !(bv && std::string(bv) == "0");
    if (use_tma_) KH_TRY(build_tma_maps());
    zplanes_ = choose_zplanes();
    if (const char* xv = std::getenv("KHRONOS_GB300_XPREFETCH")) xprefetch_ = std::min(2, std::max(0, std::atoi(xv)));
    if (const char* dv = std::getenv("KHRONOS_GB300_XPF_DIST")) xpf_dist_ = std::min(8, std::max(1, std::atoi(dv)));
    if (const char* sv = std::getenv("KHRONOS_GB300_TEST_STALL")) stall_tx_ = std::string(sv) == "1" ? 16u : 0u;
    // the zeroing and uploads above ran on the legacy default stream; wait for
    // them only (work of other simulations on non-blocking streams goes on)
    KH_CUDA(cudaStreamSynchronize(cudaStreamLegacy));
    special_in_region_[0] = special_in_region_[1] = false;
    if (region_flags) {
      unsigned int rf = 0;
      KH_CUDA(cudaMemcpy(&rf, region_flags, sizeof(rf), cudaMemcpyDeviceToHost));
      special_in_region_[0] = (rf & 1u) != 0;
      special_in_region_[1] = (rf & 2u) != 0;
    }
    // χ3 and pole cells updated by the LEAN E launch plus the dispersive-cell
    // pass, unless something else needs the FULL launch anyway (material
    // conductivity, the CPU-path semantics with special cells in CPML, or a
    // periodic axis, whose wrap must see E before the Kerr correction).
    // KHRONOS_GB300_DISP_FIX=0 keeps them in the FULL launch.
    {
      const char* dv = std::getenv("KHRONOS_GB300_DISP_FIX");
      const bool dispersive = chi3_ != nullptr || !poles_d_.empty();
      const bool msd_any = msigd_[0] || msigd_[1] || msigd_[2];
      disp_fix_ = dispersive && !(dv && std::string(dv) == "0") && !msd_any && d_.periodic == 0 &&
                  !(d_.semantics == KH_SEM_REFERENCE_CPU && special_in_region_[0]) && cls_ != nullptr;
      const long long nseg = (long long)n_[2] * n_[1] * nxb_;
      if (disp_fix_ && nseg >= (1LL << 31)) disp_fix_ = false;  // list entries carry 31-bit indices
      if (disp_fix_) {
        // the row segments holding χ3 or pole cells, in grid order
        unsigned char* flags = nullptr;
        KH_CUDA(kh_host::dev_alloc((void**)&flags, size_t(nseg), cudaStreamLegacy));
        int* cnt = nullptr;
        KH_TRY(alloc_raw(size_t(nseg) * sizeof(uint32_t), (void**)&disp_list_, false));
        KH_TRY(alloc_raw(sizeof(int), (void**)&cnt, false));
        kh::DispListArgs la;
        for (int a = 0; a < 3; ++a) la.n[a] = n_[a];
        la.pitch = pitch_;
        la.plane = plane_;
        la.origin = origin_;
        la.nxb = nxb_;
        la.cls = cls_;
        la.flags = flags;
        la.list = disp_list_;
        la.count = cnt;
        kh::launch_disp_list(la, cudaStreamLegacy);
        cudaError_t e = cudaGetLastError();
        int count = 0;
        if (e == cudaSuccess) e = cudaMemcpy(&count, cnt, sizeof(int), cudaMemcpyDeviceToHost);
        kh_host::dev_free(flags, cudaStreamLegacy);
        if (e != cudaSuccess) return fail(KH_ERR_CUDA, std::string("segment list: ") + cudaGetErrorString(e));
        n_disp_list_ = count;
      }
      // a source on a χ3 or pole cell: LEAN with the dispersive-cell pass,
      // else the FULL launch while sources are active
      if (src_on_dispersive_ && !disp_fix_) src_lean_ok_[0] = false;
    }
    prepared_ = true;
    return KH_OK;
#undef KH_TRY
  }

  // ---------------- stepping ----------------
  kh_status step(int64_t nsteps, cudaStream_t stream) override {
    if (!prepared_) return fail(KH_ERR_INVALID, "step before prepare");
    if (nsteps < 0) return fail(KH_ERR_INVALID, "negative step count");
    // Batches end on multiples of batch_len_ (a multiple of every monitor's
    // decimation), so steady-state batches repeat their launch sequence and
    // replay one captured graph.
    int64_t done = 0;
    while (done < nsteps) {
      const int64_t to_edge = batch_len_ - timestep_ % batch_len_;
      const int nb = int(std::min<int64_t>(to_edge, nsteps - done));
      kh_status st = run_batch(nb, stream);
      if (st != KH_OK) return st;
      done += nb;
    }
    return KH_OK;
  }

  int step_alignment() const override { return align_; }
  int64_t graph_replays() const override { return graph_replays_; }

  int64_t timestep() const override { return timestep_; }
  int sources_active() const override { return sources_active_ ? 1 : 0; }
  bool is_prepared() const override { return prepared_; }
  int64_t cells() const override { return int64_t(n_[0]) * n_[1] * n_[2]; }
  int64_t device_bytes() const override { return device_bytes_; }

  kh_status wait_idle() override {
    if (batch_recorded_) KH_CUDA(cudaEventSynchronize(batch_done_));
    return check_device_error();
  }

  // The allocations prepare() makes, from the same decisions (an upper bound
  // where a decision depends on cell classification).
  int64_t estimate_bytes() const override {
    const int64_t field = total_ * int64_t(sizeof(T));
    bool any_pml = false, pml[3];
    for (int a = 0; a < 3; ++a) {
      pml[a] = d_.pml_lo[a] > 0 || d_.pml_hi[a] > 0;
      any_pml |= pml[a];
    }
    bool src_e = false, src_h = false;
    int64_t src_cells = 0;
    for (auto& sr : srcs_) {
      (sr.d.component < 3 ? src_e : src_h) = true;
      src_cells += int64_t(sr.d.dims[0]) * sr.d.dims[1] * sr.d.dims[2];
    }
    const bool spec_e = src_e || !chi3_h_.empty() || !poles_.empty();
    const bool msb = !msigb_h_[0].empty() || !msigb_h_[1].empty() || !msigb_h_[2].empty();
    const bool msd = !msigd_h_[0].empty() || !msigd_h_[1].empty() || !msigd_h_[2].empty();
    int64_t b = 6 * field;
    for (int c = 0; c < 3; ++c) {
      const int nx = (c + 1) % 3, pv = (c + 2) % 3;
      if (any_pml || src_h) b += field;
      if (any_pml || spec_e) b += field;
      if (pml[nx]) b += 2 * field;
      if (pml[c]) b += 2 * field;
      if (msb && (pml[nx] || pml[pv])) b += field;
      if (msd && (pml[nx] || pml[pv])) b += field;
      if (has_eps(c) || geo_set_) b += field;
      if (has_mu(c)) b += field;
      if (!msigd_h_[c].empty()) b += field;
      if (!msigb_h_[c].empty()) b += field;
    }
    if (!chi3_h_.empty()) b += field;
    b += int64_t(poles_.size()) * 7 * field;
    for (int a = 0; a < 3; ++a) b += 2 * int64_t(n_[a]) * int64_t(sizeof(kh::AxisCoef<T>));
    if (spec_e || src_h) {
      b += total_ * 4;
      b += 2 * int64_t((n_[2] + 63) / 64) * n_[1] * nxb_ * 8;
    }
    b += src_cells * int64_t(4 + 4 + sizeof(Cplx<T>) + 8) + 4 * (src_cells + 1);
    for (auto& m : mons_) {
      const int64_t cnt = int64_t(m.dims[0]) * m.dims[1] * m.dims[2] * m.nf * int64_t(sizeof(Cplx<T>));
      b += cnt * (sizeof(T) == 4 ? 2 : 1);
    }
    b += 2 * int64_t(table_capacity() * sizeof(Cplx<T>)) + int64_t(sizeof(int));
    for (auto& h : hists_) b += h.ncell * h.cap * int64_t(sizeof(T));
    return b;
  }

  // ---------------- results ----------------
  kh_status get_field(int comp, double* out) override {
    if (!prepared_) return fail(KH_ERR_INVALID, "get_field before prepare");
    if (comp < 0 || comp > 5 || !out) return fail(KH_ERR_INVALID, "bad get_field arguments");
    std::vector<T> h(static_cast<size_t>(total_));
    if (kh_status es = wait_idle(); es != KH_OK) return es;
    KH_CUDA(cudaMemcpy(h.data(), comp < 3 ? E_[comp] : H_[comp - 3], total_ * sizeof(T),
                       cudaMemcpyDeviceToHost));
    const int cd[3] = {n_[0] + kStagger[comp][0], n_[1] + kStagger[comp][1], n_[2] + kStagger[comp][2]};
    for (int k = 0; k < cd[2]; ++k)
      for (int j = 0; j < cd[1]; ++j)
        for (int i = 0; i < cd[0]; ++i)
          out[(size_t(k) * cd[1] + j) * cd[0] + i] =
              double(h[origin_ + (long long)k * plane_ + (long long)j * pitch_ + i]);
    return KH_OK;
  }

  kh_status read_dft(int id, double* out) override {
    if (id < 0 || id >= int(mons_.size()) || !out) return fail(KH_ERR_INVALID, "bad monitor id");
    if (!prepared_) return fail(KH_ERR_INVALID, "read_dft before prepare");
    const Mon& m = mons_[id];
    const size_t cnt = size_t(m.ncell) * m.nf;
    if (kh_status es = wait_idle(); es != KH_OK) return es;
    // F − C in FP64 on the device, then one copy into the caller's array
    double* dout = nullptr;
    KH_CUDA(kh_host::dev_alloc((void**)&dout, cnt * 2 * sizeof(double), cudaStreamLegacy));
    kh::launch_dft_read<T>(m.F, m.C, dout, (long long)cnt, cudaStreamLegacy);
    ++launches;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(out, dout, cnt * 2 * sizeof(double), cudaMemcpyDeviceToHost);
    kh_host::dev_free(dout, cudaStreamLegacy);
    if (e != cudaSuccess) return fail(KH_ERR_CUDA, std::string("read_dft: ") + cudaGetErrorString(e));
    return KH_OK;
  }

  kh_status monitor_info(int id, int32_t* dims, int32_t* nf) const override {
    if (id < 0 || id >= int(mons_.size())) return KH_ERR_INVALID;
    for (int a = 0; a < 3; ++a) dims[a] = mons_[id].dims[a];
    *nf = mons_[id].nf;
    return KH_OK;
  }

  kh_status flux(const int32_t* ids, int normal, double dA, double* out) override {
    if (!prepared_) return fail(KH_ERR_INVALID, "flux before prepare");
    if (!ids || !out || normal < 0 || normal > 2) return fail(KH_ERR_INVALID, "bad flux arguments");
    const Mon* m[4];
    for (int q = 0; q < 4; ++q) {
      if (ids[q] < 0 || ids[q] >= int(mons_.size())) return fail(KH_ERR_INVALID, "bad monitor id");
      m[q] = &mons_[ids[q]];
      if (m[q]->nf != m[0]->nf) return fail(KH_ERR_INVALID, "flux monitors differ in frequencies");
    }
    // Ordered after this simulation's last batch on its own stream: the
    // per-frequency buffer comes from the memory pool, the result is copied
    // into a recycled pinned buffer, and only that stream is waited for.
    cudaStream_t st = last_stream_;
    const size_t bytes = sizeof(double) * m[0]->nf;
    const int cap = kFluxMaxBlocks * m[0]->nf;
    double* dout = nullptr;
    KH_CUDA(kh_host::dev_alloc((void**)&dout, bytes + sizeof(double) * size_t(cap), st));
    kh::launch_flux<T>(m[0]->F, m[1]->F, m[2]->F, m[3]->F, m[0]->C, m[1]->C, m[2]->C, m[3]->C,
                       m[0]->dims, m[1]->dims, m[2]->dims, m[3]->dims, normal, m[0]->nf, dA, dout,
                       dout + m[0]->nf, cap, st);
    ++launches;
    double* host = static_cast<double*>(kh_host::pinned_get(bytes));
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && !host) e = cudaErrorMemoryAllocation;
    if (e == cudaSuccess) e = cudaMemcpyAsync(host, dout, bytes, cudaMemcpyDeviceToHost, st);
    kh_host::dev_free(dout, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) std::memcpy(out, host, bytes);
    if (host) kh_host::pinned_put(host, bytes);
    if (e != cudaSuccess) return fail(KH_ERR_CUDA, cudaGetErrorString(e));
    return check_device_error();
  }

  // flux() with the per-frequency sums in the static device scratch instead of
  // a cudaMalloc'd buffer: no device allocation or free.
  kh_status flux_static(const int32_t* ids, int normal, double dA, double* out) override {
    if (!prepared_) return fail(KH_ERR_INVALID, "flux before prepare");
    if (!ids || !out || normal < 0 || normal > 2) return fail(KH_ERR_INVALID, "bad flux arguments");
    const Mon* m[4];
    for (int q = 0; q < 4; ++q) {
      if (ids[q] < 0 || ids[q] >= int(mons_.size())) return fail(KH_ERR_INVALID, "bad monitor id");
      m[q] = &mons_[ids[q]];
      if (m[q]->nf != m[0]->nf) return fail(KH_ERR_INVALID, "flux monitors differ in frequencies");
    }
    const int nf = m[0]->nf;
    if (nf > kFluxStaticMaxFreqs)
      return fail(KH_ERR_INVALID, "kh_sim_flux_static: " + std::to_string(nf) +
                                      " frequencies exceed its fixed scratch of " +
                                      std::to_string(kFluxStaticMaxFreqs) + "; use kh_sim_flux");
    if (kh_status es = wait_idle(); es != KH_OK) return es;
    double* scratch = nullptr;
    const kh_status st = flux_static_scratch(&scratch, err);
    if (st != KH_OK) return st;
    kh::launch_flux<T>(m[0]->F, m[1]->F, m[2]->F, m[3]->F, m[0]->C, m[1]->C, m[2]->C, m[3]->C,
                       m[0]->dims, m[1]->dims, m[2]->dims, m[3]->dims, normal, nf, dA, scratch,
                       scratch + kFluxStaticMaxFreqs, std::min(kFluxStaticPartials, kFluxMaxBlocks * nf),
                       nullptr);
    ++launches;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(out, scratch, sizeof(double) * nf, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return fail(KH_ERR_CUDA, cudaGetErrorString(e));
    return KH_OK;
  }

  // Design update: per-voxel ε⁻¹ (or μ⁻¹) of one component in a cell box,
  // values x fastest over the box.  Cell classes do not depend on these
  // values, so nothing else is rebuilt.
  kh_status update_material_box(int kind, int comp, const int32_t* st, const int32_t* dm,
                                const double* v) override {
    if (!prepared_) return fail(KH_ERR_INVALID, "update_material_box before prepare");
    if (!st || !dm || !v) return fail(KH_ERR_INVALID, "null update_material_box argument");
    if (comp < 0 || comp > 2) return fail(KH_ERR_INVALID, "material component must be 0..2");
    T* dst = nullptr;
    std::vector<T>* host = nullptr;
    if (kind == KH_MAT_EPS_INV) { dst = eps_[comp]; host = &eps_h_[comp]; }
    else if (kind == KH_MAT_MU_INV) { dst = mu_[comp]; host = &mu_h_[comp]; }
    else return fail(KH_ERR_UNSUPPORTED, "only ε⁻¹ and μ⁻¹ can be updated after prepare");
    if (!dst) return fail(KH_ERR_INVALID, "no per-voxel array of this kind was set before prepare");
    for (int a = 0; a < 3; ++a)
      if (dm[a] <= 0 || st[a] < 0 || st[a] + dm[a] > n_[a]) return fail(KH_ERR_INVALID, "box outside the grid");
    if (kh_status es = wait_idle(); es != KH_OK) return es;
    std::vector<T> plane(size_t(dm[0]) * dm[1]);
    for (int k = 0; k < dm[2]; ++k) {
      for (int j = 0; j < dm[1]; ++j)
        for (int i = 0; i < dm[0]; ++i) {
          const T val = T(v[(size_t(k) * dm[1] + j) * dm[0] + i]);
          plane[size_t(j) * dm[0] + i] = val;
          if (!host->empty()) (*host)[(size_t(st[2] + k) * n_[1] + (st[1] + j)) * n_[0] + (st[0] + i)] = val;
        }
      T* row0 = dst + origin_ + (long long)(st[2] + k) * plane_ + (long long)st[1] * pitch_ + st[0];
      KH_CUDA(cudaMemcpy2D(row0, size_t(pitch_) * sizeof(T), plane.data(), size_t(dm[0]) * sizeof(T),
                           size_t(dm[0]) * sizeof(T), size_t(dm[1]), cudaMemcpyHostToDevice));
    }
    return KH_OK;
  }

  // Replace source `index`'s amplitudes (the cells it injects into stay the
  // same: an element that was zero at prepare must stay zero) and, for a
  // KH_TIME_TABLE source, its table and end time.
  kh_status update_source(int index, const double* amp, int64_t table_len, const double* table,
                          double cutoff) override {
    if (!prepared_) return fail(KH_ERR_INVALID, "update_source before prepare");
    if (index < 0 || index >= int(srcs_.size())) return fail(KH_ERR_INVALID, "bad source index");
    SrcH& s = srcs_[index];
    if (table && s.d.time_kind != KH_TIME_TABLE)
      return fail(KH_ERR_INVALID, "a time table can only replace a KH_TIME_TABLE profile");
    if (table && table_len < 0) return fail(KH_ERR_INVALID, "negative table length");
    const size_t cnt = size_t(s.d.dims[0]) * s.d.dims[1] * s.d.dims[2];
    std::vector<Cplx<T>> amp_new = ent_amp_h_;
    if (amp) {
      std::vector<int> where(cnt, -1);
      for (auto& pe : src_ent_[index]) where[size_t(pe.first)] = pe.second;
      for (size_t q = 0; q < cnt; ++q) {
        const Cplx<T> a{T(amp[2 * q]), T(amp[2 * q + 1])};
        if (where[q] >= 0) amp_new[size_t(where[q])] = a;
        else if (a.re != T(0) || a.im != T(0))
          return fail(KH_ERR_INVALID, "update_source: nonzero amplitude outside the source's prepared cells");
      }
    }
    if (kh_status es = wait_idle(); es != KH_OK) return es;
    if (amp) {
      for (size_t q = 0; q < cnt; ++q) s.amp[q] = std::complex<double>(amp[2 * q], amp[2 * q + 1]);
      if (!amp_new.empty())
        KH_CUDA(cudaMemcpy(ent_amp_, amp_new.data(), amp_new.size() * sizeof(Cplx<T>), cudaMemcpyHostToDevice));
      ent_amp_h_.swap(amp_new);
      if (slot_pack_) {
        std::vector<kh::SlotPack<T>> pack = pack_slots();
        KH_CUDA(cudaMemcpy(slot_pack_, pack.data(), pack.size() * sizeof(kh::SlotPack<T>), cudaMemcpyHostToDevice));
      }
    }
    if (table) {
      s.table.assign(size_t(2 * table_len), std::complex<T>(T(0), T(0)));
      for (int64_t q = 0; q < 2 * table_len; ++q)
        s.table[size_t(q)] = std::complex<T>(T(table[2 * q]), T(table[2 * q + 1]));
      s.d.table_len = table_len;
      s.d.cutoff = cutoff;
      has_cw_ = false;
      last_time_ = -INFINITY;
      for (auto& x : srcs_) {
        if (x.d.time_kind == KH_TIME_CW) has_cw_ = true;
        else last_time_ = std::max(last_time_, double(T(x.d.cutoff)));
      }
    }
    return KH_OK;
  }

  kh_status monitor_view(int id, kh_host::MonitorView* out) override {
    if (!prepared_) return fail(KH_ERR_INVALID, "monitor read before prepare");
    if (id < 0 || id >= int(mons_.size()) || !out) return fail(KH_ERR_INVALID, "bad monitor id");
    const Mon& m = mons_[id];
    out->F = m.F;
    out->C = m.C;
    for (int a = 0; a < 3; ++a) out->dims[a] = m.dims[a];
    out->nf = m.nf;
    out->dtype = sizeof(T) == 4 ? KH_F32 : KH_F64;
    return KH_OK;
  }

  int monitor_count() const override { return int(mons_.size()); }

  int dtype() const override { return sizeof(T) == 4 ? KH_F32 : KH_F64; }

  kh_status field_arrays(const void* out[6], long long* count) override {
    if (!prepared_) return fail(KH_ERR_INVALID, "field read before prepare");
    for (int c = 0; c < 3; ++c) {
      out[c] = E_[c];
      out[3 + c] = H_[c];
    }
    *count = total_;
    return KH_OK;
  }

  kh_status field_view(int comp, kh_field_view* out) override {
    if (!prepared_) return fail(KH_ERR_INVALID, "field view before prepare");
    if (comp < 0 || comp > 5 || !out) return fail(KH_ERR_INVALID, "bad field view arguments");
    T* base = comp < 3 ? E_[comp] : H_[comp - 3];
    out->data = base + origin_;
    out->dtype = dtype();
    for (int a = 0; a < 3; ++a) out->dims[a] = n_[a] + kStagger[comp][a];
    out->strides[0] = 1;
    out->strides[1] = pitch_;
    out->strides[2] = plane_;
    return KH_OK;
  }

  kh_status reset() override {
    if (!prepared_) return fail(KH_ERR_INVALID, "reset before prepare");
    if (kh_status es = wait_idle(); es != KH_OK) return es;
    for (auto& s : state_) KH_CUDA(cudaMemset(s.first, 0, s.second));
    KH_CUDA(cudaStreamSynchronize(cudaStreamLegacy));
    timestep_ = 0;
    sources_active_ = true;
    return KH_OK;
  }

  int64_t state_bytes() const override {
    int64_t b = 16;
    for (auto& s : state_) b += int64_t(s.second);
    return b;
  }

  kh_status export_state(void* dst, int64_t bytes) override {
    if (!prepared_ || !dst || bytes != state_bytes()) return fail(KH_ERR_INVALID, "bad export buffer");
    if (kh_status es = wait_idle(); es != KH_OK) return es;
    char* p = static_cast<char*>(dst);
    int64_t hdr[2] = {timestep_, sources_active_ ? 1 : 0};
    std::memcpy(p, hdr, 16);
    p += 16;
    for (auto& s : state_) {
      KH_CUDA(cudaMemcpy(p, s.first, s.second, cudaMemcpyDeviceToHost));
      p += s.second;
    }
    return KH_OK;
  }

  kh_status import_state(const void* src, int64_t bytes) override {
    if (!prepared_ || !src || bytes != state_bytes()) return fail(KH_ERR_INVALID, "bad import buffer");
    if (kh_status es = wait_idle(); es != KH_OK) return es;
    const char* p = static_cast<const char*>(src);
    int64_t hdr[2];
    std::memcpy(hdr, p, 16);
    p += 16;
    for (auto& s : state_) {
      KH_CUDA(cudaMemcpy(s.first, p, s.second, cudaMemcpyHostToDevice));
      p += s.second;
    }
    timestep_ = hdr[0];
    sources_active_ = hdr[1] != 0;
    return KH_OK;
  }

  // Compulsory-traffic model: the reference's 9 + 12 words per cell
  // (benchmark/benchmark_metrics.jl:236-241) plus CPML auxiliaries of each
  // region (2 words per auxiliary per component: read + write, with the B/D
  // state counted where a U or W exists), dispersive and χ3 terms, and DFT
  // monitor traffic amortised over the decimation.
  double model_bytes_per_step() const override {
    double h, e, d;
    model_split(h, e, d);
    return h + e + d;
  }

  void model_split(double& h_bytes, double& e_bytes, double& dft_bytes) const override {
    const bool pervox_eps = has_eps(0) || geo_set_;
    const bool pervox_mu = has_mu(0);
    const long long cells = 1LL * n_[0] * n_[1] * n_[2];
    // H: E 3 rd + H 3 rd + H 3 wr (+ μ⁻¹ 3 rd); E: H 3 rd + E 3 rd + E 3 wr (+ ε⁻¹ 3 rd)
    double hw = (9 + (pervox_mu ? 3 : 0)) * double(cells);
    double ew = (9 + (pervox_eps ? 3 : 0)) * double(cells);
    for (int r = 0; r < 27; ++r) {
      const int rr[3] = {r % 3, (r / 3) % 3, r / 9};
      long long cnt = 1;
      bool f[3];
      for (int a = 0; a < 3; ++a) {
        int lo, hi;
        axis_interval(a, rr[a], lo, hi);
        cnt *= std::max(0, hi - lo);
        f[a] = rr[a] != 1;
      }
      if (cnt == 0 || !(f[0] || f[1] || f[2])) continue;
      // Σ_c 2·(U_c + W_c + T_c): T_c = U_c ∨ W_c on the CPU path; the CUDA-path
      // stages also keep T_c where only the prev axis is PML (σ_prev stage).
      const bool cpml = d_.semantics == KH_SEM_CPML;
      int aux = 0;
      for (int c = 0; c < 3; ++c) {
        const int u = f[(c + 1) % 3] ? 1 : 0, w = f[c] ? 1 : 0;
        const int t = (u || w || (cpml && f[(c + 2) % 3])) ? 1 : 0;
        aux += 2 * (u + w + t);
      }
      hw += double(aux) * double(cnt);  // B side
      ew += double(aux) * double(cnt);  // D side
    }
    if (!chi3_h_.empty() || !poles_.empty()) {
      const size_t ncenter = size_t(n_[0]) * n_[1] * n_[2];
      for (size_t q = 0; q < ncenter; ++q) {
        double w = 0;
        bool sp = false;
        if (!chi3_h_.empty() && chi3_h_[q] != T(0)) { w += 1; sp = true; }
        for (auto& p : poles_)
          if (p.sigma[q] != T(0)) { w += 1 + 12; sp = true; }  // σ + P, P_prev read + write
        if (sp) w += 6;  // D state read + write
        ew += w;
      }
    }
    h_bytes = hw * sizeof(T);
    e_bytes = ew * sizeof(T);
    dft_bytes = 0;
    for (auto& m : mons_) {
      // field read + accumulator (and Kahan term) read + write per frequency
      const double per = double(m.ncell) * (sizeof(T) + m.nf * 2.0 * sizeof(Cplx<T>) * (m.C ? 2 : 1));
      dft_bytes += per / double(m.dec);
    }
  }

  kh_status step_timed(int64_t nsteps, cudaStream_t stream, double* h_ms, double* e_ms,
                       double* dft_ms) override {
    if (!prepared_) return fail(KH_ERR_INVALID, "step before prepare");
    if (nsteps < 0) return fail(KH_ERR_INVALID, "negative step count");
    Timing t;
    int64_t done = 0;
    while (done < nsteps) {
      const int nb = int(std::min<int64_t>(kBatch, nsteps - done));
      kh_status st = run_batch(nb, stream, &t);
      if (st != KH_OK) return st;
      done += nb;
    }
    // the sampled steps stand for all nsteps
    const double scale = t.sampled > 0 ? double(nsteps) / double(t.sampled) : 0.0;
    if (h_ms) *h_ms = t.h * scale;
    if (e_ms) *e_ms = t.e * scale;
    if (dft_ms) *dft_ms = t.dft * scale;
    return KH_OK;
  }

 private:
  static constexpr int kBatch = 512;
  static constexpr int kCaptureNow = 128;

  // Entries of the largest per-batch table: both halves' source factors on
  // every step, plus each monitor's phases on its decimation steps.
  size_t table_capacity() const {
    size_t n = size_t(kBatch) * 2 * srcs_.size();
    for (auto& m : mons_) {
      const int dec = m.dec < 1 ? 1 : m.dec;
      n += size_t(m.nf) * size_t((kBatch + dec - 1) / dec + 1);
    }
    return std::max<size_t>(n, 1);
  }

  struct Timing {
    double h = 0, e = 0, dft = 0;
    int64_t sampled = 0;  // steps whose launches were bracketed with events
    int64_t done = 0;     // steps of the timed call issued so far
  };
  // Timed runs bracket the launches of every kTimeSample-th step of the call
  // (its first step included) with events; one event pair per launch group on
  // every step would itself cost ~4 % of the step time.
  static constexpr int kTimeSample = 8;
  struct PoleH {
    kh_pole_coeffs c;
    std::vector<T> sigma;
  };
  struct PoleD {
    kh_pole_coeffs c;
    T* sigma = nullptr;
    T* P[3] = {nullptr, nullptr, nullptr};
    T* Pp[3] = {nullptr, nullptr, nullptr};
  };
  struct SrcH {
    kh_source_desc d;
    std::vector<std::complex<double>> amp;
    std::vector<std::complex<T>> table;
  };
  struct GraphEntry {
    std::vector<int64_t> sig;
    cudaGraphExec_t exec;
    int64_t nlaunch;
    uint64_t last_use;
  };
  static constexpr size_t kMaxGraphs = 24;
  struct Hist {
    int comp, start[3], dims[3];
    long long ncell = 0;
    int64_t cap = 0;
    T* buf = nullptr;
  };
  struct Mon {
    int comp, start[3], dims[3], nf, dec;
    std::vector<double> freqs;
    long long ncell = 0;
    Cplx<T>* F = nullptr;
    Cplx<T>* C = nullptr;
  };

  kh_status fail(kh_status s, const std::string& msg) {
    err = msg;
    return s;
  }

  void axis_interval(int a, int r, int& lo, int& hi) const {
    if (d_.pml_lo[a] >= n_[a] && n_[a] > 0) {  // whole axis flagged
      if (r == 0) { lo = 0; hi = n_[a]; } else { lo = hi = 0; }
      return;
    }
    if (r == 0) { lo = 0; hi = d_.pml_lo[a]; }
    else if (r == 1) { lo = d_.pml_lo[a]; hi = n_[a] - d_.pml_hi[a]; }
    else { lo = n_[a] - d_.pml_hi[a]; hi = n_[a]; }
    if (hi < lo) hi = lo;
  }

  bool region_nonempty(const int* rr) const {
    for (int a = 0; a < 3; ++a) {
      int lo, hi;
      axis_interval(a, rr[a], lo, hi);
      if (hi <= lo) return false;
    }
    return true;
  }

  uint32_t region_mask(const std::vector<T>* msig) const {
    uint32_t mask = 0;
    for (int r = 0; r < 27; ++r) {
      const int rr[3] = {r % 3, (r / 3) % 3, r / 9};
      if (!region_nonempty(rr)) continue;
      int b[3][2];
      for (int a = 0; a < 3; ++a) axis_interval(a, rr[a], b[a][0], b[a][1]);
      bool nz = false;
      for (int c = 0; c < 3 && !nz; ++c) {
        if (msig[c].empty()) continue;
        for (int k = b[2][0]; k < b[2][1] && !nz; ++k)
          for (int j = b[1][0]; j < b[1][1] && !nz; ++j)
            for (int i = b[0][0]; i < b[0][1]; ++i)
              if (msig[c][(size_t(k) * n_[1] + j) * n_[0] + i] != T(0)) { nz = true; break; }
      }
      if (nz) mask |= 1u << r;
    }
    return mask;
  }

  kh_status alloc_raw(size_t bytes, void** out, bool is_state) {
    void* p = nullptr;
    KH_CUDA(kh_host::dev_alloc(&p, bytes, cudaStreamLegacy));
    allocs_.push_back(p);
    device_bytes_ += int64_t(bytes);
    KH_CUDA(cudaMemsetAsync(p, 0, bytes, cudaStreamLegacy));
    if (is_state) state_.push_back({p, bytes});
    *out = p;
    return KH_OK;
  }
  // One row of slack past the last plane: a dense wrapper that starts at the
  // (-1, -1, -1) ghost cell of a component and spans dims[2] + 1 whole planes
  // (the reference's raw layout, kh_sim_field_view) stays inside the block.
  kh_status alloc_field(T** out) {
    return alloc_raw(size_t(total_ + pitch_) * sizeof(T), (void**)out, true);
  }

  kh_status upload_raw(const void* h, size_t bytes, void** out) {
    KH_CUDA(kh_host::dev_alloc(out, bytes, cudaStreamLegacy));
    allocs_.push_back(*out);
    device_bytes_ += int64_t(bytes);
    KH_CUDA(cudaMemcpy(*out, h, bytes, cudaMemcpyHostToDevice));
    return KH_OK;
  }

  // Center-range host array (x fastest, float or double) → padded device
  // layout in the run's precision: one compact host-to-device copy into a
  // pool buffer, then a scatter kernel (the ring and row padding stay zero).
  kh_status upload_center(const void* src, int src_dtype, T** out) {
    void* p = nullptr;
    kh_status st = alloc_raw(size_t(total_) * sizeof(T), &p, false);
    if (st != KH_OK) return st;
    *out = static_cast<T*>(p);
    const size_t cnt = size_t(n_[0]) * n_[1] * n_[2];
    if (cnt == 0) return KH_OK;
    const size_t bytes = cnt * (src_dtype == KH_F32 ? sizeof(float) : sizeof(double));
    void* tmp = nullptr;
    KH_CUDA(kh_host::dev_alloc(&tmp, bytes, cudaStreamLegacy));
    cudaError_t e = cudaMemcpyAsync(tmp, src, bytes, cudaMemcpyHostToDevice, cudaStreamLegacy);
    if (e == cudaSuccess) {
      if (src_dtype == KH_F32)
        kh::launch_scatter_center<float, T>(static_cast<const float*>(tmp), *out, n_, pitch_, plane_, origin_,
                                            cudaStreamLegacy);
      else
        kh::launch_scatter_center<double, T>(static_cast<const double*>(tmp), *out, n_, pitch_, plane_, origin_,
                                             cudaStreamLegacy);
      ++launches;
      e = cudaGetLastError();
    }
    kh_host::dev_free(tmp, cudaStreamLegacy);
    if (e != cudaSuccess) return fail(KH_ERR_CUDA, std::string("material upload: ") + cudaGetErrorString(e));
    return KH_OK;
  }

  // Single-entry slots packed for one load (src = -1: several entries).
  std::vector<kh::SlotPack<T>> pack_slots() const {
    std::vector<kh::SlotPack<T>> pack(slot_off_h_.empty() ? 0 : slot_off_h_.size() - 1);
    for (size_t sl = 0; sl < pack.size(); ++sl) {
      const int e0 = slot_off_h_[sl], e1 = slot_off_h_[sl + 1];
      if (e1 - e0 == 1) pack[sl] = {ent_src_h_[e0], ent_comp_h_[e0], ent_amp_h_[e0]};
      else pack[sl] = {-1, -1, {T(0), T(0)}};
    }
    return pack;
  }

  bool has_eps(int c) const { return !eps_h_[c].empty() || att_eps_[c].ptr; }
  bool has_mu(int c) const { return !mu_h_[c].empty() || att_mu_[c].ptr; }

  // eval_time_source in the run's precision (TimeSources.jl:61-64, 123-132, 178-184)
  std::complex<T> eval_time(const SrcH& s, double t, int64_t step, bool h_half) const {
    const T two_pi = T(2) * T(M_PI);
    if (s.d.time_kind == KH_TIME_GAUSSIAN) {
      const T tt = T(t) - T(s.d.peak_time);
      if (tt > T(s.d.cutoff)) return {T(0), T(0)};
      const T w = T(s.d.width);
      const T g = std::exp((-tt) * tt / ((T(2) * w) * w));
      const T b = ((-two_pi) * T(s.d.fcen)) * tt;
      return {g * std::cos(b), g * std::sin(b)};
    }
    if (s.d.time_kind == KH_TIME_CW) {
      const T b = ((-two_pi) * T(s.d.fcen)) * T(t);
      return {std::cos(b), std::sin(b)};
    }
    if (T(t) > T(s.d.cutoff)) return {T(0), T(0)};
    const int64_t q = 2 * step + (h_half ? 0 : 1);
    if (q >= int64_t(s.table.size())) return {T(0), T(0)};
    return s.table[q];
  }

  kh_status run_batch(int nb, cudaStream_t stream, Timing* timing = nullptr) {
    // A batch on a new stream waits for the previous batch, whose kernels read
    // the shared time-factor table this batch is about to overwrite.
    if (last_stream_ != stream && batch_done_) KH_CUDA(cudaStreamWaitEvent(stream, batch_done_, 0));
    // Graph replay (the steady-state step graphs of _try_capture_graphs!,
    // Kernels.jl:99-145): the batch runs on the simulation's own stream, which
    // waits for the caller's stream and is waited on by it afterwards.  Not
    // for timed batches (events around every launch) nor while a history
    // monitor records (its destination moves every step).
    bool use_graph = graphs_on_ && !timing;
    for (auto& h : hists_)
      if (timestep_ < h.cap) use_graph = false;
    cudaStream_t ws = stream;  // stream the batch's work is issued on
    if (use_graph) {
      KH_CUDA(cudaEventRecord(ev_in_, stream));
      KH_CUDA(cudaStreamWaitEvent(gstream_, ev_in_, 0));
      ws = gstream_;
    }
    // Host pass: source activity, time factors and DFT phases for nb steps.
    struct StepPlan {
      bool sa;
      size_t fH, fE;                      // offsets into the table (Cplx<T> units)
      std::vector<std::pair<int, size_t>> dftH, dftE;  // (monitor, phase offset)
    };
    std::vector<StepPlan> plan(nb);
    std::vector<Cplx<T>> tab;
    for (int s = 0; s < nb; ++s) {
      const int64_t ts = timestep_ + s;
      const double t = double(T(ts) * dt_);  // round_time
      if (sources_active_ && !has_cw_ && nsrc_ > 0 && t > last_time_) sources_active_ = false;
      StepPlan& P = plan[s];
      P.sa = sources_active_ && nsrc_ > 0 && ent_src_ != nullptr;
      const double tE = t + double(dt_ / T(2));
      P.fH = tab.size();
      if (P.sa)
        for (auto& src : srcs_) {
          std::complex<T> f = eval_time(src, t, ts, true);
          tab.push_back({f.real(), f.imag()});
        }
      P.fE = tab.size();
      if (P.sa)
        for (auto& src : srcs_) {
          std::complex<T> f = eval_time(src, tE, ts, false);
          tab.push_back({f.real(), f.imag()});
        }
      for (int mi = 0; mi < int(mons_.size()); ++mi) {
        const Mon& m = mons_[mi];
        if (m.dec > 1 && ts % m.dec != 0) continue;
        const bool hm = m.comp >= 3;
        const double time = hm ? t : tE;
        const size_t off = tab.size();
        for (int f = 0; f < m.nf; ++f) {
          // Δt·exp(i·f·2π·time): θ formed as the reference forms it
          // (complex_backend_number(im*2π*time), Monitors.jl:287-297); FP32 runs
          // evaluate the phase in FP64 and round once.
          double re, im;
          if (sizeof(T) == 8) {
            const double th = double(T(m.freqs[f])) * double(T(6.283185307179586 * time));
            re = double(dt_) * std::cos(th);
            im = double(dt_) * std::sin(th);
          } else {
            const double th = double(T(m.freqs[f])) * (6.283185307179586 * time);
            re = double(dt_) * std::cos(th);
            im = double(dt_) * std::sin(th);
          }
          tab.push_back({T(re), T(im)});
        }
        (hm ? P.dftH : P.dftE).push_back({mi, off});
      }
    }
    // Upload the table: staging buffer b was last copied from two batches ago;
    // wait for that copy before overwriting it.
    const int b = tab_par_;
    tab_par_ ^= 1;
    const size_t bytes = tab.size() * sizeof(Cplx<T>);
    if (bytes > tab_cap_) return fail(KH_ERR_INVALID, "time-factor table exceeds its capacity");
    if (copy_pending_[b]) {
      KH_CUDA(cudaEventSynchronize(copy_ev_[b]));
      copy_pending_[b] = false;
    }
    if (!tab.empty()) {
      std::memcpy(pinned_[b], tab.data(), bytes);
      KH_CUDA(cudaMemcpyAsync(tab_dev_[b], pinned_[b], bytes, cudaMemcpyHostToDevice, ws));
      KH_CUDA(cudaEventRecord(copy_ev_[b], ws));
      copy_pending_[b] = true;
    }
    const Cplx<T>* dtab = static_cast<const Cplx<T>*>(tab_dev_[b]);

    // Timed runs bracket every launch group with events: 5 per step.
    if (timing) {
      while (events_.size() < size_t(5 * nb)) {
        cudaEvent_t ev;
        KH_CUDA(cudaEventCreate(&ev));
        events_.push_back(ev);
      }
    }
    auto sampled = [&](int s) { return timing && (timing->done + s) % kTimeSample == 0; };
    auto mark = [&](int s, int k) {
      if (sampled(s)) cudaEventRecord(events_[5 * s + k], stream);
    };
    kh::HalfStepParams<T> ph = base_params(true), pe = base_params(false);
    // LEAN unless this half needs the in-kernel general path (see prepare()).
    const bool msb = msigb_[0] || msigb_[1] || msigb_[2];
    const bool msd = msigd_[0] || msigd_[1] || msigd_[2];
    const bool ref_cpu = d_.semantics == KH_SEM_REFERENCE_CPU;
    const bool full_h_base = msb || (ref_cpu && special_in_region_[1]);
    // χ3 and pole cells: in the LEAN E launch plus the dispersive-cell pass
    // (disp_fix_), or in the FULL launch
    const bool dispersive = chi3_ != nullptr || !poles_d_.empty();
    const bool full_e_base = msd || (dispersive && !disp_fix_) || (ref_cpu && special_in_region_[0]);
    const kh::WrapParams<T> wh = wrap_params(true), we = wrap_params(false);
    kh::SourceFixParams<T> fh = fix_params(true), fe = fix_params(false);
    kh::DispFixParams<T> dfix = disp_params(pe);
    auto issue_all = [&](cudaStream_t st) {
    for (int s = 0; s < nb; ++s) {
      const StepPlan& P = plan[s];
      ph.sources_active = P.sa ? 1 : 0;
      ph.f_now = dtab + P.fH;
      const bool src_h = P.sa && has_src_[1];
      ph.full = (full_h_base || (src_h && !src_lean_ok_[1])) ? 1 : 0;
      mark(s, 0);
      if (use_tma_) kh::launch_half_step_tma<T>(true, ph, maps_h_, st);
      else kh::launch_half_step<T>(true, ph, st);
      ++launches;
      if (src_h && !ph.full) {
        fh.f_now = dtab + P.fH;
        kh::launch_source_fix<T>(fh, st);
        ++launches;
      }
      if (d_.periodic) {
        kh::launch_wrap<T>(wh, st);
        ++launches;
      }
      mark(s, 1);
      launch_dfts(P.dftH, dtab, st);
      record_histories(true, timestep_ + s, st);
      mark(s, 2);
      pe.sources_active = P.sa ? 1 : 0;
      pe.f_now = dtab + P.fE;
      const bool src_e = P.sa && has_src_[0];
      pe.full = (full_e_base || (src_e && !src_lean_ok_[0])) ? 1 : 0;
      if (use_tma_) kh::launch_half_step_tma<T>(false, pe, maps_e_, st);
      else kh::launch_half_step<T>(false, pe, st);
      ++launches;
      if (src_e && !pe.full) {
        fe.f_now = dtab + P.fE;
        kh::launch_source_fix<T>(fe, st);
        ++launches;
      }
      if (disp_fix_ && !pe.full) {
        dfix.sources_active = P.sa ? 1 : 0;
        dfix.f_now = dtab + P.fE;
        kh::launch_disp_fix<T>(dfix, st);
        ++launches;
      }
      if (d_.periodic) {
        kh::launch_wrap<T>(we, st);
        ++launches;
      }
      mark(s, 3);
      launch_dfts(P.dftE, dtab, st);
      record_histories(false, timestep_ + s, st);
      mark(s, 4);
    }
    };
    if (!use_graph) {
      issue_all(stream);
    } else {
      // signature of the batch's launch sequence: equal signatures issue the
      // same kernels with the same arguments (only the table contents differ)
      std::vector<int64_t> sig;
      sig.reserve(size_t(nb) * 8 + 4);
      sig.push_back(nb);
      sig.push_back(b);
      for (int q = 0; q < nb; ++q) {
        const StepPlan& P = plan[q];
        sig.push_back(P.sa ? 1 : 0);
        sig.push_back(int64_t(P.fH));
        sig.push_back(int64_t(P.fE));
        for (auto& dm : P.dftH) { sig.push_back(-1 - dm.first); sig.push_back(int64_t(dm.second)); }
        for (auto& dm : P.dftE) { sig.push_back(-1000000 - dm.first); sig.push_back(int64_t(dm.second)); }
      }
      GraphEntry* g = nullptr;
      for (auto& ge : graphs_)
        if (ge.sig == sig) { g = &ge; break; }
      // A short sequence is captured the second time it is seen: batches that
      // occur once (a short run, the last partial batch) are issued directly
      // rather than paying a capture and an instantiation they never
      // amortise.  Batches of kCaptureNow steps or more are captured at once:
      // one replay of them already repays the capture.
      bool seen_before = nb >= kCaptureNow;
      if (!g && !seen_before) {
        for (auto& sv : seen_)
          if (sv == sig) { seen_before = true; break; }
        if (!seen_before) {
          if (seen_.size() >= kMaxGraphs) seen_.erase(seen_.begin());
          seen_.push_back(sig);
        }
      }
      if (g) ++graph_hits_;
      else if (seen_before) ++graph_misses_;
      if (!g && !seen_before) {
        issue_all(ws);
      } else if (!g) {
        if (graphs_.size() >= kMaxGraphs) {  // evict the least recently used
          size_t lru = 0;
          for (size_t q = 1; q < graphs_.size(); ++q)
            if (graphs_[q].last_use < graphs_[lru].last_use) lru = q;
          cudaGraphExecDestroy(graphs_[lru].exec);
          graphs_.erase(graphs_.begin() + long(lru));
        }
        const int64_t l0 = launches;
        KH_CUDA(cudaStreamBeginCapture(ws, cudaStreamCaptureModeThreadLocal));
        issue_all(ws);
        cudaGraph_t graph = nullptr;
        cudaError_t ce = cudaStreamEndCapture(ws, &graph);
        cudaGraphExec_t exec = nullptr;
        if (ce == cudaSuccess) ce = cudaGraphInstantiate(&exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        if (ce != cudaSuccess) return fail(KH_ERR_CUDA, std::string("step graph capture: ") + cudaGetErrorString(ce));
        graphs_.push_back({std::move(sig), exec, launches - l0, 0});
        launches = l0;
        g = &graphs_.back();
      }
      if (g) {
        g->last_use = ++graph_clock_;
        KH_CUDA(cudaGraphLaunch(g->exec, ws));
        launches += g->nlaunch;
        ++graph_replays_;
      }
      KH_CUDA(cudaEventRecord(ev_out_, ws));
      KH_CUDA(cudaStreamWaitEvent(stream, ev_out_, 0));
      // batches that rarely repeat (irregular step counts) capture more than
      // they replay: issue directly from then on
      if (graph_misses_ > 16 && graph_hits_ < graph_misses_) graphs_on_ = false;
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(KH_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
    KH_CUDA(cudaEventRecord(batch_done_, stream));
    batch_recorded_ = true;
    last_stream_ = stream;
    timestep_ += nb;
    if (timing) {
      KH_CUDA(cudaEventSynchronize(batch_done_));
      for (int s = 0; s < nb; ++s) {
        if (!sampled(s)) continue;
        ++timing->sampled;
        float a = 0, b = 0, c = 0, d = 0;
        KH_CUDA(cudaEventElapsedTime(&a, events_[5 * s], events_[5 * s + 1]));
        KH_CUDA(cudaEventElapsedTime(&b, events_[5 * s + 1], events_[5 * s + 2]));
        KH_CUDA(cudaEventElapsedTime(&c, events_[5 * s + 2], events_[5 * s + 3]));
        KH_CUDA(cudaEventElapsedTime(&d, events_[5 * s + 3], events_[5 * s + 4]));
        timing->h += a;
        timing->dft += b + d;
        timing->e += c;
      }
      timing->done += nb;
    }
    return KH_OK;
  }

  // History monitors of one half: the component values after that half-step
  // of step `ts` go to slot ts (steps past the capacity are not recorded).
  void record_histories(bool h_half, int64_t ts, cudaStream_t stream) {
    for (auto& h : hists_) {
      if ((h.comp >= 3) != h_half || ts >= h.cap) continue;
      kh::RecordParams<T> p;
      p.field = h.comp < 3 ? E_[h.comp] : H_[h.comp - 3];
      p.pitch = pitch_;
      p.plane = plane_;
      p.origin = origin_;
      p.total = total_;
      for (int a = 0; a < 3; ++a) {
        p.start[a] = h.start[a];
        p.dims[a] = h.dims[a];
      }
      p.dst = h.buf + ts * h.ncell;
      kh::launch_record<T>(p, stream);
      ++launches;
    }
  }

  // kh_sim_set_geometry: rasterise (and smooth) each E component's ε⁻¹ on the
  // device at its Yee positions.
  kh_status build_geometry() {
    kh::GeomObj* dobjs = nullptr;
    if (!geo_.empty()) {
      const kh_status su = upload_raw(geo_.data(), geo_.size() * sizeof(kh::GeomObj), (void**)&dobjs);
      if (su != KH_OK) return su;
    }
    void* scratch = nullptr;
    if (geo_smooth_ != KH_SMOOTH_NONE) KH_CUDA(kh_host::dev_alloc(&scratch, size_t(total_) * sizeof(T), cudaStreamLegacy));
    kh_status st = KH_OK;
    for (int c = 0; c < 3 && st == KH_OK; ++c) {
      st = alloc_raw(size_t(total_) * sizeof(T), (void**)&eps_[c], false);
      if (st != KH_OK) break;
      kh::GeomArgs a;
      a.objs = dobjs;
      a.nobj = int(geo_.size());
      for (int q = 0; q < 3; ++q) {
        a.n[q] = n_[q];
        a.d[q] = double(delta_[q]);
        // Yee shift of E_c: −Δ/2 along both axes other than c (utils.jl:139-170)
        a.org[q] = geo_origin_[q] - (q == c ? 0.0 : 0.5 * double(delta_[q]));
      }
      a.pitch = pitch_;
      a.plane = plane_;
      a.origin = origin_;
      a.total = total_;
      a.background = geo_bg_;
      a.smoothing = geo_smooth_;
      a.comp = c;
      kh::launch_geometry<T>(a, eps_[c], static_cast<T*>(scratch), cudaStreamLegacy);
      launches += geo_smooth_ != KH_SMOOTH_NONE ? 2 : 1;
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) st = fail(KH_ERR_CUDA, std::string("geometry kernels: ") + cudaGetErrorString(e));
    }
    if (scratch) kh_host::dev_free(scratch, cudaStreamLegacy);
    return st;
  }

  // The DFT monitors updated after one half-step of one step: one launch for
  // all of them (KHRONOS_GB300_DFT_BATCH=0: one launch per monitor, the same
  // arithmetic).
  void launch_dfts(const std::vector<std::pair<int, size_t>>& dms, const Cplx<T>* dtab, cudaStream_t st) {
    if (dms.empty()) return;
    if (!dft_batch_) {
      for (auto& dm : dms) launch_dft_for(dm.first, dtab + dm.second, st);
      return;
    }
    for (size_t b0 = 0; b0 < dms.size(); b0 += kh::kMaxDftBatch) {
      kh::DftBatchParams<T> bp;
      std::memset(&bp, 0, sizeof(bp));
      bp.pitch = pitch_;
      bp.plane = plane_;
      bp.origin = origin_;
      bp.total = total_;
      bp.first[0] = 0;
      for (size_t q = b0; q < dms.size() && bp.n < kh::kMaxDftBatch; ++q) {
        const Mon& m = mons_[dms[q].first];
        auto& M = bp.mon[bp.n];
        M.field = m.comp < 3 ? E_[m.comp] : H_[m.comp - 3];
        for (int a = 0; a < 3; ++a) {
          M.start[a] = m.start[a];
          M.dims[a] = m.dims[a];
        }
        M.nf = m.nf;
        M.phase = dtab + dms[q].second;
        M.F = m.F;
        M.comp = m.C;
        bp.first[bp.n + 1] = bp.first[bp.n] + (long long)m.ncell * m.nf;
        ++bp.n;
      }
      kh::launch_dft_batch<T>(bp, st);
      ++launches;
    }
  }

  void launch_dft_for(int mi, const Cplx<T>* phase, cudaStream_t stream) {
    const Mon& m = mons_[mi];
    kh::DftParams<T> p;
    p.field = m.comp < 3 ? E_[m.comp] : H_[m.comp - 3];
    p.pitch = pitch_;
    p.plane = plane_;
    p.origin = origin_;
    p.total = total_;
    for (int a = 0; a < 3; ++a) {
      p.start[a] = m.start[a];
      p.dims[a] = m.dims[a];
    }
    p.nf = m.nf;
    p.phase = phase;
    p.F = m.F;
    p.comp = m.C;
    kh::launch_dft<T>(p, stream);
    ++launches;
  }

  // Tensor maps over the padded layout for the TMA-staged kernel.
  kh_status build_tma_maps() {
    // the attribute is per device: set it once for each device a simulation runs on
    static std::atomic<bool> attr_done[kMaxDevices];
    int dev = 0;
    KH_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(KH_ERR_UNSUPPORTED, "device ordinal above the supported range");
    if (!attr_done[dev]) {
      if (kh::prepare_tma_kernels<T>() != 0)
        return fail(KH_ERR_CUDA, "cudaFuncSetAttribute on the TMA half-step kernels failed");
      attr_done[dev] = true;
    }
    int sms = 0;
    KH_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    tma_slots_ = sms * kh::tma_resident_ctas<T>();
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult qr;
    KH_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &qr));
    if (!fn || qr != cudaDriverEntryPointSuccess) return fail(KH_ERR_CUDA, "cuTensorMapEncodeTiled not available");
    auto encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    const int hx = 16 / int(sizeof(T));
    const cuuint64_t dims[3] = {cuuint64_t(pitch_), cuuint64_t(n_[1] + 2), cuuint64_t(n_[2] + 2)};
    const cuuint64_t strides[2] = {cuuint64_t(pitch_) * sizeof(T), cuuint64_t(plane_) * sizeof(T)};
    const cuuint32_t box_a[3] = {cuuint32_t(kh::kTmaX + hx), cuuint32_t(kh::kTmaY + 1), 1};
    const cuuint32_t box_o[3] = {cuuint32_t(kh::kTmaX), cuuint32_t(kh::kTmaY), 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    const CUtensorMapDataType dt = sizeof(T) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
    auto mk = [&](CUtensorMap* m, T* base, const cuuint32_t* box) -> kh_status {
      // base points at element (-1,-1,-1) - XOFF + ... : the allocation start
      CUresult r = encode(m, dt, 3, static_cast<void*>(base), dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
      if (r != CUDA_SUCCESS) return fail(KH_ERR_CUDA, "cuTensorMapEncodeTiled failed");
      return KH_OK;
    };
    std::memset(&maps_h_, 0, sizeof(maps_h_));
    std::memset(&maps_e_, 0, sizeof(maps_e_));
    for (int c = 0; c < 3; ++c) {
      kh_status st;
      if ((st = mk(&maps_h_.a[c], E_[c], box_a)) != KH_OK) return st;
      if ((st = mk(&maps_h_.o[c], H_[c], box_o)) != KH_OK) return st;
      if (mu_[c] && (st = mk(&maps_h_.m[c], mu_[c], box_o)) != KH_OK) return st;
      if ((st = mk(&maps_e_.a[c], H_[c], box_a)) != KH_OK) return st;
      if ((st = mk(&maps_e_.o[c], E_[c], box_o)) != KH_OK) return st;
      if (eps_[c] && (st = mk(&maps_e_.m[c], eps_[c], box_o)) != KH_OK) return st;
      if (B_[c] && (st = mk(&maps_h_.t[c], B_[c], box_o)) != KH_OK) return st;
      if (UB_[c] && (st = mk(&maps_h_.u[c], UB_[c], box_o)) != KH_OK) return st;
      if (WB_[c] && (st = mk(&maps_h_.w[c], WB_[c], box_o)) != KH_OK) return st;
      if (D_[c] && (st = mk(&maps_e_.t[c], D_[c], box_o)) != KH_OK) return st;
      if (UD_[c] && (st = mk(&maps_e_.u[c], UD_[c], box_o)) != KH_OK) return st;
      if (WD_[c] && (st = mk(&maps_e_.w[c], WD_[c], box_o)) != KH_OK) return st;
    }
    return KH_OK;
  }

  // z planes per CTA of the TMA-staged kernel; KHRONOS_GB300_ZPLANES overrides.
  int choose_zplanes() const {
    if (const char* zv = std::getenv("KHRONOS_GB300_ZPLANES")) {
      const int z = std::atoi(zv);
      if (z >= 1) return std::min(z, n_[2]);
    }
    // 10 planes: a measured optimum on 128- and 256-plane grids (one plane of
    // curl-source halo re-read per CTA against enough CTAs to balance the
    // SMs); shallower when the launch would not fill two rounds of resident CTAs.
    int z = 10;
    if (use_tma_ && tma_slots_ > 0) {
      const long long xy = (long long)((n_[0] + kh::kTmaX - 1) / kh::kTmaX) * ((n_[1] + kh::kTmaY - 1) / kh::kTmaY);
      const long long fill = xy * n_[2] / (2LL * tma_slots_);
      z = int(std::max(2LL, std::min<long long>(z, fill)));
    }
    return std::min(z, n_[2]);
  }

  kh_status device_error() override { return check_device_error(); }

  // A kernel whose bounded wait gave up leaves KH_ERR_TIMEOUT in err_dev_.
  kh_status check_device_error() {
    if (!err_dev_) return KH_OK;
    int e = 0;
    KH_CUDA(cudaMemcpy(&e, err_dev_, sizeof(int), cudaMemcpyDeviceToHost));
    if (e != 0) return fail(KH_ERR_TIMEOUT, "a half-step kernel gave up waiting on its TMA copies");
    return KH_OK;
  }

  kh::SourceFixParams<T> fix_params(bool h) const {
    kh::SourceFixParams<T> f;
    std::memset(&f, 0, sizeof(f));
    f.nslots = nslots_;
    f.n_ent = int(ent_amp_h_.size());
    f.n_src = nsrc_;
    f.total = total_;
    f.slot_cell = slot_cell_;
    f.slot_pack = slot_pack_;
    f.slot_off = slot_off_;
    f.ent_src = ent_src_;
    f.ent_comp = ent_comp_;
    f.ent_amp = ent_amp_;
    for (int c = 0; c < 3; ++c) {
      f.O[c] = h ? H_[c] : E_[c];
      f.Ts[c] = h ? B_[c] : D_[c];
      f.m_inv[c] = h ? mu_[c] : eps_[c];
    }
    f.m_scalar = h ? T(d_.mu_inv) : T(d_.eps_inv);
    f.h_half = h ? 1 : 0;
    if (d_.semantics == KH_SEM_CPML)
      for (int c = 0; c < 3; ++c) f.W[c] = h ? WB_[c] : WD_[c];
    for (int a = 0; a < 3; ++a) {
      f.ax[a] = h ? axb_[a] : axd_[a];
      f.n[a] = n_[a];
      f.pml_lo[a] = lo_[a];
      f.pml_hi[a] = hi_[a];
    }
    f.pitch = pitch_;
    f.plane = plane_;
    f.origin = origin_;
    return f;
  }

  kh::DispFixParams<T> disp_params(const kh::HalfStepParams<T>& pe) const {
    kh::DispFixParams<T> d;
    std::memset(&d, 0, sizeof(d));
    d.nx = n_[0];
    d.ny = n_[1];
    d.nz = n_[2];
    d.pitch = pitch_;
    d.plane = plane_;
    d.origin = origin_;
    d.total = total_;
    d.cell_class = cls_;
    d.nxb = nxb_;
    d.list = disp_list_;
    d.n_list = n_disp_list_;
    d.chi3 = chi3_;
    for (int c = 0; c < 3; ++c) {
      d.D[c] = D_[c];
      d.E[c] = E_[c];
      d.m_inv[c] = eps_[c];
    }
    d.m_scalar = T(d_.eps_inv);
    d.npoles = pe.npoles;
    for (int q = 0; q < kh::kMaxPoles; ++q) d.poles[q] = pe.poles[q];
    for (int c = 0; c < 3; ++c) {
      d.W[c] = pe.cpml ? pe.W[c] : nullptr;  // the CPU-path semantics do not use the pass in a CPML region
      d.ax[c] = pe.ax[c];
      d.pml_lo[c] = pe.pml_lo[c];
      d.pml_hi[c] = pe.pml_hi[c];
    }
    d.slot_off = slot_off_;
    d.ent_src = ent_src_;
    d.ent_comp = ent_comp_;
    d.ent_amp = ent_amp_;
    d.n_slots = nslots_;
    d.n_ent = int(ent_amp_h_.size());
    d.n_src = nsrc_;
    return d;
  }

  kh::WrapParams<T> wrap_params(bool h) const {
    kh::WrapParams<T> w;
    std::memset(&w, 0, sizeof(w));
    for (int a = 0; a < 3; ++a) w.n[a] = n_[a];
    w.pitch = pitch_;
    w.plane = plane_;
    w.origin = origin_;
    w.total = total_;
    w.periodic = uint32_t(d_.periodic);
    for (int c = 0; c < 3; ++c) w.O[c] = h ? H_[c] : E_[c];
    w.chi3 = h ? nullptr : chi3_;
    return w;
  }

  kh::HalfStepParams<T> base_params(bool h) const {
    kh::HalfStepParams<T> p;
    std::memset(&p, 0, sizeof(p));
    p.nx = n_[0];
    p.ny = n_[1];
    p.nz = n_[2];
    p.pitch = pitch_;
    p.plane = plane_;
    p.origin = origin_;
    p.total = total_;
    p.nxb = nxb_;
    p.zplanes = zplanes_;
    p.xprefetch = xprefetch_;
    p.xpf_dist = xpf_dist_;
    p.dt = dt_;
    for (int a = 0; a < 3; ++a) {
      p.inv_d[a] = T(1) / delta_[a];
      p.cd[a] = dt_ * p.inv_d[a];
    }
    for (int c = 0; c < 3; ++c) {
      p.A[c] = h ? E_[c] : H_[c];
      p.O[c] = h ? H_[c] : E_[c];
      p.Ts[c] = h ? B_[c] : D_[c];
      p.U[c] = h ? UB_[c] : UD_[c];
      p.W[c] = h ? WB_[c] : WD_[c];
      p.C[c] = h ? CB_[c] : CD_[c];
      p.m_inv[c] = h ? mu_[c] : eps_[c];
      p.msig[c] = h ? msigb_[c] : msigd_[c];
      p.ax[c] = h ? axb_[c] : axd_[c];
      p.pml_lo[c] = lo_[c];
      p.pml_hi[c] = hi_[c];
    }
    p.cpml = d_.semantics == KH_SEM_CPML ? 1 : 0;
    p.m_scalar = h ? T(d_.mu_inv) : T(d_.eps_inv);
    p.sigma_region_mask = h ? sigmask_b_ : sigmask_d_;
    p.tile_bits = h ? tbits_h_ : tbits_e_;
    p.n_tile_words = p.tile_bits ? (long long)((n_[2] + 63) / 64) * n_[1] * nxb_ : 0;
    p.n_slots = nslots_;
    p.n_ent = int(ent_amp_h_.size());
    p.n_src = nsrc_;
    p.cell_class = cls_;
    p.err = err_dev_;
    p.stall_tx = stall_tx_;
    p.periodic = h ? 0u : uint32_t(d_.periodic);
    p.slot_off = slot_off_;
    p.ent_src = ent_src_;
    p.ent_comp = ent_comp_;
    p.ent_amp = ent_amp_;
    p.chi3 = h ? nullptr : chi3_;
    p.npoles = h ? 0 : int(poles_d_.size());
    if (!h)
      for (size_t q = 0; q < poles_d_.size(); ++q) {
        const PoleD& d = poles_d_[q];
        kh::PoleParams<T>& pp = p.poles[q];
        pp.gamma1_inv = T(d.c.gamma1_inv);
        pp.gamma1 = T(d.c.gamma1);
        pp.coeff_p = T(2) - T(d.c.omega0_dt_sq);
        pp.drive = d.c.is_drude ? T(d.c.drude_coeff) : T(d.c.sigma_omega0_dt_sq);
        pp.is_drude = d.c.is_drude;
        pp.sigma = d.sigma;
        for (int c = 0; c < 3; ++c) {
          pp.P[c] = d.P[c];
          pp.Pprev[c] = d.Pp[c];
        }
      }
    return p;
  }

  kh_sim_desc d_;
  int n_[3];
  T dt_, delta_[3];
  long long pitch_, plane_, origin_, total_;
  int nxb_;
  int lo_[3] = {0, 0, 0}, hi_[3] = {0, 0, 0};
  bool pml_axis_[3] = {false, false, false};
  uint32_t sigmask_b_ = 0, sigmask_d_ = 0;
  bool prepared_ = false;

  std::vector<T> sigb_h_[3], sigd_h_[3], eps_h_[3], mu_h_[3], msigd_h_[3], msigb_h_[3], chi3_h_;
  // ε⁻¹ / μ⁻¹ attached with kh_sim_attach_material: the caller's array, read at prepare
  struct Attached {
    const void* ptr = nullptr;
    int dtype = KH_F32;
  };
  Attached att_eps_[3], att_mu_[3];
  std::vector<PoleH> poles_;
  std::vector<PoleD> poles_d_;
  std::vector<SrcH> srcs_;
  std::vector<Mon> mons_;
  std::vector<Hist> hists_;
  std::vector<kh::GeomObj> geo_;
  bool geo_set_ = false;
  double geo_bg_ = 1.0, geo_origin_[3] = {0, 0, 0};
  int geo_smooth_ = KH_SMOOTH_NONE;
  bool graphs_on_ = false;
  int align_ = 1, batch_len_ = 512;
  int64_t graph_misses_ = 0, graph_hits_ = 0;
  cudaStream_t gstream_ = nullptr;
  cudaEvent_t ev_in_ = nullptr, ev_out_ = nullptr;
  std::vector<GraphEntry> graphs_;
  std::vector<std::vector<int64_t>> seen_;  // signatures issued once, not yet captured
  uint64_t graph_clock_ = 0;
  int64_t graph_replays_ = 0;
  int nsrc_ = 0;
  bool has_src_[2] = {false, false};         // [E half, H half]
  bool src_lean_ok_[2] = {true, true};
  bool src_on_dispersive_ = false;  // an E source cell carries χ3 or a pole
  bool special_in_region_[2] = {false, false};
  long long* slot_cell_ = nullptr;
  int nslots_ = 0;
  int* err_dev_ = nullptr;
  // KHRONOS_GB300_TEST_STALL=1 at prepare: the TMA half-step kernels wait for
  // bytes that never arrive and give up (tests of the timeout status only)
  uint32_t stall_tx_ = 0;
  bool use_tma_ = true;
  bool dft_batch_ = true;
  bool disp_fix_ = false;      // χ3 / pole cells by the dispersive-cell pass after a LEAN E launch
  uint32_t* disp_list_ = nullptr;  // its row-segment list (DispFixParams::list)
  int n_disp_list_ = 0;
  int zplanes_ = 10;
  int xprefetch_ = 2;        // x-CPML state prefetch mode (HalfStepParams::xprefetch)
  int xpf_dist_ = 3;
  int tma_slots_ = 0;  // SMs × resident TMA-kernel CTAs per SM
  kh::TmaMaps maps_h_, maps_e_;

  std::vector<void*> allocs_;
  std::vector<std::pair<void*, size_t>> state_;
  T *E_[3] = {}, *H_[3] = {}, *B_[3] = {}, *D_[3] = {};
  T *UB_[3] = {}, *UD_[3] = {}, *WB_[3] = {}, *WD_[3] = {}, *CB_[3] = {}, *CD_[3] = {};
  T *eps_[3] = {}, *mu_[3] = {}, *msigd_[3] = {}, *msigb_[3] = {}, *chi3_ = nullptr;
  kh::AxisCoef<T> *axb_[3] = {}, *axd_[3] = {};
  uint32_t* cls_ = nullptr;
  uint64_t *tbits_e_ = nullptr, *tbits_h_ = nullptr;
  int *slot_off_ = nullptr, *ent_src_ = nullptr, *ent_comp_ = nullptr;
  Cplx<T>* ent_amp_ = nullptr;
  kh::SlotPack<T>* slot_pack_ = nullptr;
  std::vector<int> slot_off_h_, ent_src_h_, ent_comp_h_;  // host copies of the source table
  std::vector<Cplx<T>> ent_amp_h_;  // host copy of ent_amp_
  // per source: (amplitude element index, entry index) of every injected cell
  std::vector<std::vector<std::pair<long long, int>>> src_ent_;

  void* tab_dev_[2] = {nullptr, nullptr};
  void* pinned_[2] = {nullptr, nullptr};
  size_t tab_cap_ = 0;  // bytes per buffer
  int tab_par_ = 0;
  bool copy_pending_[2] = {false, false};
  cudaEvent_t copy_ev_[2] = {nullptr, nullptr};
  cudaEvent_t batch_done_ = nullptr;
  bool batch_recorded_ = false;
  int64_t device_bytes_ = 0;
  cudaStream_t last_stream_ = nullptr;
  std::vector<cudaEvent_t> events_;

  int64_t timestep_ = 0;
  bool sources_active_ = true, has_cw_ = false;
  double last_time_ = 0;
};

}  // namespace

extern "C" {

const char* kh_version(void) { return kVersion; }

kh_status kh_device_alloc_count(int64_t* out) {
  if (!out) return KH_ERR_INVALID;
  *out = kh_host::g_alloc_count.load();
  return KH_OK;
}

kh_status kh_device_info(int32_t* sm_count, int32_t* cc_major, int32_t* cc_minor) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return KH_ERR_CUDA;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) return KH_ERR_CUDA;
  if (sm_count) *sm_count = prop.multiProcessorCount;
  if (cc_major) *cc_major = prop.major;
  if (cc_minor) *cc_minor = prop.minor;
  return KH_OK;
}

kh_status kh_sim_create(const kh_sim_desc* desc, kh_sim** out) {
  if (!desc || !out) return KH_ERR_INVALID;
  *out = nullptr;
  if (desc->n[0] <= 0 || desc->n[1] <= 0 || desc->n[2] <= 0) return KH_ERR_INVALID;
  if (desc->dtype != KH_F32 && desc->dtype != KH_F64) return KH_ERR_INVALID;
  if (!(desc->dt > 0) || !(desc->delta[0] > 0) || !(desc->delta[1] > 0) || !(desc->delta[2] > 0))
    return KH_ERR_INVALID;
  kh_sim* s = new (std::nothrow) kh_sim();
  if (!s) return KH_ERR_OOM;
  if (desc->dtype == KH_F32) s->impl.reset(new Sim<float>(*desc));
  else s->impl.reset(new Sim<double>(*desc));
  *out = s;
  return KH_OK;
}

void kh_sim_destroy(kh_sim* sim) { delete sim; }

const char* kh_last_error(const kh_sim* sim) {
  if (!sim) return "null handle";
  return sim->impl->err.c_str();
}

kh_status kh_sim_set_material(kh_sim* sim, int32_t kind, int32_t comp, const double* values) {
  if (!sim) return KH_ERR_INVALID;
  return sim->impl->set_material(kind, comp, values);
}

kh_status kh_sim_attach_material(kh_sim* sim, int32_t kind, int32_t comp, const void* values, int32_t dtype) {
  if (!sim) return KH_ERR_INVALID;
  return sim->impl->attach_material(kind, comp, values, dtype);
}

kh_status kh_sim_add_pole(kh_sim* sim, const kh_pole_coeffs* coeffs, const double* sigma) {
  if (!sim || !coeffs) return KH_ERR_INVALID;
  return sim->impl->add_pole(*coeffs, sigma);
}

kh_status kh_sim_add_source(kh_sim* sim, const kh_source_desc* src) {
  if (!sim || !src) return KH_ERR_INVALID;
  return sim->impl->add_source(*src);
}

kh_status kh_sim_add_dft_monitor(kh_sim* sim, int32_t component, const int32_t start[3],
                                 const int32_t dims[3], int32_t nfreq, const double* freqs,
                                 int32_t decimation, int32_t* out_id) {
  if (!sim) return KH_ERR_INVALID;
  return sim->impl->add_monitor(component, start, dims, nfreq, freqs, decimation, out_id);
}

kh_status kh_sim_prepare(kh_sim* sim) {
  if (!sim) return KH_ERR_INVALID;
  return sim->impl->prepare();
}

kh_status kh_sim_step(kh_sim* sim, int64_t nsteps, void* stream) {
  if (!sim) return KH_ERR_INVALID;
  return sim->impl->step(nsteps, static_cast<cudaStream_t>(stream));
}

kh_status kh_sim_synchronize(kh_sim* sim) {
  if (!sim) return KH_ERR_INVALID;
  if (!sim->impl->is_prepared()) return KH_OK;
  return sim->impl->wait_idle();
}

kh_status kh_sim_timestep(const kh_sim* sim, int64_t* out) {
  if (!sim || !out) return KH_ERR_INVALID;
  *out = sim->impl->timestep();
  return KH_OK;
}

kh_status kh_sim_sources_active(const kh_sim* sim, int32_t* out) {
  if (!sim || !out) return KH_ERR_INVALID;
  *out = sim->impl->sources_active();
  return KH_OK;
}

kh_status kh_sim_launch_count(const kh_sim* sim, int64_t* out) {
  if (!sim || !out) return KH_ERR_INVALID;
  *out = sim->impl->launches;
  return KH_OK;
}

kh_status kh_debug_bounds(int64_t* count, int64_t* index, int32_t* site) {
  if (!count || !index || !site) return KH_ERR_INVALID;
  *count = 0;
  *index = 0;
  *site = 0;
#ifdef KH_DEBUG_BOUNDS
  if (cudaDeviceSynchronize() != cudaSuccess) return KH_ERR_CUDA;
  void (*readers[])(unsigned long long*, long long*, int*) = {kh::dbg_read_tma, kh::dbg_read_kernels};
  for (auto rd : readers) {
    unsigned long long c = 0;
    long long ix = 0;
    int st = 0;
    rd(&c, &ix, &st);
    if (c && !*count) {
      *index = ix;
      *site = st;
    }
    *count += int64_t(c);
  }
  return KH_OK;
#else
  return KH_ERR_UNSUPPORTED;
#endif
}

kh_status kh_sim_get_field(kh_sim* sim, int32_t component, double* out) {
  if (!sim) return KH_ERR_INVALID;
  return sim->impl->get_field(component, out);
}

kh_status kh_sim_field_view(kh_sim* sim, int32_t component, kh_field_view* out) {
  if (!sim) return KH_ERR_INVALID;
  return sim->impl->field_view(component, out);
}

kh_status kh_sim_read_dft(kh_sim* sim, int32_t monitor_id, double* out) {
  if (!sim) return KH_ERR_INVALID;
  return sim->impl->read_dft(monitor_id, out);
}

kh_status kh_sim_monitor_info(const kh_sim* sim, int32_t monitor_id, int32_t dims[3], int32_t* nfreq) {
  if (!sim || !dims || !nfreq) return KH_ERR_INVALID;
  return sim->impl->monitor_info(monitor_id, dims, nfreq);
}

kh_status kh_sim_flux(kh_sim* sim, const int32_t ids[4], int32_t normal_axis, double dA, double* out) {
  if (!sim) return KH_ERR_INVALID;
  return sim->impl->flux(ids, normal_axis, dA, out);
}

kh_status kh_sim_flux_static(kh_sim* sim, const int32_t ids[4], int32_t normal_axis, double dA,
                             double* out) {
  if (!sim) return KH_ERR_INVALID;
  return sim->impl->flux_static(ids, normal_axis, dA, out);
}

kh_status kh_sim_memory_bytes(const kh_sim* sim, int64_t* estimate, int64_t* allocated) {
  if (!sim) return KH_ERR_INVALID;
  if (estimate) *estimate = sim->impl->estimate_bytes();
  if (allocated) *allocated = sim->impl->device_bytes();
  return KH_OK;
}

kh_status kh_sim_reset(kh_sim* sim) {
  if (!sim) return KH_ERR_INVALID;
  return sim->impl->reset();
}

kh_status kh_sim_state_bytes(const kh_sim* sim, int64_t* out) {
  if (!sim || !out) return KH_ERR_INVALID;
  *out = sim->impl->state_bytes();
  return KH_OK;
}

kh_status kh_sim_export_state(kh_sim* sim, void* host_dst, int64_t bytes) {
  if (!sim) return KH_ERR_INVALID;
  return sim->impl->export_state(host_dst, bytes);
}

kh_status kh_sim_import_state(kh_sim* sim, const void* host_src, int64_t bytes) {
  if (!sim) return KH_ERR_INVALID;
  return sim->impl->import_state(host_src, bytes);
}

kh_status kh_sim_model_bytes_split(const kh_sim* sim, double* h_half, double* e_half, double* dft) {
  if (!sim || !h_half || !e_half || !dft) return KH_ERR_INVALID;
  sim->impl->model_split(*h_half, *e_half, *dft);
  return KH_OK;
}

kh_status kh_sim_step_timed(kh_sim* sim, int64_t nsteps, void* stream, double* h_ms, double* e_ms,
                            double* dft_ms) {
  if (!sim) return KH_ERR_INVALID;
  return sim->impl->step_timed(nsteps, static_cast<cudaStream_t>(stream), h_ms, e_ms, dft_ms);
}

kh_status kh_sim_model_bytes_per_step(const kh_sim* sim, double* out) {
  if (!sim || !out) return KH_ERR_INVALID;
  *out = sim->impl->model_bytes_per_step();
  return KH_OK;
}

kh_status kh_sim_set_geometry(kh_sim* sim, const kh_object* objects, int32_t n, double background_eps,
                              const double origin[3], int32_t smoothing) {
  if (!sim) return KH_ERR_INVALID;
  return sim->impl->set_geometry(objects, n, background_eps, origin, smoothing);
}

kh_status kh_sim_read_material(kh_sim* sim, int32_t kind, int32_t comp, double* out) {
  if (!sim) return KH_ERR_INVALID;
  return sim->impl->read_material(kind, comp, out);
}

kh_status kh_sim_graph_replays(const kh_sim* sim, int64_t* out) {
  if (!sim || !out) return KH_ERR_INVALID;
  *out = sim->impl->graph_replays();
  return KH_OK;
}

kh_status kh_sim_add_history_monitor(kh_sim* sim, int32_t component, const int32_t start[3],
                                     const int32_t dims[3], int64_t capacity_steps, int32_t* out_id) {
  if (!sim) return KH_ERR_INVALID;
  return sim->impl->add_history(component, start, dims, capacity_steps, out_id);
}

kh_status kh_sim_update_material_box(kh_sim* sim, int32_t kind, int32_t comp, const int32_t start[3],
                                     const int32_t dims[3], const double* values) {
  if (!sim) return KH_ERR_INVALID;
  return sim->impl->update_material_box(kind, comp, start, dims, values);
}

kh_status kh_sim_update_source(kh_sim* sim, int32_t index, const double* amp, int64_t table_len,
                               const double* table, double cutoff) {
  if (!sim) return KH_ERR_INVALID;
  return sim->impl->update_source(index, amp, table_len, table, cutoff);
}

}  // extern "C"
