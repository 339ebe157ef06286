// ORACLE — test infrastructure, not product code.
//
// CPU restatement of Khronos.jl's CPU-backend FDTD step loop (the
// KernelAbstractions path that `step!` takes when backend_engine isa CPU).
// It exists only to check the CUDA library: tests/, __graft_entry__.smoke()
// and bench.py's CPU-baseline leg call it; nothing in the product links it.
//
// Parity status: setup functions are pinned by the reference's own known-answer
// tests (grid volumes, interpolation weights, ADE coefficients: see
// tests/test_oracle_kats.py).  Field and DFT values are "parity unpinned": the
// reference ships no field golden vectors and Julia is not available to run it,
// so this restatement is the pin for them.
//
// The structure follows the reference file by file:
//   step!                      src/Kernels/Kernels.jl:20-88
//   chunk plan (PML grid)      src/Chunking.jl:622-738, 907-966
//   aux allocation rule        src/Chunking.jl:1069-1146
//   σ slicing per chunk        src/Chunking.jl:1333-1378
//   interior fused kernel      src/Kernels/ReferenceKernels.jl:323-362
//   PML curl kernel            src/Kernels/ReferenceKernels.jl:276-313
//   PML update kernel          src/Kernels/ReferenceKernels.jl:468-512
//   curl cascade dispatch      src/Kernels/Helpers.jl:30-270
//   update dispatch            src/Kernels/Helpers.jl:313-366, 411-416
//   sources                    src/Sources/Sources.jl:288-357, TimeSources.jl:40-132
//   DFT monitors               src/Monitors/Monitors.jl:274-379
//   χ3 correction              src/Kernels/Dispersive.jl:127-173
//   ADE poles                  src/Kernels/Dispersive.jl:25-117, 186-228
//   periodic halo wrap         src/Chunking.jl:1751-1768, 2138-2172 (single chunk)
// Field arrays are one global domain; the reference's multi-chunk halo
// exchange (Chunking.jl:2082-2214) copies exactly the neighbour values a
// single domain reads, so per-region loops over global arrays reproduce it.
//
// Build: see oracle/Makefile (-O3 -fopenmp -ffp-contract=off so that no FMA
// changes the reference's rounding).

#include "../include/khronos_gb300.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <memory>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr int kNone = -1;

// A full-domain field array with the reference's raw layout: one ghost layer
// on each side plus room for the staggered N+1 layer (raw index N+2) and its
// ghost, all held at zero unless a kernel writes them.
template <class T>
struct Field3 {
  int sx = 0, sy = 0, sz = 0;
  std::vector<T> v;
  void alloc(int nx, int ny, int nz) {
    sx = nx + 3; sy = ny + 3; sz = nz + 3;
    v.assign(size_t(sx) * sy * sz, T(0));
  }
  bool ok() const { return !v.empty(); }
  // 1-based raw indices as in the Julia arrays (interior = 2..N+1).
  T& r(int fx, int fy, int fz) { return v[(size_t(fz - 1) * sy + (fy - 1)) * sx + (fx - 1)]; }
  T r(int fx, int fy, int fz) const { return v[(size_t(fz - 1) * sy + (fy - 1)) * sx + (fx - 1)]; }
};

// Center-range (Nx, Ny, Nz) geometry array, 1-based gidx like the reference.
template <class T>
struct Geo3 {
  int nx = 0, ny = 0, nz = 0;
  std::vector<T> v;
  bool ok() const { return !v.empty(); }
  T g(int ix, int iy, int iz) const { return v[(size_t(iz - 1) * ny + (iy - 1)) * nx + (ix - 1)]; }
};

// Region-local auxiliary array (CPML C/U/W), cell-local, no ghosts.
template <class T>
struct Aux3 {
  int nx = 0, ny = 0, nz = 0, ox = 0, oy = 0, oz = 0;
  std::vector<T> v;
  bool ok() const { return !v.empty(); }
  void alloc(int x0, int y0, int z0, int x1, int y1, int z1) {
    ox = x0; oy = y0; oz = z0; nx = x1 - x0 + 1; ny = y1 - y0 + 1; nz = z1 - z0 + 1;
    v.assign(size_t(nx) * ny * nz, T(0));
  }
  // Global 1-based Center indices.
  T& a(int ix, int iy, int iz) { return v[(size_t(iz - oz) * ny + (iy - oy)) * nx + (ix - ox)]; }
};

template <class T>
struct Region {
  int s[3], e[3];     // 1-based inclusive Center bounds
  bool pml[3];
  bool any_pml;
  // Region σ arrays per axis (value at global cell index), present on every
  // axis of a PML region (zeros on its non-PML axes), absent otherwise
  // (Chunking.jl:1355-1378).
  std::vector<T> sig_b[3], sig_d[3];
  Aux3<T> CB[3], UB[3], WB[3], CD[3], UD[3], WD[3];
};

struct Source {
  int comp;
  int start[3], dims[3];
  std::vector<std::complex<double>> amp;  // already rounded to T, stored as double
  int kind;
  double fcen, width, peak, cutoff;
  std::vector<std::complex<double>> table;
};

template <class T>
struct Monitor {
  int comp;
  int start[3], dims[3];
  std::vector<T> freqs;
  int decimation;
  std::vector<std::complex<T>> F;  // (dims..., nf), x fastest
};

struct Pole {
  kh_pole_coeffs c;
};

template <class T>
class Oracle {
 public:
  explicit Oracle(const kh_sim_desc& d) : desc(d) {
    for (int a = 0; a < 3; ++a) n[a] = d.n[a];
    dt = T(d.dt);
    for (int a = 0; a < 3; ++a) delta[a] = T(d.delta[a]);
    for (int a = 0; a < 3; ++a) {
      sigb[a].assign(n[a], T(0));
      sigd[a].assign(n[a], T(0));
      if (d.sigma_b[a]) for (int i = 0; i < n[a]; ++i) sigb[a][i] = T(d.sigma_b[a][i]);
      if (d.sigma_d[a]) for (int i = 0; i < n[a]; ++i) sigd[a][i] = T(d.sigma_d[a][i]);
    }
    eps_inv = T(d.eps_inv);
    mu_inv = T(d.mu_inv);
    for (int c = 0; c < 3; ++c) {
      E[c].alloc(n[0], n[1], n[2]);
      H[c].alloc(n[0], n[1], n[2]);
      B[c].alloc(n[0], n[1], n[2]);
      D[c].alloc(n[0], n[1], n[2]);
    }
  }

  std::string err;

  int set_material(int kind, int comp, const double* vals) {
    if (prepared) { err = "set_material after prepare"; return KH_ERR_INVALID; }
    Geo3<T>* g = nullptr;
    if (kind == KH_MAT_CHI3) g = &chi3;
    else if (comp < 0 || comp > 2) { err = "bad component"; return KH_ERR_INVALID; }
    else if (kind == KH_MAT_EPS_INV) g = &epsx[comp];
    else if (kind == KH_MAT_MU_INV) g = &mux[comp];
    else if (kind == KH_MAT_SIGMA_D) g = &sigD[comp];
    else if (kind == KH_MAT_SIGMA_B) g = &sigB[comp];
    else { err = "bad material kind"; return KH_ERR_INVALID; }
    g->nx = n[0]; g->ny = n[1]; g->nz = n[2];
    g->v.resize(size_t(n[0]) * n[1] * n[2]);
    for (size_t q = 0; q < g->v.size(); ++q) g->v[q] = T(vals[q]);
    return KH_OK;
  }

  int add_pole(const kh_pole_coeffs& c, const double* sigma) {
    if (prepared) { err = "add_pole after prepare"; return KH_ERR_INVALID; }
    poles.push_back({c});
    Geo3<T> s; s.nx = n[0]; s.ny = n[1]; s.nz = n[2];
    s.v.resize(size_t(n[0]) * n[1] * n[2]);
    for (size_t q = 0; q < s.v.size(); ++q) s.v[q] = T(sigma[q]);
    pole_sigma.push_back(std::move(s));
    return KH_OK;
  }

  int add_source(const kh_source_desc& s) {
    if (prepared) { err = "add_source after prepare"; return KH_ERR_INVALID; }
    if (s.component < 0 || s.component > 5) { err = "bad source component"; return KH_ERR_INVALID; }
    Source q;
    q.comp = s.component;
    for (int a = 0; a < 3; ++a) { q.start[a] = s.start[a]; q.dims[a] = s.dims[a]; }
    size_t cnt = size_t(s.dims[0]) * s.dims[1] * s.dims[2];
    q.amp.resize(cnt);
    for (size_t i = 0; i < cnt; ++i)  // complex_backend_number.(amplitude) (Sources.jl:80)
      q.amp[i] = std::complex<double>(double(T(s.amp[2 * i])), double(T(s.amp[2 * i + 1])));
    q.kind = s.time_kind;
    q.fcen = s.fcen; q.width = s.width; q.peak = s.peak_time; q.cutoff = s.cutoff;
    if (s.time_kind == KH_TIME_TABLE) {
      q.table.resize(size_t(2 * s.table_len));
      for (int64_t i = 0; i < 2 * s.table_len; ++i)
        q.table[i] = std::complex<double>(s.table[2 * i], s.table[2 * i + 1]);
    }
    sources.push_back(std::move(q));
    return KH_OK;
  }

  int add_monitor(int comp, const int32_t* st, const int32_t* dm, int nf, const double* f, int dec,
                  int32_t* id) {
    if (prepared) { err = "add_monitor after prepare"; return KH_ERR_INVALID; }
    Monitor<T> m;
    m.comp = comp;
    for (int a = 0; a < 3; ++a) { m.start[a] = st[a]; m.dims[a] = dm[a]; }
    for (int i = 0; i < nf; ++i) m.freqs.push_back(T(f[i]));  // backend_array(frequencies)
    m.decimation = dec;
    m.F.assign(size_t(dm[0]) * dm[1] * dm[2] * nf, std::complex<T>(0, 0));
    monitors.push_back(std::move(m));
    *id = int32_t(monitors.size() - 1);
    return KH_OK;
  }

  int prepare() {
    build_regions();
    for (auto& r : regions) {
      if (!r.any_pml) continue;
      // PhysicsFlags.has_sigma_{B,D} of the region (Chunking.jl:150-247): a
      // conductive object overlaps the region; here, a nonzero conductivity
      // value inside the region box.
      const bool needC_b = region_has_nonzero(r, sigB), needC_d = region_has_nonzero(r, sigD);
      for (int c = 0; c < 3; ++c) {
        const int nx_ = (c + 1) % 3, pv = (c + 2) % 3;
        // Chunking.jl:1110-1131: C iff conductivity and PML on next/prev;
        // U iff PML on next; W iff PML on own axis.
        bool hasC_b = needC_b && (r.pml[nx_] || r.pml[pv]);
        bool hasC_d = needC_d && (r.pml[nx_] || r.pml[pv]);
        bool hasU = r.pml[nx_], hasW = r.pml[c];
        auto mk = [&](Aux3<T>& A, bool on) { if (on) A.alloc(r.s[0], r.s[1], r.s[2], r.e[0], r.e[1], r.e[2]); };
        mk(r.CB[c], hasC_b); mk(r.UB[c], hasU); mk(r.WB[c], hasW);
        mk(r.CD[c], hasC_d); mk(r.UD[c], hasU); mk(r.WD[c], hasW);
        if (desc.semantics == KH_SEM_CPML && (hasC_b || hasC_d || sigB[c].ok() || sigD[c].ok())) {
          err = "the CUDA-path CPML kernels take no material conductivity (CUDAKernels.jl:122-124)";
          return KH_ERR_UNSUPPORTED;
        }
        // Combinations for which the reference's generic_curl! has no method
        // (Helpers.jl:39-270): C without U, or a material σ array with U but no C.
        bool sigmaB_arr = sigB[c].ok(), sigmaD_arr = sigD[c].ok();
        if ((hasC_b && !hasU) || (hasC_d && !hasU) || (!hasC_b && hasU && sigmaB_arr) ||
            (!hasC_d && hasU && sigmaD_arr)) {
          err = "material conductivity with this PML region combination has no generic_curl! method in the reference";
          return KH_ERR_UNSUPPORTED;
        }
      }
      for (int a = 0; a < 3; ++a) {
        r.sig_b[a].assign(n[a], T(0));
        r.sig_d[a].assign(n[a], T(0));
        if (r.pml[a]) { r.sig_b[a] = sigb[a]; r.sig_d[a] = sigd[a]; }
      }
    }
    // Source arrays S: allocated for each source component (Chunking.jl:1133-1139).
    for (auto& s : sources) {
      if (!S[s.comp].ok()) S[s.comp].alloc(n[0], n[1], n[2]);
    }
    if (!poles.empty()) for (int c = 0; c < 3; ++c) PD[c].alloc(n[0], n[1], n[2]);
    P.resize(poles.size()); Pprev.resize(poles.size());
    for (size_t p = 0; p < poles.size(); ++p) for (int c = 0; c < 3; ++c) {
      P[p][c].alloc(n[0], n[1], n[2]);
      Pprev[p][c].alloc(n[0], n[1], n[2]);
    }
    // last_source_time (TimeSources.jl:40-47): max cutoff; a CW source makes
    // get_cutoff throw and `step!` keeps sources active forever (Kernels.jl:27-35).
    has_cw = false;
    last_time = -INFINITY;
    for (auto& s : sources) {
      if (s.kind == KH_TIME_CW) has_cw = true;
      else last_time = std::max(last_time, double(T(s.cutoff)));
    }
    prepared = true;
    return KH_OK;
  }

  void step() {
    // round_time(sim) = Float64(timestep * Δt) with Δt in the run's precision
    const double t = double(T(timestep) * dt);
    if (sources_active && !has_cw && !sources.empty() && t > last_time) sources_active = false;
    const bool sa = sources_active;
    if (sa) inject(true, t);
    half_step(true, sa);
    exchange_periodic(true);  // exchange_halos!(:H) ends step_H_fused! (Kernels.jl:294)
    update_monitors(true, t);
    const double tE = t + double(dt / T(2));
    if (sa) inject(false, tE);
    half_step(false, sa);
    exchange_periodic(false);  // exchange_halos!(:E) ends step_E_fused! (Kernels.jl:452)
    chi3_correction();
    polarization();
    update_monitors(false, tE);
    ++timestep;
  }

  // ---------------- results ----------------
  void get_field(int comp, double* out) const {
    const Field3<T>& A = comp < 3 ? E[comp] : H[comp - 3];
    int cd[3];
    comp_dims(comp, cd);
    for (int k = 0; k < cd[2]; ++k)
      for (int j = 0; j < cd[1]; ++j)
        for (int i = 0; i < cd[0]; ++i)
          out[(size_t(k) * cd[1] + j) * cd[0] + i] = double(A.r(i + 2, j + 2, k + 2));
  }

  void comp_dims(int comp, int* cd) const {  // utils.jl:26-37
    static const int add[6][3] = {{0, 1, 1}, {1, 0, 1}, {1, 1, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int a = 0; a < 3; ++a) cd[a] = n[a] + add[comp][a];
  }

  kh_sim_desc desc;
  int n[3];
  T dt, delta[3], eps_inv, mu_inv;
  std::vector<T> sigb[3], sigd[3];
  Field3<T> E[3], H[3], B[3], D[3], S[6], PD[3];
  std::vector<std::array<Field3<T>, 3>> P, Pprev;
  Geo3<T> epsx[3], mux[3], sigD[3], sigB[3], chi3;
  std::vector<Pole> poles;
  std::vector<Geo3<T>> pole_sigma;
  std::vector<Source> sources;
  std::vector<Monitor<T>> monitors;
  std::vector<Region<T>> regions;
  int64_t timestep = 0;
  bool sources_active = true, prepared = false, has_cw = false;
  double last_time = 0;

 private:
  // _pml_grid_regions + plan_chunks fallback (Chunking.jl:622-738, 907-966),
  // expressed on the per-axis widths of kh_sim_desc.
  void build_regions() {
    std::vector<std::array<int, 3>> iv[3];  // (start, end, flagged)
    for (int a = 0; a < 3; ++a) {
      int lo = desc.pml_lo[a], hi = desc.pml_hi[a];
      if (lo >= n[a]) { iv[a].push_back({1, n[a], 1}); continue; }
      if (lo > 0) iv[a].push_back({1, lo, 1});
      if (lo + 1 <= n[a] - hi) iv[a].push_back({lo + 1, n[a] - hi, 0});
      if (hi > 0) iv[a].push_back({n[a] - hi + 1, n[a], 1});
    }
    regions.clear();
    for (auto& x : iv[0]) for (auto& y : iv[1]) for (auto& z : iv[2]) {
      Region<T> r;
      r.s[0] = x[0]; r.e[0] = x[1]; r.pml[0] = x[2];
      r.s[1] = y[0]; r.e[1] = y[1]; r.pml[1] = y[2];
      r.s[2] = z[0]; r.e[2] = z[1]; r.pml[2] = z[2];
      r.any_pml = r.pml[0] || r.pml[1] || r.pml[2];
      regions.push_back(std::move(r));
    }
  }

  bool region_has_nonzero(const Region<T>& r, const Geo3<T>* g) const {
    for (int c = 0; c < 3; ++c) {
      if (!g[c].ok()) continue;
      for (int iz = r.s[2]; iz <= r.e[2]; ++iz)
        for (int iy = r.s[1]; iy <= r.e[1]; ++iy)
          for (int ix = r.s[0]; ix <= r.e[0]; ++ix)
            if (g[c].g(ix, iy, iz) != T(0)) return true;
    }
    return false;
  }

  // Single-chunk periodic connections (_add_periodic_connections!,
  // Chunking.jl:1751-1768) as _exchange_halos_local! copies them
  // (Chunking.jl:2138-2172): per periodic axis and component, Julia layer N
  // → ghost 0 and layer 1 → layer N+1, over the Center range 1..N of the
  // other axes (_component_send_range / _component_recv_range clamp it to
  // the component, which it never exceeds).
  void exchange_periodic(bool h) {
    if (!desc.periodic) return;
    for (int a = 0; a < 3; ++a) {
      if (!((desc.periodic >> a) & 1)) continue;
      const int t1 = (a + 1) % 3, t2 = (a + 2) % 3;
      for (int c = 0; c < 3; ++c) {
        Field3<T>& F = h ? H[c] : E[c];
        for (int v = 2; v <= n[t2] + 1; ++v)
          for (int u = 2; u <= n[t1] + 1; ++u) {
            int g_lo[3], s_hi[3], g_hi[3], s_lo[3];
            g_lo[t1] = s_hi[t1] = g_hi[t1] = s_lo[t1] = u;
            g_lo[t2] = s_hi[t2] = g_hi[t2] = s_lo[t2] = v;
            g_lo[a] = 1; s_hi[a] = n[a] + 1; g_hi[a] = n[a] + 2; s_lo[a] = 2;
            F.r(g_lo[0], g_lo[1], g_lo[2]) = F.r(s_hi[0], s_hi[1], s_hi[2]);
            F.r(g_hi[0], g_hi[1], g_hi[2]) = F.r(s_lo[0], s_lo[1], s_lo[2]);
          }
      }
    }
  }

  const Field3<T>& src_field(bool h, int c) const { return h ? E[c] : H[c]; }

  // curl_x!/curl_y!/curl_z! with d_dx!… (Helpers.jl:283-298); s = +1 for the
  // H half-step (curl E → B), -1 for the E half-step (curl H → D).
  T curl(bool h, int c, int fx, int fy, int fz) const {
    const int s = h ? 1 : -1;
    const Field3<T>& Ax = src_field(h, 0);
    const Field3<T>& Ay = src_field(h, 1);
    const Field3<T>& Az = src_field(h, 2);
    const T ix = T(1) / delta[0], iy = T(1) / delta[1], iz = T(1) / delta[2];
    if (c == 0) {
      T dz = iz * (Ay.r(fx, fy, fz + s) - Ay.r(fx, fy, fz));
      T dy = iy * (Az.r(fx, fy + s, fz) - Az.r(fx, fy, fz));
      return dt * (dz - dy);
    } else if (c == 1) {
      T dx = ix * (Az.r(fx + s, fy, fz) - Az.r(fx, fy, fz));
      T dz = iz * (Ax.r(fx, fy, fz + s) - Ax.r(fx, fy, fz));
      return dt * (dx - dz);
    } else {
      T dy = iy * (Ax.r(fx, fy + s, fz) - Ax.r(fx, fy, fz));
      T dx = ix * (Ay.r(fx + s, fy, fz) - Ay.r(fx, fy, fz));
      return dt * (dy - dx);
    }
  }

  T m_inv(bool h, int c, int ix, int iy, int iz) const {  // get_m_inv, Helpers.jl:411-416
    const Geo3<T>& g = h ? mux[c] : epsx[c];
    return g.ok() ? g.g(ix, iy, iz) : (h ? mu_inv : eps_inv);
  }

  // update_field_from_curl (Helpers.jl:30-33)
  static T ufc(T A, T Bn, const T* Bo, const T* s) {
    if (s) return Bo ? (((T(1) - *s) * A + Bn) - *Bo) / (T(1) + *s) : ((T(1) - *s) * A + Bn) / (T(1) + *s);
    return Bo ? (A + Bn) - *Bo : A + Bn;
  }

  void half_step(bool h, bool sa) {
    for (auto& r : regions) {
      if (!r.any_pml) interior_fused(r, h, sa);
      else pml_curl_update(r, h, sa);
    }
  }

  // step_curl_and_update! (ReferenceKernels.jl:323-362)
  void interior_fused(Region<T>& r, bool h, bool sa) {
    Field3<T>* Tf = h ? B : D;
    Field3<T>* Of = h ? H : E;
#pragma omp parallel for schedule(static)
    for (int iz = r.s[2]; iz <= r.e[2]; ++iz)
      for (int iy = r.s[1]; iy <= r.e[1]; ++iy)
        for (int ix = r.s[0]; ix <= r.e[0]; ++ix) {
          const int fx = ix + 1, fy = iy + 1, fz = iz + 1;
          for (int c = 0; c < 3; ++c) {
            T K = curl(h, c, fx, fy, fz);
            T& Tc = Tf[c].r(fx, fy, fz);
            Tc = Tc + K;
            T net = Tc;
            Field3<T>& Sc = S[(h ? 3 : 0) + c];
            if (sa && Sc.ok()) { net += Sc.r(fx, fy, fz); Sc.r(fx, fy, fz) = T(0); }
            if (!h && PD[c].ok()) net -= PD[c].r(fx, fy, fz);
            Of[c].r(fx, fy, fz) = m_inv(h, c, ix, iy, iz) * net;
          }
        }
  }

  // step_curl! (ReferenceKernels.jl:276-313) followed by update_field!
  // (ReferenceKernels.jl:468-512) on one PML region.
  void pml_curl_update(Region<T>& r, bool h, bool sa) {
    Field3<T>* Tf = h ? B : D;
    Field3<T>* Of = h ? H : E;
    auto& Cc = h ? r.CB : r.CD;
    auto& Uc = h ? r.UB : r.UD;
    auto& Wc = h ? r.WB : r.WD;
    auto& sg = h ? r.sig_b : r.sig_d;
    Geo3<T>* matsig = h ? sigB : sigD;
    // curl stage
#pragma omp parallel for schedule(static)
    for (int iz = r.s[2]; iz <= r.e[2]; ++iz)
      for (int iy = r.s[1]; iy <= r.e[1]; ++iy)
        for (int ix = r.s[0]; ix <= r.e[0]; ++ix) {
          const int fx = ix + 1, fy = iy + 1, fz = iz + 1;
          const int idx[3] = {ix, iy, iz};
          for (int c = 0; c < 3; ++c) {
            const int nx_ = (c + 1) % 3, pv = (c + 2) % 3;
            T K = curl(h, c, fx, fy, fz);
            // get_σD: 0.5·(Δt·σD[gidx]) or nothing (Helpers.jl:278-279)
            bool hasSD = matsig[c].ok();
            T sD = hasSD ? T(0.5) * (dt * matsig[c].g(ix, iy, iz)) : T(0);
            T sn = sg[nx_][idx[nx_] - 1];  // get_σ(σ, i) = σ[2i-1]
            T sp = sg[pv][idx[pv] - 1];
            T& Tv = Tf[c].r(fx, fy, fz);
            bool hasC = Cc[c].ok(), hasU = Uc[c].ok();
            if (desc.semantics == KH_SEM_CPML) {
              // _cuda_pml_BH_kernel!/_cuda_pml_DE_kernel! stages (CUDAKernels.jl:150-281):
              // U with σ_next, T with σ_prev, each whenever its axis is PML here.
              T in_t = K;
              if (r.pml[nx_] && sn != T(0)) {
                T& U = Uc[c].a(ix, iy, iz);
                T u_old = U;
                U = ((T(1) - sn) * u_old + K) / (T(1) + sn);
                in_t = U - u_old;
              }
              if (r.pml[pv] && sp != T(0)) Tv = ((T(1) - sp) * Tv + in_t) / (T(1) + sp);
              else Tv = Tv + in_t;
              continue;
            }
            if (hasC && hasU) {
              T& U = Uc[c].a(ix, iy, iz);
              if (hasSD && sD != T(0)) {  // Helpers.jl:60-67 three-stage cascade
                T& Cv = Cc[c].a(ix, iy, iz);
                T C_old = Cv;
                Cv = ufc(Cv, K, nullptr, &sD);
                T U_old = U;
                U = ufc(U, Cv, &C_old, &sn);
                Tv = ufc(Tv, U, &U_old, &sp);
              } else {  // Helpers.jl:53-59 (σD == 0) and 72-78 (σD nothing)
                T U_old = U;
                U = ufc(U, K, nullptr, &sn);
                Tv = ufc(Tv, U, &U_old, &sp);
              }
            } else if (!hasC && hasU) {  // Helpers.jl:113-139 (σD nothing)
              if (sn == T(0)) {
                Tv = ufc(Tv, K, nullptr, &sp);
              } else {
                T& U = Uc[c].a(ix, iy, iz);
                T U_old = U;
                U = ufc(U, K, nullptr, &sn);
                Tv = ufc(Tv, U, &U_old, &sp);
              }
            } else {  // C and U absent
              if (hasSD) Tv = ufc(Tv, K, nullptr, &sD);  // Helpers.jl:225-240
              else Tv = ufc(Tv, K, nullptr, nullptr);      // Helpers.jl:208-223 drops σ_prev
            }
          }
        }
    // update stage: update_field_generic (Helpers.jl:323-366)
#pragma omp parallel for schedule(static)
    for (int iz = r.s[2]; iz <= r.e[2]; ++iz)
      for (int iy = r.s[1]; iy <= r.e[1]; ++iy)
        for (int ix = r.s[0]; ix <= r.e[0]; ++ix) {
          const int fx = ix + 1, fy = iy + 1, fz = iz + 1;
          const int idx[3] = {ix, iy, iz};
          for (int c = 0; c < 3; ++c) {
            T net = Tf[c].r(fx, fy, fz);
            Field3<T>& Sc = S[(h ? 3 : 0) + c];
            if (sa && Sc.ok()) { net += Sc.r(fx, fy, fz); Sc.r(fx, fy, fz) = T(0); }
            if (!h && PD[c].ok()) net -= PD[c].r(fx, fy, fz);
            const T m = m_inv(h, c, ix, iy, iz);
            const T sc = sg[c][idx[c] - 1];
            T& A = Of[c].r(fx, fy, fz);
            if (Wc[c].ok() && sc != T(0)) {
              T& W = Wc[c].a(ix, iy, iz);
              T W_old = W;
              W = m * net;
              A = (A + (T(1) + sc) * W) - (T(1) - sc) * W_old;
            } else {
              A = m * net;
            }
          }
        }
  }

  // eval_time_source in the run's precision (TimeSources.jl:61-64, 123-132, 178-184).
  std::complex<T> eval_time(const Source& s, double t, bool h_half) const {
    if (s.kind == KH_TIME_GAUSSIAN) {
      T tt = T(t) - T(s.peak);
      if (tt > T(s.cutoff)) return std::complex<T>(0, 0);
      const T two_pi = T(2) * T(M_PI);
      const T w = T(s.width);
      T g = std::exp((-tt) * tt / ((T(2) * w) * w));
      T b = ((-two_pi) * T(s.fcen)) * tt;
      return std::complex<T>(g * std::cos(b), g * std::sin(b));
    } else if (s.kind == KH_TIME_CW) {
      const T two_pi = T(2) * T(M_PI);
      T b = ((-two_pi) * T(s.fcen)) * T(t);
      return std::complex<T>(std::cos(b), std::sin(b));
    } else {
      if (T(t) > T(s.cutoff)) return std::complex<T>(0, 0);
      int64_t step = timestep;
      int64_t q = 2 * step + (h_half ? 0 : 1);
      if (q >= int64_t(s.table.size())) return std::complex<T>(0, 0);
      return std::complex<T>(T(s.table[q].real()), T(s.table[q].imag()));
    }
  }

  // update_magnetic_sources!/update_electric_sources! → update_source! (Sources.jl:330-357)
  void inject(bool h, double t) {
    const int c0 = h ? 3 : 0;
    for (int c = c0; c < c0 + 3; ++c)
      for (auto& s : sources) {
        if (s.comp != c) continue;
        std::complex<T> f = eval_time(s, t, h);
        Field3<T>& A = S[c];
        for (int k = 0; k < s.dims[2]; ++k)
          for (int j = 0; j < s.dims[1]; ++j)
            for (int i = 0; i < s.dims[0]; ++i) {
              const std::complex<double>& a = s.amp[(size_t(k) * s.dims[1] + j) * s.dims[0] + i];
              // real(scalar_amplitude * spatial_amplitude) with Complex{T} operands
              T re = f.real() * T(a.real()) - f.imag() * T(a.imag());
              // raw index = i + offset, offset = start_idx (1-based) → 0-based start + 1
              int fx = i + 1 + s.start[0] + 1, fy = j + 1 + s.start[1] + 1, fz = k + 1 + s.start[2] + 1;
              if (fx < 1 || fy < 1 || fz < 1 || fx > A.sx || fy > A.sy || fz > A.sz) continue;
              A.r(fx, fy, fz) += re;
            }
      }
  }

  // update_monitor(::DFTMonitorData) single-domain form (Monitors.jl:274-379)
  void update_monitors(bool h, double time) {
    for (auto& m : monitors) {
      if ((m.comp >= 3) != h) continue;
      if (m.decimation > 1 && timestep % m.decimation != 0) continue;
      const Field3<T>& A = m.comp < 3 ? E[m.comp] : H[m.comp - 3];
      // complex_backend_number(im * 2 * π * time)
      const T tf_im = T(6.283185307179586 * time);
      const int nf = int(m.freqs.size());
      const size_t ncell = size_t(m.dims[0]) * m.dims[1] * m.dims[2];
      for (int f = 0; f < nf; ++f) {
        T th = m.freqs[f] * tf_im;
        std::complex<T> ph(dt * std::cos(th), dt * std::sin(th));  // dt_scale * exp(i θ)
#pragma omp parallel for schedule(static)
        for (int k = 0; k < m.dims[2]; ++k)
          for (int j = 0; j < m.dims[1]; ++j)
            for (int i = 0; i < m.dims[0]; ++i) {
              T v = A.r(i + 1 + m.start[0] + 1, j + 1 + m.start[1] + 1, k + 1 + m.start[2] + 1);
              size_t q = f * ncell + (size_t(k) * m.dims[1] + j) * m.dims[0] + i;
              m.F[q] += std::complex<T>(ph.real() * v, ph.imag() * v);
            }
      }
    }
  }

  // _chi3_correction_kernel! (Dispersive.jl:127-147)
  void chi3_correction() {
    if (!chi3.ok()) return;
#pragma omp parallel for schedule(static)
    for (int iz = 1; iz <= n[2]; ++iz)
      for (int iy = 1; iy <= n[1]; ++iy)
        for (int ix = 1; ix <= n[0]; ++ix) {
          T c3 = chi3.g(ix, iy, iz);
          if (c3 == T(0)) continue;
          T& ex = E[0].r(ix + 1, iy + 1, iz + 1);
          T& ey = E[1].r(ix + 1, iy + 1, iz + 1);
          T& ez = E[2].r(ix + 1, iy + 1, iz + 1);
          T esq = (ex * ex + ey * ey) + ez * ez;
          T corr = T(1) / (T(1) + c3 * esq);
          ex = ex * corr; ey = ey * corr; ez = ez * corr;
        }
  }

  // step_polarization! (Dispersive.jl:186-228)
  void polarization() {
    if (poles.empty()) return;
#pragma omp parallel for schedule(static)
    for (int iz = 1; iz <= n[2]; ++iz)
      for (int iy = 1; iy <= n[1]; ++iy)
        for (int ix = 1; ix <= n[0]; ++ix)
          for (int c = 0; c < 3; ++c) PD[c].r(ix + 1, iy + 1, iz + 1) = T(0);
    for (size_t p = 0; p < poles.size(); ++p) {
      const kh_pole_coeffs& c = poles[p].c;
      const T g1i = T(c.gamma1_inv), g1 = T(c.gamma1), w0 = T(c.omega0_dt_sq);
      const T sw0 = T(c.sigma_omega0_dt_sq), dc = T(c.drude_coeff);
#pragma omp parallel for schedule(static)
      for (int iz = 1; iz <= n[2]; ++iz)
        for (int iy = 1; iy <= n[1]; ++iy)
          for (int ix = 1; ix <= n[0]; ++ix) {
            T s = pole_sigma[p].g(ix, iy, iz);
            const int fx = ix + 1, fy = iy + 1, fz = iz + 1;
            if (s != T(0)) {
              for (int q = 0; q < 3; ++q) {
                T& Pv = P[p][q].r(fx, fy, fz);
                T& Pp = Pprev[p][q].r(fx, fy, fz);
                T e = E[q].r(fx, fy, fz);
                T px = Pv;
                if (c.is_drude) Pv = g1i * ((T(2) * px - g1 * Pp) + (dc * s) * e);
                else Pv = g1i * (((T(2) - w0) * px - g1 * Pp) + (sw0 * s) * e);
                Pp = px;
              }
            }
            for (int q = 0; q < 3; ++q) PD[q].r(fx, fy, fz) += P[p][q].r(fx, fy, fz);
          }
    }
  }
};

struct Handle {
  int dtype;
  std::unique_ptr<Oracle<float>> f;
  std::unique_ptr<Oracle<double>> d;
  std::string err;
};

template <class F>
int with(void* h, F&& fn) {
  Handle* H = static_cast<Handle*>(h);
  if (!H) return KH_ERR_INVALID;
  if (H->f) return fn(*H->f);
  return fn(*H->d);
}

}  // namespace

extern "C" {

void* khref_create(const kh_sim_desc* d) {
  if (!d || d->n[0] <= 0 || d->n[1] <= 0 || d->n[2] <= 0) return nullptr;
  Handle* h = new Handle();
  h->dtype = d->dtype;
  if (d->dtype == KH_F32) h->f.reset(new Oracle<float>(*d));
  else h->d.reset(new Oracle<double>(*d));
  return h;
}

void khref_destroy(void* h) { delete static_cast<Handle*>(h); }

const char* khref_last_error(void* h) {
  Handle* H = static_cast<Handle*>(h);
  if (!H) return "null handle";
  H->err = H->f ? H->f->err : H->d->err;
  return H->err.c_str();
}

int khref_set_material(void* h, int kind, int comp, const double* v) {
  return with(h, [&](auto& o) { return o.set_material(kind, comp, v); });
}
int khref_add_pole(void* h, const kh_pole_coeffs* c, const double* s) {
  return with(h, [&](auto& o) { return o.add_pole(*c, s); });
}
int khref_add_source(void* h, const kh_source_desc* s) {
  return with(h, [&](auto& o) { return o.add_source(*s); });
}
int khref_add_dft_monitor(void* h, int comp, const int32_t* st, const int32_t* dm, int nf,
                          const double* f, int dec, int32_t* id) {
  return with(h, [&](auto& o) { return o.add_monitor(comp, st, dm, nf, f, dec, id); });
}
int khref_prepare(void* h) {
  return with(h, [&](auto& o) { return o.prepare(); });
}
int khref_step(void* h, int64_t nsteps) {
  return with(h, [&](auto& o) {
    if (!o.prepared) { o.err = "step before prepare"; return int(KH_ERR_INVALID); }
    for (int64_t s = 0; s < nsteps; ++s) o.step();
    return int(KH_OK);
  });
}
int64_t khref_timestep(void* h) {
  Handle* H = static_cast<Handle*>(h);
  return H->f ? H->f->timestep : H->d->timestep;
}
int khref_sources_active(void* h) {
  Handle* H = static_cast<Handle*>(h);
  return H->f ? H->f->sources_active : H->d->sources_active;
}
int khref_get_field(void* h, int comp, double* out) {
  return with(h, [&](auto& o) {
    if (comp < 0 || comp > 5) return int(KH_ERR_INVALID);
    o.get_field(comp, out);
    return int(KH_OK);
  });
}
int khref_read_dft(void* h, int id, double* out) {
  return with(h, [&](auto& o) {
    if (id < 0 || id >= int(o.monitors.size())) return int(KH_ERR_INVALID);
    auto& m = o.monitors[id];
    for (size_t q = 0; q < m.F.size(); ++q) {
      out[2 * q] = double(m.F[q].real());
      out[2 * q + 1] = double(m.F[q].imag());
    }
    return int(KH_OK);
  });
}
int khref_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
