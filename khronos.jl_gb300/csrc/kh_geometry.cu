// Geometry set-up on the device: per-voxel ε⁻¹ of the three E components
// from a list of objects, with optional subpixel smoothing.
//
// Restates the reference's host set-up (src/Geometry.jl):
//   _rasterize_geometry_3d! (:223-250)   objects painted in reverse order so the
//                                        first object containing a point wins;
//                                        each component samples at its Yee position
//   _smooth_component_yrange! (:880-990) a voxel is an interface voxel when a
//                                        face neighbour's ε⁻¹ differs by more than
//                                        1e-6 relative; its value becomes the fill-
//                                        fraction average over the nearest object
//                                        surface (volume or anisotropic average)
// The shape predicates (inside test, nearest surface point with its outward
// normal, half-space fill fraction of a voxel) are those of GeometryPrimitives
// (Ball, Cuboid, Cylinder; not part of the reference tree), restated here:
// inside tests are inclusive, the fill fraction is the exact volume of the
// voxel box on the inner side of the tangent plane.
#include <cuda_runtime.h>

#include <cmath>

#include "../../include/khronos_gb300.h"
#include "kh_kernels.cuh"

namespace kh {

namespace {

__device__ __forceinline__ bool inside(const GeomObj& o, const double p[3]) {
  if (o.shape == KH_SHAPE_BALL) {
    const double dx = p[0] - o.c[0], dy = p[1] - o.c[1], dz = p[2] - o.c[2];
    return sqrt(dx * dx + dy * dy + dz * dz) <= o.s[0];
  }
  if (o.shape == KH_SHAPE_CUBOID) {
    for (int a = 0; a < 3; ++a)
      if (fabs(p[a] - o.c[a]) > 0.5 * o.s[a]) return false;
    return true;
  }
  // cylinder: radial distance and axial extent
  const int ax = o.axis, a1 = (ax + 1) % 3, a2 = (ax + 2) % 3;
  const double r1 = p[a1] - o.c[a1], r2 = p[a2] - o.c[a2];
  return sqrt(r1 * r1 + r2 * r2) <= o.s[0] && fabs(p[ax] - o.c[ax]) <= 0.5 * o.s[1];
}

__device__ __forceinline__ double sgn(double v) { return v < 0 ? -1.0 : 1.0; }

// Nearest surface point sp of object o to p and the outward normal there.
__device__ void surfpt(const GeomObj& o, const double p[3], double sp[3], double n[3]) {
  if (o.shape == KH_SHAPE_BALL) {
    const double v[3] = {p[0] - o.c[0], p[1] - o.c[1], p[2] - o.c[2]};
    const double l = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    for (int a = 0; a < 3; ++a) n[a] = l > 0 ? v[a] / l : (a == 0 ? 1.0 : 0.0);
    for (int a = 0; a < 3; ++a) sp[a] = o.c[a] + o.s[0] * n[a];
    return;
  }
  if (o.shape == KH_SHAPE_CUBOID) {
    double d[3], out[3];
    int nout = 0, best = 0;
    for (int a = 0; a < 3; ++a) {
      d[a] = p[a] - o.c[a];
      out[a] = fabs(d[a]) - 0.5 * o.s[a];
      if (out[a] > 0) ++nout;
      if (out[a] > out[best]) best = a;
    }
    for (int a = 0; a < 3; ++a) n[a] = 0.0;
    if (nout == 0) {  // inside or on the surface: the nearest face
      for (int a = 0; a < 3; ++a) sp[a] = p[a];
      sp[best] = o.c[best] + sgn(d[best]) * 0.5 * o.s[best];
      n[best] = sgn(d[best]);
      return;
    }
    for (int a = 0; a < 3; ++a) sp[a] = o.c[a] + fmin(fmax(d[a], -0.5 * o.s[a]), 0.5 * o.s[a]);
    if (nout == 1) {
      n[best] = sgn(d[best]);
    } else {  // beyond an edge or a corner
      double l = 0;
      for (int a = 0; a < 3; ++a) l += (p[a] - sp[a]) * (p[a] - sp[a]);
      l = sqrt(l);
      for (int a = 0; a < 3; ++a) n[a] = (p[a] - sp[a]) / l;
    }
    return;
  }
  const int ax = o.axis, a1 = (ax + 1) % 3, a2 = (ax + 2) % 3;
  const double t = p[ax] - o.c[ax];
  const double r1 = p[a1] - o.c[a1], r2 = p[a2] - o.c[a2];
  const double rl = sqrt(r1 * r1 + r2 * r2);
  const double u1 = rl > 0 ? r1 / rl : 1.0, u2 = rl > 0 ? r2 / rl : 0.0;
  const double dr = rl - o.s[0], dz = fabs(t) - 0.5 * o.s[1];
  for (int a = 0; a < 3; ++a) n[a] = 0.0;
  bool side;
  if (dr <= 0 && dz <= 0) side = (-dr) < (-dz);  // inside: the nearer of side and cap
  else if (dr > 0 && dz <= 0) side = true;
  else if (dz > 0 && dr <= 0) side = false;
  else {  // beyond the rim
    sp[ax] = o.c[ax] + sgn(t) * 0.5 * o.s[1];
    sp[a1] = o.c[a1] + o.s[0] * u1;
    sp[a2] = o.c[a2] + o.s[0] * u2;
    double l = 0;
    for (int a = 0; a < 3; ++a) l += (p[a] - sp[a]) * (p[a] - sp[a]);
    l = sqrt(l);
    for (int a = 0; a < 3; ++a) n[a] = (p[a] - sp[a]) / l;
    return;
  }
  if (side) {
    sp[ax] = p[ax];
    sp[a1] = o.c[a1] + o.s[0] * u1;
    sp[a2] = o.c[a2] + o.s[0] * u2;
    n[a1] = u1;
    n[a2] = u2;
  } else {
    sp[ax] = o.c[ax] + sgn(t) * 0.5 * o.s[1];
    sp[a1] = p[a1];
    sp[a2] = p[a2];
    n[ax] = sgn(t);
  }
}

__device__ __forceinline__ double ramp_pow(double v, int k) {
  if (v <= 0) return 0.0;
  return k == 1 ? v : (k == 2 ? v * v : v * v * v);
}

// Fraction of the box [lo, hi] on the inner side {x : n·(x − r0) ≤ 0}.  In
// unit-cube coordinates u the side is Σ w_a·u_a ≤ t (w_a = |n_a|·L_a after
// flipping axes so all w_a ≥ 0); the fraction is the corner inclusion–
// exclusion Σ_S (−1)^|S| ramp(t − Σ_S w)^k / (k!·Π w) over the k axes kept.
// An axis with w_a ≤ 1e-3·max w is integrated out at its midpoint (t −= w_a/2,
// error O((w_a/w_max)²)); the closed form would divide by that tiny w_a and
// cancel catastrophically for nearly axis-aligned surfaces.
__device__ double volfrac(const double lo[3], const double hi[3], const double n_in[3], const double r0[3]) {
  double w[3], t = 0, wmax = 0;
  for (int a = 0; a < 3; ++a) t += n_in[a] * (r0[a] - lo[a]);
  for (int a = 0; a < 3; ++a) {
    const double L = hi[a] - lo[a];
    w[a] = n_in[a] * L;
    if (w[a] < 0) {
      t -= w[a];
      w[a] = -w[a];
    }
    wmax = fmax(wmax, w[a]);
  }
  int act[3], k = 0;
  double den = 1;
  for (int a = 0; a < 3; ++a) {
    if (w[a] <= 1e-3 * wmax) {
      t -= 0.5 * w[a];
    } else {
      act[k++] = a;
      den *= w[a];
    }
  }
  if (k == 0) return t >= 0 ? 1.0 : 0.0;
  double vol = 0;
  for (int mask = 0; mask < (1 << k); ++mask) {
    double v = t;
    int bits = 0;
    for (int q = 0; q < k; ++q)
      if (mask & (1 << q)) {
        v -= w[act[q]];
        ++bits;
      }
    const double r = ramp_pow(v, k);
    vol += (bits & 1) ? -r : r;
  }
  const double fact = k == 1 ? 1.0 : (k == 2 ? 2.0 : 6.0);
  const double f = vol / (fact * den);
  return fmin(fmax(f, 0.0), 1.0);
}

template <typename T>
__global__ void rasterize_kernel(const GeomArgs a, T* eps_inv) {
  const long long total = (long long)a.n[0] * a.n[1] * a.n[2];
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    const int i = int(q % a.n[0]);
    const long long r = q / a.n[0];
    const int j = int(r % a.n[1]), k = int(r / a.n[1]);
    const double p[3] = {a.org[0] + i * a.d[0], a.org[1] + j * a.d[1], a.org[2] + k * a.d[2]};
    double eps = a.background;
    for (int o = 0; o < a.nobj; ++o)
      if (inside(a.objs[o], p)) {
        eps = a.objs[o].eps;
        break;
      }
    eps_inv[a.origin + (long long)k * a.plane + (long long)j * a.pitch + i] = T(1.0 / eps);
  }
}

template <typename T>
__global__ void smooth_kernel(const GeomArgs a, const T* orig, T* eps_inv) {
  const long long total = (long long)a.n[0] * a.n[1] * a.n[2];
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    const int i = int(q % a.n[0]);
    const long long r = q / a.n[0];
    const int j = int(r % a.n[1]), k = int(r / a.n[1]);
    const long long idx = a.origin + (long long)k * a.plane + (long long)j * a.pitch + i;
    const T vc = orig[idx];
    // interface test over the six face neighbours, in the reference's order
    const int off[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
    bool iface = false;
    T vn = vc;
    for (int m = 0; m < 6 && !iface; ++m) {
      const int ii = i + off[m][0], jj = j + off[m][1], kk = k + off[m][2];
      if (ii < 0 || jj < 0 || kk < 0 || ii >= a.n[0] || jj >= a.n[1] || kk >= a.n[2]) continue;
      const T nb = orig[a.origin + (long long)kk * a.plane + (long long)jj * a.pitch + ii];
      if (fabs(double(nb) - double(vc)) > double(T(1e-6)) * fmax(fabs(double(nb)), fabs(double(vc)))) {
        iface = true;
        vn = nb;
      }
    }
    if (!iface) continue;
    const double p[3] = {a.org[0] + i * a.d[0], a.org[1] + j * a.d[1], a.org[2] + k * a.d[2]};
    const double eps_c = double(T(1) / vc), eps_n = double(T(1) / vn);
    double best = INFINITY, bsp[3] = {p[0], p[1], p[2]}, bn[3] = {0, 0, 1};
    int bo = -1;
    for (int o = 0; o < a.nobj; ++o) {
      const GeomObj& g = a.objs[o];
      double bb = 0;
      for (int ax = 0; ax < 3; ++ax) {
        if (p[ax] < g.lo[ax]) bb += (g.lo[ax] - p[ax]) * (g.lo[ax] - p[ax]);
        else if (p[ax] > g.hi[ax]) bb += (p[ax] - g.hi[ax]) * (p[ax] - g.hi[ax]);
      }
      if (bb >= best) continue;
      double sp[3], nn[3];
      surfpt(g, p, sp, nn);
      const double d2 = (sp[0] - p[0]) * (sp[0] - p[0]) + (sp[1] - p[1]) * (sp[1] - p[1]) +
                        (sp[2] - p[2]) * (sp[2] - p[2]);
      if (d2 < best) {
        best = d2;
        bo = o;
        for (int ax = 0; ax < 3; ++ax) {
          bsp[ax] = sp[ax];
          bn[ax] = nn[ax];
        }
      }
    }
    if (bo < 0) continue;
    const double nl = sqrt(bn[0] * bn[0] + bn[1] * bn[1] + bn[2] * bn[2]);
    double nh[3];
    for (int ax = 0; ax < 3; ++ax) nh[ax] = nl > 0 ? bn[ax] / nl : (ax == 2 ? 1.0 : 0.0);
    double lo[3], hi[3];
    for (int ax = 0; ax < 3; ++ax) {
      lo[ax] = p[ax] - 0.5 * a.d[ax];
      hi[ax] = p[ax] + 0.5 * a.d[ax];
    }
    const double f = volfrac(lo, hi, nh, bsp);
    const bool in = inside(a.objs[bo], p);
    const double e_shape = in ? eps_c : eps_n, e_bg = in ? eps_n : eps_c;
    const double e_avg = f * e_shape + (1 - f) * e_bg;
    const double inv_harm = f / e_shape + (1 - f) / e_bg;
    double v;
    if (a.smoothing == KH_SMOOTH_ANISOTROPIC) {
      const double nc2 = nh[a.comp] * nh[a.comp];
      v = (1 - nc2) * inv_harm + nc2 / e_avg;
    } else {
      v = 1.0 / e_avg;
    }
    eps_inv[idx] = T(v);
  }
}

}  // namespace

template <typename T>
void launch_geometry(const GeomArgs& a, T* eps_inv, T* scratch, void* stream) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const long long total = (long long)a.n[0] * a.n[1] * a.n[2];
  int blocks = int((total + 255) / 256);
  if (blocks > 152 * 32) blocks = 152 * 32;
  if (blocks < 1) blocks = 1;
  rasterize_kernel<T><<<blocks, 256, 0, st>>>(a, eps_inv);
  if (a.smoothing != KH_SMOOTH_NONE) {
    cudaMemcpyAsync(scratch, eps_inv, size_t(a.total) * sizeof(T), cudaMemcpyDeviceToDevice, st);
    smooth_kernel<T><<<blocks, 256, 0, st>>>(a, scratch, eps_inv);
  }
}

template void launch_geometry<float>(const GeomArgs&, float*, float*, void*);
template void launch_geometry<double>(const GeomArgs&, double*, double*, void*);

}  // namespace kh
