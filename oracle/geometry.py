"""ORACLE — test infrastructure, not product code.

CPU restatement (numpy, FP64) of the geometry set-up the device runs for
kh_sim_set_geometry, used by tests/ as its checker and to give the CPU step
oracle the same ε⁻¹ arrays:

* rasterisation  _rasterize_geometry_3d! / _rasterize_object_yrange!
                 (src/Geometry.jl:156-250): objects painted in reverse order,
                 so the first object containing a point wins; points sampled at
                 each E component's Yee position
* smoothing      _smooth_component_yrange! (src/Geometry.jl:880-990)
* shapes         GeometryPrimitives (pinned by Khronos.jl's Project.toml at
                 0.5; not in the reference tree): inclusive inside tests of
                 Ball, Cuboid and axis-aligned Cylinder, nearest surface point
                 with its outward normal, and the half-space fill fraction of
                 a voxel (exact corner inclusion–exclusion)
"""
from __future__ import annotations

import math

import numpy as np


def _inside(o, p):
    shape, axis, c, s, _ = o
    if shape == 0:
        dx, dy, dz = p[0] - c[0], p[1] - c[1], p[2] - c[2]
        return math.sqrt(dx * dx + dy * dy + dz * dz) <= s[0]
    if shape == 1:
        return all(abs(p[a] - c[a]) <= 0.5 * s[a] for a in range(3))
    a1, a2 = (axis + 1) % 3, (axis + 2) % 3
    r1, r2 = p[a1] - c[a1], p[a2] - c[a2]
    return math.sqrt(r1 * r1 + r2 * r2) <= s[0] and abs(p[axis] - c[axis]) <= 0.5 * s[1]


def _sgn(v):
    return -1.0 if v < 0 else 1.0


def _surfpt(o, p):
    shape, axis, c, s, _ = o
    if shape == 0:
        v = [p[a] - c[a] for a in range(3)]
        l = math.sqrt(sum(x * x for x in v))
        n = [x / l for x in v] if l > 0 else [1.0, 0.0, 0.0]
        return [c[a] + s[0] * n[a] for a in range(3)], n
    if shape == 1:
        d = [p[a] - c[a] for a in range(3)]
        out = [abs(d[a]) - 0.5 * s[a] for a in range(3)]
        nout = sum(1 for a in range(3) if out[a] > 0)
        best = 0
        for a in range(3):
            if out[a] > out[best]:
                best = a
        n = [0.0, 0.0, 0.0]
        if nout == 0:
            sp = list(p)
            sp[best] = c[best] + _sgn(d[best]) * 0.5 * s[best]
            n[best] = _sgn(d[best])
            return sp, n
        sp = [c[a] + min(max(d[a], -0.5 * s[a]), 0.5 * s[a]) for a in range(3)]
        if nout == 1:
            n[best] = _sgn(d[best])
        else:
            l = math.sqrt(sum((p[a] - sp[a]) ** 2 for a in range(3)))
            n = [(p[a] - sp[a]) / l for a in range(3)]
        return sp, n
    a1, a2 = (axis + 1) % 3, (axis + 2) % 3
    t = p[axis] - c[axis]
    r1, r2 = p[a1] - c[a1], p[a2] - c[a2]
    rl = math.sqrt(r1 * r1 + r2 * r2)
    u1, u2 = (r1 / rl, r2 / rl) if rl > 0 else (1.0, 0.0)
    dr, dz = rl - s[0], abs(t) - 0.5 * s[1]
    n = [0.0, 0.0, 0.0]
    sp = [0.0, 0.0, 0.0]
    if dr <= 0 and dz <= 0:
        side = (-dr) < (-dz)
    elif dr > 0 and dz <= 0:
        side = True
    elif dz > 0 and dr <= 0:
        side = False
    else:
        sp[axis] = c[axis] + _sgn(t) * 0.5 * s[1]
        sp[a1] = c[a1] + s[0] * u1
        sp[a2] = c[a2] + s[0] * u2
        l = math.sqrt(sum((p[a] - sp[a]) ** 2 for a in range(3)))
        return sp, [(p[a] - sp[a]) / l for a in range(3)]
    if side:
        sp[axis], sp[a1], sp[a2] = p[axis], c[a1] + s[0] * u1, c[a2] + s[0] * u2
        n[a1], n[a2] = u1, u2
    else:
        sp[axis], sp[a1], sp[a2] = c[axis] + _sgn(t) * 0.5 * s[1], p[a1], p[a2]
        n[axis] = _sgn(t)
    return sp, n


def volfrac(lo, hi, n_in, r0):
    """Fraction of the box [lo, hi] with n·(x − r0) ≤ 0: corner inclusion–
    exclusion in unit-cube coordinates, axes with |n_a|·L_a ≤ 1e-3 of the
    largest integrated out at their midpoint (same operation order as the
    device code)."""
    t = 0.0
    for a in range(3):
        t += n_in[a] * (r0[a] - lo[a])
    w = [0.0, 0.0, 0.0]
    wmax = 0.0
    for a in range(3):
        L = hi[a] - lo[a]
        w[a] = n_in[a] * L
        if w[a] < 0:
            t -= w[a]
            w[a] = -w[a]
        wmax = max(wmax, w[a])
    act = []
    den = 1.0
    for a in range(3):
        if w[a] <= 1e-3 * wmax:
            t -= 0.5 * w[a]
        else:
            act.append(a)
            den *= w[a]
    k = len(act)
    if k == 0:
        return 1.0 if t >= 0 else 0.0
    vol = 0.0
    for mask in range(1 << k):
        v = t
        bits = 0
        for q in range(k):
            if mask & (1 << q):
                v -= w[act[q]]
                bits += 1
        if v <= 0:
            r = 0.0
        elif k == 1:
            r = v
        elif k == 2:
            r = v * v
        else:
            r = v * v * v
        vol += -r if bits & 1 else r
    fact = {1: 1.0, 2: 2.0, 3: 6.0}[k]
    return min(max(vol / (fact * den), 0.0), 1.0)


def _bounds(o):
    shape, axis, c, s, _ = o
    if shape == 0:
        e = [s[0]] * 3
    elif shape == 1:
        e = [0.5 * s[a] for a in range(3)]
    else:
        e = [0.5 * s[1] if a == axis else s[0] for a in range(3)]
    return [c[a] - e[a] for a in range(3)], [c[a] + e[a] for a in range(3)]


def eps_inv_arrays(geo, n, delta, T=np.float64):
    """The three components' ε⁻¹ arrays (cell-indexed [i, j, k]) in precision T."""
    out = []
    d = [float(x) for x in delta]
    bounds = [_bounds(o) for o in geo.objects]
    for c in range(3):
        org = [geo.origin[a] - (0.0 if a == c else 0.5 * d[a]) for a in range(3)]
        arr = np.empty(tuple(n), dtype=T)
        for k in range(n[2]):
            for j in range(n[1]):
                for i in range(n[0]):
                    p = (org[0] + i * d[0], org[1] + j * d[1], org[2] + k * d[2])
                    eps = geo.background
                    for o in geo.objects:
                        if _inside(o, p):
                            eps = o[4]
                            break
                    arr[i, j, k] = T(1.0 / eps)
        if geo.smoothing:
            arr = _smooth(arr, c, org, d, geo, bounds, T)
        out.append(arr)
    return out


def _smooth(orig, comp, org, d, geo, bounds, T):
    res = orig.copy()
    n = orig.shape
    offs = ((1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1))
    rtol = float(T(1e-6))
    for k in range(n[2]):
        for j in range(n[1]):
            for i in range(n[0]):
                vc = orig[i, j, k]
                vn = vc
                iface = False
                for dx, dy, dz in offs:
                    ii, jj, kk = i + dx, j + dy, k + dz
                    if not (0 <= ii < n[0] and 0 <= jj < n[1] and 0 <= kk < n[2]):
                        continue
                    nb = orig[ii, jj, kk]
                    if abs(float(nb) - float(vc)) > rtol * max(abs(float(nb)), abs(float(vc))):
                        iface, vn = True, nb
                        break
                if not iface:
                    continue
                p = (org[0] + i * d[0], org[1] + j * d[1], org[2] + k * d[2])
                eps_c, eps_n = float(T(1) / vc), float(T(1) / vn)
                best, bsp, bn, bo = math.inf, list(p), [0.0, 0.0, 1.0], -1
                for oi, o in enumerate(geo.objects):
                    lo, hi = bounds[oi]
                    bb = 0.0
                    for a in range(3):
                        if p[a] < lo[a]:
                            bb += (lo[a] - p[a]) ** 2
                        elif p[a] > hi[a]:
                            bb += (p[a] - hi[a]) ** 2
                    if bb >= best:
                        continue
                    sp, nn = _surfpt(o, p)
                    d2 = sum((sp[a] - p[a]) ** 2 for a in range(3))
                    if d2 < best:
                        best, bsp, bn, bo = d2, sp, nn, oi
                if bo < 0:
                    continue
                nl = math.sqrt(sum(x * x for x in bn))
                nh = [x / nl for x in bn] if nl > 0 else [0.0, 0.0, 1.0]
                lo = [p[a] - 0.5 * d[a] for a in range(3)]
                hi = [p[a] + 0.5 * d[a] for a in range(3)]
                f = volfrac(lo, hi, nh, bsp)
                inside = _inside(geo.objects[bo], p)
                e_shape, e_bg = (eps_c, eps_n) if inside else (eps_n, eps_c)
                e_avg = f * e_shape + (1 - f) * e_bg
                inv_harm = f / e_shape + (1 - f) / e_bg
                if geo.smoothing == 2:
                    nc2 = nh[comp] ** 2
                    v = (1 - nc2) * inv_harm + nc2 / e_avg
                else:
                    v = 1.0 / e_avg
                res[i, j, k] = T(v)
    return res
