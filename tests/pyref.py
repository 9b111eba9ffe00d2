"""A second, pure-Python float32 restatement of the march (small cases only).

It re-derives, from the reference sources, the pieces the oracle and the
kernels implement -- ray generation (cuda_shading.cu:24-29), the slab test
(glm_math.hpp:58-72), ray emit (shader.hpp:113-137), CpuSampler filtering
(cpu_sampler.hpp:72-166), the transfer-function lookup (transfer_fn.hpp:16-23)
and the Volume / Isosurface main loops (volume_shader.cu:32-81,
isosurface_shader.cu:50-125) -- with numpy float32 scalars, one rounding per
operation.  Tests use it to pin the oracle on tiny volumes.
"""

from __future__ import annotations

import math

import numpy as np

F = np.float32


def fmin(a, b):
    return b if b < a else a


def fmax(a, b):
    return b if a < b else a


class Vol:
    """Padded bricks exactly as the dataset is defined (apron clamped at the border)."""

    def __init__(self, vox: np.ndarray, bs: int, pad: int):
        self.vox = vox
        self.bs, self.pad = bs, pad
        self.P = bs + 2 * pad
        nz, ny, nx = vox.shape
        self.dim = (nx, ny, nz)
        self.g = tuple((d + bs - 1) // bs for d in self.dim)
        P = self.P
        self.bricks = {}
        self.cheb = {}
        nonempty = {}
        for bz in range(self.g[2]):
            for by in range(self.g[1]):
                for bx in range(self.g[0]):
                    xs = np.clip(np.arange(P) + bx * bs - pad, 0, nx - 1)
                    ys = np.clip(np.arange(P) + by * bs - pad, 0, ny - 1)
                    zs = np.clip(np.arange(P) + bz * bs - pad, 0, nz - 1)
                    b = vox[np.ix_(zs, ys, xs)]
                    nonempty[(bx, by, bz)] = bool(np.any(b != 0))
                    if vox.dtype == np.uint8:
                        b = (b.astype(np.float32) / F(255)).astype(np.float32)
                    self.bricks[(bx, by, bz)] = b.astype(np.float32)
        cap = max(self.g)
        for key in nonempty:
            if nonempty[key]:
                self.cheb[key] = 0
                continue
            best = cap
            for k2, ne in nonempty.items():
                if ne:
                    best = min(best, max(abs(key[i] - k2[i]) for i in range(3)))
            self.cheb[key] = best
        self.k = F(F(bs) / F(P))
        self.b = F(F(F(pad) / F(bs)) * self.k)
        self.bbox = tuple(F(F(d) / F(bs)) for d in self.dim)
        self.du = F(F(1) / F(bs))

    def key(self, ip):
        out = []
        for a in range(3):
            x = fmin(fmax(ip[a], F(0)), F(self.g[a]))
            out.append(min(max(int(math.floor(x)), 0), self.g[a] - 1))
        return tuple(out)

    def sample(self, key, x):
        P = self.P
        data = self.bricks[key]
        fd = F(P)
        u = []
        for a in range(3):
            m = F(F(self.k * x[a]) + self.b)
            fx = F(fd * m)
            fx = F(fx - F(fd * F(np.floor(F(fx / fd)))))
            u.append(F(fx - F(0.5)))
        flr = [F(np.floor(c)) for c in u]
        aa = [F(u[i] - flr[i]) for i in range(3)]
        ix = [min(max(int(flr[i]), 0), P - 1) for i in range(3)]
        jx = [min(max(int(np.ceil(u[i])), 0), P - 1) for i in range(3)]

        def at(X, Y, Z):
            return data[Z, Y, X]

        def lerp(p, q, a):
            return F(F(p * F(F(1) - a)) + F(q * a))

        x00 = lerp(at(ix[0], ix[1], ix[2]), at(jx[0], ix[1], ix[2]), aa[0])
        x10 = lerp(at(ix[0], jx[1], ix[2]), at(jx[0], jx[1], ix[2]), aa[0])
        x01 = lerp(at(ix[0], ix[1], jx[2]), at(jx[0], ix[1], jx[2]), aa[0])
        x11 = lerp(at(ix[0], jx[1], jx[2]), at(jx[0], jx[1], jx[2]), aa[0])
        y0 = lerp(x00, x10, aa[1])
        y1 = lerp(x01, x11, aa[1])
        return lerp(y0, y1, aa[2])


def tf_sample(tf, s):
    n = len(tf)
    fd = F(n)
    fx = F(fd * s)
    if not (F(0) <= fx and fx <= fd):
        return [F(0)] * 4
    u = F(fx - F(0.5))
    flr = F(np.floor(u))
    a = F(u - flr)
    i = min(max(int(flr), 0), n - 1)
    j = min(max(int(np.ceil(u)), 0), n - 1)
    return [F(F(F(tf[i][c]) * F(F(1) - a)) + F(F(tf[j][c]) * a)) for c in range(4)]


def intersect(o, d, lo, hi):
    inv = [F(F(1) / d[a]) for a in range(3)]
    tb = [F(inv[a] * F(lo[a] - o[a])) for a in range(3)]
    tt = [F(inv[a] * F(hi[a] - o[a])) for a in range(3)]
    mn = [fmin(tt[a], tb[a]) for a in range(3)]
    mx = [fmax(tt[a], tb[a]) for a in range(3)]
    tn = fmax(fmax(mn[0], mn[1]), mn[2])
    tf = fmin(fmin(mx[0], mx[1]), mx[2])
    return tf > tn, tn, tf


def gen_ray(view, x, y, W, H):
    m = [F(v) for v in view[:16]]
    ctg = F(view[16])
    o = [F(v) for v in view[17:20]]
    ccx, ccy = F(F(W) / F(2)), F(F(H) / F(2))
    ux = F(F(F(F(x) - ccx) * F(2)) / F(H))
    uy = F(F(F(F(y) - ccy) * F(2)) / F(H))
    v = [ux, F(-uy), F(-ctg), F(1)]
    p = []
    for r in range(3):
        acc = F(m[r] * v[0])
        for c in range(1, 4):
            acc = F(acc + F(m[4 * c + r] * v[c]))
        p.append(acc)
    d = [F(p[a] - o[a]) for a in range(3)]
    n2 = F(F(F(d[0] * d[0]) + F(d[1] * d[1])) + F(d[2] * d[2]))
    inv = F(F(1) / F(np.sqrt(n2)))
    return o, [F(c * inv) for c in d]


def skip(o, d, ip, nblocks, cdu, step):
    _, _, tfar = intersect(o, d, ip, [F(c + F(1)) for c in ip])
    di = F(np.ceil(F(F(tfar + F(F(nblocks - 1) * cdu)) / step)))
    o2 = [F(o[a] + F(F(d[a] * di) * step)) for a in range(3)]
    return o2, int(di)


def volume_pixel(vol: Vol, tf, view, x, y, W, H, sample_rate=F(1), density=F(1),
                 max_steps=4000000):
    """Returns (v[4], theta[3], phi, samples) for one pixel of the Volume shader."""
    step = F(F(vol.du / F(4)) / F(sample_rate))
    o, d = gen_ray(view, x, y, W, H)
    v = [F(0)] * 4
    theta = [F(0)] * 3
    phi = F(1)
    hit, tn, tfar = intersect(o, d, [F(0)] * 3, list(vol.bbox))
    if not hit:
        return v, theta, phi, 0
    if tn < 0:
        tn = F(0)
    if tfar < 0:
        tfar = F(0)
    o = [F(o[a] + F(d[a] * tn)) for a in range(3)]
    nsteps = min(max_steps, int(F(F(tfar - tn) / step)))
    ss = 1
    cdu = F(F(1) / fmax(fmax(F(abs(d[0])), F(abs(d[1]))), F(abs(d[2]))))
    samples = 0
    while nsteps > 0:
        ip = [F(np.floor(c)) for c in o]
        key = vol.key(ip)
        cd = vol.cheb[key]
        if cd:
            o, di = skip(o, d, ip, cd, cdu, F(step * F(ss)))
            nsteps -= di
        else:
            s = vol.sample(key, [F(o[a] - ip[a]) for a in range(3)])
            samples += 1
            ub = tf_sample(tf, s)
            ub[3] = F(ub[3] * F(density))
            w = ub[3]
            ub = [F(ub[0] * w), F(ub[1] * w), F(ub[2] * w), ub[3]]
            theta = [F(theta[c] + F(ub[c] * phi)) for c in range(3)]
            phi = F(phi * F(F(1) - ub[3]))
            t = F(F(1) - v[3])
            v = [F(v[c] + F(ub[c] * t)) for c in range(4)]
            if float(v[3]) > 0.93:
                ss = 16
            elif float(v[3]) > 0.85:
                ss = 4
        o = [F(o[a] + F(F(d[a] * step) * F(ss))) for a in range(3)]
        nsteps -= ss
    return v, theta, phi, samples
