"""Seeded synthetic oriented point clouds for the benchmark workloads.

Every generator returns float32 positions (N, 3), float32 unit normals (N, 3) and, when
requested, uint8 colours (N, 3) computed as a linear function of position
(clip(255 * (p - min) / (max - min)) per channel).  Seeds follow the rule
``seed = workload_index * 1000 + cloud_index``.

Workloads (all single-precision inputs):
  sphere      20,000 points, unit sphere, radial normals, sigma 0.002, depth 6
  torus+ell   200,000 points, torus R=1 r=0.35 united with an ellipsoid 0.6/0.4/0.3 at
              +0.8 z, area weighted, analytic normals, sigma 0.003, depth 7, colour
  superquad   2,000,000 points, superquadric exponents 0.5/0.5 with radial displacement
              0.05 sin(8 .) and 2-degree normal jitter, depth 9
  mix         random sphere / torus / superquadric, log-uniform sizes, random scale in
              [0.5, 2] and rotation, sigma 0.002
"""
import math

import numpy as np


def _normalize(v):
    n = np.linalg.norm(v, axis=1, keepdims=True)
    n[n == 0] = 1.0
    return v / n


def colour_from_position(p):
    lo = p.min(axis=0)
    hi = p.max(axis=0)
    span = np.where(hi > lo, hi - lo, 1.0)
    return np.clip(np.round(255.0 * (p - lo) / span), 0, 255).astype(np.uint8)


def sphere(n, rng, sigma=0.002, radius=1.0):
    d = _normalize(rng.standard_normal((n, 3)))
    p = radius * d + sigma * rng.standard_normal((n, 3))
    return p.astype(np.float32), d.astype(np.float32)


def torus(n, rng, R=1.0, r=0.35, sigma=0.0):
    # area element is proportional to (R + r cos v): rejection sample v
    out_v = np.empty(0)
    while out_v.size < n:
        v = rng.uniform(0, 2 * np.pi, 2 * n)
        keep = rng.uniform(0, R + r, 2 * n) < (R + r * np.cos(v))
        out_v = np.concatenate([out_v, v[keep]])
    v = out_v[:n]
    u = rng.uniform(0, 2 * np.pi, n)
    cu, su, cv, sv = np.cos(u), np.sin(u), np.cos(v), np.sin(v)
    p = np.stack([(R + r * cv) * cu, (R + r * cv) * su, r * sv], axis=1)
    nrm = np.stack([cv * cu, cv * su, sv], axis=1)
    if sigma:
        p = p + sigma * rng.standard_normal(p.shape)
    return p, nrm


def ellipsoid(n, rng, radii=(0.6, 0.4, 0.3), offset=(0, 0, 0), sigma=0.0):
    a, b, c = radii
    fmax = max(b * c, a * c, a * b)
    acc = np.empty((0, 3))
    while acc.shape[0] < n:
        u = _normalize(rng.standard_normal((2 * n, 3)))
        f = np.sqrt((b * c * u[:, 0]) ** 2 + (a * c * u[:, 1]) ** 2 + (a * b * u[:, 2]) ** 2)
        keep = rng.uniform(0, fmax, 2 * n) < f
        acc = np.concatenate([acc, u[keep]])
    u = acc[:n]
    p = u * np.array([a, b, c])
    nrm = _normalize(p / np.array([a * a, b * b, c * c]))
    p = p + np.array(offset)
    if sigma:
        p = p + sigma * rng.standard_normal(p.shape)
    return p, nrm


def _ellipsoid_area(a, b, c):
    pw = 1.6075
    return 4 * np.pi * (((a * b) ** pw + (a * c) ** pw + (b * c) ** pw) / 3) ** (1 / pw)


def torus_ellipsoid(n, rng, sigma=0.003):
    at = 4 * np.pi ** 2 * 1.0 * 0.35
    ae = _ellipsoid_area(0.6, 0.4, 0.3)
    nt = int(round(n * at / (at + ae)))
    p1, n1 = torus(nt, rng)
    p2, n2 = ellipsoid(n - nt, rng, offset=(0, 0, 0.8))
    p = np.concatenate([p1, p2])
    nrm = np.concatenate([n1, n2])
    perm = rng.permutation(n)
    p = p[perm] + sigma * rng.standard_normal((n, 3))
    return p.astype(np.float32), _normalize(nrm[perm]).astype(np.float32)


def _sq_point(eta, om, e1, e2, amp, freq):
    def spow(x, e):
        return np.sign(x) * np.abs(x) ** e
    ce, se, co, so = np.cos(eta), np.sin(eta), np.cos(om), np.sin(om)
    x = spow(ce, e1) * spow(co, e2)
    y = spow(ce, e1) * spow(so, e2)
    z = spow(se, e1)
    s = 1.0 + amp * np.sin(freq * eta) * np.sin(freq * om)
    return np.stack([x * s, y * s, z * s], axis=-1)


def superquadric(n, rng, e1=0.5, e2=0.5, amp=0.05, freq=8, jitter_deg=2.0, sigma=0.0):
    h = 1e-5
    acc_eta = np.empty(0)
    acc_om = np.empty(0)
    acc_n = np.empty((0, 3))
    # rejection sampling on the parametric area element |P_eta x P_om|
    fmax = None
    while acc_eta.size < n:
        m = 2 * n
        eta = rng.uniform(-np.pi / 2 + 1e-4, np.pi / 2 - 1e-4, m)
        om = rng.uniform(-np.pi, np.pi, m)
        pe = (_sq_point(eta + h, om, e1, e2, amp, freq) - _sq_point(eta - h, om, e1, e2, amp, freq)) / (2 * h)
        po = (_sq_point(eta, om + h, e1, e2, amp, freq) - _sq_point(eta, om - h, e1, e2, amp, freq)) / (2 * h)
        cr = np.cross(po, pe)
        area = np.linalg.norm(cr, axis=1)
        area = np.minimum(area, np.quantile(area, 0.999))
        if fmax is None:
            fmax = float(area.max()) * 1.05
        keep = rng.uniform(0, fmax, m) < area
        acc_eta = np.concatenate([acc_eta, eta[keep]])
        acc_om = np.concatenate([acc_om, om[keep]])
        acc_n = np.concatenate([acc_n, cr[keep]])
    eta, om, cr = acc_eta[:n], acc_om[:n], acc_n[:n]
    p = _sq_point(eta, om, e1, e2, amp, freq)
    nrm = _normalize(cr)
    # make normals point outwards
    flip = np.sum(nrm * p, axis=1) < 0
    nrm[flip] *= -1
    if jitter_deg:
        t = _normalize(np.cross(nrm, rng.standard_normal((n, 3))))
        ang = np.deg2rad(jitter_deg) * rng.standard_normal(n)
        nrm = _normalize(nrm * np.cos(ang)[:, None] + t * np.sin(ang)[:, None])
    if sigma:
        p = p + sigma * rng.standard_normal(p.shape)
    return p.astype(np.float32), nrm.astype(np.float32)


def _random_rotation(rng):
    q, r = np.linalg.qr(rng.standard_normal((3, 3)))
    q = q * np.sign(np.diag(r))
    if np.linalg.det(q) < 0:
        q[:, 0] *= -1
    return q


def workload(name, cloud=0, n=None, colour=None):
    """Return (xyz, normals, rgb_or_None, depth) for a named workload."""
    if name == "sphere20k":
        rng = np.random.default_rng(1 * 1000 + cloud)
        p, nr = sphere(n or 20000, rng, sigma=0.002)
        return p, nr, (colour_from_position(p) if colour else None), 6
    if name == "torus_ellipsoid200k":
        rng = np.random.default_rng(2 * 1000 + cloud)
        p, nr = torus_ellipsoid(n or 200000, rng, sigma=0.003)
        return p, nr, (colour_from_position(p) if colour is not False else None), 7
    if name == "superquadric2m":
        rng = np.random.default_rng(3 * 1000 + cloud)
        p, nr = superquadric(n or 2000000, rng, sigma=0.0)
        return p, nr, (colour_from_position(p) if colour else None), 9
    if name in ("mix", "serve"):
        idx = 4 if name == "mix" else 5
        rng = np.random.default_rng(idx * 1000 + cloud)
        lo, hi = (5000, 150000) if name == "mix" else (10000, 500000)
        npts = n or int(math.exp(rng.uniform(math.log(lo), math.log(hi))))
        depth = int(rng.choice([6, 7, 8] if name == "mix" else [6, 7, 8, 9]))
        kind = int(rng.integers(0, 3))
        if kind == 0:
            p, nr = sphere(npts, rng, sigma=0.0)
        elif kind == 1:
            p, nr = torus(npts, rng)
        else:
            p, nr = superquadric(npts, rng, jitter_deg=0.0)
        rot = _random_rotation(rng)
        scale = rng.uniform(0.5, 2.0)
        p = (np.asarray(p, np.float64) @ rot.T) * scale + 0.002 * rng.standard_normal((npts, 3))
        nr = np.asarray(nr, np.float64) @ rot.T
        p = p.astype(np.float32)
        rgb = colour_from_position(p) if (colour or (colour is None and name == "serve")) else None
        return p, _normalize(nr).astype(np.float32), rgb, depth
    raise KeyError(name)
