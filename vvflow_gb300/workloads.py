"""Seeded synthetic inputs for the per-step velocity path.

There are no public datasets for this solver; every workload is generated here from a
seed.  Body contours follow the reference's Lua generators:

* ``cylinder_corners``  -- ``gen_cylinder{R, N}`` (utils/vvflow/gen_cylinder.cpp:6-44),
  which calls ``gen_arc_N(c=(0,0), R, a1=2*pi, a2=0, N)`` (utils/vvflow/gen_body.cpp:74-88):
  corners at angles ``2*pi*(1 - i/N)``, clockwise, so the flow is outside the body.
* ``ellipse_corners``   -- ``gen_ellipse{Rx, Ry, N}`` (utils/vvflow/gen_ellipse.cpp:7-69),
  arc-length stepping over the upper half and its point reflection.

Vortex clouds follow the named configurations:

* ``annulus_cloud``  -- uniform in ``r1 < r < r2``, circulations N(0, sigma^2) shifted
  to zero total (the 20 000-vortex cylinder case).
* ``wake_cloud``     -- x ~ U(x0, x1), y ~ N(0, (0.2 + 0.05 x)^2),
  sign = sgn(sin(2 pi x / 4.8) * y), |g| ~ LogNormal(ln 1e-5, 0.5), points inside the
  body rejected (the 1M and 4M wake cases).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


def cylinder_corners(R: float = 0.5, N: int = 500):
    """Corners of ``gen_cylinder{R=R, N=N}`` in contour order (float64 arrays)."""
    a1, a2 = 2 * math.pi, 0.0
    xs = np.empty(N)
    ys = np.empty(N)
    for i in range(N):
        ai = a1 + (a2 - a1) * float(i) / float(N)
        xs[i] = 0.0 + R * math.cos(ai)
        ys[i] = 0.0 + R * math.sin(ai)
    return xs, ys


def ellipse_corners(Rx: float = 0.5, Ry: float = 0.25, N: int = 4000, angle_deg: float = 0.0):
    """Corners of ``gen_ellipse{Rx, Ry, N}``, then rotated by ``angle_deg`` about the
    origin (positive = nose up for a free stream along +x)."""
    h = ((Rx - Ry) / (Rx + Ry)) ** 2
    slen = math.pi * (Rx + Ry) * (1.0 + 3 * h / (10 + math.sqrt(4 - 3 * h)))
    dl = slen / N
    if not dl < Ry / 1.9:
        raise ValueError("discretization too low")
    semiell = []
    a = math.asin(dl / (2 * Ry))
    while a < math.pi - math.asin(dl / (2 * Ry)):
        semiell.append(a)
        da1 = dl / math.sqrt((Rx * math.sin(a)) ** 2 + (Ry * math.cos(a)) ** 2)
        da2 = dl / math.sqrt((Rx * math.sin(a + da1)) ** 2 + (Ry * math.cos(a + da1)) ** 2)
        a += (da1 + da2) / 2
    n = len(semiell) - 1
    xs, ys = [], []
    for i in range(n + 1):
        aa = semiell[i] * (1.0 - i / n) + (math.pi - semiell[n - i]) * (i / n)
        xs.append(Rx * math.cos(aa)); ys.append(-Ry * math.sin(aa))
    for i in range(n + 1):
        aa = semiell[i] * (1.0 - i / n) + (math.pi - semiell[n - i]) * (i / n)
        xs.append(-Rx * math.cos(aa)); ys.append(Ry * math.sin(aa))
    xs = np.array(xs)
    ys = np.array(ys)
    if angle_deg:
        t = math.radians(-angle_deg)
        c, s = math.cos(t), math.sin(t)
        xs, ys = xs * c - ys * s, xs * s + ys * c
    return xs, ys


def point_in_polygon(px, py, cx, cy):
    """Even-odd test of points against a closed contour (vectorised)."""
    inside = np.zeros(px.shape, dtype=bool)
    n = len(cx)
    j = n - 1
    for i in range(n):
        xi, yi, xj, yj = cx[i], cy[i], cx[j], cy[j]
        cond = ((yi > py) != (yj > py))
        with np.errstate(divide="ignore", invalid="ignore"):
            xint = (xj - xi) * (py - yi) / (yj - yi) + xi
        inside ^= cond & (px < xint)
        j = i
    return inside


def annulus_cloud(n: int, r1: float = 0.52, r2: float = 3.0, sigma: float = 2e-4, seed: int = 1):
    rng = np.random.default_rng(seed)
    r = np.sqrt(rng.uniform(r1 * r1, r2 * r2, n))
    phi = rng.uniform(0.0, 2 * math.pi, n)
    g = rng.normal(0.0, sigma, n)
    g = g - g.mean()
    return r * np.cos(phi), r * np.sin(phi), g


def wake_cloud(n: int, x0: float = 0.5, x1: float = 40.0, body=None, seed: int = 2):
    """Karman-like synthetic wake; ``body`` = (corner_x, corner_y) to reject points inside."""
    rng = np.random.default_rng(seed)
    xs, ys = [], []
    need = n
    while need > 0:
        m = int(need * 1.05) + 16
        x = rng.uniform(x0, x1, m)
        y = rng.normal(0.0, 1.0, m) * (0.2 + 0.05 * x)
        if body is not None:
            bx, by = body
            r2 = (bx * bx + by * by).max()
            cand = (x * x + y * y) <= r2
            bad = np.zeros(m, dtype=bool)
            if cand.any():
                bad[cand] = point_in_polygon(x[cand], y[cand], bx, by)
            x, y = x[~bad], y[~bad]
        xs.append(x[:need]); ys.append(y[:need])
        need -= len(xs[-1])
    x = np.concatenate(xs)[:n]
    y = np.concatenate(ys)[:n]
    sign = np.sign(np.sin(2 * math.pi * x / 4.8) * y)
    sign[sign == 0] = 1.0
    mag = np.exp(rng.normal(math.log(1e-5), 0.5, n))
    return x, y, sign * mag


@dataclass
class Workload:
    """One synthetic configuration: bodies, vortices and solver scalars."""
    name: str
    bodies: list  # list of (corner_x, corner_y)
    x: np.ndarray
    y: np.ndarray
    g: np.ndarray
    re: float
    dt: float
    inf_vx: float = 1.0
    inf_vy: float = 0.0
    far_criteria: float = 8.0
    merge: bool = True
    extra: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(self.x.shape[0])

    @property
    def m(self) -> int:
        return int(sum(len(b[0]) for b in self.bodies))

    def node_sizes(self):
        """min/max node sizes used by the reference driver (utils/vvflow/vvflow.cpp:200-203):
        5 and 100 times the first body's average segment length slen/(N-1)."""
        if not self.bodies:
            return 0.0, float(np.finfo(np.float64).max)
        cx, cy = self.bodies[0]
        n = len(cx)
        dlx = np.roll(cx, -1) - cx
        dly = np.roll(cy, -1) - cy
        slen = 0.0
        for a, b in zip(dlx, dly):  # TBody::doFillProperties summation order
            slen += math.sqrt(a * a + b * b)
        dl = slen / (n - 1) if n > 1 else 0.0
        if dl <= 0:
            return 0.0, float(np.finfo(np.float64).max)
        return dl * 5, dl * 100


def cylinder_annulus(n: int = 20000, m: int = 500, seed: int = 1) -> Workload:
    """Impulsively started cylinder, R=0.5, M segments, N vortices in 0.52<r<3 (FP64 case)."""
    cx, cy = cylinder_corners(0.5, m)
    x, y, g = annulus_cloud(n, seed=seed)
    return Workload("cylinder_annulus", [(cx, cy)], x, y, g, re=600.0, dt=0.005)


def cylinder_wake(n: int = 1_000_000, m: int = 2000, seed: int = 2) -> Workload:
    """Cylinder with M segments and a synthetic wake of N vortices over x in (0.5, 40)."""
    cx, cy = cylinder_corners(0.5, m)
    x, y, g = wake_cloud(n, 0.5, 40.0, body=(cx, cy), seed=seed)
    return Workload("cylinder_wake", [(cx, cy)], x, y, g, re=1e4, dt=0.002)


def ellipse_wake(n: int = 4_000_000, m: int = 4000, seed: int = 3, angle_deg: float = 10.0,
                 far_criteria: float = 8.0) -> Workload:
    """Ellipse 0.5 x 0.25 at 10 degrees incidence, M segments, wake of N vortices to x<80."""
    cx, cy = ellipse_corners(0.5, 0.25, m, angle_deg)
    x, y, g = wake_cloud(n, 0.5, 80.0, body=(cx, cy), seed=seed)
    return Workload("ellipse_wake", [(cx, cy)], x, y, g, re=1e4, dt=0.002,
                    far_criteria=far_criteria)


def batched_cylinders(count: int = 256, n_lo: int = 5_000, n_hi: int = 200_000, m_lo: int = 200,
                      m_hi: int = 1_000, seed: int = 5) -> list:
    """Independent cylinder simulations for the batched sweep: per instance N log-uniform in
    [n_lo, n_hi], nu = 1/re log-uniform in [1/2000, 1/100], M uniform in [m_lo, m_hi], a wake
    cloud (x in 0.5..20) seeded per instance."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        n = int(round(math.exp(rng.uniform(math.log(n_lo), math.log(n_hi)))))
        nu = math.exp(rng.uniform(math.log(1 / 2000), math.log(1 / 100)))
        m = int(rng.integers(m_lo, m_hi + 1))
        cx, cy = cylinder_corners(0.5, m)
        x, y, g = wake_cloud(n, 0.5, 20.0, body=(cx, cy), seed=seed * 100003 + k)
        out.append(Workload(f"cylinder_{k}", [(cx, cy)], x, y, g, re=1.0 / nu, dt=0.002))
    return out
