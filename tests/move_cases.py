"""Seeded inputs for the caller-side steps around the path: MFlowmove::move_and_clean
(libvvhd/src/MFlowmove.cpp:11-215) and Space::calc_forces / zero_forces
(libvvhd/src/TSpace.cpp:94-142).

Each move case is one body configuration, a vortex list with velocities and the segment
circulations; the runners drive any backend with the oracle's method names (OracleSpace,
GpuSpace) and return everything the calls change.
"""
from __future__ import annotations

import numpy as np

from vvflow_gb300 import workloads as W


def _cloud(rng, n, r0, r1):
    r = np.sqrt(rng.uniform(r0 * r0, r1 * r1, n))
    a = rng.uniform(0, 2 * np.pi, n)
    return r * np.cos(a), r * np.sin(a)


def cases():
    out = {}
    # cylinder, vortices inside and around it moving at random; small and zero g; zero and
    # slip segments; non-zero initial dead-vortex sums
    rng = np.random.default_rng(21)
    cx, cy = W.cylinder_corners(0.5, 200)
    n = 4000
    x, y = _cloud(rng, n, 0.3, 1.2)
    g = rng.normal(0, 1e-3, n)
    g[rng.random(n) < 0.05] = 3e-11
    g[rng.random(n) < 0.02] = 0.0
    slip = np.zeros(len(cx), np.uint32)
    slip[::37] = 1
    sg = rng.normal(0, 1e-3, len(cx))
    sg[rng.random(len(cx)) < 0.1] = 0.0
    out["cyl"] = dict(bodies=[(cx, cy, slip)], x=x, y=y, g=g, vx=rng.normal(0, 2.0, n),
                      vy=rng.normal(0, 2.0, n), sg=sg, dt=0.05, g_dead=[2e-3], fdt_dead=[(1e-3, -2e-3, 5e-4)])
    # ellipse at incidence plus a second cylinder: the first body that claims a point wins
    rng = np.random.default_rng(22)
    ex, ey = W.ellipse_corners(0.5, 0.25, 300, 10.0)
    c2x, c2y = W.cylinder_corners(0.3, 120)
    c2x = c2x + 1.2
    n = 3000
    x = rng.uniform(-0.8, 1.8, n)
    y = rng.uniform(-0.6, 0.6, n)
    g = rng.normal(0, 1e-3, n)
    sg = rng.normal(0, 1e-3, len(ex) + len(c2x))
    out["two_bodies"] = dict(bodies=[(ex, ey, None), (c2x, c2y, None)], x=x, y=y, g=g,
                             vx=rng.normal(0, 1.0, n), vy=rng.normal(0, 1.0, n), sg=sg, dt=0.05,
                             g_dead=[0.0, 0.0], fdt_dead=[(0, 0, 0), (0, 0, 0)])
    # inverted body (corners counter-clockwise, area < 0): points leaving the contour are
    # the invalid ones
    rng = np.random.default_rng(23)
    bx, by = W.cylinder_corners(2.0, 160)
    bx, by = bx[::-1].copy(), by[::-1].copy()
    n = 2000
    x, y = _cloud(rng, n, 0.0, 1.95)
    g = rng.normal(0, 1e-3, n)
    out["inverted"] = dict(bodies=[(bx, by, None)], x=x, y=y, g=g, vx=rng.normal(0, 3.0, n),
                           vy=rng.normal(0, 3.0, n), sg=rng.normal(0, 1e-3, len(bx)), dt=0.05,
                           g_dead=[0.0], fdt_dead=[(0, 0, 0)])
    # nothing but a body
    cx, cy = W.cylinder_corners(0.5, 40)
    out["empty"] = dict(bodies=[(cx, cy, None)], x=np.zeros(0), y=np.zeros(0), g=np.zeros(0),
                        vx=np.zeros(0), vy=np.zeros(0), sg=np.full(40, 1e-3), dt=0.01,
                        g_dead=[0.0], fdt_dead=[(0, 0, 0)])
    return out


def run_move(S, case, remove=True, bp_factory=None):
    """Applies one case to backend ``S`` (fresh) and returns the outputs."""
    S.set_params(600.0, case["dt"], 1.0, 0.0)
    for k, (bx, by, slip) in enumerate(case["bodies"]):
        bp = bp_factory()
        bp.g_dead = case["g_dead"][k]
        bp.fdt_dead_x, bp.fdt_dead_y, bp.fdt_dead_o = case["fdt_dead"][k]
        S.add_body(bx, by, slip, bp)
    S.set_segment_g(case["sg"])
    S.set_vortices(case["x"], case["y"], case["g"])
    if len(case["x"]):
        S.set_velocities(case["vx"], case["vy"])
    cleaned = S.move_and_clean(remove)
    v = S.vortices()
    seg = S.segments()
    out = {"cleaned": np.array(cleaned), "gsum": seg["gsum"]}
    for k in ("x", "y", "g", "inv_eps", "vx", "vy", "orig"):
        out[k] = v[k]
    bps = [S.body_params(k) for k in range(len(case["bodies"]))]
    out["dead"] = np.array([[b["fdt_dead_x"], b["fdt_dead_y"], b["fdt_dead_o"], b["g_dead"]] for b in bps])
    return out


def forces_cases():
    out = {}
    for name, re in (("viscous", 600.0), ("inviscid", float("inf"))):
        rng = np.random.default_rng(31)
        bodies = [W.cylinder_corners(0.5, 300), W.ellipse_corners(0.5, 0.25, 200, 10.0)]
        m = sum(len(b[0]) for b in bodies)
        out[name] = dict(re=re, dt=0.002, bodies=bodies,
                         s1=[rng.normal(0, 1e-3, m), rng.normal(0, 1e-2, m), rng.normal(0, 1e-3, m)],
                         s2=[rng.normal(0, 1e-3, m), rng.normal(0, 1e-2, m), rng.normal(0, 1e-3, m)],
                         dead=[(2e-3, (1e-3, -2e-3, 5e-4)), (-1e-3, (0.0, 3e-4, -1e-4))])
    return out


def run_forces(S, case, bp_factory):
    """calc_forces, zero_forces, calc_forces again with new segment state."""
    S.set_params(case["re"], case["dt"], 1.0, 0.0)
    for k, (bx, by) in enumerate(case["bodies"]):
        bp = bp_factory()
        bp.g_dead = case["dead"][k][0]
        bp.fdt_dead_x, bp.fdt_dead_y, bp.fdt_dead_o = case["dead"][k][1]
        S.add_body(bx, by, None, bp)
    S.set_segment_state(*case["s1"])
    out = {"f1": S.calc_forces()}
    sf = S.segment_forces()
    out.update({k + "1": v for k, v in sf.items()})
    S.zero_forces()
    bps = [S.body_params(k) for k in range(len(case["bodies"]))]
    out["after_zero"] = np.array([[b[k] for k in ("friction_prev_x", "friction_prev_y", "friction_prev_o",
                                                    "fdt_dead_x", "fdt_dead_y", "fdt_dead_o", "g_dead")]
                                  for b in bps])
    seg = S.segments()
    out["gsum_zero"], out["fric_zero"] = seg["gsum"], seg["fric"]
    S.set_segment_state(*case["s2"])
    out["f2"] = S.calc_forces()
    sf = S.segment_forces()
    out.update({k + "2": v for k, v in sf.items()})
    return out
