"""Moving bodies: the attached vortex and source sheets of MConvectiveFast::body_list_influence
(libvvhd/src/MConvectiveFast.cpp:172-215, SegmentInfluence_linear_source :440-457).

One case, run the same way on every backend (the compiled reference, the C restatement,
the CUDA library): a cylinder translating and rotating about an axis off its centre
(speed_slae, holder + dpos) with circulation on its segments, a second body (an ellipse
with slip segments) at rest, and a vortex cloud around them with epsilon set.  Recorded:
the convective velocities of every vortex (process_all_lists), velocity(p) and the FP64
direct sum at probes, some within one segment length of the moving body's segments (the
linear-sheet branch) and some beyond (the point-singularity branch).
"""
from __future__ import annotations

import numpy as np


def case():
    from vvflow_gb300 import workloads as W
    rng = np.random.default_rng(77)
    cx, cy = W.cylinder_corners(0.5, 120)
    ex, ey = W.ellipse_corners(0.3, 0.15, 60, 20.0)
    ex = ex + 2.2
    ey = ey - 0.4
    x, y, g = W.annulus_cloud(6000, 0.53, 3.5, seed=78)
    # keep vortices out of the ellipse's neighbourhood
    far = np.hypot(x - 2.2, y + 0.4) > 0.45
    x, y, g = x[far], y[far], g[far]
    ie = rng.uniform(20.0, 200.0, len(x))
    ie[::23] = 0.0
    sg = rng.normal(0.0, 1e-3, len(cx))
    # probes: near the moving body's segment centres (inside |dl|) and farther out
    k = np.arange(0, len(cx), 7)
    mx = 0.5 * (cx[k] + np.roll(cx, -1)[k])
    my = 0.5 * (cy[k] + np.roll(cy, -1)[k])
    dl = np.hypot(np.roll(cx, -1)[k] - cx[k], np.roll(cy, -1)[k] - cy[k])
    r = np.hypot(mx, my)
    near_x = mx * (1 + 0.4 * dl / r)
    near_y = my * (1 + 0.4 * dl / r)
    far_x = rng.uniform(-3, 3, 40)
    far_y = rng.uniform(-3, 3, 40)
    px = np.concatenate([near_x, far_x])
    py = np.concatenate([near_y, far_y])
    return dict(cyl=(cx, cy), ell=(ex, ey), slip=np.arange(len(ex)) % 3 == 0, x=x, y=y, g=g, ie=ie, seg_g=sg,
                px=px, py=py, re=800.0, dt=0.004, inf=(1.0, 0.1))


def moving_params(bp):
    """The moving cylinder's parameters on a BodyParams of any backend."""
    bp.speed_slae_x = 0.3
    bp.speed_slae_y = -0.2
    bp.speed_slae_o = 0.7
    bp.holder_x = 0.1
    bp.holder_y = -0.05
    bp.dpos_x = 0.02
    bp.dpos_y = 0.01
    return bp


def run(S, c, params, direct=True, moving=True):
    """Loads the case into backend S (BodyParams factory `params`) and returns the records
    (the FP64 direct sum only with direct=True: the compiled reference has no direct sum;
    moving=False: the same cylinder at rest)."""
    S.set_params(c["re"], c["dt"], c["inf"][0], c["inf"][1])
    S.add_body(*c["cyl"], params=moving_params(params()) if moving else params())
    S.add_body(*c["ell"], slip=c["slip"].astype(np.uint32))
    m0 = len(c["cyl"][0])
    g = np.concatenate([c["seg_g"], np.full(len(c["ell"][0]), 2e-4)])
    S.set_segment_g(g)
    S.set_vortices(c["x"], c["y"], c["g"], c["ie"])
    out = {}
    dl = np.hypot(np.diff(np.append(c["cyl"][0], c["cyl"][0][0])), np.diff(np.append(c["cyl"][1], c["cyl"][1][0])))
    avg = dl.sum() / (m0 - 1)
    S.tree_build(8.0, 5 * avg, 100 * avg)
    S.convective()
    v = S.vortices()
    out["conv_vx"], out["conv_vy"], out["orig"] = v["vx"], v["vy"], v["orig"]
    out["probe_vx"], out["probe_vy"] = S.velocity_points(c["px"], c["py"])
    S.tree_destroy()
    if direct:
        out["direct_vx"], out["direct_vy"] = S.direct_velocity(c["px"], c["py"])
    return out
