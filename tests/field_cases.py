"""Seeded inputs for the grid fields of libvvhd (XVelocity.cpp, XStreamfunction.cpp,
XVorticity.cpp): body configurations, vortex clouds, sinks and the field calls made on
them.  ``run_fields`` drives any backend with the oracle's method names (OracleSpace,
GpuSpace) and returns every field as float32 arrays.
"""
from __future__ import annotations

import numpy as np

from vvflow_gb300 import workloads as W


def _cloud(rng, n, r0, r1):
    r = np.sqrt(rng.uniform(r0 * r0, r1 * r1, n))
    a = rng.uniform(0, 2 * np.pi, n)
    return r * np.cos(a), r * np.sin(a)


# (name, kind, kwargs): the calls of one case, in order
CALLS = [
    ("vel_x_o", "velocity", dict(mode="x", ref_frame="o")),
    ("vel_y_f", "velocity", dict(mode="y", ref_frame="f")),
    ("vel_x_b", "velocity", dict(mode="x", ref_frame="b")),
    ("psi_1_o", "streamfunction", dict(eps_mult=1.0, ref_frame="o")),
    ("psi_2_f", "streamfunction", dict(eps_mult=2.0, ref_frame="f")),
    ("omega_1", "vorticity", dict(eps_mult=1.0)),
    ("omega_2", "vorticity", dict(eps_mult=2.5)),
]


def cases():
    out = {}
    # cylinder with a vortex cloud around it, segment circulations, sinks (one in a cell)
    rng = np.random.default_rng(31)
    cx, cy = W.cylinder_corners(0.5, 200)
    n = 4000
    x, y = _cloud(rng, n, 0.52, 2.0)
    g = rng.normal(0, 1e-3, n)
    g[rng.random(n) < 0.03] = 0.0
    sg = rng.normal(0, 2e-3, len(cx))
    sinks = (np.array([1.234, -1.71, 0.05]), np.array([0.333, 0.9, -1.45]), np.array([0.02, -0.015, 0.01]))
    out["cyl"] = dict(bodies=[cx, cy], x=x, y=y, g=g, sg=sg, sinks=sinks, inf=(1.0, 0.1),
                      grid=(-2.1, -1.6, 0.1, 40, 32))
    # ellipse at incidence in a wake: a finer grid, leaves smaller than the cells
    rng = np.random.default_rng(32)
    ex, ey = W.ellipse_corners(0.5, 0.25, 300, 10.0)
    n = 6000
    x = rng.uniform(0.3, 4.0, n)
    y = rng.normal(0, 0.2 + 0.05 * x)
    keep = ~W.point_in_polygon(x, y, ex, ey)
    x, y = x[keep], y[keep]
    g = np.sign(np.sin(2 * np.pi * x / 1.2) * y) * rng.lognormal(np.log(1e-4), 0.5, len(x))
    sg = rng.normal(0, 1e-3, len(ex))
    out["ellipse"] = dict(bodies=[ex, ey], x=x, y=y, g=g, sg=sg, sinks=None, inf=(1.0, 0.0),
                          grid=(-0.7, -0.9, 0.037, 96, 48))
    # no free vortices: the fields of the attached layer alone
    cx, cy = W.cylinder_corners(0.5, 120)
    rng = np.random.default_rng(33)
    out["no_vortices"] = dict(bodies=[cx, cy], x=np.zeros(0), y=np.zeros(0), g=np.zeros(0),
                              sg=rng.normal(0, 1e-2, len(cx)), sinks=None, inf=(0.5, 0.0),
                              grid=(-1.0, -1.0, 0.125, 17, 17))
    return out


def load(sp, c):
    """Puts case ``c`` into a backend (OracleSpace or GpuSpace)."""
    sp.set_params(1000.0, 0.01, c["inf"][0], c["inf"][1])
    sp.add_body(c["bodies"][0], c["bodies"][1])
    sp.set_segment_g(np.asarray(c["sg"], np.float64))
    if c["sinks"] is not None:
        sp.set_sinks(*c["sinks"])
    sp.set_vortices(np.asarray(c["x"], np.float64), np.asarray(c["y"], np.float64), np.asarray(c["g"], np.float64))


def run_fields(sp, c, calls=CALLS):
    """Evaluates every call of ``calls`` on the loaded backend; returns {name: array}, plus
    the stream-function gap lists as name + "_gap_xi/_gap_yj/_gap"."""
    xmin, ymin, d, xres, yres = c["grid"]
    out = {}
    for name, kind, kw in calls:
        if kind == "velocity":
            out[name] = sp.field_velocity(xmin, ymin, d, xres, yres, **kw)
        elif kind == "streamfunction":
            f, (gx, gy, gv) = sp.field_streamfunction(xmin, ymin, d, xres, yres, **kw)
            out[name] = f
            out[name + "_gap_xi"], out[name + "_gap_yj"], out[name + "_gap"] = gx, gy, gv
        else:
            out[name] = sp.field_vorticity(xmin, ymin, d, xres, yres, **kw)
    return out


def case_arrays(c):
    """The inputs of case ``c`` as fixture arrays (in_*)."""
    kx, ky, kg = c["sinks"] if c["sinks"] is not None else (np.zeros(0),) * 3
    return dict(in_bx=np.asarray(c["bodies"][0]), in_by=np.asarray(c["bodies"][1]), in_x=np.asarray(c["x"]),
                in_y=np.asarray(c["y"]), in_g=np.asarray(c["g"]), in_sg=np.asarray(c["sg"]),
                in_kx=np.asarray(kx), in_ky=np.asarray(ky), in_kg=np.asarray(kg), in_inf=np.asarray(c["inf"]),
                in_grid=np.asarray(c["grid"], np.float64))


def case_from_fixture(d):
    """Inverse of case_arrays for a loaded fixture."""
    gr = d["in_grid"]
    sinks = (d["in_kx"], d["in_ky"], d["in_kg"]) if len(d["in_kx"]) else None
    return dict(bodies=[d["in_bx"], d["in_by"]], x=d["in_x"], y=d["in_y"], g=d["in_g"], sg=d["in_sg"],
                sinks=sinks, inf=(float(d["in_inf"][0]), float(d["in_inf"][1])),
                grid=(float(gr[0]), float(gr[1]), float(gr[2]), int(gr[3]), int(gr[4])))
