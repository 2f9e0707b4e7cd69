"""Generates the golden fixtures in this folder from the reference itself.

Run where the reference sources are present (they are compiled unmodified by
``make -C oracle ref``).  The fixtures are the reference's outputs for one full step
of the hot path (tests/protocol.py) on small seeded workloads, so parity tests on
machines without the reference sources still compare against the reference.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import oracle  # noqa: E402
from protocol import advance, run_step  # noqa: E402
from vvflow_gb300 import workloads as W  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def cases():
    """name -> (workload, full_lists, two_steps)"""
    out = {}
    out["cyl_small"] = (W.cylinder_annulus(2000, 100, seed=5), True, True)
    out["cyl_c1"] = (W.cylinder_annulus(20000, 500, seed=1), False, False)
    cx, cy = W.ellipse_corners(0.5, 0.25, 200, 10.0)
    x, y, g = W.wake_cloud(6000, 0.5, 6.0, body=(cx, cy), seed=7)
    out["ell_wake"] = (W.Workload("ell_wake", [(cx, cy)], x, y, g, re=1e4, dt=0.002), True, True)
    x, y, g = W.annulus_cloud(3000, 0.1, 2.0, seed=11)
    out["nobody"] = (W.Workload("nobody", [], x, y, g, re=600.0, dt=0.005), True, False)
    cx, cy = W.cylinder_corners(0.5, 24)
    x, y, g = W.annulus_cloud(10, 0.6, 1.0, seed=12)
    out["tiny"] = (W.Workload("tiny", [(cx, cy)], x, y, g, re=600.0, dt=0.005), True, True)
    # zero circulations, exact duplicates and a sparse far cluster
    cx, cy = W.cylinder_corners(0.5, 64)
    x, y, g = W.annulus_cloud(1500, 0.55, 1.5, seed=13)
    g[::17] = 0.0
    x[1::31] = x[0::31][: len(x[1::31])]
    y[1::31] = y[0::31][: len(y[1::31])]
    x = np.concatenate([x, 40 + 0.01 * np.arange(20)])
    y = np.concatenate([y, np.zeros(20)])
    g = np.concatenate([g, np.full(20, 1e-4)])
    out["edge"] = (W.Workload("edge", [(cx, cy)], x, y, g, re=600.0, dt=0.005), True, True)
    out["empty"] = (W.Workload("empty", [(cx, cy)], np.zeros(0), np.zeros(0), np.zeros(0),
                               re=600.0, dt=0.005), True, True)
    return out


def run_case(kind, wl, full_lists, two_steps):
    S = oracle.OracleSpace(kind)
    S.load(wl)
    res = run_step(S, wl, full_lists=full_lists)
    if two_steps:
        x, y, g, ie = advance(S, wl, res)
        S.set_params(wl.re, wl.dt, wl.inf_vx, wl.inf_vy, 0.0, wl.dt)
        S.set_vortices(x, y, g, ie)
        res2 = run_step(S, wl, full_lists=full_lists)
        res.update({"s2_" + k: v for k, v in res2.items()})
        res["s2_in_x"], res["s2_in_y"], res["s2_in_g"], res["s2_in_inv_eps"] = x, y, g, ie
    S.close()
    return res


def main():
    oracle.build(ref=True)
    if not oracle.ref_available():
        raise SystemExit("reference library not available; run where the reference sources are")
    for name, (wl, full, two) in cases().items():
        res = run_case("ref", wl, full, two)
        inp = {"in_x": wl.x, "in_y": wl.y, "in_g": wl.g, "in_re": np.array(wl.re),
               "in_dt": np.array(wl.dt), "in_inf": np.array([wl.inf_vx, wl.inf_vy]),
               "in_fc": np.array(wl.far_criteria), "in_nbodies": np.array(len(wl.bodies))}
        for i, (cx, cy) in enumerate(wl.bodies):
            inp[f"in_body{i}_cx"], inp[f"in_body{i}_cy"] = cx, cy
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **inp, **res)
        print(name, "n", wl.n, "m", wl.m, "merged", int(res["merged"]),
              "size", os.path.getsize(os.path.join(HERE, f"{name}.npz")))


if __name__ == "__main__":
    main()
