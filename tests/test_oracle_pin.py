"""Pins the CPU oracle (C restatement) to the reference.

1. Against the golden fixtures produced by the reference's own compiled sources
   (tests/golden/make_golden.py): every tree/epsilon/merge output bit-exact; sums within
   1e-13 (only libm exp/log may differ in the last bit between hosts).
2. Where the reference sources are present, against the compiled reference directly on
   further seeds.
"""
import os

import numpy as np
import pytest

import oracle
from parity import check_step, golden_cases, load_workload
from protocol import advance, run_step
from vvflow_gb300 import workloads as W

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _run(kind, wl, full_lists, d=None):
    S = oracle.OracleSpace(kind)
    S.load(wl)
    out = run_step(S, wl, full_lists=full_lists)
    if d is not None and "s2_in_x" in d:
        x, y, g, ie = advance(S, wl, out)
        assert np.array_equal(x, d["s2_in_x"]) and np.array_equal(ie, d["s2_in_inv_eps"])
        S.set_params(wl.re, wl.dt, wl.inf_vx, wl.inf_vy, 0.0, wl.dt)
        S.set_vortices(x, y, g, ie)
        out2 = run_step(S, wl, full_lists=full_lists)
        out.update({"s2_" + k: v for k, v in out2.items()})
    S.close()
    return out


@pytest.mark.parametrize("case", golden_cases(GOLDEN))
def test_port_matches_golden(case):
    wl, d = load_workload(os.path.join(GOLDEN, case + ".npz"))
    got = _run("port", wl, full_lists="t1_near_path" in d or "t2_near_path" in d, d=d)
    tol = dict(vel_tol=1e-13, diff_tol=1e-13, fric_tol=1e-13, slae_tol=1e-13)
    bad = check_step(d, got, **tol)
    if "s2_in_x" in d:
        bad += check_step(d, got, prefix="s2_", **tol)
    assert not bad, bad


@pytest.mark.skipif(not oracle.ref_available(), reason="reference sources not present")
@pytest.mark.parametrize("seed", [21, 22])
def test_port_matches_reference_live(seed):
    cx, cy = W.ellipse_corners(0.5, 0.25, 160, 5.0 * seed)
    x, y, g = W.wake_cloud(4000, 0.5, 5.0, body=(cx, cy), seed=seed)
    wl = W.Workload("live", [(cx, cy)], x, y, g, re=2000.0, dt=0.004)
    a = _run("ref", wl, True)
    b = _run("port", wl, True)
    bad = check_step(a, b, vel_tol=0, diff_tol=0, fric_tol=0, slae_tol=0)
    assert not bad, bad


# ---- MFlowmove::move_and_clean -------------------------------------------------------
from move_cases import cases as move_cases, run_move  # noqa: E402
from parity import check_move  # noqa: E402


@pytest.mark.parametrize("case", golden_cases(GOLDEN, prefix="move_"))
def test_port_move_matches_golden(case):
    d = dict(np.load(os.path.join(GOLDEN, case + ".npz")))
    c = move_cases()[case[len("move_"):]]
    for remove in (True, False):
        S = oracle.OracleSpace("port")
        got = run_move(S, c, remove, oracle.default_body_params)
        S.close()
        check_move(got, d, "rm_" if remove else "keep_")


@pytest.mark.skipif(not oracle.ref_available(), reason="reference sources not present")
def test_port_move_matches_reference_live():
    rng = np.random.default_rng(99)
    c = move_cases()["cyl"]
    c = dict(c, vx=rng.normal(0, 3.0, len(c["x"])), vy=rng.normal(0, 3.0, len(c["x"])))
    outs = []
    for kind in ("port", "ref"):
        S = oracle.OracleSpace(kind)
        outs.append(run_move(S, c, True, oracle.default_body_params))
        S.close()
    check_move(outs[0], {"rm_" + k: v for k, v in outs[1].items()}, "rm_")


# ---- Space::calc_forces / zero_forces -----------------------------------------------
from move_cases import forces_cases, run_forces  # noqa: E402


@pytest.mark.parametrize("case", golden_cases(GOLDEN, prefix="forces_"))
def test_port_forces_match_golden(case):
    d = dict(np.load(os.path.join(GOLDEN, case + ".npz")))
    S = oracle.OracleSpace("port")
    got = run_forces(S, forces_cases()[case[len("forces_"):]], oracle.default_body_params)
    S.close()
    check_move(got, d, "")
