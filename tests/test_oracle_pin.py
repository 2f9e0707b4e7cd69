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


# ---- grid fields: XVelocity / XStreamfunction / XVorticity ---------------------------
import field_cases as FC  # noqa: E402


@pytest.mark.parametrize("case", golden_cases(GOLDEN, prefix="field_"))
def test_port_fields_match_golden(case):
    """The restatement's fields are bit-identical to the reference's (same operation order
    and the same C library), the gap lists included; the space is left as it was."""
    d = dict(np.load(os.path.join(GOLDEN, case + ".npz")))
    c = FC.case_from_fixture(d)
    S = oracle.OracleSpace("port")
    FC.load(S, c)
    before = S.vortices()
    got = FC.run_fields(S, c)
    after = S.vortices()
    S.close()
    for k, v in got.items():
        assert np.array_equal(v, d[k]), k
    for k in before:
        assert np.array_equal(before[k], after[k]), k


@pytest.mark.skipif(not oracle.ref_available(), reason="reference sources not present")
def test_port_fields_match_reference_live():
    """A case the fixtures do not hold: two sinks in one cell, a finer grid over the body."""
    c = dict(FC.cases()["cyl"])
    c["sinks"] = (np.array([0.71, 0.72, -1.3]), np.array([0.41, 0.42, 0.2]), np.array([0.5, -1.7, 3.2]))
    c["grid"] = (-1.0, -0.8, 0.05, 41, 33)
    outs = []
    for kind in ("port", "ref"):
        S = oracle.OracleSpace(kind)
        FC.load(S, c)
        outs.append(FC.run_fields(S, c))
        S.close()
    for k in outs[1]:
        assert np.array_equal(outs[0][k], outs[1][k]), k


def test_port_fields_reject_bad_arguments():
    """XField / X* throw std::invalid_argument (XField.cpp:17-23, XVelocity.cpp:42-44,
    XStreamfunction.cpp:49-50, XVorticity.cpp:28-29); with the tree built the oracle says so."""
    c = FC.cases()["no_vortices"]
    S = oracle.OracleSpace("port")
    FC.load(S, c)
    for kw in (dict(xres=1), dict(yres=0), dict(dxdy=0.0), dict(dxdy=float("inf"))):
        a = dict(xmin=-1.0, ymin=-1.0, dxdy=0.1, xres=8, yres=8)
        a.update(kw)
        with pytest.raises(oracle.OracleError):
            S.field_vorticity(a["xmin"], a["ymin"], a["dxdy"], a["xres"], a["yres"])
    with pytest.raises(oracle.OracleError):
        S.field_velocity(-1.0, -1.0, 0.1, 8, 8, mode="z")
    with pytest.raises(oracle.OracleError):
        S.field_velocity(-1.0, -1.0, 0.1, 8, 8, ref_frame="q")
    with pytest.raises(oracle.OracleError):
        S.field_streamfunction(-1.0, -1.0, 0.1, 8, 8, eps_mult=0.0)
    S.tree_build(8, 0.1, 1.0)
    with pytest.raises(oracle.OracleError):
        S.field_vorticity(-1.0, -1.0, 0.1, 8, 8)
    S.close()


# ---- moving bodies: attached sheets (MConvectiveFast.cpp:172-215, 440-457) ---------------
def test_port_attached_sheets_match_golden():
    import attached_cases as AC
    d = np.load(os.path.join(GOLDEN, "attached_bodies.npz"))
    S = oracle.OracleSpace("port")
    got = AC.run(S, AC.case(), oracle.default_body_params)
    S.close()
    for k in d.files:
        assert np.array_equal(got[k], d[k], equal_nan=True), k
    # the sheets matter: the same state with the body at rest differs well beyond rounding
    R = oracle.OracleSpace("port")
    rest = AC.run(R, AC.case(), oracle.default_body_params, moving=False)
    R.close()
    assert np.abs(rest["probe_vx"] - d["probe_vx"]).max() > 1e-2


@pytest.mark.skipif(not oracle.ref_available(), reason="reference sources not present")
def test_port_attached_sheets_match_reference_live():
    import attached_cases as AC
    c = AC.case()
    out = {}
    for kind in ("ref", "port"):
        S = oracle.OracleSpace(kind)
        out[kind] = AC.run(S, c, oracle.default_body_params, direct=False)
        S.close()
    for k in out["ref"]:
        assert np.array_equal(out["port"][k], out["ref"][k], equal_nan=True), k
