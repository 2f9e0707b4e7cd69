"""Failure paths of the C ABI, each made on the host or by a wait that is told to run out;
none of them faults the GPU.

* A singular body system: the reference's LU reports a zero pivot and the reference exits
  (libvvhd/src/TMatrix.cpp:195-213); here vvgpu_slae returns VVGPU_ERR_SINGULAR.  A
  contour traversed twice gives pairs of equal rows, which the oracle's LU also rejects.
* Non-finite vortex input is reported as VVGPU_ERR_ARG by the first call that reads it.
* The epsilon/merge pass given a round limit below what it needs returns
  VVGPU_ERR_TIMEOUT and leaves the vortex list untouched.
* Tensor-core waits given a limit of zero polls run out at once: the call returns
  VVGPU_ERR_TIMEOUT, and with the default limit back the model gives the same results as
  before (the kernels let their MMAs land and release their tensor memory).
* The FP32 near field's shared-memory staging waits (bulk copies on an mbarrier), given
  zero polls, run out at once: vvgpu_convective returns VVGPU_ERR_TIMEOUT after its copies
  have landed, and with the default limit back it gives the same velocities as before.
After each failure the context (or model) keeps working."""
import numpy as np
import pytest

import oracle
from vvflow_gb300 import workloads as W

ERR_ARG, ERR_SINGULAR, ERR_TIMEOUT = -1, -5, -8


def _space(precision=0):
    from vvflow_gb300 import build as B
    from vvflow_gb300.vvgpu import GpuSpace
    B.build()
    return GpuSpace(precision)


def _err(fn, *a):
    from vvflow_gb300.vvgpu import VVGpuError
    with pytest.raises(VVGpuError) as ei:
        fn(*a)
    return ei.value.code


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
def test_singular_slae_is_reported(precision):
    wl = W.cylinder_annulus(2000, 100, seed=3)
    cx, cy = wl.bodies[0]
    twice = (np.concatenate([cx, cx]), np.concatenate([cy, cy]))
    mn, mx = wl.node_sizes()
    # the oracle (the reference's algorithm) rejects the same system
    R = oracle.OracleSpace("port")
    R.set_params(wl.re, wl.dt, 1.0, 0.0)
    R.add_body(*twice)
    R.set_vortices(wl.x, wl.y, wl.g)
    R.tree_build(8.0, mn, mx)
    with pytest.raises(oracle.OracleError):
        R.slae()
    R.close()
    S = _space(precision)
    S.set_params(wl.re, wl.dt, 1.0, 0.0)
    S.add_body(*twice)
    S.set_vortices(wl.x, wl.y, wl.g)
    S.tree_build(8.0, mn, mx)
    assert _err(S.slae) == ERR_SINGULAR
    S.tree_destroy()
    # the context keeps working: the same state with the proper contour solves
    S.clear_bodies()
    S.add_body(cx, cy)
    S.set_vortices(wl.x, wl.y, wl.g)
    S.tree_build(8.0, mn, mx)
    S.slae()
    _, _, x = S.slae_export()
    S.tree_destroy()
    S.close()
    assert np.all(np.isfinite(x))


@pytest.mark.gpu
def test_nonfinite_vortex_input_is_reported():
    wl = W.cylinder_annulus(3000, 100, seed=4)
    mn, mx = wl.node_sizes()
    S = _space(1)
    S.set_params(wl.re, wl.dt, 1.0, 0.0)
    S.add_body(*wl.bodies[0])
    for k, bad in (("x", np.nan), ("y", np.inf), ("g", -np.inf), ("ie", np.nan), ("ie", -1.0)):
        x, y, g = wl.x.copy(), wl.y.copy(), wl.g.copy()
        ie = np.zeros_like(x)
        {"x": x, "y": y, "g": g, "ie": ie}[k][17] = bad
        S.set_vortices(x, y, g, ie)
        assert _err(S.tree_build, 8.0, mn, mx) == ERR_ARG, k
        S.set_vortices(x, y, g, ie)
        assert _err(S.direct_velocity, np.array([1.0]), np.array([0.0])) == ERR_ARG, k
    # epsilon 0 (+inf inverse) is a valid state; so is the list after the failures
    ie = np.zeros_like(wl.x)
    ie[5] = np.inf
    S.set_vortices(wl.x, wl.y, wl.g, ie)
    S.tree_build(8.0, mn, mx)
    S.tree_destroy()
    S.close()


@pytest.mark.gpu
def test_eps_round_limit_times_out_and_leaves_the_list():
    wl = W.cylinder_annulus(20000, 500, seed=3)
    mn, mx = wl.node_sizes()
    S = _space(0)
    S.load(wl)
    S.tree_build(wl.far_criteria, mn, mx)
    before = S.vortices()
    S.set_eps_round_limit(1)
    assert _err(S.eps, True) == ERR_TIMEOUT
    after = S.vortices()
    for k in ("x", "y", "g", "inv_eps", "orig"):
        assert np.array_equal(before[k], after[k]), k
    S.set_eps_round_limit(4096)
    merged = S.eps(True)
    got = S.vortices()
    st = S.stats()
    S.tree_destroy()
    S.close()
    assert st["merge_rounds"] > 1
    F = _space(0)
    F.load(wl)
    F.tree_build(wl.far_criteria, mn, mx)
    assert F.eps(True) == merged
    ref = F.vortices()
    F.tree_destroy()
    F.close()
    for k in ("x", "y", "g", "inv_eps", "orig"):
        assert np.array_equal(ref[k], got[k]), k


@pytest.mark.gpu
def test_tensor_core_wait_limit_times_out_and_recovers():
    from vvflow_gb300 import build as B
    from vvflow_gb300.vvgpu import Mlp
    B.build()
    rng = np.random.default_rng(5)
    M = Mlp(seed=2)
    feat = rng.normal(0, 1, (3000, Mlp.NF)).astype(np.float32)
    lab = rng.normal(0, 1, (3000, 2)).astype(np.float32)
    y0 = M.forward(feat)
    M.set_samples(feat, lab)
    g0, _ = M.gradient()
    M.set_wait_limit(0)
    assert _err(M.forward, feat) == ERR_TIMEOUT
    assert _err(M.gradient) == ERR_TIMEOUT
    M.set_wait_limit(1 << 22)
    assert np.array_equal(M.forward(feat), y0)
    g1, _ = M.gradient()
    assert np.array_equal(g0, g1)
    M.close()


@pytest.mark.gpu
def test_staging_wait_limit_times_out_and_recovers():
    wl = W.cylinder_annulus(20000, 500, seed=3)
    mn, mx = wl.node_sizes()
    S = _space(1)
    S.load(wl)
    S.tree_build(wl.far_criteria, mn, mx)
    S.eps(False)
    zero = np.zeros(wl.n)
    S.set_velocities(zero, zero)
    S.convective()
    ref = S.vortices()
    S.set_wait_limit(0)
    S.set_velocities(zero, zero)
    assert _err(S.convective) == ERR_TIMEOUT
    S.set_wait_limit()
    S.set_velocities(zero, zero)
    S.convective()
    got = S.vortices()
    S.tree_destroy()
    S.close()
    assert np.abs(ref["vx"]).max() > 0
    for k in ("vx", "vy", "orig"):
        assert np.array_equal(ref[k], got[k]), k
