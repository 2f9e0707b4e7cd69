"""The learned far field inside the convective pass (vvgpu_convective_learned,
vvflow_gb300/csrc/learned_step.cu) and its judge.

* Each leaf's correction of its constant far-field terms equals the CPU restatement
  (oracle/mlp_oracle.py leaf_correction: the same network with the same BF16 roundings at
  the leaf's centre for every far cell): within 2e-2 of the sum of the pair corrections'
  magnitudes per leaf, and within 1e-2 of the corrections' rms over the leaves (BF16
  roundings of a hidden unit can fall the other way; the hardware tanh).
* Host-side fault injection: corrupted weights make the judge revert the pass, which then
  equals, bit for bit, the plain pass at the judge's far criterion on the same tree.  A
  sound network at a loose bound is not reverted.
* A trained network lowers the pass's error against the FP64 direct sum on a configuration
  it was not trained on, compared with the same loose tree without it.
"""
import numpy as np
import pytest

import mlp_oracle as MO
import oracle

FC08 = 3.125  # farCriteria of theta = 0.8


def _built(wl, fc, precision=1, keep_far=True, inv_eps=None):
    from vvflow_gb300 import build as B
    from vvflow_gb300.vvgpu import GpuSpace
    B.build()
    S = GpuSpace(precision)
    S.set_params(wl.re, wl.dt, wl.inf_vx, wl.inf_vy)
    for cx, cy in wl.bodies:
        S.add_body(cx, cy)
    S.set_vortices(wl.x, wl.y, wl.g, inv_eps)
    S.keep_far_lists(keep_far)
    mn, mx = wl.node_sizes()
    S.tree_build(fc, mn, mx)
    return S


def _mlp(seed=3):
    from vvflow_gb300.vvgpu import Mlp
    return Mlp(seed=seed)


def _inv_eps(wl):
    """epsilon of the list from one pass without merging (the oracle)"""
    mn, mx = wl.node_sizes()
    R = oracle.OracleSpace("port")
    R.load(wl)
    R.tree_build(wl.far_criteria, mn, mx)
    R.eps(False)
    v = R.vortices()
    R.tree_destroy()
    R.close()
    ie = np.empty(wl.n)
    ie[v["orig"]] = v["inv_eps"]
    return ie


def _zero_v(S):
    S.set_velocities(np.zeros(S.n), np.zeros(S.n))


@pytest.mark.gpu
def test_learned_leaf_corrections_match_oracle():
    from vvflow_gb300 import workloads as W
    wl = W.cylinder_annulus(20000, 500, seed=31)
    ie = _inv_eps(wl)
    rng = np.random.default_rng(4)
    M = _mlp()
    S = _built(wl, FC08, inv_eps=ie)
    # standardisation from real samples, random weights of a realistic scale
    pick = rng.choice(wl.n, 2000, replace=False)
    M.add_samples(S, wl.x[pick], wl.y[pick])
    nrm = M.fit_norm()
    p = np.zeros(MO.NPARAM, np.float32)
    w1 = rng.normal(0, 0.3, (MO.HID, MO.KIN)).astype(np.float32)
    w1[:, MO.NF:] = 0
    p[MO.P_W1:MO.P_B1] = w1.ravel()
    p[MO.P_B1:MO.P_W2] = rng.normal(0, 0.1, MO.HID)
    p[MO.P_W2:MO.P_B2] = rng.normal(0, 0.2, MO.HID * MO.HID)
    p[MO.P_B2:MO.P_W3] = rng.normal(0, 0.1, MO.HID)
    p[MO.P_W3:MO.P_B3] = rng.normal(0, 0.2, MO.NOUT * MO.HID)
    p[MO.P_B3:] = rng.normal(0, 0.1, MO.NOUT)
    M.set_params(p)
    _zero_v(S)
    S.convective()
    vp = S.vortices()
    _zero_v(S)
    out = S.convective_learned(M, targets=0)
    vl = S.vortices()
    nodes = S.tree_nodes()
    lv = S.tree_leaves()
    S.tree_destroy()
    S.close()
    M.close()
    assert out["pairs"] > 0 and out["reverted"] == 0
    got, ref, mag = [], [], []
    for L in rng.choice(len(lv["x"]), 40, replace=False):
        a, b = int(lv["vfirst"][L]), int(lv["vlast"][L])
        live = np.flatnonzero(vp["g"][a:b] != 0) + a
        if len(live) == 0:
            continue
        d = np.stack([vl["vx"][live] - vp["vx"][live], vl["vy"][live] - vp["vy"][live]], 1)
        # one constant per leaf (the difference of two FP64 sums of the same terms)
        assert np.abs(d - d[0]).max() <= 1e-12 * (np.abs(vp["vx"][live]).max() + 1.0)
        rx, ry, m = MO.leaf_correction(p, nrm, nodes, vp, float(lv["x"][L]), float(lv["y"][L]), FC08)
        got.append(d[0])
        ref.append((rx, ry))
        mag.append(m)
    got, ref, mag = np.array(got), np.array(ref), np.array(mag)
    assert len(got) >= 30
    err = np.abs(got - ref).max(1)
    assert np.all(err <= 2e-2 * mag), (err / mag).max()
    assert np.sqrt(np.mean((got - ref) ** 2)) <= 1e-2 * np.sqrt(np.mean(ref ** 2))


@pytest.mark.gpu
def test_judge_reverts_corrupted_weights_to_the_plain_tree():
    from vvflow_gb300 import workloads as W
    wl = W.cylinder_annulus(20000, 500, seed=32)
    ie = _inv_eps(wl)
    M = _mlp()
    p = M.params()
    # a sound network (all zero: no correction) passes even a tight bound against itself
    M.set_params(np.zeros_like(p))
    S = _built(wl, FC08, inv_eps=ie)
    out = S.convective_learned(M, targets=4096, far_criteria=8.0, bound=1.0, seed=3)
    assert out["reverted"] == 0 and out["judged"] > 3000 and out["gap_rms"] < 1e-2
    S.tree_destroy()
    # injected fault: output weights corrupted on the host
    bad = np.zeros_like(p)
    bad[MO.P_B3:] = 1e6
    M.set_params(bad)
    S.tree_build(FC08, *wl.node_sizes())
    _zero_v(S)
    out = S.convective_learned(M, targets=4096, far_criteria=8.0, bound=5e-3, seed=3)
    assert out["reverted"] == 1 and out["gap_rms"] > 5e-3
    got = S.vortices()
    S.tree_destroy()
    S.close()
    M.close()
    # the plain pass at theta = 0.5 on the same tree (the partition does not depend on the
    # far criterion)
    R = _built(wl, 8.0, keep_far=False, inv_eps=ie)
    R.convective()
    ref = R.vortices()
    R.tree_destroy()
    R.close()
    assert np.array_equal(got["orig"], ref["orig"])
    assert np.array_equal(got["vx"], ref["vx"]) and np.array_equal(got["vy"], ref["vy"])


@pytest.mark.gpu
def test_trained_network_lowers_the_pass_error():
    from test_gpu_learned import _training_set
    from vvflow_gb300 import workloads as W
    M = _mlp(seed=7)
    assert _training_set(M, seeds=(11, 12, 13, 14)) > 100000
    M.fit_norm()
    M.train(epochs=40, batch=4096, lr=2e-3, seed=5)
    wl = W.cylinder_annulus(20000, 500, seed=23)
    ie = _inv_eps(wl)
    S = _built(wl, FC08, inv_eps=ie)
    _zero_v(S)
    S.convective()
    vp = S.vortices()
    _zero_v(S)
    out = S.convective_learned(M, targets=0)
    vl = S.vortices()
    S.tree_destroy()
    S.close()
    M.close()
    assert out["pairs"] > 0
    rng = np.random.default_rng(9)
    pick = rng.choice(np.flatnonzero(vp["g"] != 0), 1500, replace=False)
    P = oracle.OracleSpace("port")
    P.set_params(wl.re, wl.dt, wl.inf_vx, wl.inf_vy)
    P.set_vortices(vp["x"], vp["y"], vp["g"], vp["inv_eps"])
    dx, dy = P.direct_velocity(vp["x"][pick], vp["y"][pick])
    P.close()
    e_plain = np.sqrt(np.mean((vp["vx"][pick] - dx) ** 2 + (vp["vy"][pick] - dy) ** 2))
    e_learn = np.sqrt(np.mean((vl["vx"][pick] - dx) ** 2 + (vl["vy"][pick] - dy) ** 2))
    assert e_learn < 0.8 * e_plain, (e_learn, e_plain)
