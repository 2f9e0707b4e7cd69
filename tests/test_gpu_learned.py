"""The learned far-field correction on the GPU (vvflow_gb300/csrc/learned.cu) against the
CPU restatement (oracle/mlp_oracle.py, itself pinned by finite differences):
* the tensor-core forward and gradients (BF16 operands, FP32 accumulation) against the
  restatement with the same BF16 roundings and FP64 accumulation: within 2e-2 of each
  block's largest magnitude (a BF16 rounding of a hidden unit can fall the other way);
* the samples (far cells by the reference's walk, features, FP64 direct-sum labels) within
  1e-5 of each column's largest magnitude;
* training lowers the loss, and the trained network lowers the error of the loose tree
  (theta = 0.8) against the FP64 direct sum on a configuration it was not trained on."""
import numpy as np
import pytest

import mlp_oracle as MO

FC08 = 3.125  # farCriteria of theta = 0.8


def _rand_params(rng):
    p = np.zeros(MO.NPARAM, np.float32)
    w1 = rng.normal(0, 0.3, (MO.HID, MO.KIN)).astype(np.float32)
    w1[:, MO.NF:] = 0
    p[MO.P_W1:MO.P_B1] = w1.ravel()
    p[MO.P_B1:MO.P_W2] = rng.normal(0, 0.1, MO.HID)
    p[MO.P_W2:MO.P_B2] = rng.normal(0, 0.2, MO.HID * MO.HID)
    p[MO.P_B2:MO.P_W3] = rng.normal(0, 0.1, MO.HID)
    p[MO.P_W3:MO.P_B3] = rng.normal(0, 0.2, MO.NOUT * MO.HID)
    p[MO.P_B3:] = rng.normal(0, 0.1, MO.NOUT)
    return p


def _mlp():
    from vvflow_gb300 import build as B
    from vvflow_gb300.vvgpu import Mlp
    B.build()
    return Mlp(seed=3)


def _blocks():
    return dict(W1=(MO.P_W1, MO.P_B1), b1=(MO.P_B1, MO.P_W2), W2=(MO.P_W2, MO.P_B2), b2=(MO.P_B2, MO.P_W3),
                W3=(MO.P_W3, MO.P_B3), b3=(MO.P_B3, MO.NPARAM))


@pytest.mark.gpu
def test_gpu_mlp_forward_matches_oracle():
    rng = np.random.default_rng(1)
    M = _mlp()
    p = _rand_params(rng)
    M.set_params(p)
    feat = rng.normal(0, 1, (1000, MO.NF)).astype(np.float32)
    y = M.forward(feat)
    ref, _ = MO.forward(p, feat.astype(np.float64), quant=True)
    M.close()
    err = np.abs(y - ref).max()
    assert err <= 2e-2 * np.abs(ref).max(), err


@pytest.mark.gpu
def test_gpu_mlp_gradient_matches_oracle():
    rng = np.random.default_rng(2)
    M = _mlp()
    p = _rand_params(rng)
    M.set_params(p)
    n = 1000
    feat = rng.normal(0, 1, (n, MO.NF)).astype(np.float32)
    lab = rng.normal(0, 1, (n, 2)).astype(np.float32)
    M.set_samples(feat, lab)
    g, loss = M.gradient()
    ref, rloss = MO.gradient(p, feat.astype(np.float64), lab.astype(np.float64), quant=True)
    M.close()
    assert abs(loss - rloss) <= 1e-3 * rloss
    for name, (a, b) in _blocks().items():
        err = np.abs(g[a:b] - ref[a:b]).max()
        assert err <= 2e-2 * np.abs(ref[a:b]).max(), (name, err, np.abs(ref[a:b]).max())


def _space(wl, fc, gpu=True):
    import oracle
    from vvflow_gb300.vvgpu import VVGPU_FP64, GpuSpace
    S = GpuSpace(VVGPU_FP64) if gpu else oracle.OracleSpace("port")
    S.load(wl)
    mn, mx = wl.node_sizes()
    S.tree_build(fc, mn, mx)
    return S


@pytest.mark.gpu
def test_gpu_mlp_samples_match_oracle():
    from vvflow_gb300 import workloads as W
    wl = W.cylinder_annulus(3000, 200, seed=4)
    rng = np.random.default_rng(4)
    r = np.sqrt(rng.uniform(0.55 ** 2, 3.0 ** 2, 60))
    a = rng.uniform(0, 2 * np.pi, 60)
    px, py = r * np.cos(a), r * np.sin(a)
    G = _space(wl, FC08)
    M = _mlp()
    n = M.add_samples(G, px, py)
    f, lab = M.samples()
    M.close()
    G.close()
    P = _space(wl, FC08, gpu=False)
    rf, rl, _ = MO.samples(P.tree_nodes(), P.vortices(), px, py, FC08)
    P.close()
    assert n == len(rf) and n > 0
    for k in range(MO.NF):
        sc = max(np.abs(rf[:, k]).max(), 1e-30)
        assert np.abs(f[:, k] - rf[:, k]).max() <= 1e-5 * sc, k
    for k in range(2):
        sc = np.abs(rl[:, k]).max()
        assert np.abs(lab[:, k] - rl[:, k]).max() <= 1e-5 * sc, k


def _training_set(M, seeds, n=20000, m=500, targets=4000):
    from vvflow_gb300 import workloads as W
    tot = 0
    for sd in seeds:
        wl = W.cylinder_annulus(n, m, seed=sd)
        G = _space(wl, FC08)
        rng = np.random.default_rng(100 + sd)
        pick = rng.choice(wl.n, targets, replace=False)
        tot += M.add_samples(G, wl.x[pick], wl.y[pick])
        G.tree_destroy()
        G.close()
    return tot


@pytest.mark.gpu
def test_gpu_mlp_training_lowers_tree_error():
    import oracle
    from vvflow_gb300 import workloads as W
    M = _mlp()
    nsamp = _training_set(M, seeds=(11, 12, 13, 14))
    assert nsamp > 100000
    M.fit_norm()
    losses = M.train(epochs=40, batch=4096, lr=2e-3, seed=5)
    assert losses[-1] < 0.2 * losses[0], losses
    # held-out configuration: the loose tree with and without the correction, the FP64
    # direct sum (each source's own epsilon) as the reference
    wl = W.cylinder_annulus(20000, 500, seed=21)
    G = _space(wl, FC08)
    G.eps(False)
    v = G.vortices()
    rng = np.random.default_rng(7)
    pick = rng.choice(len(v["x"]), 1500, replace=False)
    px, py = v["x"][pick], v["y"][pick]
    ux, uy = G.velocity_points(px, py)
    lx, ly, npairs = M.velocity_points(G, px, py)
    G.tree_destroy()
    G.close()
    P = oracle.OracleSpace("port")
    P.set_params(wl.re, wl.dt, wl.inf_vx, wl.inf_vy)
    P.set_vortices(v["x"], v["y"], v["g"], v["inv_eps"])
    dx, dy = P.direct_velocity(px, py)
    P.close()
    M.close()
    e_plain = np.hypot(ux - dx, uy - dy)
    e_learn = np.hypot(lx - dx, ly - dy)
    assert npairs > 0
    assert np.mean(e_learn) < 0.5 * np.mean(e_plain), (np.mean(e_learn), np.mean(e_plain))


@pytest.mark.gpu
def test_gpu_direct_sum_matches_oracle():
    """vvgpu_direct_velocity (no tree, each source's epsilon, sinks, free stream) against the
    restatement's direct sum, FP64 within 1e-12 of the largest velocity."""
    import oracle
    from vvflow_gb300 import workloads as W
    from vvflow_gb300.vvgpu import VVGPU_FP64, GpuSpace
    wl = W.cylinder_annulus(5000, 200, seed=8)
    rng = np.random.default_rng(8)
    ie = rng.uniform(5.0, 50.0, wl.n)
    ie[::17] = 0.0
    px = rng.uniform(-3, 3, 300)
    py = rng.uniform(-3, 3, 300)
    sinks = (np.array([0.8, -1.5]), np.array([0.2, 1.1]), np.array([0.3, -2.5]))
    out = []
    for S in (GpuSpace(VVGPU_FP64), oracle.OracleSpace("port")):
        S.set_params(wl.re, wl.dt, 1.0, 0.2)
        for cx, cy in wl.bodies:
            S.add_body(cx, cy)
        S.set_sinks(*sinks)
        S.set_vortices(wl.x, wl.y, wl.g, ie)
        out.append(S.direct_velocity(px, py))
        S.close()
    (gx, gy), (rx, ry) = out
    scale = np.abs(np.concatenate([rx, ry])).max()
    assert np.abs(gx - rx).max() <= 1e-12 * scale and np.abs(gy - ry).max() <= 1e-12 * scale
