"""The CPU restatement of the learned correction (oracle/mlp_oracle.py) pinned by
mathematics: gradients against central finite differences of the FP64 network, labels
against their definition (the cell's exact velocity minus the monopoles equals the
multipole tail for a distant target)."""
import math

import numpy as np

import mlp_oracle as MO


def _params(rng):
    p = np.zeros(MO.NPARAM)
    p[MO.P_W1:MO.P_B1] = rng.normal(0, 0.3, MO.HID * MO.KIN)
    p[MO.P_W1:MO.P_B1].reshape(MO.HID, MO.KIN)[:, MO.NF:] = 0
    p[MO.P_B1:MO.P_W2] = rng.normal(0, 0.1, MO.HID)
    p[MO.P_W2:MO.P_B2] = rng.normal(0, 0.2, MO.HID * MO.HID)
    p[MO.P_B2:MO.P_W3] = rng.normal(0, 0.1, MO.HID)
    p[MO.P_W3:MO.P_B3] = rng.normal(0, 0.2, MO.NOUT * MO.HID)
    p[MO.P_B3:] = rng.normal(0, 0.1, MO.NOUT)
    return p


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(5)
    p = _params(rng)
    feat = rng.normal(0, 1, (37, MO.NF))
    lab = rng.normal(0, 1, (37, 2))
    g, _ = MO.gradient(p, feat, lab, quant=False)
    idx = np.concatenate([rng.choice(np.arange(MO.P_W1, MO.P_B1).reshape(MO.HID, MO.KIN)[:, :MO.NF].ravel(), 6),
                          rng.integers(MO.P_B1, MO.NPARAM, 24)])
    h = 1e-6
    for i in idx:
        e = np.zeros(MO.NPARAM)
        e[i] = h
        fd = (MO.loss(p + e, feat, lab) - MO.loss(p - e, feat, lab)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])


def test_oracle_bf16_rounding():
    v = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 0.0, 1e-30], np.float32)
    r = MO.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0          # tie to even
    assert r[2] == np.float32(1.0078125)
    assert abs(r[3] + 3.140625) < 1e-7
    assert r[4] == 0.0


def test_oracle_label_is_multipole_tail():
    """For a cell far from the target the normalised residual approaches the quadrupole
    term of the complex expansion about each centroid, summed: (1/2pi) sum M2 / (z - c)^3,
    in the normalisation of the features."""
    rng = np.random.default_rng(3)
    n = 200
    xs = rng.uniform(-0.5, 0.5, n)
    ys = rng.uniform(-0.3, 0.3, n)
    gs = rng.normal(0, 1, n)
    pos, neg = gs > 0, gs < 0
    cp = (np.sum(gs[pos] * xs[pos]) / gs[pos].sum(), np.sum(gs[pos] * ys[pos]) / gs[pos].sum(), gs[pos].sum())
    cm = (np.sum(gs[neg] * xs[neg]) / gs[neg].sum(), np.sum(gs[neg] * ys[neg]) / gs[neg].sum(), gs[neg].sum())
    nodes = {k: np.array([v]) for k, v in dict(x=0.0, y=0.0, h=0.6, w=1.0, cmp_x=cp[0], cmp_y=cp[1], cmp_g=cp[2],
                                                 cmm_x=cm[0], cmm_y=cm[1], cmm_g=cm[2]).items()}
    nodes["vfirst"] = np.array([0])
    nodes["vlast"] = np.array([n])
    vort = dict(x=xs, y=ys, g=gs)
    px, py = 40.0, 25.0
    f, lab, back = MO.cell_sample(nodes, vort, 0, px, py)
    z = px + 1j * py
    w = 0j
    for c, sel in ((cp, pos), (cm, neg)):
        zc = c[0] + 1j * c[1]
        M2 = np.sum(gs[sel] * ((xs[sel] - c[0]) + 1j * (ys[sel] - c[1])) ** 2)
        w += M2 / (z - zc) ** 3
    # complex velocity u - i v = (1 / 2 pi i) sum g / (z - zj): the tail's (u, v)
    tail = w / (2j * math.pi)
    u, v = tail.real, -tail.imag
    got = lab * back
    assert np.allclose(got, [u, v], rtol=0.05, atol=1e-3 * abs(u + 1j * v))
