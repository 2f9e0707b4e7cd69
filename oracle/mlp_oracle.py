"""CPU restatement of the learned far-field correction -- TEST INFRASTRUCTURE ONLY.

The GPU kernels (vvflow_gb300/csrc/learned.cu) are checked against this module:
* the samples: for a target point, the far cells of its leaf by the reference's
  depth-first walk (snode::FindNearNodes, libvvhd/src/TSortedTree.cpp:199-217), the cell
  features and the label (exact FP64 Biot-Savart sum over the cell minus the two monopoles
  of MConvectiveFast::far_nodes_influence, libvvhd/src/MConvectiveFast.cpp:139-151);
* the network 20 -> 64 -> 64 -> 2 (tanh-GELU): forward and gradients of the mean squared
  error, with the tensor-core operands rounded to BF16 where the kernels round them and
  FP64 accumulation in place of the tensor cores' FP32.

The gradient formulas are themselves pinned by central finite differences of the
unrounded FP64 network (tests/test_learned_oracle.py).  No reference code exists for this
part: the reference has no learned component.
"""
from __future__ import annotations

import math

import numpy as np

NF, KIN, HID, NOUT = 20, 32, 64, 2
P_W1 = 0
P_B1 = P_W1 + HID * KIN
P_W2 = P_B1 + HID
P_B2 = P_W2 + HID * HID
P_W3 = P_B2 + HID
P_B3 = P_W3 + NOUT * HID
NPARAM = P_B3 + NOUT
GC = 0.7978845608028654
GA = 0.044715


def bf16(a):
    """Round float32 values to the nearest BF16 (ties to even), returned as float32."""
    a = np.ascontiguousarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).reshape(a.shape)


def unpack(p):
    p = np.asarray(p, np.float64)
    return (p[P_W1:P_B1].reshape(HID, KIN), p[P_B1:P_W2], p[P_W2:P_B2].reshape(HID, HID), p[P_B2:P_W3],
            p[P_W3:P_B3].reshape(NOUT, HID), p[P_B3:NPARAM])


def gelu(z):
    return 0.5 * z * (1.0 + np.tanh(GC * (z + GA * z ** 3)))


def gelu_d(z):
    t = np.tanh(GC * (z + GA * z ** 3))
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * GC * (1.0 + 3.0 * GA * z * z)


def _q(a, quant):
    return bf16(a).astype(np.float64) if quant else np.asarray(a, np.float64)


def forward(p, feat, quant=True):
    """Outputs y [n][2] and the intermediates (X, Z1, H1, Z2, H2)."""
    W1, b1, W2, b2, W3, b3 = unpack(p)
    n = len(feat)
    X = np.zeros((n, KIN))
    X[:, :NF] = feat
    Xq = _q(X, quant)
    Z1 = Xq @ _q(W1, quant).T
    H1 = _q(gelu(Z1 + b1), quant)
    Z2 = H1 @ _q(W2, quant).T
    H2 = _q(gelu(Z2 + b2), quant)
    Y = H2 @ _q(W3, quant).T + b3
    return Y, (Xq, Z1, H1, Z2, H2)


def loss(p, feat, lab, quant=False):
    Y, _ = forward(p, feat, quant)
    return float(np.sum((Y - lab) ** 2) / len(feat))


def gradient(p, feat, lab, quant=True):
    """Gradient of (1/n) sum |y - t|^2 in the parameter layout of the kernels."""
    W1, b1, W2, b2, W3, b3 = unpack(p)
    n = len(feat)
    Y, (Xq, Z1, H1, Z2, H2) = forward(p, feat, quant)
    dY = 2.0 / n * (Y - lab)
    dYq = _q(dY, quant)
    g = np.zeros(NPARAM)
    g[P_W3:P_B3] = (dYq.T @ H2).ravel()
    g[P_B3:NPARAM] = dY.sum(0)
    dH2 = dYq @ _q(W3, quant)
    dZ2 = dH2 * gelu_d(Z2 + b2)
    dZ2q = _q(dZ2, quant)
    g[P_W2:P_B2] = (dZ2q.T @ H1).ravel()
    g[P_B2:P_W3] = dZ2.sum(0)
    dH1 = dZ2q @ _q(W2, quant)
    dZ1 = dH1 * gelu_d(Z1 + b1)
    dZ1q = _q(dZ1, quant)
    dW1 = dZ1q.T @ Xq
    dW1[:, NF:] = 0.0
    g[P_W1:P_B1] = dW1.ravel()
    g[P_B1:P_W2] = dZ1.sum(0)
    return g, float(np.sum((Y - lab) ** 2) / n)


# ---- samples --------------------------------------------------------------------------

def _children(nodes):
    key = {(int(d), int(pa)): i for i, (d, pa) in enumerate(zip(nodes["depth"], nodes["path"]))}
    nn = len(nodes["x"])
    ch = np.full(nn, -1, np.int64)
    for i in range(nn):
        c = key.get((int(nodes["depth"][i]) + 1, 2 * int(nodes["path"][i])))
        if c is not None:
            ch[i] = c
    root = key[(0, 0)]
    c2 = np.full(nn, -1, np.int64)
    for i in range(nn):
        if ch[i] >= 0:
            c2[i] = key[(int(nodes["depth"][i]) + 1, 2 * int(nodes["path"][i]) + 1)]
    return root, ch, c2


def far_cells(nodes, px, py, far_criteria):
    """Far nodes of the leaf holding (px, py), in depth-first order (exact FP64 test)."""
    root, ch1, ch2 = _children(nodes)
    x, y, h, w = nodes["x"], nodes["y"], nodes["h"], nodes["w"]
    k = root
    while ch1[k] >= 0:
        if h[k] < w[k]:
            k = ch1[k] if px < x[k] else ch2[k]
        else:
            k = ch1[k] if py < y[k] else ch2[k]
    me = k
    out, stack = [], [root]
    while stack:
        u = stack.pop()
        ddx, ddy = x[u] - x[me], y[u] - y[me]
        hp = ((h[u] + w[u]) + h[me]) + w[me]
        if ddx * ddx + ddy * ddy > (far_criteria * hp) * hp:
            out.append(u)
            continue
        if ch1[u] >= 0:
            stack.append(ch2[u])
            stack.append(ch1[u])
    return out


def cell_sample(nodes, vort, u, px, py, with_label=True):
    """(features [20], label [2], factor back to velocity) of far cell u for target (px, py);
    with_label=False leaves the label (an exact sum over the cell) at 0."""
    gx, gy = nodes["x"][u], nodes["y"][u]
    sz = nodes["h"][u] + nodes["w"][u]
    cp = (nodes["cmp_x"][u], nodes["cmp_y"][u], nodes["cmp_g"][u])
    cm = (nodes["cmm_x"][u], nodes["cmm_y"][u], nodes["cmm_g"][u])
    G = cp[2] - cm[2]
    dx, dy = px - gx, py - gy
    d2 = dx * dx + dy * dy
    d = math.sqrt(d2)
    if not (G > 0 and sz > 0):
        return np.zeros(NF), np.zeros(2), 0.0
    f = np.zeros(NF)
    f[0], f[1] = cp[2] / G, cm[2] / G
    f[2], f[3] = (cp[0] - gx) / sz, (cp[1] - gy) / sz
    f[4], f[5] = (cm[0] - gx) / sz, (cm[1] - gy) / sz
    a, b = int(nodes["vfirst"][u]), int(nodes["vlast"][u])
    xs, ys, gs = vort["x"][a:b], vort["y"][a:b], vort["g"][a:b]
    for sgn, c in ((0, cp), (1, cm)):
        sel = (gs > 0) if sgn == 0 else (gs < 0)
        wz = (xs[sel] - c[0]) + 1j * (ys[sel] - c[1])
        for e, k in enumerate((2, 3, 4)):
            mk = np.sum(gs[sel] * wz ** k) / (G * sz ** k)
            f[6 + 6 * sgn + 2 * e] = mk.real
            f[6 + 6 * sgn + 2 * e + 1] = mk.imag
    f[18], f[19] = dx / sz, dy / sz
    norm = 2 * math.pi * d2 * d / (G * sz * sz)
    if not with_label:
        return f, np.zeros(2), 1.0 / norm
    nz = gs != 0
    rx, ry = px - xs[nz], py - ys[nz]
    q = gs[nz] / (rx * rx + ry * ry)
    ex, ey = np.sum(-ry * q), np.sum(rx * q)
    mx = my = 0.0
    for c in (cp, cm):
        if c[2] == 0:
            continue
        rx, ry = px - c[0], py - c[1]
        q = c[2] / (rx * rx + ry * ry)
        mx -= ry * q
        my += rx * q
    lab = np.array([(ex - mx) / (2 * math.pi) * norm, (ey - my) / (2 * math.pi) * norm])
    return f, lab, 1.0 / norm


def samples(nodes, vort, px, py, far_criteria):
    """Features, labels and factors of every (target, far cell) pair, targets in order and
    each target's cells in walk order (the GPU's sample order)."""
    F, L, B = [], [], []
    for tx, ty in zip(px, py):
        for u in far_cells(nodes, tx, ty, far_criteria):
            f, lab, back = cell_sample(nodes, vort, u, tx, ty)
            F.append(f)
            L.append(lab)
            B.append(back)
    if not F:
        return np.zeros((0, NF)), np.zeros((0, 2)), np.zeros(0)
    return np.array(F), np.array(L), np.array(B)


def leaf_correction(p, norm, nodes, vort, cx, cy, far_criteria):
    """The learned correction of one leaf's constant far-field terms (the convective pass
    with the learned far field, vvflow_gb300/csrc/learned_step.cu): the network at the
    leaf's centre (cx, cy) for every far cell of the leaf, inputs standardised by norm,
    outputs scaled back to velocity and summed.  Returns (dvx, dvy, sum of |pair
    corrections|)."""
    norm = np.asarray(norm, np.float64)
    cells = far_cells(nodes, cx, cy, far_criteria)
    if not cells:
        return 0.0, 0.0, 0.0
    F, B = [], []
    for u in cells:
        f, _, back = cell_sample(nodes, vort, u, cx, cy, with_label=False)
        F.append(f)
        B.append(back)
    F = (np.array(F) - norm[:NF]) * norm[NF:2 * NF]
    Y, _ = forward(p, F, quant=True)
    C = Y * norm[2 * NF:2 * NF + 2] * np.array(B)[:, None]
    return float(C[:, 0].sum()), float(C[:, 1].sum()), float(np.abs(C).sum())
