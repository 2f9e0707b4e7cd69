"""Kernel shapes of the FP32 pair passes (vvgpu_autotune_tiles, vvflow_gb300/csrc/autotune.cu):
sources per shared-memory tile of the convective near field (128, 192, 256) and targets
per lane of the diffusive pass (1, 2).

* The tuner times every shape on the context's tree, keeps one of them, and leaves the
  velocities and the wall friction as they were, bit for bit.
* Every shape gives the same velocities as the default one within 2e-6 of the largest
  velocity (only the grouping of the FP32 partial sums differs), in both passes.
* An FP64 context has one shape: the tuner reports -1 times and keeps the defaults.
* Other shapes are rejected with VVGPU_ERR_ARG.
"""
import numpy as np
import pytest

from vvflow_gb300 import workloads as W

ERR_ARG = -1


def _space(precision):
    from vvflow_gb300 import build as B
    from vvflow_gb300.vvgpu import GpuSpace
    B.build()
    return GpuSpace(precision)


def _prepared(precision):
    wl = W.cylinder_annulus(20000, 500, seed=5)
    mn, mx = wl.node_sizes()
    S = _space(precision)
    S.load(wl)
    S.tree_build(wl.far_criteria, mn, mx)
    S.eps(True)
    return S


@pytest.mark.gpu
def test_autotune_keeps_the_state_and_every_shape_agrees():
    S = _prepared(1)
    zero = np.zeros(S.n)
    S.set_velocities(zero, zero)
    S.diffusive()  # some friction to keep
    before, fric0 = S.vortices(), S.segments()["fric"]
    tile, dt, ms = S.autotune_tiles()
    after, fric1 = S.vortices(), S.segments()["fric"]
    assert tile in (128, 192, 256) and dt in (1, 2) and np.all(ms > 0), (tile, dt, ms)
    assert S.tiles() == (tile, dt)
    for k in ("vx", "vy", "orig"):
        assert np.array_equal(before[k], after[k]), k
    assert np.array_equal(fric0, fric1)
    got = {}
    for shape in ((192, 1), (128, 1), (256, 1), (192, 2)):
        S.set_tiles(*shape)
        S.set_velocities(zero, zero)
        S.convective()
        c = S.vortices()
        S.set_velocities(zero, zero)
        S.diffusive()
        d = S.vortices()
        got[shape] = (c["vx"], c["vy"], d["vx"], d["vy"])
    S.tree_destroy()
    S.close()
    ref = got[(192, 1)]
    for shape, v in got.items():
        for a, b in zip(v, ref):
            scale = np.abs(b).max()
            assert scale > 0
            assert np.abs(a - b).max() <= 2e-6 * scale, (shape, np.abs(a - b).max() / scale)


@pytest.mark.gpu
def test_autotune_fp64_has_one_shape_and_bad_shapes_are_rejected():
    from vvflow_gb300.vvgpu import VVGpuError
    S = _prepared(0)
    tile, dt, ms = S.autotune_tiles()
    assert (tile, dt) == (256, 1) and np.all(ms == -1)
    for shape in ((64, 1), (192, 3), (100, 2)):
        with pytest.raises(VVGpuError) as ei:
            S.set_tiles(*shape)
        assert ei.value.code == ERR_ARG
    S.tree_destroy()
    S.close()
