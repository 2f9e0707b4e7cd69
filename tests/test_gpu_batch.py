"""Batched sweep (vvgpu_batch_step): several independent simulations advanced by one call
from a pool of host threads compute exactly what each computes alone through the same
calls (simulate()'s step, utils/vvflow/vvflow.cpp:214-255, then
MFlowmove::move_and_clean): the vortex lists after two steps are bit-identical."""
import numpy as np
import pytest


def _load(wl, precision):
    from vvflow_gb300.vvgpu import GpuSpace
    S = GpuSpace(precision)
    S.set_params(wl.re, wl.dt, wl.inf_vx, wl.inf_vy, 0.0, 0.0)
    for cx, cy in wl.bodies:
        S.add_body(cx, cy)
    S.set_vortices(wl.x, wl.y, wl.g)
    return S


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_gpu_batch_matches_single_instances(precision):
    from vvflow_gb300 import build as B
    from vvflow_gb300 import workloads as W
    from vvflow_gb300.vvgpu import VVGPU_FP32, VVGPU_FP64, Batch
    B.build()
    prec = VVGPU_FP32 if precision == "fp32" else VVGPU_FP64
    wls = W.batched_cylinders(5, n_lo=2000, n_hi=12000, m_lo=60, m_hi=150, seed=9)
    batch_spaces = [_load(wl, prec) for wl in wls]
    batch = Batch(batch_spaces, 8.0, [wl.node_sizes() for wl in wls], merge=True, move=True)
    for _ in range(2):
        ms = batch.step(nthreads=3)
        assert ms.shape == (5,) and np.all(ms > 0)
    for wl, S in zip(wls, batch_spaces):
        R = _load(wl, prec)
        mn, mx = wl.node_sizes()
        for _ in range(2):
            R.tree_build(8.0, mn, mx)
            R.slae()
            R.tree_destroy()
            R.vortex_shed()
            R.tree_build(8.0, mn, mx)
            R.eps(True)
            R.convective()
            R.diffusive()
            R.tree_destroy()
            R.move_and_clean(True)
        a, b = S.vortices(), R.vortices()
        R.close()
        for k in a:
            assert np.array_equal(a[k], b[k]), (wl.name, k)
    for S in batch_spaces:
        S.close()


@pytest.mark.gpu
def test_gpu_batch_autotune_and_errors():
    from vvflow_gb300 import build as B
    from vvflow_gb300 import workloads as W
    from vvflow_gb300.vvgpu import VVGPU_FP32, Batch, VVGpuError
    B.build()
    wls = W.batched_cylinders(3, n_lo=1000, n_hi=3000, m_lo=40, m_hi=80, seed=11)
    spaces = [_load(wl, VVGPU_FP32) for wl in wls]
    batch = Batch(spaces, 8.0, [wl.node_sizes() for wl in wls])
    nt, ms = batch.autotune((1, 2, 3))
    assert nt in (1, 2, 3) and ms > 0
    for S in spaces:  # every instance timed its own kernel shapes in the first step
        t, d = S.tiles()
        assert t in (128, 192, 256) and d in (1, 2)
    # a context with a tree left built fails its own step; the others still advance
    mn, mx = wls[1].node_sizes()
    spaces[1].tree_build(8.0, mn, mx)
    n0 = spaces[0].n
    with pytest.raises(VVGpuError):
        batch.step()
    spaces[1].tree_destroy()
    assert spaces[0].n != n0 or spaces[0].n > 0
    for S in spaces:
        S.close()
