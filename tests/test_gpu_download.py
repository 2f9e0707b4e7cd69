"""The list download that runs beside the step's later calls (vvgpu_get_vortices_async,
started after the epsilon/merge pass, waited for after the diffusive pass) returns exactly
what the synchronous vvgpu_get_vortices returns after the step: the reference's list
(Space::VortexList) after MEpsilonFast, whose positions, circulations and epsilons the
convective and diffusive passes leave as they are."""
import numpy as np
import pytest


@pytest.mark.gpu
@pytest.mark.parametrize("pinned", [True, False])
def test_gpu_async_download_matches_sync(pinned):
    import torch

    from vvflow_gb300 import build as B
    from vvflow_gb300 import workloads as W
    from vvflow_gb300.vvgpu import VVGPU_FP32, GpuSpace
    B.build()
    wl = W.cylinder_wake(60000, 400, seed=4)
    S = GpuSpace(VVGPU_FP32)
    S.load(wl)
    mn, mx = wl.node_sizes()
    n0 = S.n
    cap = n0 + 2 * wl.m  # shedding adds at most two vortices per segment

    def buf(dtype):
        t = torch.zeros(cap, dtype=dtype)
        return t.pin_memory() if pinned else t

    out = {k: buf(torch.float64) for k in ("x", "y", "g", "ie")}
    orig = buf(torch.int64)
    for step in range(2):
        S.tree_build(wl.far_criteria, mn, mx)
        S.slae()
        S.tree_destroy()
        S.vortex_shed()
        S.tree_build(wl.far_criteria, mn, mx)
        S.eps(True)
        S.get_vortices_async(out["x"].data_ptr(), out["y"].data_ptr(), out["g"].data_ptr(), out["ie"].data_ptr(),
                             orig.data_ptr())
        S.convective()
        S.diffusive()
        S.tree_destroy()
        S.wait_vortices()
        S.wait_vortices()  # no download pending: returns at once
        ref = S.vortices()
        n = S.n
        for k, rk in (("x", "x"), ("y", "y"), ("g", "g"), ("ie", "inv_eps")):
            assert np.array_equal(out[k][:n].numpy(), ref[rk]), (step, k)
        assert np.array_equal(orig[:n].numpy(), ref["orig"]), step
        S.move_and_clean(True)
    # a second download waits for the first; NULL pointers are skipped
    S.tree_build(wl.far_criteria, mn, mx)
    S.get_vortices_async(out["x"].data_ptr(), 0, 0, 0, 0)
    S.get_vortices_async(0, out["y"].data_ptr(), 0, 0, 0)
    S.wait_vortices()
    ref = S.vortices()
    assert np.array_equal(out["x"][:S.n].numpy(), ref["x"])
    assert np.array_equal(out["y"][:S.n].numpy(), ref["y"])
    S.tree_destroy()
    S.close()
