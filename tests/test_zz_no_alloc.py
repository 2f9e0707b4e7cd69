"""vvgpu_velocity_points_noalloc: point velocities for callers that cannot allocate device
memory.

Such a caller might be a host program that grants the solver a fixed device-memory budget,
or a probe loop running next to the solver each step that must not stall other streams
with the device-wide synchronisation that cudaMalloc/cudaFree imply.  The entry point stages
its points and results in one fixed device array instead (VVGPU_NOALLOC_MAX_POINTS points),
so its results must equal those of vvgpu_velocity_points, which allocates a staging buffer
per call.  Checked here through the C ABI on two calls in a row (different point sets, so a
stale result from the first call would show), plus the size limit.

This file is named to be collected last; it runs alone or after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from vvflow_gb300 import workloads as W

MAX_POINTS = 16384  # VVGPU_NOALLOC_MAX_POINTS in include/vvgpu.h
TOL = 1e-12         # FP64 velocity tolerance of the parity tests


def _ptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


@pytest.mark.gpu
def test_noalloc_points_match_allocating_entry_point():
    from vvflow_gb300 import build as B
    from vvflow_gb300.vvgpu import VVGPU_FP64, GpuSpace

    B.build()
    wl = W.cylinder_annulus(3000, 120, seed=31)
    S = GpuSpace(VVGPU_FP64)
    S.load(wl)
    mn, mx = wl.node_sizes()
    S.tree_build(wl.far_criteria, mn, mx)
    S.eps(True)
    lib = S.lib
    rng = np.random.default_rng(5)
    for n in (1000, 257):  # two calls in a row, different sizes and points
        r = np.sqrt(rng.uniform(0.6 ** 2, 3.0 ** 2, n))
        a = rng.uniform(0, 2 * np.pi, n)
        px = np.ascontiguousarray(r * np.cos(a))
        py = np.ascontiguousarray(r * np.sin(a))
        ref_x, ref_y = S.velocity_points(px, py)
        vx = np.full(n, np.nan)
        vy = np.full(n, np.nan)
        rc = lib.vvgpu_velocity_points_noalloc(S.h, n, _ptr(px), _ptr(py), _ptr(vx), _ptr(vy))
        assert rc == 0, lib.vvgpu_last_error(S.h)
        scale = np.max(np.hypot(ref_x, ref_y))
        err = np.max(np.hypot(vx - ref_x, vy - ref_y)) / scale
        assert err <= TOL, err
    # beyond the maximum: a clear error, nothing written
    n = MAX_POINTS + 1
    px = np.zeros(n)
    vx = np.full(n, 7.0)
    rc = lib.vvgpu_velocity_points_noalloc(S.h, n, _ptr(px), _ptr(px), _ptr(vx), _ptr(vx))
    assert rc == -9  # VVGPU_ERR_LIMIT
    assert b"at most" in lib.vvgpu_last_error(S.h)
    assert np.all(vx == 7.0)
    S.tree_destroy()
    S.close()
