"""Parity of the caller-side steps with the reference's own outputs:
* vvgpu_move_and_clean (MFlowmove::move_and_clean, libvvhd/src/MFlowmove.cpp:11-215) against
  tests/golden/move_*.npz: positions, the kept list and its order, circulations, velocities
  reset, segment gsum and the bodies' dead-vortex sums, with and without removal inside
  bodies;
* vvgpu_calc_forces / vvgpu_zero_forces (Space::calc_forces, zero_forces,
  libvvhd/src/TSpace.cpp:94-142) against tests/golden/forces_*.npz.
All bit-exact."""
import os

import numpy as np
import pytest

from move_cases import cases as move_cases, run_move
from parity import check_move, golden_cases

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.gpu
@pytest.mark.parametrize("case", golden_cases(GOLDEN, prefix="move_"))
def test_gpu_move_matches_golden(case):
    from vvflow_gb300 import build as B
    from vvflow_gb300.vvgpu import VVGPU_FP64, GpuSpace, default_body_params
    B.build()
    d = dict(np.load(os.path.join(GOLDEN, case + ".npz")))
    c = move_cases()[case[len("move_"):]]
    for remove in (True, False):
        S = GpuSpace(VVGPU_FP64)
        got = run_move(S, c, remove, default_body_params)
        S.close()
        check_move(got, d, "rm_" if remove else "keep_")


@pytest.mark.gpu
def test_gpu_move_rejects_built_tree():
    from vvflow_gb300 import build as B
    from vvflow_gb300 import workloads as W
    from vvflow_gb300.vvgpu import VVGPU_FP64, GpuSpace, VVGpuError
    B.build()
    wl = W.cylinder_annulus(500, 40, seed=3)
    S = GpuSpace(VVGPU_FP64)
    S.load(wl)
    mn, mx = wl.node_sizes()
    S.tree_build(wl.far_criteria, mn, mx)
    with pytest.raises(VVGpuError):
        S.move_and_clean(True)
    S.tree_destroy()
    S.close()


@pytest.mark.gpu
@pytest.mark.parametrize("case", golden_cases(GOLDEN, prefix="forces_"))
def test_gpu_forces_match_golden(case):
    """Space::calc_forces / zero_forces (libvvhd/src/TSpace.cpp:94-142): friction, nusselt,
    the per-segment Cp/Fr/Nu accumulators and the zeroed state, bit-exact (NaN where the
    reference gives NaN: Nu for an inviscid run)."""
    from move_cases import forces_cases, run_forces
    from vvflow_gb300 import build as B
    from vvflow_gb300.vvgpu import VVGPU_FP64, GpuSpace, default_body_params
    B.build()
    d = dict(np.load(os.path.join(GOLDEN, case + ".npz")))
    S = GpuSpace(VVGPU_FP64)
    got = run_forces(S, forces_cases()[case[len("forces_"):]], default_body_params)
    S.close()
    check_move(got, d, "")
