"""Moving bodies on the GPU: the attached vortex and source sheets of body_list_influence
(libvvhd/src/MConvectiveFast.cpp:172-215, 440-457) in the convective pass, velocity(p) and
the direct sum, against the reference's own outputs (tests/golden/attached_bodies.npz, made
by tests/golden/make_golden_attached.py; the C restatement matches them bit for bit,
tests/test_oracle_pin.py).  A cylinder translating and rotating about an off-centre axis,
with probes inside one segment length of its segments (linear sheets) and beyond (point
singularities).  Tolerances: FP64 1e-12, FP32 convective 1e-5 (per-vortex relative error
with a 1e-3 rms floor, parity.rel_err_vec)."""
import os

import numpy as np
import pytest

import attached_cases as AC
from parity import rel_err_vec

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
def test_gpu_attached_sheets_match_reference(precision):
    from vvflow_gb300 import build as B
    from vvflow_gb300.vvgpu import GpuSpace, default_body_params
    B.build()
    d = np.load(os.path.join(GOLDEN, "attached_bodies.npz"))
    S = GpuSpace(precision)
    got = AC.run(S, AC.case(), default_body_params)
    S.close()
    assert np.array_equal(got["orig"], d["orig"])
    conv_tol = 1e-12 if precision == 0 else 1e-5
    assert rel_err_vec(got["conv_vx"], got["conv_vy"], d["conv_vx"], d["conv_vy"]) <= conv_tol
    assert rel_err_vec(got["probe_vx"], got["probe_vy"], d["probe_vx"], d["probe_vy"]) <= 1e-12
    assert rel_err_vec(got["direct_vx"], got["direct_vy"], d["direct_vx"], d["direct_vy"]) <= 1e-12
