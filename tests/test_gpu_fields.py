"""Grid fields on the GPU (vvgpu_field_velocity / _streamfunction / _vorticity) against the
reference's own XVelocity, XStreamfunction and XVorticity (libvvhd/src/X*.cpp):
* tests/golden/field_*.npz, written by the reference;
* the C restatement (bit-identical to the reference, pinned in test_oracle_pin.py) on a
  larger wake than the fixtures hold.
Tolerance: every float map value within 1e-6 of the field's largest magnitude (the FP64 sums
run in another order, and CUDA's log/exp/erf/atan2 differ from the C library's in the last
bits, before the rounding to float); the stream function's gap lists exactly.  The context
is left as it was (the reference evaluates on a private copy of Space)."""
import os

import numpy as np
import pytest

import field_cases as FC
from parity import check_fields, golden_cases

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
REL_TOL = 1e-6


def _gpu():
    from vvflow_gb300 import build as B
    from vvflow_gb300.vvgpu import VVGPU_FP64, GpuSpace
    B.build()
    return GpuSpace(VVGPU_FP64)


@pytest.mark.gpu
@pytest.mark.parametrize("case", golden_cases(GOLDEN, prefix="field_"))
def test_gpu_fields_match_golden(case):
    d = dict(np.load(os.path.join(GOLDEN, case + ".npz")))
    c = FC.case_from_fixture(d)
    S = _gpu()
    FC.load(S, c)
    before = S.vortices()
    got = FC.run_fields(S, c)
    after = S.vortices()
    S.close()
    bad = check_fields(got, d, REL_TOL)
    assert not bad, bad
    for k in before:
        assert np.array_equal(before[k], after[k]), k


@pytest.mark.gpu
def test_gpu_fields_match_port_wake():
    import oracle
    from vvflow_gb300 import workloads as W
    rng = np.random.default_rng(41)
    ex, ey = W.ellipse_corners(0.5, 0.25, 400, 10.0)
    n = 40000
    x = rng.uniform(0.3, 8.0, n)
    y = rng.normal(0, 0.2 + 0.05 * x)
    keep = ~W.point_in_polygon(x, y, ex, ey)
    x, y = x[keep], y[keep]
    g = np.sign(np.sin(2 * np.pi * x / 2.4) * y) * rng.lognormal(np.log(1e-4), 0.5, len(x))
    c = dict(bodies=[ex, ey], x=x, y=y, g=g, sg=rng.normal(0, 1e-3, len(ex)),
             sinks=(np.array([2.0]), np.array([0.31]), np.array([0.004])), inf=(1.0, 0.0),
             grid=(-0.6, -1.2, 0.05, 128, 48))
    ref = {}
    S = oracle.OracleSpace("port")
    FC.load(S, c)
    ref = FC.run_fields(S, c)
    S.close()
    S = _gpu()
    FC.load(S, c)
    got = FC.run_fields(S, c)
    S.close()
    bad = check_fields(got, ref, REL_TOL)
    assert not bad, bad


@pytest.mark.gpu
def test_gpu_fields_reject_bad_arguments():
    from vvflow_gb300.vvgpu import VVGpuError
    c = FC.cases()["no_vortices"]
    S = _gpu()
    FC.load(S, c)
    for a in ((-1.0, -1.0, 0.1, 1, 8), (-1.0, -1.0, 0.1, 8, 0), (-1.0, -1.0, 0.0, 8, 8),
              (-1.0, -1.0, float("inf"), 8, 8)):
        with pytest.raises(VVGpuError):
            S.field_vorticity(*a)
    with pytest.raises(VVGpuError):
        S.field_velocity(-1.0, -1.0, 0.1, 8, 8, mode="z")
    with pytest.raises(VVGpuError):
        S.field_velocity(-1.0, -1.0, 0.1, 8, 8, ref_frame="q")
    with pytest.raises(VVGpuError):
        S.field_streamfunction(-1.0, -1.0, 0.1, 8, 8, eps_mult=0.0)
    S.tree_build(8, 0.1, 1.0)
    with pytest.raises(VVGpuError):
        S.field_vorticity(-1.0, -1.0, 0.1, 8, 8)
    S.tree_destroy()
    # usable afterwards
    assert S.field_vorticity(-1.0, -1.0, 0.125, 17, 17).shape == (17, 17)
    S.close()
