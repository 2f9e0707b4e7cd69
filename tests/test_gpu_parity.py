"""Parity of the CUDA path (through the C ABI) with the reference.

* Golden fixtures (outputs of the reference's own compiled sources): tree geometry,
  permutation, near/far lists, centroids, merges, positions and epsilon bit-exact in both
  precisions; sums within the tolerances below.
* Larger seeded workloads against the C restatement of the reference (bit-exact with the
  reference, see test_oracle_pin.py).

Tolerances (per-vortex relative error with a floor of 1e-3 rms, parity.rel_err_vec):
  FP64 path: convective 1e-12, diffusive 1e-11, friction 1e-10, SLAE cells 1e-12, right-hand
  side 1e-11 (a sum of ~1e3 logarithms in a different order), solution 1e-10.
  FP32 path: convective 1e-5, diffusive 1e-5, friction 1e-5 (wall terms are FP64).
"""
import os

import numpy as np
import pytest

import oracle
from parity import check_step, golden_cases, load_workload
from protocol import advance, run_step
from vvflow_gb300 import workloads as W

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

TOL64 = dict(vel_tol=1e-12, diff_tol=1e-11, fric_tol=1e-10, slae_tol=1e-12)
# FP32 path: the matrix cells stay FP64; the right-hand side's tree sums run in FP32 with
# compensated accumulation (relative error ~1e-7 of the largest entry), and the solution
# carries that error times the system's conditioning.
TOL32 = dict(vel_tol=1e-5, diff_tol=1e-5, fric_tol=1e-5, slae_tol=1e-12, slae_rhs_tol=2e-6, slae_x_tol=2e-5)


def gpu_space(precision):
    from vvflow_gb300 import build as B
    from vvflow_gb300.vvgpu import GpuSpace
    B.build()
    return GpuSpace(precision)


def run_gpu(wl, precision, d=None, full_lists=True):
    """One step (two for fixtures that hold a second step).  Inputs of every call equal the
    reference's: the shed uses the reference's SLAE solution, and the second step starts
    from the reference's moved state."""
    S = gpu_space(precision)
    S.load(wl)
    out = run_step(S, wl, full_lists=full_lists, seg_g=None if d is None else d["seg_g"])
    if d is not None and "s2_in_x" in d:
        S.set_params(wl.re, wl.dt, wl.inf_vx, wl.inf_vy, 0.0, wl.dt)
        S.set_vortices(d["s2_in_x"], d["s2_in_y"], d["s2_in_g"], d["s2_in_inv_eps"])
        out2 = run_step(S, wl, full_lists=full_lists, seg_g=d["s2_seg_g"])
        out.update({"s2_" + k: v for k, v in out2.items()})
    st = S.stats()
    S.close()
    return out, st


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
@pytest.mark.parametrize("case", golden_cases(GOLDEN))
def test_gpu_matches_golden(case, precision):
    wl, d = load_workload(os.path.join(GOLDEN, case + ".npz"))
    got, _ = run_gpu(wl, precision, d, full_lists="t1_near_path" in d or "t2_near_path" in d)
    tol = TOL64 if precision == 0 else TOL32
    bad = check_step(d, got, **tol)
    if "s2_in_x" in d:
        bad += check_step(d, got, prefix="s2_", **tol)
    assert not bad, bad


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
def test_gpu_matches_oracle_wake_200k(precision):
    wl = W.cylinder_wake(200_000, 2000, seed=4)
    S = oracle.OracleSpace("port")
    S.load(wl)
    ref = run_step(S, wl, full_lists=False)
    S.close()
    got, st = run_gpu(wl, precision, d={"seg_g": ref["seg_g"]}, full_lists=False)
    tol = TOL64 if precision == 0 else TOL32
    bad = check_step(ref, got, **tol)
    assert not bad, bad
    assert st["merge_rounds"] >= 1


@pytest.fixture(scope="module")
def wake_1m_oracle():
    """One full, unsampled step of the oracle on the 1M-vortex cylinder wake (2000
    segments, farCriteria 8): about a minute on the host cores."""
    wl = W.cylinder_wake(1_000_000, 2000, seed=2)
    S = oracle.OracleSpace("port")
    S.load(wl)
    ref = run_step(S, wl, full_lists=False)
    S.close()
    return wl, ref


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
def test_gpu_matches_oracle_wake_1m(wake_1m_oracle, precision):
    """The plain method at scale: 1M vortices, a 2000-segment cylinder.  Bit-exact: both
    trees (permutation, leaf boxes and ranges, node centroids), the digests of every leaf's
    near and far lists, the merge count, the merged positions and circulations and epsilon;
    velocities, friction and the SLAE within the tolerances above."""
    wl, ref = wake_1m_oracle
    got, st = run_gpu(wl, precision, d={"seg_g": ref["seg_g"]}, full_lists=False)
    tol = TOL64 if precision == 0 else TOL32
    bad = check_step(ref, got, **tol)
    assert not bad, bad
    assert int(ref["merged"]) > 1000 and st["merge_rounds"] >= 2
    assert int(ref["t2_sizes"][1]) > 50_000  # leaves


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
def test_slae_matrix_reused_until_its_inputs_change(precision):
    """Once the matrix is filled and inverted, later solves with the same bodies and dt
    fill only the right-hand side; a change of a body parameter that enters the matrix
    refills it.  Both give the bits of a fresh context with the same state."""
    wl = W.cylinder_annulus(20000, 500, seed=3)
    mn, mx = wl.node_sizes()

    def solve(S):
        S.tree_build(wl.far_criteria, mn, mx)
        S.slae()
        A, b, x = S.slae_export()
        S.tree_destroy()
        return A, b, x

    S = gpu_space(precision)
    S.load(wl)
    A1, b1, x1 = solve(S)
    A2, b2, x2 = solve(S)
    assert np.array_equal(A1, A2) and np.array_equal(b1, b2) and np.array_equal(x1, x2)
    S.set_body_params(0, density=2.0)
    A3, b3, x3 = solve(S)
    assert not np.array_equal(A1, A3)
    F = gpu_space(precision)
    F.load(wl)
    F.set_body_params(0, density=2.0)
    A4, b4, x4 = solve(F)
    assert np.array_equal(A3, A4) and np.array_equal(b3, b4) and np.array_equal(x3, x4)
    S.close()
    F.close()


@pytest.mark.gpu
@pytest.mark.parametrize("n", [700, 1024, 1025, 5000])
def test_gpu_matches_oracle_subtree_sizes(n):
    """Body-free clouds around the size limit of the one-block subtree build (1024
    vortices): at 700 and 1024 the root's whole tree is built by one block, at 1025 and
    5000 the level loop hands its children over.  Exact duplicates and a tight cluster
    exercise empty and degenerate boxes."""
    x, y, g = W.annulus_cloud(n, 0.1, 2.0, seed=20 + n)
    x[n // 3: n // 3 + 5] = x[n // 3]
    y[n // 3: n // 3 + 5] = y[n // 3]
    x[-40:] = 1.5 + 1e-9 * np.arange(40)
    y[-40:] = -0.25
    wl = W.Workload("subtree", [], x, y, g, re=600.0, dt=0.005)
    S = oracle.OracleSpace("port")
    S.load(wl)
    ref = run_step(S, wl, full_lists=True)
    S.close()
    # FP32: inside the 1e-9 cluster single pair terms are ~1e4 times the velocities they
    # sum to (alternating signs cancel), so the FP32 rounding of each pair reaches ~1e-5 of
    # the result there; the decisions (tree, epsilon, merges) stay exact.
    tol32 = dict(TOL32, vel_tol=5e-5, diff_tol=5e-5)
    for precision in (0, 1):
        got, _ = run_gpu(wl, precision, full_lists=True)
        tol = TOL64 if precision == 0 else tol32
        bad = check_step(ref, got, **tol)
        assert not bad, (precision, bad)
