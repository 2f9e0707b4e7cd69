"""Comparison rules for one recorded step (tests/protocol.py) against a reference record.

Bit-exact (integer/index work and FP64 decisions): tree sizes, permutation, leaf geometry
and ranges, segment order, near/far lists, node centroids, merge count, post-merge
positions/circulations and epsilon.  Tolerances (stated per quantity) apply to sums
whose order differs between implementations: velocities, friction, the SLAE.
"""
from __future__ import annotations

import numpy as np

GOLDEN_EXACT_PREFIXES = ("t1_", "t2_")
EXACT_KEYS = ("merged", "n_after_shed", "eps_x", "eps_y", "eps_g", "eps_inv_eps", "eps_orig")


def golden_cases(folder, prefix=None):
    """Fixture names in ``folder``: the one-step fixtures (no prefix), or those whose name
    starts with ``prefix`` (e.g. "move_", "field_")."""
    import glob
    import os
    names = sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(folder, "*.npz")))
    if prefix is None:
        return [n for n in names if not n.startswith(("move_", "forces_", "field_", "attached_"))]
    return [n for n in names if n.startswith(prefix)]


def check_move(got: dict, d: dict, prefix: str):
    """MFlowmove::move_and_clean outputs: every array bit-exact (the FP64 bookkeeping sums
    run in the reference's order)."""
    for k, v in got.items():
        ref = d[prefix + k]
        assert np.asarray(v).shape == ref.shape, (prefix + k, np.asarray(v).shape, ref.shape)
        eq_nan = np.asarray(v).dtype.kind == "f"
        assert np.array_equal(np.asarray(v), ref, equal_nan=eq_nan), prefix + k


def load_workload(path):
    from vvflow_gb300.workloads import Workload
    d = np.load(path)
    bodies = [(d[f"in_body{i}_cx"], d[f"in_body{i}_cy"]) for i in range(int(d["in_nbodies"]))]
    inf = d["in_inf"]
    wl = Workload(str(path), bodies, d["in_x"], d["in_y"], d["in_g"], re=float(d["in_re"]),
                  dt=float(d["in_dt"]), inf_vx=float(inf[0]), inf_vy=float(inf[1]),
                  far_criteria=float(d["in_fc"]))
    return wl, d


def rel_err_vec(ax, ay, bx, by):
    """max_i |a_i - b_i| / (|b_i| + 1e-3 * rms|b|): per-vortex relative error with a floor
    that keeps near-zero velocities from dominating.  Non-finite reference values (the
    reference's own 0 * inf for coincident vortices whose epsilon is 0) must be matched
    position for position (inf is returned otherwise) and are left out of the measure."""
    if len(bx) == 0:
        return 0.0
    ax, ay, bx, by = (np.asarray(v, np.float64) for v in (ax, ay, bx, by))
    fb = np.isfinite(bx) & np.isfinite(by)
    fa = np.isfinite(ax) & np.isfinite(ay)
    if not np.array_equal(fa, fb):
        return float("inf")
    ax, ay, bx, by = ax[fb], ay[fb], bx[fb], by[fb]
    if len(bx) == 0:
        return 0.0
    mag = np.hypot(bx, by)
    floor = 1e-3 * np.sqrt(np.mean(mag * mag)) + 1e-300
    return float(np.max(np.hypot(ax - bx, ay - by) / (mag + floor)))


def rel_err(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    if a.size == 0:
        return 0.0
    scale = np.max(np.abs(b)) + 1e-300
    return float(np.max(np.abs(a - b)) / scale)


def check_exact(ref, got, keys=None, prefix=""):
    bad = []
    keys = keys if keys is not None else [k for k in ref if k.startswith(GOLDEN_EXACT_PREFIXES) or k in EXACT_KEYS]
    for k in keys:
        rk, gk = prefix + k, prefix + k
        if rk not in ref:
            continue
        if gk not in got:
            bad.append(f"{gk} missing")
            continue
        a, b = np.asarray(ref[rk]), np.asarray(got[gk])
        if a.shape != b.shape:
            bad.append(f"{gk}: shape {b.shape} != {a.shape}")
        elif not np.array_equal(a, b):
            nbad = int(np.sum(a != b)) if a.dtype.kind != "U" else 1
            d = float(np.max(np.abs(a.astype(np.float64) - b.astype(np.float64)))) if a.dtype.kind in "fiu" else -1
            bad.append(f"{gk}: {nbad}/{a.size} differ (max |d| {d:.3g})")
    return bad


def check_step(ref, got, *, vel_tol, diff_tol, fric_tol, slae_tol, slae_rhs_tol=None, slae_x_tol=None, exact=True,
               prefix=""):
    """Returns a list of failure strings (empty = pass).  The SLAE right-hand side and
    solution default to 10x and 100x the matrix tolerance."""
    slae_rhs_tol = slae_tol * 10 if slae_rhs_tol is None else slae_rhs_tol
    slae_x_tol = slae_tol * 100 if slae_x_tol is None else slae_x_tol
    bad = []
    if exact:
        keys = [k[len(prefix):] for k in ref if k.startswith(prefix)
                and (k[len(prefix):].startswith(GOLDEN_EXACT_PREFIXES) or k[len(prefix):] in EXACT_KEYS)]
        bad += check_exact(ref, got, keys, prefix)
    p = prefix
    e = rel_err_vec(got[p + "conv_vx"], got[p + "conv_vy"], ref[p + "conv_vx"], ref[p + "conv_vy"])
    if not e <= vel_tol:
        bad.append(f"{p}convective rel err {e:.3e} > {vel_tol:.1e}")
    e = rel_err_vec(got[p + "diff_vx"], got[p + "diff_vy"], ref[p + "diff_vx"], ref[p + "diff_vy"])
    if not e <= diff_tol:
        bad.append(f"{p}diffusive rel err {e:.3e} > {diff_tol:.1e}")
    e = rel_err(got[p + "fric"], ref[p + "fric"])
    if not e <= fric_tol:
        bad.append(f"{p}fric rel err {e:.3e} > {fric_tol:.1e}")
    e = rel_err_vec(got[p + "probe_vx"], got[p + "probe_vy"], ref[p + "probe_vx"], ref[p + "probe_vy"])
    if not e <= vel_tol:
        bad.append(f"{p}probe velocity rel err {e:.3e} > {vel_tol:.1e}")
    if p + "slae_A" in ref:
        e = rel_err(got[p + "slae_A"], ref[p + "slae_A"])
        if not e <= slae_tol:
            bad.append(f"{p}slae matrix rel err {e:.3e}")
        e = rel_err(got[p + "slae_b"], ref[p + "slae_b"])
        if not e <= slae_rhs_tol:
            bad.append(f"{p}slae rhs rel err {e:.3e} > {slae_rhs_tol:.1e}")
        e = rel_err(got[p + "slae_x"], ref[p + "slae_x"])
        if not e <= slae_x_tol:
            bad.append(f"{p}slae solution rel err {e:.3e} > {slae_x_tol:.1e}")
    return bad


def check_fields(got: dict, ref: dict, rel_tol: float):
    """Grid fields (XField::map, float32).  Exact: the stream function's gap lists.  Within
    ``rel_tol`` of the field's largest magnitude: every map value (the FP64 sums run in a
    different order and CUDA's log/exp/erf/atan2 differ from the C library's in the last
    bits before the rounding to float).  Returns failure strings."""
    bad = []
    for k, b in ref.items():
        if k.startswith("in_"):
            continue
        a = np.asarray(got[k])
        b = np.asarray(b)
        if a.shape != b.shape:
            bad.append(f"{k}: shape {a.shape} != {b.shape}")
            continue
        if "_gap" in k:
            if not np.array_equal(a, b):
                bad.append(f"{k}: gap lists differ")
            continue
        d = np.abs(a.astype(np.float64) - b.astype(np.float64))
        scale = float(np.max(np.abs(b))) if b.size else 0.0
        if not np.all(np.isfinite(a)) or (b.size and d.max() > rel_tol * scale):
            bad.append(f"{k}: max |d| {d.max():.3g} > {rel_tol:.0e} x {scale:.3g}")
    return bad
