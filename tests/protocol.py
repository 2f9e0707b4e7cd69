"""One simulate() iteration of the hot path, driven through any backend with the
oracle's call surface (the C restatement, the compiled reference, or the CUDA library).

The order is the reference driver's (utils/vvflow/vvflow.cpp:214-255):
tree.build -> calc_circulation -> tree.destroy -> vortex_shed -> tree.build ->
CalcEpsilonFast(merge) -> process_all_lists -> process_vort_list -> tree.destroy.
Every intermediate result the parity tests compare is recorded.
"""
from __future__ import annotations

import hashlib

import numpy as np

PROBES_X = np.array([-2.0, -1.1, -0.6, 0.0, 0.55, 0.9, 1.7, 2.5, 3.3, 6.0])
PROBES_Y = np.array([0.1, -0.7, 0.62, 0.8, -0.3, 1.2, -1.9, 0.4, 0.0, 0.25])


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        a = np.ascontiguousarray(a)
        h.update(str(a.dtype).encode())
        h.update(a.tobytes())
    return h.hexdigest()


def tree_record(S, prefix: str, out: dict, full_lists: bool, far_lists: bool = True):
    """far_lists=False: the digest covers the near lists and the far-list offsets only (the
    far nodes of every leaf at 4M vortices are ~7e8 entries)."""
    nn, nl, nnear, nfar = S.tree_sizes()
    out[prefix + "sizes"] = np.array([nn, nl, nnear, nfar], np.int64)
    v = S.vortices()
    out[prefix + "perm"] = v["orig"]
    lv = S.tree_leaves()
    for k in ("x", "y", "h", "w", "vfirst", "vlast", "depth", "path", "sfirst", "slast"):
        out[prefix + "leaf_" + k] = lv[k]
    out[prefix + "seg_order"] = S.tree_seg_order()
    li = S.tree_lists(far=far_lists or full_lists)
    out[prefix + "near_off"] = li["near_off"]
    out[prefix + "far_off"] = li["far_off"]
    if full_lists:
        for k in ("near_depth", "near_path", "far_depth", "far_path"):
            out[prefix + k] = li[k]
    if far_lists or full_lists:
        out[prefix + "lists_sha"] = np.array(digest(li["near_depth"], li["near_path"],
                                                    li["far_depth"], li["far_path"]))
    else:
        out[prefix + "near_sha"] = np.array(digest(li["near_depth"], li["near_path"]))
    del li
    nd = S.tree_nodes()
    order = np.lexsort((nd["path"], nd["depth"]))
    for k in nd:
        out[prefix + "node_" + k] = nd[k][order]


def run_step(S, wl, *, merge=None, full_lists=True, far_criteria=None, record_tree=True, seg_g=None):
    """Runs one step on backend ``S`` (already loaded with ``wl``); returns a dict.

    ``seg_g``: segment circulations to shed instead of this backend's own SLAE solution.
    Parity runs pass the reference's solution so that every call after the SLAE sees
    identical inputs (the solve itself is compared with a tolerance)."""
    out = {}
    mn, mx = wl.node_sizes()
    fc = wl.far_criteria if far_criteria is None else far_criteria
    merge = wl.merge if merge is None else merge
    if wl.bodies:
        S.tree_build(fc, mn, mx)
        if record_tree:
            tree_record(S, "t1_", out, full_lists)
        bo = S.slae()
        A, b, x = S.slae_export()
        out["slae_A"], out["slae_b"], out["slae_x"] = A, b, x
        out["slae_body"] = np.array([[d[k] for k in sorted(d)] for d in bo])
        S.tree_destroy()
        if seg_g is not None:
            S.set_segment_g(seg_g)
    S.vortex_shed()
    seg = S.segments()
    out["seg_g"] = seg["g"]
    out["seg_gsum"] = seg["gsum"]
    out["n_after_shed"] = np.array(S.n)
    S.tree_build(fc, mn, mx)
    if record_tree:
        tree_record(S, "t2_", out, full_lists)
    out["merged"] = np.array(S.eps(merge))
    v = S.vortices()
    for k in ("x", "y", "g", "inv_eps", "orig"):
        out["eps_" + k] = v[k]
    S.convective()
    v = S.vortices()
    out["conv_vx"], out["conv_vy"] = v["vx"], v["vy"]
    S.diffusive()
    v = S.vortices()
    out["diff_vx"], out["diff_vy"] = v["vx"], v["vy"]
    out["fric"] = S.segments()["fric"]
    out["probe_vx"], out["probe_vy"] = S.velocity_points(PROBES_X, PROBES_Y)
    S.tree_destroy()
    return out


def advance(S, wl, out):
    """Host-side stand-in for move_and_clean between two parity steps:
    r += v dt, drop |g| < 1e-10, keep the new epsilon (MFlowmove.cpp:107-117)."""
    v = S.vortices()
    x = v["x"] + v["vx"] * wl.dt
    y = v["y"] + v["vy"] * wl.dt
    keep = np.abs(v["g"]) >= 1e-10
    return x[keep], y[keep], v["g"][keep], v["inv_eps"][keep]
