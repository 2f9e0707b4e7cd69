"""ctypes binding of libvvgpu.so (include/vvgpu.h).

``GpuSpace`` mirrors the reference's hot-path call surface (stree::build/destroy,
MEpsilonFast::CalcEpsilonFast, MConvectiveFast::process_all_lists / velocity /
calc_circulation, MDiffusiveFast::process_vort_list, MFlowmove::vortex_shed) on one
Space held in GPU memory.  There is no CPU fallback: constructing a GpuSpace without the
compiled library or without a CUDA device raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libvvgpu.so")

VVGPU_FP64 = 0
VVGPU_FP32 = 1

ERRORS = {
    -1: "VVGPU_ERR_ARG", -2: "VVGPU_ERR_STATE", -3: "VVGPU_ERR_NOT_BUILT", -4: "VVGPU_ERR_UNSUPPORTED",
    -5: "VVGPU_ERR_SINGULAR", -6: "VVGPU_ERR_CUDA", -7: "VVGPU_ERR_NOMEM", -8: "VVGPU_ERR_TIMEOUT",
    -9: "VVGPU_ERR_LIMIT",
}


class Cfg(C.Structure):
    _fields_ = [("device", C.c_int), ("precision", C.c_int), ("reserve_vortices", C.c_int64),
                ("reserve_segments", C.c_int64)]


class BodyParams(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "holder_x", "holder_y", "holder_o", "dpos_x", "dpos_y", "dpos_o",
        "speed_x", "speed_y", "speed_o",
        "speed_slae_x", "speed_slae_y", "speed_slae_o",
        "speed_slae_prev_x", "speed_slae_prev_y", "speed_slae_prev_o",
        "friction_prev_x", "friction_prev_y", "friction_prev_o",
        "fdt_dead_x", "fdt_dead_y", "fdt_dead_o", "g_dead", "density",
        "kspring_x", "kspring_y", "kspring_o")] + [
        ("special_segment_no", C.c_int32), ("bc_kutta", C.c_int32)]


class BodyOut(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "speed_slae_x", "speed_slae_y", "speed_slae_o",
        "force_hydro_x", "force_hydro_y", "force_hydro_o",
        "force_holder_x", "force_holder_y", "force_holder_o")]


class StepCfg(C.Structure):
    _fields_ = [("far_criteria", C.c_double), ("min_node", C.c_double), ("max_node", C.c_double),
                ("merge", C.c_int32), ("move", C.c_int32)]


class JudgeCfg(C.Structure):
    _fields_ = [("targets", C.c_int64), ("far_criteria", C.c_double), ("bound", C.c_double), ("seed", C.c_uint64)]


class JudgeOut(C.Structure):
    _fields_ = [("gap_rms", C.c_double), ("gap_max", C.c_double), ("pairs", C.c_int64), ("judged", C.c_int64),
                ("reverted", C.c_int32), ("reserved", C.c_int32)]


class Stats(C.Structure):
    _fields_ = [(n, C.c_int64) for n in (
        "n_vortices", "n_segments", "n_nodes", "n_leaves", "tree_depth", "near_pairs", "far_pairs",
        "near_runs", "merge_rounds", "merged", "diff_candidates")] + [("reserved", C.c_int64 * 8)]


class VVGpuError(RuntimeError):
    def __init__(self, code, where, msg=""):
        super().__init__(f"{where}: {ERRORS.get(code, code)} {msg}".strip())
        self.code = code


_D = C.POINTER(C.c_double)
_I64 = C.POINTER(C.c_int64)
_I32 = C.POINTER(C.c_int32)
_U32 = C.POINTER(C.c_uint32)
_U16 = C.POINTER(C.c_uint16)
_F = C.POINTER(C.c_float)
_H = C.c_void_p

# name -> (restype, argtypes); the same list is the ABI surface checked by the tests
SIGNATURES = {
    "vvgpu_ctx_create": (C.c_int, [C.POINTER(Cfg), C.POINTER(_H)]),
    "vvgpu_ctx_destroy": (C.c_int, [_H]),
    "vvgpu_last_error": (C.c_char_p, [_H]),
    "vvgpu_set_precision": (C.c_int, [_H, C.c_int]),
    "vvgpu_set_stream": (C.c_int, [_H, C.c_void_p]),
    "vvgpu_synchronize": (C.c_int, [_H]),
    "vvgpu_get_stats": (C.c_int, [_H, C.POINTER(Stats)]),
    "vvgpu_set_eps_round_limit": (C.c_int, [_H, C.c_int64]),
    "vvgpu_set_wait_limit": (C.c_int, [_H, C.c_uint32]),
    "vvgpu_autotune_tiles": (C.c_int, [_H, _I32, _I32, _D]),
    "vvgpu_set_tiles": (C.c_int, [_H, C.c_int32, C.c_int32]),
    "vvgpu_get_tiles": (C.c_int, [_H, _I32, _I32]),
    "vvgpu_set_autotune": (C.c_int, [_H, C.c_int]),
    "vvgpu_set_kernel_timing": (C.c_int, [_H, C.c_int]),
    "vvgpu_get_kernel_timing": (C.c_int, [_H, _D, _I64]),
    "vvgpu_set_params": (C.c_int, [_H] + [C.c_double] * 8),
    "vvgpu_add_body": (C.c_int, [_H, C.c_int64, _D, _D, _U32, C.POINTER(BodyParams)]),
    "vvgpu_set_segment_g": (C.c_int, [_H, _D]),
    "vvgpu_set_segment_state": (C.c_int, [_H, _D, _D, _D]),
    "vvgpu_clear_bodies": (C.c_int, [_H]),
    "vvgpu_set_body_params": (C.c_int, [_H, C.c_int, C.POINTER(BodyParams)]),
    "vvgpu_set_velocities": (C.c_int, [_H, _D, _D]),
    "vvgpu_set_sinks": (C.c_int, [_H, C.c_int64, _D, _D, _D]),
    "vvgpu_set_vortices": (C.c_int, [_H, C.c_int64, _D, _D, _D, _D]),
    "vvgpu_set_vortices_device": (C.c_int, [_H, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "vvgpu_num_vortices": (C.c_int64, [_H]),
    "vvgpu_num_segments": (C.c_int64, [_H]),
    "vvgpu_get_vortices": (C.c_int, [_H, _D, _D, _D, _D, _D, _D, _I64]),
    "vvgpu_get_vortices_async": (C.c_int, [_H, _D, _D, _D, _D, _I64]),
    "vvgpu_wait_vortices": (C.c_int, [_H]),
    "vvgpu_device_arrays": (C.c_int, [_H] + [C.POINTER(C.c_void_p)] * 6),
    "vvgpu_get_segments": (C.c_int, [_H] + [_D] * 8),
    "vvgpu_get_body_geom": (C.c_int, [_H, C.c_int] + [_D] * 5),
    "vvgpu_tree_build": (C.c_int, [_H, C.c_double, C.c_double, C.c_double]),
    "vvgpu_tree_destroy": (C.c_int, [_H]),
    "vvgpu_eps": (C.c_int, [_H, C.c_int, _I64]),
    "vvgpu_convective": (C.c_int, [_H]),
    "vvgpu_diffusive": (C.c_int, [_H]),
    "vvgpu_velocity_points": (C.c_int, [_H, C.c_int64, _D, _D, _D, _D]),
    "vvgpu_velocity_points_noalloc": (C.c_int, [_H, C.c_int64, _D, _D, _D, _D]),
    "vvgpu_slae": (C.c_int, [_H, C.POINTER(BodyOut)]),
    "vvgpu_vortex_shed": (C.c_int, [_H]),
    "vvgpu_move_and_clean": (C.c_int, [_H, C.c_int, C.POINTER(C.c_int64)]),
    "vvgpu_get_body_params": (C.c_int, [_H, C.c_int, C.POINTER(BodyParams)]),
    "vvgpu_calc_forces": (C.c_int, [_H, _D]),
    "vvgpu_zero_forces": (C.c_int, [_H]),
    "vvgpu_get_segment_forces": (C.c_int, [_H, _D, _D, _D]),
    "vvgpu_gsum": (C.c_int, [_H, _D]),
    "vvgpu_direct_velocity": (C.c_int, [_H, C.c_int64, _D, _D, _D, _D]),
    "vvgpu_batch_step": (C.c_int, [C.POINTER(_H), C.c_int64, C.POINTER(StepCfg), C.c_int32, _D, _I32]),
    "vvgpu_batch_autotune": (C.c_int, [C.POINTER(_H), C.c_int64, C.POINTER(StepCfg), _I32, C.c_int32, _I32,
                                       C.POINTER(C.c_double)]),
    "vvgpu_mlp_create": (C.c_int, [C.c_int, C.c_uint64, C.POINTER(_H)]),
    "vvgpu_mlp_destroy": (C.c_int, [_H]),
    "vvgpu_mlp_last_error": (C.c_char_p, [_H]),
    "vvgpu_mlp_set_wait_limit": (C.c_int, [_H, C.c_int64]),
    "vvgpu_mlp_num_params": (C.c_int64, []),
    "vvgpu_mlp_get_params": (C.c_int, [_H, _F]),
    "vvgpu_mlp_set_params": (C.c_int, [_H, _F]),
    "vvgpu_mlp_set_norm": (C.c_int, [_H, _F]),
    "vvgpu_mlp_get_norm": (C.c_int, [_H, _F]),
    "vvgpu_mlp_fit_norm": (C.c_int, [_H]),
    "vvgpu_mlp_set_samples": (C.c_int, [_H, C.c_int64, _F, _F]),
    "vvgpu_mlp_num_samples": (C.c_int64, [_H]),
    "vvgpu_mlp_get_samples": (C.c_int, [_H, C.c_int64, C.c_int64, _F, _F]),
    "vvgpu_mlp_add_samples": (C.c_int, [_H, _H, C.c_int64, _D, _D, _I64]),
    "vvgpu_mlp_gradient": (C.c_int, [_H, C.c_int64, _F, _F]),
    "vvgpu_mlp_train": (C.c_int, [_H, C.c_int64, C.c_int64, C.c_float, C.c_uint64, _F]),
    "vvgpu_mlp_forward": (C.c_int, [_H, C.c_int64, _F, _F]),
    "vvgpu_velocity_points_learned": (C.c_int, [_H, _H, C.c_int64, _D, _D, _D, _D, _I64]),
    "vvgpu_convective_learned": (C.c_int, [_H, _H, C.POINTER(JudgeCfg), C.POINTER(JudgeOut)]),
    "vvgpu_keep_far_lists": (C.c_int, [_H, C.c_int]),
    "vvgpu_field_velocity": (C.c_int, [_H, C.c_double, C.c_double, C.c_double, C.c_int32, C.c_int32,
                                       C.c_char, C.c_char, _F]),
    "vvgpu_field_streamfunction": (C.c_int, [_H, C.c_double, C.c_double, C.c_double, C.c_int32, C.c_int32,
                                             C.c_double, C.c_char, _F, C.c_int64, _U16, _U16, _F, _I64]),
    "vvgpu_field_vorticity": (C.c_int, [_H, C.c_double, C.c_double, C.c_double, C.c_int32, C.c_int32,
                                        C.c_double, _F]),
    "vvgpu_tree_sizes": (C.c_int, [_H, _I64, _I64, _I64, _I64]),
    "vvgpu_tree_leaves": (C.c_int, [_H, _D, _D, _D, _D, _I64, _I64, _I32, _I64, _I64, _I64]),
    "vvgpu_tree_nodes": (C.c_int, [_H, _D, _D, _D, _D, _I64, _I64, _I32, _I64] + [_D] * 6),
    "vvgpu_tree_seg_order": (C.c_int, [_H, _I64]),
    "vvgpu_tree_lists": (C.c_int, [_H, _I64, _I32, _I64, _I64, _I32, _I64]),
    "vvgpu_slae_size": (C.c_int64, [_H]),
    "vvgpu_slae_export": (C.c_int, [_H, _D, _D, _D]),
}

_lib = None


def load_library(path: str = LIB_PATH):
    """Loads libvvgpu.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with `python -m vvflow_gb300.build`")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def _p(a, ct=C.c_double):
    return a.ctypes.data_as(C.POINTER(ct)) if a is not None else None


def default_body_params() -> BodyParams:
    bp = BodyParams()
    bp.density = 1.0
    bp.kspring_x = bp.kspring_y = bp.kspring_o = float("inf")
    return bp


class GpuSpace:
    """One Space on the GPU; method names follow the oracle's driver."""

    kind = "gpu"

    def __init__(self, precision: int = VVGPU_FP64, device: int = 0, reserve: int = 0):
        self.lib = load_library()
        cfg = Cfg(device, precision, reserve, 0)
        h = _H()
        rc = self.lib.vvgpu_ctx_create(C.byref(cfg), C.byref(h))
        if rc != 0:
            raise VVGpuError(rc, "vvgpu_ctx_create", "(needs a CUDA device)")
        self.h = h
        self.nbodies = 0
        self.precision = precision

    def close(self):
        if getattr(self, "h", None):
            self.lib.vvgpu_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ok(self, rc, what):
        if rc != 0:
            msg = self.lib.vvgpu_last_error(self.h)
            raise VVGpuError(rc, what, msg.decode() if msg else "")

    def stats(self):
        s = Stats()
        self._ok(self.lib.vvgpu_get_stats(self.h, C.byref(s)), "get_stats")
        d = {k: getattr(s, k) for k, _ in Stats._fields_ if k != "reserved"}
        d["launches"] = int(s.reserved[0])
        d["eps_evaluations"] = int(s.reserved[1])
        d["diff_sources"] = int(s.reserved[2])
        d["eps_records"] = int(s.reserved[3])
        d["walk_loads"] = int(s.reserved[4])
        return d

    # -- state -----------------------------------------------------------------------
    TIMING_SLOTS = ("tree_build", "walk", "eps_round", "eps_cand", "eps_pass", "convective", "diffusive", "slae",
                    "learned", "judge")

    def set_kernel_timing(self, on: bool = True):
        self._ok(self.lib.vvgpu_set_kernel_timing(self.h, int(bool(on))), "set_kernel_timing")

    def kernel_timing(self):
        """{slot: (device ms, timed launches)} since timing was switched on."""
        ms = np.zeros(len(self.TIMING_SLOTS))
        cnt = np.zeros(len(self.TIMING_SLOTS), np.int64)
        self._ok(self.lib.vvgpu_get_kernel_timing(self.h, _p(ms), _p(cnt, C.c_int64)), "get_kernel_timing")
        return {k: (float(ms[i]), int(cnt[i])) for i, k in enumerate(self.TIMING_SLOTS)}

    def keep_far_lists(self, on: bool = True):
        self._ok(self.lib.vvgpu_keep_far_lists(self.h, int(bool(on))), "keep_far_lists")

    def convective_learned(self, mlp, targets=4096, far_criteria=8.0, bound=5e-3, seed=1):
        """process_all_lists with the learned far field, judged by the plain tree at
        far_criteria on `targets` sampled vortices (0: no judge).  Returns the verdict."""
        cfg = JudgeCfg(int(targets), float(far_criteria), float(bound), int(seed))
        out = JudgeOut()
        self._ok(self.lib.vvgpu_convective_learned(self.h, mlp.h, C.byref(cfg) if targets else None,
                                                   C.byref(out)), "convective_learned")
        return {k: getattr(out, k) for k, _ in JudgeOut._fields_ if k != "reserved"}

    def set_eps_round_limit(self, max_rounds: int):
        self._ok(self.lib.vvgpu_set_eps_round_limit(self.h, int(max_rounds)), "set_eps_round_limit")

    def autotune_tiles(self):
        """Times the FP32 pair passes' kernel shapes on the current tree and keeps the fastest;
        returns (conv_tile, diff_targets, ms[5])."""
        t, d = np.zeros(1, np.int32), np.zeros(1, np.int32)
        ms = np.zeros(5)
        self._ok(self.lib.vvgpu_autotune_tiles(self.h, _p(t, C.c_int32), _p(d, C.c_int32), _p(ms, C.c_double)),
                 "autotune_tiles")
        return int(t[0]), int(d[0]), ms

    def set_tiles(self, conv_tile: int = 256, diff_targets: int = 1):
        self._ok(self.lib.vvgpu_set_tiles(self.h, int(conv_tile), int(diff_targets)), "set_tiles")

    def tiles(self):
        t, d = np.zeros(1, np.int32), np.zeros(1, np.int32)
        self._ok(self.lib.vvgpu_get_tiles(self.h, _p(t, C.c_int32), _p(d, C.c_int32)), "get_tiles")
        return int(t[0]), int(d[0])

    def set_autotune(self, on: bool = True):
        self._ok(self.lib.vvgpu_set_autotune(self.h, int(bool(on))), "set_autotune")

    STAGE_SPINS = 1 << 22  # default polls of one staging wait

    def set_wait_limit(self, spins: int = STAGE_SPINS):
        """polls of one shared-memory staging wait of the FP32 near field (0: every wait
        runs out and the call raises VVGPU_ERR_TIMEOUT)"""
        self._ok(self.lib.vvgpu_set_wait_limit(self.h, int(spins)), "set_wait_limit")

    def set_params(self, re, dt, inf_vx=1.0, inf_vy=0.0, inf_g=0.0, time=0.0, gx=0.0, gy=0.0):
        self._ok(self.lib.vvgpu_set_params(self.h, re, dt, inf_vx, inf_vy, inf_g, time, gx, gy), "set_params")

    def add_body(self, cx, cy, slip=None, params: BodyParams | None = None):
        cx = np.ascontiguousarray(cx, np.float64)
        cy = np.ascontiguousarray(cy, np.float64)
        sl = None if slip is None else np.ascontiguousarray(slip, np.uint32)
        bp = params if params is not None else default_body_params()
        self._ok(self.lib.vvgpu_add_body(self.h, len(cx), _p(cx), _p(cy), _p(sl, C.c_uint32), C.byref(bp)), "add_body")
        self.nbodies += 1

    def clear_bodies(self):
        self._ok(self.lib.vvgpu_clear_bodies(self.h), "clear_bodies")

    def set_segment_g(self, g):
        g = np.ascontiguousarray(g, np.float64)
        self._ok(self.lib.vvgpu_set_segment_g(self.h, _p(g)), "set_segment_g")

    def set_segment_state(self, g=None, fric=None, gsum=None):
        arr = [None if a is None else np.ascontiguousarray(a, np.float64) for a in (g, fric, gsum)]
        self._ok(self.lib.vvgpu_set_segment_state(self.h, *(_p(a) for a in arr)), "set_segment_state")

    def set_sinks(self, x, y, g):
        x, y, g = (np.ascontiguousarray(a, np.float64) for a in (x, y, g))
        self._ok(self.lib.vvgpu_set_sinks(self.h, len(x), _p(x), _p(y), _p(g)), "set_sinks")

    def set_vortices(self, x, y, g, inv_eps=None):
        x, y, g = (np.ascontiguousarray(a, np.float64) for a in (x, y, g))
        ie = None if inv_eps is None else np.ascontiguousarray(inv_eps, np.float64)
        self._ok(self.lib.vvgpu_set_vortices(self.h, len(x), _p(x), _p(y), _p(g), _p(ie)), "set_vortices")

    def set_vortices_device(self, n, x_ptr, y_ptr, g_ptr, ie_ptr=None):
        self._ok(self.lib.vvgpu_set_vortices_device(self.h, n, x_ptr, y_ptr, g_ptr, ie_ptr), "set_vortices_device")

    def load(self, wl, inv_eps=None, time=0.0):
        self.set_params(wl.re, wl.dt, wl.inf_vx, wl.inf_vy, 0.0, time)
        for cx, cy in wl.bodies:
            self.add_body(cx, cy)
        self.set_vortices(wl.x, wl.y, wl.g, inv_eps)

    @property
    def n(self):
        return int(self.lib.vvgpu_num_vortices(self.h))

    @property
    def m(self):
        return int(self.lib.vvgpu_num_segments(self.h))

    def vortices(self):
        n = self.n
        out = {k: np.empty(n) for k in ("x", "y", "g", "inv_eps", "vx", "vy")}
        out["orig"] = np.empty(n, np.int64)
        self._ok(self.lib.vvgpu_get_vortices(self.h, *(_p(out[k]) for k in ("x", "y", "g", "inv_eps", "vx", "vy")),
                                             _p(out["orig"], C.c_int64)), "get_vortices")
        return out

    def segments(self):
        m = self.m
        keys = ("rx", "ry", "dlx", "dly", "inv_eps", "g", "fric", "gsum")
        out = {k: np.empty(m) for k in keys}
        self._ok(self.lib.vvgpu_get_segments(self.h, *(_p(out[k]) for k in keys)), "get_segments")
        return out

    def body_geom(self, b=0):
        vals = [C.c_double() for _ in range(5)]
        self._ok(self.lib.vvgpu_get_body_geom(self.h, b, *(C.byref(v) for v in vals)), "get_body_geom")
        return dict(zip(("area", "cofm_x", "cofm_y", "moi_axis", "slen"), (v.value for v in vals)))

    # -- hot path ----------------------------------------------------------------------
    def tree_build(self, far_criteria, min_node, max_node):
        self._ok(self.lib.vvgpu_tree_build(self.h, far_criteria, min_node, max_node), "tree_build")

    def tree_destroy(self):
        self._ok(self.lib.vvgpu_tree_destroy(self.h), "tree_destroy")

    def eps(self, merge=True):
        m = C.c_int64()
        self._ok(self.lib.vvgpu_eps(self.h, int(bool(merge)), C.byref(m)), "eps")
        return m.value

    def convective(self):
        self._ok(self.lib.vvgpu_convective(self.h), "convective")

    def diffusive(self):
        self._ok(self.lib.vvgpu_diffusive(self.h), "diffusive")

    def velocity_points(self, px, py):
        px = np.ascontiguousarray(px, np.float64)
        py = np.ascontiguousarray(py, np.float64)
        vx = np.empty_like(px)
        vy = np.empty_like(px)
        self._ok(self.lib.vvgpu_velocity_points(self.h, len(px), _p(px), _p(py), _p(vx), _p(vy)), "velocity_points")
        return vx, vy

    def slae(self):
        out = (BodyOut * max(self.nbodies, 1))()
        self._ok(self.lib.vvgpu_slae(self.h, out), "slae")
        return [{k: getattr(out[i], k) for k, _ in BodyOut._fields_} for i in range(self.nbodies)]

    def slae_export(self):
        n = int(self.lib.vvgpu_slae_size(self.h))
        A = np.empty((n, n))
        b = np.empty(n)
        x = np.empty(n)
        self._ok(self.lib.vvgpu_slae_export(self.h, _p(A), _p(b), _p(x)), "slae_export")
        return A, b, x

    def vortex_shed(self):
        self._ok(self.lib.vvgpu_vortex_shed(self.h), "vortex_shed")

    def direct_velocity(self, px, py):
        """FP64 direct sum over every vortex (no tree) at the points."""
        px = np.ascontiguousarray(px, np.float64)
        py = np.ascontiguousarray(py, np.float64)
        vx = np.empty_like(px)
        vy = np.empty_like(px)
        self._ok(self.lib.vvgpu_direct_velocity(self.h, len(px), _p(px), _p(py), _p(vx), _p(vy)), "direct_velocity")
        return vx, vy

    # -- grid fields (XVelocity, XStreamfunction, XVorticity); out[yj, xi] float32 ------
    def field_velocity(self, xmin, ymin, dxdy, xres, yres, mode="x", ref_frame="o"):
        out = np.zeros((yres, xres), np.float32)
        self._ok(self.lib.vvgpu_field_velocity(self.h, xmin, ymin, dxdy, xres, yres, mode.encode(),
                                               ref_frame.encode(), _p(out, C.c_float)), "field_velocity")
        return out

    def field_streamfunction(self, xmin, ymin, dxdy, xres, yres, eps_mult=1.0, ref_frame="o", gap_cap=4096):
        out = np.zeros((yres, xres), np.float32)
        gx = np.zeros(gap_cap, np.uint16)
        gy = np.zeros(gap_cap, np.uint16)
        gv = np.zeros(gap_cap, np.float32)
        ng = C.c_int64(0)
        self._ok(self.lib.vvgpu_field_streamfunction(self.h, xmin, ymin, dxdy, xres, yres, eps_mult,
                                                     ref_frame.encode(), _p(out, C.c_float), gap_cap,
                                                     _p(gx, C.c_uint16), _p(gy, C.c_uint16),
                                                     _p(gv, C.c_float), C.byref(ng)), "field_streamfunction")
        k = min(int(ng.value), gap_cap)
        return out, (gx[:k].copy(), gy[:k].copy(), gv[:k].copy())

    def field_vorticity(self, xmin, ymin, dxdy, xres, yres, eps_mult=1.0):
        out = np.zeros((yres, xres), np.float32)
        self._ok(self.lib.vvgpu_field_vorticity(self.h, xmin, ymin, dxdy, xres, yres, eps_mult,
                                                _p(out, C.c_float)), "field_vorticity")
        return out

    def gsum(self):
        v = C.c_double()
        self._ok(self.lib.vvgpu_gsum(self.h, C.byref(v)), "gsum")
        return v.value

    def set_velocities(self, vx, vy):
        """TObj::v of every vortex (host arrays of the current list length)."""
        vx = np.ascontiguousarray(vx, dtype=np.float64)
        vy = np.ascontiguousarray(vy, dtype=np.float64)
        self._ok(self.lib.vvgpu_set_velocities(self.h, _p(vx), _p(vy)), "set_velocities")

    def move_and_clean(self, remove: bool = True) -> int:
        """MFlowmove::move_and_clean (MFlowmove.cpp:11-215); returns the number of vortices
        erased inside bodies."""
        n = C.c_int64(0)
        self._ok(self.lib.vvgpu_move_and_clean(self.h, 1 if remove else 0, C.byref(n)), "move_and_clean")
        return int(n.value)

    def body_params(self, b: int = 0) -> dict:
        bp = BodyParams()
        self._ok(self.lib.vvgpu_get_body_params(self.h, int(b), C.byref(bp)), "get_body_params")
        return {k: getattr(bp, k) for k, _ in BodyParams._fields_}

    def set_body_params(self, b: int = 0, **changes):
        """Updates the named fields of body b's parameters (vvgpu_body_params)."""
        bp = BodyParams()
        self._ok(self.lib.vvgpu_get_body_params(self.h, int(b), C.byref(bp)), "get_body_params")
        for k, v in changes.items():
            if k not in dict(BodyParams._fields_):
                raise KeyError(k)
            setattr(bp, k, v)
        self._ok(self.lib.vvgpu_set_body_params(self.h, int(b), C.byref(bp)), "set_body_params")

    def calc_forces(self) -> np.ndarray:
        """Space::calc_forces (TSpace.cpp:94-117); per body [friction x, y, o, nusselt]."""
        out = np.zeros((self.nbodies, 4))
        self._ok(self.lib.vvgpu_calc_forces(self.h, _p(out)), "calc_forces")
        return out

    def zero_forces(self):
        self._ok(self.lib.vvgpu_zero_forces(self.h), "zero_forces")

    def segment_forces(self) -> dict:
        m = self.m
        out = {k: np.empty(m) for k in ("cp", "fr", "nu")}
        self._ok(self.lib.vvgpu_get_segment_forces(self.h, _p(out["cp"]), _p(out["fr"]), _p(out["nu"])),
                 "get_segment_forces")
        return out

    def set_stream(self, stream_ptr: int | None):
        """Queues all work on the caller's CUDA stream (cudaStream_t as an integer)."""
        self._ok(self.lib.vvgpu_set_stream(self.h, C.c_void_p(stream_ptr) if stream_ptr else None), "set_stream")

    def get_vortices_into(self, x=0, y=0, g=0, ie=0, vx=0, vy=0, orig=0):
        """Copies the vortex list into caller-owned host buffers given as addresses (0 = skip)."""
        D = C.POINTER(C.c_double)
        f = lambda a, t=D: C.cast(C.c_void_p(a), t) if a else None
        self._ok(self.lib.vvgpu_get_vortices(self.h, f(x), f(y), f(g), f(ie), f(vx), f(vy),
                                             f(orig, C.POINTER(C.c_int64))), "get_vortices")

    def get_vortices_async(self, x=0, y=0, g=0, ie=0, orig=0):
        """Starts copying positions, circulations, inverse epsilons and origin indices into
        caller-owned host buffers given as addresses (0 = skip) and returns at once; the
        buffers are ready after wait_vortices()."""
        D = C.POINTER(C.c_double)
        f = lambda a, t=D: C.cast(C.c_void_p(a), t) if a else None
        self._ok(self.lib.vvgpu_get_vortices_async(self.h, f(x), f(y), f(g), f(ie), f(orig, C.POINTER(C.c_int64))),
                 "get_vortices_async")

    def wait_vortices(self):
        self._ok(self.lib.vvgpu_wait_vortices(self.h), "wait_vortices")

    def set_vortices_from(self, n, x, y, g, ie=0):
        """Replaces the vortex list from host buffers given as addresses (e.g. pinned memory)."""
        D = C.POINTER(C.c_double)
        f = lambda a: C.cast(C.c_void_p(a), D) if a else None
        self._ok(self.lib.vvgpu_set_vortices(self.h, n, f(x), f(y), f(g), f(ie)), "set_vortices")

    def synchronize(self):
        self._ok(self.lib.vvgpu_synchronize(self.h), "synchronize")

    # -- inspection -------------------------------------------------------------------
    def tree_sizes(self):
        v = [C.c_int64() for _ in range(4)]
        self._ok(self.lib.vvgpu_tree_sizes(self.h, *(C.byref(a) for a in v)), "tree_sizes")
        return tuple(a.value for a in v)

    def tree_leaves(self):
        _, nl, _, _ = self.tree_sizes()
        d = {k: np.empty(nl) for k in ("x", "y", "h", "w")}
        for k in ("vfirst", "vlast", "path", "sfirst", "slast"):
            d[k] = np.empty(nl, np.int64)
        d["depth"] = np.empty(nl, np.int32)
        self._ok(self.lib.vvgpu_tree_leaves(self.h, _p(d["x"]), _p(d["y"]), _p(d["h"]), _p(d["w"]),
                                            _p(d["vfirst"], C.c_int64), _p(d["vlast"], C.c_int64),
                                            _p(d["depth"], C.c_int32), _p(d["path"], C.c_int64),
                                            _p(d["sfirst"], C.c_int64), _p(d["slast"], C.c_int64)), "tree_leaves")
        return d

    def tree_nodes(self):
        nn, _, _, _ = self.tree_sizes()
        keys_d = ("x", "y", "h", "w")
        keys_c = ("cmp_x", "cmp_y", "cmp_g", "cmm_x", "cmm_y", "cmm_g")
        d = {k: np.empty(nn) for k in keys_d + keys_c}
        d["vfirst"] = np.empty(nn, np.int64)
        d["vlast"] = np.empty(nn, np.int64)
        d["depth"] = np.empty(nn, np.int32)
        d["path"] = np.empty(nn, np.int64)
        self._ok(self.lib.vvgpu_tree_nodes(self.h, *(_p(d[k]) for k in keys_d),
                                           _p(d["vfirst"], C.c_int64), _p(d["vlast"], C.c_int64),
                                           _p(d["depth"], C.c_int32), _p(d["path"], C.c_int64),
                                           *(_p(d[k]) for k in keys_c)), "tree_nodes")
        return d

    def tree_seg_order(self):
        so = np.empty(self.m, np.int64)
        self._ok(self.lib.vvgpu_tree_seg_order(self.h, _p(so, C.c_int64)), "tree_seg_order")
        return so

    def tree_lists(self, far=True):
        """Near and far lists of every leaf as (depth, path) of the nodes; far=False leaves
        out the far nodes (only their offsets)."""
        _, nl, nnear, nfar = self.tree_sizes()
        d = {"near_off": np.empty(nl + 1, np.int64), "far_off": np.empty(nl + 1, np.int64),
             "near_depth": np.empty(nnear, np.int32), "near_path": np.empty(nnear, np.int64),
             "far_depth": np.empty(nfar if far else 0, np.int32), "far_path": np.empty(nfar if far else 0, np.int64)}
        if not far:
            d["far_depth"] = d["far_path"] = None
        self._ok(self.lib.vvgpu_tree_lists(self.h, _p(d["near_off"], C.c_int64), _p(d["near_depth"], C.c_int32),
                                           _p(d["near_path"], C.c_int64), _p(d["far_off"], C.c_int64),
                                           _p(d["far_depth"], C.c_int32), _p(d["far_path"], C.c_int64)), "tree_lists")
        return d


class Batch:
    """Many independent GpuSpace instances advanced together (vvgpu_batch_step): each step
    is simulate()'s step (tree build, SLAE, destroy, shed, tree build, eps, convective,
    diffusive, destroy), optionally followed by move_and_clean, per instance with its own
    tree sizes."""

    def __init__(self, spaces, far_criteria, node_sizes, merge=True, move=True):
        self.lib = load_library()
        self.spaces = list(spaces)
        n = len(self.spaces)
        self.handles = (_H * n)(*[S.h for S in self.spaces])
        self.cfgs = (StepCfg * n)()
        for i, (mn, mx) in enumerate(node_sizes):
            fc = far_criteria[i] if hasattr(far_criteria, "__len__") else far_criteria
            self.cfgs[i] = StepCfg(fc, mn, mx, 1 if merge else 0, 1 if move else 0)
        self.nthreads = 0

    def step(self, nthreads=None):
        """One batched step; returns each instance's wall time in ms (stream synchronised)."""
        n = len(self.spaces)
        ms = np.zeros(n)
        st = np.zeros(n, np.int32)
        nt = self.nthreads if nthreads is None else nthreads
        rc = self.lib.vvgpu_batch_step(self.handles, n, self.cfgs, nt, _p(ms), _p(st, C.c_int32))
        if rc != 0:
            bad = [i for i in range(n) if st[i] != 0]
            i = bad[0] if bad else 0
            msg = self.lib.vvgpu_last_error(self.spaces[i].h)
            raise VVGpuError(rc, f"batch_step (instance {i})", msg.decode() if msg else "")
        return ms

    def autotune(self, candidates=(1, 2, 4, 8, 16)):
        """Times one batched step per pool size (the steps advance the instances) and keeps
        the fastest; returns (pool size, ms)."""
        cand = np.asarray(candidates, np.int32)
        best = C.c_int32(0)
        bms = C.c_double(0)
        rc = self.lib.vvgpu_batch_autotune(self.handles, len(self.spaces), self.cfgs, _p(cand, C.c_int32),
                                          len(cand), C.byref(best), C.byref(bms))
        if rc != 0:
            raise VVGpuError(rc, "batch_autotune")
        self.nthreads = int(best.value)
        return self.nthreads, float(bms.value)


class Mlp:
    """The learned far-field correction (vvgpu_mlp_*): an MLP 20 -> 64 -> 64 -> 2 trained on
    (target, far cell) pairs of a built tree with FP64 direct-sum labels."""

    NF = 20

    def __init__(self, device: int = 0, seed: int = 1):
        self.lib = load_library()
        h = _H()
        rc = self.lib.vvgpu_mlp_create(device, seed, C.byref(h))
        if rc != 0:
            raise VVGpuError(rc, "vvgpu_mlp_create", "(needs a CUDA device)")
        self.h = h
        self.nparam = int(self.lib.vvgpu_mlp_num_params())

    def close(self):
        if getattr(self, "h", None):
            self.lib.vvgpu_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ok(self, rc, what):
        if rc != 0:
            msg = self.lib.vvgpu_mlp_last_error(self.h)
            raise VVGpuError(rc, what, msg.decode() if msg else "")

    def set_wait_limit(self, spins: int):
        self._ok(self.lib.vvgpu_mlp_set_wait_limit(self.h, int(spins)), "mlp_set_wait_limit")

    def params(self):
        out = np.empty(self.nparam, np.float32)
        self._ok(self.lib.vvgpu_mlp_get_params(self.h, _p(out, C.c_float)), "mlp_get_params")
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.nparam
        self._ok(self.lib.vvgpu_mlp_set_params(self.h, _p(p, C.c_float)), "mlp_set_params")

    def norm(self):
        out = np.empty(2 * self.NF + 2, np.float32)
        self._ok(self.lib.vvgpu_mlp_get_norm(self.h, _p(out, C.c_float)), "mlp_get_norm")
        return out

    def set_norm(self, nrm):
        nrm = np.ascontiguousarray(nrm, np.float32)
        self._ok(self.lib.vvgpu_mlp_set_norm(self.h, _p(nrm, C.c_float)), "mlp_set_norm")

    def fit_norm(self):
        self._ok(self.lib.vvgpu_mlp_fit_norm(self.h), "mlp_fit_norm")
        return self.norm()

    def set_samples(self, feat, lab):
        feat = np.ascontiguousarray(feat, np.float32)
        lab = np.ascontiguousarray(lab, np.float32)
        self._ok(self.lib.vvgpu_mlp_set_samples(self.h, len(feat), _p(feat, C.c_float), _p(lab, C.c_float)),
                 "mlp_set_samples")

    @property
    def nsamples(self):
        return int(self.lib.vvgpu_mlp_num_samples(self.h))

    def samples(self, first=0, n=None):
        n = self.nsamples - first if n is None else n
        f = np.empty((n, self.NF), np.float32)
        lab = np.empty((n, 2), np.float32)
        self._ok(self.lib.vvgpu_mlp_get_samples(self.h, first, n, _p(f, C.c_float), _p(lab, C.c_float)),
                 "mlp_get_samples")
        return f, lab

    def add_samples(self, space, px, py):
        px = np.ascontiguousarray(px, np.float64)
        py = np.ascontiguousarray(py, np.float64)
        n = C.c_int64(0)
        self._ok(self.lib.vvgpu_mlp_add_samples(self.h, space.h, len(px), _p(px), _p(py), C.byref(n)),
                 "mlp_add_samples")
        return int(n.value)

    def gradient(self, n=None):
        n = self.nsamples if n is None else n
        g = np.empty(self.nparam, np.float32)
        loss = C.c_float(0)
        self._ok(self.lib.vvgpu_mlp_gradient(self.h, n, _p(g, C.c_float), C.byref(loss)), "mlp_gradient")
        return g, float(loss.value)

    def train(self, epochs, batch=8192, lr=1e-3, seed=1):
        out = np.empty(epochs, np.float32)
        self._ok(self.lib.vvgpu_mlp_train(self.h, epochs, batch, lr, seed, _p(out, C.c_float)), "mlp_train")
        return out

    def forward(self, feat):
        feat = np.ascontiguousarray(feat, np.float32)
        y = np.empty((len(feat), 2), np.float32)
        self._ok(self.lib.vvgpu_mlp_forward(self.h, len(feat), _p(feat, C.c_float), _p(y, C.c_float)), "mlp_forward")
        return y

    def velocity_points(self, space, px, py):
        """velocity(p) of the space's built tree plus the learned correction."""
        px = np.ascontiguousarray(px, np.float64)
        py = np.ascontiguousarray(py, np.float64)
        vx = np.empty(len(px))
        vy = np.empty(len(px))
        n = C.c_int64(0)
        self._ok(self.lib.vvgpu_velocity_points_learned(space.h, self.h, len(px), _p(px), _p(py), _p(vx), _p(vy),
                                                         C.byref(n)), "velocity_points_learned")
        return vx, vy, int(n.value)
