"""ctypes driver for the CPU oracle -- TEST INFRASTRUCTURE ONLY.

``OracleSpace("port")`` drives the C restatement (oracle/_build/liboracle.so);
``OracleSpace("ref")`` drives the reference's own sources compiled by ``make ref``
(oracle/_ref/libvvref.so, only buildable where the reference sources are present).
Both expose the same calls; arrays come back as numpy float64/int64.

Only tests/, the smoke entry point and bench.py's CPU-baseline leg import this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "_build", "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libvvref.so")
# the reference checkout: VVD_REFERENCE_DIR, else a sibling folder "reference" of this repository
REF_SRC = os.environ.get("VVD_REFERENCE_DIR", os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))


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


def default_body_params() -> BodyParams:
    bp = BodyParams()
    bp.density = 1.0
    bp.kspring_x = bp.kspring_y = bp.kspring_o = float("inf")
    return bp


def build(ref: bool = False) -> None:
    """Compile the restatement (and, if asked and possible, the reference)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if ref and os.path.isdir(os.path.join(REF_SRC, "libvvhd")):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REF_SRC}"], check=True)


def ref_available() -> bool:
    if os.path.exists(REF_LIB):
        try:
            C.CDLL(REF_LIB)
            return True
        except OSError:
            return False
    return False


_LIBS: dict = {}

_D = C.POINTER(C.c_double)
_I64 = C.POINTER(C.c_int64)
_I32 = C.POINTER(C.c_int32)
_U32 = C.POINTER(C.c_uint32)
_U16 = C.POINTER(C.c_uint16)
_F = C.POINTER(C.c_float)


def _load(kind: str):
    if kind in _LIBS:
        return _LIBS[kind]
    path, pre = (PORT_LIB, "vvo_") if kind == "port" else (REF_LIB, "vvr_")
    if kind == "port" and not os.path.exists(path):
        build(False)
    lib = C.CDLL(path)
    H = C.c_void_p
    sig = {
        "create": (H, []), "destroy": (None, [H]),
        "set_params": (C.c_int, [H] + [C.c_double] * 8),
        "add_body": (C.c_int, [H, C.c_int64, _D, _D, _U32, C.POINTER(BodyParams)]),
        "set_segment_g": (C.c_int, [H, _D]),
        "set_sinks": (C.c_int, [H, C.c_int64, _D, _D, _D]),
        "set_vortices": (C.c_int, [H, C.c_int64, _D, _D, _D, _D]),
        "num_vortices": (C.c_int64, [H]), "num_segments": (C.c_int64, [H]),
        "get_vortices": (C.c_int, [H, _D, _D, _D, _D, _D, _D, _I64]),
        "get_segments": (C.c_int, [H] + [_D] * 8),
        "get_body_geom": (C.c_int, [H, C.c_int] + [_D] * 5),
        "tree_build": (C.c_int, [H, C.c_double, C.c_double, C.c_double]),
        "tree_destroy": (C.c_int, [H]),
        "tree_sizes": (C.c_int, [H, _I64, _I64, _I64, _I64]),
        "tree_leaves": (C.c_int, [H, _D, _D, _D, _D, _I64, _I64, _I32, _I64, _I64, _I64]),
        "tree_nodes": (C.c_int, [H, _D, _D, _D, _D, _I64, _I64, _I32, _I64] + [_D] * 6),
        "tree_seg_order": (C.c_int, [H, _I64]),
        "tree_lists": (C.c_int, [H, _I64, _I32, _I64, _I64, _I32, _I64]),
        "eps": (C.c_int, [H, C.c_int, _I64]),
        "convective": (C.c_int, [H]), "diffusive": (C.c_int, [H]),
        "velocity_points": (C.c_int, [H, C.c_int64, _D, _D, _D, _D]),
        "slae": (C.c_int, [H, C.POINTER(BodyOut)]),
        "slae_size": (C.c_int64, [H]),
        "slae_export": (C.c_int, [H, _D, _D, _D]),
        "vortex_shed": (C.c_int, [H]),
        "gsum": (C.c_double, [H]),
        "set_velocities": (C.c_int, [H, _D, _D]),
        "move_and_clean": (C.c_int, [H, C.c_int, C.POINTER(C.c_int64)]),
        "get_body_params": (C.c_int, [H, C.c_int, C.POINTER(BodyParams)]),
        "set_segment_state": (C.c_int, [H, _D, _D, _D]),
        "calc_forces": (C.c_int, [H, _D]),
        "zero_forces": (C.c_int, [H]),
        "get_segment_forces": (C.c_int, [H, _D, _D, _D]),
        "field_velocity": (C.c_int, [H, C.c_double, C.c_double, C.c_double, C.c_int32, C.c_int32,
                                     C.c_char, C.c_char, _F]),
        "field_streamfunction": (C.c_int, [H, C.c_double, C.c_double, C.c_double, C.c_int32, C.c_int32,
                                           C.c_double, C.c_char, _F, C.c_int64, _U16, _U16, _F, _I64]),
        "field_vorticity": (C.c_int, [H, C.c_double, C.c_double, C.c_double, C.c_int32, C.c_int32,
                                      C.c_double, _F]),
    }
    if kind == "port":
        sig["direct_velocity"] = (C.c_int, [H, C.c_int64, _D, _D, _D, _D])
        sig["set_sample"] = (C.c_int, [H, C.c_int64])
        sig["slae_rhs_step"] = (C.c_int, [H, _D])
        sig["last_timings"] = (C.c_int, [H, _D])
    fns = {}
    for name, (res, args) in sig.items():
        f = getattr(lib, pre + name)
        f.restype = res
        f.argtypes = args
        fns[name] = f
    _LIBS[kind] = fns
    return fns


def _p(a, ct=C.c_double):
    return a.ctypes.data_as(C.POINTER(ct)) if a is not None else None


class OracleError(RuntimeError):
    pass


class OracleSpace:
    """One ``Space`` with the reference's hot-path modules, on the CPU."""

    def __init__(self, kind: str = "port"):
        self.kind = kind
        self.f = _load(kind)
        self.h = self.f["create"]()
        self.nbodies = 0

    def close(self):
        if self.h:
            self.f["destroy"](self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ok(self, rc, what):
        if rc != 0:
            raise OracleError(f"{self.kind}:{what} returned {rc}")

    # -- state -----------------------------------------------------------------------
    def set_params(self, re, dt, inf_vx=1.0, inf_vy=0.0, inf_g=0.0, time=0.0, gx=0.0, gy=0.0):
        self._ok(self.f["set_params"](self.h, re, dt, inf_vx, inf_vy, inf_g, time, gx, gy), "set_params")

    def add_body(self, cx, cy, slip=None, params: BodyParams | None = None):
        cx = np.ascontiguousarray(cx, np.float64)
        cy = np.ascontiguousarray(cy, np.float64)
        sl = None if slip is None else np.ascontiguousarray(slip, np.uint32)
        bp = params if params is not None else default_body_params()
        self._ok(self.f["add_body"](self.h, len(cx), _p(cx), _p(cy), _p(sl, C.c_uint32), C.byref(bp)), "add_body")
        self.nbodies += 1

    def set_segment_g(self, g):
        g = np.ascontiguousarray(g, np.float64)
        self._ok(self.f["set_segment_g"](self.h, _p(g)), "set_segment_g")

    def set_sinks(self, x, y, g):
        x, y, g = (np.ascontiguousarray(a, np.float64) for a in (x, y, g))
        self._ok(self.f["set_sinks"](self.h, len(x), _p(x), _p(y), _p(g)), "set_sinks")

    def set_vortices(self, x, y, g, inv_eps=None):
        x, y, g = (np.ascontiguousarray(a, np.float64) for a in (x, y, g))
        ie = None if inv_eps is None else np.ascontiguousarray(inv_eps, np.float64)
        self._ok(self.f["set_vortices"](self.h, len(x), _p(x), _p(y), _p(g), _p(ie)), "set_vortices")

    def load(self, wl, inv_eps=None, time=0.0):
        self.set_params(wl.re, wl.dt, wl.inf_vx, wl.inf_vy, 0.0, time)
        for cx, cy in wl.bodies:
            self.add_body(cx, cy)
        self.set_vortices(wl.x, wl.y, wl.g, inv_eps)

    @property
    def n(self):
        return int(self.f["num_vortices"](self.h))

    @property
    def m(self):
        return int(self.f["num_segments"](self.h))

    def vortices(self):
        n = self.n
        out = {k: np.empty(n) for k in ("x", "y", "g", "inv_eps", "vx", "vy")}
        out["orig"] = np.empty(n, np.int64)
        self._ok(self.f["get_vortices"](self.h, *(_p(out[k]) for k in ("x", "y", "g", "inv_eps", "vx", "vy")),
                                        _p(out["orig"], C.c_int64)), "get_vortices")
        return out

    def segments(self):
        m = self.m
        keys = ("rx", "ry", "dlx", "dly", "inv_eps", "g", "fric", "gsum")
        out = {k: np.empty(m) for k in keys}
        self._ok(self.f["get_segments"](self.h, *(_p(out[k]) for k in keys)), "get_segments")
        return out

    def body_geom(self, b=0):
        vals = [C.c_double() for _ in range(5)]
        self._ok(self.f["get_body_geom"](self.h, b, *(C.byref(v) for v in vals)), "get_body_geom")
        return dict(zip(("area", "cofm_x", "cofm_y", "moi_axis", "slen"), (v.value for v in vals)))

    # -- tree --------------------------------------------------------------------------
    def tree_build(self, far_criteria, min_node, max_node):
        self._ok(self.f["tree_build"](self.h, far_criteria, min_node, max_node), "tree_build")

    def tree_destroy(self):
        self._ok(self.f["tree_destroy"](self.h), "tree_destroy")

    def tree_sizes(self):
        v = [C.c_int64() for _ in range(4)]
        self._ok(self.f["tree_sizes"](self.h, *(C.byref(a) for a in v)), "tree_sizes")
        return tuple(a.value for a in v)

    def tree_leaves(self):
        _, nl, _, _ = self.tree_sizes()
        d = {k: np.empty(nl) for k in ("x", "y", "h", "w")}
        for k in ("vfirst", "vlast", "path", "sfirst", "slast"):
            d[k] = np.empty(nl, np.int64)
        d["depth"] = np.empty(nl, np.int32)
        self._ok(self.f["tree_leaves"](self.h, _p(d["x"]), _p(d["y"]), _p(d["h"]), _p(d["w"]),
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
        self._ok(self.f["tree_nodes"](self.h, *(_p(d[k]) for k in keys_d),
                                      _p(d["vfirst"], C.c_int64), _p(d["vlast"], C.c_int64),
                                      _p(d["depth"], C.c_int32), _p(d["path"], C.c_int64),
                                      *(_p(d[k]) for k in keys_c)), "tree_nodes")
        return d

    def tree_seg_order(self):
        so = np.empty(self.m, np.int64)
        self._ok(self.f["tree_seg_order"](self.h, _p(so, C.c_int64)), "tree_seg_order")
        return so

    def tree_lists(self, far=True):
        _, nl, nnear, nfar = self.tree_sizes()
        d = {"near_off": np.empty(nl + 1, np.int64), "far_off": np.empty(nl + 1, np.int64),
             "near_depth": np.empty(nnear, np.int32), "near_path": np.empty(nnear, np.int64),
             "far_depth": np.empty(nfar if far else 0, np.int32), "far_path": np.empty(nfar if far else 0, np.int64)}
        if not far:
            d["far_depth"] = d["far_path"] = None
        self._ok(self.f["tree_lists"](self.h, _p(d["near_off"], C.c_int64), _p(d["near_depth"], C.c_int32),
                                      _p(d["near_path"], C.c_int64), _p(d["far_off"], C.c_int64),
                                      _p(d["far_depth"], C.c_int32), _p(d["far_path"], C.c_int64)), "tree_lists")
        return d

    # -- modules -----------------------------------------------------------------------
    def eps(self, merge=True):
        m = C.c_int64()
        self._ok(self.f["eps"](self.h, int(bool(merge)), C.byref(m)), "eps")
        return m.value

    def convective(self):
        self._ok(self.f["convective"](self.h), "convective")

    def diffusive(self):
        self._ok(self.f["diffusive"](self.h), "diffusive")

    def velocity_points(self, px, py):
        px = np.ascontiguousarray(px, np.float64)
        py = np.ascontiguousarray(py, np.float64)
        vx = np.empty_like(px)
        vy = np.empty_like(px)
        self._ok(self.f["velocity_points"](self.h, len(px), _p(px), _p(py), _p(vx), _p(vy)), "velocity_points")
        return vx, vy

    def direct_velocity(self, px, py):
        px = np.ascontiguousarray(px, np.float64)
        py = np.ascontiguousarray(py, np.float64)
        vx = np.empty_like(px)
        vy = np.empty_like(px)
        self._ok(self.f["direct_velocity"](self.h, len(px), _p(px), _p(py), _p(vx), _p(vy)), "direct_velocity")
        return vx, vy

    def slae(self):
        out = (BodyOut * max(self.nbodies, 1))()
        self._ok(self.f["slae"](self.h, out), "slae")
        return [{k: getattr(out[i], k) for k, _ in BodyOut._fields_} for i in range(self.nbodies)]

    def slae_export(self):
        n = int(self.f["slae_size"](self.h))
        A = np.empty((n, n))
        b = np.empty(n)
        x = np.empty(n)
        self._ok(self.f["slae_export"](self.h, _p(A), _p(b), _p(x)), "slae_export")
        return A, b, x

    def vortex_shed(self):
        self._ok(self.f["vortex_shed"](self.h), "vortex_shed")

    def gsum(self):
        return float(self.f["gsum"](self.h))

    def set_velocities(self, vx, vy):
        vx = np.ascontiguousarray(vx, dtype=np.float64)
        vy = np.ascontiguousarray(vy, dtype=np.float64)
        self._ok(self.f["set_velocities"](self.h, _p(vx), _p(vy)), "set_velocities")

    def move_and_clean(self, remove: bool = True) -> int:
        """MFlowmove::move_and_clean (MFlowmove.cpp:11-215); returns the number of vortices
        removed inside bodies."""
        n = C.c_int64(0)
        self._ok(self.f["move_and_clean"](self.h, 1 if remove else 0, C.byref(n)), "move_and_clean")
        return int(n.value)

    def body_params(self, b: int = 0) -> dict:
        bp = BodyParams()
        self._ok(self.f["get_body_params"](self.h, int(b), C.byref(bp)), "get_body_params")
        return {k: getattr(bp, k) for k, _ in BodyParams._fields_}

    def set_segment_state(self, g=None, fric=None, gsum=None):
        arr = [None if a is None else np.ascontiguousarray(a, np.float64) for a in (g, fric, gsum)]
        self._ok(self.f["set_segment_state"](self.h, *(_p(a) for a in arr)), "set_segment_state")

    def calc_forces(self) -> np.ndarray:
        """Space::calc_forces (TSpace.cpp:94-117); per body [friction x, y, o, nusselt]."""
        out = np.zeros((self.nbodies, 4))
        self._ok(self.f["calc_forces"](self.h, _p(out)), "calc_forces")
        return out

    def zero_forces(self):
        self._ok(self.f["zero_forces"](self.h), "zero_forces")

    def segment_forces(self) -> dict:
        out = {k: np.empty(self.m) for k in ("cp", "fr", "nu")}
        self._ok(self.f["get_segment_forces"](self.h, _p(out["cp"]), _p(out["fr"]), _p(out["nu"])),
                 "get_segment_forces")
        return out

    # grid fields (XVelocity.cpp, XStreamfunction.cpp, XVorticity.cpp); out[yj, xi] float32
    def field_velocity(self, xmin, ymin, dxdy, xres, yres, mode="x", ref_frame="o"):
        out = np.zeros((yres, xres), np.float32)
        self._ok(self.f["field_velocity"](self.h, xmin, ymin, dxdy, xres, yres, mode.encode(),
                                          ref_frame.encode(), _p(out, C.c_float)), "field_velocity")
        return out

    def field_streamfunction(self, xmin, ymin, dxdy, xres, yres, eps_mult=1.0, ref_frame="o", gap_cap=4096):
        out = np.zeros((yres, xres), np.float32)
        gx = np.zeros(gap_cap, np.uint16)
        gy = np.zeros(gap_cap, np.uint16)
        gv = np.zeros(gap_cap, np.float32)
        ng = C.c_int64(0)
        self._ok(self.f["field_streamfunction"](self.h, xmin, ymin, dxdy, xres, yres, eps_mult,
                                                ref_frame.encode(), _p(out, C.c_float), gap_cap,
                                                _p(gx, C.c_uint16), _p(gy, C.c_uint16), _p(gv, C.c_float),
                                                C.byref(ng)), "field_streamfunction")
        k = min(int(ng.value), gap_cap)
        return out, (gx[:k].copy(), gy[:k].copy(), gv[:k].copy())

    def field_vorticity(self, xmin, ymin, dxdy, xres, yres, eps_mult=1.0):
        out = np.zeros((yres, xres), np.float32)
        self._ok(self.f["field_vorticity"](self.h, xmin, ymin, dxdy, xres, yres, eps_mult,
                                           _p(out, C.c_float)), "field_vorticity")
        return out

    def set_sample(self, stride: int):
        self._ok(self.f["set_sample"](self.h, int(stride)), "set_sample")

    def last_timings(self):
        out = np.zeros(3)
        self._ok(self.f["last_timings"](self.h, _p(out)), "last_timings")
        return dict(zip(("partition", "cmass", "lists"), out.tolist()))

    def slae_rhs_step(self):
        self._ok(self.f["slae_rhs_step"](self.h, None), "slae_rhs_step")
