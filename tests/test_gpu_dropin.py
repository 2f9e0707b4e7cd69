"""The C++ drop-in classes (include/vvgpu_modules.hpp) run one step on the GPU the way the
reference's simulate() runs its own classes (tests/cxx/dropin_step.cpp on the host Space of
tests/cxx/mini_space.hpp), and the Space they leave behind equals the oracle's after the same
calls: the permuted and merged vortex list and epsilon bit for bit, velocities within
1e-12, the SLAE solution scattered to the segments and the body unknowns within 1e-10,
friction within 1e-10, a velocity(p) probe within 1e-12."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle
from parity import rel_err, rel_err_vec

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _compile(tmp):
    from vvflow_gb300 import build as B
    lib = B.build()
    libdir = os.path.dirname(lib)
    cudalib = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(B.nvcc()))), "lib64")
    exe = os.path.join(tmp, "dropin_step")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"), "-I",
           os.path.join(ROOT, "tests", "cxx"), os.path.join(ROOT, "tests", "cxx", "dropin_step.cpp"),
           "-L", libdir, "-lvvgpu", f"-Wl,-rpath,{libdir}", f"-Wl,-rpath,{cudalib}", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


@pytest.mark.gpu
@pytest.mark.skipif(shutil.which("g++") is None, reason="no C++ compiler")
def test_dropin_classes_run_one_step(tmp_path):
    from vvflow_gb300 import workloads as W
    exe = _compile(str(tmp_path))
    wl = W.cylinder_annulus(20000, 500, seed=41)
    mn, mx = wl.node_sizes()
    # epsilon of a previous pass, so that the convective pass sees smoothed sources
    R = oracle.OracleSpace("port")
    R.load(wl)
    R.tree_build(wl.far_criteria, mn, mx)
    R.eps(False)
    v0 = R.vortices()
    R.tree_destroy()
    R.close()
    ie = np.empty(wl.n)
    ie[v0["orig"]] = v0["inv_eps"]
    probe = (0.9, 0.35)
    cx, cy = wl.bodies[0]
    with open(tmp_path / "in.bin", "wb") as f:
        np.array([wl.n, len(cx)], np.int64).tofile(f)
        np.array([wl.re, wl.dt, wl.inf_vx, wl.inf_vy, wl.far_criteria, probe[0], probe[1]]).tofile(f)
        np.stack([wl.x, wl.y, wl.g, ie], 1).astype(np.float64).tofile(f)
        np.stack([cx, cy], 1).astype(np.float64).tofile(f)
    r = subprocess.run([exe, str(tmp_path / "in.bin"), str(tmp_path / "out.bin")], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    raw = np.fromfile(tmp_path / "out.bin", np.uint8)
    n, m, merged = np.frombuffer(raw[:24].tobytes(), np.int64)
    body = np.frombuffer(raw[24:].tobytes(), np.float64)
    V = body[:6 * n].reshape(n, 6)
    segs = body[6 * n:6 * n + 2 * m].reshape(m, 2)
    unk = body[6 * n + 2 * m:6 * n + 2 * m + 9]
    pvx, pvy = body[6 * n + 2 * m + 9:6 * n + 2 * m + 11]

    # the same calls on the oracle
    R = oracle.OracleSpace("port")
    R.set_params(wl.re, wl.dt, wl.inf_vx, wl.inf_vy)
    R.add_body(cx, cy)
    R.set_vortices(wl.x, wl.y, wl.g, ie)
    R.tree_build(wl.far_criteria, mn, mx)
    bo = R.slae()[0]
    R.tree_destroy()
    R.tree_build(wl.far_criteria, mn, mx)
    rmerged = R.eps(True)
    R.convective()
    R.diffusive()
    qx, qy = R.velocity_points(np.array([probe[0]]), np.array([probe[1]]))
    ref = R.vortices()
    rs = R.segments()
    R.tree_destroy()
    R.close()

    assert merged == rmerged and merged > 0
    assert n == len(ref["x"]) and m == len(rs["g"])
    for col, k in enumerate(("x", "y", "g", "inv_eps")):
        assert np.array_equal(V[:, col], ref[k]), k
    assert rel_err_vec(V[:, 4], V[:, 5], ref["vx"], ref["vy"]) <= 1e-12
    assert rel_err(segs[:, 0], rs["g"]) <= 1e-10
    assert rel_err(segs[:, 1], rs["fric"]) <= 1e-10
    keys = ("speed_slae_x", "speed_slae_y", "speed_slae_o", "force_hydro_x", "force_hydro_y", "force_hydro_o",
            "force_holder_x", "force_holder_y", "force_holder_o")
    ru = np.array([bo[k] for k in keys])
    assert np.abs(unk - ru).max() <= 1e-10 * (np.abs(ru).max() + 1.0)
    assert rel_err_vec(np.array([pvx]), np.array([pvy]), qx, qy) <= 1e-12
