"""Generates attached_bodies.npz in this folder from the reference: the moving-body case of
tests/attached_cases.py (attached vortex and source sheets of
MConvectiveFast::body_list_influence, libvvhd/src/MConvectiveFast.cpp:172-215 and
:440-457) run through the reference's own compiled sources.  The inputs are regenerated
from the seeded case by the tests; the outputs are stored (the FP64 direct sum comes from
the C restatement, the reference having none).

Run where the reference sources are present (compiled unmodified by ``make -C oracle ref``):

    python tests/golden/make_golden_attached.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import attached_cases as AC  # noqa: E402
import oracle  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    oracle.build(ref=True)
    if not oracle.ref_available():
        raise SystemExit("reference library not available; run where the reference sources are")
    c = AC.case()
    S = oracle.OracleSpace("ref")
    out = AC.run(S, c, oracle.default_body_params, direct=False)
    S.close()
    P = oracle.OracleSpace("port")
    d = AC.run(P, c, oracle.default_body_params)
    P.close()
    out["direct_vx"], out["direct_vy"] = d["direct_vx"], d["direct_vy"]
    np.savez_compressed(os.path.join(HERE, "attached_bodies.npz"), **out)
    print("attached_bodies.npz", {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
