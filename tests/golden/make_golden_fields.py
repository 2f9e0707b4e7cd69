"""Generates the grid-field fixtures (field_*.npz) in this folder from the reference.

Run where the reference sources are present (compiled unmodified by ``make -C oracle
ref``, together with libvvhd/src/XField.cpp, XVelocity.cpp, XStreamfunction.cpp and
XVorticity.cpp).  A fixture holds the inputs of one case of tests/field_cases.py (in_*)
and the reference's XField::map of every call in field_cases.CALLS, plus the stream
function's gap lists sorted into grid order.

    python tests/golden/make_golden_fields.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import oracle  # noqa: E402
from field_cases import case_arrays, cases, load, run_fields  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    oracle.build(ref=True)
    if not oracle.ref_available():
        raise SystemExit("reference library not available; run where the reference sources are")
    for name, case in cases().items():
        S = oracle.OracleSpace("ref")
        load(S, case)
        out = run_fields(S, case)
        S.close()
        out.update(case_arrays(case))
        np.savez_compressed(os.path.join(HERE, f"field_{name}.npz"), **out)
        print(name, {k: float(np.abs(v).max()) for k, v in out.items() if k.startswith(("vel", "psi", "omega"))
                     and v.ndim == 2})


if __name__ == "__main__":
    main()
