"""Generates the move_and_clean and forces fixtures (move_*.npz, forces_*.npz) in this folder
from the reference.

Run where the reference sources are present (compiled unmodified by ``make -C oracle
ref``).  A move fixture holds the reference's outputs of MFlowmove::move_and_clean
(libvvhd/src/MFlowmove.cpp:11-215) for one case of tests/move_cases.py, with and without
removal inside bodies; a forces fixture those of Space::calc_forces / zero_forces
(libvvhd/src/TSpace.cpp:94-142).

    python tests/golden/make_golden_move.py
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
from move_cases import cases, forces_cases, run_forces, run_move  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    oracle.build(ref=True)
    if not oracle.ref_available():
        raise SystemExit("reference library not available; run where the reference sources are")
    for name, case in cases().items():
        out = {}
        for remove in (True, False):
            S = oracle.OracleSpace("ref")
            res = run_move(S, case, remove, oracle.default_body_params)
            S.close()
            out.update({("rm_" if remove else "keep_") + k: v for k, v in res.items()})
        np.savez_compressed(os.path.join(HERE, f"move_{name}.npz"), **out)
        print(name, "removed", int(out["rm_cleaned"]), "left", len(out["rm_x"]))
    for name, case in forces_cases().items():
        S = oracle.OracleSpace("ref")
        out = run_forces(S, case, oracle.default_body_params)
        S.close()
        np.savez_compressed(os.path.join(HERE, f"forces_{name}.npz"), **out)
        print("forces", name, out["f1"][0])


if __name__ == "__main__":
    main()
