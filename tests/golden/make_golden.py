"""Generate tests/golden/*.npz from the reference's own kernels (oracle/_ref).

Run in a checkout next to the reference tree (oracle/build_ref.py compiles its OpenCL C
kernels for the host). For every case in cases.py the reference kernels are driven like
Simulation.timeStep (Simulation.py:232-237) and the final positions, velocities, recorded
force curve and (viscoplastic) plastic state are stored. The GPU machine has no reference tree;
tests there compare against these files.

    python tests/golden/make_golden.py [reference_root] [case ...]

The reference root defaults to $NFX_REFERENCE_ROOT or the recipe's default (oracle/build_ref.py).
"""

from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402
from oracle import build_ref  # noqa: E402
from tests.golden.cases import CASES  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref_root: str | None = None, names=None) -> None:
    if build_ref.build(ref_root) is None:
        raise SystemExit("reference tree not found")
    for name, case in CASES.items():
        if names and name not in names:
            continue
        st = O.State(case.problem(), "f64")
        curve = O.ref_run(st, case.steps, case.workload.record_every)
        out = dict(points=st.positions(), velocities=st.velocities(), curve=curve, steps=case.steps)
        if case.problem().model == O.MODEL_VP:
            out.update(Fp=st.Fp.copy(), acc=st.acc.copy(), vonMises=st.vonMises.copy(), pressure=st.pressure.copy())
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
        print(f"{name}: {len(curve)} rows, final force {curve[-1, 2]:.6e}")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None, sys.argv[2:])
