"""Regenerate the golden fixtures of tests/golden/ (run from the repository root:
``python tests/golden/make_golden.py``).

The reference ships no golden vectors for this path, so these fixtures pin
the CPU oracle to the independent numpy restatement of tests/pyref.py on two
small seeded cases: the halo-filled state and the advection RHS of every
component.  The state is regenerated from the seeded generators and checked
against the stored copy, so a change of the generators shows up too.
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from tests import cases, pyref  # noqa: E402

FIXTURES = ["bubble_12x10x8", "hill_odd_13x7x9_reverse"]


def build(name):
    geo, vel, st = cases.get(name)
    g = geo.grid
    c = st.c.copy()
    # periodic halo fill (ExchangeCell) in numpy
    if g.periodic_x:
        c[:, 1:-1, 1:-1, 0] = c[:, 1:-1, 1:-1, g.nx]
        c[:, 1:-1, 1:-1, g.nx + 1] = c[:, 1:-1, 1:-1, 1]
    if g.periodic_y:
        c[:, 1:-1, 0, 1:-1] = c[:, 1:-1, g.ny, 1:-1]
        c[:, 1:-1, g.ny + 1, 1:-1] = c[:, 1:-1, 1, 1:-1]
    f = pyref.fcn(geo, c, vel)
    return {"c": c, "fcn": f}


if __name__ == "__main__":
    out = Path(__file__).resolve().parent
    for name in FIXTURES:
        data = build(name)
        np.savez_compressed(out / f"{name}.npz", **data)
        print(name, {k: v.shape for k, v in data.items()})
