"""Regenerate the golden fixtures of tests/golden/ (run from the repository root:
``python tests/golden/make_golden.py``).

The reference ships no golden vectors for this path, so these fixtures pin
the CPU oracle to the independent numpy restatement of tests/pyref.py on two
small seeded cases: the halo-filled state and the advection RHS of every
component; and the pressure projection's oracle to the numpy restatement of
the level-0 Laplacian on a closed cut-cell block.  The state is regenerated from the seeded generators and checked
against the stored copy, so a change of the generators shows up too.
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from tests import cases, pyref  # noqa: E402

FIXTURES = ["bubble_12x10x8", "hill_odd_13x7x9_reverse"]
PROJ_FIXTURE = "proj_hill_odd_13x7x9"
PROJ_BETA0, PROJ_DTP = 0.435866521508459, 2.0


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


def build_proj(name):
    """Level-0 pressure Laplacian of a closed block from the numpy restatement
    (its seeded sound weights regenerated and stored too)."""
    geo = cases.get(name)
    W, dx, dy, dz, _ = cases.proj_inputs(geo)
    arrs = pyref.lapl_level0(geo, W, dx, dy, dz, PROJ_BETA0, PROJ_DTP)
    keys = ["d", "uz", "lz", "ux", "lx", "u3", "l3"]
    data = dict(zip(keys, arrs))
    data["dut"] = W[6]
    return data


if __name__ == "__main__":
    out = Path(__file__).resolve().parent
    for name in FIXTURES:
        data = build(name)
        np.savez_compressed(out / f"{name}.npz", **data)
        print(name, {k: v.shape for k, v in data.items()})
    data = build_proj(PROJ_FIXTURE)
    np.savez_compressed(out / f"{PROJ_FIXTURE}.npz", **data)
    print(PROJ_FIXTURE, {k: v.shape for k, v in data.items()})
