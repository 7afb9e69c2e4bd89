"""The CPU oracle reproduces the committed golden fixtures bit for bit
(fixtures written by tests/golden/make_golden.py from the independent numpy
restatement; the reference itself has no golden vectors for this path)."""
from pathlib import Path

import numpy as np
import pytest

from tests import cases

GOLDEN = Path(__file__).resolve().parent / "golden"
NAMES = ["bubble_12x10x8", "hill_odd_13x7x9_reverse"]


@pytest.mark.parametrize("name", NAMES)
def test_oracle_reproduces_golden_flux(built_oracle, name):
    import oracle

    data = np.load(GOLDEN / f"{name}.npz")
    geo, vel, st = cases.get(name)
    o = oracle.Oracle(geo)
    c = o.exchange_cell(st.c)
    assert np.array_equal(c, data["c"])
    assert np.array_equal(o.fcn(c, vel), data["fcn"])


def test_oracle_reproduces_golden_laplacian(built_oracle):
    """Level-0 pressure Laplacian of the projection oracle (LaplTFullCompute)
    against the fixture written from the numpy restatement."""
    import oracle

    name = "proj_hill_odd_13x7x9"
    data = np.load(GOLDEN / f"{name}.npz")
    geo = cases.get(name)
    W, dx, dy, dz, _ = cases.proj_inputs(geo)
    assert np.array_equal(W[6], data["dut"])
    o = oracle.OracleProj(geo, dx, dy, dz, W)
    o.lapl_compute(0.435866521508459, 2.0)
    for which, key in enumerate(["d", "uz", "lz", "ux", "lx", "u3", "l3"]):
        assert np.array_equal(o.lapl_get(0, 0, which), data[key]), key
