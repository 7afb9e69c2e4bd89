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
