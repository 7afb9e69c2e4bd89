"""GPU parity of the TriDiagTB block-Thomas column solve and its product
(MULTI/TriDiagTB_Mod.f90:121-163) with the oracle: bit-exact on every shape,
including one- and two-level columns and a batch of 32768 columns of 128
levels (the columns of a 256x128 plane stack of the 512x512x128 grid)."""
import numpy as np
import pytest

import asam_gb300 as asam
import oracle
from tests.test_tritb import tb_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("ncol,n1", [(7, 12), (3, 1), (5, 2), (130, 64), (32768, 128)])
def test_tri_tb_solve_and_matvec_bitwise(built_lib, ncol, n1):
    d, u, l, b = tb_case(ncol, n1, seed=ncol + n1)
    x = asam.Solve_TB_1D(d, u, l, b)
    xr = oracle.tri_tb_solve(d, u, l, b)
    assert np.array_equal(x, xr)
    y = asam.MatVecTB_1D(d, u, l, x)
    assert np.array_equal(y, oracle.tri_tb_matvec(d, u, l, x))
    np.testing.assert_allclose(y, b, rtol=1e-10, atol=1e-11)


def test_tri_tb_bad_args(built_lib):
    from asam_gb300 import _lib

    lib = _lib.load()
    assert lib.asam_tri_tb_solve(0, 4, None, None, None, None) == 4
    assert lib.asam_tri_tb_matvec(2, 3, None, None, None, None, None) == 4
