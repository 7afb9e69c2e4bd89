"""Block-tridiagonal column solve of TriDiagTB (MULTI/TriDiagTB_Mod.f90:121-163)
in the oracle: against a dense numpy solve of the assembled block matrix, the
product and the solve inverse to each other, one-level columns.  Host only."""
import numpy as np
import pytest

import oracle


def tb_case(ncol, n1, seed=0, dominance=4.0):
    """Diagonally dominant 2x2-block columns shaped like the assembled
    TriDiagTB blocks (density row coupled to the buoyancy column)."""
    r = np.random.default_rng(seed)
    d = r.uniform(-1, 1, (ncol, n1, 4))
    d[:, :, 0] = np.abs(d[:, :, 0]) + dominance
    d[:, :, 3] = np.abs(d[:, :, 3]) + dominance
    u = r.uniform(-1, 1, (ncol, max(n1 - 1, 0), 4))
    l = r.uniform(-1, 1, (ncol, max(n1 - 1, 0), 4))
    b = r.standard_normal((ncol, n1, 2))
    return d, u, l, b


def dense(d, u, l):
    n1 = d.shape[0]
    A = np.zeros((2 * n1, 2 * n1))
    blk = lambda v: v.reshape(2, 2, order="F")  # noqa: E731
    for i in range(n1):
        A[2 * i:2 * i + 2, 2 * i:2 * i + 2] = blk(d[i])
        if i + 1 < n1:
            A[2 * i:2 * i + 2, 2 * i + 2:2 * i + 4] = blk(u[i])
            A[2 * i + 2:2 * i + 4, 2 * i:2 * i + 2] = blk(l[i])
    return A


@pytest.mark.parametrize("ncol,n1", [(5, 12), (3, 1), (4, 2), (2, 64)])
def test_oracle_block_thomas_against_dense(built_oracle, ncol, n1):
    d, u, l, b = tb_case(ncol, n1, seed=n1)
    x = oracle.tri_tb_solve(d, u, l, b)
    y = oracle.tri_tb_matvec(d, u, l, x)
    for c in range(ncol):
        A = dense(d[c], u[c], l[c])
        np.testing.assert_allclose(x[c].ravel(), np.linalg.solve(A, b[c].ravel()), rtol=1e-12, atol=1e-13)
        np.testing.assert_allclose(y[c].ravel(), A @ x[c].ravel(), rtol=1e-12, atol=1e-13)
    np.testing.assert_allclose(y, b, rtol=1e-11, atol=1e-12)


def test_oracle_diagonal_blocks_decouple(built_oracle):
    # u = l = 0: every level is its own 2x2 solve by the adjugate (Div_2)
    d, u, l, b = tb_case(2, 6, seed=3)
    u[:] = 0.0
    l[:] = 0.0
    x = oracle.tri_tb_solve(d, u, l, b)
    det = d[..., 0] * d[..., 3] - d[..., 2] * d[..., 1]
    x1 = (d[..., 3] * b[..., 0] - d[..., 2] * b[..., 1]) / det
    x2 = (-d[..., 1] * b[..., 0] + d[..., 0] * b[..., 1]) / det
    assert np.array_equal(x[..., 0], x1) and np.array_equal(x[..., 1], x2)
