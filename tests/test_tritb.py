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


def compute_inputs(ncol, n1, seed):
    r = np.random.default_rng(seed)
    faces = [r.uniform(0.2, 2.0, (ncol, n1 + 1)) for _ in range(4)]  # F, FG, DTU, DUU
    vol = r.uniform(0.5, 3.0, (ncol, n1))
    dut = r.uniform(0.1, 1.5, (ncol, n1))
    dur = r.uniform(-0.5, 0.5, (ncol, n1))
    coefs = dict(beta0_dtp=r.uniform(0.3, 3.0), fac1_l=2.0, fac1_r=1.0, grav_comp=9.81, fac_anela=0.25)
    return faces, vol, dut, dur, coefs


def numpy_compute(faces, vol, dut, dur, beta0_dtp, fac1_l, fac1_r, grav_comp, fac_anela):
    """Compute_1D restated with numpy, element by element in the order the
    reference's statements touch each entry: the first face's terms, the
    entry's share of face i (as the upper cell of that face), of face i+1 (as
    the lower cell), the last face's terms, the FacAnela/Vol diagonal."""
    F, FG, DTU, DUU = faces
    ncol, n1 = vol.shape
    tr = dur is not None
    bd2 = beta0_dtp * beta0_dtp
    eps, half = 1e-30, 0.5
    d = np.zeros((ncol, n1, 4))
    d[:, :, 0] = 1e-40
    d[:, :, 3] = 1e-40
    u = np.zeros((ncol, max(n1 - 1, 0), 4))
    l = np.zeros_like(u)
    V = vol
    # first face (column index 0 of the faces), first cell
    d[:, 0, 0] = d[:, 0, 0] + bd2 * fac1_l * F[:, 0] * DTU[:, 0] * DUU[:, 0] * FG[:, 0] * dut[:, 0] / (V[:, 0] + eps)
    if tr:
        d[:, 0, 2] = d[:, 0, 2] + bd2 * fac1_l * F[:, 0] * DTU[:, 0] * DUU[:, 0] * FG[:, 0] * dur[:, 0] / (V[:, 0] + eps)
    d[:, 0, 1] = d[:, 0, 1] + bd2 * fac1_l * F[:, 0] * DUU[:, 0] * FG[:, 0] * dut[:, 0] / (V[:, 0] + eps)
    if tr:
        d[:, 0, 3] = d[:, 0, 3] + bd2 * fac1_l * F[:, 0] * DUU[:, 0] * FG[:, 0] * dur[:, 0] / (V[:, 0] + eps)
    d[:, 0, 2] = d[:, 0, 2] - half * grav_comp * bd2 * fac1_l * F[:, 0] * DTU[:, 0] * V[:, 0] / (V[:, 0] + eps)
    d[:, 0, 3] = d[:, 0, 3] - half * grav_comp * bd2 * fac1_l * F[:, 0] * V[:, 0] / (V[:, 0] + eps)
    for i in range(n1 - 1):  # face i+1 between cells i and i+1, in the reference's loop order
        q = i + 1
        S = V[:, i] + V[:, q] + eps
        a = bd2 * 2.0 * F[:, q] * DTU[:, q] * DUU[:, q] * FG[:, q]
        b = bd2 * 2.0 * F[:, q] * DUU[:, q] * FG[:, q]
        u[:, i, 0] = -(a * dut[:, q] / S)
        u[:, i, 1] = -(b * dut[:, q] / S)
        l[:, i, 0] = -(a * dut[:, i] / S)
        l[:, i, 1] = -(b * dut[:, i] / S)
        if tr:
            u[:, i, 2] = -(a * dur[:, q] / S)
            u[:, i, 3] = -(b * dur[:, q] / S)
            l[:, i, 2] = -(a * dur[:, i] / S)
            l[:, i, 3] = -(b * dur[:, i] / S)
        g = grav_comp * bd2 * F[:, q]
        u[:, i, 2] = u[:, i, 2] - g * DTU[:, q] * V[:, q] / S
        u[:, i, 3] = u[:, i, 3] - g * V[:, q] / S
        l[:, i, 2] = l[:, i, 2] + g * DTU[:, q] * V[:, i] / S
        l[:, i, 3] = l[:, i, 3] + g * V[:, i] / S
        for c, src in ((i, i), (q, q)):
            d[:, c, 0] = d[:, c, 0] + a * dut[:, src] / S
            d[:, c, 1] = d[:, c, 1] + b * dut[:, src] / S
            if tr:
                d[:, c, 2] = d[:, c, 2] + a * dur[:, src] / S
                d[:, c, 3] = d[:, c, 3] + b * dur[:, src] / S
        d[:, i, 2] = d[:, i, 2] - g * DTU[:, q] * V[:, i] / S
        d[:, i, 3] = d[:, i, 3] - g * V[:, i] / S
        d[:, q, 2] = d[:, q, 2] + g * DTU[:, q] * V[:, q] / S
        d[:, q, 3] = d[:, q, 3] + g * V[:, q] / S
    c, q = n1 - 1, n1
    d[:, c, 0] = d[:, c, 0] + bd2 * fac1_r * F[:, q] * DTU[:, q] * DUU[:, q] * FG[:, q] * dut[:, c] / (V[:, c] + eps)
    if tr:
        d[:, c, 2] = d[:, c, 2] + bd2 * fac1_r * F[:, q] * DTU[:, q] * DUU[:, q] * FG[:, q] * dur[:, c] / (V[:, c] + eps)
    d[:, c, 1] = d[:, c, 1] + bd2 * fac1_r * F[:, q] * DUU[:, q] * FG[:, q] * dut[:, c] / (V[:, c] + eps)
    if tr:
        d[:, c, 3] = d[:, c, 3] + bd2 * fac1_r * F[:, q] * DUU[:, q] * FG[:, q] * dur[:, c] / (V[:, c] + eps)
    d[:, c, 2] = d[:, c, 2] + half * grav_comp * bd2 * fac1_r * F[:, q] * DTU[:, q] * V[:, c] / (V[:, c] + eps)
    d[:, c, 3] = d[:, c, 3] + half * grav_comp * bd2 * fac1_r * F[:, q] * V[:, c] / (V[:, c] + eps)
    d[:, :, 0] = d[:, :, 0] + fac_anela * V
    d[:, :, 3] = d[:, :, 3] + V
    return d, u, l


@pytest.mark.parametrize("variant", ["TB", "TR"])
@pytest.mark.parametrize("ncol,n1", [(4, 1), (3, 2), (5, 9), (2, 40)])
def test_oracle_compute_matches_numpy(built_oracle, variant, ncol, n1):
    """Compute_1D (MULTI/TriDiagTB_Mod.f90:32-93, TriDiagTR_Mod.f90:32-105):
    the oracle equals the numpy restatement bit for bit."""
    faces, vol, dut, dur, coefs = compute_inputs(ncol, n1, seed=n1 + (variant == "TR"))
    dr = dur if variant == "TR" else None
    got = oracle.tri_tb_compute(*faces[:2], vol, faces[2], faces[3], dut, dr, **coefs)
    ref = numpy_compute(faces, vol, dut, dr, **coefs)
    for g, r in zip(got, ref):
        assert np.array_equal(g, r)


def test_oracle_compute_known_answer(built_oracle):
    """One cell, no gravity, FacAnela 0: d(1,1) = 1e-40 + the two faces'
    terms + 0, d(2,2) = 1e-40 + Vol, the other entries 0; the (1,1) block of
    two cells without boundary faces has the row sums of a difference operator."""
    F, FG, DTU, DUU = (np.array([[2.0, 3.0]]) for _ in range(4))
    vol, dut = np.array([[4.0]]), np.array([[0.5]])
    d, u, l = oracle.tri_tb_compute(F, FG, vol, DTU, DUU, dut, beta0_dtp=1.0, fac1_l=1.0, fac1_r=1.0)
    assert d[0, 0, 0] == 1e-40 + 2.0 * 2.0 * 2.0 * 2.0 * 0.5 / (4.0 + 1e-30) + 3.0 * 3.0 * 3.0 * 3.0 * 0.5 / (4.0 + 1e-30)
    # d(2,1): the same terms without DTU
    assert d[0, 0, 1] == 0.0 + 2.0 * 2.0 * 2.0 * 0.5 / (4.0 + 1e-30) + 3.0 * 3.0 * 3.0 * 0.5 / (4.0 + 1e-30)
    assert d[0, 0, 3] == 1e-40 + 4.0 and d[0, 0, 2] == 0.0
    ones = [np.ones((1, 3)) for _ in range(4)]
    d, u, l = oracle.tri_tb_compute(*ones[:2], np.ones((1, 2)), *ones[2:], np.ones((1, 2)))
    # (1,1) entries: face between the cells only; d = 1e-40 + 2/(2+eps) each, u = l = -2/(2+eps)
    assert d[0, :, 0].tolist() == [1e-40 + 1.0, 1e-40 + 1.0] and u[0, 0, 0] == -1.0 and l[0, 0, 0] == -1.0


def compute_inputs_2d(nplane, n2, n1, seed):
    r = np.random.default_rng(seed)
    zf = [r.uniform(0.2, 2.0, (nplane, n2, n1 + 1)) for _ in range(4)]  # F1, F1G, DTU1, DUU1
    xf = [r.uniform(0.2, 2.0, (nplane, n2 + 1, n1)) for _ in range(4)]  # F2, F2G, DTU2, DUU2
    vol = r.uniform(0.5, 3.0, (nplane, n2, n1))
    dut = r.uniform(0.1, 1.5, (nplane, n2, n1))
    dur = r.uniform(-0.5, 0.5, (nplane, n2, n1))
    coefs = dict(beta0_dtp=r.uniform(0.3, 3.0), fac1_l=2.0, fac1_r=1.0, grav_comp=9.81, fac_anela=0.25, fac2_l=1.0,
                 fac2_r=2.0)
    return zf, xf, vol, dut, dur, coefs


def numpy_compute_2d(zf, xf, vol, dut, dur, fac2_l, fac2_r, **c1):
    """Compute_2D restated: every line's Compute_1D (numpy_compute over all
    lines as columns), then the faces between lines in the order the
    reference adds them to an entry -- Fac2_L on the first line, the face to
    the line before, the face to the line after, Fac2_R on the last line."""
    nplane, n2, n1 = vol.shape
    tr = dur is not None
    flat = lambda a: a.reshape(nplane * n2, -1)  # noqa: E731
    d, u1, l1 = numpy_compute([flat(a) for a in zf], flat(vol), flat(dut), flat(dur) if tr else None, **c1)
    d = d.reshape(nplane, n2, n1, 4)
    u1 = u1.reshape(nplane, n2, n1 - 1, 4)
    l1 = l1.reshape(nplane, n2, n1 - 1, 4)
    F2, F2G, DTU2, DUU2 = xf
    bd2 = c1["beta0_dtp"] * c1["beta0_dtp"]
    eps = 1e-30
    u2 = np.zeros((nplane, n2 - 1, n1, 4))
    l2 = np.zeros_like(u2)

    def add(jc, jf, fac, den):
        a = bd2 * fac * F2[:, jf] * DTU2[:, jf] * DUU2[:, jf] * F2G[:, jf]
        b = bd2 * fac * F2[:, jf] * DUU2[:, jf] * F2G[:, jf]
        d[:, jc, :, 0] = d[:, jc, :, 0] + a * dut[:, jc] / den
        if tr:
            d[:, jc, :, 2] = d[:, jc, :, 2] + a * dur[:, jc] / den
        d[:, jc, :, 1] = d[:, jc, :, 1] + b * dut[:, jc] / den
        if tr:
            d[:, jc, :, 3] = d[:, jc, :, 3] + b * dur[:, jc] / den

    add(0, 0, fac2_l, vol[:, 0] + eps)
    for j in range(1, n2):  # face j, line j as the upper one
        add(j, j, 2.0, vol[:, j - 1] + vol[:, j] + eps)
    for j in range(n2 - 1):  # face j+1, line j as the lower one, and the couplings
        q = j + 1
        S = vol[:, j] + vol[:, q] + eps
        a = bd2 * 2.0 * F2[:, q] * DTU2[:, q] * DUU2[:, q] * F2G[:, q]
        b = bd2 * 2.0 * F2[:, q] * DUU2[:, q] * F2G[:, q]
        u2[:, j, :, 0], u2[:, j, :, 1] = -(a * dut[:, q] / S), -(b * dut[:, q] / S)
        l2[:, j, :, 0], l2[:, j, :, 1] = -(a * dut[:, j] / S), -(b * dut[:, j] / S)
        if tr:
            u2[:, j, :, 2], u2[:, j, :, 3] = -(a * dur[:, q] / S), -(b * dur[:, q] / S)
            l2[:, j, :, 2], l2[:, j, :, 3] = -(a * dur[:, j] / S), -(b * dur[:, j] / S)
        add(j, q, 2.0, S)
    add(n2 - 1, n2, fac2_r, vol[:, n2 - 1] + eps)
    return d, u1, l1, u2, l2


@pytest.mark.parametrize("variant", ["TB", "TR"])
@pytest.mark.parametrize("nplane,n2,n1", [(1, 1, 1), (2, 3, 4), (3, 1, 5), (2, 5, 1), (2, 6, 9)])
def test_oracle_compute_2d_matches_numpy(built_oracle, variant, nplane, n2, n1):
    """Compute_2D (MULTI/TriDiagTB_Mod.f90:260-343, TriDiagTR_Mod.f90:273-387):
    the oracle's line-by-line sweep equals the numpy restatement bit for bit;
    one line per plane without Fac2 terms is Compute_1D of that line."""
    zf, xf, vol, dut, dur, coefs = compute_inputs_2d(nplane, n2, n1, seed=7 * n2 + n1)
    dr = dur if variant == "TR" else None
    got = oracle.tri_tb_compute_2d(zf, xf, vol, dut, dr, **coefs)
    ref = numpy_compute_2d(zf, xf, vol, dut, dr, **coefs)
    for g, r in zip(got, ref):
        assert np.array_equal(g, r)
    if n2 == 1:
        c1 = {k: v for k, v in coefs.items() if k not in ("fac2_l", "fac2_r")}
        one = oracle.tri_tb_compute_2d(zf, xf, vol, dut, dr, **c1)
        line = oracle.tri_tb_compute(*[a[:, 0] for a in zf[:2]], vol[:, 0], *[a[:, 0] for a in zf[2:]], dut[:, 0],
                                     None if dr is None else dr[:, 0], **c1)
        assert np.array_equal(one[0][:, 0], line[0]) and np.array_equal(one[1][:, 0], line[1])


def test_oracle_compute_2d_uniform(built_oracle):
    """All faces, weights and volumes 1, no boundary faces, no gravity: every
    face between two cells adds 2/(2+eps) = 1 to both cells' (1,1) entry, so
    the (1,1) diagonal counts each cell's neighbours."""
    nplane, n2, n1 = 1, 3, 4
    zf = [np.ones((nplane, n2, n1 + 1)) for _ in range(4)]
    xf = [np.ones((nplane, n2 + 1, n1)) for _ in range(4)]
    d, u1, l1, u2, l2 = oracle.tri_tb_compute_2d(zf, xf, np.ones((nplane, n2, n1)), np.ones((nplane, n2, n1)))
    nb = np.zeros((n2, n1))
    nb[:, :-1] += 1
    nb[:, 1:] += 1
    nb[:-1, :] += 1
    nb[1:, :] += 1
    assert np.array_equal(d[0, :, :, 0], 1e-40 + nb)
    assert (u1[..., 0] == -1.0).all() and (u2[..., 0] == -1.0).all() and (l2[..., 2] == 0.0).all()


def compute_inputs_3d(n3, n2, n1, seed):
    zf, xf, vol, dut, dur, coefs = compute_inputs_2d(n3, n2, n1, seed)
    r = np.random.default_rng(seed + 1000)
    yf = [r.uniform(0.2, 2.0, (n3 + 1, n2, n1)) for _ in range(4)]  # F3, F3G, DTU3, DUU3
    coefs.update(fac3_l=2.0, fac3_r=0.5)
    return zf, xf, yf, vol, dut, dur, coefs


def numpy_compute_3d(zf, xf, yf, vol, dut, dur, couple, fac3_l, fac3_r, **c2):
    """Compute_3D restated: every plane's Compute_2D (numpy_compute_2d with the
    planes as the batch), then the faces between planes in the order the
    reference adds them to an entry, DUU3 in the face terms as the branch
    has it (always in Fac3_L)."""
    n3, n2, n1 = vol.shape
    tr = dur is not None
    d, u1, l1, u2, l2 = numpy_compute_2d(zf, xf, vol, dut, dur, **c2)
    F3, F3G, DTU3, DUU3 = yf
    bd2 = c2["beta0_dtp"] * c2["beta0_dtp"]
    eps = 1e-30
    u3 = np.zeros((n3 - 1, n2, n1, 4))
    l3 = np.zeros_like(u3)

    def w(fac, q, duu):
        if duu:
            return (bd2 * fac * F3[q] * DTU3[q] * DUU3[q] * F3G[q], bd2 * fac * F3[q] * DUU3[q] * F3G[q])
        return bd2 * fac * F3[q] * DTU3[q] * F3G[q], bd2 * fac * F3[q] * F3G[q]

    def add(k, ab, den):
        a, b = ab
        d[k, :, :, 0] = d[k, :, :, 0] + a * dut[k] / den
        if tr:
            d[k, :, :, 2] = d[k, :, :, 2] + a * dur[k] / den
        d[k, :, :, 1] = d[k, :, :, 1] + b * dut[k] / den
        if tr:
            d[k, :, :, 3] = d[k, :, :, 3] + b * dur[k] / den

    inner = not couple
    add(0, w(fac3_l, 0, True), vol[0] + eps)
    for k in range(1, n3):
        add(k, w(2.0, k, inner), vol[k - 1] + vol[k] + eps)
    for k in range(n3 - 1):
        q = k + 1
        S = vol[k] + vol[q] + eps
        a, b = w(2.0, q, inner)
        if couple:
            u3[k, :, :, 0], u3[k, :, :, 1] = -(a * dut[q] / S), -(b * dut[q] / S)
            l3[k, :, :, 0], l3[k, :, :, 1] = -(a * dut[k] / S), -(b * dut[k] / S)
            if tr:
                u3[k, :, :, 2], u3[k, :, :, 3] = -(a * dur[q] / S), -(b * dur[q] / S)
                l3[k, :, :, 2], l3[k, :, :, 3] = -(a * dur[k] / S), -(b * dur[k] / S)
        add(k, (a, b), S)
    add(n3 - 1, w(fac3_r, n3, inner), vol[n3 - 1] + eps)
    return d, u1, l1, u2, l2, u3, l3


@pytest.mark.parametrize("couple", [True, False])
@pytest.mark.parametrize("variant", ["TB", "TR"])
@pytest.mark.parametrize("n3,n2,n1", [(1, 1, 1), (2, 3, 4), (4, 1, 3), (3, 2, 1), (5, 4, 6)])
def test_oracle_compute_3d_matches_numpy(built_oracle, couple, variant, n3, n2, n1):
    """Compute_3D (MULTI/TriDiagTB_Mod.f90:663-780, TriDiagTR_Mod.f90:707-864),
    both of the reference's branches: the oracle's plane-by-plane sweep
    equals the numpy restatement bit for bit; one plane without Fac3 terms
    is Compute_2D of that plane."""
    zf, xf, yf, vol, dut, dur, coefs = compute_inputs_3d(n3, n2, n1, seed=11 * n3 + 3 * n2 + n1)
    dr = dur if variant == "TR" else None
    got = oracle.tri_tb_compute_3d(zf, xf, yf, vol, dut, dr, couple=couple, **coefs)
    ref = numpy_compute_3d(zf, xf, yf, vol, dut, dr, couple, **coefs)
    for g, r in zip(got, ref):
        assert np.array_equal(g, r)
    if n3 == 1:
        c2 = {k: v for k, v in coefs.items() if k not in ("fac3_l", "fac3_r")}
        one = oracle.tri_tb_compute_3d(zf, xf, yf, vol, dut, dr, couple=couple, **c2)
        plane = oracle.tri_tb_compute_2d(zf, xf, vol, dut, dr, **c2)
        assert np.array_equal(one[0], plane[0])


def test_oracle_compute_3d_branches_differ_by_duu3(built_oracle):
    """The two branches agree when DUU3 = 1 and differ otherwise (the
    interior faces and Fac3_R of the branch with couplings leave DUU3 out)."""
    zf, xf, yf, vol, dut, dur, coefs = compute_inputs_3d(3, 2, 4, seed=1)
    a = oracle.tri_tb_compute_3d(zf, xf, yf, vol, dut, couple=True, **coefs)[0]
    b = oracle.tri_tb_compute_3d(zf, xf, yf, vol, dut, couple=False, **coefs)[0]
    assert not np.array_equal(a, b)
    yf[3] = np.ones_like(yf[3])
    a = oracle.tri_tb_compute_3d(zf, xf, yf, vol, dut, couple=True, **coefs)[0]
    b = oracle.tri_tb_compute_3d(zf, xf, yf, vol, dut, couple=False, **coefs)[0]
    assert np.array_equal(a, b)


def dense_level(blocks, tr):
    """The level's operator as a dense matrix: unknown (i, j, k, r) at
    ((k*n2 + j)*n1 + i)*2 + r; TriDiagTB's couplings between lines and
    planes act on the neighbour's first component only."""
    d, u1, l1, u2, l2, u3, l3 = blocks
    n3, n2, n1 = d.shape[:3]
    N = 2 * n1 * n2 * n3
    A = np.zeros((N, N))
    idx = lambda i, j, k: ((k * n2 + j) * n1 + i) * 2  # noqa: E731
    blk = lambda v: v.reshape(2, 2, order="F")  # noqa: E731
    cpl = lambda v: blk(v) if tr else np.array([[v[0], 0.0], [v[1], 0.0]])  # noqa: E731
    for k in range(n3):
        for j in range(n2):
            for i in range(n1):
                a = idx(i, j, k)
                A[a:a + 2, a:a + 2] = blk(d[k, j, i])
                if i + 1 < n1:
                    A[a:a + 2, idx(i + 1, j, k):idx(i + 1, j, k) + 2] = blk(u1[k, j, i])
                    A[idx(i + 1, j, k):idx(i + 1, j, k) + 2, a:a + 2] = blk(l1[k, j, i])
                if j + 1 < n2:
                    A[a:a + 2, idx(i, j + 1, k):idx(i, j + 1, k) + 2] = cpl(u2[k, j, i])
                    A[idx(i, j + 1, k):idx(i, j + 1, k) + 2, a:a + 2] = cpl(l2[k, j, i])
                if k + 1 < n3:
                    A[a:a + 2, idx(i, j, k + 1):idx(i, j, k + 1) + 2] = cpl(u3[k, j, i])
                    A[idx(i, j, k + 1):idx(i, j, k + 1) + 2, a:a + 2] = cpl(l3[k, j, i])
    return A


@pytest.mark.parametrize("variant", ["TB", "TR"])
@pytest.mark.parametrize("n3,n2,n1", [(1, 1, 4), (1, 3, 4), (3, 2, 1), (3, 4, 5)])
def test_oracle_level_matvec_against_dense(built_oracle, variant, n3, n2, n1):
    """MatVecTB_2D/3D and MatVecTR_2D/3D (MULTI/TriDiagTB_Mod.f90:345-372,
    782-816; TriDiagTR_Mod.f90:389-416, 866-900) of an assembled level equal
    the dense product of the same operator (1e-13)."""
    zf, xf, yf, vol, dut, dur, coefs = compute_inputs_3d(n3, n2, n1, seed=3 * n3 + n2 + 7 * n1)
    tr = variant == "TR"
    blocks = oracle.tri_tb_compute_3d(zf, xf, yf, vol, dut, dur if tr else None, couple=True, **coefs)
    x = np.random.default_rng(n1).standard_normal((n3, n2, n1, 2))
    y = oracle.tri_tb_matvec_3d(blocks, x, tr)
    ref = (dense_level(blocks, tr) @ x.reshape(-1)).reshape(x.shape)
    assert np.max(np.abs(y - ref)) <= 1e-13 * np.max(np.abs(ref))


def plane_case(nplane, n2, n1, seed, dominance=6.0):
    """Diagonally dominant plane systems in the layout of Compute_2D."""
    r = np.random.default_rng(seed)
    d, u1, l1, _ = tb_case(nplane * n2, n1, seed=seed, dominance=dominance)
    d = d.reshape(nplane, n2, n1, 4)
    u1 = u1.reshape(nplane, n2, n1 - 1, 4)
    l1 = l1.reshape(nplane, n2, n1 - 1, 4)
    u2 = r.uniform(-1, 1, (nplane, n2 - 1, n1, 4))
    l2 = r.uniform(-1, 1, (nplane, n2 - 1, n1, 4))
    b = r.standard_normal((nplane, n2, n1, 2))
    return (d, u1, l1, u2, l2), b


@pytest.mark.parametrize("variant", ["TB", "TR"])
@pytest.mark.parametrize("nplane,n2,n1", [(2, 1, 5), (2, 2, 3), (3, 5, 4), (1, 7, 1)])
def test_oracle_gauss_seidel_2d_converges(built_oracle, variant, nplane, n2, n1):
    """GaussSeidel_2D (MULTI/TriDiagTB_Mod.f90:374-418, TriDiagTR_Mod.f90:418-462):
    the symmetric line sweeps of a diagonally dominant plane converge to the
    dense solution (TriDiagTB's couplings act on the first component only);
    one line is Solve_1D of that line, bit for bit."""
    tr = variant == "TR"
    blocks, b = plane_case(nplane, n2, n1, seed=n2 * 10 + n1)
    x = oracle.tri_tb_gauss_seidel_2d(blocks, b, np.zeros_like(b), 40, tr)
    d, u1, l1, u2, l2 = blocks
    for p in range(nplane):
        lvl = (d[p][None], u1[p][None], l1[p][None], u2[p][None], l2[p][None], np.zeros((0, n2, n1, 4)),
               np.zeros((0, n2, n1, 4)))
        ref = np.linalg.solve(dense_level(lvl, tr), b[p].reshape(-1)).reshape(n2, n1, 2)
        assert np.max(np.abs(x[p] - ref)) <= 1e-11 * np.max(np.abs(ref))
    if n2 == 1:
        for p in range(nplane):
            assert np.array_equal(x[p, 0], oracle.tri_tb_solve(d[p], u1[p], l1[p], b[p])[0])


@pytest.mark.parametrize("n2,n1", [(1, 1), (2, 2), (3, 5), (4, 7), (5, 4)])
def test_oracle_restrict_prolong(built_oracle, n2, n1):
    """RestrictTB_2D / ProlongateTB_2D (MULTI/TriDiagTB_Mod.f90:495-560): the
    coarse entry sums its 2x2 fine cells in the reference's order (an odd
    last line or level alone), the prolongation copies it back."""
    res = np.random.default_rng(n2 + n1).standard_normal((2, n2, n1, 2))
    got = oracle.tri_tb_restrict_2d(res)
    n2c, n1c = (n2 + 1) // 2, (n1 + 1) // 2
    ref = np.zeros((2, n2c, n1c, 2))
    for jc in range(n2c):
        for ic in range(n1c):
            js = [2 * jc] + ([2 * jc + 1] if 2 * jc + 1 < n2 else [])
            is_ = [2 * ic] + ([2 * ic + 1] if 2 * ic + 1 < n1 else [])
            acc = None
            for j in js:  # (i, j), (i+1, j), (i, j+1), (i+1, j+1)
                for i in is_:
                    acc = res[:, j, i] if acc is None else acc + res[:, j, i]
            ref[:, jc, ic] = acc
    assert np.array_equal(got, ref)
    back = oracle.tri_tb_prolong_2d(got, n2, n1)
    for j in range(n2):
        for i in range(n1):
            assert np.array_equal(back[:, j, i], got[:, j // 2, i // 2])


def galerkin_coarse(blocks, tr):
    """The coarse plane R A P of a plane level (P copies a coarse entry to
    its 2x2 fine cells, R sums them): again five blocks, the couplings
    between coarse lines of TriDiagTB acting on the first component only."""
    d, u1, l1, u2, l2 = blocks
    nplane, n2, n1 = d.shape[:3]
    n2c, n1c = (n2 + 1) // 2, (n1 + 1) // 2
    out = (np.zeros((nplane, n2c, n1c, 4)), np.zeros((nplane, n2c, max(n1c - 1, 0), 4)),
           np.zeros((nplane, n2c, max(n1c - 1, 0), 4)), np.zeros((nplane, max(n2c - 1, 0), n1c, 4)),
           np.zeros((nplane, max(n2c - 1, 0), n1c, 4)))
    idx = lambda i, j: (j * n1 + i) * 2  # noqa: E731
    cidx = lambda i, j: (j * n1c + i) * 2  # noqa: E731
    P = np.zeros((n2 * n1 * 2, n2c * n1c * 2))
    for j in range(n2):
        for i in range(n1):
            P[idx(i, j):idx(i, j) + 2, cidx(i // 2, j // 2):cidx(i // 2, j // 2) + 2] = np.eye(2)
    z = np.zeros((0, n2, n1, 4))
    for p in range(nplane):
        A = dense_level((d[p][None], u1[p][None], l1[p][None], u2[p][None], l2[p][None], z, z), tr)
        Ac = P.T @ A @ P
        blk = lambda a, c: Ac[a:a + 2, c:c + 2].reshape(-1, order="F")  # noqa: E731
        for jc in range(n2c):
            for ic in range(n1c):
                a = cidx(ic, jc)
                out[0][p, jc, ic] = blk(a, a)
                if ic + 1 < n1c:
                    out[1][p, jc, ic] = blk(a, cidx(ic + 1, jc))
                    out[2][p, jc, ic] = blk(cidx(ic + 1, jc), a)
                if jc + 1 < n2c:
                    out[3][p, jc, ic] = blk(a, cidx(ic, jc + 1))
                    out[4][p, jc, ic] = blk(cidx(ic, jc + 1), a)
        zc = np.zeros((0, n2c, n1c, 4))
        assert np.allclose(dense_level(tuple(o[p][None] for o in out) + (zc, zc), tr), Ac, atol=1e-12)
    return out


def plane_hierarchy(nplane, n2, n1, seed, tr, dominance=6.0):
    blocks, b = plane_case(nplane, n2, n1, seed, dominance)
    levels = [blocks]
    while levels[-1][0].shape[1] > 1 or levels[-1][0].shape[2] > 1:
        levels.append(galerkin_coarse(levels[-1], tr))
    return levels, b


def compose_multigrid_2d(levels, b, x, gauss_iter2, mult_iter, tr):
    """Multigrid_2D (MULTI/TriDiagTB_Mod.f90:433-494) cycle by cycle from the
    oracle's pinned pieces: the smoother, the level product of each plane, the
    transfers."""
    z = lambda n2, n1: np.zeros((0, n2, n1, 4))  # noqa: E731
    x = x.copy()
    nlev = len(levels)
    for _ in range(mult_iter):
        bl, xl = [b] + [None] * (nlev - 1), [x] + [None] * (nlev - 1)
        gi, lv = 1, 0
        while True:
            xl[lv] = oracle.tri_tb_gauss_seidel_2d(levels[lv], bl[lv], xl[lv], gi, tr)
            gi += gauss_iter2
            if lv + 1 == nlev:
                gi -= gauss_iter2
                break
            d = levels[lv][0]
            n2, n1 = d.shape[1:3]
            ax = np.stack([oracle.tri_tb_matvec_3d(tuple(a[p][None] for a in levels[lv]) + (z(n2, n1), z(n2, n1)),
                                                   xl[lv][p][None], tr)[0] for p in range(d.shape[0])])
            bl[lv + 1] = oracle.tri_tb_restrict_2d(bl[lv] - ax)
            xl[lv + 1] = np.zeros_like(bl[lv + 1])
            lv += 1
        while True:
            xl[lv] = oracle.tri_tb_gauss_seidel_2d(levels[lv], bl[lv], xl[lv], gi, tr)
            gi -= gauss_iter2
            if lv == 0:
                break
            lv -= 1
            n2, n1 = levels[lv][0].shape[1:3]
            xl[lv] = xl[lv] + oracle.tri_tb_prolong_2d(xl[lv + 1], n2, n1)
        x = xl[0]
    return x


@pytest.mark.parametrize("variant", ["TB", "TR"])
@pytest.mark.parametrize("nplane,n2,n1,gi2,cycles", [(2, 8, 8, 1, 2), (1, 7, 5, 2, 3), (3, 1, 9, 1, 1), (2, 6, 1, 0, 2),
                                                      (1, 1, 1, 1, 2)])
def test_oracle_multigrid_2d_composes_pieces(built_oracle, variant, nplane, n2, n1, gi2, cycles):
    """Solve_2D / Multigrid_2D (MULTI/TriDiagTB_Mod.f90:419-494,
    TriDiagTR_Mod.f90:463-538) in the oracle equal, bit for bit, the V-cycle
    composed from the separately pinned smoother, product and transfers: the
    GaussIter counts (1 growing by GaussIter2 per level, the coarsest twice),
    the zero coarse guess and the added correction."""
    tr = variant == "TR"
    levels, b = plane_hierarchy(nplane, n2, n1, seed=n2 * 7 + n1, tr=tr)
    x0 = np.random.default_rng(1).standard_normal(b.shape)
    got = oracle.tri_tb_multigrid_2d(levels, b, x0, gi2, cycles, tr)
    ref = compose_multigrid_2d(levels, b, x0, gi2, cycles, tr)
    assert np.array_equal(got, ref)
    assert np.array_equal(oracle.tri_tb_multigrid_2d(levels, b, x0, gi2, 0, tr), x0)


@pytest.mark.parametrize("variant", ["TB", "TR"])
def test_oracle_multigrid_2d_converges(built_oracle, variant):
    """V-cycles over a Galerkin hierarchy of a weakly dominant plane reach
    the dense solution, the error falling every cycle."""
    tr = variant == "TR"
    n2 = n1 = 16
    levels, b = plane_hierarchy(2, n2, n1, seed=3, tr=tr, dominance=2.5)
    z = np.zeros((0, n2, n1, 4))
    d, u1, l1, u2, l2 = levels[0]
    refs = [np.linalg.solve(dense_level((d[p][None], u1[p][None], l1[p][None], u2[p][None], l2[p][None], z, z), tr),
                            b[p].reshape(-1)).reshape(n2, n1, 2) for p in range(2)]
    ref = np.stack(refs)
    x = np.zeros_like(b)
    errs = []
    for _ in range(12):
        x = oracle.tri_tb_multigrid_2d(levels, b, x, 1, 1, tr)
        errs.append(np.max(np.abs(x - ref)) / np.max(np.abs(ref)))
    assert errs[-1] <= 1e-10, errs
    assert all(e1 < e0 for e0, e1 in zip(errs, errs[1:]) if e0 > 1e-14), errs


def restrict_3d_loops(res):
    """RestrictTB_3D (MULTI/TriDiagTB_Mod.f90:954-1026) as the reference's
    overwriting loops, statement by statement (0-based)."""
    n3, n2, n1 = res.shape[:3]
    n1c, n2c, n3c = (n1 + 1) // 2, (n2 + 1) // 2, (n3 + 1) // 2
    R = lambda i, j, k: res[k, j, i]  # noqa: E731
    out = np.zeros((n3c, n2c, n1c, 2))
    out[n3c - 1, n2c - 1, n1c - 1] = R(n1 - 1, n2 - 1, n3 - 1)
    for ic in range(n1 // 2):
        out[n3c - 1, n2c - 1, ic] = R(2 * ic, n2 - 1, n3 - 1) + R(2 * ic + 1, n2 - 1, n3 - 1)
    for jc in range(n2 // 2):
        j = 2 * jc
        out[n3c - 1, jc, n1c - 1] = R(n1 - 1, j, n3 - 1) + R(n1 - 1, j + 1, n3 - 1)
        for ic in range(n1 // 2):
            i = 2 * ic
            out[n3c - 1, jc, ic] = R(i, j, n3 - 1) + R(i + 1, j, n3 - 1) + R(i, j + 1, n3 - 1) + R(i + 1, j + 1, n3 - 1)
    for kc in range(n3 // 2):
        k = 2 * kc
        out[kc, n2c - 1, n1c - 1] = R(n1 - 1, n2 - 1, k) + R(n1 - 1, n2 - 1, k + 1)
        for ic in range(n1 // 2):
            i = 2 * ic
            out[kc, n2c - 1, ic] = R(i, n2 - 1, k) + R(i + 1, n2 - 1, k) + R(i, n2 - 1, k + 1) + R(i + 1, n2 - 1, k + 1)
        for jc in range(n2 // 2):
            j = 2 * jc
            out[kc, jc, n1c - 1] = R(n1 - 1, j, k) + R(n1 - 1, j + 1, k) + R(n1 - 1, j, k + 1) + R(n1 - 1, j + 1, k + 1)
            for ic in range(n1 // 2):
                i = 2 * ic
                out[kc, jc, ic] = (R(i, j, k) + R(i + 1, j, k) + R(i, j + 1, k) + R(i, j, k + 1) + R(i + 1, j + 1, k)
                                   + R(i + 1, j, k + 1) + R(i, j + 1, k + 1) + R(i + 1, j + 1, k + 1))
    return out


@pytest.mark.parametrize("n3,n2,n1", [(1, 1, 1), (2, 2, 2), (3, 5, 4), (4, 7, 6), (5, 3, 9), (2, 1, 3)])
def test_oracle_restrict_prolong_3d(built_oracle, n3, n2, n1):
    """RestrictTB_3D / ProlongateTB_3D (MULTI/TriDiagTB_Mod.f90:954-1100) bit
    for bit against the reference's overwriting loops; the prolongation
    copies each coarse entry to its fine cells."""
    res = np.random.default_rng(n3 + n2 + n1).standard_normal((n3, n2, n1, 2))
    got = oracle.tri_tb_restrict_3d(res)
    assert np.array_equal(got, restrict_3d_loops(res))
    back = oracle.tri_tb_prolong_3d(got, n3, n2, n1)
    k, j, i = np.meshgrid(np.arange(n3), np.arange(n2), np.arange(n1), indexing="ij")
    assert np.array_equal(back, got[k // 2, j // 2, i // 2])


def couple_sub_np(t, c, x, tr):
    """t - (coupling) x as the oracle forms it: TriDiagTB's vector times the
    neighbour's first component, TriDiagTR's Mult_2 (CG/Matrix_Mod.f90)."""
    if tr:
        v0 = c[..., 0] * x[..., 0] + c[..., 2] * x[..., 1]
        v1 = c[..., 1] * x[..., 0] + c[..., 3] * x[..., 1]
        return np.stack([t[..., 0] - v0, t[..., 1] - v1], axis=-1)
    return np.stack([t[..., 0] - c[..., 0] * x[..., 0], t[..., 1] - c[..., 1] * x[..., 0]], axis=-1)


def plane_levels_of(blocks, tr):
    levels = [tuple(blocks)]
    while levels[-1][0].shape[1] > 1 or levels[-1][0].shape[2] > 1:
        levels.append(galerkin_coarse(levels[-1], tr))
    return levels


def galerkin_coarse_3d(blocks7, tr):
    """R A P of a level (7 blocks), 2x2x2 cells to one: again 7 blocks."""
    n3, n2, n1 = blocks7[0].shape[:3]
    c3, c2, c1 = (n3 + 1) // 2, (n2 + 1) // 2, (n1 + 1) // 2
    idx = lambda i, j, k, a, b: ((k * a + j) * b + i) * 2  # noqa: E731
    P = np.zeros((n3 * n2 * n1 * 2, c3 * c2 * c1 * 2))
    for k in range(n3):
        for j in range(n2):
            for i in range(n1):
                f, c = idx(i, j, k, n2, n1), idx(i // 2, j // 2, k // 2, c2, c1)
                P[f:f + 2, c:c + 2] = np.eye(2)
    Ac = P.T @ dense_level(blocks7, tr) @ P
    blk = lambda a, c: Ac[a:a + 2, c:c + 2].reshape(-1, order="F")  # noqa: E731
    out = [np.zeros((c3, c2, c1, 4)), np.zeros((c3, c2, max(c1 - 1, 0), 4)), np.zeros((c3, c2, max(c1 - 1, 0), 4)),
           np.zeros((c3, max(c2 - 1, 0), c1, 4)), np.zeros((c3, max(c2 - 1, 0), c1, 4)),
           np.zeros((max(c3 - 1, 0), c2, c1, 4)), np.zeros((max(c3 - 1, 0), c2, c1, 4))]
    for k in range(c3):
        for j in range(c2):
            for i in range(c1):
                a = idx(i, j, k, c2, c1)
                out[0][k, j, i] = blk(a, a)
                for ax, (di, dj, dk) in ((1, (1, 0, 0)), (3, (0, 1, 0)), (5, (0, 0, 1))):
                    if i + di < c1 and j + dj < c2 and k + dk < c3:
                        b_ = idx(i + di, j + dj, k + dk, c2, c1)
                        out[ax][k, j, i] = blk(a, b_)
                        out[ax + 1][k, j, i] = blk(b_, a)
    assert np.allclose(dense_level(out, tr), Ac, atol=1e-12)
    return out


def level_hierarchy_3d(n3, n2, n1, seed, tr, dominance=8.0):
    """A random diagonally dominant level and its Galerkin levels down to one
    cell, each as (plane_levels, u3, l3) with Galerkin plane hierarchies."""
    r = np.random.default_rng(seed)
    blocks, _ = plane_case(n3, n2, n1, seed, dominance)
    u3 = r.uniform(-1, 1, (n3 - 1, n2, n1, 4))
    l3 = r.uniform(-1, 1, (n3 - 1, n2, n1, 4))
    b = r.standard_normal((n3, n2, n1, 2))
    b7 = list(blocks) + [u3, l3]
    levels = []
    while True:
        levels.append((plane_levels_of(b7[:5], tr), b7[5], b7[6]))
        if b7[0].shape[:3] == (1, 1, 1):
            return levels, b
        b7 = galerkin_coarse_3d(b7, tr)


def compose_gauss_seidel_3d(level, b, x, iters, gi2, mi2, tr):
    """GaussSeidel_3D (MULTI/TriDiagTB_Mod.f90:818-874) statement by
    statement, each plane solved by the oracle's Solve_2D."""
    planes, u3, l3 = level
    n3 = planes[0][0].shape[0]
    x = x.copy()

    def solve(k, t):
        lv = [tuple(a[k:k + 1] for a in p) for p in planes]
        x[k] = oracle.tri_tb_multigrid_2d(lv, t[None], x[k:k + 1], gi2, mi2, tr)[0]

    if n3 == 1:
        solve(0, b[0])
        return x
    for _ in range(iters):
        t = b[0].copy()
        for k in range(n3 - 1):
            t = couple_sub_np(t, u3[k], x[k + 1], tr)
            solve(k, t)
            t = couple_sub_np(b[k + 1], l3[k], x[k], tr)
        solve(n3 - 1, t)
        t = couple_sub_np(b[n3 - 2], u3[n3 - 2], x[n3 - 1], tr)
        for k in range(n3 - 2, 0, -1):
            t = couple_sub_np(t, l3[k - 1], x[k - 1], tr)
            solve(k, t)
            t = couple_sub_np(b[k - 1], u3[k - 1], x[k], tr)
    solve(0, t)
    t = couple_sub_np(b[n3 - 1], l3[n3 - 2], x[n3 - 2], tr)
    solve(n3 - 1, t)
    return x


@pytest.mark.parametrize("variant", ["TB", "TR"])
@pytest.mark.parametrize("n3,n2,n1,iters", [(1, 3, 4, 1), (2, 2, 3, 1), (4, 3, 5, 2), (3, 1, 1, 3)])
def test_oracle_gauss_seidel_3d_composes(built_oracle, variant, n3, n2, n1, iters):
    """GaussSeidel_3D in the oracle (MULTI/TriDiagTB_Mod.f90:818-874,
    TriDiagTR_Mod.f90:902-961) equals its statement-by-statement composition
    from the pinned Solve_2D bit for bit: the forward and backward plane
    sweeps, then plane 1 and plane n3 once more."""
    tr = variant == "TR"
    levels, b = level_hierarchy_3d(n3, n2, n1, seed=n3 * 13 + n2 + n1, tr=tr)
    x0 = np.random.default_rng(2).standard_normal(b.shape)
    got = oracle.tri_tb_gauss_seidel_3d(levels[0], b, x0, iters, 1, 2, tr)
    assert np.array_equal(got, compose_gauss_seidel_3d(levels[0], b, x0, iters, 1, 2, tr))


@pytest.mark.parametrize("variant", ["TB", "TR"])
def test_oracle_gauss_seidel_3d_converges(built_oracle, variant):
    """Plane sweeps with near-exact plane solves reach the dense solution of
    a diagonally dominant level."""
    tr = variant == "TR"
    levels, b = level_hierarchy_3d(4, 4, 5, seed=5, tr=tr)
    planes, u3, l3 = levels[0]
    ref = np.linalg.solve(dense_level(tuple(planes[0]) + (u3, l3), tr), b.reshape(-1)).reshape(b.shape)
    x = oracle.tri_tb_gauss_seidel_3d(levels[0], b, np.zeros_like(b), 30, 1, 30, tr)
    assert np.max(np.abs(x - ref)) <= 1e-11 * np.max(np.abs(ref))


def compose_multigrid_3d(levels, b, x, gi2, mi2, gi3, mi3, tr):
    """Multigrid_3D (MULTI/TriDiagTB_Mod.f90:876-938) from the oracle's pinned
    smoother, level product and transfers."""
    nlev = len(levels)
    x = x.copy()
    for _ in range(mi3):
        bl, xl = [b] + [None] * (nlev - 1), [x] + [None] * (nlev - 1)
        gi, L = 1, 0
        while True:
            xl[L] = oracle.tri_tb_gauss_seidel_3d(levels[L], bl[L], xl[L], gi, gi2, mi2, tr)
            gi += gi3
            if L + 1 == nlev:
                gi -= gi3
                break
            planes, u3, l3 = levels[L]
            ax = oracle.tri_tb_matvec_3d(tuple(planes[0]) + (u3, l3), xl[L], tr)
            bl[L + 1] = oracle.tri_tb_restrict_3d(bl[L] - ax)
            xl[L + 1] = np.zeros_like(bl[L + 1])
            L += 1
        while True:
            xl[L] = oracle.tri_tb_gauss_seidel_3d(levels[L], bl[L], xl[L], gi, gi2, mi2, tr)
            gi -= gi3
            if L == 0:
                break
            L -= 1
            xl[L] = xl[L] + oracle.tri_tb_prolong_3d(xl[L + 1], *xl[L].shape[:3])
        x = xl[0]
    return x


@pytest.mark.parametrize("variant", ["TB", "TR"])
@pytest.mark.parametrize("n3,n2,n1,gi3,cycles", [(4, 4, 4, 1, 2), (3, 5, 2, 2, 1), (1, 1, 1, 1, 2), (5, 1, 3, 0, 2)])
def test_oracle_multigrid_3d_composes(built_oracle, variant, n3, n2, n1, gi3, cycles):
    """Solve_3D / Multigrid_3D (MULTI/TriDiagTB_Mod.f90:876-952,
    TriDiagTR_Mod.f90:963-1041) in the oracle equal their composition from
    the pinned pieces bit for bit."""
    tr = variant == "TR"
    levels, b = level_hierarchy_3d(n3, n2, n1, seed=n3 + 5 * n2 + 11 * n1, tr=tr)
    x0 = np.random.default_rng(4).standard_normal(b.shape)
    got = oracle.tri_tb_multigrid_3d(levels, b, x0, 1, 1, gi3, cycles, tr)
    assert np.array_equal(got, compose_multigrid_3d(levels, b, x0, 1, 1, gi3, cycles, tr))
    assert np.array_equal(oracle.tri_tb_multigrid_3d(levels, b, x0, 1, 1, gi3, 0, tr), x0)


@pytest.mark.parametrize("variant", ["TB", "TR"])
def test_oracle_multigrid_3d_converges(built_oracle, variant):
    """V-cycles over a Galerkin hierarchy of a weakly dominant 8x8x8 level
    reach the dense solution, the error falling every cycle."""
    tr = variant == "TR"
    levels, b = level_hierarchy_3d(8, 8, 8, seed=9, tr=tr, dominance=4.0)
    planes, u3, l3 = levels[0]
    ref = np.linalg.solve(dense_level(tuple(planes[0]) + (u3, l3), tr), b.reshape(-1)).reshape(b.shape)
    x = np.zeros_like(b)
    errs = []
    for _ in range(8):
        x = oracle.tri_tb_multigrid_3d(levels, b, x, 1, 1, 1, 1, tr)
        errs.append(np.max(np.abs(x - ref)) / np.max(np.abs(ref)))
    assert errs[-1] <= 1e-9, errs
    assert all(e1 < e0 for e0, e1 in zip(errs, errs[1:]) if e0 > 1e-14), errs


LAPL_COEFS = dict(beta0_dtp=0.5, fac1_l=1.0, fac1_r=1.0, grav_comp=1.0, fac_anela=0.25, fac2_l=1.0, fac2_r=1.0,
                  fac3_l=1.0, fac3_r=1.0)


def coarsen_loops(zf, xf, yf, vol, dut, dur, s1, s2, s3):
    """FaceCoarse, CFaceCoarse, VolCoarse, CVolCoarse (MULTI/JacAccGrav_Mod.f90:
    685-891) as the reference's loops over the fine cells, accumulating into
    the coarse arrays (0-based; direction 1 = the arrays' last axis)."""
    eps = 1.0e-30
    n3, n2, n1 = vol.shape
    c1, c2, c3 = (n1 + s1) // (s1 + 1), (n2 + s2) // (s2 + 1), (n3 + s3) // (s3 + 1)
    cc = lambda i, s: (i + 1 + s) // (s + 1) - 1  # noqa: E731  (1-based (i+s)/(s+1), back to 0-based)
    out = []
    for a, (F, FG, DT, DU) in enumerate((zf, xf, yf)):
        shape = [(c3, c2, c1 + 1), (c3, c2 + 1, c1), (c3 + 1, c2, c1)][a]
        Fc, FGc, Tc, Uc = (np.zeros(shape) for _ in range(4))
        if a == 0:
            it = ((ic, min((s1 + 1) * ic, n1), j, k) for ic in range(c1 + 1) for j in range(n2) for k in range(n3))
            for ic, i, j, k in it:
                q, r = (k, j, i), (cc(k, s3), cc(j, s2), ic)
                Fc[r] += F[q]; FGc[r] += FG[q]; Tc[r] += DT[q] * F[q]; Uc[r] += DU[q] * FG[q]  # noqa: E702
        elif a == 1:
            it = ((i, jc, min((s2 + 1) * jc, n2), k) for i in range(n1) for jc in range(c2 + 1) for k in range(n3))
            for i, jc, j, k in it:
                q, r = (k, j, i), (cc(k, s3), jc, cc(i, s1))
                Fc[r] += F[q]; FGc[r] += FG[q]; Tc[r] += DT[q] * F[q]; Uc[r] += DU[q] * FG[q]  # noqa: E702
        else:
            it = ((i, j, kc, min((s3 + 1) * kc, n3)) for i in range(n1) for j in range(n2) for kc in range(c3 + 1))
            for i, j, kc, k in it:
                q, r = (k, j, i), (kc, cc(j, s2), cc(i, s1))
                Fc[r] += F[q]; FGc[r] += FG[q]; Tc[r] += DT[q] * F[q]; Uc[r] += DU[q] * FG[q]  # noqa: E702
        out.append((Fc, FGc, Tc / (Fc + eps), Uc / (FGc + eps)))
    V, TV, RV = np.zeros((c3, c2, c1)), np.zeros((c3, c2, c1)), np.zeros((c3, c2, c1))
    for i in range(n1):
        for j in range(n2):
            for k in range(n3):
                r = (cc(k, s3), cc(j, s2), cc(i, s1))
                V[r] += vol[k, j, i]
                TV[r] += dut[k, j, i] * vol[k, j, i]
                if dur is not None:
                    RV[r] += dur[k, j, i] * vol[k, j, i]
    return out[0], out[1], out[2], V, TV / (V + eps), (RV / (V + eps) if dur is not None else None)


@pytest.mark.parametrize("variant", ["TB", "TR"])
@pytest.mark.parametrize("n3,n2,n1,level3,level2", [(5, 6, 7, 0, 0), (5, 6, 7, 1, 1), (5, 6, 7, 1, 2), (4, 3, 9, 0, 2),
                                                     (3, 3, 3, 2, 2)])
def test_oracle_lapl_level_matches_reference_loops(built_oracle, variant, n3, n2, n1, level3, level2):
    """A level of LaplTBCompute / LaplTRCompute (MULTI/JacAccGrav_Mod.f90:
    1312-1667) is Compute_3D of the finest fields coarsened by the
    reference's loops with shifts 2^level2-1, 2^level2-1, 2^level3-1 -- level
    0 too (shift 0 turns DTU into DTU*F/(F+Eps)) -- bit for bit, with the
    couplings between planes on the level itself and without them on its
    plane levels."""
    tr = variant == "TR"
    zf, xf, yf, vol, dut, dur, coefs = compute_inputs_3d(n3, n2, n1, seed=n3 + n2 + n1 + level2)
    s12, s3 = 2 ** level2 - 1, 2 ** level3 - 1
    z, x, y, V, T, R = coarsen_loops(zf, xf, yf, vol, dut, dur if tr else None, s12, s12, s3)
    got = oracle.tri_tb_lapl_level(zf, xf, yf, vol, dut, dur if tr else None, level3, level2, coefs)
    ref = oracle.tri_tb_compute_3d(z, x, y, V, T, R, couple=level2 == level3, **coefs)
    for g, r in zip(got, ref):
        assert np.array_equal(g, r)


@pytest.mark.parametrize("variant", ["TB", "TR"])
def test_oracle_lapl_hierarchy_vcycle_converges(built_oracle, variant):
    """The V-cycle over the hierarchy LaplTBCompute builds (four levels, the
    plane levels of each) reaches the dense solution of the finest level,
    each cycle faster than a plane sweep of GaussSeidel_3D on that level."""
    tr = variant == "TR"
    zf, xf, yf, vol, dut, dur, _ = compute_inputs_3d(8, 8, 8, seed=1)
    levels = oracle.tri_tb_lapl_compute(zf, xf, yf, vol, dut, dur if tr else None, ref_level=4, **LAPL_COEFS)
    assert [(p[0][0].shape[:3], len(p)) for p, _, _ in levels] == [((8, 8, 8), 4), ((4, 4, 4), 3), ((2, 2, 2), 2),
                                                                  ((1, 1, 1), 1)]
    planes, u3, l3 = levels[0]
    b = np.random.default_rng(0).standard_normal((8, 8, 8, 2))
    ref = np.linalg.solve(dense_level(tuple(planes[0]) + (u3, l3), tr), b.reshape(-1)).reshape(b.shape)
    x, xg = np.zeros_like(b), np.zeros_like(b)
    for _ in range(6):
        x = oracle.tri_tb_multigrid_3d(levels, b, x, 1, 1, 1, 1, tr)
        xg = oracle.tri_tb_gauss_seidel_3d(levels[0], b, xg, 1, 1, 1, tr)
    err = lambda v: np.max(np.abs(v - ref)) / np.max(np.abs(ref))  # noqa: E731
    assert err(x) <= 1e-8 and err(x) < 1e-3 * err(xg), (err(x), err(xg))


@pytest.mark.parametrize("variant", ["TB", "TR"])
def test_oracle_zebra_order_converges_like_the_reference(built_oracle, variant):
    """The zebra order of the smoothers (lines and planes of one parity at
    once, the GPU's parallel order) solves the same systems: V-cycles over
    the built hierarchy reach the dense solution (about 17 times per cycle
    where the reference order gains 45), and a plane of one line is the
    reference's relaxation bit for bit."""
    tr = variant == "TR"
    zf, xf, yf, vol, dut, dur, _ = compute_inputs_3d(8, 8, 8, seed=1)
    levels = oracle.tri_tb_lapl_compute(zf, xf, yf, vol, dut, dur if tr else None, ref_level=4, **LAPL_COEFS)
    planes, u3, l3 = levels[0]
    b = np.random.default_rng(0).standard_normal((8, 8, 8, 2))
    ref = np.linalg.solve(dense_level(tuple(planes[0]) + (u3, l3), tr), b.reshape(-1)).reshape(b.shape)
    err = lambda v: np.max(np.abs(v - ref)) / np.max(np.abs(ref))  # noqa: E731
    out = {}
    try:
        for z in (0, 1):
            oracle.tri_tb_set_zebra(z)
            x = np.zeros_like(b)
            errs = []
            for _ in range(6):
                x = oracle.tri_tb_multigrid_3d(levels, b, x, 1, 1, 1, 1, tr)
                errs.append(err(x))
            out[z] = (errs, x)
        line = (planes[0][0][:1, :1],) + tuple(a[:1, :1] for a in planes[0][1:3]) + (planes[0][3][:1, :0],
                                                                                      planes[0][4][:1, :0])
        oracle.tri_tb_set_zebra(1)
        y1 = oracle.tri_tb_gauss_seidel_2d(line, b[:1, :1], np.zeros_like(b[:1, :1]), 2, tr)
        oracle.tri_tb_set_zebra(0)
        y0 = oracle.tri_tb_gauss_seidel_2d(line, b[:1, :1], np.zeros_like(b[:1, :1]), 2, tr)
    finally:
        oracle.tri_tb_set_zebra(0)
    (e0, _), (e1, xz) = out[0], out[1]
    assert e1[-1] <= 2e-8 and e1[-1] <= 100 * e0[-1], (e0, e1)  # about 17x per cycle against 45x
    assert all(b_ < a_ for a_, b_ in zip(e1, e1[1:])), e1
    assert not np.array_equal(xz, out[0][1])  # the order differs
    assert np.array_equal(y1, y0)  # one line: no order to change
