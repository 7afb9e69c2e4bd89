"""GPU parity of the TriDiagTB block-Thomas column solve and its product
(MULTI/TriDiagTB_Mod.f90:121-163, the same statements as TriDiagTR's) and of
the columns' assembly Compute_1D of both variants (TriDiagTB_Mod.f90:32-93,
TriDiagTR_Mod.f90:32-105) with the oracle: bit-exact on every shape,
including one- and two-level columns and a batch of 32768 columns of 128
levels (the columns of a 256x128 plane stack of the 512x512x128 grid); the
planes' and levels' assembly, product, smoothers, transfers and V-cycles
(Compute_2D/3D, MatVecTB_2D/3D, GaussSeidel_2D/3D, RestrictTB_2D/3D,
ProlongateTB_2D/3D, Multigrid_2D/3D), the resident hierarchy of
LaplTBCompute / LaplTRCompute (MULTI/JacAccGrav_Mod.f90:1312-1667) and its
V-cycle in the reference's order and in zebra order bit for bit as well."""
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


@pytest.mark.parametrize("variant", ["TB", "TR"])
@pytest.mark.parametrize("ncol,n1", [(3, 1), (4, 2), (129, 17), (4096, 128)])
def test_tri_tb_compute_bitwise(built_lib, variant, ncol, n1):
    """Compute_1D of TriDiagTB / TriDiagTR on the GPU equals the oracle bit
    for bit, and the assembled columns solve to the oracle's solution of its
    own assembly bit for bit."""
    from tests.test_tritb import compute_inputs

    faces, vol, dut, dur, coefs = compute_inputs(ncol, n1, seed=3 * n1 + ncol)
    dr = dur if variant == "TR" else None
    got = asam.Compute_TB_1D(*faces[:2], vol, faces[2], faces[3], dut, dr, **coefs)
    ref = oracle.tri_tb_compute(*faces[:2], vol, faces[2], faces[3], dut, dr, **coefs)
    for g, r in zip(got, ref):
        assert np.array_equal(g, r)
    b = np.random.default_rng(n1).standard_normal((ncol, n1, 2))
    assert np.array_equal(asam.Solve_TB_1D(*got, b), oracle.tri_tb_solve(*ref, b))
    from asam_gb300 import _lib

    lib = _lib.load()
    co = _lib.AsamTriTbCoefs(1.0, 0.0, 0.0, 0.0, 0.0)
    assert lib.asam_tri_tb_compute(2, 1, 1, co, None, None, None, None, None, None, None, None, None, None) == 4


@pytest.mark.parametrize("variant", ["TB", "TR"])
@pytest.mark.parametrize("nplane,n2,n1", [(1, 1, 1), (2, 3, 4), (3, 1, 5), (2, 5, 1), (16, 64, 32), (4, 256, 128)])
def test_tri_tb_compute_2d_bitwise(built_lib, variant, nplane, n2, n1):
    """Compute_2D of TriDiagTB / TriDiagTR, every element at once on the GPU,
    equals the oracle's line-by-line sweep bit for bit."""
    from tests.test_tritb import compute_inputs_2d

    zf, xf, vol, dut, dur, coefs = compute_inputs_2d(nplane, n2, n1, seed=5 * n2 + n1 + nplane)
    dr = dur if variant == "TR" else None
    got = asam.Compute_TB_2D(zf, xf, vol, dut, dr, **coefs)
    ref = oracle.tri_tb_compute_2d(zf, xf, vol, dut, dr, **coefs)
    for g, r in zip(got, ref):
        assert np.array_equal(g, r)


@pytest.mark.parametrize("couple", [True, False])
@pytest.mark.parametrize("variant", ["TB", "TR"])
@pytest.mark.parametrize("n3,n2,n1", [(1, 1, 1), (2, 3, 4), (4, 1, 3), (3, 2, 1), (16, 32, 64)])
def test_tri_tb_compute_3d_bitwise(built_lib, couple, variant, n3, n2, n1):
    """Compute_3D of TriDiagTB / TriDiagTR, both branches of the reference,
    every element at once on the GPU, equals the oracle's plane-by-plane
    sweep bit for bit."""
    from tests.test_tritb import compute_inputs_3d

    zf, xf, yf, vol, dut, dur, coefs = compute_inputs_3d(n3, n2, n1, seed=13 * n3 + n2 + n1)
    dr = dur if variant == "TR" else None
    got = asam.Compute_TB_3D(zf, xf, yf, vol, dut, dr, couple=couple, **coefs)
    ref = oracle.tri_tb_compute_3d(zf, xf, yf, vol, dut, dr, couple=couple, **coefs)
    for g, r in zip(got, ref):
        assert np.array_equal(g, r)


@pytest.mark.parametrize("variant", ["TB", "TR"])
@pytest.mark.parametrize("n3,n2,n1", [(1, 1, 4), (1, 3, 4), (3, 2, 1), (3, 4, 5), (16, 32, 64)])
def test_tri_tb_matvec_3d_bitwise(built_lib, variant, n3, n2, n1):
    """The level product MatVecTB/TR_2D/3D on the GPU, one thread per
    element, equals the oracle's loop nest bit for bit."""
    from tests.test_tritb import compute_inputs_3d

    zf, xf, yf, vol, dut, dur, coefs = compute_inputs_3d(n3, n2, n1, seed=n3 + 5 * n2 + n1)
    tr = variant == "TR"
    blocks = oracle.tri_tb_compute_3d(zf, xf, yf, vol, dut, dur if tr else None, couple=True, **coefs)
    x = np.random.default_rng(n2).standard_normal((n3, n2, n1, 2))
    assert np.array_equal(asam.MatVecTB_3D(blocks, x, tr), oracle.tri_tb_matvec_3d(blocks, x, tr))


@pytest.mark.parametrize("variant", ["TB", "TR"])
@pytest.mark.parametrize("nplane,n2,n1", [(2, 1, 5), (2, 2, 3), (3, 5, 4), (1, 7, 1), (64, 32, 48)])
def test_tri_tb_gauss_seidel_2d_bitwise(built_lib, variant, nplane, n2, n1):
    """GaussSeidel_2D on the GPU (planes in parallel, each plane's symmetric
    line sweep in the reference's order) equals the oracle bit for bit."""
    from tests.test_tritb import plane_case

    tr = variant == "TR"
    blocks, b = plane_case(nplane, n2, n1, seed=n2 + 3 * n1 + nplane)
    x0 = np.random.default_rng(nplane).standard_normal(b.shape)
    for iters in (1, 3):
        assert np.array_equal(asam.GaussSeidelTB_2D(blocks, b, x0, iters, tr),
                              oracle.tri_tb_gauss_seidel_2d(blocks, b, x0, iters, tr))


@pytest.mark.parametrize("n2,n1", [(1, 1), (2, 2), (3, 5), (4, 7), (65, 130)])
def test_tri_tb_restrict_prolong_bitwise(built_lib, n2, n1):
    res = np.random.default_rng(n1).standard_normal((3, n2, n1, 2))
    rc = asam.RestrictTB_2D(res)
    assert np.array_equal(rc, oracle.tri_tb_restrict_2d(res))
    assert np.array_equal(asam.ProlongateTB_2D(rc, n2, n1), oracle.tri_tb_prolong_2d(rc, n2, n1))


def random_hierarchy(nplane, n2, n1, seed):
    """Independent diagonally dominant planes on every level (the V-cycle's
    bits do not need a consistent hierarchy)."""
    from tests.test_tritb import plane_case

    levels = []
    while True:
        blocks, b = plane_case(nplane, n2, n1, seed=seed + len(levels))
        levels.append(blocks)
        if len(levels) == 1:
            b0 = b
        if n2 == 1 and n1 == 1:
            return levels, b0
        n2, n1 = (n2 + 1) // 2, (n1 + 1) // 2


@pytest.mark.parametrize("variant", ["TB", "TR"])
@pytest.mark.parametrize("nplane,n2,n1,gi2,cycles", [(2, 8, 8, 1, 2), (1, 7, 5, 2, 3), (3, 1, 9, 1, 1), (2, 6, 1, 0, 2),
                                                      (1, 1, 1, 1, 2), (32, 64, 96, 1, 2)])
def test_tri_tb_multigrid_2d_bitwise(built_lib, variant, nplane, n2, n1, gi2, cycles):
    """Solve_2D / Multigrid_2D on the GPU (smoother, residual, restriction
    and correction as kernels on one stream, the level loop on the host)
    equals the oracle bit for bit, on Galerkin hierarchies and on a 32-plane
    stack of 64x96 planes with seven levels."""
    from tests.test_tritb import plane_hierarchy

    tr = variant == "TR"
    if nplane * n2 * n1 <= 256:
        levels, b = plane_hierarchy(nplane, n2, n1, seed=n2 * 7 + n1, tr=tr)
    else:
        levels, b = random_hierarchy(nplane, n2, n1, seed=11)
    x0 = np.random.default_rng(1).standard_normal(b.shape)
    assert np.array_equal(asam.SolveTB_2D(levels, b, x0, gi2, cycles, tr),
                          oracle.tri_tb_multigrid_2d(levels, b, x0, gi2, cycles, tr))


def test_tri_tb_multigrid_2d_bad_args(built_lib):
    from asam_gb300._lib import AsamError

    levels, b = random_hierarchy(1, 6, 4, seed=2)
    with pytest.raises(AsamError):  # a level of the wrong size
        asam.SolveTB_2D([levels[0], levels[0]], b, b, 1, 1)
    with pytest.raises(AsamError):
        asam.SolveTB_2D(levels, b, b, -1, 1)


def random_levels_3d(n3, n2, n1, seed):
    """Independent diagonally dominant levels and plane levels (bits only)."""
    from tests.test_tritb import plane_case

    levels, b0 = [], None
    while True:
        r = np.random.default_rng(seed + len(levels))
        planes, p2, p1 = [], n2, n1
        while True:
            blocks, b = plane_case(n3, p2, p1, seed=seed + 100 * len(levels) + len(planes))
            if b0 is None:
                b0 = b
            planes.append(blocks)
            if p2 == 1 and p1 == 1:
                break
            p2, p1 = (p2 + 1) // 2, (p1 + 1) // 2
        levels.append((planes, r.uniform(-1, 1, (n3 - 1, n2, n1, 4)), r.uniform(-1, 1, (n3 - 1, n2, n1, 4))))
        if (n3, n2, n1) == (1, 1, 1):
            return levels, b0
        n3, n2, n1 = (n3 + 1) // 2, (n2 + 1) // 2, (n1 + 1) // 2


@pytest.mark.parametrize("variant", ["TB", "TR"])
@pytest.mark.parametrize("n3,n2,n1,gi3,cycles", [(4, 4, 4, 1, 2), (3, 5, 2, 2, 1), (1, 1, 1, 1, 2), (5, 1, 3, 0, 2),
                                                  (12, 24, 20, 1, 1)])
def test_tri_tb_multigrid_3d_bitwise(built_lib, variant, n3, n2, n1, gi3, cycles):
    """Solve_3D / Multigrid_3D on the GPU (the plane sweeps of GaussSeidel_3D,
    each plane's Solve_2D, the residual, RestrictTB_3D and the correction as
    kernels on one stream) equals the oracle bit for bit, on Galerkin
    hierarchies and on a 12x24x20 level with five levels."""
    from tests.test_tritb import level_hierarchy_3d

    tr = variant == "TR"
    if n3 * n2 * n1 <= 64:
        levels, b = level_hierarchy_3d(n3, n2, n1, seed=n3 + 5 * n2 + 11 * n1, tr=tr)
    else:
        levels, b = random_levels_3d(n3, n2, n1, seed=21)
    x0 = np.random.default_rng(4).standard_normal(b.shape)
    for gi2, mi2 in ((1, 1), (2, 2)):
        assert np.array_equal(asam.SolveTB_3D(levels, b, x0, gi2, mi2, gi3, cycles, tr),
                              oracle.tri_tb_multigrid_3d(levels, b, x0, gi2, mi2, gi3, cycles, tr))


def test_tri_tb_multigrid_3d_bad_args(built_lib):
    from asam_gb300._lib import AsamError

    levels, b = random_levels_3d(3, 4, 4, seed=2)
    with pytest.raises(AsamError):  # a level of the wrong size
        asam.SolveTB_3D([levels[0], levels[0]], b, b)
    planes, u3, l3 = levels[0]
    with pytest.raises(ValueError):  # a plane level of the wrong size
        asam.SolveTB_3D([(planes[:1] + planes[:1], u3, l3)] + levels[1:], b, b)
    with pytest.raises(AsamError):
        asam.SolveTB_3D(levels, b, b, mult_iter3=-1)


@pytest.mark.parametrize("variant", ["TB", "TR"])
@pytest.mark.parametrize("n3,n2,n1,ref_level", [(5, 6, 7, 3), (8, 8, 8, 4), (3, 1, 9, 2), (16, 48, 40, 5)])
def test_tri_tb_hierarchy_bitwise(built_lib, variant, n3, n2, n1, ref_level):
    """LaplTBCompute / LaplTRCompute on the GPU (the coarsening of the finest
    fields and Compute_3D of every level and plane level, resident on the
    device) equal the oracle's arrays bit for bit, and a V-cycle over the
    resident hierarchy from x = 0 (VCycleCG) equals the oracle's Solve_3D
    over the oracle's hierarchy."""
    from tests.test_tritb import LAPL_COEFS, compute_inputs_3d

    tr = variant == "TR"
    zf, xf, yf, vol, dut, dur, _ = compute_inputs_3d(n3, n2, n1, seed=n3 * n2 + n1)
    dd = dur if tr else None
    with asam.TriTBHierarchy(zf, xf, yf, vol, dut, dd, ref_level=ref_level, **LAPL_COEFS) as h:
        for L3 in range(ref_level):
            for L2 in range(L3, ref_level):
                got = h.level(L3, L2)
                ref = oracle.tri_tb_lapl_level(zf, xf, yf, vol, dut, dd, L3, L2, LAPL_COEFS)
                for g, r in zip(got, ref[:len(got)]):
                    assert np.array_equal(g, r), (L3, L2)
        b = np.random.default_rng(n1).standard_normal((n3, n2, n1, 2))
        levels = oracle.tri_tb_lapl_compute(zf, xf, yf, vol, dut, dd, ref_level=ref_level, **LAPL_COEFS)
        assert np.array_equal(h.vcycle(b), oracle.tri_tb_multigrid_3d(levels, b, np.zeros_like(b), 1, 1, 1, 1, tr))
        x0 = np.random.default_rng(2).standard_normal(b.shape)
        assert np.array_equal(h.vcycle(b, x0, 2, 2, 1, 2),
                              oracle.tri_tb_multigrid_3d(levels, b, x0, 2, 2, 1, 2, tr))


@pytest.mark.parametrize("variant", ["TB", "TR"])
@pytest.mark.parametrize("n3,n2,n1,ref_level", [(5, 6, 7, 3), (8, 8, 8, 4), (3, 1, 9, 2), (16, 48, 40, 5)])
def test_tri_tb_hierarchy_zebra_bitwise(built_lib, variant, n3, n2, n1, ref_level):
    """The zebra order on the GPU (every line of a parity in parallel, the
    2D V-cycles of every plane of a parity at once) equals the oracle's zebra
    order bit for bit."""
    from tests.test_tritb import LAPL_COEFS, compute_inputs_3d

    tr = variant == "TR"
    zf, xf, yf, vol, dut, dur, _ = compute_inputs_3d(n3, n2, n1, seed=n3 * n2 + n1)
    dd = dur if tr else None
    levels = oracle.tri_tb_lapl_compute(zf, xf, yf, vol, dut, dd, ref_level=ref_level, **LAPL_COEFS)
    b = np.random.default_rng(n1).standard_normal((n3, n2, n1, 2))
    x0 = np.random.default_rng(2).standard_normal(b.shape)
    with asam.TriTBHierarchy(zf, xf, yf, vol, dut, dd, ref_level=ref_level, **LAPL_COEFS) as h:
        h.set_zebra(True)
        try:
            oracle.tri_tb_set_zebra(1)
            ref1 = oracle.tri_tb_multigrid_3d(levels, b, np.zeros_like(b), 1, 1, 1, 1, tr)
            ref2 = oracle.tri_tb_multigrid_3d(levels, b, x0, 2, 2, 1, 2, tr)
        finally:
            oracle.tri_tb_set_zebra(0)
        assert np.array_equal(h.vcycle(b), ref1)
        assert np.array_equal(h.vcycle(b, x0, 2, 2, 1, 2), ref2)
        h.set_zebra(False)
        assert np.array_equal(h.vcycle(b), oracle.tri_tb_multigrid_3d(levels, b, np.zeros_like(b), 1, 1, 1, 1, tr))


def test_tri_tb_hierarchy_bad_args(built_lib):
    from asam_gb300._lib import AsamError
    from tests.test_tritb import LAPL_COEFS, compute_inputs_3d

    zf, xf, yf, vol, dut, dur, _ = compute_inputs_3d(3, 4, 5, seed=1)
    for ref_level in (0, 25):
        with pytest.raises(AsamError):
            asam.TriTBHierarchy(zf, xf, yf, vol, dut, None, ref_level=ref_level, **LAPL_COEFS)
    with pytest.raises(ValueError):  # faces of the wrong shape
        asam.TriTBHierarchy(zf, xf[::-1][:3] + [xf[3][:, :-1]], yf, vol, dut, None, ref_level=2, **LAPL_COEFS)
    with asam.TriTBHierarchy(zf, xf, yf, vol, dut, None, ref_level=2, **LAPL_COEFS) as h:
        with pytest.raises(AsamError):
            h.level(1, 0)  # plane levels start at the level itself
        with pytest.raises(ValueError):
            h.vcycle(np.zeros((3, 4, 4, 2)))
