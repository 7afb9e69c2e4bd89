"""Independent numpy restatement of the transport-stage operators (test-only).

Written in gather form (face fluxes first, then each cell sums its faces in
the order the reference's scatter loop touches it), so it shares no code and
no loop structure with the C oracle, yet follows the same floating-point
operation order -- agreement with the oracle is therefore expected to be
bit-exact.  Sources: ADVECT/Advection_Mod.f90:737-1054 (AdvectionComputeP),
:2106-2134 (hLF..PhiLim), :2220-2872 (JacAdvectionCompute),
ADVECT/Function_Mod.f90:1782-1862 (JacScaleCompute),
CG/MatSpDiag_Mod.f90:87-235 (SpAVec, GaussSeidel).
"""
from __future__ import annotations

import numpy as np

EPS = 1e-30


def _k1(hL, hC, hR):
    return (hC / (hC + hR + EPS)) * ((hL + hC) / (hL + hC + hR + EPS))


def _k2(hL, hC, hR):
    return (hC / (hL + hC + EPS)) * (hR / (hL + hC + hR + EPS))


def _koren(r, k1, k2):
    a = k1 * r + k2
    m = np.where(a < 1.0, a, 1.0)
    m = np.where(r < m, r, m)
    return np.where(0.0 > m, 0.0, m)


def _upwind(cL, cC, cR, VL, VC, VR, FL, FR, vel, right, vblend):
    with np.errstate(divide="ignore", invalid="ignore"):
        if vblend:
            cL = np.where(VL < VC, ((VC - VL) * cC + VL * cL) / VC, cL)
            cR = np.where(VR < VC, ((VC - VR) * cC + VR * cR) / VC, cR)
        cL = np.where(FL < FR, ((FR - FL) * cC + FL * cL) / FR, cL)
        cR = np.where(FR < FL, ((FL - FR) * cC + FR * cR) / FL, cR)
        if not right:
            k1 = _k1(VR, VC, VL)
            k2 = _k2(VR, VC, VL)
            r = (cC - cL + EPS) / ((cR - cC) + EPS)
            return 0.5 * (np.abs(vel) - vel) * FL * (cC + FR / (FR + EPS) * (_koren(r, k1, k2) * (cC - cR)))
        k1 = _k1(VL, VC, VR)
        k2 = _k2(VL, VC, VR)
        r = (cR - cC + EPS) / ((cC - cL) + EPS)
        return 0.5 * (np.abs(vel) + vel) * FR * (cC + FL / (FL + EPS) * (_koren(r, k1, k2) * (cC - cL)))


def face_fluxes(geo, phi, vel):
    """Upwind-cell flux of every x/y/z face for one component field phi (padded, k,j,i)."""
    g = geo.grid
    nx, ny, nz = g.nx, g.ny, g.nz
    V = geo.volc
    uf, vf, wf = vel
    out = []
    # x faces i=0..nx between padded cells i,i+1 (j,k interior)
    J, K = slice(1, ny + 1), slice(1, nz + 1)
    gx = np.zeros((nz, ny, nx + 1))
    for i in range(nx + 1):
        u = uf[:, :, i]
        res = np.zeros((nz, ny))
        if i >= 1:  # upwind = cell i (right face of i)
            c = i
            val = _upwind(phi[K, J, c - 1], phi[K, J, c], phi[K, J, c + 1], V[K, J, c - 1], V[K, J, c], V[K, J, c + 1],
                          geo.fu[:, :, c], geo.fu[:, :, c + 1], u, True, True)
            res = np.where(u > 0, val, res)
        if i + 1 <= nx:  # upwind = cell i+1 (left face of i+1)
            c = i + 1
            val = _upwind(phi[K, J, c - 1], phi[K, J, c], phi[K, J, c + 1], V[K, J, c - 1], V[K, J, c], V[K, J, c + 1],
                          geo.fu[:, :, c], geo.fu[:, :, c + 1], u, False, True)
            res = np.where(u < 0, val, res)
        gx[:, :, i] = res
    out.append(gx)
    I = slice(1, nx + 1)
    gy = np.zeros((nz, ny + 1, nx))
    for j in range(ny + 1):
        v = vf[:, j, :]
        res = np.zeros((nz, nx))
        if j >= 1:
            c = j
            val = _upwind(phi[K, c - 1, I], phi[K, c, I], phi[K, c + 1, I], V[K, c - 1, I], V[K, c, I], V[K, c + 1, I],
                          geo.fv[:, c, :], geo.fv[:, c + 1, :], v, True, False)
            res = np.where(v > 0, val, res)
        if j + 1 <= ny:
            c = j + 1
            val = _upwind(phi[K, c - 1, I], phi[K, c, I], phi[K, c + 1, I], V[K, c - 1, I], V[K, c, I], V[K, c + 1, I],
                          geo.fv[:, c, :], geo.fv[:, c + 1, :], v, False, False)
            res = np.where(v < 0, val, res)
        gy[:, j, :] = res
    out.append(gy)
    gz = np.zeros((nz + 1, ny, nx))
    for k in range(nz + 1):
        w = wf[k]
        res = np.zeros((ny, nx))
        if k >= 1:
            c = k
            val = _upwind(phi[c - 1, J, I], phi[c, J, I], phi[c + 1, J, I], V[c - 1, J, I], V[c, J, I], V[c + 1, J, I],
                          geo.fw[c], geo.fw[c + 1], w, True, False)
            res = np.where(w > 0, val, res)
        if k + 1 <= nz:
            c = k + 1
            val = _upwind(phi[c - 1, J, I], phi[c, J, I], phi[c + 1, J, I], V[c - 1, J, I], V[c, J, I], V[c + 1, J, I],
                          geo.fw[c], geo.fw[c + 1], w, False, False)
            res = np.where(w < 0, val, res)
        gz[k] = res
    out.append(gz)
    return out


def fcn(geo, c, vel, rho_pos=0):
    """FcnMet advection terms of all components (gather form)."""
    g = geo.grid
    nx, ny, nz = g.nx, g.ny, g.nz
    V = geo.volc
    uf, vf, wf = vel
    rho = c[rho_pos]
    out = np.zeros_like(c)
    for ic in range(c.shape[0]):
        phi = c[ic] / (rho + EPS)
        gx, gy, gz = face_fluxes(geo, phi, vel)
        f = np.zeros_like(phi)
        a = np.zeros((nz, ny, nx))
        uL, uR = uf[:, :, :-1], uf[:, :, 1:]
        vL, vR = vf[:, :-1, :], vf[:, 1:, :]
        wL, wR = wf[:-1], wf[1:]
        GxL, GxR = gx[:, :, :-1], gx[:, :, 1:]
        GyL, GyR = gy[:, :-1, :], gy[:, 1:, :]
        GzL, GzR = gz[:-1], gz[1:]
        for cond, term, sign in ((wL > 0, GzL, 1), (vL > 0, GyL, 1), (uL > 0, GxL, 1), (uL < 0, GxL, -1),
                                 (uR > 0, GxR, -1), (vL < 0, GyL, -1), (vR > 0, GyR, -1), (wL < 0, GzL, -1),
                                 (wR > 0, GzR, -1), (uR < 0, GxR, 1), (vR < 0, GyR, 1), (wR < 0, GzR, 1)):
            a = np.where(cond, a + term if sign > 0 else a - term, a)
        # first-order inflow through the faces of the outer walls from the halo
        # cells, W, E, S, N, B, T (the bottom divides by the interior density)
        ci = c[ic]
        if not g.periodic_x:
            u = uf[:, :, 0]
            a[:, :, 0] = a[:, :, 0] + 0.5 * (np.abs(u) + u) * ci[1:-1, 1:-1, 0] / (rho[1:-1, 1:-1, 0] + EPS) * geo.fu[:, :, 1]
            u = uf[:, :, nx]
            a[:, :, nx - 1] = (a[:, :, nx - 1] + 0.5 * (np.abs(u) - u) * ci[1:-1, 1:-1, nx + 1]
                               / (rho[1:-1, 1:-1, nx + 1] + EPS) * geo.fu[:, :, nx + 1])
        if not g.periodic_y:
            v = vf[:, 0, :]
            a[:, 0, :] = a[:, 0, :] + 0.5 * (np.abs(v) + v) * ci[1:-1, 0, 1:-1] / (rho[1:-1, 0, 1:-1] + EPS) * geo.fv[:, 1, :]
            v = vf[:, ny, :]
            a[:, ny - 1, :] = (a[:, ny - 1, :] + 0.5 * (np.abs(v) - v) * ci[1:-1, ny + 1, 1:-1]
                               / (rho[1:-1, ny + 1, 1:-1] + EPS) * geo.fv[:, ny + 1, :])
        if not g.periodic_z:
            w = wf[0]
            a[0] = a[0] + 0.5 * (np.abs(w) + w) * ci[0, 1:-1, 1:-1] / (rho[1, 1:-1, 1:-1] + EPS) * geo.fw[1]
            w = wf[nz]
            a[nz - 1] = a[nz - 1] + 0.5 * (np.abs(w) - w) * ci[nz + 1, 1:-1, 1:-1] / (rho[nz + 1, 1:-1, 1:-1] + EPS) * geo.fw[nz + 1]
        f[1:nz + 1, 1:ny + 1, 1:nx + 1] = a
        # halo cells next to the interior: the outflow a periodic side hands on;
        # an outer wall's halo is zeroed
        f[1:nz + 1, 1:ny + 1, 0] = np.where(uf[:, :, 0] < 0, gx[:, :, 0], 0.0) if g.periodic_x else 0.0
        f[1:nz + 1, 1:ny + 1, nx + 1] = np.where(uf[:, :, nx] > 0, gx[:, :, nx], 0.0) if g.periodic_x else 0.0
        f[1:nz + 1, 0, 1:nx + 1] = np.where(vf[:, 0, :] < 0, gy[:, 0, :], 0.0) if g.periodic_y else 0.0
        f[1:nz + 1, ny + 1, 1:nx + 1] = np.where(vf[:, ny, :] > 0, gy[:, ny, :], 0.0) if g.periodic_y else 0.0
        f[0, 1:ny + 1, 1:nx + 1] = np.where(wf[0] < 0, gz[0], 0.0) if g.periodic_z else 0.0
        f[nz + 1, 1:ny + 1, 1:nx + 1] = np.where(wf[nz] > 0, gz[nz], 0.0) if g.periodic_z else 0.0
        f = f * V / (V + EPS)
        if g.periodic_x:
            f[1:nz + 1, 1:ny + 1, 1] = f[1:nz + 1, 1:ny + 1, 1] + f[1:nz + 1, 1:ny + 1, nx + 1]
            f[1:nz + 1, 1:ny + 1, nx] = f[1:nz + 1, 1:ny + 1, nx] + f[1:nz + 1, 1:ny + 1, 0]
        if g.periodic_y:
            f[1:nz + 1, 1, 1:nx + 1] = f[1:nz + 1, 1, 1:nx + 1] + f[1:nz + 1, ny + 1, 1:nx + 1]
            f[1:nz + 1, ny, 1:nx + 1] = f[1:nz + 1, ny, 1:nx + 1] + f[1:nz + 1, 0, 1:nx + 1]
        out[ic] = f / (V + EPS)
    return out


def upwind_rhs(geo, c, vel, rho):
    """First-order upwind advection RHS (what the Jacobian linearises): per
    interior cell sum of inflow u*F*c_up/rho_up minus outflow u*F*c/rho, over V."""
    g = geo.grid
    nx, ny, nz = g.nx, g.ny, g.nz
    V = geo.volc
    uf, vf, wf = vel
    phi = c / (rho + EPS)
    out = np.zeros_like(c)
    I, J, K = slice(1, nx + 1), slice(1, ny + 1), slice(1, nz + 1)
    acc = np.zeros((nz, ny, nx))
    fu = geo.fu[:, :, 1:nx + 2]
    fv = geo.fv[:, 1:ny + 2, :]
    fw = geo.fw[1:nz + 2]
    # flux through each face, positive in +axis direction (upwind value)
    px = np.where(uf > 0, uf * fu * phi[K, J, 0:nx + 1], uf * fu * phi[K, J, 1:nx + 2])
    py = np.where(vf > 0, vf * fv * phi[K, 0:ny + 1, I], vf * fv * phi[K, 1:ny + 2, I])
    pz = np.where(wf > 0, wf * fw * phi[0:nz + 1, J, I], wf * fw * phi[1:nz + 2, J, I])
    # an outer wall keeps the outflow of the interior cell (the inflow from
    # the halo does not depend on the interior state)
    if not g.periodic_x:
        px[:, :, 0] = np.minimum(px[:, :, 0], 0.0)
        px[:, :, nx] = np.maximum(px[:, :, nx], 0.0)
    if not g.periodic_y:
        py[:, 0, :] = np.minimum(py[:, 0, :], 0.0)
        py[:, ny, :] = np.maximum(py[:, ny, :], 0.0)
    pz[0] = np.minimum(pz[0], 0.0)
    pz[nz] = np.maximum(pz[nz], 0.0)
    acc = (px[:, :, :-1] - px[:, :, 1:]) + (py[:, :-1, :] - py[:, 1:, :]) + (pz[:-1] - pz[1:])
    out[K, J, I] = acc / (V[K, J, I] + EPS)
    return out


def dia_scipy(val, grid):
    """The column-oriented DIA matrix as scipy.sparse (A[col-shift, col] = Val(col, d))."""
    import scipy.sparse as sp

    NX, NY = grid.nx + 2, grid.ny + 2
    n = grid.npad
    shifts = [-NX * NY, -NX, -1, 0, 1, NX, NX * NY]
    # scipy dia: A[i, i+k] = data[d, i+k]  ->  offset k = shift
    return sp.dia_matrix((np.asarray(val), shifts), shape=(n, n)).tocsr()


def gauss_seidel(val, grid, b, iterg=5):
    """x = (L+D)^-1 b, then IterG sweeps x = (L+D)^-1 (b - U x) (scipy triangular solves)."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl

    A = dia_scipy(val, grid)
    L = sp.tril(A, 0).tocsr()
    U = sp.triu(A, 1).tocsr()
    x = spl.spsolve_triangular(L, b, lower=True)
    for _ in range(iterg):
        x = spl.spsolve_triangular(L, b - U @ x, lower=True)
    return x


def line_solve(val, grid, b, axis):
    """x = T^-1 b with T the tridiagonal part of the stage matrix along one axis
    (0: x, 1: y, 2: z): the diagonal and the couplings to the two neighbours on
    that axis inside the padded box, every line solved on its own."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl

    NX, NY, NZ = grid.nx + 2, grid.ny + 2, grid.nz + 2
    A = dia_scipy(val, grid).tocoo()
    st = [1, NX, NX * NY][axis]
    length = [NX, NY, NZ][axis]
    d = A.col - A.row
    pos = lambda r: (r // st) % length  # noqa: E731  index of a cell along the axis
    keep = (d == 0) | (((d == st) | (d == -st)) & (np.abs(pos(A.col) - pos(A.row)) == 1))
    T = sp.csc_matrix((A.data[keep], (A.row[keep], A.col[keep])), shape=A.shape)
    lu = spl.splu(T)
    bb = np.asarray(b, dtype=np.float64).reshape(-1, grid.npad)
    return np.stack([lu.solve(r) for r in bb]).reshape(np.shape(b))


def lapl_level0(geo, W, dx, dy, dz, beta0, dtp, facs=(0.0, 0.0, 0.0)):
    """Level-0 pressure Laplacian of LaplTFullCompute (MULTI/JacAccGrav_Mod.f90:
    1056-1310 with ComputeFull_1D/2D/3D of MULTI/TriDiagT_Mod.f90; shift 0,
    Cartesian metric), restated in numpy: the arrays d, u/l along z, along x
    and along y in the reversed order (z fastest, then x, then y), entries past
    the last row/line/plane 0.  facs = the boundary factors (Fac1, Fac2, Fac3)
    of both ends of the z, x and y axes: 0 for LaplNeumann (SetFactorN), 2 on
    the periodic axes for LaplDirichlet (SetFactorD)."""
    f1, f2, f3 = (float(f) for f in facs)
    g = geo.grid
    nx, ny, nz = g.nx, g.ny, g.nz
    eps = 1.0e-30
    dtu, dtv, dtw, duu, duv, duw, dut, _ = W
    rv = lambda a: np.ascontiguousarray(np.transpose(a, (1, 2, 0)))  # [z,y,x] -> [y,x,z]
    F1, T1, U1 = rv(geo.fw[1:nz + 2]), rv(dtw), rv(duw)
    F2, T2, U2 = rv(geo.fu[:, :, 1:nx + 2]), rv(dtu), rv(duu)
    F3, T3, U3 = rv(geo.fv[:, 1:ny + 2, :]), rv(dtv), rv(duv)
    # CFaceCoarse with shift 0
    T1, U1 = (T1 * F1) / (F1 + eps), (U1 * F1) / (F1 + eps)
    T2, U2 = (T2 * F2) / (F2 + eps), (U2 * F2) / (F2 + eps)
    T3, U3 = (T3 * F3) / (F3 + eps), (U3 * F3) / (F3 + eps)
    vol = rv(geo.volc[1:-1, 1:-1, 1:-1])
    vol = 0.0 + vol
    D = (rv(dut) * vol) / (vol + eps)
    bd = beta0 * dtp
    bd2 = bd * bd
    one = 1.0
    d = np.full((ny, nx, nz), 1.0e-40)
    z = np.zeros_like(d)
    # z terms: face f (1..nz-1) between cells f-1, f (0-based)
    dzc = 0.0 + np.asarray(dz)
    if nz > 1:
        den = (dzc[:-1] + dzc[1:]) * one * one
        base = bd2 * 2.0 * F1[:, :, 1:nz] * T1[:, :, 1:nz] * U1[:, :, 1:nz]
        below = base * D[:, :, 1:] / den   # cell f, face below
        above = base * D[:, :, :-1] / den  # cell f-1, face above
        first = np.concatenate([bd2 * f1 * F1[:, :, :1] * T1[:, :, :1] * U1[:, :, :1] * D[:, :, :1] / (dzc[0] * one * one),
                                below], axis=2)
        second = np.concatenate([above, bd2 * f1 * F1[:, :, nz:] * T1[:, :, nz:] * U1[:, :, nz:] * D[:, :, -1:] /
                                 (dzc[-1] * one * one)], axis=2)
        uz = np.concatenate([-(base * D[:, :, 1:] / den), z[:, :, :1]], axis=2)
        lz = np.concatenate([-(base * D[:, :, :-1] / den), z[:, :, :1]], axis=2)
    else:
        first = bd2 * f1 * F1[:, :, :1] * T1[:, :, :1] * U1[:, :, :1] * D / (dzc[0] * one * one)
        second = bd2 * f1 * F1[:, :, 1:] * T1[:, :, 1:] * U1[:, :, 1:] * D / (dzc[0] * one * one)
        uz = lz = z.copy()
    d = d + first
    d = d + second
    d = d + 1.0 * vol
    # x terms: face f (1..nx-1) between columns f-1, f
    dxc = 0.0 + np.asarray(dx)
    if nx > 1:
        den = ((dxc[:-1] + dxc[1:]) * one)[None, :, None] * one
        base = bd2 * 2.0 * F2[:, 1:nx] * T2[:, 1:nx] * U2[:, 1:nx]
        first = np.concatenate([bd2 * f2 * F2[:, :1] * T2[:, :1] * U2[:, :1] * D[:, :1] / (dxc[0] * one * one),
                                base * D[:, 1:] / den], axis=1)
        second = np.concatenate([base * D[:, :-1] / den,
                                 bd2 * f2 * F2[:, nx:] * T2[:, nx:] * U2[:, nx:] * D[:, -1:] / (dxc[-1] * one * one)],
                                axis=1)
        ux = np.concatenate([-(base * D[:, 1:] / den), z[:, :1]], axis=1)
        lx = np.concatenate([-(base * D[:, :-1] / den), z[:, :1]], axis=1)
    else:
        first = bd2 * f2 * F2[:, :1] * T2[:, :1] * U2[:, :1] * D / (dxc[0] * one * one)
        second = bd2 * f2 * F2[:, 1:] * T2[:, 1:] * U2[:, 1:] * D / (dxc[0] * one * one)
        ux = lx = z.copy()
    d = d + first
    d = d + second
    # y terms (no DUU3 in the couplings, the interior diagonal terms and the high boundary term)
    dyc = 0.0 + np.asarray(dy)
    if ny > 1:
        den = ((dyc[:-1] + dyc[1:]) * one)[:, None, None] * one
        base = bd2 * 2.0 * F3[1:ny] * T3[1:ny]
        first = np.concatenate([bd2 * f3 * F3[:1] * T3[:1] * U3[:1] * D[:1] / (dyc[0] * one * one),
                                base * D[1:] / den], axis=0)
        second = np.concatenate([base * D[:-1] / den, bd2 * f3 * F3[ny:] * T3[ny:] * D[-1:] / (dyc[-1] * one * one)],
                                axis=0)
        u3 = np.concatenate([-(base * D[1:] / den), z[:1]], axis=0)
        l3 = np.concatenate([-(base * D[:-1] / den), z[:1]], axis=0)
    else:
        first = bd2 * f3 * F3[:1] * T3[:1] * U3[:1] * D / (dyc[0] * one * one)
        second = bd2 * f3 * F3[1:] * T3[1:] * D / (dyc[0] * one * one)
        u3 = l3 = z.copy()
    d = d + first
    d = d + second
    return [a.ravel() for a in (d, uz, lz, ux, lx, u3, l3)]


# ---------------------------------------------------------------------------
# Dynamical-core pieces (numpy, vectorised; independent of oracle/asam_dyn.c)
# ---------------------------------------------------------------------------
CPD, CVD, CPV, RV, CPL, CPI, P0 = 1004.0, 717.0, 1885.0, 461.0, 4186.0, 2110.0, 1.0e5
RD = CPD - CVD


def bound_cond(c, kinds, periodic=(False, False, False), mean=None, fval=None, amb=None, vel=None, rho_pos=0):
    """BoundaryCompute on the face halos of the non-periodic sides
    (ADVECT/BoundaryCondition_Mod.f90:70-346); c (ncomp, NZ, NY, NX).  Kinds
    1 ZeroGrad, 2 ZeroValue, 3 MeanValue (mean (ncomp, nz)), 4 Function
    (fval: the halo values F), 5 InFlowOutFlow on the lateral sides (amb: the
    ambient state, vel: the face velocities), 6 Extrapolation on the bottom
    and top; components in order."""
    out = c.copy()
    nz = c.shape[1] - 2
    for ic in range(c.shape[0]):
        a = out[ic]
        k = kinds[ic]
        rho = out[rho_pos]
        # (side, halo index, interior index, next interior index) per side
        sides = []
        if not periodic[0]:
            sides += [(0, np.s_[1:-1, 1:-1, 0], np.s_[1:-1, 1:-1, 1], np.s_[1:-1, 1:-1, 2]),
                      (1, np.s_[1:-1, 1:-1, -1], np.s_[1:-1, 1:-1, -2], np.s_[1:-1, 1:-1, -3])]
        if not periodic[1]:
            sides += [(2, np.s_[1:-1, 0, 1:-1], np.s_[1:-1, 1, 1:-1], np.s_[1:-1, 2, 1:-1]),
                      (3, np.s_[1:-1, -1, 1:-1], np.s_[1:-1, -2, 1:-1], np.s_[1:-1, -3, 1:-1])]
        if not periodic[2]:
            sides += [(4, np.s_[0, 1:-1, 1:-1], np.s_[1, 1:-1, 1:-1], np.s_[2, 1:-1, 1:-1]),
                      (5, np.s_[-1, 1:-1, 1:-1], np.s_[-2, 1:-1, 1:-1], np.s_[-3, 1:-1, 1:-1])]
        for side, H, S, S2 in sides:
            kind = k[side]
            if kind == 1:
                a[H] = a[S]
            elif kind == 2:
                a[H] = -a[S]
            elif kind == 3:
                if side < 4:
                    prof = mean[ic][:, None]
                else:
                    prof = mean[ic][0 if side == 4 else nz - 1]
                a[H] = 2.0 * prof - a[S]
            elif kind == 4:
                a[H] = 2.0 * fval[ic][H] - a[S]
            elif kind == 5 and side < 4:
                uf, vf = vel[0], vel[1]
                u = {0: uf[:, :, 0], 1: uf[:, :, -1], 2: vf[:, 0, :], 3: vf[:, -1, :]}[side]
                inflow = u <= 0 if side & 1 else u >= 0
                a[H] = np.where(inflow, rho[H] * amb[ic][H], a[S])
            elif kind == 6 and side >= 4:
                a[H] = 2.0 * a[S] - a[S2]
    return out


def thermo(rho, rth, rv=None, rc=None, rr=None, ri=None):
    """AbsTCompute 'Density' and PreCompute default branch
    (ADVECT/Diagnostic_Mod.f90:602-615, 805-811), element-wise."""
    z = np.zeros_like(rho)
    rv = z if rv is None else rv
    rl, rrr = (z if rc is None else rc), (z if rr is None else rr)
    ri = z if ri is None else ri
    rll = rl + rrr
    rd = rho - rv - rll - ri + EPS
    rm = RD * rd + RV * rv + EPS
    cpml = CPD * rd + CPV * rv + CPL * rll + CPI * ri + EPS
    kap = rm / cpml
    with np.errstate(invalid="ignore"):
        t = np.power(RD * rth / np.power(P0, kap), 1.0 / (1.0 - kap)) / rm + EPS
    p = (RD * (rho - rl - rrr) + (RV - RD) * rv) * t
    return t, p


def momentum_sources(geo, p, rho, dx, dy, dz, grav=9.81):
    """Pressure gradient (ADVECT/PressureGrad_Mod.f90:252-276, before
    AdvectionScale: -2 VolC Grad per LR component) and buoyancy
    (ADVECT/Buoyancy_Mod.f90:51-63, after the scale: -RhoLoc Grav) on the
    interior cells of a block with closed or periodic x/y sides.  Returns (pg[6], bu[2]) as (nz, ny, nx)
    arrays in the order uL, uR, vL, vR, wL, wR and wL, wR."""
    g = geo.grid
    nx, ny, nz = g.nx, g.ny, g.nz
    V = geo.volc[1:nz + 1, 1:ny + 1, 1:nx + 1]
    P = p
    pg = [np.zeros((nz, ny, nx)) for _ in range(6)]
    # x faces between interior cells i and i+1 (i = 1..nx-1): native FU index i+1
    F = geo.fu[:, :, 2:nx + 1]
    gx = F / (F + EPS) * F / (F + EPS) * (P[1:-1, 1:-1, 2:nx + 1] - P[1:-1, 1:-1, 1:nx]) / (
        1.0 * (dx[1:] + dx[:-1] + EPS))
    pg[0][:, :, 1:] = -2.0 * V[:, :, 1:] * gx
    pg[1][:, :, :-1] = -2.0 * V[:, :, :-1] * gx
    F = geo.fv[:, 2:ny + 1, :]
    gy = F / (F + EPS) * F / (F + EPS) * (P[1:-1, 2:ny + 1, 1:-1] - P[1:-1, 1:ny, 1:-1]) / (
        1.0 * (dy[1:] + dy[:-1] + EPS))[None, :, None]
    pg[2][:, 1:, :] = -2.0 * V[:, 1:, :] * gy
    pg[3][:, :-1, :] = -2.0 * V[:, :-1, :] * gy
    F = geo.fw[2:nz + 1]
    gz = F / (F + EPS) * F / (F + EPS) * (P[2:nz + 1, 1:-1, 1:-1] - P[1:nz, 1:-1, 1:-1]) / (
        dz[1:] + dz[:-1] + EPS)[:, None, None]
    pg[4][1:] = -2.0 * V[1:] * gz
    pg[5][:-1] = -2.0 * V[:-1] * gz
    # periodic sides: the neighbour loop ('iw'/'ie'/'is'/'in'), no DUU factor,
    # the partner cell's width in the denominator; p's halos hold the images
    if g.periodic_x:
        Fb = geo.fu[:, :, 1]
        gw = Fb / (Fb + EPS) * (P[1:-1, 1:-1, 1] - P[1:-1, 1:-1, 0]) / (1.0 * (dx[0] + dx[-1] + EPS))
        pg[0][:, :, 0] = -2.0 * V[:, :, 0] * gw
        Fb = geo.fu[:, :, nx + 1]
        ge = Fb / (Fb + EPS) * (P[1:-1, 1:-1, nx + 1] - P[1:-1, 1:-1, nx]) / (1.0 * (dx[-1] + dx[0] + EPS))
        pg[1][:, :, -1] = -2.0 * V[:, :, -1] * ge
    if g.periodic_y:
        Fb = geo.fv[:, 1, :]
        gs = Fb / (Fb + EPS) * (P[1:-1, 1, 1:-1] - P[1:-1, 0, 1:-1]) / (1.0 * (dy[0] + dy[-1] + EPS))
        pg[2][:, 0, :] = -2.0 * V[:, 0, :] * gs
        Fb = geo.fv[:, ny + 1, :]
        gn = Fb / (Fb + EPS) * (P[1:-1, ny + 1, 1:-1] - P[1:-1, ny, 1:-1]) / (1.0 * (dy[0] + dy[-1] + EPS))
        pg[3][:, -1, :] = -2.0 * V[:, -1, :] * gn
    R = rho[1:-1, 1:-1, 1:-1]
    rl = F / (F + EPS) * (dz[:-1, None, None] * R[:-1] + dz[1:, None, None] * R[1:]) / (
        dz[:-1] + dz[1:] + EPS)[:, None, None]
    bu = [np.zeros((nz, ny, nx)) for _ in range(2)]
    bu[0][1:] = -rl * grav
    bu[1][:-1] = -rl * grav
    return pg, bu


def diffusion(geo, c, rho, dh, dv):
    """DiffusionCompute (ADVECT/Diffusion_Mod.f90:11-275) for one component
    on the padded box, in gather form: each cell sums its face fluxes in the
    reference's order (x left, x right, y left, y right, z left, z right),
    then f*VolC/(VolC+Eps).  Periodic sides carry half a flux from each side
    (the halo cells receive theirs); walls use the interior coefficient."""
    g = geo.grid
    nx, ny, nz = g.nx, g.ny, g.nz
    V = geo.volc
    phi = c / (rho + EPS)
    f = np.zeros_like(c)

    def face(axis):
        # coefficient arrays of the faces 0..n along axis between padded cells (f, f+1)
        per = (g.periodic_x, g.periodic_y, g.periodic_z)[axis]
        D = dv if axis == 2 else dh
        if axis == 0:
            F = geo.fu[:, :, 1:nx + 2]
            sl = lambda a, o: a[1:-1, 1:-1, o:o + nx + 1]
        elif axis == 1:
            F = geo.fv[:, 1:ny + 2, :]
            sl = lambda a, o: a[1:-1, o:o + ny + 1, 1:-1]
        else:
            F = geo.fw[1:nz + 2]
            sl = lambda a, o: a[o:o + nz + 1, 1:-1, 1:-1]
        VL, VR, DL, DR = sl(V, 0), sl(V, 1), sl(D, 0), sl(D, 1)
        dfm = (DL * VR + DR * VL) / (VL + VR + EPS)
        npax = 2 - axis  # numpy axis of the face direction (arrays are (z, y, x))
        n = F.shape[npax]
        idx = np.arange(n).reshape([-1 if a == npax else 1 for a in range(3)])
        if per:
            DR_ = dfm
            two = np.where((idx >= 1) & (idx <= n - 2), 2.0, 1.0)
        else:
            DR_ = np.where(idx == 0, DR, np.where(idx == n - 1, DL, dfm))
            two = 2.0
        flux = two * DR_ * F * F / (VL + VR + EPS) * (sl(phi, 1) - sl(phi, 0))
        return flux, per

    out = f.copy()
    I = (slice(1, -1),) * 3
    fx, px = face(0)
    fy, py = face(1)
    fz, pz = face(2)
    a = out[I]
    a = a - fx[:, :, :-1]
    a = a + fx[:, :, 1:]
    a = a - fy[:, :-1, :]
    a = a + fy[:, 1:, :]
    a = a - fz[:-1]
    a = a + fz[1:]
    out[I] = a
    if px:
        out[1:-1, 1:-1, 0] += fx[:, :, 0]
        out[1:-1, 1:-1, -1] -= fx[:, :, -1]
    if py:
        out[1:-1, 0, 1:-1] += fy[:, 0, :]
        out[1:-1, -1, 1:-1] -= fy[:, -1, :]
    if pz:
        out[0, 1:-1, 1:-1] += fz[0]
        out[-1, 1:-1, 1:-1] -= fz[-1]
    return out * V / (V + EPS)
