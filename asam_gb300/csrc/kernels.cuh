// Templated CUDA kernels of the transport stage.  Included by k64.cu (FP64,
// compiled with -fmad=false so every product and sum is rounded exactly as in
// the reference Fortran) and by k32.cu (FP32 inner solver of the refined mode).
// Everything here lives in an anonymous namespace: each translation unit gets
// its own copy, and the launch wrappers of launch.h are the only exports.
#pragma once
#include "asam_common.cuh"
#include "launch.h"

namespace {

using asam::Dims;
using asam::kMaxComp;
using asam::GsTileSched;
using asam::MomSrc;
using asam::DiffSrc;
using asam::WallIn;

template <typename T>
__device__ __forceinline__ T eps_t() {
  return (T)1.0e-30;
}

// Correctly rounded quotient x/d from a precomputed rinv = RN(1/d), by one
// FMA correction step (Markstein, "Computation of elementary functions on the
// IBM RISC System/6000 processor", IBM J. Res. Dev. 34, 1990): q0 = RN(x*rinv),
// e = x - q0*d (exact with an FMA), q = RN(q0 + e*rinv).  Agreement with the
// IEEE quotient is checked on the device by asam_probe_div.
__device__ __forceinline__ double div_rn(double x, double d, double rinv) {
  const double q0 = __dmul_rn(x, rinv);
  const double e = __fma_rn(-q0, d, x);
  return __fma_rn(e, rinv, q0);
}
__device__ __forceinline__ float div_rn(float x, float d, float rinv) {
  const float q0 = __fmul_rn(x, rinv);
  const float e = __fmaf_rn(-q0, d, x);
  return __fmaf_rn(e, rinv, q0);
}

// ---------------------------------------------------------------------------
// Limiter and stencil coefficients: ADVECT/Advection_Mod.f90:2118-2134
// (k1F, k2F, PhiLim with MethAdv='Koren').
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T k1f(T hL, T hC, T hR) {
  const T e = eps_t<T>();
  return (hC / (hC + hR + e)) * ((hL + hC) / (hL + hC + hR + e));
}
template <typename T>
__device__ __forceinline__ T k2f(T hL, T hC, T hR) {
  const T e = eps_t<T>();
  return (hC / (hL + hC + e)) * (hR / (hL + hC + hR + e));
}
template <typename T>
__device__ __forceinline__ T koren(T r, T k1, T k2) {
  T a = k1 * r + k2;
  T m = a < (T)1 ? a : (T)1;
  m = r < m ? r : m;
  return (T)0 > m ? (T)0 : m;
}

using asam::GeomT;

// phi = c/(Rho+Eps) over the padded box, all components.  One IEEE
// reciprocal of Rho+Eps per cell, then the correctly rounded quotient per
// component (div_rn), identical to the reference's c/(Rho+Eps).
template <typename T>
__global__ void k_phi(Dims d, int ncomp, int rho_pos, const T* __restrict__ c, T* __restrict__ phi) {
  const size_t n = d.npad();
  const T e = eps_t<T>();
  const T* rho = c + (size_t)rho_pos * n;
  for (size_t P = blockIdx.x * (size_t)blockDim.x + threadIdx.x; P < n; P += (size_t)gridDim.x * blockDim.x) {
    const T rp = rho[P] + e;
    const T rr = (T)1 / rp;
    for (int ic = 0; ic < ncomp; ++ic) phi[ic * n + P] = div_rn(c[ic * n + P], rp, rr);
  }
}

// Per-face coefficients of the flux (geometry and face velocity only, so
// they are computed once when the velocities are set):
//   coef[0] = +/- Half*(ABS(u)+/-u)*F  (sign: + upwind cell left of the face,
//             - upwind cell right of it, 0 no flux in the reference's loop)
//   coef[1] = F_other/(F_other+Eps), coef[2] = k1, coef[3] = k2 of the upwind cell
//   mask bits: 1 VL<VC, 2 VR<VC (x only), 4 FL<FR, 8 FR<FL (blends of :868-871)
// with the upwind cell's VL, VC, VR, FL, FR as in ADVECT/Advection_Mod.f90:854-974.
template <typename T, int AXIS>
__global__ void k_face_coef(Dims d, GeomT<T> g, T* __restrict__ coef, unsigned char* __restrict__ mask) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const int ex = AXIS == 0 ? nx + 1 : nx;
  const int ey = AXIS == 1 ? ny + 1 : ny;
  const int ez = AXIS == 2 ? nz + 1 : nz;
  const size_t nface = (size_t)ex * ey * ez;
  const T e = eps_t<T>();
  const T half = (T)0.5;
  for (size_t f = blockIdx.x * (size_t)blockDim.x + threadIdx.x; f < nface; f += (size_t)gridDim.x * blockDim.x) {
    const int a = (int)(f % ex);
    const size_t rest = f / ex;
    const int b = (int)(rest % ey);
    const int cc = (int)(rest / ey);
    int i, j, k;
    T vel;
    if (AXIS == 0) {
      i = a; j = b + 1; k = cc + 1;
      vel = g.uf[d.UF(i, j, k)];
    } else if (AXIS == 1) {
      i = a + 1; j = b; k = cc + 1;
      vel = g.vf[d.VF(i, j, k)];
    } else {
      i = a + 1; j = b + 1; k = cc;
      vel = g.wf[d.WF(i, j, k)];
    }
    const int s = AXIS == 0 ? i : (AXIS == 1 ? j : k);
    const int smax = AXIS == 0 ? nx : (AXIS == 1 ? ny : nz);
    int orient = 0;
    if (vel > (T)0 && s >= 1) orient = 1;           // upwind = left cell, its right face
    else if (vel < (T)0 && s + 1 <= smax) orient = -1;  // upwind = right cell, its left face
    T c0 = (T)0, c1 = (T)0, c2 = (T)0, c3 = (T)0;
    unsigned char m = 0;
    if (orient != 0) {
      const int ci = i + (orient < 0 && AXIS == 0), cj = j + (orient < 0 && AXIS == 1),
                ck = k + (orient < 0 && AXIS == 2);
      const size_t PC = d.P(ci, cj, ck);
      const size_t stride = AXIS == 0 ? 1 : (AXIS == 1 ? (size_t)d.NX() : (size_t)d.NX() * d.NY());
      T FL, FR;
      if (AXIS == 0) {
        FR = g.fu[d.FU(ci, cj, ck)];
        FL = g.fu[d.FU(ci - 1, cj, ck)];
      } else if (AXIS == 1) {
        FR = g.fv[d.FV(ci, cj, ck)];
        FL = g.fv[d.FV(ci, cj - 1, ck)];
      } else {
        FR = g.fw[d.FW(ci, cj, ck)];
        FL = g.fw[d.FW(ci, cj, ck - 1)];
      }
      const T VL = g.volc[PC - stride], VC = g.volc[PC], VR = g.volc[PC + stride];
      if (orient > 0) {
        c0 = half * (fabs(vel) + vel) * FR;
        c1 = FL / (FL + e);
        c2 = k1f(VL, VC, VR);
        c3 = k2f(VL, VC, VR);
      } else {
        c0 = -(half * (fabs(vel) - vel) * FL);
        c1 = FR / (FR + e);
        c2 = k1f(VR, VC, VL);
        c3 = k2f(VR, VC, VL);
      }
      if (AXIS == 0 && VL < VC) m |= 1;
      if (AXIS == 0 && VR < VC) m |= 2;
      if (FL < FR) m |= 4;
      if (FR < FL) m |= 8;
    }
    coef[0 * nface + f] = c0;
    coef[1 * nface + f] = c1;
    coef[2 * nface + f] = c2;
    coef[3 * nface + f] = c3;
    mask[f] = m;
  }
}

// Face fluxes.  axis 0: x faces (i in [0,nx], j,k interior) stored at UF(i,j,k);
// axis 1: y faces at VF; axis 2: z faces at WF.  gout[ic*nface + face] holds the
// flux the reference's loop computes for the upwind interior cell of the face
// (zero when the upwind cell is a halo cell or the velocity is zero):
//   Half*(ABS(u)+-u)*F*(cC + Fo/(Fo+Eps)*PhiLim(r,k1,k2,...))   (:875-894)
template <typename T, int AXIS>
__global__ void k_face_flux(Dims d, GeomT<T> g, int ncomp, const T* __restrict__ coef,
                            const unsigned char* __restrict__ mask, const T* __restrict__ phi,
                            T* __restrict__ gout) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const int ex = AXIS == 0 ? nx + 1 : nx;
  const int ey = AXIS == 1 ? ny + 1 : ny;
  const int ez = AXIS == 2 ? nz + 1 : nz;
  const size_t nface = (size_t)ex * ey * ez;
  const size_t n = d.npad();
  const T e = eps_t<T>();
  for (size_t f = blockIdx.x * (size_t)blockDim.x + threadIdx.x; f < nface; f += (size_t)gridDim.x * blockDim.x) {
    const T pref_s = coef[f];
    if (pref_s == (T)0) {
      for (int ic = 0; ic < ncomp; ++ic) gout[ic * nface + f] = (T)0;
      continue;
    }
    const bool right = pref_s > (T)0;
    const T pref = right ? pref_s : -pref_s;
    const T ratio = coef[nface + f], k1 = coef[2 * nface + f], k2 = coef[3 * nface + f];
    const unsigned char m = mask[f];
    const int a = (int)(f % ex);
    const size_t rest = f / ex;
    const int b = (int)(rest % ey);
    const int cc = (int)(rest / ey);
    int ci, cj, ck;
    if (AXIS == 0) {
      ci = a + !right; cj = b + 1; ck = cc + 1;
    } else if (AXIS == 1) {
      ci = a + 1; cj = b + !right; ck = cc + 1;
    } else {
      ci = a + 1; cj = b + 1; ck = cc + !right;
    }
    const size_t PC = d.P(ci, cj, ck);
    const size_t stride = AXIS == 0 ? 1 : (AXIS == 1 ? (size_t)d.NX() : (size_t)d.NX() * d.NY());
    const size_t PL = PC - stride, PR = PC + stride;
    T VL = (T)0, VC = (T)0, VR = (T)0, FL = (T)0, FR = (T)0;
    if (m) {  // cut-cell blends (rare): geometry of the upwind cell
      VL = g.volc[PL];
      VC = g.volc[PC];
      VR = g.volc[PR];
      if (AXIS == 0) {
        FR = g.fu[d.FU(ci, cj, ck)];
        FL = g.fu[d.FU(ci - 1, cj, ck)];
      } else if (AXIS == 1) {
        FR = g.fv[d.FV(ci, cj, ck)];
        FL = g.fv[d.FV(ci, cj - 1, ck)];
      } else {
        FR = g.fw[d.FW(ci, cj, ck)];
        FL = g.fw[d.FW(ci, cj, ck - 1)];
      }
    }
    for (int ic = 0; ic < ncomp; ++ic) {
      const T* ph = phi + ic * n;
      T cL = ph[PL], cC = ph[PC], cR = ph[PR];
      if (m) {
        if (m & 1) cL = ((VC - VL) * cC + VL * cL) / VC;
        if (m & 2) cR = ((VC - VR) * cC + VR * cR) / VC;
        if (m & 4) cL = ((FR - FL) * cC + FL * cL) / FR;
        if (m & 8) cR = ((FL - FR) * cC + FR * cR) / FL;
      }
      T flux;
      if (right) {
        const T r = (cR - cC + e) / ((cC - cL) + e);
        flux = pref * (cC + ratio * (koren(r, k1, k2) * (cC - cL)));
      } else {
        const T r = (cC - cL + e) / ((cR - cC) + e);
        flux = pref * (cC + ratio * (koren(r, k1, k2) * (cC - cR)));
      }
      gout[ic * nface + f] = flux;
    }
  }
}

// Grad of PGradComputeCFull (ADVECT/PressureGrad_Mod.f90:252-276) on the
// interior face between padded cells (i,j,k) and their +1 neighbour along
// axis, with DUU = F/(F+Eps) of IniJacAccGrav (MULTI/JacAccGrav_Mod.f90:297):
//   DUU*F/(F+Eps)*(p(+1)-p)/(Metr*(d(+1)+d+Eps)), evaluated left to right.
template <typename T>
__device__ __forceinline__ T pgrad_face(const Dims& d, const GeomT<T>& g, const MomSrc<T>& ms, int axis, int i, int j,
                                        int k) {
  const T e = eps_t<T>();
  if (axis == 0) {
    const T F = g.fu[d.FU(i, j, k)];
    const T du = F / (F + e);
    return du * F / (F + e) * (ms.p[d.P(i + 1, j, k)] - ms.p[d.P(i, j, k)]) /
           (ms.mxy[j - 1] * (ms.dx[i] + ms.dx[i - 1] + e));
  }
  if (axis == 1) {
    const T F = g.fv[d.FV(i, j, k)];
    const T du = F / (F + e);
    return du * F / (F + e) * (ms.p[d.P(i, j + 1, k)] - ms.p[d.P(i, j, k)]) /
           (ms.myx[i - 1] * (ms.dy[j] + ms.dy[j - 1] + e));
  }
  const T F = g.fw[d.FW(i, j, k)];
  const T du = F / (F + e);
  return du * F / (F + e) * (ms.p[d.P(i, j, k + 1)] - ms.p[d.P(i, j, k)]) / (ms.dz[k] + ms.dz[k - 1] + e);
}

// Grad of PGradComputeCFull's neighbour loop on a periodic side ('iw', 'ie',
// 'is', 'in' with equal refinement, ADVECT/PressureGrad_Mod.f90:307-313,
// 340-346, 373-379, 406-412): no DUU factor, and the width dLoc of the
// partner cell across the side (the block's own last cell for 'iw', its
// first for 'ie'); p's halo holds the periodic image.  side 0 W, 1 E, 2 S, 3 N.
template <typename T>
__device__ __forceinline__ T pgrad_side(const Dims& d, const GeomT<T>& g, const MomSrc<T>& ms, int side, int i, int j,
                                        int k) {
  const T e = eps_t<T>();
  const int nx = d.nx, ny = d.ny;
  if (side == 0) {
    const T F = g.fu[d.FU(0, j, k)];
    return F / (F + e) * (ms.p[d.P(1, j, k)] - ms.p[d.P(0, j, k)]) / (ms.mxy[j - 1] * (ms.dx[0] + ms.dx[nx - 1] + e));
  }
  if (side == 1) {
    const T F = g.fu[d.FU(nx, j, k)];
    return F / (F + e) * (ms.p[d.P(nx + 1, j, k)] - ms.p[d.P(nx, j, k)]) /
           (ms.mxy[j - 1] * (ms.dx[nx - 1] + ms.dx[0] + e));
  }
  if (side == 2) {
    const T F = g.fv[d.FV(i, 0, k)];
    return F / (F + e) * (ms.p[d.P(i, 1, k)] - ms.p[d.P(i, 0, k)]) / (ms.myx[i - 1] * (ms.dy[0] + ms.dy[ny - 1] + e));
  }
  const T F = g.fv[d.FV(i, ny, k)];
  return F / (F + e) * (ms.p[d.P(i, ny + 1, k)] - ms.p[d.P(i, ny, k)]) /
         (ms.myx[i - 1] * (ms.dy[0] + ms.dy[ny - 1] + e));
}

// RhoLoc of AuftriebDryComputeLRFull (ADVECT/Buoyancy_Mod.f90:51-63) on the
// face between levels k and k+1.
template <typename T>
__device__ __forceinline__ T buoy_rho_face(const Dims& d, const GeomT<T>& g, const MomSrc<T>& ms, int i, int j,
                                           int k) {
  const T e = eps_t<T>();
  const T F = g.fw[d.FW(i, j, k)];
  return F / (F + e) * (ms.dz[k - 1] * ms.rho[d.P(i, j, k)] + ms.dz[k] * ms.rho[d.P(i, j, k + 1)]) /
         (ms.dz[k - 1] + ms.dz[k] + e);
}

// Gather of the face fluxes into the cell right-hand side in the exact order
// in which the reference's scatter loop touches f(ix,iy,iz), then (wl set)
// the first-order inflow through the faces of the outer walls from their
// halo cells and the zeroed wall halos, the zero-volume mask (:1045-1051),
// the periodic ExchangeFlux (neighbour order W,E,S,N,B,T) and AdvectionScale
// (:2888-2898).  One thread per padded cell.
// kMom adds the momentum sources of ms (closed or periodic x/y sides); kDiff the diffusion
// fluxes of df with DiffusionCompute's second zero-volume mask (the halo
// cells of a periodic side included, before ExchangeFlux reads them).
template <typename T, bool kMom = false, bool kDiff = false>
__global__ void k_flux_gather(Dims d, GeomT<T> g, int ncomp, const T* __restrict__ gx, const T* __restrict__ gy,
                              const T* __restrict__ gz, const T* __restrict__ rvol, T* __restrict__ f,
                              MomSrc<T> ms, DiffSrc<T> df = DiffSrc<T>{}, WallIn<T> wl = WallIn<T>{}) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const int NX = d.NX(), NY = d.NY(), NZ = d.NZ();
  const size_t n = d.npad();
  const size_t nfx = (size_t)(nx + 1) * ny * nz, nfy = (size_t)nx * (ny + 1) * nz, nfz = (size_t)nx * ny * (nz + 1);
  const T e = eps_t<T>();
  for (size_t P = blockIdx.x * (size_t)blockDim.x + threadIdx.x; P < n; P += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(P % NX);
    const int j = (int)((P / NX) % NY);
    const int k = (int)(P / ((size_t)NX * NY));
    const T V = g.volc[P];
    const T Ve = V + e, rV = rvol[P];
    const bool ii = i >= 1 && i <= nx, jj = j >= 1 && j <= ny, kk = k >= 1 && k <= nz;
    if (ii && jj && kk) {
      const size_t fxL = d.UF(i - 1, j, k), fxR = d.UF(i, j, k);
      const size_t fyL = d.VF(i, j - 1, k), fyR = d.VF(i, j, k);
      const size_t fzL = d.WF(i, j, k - 1), fzR = d.WF(i, j, k);
      const T uL = g.uf[fxL], uR = g.uf[fxR];
      const T vL = g.vf[fyL], vR = g.vf[fyR];
      const T wL = g.wf[fzL], wR = g.wf[fzR];
      // periodic exchange sources (masked halo values of the opposite side)
      const bool exW = d.per_x && i == 1, exE = d.per_x && i == nx;
      const bool exS = d.per_y && j == 1, exN = d.per_y && j == ny;
      const bool exB = d.per_z && k == 1, exT = d.per_z && k == nz;
      for (int ic = 0; ic < ncomp; ++ic) {
        const T* GX = gx + ic * nfx;
        const T* GY = gy + ic * nfy;
        const T* GZ = gz + ic * nfz;
        T a = (T)0;
        if (wL > (T)0) a = a + GZ[fzL];  // FluxZR of the cell below
        if (vL > (T)0) a = a + GY[fyL];  // FluxYR of the cell south
        if (uL > (T)0) a = a + GX[fxL];  // FluxXR of the cell west
        if (uL < (T)0) a = a - GX[fxL];  // own x-left
        if (uR > (T)0) a = a - GX[fxR];  // own x-right
        if (vL < (T)0) a = a - GY[fyL];
        if (vR > (T)0) a = a - GY[fyR];
        if (wL < (T)0) a = a - GZ[fzL];
        if (wR > (T)0) a = a - GZ[fzR];
        if (uR < (T)0) a = a + GX[fxR];  // FluxXL of the cell east
        if (vR < (T)0) a = a + GY[fyR];
        if (wR < (T)0) a = a + GZ[fzR];
        if (wl.c) {  // inflow through the outer walls' faces, W, E, S, N, B, T (:975-1044)
          const T* cc = wl.c + ic * n;
          const T half = (T)0.5;
          if (!d.per_x && i == 1) {
            const size_t H = d.P(0, j, k);
            a = a + half * (fabs(uL) + uL) * cc[H] / (wl.rho[H] + e) * g.fu[d.FU(0, j, k)];
          }
          if (!d.per_x && i == nx) {
            const size_t H = d.P(nx + 1, j, k);
            a = a + half * (fabs(uR) - uR) * cc[H] / (wl.rho[H] + e) * g.fu[d.FU(nx, j, k)];
          }
          if (!d.per_y && j == 1) {
            const size_t H = d.P(i, 0, k);
            a = a + half * (fabs(vL) + vL) * cc[H] / (wl.rho[H] + e) * g.fv[d.FV(i, 0, k)];
          }
          if (!d.per_y && j == ny) {
            const size_t H = d.P(i, ny + 1, k);
            a = a + half * (fabs(vR) - vR) * cc[H] / (wl.rho[H] + e) * g.fv[d.FV(i, ny, k)];
          }
          if (!d.per_z && k == 1) {  // the bottom divides by the interior cell's density
            const size_t H = d.P(i, j, 0);
            a = a + half * (fabs(wL) + wL) * cc[H] / (wl.rho[P] + e) * g.fw[d.FW(i, j, 0)];
          }
          if (!d.per_z && k == nz) {
            const size_t H = d.P(i, j, nz + 1);
            a = a + half * (fabs(wR) - wR) * cc[H] / (wl.rho[H] + e) * g.fw[d.FW(i, j, nz)];
          }
        }
        a = div_rn(a * V, Ve, rV);
        if (kDiff) {  // f(R) - Flux, f(L) + Flux per face, x then y then z; then the mask
          const T* ph = df.phi + ic * n;
          const T pc = ph[P];
          const bool ix0 = i >= 2, ix1 = i <= nx - 1;  // faces i-1 and i between two cells of the block
          const bool iy0 = j >= 2, iy1 = j <= ny - 1;
          const bool iz0 = k >= 2, iz1 = k <= nz - 1;
          const T kxl = df.kx[fxL], kxr = df.kx[fxR], kyl = df.ky[fyL], kyr = df.ky[fyR];
          const T kzl = df.kz[fzL], kzr = df.kz[fzR];
          a = a - ((ix0 || !d.per_x) ? (T)2 * kxl : kxl) * (pc - ph[P - 1]);
          a = a + ((ix1 || !d.per_x) ? (T)2 * kxr : kxr) * (ph[P + 1] - pc);
          a = a - ((iy0 || !d.per_y) ? (T)2 * kyl : kyl) * (pc - ph[P - (size_t)NX]);
          a = a + ((iy1 || !d.per_y) ? (T)2 * kyr : kyr) * (ph[P + (size_t)NX] - pc);
          a = a - ((iz0 || !d.per_z) ? (T)2 * kzl : kzl) * (pc - ph[P - (size_t)NX * NY]);
          a = a + ((iz1 || !d.per_z) ? (T)2 * kzr : kzr) * (ph[P + (size_t)NX * NY] - pc);
          a = div_rn(a * V, Ve, rV);
        }
        if (kMom && ms.pgrad) {  // uRhsL(ix+1) - Two*VolC(ix+1)*Grad, uRhsR(ix) - Two*VolC(ix)*Grad
          int axis = -1, lo = 0;
          if (ic == ms.pos[0] && i >= 2) axis = 0, lo = 1;
          else if (ic == ms.pos[1] && i <= nx - 1) axis = 0;
          else if (ic == ms.pos[2] && j >= 2) axis = 1, lo = 1;
          else if (ic == ms.pos[3] && j <= ny - 1) axis = 1;
          else if (ic == ms.pos[4] && k >= 2) axis = 2, lo = 1;
          else if (ic == ms.pos[5] && k <= nz - 1) axis = 2;
          if (axis >= 0) {
            const T gr = pgrad_face(d, g, ms, axis, i - (axis == 0 ? lo : 0), j - (axis == 1 ? lo : 0),
                                    k - (axis == 2 ? lo : 0));
            a = a - (T)2 * V * gr;
          } else {  // the shared face of a periodic side
            int side = -1;
            if (ic == ms.pos[0] && d.per_x) side = 0;
            else if (ic == ms.pos[1] && d.per_x) side = 1;
            else if (ic == ms.pos[2] && d.per_y) side = 2;
            else if (ic == ms.pos[3] && d.per_y) side = 3;
            if (side >= 0) a = a - (T)2 * V * pgrad_side(d, g, ms, side, i, j, k);
          }
        }
        if (exW) {
          const size_t PH = d.P(nx + 1, j, k), fh = d.UF(nx, j, k);
          T h = g.uf[fh] > (T)0 ? GX[fh] : (T)0;
          T VH = g.volc[PH];
          T hv = div_rn(h * VH, VH + e, rvol[PH]);
          if (kDiff) {  // the halo's diffusion deposit and second mask
            const T* ph = df.phi + ic * n;
            hv = hv - df.kx[fh] * (ph[PH] - ph[d.P(nx, j, k)]);
            hv = div_rn(hv * VH, VH + e, rvol[PH]);
          }
          a = a + hv;
        }
        if (exE) {
          const size_t PH = d.P(0, j, k), fh = d.UF(0, j, k);
          T h = g.uf[fh] < (T)0 ? GX[fh] : (T)0;
          T VH = g.volc[PH];
          T hv = div_rn(h * VH, VH + e, rvol[PH]);
          if (kDiff) {  // the halo's diffusion deposit and second mask
            const T* ph = df.phi + ic * n;
            hv = hv + df.kx[fh] * (ph[d.P(1, j, k)] - ph[PH]);
            hv = div_rn(hv * VH, VH + e, rvol[PH]);
          }
          a = a + hv;
        }
        if (exS) {
          const size_t PH = d.P(i, ny + 1, k), fh = d.VF(i, ny, k);
          T h = g.vf[fh] > (T)0 ? GY[fh] : (T)0;
          T VH = g.volc[PH];
          T hv = div_rn(h * VH, VH + e, rvol[PH]);
          if (kDiff) {  // the halo's diffusion deposit and second mask
            const T* ph = df.phi + ic * n;
            hv = hv - df.ky[fh] * (ph[PH] - ph[d.P(i, ny, k)]);
            hv = div_rn(hv * VH, VH + e, rvol[PH]);
          }
          a = a + hv;
        }
        if (exN) {
          const size_t PH = d.P(i, 0, k), fh = d.VF(i, 0, k);
          T h = g.vf[fh] < (T)0 ? GY[fh] : (T)0;
          T VH = g.volc[PH];
          T hv = div_rn(h * VH, VH + e, rvol[PH]);
          if (kDiff) {  // the halo's diffusion deposit and second mask
            const T* ph = df.phi + ic * n;
            hv = hv + df.ky[fh] * (ph[d.P(i, 1, k)] - ph[PH]);
            hv = div_rn(hv * VH, VH + e, rvol[PH]);
          }
          a = a + hv;
        }
        if (exB) {
          const size_t PH = d.P(i, j, nz + 1), fh = d.WF(i, j, nz);
          T h = g.wf[fh] > (T)0 ? GZ[fh] : (T)0;
          T VH = g.volc[PH];
          T hv = div_rn(h * VH, VH + e, rvol[PH]);
          if (kDiff) {  // the halo's diffusion deposit and second mask
            const T* ph = df.phi + ic * n;
            hv = hv - df.kz[fh] * (ph[PH] - ph[d.P(i, j, nz)]);
            hv = div_rn(hv * VH, VH + e, rvol[PH]);
          }
          a = a + hv;
        }
        if (exT) {
          const size_t PH = d.P(i, j, 0), fh = d.WF(i, j, 0);
          T h = g.wf[fh] < (T)0 ? GZ[fh] : (T)0;
          T VH = g.volc[PH];
          T hv = div_rn(h * VH, VH + e, rvol[PH]);
          if (kDiff) {  // the halo's diffusion deposit and second mask
            const T* ph = df.phi + ic * n;
            hv = hv + df.kz[fh] * (ph[d.P(i, j, 1)] - ph[PH]);
            hv = div_rn(hv * VH, VH + e, rvol[PH]);
          }
          a = a + hv;
        }
        T fv = div_rn(a, Ve, rV);
        if (kMom && ms.buoy) {  // fL(iz+1) - RhoLoc*Grav, fR(iz) - RhoLoc*Grav
          if (ic == ms.pos[4] && k >= 2) fv = fv - buoy_rho_face(d, g, ms, i, j, k - 1) * ms.grav;
          else if (ic == ms.pos[5] && k <= nz - 1) fv = fv - buoy_rho_face(d, g, ms, i, j, k) * ms.grav;
        }
        f[ic * n + P] = fv;
      }
    } else {
      // halo cell: only the face-halo cells next to the interior receive a flux
      int axis = -1;
      size_t fidx = 0;
      bool take_pos = false;
      if (jj && kk && (i == 0 || i == NX - 1)) {
        axis = 0;
        fidx = d.UF(i == 0 ? 0 : nx, j, k);
        take_pos = i != 0;
      } else if (ii && kk && (j == 0 || j == NY - 1)) {
        axis = 1;
        fidx = d.VF(i, j == 0 ? 0 : ny, k);
        take_pos = j != 0;
      } else if (ii && jj && (k == 0 || k == NZ - 1)) {
        axis = 2;
        fidx = d.WF(i, j, k == 0 ? 0 : nz);
        take_pos = k != 0;
      }
      T vel = (T)0;
      if (axis == 0) vel = g.uf[fidx];
      if (axis == 1) vel = g.vf[fidx];
      if (axis == 2) vel = g.wf[fidx];
      // an outer wall's face halo is zeroed after the inflow (:975-1044)
      const bool wall = (axis == 0 && !d.per_x) || (axis == 1 && !d.per_y) || (axis == 2 && !d.per_z);
      const bool has = axis >= 0 && !(wl.c && wall) && (take_pos ? vel > (T)0 : vel < (T)0);
      for (int ic = 0; ic < ncomp; ++ic) {
        T a = (T)0;
        if (has) {
          if (axis == 0) a = a + gx[ic * nfx + fidx];
          if (axis == 1) a = a + gy[ic * nfy + fidx];
          if (axis == 2) a = a + gz[ic * nfz + fidx];
        }
        a = div_rn(a * V, Ve, rV);
        if (kDiff) {  // periodic face halos receive the half flux of their face; every halo is masked again
          const T* ph = df.phi + ic * n;
          if (axis == 0 && d.per_x) {
            if (i == 0) a = a + df.kx[fidx] * (ph[P + 1] - ph[P]);
            else a = a - df.kx[fidx] * (ph[P] - ph[P - 1]);
          } else if (axis == 1 && d.per_y) {
            if (j == 0) a = a + df.ky[fidx] * (ph[P + (size_t)NX] - ph[P]);
            else a = a - df.ky[fidx] * (ph[P] - ph[P - (size_t)NX]);
          } else if (axis == 2 && d.per_z) {
            if (k == 0) a = a + df.kz[fidx] * (ph[P + (size_t)NX * NY] - ph[P]);
            else a = a - df.kz[fidx] * (ph[P] - ph[P - (size_t)NX * NY]);
          }
          a = div_rn(a * V, Ve, rV);
        }
        f[ic * n + P] = div_rn(a, Ve, rV);
      }
    }
  }
}

// Face coefficients of DiffusionCompute: K = DRhoF*F*F/(VL+VR+Eps), DRhoF =
// DF(D_L, VL, D_R, VR) = (D_L*VR + D_R*VL)/(VL+VR+Eps) on faces between two
// cells of the block or on a periodic side, the interior cell's D on an
// outer wall (ADVECT/Diffusion_Mod.f90:24-52 and the matching branches);
// D = DH on x and y faces, DV on z faces.
template <typename T>
__global__ void k_diff_coef(Dims d, GeomT<T> g, const T* __restrict__ dh, const T* __restrict__ dv,
                            T* __restrict__ kx, T* __restrict__ ky, T* __restrict__ kz) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const size_t nu = d.n_uf(), nv = d.n_vf(), nw = d.n_wf();
  const T e = eps_t<T>();
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < nu + nv + nw; q += (size_t)gridDim.x * blockDim.x) {
    size_t L, R;
    T F;
    bool wall_lo, wall_hi;
    const T* D;
    T* out;
    size_t o;
    if (q < nu) {
      const int i = (int)(q % (nx + 1)), j = (int)((q / (nx + 1)) % ny) + 1, k = (int)(q / ((size_t)(nx + 1) * ny)) + 1;
      L = d.P(i, j, k);
      R = d.P(i + 1, j, k);
      F = g.fu[d.FU(i, j, k)];
      wall_lo = !d.per_x && i == 0;
      wall_hi = !d.per_x && i == nx;
      D = dh;
      out = kx;
      o = q;
    } else if (q < nu + nv) {
      o = q - nu;
      const int i = (int)(o % nx) + 1, j = (int)((o / nx) % (ny + 1)), k = (int)(o / ((size_t)nx * (ny + 1))) + 1;
      L = d.P(i, j, k);
      R = d.P(i, j + 1, k);
      F = g.fv[d.FV(i, j, k)];
      wall_lo = !d.per_y && j == 0;
      wall_hi = !d.per_y && j == ny;
      D = dh;
      out = ky;
    } else {
      o = q - nu - nv;
      const int i = (int)(o % nx) + 1, j = (int)((o / nx) % ny) + 1, k = (int)(o / ((size_t)nx * ny));
      L = d.P(i, j, k);
      R = d.P(i, j, k + 1);
      F = g.fw[d.FW(i, j, k)];
      wall_lo = !d.per_z && k == 0;
      wall_hi = !d.per_z && k == nz;
      D = dv;
      out = kz;
    }
    const T VL = g.volc[L], VR = g.volc[R];
    T DRhoF;
    if (wall_lo) DRhoF = D[R];
    else if (wall_hi) DRhoF = D[L];
    else DRhoF = (D[L] * VR + D[R] * VL) / (VL + VR + e);
    out[o] = DRhoF * F * F / (VL + VR + e);
  }
}

// rv = 1/(v + Eps) over n values (IEEE division)
template <typename T>
__global__ void k_recip_eps(size_t len, const T* __restrict__ v, T* __restrict__ rv) {
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < len; q += (size_t)gridDim.x * blockDim.x)
    rv[q] = (T)1 / (v[q] + eps_t<T>());
}

// DivCompute, ADVECT/Advection_Mod.f90:2901-2916 (rhs accumulated)
template <typename T>
__global__ void k_div(Dims d, GeomT<T> g, T* __restrict__ rhs) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const size_t n = (size_t)nx * ny * nz;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
    int i = (int)(q % nx) + 1;
    int j = (int)((q / nx) % ny) + 1;
    int k = (int)(q / ((size_t)nx * ny)) + 1;
    size_t P = d.P(i, j, k);
    rhs[P] = rhs[P] - (g.uf[d.UF(i, j, k)] * g.fu[d.FU(i, j, k)] - g.uf[d.UF(i - 1, j, k)] * g.fu[d.FU(i - 1, j, k)] +
                       g.vf[d.VF(i, j, k)] * g.fv[d.FV(i, j, k)] - g.vf[d.VF(i, j - 1, k)] * g.fv[d.FV(i, j - 1, k)] +
                       g.wf[d.WF(i, j, k)] * g.fw[d.FW(i, j, k)] - g.wf[d.WF(i, j, k - 1)] * g.fw[d.FW(i, j, k - 1)]);
  }
}

// ---------------------------------------------------------------------------
// Jacobian: JacAdvectionCompute (ADVECT/Advection_Mod.f90:2220-2872) followed by
// JacScaleCompute (ADVECT/Function_Mod.f90:1782-1862), one thread per padded
// cell computing its column of the 7-diagonal matrix in the reference's
// accumulation order.
// ---------------------------------------------------------------------------
// Half*(ABS(u)+/-u)*F/V/(Rho+Eps), both divisions correctly rounded from the
// precomputed reciprocals of V (= VolC+Eps of that cell: rvol) and of
// Rho+Eps (one per column), so the result is the reference's expression
template <typename T>
__device__ __forceinline__ T jac_term(T vel, bool plus, T F, T Vden, T rVden, T rhoe, T rrhoe) {
  const T half = (T)0.5;
  T s = plus ? (fabs(vel) + vel) : (fabs(vel) - vel);
  return div_rn(div_rn(half * s * F, Vden, rVden), rhoe, rrhoe);
}

template <typename T>
__global__ void k_jac(Dims d, GeomT<T> g, const T* __restrict__ rho, const T* __restrict__ rvol, T bdt,
                      T* __restrict__ val, const T* __restrict__ dkx = nullptr, const T* __restrict__ dky = nullptr,
                      const T* __restrict__ dkz = nullptr) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const int NX = d.NX(), NY = d.NY();
  const size_t n = d.npad();
  const T e = eps_t<T>();
  const size_t sx = 1, sy = (size_t)NX, sz = (size_t)NX * NY;
  for (size_t P = blockIdx.x * (size_t)blockDim.x + threadIdx.x; P < n; P += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(P % NX);
    const int j = (int)((P / NX) % NY);
    const int k = (int)(P / ((size_t)NX * NY));
    const bool ii = i >= 1 && i <= nx, jj = j >= 1 && j <= ny, kk = k >= 1 && k <= nz;
    const T rP = rho[P];
    const T rPe = rP + e, rrP = (T)1 / rPe;
    const T VP = g.volc[P] + e, rVP = rvol[P];
    T v[7] = {(T)0, (T)0, (T)0, (T)0, (T)0, (T)0, (T)0};
    // face activity: interior faces, plus boundary faces of periodic sides
    auto actx = [&](int fi) { return jj && kk && fi >= 0 && fi <= nx && ((fi >= 1 && fi <= nx - 1) || d.per_x); };
    auto acty = [&](int fj) { return ii && kk && fj >= 0 && fj <= ny && ((fj >= 1 && fj <= ny - 1) || d.per_y); };
    auto actz = [&](int fk) { return ii && jj && fk >= 0 && fk <= nz && ((fk >= 1 && fk <= nz - 1) || d.per_z); };
    // off-diagonals (each a single term)
    if (actx(i)) v[2] = v[2] + jac_term(g.uf[d.UF(i, j, k)], true, g.fu[d.FU(i, j, k)], g.volc[P + sx] + e, rvol[P + sx], rPe, rrP);
    if (actx(i - 1))
      v[4] = v[4] + jac_term(g.uf[d.UF(i - 1, j, k)], false, g.fu[d.FU(i - 1, j, k)], g.volc[P - sx] + e, rvol[P - sx], rPe, rrP);
    if (acty(j)) v[1] = v[1] + jac_term(g.vf[d.VF(i, j, k)], true, g.fv[d.FV(i, j, k)], g.volc[P + sy] + e, rvol[P + sy], rPe, rrP);
    if (acty(j - 1))
      v[5] = v[5] + jac_term(g.vf[d.VF(i, j - 1, k)], false, g.fv[d.FV(i, j - 1, k)], g.volc[P - sy] + e, rvol[P - sy], rPe, rrP);
    if (actz(k)) v[0] = v[0] + jac_term(g.wf[d.WF(i, j, k)], true, g.fw[d.FW(i, j, k)], g.volc[P + sz] + e, rvol[P + sz], rPe, rrP);
    if (actz(k - 1))
      v[6] = v[6] + jac_term(g.wf[d.WF(i, j, k - 1)], false, g.fw[d.FW(i, j, k - 1)], g.volc[P - sz] + e, rvol[P - sz], rPe, rrP);
    // diagonal: interior loops x, y, z (face left of P then face right of P)
    T dg = (T)0;
    if (jj && kk && i - 1 >= 1 && i - 1 <= nx - 1)
      dg = dg - jac_term(g.uf[d.UF(i - 1, j, k)], false, g.fu[d.FU(i - 1, j, k)], VP, rVP, rPe, rrP);
    if (jj && kk && i >= 1 && i <= nx - 1) dg = dg - jac_term(g.uf[d.UF(i, j, k)], true, g.fu[d.FU(i, j, k)], VP, rVP, rPe, rrP);
    if (ii && kk && j - 1 >= 1 && j - 1 <= ny - 1)
      dg = dg - jac_term(g.vf[d.VF(i, j - 1, k)], false, g.fv[d.FV(i, j - 1, k)], VP, rVP, rPe, rrP);
    if (ii && kk && j >= 1 && j <= ny - 1) dg = dg - jac_term(g.vf[d.VF(i, j, k)], true, g.fv[d.FV(i, j, k)], VP, rVP, rPe, rrP);
    if (ii && jj && k - 1 >= 1 && k - 1 <= nz - 1)
      dg = dg - jac_term(g.wf[d.WF(i, j, k - 1)], false, g.fw[d.FW(i, j, k - 1)], VP, rVP, rPe, rrP);
    if (ii && jj && k >= 1 && k <= nz - 1) dg = dg - jac_term(g.wf[d.WF(i, j, k)], true, g.fw[d.FW(i, j, k)], VP, rVP, rPe, rrP);
    // neighbour branches W, E, S, N, B, T of a periodic block
    if (d.per_x && jj && kk) {
      if (i == 0) dg = dg - jac_term(g.uf[d.UF(0, j, k)], true, g.fu[d.FU(0, j, k)], VP, rVP, rPe, rrP);
      if (i == 1) dg = dg - jac_term(g.uf[d.UF(0, j, k)], false, g.fu[d.FU(0, j, k)], VP, rVP, rPe, rrP);
      if (i == nx) dg = dg - jac_term(g.uf[d.UF(nx, j, k)], true, g.fu[d.FU(nx, j, k)], VP, rVP, rPe, rrP);
      if (i == nx + 1) dg = dg - jac_term(g.uf[d.UF(nx, j, k)], false, g.fu[d.FU(nx, j, k)], VP, rVP, rPe, rrP);
    }
    // outer walls 'ow'/'oe' (ADVECT/Advection_Mod.f90:2390-2410, 2469-2489): the
    // outflow through the wall face on the interior cell's diagonal
    if (!d.per_x && jj && kk) {
      if (i == 1) dg = dg - jac_term(g.uf[d.UF(0, j, k)], false, g.fu[d.FU(0, j, k)], VP, rVP, rPe, rrP);
      if (i == nx) dg = dg - jac_term(g.uf[d.UF(nx, j, k)], true, g.fu[d.FU(nx, j, k)], VP, rVP, rPe, rrP);
    }
    if (d.per_y && ii && kk) {
      if (j == 0) dg = dg - jac_term(g.vf[d.VF(i, 0, k)], true, g.fv[d.FV(i, 0, k)], VP, rVP, rPe, rrP);
      if (j == 1) dg = dg - jac_term(g.vf[d.VF(i, 0, k)], false, g.fv[d.FV(i, 0, k)], VP, rVP, rPe, rrP);
      if (j == ny) dg = dg - jac_term(g.vf[d.VF(i, ny, k)], true, g.fv[d.FV(i, ny, k)], VP, rVP, rPe, rrP);
      if (j == ny + 1) dg = dg - jac_term(g.vf[d.VF(i, ny, k)], false, g.fv[d.FV(i, ny, k)], VP, rVP, rPe, rrP);
    }
    if (!d.per_y && ii && kk) {  // 'os'/'on'
      if (j == 1) dg = dg - jac_term(g.vf[d.VF(i, 0, k)], false, g.fv[d.FV(i, 0, k)], VP, rVP, rPe, rrP);
      if (j == ny) dg = dg - jac_term(g.vf[d.VF(i, ny, k)], true, g.fv[d.FV(i, ny, k)], VP, rVP, rPe, rrP);
    }
    if (d.per_z && ii && jj) {
      if (k == 0) dg = dg - jac_term(g.wf[d.WF(i, j, 0)], true, g.fw[d.FW(i, j, 0)], VP, rVP, rPe, rrP);
      if (k == 1) dg = dg - jac_term(g.wf[d.WF(i, j, 0)], false, g.fw[d.FW(i, j, 0)], VP, rVP, rPe, rrP);
      if (k == nz) dg = dg - jac_term(g.wf[d.WF(i, j, nz)], true, g.fw[d.FW(i, j, nz)], VP, rVP, rPe, rrP);
      if (k == nz + 1) dg = dg - jac_term(g.wf[d.WF(i, j, nz)], false, g.fw[d.FW(i, j, nz)], VP, rVP, rPe, rrP);
    }
    if (!d.per_z && ii && jj) {  // 'ob'/'ot'
      if (k == 1) dg = dg - jac_term(g.wf[d.WF(i, j, 0)], false, g.fw[d.FW(i, j, 0)], VP, rVP, rPe, rrP);
      if (k == nz) dg = dg - jac_term(g.wf[d.WF(i, j, nz)], true, g.fw[d.FW(i, j, nz)], VP, rVP, rPe, rrP);
    }
    // JacDiffusionCompute (ADVECT/Diffusion_Mod.f90:1504-1708): per face with
    // a neighbour Temp = 2K; the off-diagonal of each column and its diagonal
    // (face left of P, then face right of P; x, y, z) get
    // Temp/(VolC_row+Eps)/(Rho_col+Eps)
    if (dkx) {
      auto term = [&](T K, size_t Q) { return div_rn(div_rn((T)2 * K, g.volc[Q] + e, rvol[Q]), rPe, rrP); };
      if (actx(i - 1)) {
        const T K = dkx[d.UF(i - 1, j, k)];
        v[4] = v[4] + term(K, P - sx);
        dg = dg - term(K, P);
      }
      if (actx(i)) {
        const T K = dkx[d.UF(i, j, k)];
        v[2] = v[2] + term(K, P + sx);
        dg = dg - term(K, P);
      }
      if (acty(j - 1)) {
        const T K = dky[d.VF(i, j - 1, k)];
        v[5] = v[5] + term(K, P - sy);
        dg = dg - term(K, P);
      }
      if (acty(j)) {
        const T K = dky[d.VF(i, j, k)];
        v[1] = v[1] + term(K, P + sy);
        dg = dg - term(K, P);
      }
      if (actz(k - 1)) {
        const T K = dkz[d.WF(i, j, k - 1)];
        v[6] = v[6] + term(K, P - sz);
        dg = dg - term(K, P);
      }
      if (actz(k)) {
        const T K = dkz[d.WF(i, j, k)];
        v[0] = v[0] + term(K, P + sz);
        dg = dg - term(K, P);
      }
    }
    // JacScaleCompute fold of the face-halo rows (:1791-1856)
    if (jj && kk && i == 0) dg = dg - v[2];
    if (jj && kk && i == nx + 1) dg = dg - v[4];
    if (ii && kk && j == 0) dg = dg - v[1];
    if (ii && kk && j == ny + 1) dg = dg - v[5];
    if (ii && jj && k == 0) dg = dg - v[0];
    if (ii && jj && k == nz + 1) dg = dg - v[6];
    // scale to I - beta0*dt*J (:1857-1862); slot 7 holds 1/diagonal for the
    // correctly rounded divisions of the Gauss-Seidel sweeps
    const T diag = (T)1 - bdt * dg;
    val[3 * n + P] = diag;
    val[7 * n + P] = (T)1 / diag;
    val[0 * n + P] = -(bdt * v[0]);
    val[1 * n + P] = -(bdt * v[1]);
    val[2 * n + P] = -(bdt * v[2]);
    val[4 * n + P] = -(bdt * v[4]);
    val[5 * n + P] = -(bdt * v[5]);
    val[6 * n + P] = -(bdt * v[6]);
  }
}

// ---------------------------------------------------------------------------
// Stage operator: MatVecMet_Vec4CellSp (MODULE/SpMatrix4CellPar_Mod.f90:70-84):
// y = T*x (SpAVec_SpDiag, CG/MatSpDiag_Mod.f90:87-108, row sums in diagonal
// order), then y = -1*x + y, y = x + y (identity source block).
// ---------------------------------------------------------------------------
template <typename TM, typename T>
__global__ void k_matvec(Dims d, int ncomp, const TM* __restrict__ val, const T* __restrict__ x, T* __restrict__ y,
                         int plain_spmv) {
  const int NX = d.NX(), NY = d.NY(), NZ = d.NZ();
  const size_t n = d.npad();
  const size_t sy = (size_t)NX, sz = (size_t)NX * NY;
  for (size_t P = blockIdx.x * (size_t)blockDim.x + threadIdx.x; P < n; P += (size_t)gridDim.x * blockDim.x) {
    int i, j, k;
    d.ijk(P, i, j, k);
    const T v0 = k > 0 ? (T)val[0 * n + P - sz] : (T)0;
    const T v1 = j > 0 ? (T)val[1 * n + P - sy] : (T)0;
    const T v2 = i > 0 ? (T)val[2 * n + P - 1] : (T)0;
    const T v3 = (T)val[3 * n + P];
    const T v4 = i < NX - 1 ? (T)val[4 * n + P + 1] : (T)0;
    const T v5 = j < NY - 1 ? (T)val[5 * n + P + sy] : (T)0;
    const T v6 = k < NZ - 1 ? (T)val[6 * n + P + sz] : (T)0;
    for (int ic = 0; ic < ncomp; ++ic) {
      const T* xa = x + ic * n;
      T s = (T)0;
      if (k > 0) s = s + v0 * xa[P - sz];
      if (j > 0) s = s + v1 * xa[P - sy];
      if (i > 0) s = s + v2 * xa[P - 1];
      s = s + v3 * xa[P];
      if (i < NX - 1) s = s + v4 * xa[P + 1];
      if (j < NY - 1) s = s + v5 * xa[P + sy];
      if (k < NZ - 1) s = s + v6 * xa[P + sz];
      if (!plain_spmv) {
        const T xp = xa[P];
        s = (T)(-1) * xp + s;
        s = xp + s;
      }
      y[ic * n + P] = s;
    }
  }
}

// ---------------------------------------------------------------------------
// Gauss-Seidel preconditioner GaussSeidel_SpDiag (CG/MatSpDiag_Mod.f90:191-235),
// restated as: sweep 0 solves (L+D)x=b; sweeps 1..IterG solve
// (L+D)x_new = b - U*x_old.  Row r of the column-oriented storage receives
//   U part: columns r+1, r+NX, r+NXY (in that order),
//   L part: columns r-NXY, r-NX, r-1 (in that order), then the division.
// The padded box is cut into tiles of GS_TX x GS_TY x GS_TZ cells; tile
// (I,J,K) depends only on tiles (I-1,J,K), (I,J-1,K), (I,J,K-1) in the lower
// solve, so all tiles with I+J+K = level are independent.  Inside a tile the
// cells are visited by hyperplanes a+b+c = l: each thread owns one (b,c) line
// of one component and walks it in x, so the x-neighbour is in a register;
// the 16 lines of a component sit in one warp, so the y/z-neighbours computed
// at the previous hyperplane arrive by warp shuffle, and neighbours in the
// previous tiles come from an earlier launch.
// ---------------------------------------------------------------------------
constexpr int GS_TX = 32;
constexpr int GS_TY = 4;
constexpr int GS_TZ = 4;

// All 1+IterG sweeps of GaussSeidel_SpDiag in one pipelined wavefront.
// Sweep s solves (L+D) x^s = b - U x^{s-1} (x^{-1} = 0, i.e. no U part in
// sweep 0) and trails sweep s-1 by two tile levels: its U-neighbour tiles
// (I+1,J,K), (I,J+1,K), (I,J,K+1) hold x^{s-1} from the previous launch, so one
// launch (index tau) runs tile level tau-2s of every sweep s.  x^s lives in
// buffer s%2 relative to the last sweep (the last sweep writes `out`); within
// one launch the tile levels read and written in each buffer are disjoint.
// Per cell the operation order is the reference's: b, U part (columns r+1,
// r+NX, r+NXY), L part (columns r-NXY, r-NX, r-1), division.
// Variant for the FP64 pipe (occupancy matters more than latency): each
// thread prefetches its next two cells' operands into registers, two
// hyperplanes ahead; no shared memory, so many tiles fit on an SM.
template <typename TM, typename T>
__global__ void __launch_bounds__(256) k_gs_pipe_reg(Dims d, int ncomp, const TM* __restrict__ val,
                                                     const T* __restrict__ b, T* buf_last, T* buf_other, int tau,
                                                     int nsweep, int ntx, int nty, int ntz, int nlev) {
  static_assert(GS_TY * GS_TZ == 16, "one component's tile lines fill half a warp");
  const int s = blockIdx.z;
  const int L = tau - 2 * s;
  if (L < 0 || L >= nlev) return;
  const int K = blockIdx.y;
  const int Jlo = max(0, L - K - (ntx - 1));
  const int J = Jlo + (int)blockIdx.x;
  const int I = L - J - K;
  if (J >= nty || I < 0 || I >= ntx) return;  // uniform over the block
  const int NX = d.NX(), NY = d.NY(), NZ = d.NZ();
  const size_t n = d.npad();
  const size_t sy = (size_t)NX, sz = (size_t)NX * NY;
  const bool last_parity = ((nsweep - 1 - s) & 1) == 0;
  T* xn_all = last_parity ? buf_last : buf_other;        // x^s
  const T* xo_all = last_parity ? buf_other : buf_last;  // x^{s-1}
  // lane = tb + GS_TY*tc + 16*(ic&1): the y-neighbour line is lane-1 and the
  // z-neighbour line lane-GS_TY, both in this warp
  const int lb = threadIdx.x % (GS_TY * GS_TZ);
  const int ic = threadIdx.x / (GS_TY * GS_TZ);
  const int tb = lb % GS_TY, tc = lb / GS_TY;
  const int j = J * GS_TY + tb, k = K * GS_TZ + tc;
  const bool line_ok = ic < ncomp && j < NY && k < NZ;
  const size_t off = (size_t)(line_ok ? ic : 0) * n;
  const T* bb = b + off;
  T* xn = xn_all + off;
  const T* xo = xo_all + off;
  const int i0 = I * GS_TX;
  const size_t rowP = sy * (size_t)j + sz * (size_t)k;
  const bool up = s > 0;

  // operands of one cell that do not depend on this sweep's current results
  struct Cell {
    T bb, u4, u5, u6, xo4, xo5, xo6, l0, l1, l2, dg, rd, xz, xy, xx;
  };
  auto load = [&](int a, Cell& c) {
    const int i = i0 + a;
    const size_t P = (size_t)i + rowP;
    c.bb = bb[P];
    c.u4 = c.u5 = c.u6 = c.xo4 = c.xo5 = c.xo6 = (T)0;
    if (up) {
      if (i < NX - 1) { c.u4 = (T)val[4 * n + P + 1]; c.xo4 = xo[P + 1]; }
      if (j < NY - 1) { c.u5 = (T)val[5 * n + P + sy]; c.xo5 = xo[P + sy]; }
      if (k < NZ - 1) { c.u6 = (T)val[6 * n + P + sz]; c.xo6 = xo[P + sz]; }
    }
    c.l0 = k > 0 ? (T)val[0 * n + P - sz] : (T)0;
    c.l1 = j > 0 ? (T)val[1 * n + P - sy] : (T)0;
    c.l2 = i > 0 ? (T)val[2 * n + P - 1] : (T)0;
    c.dg = (T)val[3 * n + P];
    c.rd = (T)val[7 * n + P];
    // neighbours in the previous tiles (written by an earlier launch)
    c.xz = (tc == 0 && k > 0) ? xn[P - sz] : (T)0;
    c.xy = (tb == 0 && j > 0) ? xn[P - sy] : (T)0;
    c.xx = (a == 0 && i > 0) ? xn[P - 1] : (T)0;
  };

  const int amax = min(GS_TX, NX - i0);  // cells of this line inside the box
  Cell cur, nxt, nxt2;  // operands of cells a, a+1, a+2
  if (line_ok && amax > 0) load(0, nxt);
  if (line_ok && amax > 1) load(1, nxt2);
  T last = (T)0;
  const unsigned full = 0xffffffffu;
  const int nlev_in = GS_TX + GS_TY + GS_TZ - 2;
  for (int l = 0; l < nlev_in; ++l) {
    const T from_y = __shfl_up_sync(full, last, 1);
    const T from_z = __shfl_up_sync(full, last, GS_TY);
    const int a = l - tb - tc;
    if (line_ok && a >= 0 && a < amax) {
      cur = nxt;
      nxt = nxt2;
      if (a + 2 < amax) load(a + 2, nxt2);
      const int i = i0 + a;
      T t = cur.bb;
      if (up) {
        if (i < NX - 1) t = t - cur.u4 * cur.xo4;
        if (j < NY - 1) t = t - cur.u5 * cur.xo5;
        if (k < NZ - 1) t = t - cur.u6 * cur.xo6;
      }
      if (k > 0) t = t - cur.l0 * (tc > 0 ? from_z : cur.xz);
      if (j > 0) t = t - cur.l1 * (tb > 0 ? from_y : cur.xy);
      if (i > 0) t = t - cur.l2 * (a > 0 ? last : cur.xx);
      t = div_rn(t, cur.dg, cur.rd);
      xn[(size_t)i + rowP] = t;
      last = t;
    }
  }
}

// Shared-memory layout of one tile of k_gs_pipe_smem (in units of T):
//   ts [ncomp][TZ][TY][TX]       b, then b - U x^{s-1}
//   ls [8][TZ][TY][TX]           lower-part coefficients for columns r-NXY, r-NX,
//                                r-1, the diagonal, its reciprocal, and the
//                                upper-part coefficients for columns r+1, r+NX, r+NXY
//   xs [ncomp][TZ+1][TY+1][TX+1] x^{s-1} on the tile grown by one cell in +x,
//                                +y and +z (the upper-part neighbours)
//   zb [ncomp][TY][TX]           x^s of the cells below the tile's bottom plane
//   yb [ncomp][TZ][TX]           x^s of the cells south of the tile's first row
//   xb [ncomp][TZ][TY]           x^s of the cells west of the tile's first column
constexpr int GS_TILE = GS_TX * GS_TY * GS_TZ;
constexpr int GS_BX = GS_TX + 1, GS_BY = GS_TY + 1, GS_BZ = GS_TZ + 1;
constexpr int GS_BOX = GS_BX * GS_BY * GS_BZ;
inline size_t gs_smem_elems(int ncomp) {
  return (size_t)ncomp * (GS_TILE + GS_BOX + GS_TY * GS_TX + GS_TZ * GS_TX + GS_TZ * GS_TY) + 8 * (size_t)GS_TILE;
}

// Asynchronous global->shared copy of one element (cp.async, no register
// staging); when `pred` is false nothing is read and the element is zeroed.
template <typename T>
__device__ __forceinline__ void cp_async_elem(T* smem, const T* gmem, bool pred) {
  static_assert(sizeof(T) == 4 || sizeof(T) == 8, "cp.async element of 4 or 8 bytes");
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  const unsigned src_size = pred ? (unsigned)sizeof(T) : 0u;
  if constexpr (sizeof(T) == 4)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(sa), "l"(gmem), "r"(src_size) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(sa), "l"(gmem), "r"(src_size) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// One tile of one sweep with its operands staged in shared memory (the FP32
// variants): every operand that does not depend on this sweep's new values is
// copied by cp.async in one batch (one memory round trip instead of one per
// load), b - U x^{s-1} is formed in shared memory, and the wavefront then reads
// only shared memory and registers.  The copies are issued in two groups so
// that a scheduler can wait for the tile's dependencies in between: the
// coefficients and b never change during the sweeps; x^{s-1} and the x^s halo
// are written by other tiles.
template <typename TM, typename T>
struct GsTile {
  static_assert(sizeof(TM) == sizeof(T), "coefficients are copied as they are stored");
  int ncomp, NX, NY, NZ;
  size_t n, sy, sz;
  const TM* val;
  const T* b;
  T* xn_all;        // x^s
  const T* xo_all;  // x^{s-1}
  bool up;
  int i0, j0, k0;
  T *ts, *ls, *xs, *zb, *yb, *xb;

  // components c0 .. c0+ncomp_-1 of the fields (the sweeps of different
  // components are independent: one matrix, no coupling)
  __device__ GsTile(const Dims& d, int c0, int ncomp_, const TM* val_, const T* b_, T* buf_last, T* buf_other,
                    int nsweep, int I, int J, int K, int s, unsigned char* smem)
      : ncomp(ncomp_), NX(d.NX()), NY(d.NY()), NZ(d.NZ()), n(d.npad()), sy((size_t)d.NX()),
        sz((size_t)d.NX() * d.NY()), val(val_), b(b_ + (size_t)c0 * d.npad()), up(s > 0), i0(I * GS_TX),
        j0(J * GS_TY), k0(K * GS_TZ) {
    const bool last_parity = ((nsweep - 1 - s) & 1) == 0;
    xn_all = (last_parity ? buf_last : buf_other) + (size_t)c0 * n;
    xo_all = (last_parity ? buf_other : buf_last) + (size_t)c0 * n;
    ts = reinterpret_cast<T*>(smem);
    ls = ts + (size_t)ncomp * GS_TILE;
    xs = ls + 8 * (size_t)GS_TILE;
    zb = xs + (size_t)ncomp * GS_BOX;
    yb = zb + (size_t)ncomp * GS_TY * GS_TX;
    xb = yb + (size_t)ncomp * GS_TZ * GS_TX;
  }

  // The copies are issued per x-row of the tile: warp w takes rows w, w+nwarp,
  // ...; lane a copies cell i0+a of the row (coalesced, one address per lane).
  // group 1: the eight coefficient slots and b
  __device__ void issue_fixed() const {
    TM* lsm = reinterpret_cast<TM*>(ls);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    const int i = i0 + lane;
    constexpr int ROWS = GS_TY * GS_TZ;
    for (int r = warp; r < 8 * ROWS; r += nwarp) {
      const int m = r / ROWS, line = r % ROWS;
      const int j = j0 + line % GS_TY, k = k0 + line / GS_TY;
      const bool in = i < NX && j < NY && k < NZ;
      const size_t P = in ? (size_t)i + sy * j + sz * k : 0;
      // slot m of the shared tile: (matrix column, cell offset, condition)
      const TM* src = val;
      bool p = false;
      switch (m) {
        case 0: p = in && k > 0; src = val + 0 * n + P - sz; break;
        case 1: p = in && j > 0; src = val + 1 * n + P - sy; break;
        case 2: p = in && i > 0; src = val + 2 * n + P - 1; break;
        case 3: p = in; src = val + 3 * n + P; break;
        case 4: p = in; src = val + 7 * n + P; break;
        case 5: p = in && up && i < NX - 1; src = val + 4 * n + P + 1; break;
        case 6: p = in && up && j < NY - 1; src = val + 5 * n + P + sy; break;
        default: p = in && up && k < NZ - 1; src = val + 6 * n + P + sz; break;
      }
      cp_async_elem(lsm + m * GS_TILE + line * GS_TX + lane, p ? src : val, p);
    }
    for (int r = warp; r < ncomp * ROWS; r += nwarp) {
      const int ic = r / ROWS, line = r % ROWS;
      const int j = j0 + line % GS_TY, k = k0 + line / GS_TY;
      const bool in = i < NX && j < NY && k < NZ;
      cp_async_elem(ts + r * GS_TX + lane, in ? b + (size_t)ic * n + (size_t)i + sy * j + sz * k : b, in);
    }
  }

  // group 2: x^{s-1} on the tile grown by one cell in +x, +y, +z (the edges
  // and the corner of the grown part are never read, and may be written by
  // sweep s-1 meanwhile: they are skipped), and the x^s faces of the three
  // lower neighbour tiles
  __device__ void issue_neighbours() const {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    const int i = i0 + lane;
    if (up) {
      constexpr int BROWS = GS_BY * GS_BZ;
      for (int r = warp; r < ncomp * BROWS; r += nwarp) {
        const int ic = r / BROWS, line = r % BROWS;
        const int tb = line % GS_BY, tc = line / GS_BY;
        if (tb == GS_TY && tc == GS_TZ) continue;  // edge of the grown part: never read
        const int j = j0 + tb, k = k0 + tc;
        const bool row = j < NY && k < NZ;
        const T* src = xo_all + (size_t)ic * n + sy * j + sz * k;
        T* dst = xs + (size_t)ic * GS_BOX + line * GS_BX;
        cp_async_elem(dst + lane, row && i < NX ? src + i : xo_all, row && i < NX);
        if (lane == 0 && tb < GS_TY && tc < GS_TZ) {  // the +x cell of the row
          const bool p = row && i0 + GS_TX < NX;
          cp_async_elem(dst + GS_TX, p ? src + i0 + GS_TX : xo_all, p);
        }
      }
    }
    for (int r = warp; r < ncomp * GS_TY; r += nwarp) {  // plane below: rows tb
      const int ic = r / GS_TY, tb = r % GS_TY;
      const int j = j0 + tb, k = k0;
      const bool in = k > 0 && i < NX && j < NY;
      cp_async_elem(zb + r * GS_TX + lane, in ? xn_all + (size_t)ic * n + (size_t)i + sy * j + sz * (k - 1) : xn_all,
                    in);
    }
    for (int r = warp; r < ncomp * GS_TZ; r += nwarp) {  // row to the south: rows tc
      const int ic = r / GS_TZ, tc = r % GS_TZ;
      const int j = j0, k = k0 + tc;
      const bool in = j > 0 && i < NX && k < NZ;
      cp_async_elem(yb + r * GS_TX + lane, in ? xn_all + (size_t)ic * n + (size_t)i + sy * (j - 1) + sz * k : xn_all,
                    in);
    }
    for (int q = threadIdx.x; q < ncomp * GS_TZ * GS_TY; q += blockDim.x) {  // column to the west
      const int ic = q / (GS_TZ * GS_TY), c = q % (GS_TZ * GS_TY);
      const int tb = c % GS_TY, tc = c / GS_TY;
      const int j = j0 + tb, k = k0 + tc;
      const bool in = i0 > 0 && j < NY && k < NZ;
      cp_async_elem(xb + q, in ? xn_all + (size_t)ic * n + (size_t)(i0 - 1) + sy * j + sz * k : xn_all, in);
    }
  }

  // waits for both groups, forms b - U x^{s-1}, runs the wavefront and stores x^s
  __device__ void compute() const {
    cp_async_wait_all();
    __syncthreads();
    if (up) {  // b - U x^{s-1} in the reference's column order, one x-row per warp
      const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
      const int i = i0 + lane;
      constexpr int ROWS = GS_TY * GS_TZ;
      for (int r = warp; r < ncomp * ROWS; r += nwarp) {
        const int ic = r / ROWS, line = r % ROWS;
        const int tb = line % GS_TY, tc = line / GS_TY;
        const int j = j0 + tb, k = k0 + tc;
        if (i < NX && j < NY && k < NZ) {
          const int c = line * GS_TX + lane;
          const T* xq = xs + (size_t)ic * GS_BOX + (tc * GS_BY + tb) * GS_BX + lane;
          T t = ts[r * GS_TX + lane];
          if (i < NX - 1) t = t - ls[5 * GS_TILE + c] * xq[1];
          if (j < NY - 1) t = t - ls[6 * GS_TILE + c] * xq[GS_BX];
          if (k < NZ - 1) t = t - ls[7 * GS_TILE + c] * xq[GS_BX * GS_BY];
          ts[r * GS_TX + lane] = t;
        }
      }
      __syncthreads();
    }
    // wavefront over the tile's hyperplanes.  lane = tb + GS_TY*tc + 16*(ic&1):
    // the y-neighbour line is lane-1 and the z-neighbour line lane-GS_TY.
    const int lb = threadIdx.x % (GS_TY * GS_TZ);
    const int ic = threadIdx.x / (GS_TY * GS_TZ);
    const int tb = lb % GS_TY, tc = lb / GS_TY;
    const int j = j0 + tb, k = k0 + tc;
    const bool line_ok = ic < ncomp && j < NY && k < NZ;
    const int icc = line_ok ? ic : 0;
    T* xn = xn_all + (size_t)icc * n;
    const size_t rowP = sy * (size_t)j + sz * (size_t)k;
    const int amax = min(GS_TX, NX - i0);
    const T* tl = ts + (size_t)icc * GS_TILE + (tc * GS_TY + tb) * GS_TX;
    const int lq = (tc * GS_TY + tb) * GS_TX;
    T last = line_ok ? xb[(icc * GS_TZ + tc) * GS_TY + tb] : (T)0;  // x-neighbour of cell 0
    const unsigned full = 0xffffffffu;
    const int nlev_in = GS_TX + GS_TY + GS_TZ - 2;
    for (int l = 0; l < nlev_in; ++l) {
      const T from_y = __shfl_up_sync(full, last, 1);
      const T from_z = __shfl_up_sync(full, last, GS_TY);
      const int a = l - tb - tc;
      if (line_ok && a >= 0 && a < amax) {
        const int i = i0 + a;
        const int q = lq + a;
        T t = tl[a];
        if (k > 0) t = t - ls[0 * GS_TILE + q] * (tc > 0 ? from_z : zb[(icc * GS_TY + tb) * GS_TX + a]);
        if (j > 0) t = t - ls[1 * GS_TILE + q] * (tb > 0 ? from_y : yb[(icc * GS_TZ + tc) * GS_TX + a]);
        if (i > 0) t = t - ls[2 * GS_TILE + q] * last;
        t = div_rn(t, ls[3 * GS_TILE + q], ls[4 * GS_TILE + q]);
        xn[(size_t)i + rowP] = t;
        last = t;
      }
    }
  }
};

// The shared-memory variants run `group` components per CTA (16 tile lines
// per component, whole warps): the sweeps of different components are
// independent wavefronts, so smaller groups give more, smaller CTAs (more per
// SM, shorter copy phases) at the price of copying the tile's coefficients
// once per group.
__host__ __device__ inline int gs_ngroups(int ncomp, int group) { return (ncomp + group - 1) / group; }

// Level-synchronous schedule: launch tau runs tile level tau-2s of every sweep
// s and component group g (blockIdx.z = s*ngroups + g).
template <typename TM, typename T>
__global__ void __launch_bounds__(256) k_gs_pipe_smem(Dims d, int ncomp, int group, const TM* __restrict__ val,
                                                      const T* __restrict__ b, T* buf_last, T* buf_other, int tau,
                                                      int nsweep, int ntx, int nty, int ntz, int nlev) {
  static_assert(GS_TY * GS_TZ == 16, "one component's tile lines fill half a warp");
  const int ngroups = gs_ngroups(ncomp, group);
  const int s = blockIdx.z / ngroups, g = blockIdx.z % ngroups;
  const int L = tau - 2 * s;
  if (L < 0 || L >= nlev) return;
  const int K = blockIdx.y;
  const int Jlo = max(0, L - K - (ntx - 1));
  const int J = Jlo + (int)blockIdx.x;
  const int I = L - J - K;
  if (J >= nty || I < 0 || I >= ntx) return;  // uniform over the block
  extern __shared__ __align__(16) unsigned char gs_smem_raw[];
  const int c0 = g * group;
  const GsTile<TM, T> tile(d, c0, min(group, ncomp - c0), val, b, buf_last, buf_other, nsweep, I, J, K, s,
                           gs_smem_raw);
  tile.issue_fixed();
  tile.issue_neighbours();
  tile.compute();
}

// ---------------------------------------------------------------------------
// Persistent schedule of the same sweeps: one launch, CTAs take tickets
// (tile, sweep, component group) from an atomic counter in pipelined-level
// order (level + 2*sweep, the launch index of the level-synchronous schedule)
// and wait for the tickets their tile depends on through per-(tile, group)
// completion counters:
//   sweep s of tile (I,J,K) needs sweep s of (I-1,J,K), (I,J-1,K), (I,J,K-1)
//   (lower part) and, for s > 0, sweep s-1 of the tile itself and of
//   (I+1,J,K), (I,J+1,K), (I,J,K+1) (upper part, x^{s-1}), same group.
// Every dependency has a smaller ticket, and a CTA only takes a ticket while
// it runs, so the smallest unfinished ticket can always proceed: no deadlock
// whatever the number of resident CTAs.  The buffer reuse (x^s overwrites
// x^{s-2}) is safe by the same chain: every reader of x^{s-2} of a tile is a
// dependency, direct or transitive, of its sweep s.
// Waits are bounded: a CTA that gives up sets the error flag, lets its own
// copies in flight land and returns; the other CTAs see the flag and return.
// ---------------------------------------------------------------------------

__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(int* p, int v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;\n" ::"l"(p), "r"(v) : "memory");
}

// counter reached target, in wrap-around (serial number) arithmetic
__device__ bool gs_wait_flag(const int* f, unsigned target, const int* err, int spin) {
  for (int it = 0; it < spin; ++it) {
    if ((int)((unsigned)ld_acquire(f) - target) >= 0) return true;
    if (*(volatile const int*)err) return false;
    __nanosleep(32);
  }
  return false;
}

template <typename TM, typename T>
__global__ void __launch_bounds__(256) k_gs_persist(Dims d, int ncomp, const TM* __restrict__ val,
                                                    const T* __restrict__ b, T* buf_last, T* buf_other, int nsweep,
                                                    int ntx, int nty, int ntz, GsTileSched sch) {
  static_assert(GS_TY * GS_TZ == 16, "one component's tile lines fill half a warp");
  extern __shared__ __align__(16) unsigned char gs_smem_raw[];
  __shared__ int s_ticket, s_ok;
  const int group = sch.group;
  const int ngroups = gs_ngroups(ncomp, group);
  const unsigned base = *sch.base;  // advanced by k_gs_advance after this launch
  for (;;) {
    if (threadIdx.x == 0) s_ticket = *(volatile const int*)sch.err ? sch.nticket : atomicAdd(sch.counter, 1);
    __syncthreads();
    const int tk = s_ticket;
    if (tk >= sch.nticket) return;  // uniform over the block
    const int4 e = sch.order[tk];
    const int I = e.x, J = e.y, K = e.z, s = e.w / ngroups, g = e.w % ngroups;
    const int c0 = g * group;
    const GsTile<TM, T> tile(d, c0, min(group, ncomp - c0), val, b, buf_last, buf_other, nsweep, I, J, K, s,
                             gs_smem_raw);
    tile.issue_fixed();
    if (threadIdx.x == 0) {
      const int* f = sch.flags;
      const unsigned now = base + s + 1, prev = base + s;  // sweep s done, sweep s-1 done
      const int id = ((K * nty + J) * ntx + I) * ngroups + g;
      const int sx = ngroups, sy_ = ntx * ngroups, sz_ = ntx * nty * ngroups;
      bool ok = true;
      if (I > 0) ok = ok && gs_wait_flag(f + id - sx, now, sch.err, sch.spin);
      if (J > 0) ok = ok && gs_wait_flag(f + id - sy_, now, sch.err, sch.spin);
      if (K > 0) ok = ok && gs_wait_flag(f + id - sz_, now, sch.err, sch.spin);
      if (s > 0) {
        ok = ok && gs_wait_flag(f + id, prev, sch.err, sch.spin);
        if (I + 1 < ntx) ok = ok && gs_wait_flag(f + id + sx, prev, sch.err, sch.spin);
        if (J + 1 < nty) ok = ok && gs_wait_flag(f + id + sy_, prev, sch.err, sch.spin);
        if (K + 1 < ntz) ok = ok && gs_wait_flag(f + id + sz_, prev, sch.err, sch.spin);
      }
      if (!ok) atomicExch(sch.err, 1);
      s_ok = ok;
    }
    __syncthreads();
    if (!s_ok) {  // give up: let this CTA's copies land, then leave
      cp_async_wait_all();
      return;
    }
    __threadfence();
    tile.issue_neighbours();
    tile.compute();
    // publish: every thread's stores are ordered before the counter update
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0)
      st_release(sch.flags + ((K * nty + J) * ntx + I) * ngroups + g, (int)(base + s + 1));
  }
}

// next epoch of the persistent schedule's completion counters
__global__ void k_gs_advance(unsigned* base, int nsweep) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *base += (unsigned)nsweep;
}

// Line preconditioners of the refined mode's inner solver: x = T^{-1} b with
// T the tridiagonal part of the stage matrix along one axis (the diagonal and
// the couplings to the two neighbours on the axis), solved by the Thomas
// algorithm along every padded line of that axis; the other couplings are
// dropped (block Jacobi over lines).  Along the wind the dropped part is small
// and one application is nearly an exact inverse.
//
// y and z lines: one thread per line handles all components (the elimination
// factors depend on the matrix only and are kept in `w`, one value per cell);
// consecutive threads take consecutive i, so every access is coalesced.
// axis 1: lines along y (columns (i,k)); axis 2: along z (columns (i,j)).
template <typename TM, typename T>
__global__ void k_line_psolve(Dims d, int ncomp, int axis, const TM* __restrict__ val, const T* __restrict__ b,
                              T* __restrict__ x, T* __restrict__ w) {
  const int NX = d.NX(), NY = d.NY(), NZ = d.NZ();
  const size_t n = d.npad();
  const size_t sy = (size_t)NX, sz = (size_t)NX * NY;
  const bool alz = axis == 2;
  const size_t st = alz ? sz : sy;          // stride along the line
  const int len = alz ? NZ : NY;            // cells on the line
  const int lo = alz ? 0 : 1, hi = alz ? 6 : 5;  // matrix slots of the two neighbours
  const size_t ncols = (size_t)NX * (alz ? NY : NZ);
  for (size_t col = blockIdx.x * (size_t)blockDim.x + threadIdx.x; col < ncols;
       col += (size_t)gridDim.x * blockDim.x) {
    const size_t i = col % NX, o = col / NX;
    const size_t P0 = i + (alz ? sy * o : sz * o);
    T g[kMaxComp];
    // forward elimination
    T wprev = (T)0;
    for (int k = 0; k < len; ++k) {
      const size_t P = P0 + st * (size_t)k;
      const T a = k > 0 ? (T)val[lo * n + P - st] : (T)0;
      const T c = k < len - 1 ? (T)val[hi * n + P + st] : (T)0;
      const T den = (T)val[3 * n + P] - a * wprev;
      const T rden = (T)1 / den;
      const T wk = c * rden;
      w[P] = wk;
      for (int ic = 0; ic < ncomp; ++ic) {
        const T gk = (b[ic * n + P] - a * (k > 0 ? g[ic] : (T)0)) * rden;
        g[ic] = gk;
        x[ic * n + P] = gk;
      }
      wprev = wk;
    }
    // back substitution
    for (int k = len - 2; k >= 0; --k) {
      const size_t P = P0 + st * (size_t)k;
      const T wk = w[P];
      for (int ic = 0; ic < ncomp; ++ic) {
        const T xk = x[ic * n + P] - wk * g[ic];
        g[ic] = xk;
        x[ic * n + P] = xk;
      }
    }
  }
}

// x lines (the memory-contiguous axis): the padded rows of the box are
// consecutive, so 32 consecutive rows form one contiguous 32 x NX block.  A
// warp takes 32 rows and walks them in chunks of 32 columns: each chunk of
// every operand is copied row by row (lanes along x, coalesced, cp.async, one
// memory round trip per chunk) into a shared 32 x 33 tile, lane q then runs
// the recurrence of row q through the chunk from the tile (conflict-free: row
// pitch 33), and results leave through the tile the same way.
// The elimination factors depend on the matrix only, so they are computed
// once per stage matrix (k_xline_factor: w_i = c_i/den_i and 1/den_i with
// den_i = d_i - a_i w_{i-1}); every application (k_xline_solve, one warp per
// 32 rows and component) then runs g_i = (b_i - a_i g_{i-1})/den_i forward
// and x_i = g_i - w_i x_{i+1} backward.
template <typename T>
__host__ __device__ constexpr int xl_warps() {  // warps per CTA: three 32 x 33 tiles per warp within 48 KB
  return sizeof(T) == 4 ? 3 : 1;
}

template <typename T>
__device__ __forceinline__ void xl_load(T (*t)[33], const T* src, int r0, int nr, int NX, int ch, int lane,
                                        int shift, bool lo_ok, bool hi_ok) {
  const int i = ch * 32 + lane;
  for (int q = 0; q < nr; ++q) {
    const size_t P = (size_t)(r0 + q) * NX + i;
    const bool in = i < NX && (lo_ok || i > 0) && (hi_ok || i < NX - 1);
    cp_async_elem(&t[q][lane], in ? src + P + shift : src, in);
  }
}
template <typename T>
__device__ __forceinline__ void xl_store(T (*t)[33], T* dst, int r0, int nr, int NX, int ch, int lane) {
  const int i = ch * 32 + lane;
  if (i < NX)
    for (int q = 0; q < nr; ++q) dst[(size_t)(r0 + q) * NX + i] = t[q][lane];
}

template <typename TM, typename T>
__global__ void __launch_bounds__(32 * xl_warps<T>()) k_xline_factor(Dims d, const TM* __restrict__ val,
                                                                    T* __restrict__ fw, T* __restrict__ fr) {
  constexpr int XW = xl_warps<T>();
  __shared__ T tile[XW][3][32][33];  // a, c (then w), d (then 1/den)
  const int NX = d.NX();
  const size_t n = d.npad();
  const int nrows = d.NY() * d.NZ();
  const int lane = threadIdx.x & 31, wq = threadIdx.x >> 5;
  const int grp = blockIdx.x * XW + wq;
  if (grp * 32 >= nrows) return;  // whole warp
  const int r0 = grp * 32, nr = min(32, nrows - r0);
  T(*ta)[33] = tile[wq][0];
  T(*tc)[33] = tile[wq][1];
  T(*td)[33] = tile[wq][2];
  const int nch = (NX + 31) / 32;
  T wprev = (T)0;
  for (int ch = 0; ch < nch; ++ch) {
    xl_load(ta, val + 2 * n, r0, nr, NX, ch, lane, -1, false, true);
    xl_load(tc, val + 4 * n, r0, nr, NX, ch, lane, +1, true, false);
    xl_load(td, val + 3 * n, r0, nr, NX, ch, lane, 0, true, true);
    cp_async_wait_all();
    __syncwarp();
    if (lane < nr) {
      const int m = min(32, NX - ch * 32);
      for (int k = 0; k < m; ++k) {
        const T rden = (T)1 / (td[lane][k] - ta[lane][k] * wprev);
        wprev = tc[lane][k] * rden;
        tc[lane][k] = wprev;
        td[lane][k] = rden;
      }
    }
    __syncwarp();
    xl_store(tc, fw, r0, nr, NX, ch, lane);
    xl_store(td, fr, r0, nr, NX, ch, lane);
    __syncwarp();
  }
}

template <typename TM, typename T>
__global__ void __launch_bounds__(32 * xl_warps<T>()) k_xline_solve(Dims d, int ncomp, const TM* __restrict__ val,
                                                                   const T* __restrict__ fw,
                                                                   const T* __restrict__ fr, const T* __restrict__ b,
                                                                   T* __restrict__ x) {
  constexpr int XW = xl_warps<T>();
  __shared__ T tile[XW][3][32][33];  // forward: a, 1/den, b (then g); backward: w, g (then x)
  const int NX = d.NX();
  const size_t n = d.npad();
  const int nrows = d.NY() * d.NZ();
  const int ngrp = (nrows + 31) / 32;
  const int lane = threadIdx.x & 31, wq = threadIdx.x >> 5;
  const long long task = (long long)blockIdx.x * XW + wq;  // (row group, component), component fastest
  if (task >= (long long)ngrp * ncomp) return;             // whole warp
  const int ic = (int)(task % ncomp), grp = (int)(task / ncomp);
  const int r0 = grp * 32, nr = min(32, nrows - r0);
  T(*t0)[33] = tile[wq][0];
  T(*t1)[33] = tile[wq][1];
  T(*t2)[33] = tile[wq][2];
  const T* bc = b + (size_t)ic * n;
  T* xc = x + (size_t)ic * n;
  const int nch = (NX + 31) / 32;
  T gprev = (T)0;
  for (int ch = 0; ch < nch; ++ch) {
    xl_load(t0, val + 2 * n, r0, nr, NX, ch, lane, -1, false, true);
    xl_load(t1, fr, r0, nr, NX, ch, lane, 0, true, true);
    xl_load(t2, bc, r0, nr, NX, ch, lane, 0, true, true);
    cp_async_wait_all();
    __syncwarp();
    if (lane < nr) {
      const int m = min(32, NX - ch * 32);
      for (int k = 0; k < m; ++k) {
        gprev = (t2[lane][k] - t0[lane][k] * gprev) * t1[lane][k];
        t2[lane][k] = gprev;
      }
    }
    __syncwarp();
    xl_store(t2, xc, r0, nr, NX, ch, lane);
    __syncwarp();
  }
  __threadfence_block();  // the partial solution is re-read by this warp's copies below
  T xnext = (T)0;
  for (int ch = nch - 1; ch >= 0; --ch) {
    xl_load(t0, fw, r0, nr, NX, ch, lane, 0, true, true);
    xl_load(t1, static_cast<const T*>(xc), r0, nr, NX, ch, lane, 0, true, true);
    cp_async_wait_all();
    __syncwarp();
    if (lane < nr) {
      const int m = min(32, NX - ch * 32);
      for (int k = m - 1; k >= 0; --k) {
        xnext = (ch == nch - 1 && k == m - 1) ? t1[lane][k] : t1[lane][k] - t0[lane][k] * xnext;
        t1[lane][k] = xnext;
      }
    }
    __syncwarp();
    xl_store(t1, xc, r0, nr, NX, ch, lane);
    __syncwarp();
  }
}

// zero the whole halo layer (PSolveSp, MODULE/Vector4Cell_Mod.f90:732-737)
template <typename T>
__global__ void k_zero_halo(Dims d, int ncomp, T* __restrict__ x) {
  const int NX = d.NX(), NY = d.NY(), NZ = d.NZ();
  const size_t n = d.npad();
  for (size_t P = blockIdx.x * (size_t)blockDim.x + threadIdx.x; P < n; P += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(P % NX);
    const int j = (int)((P / NX) % NY);
    const int k = (int)(P / ((size_t)NX * NY));
    if (i == 0 || i == NX - 1 || j == 0 || j == NY - 1 || k == 0 || k == NZ - 1)
      for (int ic = 0; ic < ncomp; ++ic) x[ic * n + P] = (T)0;
  }
}

// periodic halo fill (ExchangeCell of a single periodic block)
template <typename T>
__global__ void k_exchange_cell(Dims d, int ncomp, T* __restrict__ c) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const size_t n = d.npad();
  const size_t nxf = d.per_x ? (size_t)ny * nz : 0;
  const size_t nyf = d.per_y ? (size_t)nx * nz : 0;
  const size_t nzf = d.per_z ? (size_t)nx * ny : 0;
  const size_t tot = nxf + nyf + nzf;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < tot; q += (size_t)gridDim.x * blockDim.x) {
    size_t lo, hi_src, lo_src, hi;
    if (q < nxf) {
      int j = (int)(q % ny) + 1, k = (int)(q / ny) + 1;
      lo = d.P(0, j, k); lo_src = d.P(nx, j, k); hi = d.P(nx + 1, j, k); hi_src = d.P(1, j, k);
    } else if (q < nxf + nyf) {
      size_t r = q - nxf;
      int i = (int)(r % nx) + 1, k = (int)(r / nx) + 1;
      lo = d.P(i, 0, k); lo_src = d.P(i, ny, k); hi = d.P(i, ny + 1, k); hi_src = d.P(i, 1, k);
    } else {
      size_t r = q - nxf - nyf;
      int i = (int)(r % nx) + 1, j = (int)(r / nx) + 1;
      lo = d.P(i, j, 0); lo_src = d.P(i, j, nz); hi = d.P(i, j, nz + 1); hi_src = d.P(i, j, 1);
    }
    for (int ic = 0; ic < ncomp; ++ic) {
      T* a = c + ic * n;
      a[lo] = a[lo_src];
      a[hi] = a[hi_src];
    }
  }
}

// Halo rule of the outer walls (BoundaryCondition / BoundaryVelocity at the
// start of a stage, ADVECT/Int_Mod.f90:283-287): every face halo cell of a
// side that is not periodic takes the rule of its component and side (the
// kinds of BcKind).  comp0 is the first component's index in bc; one thread
// handles one halo location for every component in order, so a density halo
// that InFlowOutFlow reads is updated before the components after the
// density, as in the reference's component loop.
template <typename T>
__device__ __forceinline__ void bc_apply(const asam::BcKinds& bc, signed char kind, int side, int q, size_t n, T* a,
                                         const T* rho, size_t h, size_t src, size_t src2, int level, int nz,
                                         double vel) {
  switch (kind) {
    case asam::kBcZeroGrad: a[h] = a[src]; break;
    case asam::kBcZeroValue: a[h] = -a[src]; break;
    case asam::kBcMeanValue: a[h] = (T)2 * (T)bc.mean[(size_t)q * nz + (level - 1)] - a[src]; break;
    case asam::kBcFunction: a[h] = (T)2 * (T)bc.fval[(size_t)q * n + h] - a[src]; break;
    case asam::kBcInflowOutflow:
      if (side < 4 && rho) {
        const bool in = (side & 1) ? vel <= 0.0 : vel >= 0.0;
        a[h] = in ? rho[h] * (T)bc.amb[(size_t)q * n + h] : a[src];
      }
      break;
    case asam::kBcExtrapolation:
      if (side >= 4) a[h] = (T)2 * a[src] - a[src2];
      break;
    default: break;
  }
}

template <typename T>
__global__ void k_bound_cond(Dims d, int ncomp, int comp0, asam::BcKinds bc, T* __restrict__ c) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const size_t n = d.npad();
  const size_t nxf = d.per_x ? 0 : (size_t)ny * nz;
  const size_t nyf = d.per_y ? 0 : (size_t)nx * nz;
  const size_t nzf = d.per_z ? 0 : (size_t)nx * ny;
  const size_t tot = nxf + nyf + nzf;
  const T* rho = comp0 == 0 ? c + (size_t)bc.rho * n : nullptr;  // the density, read by InFlowOutFlow
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < tot; q += (size_t)gridDim.x * blockDim.x) {
    size_t lo, lo_src, lo_src2, hi, hi_src, hi_src2;
    int side;  // W/E = 0, S/N = 2, B/T = 4
    int lev_lo, lev_hi;
    double vel_lo = 0.0, vel_hi = 0.0;
    if (q < nxf) {
      int j = (int)(q % ny) + 1, k = (int)(q / ny) + 1;
      lo = d.P(0, j, k); lo_src = d.P(1, j, k); lo_src2 = d.P(2, j, k);
      hi = d.P(nx + 1, j, k); hi_src = d.P(nx, j, k); hi_src2 = d.P(nx - 1, j, k);
      side = 0;
      lev_lo = lev_hi = k;
      if (bc.uf) vel_lo = bc.uf[d.UF(0, j, k)], vel_hi = bc.uf[d.UF(nx, j, k)];
    } else if (q < nxf + nyf) {
      size_t r = q - nxf;
      int i = (int)(r % nx) + 1, k = (int)(r / nx) + 1;
      lo = d.P(i, 0, k); lo_src = d.P(i, 1, k); lo_src2 = d.P(i, 2, k);
      hi = d.P(i, ny + 1, k); hi_src = d.P(i, ny, k); hi_src2 = d.P(i, ny - 1, k);
      side = 2;
      lev_lo = lev_hi = k;
      if (bc.vf) vel_lo = bc.vf[d.VF(i, 0, k)], vel_hi = bc.vf[d.VF(i, ny, k)];
    } else {
      size_t r = q - nxf - nyf;
      int i = (int)(r % nx) + 1, j = (int)(r / nx) + 1;
      lo = d.P(i, j, 0); lo_src = d.P(i, j, 1); lo_src2 = d.P(i, j, 2);
      hi = d.P(i, j, nz + 1); hi_src = d.P(i, j, nz); hi_src2 = d.P(i, j, nz - 1);
      side = 4;
      lev_lo = 1, lev_hi = nz;
    }
    for (int ic = 0; ic < ncomp; ++ic) {
      T* a = c + ic * n;
      const int cq = comp0 + ic;
      const signed char kl = bc.k[cq][side], kh = bc.k[cq][side + 1];
      if (kl != asam::kBcNone) bc_apply(bc, kl, side, cq, n, a, rho, lo, lo_src, lo_src2, lev_lo, nz, vel_lo);
      if (kh != asam::kBcNone) bc_apply(bc, kh, side + 1, cq, n, a, rho, hi, hi_src, hi_src2, lev_hi, nz, vel_hi);
    }
  }
}

// Transpose of k_bound_cond for one field of component comp: every interior
// cell next to a wall adds the halo cells that were derived from it (with
// the rule's sign) and those halo cells become 0.  Each halo cell has exactly
// one source cell, so the gather needs no atomics.
template <typename T>
__global__ void k_bound_cond_T(Dims d, int comp, asam::BcKinds bc, T* __restrict__ x) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const size_t nint = (size_t)nx * ny * nz;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < nint; q += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(q % nx) + 1, j = (int)((q / nx) % ny) + 1, k = (int)(q / ((size_t)nx * ny)) + 1;
    const bool on[6] = {!d.per_x && i == 1, !d.per_x && i == nx, !d.per_y && j == 1,
                        !d.per_y && j == ny, !d.per_z && k == 1, !d.per_z && k == nz};
    T add = (T)0;
    for (int s = 0; s < 6; ++s) {
      if (!on[s]) continue;
      const signed char kind = bc.k[comp][s];
      if (kind != asam::kBcZeroGrad && kind != asam::kBcZeroValue) continue;
      const size_t H = s == 0 ? d.P(0, j, k) : s == 1 ? d.P(nx + 1, j, k) : s == 2 ? d.P(i, 0, k)
                     : s == 3 ? d.P(i, ny + 1, k) : s == 4 ? d.P(i, j, 0) : d.P(i, j, nz + 1);
      add = kind == asam::kBcZeroGrad ? add + x[H] : add - x[H];
      x[H] = (T)0;
    }
    if (add != (T)0) x[d.P(i, j, k)] += add;
  }
}

// ---------------------------------------------------------------------------
// Interior dot products (Dot_VectorCell, MODULE/Vector4Cell_Mod.f90:1120-1132),
// deterministic two-stage reduction.
// ---------------------------------------------------------------------------
constexpr int RED_BLOCK = 256;
constexpr int RED_GRID = 1024;

// Per-thread accumulator of a dot product.  FP64 operands accumulate in FP64.
// FP32 operands use the compensated Dot2 scheme of Ogita, Rump and Oishi
// ("Accurate sum and dot product", SIAM J. Sci. Comput. 26 (2005)): the
// rounding error of each product (recovered exactly by an FMA) and of each
// running sum (Knuth's TwoSum) is carried in a second float, so a thread's
// partial is as accurate as if accumulated in twice the working precision,
// at FP32-pipe cost; the partials are then summed in FP64.
template <typename T>
struct DotAcc;
template <>
struct DotAcc<double> {
  double s = 0.0;
  __device__ __forceinline__ void add(double x, double y) { s += x * y; }
  __device__ __forceinline__ double value() const { return s; }
};
template <>
struct DotAcc<float> {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(float x, float y) {
    const float p = __fmul_rn(x, y);
    const float pe = __fmaf_rn(x, y, -p);  // x*y - p exactly
    const float t = __fadd_rn(hi, p);
    const float bp = __fsub_rn(t, hi);
    const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(t, bp)), __fsub_rn(p, bp));  // hi + p - t exactly
    hi = t;
    lo = __fadd_rn(lo, __fadd_rn(e, pe));
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

// Sum of one double per thread over a block of at most RED_BLOCK threads, in a fixed
// order (warp shuffles, then the warp sums by the first warp): the value is
// complete in thread 0.  `ws` holds RED_BLOCK/32 doubles of shared memory;
// the call ends with the block synchronised, so `ws` may be reused.
__device__ __forceinline__ double block_sum(double v, double* ws) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if (lane == 0) ws[warp] = v;
  __syncthreads();
  if (warp == 0) {
    v = lane < (int)((blockDim.x + 31) >> 5) ? ws[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  }
  __syncthreads();
  return v;
}

// One warp per interior x-row of one component at a time (lanes along x, so
// every load is coalesced and no per-element index division is needed).
template <typename T>
__global__ void k_dot_partial(Dims d, int ncomp, const T* __restrict__ x, const T* __restrict__ y,
                              double* __restrict__ partial) {
  const int nx = d.nx, ny = d.ny;
  const long long rows_c = (long long)ny * d.nz;
  const long long nrow = rows_c * ncomp;
  const size_t n = d.npad();
  const size_t sy = (size_t)d.NX(), sz = (size_t)d.NX() * d.NY();
  const int lane = threadIdx.x & 31;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  DotAcc<T> acc;
  for (long long r = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5; r < nrow; r += nw) {
    const int ic = (int)(r / rows_c);
    const int jk = (int)(r - ic * rows_c);
    const int j = jk % ny + 1, k = jk / ny + 1;
    const size_t base = (size_t)ic * n + 1 + sy * j + sz * k;
    const T* xr = x + base;
    const T* yr = y + base;
    int i = lane;
    for (; i + 96 < nx; i += 128) {
      const T x0 = xr[i], x1 = xr[i + 32], x2 = xr[i + 64], x3 = xr[i + 96];
      const T y0 = yr[i], y1 = yr[i + 32], y2 = yr[i + 64], y3 = yr[i + 96];
      acc.add(x0, y0);
      acc.add(x1, y1);
      acc.add(x2, y2);
      acc.add(x3, y3);
    }
    for (; i < nx; i += 32) acc.add(xr[i], yr[i]);
  }
  __shared__ double ws[RED_BLOCK / 32];
  const double t = block_sum(acc.value(), ws);
  if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

// SpMV fused with the dot products that read its result (BiCGStab's
// v = A p-hat with (r~, v), and t = A r-hat with (t, r) and (t, t)): y =
// MatVecMet(x) exactly as k_matvec, and per-block partial sums over the
// interior cells of (a, y) -- with kTwo, of (y, a) and (y, y) -- for
// k_dot_final, so the product is not read back.  RED_GRID blocks of
// RED_BLOCK threads stride over the padded cells.
template <typename TM, typename T, bool kTwo>
__global__ void __launch_bounds__(RED_BLOCK) k_matvec_dot(Dims d, int ncomp, const TM* __restrict__ val,
                                                          const T* __restrict__ x, T* __restrict__ y,
                                                          const T* __restrict__ a, double* __restrict__ partial,
                                                          double* __restrict__ partial2) {
  const int NX = d.NX(), NY = d.NY(), NZ = d.NZ();
  const size_t n = d.npad();
  const size_t sy = (size_t)NX, sz = (size_t)NX * NY;
  DotAcc<T> acc, acc2;
  for (size_t P = blockIdx.x * (size_t)blockDim.x + threadIdx.x; P < n; P += (size_t)gridDim.x * blockDim.x) {
    int i, j, k;
    d.ijk(P, i, j, k);
    const bool in = i >= 1 && i <= d.nx && j >= 1 && j <= d.ny && k >= 1 && k <= d.nz;
    const T v0 = k > 0 ? (T)val[0 * n + P - sz] : (T)0;
    const T v1 = j > 0 ? (T)val[1 * n + P - sy] : (T)0;
    const T v2 = i > 0 ? (T)val[2 * n + P - 1] : (T)0;
    const T v3 = (T)val[3 * n + P];
    const T v4 = i < NX - 1 ? (T)val[4 * n + P + 1] : (T)0;
    const T v5 = j < NY - 1 ? (T)val[5 * n + P + sy] : (T)0;
    const T v6 = k < NZ - 1 ? (T)val[6 * n + P + sz] : (T)0;
    for (int ic = 0; ic < ncomp; ++ic) {
      const T* xa = x + ic * n;
      T s = (T)0;
      if (k > 0) s = s + v0 * xa[P - sz];
      if (j > 0) s = s + v1 * xa[P - sy];
      if (i > 0) s = s + v2 * xa[P - 1];
      s = s + v3 * xa[P];
      if (i < NX - 1) s = s + v4 * xa[P + 1];
      if (j < NY - 1) s = s + v5 * xa[P + sy];
      if (k < NZ - 1) s = s + v6 * xa[P + sz];
      const T xp = xa[P];
      s = (T)(-1) * xp + s;
      s = xp + s;
      y[ic * n + P] = s;
      if (in) {
        if (kTwo) {
          acc.add(s, a[ic * n + P]);
          acc2.add(s, s);
        } else {
          acc.add(a[ic * n + P], s);
        }
      }
    }
  }
  __shared__ double ws[RED_BLOCK / 32];
  const double t1 = block_sum(acc.value(), ws);
  if (threadIdx.x == 0) partial[blockIdx.x] = t1;
  if (kTwo) {
    const double t2 = block_sum(acc2.value(), ws);
    if (threadIdx.x == 0) partial2[blockIdx.x] = t2;
  }
}

__device__ __forceinline__ double block_sum_partials(const double* partial, int npart) {
  __shared__ double ws[RED_BLOCK / 32];
  double s = 0.0;
  for (int q = threadIdx.x; q < npart; q += blockDim.x) s += partial[q];
  return block_sum(s, ws);  // complete in thread 0
}

// final reduction + the scalar recurrences of BiCGStabMet_Vec4CellSp
// (MODULE/SpMatrix4CellPar_Mod.f90:283-338); op (asam::ScalarOp) selects what
// the dot product is.
using namespace asam;

__global__ void k_dot_final(const double* __restrict__ partial, int npart, asam::KrylovScalars* sc, int op,
                            double* out) {
  double s = block_sum_partials(partial, npart);
  if (threadIdx.x != 0) return;
  if (out) *out = s;
  switch (op) {
    case OP_STORE_A: sc->dot_a = s; break;
    case OP_STORE_B: sc->dot_b = s; break;
    case OP_RNORM0: sc->rnorm0 = sqrt(s); break;
    case OP_RHO:
      sc->rho_old = sc->rho;
      sc->rho = s;
      if (s == 0.0 && sc->done == 0) sc->done = 3;
      break;
    case OP_ALPHA: sc->alpha = sc->rho / s; break;
    case OP_RNORM_HALF:
      sc->rnorm = sqrt(s);
      if (sc->done == 0 && sc->rnorm <= sc->tol * sc->rnorm0) sc->done = 1;
      break;
    case OP_OMEGA: sc->omega = sc->dot_a / s; break;
    case OP_RNORM_FULL:
      sc->rnorm = sqrt(s);
      if (sc->done == 0 && sc->rnorm <= sc->tol * sc->rnorm0) sc->done = 2;
      break;
  }
}

// beta = (rho/rho_old)*(alpha/omega), computed on the device
__global__ void k_beta(asam::KrylovScalars* sc) {
  if (threadIdx.x == 0 && blockIdx.x == 0) sc->beta = (sc->rho / sc->rho_old) * (sc->alpha / sc->omega);
}

// Vector updates over the whole padded arrays.  The coefficient comes from
// the scalar block (sel) times sign, and an Axpy with a zero coefficient is
// skipped as in Axpy_VectorCell (MODULE/Vector4Cell_Mod.f90:1237-1250).
__device__ __forceinline__ double pick(const asam::KrylovScalars* sc, int sel) {
  return sel == SEL_ALPHA ? sc->alpha : (sel == SEL_OMEGA ? sc->omega : sc->beta);
}

template <typename T>
__global__ void k_axpy_sc(size_t len, const asam::KrylovScalars* sc, int sel, double sign, const T* __restrict__ x,
                          T* __restrict__ y) {
  const T a = (T)(sign * pick(sc, sel));
  if (a == (T)0) return;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < len; q += (size_t)gridDim.x * blockDim.x)
    y[q] = a * x[q] + y[q];
}

// y = y + sign*coef*x (skipped when the coefficient is 0, as k_axpy_sc)
// fused with the partial sums of (y, y) over the interior cells that the
// residual norm test reads next.  One warp per padded x-row of one
// component (every cell updated; the interior rows and cells counted).
template <typename T>
__global__ void __launch_bounds__(RED_BLOCK) k_axpy_dot(Dims d, int ncomp, const asam::KrylovScalars* sc, int sel,
                                                        double sign, const T* __restrict__ x, T* __restrict__ y,
                                                        double* __restrict__ partial) {
  const T a = (T)(sign * pick(sc, sel));
  const int NX = d.NX(), NY = d.NY();
  const long long rows_c = (long long)NY * d.NZ();
  const long long nrow = rows_c * ncomp;
  const size_t n = d.npad();
  const int lane = threadIdx.x & 31;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  DotAcc<T> acc;
  for (long long r = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5; r < nrow; r += nw) {
    const int ic = (int)(r / rows_c);
    const long long jk = r - ic * rows_c;
    const int j = (int)(jk % NY), k = (int)(jk / NY);
    const bool row_in = j >= 1 && j <= d.ny && k >= 1 && k <= d.nz;
    const size_t base = (size_t)ic * n + (size_t)jk * NX;
    for (int i = lane; i < NX; i += 32) {
      T v = y[base + i];
      if (a != (T)0) {
        v = a * x[base + i] + v;
        y[base + i] = v;
      }
      if (row_in && i >= 1 && i <= d.nx) acc.add(v, v);
    }
  }
  __shared__ double ws[RED_BLOCK / 32];
  const double t = block_sum(acc.value(), ws);
  if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

// p = beta*(p - omega*v) + r in the reference's two steps:
// Axpy(-omega,v,p) then Xpay(r,beta,p)
template <typename T>
__global__ void k_pupdate(size_t len, const asam::KrylovScalars* sc, const T* __restrict__ r, const T* __restrict__ v,
                          T* __restrict__ p) {
  const T mo = (T)(-sc->omega);
  const T be = (T)sc->beta;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < len; q += (size_t)gridDim.x * blockDim.x) {
    T pp = p[q];
    if (mo != (T)0) pp = mo * v[q] + pp;
    p[q] = be * pp + r[q];
  }
}

// x = x + alpha*ph (+ omega*rh), the two Axpy calls of :322-323
template <typename T>
__global__ void k_xupdate(size_t len, const asam::KrylovScalars* sc, int with_omega, const T* __restrict__ ph,
                          const T* __restrict__ rh, T* __restrict__ x) {
  const T al = (T)sc->alpha;
  const T om = (T)sc->omega;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < len; q += (size_t)gridDim.x * blockDim.x) {
    T xx = x[q];
    if (al != (T)0) xx = al * ph[q] + xx;
    if (with_omega && om != (T)0) xx = om * rh[q] + xx;
    x[q] = xx;
  }
}

// The device-driven BiCGStab's updates (graph WHILE loop): p = r on the
// first iteration, else beta = (rho/rho_old)*(alpha/omega) and
// p = beta*(p - omega*v) + r -- the operations of k_beta + k_pupdate, in the
// same expressions, compiled in the same translation unit per precision, so
// the rounding (and any contraction) is theirs; and the half-step exit's
// x += alpha*ph when the first half converged (k_xupdate's first term).
template <typename T>
__global__ void k_pupdate_auto(size_t len, const asam::KrylovScalars* sc, const T* __restrict__ r,
                               const T* __restrict__ v, T* __restrict__ p) {
  const bool first = sc->iter == 0;
  const T be = (T)((sc->rho / sc->rho_old) * (sc->alpha / sc->omega));
  const T mo = (T)(-sc->omega);
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < len; q += (size_t)gridDim.x * blockDim.x) {
    if (first) {
      p[q] = r[q];
    } else {
      T pp = p[q];
      if (mo != (T)0) pp = mo * v[q] + pp;
      p[q] = be * pp + r[q];
    }
  }
}
template <typename T>
__global__ void k_xupdate_half(size_t len, const asam::KrylovScalars* sc, const T* __restrict__ ph,
                               T* __restrict__ x) {
  if (sc->done != 1) return;
  const T al = (T)sc->alpha;
  if (al == (T)0) return;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < len; q += (size_t)gridDim.x * blockDim.x) {
    T xx = x[q];
    xx = al * ph[q] + xx;
    x[q] = xx;
  }
}

// y = a*x + y with a host coefficient (skipped when a == 0)
template <typename T>
__global__ void k_axpy_host(size_t len, T a, const T* __restrict__ x, T* __restrict__ y) {
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < len; q += (size_t)gridDim.x * blockDim.x)
    y[q] = a * x[q] + y[q];
}
// y = a*y + x
template <typename T>
__global__ void k_xpay_host(size_t len, const T* __restrict__ x, T a, T* __restrict__ y) {
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < len; q += (size_t)gridDim.x * blockDim.x)
    y[q] = a * y[q] + x[q];
}
template <typename T>
__global__ void k_scale_host(size_t len, T a, T* __restrict__ y) {
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < len; q += (size_t)gridDim.x * blockDim.x)
    y[q] = a * y[q];
}

// ---------------------------------------------------------------------------
// Batched Thomas solve / tridiagonal product on vertical columns:
// MULTI/TriDiagT_Mod.f90:135-155 Solve_1D and :113-133 MatVecT_1D.
// Columns are contiguous (col*n1 + i).
// ---------------------------------------------------------------------------
// The solve, with every global access coalesced.  One warp owns 32
// consecutive columns; since columns are contiguous, a chunk of kTriRows rows
// of those columns is 32 runs of kTriRows consecutive values, which the warp
// copies with consecutive lanes on consecutive addresses of a run (each
// 32-byte sector read whole by one instruction) into a shared tile
// [row][column] (pitch 34 doubles: the sixteen lanes of a half-warp
// touch sixteen different banks in the copy, and the per-column walk reads
// consecutive words).  Each lane then runs its own column's recurrence over the
// chunk from the tile, with the reference's operations in its order, and the
// elimination factors w and the forward values are written back through the
// tile the same way; the back substitution walks the chunks downwards.
constexpr int kTriRows = 8;
constexpr int kTriWarps = 4;  // warps per block, each independent
constexpr int kTriPitch = 34;

template <typename T>
__device__ __forceinline__ void tri_tile_load(T (*tile)[kTriPitch], const T* __restrict__ src, int stride, int c0, int ncol,
                                              int r0, int nrow, int lane) {
  // element e of the chunk: column e / kTriRows, row e % kTriRows
#pragma unroll
  for (int e = lane; e < 32 * kTriRows; e += 32) {
    const int c = e / kTriRows, r = e % kTriRows;
    const int row = r0 + r;
    if (c0 + c < ncol && row >= 0 && row < nrow) tile[r][c] = src[(size_t)(c0 + c) * stride + row];
  }
}
template <typename T>
__device__ __forceinline__ void tri_tile_store(const T (*tile)[kTriPitch], T* __restrict__ dst, int stride, int c0, int ncol,
                                               int r0, int nrow, int lane) {
#pragma unroll
  for (int e = lane; e < 32 * kTriRows; e += 32) {
    const int c = e / kTriRows, r = e % kTriRows;
    const int row = r0 + r;
    if (c0 + c < ncol && row >= 0 && row < nrow) dst[(size_t)(c0 + c) * stride + row] = tile[r][c];
  }
}

template <typename T>
__global__ void __launch_bounds__(32 * kTriWarps) k_tri_solve_w(int ncol, int n1, const T* __restrict__ dd,
                                                                 const T* __restrict__ uu, const T* __restrict__ ll,
                                                                 T* __restrict__ bb, T* __restrict__ ww) {
  __shared__ T sh[kTriWarps][4][kTriRows][kTriPitch];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int c0 = (blockIdx.x * kTriWarps + warp) * 32;
  if (c0 >= ncol) return;  // uniform over the warp
  T(*td)[kTriPitch] = sh[warp][0];
  T(*tu)[kTriPitch] = sh[warp][1];  // u(i-1) in, w(i-1) out
  T(*tl)[kTriPitch] = sh[warp][2];  // l(i-1)
  T(*tb)[kTriPitch] = sh[warp][3];  // b(i) in, forward value out
  const int m = n1 - 1;      // length of u, l and w's used part
  const bool live = c0 + lane < ncol;
  T t = (T)0, g = (T)0;
  // forward elimination, rows [r0, r0 + kTriRows); u, l and w at rows r0-1 ...
  for (int r0 = 0; r0 < n1; r0 += kTriRows) {
    tri_tile_load(td, dd, n1, c0, ncol, r0, n1, lane);
    tri_tile_load(tb, bb, n1, c0, ncol, r0, n1, lane);
    tri_tile_load(tu, uu, m, c0, ncol, r0 - 1, m, lane);
    tri_tile_load(tl, ll, m, c0, ncol, r0 - 1, m, lane);
    __syncwarp();
    if (live) {
      const int nr = min(kTriRows, n1 - r0);
      for (int r = 0; r < nr; ++r) {
        const int i = r0 + r;
        if (i == 0) {
          t = td[r][lane];
          g = tb[r][lane] / t;
        } else {
          const T wi = tu[r][lane] / t;
          tu[r][lane] = wi;
          t = td[r][lane] - tl[r][lane] * wi;
          g = (tb[r][lane] - tl[r][lane] * g) / t;
        }
        tb[r][lane] = g;
      }
    }
    __syncwarp();
    tri_tile_store(tb, bb, n1, c0, ncol, r0, n1, lane);
    tri_tile_store(tu, ww, n1, c0, ncol, r0 - 1, m, lane);
    __syncwarp();
  }
  // back substitution x(i) = g(i) - w(i) x(i+1), i = n1-2 ... 0, chunks downwards
  T x = g;  // x(n1-1) = g(n1-1), already stored
  for (int r0 = ((m - 1) / kTriRows) * kTriRows; m > 0 && r0 >= 0; r0 -= kTriRows) {
    tri_tile_load(tb, bb, n1, c0, ncol, r0, m, lane);
    tri_tile_load(tu, ww, n1, c0, ncol, r0, m, lane);
    __syncwarp();
    if (live) {
      const int nr = min(kTriRows, m - r0);
      for (int r = nr - 1; r >= 0; --r) {
        x = tb[r][lane] - tu[r][lane] * x;
        tb[r][lane] = x;
      }
    }
    __syncwarp();
    tri_tile_store(tb, bb, n1, c0, ncol, r0, m, lane);
    __syncwarp();
  }
}

template <typename T>
__global__ void k_tri_matvec(int ncol, int n1, const T* __restrict__ dd, const T* __restrict__ uu,
                             const T* __restrict__ ll, const T* __restrict__ xx, T* __restrict__ yy) {
  size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (q >= (size_t)ncol * n1) return;
  int col = (int)(q / n1), i = (int)(q % n1);
  const T* d = dd + (size_t)col * n1;
  const T* u = uu + (size_t)col * (n1 - 1);
  const T* l = ll + (size_t)col * (n1 - 1);
  const T* x = xx + (size_t)col * n1;
  T y;
  if (n1 == 1) {
    y = d[0] * x[0];
  } else if (i == 0) {
    y = d[0] * x[0] + u[0] * x[1];
  } else if (i == n1 - 1) {
    y = l[n1 - 2] * x[n1 - 2] + d[n1 - 1] * x[n1 - 1];
  } else {
    y = l[i - 1] * x[i - 1] + d[i] * x[i] + u[i] * x[i + 1];
  }
  yy[q] = y;
}

// Residual of the refinement loop in one pass: r = b + (-1)*MatVecMet(x) (the
// rounding of the separate MatVecMet and Xpay passes), with the per-block
// partial sums of r.r over the interior cells for a following k_dot_final.
template <typename T>
__global__ void k_resid_dot(Dims d, int ncomp, const T* __restrict__ val, const T* __restrict__ x,
                            const T* __restrict__ b, T* __restrict__ r, double* __restrict__ partial) {
  const int NX = d.NX(), NY = d.NY(), NZ = d.NZ();
  const size_t n = d.npad();
  const size_t sy = (size_t)NX, sz = (size_t)NX * NY;
  double acc = 0.0;
  for (size_t P = blockIdx.x * (size_t)blockDim.x + threadIdx.x; P < n; P += (size_t)gridDim.x * blockDim.x) {
    int i, j, k;
    d.ijk(P, i, j, k);
    const bool interior = i > 0 && i < NX - 1 && j > 0 && j < NY - 1 && k > 0 && k < NZ - 1;
    const T v0 = k > 0 ? val[0 * n + P - sz] : (T)0;
    const T v1 = j > 0 ? val[1 * n + P - sy] : (T)0;
    const T v2 = i > 0 ? val[2 * n + P - 1] : (T)0;
    const T v3 = val[3 * n + P];
    const T v4 = i < NX - 1 ? val[4 * n + P + 1] : (T)0;
    const T v5 = j < NY - 1 ? val[5 * n + P + sy] : (T)0;
    const T v6 = k < NZ - 1 ? val[6 * n + P + sz] : (T)0;
    for (int ic = 0; ic < ncomp; ++ic) {
      const T* xa = x + ic * n;
      T s = (T)0;
      if (k > 0) s = s + v0 * xa[P - sz];
      if (j > 0) s = s + v1 * xa[P - sy];
      if (i > 0) s = s + v2 * xa[P - 1];
      s = s + v3 * xa[P];
      if (i < NX - 1) s = s + v4 * xa[P + 1];
      if (j < NY - 1) s = s + v5 * xa[P + sy];
      if (k < NZ - 1) s = s + v6 * xa[P + sz];
      const T xp = xa[P];
      s = (T)(-1) * xp + s;
      s = xp + s;
      const T rv = b[ic * n + P] + (T)(-1) * s;
      r[ic * n + P] = rv;
      if (interior) acc += (double)rv * (double)rv;
    }
  }
  __shared__ double sh[RED_BLOCK];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int w = RED_BLOCK / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

// TotalScalar partials: sum(c*VolB) over the interior (ADVECT/Diagnostic_Mod.f90:13-31)
__global__ void k_mass_partial(Dims d, const double* __restrict__ c, const double* __restrict__ volc,
                               double* __restrict__ partial) {
  const int nx = d.nx, ny = d.ny;
  const size_t nint = (size_t)nx * ny * d.nz;
  double s = 0.0;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < nint; q += (size_t)gridDim.x * blockDim.x) {
    int i = (int)(q % nx) + 1;
    int j = (int)((q / nx) % ny) + 1;
    int k = (int)(q / ((size_t)nx * ny)) + 1;
    size_t P = d.P(i, j, k);
    s += c[P] * volc[P];
  }
  __shared__ double sh[RED_BLOCK];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = RED_BLOCK / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

}  // namespace
