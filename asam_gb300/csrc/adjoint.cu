// Tangent-linear and adjoint (transpose) of the transport stage for one
// passive component, with density and face velocities held fixed.
//
// Forward map of one step (ADVECT/Int_Mod.f90:263-374, transport part), on the
// interior values u of the component (halos are derived by ExchangeCell E):
//   u_i   = u_0 + sum_{j<i} alpha(i-1,j) k_j            (stage state)
//   b_i   = dt * R F(E u_i) + sum_{j<i} beta(i,j) k_j   (R: restriction to the interior)
//   k_i   = A_per^{-1} b_i,  A_per = R A E               (the periodic stage system)
//   u_new = u_0 + sum_j alpha(nS-1,j) k_j
// F is piecewise linear in the component (the Koren limiter switches branch
// with the local gradient ratio), so the tangent-linear model freezes the
// branches of the forward state; A does not depend on the component.  Every
// linear piece has a hand-written transpose here:
//   flux:  dF = G . dphi  (G: per-face derivative coefficients, gather of
//          ADVECT/Advection_Mod.f90:854-1054 and ExchangeFlux/AdvectionScale),
//          dF^T = dphi^T . gather^T
//   DIA:   (A^T x)(c) = sum_d Val(c,d) x(c - shift_d)  -- a gather from the
//          same column-oriented storage (CG/MatSpDiag_Mod.f90:87-108)
//   E^T:   halo values are added back to the interior cells they were copied from
// The adjoint stage solve A_per^T y = b is a BiCGStab on the transposed
// operator with a diagonal preconditioner.
#include <cmath>
#include <cstring>
#include <vector>

#include "context.h"
#include "kernels.cuh"

using namespace asam;

namespace {

constexpr int kB = 256;
inline int grid_of(const Launch& L, size_t n) {
  size_t g = (n + kB - 1) / kB, cap = (size_t)L.sm_count * 16;
  return (int)(g > cap ? cap : (g < 1 ? 1 : g));
}

// d(face flux)/d(phi) along (dL,dC,dR) for the upwind stencil, branches frozen.
__device__ double flux_deriv(double cL, double cC, double cR, double dL, double dC, double dR, double VL,
                             double VC, double VR, double FL, double FR, unsigned char m, bool right, double pref,
                             double ratio, double k1, double k2) {
  const double e = 1.0e-30;
  if (m & 1) {
    dL = ((VC - VL) * dC + VL * dL) / VC;
    cL = ((VC - VL) * cC + VL * cL) / VC;
  }
  if (m & 2) {
    dR = ((VC - VR) * dC + VR * dR) / VC;
    cR = ((VC - VR) * cC + VR * cR) / VC;
  }
  if (m & 4) {
    dL = ((FR - FL) * dC + FL * dL) / FR;
    cL = ((FR - FL) * cC + FL * cL) / FR;
  }
  if (m & 8) {
    dR = ((FL - FR) * dC + FR * dR) / FL;
    cR = ((FL - FR) * cC + FR * cR) / FL;
  }
  // r = (N+e)/(D+e); limiter term S = lim(r)*X with X = cC - cL (right) or cC - cR (left)
  double N, D, dN, dD, X, dX;
  if (right) {
    N = cR - cC; dN = dR - dC;
    D = cC - cL; dD = dC - dL;
    X = cC - cL; dX = dC - dL;
  } else {
    N = cC - cL; dN = dC - dL;
    D = cR - cC; dD = dR - dC;
    X = cC - cR; dX = dC - dR;
  }
  const double r = (N + e) / (D + e);
  const double dr = (dN - r * dD) / (D + e);
  // Koren branch of the forward evaluation (same comparisons as koren())
  const double a = k1 * r + k2;
  double lim, dlim;
  if (a < 1.0) {
    lim = a;
    dlim = k1 * dr;
  } else {
    lim = 1.0;
    dlim = 0.0;
  }
  if (r < lim) {
    lim = r;
    dlim = dr;
  }
  if (0.0 > lim) {
    lim = 0.0;
    dlim = 0.0;
  }
  const double dS = dlim * X + lim * dX;
  return pref * (dC + ratio * dS);
}

// Per-face derivative coefficients (gL, gC, gR) of one component's face flux
// with respect to phi at the upwind cell's left, centre and right neighbours.
template <int AXIS>
__global__ void k_face_dcoef(Dims d, GeomT<double> g, const double* __restrict__ coef,
                             const unsigned char* __restrict__ mask, const double* __restrict__ phi,
                             double* __restrict__ dcoef) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const int ex = AXIS == 0 ? nx + 1 : nx, ey = AXIS == 1 ? ny + 1 : ny, ez = AXIS == 2 ? nz + 1 : nz;
  const size_t nface = (size_t)ex * ey * ez;
  for (size_t f = blockIdx.x * (size_t)blockDim.x + threadIdx.x; f < nface; f += (size_t)gridDim.x * blockDim.x) {
    const double ps = coef[f];
    double gl = 0, gc = 0, gr = 0;
    if (ps != 0.0) {
      const bool right = ps > 0.0;
      const double pref = right ? ps : -ps;
      const double ratio = coef[nface + f], k1 = coef[2 * nface + f], k2 = coef[3 * nface + f];
      const unsigned char m = mask[f];
      const int a = (int)(f % ex);
      const size_t rest = f / ex;
      const int b = (int)(rest % ey), cc = (int)(rest / ey);
      int ci, cj, ck;
      if (AXIS == 0) { ci = a + !right; cj = b + 1; ck = cc + 1; }
      else if (AXIS == 1) { ci = a + 1; cj = b + !right; ck = cc + 1; }
      else { ci = a + 1; cj = b + 1; ck = cc + !right; }
      const size_t PC = d.P(ci, cj, ck);
      const size_t st = AXIS == 0 ? 1 : (AXIS == 1 ? (size_t)d.NX() : (size_t)d.NX() * d.NY());
      const double VL = g.volc[PC - st], VC = g.volc[PC], VR = g.volc[PC + st];
      double FL, FR;
      if (AXIS == 0) { FR = g.fu[d.FU(ci, cj, ck)]; FL = g.fu[d.FU(ci - 1, cj, ck)]; }
      else if (AXIS == 1) { FR = g.fv[d.FV(ci, cj, ck)]; FL = g.fv[d.FV(ci, cj - 1, ck)]; }
      else { FR = g.fw[d.FW(ci, cj, ck)]; FL = g.fw[d.FW(ci, cj, ck - 1)]; }
      const double cL = phi[PC - st], cC = phi[PC], cR = phi[PC + st];
      gl = flux_deriv(cL, cC, cR, 1, 0, 0, VL, VC, VR, FL, FR, m, right, pref, ratio, k1, k2);
      gc = flux_deriv(cL, cC, cR, 0, 1, 0, VL, VC, VR, FL, FR, m, right, pref, ratio, k1, k2);
      gr = flux_deriv(cL, cC, cR, 0, 0, 1, VL, VC, VR, FL, FR, m, right, pref, ratio, k1, k2);
    }
    dcoef[f] = gl;
    dcoef[nface + f] = gc;
    dcoef[2 * nface + f] = gr;
  }
}

// dg(face) = gL dphi(L) + gC dphi(C) + gR dphi(R)
template <int AXIS>
__global__ void k_face_tlm(Dims d, const double* __restrict__ coef, const double* __restrict__ dcoef,
                           const double* __restrict__ dphi, double* __restrict__ dg) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const int ex = AXIS == 0 ? nx + 1 : nx, ey = AXIS == 1 ? ny + 1 : ny, ez = AXIS == 2 ? nz + 1 : nz;
  const size_t nface = (size_t)ex * ey * ez;
  for (size_t f = blockIdx.x * (size_t)blockDim.x + threadIdx.x; f < nface; f += (size_t)gridDim.x * blockDim.x) {
    const double ps = coef[f];
    double v = 0.0;
    if (ps != 0.0) {
      const bool right = ps > 0.0;
      const int a = (int)(f % ex);
      const size_t rest = f / ex;
      const int b = (int)(rest % ey), cc = (int)(rest / ey);
      int ci, cj, ck;
      if (AXIS == 0) { ci = a + !right; cj = b + 1; ck = cc + 1; }
      else if (AXIS == 1) { ci = a + 1; cj = b + !right; ck = cc + 1; }
      else { ci = a + 1; cj = b + 1; ck = cc + !right; }
      const size_t PC = d.P(ci, cj, ck);
      const size_t st = AXIS == 0 ? 1 : (AXIS == 1 ? (size_t)d.NX() : (size_t)d.NX() * d.NY());
      v = dcoef[f] * dphi[PC - st] + dcoef[nface + f] * dphi[PC] + dcoef[2 * nface + f] * dphi[PC + st];
    }
    dg[f] = v;
  }
}

// Transpose of k_flux_gather (one component): lg(face) from lf(padded).
// A face enters the cells on both sides (signs of the scatter order), the
// halo cell beyond a boundary face, and, across a periodic side, the interior
// cell that receives that halo's flux (ExchangeFlux).
template <int AXIS>
__global__ void k_gather_T(Dims d, GeomT<double> g, const double* __restrict__ rvol, const double* __restrict__ lf,
                           double* __restrict__ lg) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const int ex = AXIS == 0 ? nx + 1 : nx, ey = AXIS == 1 ? ny + 1 : ny, ez = AXIS == 2 ? nz + 1 : nz;
  const size_t nface = (size_t)ex * ey * ez;
  const double e = 1.0e-30;
  const int smax = AXIS == 0 ? nx : (AXIS == 1 ? ny : nz);
  const int per = AXIS == 0 ? d.per_x : (AXIS == 1 ? d.per_y : d.per_z);
  for (size_t f = blockIdx.x * (size_t)blockDim.x + threadIdx.x; f < nface; f += (size_t)gridDim.x * blockDim.x) {
    const int a = (int)(f % ex);
    const size_t rest = f / ex;
    const int b = (int)(rest % ey), cc = (int)(rest / ey);
    int i, j, k;
    double vel;
    if (AXIS == 0) { i = a; j = b + 1; k = cc + 1; vel = g.uf[f]; }
    else if (AXIS == 1) { i = a + 1; j = b; k = cc + 1; vel = g.vf[f]; }
    else { i = a + 1; j = b + 1; k = cc; vel = g.wf[f]; }
    const int s = AXIS == 0 ? i : (AXIS == 1 ? j : k);
    const size_t st = AXIS == 0 ? 1 : (AXIS == 1 ? (size_t)d.NX() : (size_t)d.NX() * d.NY());
    const size_t PL = d.P(i, j, k), PR = PL + st;
    // f(P) = ((a*V)/Ve + ex)/Ve for interior P: d f / d a = V/Ve^2
    auto wint = [&](size_t P) { const double V = g.volc[P]; return V * rvol[P] * rvol[P]; };
    double acc = 0.0;
    if (vel != 0.0) {
      const double sL = vel > 0.0 ? -1.0 : 1.0;  // the face is the right face of the left cell
      const double sR = -sL;                     // ... and the left face of the right cell
      if (s >= 1) acc += sL * wint(PL) * lf[PL];
      if (s + 1 <= smax) acc += sR * wint(PR) * lf[PR];
      // boundary faces: the halo beyond the face and the periodic receiver
      if (s == smax && vel > 0.0) {  // halo at s+1 holds the flux
        const double VH = g.volc[PR];
        const double wh = VH / (VH + e);
        acc += wh * rvol[PR] * lf[PR];
        if (per) {
          const size_t Q = PR - (size_t)smax * st;  // interior cell 1 on the axis
          acc += wh * rvol[Q] * lf[Q];
        }
      }
      if (s == 0 && vel < 0.0) {  // halo at s=0 holds the flux
        const double VH = g.volc[PL];
        const double wh = VH / (VH + e);
        acc += wh * rvol[PL] * lf[PL];
        if (per) {
          const size_t Q = PL + (size_t)smax * st;  // interior cell smax
          acc += wh * rvol[Q] * lf[Q];
        }
      }
    }
    lg[f] = acc;
  }
}

// lphi(P) = sum over faces whose upwind stencil contains P of the face's
// derivative coefficient for P's position times lg(face); then lc = lphi/(Rho+Eps).
__global__ void k_phi_T(Dims d, const double* __restrict__ cx, const double* __restrict__ cy,
                        const double* __restrict__ cz, const double* __restrict__ dx_, const double* __restrict__ dy_,
                        const double* __restrict__ dz_, const double* __restrict__ lgx, const double* __restrict__ lgy,
                        const double* __restrict__ lgz, const double* __restrict__ rho, double* __restrict__ lc) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const int NX = d.NX(), NY = d.NY();
  const size_t n = d.npad();
  const size_t nfx = (size_t)(nx + 1) * ny * nz, nfy = (size_t)nx * (ny + 1) * nz, nfz = (size_t)nx * ny * (nz + 1);
  for (size_t P = blockIdx.x * (size_t)blockDim.x + threadIdx.x; P < n; P += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(P % NX), j = (int)((P / NX) % NY), k = (int)(P / ((size_t)NX * NY));
    double acc = 0.0;
    // x faces: face fi between cells fi, fi+1 exists for fi in [0,nx], j,k interior
    if (j >= 1 && j <= ny && k >= 1 && k <= nz) {
      for (int fi = i - 2; fi <= i + 1; ++fi) {
        if (fi < 0 || fi > nx) continue;
        const size_t f = d.UF(fi, j, k);
        const double ps = cx[f];
        if (ps == 0.0) continue;
        const int C = ps > 0.0 ? fi : fi + 1;
        const int pos = i - C;  // -1 L, 0 C, +1 R
        if (pos < -1 || pos > 1) continue;
        acc += dx_[(size_t)(pos + 1) * nfx + f] * lgx[f];
      }
    }
    if (i >= 1 && i <= nx && k >= 1 && k <= nz) {
      for (int fj = j - 2; fj <= j + 1; ++fj) {
        if (fj < 0 || fj > ny) continue;
        const size_t f = d.VF(i, fj, k);
        const double ps = cy[f];
        if (ps == 0.0) continue;
        const int C = ps > 0.0 ? fj : fj + 1;
        const int pos = j - C;
        if (pos < -1 || pos > 1) continue;
        acc += dy_[(size_t)(pos + 1) * nfy + f] * lgy[f];
      }
    }
    if (i >= 1 && i <= nx && j >= 1 && j <= ny) {
      for (int fk = k - 2; fk <= k + 1; ++fk) {
        if (fk < 0 || fk > nz) continue;
        const size_t f = d.WF(i, j, fk);
        const double ps = cz[f];
        if (ps == 0.0) continue;
        const int C = ps > 0.0 ? fk : fk + 1;
        const int pos = k - C;
        if (pos < -1 || pos > 1) continue;
        acc += dz_[(size_t)(pos + 1) * nfz + f] * lgz[f];
      }
    }
    lc[P] = acc / (rho[P] + 1.0e-30);
  }
}

__global__ void k_div_rho(size_t n, const double* __restrict__ x, const double* __restrict__ rho,
                          double* __restrict__ y) {
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
    y[q] = x[q] / (rho[q] + 1.0e-30);
}

// Transpose of the periodic ExchangeCell: every interior cell adds the halo
// cells that were copied from it; afterwards the whole halo layer is zero.
__global__ void k_exchange_T(Dims d, double* __restrict__ x) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const size_t nint = (size_t)nx * ny * nz;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < nint; q += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(q % nx) + 1, j = (int)((q / nx) % ny) + 1, k = (int)(q / ((size_t)nx * ny)) + 1;
    const size_t P = d.P(i, j, k);
    double add = 0.0;
    if (d.per_x) {
      if (i == nx) add += x[d.P(0, j, k)];
      if (i == 1) add += x[d.P(nx + 1, j, k)];
    }
    if (d.per_y) {
      if (j == ny) add += x[d.P(i, 0, k)];
      if (j == 1) add += x[d.P(i, ny + 1, k)];
    }
    if (d.per_z) {
      if (k == nz) add += x[d.P(i, j, 0)];
      if (k == 1) add += x[d.P(i, j, nz + 1)];
    }
    if (add != 0.0) x[P] += add;
  }
}

__global__ void k_zero_halo1(Dims d, double* __restrict__ x) {
  const int NX = d.NX(), NY = d.NY(), NZ = d.NZ();
  const size_t n = d.npad();
  for (size_t P = blockIdx.x * (size_t)blockDim.x + threadIdx.x; P < n; P += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(P % NX), j = (int)((P / NX) % NY), k = (int)(P / ((size_t)NX * NY));
    if (i == 0 || i == NX - 1 || j == 0 || j == NY - 1 || k == 0 || k == NZ - 1) x[P] = 0.0;
  }
}

// y = A^T x for the column-oriented DIA storage: (A^T x)(c) = sum_d Val(c,d) x(c - shift_d)
__global__ void k_matvec_T(Dims d, const double* __restrict__ val, const double* __restrict__ x,
                           double* __restrict__ y) {
  const int NX = d.NX(), NY = d.NY(), NZ = d.NZ();
  const size_t n = d.npad();
  const size_t sy = (size_t)NX, sz = (size_t)NX * NY;
  for (size_t P = blockIdx.x * (size_t)blockDim.x + threadIdx.x; P < n; P += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(P % NX), j = (int)((P / NX) % NY), k = (int)(P / sz);
    double s = 0.0;
    if (k < NZ - 1) s += val[0 * n + P] * x[P + sz];
    if (j < NY - 1) s += val[1 * n + P] * x[P + sy];
    if (i < NX - 1) s += val[2 * n + P] * x[P + 1];
    s += val[3 * n + P] * x[P];
    if (i > 0) s += val[4 * n + P] * x[P - 1];
    if (j > 0) s += val[5 * n + P] * x[P - sy];
    if (k > 0) s += val[6 * n + P] * x[P - sz];
    y[P] = s;
  }
}

// interior-only dot product of two single fields
__global__ void k_dot1_partial(Dims d, const double* __restrict__ x, const double* __restrict__ y,
                               double* __restrict__ partial) {
  const int nx = d.nx, ny = d.ny;
  const size_t nint = (size_t)nx * ny * d.nz;
  double s = 0.0;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < nint; q += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(q % nx) + 1, j = (int)((q / nx) % ny) + 1, k = (int)(q / ((size_t)nx * ny)) + 1;
    const size_t P = d.P(i, j, k);
    s += x[P] * y[P];
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

__global__ void k_sum_partials(const double* __restrict__ partial, int npart, double* out) {
  double s = block_sum_partials(partial, npart);
  if (threadIdx.x == 0) *out = s;
}

__global__ void k_axpby(size_t n, double a, const double* __restrict__ x, double b, double* __restrict__ y) {
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
    y[q] = a * x[q] + b * y[q];
}

__global__ void k_div_diag(size_t n, const double* __restrict__ val, const double* __restrict__ x,
                           double* __restrict__ y) {
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
    y[q] = x[q] * val[7 * n + q];
}

// J = sum_box (c/rho)^2 V and dJ/dc = 2 c V / rho^2 on the box (interior cells)
__global__ void k_objective(Dims d, const double* __restrict__ c, const double* __restrict__ rho,
                            const double* __restrict__ volc, int i0, int i1, int j0, int j1, int k0, int k1,
                            double* __restrict__ grad, double* __restrict__ partial) {
  const int nx = d.nx, ny = d.ny;
  const size_t nint = (size_t)nx * ny * d.nz;
  double s = 0.0;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < nint; q += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(q % nx) + 1, j = (int)((q / nx) % ny) + 1, k = (int)(q / ((size_t)nx * ny)) + 1;
    const size_t P = d.P(i, j, k);
    double gv = 0.0;
    if (i >= i0 && i <= i1 && j >= j0 && j <= j1 && k >= k0 && k <= k1) {
      const double r = rho[P] + 1.0e-30;
      const double qv = c[P] / r;
      s += qv * qv * volc[P];
      gv = 2.0 * qv * volc[P] / r;
    }
    if (grad) grad[P] = gv;
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

// ---------------------------------------------------------------------------
// Wind and density derivatives (coupled density-component adjoint).
//
// Stage operator: A = I - bdt*J with every entry of column P of J a sum of
// jac_term(u_f, ., F, V, Rho_P) = Half*(|u_f| +/- u_f)*F/V/(Rho_P+Eps) terms
// (k_jac), each depending on one face velocity u_f (homogeneous of degree 1
// on either side of u_f = 0) and on Rho_P only through 1/(Rho_P+Eps):
//   d term/d u_f = term/u_f,  d term/d Rho_P = -term/(Rho_P+Eps).
// For the stage solve A k = b the adjoint contribution of dA is
//   -lb^T dA k = bdt * sum_terms sigma * d(term) * lb(row) * k(P)
// (sigma the term's sign in J(row, P)), summed over the components.  Faces
// with u_f = 0 are not differentiable (the upwind side switches) and get 0.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double jac_term_d(double vel, bool plus, double F, double Vden, double rho) {
  const double s = plus ? (fabs(vel) + vel) : (fabs(vel) - vel);
  return 0.5 * s * F / Vden / (rho + 1.0e-30);
}

// k (exchanged) and lb (zero halos) hold nc fields each, `stride` apart.
__global__ void k_jac_adj(Dims d, GeomT<double> g, const double* __restrict__ rho, double bdt, int nc,
                          size_t stride, const double* __restrict__ lb, const double* __restrict__ kk_,
                          double* __restrict__ gu, double* __restrict__ gv, double* __restrict__ gw,
                          double* __restrict__ grho) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const int NX = d.NX(), NY = d.NY();
  const size_t n = d.npad();
  const double e = 1.0e-30;
  const size_t sx = 1, sy = (size_t)NX, sz = (size_t)NX * NY;
  for (size_t P = blockIdx.x * (size_t)blockDim.x + threadIdx.x; P < n; P += (size_t)gridDim.x * blockDim.x) {
    int i, j, k;
    d.ijk(P, i, j, k);
    const bool ii = i >= 1 && i <= nx, jj = j >= 1 && j <= ny, kk = k >= 1 && k <= nz;
    const double rP = rho[P];
    const double VP = g.volc[P] + e;
    // w(row) = sum over components of lb(row) * k(P)
    auto wrow = [&](size_t row) {
      double s = 0.0;
      for (int m = 0; m < nc; ++m) s += lb[m * stride + row] * kk_[m * stride + P];
      return s;
    };
    double drho = 0.0;
    // one term of J(row, P) with sign sigma, velocity u (array a at index f)
    auto term = [&](double* ga, size_t fidx, double u, bool plus, double F, double Vden, size_t row, double sigma) {
      const double t = jac_term_d(u, plus, F, Vden, rP);
      if (t == 0.0) return;
      const double c = bdt * sigma * t * wrow(row);
      if (u != 0.0) atomicAdd(ga + fidx, c / u);
      drho += -c / (rP + e);
    };
    auto actx = [&](int fi) { return jj && kk && fi >= 0 && fi <= nx && ((fi >= 1 && fi <= nx - 1) || d.per_x); };
    auto acty = [&](int fj) { return ii && kk && fj >= 0 && fj <= ny && ((fj >= 1 && fj <= ny - 1) || d.per_y); };
    auto actz = [&](int fk) { return ii && jj && fk >= 0 && fk <= nz && ((fk >= 1 && fk <= nz - 1) || d.per_z); };
    // off-diagonals: slot 2 -> row P+1, 4 -> P-1, 1 -> P+NX, 5 -> P-NX, 0 -> P+NXY, 6 -> P-NXY;
    // the face-halo rows fold the same term into the diagonal with sign -1
    if (actx(i)) {
      const size_t f = d.UF(i, j, k);
      term(gu, f, g.uf[f], true, g.fu[d.FU(i, j, k)], g.volc[P + sx] + e, P + sx, 1.0);
      if (i == 0) term(gu, f, g.uf[f], true, g.fu[d.FU(i, j, k)], g.volc[P + sx] + e, P, -1.0);
    }
    if (actx(i - 1)) {
      const size_t f = d.UF(i - 1, j, k);
      term(gu, f, g.uf[f], false, g.fu[d.FU(i - 1, j, k)], g.volc[P - sx] + e, P - sx, 1.0);
      if (i == nx + 1) term(gu, f, g.uf[f], false, g.fu[d.FU(i - 1, j, k)], g.volc[P - sx] + e, P, -1.0);
    }
    if (acty(j)) {
      const size_t f = d.VF(i, j, k);
      term(gv, f, g.vf[f], true, g.fv[d.FV(i, j, k)], g.volc[P + sy] + e, P + sy, 1.0);
      if (j == 0) term(gv, f, g.vf[f], true, g.fv[d.FV(i, j, k)], g.volc[P + sy] + e, P, -1.0);
    }
    if (acty(j - 1)) {
      const size_t f = d.VF(i, j - 1, k);
      term(gv, f, g.vf[f], false, g.fv[d.FV(i, j - 1, k)], g.volc[P - sy] + e, P - sy, 1.0);
      if (j == ny + 1) term(gv, f, g.vf[f], false, g.fv[d.FV(i, j - 1, k)], g.volc[P - sy] + e, P, -1.0);
    }
    if (actz(k)) {
      const size_t f = d.WF(i, j, k);
      term(gw, f, g.wf[f], true, g.fw[d.FW(i, j, k)], g.volc[P + sz] + e, P + sz, 1.0);
      if (k == 0) term(gw, f, g.wf[f], true, g.fw[d.FW(i, j, k)], g.volc[P + sz] + e, P, -1.0);
    }
    if (actz(k - 1)) {
      const size_t f = d.WF(i, j, k - 1);
      term(gw, f, g.wf[f], false, g.fw[d.FW(i, j, k - 1)], g.volc[P - sz] + e, P - sz, 1.0);
      if (k == nz + 1) term(gw, f, g.wf[f], false, g.fw[d.FW(i, j, k - 1)], g.volc[P - sz] + e, P, -1.0);
    }
    // diagonal terms (sign -1 in J(P, P)), the interior loops and the periodic branches of k_jac
    if (jj && kk && i - 1 >= 1 && i - 1 <= nx - 1) {
      const size_t f = d.UF(i - 1, j, k);
      term(gu, f, g.uf[f], false, g.fu[d.FU(i - 1, j, k)], VP, P, -1.0);
    }
    if (jj && kk && i >= 1 && i <= nx - 1) {
      const size_t f = d.UF(i, j, k);
      term(gu, f, g.uf[f], true, g.fu[d.FU(i, j, k)], VP, P, -1.0);
    }
    if (ii && kk && j - 1 >= 1 && j - 1 <= ny - 1) {
      const size_t f = d.VF(i, j - 1, k);
      term(gv, f, g.vf[f], false, g.fv[d.FV(i, j - 1, k)], VP, P, -1.0);
    }
    if (ii && kk && j >= 1 && j <= ny - 1) {
      const size_t f = d.VF(i, j, k);
      term(gv, f, g.vf[f], true, g.fv[d.FV(i, j, k)], VP, P, -1.0);
    }
    if (ii && jj && k - 1 >= 1 && k - 1 <= nz - 1) {
      const size_t f = d.WF(i, j, k - 1);
      term(gw, f, g.wf[f], false, g.fw[d.FW(i, j, k - 1)], VP, P, -1.0);
    }
    if (ii && jj && k >= 1 && k <= nz - 1) {
      const size_t f = d.WF(i, j, k);
      term(gw, f, g.wf[f], true, g.fw[d.FW(i, j, k)], VP, P, -1.0);
    }
    if (d.per_x && jj && kk) {
      if (i == 0) term(gu, d.UF(0, j, k), g.uf[d.UF(0, j, k)], true, g.fu[d.FU(0, j, k)], VP, P, -1.0);
      if (i == 1) term(gu, d.UF(0, j, k), g.uf[d.UF(0, j, k)], false, g.fu[d.FU(0, j, k)], VP, P, -1.0);
      if (i == nx) term(gu, d.UF(nx, j, k), g.uf[d.UF(nx, j, k)], true, g.fu[d.FU(nx, j, k)], VP, P, -1.0);
      if (i == nx + 1) term(gu, d.UF(nx, j, k), g.uf[d.UF(nx, j, k)], false, g.fu[d.FU(nx, j, k)], VP, P, -1.0);
    }
    if (d.per_y && ii && kk) {
      if (j == 0) term(gv, d.VF(i, 0, k), g.vf[d.VF(i, 0, k)], true, g.fv[d.FV(i, 0, k)], VP, P, -1.0);
      if (j == 1) term(gv, d.VF(i, 0, k), g.vf[d.VF(i, 0, k)], false, g.fv[d.FV(i, 0, k)], VP, P, -1.0);
      if (j == ny) term(gv, d.VF(i, ny, k), g.vf[d.VF(i, ny, k)], true, g.fv[d.FV(i, ny, k)], VP, P, -1.0);
      if (j == ny + 1) term(gv, d.VF(i, ny, k), g.vf[d.VF(i, ny, k)], false, g.fv[d.FV(i, ny, k)], VP, P, -1.0);
    }
    if (d.per_z && ii && jj) {
      if (k == 0) term(gw, d.WF(i, j, 0), g.wf[d.WF(i, j, 0)], true, g.fw[d.FW(i, j, 0)], VP, P, -1.0);
      if (k == 1) term(gw, d.WF(i, j, 0), g.wf[d.WF(i, j, 0)], false, g.fw[d.FW(i, j, 0)], VP, P, -1.0);
      if (k == nz) term(gw, d.WF(i, j, nz), g.wf[d.WF(i, j, nz)], true, g.fw[d.FW(i, j, nz)], VP, P, -1.0);
      if (k == nz + 1) term(gw, d.WF(i, j, nz), g.wf[d.WF(i, j, nz)], false, g.fw[d.FW(i, j, nz)], VP, P, -1.0);
    }
    grho[P] += drho;
  }
}

// Wind part of the flux adjoint: the stored face flux g = |u| F recon (the
// upwind reconstruction) gives dg/du = g/u on faces with u != 0, so
// gface += scale * lg * g / u with lg the face adjoint of the gather transpose.
__global__ void k_wind_flux_T(size_t nface, const double* __restrict__ vel, const double* __restrict__ lg,
                              const double* __restrict__ gfl, double scale, double* __restrict__ gface) {
  for (size_t f = blockIdx.x * (size_t)blockDim.x + threadIdx.x; f < nface; f += (size_t)gridDim.x * blockDim.x) {
    const double u = vel[f];
    if (u != 0.0) gface[f] += scale * lg[f] * gfl[f] / u;
  }
}

// density part of a component's flux adjoint: phi = c/(Rho+Eps) gives
// d phi/d Rho = -phi/(Rho+Eps), so lr = -phi * lc with lc = lphi/(Rho+Eps)
__global__ void k_rho_from_phi(size_t n, const double* __restrict__ phi, const double* __restrict__ lc,
                               double* __restrict__ lr) {
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
    lr[q] = -phi[q] * lc[q];
}

// J = sum_box (c/(Rho+Eps))^2 V, dJ/dc = 2 q V/(Rho+Eps), dJ/dRho = -2 q^2 V/(Rho+Eps)
__global__ void k_objective2(Dims d, const double* __restrict__ c, const double* __restrict__ rho,
                             const double* __restrict__ volc, int i0, int i1, int j0, int j1, int k0, int k1,
                             double* __restrict__ gc, double* __restrict__ gr, double* __restrict__ partial) {
  const int nx = d.nx, ny = d.ny;
  const size_t nint = (size_t)nx * ny * d.nz;
  double s = 0.0;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < nint; q += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(q % nx) + 1, j = (int)((q / nx) % ny) + 1, k = (int)(q / ((size_t)nx * ny)) + 1;
    const size_t P = d.P(i, j, k);
    double a = 0.0, b = 0.0;
    if (i >= i0 && i <= i1 && j >= j0 && j <= j1 && k >= k0 && k <= k1) {
      const double r = rho[P] + 1.0e-30;
      const double qv = c[P] / r;
      s += qv * qv * volc[P];
      a = 2.0 * qv * volc[P] / r;
      b = -2.0 * qv * qv * volc[P] / r;
    }
    gc[P] = a;
    gr[P] = b;
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

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct AdjWork {
  size_t npad = 0;
  double *dcx = nullptr, *dcy = nullptr, *dcz = nullptr;  // derivative coefficients
  double *gx = nullptr, *gy = nullptr, *gz = nullptr;     // face (adjoint) fluxes, one component
  double *phi = nullptr, *t1 = nullptr, *t2 = nullptr;
  // adjoint BiCGStab vectors
  double *r = nullptr, *rt = nullptr, *p = nullptr, *v = nullptr, *s = nullptr, *tt = nullptr, *ph = nullptr,
         *sh = nullptr;
  // stage vectors of the tangent-linear / adjoint steps
  double *ui = nullptr, *bi = nullptr, *lb = nullptr, *lu = nullptr, *l0 = nullptr, *lam = nullptr;
  std::vector<double*> all() {
    return {dcx, dcy, dcz, gx, gy, gz, phi, t1, t2, r, rt, p, v, s, tt, ph, sh, ui, bi, lb, lu, l0, lam};
  }
};

int adj_alloc(asam_ctx* h, AdjWork& w) {
  const Dims& d = h->d;
  w.npad = h->npad;
  struct A {
    double** p;
    size_t n;
  } al[] = {{&w.dcx, 3 * d.n_uf()}, {&w.dcy, 3 * d.n_vf()}, {&w.dcz, 3 * d.n_wf()}, {&w.gx, d.n_uf()},
            {&w.gy, d.n_vf()},      {&w.gz, d.n_wf()},      {&w.phi, h->npad},      {&w.t1, h->npad},
            {&w.t2, h->npad},       {&w.r, h->npad},        {&w.rt, h->npad},       {&w.p, h->npad},
            {&w.v, h->npad},        {&w.s, h->npad},        {&w.tt, h->npad},       {&w.ph, h->npad},
            {&w.sh, h->npad},       {&w.ui, h->npad},       {&w.bi, h->npad},       {&w.lb, h->npad},
            {&w.lu, h->npad},       {&w.l0, h->npad},       {&w.lam, h->npad}};
  for (auto& a : al) CK(cudaMalloc((void**)a.p, a.n * sizeof(double)));
  return kOk;
}
void adj_free(AdjWork& w) {
  for (double* p : w.all())
    if (p) cudaFree(p);
  w = AdjWork();
}

double* comp_ptr(asam_ctx* h, const double* c, int comp) { return const_cast<double*>(c) + (size_t)comp * h->npad; }

// derivative coefficients of component `comp` of state c (halos current)
void flux_dcoef(asam_ctx* h, AdjWork& w, const double* c, int comp) {
  const Launch& L = h->L;
  const Dims& d = h->d;
  const double* rho = c + (size_t)h->cfg.rho_pos * h->npad;
  k_div_rho<<<grid_of(L, h->npad), kB, 0, L.stream>>>(h->npad, comp_ptr(h, c, comp), rho, w.phi);
  k_face_dcoef<0><<<grid_of(L, d.n_uf()), kB, 0, L.stream>>>(d, h->geom(), h->coef_x, h->mask_x, w.phi, w.dcx);
  k_face_dcoef<1><<<grid_of(L, d.n_vf()), kB, 0, L.stream>>>(d, h->geom(), h->coef_y, h->mask_y, w.phi, w.dcy);
  k_face_dcoef<2><<<grid_of(L, d.n_wf()), kB, 0, L.stream>>>(d, h->geom(), h->coef_z, h->mask_z, w.phi, w.dcz);
  count_launches(4);
}

// df = F'(c) dc for the coefficients in w (padded single fields)
void flux_tlm(asam_ctx* h, AdjWork& w, const double* rho, const double* dc, double* df) {
  const Launch& L = h->L;
  const Dims& d = h->d;
  k_div_rho<<<grid_of(L, h->npad), kB, 0, L.stream>>>(h->npad, dc, rho, w.t1);
  k_face_tlm<0><<<grid_of(L, d.n_uf()), kB, 0, L.stream>>>(d, h->coef_x, w.dcx, w.t1, w.gx);
  k_face_tlm<1><<<grid_of(L, d.n_vf()), kB, 0, L.stream>>>(d, h->coef_y, w.dcy, w.t1, w.gy);
  k_face_tlm<2><<<grid_of(L, d.n_wf()), kB, 0, L.stream>>>(d, h->coef_z, w.dcz, w.t1, w.gz);
  launch_flux_gather(L, d, h->geom(), 1, w.gx, w.gy, w.gz, h->rvol, df, nullptr);
  count_launches(4);
}

// lc = F'(c)^T lf
void flux_adj(asam_ctx* h, AdjWork& w, const double* rho, const double* lf, double* lc) {
  const Launch& L = h->L;
  const Dims& d = h->d;
  k_gather_T<0><<<grid_of(L, d.n_uf()), kB, 0, L.stream>>>(d, h->geom(), h->rvol, lf, w.gx);
  k_gather_T<1><<<grid_of(L, d.n_vf()), kB, 0, L.stream>>>(d, h->geom(), h->rvol, lf, w.gy);
  k_gather_T<2><<<grid_of(L, d.n_wf()), kB, 0, L.stream>>>(d, h->geom(), h->rvol, lf, w.gz);
  k_phi_T<<<grid_of(L, h->npad), kB, 0, L.stream>>>(d, h->coef_x, h->coef_y, h->coef_z, w.dcx, w.dcy, w.dcz, w.gx,
                                                    w.gy, w.gz, rho, lc);
  count_launches(4);
}

int dot1(asam_ctx* h, const double* x, const double* y, double* out) {
  k_dot1_partial<<<RED_GRID, RED_BLOCK, 0, h->L.stream>>>(h->d, x, y, h->partial);
  k_sum_partials<<<1, RED_BLOCK, 0, h->L.stream>>>(h->partial, RED_GRID, h->red_out);
  count_launches(2);
  return reduce_to_host(h, out);
}

void axpby(asam_ctx* h, double a, const double* x, double b, double* y) {
  k_axpby<<<grid_of(h->L, h->npad), kB, 0, h->L.stream>>>(h->npad, a, x, b, y);
  count_launches(1);
}

// Transpose of the halo derivation of a state field of component comp at the
// start of a stage: the periodic ExchangeCell and the outer-wall rule
// (k_bound_cond); both read interior cells only and write disjoint halos, so
// their transposes add independently.  The halo layer is left to the caller.
void state_halo_T(asam_ctx* h, int comp, double* x) {
  const Launch& L = h->L;
  const size_t nint = (size_t)h->d.nx * h->d.ny * h->d.nz;
  k_exchange_T<<<grid_of(L, nint), kB, 0, L.stream>>>(h->d, x);
  k_bound_cond_T<double><<<grid_of(L, nint), kB, 0, L.stream>>>(h->d, comp, h->bc, x);
  count_launches(2);
}

// y = A_per^T x = E^T A^T Z x  (x: interior values, halos ignored; y: zero halos)
void matvec_per_T(asam_ctx* h, AdjWork& w, const double* x, double* y) {
  const Launch& L = h->L;
  cudaMemcpyAsync(w.t2, x, h->npad * sizeof(double), cudaMemcpyDeviceToDevice, L.stream);
  k_zero_halo1<<<grid_of(L, h->npad), kB, 0, L.stream>>>(h->d, w.t2);
  k_matvec_T<<<grid_of(L, h->npad), kB, 0, L.stream>>>(h->d, h->val, w.t2, y);
  k_exchange_T<<<grid_of(L, (size_t)h->d.nx * h->d.ny * h->d.nz), kB, 0, L.stream>>>(h->d, y);
  k_zero_halo1<<<grid_of(L, h->npad), kB, 0, L.stream>>>(h->d, y);
  count_launches(4);
}

// Solve A_per^T x = b (interior) by BiCGStab with a diagonal preconditioner.
int bicgstab_T(asam_ctx* h, AdjWork& w, double* x, const double* b, int maxiter, double tol, int* iters) {
  const Launch& L = h->L;
  const size_t n = h->npad;
  CK(cudaMemsetAsync(x, 0, n * sizeof(double), L.stream));
  CK(cudaMemcpyAsync(w.r, b, n * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));
  k_zero_halo1<<<grid_of(L, n), kB, 0, L.stream>>>(h->d, w.r);
  CK(cudaMemcpyAsync(w.rt, w.r, n * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));
  CK(cudaMemsetAsync(w.p, 0, n * sizeof(double), L.stream));
  CK(cudaMemsetAsync(w.v, 0, n * sizeof(double), L.stream));
  double rr0 = 0;
  int rc = dot1(h, w.r, w.r, &rr0);
  if (rc) return rc;
  const double rn0 = std::sqrt(rr0);
  if (iters) *iters = 0;
  if (rn0 == 0.0) return kOk;
  double rho = 1, alpha = 1, omega = 1;
  for (int it = 1; it <= maxiter; ++it) {
    double rho_new = 0;
    if ((rc = dot1(h, w.rt, w.r, &rho_new))) return rc;
    if (rho_new == 0.0) return kBreakdown;
    const double beta = (rho_new / rho) * (alpha / omega);
    rho = rho_new;
    // p = r + beta (p - omega v)
    axpby(h, -omega, w.v, 1.0, w.p);
    axpby(h, 1.0, w.r, beta, w.p);
    k_div_diag<<<grid_of(L, n), kB, 0, L.stream>>>(n, h->val, w.p, w.ph);
    matvec_per_T(h, w, w.ph, w.v);
    double rtv = 0;
    if ((rc = dot1(h, w.rt, w.v, &rtv))) return rc;
    alpha = rho / rtv;
    // s = r - alpha v
    CK(cudaMemcpyAsync(w.s, w.r, n * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));
    axpby(h, -alpha, w.v, 1.0, w.s);
    axpby(h, alpha, w.ph, 1.0, x);
    double ss = 0;
    if ((rc = dot1(h, w.s, w.s, &ss))) return rc;
    if (std::sqrt(ss) <= tol * rn0) {
      if (iters) *iters = it;
      return kOk;
    }
    k_div_diag<<<grid_of(L, n), kB, 0, L.stream>>>(n, h->val, w.s, w.sh);
    matvec_per_T(h, w, w.sh, w.tt);
    double ts = 0, tt = 0;
    if ((rc = dot1(h, w.tt, w.s, &ts))) return rc;
    if ((rc = dot1(h, w.tt, w.tt, &tt))) return rc;
    omega = ts / tt;
    axpby(h, omega, w.sh, 1.0, x);
    CK(cudaMemcpyAsync(w.r, w.s, n * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));
    axpby(h, -omega, w.tt, 1.0, w.r);
    double r2 = 0;
    if ((rc = dot1(h, w.r, w.r, &r2))) return rc;
    if (std::sqrt(r2) <= tol * rn0) {
      if (iters) *iters = it;
      return kOk;
    }
    count_launches(4);
  }
  if (iters) *iters = 2 * maxiter;
  return kNotConverged;
}

// forward solve A_per x = b for one field through the multi-component driver:
// the field is placed in component slot 0 of a 1-component view.
int solve_per(asam_ctx* h, double* x, const double* b, double tol) {
  // the library's BiCGStab works on ncomp fields; run it on a state whose
  // other components are zero (their solution stays zero)
  const size_t n = h->npad;
  double* bb = h->stage_a;
  double* xx = h->stage_b;
  CK(cudaMemsetAsync(bb, 0, h->len * sizeof(double), h->L.stream));
  CK(cudaMemsetAsync(xx, 0, h->len * sizeof(double), h->L.stream));
  CK(cudaMemcpyAsync(bb, b, n * sizeof(double), cudaMemcpyDeviceToDevice, h->L.stream));
  int it = 200;
  double t = tol;
  int rc = bicgstab_dev<double>(h, h->val, xx, bb, &it, &t, h->w64, true);
  if (rc != kOk && rc != kNotConverged) return rc;
  CK(cudaMemcpyAsync(x, xx, n * sizeof(double), cudaMemcpyDeviceToDevice, h->L.stream));
  return kOk;
}

struct StepTraj {
  std::vector<double*> stage;  // full states at the start of each stage (halos current)
};

// forward step from c (device, full state), recording the stage states
int forward_record(asam_ctx* h, const double* c, double dt, double tol, std::vector<double*>& stage_states) {
  const Launch& L = h->L;
  const size_t len = h->len;
  // run the forward step stage by stage with the library's driver on a copy;
  // the stage states are reconstructed from the increments
  double* cur = stage_states[h->nstage];  // scratch full state
  CK(cudaMemcpyAsync(cur, c, len * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));
  CK(cudaMemcpyAsync(h->cold, cur, len * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));
  const Dims& d = h->d;
  const int nc = h->cfg.ncomp;
  for (int is = 0; is < h->nstage; ++is) {
    launch_exchange_cell(L, d, nc, cur);
    launch_bound_cond(L, d, nc, 0, h->bc, cur);
    CK(cudaMemcpyAsync(stage_states[is], cur, len * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));
    if (is == 0) {
      int rc = jac_dev(h, cur, dt);
      if (rc) return rc;
    }
    int rc = fcn_dev(h, cur, h->rhs);
    if (rc) return rc;
    launch_scale_host(L, len, dt, h->rhs);
    for (int js = 0; js < is; ++js)
      launch_axpy_host(L, len, h->beta[is * 4 + js], h->incr + (size_t)js * len, h->rhs);
    double* x = h->incr + (size_t)is * len;
    CK(cudaMemsetAsync(x, 0, len * sizeof(double), L.stream));
    int it = 200;
    double t = tol;
    rc = bicgstab_dev<double>(h, h->val, x, h->rhs, &it, &t, h->w64, true);
    if (rc != kOk && rc != kNotConverged) return rc;
    launch_exchange_cell(L, d, nc, x);
    CK(cudaMemcpyAsync(cur, h->cold, len * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));
    for (int js = 0; js <= is; ++js) launch_axpy_host(L, len, h->alpha[is * 4 + js], h->incr + (size_t)js * len, cur);
  }
  return check_launch();
}

// tangent-linear step: du (interior of component comp) -> du_out, around state c
int step_tlm(asam_ctx* h, AdjWork& w, const std::vector<double*>& stage_states, int comp, const double* du,
             double* du_out, double dt, double tol, std::vector<double*>& dk) {
  const Launch& L = h->L;
  const size_t n = h->npad;
  const double* rho = stage_states[0] + (size_t)h->cfg.rho_pos * n;
  double* ui = w.ui;  // stage perturbation (padded)
  double* bi = w.bi;
  for (int is = 0; is < h->nstage; ++is) {
    CK(cudaMemcpyAsync(ui, du, n * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));
    for (int js = 0; js < is; ++js) axpby(h, h->alpha[(is - 1) * 4 + js], dk[js], 1.0, ui);
    k_zero_halo1<<<grid_of(L, n), kB, 0, L.stream>>>(h->d, ui);
    launch_exchange_cell(L, h->d, 1, ui);
    launch_bound_cond(L, h->d, 1, comp, h->bc, ui);
    flux_dcoef(h, w, stage_states[is], comp);
    flux_tlm(h, w, rho, ui, bi);
    k_axpby<<<grid_of(L, n), kB, 0, L.stream>>>(n, 0.0, bi, dt, bi);
    for (int js = 0; js < is; ++js) axpby(h, h->beta[is * 4 + js], dk[js], 1.0, bi);
    k_zero_halo1<<<grid_of(L, n), kB, 0, L.stream>>>(h->d, bi);
    count_launches(3);
    int rc = solve_per(h, dk[is], bi, tol);
    if (rc) return rc;
    k_zero_halo1<<<grid_of(L, n), kB, 0, L.stream>>>(h->d, dk[is]);
    count_launches(1);
  }
  CK(cudaMemcpyAsync(du_out, du, n * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));
  for (int js = 0; js < h->nstage; ++js) axpby(h, h->alpha[(h->nstage - 1) * 4 + js], dk[js], 1.0, du_out);
  k_zero_halo1<<<grid_of(L, n), kB, 0, L.stream>>>(h->d, du_out);
  count_launches(1);
  return check_launch();
}

// adjoint step: lam (interior) -> lam_out, transpose of step_tlm
int step_adj(asam_ctx* h, AdjWork& w, const std::vector<double*>& stage_states, int comp, const double* lam,
             double* lam_out, double dt, double tol, std::vector<double*>& lk) {
  const Launch& L = h->L;
  const size_t n = h->npad;
  const int ns = h->nstage;
  const double* rho = stage_states[0] + (size_t)h->cfg.rho_pos * n;
  double* lb = w.lb;
  double* lu = w.lu;
  double* l0 = w.l0;
  CK(cudaMemcpyAsync(l0, lam, n * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));
  k_zero_halo1<<<grid_of(L, n), kB, 0, L.stream>>>(h->d, l0);
  count_launches(1);
  for (int j = 0; j < ns; ++j) {
    CK(cudaMemsetAsync(lk[j], 0, n * sizeof(double), L.stream));
    axpby(h, h->alpha[(ns - 1) * 4 + j], l0, 1.0, lk[j]);
  }
  // lam_out accumulates the direct path u_new = u_0 + ...
  double* acc = lam_out;
  CK(cudaMemcpyAsync(acc, l0, n * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));
  for (int is = ns - 1; is >= 0; --is) {
    int rc = bicgstab_T(h, w, lb, lk[is], 400, tol, nullptr);
    if (rc != kOk && rc != kNotConverged) return rc;
    for (int js = 0; js < is; ++js) axpby(h, h->beta[is * 4 + js], lb, 1.0, lk[js]);
    // lu = dt * E^T F'^T Z lb
    k_zero_halo1<<<grid_of(L, n), kB, 0, L.stream>>>(h->d, lb);
    flux_dcoef(h, w, stage_states[is], comp);
    flux_adj(h, w, rho, lb, lu);
    state_halo_T(h, comp, lu);
    k_zero_halo1<<<grid_of(L, n), kB, 0, L.stream>>>(h->d, lu);
    count_launches(1);
    axpby(h, dt, lu, 1.0, acc);
    for (int js = 0; js < is; ++js) axpby(h, dt * h->alpha[(is - 1) * 4 + js], lu, 1.0, lk[js]);
  }
  return check_launch();
}

// Coupled adjoint step of (Rho, component comp) with the face velocities as
// parameters: (lr, lc) adjoints of the step's end state (interior) ->
// (lr_out, lc_out) adjoints of its start state; the wind gradient of the step
// is added to (gu, gv, gw).  Needs the stage states of the step
// (stage_states[0..nS-1], halos current), its increments in h->incr
// (exchanged) and its stage matrix in h->val.  Density enters through the
// mixing ratio of the component's flux and through the stage matrix; its own
// flux does not depend on it (phi_Rho = Rho/(Rho+Eps) = 1 in FP64).
struct CoupledWork {
  double *lkc[4], *lkr[4];  // adjoints of the increments
  double *lbc, *lbr, *luc, *lur, *accc, *accr, *grho, *lrp;
  std::vector<double*> own;
  int alloc(asam_ctx* h) {
    const size_t n = h->npad;
    for (int q = 0; q < 4; ++q) {
      lkc[q] = lkr[q] = nullptr;
    }
    double** ptrs[] = {&lbc, &lbr, &luc, &lur, &accc, &accr, &grho, &lrp};
    for (double** q : ptrs) {
      CK(cudaMalloc((void**)q, n * sizeof(double)));
      own.push_back(*q);
    }
    for (int q = 0; q < h->nstage; ++q) {
      CK(cudaMalloc((void**)&lkc[q], n * sizeof(double)));
      own.push_back(lkc[q]);
      CK(cudaMalloc((void**)&lkr[q], n * sizeof(double)));
      own.push_back(lkr[q]);
    }
    return kOk;
  }
  ~CoupledWork() {
    for (double* q : own) cudaFree(q);
  }
};

// kr[is], kc[is]: the step's increments of Rho and of the component (exchanged)
int step_adj_coupled(asam_ctx* h, AdjWork& w, CoupledWork& cw, const std::vector<double*>& stage_states, int comp,
                     const double* const* kr, const double* const* kc, const double* lr_in, const double* lc_in,
                     double* lr_out, double* lc_out, double dt, double tol, double* gu, double* gv, double* gw) {
  const Launch& L = h->L;
  const Dims& d = h->d;
  const size_t n = h->npad;
  const int ns = h->nstage;
  const int rp = h->cfg.rho_pos;
  const double bdt = h->beta0 * dt;
  const int gn = grid_of(L, n);
  const size_t nint = (size_t)d.nx * d.ny * d.nz;
  CK(cudaMemcpyAsync(cw.accc, lc_in, n * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));
  CK(cudaMemcpyAsync(cw.accr, lr_in, n * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));
  k_zero_halo1<<<gn, kB, 0, L.stream>>>(d, cw.accc);
  k_zero_halo1<<<gn, kB, 0, L.stream>>>(d, cw.accr);
  count_launches(2);
  for (int j = 0; j < ns; ++j) {
    CK(cudaMemsetAsync(cw.lkc[j], 0, n * sizeof(double), L.stream));
    CK(cudaMemsetAsync(cw.lkr[j], 0, n * sizeof(double), L.stream));
    axpby(h, h->alpha[(ns - 1) * 4 + j], cw.accc, 1.0, cw.lkc[j]);
    axpby(h, h->alpha[(ns - 1) * 4 + j], cw.accr, 1.0, cw.lkr[j]);
  }
  CK(cudaMemsetAsync(cw.grho, 0, n * sizeof(double), L.stream));
  const double* rho0 = stage_states[0] + (size_t)rp * n;
  for (int is = ns - 1; is >= 0; --is) {
    // stage solve A k = b: lb = A_per^-T lk for both components
    int rc = bicgstab_T(h, w, cw.lbc, cw.lkc[is], 400, tol, nullptr);
    if (rc != kOk && rc != kNotConverged) return rc;
    rc = bicgstab_T(h, w, cw.lbr, cw.lkr[is], 400, tol, nullptr);
    if (rc != kOk && rc != kNotConverged) return rc;
    k_zero_halo1<<<gn, kB, 0, L.stream>>>(d, cw.lbc);
    k_zero_halo1<<<gn, kB, 0, L.stream>>>(d, cw.lbr);
    count_launches(2);
    // the stage matrix's dependence on the wind and on Rho_0: lb of (Rho, comp)
    // against the increments k_is of (Rho, comp)
    k_jac_adj<<<gn, kB, 0, L.stream>>>(d, h->geom(), rho0, bdt, 1, 0, cw.lbr, kr[is], gu, gv, gw, cw.grho);
    k_jac_adj<<<gn, kB, 0, L.stream>>>(d, h->geom(), rho0, bdt, 1, 0, cw.lbc, kc[is], gu, gv, gw, cw.grho);
    count_launches(2);
    for (int js = 0; js < is; ++js) {
      axpby(h, h->beta[is * 4 + js], cw.lbc, 1.0, cw.lkc[js]);
      axpby(h, h->beta[is * 4 + js], cw.lbr, 1.0, cw.lkr[js]);
    }
    // flux RHS b = dt R F(E y): forward face fluxes at the stage state
    if ((rc = fcn_dev(h, stage_states[is], h->rhs))) return rc;
    const double* rho_s = stage_states[is] + (size_t)rp * n;
    // component: lc = F_c'^T lb (w.gx/gy/gz: face adjoints), wind and density parts
    flux_dcoef(h, w, stage_states[is], comp);
    flux_adj(h, w, rho_s, cw.lbc, cw.luc);
    k_wind_flux_T<<<grid_of(L, d.n_uf()), kB, 0, L.stream>>>(d.n_uf(), h->uf, w.gx, h->gx + (size_t)comp * d.n_uf(),
                                                             dt, gu);
    k_wind_flux_T<<<grid_of(L, d.n_vf()), kB, 0, L.stream>>>(d.n_vf(), h->vf, w.gy, h->gy + (size_t)comp * d.n_vf(),
                                                             dt, gv);
    k_wind_flux_T<<<grid_of(L, d.n_wf()), kB, 0, L.stream>>>(d.n_wf(), h->wf, w.gz, h->gz + (size_t)comp * d.n_wf(),
                                                             dt, gw);
    k_rho_from_phi<<<gn, kB, 0, L.stream>>>(n, w.phi, cw.luc, cw.lur);
    count_launches(4);
    // Rho: its flux depends on the wind only
    k_gather_T<0><<<grid_of(L, d.n_uf()), kB, 0, L.stream>>>(d, h->geom(), h->rvol, cw.lbr, w.gx);
    k_gather_T<1><<<grid_of(L, d.n_vf()), kB, 0, L.stream>>>(d, h->geom(), h->rvol, cw.lbr, w.gy);
    k_gather_T<2><<<grid_of(L, d.n_wf()), kB, 0, L.stream>>>(d, h->geom(), h->rvol, cw.lbr, w.gz);
    k_wind_flux_T<<<grid_of(L, d.n_uf()), kB, 0, L.stream>>>(d.n_uf(), h->uf, w.gx, h->gx + (size_t)rp * d.n_uf(),
                                                             dt, gu);
    k_wind_flux_T<<<grid_of(L, d.n_vf()), kB, 0, L.stream>>>(d.n_vf(), h->vf, w.gy, h->gy + (size_t)rp * d.n_vf(),
                                                             dt, gv);
    k_wind_flux_T<<<grid_of(L, d.n_wf()), kB, 0, L.stream>>>(d.n_wf(), h->wf, w.gz, h->gz + (size_t)rp * d.n_wf(),
                                                             dt, gw);
    count_launches(6);
    // stage state y = u0 + sum alpha k: lu = dt E^T Z (lc, lr)
    double* lus[2] = {cw.luc, cw.lur};
    const int lcomp[2] = {comp, rp};
    for (int q = 0; q < 2; ++q) {
      state_halo_T(h, lcomp[q], lus[q]);
      k_zero_halo1<<<gn, kB, 0, L.stream>>>(d, lus[q]);
      count_launches(1);
    }
    axpby(h, dt, cw.luc, 1.0, cw.accc);
    axpby(h, dt, cw.lur, 1.0, cw.accr);
    for (int js = 0; js < is; ++js) {
      axpby(h, dt * h->alpha[(is - 1) * 4 + js], cw.luc, 1.0, cw.lkc[js]);
      axpby(h, dt * h->alpha[(is - 1) * 4 + js], cw.lur, 1.0, cw.lkr[js]);
    }
  }
  // Rho_0 of the stage matrix is the exchanged start state: E^T, then add
  state_halo_T(h, rp, cw.grho);
  k_zero_halo1<<<gn, kB, 0, L.stream>>>(d, cw.grho);
  count_launches(1);
  axpby(h, 1.0, cw.grho, 1.0, cw.accr);
  CK(cudaMemcpyAsync(lc_out, cw.accc, n * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));
  CK(cudaMemcpyAsync(lr_out, cw.accr, n * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));
  return check_launch();
}

struct AdjScratch {
  AdjWork w;
  std::vector<double*> stage;  // nstage+1 full states
  std::vector<double*> k;      // nstage single fields
  int alloc(asam_ctx* h) {
    int rc = adj_alloc(h, w);
    if (rc) return rc;
    stage.assign(h->nstage + 1, nullptr);
    k.assign(h->nstage, nullptr);
    for (auto& p : stage) CK(cudaMalloc((void**)&p, h->len * sizeof(double)));
    for (auto& p : k) CK(cudaMalloc((void**)&p, h->npad * sizeof(double)));
    return kOk;
  }
  ~AdjScratch() {
    adj_free(w);
    for (auto p : stage)
      if (p) cudaFree(p);
    for (auto p : k)
      if (p) cudaFree(p);
  }
};

int dev_copy_in(asam_ctx* h, const double* src, size_t n, double** dst, std::vector<double*>& owned) {
  if (is_device_ptr(src)) {
    *dst = const_cast<double*>(src);
    return kOk;
  }
  double* p;
  CK(cudaMalloc((void**)&p, n * sizeof(double)));
  owned.push_back(p);
  CK(cudaMemcpyAsync(p, src, n * sizeof(double), cudaMemcpyHostToDevice, h->L.stream));
  *dst = p;
  return kOk;
}

struct Owned {
  std::vector<double*> p;
  ~Owned() {
    for (auto q : p) cudaFree(q);
  }
};

int dev_out(asam_ctx* h, double* user, size_t n, double** dst, Owned& o) {
  if (is_device_ptr(user)) {
    *dst = user;
    return kOk;
  }
  double* p;
  CK(cudaMalloc((void**)&p, n * sizeof(double)));
  o.p.push_back(p);
  *dst = p;
  return kOk;
}
int dev_out_finish(asam_ctx* h, double* user, size_t n, double* dev) {
  if (dev != user) {
    CK(cudaMemcpyAsync(user, dev, n * sizeof(double), cudaMemcpyDeviceToHost, h->L.stream));
  }
  CK(cudaStreamSynchronize(h->L.stream));
  return kOk;
}

// the tangent-linear and adjoint flux cover the advection with closed walls; a
// context with diffusion (asam_set_diffusion) or with open-boundary wall
// rules is refused rather than differentiated wrongly
bool valid_comp(asam_ctx* h, int comp) {
  if (h->dkx) {
    set_last_error("the adjoint covers the advection flux; switch diffusion off first", __FILE__, __LINE__);
    return false;
  }
  if (h->bc_open()) {
    set_last_error("the adjoint covers the ZeroGrad and ZeroValue wall rules only", __FILE__, __LINE__);
    return false;
  }
  return comp >= 0 && comp < h->cfg.ncomp && comp != h->cfg.rho_pos;
}

}  // namespace

// ---------------------------------------------------------------------------
extern "C" {

int asam_fcn_tlm(asam_ctx* h, const double* c, int comp, const double* dc, double* df) {
  if (!h || !c || !dc || !df || !valid_comp(h, comp)) return kBadArg;
  Owned o;
  double *dcs, *dd, *out;
  int rc;
  if ((rc = dev_copy_in(h, c, h->len, &dcs, o.p)) || (rc = dev_copy_in(h, dc, h->npad, &dd, o.p)) ||
      (rc = dev_out(h, df, h->npad, &out, o)))
    return rc;
  AdjWork w;
  if ((rc = adj_alloc(h, w))) return rc;
  flux_dcoef(h, w, dcs, comp);
  flux_tlm(h, w, dcs + (size_t)h->cfg.rho_pos * h->npad, dd, out);
  rc = check_launch();
  if (!rc) rc = dev_out_finish(h, df, h->npad, out);
  adj_free(w);
  return rc;
}

int asam_fcn_adj(asam_ctx* h, const double* c, int comp, const double* lf, double* lc) {
  if (!h || !c || !lf || !lc || !valid_comp(h, comp)) return kBadArg;
  Owned o;
  double *dcs, *dl, *out;
  int rc;
  if ((rc = dev_copy_in(h, c, h->len, &dcs, o.p)) || (rc = dev_copy_in(h, lf, h->npad, &dl, o.p)) ||
      (rc = dev_out(h, lc, h->npad, &out, o)))
    return rc;
  AdjWork w;
  if ((rc = adj_alloc(h, w))) return rc;
  flux_dcoef(h, w, dcs, comp);
  flux_adj(h, w, dcs + (size_t)h->cfg.rho_pos * h->npad, dl, out);
  rc = check_launch();
  if (!rc) rc = dev_out_finish(h, lc, h->npad, out);
  adj_free(w);
  return rc;
}

int asam_matvec_adj(asam_ctx* h, const double* x, double* y) {
  if (!h || !x || !y) return kBadArg;
  Owned o;
  double *dx, *dy;
  int rc;
  if ((rc = dev_copy_in(h, x, h->npad, &dx, o.p)) || (rc = dev_out(h, y, h->npad, &dy, o))) return rc;
  k_matvec_T<<<grid_of(h->L, h->npad), kB, 0, h->L.stream>>>(h->d, h->val, dx, dy);
  count_launches(1);
  rc = check_launch();
  if (!rc) rc = dev_out_finish(h, y, h->npad, dy);
  return rc;
}

int asam_bicgstab_adj(asam_ctx* h, double* x, const double* b, int* maxiter, double* tol) {
  if (!h || !x || !b || !maxiter || !tol || *maxiter < 1) return kBadArg;
  Owned o;
  double *db, *dx;
  int rc;
  if ((rc = dev_copy_in(h, b, h->npad, &db, o.p)) || (rc = dev_out(h, x, h->npad, &dx, o))) return rc;
  AdjWork w;
  if ((rc = adj_alloc(h, w))) return rc;
  int it = 0;
  int st = bicgstab_T(h, w, dx, db, *maxiter, *tol, &it);
  *maxiter = it;
  adj_free(w);
  if (st != kOk && st != kNotConverged) return st;
  rc = dev_out_finish(h, x, h->npad, dx);
  return rc ? rc : st;
}

int asam_ros_step_tlm(asam_ctx* h, const double* c, int comp, const double* du, double* du_out, double dt,
                      double tol) {
  if (!h || !c || !du || !du_out || !valid_comp(h, comp)) return kBadArg;
  Owned o;
  double *dcs, *ddu, *out;
  int rc;
  if ((rc = dev_copy_in(h, c, h->len, &dcs, o.p)) || (rc = dev_copy_in(h, du, h->npad, &ddu, o.p)) ||
      (rc = dev_out(h, du_out, h->npad, &out, o)))
    return rc;
  AdjScratch sc;
  if ((rc = sc.alloc(h))) return rc;
  if ((rc = forward_record(h, dcs, dt, tol, sc.stage))) return rc;
  if ((rc = step_tlm(h, sc.w, sc.stage, comp, ddu, out, dt, tol, sc.k))) return rc;
  return dev_out_finish(h, du_out, h->npad, out);
}

int asam_ros_step_adj(asam_ctx* h, const double* c, int comp, const double* lam, double* lam_out, double dt,
                      double tol) {
  if (!h || !c || !lam || !lam_out || !valid_comp(h, comp)) return kBadArg;
  Owned o;
  double *dcs, *dl, *out;
  int rc;
  if ((rc = dev_copy_in(h, c, h->len, &dcs, o.p)) || (rc = dev_copy_in(h, lam, h->npad, &dl, o.p)) ||
      (rc = dev_out(h, lam_out, h->npad, &out, o)))
    return rc;
  AdjScratch sc;
  if ((rc = sc.alloc(h))) return rc;
  if ((rc = forward_record(h, dcs, dt, tol, sc.stage))) return rc;
  if ((rc = step_adj(h, sc.w, sc.stage, comp, dl, out, dt, tol, sc.k))) return rc;
  return dev_out_finish(h, lam_out, h->npad, out);
}

int asam_tracer_gradient(asam_ctx* h, const double* c0, int comp, int nsteps, double dt, int ckpt_every,
                         const int* box, double tol, double* J, double* grad) {
  if (!h || !c0 || !box || !J || !grad || !valid_comp(h, comp) || nsteps < 1 || ckpt_every < 1) return kBadArg;
  const Launch& L = h->L;
  const size_t len = h->len, n = h->npad;
  Owned o;
  double *dc0, *dgrad;
  int rc;
  if ((rc = dev_copy_in(h, c0, len, &dc0, o.p)) || (rc = dev_out(h, grad, n, &dgrad, o))) return rc;
  AdjScratch sc;
  if ((rc = sc.alloc(h))) return rc;
  // checkpoints every ckpt_every steps (nsteps/k states); in the reverse sweep
  // one segment of k steps is recomputed once from its checkpoint with the
  // stage states of every step recorded (k*nStage states, plus two for the
  // running state), so each step costs one forward recomputation, the rebuild
  // of its stage matrix and its adjoint
  const int nck = (nsteps + ckpt_every - 1) / ckpt_every;
  const int ns = h->nstage;
  std::vector<double*> ckpt(nck, nullptr), recbuf((size_t)ckpt_every * ns + 2, nullptr);
  struct Free {
    std::vector<double*>* a;
    ~Free() {
      for (auto p : *a)
        if (p) cudaFree(p);
    }
  };
  Free f1{&ckpt}, f2{&recbuf};
  for (auto& p : ckpt) CK(cudaMalloc((void**)&p, len * sizeof(double)));
  for (auto& p : recbuf) CK(cudaMalloc((void**)&p, len * sizeof(double)));
  // rec[m]: stage states of step s0+m, then the state after the step (one of
  // two alternating buffers)
  std::vector<std::vector<double*>> rec(ckpt_every, std::vector<double*>(ns + 1, nullptr));
  for (int m = 0; m < ckpt_every; ++m) {
    for (int is = 0; is < ns; ++is) rec[m][is] = recbuf[(size_t)m * ns + is];
    rec[m][ns] = recbuf[(size_t)ckpt_every * ns + (m & 1)];
  }
  struct TolGuard {
    asam_ctx* h;
    double saved;
    ~TolGuard() { h->cfg.bicgstab_tol = saved; }
  } tg{h, h->cfg.bicgstab_tol};
  h->cfg.bicgstab_tol = tol;  // the forward sweeps solve to the adjoint's tolerance
  double* cur = h->c;
  CK(cudaMemcpyAsync(cur, dc0, len * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));
  for (int s = 0; s < nsteps; ++s) {
    if (s % ckpt_every == 0)
      CK(cudaMemcpyAsync(ckpt[s / ckpt_every], cur, len * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));
    int it[4];
    double rs[4];
    rc = ros_step_dev(h, cur, dt, it, rs);
    if (rc != kOk && rc != kNotConverged) return rc;
  }
  // objective at the final state
  launch_exchange_cell(L, h->d, h->cfg.ncomp, cur);
  double* lam = sc.w.lam;
  k_objective<<<RED_GRID, RED_BLOCK, 0, L.stream>>>(h->d, cur + (size_t)comp * n, cur + (size_t)h->cfg.rho_pos * n,
                                                    h->volc, box[0], box[1], box[2], box[3], box[4], box[5], lam,
                                                    h->partial);
  k_sum_partials<<<1, RED_BLOCK, 0, L.stream>>>(h->partial, RED_GRID, h->red_out);
  count_launches(2);
  if ((rc = reduce_to_host(h, J))) return rc;
  // reverse sweep over segments
  double* lam_next = dgrad;
  for (int sgi = nck - 1; sgi >= 0; --sgi) {
    const int s0 = sgi * ckpt_every;
    const int s1 = std::min(nsteps, s0 + ckpt_every);
    const double* src = ckpt[sgi];
    for (int s = s0; s < s1; ++s) {
      if ((rc = forward_record(h, src, dt, tol, rec[s - s0]))) return rc;
      src = rec[s - s0][ns];
    }
    for (int s = s1 - 1; s >= s0; --s) {
      if ((rc = jac_dev(h, rec[s - s0][0], dt))) return rc;  // the step's stage matrix
      if ((rc = step_adj(h, sc.w, rec[s - s0], comp, lam, lam_next, dt, tol, sc.k))) return rc;
      CK(cudaMemcpyAsync(lam, lam_next, n * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));
    }
  }
  CK(cudaMemcpyAsync(dgrad, lam, n * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));
  rc = check_launch();
  if (rc) return rc;
  return dev_out_finish(h, grad, n, dgrad);
}

int asam_tracer_wind_gradient(asam_ctx* h, const double* c0, int comp, int nsteps, double dt, int ckpt_every,
                              const int* box, double tol, double* J, double* grad_c, double* grad_rho,
                              double* grad_uf, double* grad_vf, double* grad_wf) {
  if (!h || !c0 || !box || !J || !grad_c || !grad_rho || !grad_uf || !grad_vf || !grad_wf || !valid_comp(h, comp) ||
      nsteps < 1 || ckpt_every < 1)
    return kBadArg;
  const Launch& L = h->L;
  const Dims& d = h->d;
  const size_t len = h->len, n = h->npad;
  const int rp = h->cfg.rho_pos;
  Owned o;
  double *dc0, *dgc, *dgr, *dgu, *dgv, *dgw;
  int rc;
  if ((rc = dev_copy_in(h, c0, len, &dc0, o.p)) || (rc = dev_out(h, grad_c, n, &dgc, o)) ||
      (rc = dev_out(h, grad_rho, n, &dgr, o)) || (rc = dev_out(h, grad_uf, d.n_uf(), &dgu, o)) ||
      (rc = dev_out(h, grad_vf, d.n_vf(), &dgv, o)) || (rc = dev_out(h, grad_wf, d.n_wf(), &dgw, o)))
    return rc;
  AdjScratch sc;
  if ((rc = sc.alloc(h))) return rc;
  CoupledWork cw;
  if ((rc = cw.alloc(h))) return rc;
  const int nck = (nsteps + ckpt_every - 1) / ckpt_every;
  const int ns = h->nstage;
  std::vector<double*> ckpt(nck, nullptr), recbuf((size_t)ckpt_every * ns + 2, nullptr);
  double *lr = nullptr, *lr2 = nullptr, *lc2 = nullptr;
  struct Free {
    std::vector<double*>* a;
    ~Free() {
      for (auto p : *a)
        if (p) cudaFree(p);
    }
  };
  std::vector<double*> extra;
  // increments of Rho and of the component for every stage of every step of a
  // segment: [(m*ns + is)*2 + 0 | 1]
  std::vector<double*> incs((size_t)ckpt_every * ns * 2, nullptr);
  Free f1{&ckpt}, f2{&recbuf}, f3{&extra}, f4{&incs};
  for (auto& p : ckpt) CK(cudaMalloc((void**)&p, len * sizeof(double)));
  for (auto& p : recbuf) CK(cudaMalloc((void**)&p, len * sizeof(double)));
  for (auto& p : incs) CK(cudaMalloc((void**)&p, n * sizeof(double)));
  for (double** q : {&lr, &lr2, &lc2}) {
    CK(cudaMalloc((void**)q, n * sizeof(double)));
    extra.push_back(*q);
  }
  std::vector<std::vector<double*>> rec(ckpt_every, std::vector<double*>(ns + 1, nullptr));
  for (int m = 0; m < ckpt_every; ++m) {
    for (int is = 0; is < ns; ++is) rec[m][is] = recbuf[(size_t)m * ns + is];
    rec[m][ns] = recbuf[(size_t)ckpt_every * ns + (m & 1)];
  }
  struct TolGuard {
    asam_ctx* h;
    double saved;
    ~TolGuard() { h->cfg.bicgstab_tol = saved; }
  } tg{h, h->cfg.bicgstab_tol};
  h->cfg.bicgstab_tol = tol;
  double* cur = h->c;
  CK(cudaMemcpyAsync(cur, dc0, len * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));
  for (int s = 0; s < nsteps; ++s) {
    if (s % ckpt_every == 0)
      CK(cudaMemcpyAsync(ckpt[s / ckpt_every], cur, len * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));
    int it[4];
    double rs[4];
    rc = ros_step_dev(h, cur, dt, it, rs);
    if (rc != kOk && rc != kNotConverged) return rc;
  }
  launch_exchange_cell(L, d, h->cfg.ncomp, cur);
  double* lc = sc.w.lam;
  k_objective2<<<RED_GRID, RED_BLOCK, 0, L.stream>>>(d, cur + (size_t)comp * n, cur + (size_t)rp * n, h->volc, box[0],
                                                     box[1], box[2], box[3], box[4], box[5], lc, lr, h->partial);
  k_sum_partials<<<1, RED_BLOCK, 0, L.stream>>>(h->partial, RED_GRID, h->red_out);
  count_launches(2);
  if ((rc = reduce_to_host(h, J))) return rc;
  CK(cudaMemsetAsync(dgu, 0, d.n_uf() * sizeof(double), L.stream));
  CK(cudaMemsetAsync(dgv, 0, d.n_vf() * sizeof(double), L.stream));
  CK(cudaMemsetAsync(dgw, 0, d.n_wf() * sizeof(double), L.stream));
  for (int sgi = nck - 1; sgi >= 0; --sgi) {
    const int s0 = sgi * ckpt_every;
    const int s1 = std::min(nsteps, s0 + ckpt_every);
    const double* src = ckpt[sgi];
    for (int s = s0; s < s1; ++s) {
      const int m = s - s0;
      if ((rc = forward_record(h, src, dt, tol, rec[m]))) return rc;
      for (int is = 0; is < ns; ++is) {
        const double* k = h->incr + (size_t)is * len;
        CK(cudaMemcpyAsync(incs[((size_t)m * ns + is) * 2], k + (size_t)rp * n, n * sizeof(double),
                           cudaMemcpyDeviceToDevice, L.stream));
        CK(cudaMemcpyAsync(incs[((size_t)m * ns + is) * 2 + 1], k + (size_t)comp * n, n * sizeof(double),
                           cudaMemcpyDeviceToDevice, L.stream));
      }
      src = rec[m][ns];
    }
    for (int s = s1 - 1; s >= s0; --s) {
      const int m = s - s0;
      if ((rc = jac_dev(h, rec[m][0], dt))) return rc;  // the step's stage matrix
      double* kr[4];
      double* kc[4];
      for (int is = 0; is < ns; ++is) {
        kr[is] = incs[((size_t)m * ns + is) * 2];
        kc[is] = incs[((size_t)m * ns + is) * 2 + 1];
      }
      if ((rc = step_adj_coupled(h, sc.w, cw, rec[m], comp, kr, kc, lr, lc, lr2, lc2, dt, tol, dgu, dgv, dgw)))
        return rc;
      CK(cudaMemcpyAsync(lc, lc2, n * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));
      CK(cudaMemcpyAsync(lr, lr2, n * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));
    }
  }
  CK(cudaMemcpyAsync(dgc, lc, n * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));
  CK(cudaMemcpyAsync(dgr, lr, n * sizeof(double), cudaMemcpyDeviceToDevice, L.stream));
  if ((rc = check_launch())) return rc;
  if ((rc = dev_out_finish(h, grad_c, n, dgc)) || (rc = dev_out_finish(h, grad_rho, n, dgr)) ||
      (rc = dev_out_finish(h, grad_uf, d.n_uf(), dgu)) || (rc = dev_out_finish(h, grad_vf, d.n_vf(), dgv)))
    return rc;
  return dev_out_finish(h, grad_wf, d.n_wf(), dgw);
}

}  // extern "C"
