// Block-tridiagonal column solve of the density/buoyancy-coupled line
// preconditioner (MULTI/TriDiagTB_Mod.f90): Solve_1D (:143-163), a Thomas
// elimination with 2x2 blocks, and MatVecTB_1D (:121-141), over independent
// columns.  The 2x2 helpers are those of CG/Matrix_Mod.f90 (Mult_2, Mult_22,
// Div_2, Div_22), evaluated in their operation order without contraction, so
// the results are bit-identical to a scalar CPU evaluation.
//
// Layout at the boundary (the reference's per-column arrays back to back):
//   d[(col*n1 + i)*4 + r + 2*c]        = A%d(r+1,c+1,i+1)
//   u, l[(col*(n1-1) + i)*4 + r + 2*c] = A%u / A%l(r+1,c+1,i+1)
//   b, x, y[(col*n1 + i)*2 + r]        = b(r+1,i+1)
// One thread per column; the elimination factors w go to a scratch array
// laid out level-major ([i][e][col]) so that a warp's stores are coalesced.
#include <memory>

#include "context.h"

namespace {

struct M2 {
  double a11, a21, a12, a22;  // column-major like the Fortran 2x2 block
};
struct V2 {
  double x1, x2;
};

__device__ __forceinline__ M2 ld_m(const double* p) {
  const double2 a = *reinterpret_cast<const double2*>(p);
  const double2 b = *reinterpret_cast<const double2*>(p + 2);
  return M2{a.x, a.y, b.x, b.y};
}
__device__ __forceinline__ V2 ld_v(const double* p) {
  const double2 a = *reinterpret_cast<const double2*>(p);
  return V2{a.x, a.y};
}
__device__ __forceinline__ void st_v(double* p, V2 v) { *reinterpret_cast<double2*>(p) = make_double2(v.x1, v.x2); }

// Mult_2(b,c): temp(1)=b(1,1)*c(1)+b(1,2)*c(2); temp(2)=b(2,1)*c(1)+b(2,2)*c(2)
__device__ __forceinline__ V2 mult_2(const M2& b, const V2& c) {
  return V2{__dadd_rn(__dmul_rn(b.a11, c.x1), __dmul_rn(b.a12, c.x2)),
            __dadd_rn(__dmul_rn(b.a21, c.x1), __dmul_rn(b.a22, c.x2))};
}
// Mult_22(b,c): temp(r,s)=b(r,1)*c(1,s)+b(r,2)*c(2,s)
__device__ __forceinline__ M2 mult_22(const M2& b, const M2& c) {
  return M2{__dadd_rn(__dmul_rn(b.a11, c.a11), __dmul_rn(b.a12, c.a21)),
            __dadd_rn(__dmul_rn(b.a21, c.a11), __dmul_rn(b.a22, c.a21)),
            __dadd_rn(__dmul_rn(b.a11, c.a12), __dmul_rn(b.a12, c.a22)),
            __dadd_rn(__dmul_rn(b.a21, c.a12), __dmul_rn(b.a22, c.a22))};
}
__device__ __forceinline__ double det(const M2& c) {
  return __dsub_rn(__dmul_rn(c.a11, c.a22), __dmul_rn(c.a12, c.a21));
}
// Div_2(b,c): c^-1 b by the adjugate over Det
__device__ __forceinline__ V2 div_2(const V2& b, const M2& c) {
  const double dt = det(c);
  return V2{__ddiv_rn(__dsub_rn(__dmul_rn(c.a22, b.x1), __dmul_rn(c.a12, b.x2)), dt),
            __ddiv_rn(__dadd_rn(__dmul_rn(-c.a21, b.x1), __dmul_rn(c.a11, b.x2)), dt)};
}
// Div_22(b,c): c^-1 b column by column
__device__ __forceinline__ M2 div_22(const M2& b, const M2& c) {
  const double dt = det(c);
  return M2{__ddiv_rn(__dsub_rn(__dmul_rn(c.a22, b.a11), __dmul_rn(c.a12, b.a21)), dt),
            __ddiv_rn(__dadd_rn(__dmul_rn(-c.a21, b.a11), __dmul_rn(c.a11, b.a21)), dt),
            __ddiv_rn(__dsub_rn(__dmul_rn(c.a22, b.a12), __dmul_rn(c.a12, b.a22)), dt),
            __ddiv_rn(__dadd_rn(__dmul_rn(-c.a21, b.a12), __dmul_rn(c.a11, b.a22)), dt)};
}
__device__ __forceinline__ M2 sub_m(const M2& a, const M2& b) {
  return M2{__dsub_rn(a.a11, b.a11), __dsub_rn(a.a21, b.a21), __dsub_rn(a.a12, b.a12), __dsub_rn(a.a22, b.a22)};
}
__device__ __forceinline__ V2 sub_v(const V2& a, const V2& b) {
  return V2{__dsub_rn(a.x1, b.x1), __dsub_rn(a.x2, b.x2)};
}
__device__ __forceinline__ V2 add_v(const V2& a, const V2& b) {
  return V2{__dadd_rn(a.x1, b.x1), __dadd_rn(a.x2, b.x2)};
}

// Solve_1D of one column (dc, uc, lc, bc of that column); the factors w of
// level i at w[(i*4 + e)*ws] (ws the stride between the columns' slots)
__device__ void solve_col(int n1, const double* __restrict__ dc, const double* __restrict__ uc,
                          const double* __restrict__ lc, double* __restrict__ bc, double* __restrict__ w, size_t ws) {
  // the next row's inputs are loaded before this row's arithmetic, so their
  // latency overlaps the recurrence (the operations and their order are the
  // same as a row-by-row evaluation)
  M2 t = ld_m(dc);
  V2 bp = div_2(ld_v(bc), t);
  st_v(bc, bp);
  if (n1 > 1) {
    M2 ln = ld_m(lc), un = ld_m(uc), dn = ld_m(dc + 4);
    V2 bn = ld_v(bc + 2);
    for (int i = 1; i < n1; ++i) {
      const M2 li = ln, ui = un, di = dn;
      const V2 bi = bn;
      if (i + 1 < n1) {
        ln = ld_m(lc + (size_t)i * 4);
        un = ld_m(uc + (size_t)i * 4);
        dn = ld_m(dc + (size_t)(i + 1) * 4);
        bn = ld_v(bc + (size_t)(i + 1) * 2);
      }
      const M2 wi = div_22(ui, t);
      double* wp = w + (size_t)(i - 1) * 4 * ws;
      wp[0] = wi.a11;
      wp[ws] = wi.a21;
      wp[2 * ws] = wi.a12;
      wp[3 * ws] = wi.a22;
      t = sub_m(di, mult_22(li, wi));
      bp = div_2(sub_v(bi, mult_2(li, bp)), t);
      st_v(bc + (size_t)i * 2, bp);
    }
    const double* wp0 = w + (size_t)(n1 - 2) * 4 * ws;
    M2 wn{wp0[0], wp0[ws], wp0[2 * ws], wp0[3 * ws]};
    V2 cn = ld_v(bc + (size_t)(n1 - 2) * 2);
    for (int i = n1 - 2; i >= 0; --i) {
      const M2 wi = wn;
      const V2 ci = cn;
      if (i > 0) {
        const double* wp = w + (size_t)(i - 1) * 4 * ws;
        wn = M2{wp[0], wp[ws], wp[2 * ws], wp[3 * ws]};
        cn = ld_v(bc + (size_t)(i - 1) * 2);
      }
      bp = sub_v(ci, mult_2(wi, bp));
      st_v(bc + (size_t)i * 2, bp);
    }
  }
}

__global__ void k_tri_tb_solve(int ncol, int n1, const double* __restrict__ d, const double* __restrict__ u,
                               const double* __restrict__ l, double* __restrict__ b, double* __restrict__ w) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= ncol) return;
  solve_col(n1, d + (size_t)col * n1 * 4, u + (size_t)col * (n1 - 1) * 4, l + (size_t)col * (n1 - 1) * 4,
            b + (size_t)col * n1 * 2, w + col, (size_t)ncol);
}

// GaussSeidel_2D (MULTI/TriDiagTB_Mod.f90:374-418, TriDiagTR_Mod.f90:418-462), one
// thread per plane: the reference's symmetric line sweep, statement by
// statement; t and the Thomas factors in slots strided by the plane count.
__device__ __forceinline__ V2 couple_sub(int tr, const V2& t, const double* c, const V2& x) {
  if (tr) return sub_v(t, mult_2(ld_m(c), x));
  return V2{__dsub_rn(t.x1, __dmul_rn(c[0], x.x1)), __dsub_rn(t.x2, __dmul_rn(c[1], x.x1))};
}

__global__ void k_tri_tb_gs_2d(int tr, int nplane, int n2, int n1, const double* __restrict__ d,
                               const double* __restrict__ u1, const double* __restrict__ l1,
                               const double* __restrict__ u2, const double* __restrict__ l2,
                               const double* __restrict__ b, double* __restrict__ x, int iters,
                               double* __restrict__ tbuf, double* __restrict__ w) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nplane) return;
  const size_t L0 = (size_t)p * n2, ws = (size_t)nplane;
  double* wp = w + p;
  auto T = [&](int i) -> V2 { return V2{tbuf[((size_t)i * 2) * ws + p], tbuf[((size_t)i * 2 + 1) * ws + p]}; };
  auto setT = [&](int i, const V2& v) {
    tbuf[((size_t)i * 2) * ws + p] = v.x1;
    tbuf[((size_t)i * 2 + 1) * ws + p] = v.x2;
  };
  auto XL = [&](int j) { return x + (L0 + j) * n1 * 2; };
  auto BL = [&](int j) { return b + (L0 + j) * n1 * 2; };
  auto C2 = [&](const double* a, int i, int j) { return a + (((size_t)p * (n2 - 1) + j) * n1 + i) * 4; };
  auto solve = [&](int j) {
    solve_col(n1, d + (L0 + j) * n1 * 4, u1 + (L0 + j) * (n1 - 1) * 4, l1 + (L0 + j) * (n1 - 1) * 4, XL(j), wp, ws);
  };
  if (n2 > 1) {
    for (int it = 0; it < iters; ++it) {
      for (int i = 0; i < n1; ++i) setT(i, ld_v(BL(0) + 2 * i));
      for (int j = 0; j < n2 - 1; ++j) {
        for (int i = 0; i < n1; ++i) st_v(XL(j) + 2 * i, couple_sub(tr, T(i), C2(u2, i, j), ld_v(XL(j + 1) + 2 * i)));
        solve(j);
        for (int i = 0; i < n1; ++i) setT(i, couple_sub(tr, ld_v(BL(j + 1) + 2 * i), C2(l2, i, j), ld_v(XL(j) + 2 * i)));
      }
      for (int i = 0; i < n1; ++i) st_v(XL(n2 - 1) + 2 * i, T(i));
      solve(n2 - 1);
      for (int i = 0; i < n1; ++i)
        setT(i, couple_sub(tr, ld_v(BL(n2 - 2) + 2 * i), C2(u2, i, n2 - 2), ld_v(XL(n2 - 1) + 2 * i)));
      for (int j = n2 - 2; j >= 1; --j) {
        for (int i = 0; i < n1; ++i)
          st_v(XL(j) + 2 * i, couple_sub(tr, T(i), C2(l2, i, j - 1), ld_v(XL(j - 1) + 2 * i)));
        solve(j);
        for (int i = 0; i < n1; ++i)
          setT(i, couple_sub(tr, ld_v(BL(j - 1) + 2 * i), C2(u2, i, j - 1), ld_v(XL(j) + 2 * i)));
      }
    }
    for (int i = 0; i < n1; ++i) st_v(XL(0) + 2 * i, T(i));
    solve(0);
  } else {
    for (int i = 0; i < n1; ++i) st_v(XL(0) + 2 * i, ld_v(BL(0) + 2 * i));
    solve(0);
  }
}

// RestrictTB_2D (TriDiagTB_Mod.f90:495-525) per coarse entry: the value the
// reference's overwriting loops leave there
__device__ __forceinline__ void restrict_2d_entry(int n2, int n1, const double* __restrict__ res,
                                                  double* __restrict__ resc, size_t e) {
  const int n1c = (n1 + 1) / 2, n2c = (n2 + 1) / 2;
  const int ic = (int)(e % n1c);
  const int jc = (int)((e / n1c) % n2c);
  const size_t p = e / ((size_t)n1c * n2c);
  const double* R = res + p * n2 * n1 * 2;
  auto rf = [&](int i, int j) { return ld_v(R + ((size_t)j * n1 + i) * 2); };
  V2 v;
  if (jc < n2 / 2) {
    const int jf = 2 * jc;
    if (ic < n1 / 2) {
      const int i = 2 * ic;
      v = add_v(add_v(add_v(rf(i, jf), rf(i + 1, jf)), rf(i, jf + 1)), rf(i + 1, jf + 1));
    } else {
      v = add_v(rf(n1 - 1, jf), rf(n1 - 1, jf + 1));
    }
  } else {
    v = ic < n1 / 2 ? add_v(rf(2 * ic, n2 - 1), rf(2 * ic + 1, n2 - 1)) : rf(n1 - 1, n2 - 1);
  }
  st_v(resc + e * 2, v);
}

__global__ void k_tri_tb_restrict_2d(int nplane, int n2, int n1, const double* __restrict__ res,
                                     double* __restrict__ resc) {
  const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= (size_t)nplane * ((n2 + 1) / 2) * ((n1 + 1) / 2)) return;
  restrict_2d_entry(n2, n1, res, resc, e);
}

// ProlongateTB_2D (TriDiagTB_Mod.f90:527-560): each fine entry its coarse cell's value
__global__ void k_tri_tb_prolong_2d(int nplane, int n2, int n1, const double* __restrict__ xc,
                                    double* __restrict__ x) {
  const int n1c = (n1 + 1) / 2, n2c = (n2 + 1) / 2;
  const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= (size_t)nplane * n2 * n1) return;
  const int i = (int)(e % n1);
  const int j = (int)((e / n1) % n2);
  const size_t p = e / ((size_t)n1 * n2);
  st_v(x + e * 2, ld_v(xc + ((p * n2c + j / 2) * n1c + i / 2) * 2));
}

__global__ void k_tri_tb_matvec(int ncol, int n1, const double* __restrict__ d, const double* __restrict__ u,
                                const double* __restrict__ l, const double* __restrict__ x, double* __restrict__ y) {
  const size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (q >= (size_t)ncol * n1) return;
  const size_t col = q / n1;
  const int i = (int)(q % n1);
  const double* xc = x + col * n1 * 2;
  const M2 di = ld_m(d + q * 4);
  V2 r;
  if (n1 == 1) {
    r = mult_2(di, ld_v(xc));
  } else if (i == 0) {
    r = add_v(mult_2(di, ld_v(xc)), mult_2(ld_m(u + col * (n1 - 1) * 4), ld_v(xc + 2)));
  } else if (i == n1 - 1) {
    r = add_v(mult_2(ld_m(l + (col * (n1 - 1) + i - 1) * 4), ld_v(xc + (size_t)(i - 1) * 2)),
              mult_2(di, ld_v(xc + (size_t)i * 2)));
  } else {
    r = add_v(add_v(mult_2(ld_m(l + (col * (n1 - 1) + i - 1) * 4), ld_v(xc + (size_t)(i - 1) * 2)),
                    mult_2(di, ld_v(xc + (size_t)i * 2))),
              mult_2(ld_m(u + (col * (n1 - 1) + i) * 4), ld_v(xc + (size_t)(i + 1) * 2)));
  }
  st_v(y + q * 2, r);
}

// Compute_1D (Allocate_1D, then MULTI/TriDiagTB_Mod.f90:32-93; with tr the
// DUR terms of MULTI/TriDiagTR_Mod.f90:32-105) of one column, statement by
// statement in the reference's order (the GradFull branches are the same
// statements).  s = {beta0*dtp, Fac1_L, Fac1_R, GravComp, FacAnela}.
__global__ void k_tri_tb_compute(int tr, int ncol, int n1, asam_tri_tb_coefs s, const double* __restrict__ f,
                                 const double* __restrict__ fg, const double* __restrict__ vol,
                                 const double* __restrict__ dtu, const double* __restrict__ duu,
                                 const double* __restrict__ dut, const double* __restrict__ dur,
                                 double* __restrict__ d, double* __restrict__ u, double* __restrict__ l) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= ncol) return;
  const double bd = s.beta0_dtp, fl = s.fac1_l, fr = s.fac1_r, grav = s.grav_comp, anela = s.fac_anela;
  const double bd2 = bd * bd, half = 0.5, eps = 1.0e-30;
  const double *F = f + (size_t)col * (n1 + 1), *FG = fg + (size_t)col * (n1 + 1);
  const double *DTU = dtu + (size_t)col * (n1 + 1), *DUU = duu + (size_t)col * (n1 + 1);
  const double *V = vol + (size_t)col * n1, *DUT = dut + (size_t)col * n1;
  const double* DUR = tr ? dur + (size_t)col * n1 : nullptr;
  double* D = d + (size_t)col * n1 * 4;
  double *U = u + (size_t)col * (n1 - 1) * 4, *L = l + (size_t)col * (n1 - 1) * 4;
  auto DD = [&](int r, int c, int i) -> double& { return D[(size_t)i * 4 + r + 2 * c]; };
  auto UU = [&](int r, int c, int i) -> double& { return U[(size_t)i * 4 + r + 2 * c]; };
  auto LL = [&](int r, int c, int i) -> double& { return L[(size_t)i * 4 + r + 2 * c]; };
  for (int i = 0; i < n1; ++i) {
    DD(0, 0, i) = 1.0e-40;
    DD(1, 0, i) = 0.0;
    DD(0, 1, i) = 0.0;
    DD(1, 1, i) = 1.0e-40;
  }
  for (int i = 0; i < n1 - 1; ++i)
    for (int e = 0; e < 4; ++e) U[(size_t)i * 4 + e] = L[(size_t)i * 4 + e] = 0.0;
  DD(0, 0, 0) = DD(0, 0, 0) + bd2 * fl * F[0] * DTU[0] * DUU[0] * FG[0] * DUT[0] / (V[0] + eps);
  if (tr) DD(0, 1, 0) = DD(0, 1, 0) + bd2 * fl * F[0] * DTU[0] * DUU[0] * FG[0] * DUR[0] / (V[0] + eps);
  DD(1, 0, 0) = DD(1, 0, 0) + bd2 * fl * F[0] * DUU[0] * FG[0] * DUT[0] / (V[0] + eps);
  if (tr) DD(1, 1, 0) = DD(1, 1, 0) + bd2 * fl * F[0] * DUU[0] * FG[0] * DUR[0] / (V[0] + eps);
  DD(0, 1, 0) = DD(0, 1, 0) - half * grav * bd2 * fl * F[0] * DTU[0] * V[0] / (V[0] + eps);
  DD(1, 1, 0) = DD(1, 1, 0) - half * grav * bd2 * fl * F[0] * V[0] / (V[0] + eps);
  for (int i = 0; i < n1 - 1; ++i) {
    const int q = i + 1;
    const double S = V[i] + V[q] + eps;
    UU(0, 0, i) = -(bd2 * 2.0 * F[q] * DTU[q] * DUU[q] * FG[q] * DUT[q] / S);
    if (tr) UU(0, 1, i) = -(bd2 * 2.0 * F[q] * DTU[q] * DUU[q] * FG[q] * DUR[q] / S);
    UU(1, 0, i) = -(bd2 * 2.0 * F[q] * DUU[q] * FG[q] * DUT[q] / S);
    if (tr) UU(1, 1, i) = -(bd2 * 2.0 * F[q] * DUU[q] * FG[q] * DUR[q] / S);
    LL(0, 0, i) = -(bd2 * 2.0 * F[q] * DTU[q] * DUU[q] * FG[q] * DUT[i] / S);
    if (tr) LL(0, 1, i) = -(bd2 * 2.0 * F[q] * DTU[q] * DUU[q] * FG[q] * DUR[i] / S);
    LL(1, 0, i) = -(bd2 * 2.0 * F[q] * DUU[q] * FG[q] * DUT[i] / S);
    if (tr) LL(1, 1, i) = -(bd2 * 2.0 * F[q] * DUU[q] * FG[q] * DUR[i] / S);
    UU(0, 1, i) = UU(0, 1, i) - grav * bd2 * F[q] * DTU[q] * V[q] / S;
    UU(1, 1, i) = UU(1, 1, i) - grav * bd2 * F[q] * V[q] / S;
    LL(0, 1, i) = LL(0, 1, i) + grav * bd2 * F[q] * DTU[q] * V[i] / S;
    LL(1, 1, i) = LL(1, 1, i) + grav * bd2 * F[q] * V[i] / S;
    DD(0, 0, i) = DD(0, 0, i) + bd2 * 2.0 * F[q] * DTU[q] * DUU[q] * FG[q] * DUT[i] / S;
    if (tr) DD(0, 1, i) = DD(0, 1, i) + bd2 * 2.0 * F[q] * DTU[q] * DUU[q] * FG[q] * DUR[i] / S;
    DD(1, 0, i) = DD(1, 0, i) + bd2 * 2.0 * F[q] * DUU[q] * FG[q] * DUT[i] / S;
    if (tr) DD(1, 1, i) = DD(1, 1, i) + bd2 * 2.0 * F[q] * DUU[q] * FG[q] * DUR[i] / S;
    DD(0, 0, q) = DD(0, 0, q) + bd2 * 2.0 * F[q] * DTU[q] * DUU[q] * FG[q] * DUT[q] / S;
    if (tr) DD(0, 1, q) = DD(0, 1, q) + bd2 * 2.0 * F[q] * DTU[q] * DUU[q] * FG[q] * DUR[q] / S;
    DD(1, 0, q) = DD(1, 0, q) + bd2 * 2.0 * F[q] * DUU[q] * FG[q] * DUT[q] / S;
    if (tr) DD(1, 1, q) = DD(1, 1, q) + bd2 * 2.0 * F[q] * DUU[q] * FG[q] * DUR[q] / S;
    DD(0, 1, i) = DD(0, 1, i) - grav * bd2 * F[q] * DTU[q] * V[i] / S;
    DD(1, 1, i) = DD(1, 1, i) - grav * bd2 * F[q] * V[i] / S;
    DD(0, 1, q) = DD(0, 1, q) + grav * bd2 * F[q] * DTU[q] * V[q] / S;
    DD(1, 1, q) = DD(1, 1, q) + grav * bd2 * F[q] * V[q] / S;
  }
  {
    const int c = n1 - 1, q = n1;
    DD(0, 0, c) = DD(0, 0, c) + bd2 * fr * F[q] * DTU[q] * DUU[q] * FG[q] * DUT[c] / (V[c] + eps);
    if (tr) DD(0, 1, c) = DD(0, 1, c) + bd2 * fr * F[q] * DTU[q] * DUU[q] * FG[q] * DUR[c] / (V[c] + eps);
    DD(1, 0, c) = DD(1, 0, c) + bd2 * fr * F[q] * DUU[q] * FG[q] * DUT[c] / (V[c] + eps);
    if (tr) DD(1, 1, c) = DD(1, 1, c) + bd2 * fr * F[q] * DUU[q] * FG[q] * DUR[c] / (V[c] + eps);
    DD(0, 1, c) = DD(0, 1, c) + half * grav * bd2 * fr * F[q] * DTU[q] * V[c] / (V[c] + eps);
    DD(1, 1, c) = DD(1, 1, c) + half * grav * bd2 * fr * F[q] * V[c] / (V[c] + eps);
  }
  for (int i = 0; i < n1; ++i) {
    DD(0, 0, i) = DD(0, 0, i) + anela * V[i];
    DD(1, 1, i) = DD(1, 1, i) + V[i];
  }
}

// Compute_2D (MULTI/TriDiagTB_Mod.f90:260-343; TriDiagTR_Mod.f90:273-387) over
// planes, one thread per element (plane p, line j, level i).  Every entry is
// a sum whose terms the reference adds in a fixed order: its line's
// Compute_1D (the first z face, the face below as the upper cell, the face
// above as the lower cell, the last z face, FacAnela/Vol), then the faces
// between lines (Fac2_L on line 1, the face to the line before, the face to
// the line after, Fac2_R on the last line).  The thread adds them in that
// order, so the entries equal the reference's line-by-line sweep bit for bit
// while all elements are assembled at once.
struct Plane2D {  // the inputs and couplings of the plane systems (layouts of asam_tri_tb_compute_2d)
  const double *f1, *f1g, *dtu1, *duu1, *f2, *f2g, *dtu2, *duu2, *vol, *dut, *dur;
  double *u1, *l1, *u2, *l2;
};

// entry e = (p*n2 + j)*n1 + i of plane p: its block (out[4]) and, for i < n1-1
// and j < n2-1, the couplings to the next level and to the next line
__device__ void element_2d(int tr, int n2, int n1, const asam_tri_tb_coefs& s, const Plane2D& P, size_t e,
                           double* out) {
  const double *f1 = P.f1, *f1g = P.f1g, *dtu1 = P.dtu1, *duu1 = P.duu1, *f2 = P.f2, *f2g = P.f2g;
  const double *dtu2 = P.dtu2, *duu2 = P.duu2, *vol = P.vol, *dut = P.dut, *dur = P.dur;
  double *u1 = P.u1, *l1 = P.l1, *u2 = P.u2, *l2 = P.l2;
  const int i = (int)(e % n1);
  const size_t line = e / n1;  // p*n2 + j
  const int j = (int)(line % n2);
  const size_t p = line / n2;
  const double bd = s.beta0_dtp, fl = s.fac1_l, fr = s.fac1_r, grav = s.grav_comp, anela = s.fac_anela;
  const double bd2 = bd * bd, half = 0.5, eps = 1.0e-30;
  // this line's z faces and cells
  const double *F = f1 + line * (n1 + 1), *FG = f1g + line * (n1 + 1);
  const double *DTU = dtu1 + line * (n1 + 1), *DUU = duu1 + line * (n1 + 1);
  const double *V = vol + line * n1, *DUT = dut + line * n1;
  const double* DUR = tr ? dur + line * n1 : nullptr;
  // ---- Compute_1D of the line: entry i
  double e0 = 1.0e-40, e1 = 0.0, e2 = 0.0, e3 = 1.0e-40;
  if (i == 0) {
    e0 = e0 + bd2 * fl * F[0] * DTU[0] * DUU[0] * FG[0] * DUT[0] / (V[0] + eps);
    if (tr) e2 = e2 + bd2 * fl * F[0] * DTU[0] * DUU[0] * FG[0] * DUR[0] / (V[0] + eps);
    e1 = e1 + bd2 * fl * F[0] * DUU[0] * FG[0] * DUT[0] / (V[0] + eps);
    if (tr) e3 = e3 + bd2 * fl * F[0] * DUU[0] * FG[0] * DUR[0] / (V[0] + eps);
    e2 = e2 - half * grav * bd2 * fl * F[0] * DTU[0] * V[0] / (V[0] + eps);
    e3 = e3 - half * grav * bd2 * fl * F[0] * V[0] / (V[0] + eps);
  }
  if (i > 0) {  // face i, entry i as its upper cell
    const int q = i, c = i - 1;
    const double S = V[c] + V[q] + eps;
    e0 = e0 + bd2 * 2.0 * F[q] * DTU[q] * DUU[q] * FG[q] * DUT[q] / S;
    if (tr) e2 = e2 + bd2 * 2.0 * F[q] * DTU[q] * DUU[q] * FG[q] * DUR[q] / S;
    e1 = e1 + bd2 * 2.0 * F[q] * DUU[q] * FG[q] * DUT[q] / S;
    if (tr) e3 = e3 + bd2 * 2.0 * F[q] * DUU[q] * FG[q] * DUR[q] / S;
    e2 = e2 + grav * bd2 * F[q] * DTU[q] * V[q] / S;
    e3 = e3 + grav * bd2 * F[q] * V[q] / S;
  }
  if (i < n1 - 1) {  // face i+1, entry i as its lower cell; the couplings of that face
    const int q = i + 1;
    const double S = V[i] + V[q] + eps;
    double* U = u1 + (line * (n1 - 1) + i) * 4;
    double* L = l1 + (line * (n1 - 1) + i) * 4;
    U[0] = -(bd2 * 2.0 * F[q] * DTU[q] * DUU[q] * FG[q] * DUT[q] / S);
    double u12 = tr ? -(bd2 * 2.0 * F[q] * DTU[q] * DUU[q] * FG[q] * DUR[q] / S) : 0.0;
    U[1] = -(bd2 * 2.0 * F[q] * DUU[q] * FG[q] * DUT[q] / S);
    double u22 = tr ? -(bd2 * 2.0 * F[q] * DUU[q] * FG[q] * DUR[q] / S) : 0.0;
    L[0] = -(bd2 * 2.0 * F[q] * DTU[q] * DUU[q] * FG[q] * DUT[i] / S);
    double l12 = tr ? -(bd2 * 2.0 * F[q] * DTU[q] * DUU[q] * FG[q] * DUR[i] / S) : 0.0;
    L[1] = -(bd2 * 2.0 * F[q] * DUU[q] * FG[q] * DUT[i] / S);
    double l22 = tr ? -(bd2 * 2.0 * F[q] * DUU[q] * FG[q] * DUR[i] / S) : 0.0;
    U[2] = u12 - grav * bd2 * F[q] * DTU[q] * V[q] / S;
    U[3] = u22 - grav * bd2 * F[q] * V[q] / S;
    L[2] = l12 + grav * bd2 * F[q] * DTU[q] * V[i] / S;
    L[3] = l22 + grav * bd2 * F[q] * V[i] / S;
    e0 = e0 + bd2 * 2.0 * F[q] * DTU[q] * DUU[q] * FG[q] * DUT[i] / S;
    if (tr) e2 = e2 + bd2 * 2.0 * F[q] * DTU[q] * DUU[q] * FG[q] * DUR[i] / S;
    e1 = e1 + bd2 * 2.0 * F[q] * DUU[q] * FG[q] * DUT[i] / S;
    if (tr) e3 = e3 + bd2 * 2.0 * F[q] * DUU[q] * FG[q] * DUR[i] / S;
    e2 = e2 - grav * bd2 * F[q] * DTU[q] * V[i] / S;
    e3 = e3 - grav * bd2 * F[q] * V[i] / S;
  }
  if (i == n1 - 1) {
    const int c = i, q = n1;
    e0 = e0 + bd2 * fr * F[q] * DTU[q] * DUU[q] * FG[q] * DUT[c] / (V[c] + eps);
    if (tr) e2 = e2 + bd2 * fr * F[q] * DTU[q] * DUU[q] * FG[q] * DUR[c] / (V[c] + eps);
    e1 = e1 + bd2 * fr * F[q] * DUU[q] * FG[q] * DUT[c] / (V[c] + eps);
    if (tr) e3 = e3 + bd2 * fr * F[q] * DUU[q] * FG[q] * DUR[c] / (V[c] + eps);
    e2 = e2 + half * grav * bd2 * fr * F[q] * DTU[q] * V[c] / (V[c] + eps);
    e3 = e3 + half * grav * bd2 * fr * F[q] * V[c] / (V[c] + eps);
  }
  e0 = e0 + anela * V[i];
  e3 = e3 + V[i];
  // ---- the faces between lines: face j (to line j-1) and face j+1 (to line j+1)
  const double* F2 = f2 + p * (n2 + 1) * n1;
  const double* F2G = f2g + p * (n2 + 1) * n1;
  const double* DTU2 = dtu2 + p * (n2 + 1) * n1;
  const double* DUU2 = duu2 + p * (n2 + 1) * n1;
  const double* Vp = vol + p * n2 * n1;
  const double* DUTp = dut + p * n2 * n1;
  const double* DURp = tr ? dur + p * n2 * n1 : nullptr;
  auto fc = [&](const double* a, int jf) { return a[(size_t)jf * n1 + i]; };  // face jf of level i
  auto cl = [&](const double* a, int jc) { return a[(size_t)jc * n1 + i]; };  // cell (i, jc)
  if (j == 0) {
    const double a = bd2 * s.fac2_l * fc(F2, 0) * fc(DTU2, 0) * fc(DUU2, 0) * fc(F2G, 0);
    const double b = bd2 * s.fac2_l * fc(F2, 0) * fc(DUU2, 0) * fc(F2G, 0);
    const double den = cl(Vp, 0) + eps;
    e0 = e0 + a * cl(DUTp, 0) / den;
    if (tr) e2 = e2 + a * cl(DURp, 0) / den;
    e1 = e1 + b * cl(DUTp, 0) / den;
    if (tr) e3 = e3 + b * cl(DURp, 0) / den;
  }
  if (j > 0) {  // face j, this line as the upper one
    const int q = j, c = j - 1;
    const double S = cl(Vp, c) + cl(Vp, q) + eps;
    const double a = bd2 * 2.0 * fc(F2, q) * fc(DTU2, q) * fc(DUU2, q) * fc(F2G, q);
    const double b = bd2 * 2.0 * fc(F2, q) * fc(DUU2, q) * fc(F2G, q);
    e0 = e0 + a * cl(DUTp, q) / S;
    if (tr) e2 = e2 + a * cl(DURp, q) / S;
    e1 = e1 + b * cl(DUTp, q) / S;
    if (tr) e3 = e3 + b * cl(DURp, q) / S;
  }
  if (j < n2 - 1) {  // face j+1, this line as the lower one; the couplings between the lines
    const int q = j + 1;
    const double S = cl(Vp, j) + cl(Vp, q) + eps;
    const double a = bd2 * 2.0 * fc(F2, q) * fc(DTU2, q) * fc(DUU2, q) * fc(F2G, q);
    const double b = bd2 * 2.0 * fc(F2, q) * fc(DUU2, q) * fc(F2G, q);
    double* U = u2 + ((p * (n2 - 1) + j) * n1 + i) * 4;
    double* L = l2 + ((p * (n2 - 1) + j) * n1 + i) * 4;
    U[0] = -(a * cl(DUTp, q) / S);
    U[2] = tr ? -(a * cl(DURp, q) / S) : 0.0;
    U[1] = -(b * cl(DUTp, q) / S);
    U[3] = tr ? -(b * cl(DURp, q) / S) : 0.0;
    L[0] = -(a * cl(DUTp, j) / S);
    L[2] = tr ? -(a * cl(DURp, j) / S) : 0.0;
    L[1] = -(b * cl(DUTp, j) / S);
    L[3] = tr ? -(b * cl(DURp, j) / S) : 0.0;
    e0 = e0 + a * cl(DUTp, j) / S;
    if (tr) e2 = e2 + a * cl(DURp, j) / S;
    e1 = e1 + b * cl(DUTp, j) / S;
    if (tr) e3 = e3 + b * cl(DURp, j) / S;
  }
  if (j == n2 - 1) {
    const int q = n2;
    const double a = bd2 * s.fac2_r * fc(F2, q) * fc(DTU2, q) * fc(DUU2, q) * fc(F2G, q);
    const double b = bd2 * s.fac2_r * fc(F2, q) * fc(DUU2, q) * fc(F2G, q);
    const double den = cl(Vp, j) + eps;
    e0 = e0 + a * cl(DUTp, j) / den;
    if (tr) e2 = e2 + a * cl(DURp, j) / den;
    e1 = e1 + b * cl(DUTp, j) / den;
    if (tr) e3 = e3 + b * cl(DURp, j) / den;
  }
  out[0] = e0, out[1] = e1, out[2] = e2, out[3] = e3;
}

__global__ void k_tri_tb_compute_2d(int tr, int nplane, int n2, int n1, asam_tri_tb_coefs s, Plane2D P,
                                    double* __restrict__ d) {
  const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= (size_t)nplane * n2 * n1) return;
  element_2d(tr, n2, n1, s, P, e, d + e * 4);
}

// Compute_3D (MULTI/TriDiagTB_Mod.f90:663-780; TriDiagTR_Mod.f90:707-864) of
// n3 planes coupled through the y faces, one thread per element: the plane's
// Compute_2D entry (element_2d), then the faces between planes in the
// reference's order -- Fac3_L on plane 1, the face to the plane before, the
// face to the plane after, Fac3_R on the last plane.  The reference's two
// branches differ: with the couplings between planes stored (the level's
// u/l associated) the interior faces and Fac3_R leave DUU3 out, without them
// every face term has it; Fac3_L has it in both.
__global__ void k_tri_tb_compute_3d(int tr, int couple, int n3, int n2, int n1, asam_tri_tb_coefs s, Plane2D P,
                                    const double* __restrict__ f3, const double* __restrict__ f3g,
                                    const double* __restrict__ dtu3, const double* __restrict__ duu3,
                                    double* __restrict__ d, double* __restrict__ u3, double* __restrict__ l3) {
  const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t npl = (size_t)n2 * n1;
  if (e >= (size_t)n3 * npl) return;
  double v[4];
  element_2d(tr, n2, n1, s, P, e, v);
  double e0 = v[0], e1 = v[1], e2 = v[2], e3 = v[3];
  const size_t r = e % npl;  // (j, i) in the plane
  const int k = (int)(e / npl);
  const double bd = s.beta0_dtp, bd2 = bd * bd, eps = 1.0e-30;
  auto fc = [&](const double* a, int kf) { return a[(size_t)kf * npl + r]; };  // face kf of (i, j)
  auto cl = [&](const double* a, int kc) { return a[(size_t)kc * npl + r]; };  // cell (i, j, kc)
  const double* dur = P.dur;
  auto add = [&](double a, double b, int kc, double den) {
    e0 = e0 + a * cl(P.dut, kc) / den;
    if (tr) e2 = e2 + a * cl(dur, kc) / den;
    e1 = e1 + b * cl(P.dut, kc) / den;
    if (tr) e3 = e3 + b * cl(dur, kc) / den;
  };
  // face weights: a (first block row), b (second); DUU3 as the branch has it
  auto wa = [&](double fac, int q, bool duu) {
    return duu ? bd2 * fac * fc(f3, q) * fc(dtu3, q) * fc(duu3, q) * fc(f3g, q)
               : bd2 * fac * fc(f3, q) * fc(dtu3, q) * fc(f3g, q);
  };
  auto wb = [&](double fac, int q, bool duu) {
    return duu ? bd2 * fac * fc(f3, q) * fc(duu3, q) * fc(f3g, q) : bd2 * fac * fc(f3, q) * fc(f3g, q);
  };
  const bool inner_duu = !couple;
  if (k == 0) add(wa(s.fac3_l, 0, true), wb(s.fac3_l, 0, true), 0, cl(P.vol, 0) + eps);
  if (k > 0) {  // face k, this plane as the upper one
    const double S = cl(P.vol, k - 1) + cl(P.vol, k) + eps;
    add(wa(2.0, k, inner_duu), wb(2.0, k, inner_duu), k, S);
  }
  if (k < n3 - 1) {  // face k+1, this plane as the lower one; the couplings between the planes
    const int q = k + 1;
    const double S = cl(P.vol, k) + cl(P.vol, q) + eps;
    const double a = wa(2.0, q, inner_duu), b = wb(2.0, q, inner_duu);
    if (couple) {
      double* U = u3 + ((size_t)k * npl + r) * 4;
      double* L = l3 + ((size_t)k * npl + r) * 4;
      U[0] = -(a * cl(P.dut, q) / S);
      U[2] = tr ? -(a * cl(dur, q) / S) : 0.0;
      U[1] = -(b * cl(P.dut, q) / S);
      U[3] = tr ? -(b * cl(dur, q) / S) : 0.0;
      L[0] = -(a * cl(P.dut, k) / S);
      L[2] = tr ? -(a * cl(dur, k) / S) : 0.0;
      L[1] = -(b * cl(P.dut, k) / S);
      L[3] = tr ? -(b * cl(dur, k) / S) : 0.0;
    }
    add(a, b, k, S);
  }
  if (k == n3 - 1) add(wa(s.fac3_r, n3, inner_duu), wb(s.fac3_r, n3, inner_duu), k, cl(P.vol, k) + eps);
  double* D = d + e * 4;
  D[0] = e0, D[1] = e1, D[2] = e2, D[3] = e3;
}

// MatVecTB_2D/3D (MULTI/TriDiagTB_Mod.f90:345-372, 782-816) and MatVecTR_2D/3D
// (TriDiagTR_Mod.f90:389-416, 866-900) of one level, one thread per element:
// the line product MatVecTB_1D, then the couplings between lines (line 1:
// + u x(j+1); inner lines: + l x(j-1), then + u x(j+1); last line: + l x(j-1)),
// then those between planes the same way.  TriDiagTB's couplings are vectors
// that multiply the neighbour's first component; TriDiagTR's are 2x2 blocks
// (Mult_2).
__device__ __forceinline__ V2 couple_mul(int tr, const double* c, const V2& x) {
  if (tr) return mult_2(ld_m(c), x);
  return V2{__dmul_rn(c[0], x.x1), __dmul_rn(c[1], x.x1)};
}

// entry e of the level product; planes are coupled only when u3 is given
// (otherwise n3 counts independent planes)
__device__ __forceinline__ V2 level_entry(int tr, int n3, int n2, int n1, const double* __restrict__ d,
                                          const double* __restrict__ u1, const double* __restrict__ l1,
                                          const double* __restrict__ u2, const double* __restrict__ l2,
                                          const double* __restrict__ u3, const double* __restrict__ l3,
                                          const double* __restrict__ x, size_t e) {
  const size_t npl = (size_t)n2 * n1;
  const int i = (int)(e % n1);
  const size_t line = e / n1;
  const int j = (int)(line % n2);
  const int k = (int)(line / n2);
  const double* xl = x + line * n1 * 2;
  const M2 di = ld_m(d + e * 4);
  V2 r;  // MatVecTB_1D of the line, entry i
  if (n1 == 1) {
    r = mult_2(di, ld_v(xl));
  } else if (i == 0) {
    r = add_v(mult_2(di, ld_v(xl)), mult_2(ld_m(u1 + line * (n1 - 1) * 4), ld_v(xl + 2)));
  } else if (i == n1 - 1) {
    r = add_v(mult_2(ld_m(l1 + (line * (n1 - 1) + i - 1) * 4), ld_v(xl + (size_t)(i - 1) * 2)),
              mult_2(di, ld_v(xl + (size_t)i * 2)));
  } else {
    r = add_v(add_v(mult_2(ld_m(l1 + (line * (n1 - 1) + i - 1) * 4), ld_v(xl + (size_t)(i - 1) * 2)),
                    mult_2(di, ld_v(xl + (size_t)i * 2))),
              mult_2(ld_m(u1 + (line * (n1 - 1) + i) * 4), ld_v(xl + (size_t)(i + 1) * 2)));
  }
  if (n2 > 1) {  // between lines of plane k
    const size_t c0 = (size_t)k * (n2 - 1) * n1;
    if (j > 0) r = add_v(r, couple_mul(tr, l2 + (c0 + (size_t)(j - 1) * n1 + i) * 4, ld_v(x + (e - n1) * 2)));
    if (j < n2 - 1) r = add_v(r, couple_mul(tr, u2 + (c0 + (size_t)j * n1 + i) * 4, ld_v(x + (e + n1) * 2)));
  }
  if (n3 > 1 && u3) {  // between planes
    const size_t r0 = e % npl;
    if (k > 0) r = add_v(r, couple_mul(tr, l3 + ((size_t)(k - 1) * npl + r0) * 4, ld_v(x + (e - npl) * 2)));
    if (k < n3 - 1) r = add_v(r, couple_mul(tr, u3 + ((size_t)k * npl + r0) * 4, ld_v(x + (e + npl) * 2)));
  }
  return r;
}

__global__ void k_tri_tb_matvec_3d(int tr, int n3, int n2, int n1, const double* __restrict__ d,
                                   const double* __restrict__ u1, const double* __restrict__ l1,
                                   const double* __restrict__ u2, const double* __restrict__ l2,
                                   const double* __restrict__ u3, const double* __restrict__ l3,
                                   const double* __restrict__ x, double* __restrict__ y) {
  const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= (size_t)n3 * n2 * n1) return;
  st_v(y + e * 2, level_entry(tr, n3, n2, n1, d, u1, l1, u2, l2, u3, l3, x, e));
}

// Multigrid_2D/3D's residual b - A x (MULTI/TriDiagTB_Mod.f90:458-459, 901-902)
// of n3 planes, coupled by u3, l3 or independent when u3 is null: the
// product rounded, then the difference
__global__ void k_tri_tb_residual(int tr, int n3, int n2, int n1, const double* __restrict__ d,
                                  const double* __restrict__ u1, const double* __restrict__ l1,
                                  const double* __restrict__ u2, const double* __restrict__ l2,
                                  const double* __restrict__ u3, const double* __restrict__ l3,
                                  const double* __restrict__ b, const double* __restrict__ x,
                                  double* __restrict__ res) {
  const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= (size_t)n3 * n2 * n1) return;
  st_v(res + e * 2, sub_v(ld_v(b + e * 2), level_entry(tr, n3, n2, n1, d, u1, l1, u2, l2, u3, l3, x, e)));
}

// Multigrid_2D/3D's correction x = x + Prolongate(xc) (MULTI/TriDiagTB_Mod.f90:
// 480-488, 924-932): the coarse cell of fine entry (i, j, k) is (i/2, j/2,
// k/2) on a coarser level, (i/2, j/2, k) for independent planes (halve3 0)
__global__ void k_tri_tb_prolong_add(int halve3, int n3, int n2, int n1, const double* __restrict__ xc,
                                     double* __restrict__ x) {
  const int n1c = (n1 + 1) / 2, n2c = (n2 + 1) / 2;
  const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= (size_t)n3 * n2 * n1) return;
  const int i = (int)(e % n1);
  const int j = (int)((e / n1) % n2);
  const size_t k = e / ((size_t)n1 * n2);
  const size_t kc = halve3 ? k / 2 : k;
  st_v(x + e * 2, add_v(ld_v(x + e * 2), ld_v(xc + ((kc * n2c + j / 2) * n1c + i / 2) * 2)));
}

// RestrictTB_3D (MULTI/TriDiagTB_Mod.f90:954-1026) per coarse entry: the value
// the reference's overwriting loops leave there -- the fine cells summed
// along the axes where the entry has two (an odd axis's last cell alone), in
// the reference's term order (i,j,k), (i+1,j,k), (i,j+1,k), (i,j,k+1),
// (i+1,j+1,k), (i+1,j,k+1), (i,j+1,k+1), (i+1,j+1,k+1) of the cells present
__global__ void k_tri_tb_restrict_3d(int n3, int n2, int n1, const double* __restrict__ res,
                                     double* __restrict__ resc) {
  const int n1c = (n1 + 1) / 2, n2c = (n2 + 1) / 2, n3c = (n3 + 1) / 2;
  const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= (size_t)n3c * n2c * n1c) return;
  const int ic = (int)(e % n1c);
  const int jc = (int)((e / n1c) % n2c);
  const int kc = (int)(e / ((size_t)n1c * n2c));
  const bool pi = ic < n1 / 2, pj = jc < n2 / 2, pk = kc < n3 / 2;
  const int i0 = pi ? 2 * ic : n1 - 1, j0 = pj ? 2 * jc : n2 - 1, k0 = pk ? 2 * kc : n3 - 1;
  constexpr int ord[8] = {0, 1, 2, 4, 3, 5, 6, 7};  // bit 0: i+1, bit 1: j+1, bit 2: k+1
  V2 v{0.0, 0.0};
  bool first = true;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int di = ord[q] & 1, dj = (ord[q] >> 1) & 1, dk = (ord[q] >> 2) & 1;
    if ((di && !pi) || (dj && !pj) || (dk && !pk)) continue;
    const V2 r = ld_v(res + ((((size_t)(k0 + dk) * n2 + j0 + dj) * n1) + i0 + di) * 2);
    v = first ? r : add_v(v, r);
    first = false;
  }
  st_v(resc + e * 2, v);
}

// t - (coupling) x of every entry of a plane (GaussSeidel_3D's right-hand
// sides, MULTI/TriDiagTB_Mod.f90:830-862); t and o may be the same array
__global__ void k_tri_tb_couple_sub(int tr, int n, const double* t, const double* __restrict__ c,
                                    const double* __restrict__ x, double* o) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  st_v(o + (size_t)e * 2, couple_sub(tr, ld_v(t + (size_t)e * 2), c + (size_t)e * 4, ld_v(x + (size_t)e * 2)));
}

// The finest fields of LaplTBCompute / LaplTRCompute (MULTI/JacAccGrav_Mod.f90:
// 1312-1667) and one coarsening of them: faces f[4a + q] of direction a
// (q: F, FG, DTU, DUU; layouts of asam_tri_tb_compute_3d), cells vol, dut,
// dur (dur null for TriDiagTB)
struct TbFields {
  const double* f[12];
  const double *vol, *dut, *dur;
};
struct TbCoarse {
  double* f[12];
  double *vol, *dut, *dur;
};

__device__ __forceinline__ int tb_lo(int c, int s) { return (c - 1) * (s + 1) + 1; }
__device__ __forceinline__ int tb_hi(int c, int s, int n) { return min(c * (s + 1), n); }

// FaceCoarse of F and FG, CFaceCoarse of DTU (weighted by F) and DUU (by FG)
// (JacAccGrav_Mod.f90:784-891), one thread per coarse face: the face
// direction's fine face min((shift+1)*c, n), the other two directions'
// cells summed with direction 1 slowest (the reference's loop order), then
// the weighted sums divided by the coarse weight + Eps
__global__ void k_tb_coarse_faces(int n3, int n2, int n1, TbFields g, int c3, int c2, int c1, TbCoarse c, int s12,
                                  int s3) {
  const size_t nz = (size_t)c3 * c2 * (c1 + 1), nx = (size_t)c3 * (c2 + 1) * c1, ny = (size_t)(c3 + 1) * c2 * c1;
  const size_t e0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e0 >= nz + nx + ny) return;
  int a, ic, jc, kc;
  size_t e = e0;
  if (e < nz) {
    a = 0;
    ic = (int)(e % (c1 + 1));
    jc = (int)((e / (c1 + 1)) % c2) + 1;
    kc = (int)(e / ((size_t)(c1 + 1) * c2)) + 1;
  } else if ((e -= nz) < nx) {
    a = 1;
    ic = (int)(e % c1) + 1;
    jc = (int)((e / c1) % (c2 + 1));
    kc = (int)(e / ((size_t)c1 * (c2 + 1))) + 1;
  } else {
    e -= nx;
    a = 2;
    ic = (int)(e % c1) + 1;
    jc = (int)((e / c1) % c2) + 1;
    kc = (int)(e / ((size_t)c1 * c2));
  }
  const int e1 = a == 0, e2 = a == 1, e3 = a == 2;
  const int ilo = e1 ? min((s12 + 1) * ic, n1) : tb_lo(ic, s12), ihi = e1 ? ilo : tb_hi(ic, s12, n1);
  const int jlo = e2 ? min((s12 + 1) * jc, n2) : tb_lo(jc, s12), jhi = e2 ? jlo : tb_hi(jc, s12, n2);
  const int klo = e3 ? min((s3 + 1) * kc, n3) : tb_lo(kc, s3), khi = e3 ? klo : tb_hi(kc, s3, n3);
  const double *F = g.f[4 * a], *FG = g.f[4 * a + 1], *DT = g.f[4 * a + 2], *DU = g.f[4 * a + 3];
  double f = 0.0, fg = 0.0, tf = 0.0, ug = 0.0;
  for (int i = ilo; i <= ihi; ++i)
    for (int j = jlo; j <= jhi; ++j)
      for (int k = klo; k <= khi; ++k) {
        const size_t q = ((size_t)(e3 ? k : k - 1) * (n2 + e2) + (e2 ? j : j - 1)) * (n1 + e1) + (e1 ? i : i - 1);
        const double fq = F[q], gq = FG[q];
        f = __dadd_rn(f, fq);
        fg = __dadd_rn(fg, gq);
        tf = __dadd_rn(tf, __dmul_rn(DT[q], fq));
        ug = __dadd_rn(ug, __dmul_rn(DU[q], gq));
      }
  const size_t qc = ((size_t)(e3 ? kc : kc - 1) * (c2 + e2) + (e2 ? jc : jc - 1)) * (c1 + e1) + (e1 ? ic : ic - 1);
  c.f[4 * a][qc] = f;
  c.f[4 * a + 1][qc] = fg;
  c.f[4 * a + 2][qc] = __ddiv_rn(tf, __dadd_rn(f, asam::kEps));
  c.f[4 * a + 3][qc] = __ddiv_rn(ug, __dadd_rn(fg, asam::kEps));
}

// VolCoarse of Vol, CVolCoarse of DUT and DUR weighted by Vol
// (JacAccGrav_Mod.f90:685-782), one thread per coarse cell
__global__ void k_tb_coarse_cells(int n3, int n2, int n1, TbFields g, int c3, int c2, int c1, TbCoarse c, int s12,
                                  int s3) {
  const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= (size_t)c3 * c2 * c1) return;
  const int ic = (int)(e % c1) + 1, jc = (int)((e / c1) % c2) + 1, kc = (int)(e / ((size_t)c1 * c2)) + 1;
  double v = 0.0, tv = 0.0, rv = 0.0;
  for (int i = tb_lo(ic, s12); i <= tb_hi(ic, s12, n1); ++i)
    for (int j = tb_lo(jc, s12); j <= tb_hi(jc, s12, n2); ++j)
      for (int k = tb_lo(kc, s3); k <= tb_hi(kc, s3, n3); ++k) {
        const size_t q = ((size_t)(k - 1) * n2 + (j - 1)) * n1 + (i - 1);
        const double vq = g.vol[q];
        v = __dadd_rn(v, vq);
        tv = __dadd_rn(tv, __dmul_rn(g.dut[q], vq));
        if (g.dur) rv = __dadd_rn(rv, __dmul_rn(g.dur[q], vq));
      }
  c.vol[e] = v;
  c.dut[e] = __ddiv_rn(tv, __dadd_rn(v, asam::kEps));
  c.dur[e] = __ddiv_rn(rv, __dadd_rn(v, asam::kEps));
}

// Zebra half-sweep of GaussSeidel_2D (the GPU's parallel order): one thread per
// line j = j0 + m*jstep (m < jcount) of every plane, its right-hand side with
// the forward ((b - l x(j-1)) - u x(j+1)) or backward ((b - u x(j+1)) -
// l x(j-1)) operation order written over x(j), then Solve_1D in place; the
// lines of one parity read only lines of the other
__device__ __forceinline__ void relax_line(int tr, int n2, int n1, const double* __restrict__ d,
                                           const double* __restrict__ u1, const double* __restrict__ l1,
                                           const double* __restrict__ u2, const double* __restrict__ l2,
                                           const double* __restrict__ b, double* __restrict__ x, size_t p, int j,
                                           int bwd, double* __restrict__ w, size_t ws) {
  const size_t line = p * n2 + j;
  double* xl = x + line * n1 * 2;
  const double* bl = b + line * n1 * 2;
  for (int i = 0; i < n1; ++i) {
    V2 v = ld_v(bl + 2 * i);
    const double* cl = j > 0 ? l2 + ((p * (n2 - 1) + j - 1) * n1 + i) * 4 : nullptr;
    const double* cu = j < n2 - 1 ? u2 + ((p * (n2 - 1) + j) * n1 + i) * 4 : nullptr;
    if (!bwd) {
      if (cl) v = couple_sub(tr, v, cl, ld_v(xl - (size_t)n1 * 2 + 2 * i));
      if (cu) v = couple_sub(tr, v, cu, ld_v(xl + (size_t)n1 * 2 + 2 * i));
    } else {
      if (cu) v = couple_sub(tr, v, cu, ld_v(xl + (size_t)n1 * 2 + 2 * i));
      if (cl) v = couple_sub(tr, v, cl, ld_v(xl - (size_t)n1 * 2 + 2 * i));
    }
    st_v(xl + 2 * i, v);
  }
  solve_col(n1, d + line * n1 * 4, u1 + line * (n1 - 1) * 4, l1 + line * (n1 - 1) * 4, xl, w, ws);
}

__global__ void k_tri_tb_gs_2d_lines(int tr, int nplane, int n2, int n1, const double* __restrict__ d,
                                     const double* __restrict__ u1, const double* __restrict__ l1,
                                     const double* __restrict__ u2, const double* __restrict__ l2,
                                     const double* __restrict__ b, double* __restrict__ x, int j0, int jstep,
                                     int jcount, int bwd, double* __restrict__ w) {
  const size_t tid = blockIdx.x * (size_t)blockDim.x + threadIdx.x, nth = (size_t)nplane * jcount;
  if (tid >= nth) return;
  relax_line(tr, n2, n1, d, u1, l1, u2, l2, b, x, tid / jcount, j0 + (int)(tid % jcount) * jstep, bwd, w + tid, nth);
}

// Solve_2D on nplane planes in zebra order as one launch: one CTA per plane
// runs all mult_iter V-cycles of its plane hierarchy, its threads taking the
// lines of one parity (or the entries of a residual, restriction or
// correction) between block barriers; every relaxation, residual and
// transfer is the multi-launch path's arithmetic, so the bits are the same.
constexpr int kPlaneHierMax = 12;
struct PlaneHierDev {
  int nlev;
  int n2[kPlaneHierMax], n1[kPlaneHierMax];
  const double* a[kPlaneHierMax][5];
  double *b[kPlaneHierMax], *x[kPlaneHierMax], *res[kPlaneHierMax];
};

__global__ void __launch_bounds__(128) k_tb_plane_vcycles(int tr, int nplane, PlaneHierDev H, int gauss_iter2,
                                                          int mult_iter, double* __restrict__ w) {
  const size_t p = blockIdx.x;
  if (p >= (size_t)nplane) return;
  const int tid = threadIdx.x, nt = blockDim.x;
  const size_t ws = (size_t)nplane * H.n2[0];  // one factor slot per line of the finest level
  auto gs = [&](int l, int gi) {
    const int n2 = H.n2[l], n1 = H.n1[l];
    const double *d = H.a[l][0], *u1 = H.a[l][1], *l1 = H.a[l][2], *u2 = H.a[l][3], *l2 = H.a[l][4];
    if (n2 > 1)
      for (int it = 0; it < gi; ++it)
        for (int half = 0; half < 4; ++half) {
          const int par = half == 1 || half == 2;
          for (int j = par + 2 * tid; j < n2; j += 2 * nt)
            relax_line(tr, n2, n1, d, u1, l1, u2, l2, H.b[l], H.x[l], p, j, half >= 2, w + p * H.n2[0] + j, ws);
          __syncthreads();
        }
    if (tid == 0) relax_line(tr, n2, n1, d, u1, l1, u2, l2, H.b[l], H.x[l], p, 0, 1, w + p * H.n2[0], ws);
    __syncthreads();
  };
  for (int it = 0; it < mult_iter; ++it) {
    int gi = 1, l = 0;
    for (;;) {  // the way down (MULTI/TriDiagTB_Mod.f90:449-470)
      gs(l, gi);
      gi += gauss_iter2;
      if (l + 1 == H.nlev) {
        gi -= gauss_iter2;
        break;
      }
      const int n2 = H.n2[l], n1 = H.n1[l];
      const size_t np = (size_t)n2 * n1, base = p * np;
      for (size_t e = tid; e < np; e += nt)
        st_v(H.res[l] + (base + e) * 2,
             sub_v(ld_v(H.b[l] + (base + e) * 2), level_entry(tr, nplane, n2, n1, H.a[l][0], H.a[l][1], H.a[l][2],
                                                              H.a[l][3], H.a[l][4], nullptr, nullptr, H.x[l], base + e)));
      __syncthreads();
      const size_t npc = (size_t)H.n2[l + 1] * H.n1[l + 1], basec = p * npc;
      for (size_t e = tid; e < npc; e += nt) {
        restrict_2d_entry(n2, n1, H.res[l], H.b[l + 1], basec + e);
        st_v(H.x[l + 1] + (basec + e) * 2, V2{0.0, 0.0});
      }
      __syncthreads();
      ++l;
    }
    for (;;) {  // and up (:471-493)
      gs(l, gi);
      gi -= gauss_iter2;
      if (l == 0) break;
      --l;
      const int n2 = H.n2[l], n1 = H.n1[l], n1c = (n1 + 1) / 2, n2c = (n2 + 1) / 2;
      const size_t np = (size_t)n2 * n1;
      for (size_t e = tid; e < np; e += nt) {
        const int i = (int)(e % n1), j = (int)(e / n1);
        const size_t q = (p * np + e) * 2;
        st_v(H.x[l] + q, add_v(ld_v(H.x[l] + q), ld_v(H.x[l + 1] + ((p * n2c + j / 2) * n1c + i / 2) * 2)));
      }
      __syncthreads();
    }
  }
}

// the right-hand sides of every plane of a level at once (zebra order of
// GaussSeidel_3D): b(k) minus its couplings to planes k-1 and k+1 in the
// forward or backward operation order
__global__ void k_tri_tb_rhs3(int tr, int n3, size_t npl, const double* __restrict__ b,
                              const double* __restrict__ u3, const double* __restrict__ l3,
                              const double* __restrict__ x, int bwd, double* __restrict__ t) {
  const size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (e >= (size_t)n3 * npl) return;
  const int k = (int)(e / npl);
  const size_t r = e % npl;
  V2 v = ld_v(b + e * 2);
  const double* cl = k > 0 ? l3 + ((size_t)(k - 1) * npl + r) * 4 : nullptr;
  const double* cu = k < n3 - 1 ? u3 + ((size_t)k * npl + r) * 4 : nullptr;
  if (!bwd) {
    if (cl) v = couple_sub(tr, v, cl, ld_v(x + (e - npl) * 2));
    if (cu) v = couple_sub(tr, v, cu, ld_v(x + (e + npl) * 2));
  } else {
    if (cu) v = couple_sub(tr, v, cu, ld_v(x + (e + npl) * 2));
    if (cl) v = couple_sub(tr, v, cl, ld_v(x + (e - npl) * 2));
  }
  st_v(t + e * 2, v);
}

struct DevBufs {
  double* p[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  ~DevBufs() {
    for (double* q : p)
      if (q) cudaFree(q);
  }
};

int cu_fail(cudaError_t e) {
  asam::set_last_error(cudaGetErrorString(e), __FILE__, __LINE__);
  return ASAM_CUDA_ERROR;
}
#define TCU(expr)                               \
  do {                                          \
    cudaError_t e_ = (expr);                    \
    if (e_ != cudaSuccess) return cu_fail(e_);  \
  } while (0)

constexpr int kTbBlock = 128;

// One plane level of a V-cycle on the device: its blocks (all planes), its
// right-hand side, guess and residual.
struct PlaneLevel {
  int n2 = 0, n1 = 0;
  const double* a[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  double *b = nullptr, *x = nullptr, *res = nullptr;
};
// the smoother's per-plane scratch, sized for the finest plane
struct Scratch {
  double *t, *w;
  // zebra order: the line solves' factors (nplane x ceil(n2/2) lines of the
  // finest plane level), every plane's right-hand side and a copy of x
  double *wz = nullptr, *tall = nullptr, *xtmp = nullptr;
  // the one-launch plane V-cycle's factors: a slot per line of the finest
  // plane level of every plane
  double* wl = nullptr;
};

size_t plane_block_len(int nplane, int n2, int n1) {
  return (size_t)nplane * ((size_t)n2 * n1 * 4 + 2 * (size_t)n2 * (n1 - 1) * 4 + 2 * (size_t)(n2 - 1) * n1 * 4);
}
size_t plane_vec_len(int nplane, int n2, int n1) { return (size_t)nplane * n2 * n1 * 2; }

// the hierarchy's sizes halve (rounding up) from the finest n2 x n1 and every
// level's arrays are present
bool plane_levels_ok(int nlev, const int* n2s, const int* n1s, const double* const* d, const double* const* u1,
                     const double* const* l1, const double* const* u2, const double* const* l2, int n2, int n1) {
  if (nlev < 1 || nlev > 32 || !n2s || !n1s || !d || !u1 || !l1 || !u2 || !l2 || n2 < 1 || n1 < 1) return false;
  for (int l = 0; l < nlev; ++l) {
    if (n2s[l] != n2 || n1s[l] != n1 || !d[l] || (n1 > 1 && (!u1[l] || !l1[l])) || (n2 > 1 && (!u2[l] || !l2[l])))
      return false;
    n2 = (n2 + 1) / 2;
    n1 = (n1 + 1) / 2;
  }
  return true;
}

// copy a level's five block arrays (host or device; src null: carve only)
// into cur and carve its b, x and residual after them; cur advances past all
// of it
cudaError_t stage_plane_level(PlaneLevel& L, int nplane, int n2, int n1, const double* const src[5], double*& cur) {
  L.n2 = n2;
  L.n1 = n1;
  const size_t nl = (size_t)nplane * n2;
  const size_t len[5] = {nl * n1 * 4, nl * (n1 - 1) * 4, nl * (n1 - 1) * 4, (size_t)nplane * (n2 - 1) * n1 * 4,
                         (size_t)nplane * (n2 - 1) * n1 * 4};
  for (int q = 0; q < 5; ++q) {
    L.a[q] = cur;
    if (len[q] && src) {
      cudaError_t e = cudaMemcpy(cur, src[q], len[q] * sizeof(double), cudaMemcpyDefault);
      if (e != cudaSuccess) return e;
    }
    cur += len[q];
  }
  const size_t nv = plane_vec_len(nplane, n2, n1);
  L.b = cur;
  L.x = cur + nv;
  L.res = cur + 2 * nv;
  cur += 3 * nv;
  return cudaSuccess;
}

// Solve_2D: mult_iter V-cycles of Multigrid_2D (MULTI/TriDiagTB_Mod.f90:419-494)
// on nplane independent planes, from lv[0].b and the guess lv[0].x; the
// coarse levels' b, x and every residual are work space.  Kernels on the
// legacy stream, the level loop here.
cudaError_t plane_cycles(int variant, int nplane, int nlev, PlaneLevel* lv, const Scratch& sc, int gauss_iter2,
                         int mult_iter, long& launches, int zebra = 0) {
  if (zebra && sc.wl && nlev <= kPlaneHierMax) {  // the whole Solve_2D as one launch, a CTA per plane
    PlaneHierDev H;
    H.nlev = nlev;
    for (int l = 0; l < nlev; ++l) {
      H.n2[l] = lv[l].n2;
      H.n1[l] = lv[l].n1;
      for (int q = 0; q < 5; ++q) H.a[l][q] = lv[l].a[q];
      H.b[l] = lv[l].b;
      H.x[l] = lv[l].x;
      H.res[l] = lv[l].res;
    }
    k_tb_plane_vcycles<<<nplane, 128>>>(variant, nplane, H, gauss_iter2, mult_iter, sc.wl);
    ++launches;
    return cudaGetLastError();
  }
  auto grid = [&](const PlaneLevel& L) { return (unsigned)(((size_t)nplane * L.n2 * L.n1 + 255) / 256); };
  // GaussSeidel_2D of one level in zebra order: four half-sweeps per
  // iteration, then line 1 with the backward right-hand side
  auto gs_zebra = [&](const PlaneLevel& L, int gi) {
    auto lines = [&](int j0, int jstep, int jcount, int bwd) {
      const size_t nth = (size_t)nplane * jcount;
      k_tri_tb_gs_2d_lines<<<(unsigned)((nth + 127) / 128), 128>>>(variant, nplane, L.n2, L.n1, L.a[0], L.a[1], L.a[2],
                                                                   L.a[3], L.a[4], L.b, L.x, j0, jstep, jcount, bwd,
                                                                   sc.wz);
      ++launches;
    };
    if (L.n2 > 1)
      for (int it = 0; it < gi; ++it)
        for (int half = 0; half < 4; ++half) {
          const int par = half == 1 || half == 2;
          lines(par, 2, (L.n2 - par + 1) / 2, half >= 2);
        }
    lines(0, 1, 1, 1);
  };
#define TB_LEVEL(L) variant, nplane, (L).n2, (L).n1, (L).a[0], (L).a[1], (L).a[2], (L).a[3], (L).a[4]
  for (int it = 0; it < mult_iter; ++it) {
    int gi = 1, l = 0;
    for (;;) {  // the way down (:449-470)
      if (zebra) {
        gs_zebra(lv[l], gi);
      } else {
        k_tri_tb_gs_2d<<<(nplane + 63) / 64, 64>>>(TB_LEVEL(lv[l]), lv[l].b, lv[l].x, gi, sc.t, sc.w);
        ++launches;
      }
      gi += gauss_iter2;
      if (l + 1 == nlev) {
        gi -= gauss_iter2;
        break;
      }
      k_tri_tb_residual<<<grid(lv[l]), 256>>>(TB_LEVEL(lv[l]), nullptr, nullptr, lv[l].b, lv[l].x, lv[l].res);
      k_tri_tb_restrict_2d<<<grid(lv[l + 1]), 256>>>(nplane, lv[l].n2, lv[l].n1, lv[l].res, lv[l + 1].b);
      cudaError_t e = cudaMemsetAsync(lv[l + 1].x, 0, plane_vec_len(nplane, lv[l + 1].n2, lv[l + 1].n1) * sizeof(double));
      if (e != cudaSuccess) return e;
      launches += 2;
      ++l;
    }
    for (;;) {  // and up (:471-493)
      if (zebra) {
        gs_zebra(lv[l], gi);
      } else {
        k_tri_tb_gs_2d<<<(nplane + 63) / 64, 64>>>(TB_LEVEL(lv[l]), lv[l].b, lv[l].x, gi, sc.t, sc.w);
        ++launches;
      }
      gi -= gauss_iter2;
      if (l == 0) break;
      --l;
      k_tri_tb_prolong_add<<<grid(lv[l]), 256>>>(0, nplane, lv[l].n2, lv[l].n1, lv[l + 1].x, lv[l].x);
      ++launches;
    }
  }
#undef TB_LEVEL
  return cudaGetLastError();
}

// GaussSeidel_3D (MULTI/TriDiagTB_Mod.f90:818-874, TriDiagTR_Mod.f90:902-961) of
// one level of n3 planes whose plane hierarchy pl[0..nlev2) holds all n3
// planes (pl[0]'s b and x the level's, its residual free while the level is
// smoothed, the coarser plane levels' b, x and residual work space): the
// forward and backward plane sweeps, each plane solved by Solve_2D from the
// current guess, then plane 1 and plane n3 once more.  t: one plane.
cudaError_t level_gs(int variant, int n3, const PlaneLevel* pl, int nlev2, const double* u3, const double* l3,
                     double* t, const Scratch& sc, int gauss_iter, int gauss_iter2, int mult_iter2, long& launches,
                     int zebra = 0) {
  const size_t npl = (size_t)pl[0].n2 * pl[0].n1;
  const double* b = pl[0].b;
  double* x = pl[0].x;
  auto solve = [&](int k, const double* rhs) {
    PlaneLevel one[32];
    for (int m = 0; m < nlev2; ++m) {
      const size_t a2 = pl[m].n2, a1 = pl[m].n1;
      const size_t per[5] = {a2 * a1 * 4, a2 * (a1 - 1) * 4, a2 * (a1 - 1) * 4, (a2 - 1) * a1 * 4, (a2 - 1) * a1 * 4};
      one[m] = pl[m];
      for (int q = 0; q < 5; ++q) one[m].a[q] = pl[m].a[q] + (size_t)k * per[q];
    }
    one[0].b = const_cast<double*>(rhs);
    one[0].x = x + (size_t)k * npl * 2;
    return plane_cycles(variant, 1, nlev2, one, sc, gauss_iter2, mult_iter2, launches, zebra);
  };
  const unsigned g = (unsigned)((npl + 255) / 256);
  auto couple = [&](const double* tin, const double* c, const double* xn) {
    k_tri_tb_couple_sub<<<g, 256>>>(variant, (int)npl, tin, c, xn, t);
    ++launches;
  };
#define TB_CHECK(expr)                       \
  do {                                       \
    cudaError_t e_ = (expr);                 \
    if (e_ != cudaSuccess) return e_;        \
  } while (0)
  auto X = [&](int k) { return x + (size_t)k * npl * 2; };
  auto B = [&](int k) { return b + (size_t)k * npl * 2; };
  auto U = [&](int k) { return u3 + (size_t)k * npl * 4; };
  auto Lo = [&](int k) { return l3 + (size_t)k * npl * 4; };
  if (n3 > 1 && zebra) {
    // the planes of one parity at once: every plane's right-hand side, the 2D
    // V-cycles of all planes on a copy of x, the parity's planes copied back
    const size_t nv = (size_t)n3 * npl * 2;
    const unsigned g3 = (unsigned)((n3 * npl + 255) / 256);
    PlaneLevel all[32];
    for (int m = 0; m < nlev2; ++m) all[m] = pl[m];
    all[0].b = sc.tall;
    all[0].x = sc.xtmp;
    for (int it = 0; it < gauss_iter; ++it)
      for (int half = 0; half < 4; ++half) {
        const int par = half == 1 || half == 2;
        k_tri_tb_rhs3<<<g3, 256>>>(variant, n3, npl, b, u3, l3, x, half >= 2, sc.tall);
        ++launches;
        TB_CHECK(cudaMemcpyAsync(sc.xtmp, x, nv * sizeof(double), cudaMemcpyDeviceToDevice));
        TB_CHECK(plane_cycles(variant, n3, nlev2, all, sc, gauss_iter2, mult_iter2, launches, 1));
        TB_CHECK(cudaMemcpy2DAsync(x + par * npl * 2, 2 * npl * 2 * sizeof(double), sc.xtmp + par * npl * 2,
                                   2 * npl * 2 * sizeof(double), npl * 2 * sizeof(double), (n3 - par + 1) / 2,
                                   cudaMemcpyDeviceToDevice));
      }
    couple(B(0), U(0), X(1));
    TB_CHECK(solve(0, t));
    couple(B(n3 - 1), Lo(n3 - 2), X(n3 - 2));
    TB_CHECK(solve(n3 - 1, t));
  } else if (n3 > 1) {
    for (int it = 0; it < gauss_iter; ++it) {
      TB_CHECK(cudaMemcpyAsync(t, b, npl * 2 * sizeof(double), cudaMemcpyDeviceToDevice));
      for (int k = 0; k < n3 - 1; ++k) {
        couple(t, U(k), X(k + 1));
        TB_CHECK(solve(k, t));
        couple(B(k + 1), Lo(k), X(k));
      }
      TB_CHECK(solve(n3 - 1, t));
      couple(B(n3 - 2), U(n3 - 2), X(n3 - 1));
      for (int k = n3 - 2; k >= 1; --k) {
        couple(t, Lo(k - 1), X(k - 1));
        TB_CHECK(solve(k, t));
        couple(B(k - 1), U(k - 1), X(k));
      }
    }
    TB_CHECK(solve(0, t));
    couple(B(n3 - 1), Lo(n3 - 2), X(n3 - 2));
    TB_CHECK(solve(n3 - 1, t));
  } else {
    TB_CHECK(solve(0, b));
  }
#undef TB_CHECK
  return cudaGetLastError();
}

// Solve_3D: mult_iter3 V-cycles of Multigrid_3D (MULTI/TriDiagTB_Mod.f90:876-952)
// over levels pl[L] (plane hierarchies of all planes, pl[L][0] the level's b,
// x, residual) with couplings du3[L], dl3[L], from pl[0][0].b and the guess
// pl[0][0].x
cudaError_t level_cycles(int variant, int nlev3, const int* n3s, const int* n2s, const int* n1s, const int* nlev2s,
                         PlaneLevel (*pl)[32], double* const* du3, double* const* dl3, double* t, const Scratch& sc,
                         int gauss_iter2, int mult_iter2, int gauss_iter3, int mult_iter3, long& launches,
                         int zebra = 0) {
  auto grid = [&](int L) { return (unsigned)(((size_t)n3s[L] * n2s[L] * n1s[L] + 255) / 256); };
  cudaError_t e;
  for (int it = 0; it < mult_iter3; ++it) {
    int gi = 1, L = 0;
    for (;;) {  // the way down (:891-914)
      e = level_gs(variant, n3s[L], pl[L], nlev2s[L], du3[L], dl3[L], t, sc, gi, gauss_iter2, mult_iter2, launches,
                   zebra);
      if (e != cudaSuccess) return e;
      gi += gauss_iter3;
      if (L + 1 == nlev3) {
        gi -= gauss_iter3;
        break;
      }
      const PlaneLevel& F = pl[L][0];
      k_tri_tb_residual<<<grid(L), 256>>>(variant, n3s[L], n2s[L], n1s[L], F.a[0], F.a[1], F.a[2], F.a[3], F.a[4],
                                          du3[L], dl3[L], F.b, F.x, F.res);
      k_tri_tb_restrict_3d<<<grid(L + 1), 256>>>(n3s[L], n2s[L], n1s[L], F.res, pl[L + 1][0].b);
      e = cudaMemsetAsync(pl[L + 1][0].x, 0, plane_vec_len(n3s[L + 1], n2s[L + 1], n1s[L + 1]) * sizeof(double));
      if (e != cudaSuccess) return e;
      launches += 2;
      ++L;
    }
    for (;;) {  // and up (:915-937)
      e = level_gs(variant, n3s[L], pl[L], nlev2s[L], du3[L], dl3[L], t, sc, gi, gauss_iter2, mult_iter2, launches,
                   zebra);
      if (e != cudaSuccess) return e;
      gi -= gauss_iter3;
      if (L == 0) break;
      --L;
      k_tri_tb_prolong_add<<<grid(L), 256>>>(1, n3s[L], n2s[L], n1s[L], pl[L + 1][0].x, pl[L][0].x);
      ++launches;
    }
  }
  return cudaGetLastError();
}

}  // namespace

// The device-resident hierarchy of LaplTBCompute / LaplTRCompute: per level its
// plane hierarchy (all planes; plane level 0 carries the level's b, x and
// residual) and its couplings between planes, one allocation.
struct asam_tri_tb_hier {
  int variant = 0, nlev3 = 0, zebra = 0;
  int n3s[32] = {}, n2s[32] = {}, n1s[32] = {}, nlev2s[32] = {};
  PlaneLevel pl[32][32];
  double* du3[32] = {};
  double* dl3[32] = {};
  double* mem = nullptr;
  double* t = nullptr;
  Scratch sc{nullptr, nullptr};
  ~asam_tri_tb_hier() {
    if (mem) cudaFree(mem);
  }
};

extern "C" {

int asam_tri_tb_compute(int variant, int ncol, int n1, const asam_tri_tb_coefs* coefs, const double* f,
                        const double* fg, const double* vol, const double* dtu, const double* duu, const double* dut,
                        const double* dur, double* d, double* u, double* l) {
  if ((variant != 0 && variant != 1) || ncol < 1 || n1 < 1 || !coefs || !f || !fg || !vol || !dtu || !duu ||
      !dut || (variant == 1 && !dur) || !d || (n1 > 1 && (!u || !l))) {
    asam::set_last_error("asam_tri_tb_compute: bad argument", __FILE__, __LINE__);
    return ASAM_BAD_ARG;
  }
  const size_t nf = (size_t)ncol * (n1 + 1), nc = (size_t)ncol * n1;
  const size_t nd = nc * 4, no = (size_t)ncol * (n1 - 1) * 4;
  // inputs: f, fg, dtu, duu (faces), vol, dut, dur (cells) packed in one buffer
  DevBufs m;
  TCU(cudaMalloc((void**)&m.p[0], (4 * nf + 3 * nc) * sizeof(double)));
  TCU(cudaMalloc((void**)&m.p[1], (nd + 2 * no + 1) * sizeof(double)));
  double* in = m.p[0];
  const double* src[7] = {f, fg, dtu, duu, vol, dut, variant == 1 ? dur : vol};
  const size_t len[7] = {nf, nf, nf, nf, nc, nc, nc};
  double* dev[7];
  size_t off = 0;
  for (int q = 0; q < 7; ++q) {
    dev[q] = in + off;
    TCU(cudaMemcpy(dev[q], src[q], len[q] * sizeof(double), cudaMemcpyDefault));
    off += len[q];
  }
  double *dd = m.p[1], *du = dd + nd, *dl = du + no;
  k_tri_tb_compute<<<(ncol + kTbBlock - 1) / kTbBlock, kTbBlock>>>(variant, ncol, n1, *coefs, dev[0], dev[1], dev[4],
                                                                   dev[2], dev[3], dev[5], dev[6], dd, du, dl);
  asam::count_launches(1);
  TCU(cudaGetLastError());
  TCU(cudaMemcpy(d, dd, nd * sizeof(double), cudaMemcpyDefault));
  if (no) {
    TCU(cudaMemcpy(u, du, no * sizeof(double), cudaMemcpyDefault));
    TCU(cudaMemcpy(l, dl, no * sizeof(double), cudaMemcpyDefault));
  }
  return ASAM_OK;
}

int asam_tri_tb_compute_2d(int variant, int nplane, int n2, int n1, const asam_tri_tb_coefs* coefs,
                           const double* f1, const double* f1g, const double* dtu1, const double* duu1,
                           const double* f2, const double* f2g, const double* dtu2, const double* duu2,
                           const double* vol, const double* dut, const double* dur, double* d, double* u1,
                           double* l1, double* u2, double* l2) {
  if ((variant != 0 && variant != 1) || nplane < 1 || n2 < 1 || n1 < 1 || !coefs || !f1 || !f1g || !dtu1 ||
      !duu1 || !f2 || !f2g || !dtu2 || !duu2 || !vol || !dut || (variant == 1 && !dur) || !d ||
      (n1 > 1 && (!u1 || !l1)) || (n2 > 1 && (!u2 || !l2))) {
    asam::set_last_error("asam_tri_tb_compute_2d: bad argument", __FILE__, __LINE__);
    return ASAM_BAD_ARG;
  }
  const size_t nl = (size_t)nplane * n2, nz = nl * (n1 + 1), nx = (size_t)nplane * (n2 + 1) * n1;
  const size_t nc = nl * n1, nd = nc * 4, no1 = nl * (n1 - 1) * 4, no2 = (size_t)nplane * (n2 - 1) * n1 * 4;
  DevBufs m;
  TCU(cudaMalloc((void**)&m.p[0], (4 * nz + 4 * nx + 3 * nc) * sizeof(double)));
  TCU(cudaMalloc((void**)&m.p[1], (nd + 2 * no1 + 2 * no2 + 1) * sizeof(double)));
  const double* src[11] = {f1, f1g, dtu1, duu1, f2, f2g, dtu2, duu2, vol, dut, variant == 1 ? dur : vol};
  const size_t len[11] = {nz, nz, nz, nz, nx, nx, nx, nx, nc, nc, nc};
  double* dev[11];
  size_t off = 0;
  for (int q = 0; q < 11; ++q) {
    dev[q] = m.p[0] + off;
    TCU(cudaMemcpy(dev[q], src[q], len[q] * sizeof(double), cudaMemcpyDefault));
    off += len[q];
  }
  double *dd = m.p[1], *du1 = dd + nd, *dl1 = du1 + no1, *du2 = dl1 + no1, *dl2 = du2 + no2;
  const Plane2D P{dev[0], dev[1], dev[2], dev[3], dev[4], dev[5], dev[6], dev[7], dev[8], dev[9], dev[10],
                  du1, dl1, du2, dl2};
  k_tri_tb_compute_2d<<<(unsigned)((nc + 255) / 256), 256>>>(variant, nplane, n2, n1, *coefs, P, dd);
  asam::count_launches(1);
  TCU(cudaGetLastError());
  TCU(cudaMemcpy(d, dd, nd * sizeof(double), cudaMemcpyDefault));
  if (no1) {
    TCU(cudaMemcpy(u1, du1, no1 * sizeof(double), cudaMemcpyDefault));
    TCU(cudaMemcpy(l1, dl1, no1 * sizeof(double), cudaMemcpyDefault));
  }
  if (no2) {
    TCU(cudaMemcpy(u2, du2, no2 * sizeof(double), cudaMemcpyDefault));
    TCU(cudaMemcpy(l2, dl2, no2 * sizeof(double), cudaMemcpyDefault));
  }
  return ASAM_OK;
}

int asam_tri_tb_compute_3d(int variant, int couple, int n3, int n2, int n1, const asam_tri_tb_coefs* coefs,
                           const double* f1, const double* f1g, const double* dtu1, const double* duu1,
                           const double* f2, const double* f2g, const double* dtu2, const double* duu2,
                           const double* f3, const double* f3g, const double* dtu3, const double* duu3,
                           const double* vol, const double* dut, const double* dur, double* d, double* u1,
                           double* l1, double* u2, double* l2, double* u3, double* l3) {
  if ((variant != 0 && variant != 1) || n3 < 1 || n2 < 1 || n1 < 1 || !coefs || !f1 || !f1g || !dtu1 || !duu1 ||
      !f2 || !f2g || !dtu2 || !duu2 || !f3 || !f3g || !dtu3 || !duu3 || !vol || !dut || (variant == 1 && !dur) ||
      !d || (n1 > 1 && (!u1 || !l1)) || (n2 > 1 && (!u2 || !l2)) || (couple && n3 > 1 && (!u3 || !l3))) {
    asam::set_last_error("asam_tri_tb_compute_3d: bad argument", __FILE__, __LINE__);
    return ASAM_BAD_ARG;
  }
  const size_t npl = (size_t)n2 * n1, nl = (size_t)n3 * n2, nc = (size_t)n3 * npl;
  const size_t nz = nl * (n1 + 1), nx = (size_t)n3 * (n2 + 1) * n1, ny = (size_t)(n3 + 1) * npl;
  const size_t nd = nc * 4, no1 = nl * (n1 - 1) * 4, no2 = (size_t)n3 * (n2 - 1) * n1 * 4;
  const size_t no3 = couple ? (size_t)(n3 - 1) * npl * 4 : 0;
  DevBufs m;
  TCU(cudaMalloc((void**)&m.p[0], (4 * nz + 4 * nx + 4 * ny + 3 * nc) * sizeof(double)));
  TCU(cudaMalloc((void**)&m.p[1], (nd + 2 * no1 + 2 * no2 + 2 * no3 + 1) * sizeof(double)));
  const double* src[15] = {f1, f1g, dtu1, duu1, f2, f2g, dtu2, duu2, f3, f3g, dtu3, duu3,
                           vol, dut, variant == 1 ? dur : vol};
  const size_t len[15] = {nz, nz, nz, nz, nx, nx, nx, nx, ny, ny, ny, ny, nc, nc, nc};
  double* dev[15];
  size_t off = 0;
  for (int q = 0; q < 15; ++q) {
    dev[q] = m.p[0] + off;
    TCU(cudaMemcpy(dev[q], src[q], len[q] * sizeof(double), cudaMemcpyDefault));
    off += len[q];
  }
  double *dd = m.p[1], *du1 = dd + nd, *dl1 = du1 + no1, *du2 = dl1 + no1, *dl2 = du2 + no2;
  double *du3 = dl2 + no2, *dl3 = du3 + no3;
  const Plane2D P{dev[0], dev[1], dev[2], dev[3], dev[4], dev[5], dev[6], dev[7], dev[12], dev[13], dev[14],
                  du1, dl1, du2, dl2};
  k_tri_tb_compute_3d<<<(unsigned)((nc + 255) / 256), 256>>>(variant, couple ? 1 : 0, n3, n2, n1, *coefs, P, dev[8],
                                                              dev[9], dev[10], dev[11], dd, du3, dl3);
  asam::count_launches(1);
  TCU(cudaGetLastError());
  TCU(cudaMemcpy(d, dd, nd * sizeof(double), cudaMemcpyDefault));
  double* outs[6] = {u1, l1, u2, l2, u3, l3};
  const double* ins[6] = {du1, dl1, du2, dl2, du3, dl3};
  const size_t lens[6] = {no1, no1, no2, no2, no3, no3};
  for (int q = 0; q < 6; ++q)
    if (lens[q]) TCU(cudaMemcpy(outs[q], ins[q], lens[q] * sizeof(double), cudaMemcpyDefault));
  return ASAM_OK;
}

int asam_tri_tb_matvec_3d(int variant, int n3, int n2, int n1, const double* d, const double* u1, const double* l1,
                          const double* u2, const double* l2, const double* u3, const double* l3, const double* x,
                          double* y) {
  if ((variant != 0 && variant != 1) || n3 < 1 || n2 < 1 || n1 < 1 || !d || !x || !y || (n1 > 1 && (!u1 || !l1)) ||
      (n2 > 1 && (!u2 || !l2)) || (n3 > 1 && (!u3 || !l3))) {
    asam::set_last_error("asam_tri_tb_matvec_3d: bad argument", __FILE__, __LINE__);
    return ASAM_BAD_ARG;
  }
  const size_t npl = (size_t)n2 * n1, nc = (size_t)n3 * npl;
  const size_t len[8] = {nc * 4, (size_t)n3 * n2 * (n1 - 1) * 4, (size_t)n3 * n2 * (n1 - 1) * 4,
                         (size_t)n3 * (n2 - 1) * n1 * 4, (size_t)n3 * (n2 - 1) * n1 * 4, (size_t)(n3 - 1) * npl * 4,
                         (size_t)(n3 - 1) * npl * 4, nc * 2};
  const double* src[8] = {d, u1, l1, u2, l2, u3, l3, x};
  size_t tot = nc * 2 + 1;
  for (size_t q : len) tot += q;
  DevBufs m;
  TCU(cudaMalloc((void**)&m.p[0], tot * sizeof(double)));
  double* dev[8];
  size_t off = 0;
  for (int q = 0; q < 8; ++q) {
    dev[q] = m.p[0] + off;
    if (len[q]) TCU(cudaMemcpy(dev[q], src[q], len[q] * sizeof(double), cudaMemcpyDefault));
    off += len[q];
  }
  double* dy = m.p[0] + off;
  k_tri_tb_matvec_3d<<<(unsigned)((nc + 255) / 256), 256>>>(variant, n3, n2, n1, dev[0], dev[1], dev[2], dev[3],
                                                             dev[4], dev[5], dev[6], dev[7], dy);
  asam::count_launches(1);
  TCU(cudaGetLastError());
  TCU(cudaMemcpy(y, dy, nc * 2 * sizeof(double), cudaMemcpyDefault));
  return ASAM_OK;
}

int asam_tri_tb_gauss_seidel_2d(int variant, int nplane, int n2, int n1, const double* d, const double* u1,
                                const double* l1, const double* u2, const double* l2, const double* b, double* x,
                                int gauss_iter) {
  if ((variant != 0 && variant != 1) || nplane < 1 || n2 < 1 || n1 < 1 || !d || !b || !x ||
      (n1 > 1 && (!u1 || !l1)) || (n2 > 1 && (!u2 || !l2 || gauss_iter < 1))) {
    asam::set_last_error("asam_tri_tb_gauss_seidel_2d: bad argument", __FILE__, __LINE__);
    return ASAM_BAD_ARG;
  }
  const size_t nl = (size_t)nplane * n2;
  const size_t len[7] = {nl * n1 * 4, nl * (n1 - 1) * 4, nl * (n1 - 1) * 4, (size_t)nplane * (n2 - 1) * n1 * 4,
                         (size_t)nplane * (n2 - 1) * n1 * 4, nl * n1 * 2, nl * n1 * 2};
  const double* src[7] = {d, u1, l1, u2, l2, b, x};
  const size_t nt = (size_t)nplane * n1 * 2, nw = (size_t)nplane * (n1 > 1 ? n1 - 1 : 1) * 4;
  size_t tot = nt + nw + 1;
  for (size_t q : len) tot += q;
  DevBufs m;
  TCU(cudaMalloc((void**)&m.p[0], tot * sizeof(double)));
  double* dev[7];
  size_t off = 0;
  for (int q = 0; q < 7; ++q) {
    dev[q] = m.p[0] + off;
    if (len[q]) TCU(cudaMemcpy(dev[q], src[q], len[q] * sizeof(double), cudaMemcpyDefault));
    off += len[q];
  }
  double *tb = m.p[0] + off, *wb = tb + nt;
  k_tri_tb_gs_2d<<<(nplane + 63) / 64, 64>>>(variant, nplane, n2, n1, dev[0], dev[1], dev[2], dev[3], dev[4], dev[5],
                                             dev[6], gauss_iter, tb, wb);
  asam::count_launches(1);
  TCU(cudaGetLastError());
  TCU(cudaMemcpy(x, dev[6], len[6] * sizeof(double), cudaMemcpyDefault));
  return ASAM_OK;
}

int asam_tri_tb_multigrid_2d(int variant, int nplane, int nlev, const int* n2s, const int* n1s,
                             const double* const* d, const double* const* u1, const double* const* l1,
                             const double* const* u2, const double* const* l2, const double* b, double* x,
                             int gauss_iter2, int mult_iter) {
  bool ok = (variant == 0 || variant == 1) && nplane >= 1 && b && x && gauss_iter2 >= 0 && mult_iter >= 0 &&
            plane_levels_ok(nlev, n2s, n1s, d, u1, l1, u2, l2, (nlev >= 1 && n2s) ? n2s[0] : 0,
                            (nlev >= 1 && n1s) ? n1s[0] : 0);
  if (!ok) {
    asam::set_last_error("asam_tri_tb_multigrid_2d: bad argument", __FILE__, __LINE__);
    return ASAM_BAD_ARG;
  }
  // one allocation: the levels' blocks, b, x and the residual of every level
  size_t tot = 0;
  for (int l = 0; l < nlev; ++l) tot += plane_block_len(nplane, n2s[l], n1s[l]) + 3 * plane_vec_len(nplane, n2s[l], n1s[l]);
  const size_t nt = (size_t)nplane * n1s[0] * 2, nw = (size_t)nplane * (n1s[0] > 1 ? n1s[0] - 1 : 1) * 4;
  DevBufs m;
  TCU(cudaMalloc((void**)&m.p[0], (tot + nt + nw) * sizeof(double)));
  PlaneLevel lv[32];
  double* cur = m.p[0];
  for (int l = 0; l < nlev; ++l) {
    const double* src[5] = {d[l], u1[l], l1[l], u2[l], l2[l]};
    TCU(stage_plane_level(lv[l], nplane, n2s[l], n1s[l], src, cur));
  }
  Scratch sc{cur, cur + nt};
  TCU(cudaMemcpy(lv[0].b, b, plane_vec_len(nplane, n2s[0], n1s[0]) * sizeof(double), cudaMemcpyDefault));
  TCU(cudaMemcpy(lv[0].x, x, plane_vec_len(nplane, n2s[0], n1s[0]) * sizeof(double), cudaMemcpyDefault));
  long launches = 0;
  TCU(plane_cycles(variant, nplane, nlev, lv, sc, gauss_iter2, mult_iter, launches));
  asam::count_launches(launches);
  TCU(cudaMemcpy(x, lv[0].x, plane_vec_len(nplane, n2s[0], n1s[0]) * sizeof(double), cudaMemcpyDefault));
  return ASAM_OK;
}

int asam_tri_tb_multigrid_3d(int variant, int nlev3, const int* n3s, const int* n2s, const int* n1s, const int* nlev2s,
                             const double* const* u3, const double* const* l3, const double* const* d,
                             const double* const* u1, const double* const* l1, const double* const* u2,
                             const double* const* l2, const double* b, double* x, int gauss_iter2, int mult_iter2,
                             int gauss_iter3, int mult_iter3) {
  bool ok = (variant == 0 || variant == 1) && nlev3 >= 1 && nlev3 <= 32 && n3s && n2s && n1s && nlev2s && u3 && l3 &&
            d && u1 && l1 && u2 && l2 && b && x && gauss_iter2 >= 0 && mult_iter2 >= 0 && gauss_iter3 >= 0 &&
            mult_iter3 >= 0;
  int p2[32][32], p1[32][32], off[32];
  for (int L = 0, o = 0; ok && L < nlev3; ++L) {
    ok = n3s[L] >= 1 && n2s[L] >= 1 && n1s[L] >= 1 && nlev2s[L] >= 1 && nlev2s[L] <= 32 && o + nlev2s[L] <= 1024 &&
         (n3s[L] == 1 || (u3[L] && l3[L]));
    if (ok && L > 0)
      ok = n3s[L] == (n3s[L - 1] + 1) / 2 && n2s[L] == (n2s[L - 1] + 1) / 2 && n1s[L] == (n1s[L - 1] + 1) / 2;
    if (!ok) break;
    p2[L][0] = n2s[L];
    p1[L][0] = n1s[L];
    for (int m = 1; m < nlev2s[L]; ++m) {
      p2[L][m] = (p2[L][m - 1] + 1) / 2;
      p1[L][m] = (p1[L][m - 1] + 1) / 2;
    }
    ok = plane_levels_ok(nlev2s[L], p2[L], p1[L], d + o, u1 + o, l1 + o, u2 + o, l2 + o, n2s[L], n1s[L]);
    off[L] = o;
    o += nlev2s[L];
  }
  if (!ok) {
    asam::set_last_error("asam_tri_tb_multigrid_3d: bad argument", __FILE__, __LINE__);
    return ASAM_BAD_ARG;
  }
  // one allocation: every level's plane hierarchy (blocks, b, x, residual
  // for all its planes), its couplings between planes, the smoother's plane
  // right-hand side and scratch
  size_t tot = 0;
  for (int L = 0; L < nlev3; ++L) {
    for (int m = 0; m < nlev2s[L]; ++m)
      tot += plane_block_len(n3s[L], p2[L][m], p1[L][m]) + 3 * plane_vec_len(n3s[L], p2[L][m], p1[L][m]);
    tot += 2 * (size_t)(n3s[L] - 1) * n2s[L] * n1s[L] * 4;
  }
  const size_t npl = (size_t)n2s[0] * n1s[0], nt = (size_t)n1s[0] * 2, nw = (size_t)(n1s[0] > 1 ? n1s[0] - 1 : 1) * 4;
  DevBufs m;
  TCU(cudaMalloc((void**)&m.p[0], (tot + npl * 2 + nt + nw) * sizeof(double)));
  static thread_local PlaneLevel pl[32][32];
  double* cur = m.p[0];
  double *du3[32], *dl3[32];
  for (int L = 0; L < nlev3; ++L) {
    for (int q = 0; q < nlev2s[L]; ++q) {
      const int o = off[L] + q;
      const double* src[5] = {d[o], u1[o], l1[o], u2[o], l2[o]};
      TCU(stage_plane_level(pl[L][q], n3s[L], p2[L][q], p1[L][q], src, cur));
    }
    const size_t nc = (size_t)(n3s[L] - 1) * n2s[L] * n1s[L] * 4;
    du3[L] = nc ? cur : nullptr;
    dl3[L] = nc ? cur + nc : nullptr;
    if (nc) {
      TCU(cudaMemcpy(du3[L], u3[L], nc * sizeof(double), cudaMemcpyDefault));
      TCU(cudaMemcpy(dl3[L], l3[L], nc * sizeof(double), cudaMemcpyDefault));
    }
    cur += 2 * nc;
  }
  double* t = cur;
  Scratch sc{cur + npl * 2, cur + npl * 2 + nt};
  const size_t nv0 = plane_vec_len(n3s[0], n2s[0], n1s[0]);
  TCU(cudaMemcpy(pl[0][0].b, b, nv0 * sizeof(double), cudaMemcpyDefault));
  TCU(cudaMemcpy(pl[0][0].x, x, nv0 * sizeof(double), cudaMemcpyDefault));
  long launches = 0;
  TCU(level_cycles(variant, nlev3, n3s, n2s, n1s, nlev2s, pl, du3, dl3, t, sc, gauss_iter2, mult_iter2, gauss_iter3,
                   mult_iter3, launches));
  asam::count_launches(launches);
  TCU(cudaMemcpy(x, pl[0][0].x, nv0 * sizeof(double), cudaMemcpyDefault));
  return ASAM_OK;
}

int asam_tri_tb_hier_create(int variant, int ref_level, int n3, int n2, int n1, const asam_tri_tb_coefs* coefs,
                            const double* const* faces, const double* vol, const double* dut, const double* dur,
                            asam_tri_tb_hier** out) {
  // ref_level <= 24: the shifts 2^L - 1 stay within int, and 2^23 cells per
  // direction already coarsen to one
  bool ok = (variant == 0 || variant == 1) && ref_level >= 1 && ref_level <= 24 && n3 >= 1 && n2 >= 1 && n1 >= 1 &&
            coefs && faces && vol && dut && (variant == 0 || dur) && out;
  for (int q = 0; ok && q < 12; ++q) ok = faces[q] != nullptr;
  if (!ok) {
    asam::set_last_error("asam_tri_tb_hier_create: bad argument", __FILE__, __LINE__);
    return ASAM_BAD_ARG;
  }
  *out = nullptr;
  std::unique_ptr<asam_tri_tb_hier> h(new asam_tri_tb_hier);
  h->variant = variant;
  h->nlev3 = ref_level;
  // level L3: n3 halved L3 times (rounding up); its plane level m: n2, n1
  // halved L3 + m times (LaplTBCompute's (n + Shift)/(Shift + 1))
  auto cdiv = [](int n, int L) { return (int)(((long long)n + (1LL << L) - 1) >> L); };
  size_t tot = 0;
  for (int L = 0; L < ref_level; ++L) {
    h->n3s[L] = cdiv(n3, L);
    h->n2s[L] = cdiv(n2, L);
    h->n1s[L] = cdiv(n1, L);
    h->nlev2s[L] = ref_level - L;
    for (int m = 0; m < h->nlev2s[L]; ++m)
      tot += plane_block_len(h->n3s[L], cdiv(n2, L + m), cdiv(n1, L + m)) +
             3 * plane_vec_len(h->n3s[L], cdiv(n2, L + m), cdiv(n1, L + m));
    tot += 2 * (size_t)(h->n3s[L] - 1) * h->n2s[L] * h->n1s[L] * 4;
  }
  const size_t npl = (size_t)n2 * n1, nc = (size_t)n3 * npl;
  const size_t nz = (size_t)n3 * n2 * (n1 + 1), nx = (size_t)n3 * (n2 + 1) * n1, ny = (size_t)(n3 + 1) * npl;
  const size_t nt = (size_t)n1 * 2, nw = (size_t)(n1 > 1 ? n1 - 1 : 1) * 4;
  const size_t fields = 4 * (nz + nx + ny) + 3 * nc;  // the finest fields, and room for one coarsening of them
  const size_t nwz = (size_t)n3 * ((n2 + 1) / 2) * (n1 > 1 ? n1 - 1 : 1) * 4;
  const size_t nwl = (size_t)n3 * n2 * (n1 > 1 ? n1 - 1 : 1) * 4;
  TCU(cudaMalloc((void**)&h->mem, (tot + npl * 2 + nt + nw + nwz + 2 * nc * 2 + nwl) * sizeof(double)));
  DevBufs work;
  TCU(cudaMalloc((void**)&work.p[0], 2 * fields * sizeof(double)));
  double* cur = h->mem;
  for (int L = 0; L < ref_level; ++L) {
    for (int m = 0; m < h->nlev2s[L]; ++m)
      TCU(stage_plane_level(h->pl[L][m], h->n3s[L], cdiv(n2, L + m), cdiv(n1, L + m), nullptr, cur));
    const size_t ncp = (size_t)(h->n3s[L] - 1) * h->n2s[L] * h->n1s[L] * 4;
    h->du3[L] = ncp ? cur : nullptr;
    h->dl3[L] = ncp ? cur + ncp : nullptr;
    cur += 2 * ncp;
  }
  h->t = cur;
  h->sc = Scratch{cur + npl * 2, cur + npl * 2 + nt};
  h->sc.wz = cur + npl * 2 + nt + nw;
  h->sc.tall = h->sc.wz + nwz;
  h->sc.xtmp = h->sc.tall + nc * 2;
  h->sc.wl = h->sc.xtmp + nc * 2;
  // the finest fields on the device
  TbFields g;
  double* fp = work.p[0];
  const size_t flen[3] = {nz, nx, ny};
  for (int q = 0; q < 12; ++q) {
    TCU(cudaMemcpy(fp, faces[q], flen[q / 4] * sizeof(double), cudaMemcpyDefault));
    g.f[q] = fp;
    fp += flen[q / 4];
  }
  const double* cells[3] = {vol, dut, variant == 1 ? dur : nullptr};
  const double* gc[3];
  for (int q = 0; q < 3; ++q) {
    if (cells[q]) TCU(cudaMemcpy(fp, cells[q], nc * sizeof(double), cudaMemcpyDefault));
    gc[q] = cells[q] ? fp : nullptr;
    fp += nc;
  }
  g.vol = gc[0];
  g.dut = gc[1];
  g.dur = gc[2];
  long launches = 0;
  for (int L3 = 0; L3 < ref_level; ++L3)
    for (int L2 = L3; L2 < ref_level; ++L2) {
      const int s12 = (1 << L2) - 1, s3 = (1 << L3) - 1;
      const int c3 = cdiv(n3, L3), c2 = cdiv(n2, L2), c1 = cdiv(n1, L2);
      const size_t cz = (size_t)c3 * c2 * (c1 + 1), cx = (size_t)c3 * (c2 + 1) * c1, cy = (size_t)(c3 + 1) * c2 * c1;
      const size_t ccl = (size_t)c3 * c2 * c1;
      TbCoarse c;
      double* cp = work.p[0] + fields;
      const size_t clen[3] = {cz, cx, cy};
      for (int q = 0; q < 12; ++q) {
        c.f[q] = cp;
        cp += clen[q / 4];
      }
      c.vol = cp;
      c.dut = cp + ccl;
      c.dur = cp + 2 * ccl;
      k_tb_coarse_faces<<<(unsigned)((cz + cx + cy + 255) / 256), 256>>>(n3, n2, n1, g, c3, c2, c1, c, s12, s3);
      k_tb_coarse_cells<<<(unsigned)((ccl + 255) / 256), 256>>>(n3, n2, n1, g, c3, c2, c1, c, s12, s3);
      PlaneLevel& P = h->pl[L3][L2 - L3];
      const Plane2D P2{c.f[0], c.f[1], c.f[2], c.f[3], c.f[4], c.f[5], c.f[6], c.f[7], c.vol, c.dut, c.dur,
                       const_cast<double*>(P.a[1]), const_cast<double*>(P.a[2]), const_cast<double*>(P.a[3]),
                       const_cast<double*>(P.a[4])};
      const bool couple = L2 == L3;
      k_tri_tb_compute_3d<<<(unsigned)((ccl + 255) / 256), 256>>>(variant, couple ? 1 : 0, c3, c2, c1, *coefs, P2,
                                                                   c.f[8], c.f[9], c.f[10], c.f[11],
                                                                   const_cast<double*>(P.a[0]),
                                                                   couple ? h->du3[L3] : nullptr,
                                                                   couple ? h->dl3[L3] : nullptr);
      launches += 3;
      TCU(cudaGetLastError());
    }
  TCU(cudaDeviceSynchronize());
  asam::count_launches(launches);
  *out = h.release();
  return ASAM_OK;
}

int asam_tri_tb_hier_get(const asam_tri_tb_hier* h, int level3, int level2, int which, double* dst) {
  if (!h || level3 < 0 || level3 >= h->nlev3 || level2 < level3 || level2 - level3 >= h->nlev2s[level3] || which < 0 ||
      which > 6 || !dst) {
    asam::set_last_error("asam_tri_tb_hier_get: bad argument", __FILE__, __LINE__);
    return ASAM_BAD_ARG;
  }
  const PlaneLevel& P = h->pl[level3][level2 - level3];
  const size_t n3 = h->n3s[level3], n2 = P.n2, n1 = P.n1;
  const size_t len[7] = {n3 * n2 * n1 * 4,      n3 * n2 * (n1 - 1) * 4, n3 * n2 * (n1 - 1) * 4, n3 * (n2 - 1) * n1 * 4,
                         n3 * (n2 - 1) * n1 * 4, (n3 - 1) * n2 * n1 * 4, (n3 - 1) * n2 * n1 * 4};
  const double* src = which < 5 ? P.a[which] : (level2 == level3 ? (which == 5 ? h->du3[level3] : h->dl3[level3]) : nullptr);
  if (which >= 5 && level2 != level3) {
    asam::set_last_error("asam_tri_tb_hier_get: couplings between planes exist on a level's own planes only", __FILE__,
                         __LINE__);
    return ASAM_BAD_ARG;
  }
  if (len[which]) TCU(cudaMemcpy(dst, src, len[which] * sizeof(double), cudaMemcpyDefault));
  return ASAM_OK;
}

int asam_tri_tb_hier_vcycle(asam_tri_tb_hier* h, const double* b, double* x, int gauss_iter2, int mult_iter2,
                            int gauss_iter3, int mult_iter3) {
  if (!h || !b || !x || gauss_iter2 < 0 || mult_iter2 < 0 || gauss_iter3 < 0 || mult_iter3 < 0) {
    asam::set_last_error("asam_tri_tb_hier_vcycle: bad argument", __FILE__, __LINE__);
    return ASAM_BAD_ARG;
  }
  const size_t nv0 = plane_vec_len(h->n3s[0], h->n2s[0], h->n1s[0]);
  TCU(cudaMemcpy(h->pl[0][0].b, b, nv0 * sizeof(double), cudaMemcpyDefault));
  TCU(cudaMemcpy(h->pl[0][0].x, x, nv0 * sizeof(double), cudaMemcpyDefault));
  long launches = 0;
  TCU(level_cycles(h->variant, h->nlev3, h->n3s, h->n2s, h->n1s, h->nlev2s, h->pl, h->du3, h->dl3, h->t, h->sc,
                   gauss_iter2, mult_iter2, gauss_iter3, mult_iter3, launches, h->zebra));
  asam::count_launches(launches);
  TCU(cudaMemcpy(x, h->pl[0][0].x, nv0 * sizeof(double), cudaMemcpyDefault));
  return ASAM_OK;
}

int asam_tri_tb_hier_set_zebra(asam_tri_tb_hier* h, int on) {
  if (!h) {
    asam::set_last_error("asam_tri_tb_hier_set_zebra: bad argument", __FILE__, __LINE__);
    return ASAM_BAD_ARG;
  }
  h->zebra = on != 0;
  return ASAM_OK;
}

void asam_tri_tb_hier_destroy(asam_tri_tb_hier* h) { delete h; }

int asam_tri_tb_restrict_2d(int nplane, int n2, int n1, const double* res, double* resc) {
  if (nplane < 1 || n2 < 1 || n1 < 1 || !res || !resc) {
    asam::set_last_error("asam_tri_tb_restrict_2d: bad argument", __FILE__, __LINE__);
    return ASAM_BAD_ARG;
  }
  const size_t nf = (size_t)nplane * n2 * n1 * 2, nc = (size_t)nplane * ((n2 + 1) / 2) * ((n1 + 1) / 2) * 2;
  DevBufs m;
  TCU(cudaMalloc((void**)&m.p[0], (nf + nc) * sizeof(double)));
  TCU(cudaMemcpy(m.p[0], res, nf * sizeof(double), cudaMemcpyDefault));
  k_tri_tb_restrict_2d<<<(unsigned)((nc / 2 + 255) / 256), 256>>>(nplane, n2, n1, m.p[0], m.p[0] + nf);
  asam::count_launches(1);
  TCU(cudaGetLastError());
  TCU(cudaMemcpy(resc, m.p[0] + nf, nc * sizeof(double), cudaMemcpyDefault));
  return ASAM_OK;
}

int asam_tri_tb_prolong_2d(int nplane, int n2, int n1, const double* xc, double* x) {
  if (nplane < 1 || n2 < 1 || n1 < 1 || !xc || !x) {
    asam::set_last_error("asam_tri_tb_prolong_2d: bad argument", __FILE__, __LINE__);
    return ASAM_BAD_ARG;
  }
  const size_t nf = (size_t)nplane * n2 * n1 * 2, nc = (size_t)nplane * ((n2 + 1) / 2) * ((n1 + 1) / 2) * 2;
  DevBufs m;
  TCU(cudaMalloc((void**)&m.p[0], (nf + nc) * sizeof(double)));
  TCU(cudaMemcpy(m.p[0], xc, nc * sizeof(double), cudaMemcpyDefault));
  k_tri_tb_prolong_2d<<<(unsigned)((nf / 2 + 255) / 256), 256>>>(nplane, n2, n1, m.p[0], m.p[0] + nc);
  asam::count_launches(1);
  TCU(cudaGetLastError());
  TCU(cudaMemcpy(x, m.p[0] + nc, nf * sizeof(double), cudaMemcpyDefault));
  return ASAM_OK;
}

int asam_tri_tb_solve(int ncol, int n1, const double* d, const double* u, const double* l, double* b) {
  if (ncol < 1 || n1 < 1 || !d || !b || (n1 > 1 && (!u || !l))) {
    asam::set_last_error("asam_tri_tb_solve: bad argument", __FILE__, __LINE__);
    return ASAM_BAD_ARG;
  }
  const size_t nd = (size_t)ncol * n1 * 4, no = (size_t)ncol * (n1 - 1) * 4, nb = (size_t)ncol * n1 * 2;
  DevBufs m;
  TCU(cudaMalloc((void**)&m.p[0], nd * sizeof(double)));
  TCU(cudaMalloc((void**)&m.p[1], nb * sizeof(double)));
  if (no) {
    TCU(cudaMalloc((void**)&m.p[2], no * sizeof(double)));
    TCU(cudaMalloc((void**)&m.p[3], no * sizeof(double)));
    TCU(cudaMalloc((void**)&m.p[4], no * sizeof(double)));
    TCU(cudaMemcpy(m.p[2], u, no * sizeof(double), cudaMemcpyDefault));
    TCU(cudaMemcpy(m.p[3], l, no * sizeof(double), cudaMemcpyDefault));
  }
  TCU(cudaMemcpy(m.p[0], d, nd * sizeof(double), cudaMemcpyDefault));
  TCU(cudaMemcpy(m.p[1], b, nb * sizeof(double), cudaMemcpyDefault));
  k_tri_tb_solve<<<(ncol + kTbBlock - 1) / kTbBlock, kTbBlock>>>(ncol, n1, m.p[0], m.p[2], m.p[3], m.p[1], m.p[4]);
  asam::count_launches(1);
  TCU(cudaGetLastError());
  TCU(cudaMemcpy(b, m.p[1], nb * sizeof(double), cudaMemcpyDefault));
  return ASAM_OK;
}

int asam_tri_tb_matvec(int ncol, int n1, const double* d, const double* u, const double* l, const double* x,
                       double* y) {
  if (ncol < 1 || n1 < 1 || !d || !x || !y || (n1 > 1 && (!u || !l))) {
    asam::set_last_error("asam_tri_tb_matvec: bad argument", __FILE__, __LINE__);
    return ASAM_BAD_ARG;
  }
  const size_t nd = (size_t)ncol * n1 * 4, no = (size_t)ncol * (n1 - 1) * 4, nb = (size_t)ncol * n1 * 2;
  DevBufs m;
  TCU(cudaMalloc((void**)&m.p[0], nd * sizeof(double)));
  TCU(cudaMalloc((void**)&m.p[1], nb * sizeof(double)));
  TCU(cudaMalloc((void**)&m.p[5], nb * sizeof(double)));
  if (no) {
    TCU(cudaMalloc((void**)&m.p[2], no * sizeof(double)));
    TCU(cudaMalloc((void**)&m.p[3], no * sizeof(double)));
    TCU(cudaMemcpy(m.p[2], u, no * sizeof(double), cudaMemcpyDefault));
    TCU(cudaMemcpy(m.p[3], l, no * sizeof(double), cudaMemcpyDefault));
  }
  TCU(cudaMemcpy(m.p[0], d, nd * sizeof(double), cudaMemcpyDefault));
  TCU(cudaMemcpy(m.p[1], x, nb * sizeof(double), cudaMemcpyDefault));
  const size_t n = (size_t)ncol * n1;
  k_tri_tb_matvec<<<(unsigned)((n + 255) / 256), 256>>>(ncol, n1, m.p[0], m.p[2], m.p[3], m.p[1], m.p[5]);
  asam::count_launches(1);
  TCU(cudaGetLastError());
  TCU(cudaMemcpy(y, m.p[5], nb * sizeof(double), cudaMemcpyDefault));
  return ASAM_OK;
}

}  // extern "C"
