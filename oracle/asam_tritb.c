/* Oracle (test infrastructure only) of the block-tridiagonal column solve of
 * MULTI/TriDiagTB_Mod.f90: Solve_1D (:143-163) and MatVecTB_1D (:121-141),
 * with the 2x2 helpers of CG/Matrix_Mod.f90 (Mult_2, Mult_22, Div_2, Div_22)
 * in their operation order.  Compiled without contraction.  Layout: the
 * reference's per-column arrays back to back, 2x2 blocks column-major
 * (index r + 2c), vectors (index r) per level. */
#include <stddef.h>
#include <stdlib.h>
#include <string.h>

#define EPS_TB 1.0e-30 /* CG/Kind_Mod_gf.f90 Eps */

static void mult_2(const double *b, const double *c, double *o) {
  double t1 = b[0] * c[0] + b[2] * c[1];
  double t2 = b[1] * c[0] + b[3] * c[1];
  o[0] = t1;
  o[1] = t2;
}

static void mult_22(const double *b, const double *c, double *o) {
  double t11 = b[0] * c[0] + b[2] * c[1];
  double t12 = b[0] * c[2] + b[2] * c[3];
  double t21 = b[1] * c[0] + b[3] * c[1];
  double t22 = b[1] * c[2] + b[3] * c[3];
  o[0] = t11;
  o[1] = t21;
  o[2] = t12;
  o[3] = t22;
}

static void div_2(const double *b, const double *c, double *o) {
  double det = c[0] * c[3] - c[2] * c[1];
  double t1 = (c[3] * b[0] - c[2] * b[1]) / det;
  double t2 = (-c[1] * b[0] + c[0] * b[1]) / det;
  o[0] = t1;
  o[1] = t2;
}

static void div_22(const double *b, const double *c, double *o) {
  double det = c[0] * c[3] - c[2] * c[1];
  double t11 = (c[3] * b[0] - c[2] * b[1]) / det;
  double t12 = (c[3] * b[2] - c[2] * b[3]) / det;
  double t21 = (-c[1] * b[0] + c[0] * b[1]) / det;
  double t22 = (-c[1] * b[2] + c[0] * b[3]) / det;
  o[0] = t11;
  o[1] = t21;
  o[2] = t12;
  o[3] = t22;
}

void ora_tri_tb_solve(int ncol, int n1, const double *d, const double *u, const double *l, double *b,
                      double *w) {
  for (int col = 0; col < ncol; ++col) {
    const double *dc = d + (size_t)col * n1 * 4;
    const double *uc = u + (size_t)col * (n1 - 1) * 4;
    const double *lc = l + (size_t)col * (n1 - 1) * 4;
    double *bc = b + (size_t)col * n1 * 2;
    double t[4] = {dc[0], dc[1], dc[2], dc[3]}, m[4], v[2];
    div_2(bc, t, bc);
    for (int i = 1; i < n1; ++i) {
      div_22(uc + (size_t)(i - 1) * 4, t, w + (size_t)(i - 1) * 4);
      mult_22(lc + (size_t)(i - 1) * 4, w + (size_t)(i - 1) * 4, m);
      for (int e = 0; e < 4; ++e) t[e] = dc[(size_t)i * 4 + e] - m[e];
      mult_2(lc + (size_t)(i - 1) * 4, bc + (size_t)(i - 1) * 2, v);
      v[0] = bc[(size_t)i * 2] - v[0];
      v[1] = bc[(size_t)i * 2 + 1] - v[1];
      div_2(v, t, bc + (size_t)i * 2);
    }
    for (int i = n1 - 2; i >= 0; --i) {
      mult_2(w + (size_t)i * 4, bc + (size_t)(i + 1) * 2, v);
      bc[(size_t)i * 2] -= v[0];
      bc[(size_t)i * 2 + 1] -= v[1];
    }
  }
}

void ora_tri_tb_matvec(int ncol, int n1, const double *d, const double *u, const double *l, const double *x,
                       double *y) {
  for (int col = 0; col < ncol; ++col) {
    const double *dc = d + (size_t)col * n1 * 4;
    const double *uc = u + (size_t)col * (n1 - 1) * 4;
    const double *lc = l + (size_t)col * (n1 - 1) * 4;
    const double *xc = x + (size_t)col * n1 * 2;
    double *yc = y + (size_t)col * n1 * 2;
    double a[2], b[2], c[2];
    for (int i = 0; i < n1; ++i) {
      mult_2(dc + (size_t)i * 4, xc + (size_t)i * 2, b);
      if (n1 == 1) {
        yc[0] = b[0];
        yc[1] = b[1];
      } else if (i == 0) {
        mult_2(uc, xc + 2, c);
        yc[0] = b[0] + c[0];
        yc[1] = b[1] + c[1];
      } else if (i == n1 - 1) {
        mult_2(lc + (size_t)(i - 1) * 4, xc + (size_t)(i - 1) * 2, a);
        yc[(size_t)i * 2] = a[0] + b[0];
        yc[(size_t)i * 2 + 1] = a[1] + b[1];
      } else {
        mult_2(lc + (size_t)(i - 1) * 4, xc + (size_t)(i - 1) * 2, a);
        mult_2(uc + (size_t)i * 4, xc + (size_t)(i + 1) * 2, c);
        yc[(size_t)i * 2] = (a[0] + b[0]) + c[0];
        yc[(size_t)i * 2 + 1] = (a[1] + b[1]) + c[1];
      }
    }
  }
}

/* Compute_1D of the block-tridiagonal line systems: Allocate_1D (d = 1e-40 on
 * the diagonal of each block, u = l = 0) then the assembly of
 * MULTI/TriDiagTB_Mod.f90:32-93 (variant 0) or MULTI/TriDiagTR_Mod.f90:32-105
 * (variant 1, with the DUR terms of the second block column), statement by
 * statement; the GradFull and .NOT.GradFull branches of the reference are the
 * same statements.  s = {beta0*dtp, Fac1_L, Fac1_R, GravComp, FacAnela};
 * face arrays f, fg, dtu, duu [col*(n1+1) + i], cell arrays vol, dut, dur
 * [col*n1 + i]; d [col*n1 + i][4], u, l [col*(n1-1) + i][4], blocks
 * column-major (r + 2c). */
void ora_tri_tb_compute(int variant, int ncol, int n1, const double *s, const double *f, const double *fg,
                        const double *vol, const double *dtu, const double *duu, const double *dut,
                        const double *dur, double *d, double *u, double *l) {
  const double bd = s[0], fl = s[1], fr = s[2], grav = s[3], anela = s[4];
  const double bd2 = bd * bd, half = 0.5, eps = 1.0e-30;
  const int tr = variant == 1;
  for (int col = 0; col < ncol; ++col) {
    const double *F = f + (size_t)col * (n1 + 1), *FG = fg + (size_t)col * (n1 + 1);
    const double *DTU = dtu + (size_t)col * (n1 + 1), *DUU = duu + (size_t)col * (n1 + 1);
    const double *V = vol + (size_t)col * n1, *DUT = dut + (size_t)col * n1;
    const double *DUR = tr ? dur + (size_t)col * n1 : 0;
    double *D = d + (size_t)col * n1 * 4;
    double *U = u + (size_t)col * (n1 - 1) * 4, *L = l + (size_t)col * (n1 - 1) * 4;
#define DD(r, c, i) D[(size_t)(i) * 4 + (r) + 2 * (c)]
#define UU(r, c, i) U[(size_t)(i) * 4 + (r) + 2 * (c)]
#define LL(r, c, i) L[(size_t)(i) * 4 + (r) + 2 * (c)]
    for (int i = 0; i < n1; ++i) {
      DD(0, 0, i) = 1.0e-40;
      DD(1, 0, i) = 0.0;
      DD(0, 1, i) = 0.0;
      DD(1, 1, i) = 1.0e-40;
    }
    for (int i = 0; i < n1 - 1; ++i)
      for (int e = 0; e < 4; ++e) U[(size_t)i * 4 + e] = L[(size_t)i * 4 + e] = 0.0;
    /* first cell, face 1 */
    DD(0, 0, 0) = DD(0, 0, 0) + bd2 * fl * F[0] * DTU[0] * DUU[0] * FG[0] * DUT[0] / (V[0] + eps);
    if (tr) DD(0, 1, 0) = DD(0, 1, 0) + bd2 * fl * F[0] * DTU[0] * DUU[0] * FG[0] * DUR[0] / (V[0] + eps);
    DD(1, 0, 0) = DD(1, 0, 0) + bd2 * fl * F[0] * DUU[0] * FG[0] * DUT[0] / (V[0] + eps);
    if (tr) DD(1, 1, 0) = DD(1, 1, 0) + bd2 * fl * F[0] * DUU[0] * FG[0] * DUR[0] / (V[0] + eps);
    DD(0, 1, 0) = DD(0, 1, 0) - half * grav * bd2 * fl * F[0] * DTU[0] * V[0] / (V[0] + eps);
    DD(1, 1, 0) = DD(1, 1, 0) - half * grav * bd2 * fl * F[0] * V[0] / (V[0] + eps);
    for (int i = 0; i < n1 - 1; ++i) { /* face i+1 (0-based) between cells i and i+1 */
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
    /* last cell, face n1+1 */
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
#undef DD
#undef UU
#undef LL
  }
}

/* Compute_2D of the plane systems (MULTI/TriDiagTB_Mod.f90:260-343, variant 0;
 * MULTI/TriDiagTR_Mod.f90:273-387, variant 1): per plane, line 1's Compute_1D
 * and its Fac2_L terms, then for every face j+1 between lines j and j+1 the
 * couplings u2/l2, line j's share, line j+1's Compute_1D and line j+1's share,
 * finally line n2's Fac2_R terms -- the reference's loops as they stand.
 * s = {beta0*dtp, Fac1_L, Fac1_R, GravComp, FacAnela, Fac2_L, Fac2_R}.
 * Per plane p: z faces f1, f1g, dtu1, duu1 [(p*n2 + j)*(n1+1) + i]; faces
 * between lines f2, f2g, dtu2, duu2 [(p*(n2+1) + j)*n1 + i]; cells vol, dut,
 * dur [(p*n2 + j)*n1 + i].  Out: d [(p*n2 + j)*n1 + i][4] and u1, l1
 * [(p*n2 + j)*(n1-1) + i][4] of the lines; u2, l2 [(p*(n2-1) + j)*n1 + i][4]
 * between lines j and j+1 (TriDiagTB keeps the first block column, entries
 * 2 and 3 are 0). */
void ora_tri_tb_compute_2d(int variant, int nplane, int n2, int n1, const double *s, const double *f1,
                           const double *f1g, const double *dtu1, const double *duu1, const double *f2,
                           const double *f2g, const double *dtu2, const double *duu2, const double *vol,
                           const double *dut, const double *dur, double *d, double *u1, double *l1, double *u2,
                           double *l2) {
  const double bd = s[0], fac2l = s[5], fac2r = s[6];
  const double bd2 = bd * bd, eps = 1.0e-30;
  const int tr = variant == 1;
  for (int p = 0; p < nplane; ++p) {
    const size_t lines = (size_t)p * n2;
    const double *F2 = f2 + (size_t)p * (n2 + 1) * n1, *F2G = f2g + (size_t)p * (n2 + 1) * n1;
    const double *DTU2 = dtu2 + (size_t)p * (n2 + 1) * n1, *DUU2 = duu2 + (size_t)p * (n2 + 1) * n1;
    const double *V = vol + lines * n1, *DUT = dut + lines * n1, *DUR = tr ? dur + lines * n1 : 0;
    double *D = d + lines * n1 * 4;
    double *U2 = u2 + (size_t)p * (n2 - 1) * n1 * 4, *L2 = l2 + (size_t)p * (n2 - 1) * n1 * 4;
#define LINE(j)                                                                                                  \
  ora_tri_tb_compute(variant, 1, n1, s, f1 + (lines + (j)) * (n1 + 1), f1g + (lines + (j)) * (n1 + 1),        \
                     vol + (lines + (j)) * n1, dtu1 + (lines + (j)) * (n1 + 1), duu1 + (lines + (j)) * (n1 + 1), \
                     dut + (lines + (j)) * n1, tr ? dur + (lines + (j)) * n1 : 0, d + (lines + (j)) * n1 * 4,    \
                     u1 + (lines + (j)) * (n1 - 1) * 4, l1 + (lines + (j)) * (n1 - 1) * 4)
#define DD(i, j, e) D[((size_t)(j) * n1 + (i)) * 4 + (e)]
#define CELL(a, i, j) a[(size_t)(j) * n1 + (i)]
#define FACE(a, i, j) a[(size_t)(j) * n1 + (i)]
    LINE(0);
    for (int i = 0; i < n1; ++i) {
      const double a = bd2 * fac2l * FACE(F2, i, 0) * FACE(DTU2, i, 0) * FACE(DUU2, i, 0) * FACE(F2G, i, 0);
      const double b = bd2 * fac2l * FACE(F2, i, 0) * FACE(DUU2, i, 0) * FACE(F2G, i, 0);
      const double den = CELL(V, i, 0) + eps;
      DD(i, 0, 0) = DD(i, 0, 0) + a * CELL(DUT, i, 0) / den;
      if (tr) DD(i, 0, 2) = DD(i, 0, 2) + a * CELL(DUR, i, 0) / den;
      DD(i, 0, 1) = DD(i, 0, 1) + b * CELL(DUT, i, 0) / den;
      if (tr) DD(i, 0, 3) = DD(i, 0, 3) + b * CELL(DUR, i, 0) / den;
    }
    for (int j = 0; j < n2 - 1; ++j) {
      const int q = j + 1;
      for (int i = 0; i < n1; ++i) {
        const double S = CELL(V, i, j) + CELL(V, i, q) + eps;
        const double a = bd2 * 2.0 * FACE(F2, i, q) * FACE(DTU2, i, q) * FACE(DUU2, i, q) * FACE(F2G, i, q);
        const double b = bd2 * 2.0 * FACE(F2, i, q) * FACE(DUU2, i, q) * FACE(F2G, i, q);
        double *u = U2 + ((size_t)j * n1 + i) * 4, *l = L2 + ((size_t)j * n1 + i) * 4;
        u[0] = -(a * CELL(DUT, i, q) / S);
        u[2] = tr ? -(a * CELL(DUR, i, q) / S) : 0.0;
        u[1] = -(b * CELL(DUT, i, q) / S);
        u[3] = tr ? -(b * CELL(DUR, i, q) / S) : 0.0;
        l[0] = -(a * CELL(DUT, i, j) / S);
        l[2] = tr ? -(a * CELL(DUR, i, j) / S) : 0.0;
        l[1] = -(b * CELL(DUT, i, j) / S);
        l[3] = tr ? -(b * CELL(DUR, i, j) / S) : 0.0;
        DD(i, j, 0) = DD(i, j, 0) + a * CELL(DUT, i, j) / S;
        if (tr) DD(i, j, 2) = DD(i, j, 2) + a * CELL(DUR, i, j) / S;
        DD(i, j, 1) = DD(i, j, 1) + b * CELL(DUT, i, j) / S;
        if (tr) DD(i, j, 3) = DD(i, j, 3) + b * CELL(DUR, i, j) / S;
      }
      LINE(q);
      for (int i = 0; i < n1; ++i) {
        const double S = CELL(V, i, j) + CELL(V, i, q) + eps;
        const double a = bd2 * 2.0 * FACE(F2, i, q) * FACE(DTU2, i, q) * FACE(DUU2, i, q) * FACE(F2G, i, q);
        const double b = bd2 * 2.0 * FACE(F2, i, q) * FACE(DUU2, i, q) * FACE(F2G, i, q);
        DD(i, q, 0) = DD(i, q, 0) + a * CELL(DUT, i, q) / S;
        if (tr) DD(i, q, 2) = DD(i, q, 2) + a * CELL(DUR, i, q) / S;
        DD(i, q, 1) = DD(i, q, 1) + b * CELL(DUT, i, q) / S;
        if (tr) DD(i, q, 3) = DD(i, q, 3) + b * CELL(DUR, i, q) / S;
      }
    }
    for (int i = 0; i < n1; ++i) {
      const int j = n2 - 1, q = n2;
      const double a = bd2 * fac2r * FACE(F2, i, q) * FACE(DTU2, i, q) * FACE(DUU2, i, q) * FACE(F2G, i, q);
      const double b = bd2 * fac2r * FACE(F2, i, q) * FACE(DUU2, i, q) * FACE(F2G, i, q);
      const double den = CELL(V, i, j) + eps;
      DD(i, j, 0) = DD(i, j, 0) + a * CELL(DUT, i, j) / den;
      if (tr) DD(i, j, 2) = DD(i, j, 2) + a * CELL(DUR, i, j) / den;
      DD(i, j, 1) = DD(i, j, 1) + b * CELL(DUT, i, j) / den;
      if (tr) DD(i, j, 3) = DD(i, j, 3) + b * CELL(DUR, i, j) / den;
    }
#undef LINE
#undef DD
#undef CELL
#undef FACE
  }
}

/* Compute_3D (MULTI/TriDiagTB_Mod.f90:663-780, variant 0; TriDiagTR_Mod.f90:707-864,
 * variant 1) of one 3D level, the reference's loops as they stand: plane 1's
 * Compute_2D and Fac3_L terms, then per face k+1 between planes k and k+1 the
 * couplings, plane k's share, plane k+1's Compute_2D and its share, finally
 * the last plane's Fac3_R terms.  couple = 1: the branch with the couplings
 * between planes stored, whose interior and Fac3_R terms have no DUU3;
 * couple = 0: the branch without them, every face term with DUU3.
 * s = {beta0*dtp, Fac1_L, Fac1_R, GravComp, FacAnela, Fac2_L, Fac2_R, Fac3_L,
 * Fac3_R}; faces between planes f3.. [(k*n2 + j)*n1 + i], k = 0..n3; the rest
 * as ora_tri_tb_compute_2d with p = k; u3, l3 [(k*n2 + j)*n1 + i][4]. */
void ora_tri_tb_compute_3d(int variant, int couple, int n3, int n2, int n1, const double *s, const double *f1,
                           const double *f1g, const double *dtu1, const double *duu1, const double *f2,
                           const double *f2g, const double *dtu2, const double *duu2, const double *f3,
                           const double *f3g, const double *dtu3, const double *duu3, const double *vol,
                           const double *dut, const double *dur, double *d, double *u1, double *l1, double *u2,
                           double *l2, double *u3, double *l3) {
  const double bd = s[0], fac3l = s[7], fac3r = s[8];
  const double bd2 = bd * bd, eps = 1.0e-30;
  const int tr = variant == 1;
  const size_t npl = (size_t)n2 * n1;
#define PLANE(k)                                                                                                   \
  ora_tri_tb_compute_2d(variant, 1, n2, n1, s, f1 + (size_t)(k)*n2 * (n1 + 1), f1g + (size_t)(k)*n2 * (n1 + 1),    \
                        dtu1 + (size_t)(k)*n2 * (n1 + 1), duu1 + (size_t)(k)*n2 * (n1 + 1),                          \
                        f2 + (size_t)(k) * (n2 + 1) * n1, f2g + (size_t)(k) * (n2 + 1) * n1,                         \
                        dtu2 + (size_t)(k) * (n2 + 1) * n1, duu2 + (size_t)(k) * (n2 + 1) * n1, vol + (k)*npl,       \
                        dut + (k)*npl, tr ? dur + (k)*npl : 0, d + (k)*npl * 4, u1 + (size_t)(k)*n2 * (n1 - 1) * 4, \
                        l1 + (size_t)(k)*n2 * (n1 - 1) * 4, u2 + (size_t)(k) * (n2 - 1) * n1 * 4,                    \
                        l2 + (size_t)(k) * (n2 - 1) * n1 * 4)
#define C3(a, r, k) a[(size_t)(k)*npl + (r)]
#define D3(r, k, e) d[((size_t)(k)*npl + (r)) * 4 + (e)]
  PLANE(0);
  for (size_t r = 0; r < npl; ++r) {
    const double a = bd2 * fac3l * C3(f3, r, 0) * C3(dtu3, r, 0) * C3(duu3, r, 0) * C3(f3g, r, 0);
    const double b = bd2 * fac3l * C3(f3, r, 0) * C3(duu3, r, 0) * C3(f3g, r, 0);
    const double den = C3(vol, r, 0) + eps;
    D3(r, 0, 0) = D3(r, 0, 0) + a * C3(dut, r, 0) / den;
    if (tr) D3(r, 0, 2) = D3(r, 0, 2) + a * C3(dur, r, 0) / den;
    D3(r, 0, 1) = D3(r, 0, 1) + b * C3(dut, r, 0) / den;
    if (tr) D3(r, 0, 3) = D3(r, 0, 3) + b * C3(dur, r, 0) / den;
  }
  for (int k = 0; k < n3 - 1; ++k) {
    const int q = k + 1;
    for (size_t r = 0; r < npl; ++r) {
      const double S = C3(vol, r, k) + C3(vol, r, q) + eps;
      const double a = couple ? bd2 * 2.0 * C3(f3, r, q) * C3(dtu3, r, q) * C3(f3g, r, q)
                              : bd2 * 2.0 * C3(f3, r, q) * C3(dtu3, r, q) * C3(duu3, r, q) * C3(f3g, r, q);
      const double b = couple ? bd2 * 2.0 * C3(f3, r, q) * C3(f3g, r, q)
                              : bd2 * 2.0 * C3(f3, r, q) * C3(duu3, r, q) * C3(f3g, r, q);
      if (couple) {
        double *u = u3 + ((size_t)k * npl + r) * 4, *l = l3 + ((size_t)k * npl + r) * 4;
        u[0] = -(a * C3(dut, r, q) / S);
        u[2] = tr ? -(a * C3(dur, r, q) / S) : 0.0;
        u[1] = -(b * C3(dut, r, q) / S);
        u[3] = tr ? -(b * C3(dur, r, q) / S) : 0.0;
        l[0] = -(a * C3(dut, r, k) / S);
        l[2] = tr ? -(a * C3(dur, r, k) / S) : 0.0;
        l[1] = -(b * C3(dut, r, k) / S);
        l[3] = tr ? -(b * C3(dur, r, k) / S) : 0.0;
      }
      D3(r, k, 0) = D3(r, k, 0) + a * C3(dut, r, k) / S;
      if (tr) D3(r, k, 2) = D3(r, k, 2) + a * C3(dur, r, k) / S;
      D3(r, k, 1) = D3(r, k, 1) + b * C3(dut, r, k) / S;
      if (tr) D3(r, k, 3) = D3(r, k, 3) + b * C3(dur, r, k) / S;
    }
    PLANE(q);
    for (size_t r = 0; r < npl; ++r) {
      const double S = C3(vol, r, k) + C3(vol, r, q) + eps;
      const double a = couple ? bd2 * 2.0 * C3(f3, r, q) * C3(dtu3, r, q) * C3(f3g, r, q)
                              : bd2 * 2.0 * C3(f3, r, q) * C3(dtu3, r, q) * C3(duu3, r, q) * C3(f3g, r, q);
      const double b = couple ? bd2 * 2.0 * C3(f3, r, q) * C3(f3g, r, q)
                              : bd2 * 2.0 * C3(f3, r, q) * C3(duu3, r, q) * C3(f3g, r, q);
      D3(r, q, 0) = D3(r, q, 0) + a * C3(dut, r, q) / S;
      if (tr) D3(r, q, 2) = D3(r, q, 2) + a * C3(dur, r, q) / S;
      D3(r, q, 1) = D3(r, q, 1) + b * C3(dut, r, q) / S;
      if (tr) D3(r, q, 3) = D3(r, q, 3) + b * C3(dur, r, q) / S;
    }
  }
  for (size_t r = 0; r < npl; ++r) {
    const int k = n3 - 1, q = n3;
    const double a = couple ? bd2 * fac3r * C3(f3, r, q) * C3(dtu3, r, q) * C3(f3g, r, q)
                            : bd2 * fac3r * C3(f3, r, q) * C3(dtu3, r, q) * C3(duu3, r, q) * C3(f3g, r, q);
    const double b = couple ? bd2 * fac3r * C3(f3, r, q) * C3(f3g, r, q)
                            : bd2 * fac3r * C3(f3, r, q) * C3(duu3, r, q) * C3(f3g, r, q);
    const double den = C3(vol, r, k) + eps;
    D3(r, k, 0) = D3(r, k, 0) + a * C3(dut, r, k) / den;
    if (tr) D3(r, k, 2) = D3(r, k, 2) + a * C3(dur, r, k) / den;
    D3(r, k, 1) = D3(r, k, 1) + b * C3(dut, r, k) / den;
    if (tr) D3(r, k, 3) = D3(r, k, 3) + b * C3(dur, r, k) / den;
  }
#undef PLANE
#undef C3
#undef D3
}

/* MatVecTB_2D / MatVecTR_2D (MULTI/TriDiagTB_Mod.f90:345-372, TriDiagTR_Mod.f90:389-416)
 * of one plane, as the reference loops: line 1's product and its coupling to
 * line 2, each inner line's product, + l x(j-1), + u x(j+1), the last line's
 * product and + l x(n2-1).  TriDiagTB's couplings are vectors times the
 * neighbour's first component, TriDiagTR's 2x2 blocks (Mult_2). */
static void couple_add(int tr, const double *c, const double *x, double *y) {
  double v[2];
  if (tr) {
    mult_2(c, x, v);
  } else {
    v[0] = c[0] * x[0];
    v[1] = c[1] * x[0];
  }
  y[0] = y[0] + v[0];
  y[1] = y[1] + v[1];
}
static void matvec_2d(int tr, int n2, int n1, const double *d, const double *u1, const double *l1, const double *u2,
                      const double *l2, const double *x, double *y) {
#define LINEMV(j)                                                                                               \
  ora_tri_tb_matvec(1, n1, d + (size_t)(j)*n1 * 4, u1 + (size_t)(j) * (n1 - 1) * 4,                            \
                    l1 + (size_t)(j) * (n1 - 1) * 4, x + (size_t)(j)*n1 * 2, y + (size_t)(j)*n1 * 2)
#define XY(a, i, j) (a + ((size_t)(j)*n1 + (i)) * 2)
#define CP(a, i, j) (a + ((size_t)(j)*n1 + (i)) * 4)
  LINEMV(0);
  if (n2 > 1) {
    for (int i = 0; i < n1; ++i) couple_add(tr, CP(u2, i, 0), XY(x, i, 1), XY(y, i, 0));
    for (int j = 1; j < n2 - 1; ++j) {
      LINEMV(j);
      for (int i = 0; i < n1; ++i) {
        couple_add(tr, CP(l2, i, j - 1), XY(x, i, j - 1), XY(y, i, j));
        couple_add(tr, CP(u2, i, j), XY(x, i, j + 1), XY(y, i, j));
      }
    }
    LINEMV(n2 - 1);
    for (int i = 0; i < n1; ++i) couple_add(tr, CP(l2, i, n2 - 2), XY(x, i, n2 - 2), XY(y, i, n2 - 1));
  }
#undef LINEMV
#undef XY
#undef CP
}

/* MatVecTB_3D / MatVecTR_3D (TriDiagTB_Mod.f90:782-816, TriDiagTR_Mod.f90:866-900):
 * the same over planes with the couplings u3, l3. */
void ora_tri_tb_matvec_3d(int variant, int n3, int n2, int n1, const double *d, const double *u1, const double *l1,
                          const double *u2, const double *l2, const double *u3, const double *l3, const double *x,
                          double *y) {
  const int tr = variant == 1;
  const size_t npl = (size_t)n2 * n1;
#define PLANEMV(k)                                                                                               \
  matvec_2d(tr, n2, n1, d + (size_t)(k)*npl * 4, u1 + (size_t)(k)*n2 * (n1 - 1) * 4,                           \
            l1 + (size_t)(k)*n2 * (n1 - 1) * 4, u2 + (size_t)(k) * (n2 - 1) * n1 * 4,                          \
            l2 + (size_t)(k) * (n2 - 1) * n1 * 4, x + (size_t)(k)*npl * 2, y + (size_t)(k)*npl * 2)
#define X3(a, r, k) (a + ((size_t)(k)*npl + (r)) * 2)
#define C3(a, r, k) (a + ((size_t)(k)*npl + (r)) * 4)
  PLANEMV(0);
  if (n3 > 1) {
    for (size_t r = 0; r < npl; ++r) couple_add(tr, C3(u3, r, 0), X3(x, r, 1), X3(y, r, 0));
    for (int k = 1; k < n3 - 1; ++k) {
      PLANEMV(k);
      for (size_t r = 0; r < npl; ++r) {
        couple_add(tr, C3(l3, r, k - 1), X3(x, r, k - 1), X3(y, r, k));
        couple_add(tr, C3(u3, r, k), X3(x, r, k + 1), X3(y, r, k));
      }
    }
    PLANEMV(n3 - 1);
    for (size_t r = 0; r < npl; ++r) couple_add(tr, C3(l3, r, n3 - 2), X3(x, r, n3 - 2), X3(y, r, n3 - 1));
  }
#undef PLANEMV
#undef X3
#undef C3
}

/* GaussSeidel_2D (MULTI/TriDiagTB_Mod.f90:374-418, TriDiagTR_Mod.f90:418-462) on
 * nplane planes: the symmetric line sweep of the reference -- per iteration
 * lines 1..n2-1 forward, then n2..2 backward, each line's right-hand side
 * minus its couplings to the neighbour lines and a Solve_1D -- and line 1
 * once more after the iterations.  x holds the initial guess and is
 * overwritten; gauss_iter >= 1 when n2 > 1 (the reference reads t
 * unset otherwise). */
static void couple_sub(int tr, const double *t, const double *c, const double *x, double *o) {
  double v[2];
  if (tr) {
    mult_2(c, x, v);
  } else {
    v[0] = c[0] * x[0];
    v[1] = c[1] * x[0];
  }
  o[0] = t[0] - v[0];
  o[1] = t[1] - v[1];
}
/* Zebra order of the plane and level smoothers (the GPU's parallel order, not
 * the reference's): per Gauss-Seidel iteration the lines (planes) of parity
 * 0 with the forward right-hand side (b - l x(j-1)) - u x(j+1), parity 1
 * forward, parity 1 backward ((b - u x(j+1)) - l x(j-1)), parity 0
 * backward; then the reference's closing solves (line 1; planes 1 and n3)
 * with its right-hand sides.  Every single relaxation is the reference's
 * arithmetic, only the order of the lines (planes) differs. */
static int g_tb_zebra = 0;
void ora_tri_tb_set_zebra(int on) { g_tb_zebra = on != 0; }

static void gs2d_zebra(int tr, int nplane, int n2, int n1, const double *d, const double *u1, const double *l1,
                       const double *u2, const double *l2, const double *b, double *x, int gauss_iter, double *w) {
  for (int p = 0; p < nplane; ++p) {
    const size_t L0 = (size_t)p * n2;
#define XL(j) (x + (L0 + (j)) * n1 * 2)
#define BL(j) (b + (L0 + (j)) * n1 * 2)
#define C2(a, i, j) (a + (((size_t)p * (n2 - 1) + (j)) * n1 + (i)) * 4)
#define SOLVE(j)                                                                                                \
  ora_tri_tb_solve(1, n1, d + (L0 + (j)) * n1 * 4, u1 + (L0 + (j)) * (n1 - 1) * 4, l1 + (L0 + (j)) * (n1 - 1) * 4, \
                   XL(j), w)
    if (n2 > 1) {
      for (int it = 0; it < gauss_iter; ++it)
        for (int half = 0; half < 4; ++half) {
          const int par = half == 1 || half == 2, bwd = half >= 2;
          for (int j = par; j < n2; j += 2) {
            for (int i = 0; i < n1; ++i) {
              double *o = XL(j) + 2 * i;
              o[0] = BL(j)[2 * i];
              o[1] = BL(j)[2 * i + 1];
              if (!bwd) {
                if (j > 0) couple_sub(tr, o, C2(l2, i, j - 1), XL(j - 1) + 2 * i, o);
                if (j < n2 - 1) couple_sub(tr, o, C2(u2, i, j), XL(j + 1) + 2 * i, o);
              } else {
                if (j < n2 - 1) couple_sub(tr, o, C2(u2, i, j), XL(j + 1) + 2 * i, o);
                if (j > 0) couple_sub(tr, o, C2(l2, i, j - 1), XL(j - 1) + 2 * i, o);
              }
            }
            SOLVE(j);
          }
        }
      for (int i = 0; i < n1; ++i) couple_sub(tr, BL(0) + 2 * i, C2(u2, i, 0), XL(1) + 2 * i, XL(0) + 2 * i);
      SOLVE(0);
    } else {
      memcpy(XL(0), BL(0), sizeof(double) * 2 * (size_t)n1);
      SOLVE(0);
    }
#undef XL
#undef BL
#undef C2
#undef SOLVE
  }
}

void ora_tri_tb_gauss_seidel_2d(int variant, int nplane, int n2, int n1, const double *d, const double *u1,
                                const double *l1, const double *u2, const double *l2, const double *b, double *x,
                                int gauss_iter) {
  const int tr = variant == 1;
  double *t = (double *)malloc(sizeof(double) * 2 * (size_t)n1);
  double *w = (double *)malloc(sizeof(double) * 4 * (size_t)(n1 > 1 ? n1 - 1 : 1));
  if (g_tb_zebra) {
    gs2d_zebra(tr, nplane, n2, n1, d, u1, l1, u2, l2, b, x, gauss_iter, w);
    free(t);
    free(w);
    return;
  }
  for (int p = 0; p < nplane; ++p) {
    const size_t L0 = (size_t)p * n2;
#define XL(j) (x + (L0 + (j)) * n1 * 2)
#define BL(j) (b + (L0 + (j)) * n1 * 2)
#define C2(a, i, j) (a + (((size_t)p * (n2 - 1) + (j)) * n1 + (i)) * 4)
#define SOLVE(j)                                                                                                \
  ora_tri_tb_solve(1, n1, d + (L0 + (j)) * n1 * 4, u1 + (L0 + (j)) * (n1 - 1) * 4, l1 + (L0 + (j)) * (n1 - 1) * 4, \
                   XL(j), w)
    if (n2 > 1) {
      for (int it = 0; it < gauss_iter; ++it) {
        memcpy(t, BL(0), sizeof(double) * 2 * (size_t)n1);
        for (int j = 0; j < n2 - 1; ++j) {
          for (int i = 0; i < n1; ++i) couple_sub(tr, t + 2 * i, C2(u2, i, j), XL(j + 1) + 2 * i, XL(j) + 2 * i);
          SOLVE(j);
          for (int i = 0; i < n1; ++i) couple_sub(tr, BL(j + 1) + 2 * i, C2(l2, i, j), XL(j) + 2 * i, t + 2 * i);
        }
        memcpy(XL(n2 - 1), t, sizeof(double) * 2 * (size_t)n1);
        SOLVE(n2 - 1);
        for (int i = 0; i < n1; ++i)
          couple_sub(tr, BL(n2 - 2) + 2 * i, C2(u2, i, n2 - 2), XL(n2 - 1) + 2 * i, t + 2 * i);
        for (int j = n2 - 2; j >= 1; --j) {
          for (int i = 0; i < n1; ++i) couple_sub(tr, t + 2 * i, C2(l2, i, j - 1), XL(j - 1) + 2 * i, XL(j) + 2 * i);
          SOLVE(j);
          for (int i = 0; i < n1; ++i) couple_sub(tr, BL(j - 1) + 2 * i, C2(u2, i, j - 1), XL(j) + 2 * i, t + 2 * i);
        }
      }
      memcpy(XL(0), t, sizeof(double) * 2 * (size_t)n1);
      SOLVE(0);
    } else {
      memcpy(XL(0), BL(0), sizeof(double) * 2 * (size_t)n1);
      SOLVE(0);
    }
#undef XL
#undef BL
#undef C2
#undef SOLVE
  }
  free(t);
  free(w);
}

/* RestrictTB_2D / RestrictTR_2D (TriDiagTB_Mod.f90:495-525): the coarse residual of
 * a plane of n2 x n1 fine entries, (n2+1)/2 x (n1+1)/2, sums of 2x2 fine cells
 * in the reference's order (an odd last row or line on its own). */
void ora_tri_tb_restrict_2d(int nplane, int n2, int n1, const double *res, double *resc) {
  const int n1c = (n1 + 1) / 2, n2c = (n2 + 1) / 2;
  for (int p = 0; p < nplane; ++p) {
    const double *R = res + (size_t)p * n2 * n1 * 2;
    double *C = resc + (size_t)p * n2c * n1c * 2;
#define RF(i, j, r) R[((size_t)(j)*n1 + (i)) * 2 + (r)]
#define RC(i, j, r) C[((size_t)(j)*n1c + (i)) * 2 + (r)]
    for (int r = 0; r < 2; ++r) RC(n1c - 1, n2c - 1, r) = RF(n1 - 1, n2 - 1, r);
    for (int ic = 0; ic < n1 / 2; ++ic)
      for (int r = 0; r < 2; ++r) RC(ic, n2c - 1, r) = RF(2 * ic, n2 - 1, r) + RF(2 * ic + 1, n2 - 1, r);
    for (int jc = 0; jc < n2 / 2; ++jc) {
      const int jf = 2 * jc;
      for (int r = 0; r < 2; ++r) RC(n1c - 1, jc, r) = RF(n1 - 1, jf, r) + RF(n1 - 1, jf + 1, r);
      for (int ic = 0; ic < n1 / 2; ++ic) {
        const int i = 2 * ic;
        for (int r = 0; r < 2; ++r)
          RC(ic, jc, r) = RF(i, jf, r) + RF(i + 1, jf, r) + RF(i, jf + 1, r) + RF(i + 1, jf + 1, r);
      }
    }
#undef RF
#undef RC
  }
}

/* ProlongateTB_2D / ProlongateTR_2D (TriDiagTB_Mod.f90:527-560): every fine entry
 * takes the value of its coarse cell. */
void ora_tri_tb_prolong_2d(int nplane, int n2, int n1, const double *xc, double *x) {
  const int n1c = (n1 + 1) / 2, n2c = (n2 + 1) / 2;
  for (int p = 0; p < nplane; ++p)
    for (int j = 0; j < n2; ++j)
      for (int i = 0; i < n1; ++i)
        for (int r = 0; r < 2; ++r)
          x[(((size_t)p * n2 + j) * n1 + i) * 2 + r] = xc[(((size_t)p * n2c + j / 2) * n1c + i / 2) * 2 + r];
}

/* Multigrid_2D (MULTI/TriDiagTB_Mod.f90:433-494, TriDiagTR_Mod.f90:477-538) repeated
 * mult_iter times (Solve_2D, :419-431) on nplane planes whose hierarchy of
 * nlev levels the caller assembled (level l: n2s[l] lines of n1s[l] levels,
 * blocks d[l], u1[l], l1[l], u2[l], l2[l] as ora_tri_tb_compute_2d writes
 * them; level l+1 has ((n2s[l]+1)/2, (n1s[l]+1)/2)).  Down: GaussSeidel_2D
 * with GaussIter 1, 1+GaussIter2, ..., the residual b - A x, its
 * restriction, a zero coarse guess; up: GaussSeidel_2D again (the coarsest
 * a second time with its count), the prolongation added to the finer guess. */
static void matvec_planes(int variant, int nplane, int n2, int n1, const double *d, const double *u1,
                          const double *l1, const double *u2, const double *l2, const double *x, double *y) {
  for (int p = 0; p < nplane; ++p) {
    const size_t L = (size_t)p * n2;
    ora_tri_tb_matvec_3d(variant, 1, n2, n1, d + L * n1 * 4, u1 + L * (n1 - 1) * 4, l1 + L * (n1 - 1) * 4,
                         u2 + (size_t)p * (n2 - 1) * n1 * 4, l2 + (size_t)p * (n2 - 1) * n1 * 4, 0, 0,
                         x + L * n1 * 2, y + L * n1 * 2);
  }
}
void ora_tri_tb_multigrid_2d(int variant, int nplane, int nlev, const int *n2s, const int *n1s,
                             const double *const *d, const double *const *u1, const double *const *l1,
                             const double *const *u2, const double *const *l2, const double *b, double *x,
                             int gauss_iter2, int mult_iter) {
  double *bl[32], *xl[32], *res[32];
  for (int l = 0; l < nlev; ++l) {
    const size_t n = (size_t)nplane * n2s[l] * n1s[l] * 2;
    res[l] = (double *)malloc(sizeof(double) * n);
    bl[l] = l ? (double *)malloc(sizeof(double) * n) : (double *)b;
    xl[l] = l ? (double *)malloc(sizeof(double) * n) : x;
  }
#define LV(l) variant, nplane, n2s[l], n1s[l], d[l], u1[l], l1[l], u2[l], l2[l]
  for (int it = 0; it < mult_iter; ++it) {
    int gi = 1, l = 0;
    for (;;) {
      ora_tri_tb_gauss_seidel_2d(LV(l), bl[l], xl[l], gi);
      gi += gauss_iter2;
      if (l + 1 < nlev) {
        const size_t n = (size_t)nplane * n2s[l] * n1s[l] * 2;
        matvec_planes(LV(l), xl[l], res[l]);
        for (size_t q = 0; q < n; ++q) res[l][q] = bl[l][q] - res[l][q];
        ora_tri_tb_restrict_2d(nplane, n2s[l], n1s[l], res[l], bl[l + 1]);
        memset(xl[l + 1], 0, sizeof(double) * (size_t)nplane * n2s[l + 1] * n1s[l + 1] * 2);
        ++l;
      } else {
        gi -= gauss_iter2;
        break;
      }
    }
    for (;;) {
      ora_tri_tb_gauss_seidel_2d(LV(l), bl[l], xl[l], gi);
      gi -= gauss_iter2;
      if (l == 0) break;
      --l;
      const size_t n = (size_t)nplane * n2s[l] * n1s[l] * 2;
      ora_tri_tb_prolong_2d(nplane, n2s[l], n1s[l], xl[l + 1], res[l]);
      for (size_t q = 0; q < n; ++q) xl[l][q] = xl[l][q] + res[l][q];
    }
  }
#undef LV
  for (int l = 0; l < nlev; ++l) {
    free(res[l]);
    if (l) {
      free(bl[l]);
      free(xl[l]);
    }
  }
}

/* The plane solve Solve(A%d(k)%P, t, x(:,:,:,k)) of GaussSeidel_3D: Solve_2D on
 * plane k of a level whose planes carry nlev2 plane levels (the 2D level m
 * of all n3 planes at d[m] .. l2[m], n2 x n1 halved m times). */
static void solve_plane(int variant, int k, int nlev2, const int *n2s, const int *n1s, const double *const *d,
                        const double *const *u1, const double *const *l1, const double *const *u2,
                        const double *const *l2, const double *t, double *x, int gauss_iter2, int mult_iter2) {
  const double *pd[32], *pu1[32], *pl1[32], *pu2[32], *pl2[32];
  for (int m = 0; m < nlev2; ++m) {
    const size_t n2 = (size_t)n2s[m], n1 = (size_t)n1s[m];
    pd[m] = d[m] + k * n2 * n1 * 4;
    pu1[m] = u1[m] + k * n2 * (n1 - 1) * 4;
    pl1[m] = l1[m] + k * n2 * (n1 - 1) * 4;
    pu2[m] = u2[m] + k * (n2 - 1) * n1 * 4;
    pl2[m] = l2[m] + k * (n2 - 1) * n1 * 4;
  }
  ora_tri_tb_multigrid_2d(variant, 1, nlev2, n2s, n1s, pd, pu1, pl1, pu2, pl2, t, x, gauss_iter2, mult_iter2);
}

/* GaussSeidel_3D (MULTI/TriDiagTB_Mod.f90:818-874, TriDiagTR_Mod.f90:902-961) of
 * one level of n3 planes: per iteration the planes 1..n3-1 forward and n3..2
 * backward, each plane's right-hand side minus its couplings to the planes
 * either side (u3, l3 as ora_tri_tb_compute_3d writes them), each plane
 * solved by Solve_2D from the current guess; then plane 1 and, additionally,
 * plane n3 once more.  n2s, n1s: the plane levels' sizes, n2s[0] = n2. */
void ora_tri_tb_gauss_seidel_3d(int variant, int n3, int nlev2, const int *n2s, const int *n1s,
                                const double *const *d, const double *const *u1, const double *const *l1,
                                const double *const *u2, const double *const *l2, const double *u3, const double *l3,
                                const double *b, double *x, int gauss_iter, int gauss_iter2, int mult_iter2) {
  const int tr = variant == 1;
  const size_t npl = (size_t)n2s[0] * n1s[0];
  double *t = (double *)malloc(sizeof(double) * npl * 2);
#define SOLVE(k, rhs) \
  solve_plane(variant, k, nlev2, n2s, n1s, d, u1, l1, u2, l2, rhs, x + (size_t)(k)*npl * 2, gauss_iter2, mult_iter2)
#define XP(a, r, k) (a + ((size_t)(k)*npl + (r)) * 2)
#define CP(a, r, k) (a + ((size_t)(k)*npl + (r)) * 4)
  if (n3 > 1 && g_tb_zebra) {
    for (int it = 0; it < gauss_iter; ++it)
      for (int half = 0; half < 4; ++half) {
        const int par = half == 1 || half == 2, bwd = half >= 2;
        for (int k = par; k < n3; k += 2) {
          for (size_t r = 0; r < npl; ++r) {
            double *o = t + r * 2;
            o[0] = XP(b, r, k)[0];
            o[1] = XP(b, r, k)[1];
            if (!bwd) {
              if (k > 0) couple_sub(tr, o, CP(l3, r, k - 1), XP(x, r, k - 1), o);
              if (k < n3 - 1) couple_sub(tr, o, CP(u3, r, k), XP(x, r, k + 1), o);
            } else {
              if (k < n3 - 1) couple_sub(tr, o, CP(u3, r, k), XP(x, r, k + 1), o);
              if (k > 0) couple_sub(tr, o, CP(l3, r, k - 1), XP(x, r, k - 1), o);
            }
          }
          SOLVE(k, t);
        }
      }
    for (size_t r = 0; r < npl; ++r) couple_sub(tr, XP(b, r, 0), CP(u3, r, 0), XP(x, r, 1), t + r * 2);
    SOLVE(0, t);
    for (size_t r = 0; r < npl; ++r) couple_sub(tr, XP(b, r, n3 - 1), CP(l3, r, n3 - 2), XP(x, r, n3 - 2), t + r * 2);
    SOLVE(n3 - 1, t);
  } else if (n3 > 1) {
    for (int it = 0; it < gauss_iter; ++it) {
      memcpy(t, b, sizeof(double) * npl * 2);
      for (int k = 0; k < n3 - 1; ++k) {
        for (size_t r = 0; r < npl; ++r) couple_sub(tr, t + r * 2, CP(u3, r, k), XP(x, r, k + 1), t + r * 2);
        SOLVE(k, t);
        for (size_t r = 0; r < npl; ++r) {
          couple_sub(tr, XP(b, r, k + 1), CP(l3, r, k), XP(x, r, k), t + r * 2);
        }
      }
      SOLVE(n3 - 1, t);
      for (size_t r = 0; r < npl; ++r) {
        couple_sub(tr, XP(b, r, n3 - 2), CP(u3, r, n3 - 2), XP(x, r, n3 - 1), t + r * 2);
      }
      for (int k = n3 - 2; k >= 1; --k) {
        for (size_t r = 0; r < npl; ++r) couple_sub(tr, t + r * 2, CP(l3, r, k - 1), XP(x, r, k - 1), t + r * 2);
        SOLVE(k, t);
        for (size_t r = 0; r < npl; ++r) {
          couple_sub(tr, XP(b, r, k - 1), CP(u3, r, k - 1), XP(x, r, k), t + r * 2);
        }
      }
    }
    SOLVE(0, t);
    for (size_t r = 0; r < npl; ++r) {
      couple_sub(tr, XP(b, r, n3 - 1), CP(l3, r, n3 - 2), XP(x, r, n3 - 2), t + r * 2);
    }
    SOLVE(n3 - 1, t);
  } else {
    SOLVE(0, b);
  }
#undef SOLVE
#undef XP
#undef CP
  free(t);
}

/* RestrictTB_3D (MULTI/TriDiagTB_Mod.f90:954-1026): the value the reference's
 * overwriting loops leave in each coarse entry -- its fine cells summed along
 * the axes where it has two (the last cell of an odd axis alone), in the
 * order (i,j,k), (i+1,j,k), (i,j+1,k), (i,j,k+1), (i+1,j+1,k), (i+1,j,k+1),
 * (i,j+1,k+1), (i+1,j+1,k+1) of the cells that exist; with two paired axes
 * a, b: (a,b), (a+1,b), (a,b+1), (a+1,b+1). */
void ora_tri_tb_restrict_3d(int n3, int n2, int n1, const double *res, double *resc) {
  const int n1c = (n1 + 1) / 2, n2c = (n2 + 1) / 2, n3c = (n3 + 1) / 2;
  static const int ord[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1},
                                {1, 1, 0}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};
  for (int kc = 0; kc < n3c; ++kc)
    for (int jc = 0; jc < n2c; ++jc)
      for (int ic = 0; ic < n1c; ++ic) {
        const int pi = ic < n1 / 2, pj = jc < n2 / 2, pk = kc < n3 / 2;
        const int i0 = pi ? 2 * ic : n1 - 1, j0 = pj ? 2 * jc : n2 - 1, k0 = pk ? 2 * kc : n3 - 1;
        double s0 = 0.0, s1 = 0.0;
        int first = 1;
        for (int q = 0; q < 8; ++q) {
          if ((ord[q][0] && !pi) || (ord[q][1] && !pj) || (ord[q][2] && !pk)) continue;
          const double *v = res + ((((size_t)(k0 + ord[q][2]) * n2 + j0 + ord[q][1]) * n1) + i0 + ord[q][0]) * 2;
          if (first) {
            s0 = v[0];
            s1 = v[1];
            first = 0;
          } else {
            s0 = s0 + v[0];
            s1 = s1 + v[1];
          }
        }
        double *o = resc + (((size_t)kc * n2c + jc) * n1c + ic) * 2;
        o[0] = s0;
        o[1] = s1;
      }
}

/* ProlongateTB_3D (MULTI/TriDiagTB_Mod.f90:1028-1100): each fine entry its
 * coarse cell's value. */
void ora_tri_tb_prolong_3d(int n3, int n2, int n1, const double *xc, double *x) {
  const int n1c = (n1 + 1) / 2, n2c = (n2 + 1) / 2;
  for (int k = 0; k < n3; ++k)
    for (int j = 0; j < n2; ++j)
      for (int i = 0; i < n1; ++i) {
        const double *c = xc + (((size_t)(k / 2) * n2c + j / 2) * n1c + i / 2) * 2;
        double *o = x + (((size_t)k * n2 + j) * n1 + i) * 2;
        o[0] = c[0];
        o[1] = c[1];
      }
}

/* Solve_3D (MULTI/TriDiagTB_Mod.f90:940-952, TriDiagTR_Mod.f90:1028-1041):
 * mult_iter3 V-cycles of Multigrid_3D (TriDiagTB_Mod.f90:876-938) over nlev3
 * levels, level L of n3s[L] planes of n2s[L] x n1s[L] (each halved, rounding
 * up, on the next level), its couplings between planes u3[L], l3[L] and its
 * planes' nlev2s[L] plane levels at d[o + m] .. l2[o + m], o = the sum of
 * nlev2s[0..L-1].  Down: GaussSeidel_3D with GaussIter 1, raised by
 * gauss_iter3 per level, the residual b - A x restricted, a zero coarse
 * guess; up: GaussSeidel_3D again, the prolonged guess added.  Each plane
 * solve is Solve_2D with gauss_iter2, mult_iter2. */
void ora_tri_tb_multigrid_3d(int variant, int nlev3, const int *n3s, const int *n2s, const int *n1s, const int *nlev2s,
                             const double *const *u3, const double *const *l3, const double *const *d,
                             const double *const *u1, const double *const *l1, const double *const *u2,
                             const double *const *l2, const double *b, double *x, int gauss_iter2, int mult_iter2,
                             int gauss_iter3, int mult_iter3) {
  double *bl[32], *xl[32], *res[32];
  int off[32], p2[32][32], p1[32][32];
  for (int L = 0, o = 0; L < nlev3; ++L) {
    const size_t n = (size_t)n3s[L] * n2s[L] * n1s[L] * 2;
    res[L] = (double *)malloc(sizeof(double) * n);
    bl[L] = L ? (double *)malloc(sizeof(double) * n) : (double *)b;
    xl[L] = L ? (double *)malloc(sizeof(double) * n) : x;
    off[L] = o;
    o += nlev2s[L];
    p2[L][0] = n2s[L];
    p1[L][0] = n1s[L];
    for (int m = 1; m < nlev2s[L]; ++m) {
      p2[L][m] = (p2[L][m - 1] + 1) / 2;
      p1[L][m] = (p1[L][m - 1] + 1) / 2;
    }
  }
#define GS3(L, gi)                                                                                                 \
  ora_tri_tb_gauss_seidel_3d(variant, n3s[L], nlev2s[L], p2[L], p1[L], d + off[L], u1 + off[L], l1 + off[L],    \
                             u2 + off[L], l2 + off[L], u3[L], l3[L], bl[L], xl[L], gi, gauss_iter2, mult_iter2)
  for (int it = 0; it < mult_iter3; ++it) {
    int gi = 1, L = 0;
    for (;;) {
      GS3(L, gi);
      gi += gauss_iter3;
      if (L + 1 == nlev3) {
        gi -= gauss_iter3;
        break;
      }
      const size_t n = (size_t)n3s[L] * n2s[L] * n1s[L] * 2;
      ora_tri_tb_matvec_3d(variant, n3s[L], n2s[L], n1s[L], d[off[L]], u1[off[L]], l1[off[L]], u2[off[L]],
                           l2[off[L]], u3[L], l3[L], xl[L], res[L]);
      for (size_t q = 0; q < n; ++q) res[L][q] = bl[L][q] - res[L][q];
      ora_tri_tb_restrict_3d(n3s[L], n2s[L], n1s[L], res[L], bl[L + 1]);
      memset(xl[L + 1], 0, sizeof(double) * (size_t)n3s[L + 1] * n2s[L + 1] * n1s[L + 1] * 2);
      ++L;
    }
    for (;;) {
      GS3(L, gi);
      gi -= gauss_iter3;
      if (L == 0) break;
      --L;
      const size_t n = (size_t)n3s[L] * n2s[L] * n1s[L] * 2;
      ora_tri_tb_prolong_3d(n3s[L], n2s[L], n1s[L], xl[L + 1], res[L]);
      for (size_t q = 0; q < n; ++q) xl[L][q] = xl[L][q] + res[L][q];
    }
  }
#undef GS3
  for (int L = 0; L < nlev3; ++L) {
    free(res[L]);
    if (L) {
      free(bl[L]);
      free(xl[L]);
    }
  }
}

/* One level of LaplTBCompute / LaplTRCompute (MULTI/JacAccGrav_Mod.f90:1312-1482,
 * 1485-1667): the finest fields coarsened with the shifts 2^level2-1 along
 * directions 1 and 2 and 2^level3-1 along direction 3 (level2 >= level3) --
 * FaceCoarse of F and FG, CFaceCoarse of DTU weighted by F and of DUU
 * weighted by FG, VolCoarse of Vol, CVolCoarse of DUT and DUR weighted by Vol
 * (:685-891; every coarse value sums its fine values with direction 1
 * slowest, then direction 2, then 3, the weighted ones then divided by the
 * coarse weight + Eps) -- and assembled by Compute_3D: with the couplings
 * between planes (the level itself, level2 == level3) or without (the
 * level2-level3'th plane level of its planes).  Face and cell layouts as
 * ora_tri_tb_compute_3d; level 0 too is the coarsening with shift 0. */
static size_t tb_blo(int c, int s) { return (size_t)(c - 1) * (s + 1) + 1; }
static size_t tb_bhi(int c, int s, int n) { return (size_t)c * (s + 1) < (size_t)n ? (size_t)c * (s + 1) : (size_t)n; }

void ora_tri_tb_lapl_level(int variant, int n3, int n2, int n1, const double *s, const double *const *faces,
                           const double *vol, const double *dut, const double *dur, int level3, int level2, double *d,
                           double *u1, double *l1, double *u2, double *l2, double *u3, double *l3) {
  const int s3 = (1 << level3) - 1, s12 = (1 << level2) - 1;
  const int c1 = (n1 + s12) / (s12 + 1), c2 = (n2 + s12) / (s12 + 1), c3 = (n3 + s3) / (s3 + 1);
  const size_t cz = (size_t)c3 * c2 * (c1 + 1), cx = (size_t)c3 * (c2 + 1) * c1, cy = (size_t)(c3 + 1) * c2 * c1;
  const size_t cc = (size_t)c3 * c2 * c1;
  double *buf = (double *)malloc(sizeof(double) * (4 * (cz + cx + cy) + 3 * cc));
  double *cf[12];
  const size_t clen[3] = {cz, cx, cy};
  double *p = buf;
  for (int q = 0; q < 12; ++q) {
    cf[q] = p;
    p += clen[q / 4];
  }
  double *vc = p, *dutc = p + cc, *durc = p + 2 * cc;
  /* faces: direction a's index on the coarse face fixed (the fine face at
   * min((shift+1)*c, n)), the other two summed over their cells */
  for (int a = 0; a < 3; ++a) {
    const double *F = faces[4 * a], *FG = faces[4 * a + 1], *DT = faces[4 * a + 2], *DU = faces[4 * a + 3];
    const int e1 = a == 0, e2 = a == 1, e3 = a == 2; /* the face direction has one more entry */
    for (int kc = 1 - e3; kc <= c3; ++kc)
      for (int jc = 1 - e2; jc <= c2; ++jc)
        for (int ic = 1 - e1; ic <= c1; ++ic) {
          size_t ilo, ihi, jlo, jhi, klo, khi;
          if (e1) ilo = ihi = (size_t)(s12 + 1) * ic < (size_t)n1 ? (size_t)(s12 + 1) * ic : (size_t)n1;
          else { ilo = tb_blo(ic, s12); ihi = tb_bhi(ic, s12, n1); }
          if (e2) jlo = jhi = (size_t)(s12 + 1) * jc < (size_t)n2 ? (size_t)(s12 + 1) * jc : (size_t)n2;
          else { jlo = tb_blo(jc, s12); jhi = tb_bhi(jc, s12, n2); }
          if (e3) klo = khi = (size_t)(s3 + 1) * kc < (size_t)n3 ? (size_t)(s3 + 1) * kc : (size_t)n3;
          else { klo = tb_blo(kc, s3); khi = tb_bhi(kc, s3, n3); }
          double f = 0.0, fg = 0.0, tf = 0.0, ug = 0.0;
          for (size_t i = ilo; i <= ihi; ++i)
            for (size_t j = jlo; j <= jhi; ++j)
              for (size_t k = klo; k <= khi; ++k) {
                /* fine index: 0-based on the face direction, 1-based cells */
                const size_t ii = e1 ? i : i - 1, jj = e2 ? j : j - 1, kk = e3 ? k : k - 1;
                const size_t q = ((kk * (size_t)(n2 + e2) + jj) * (size_t)(n1 + e1)) + ii;
                f = f + F[q];
                fg = fg + FG[q];
                tf = tf + DT[q] * F[q];
                ug = ug + DU[q] * FG[q];
              }
          const size_t ici = e1 ? (size_t)ic : (size_t)ic - 1, jci = e2 ? (size_t)jc : (size_t)jc - 1,
                       kci = e3 ? (size_t)kc : (size_t)kc - 1;
          const size_t qc = ((kci * (size_t)(c2 + e2) + jci) * (size_t)(c1 + e1)) + ici;
          cf[4 * a][qc] = f;
          cf[4 * a + 1][qc] = fg;
          cf[4 * a + 2][qc] = tf / (f + EPS_TB);
          cf[4 * a + 3][qc] = ug / (fg + EPS_TB);
        }
  }
  for (int kc = 1; kc <= c3; ++kc)
    for (int jc = 1; jc <= c2; ++jc)
      for (int ic = 1; ic <= c1; ++ic) {
        double v = 0.0, tv = 0.0, rv = 0.0;
        for (size_t i = tb_blo(ic, s12); i <= tb_bhi(ic, s12, n1); ++i)
          for (size_t j = tb_blo(jc, s12); j <= tb_bhi(jc, s12, n2); ++j)
            for (size_t k = tb_blo(kc, s3); k <= tb_bhi(kc, s3, n3); ++k) {
              const size_t q = ((k - 1) * n2 + (j - 1)) * n1 + (i - 1);
              v = v + vol[q];
              tv = tv + dut[q] * vol[q];
              if (dur) rv = rv + dur[q] * vol[q];
            }
        const size_t qc = ((size_t)(kc - 1) * c2 + (jc - 1)) * c1 + (ic - 1);
        vc[qc] = v;
        dutc[qc] = tv / (v + EPS_TB);
        durc[qc] = rv / (v + EPS_TB);
      }
  ora_tri_tb_compute_3d(variant, level2 == level3, c3, c2, c1, s, cf[0], cf[1], cf[2], cf[3], cf[4], cf[5], cf[6],
                        cf[7], cf[8], cf[9], cf[10], cf[11], vc, dutc, durc, d, u1, l1, u2, l2, u3, l3);
  free(buf);
}
