/* Oracle (test infrastructure only) of the block-tridiagonal column solve of
 * MULTI/TriDiagTB_Mod.f90: Solve_1D (:143-163) and MatVecTB_1D (:121-141),
 * with the 2x2 helpers of CG/Matrix_Mod.f90 (Mult_2, Mult_22, Div_2, Div_22)
 * in their operation order.  Compiled without contraction.  Layout: the
 * reference's per-column arrays back to back, 2x2 blocks column-major
 * (index r + 2c), vectors (index r) per level. */
#include <stddef.h>

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
