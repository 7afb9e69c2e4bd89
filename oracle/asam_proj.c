/*
 * CPU oracle of the ASAM pressure projection (sound solve) of one block.
 *
 * TEST INFRASTRUCTURE ONLY.  The parity tests and the CPU-baseline leg of the
 * benchmark call it as the checker; the CUDA library never links or calls it.
 *
 * It restates, loop for loop and in the same floating-point operation order,
 * the Fortran routines of ASAM (OsKnoth/ASAM) on the projection path with the
 * configuration's switches (MultiTriT, GradFull, MethSound='FGMRES', default
 * orders xOrder=2, yOrder=3, zOrder=1, coarsening factors 2):
 *
 *   LaplTFullCompute          MULTI/JacAccGrav_Mod.f90:1056-1310
 *   FaceCoarse, CFaceCoarse, VolCoarse, CVolCoarse, IncrCoarse, CIncrCoarse
 *                             MULTI/JacAccGrav_Mod.f90:709-903
 *   ComputeFull_1D/2D/3D      MULTI/TriDiagT_Mod.f90:62-90, 330-403, 790-883
 *   MatVecT_1D/2D/3D          MULTI/TriDiagT_Mod.f90:113-133, 405-431, 885-917
 *   Solve_1D (Thomas)         MULTI/TriDiagT_Mod.f90:135-155
 *   GaussSeidel_2D/3D         MULTI/TriDiagT_Mod.f90:433-471, 931-983
 *   Multigrid_2D/3D, Solve_2D/3D, RestrictT_2D/3D, ProlongateT_2D/3D
 *                             MULTI/TriDiagT_Mod.f90:472-589, 985-1131
 *   Reverse, ReverseBack      MULTI/Reverse_Mod.f90:565-588 ((x,y,z) -> (z,x,y))
 *   MatVecP_Tri, VCycleCG     MULTI/JacAccGrav_Mod.f90:531-545, 4466-4517
 *   MatVecFull (MultiTriT)    MATRIX/MatVec_Mod.f90:184-258
 *   PSolve1, PressurePre, b1pBTx2Full, SchurPreFull
 *                             MATRIX/PreCond_Mod.f90:1555-1571, 599-622, 624-665, 20-597
 *   FGMRES                    SOLU/Iter_Mod.f90:121-199
 *   Rhs, DivergenceS          MATRIX/Rhs_Mod.f90:110-187, 41-78
 *   UpdateVelocity            MATRIX/Rhs_Mod.f90:589-952 (GradFull, MultiTriT)
 *   ProjectVelFace            ADVECT/IntSub_Mod.f90:25-71
 *
 * Scope: one block whose sides are either closed outer boundaries
 * (TypeW='ow' ... with BCP=0 and a velocity rule other than 'OutFlow') or
 * periodic, i.e. the block is its own neighbour across the side pair
 * (nType 'iw'/'ie', 'is'/'in', 'ib'/'it' with equal refinement).  A periodic
 * side carries the boundary face unknowns u_w ... w_t of PressureVelocity
 * (MODULE/VecPrVel_Mod.f90:10-18); a closed side has none.  With face
 * unknowns the routines restated here are
 *   MatVecFull face terms      MATRIX/MatVec_Mod.f90:184-258
 *   Exchange / RandCopy / CopyFluxVel (EqualEqual)
 *                              MODULE/VecPrVel_Mod.f90:809-974,
 *                              MODULE/Exchange_Mod.f90:769-859
 *   DOT2                       MODULE/VecPrVel_Mod.f90:112-172
 *   PSolve1 = PressurePre, b2pBx1Full, Exchange, SchurPreFull, Exchange,
 *   b1pBTx2Full, PressurePre   MATRIX/PreCond_Mod.f90:1555-1571, 599-844, 20-597
 *   SetFactorD (Fac=2 on the periodic sides) for the Dirichlet hierarchy
 *   LaplDirichlet               MULTI/Reverse_Mod.f90:95-213,
 *                              MULTI/JacAccGrav_Mod.f90:453-469
 *   UpdateVelocity boundary faces MATRIX/Rhs_Mod.f90:636-660
 * The Neumann hierarchy LaplNeumann keeps the factors 0 of SetFactorN
 * (MULTI/Reverse_Mod.f90:215-292) on every side.
 *
 * PressureVelocity vectors of this file: the pressure (natural interior
 * order, nx*ny*nz) followed by the face unknowns of the periodic sides in the
 * order u_w, u_e (ny*nz each, y fastest), v_s, v_n (nx*nz, x fastest), w_b,
 * w_t (nx*ny, x fastest); ora_proj_nvec() gives the length.
 *
 * Besides the reference's lexicographic plane/line Gauss-Seidel smoother the
 * file also holds the zebra (two-colour) ordering of the same smoother that the
 * GPU runs (planes, then x-lines, of one parity are independent): with
 * zebra=1 every plane and line relaxation uses exactly the reference's
 * arithmetic, only the order of the relaxations changes.
 *
 * Layout: inputs are Fortran arrays in natural (x fastest) order; internally
 * everything is in the reversed index space (n1,n2,n3) = (nz,nx,ny) of
 * Reverse_Mod, column-major with 1-based logical indices.
 *
 * Build with -O2 -ffp-contract=off.  Parity with the Fortran binary itself is
 * unpinned (no Fortran compiler is available).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define EPS 1.0e-30

typedef struct {
  int n1;
  double *d, *u, *l; /* d(1:n1), u(1:n1-1), l(1:n1-1) */
} T1;

typedef struct T2 {
  int n1, n2;
  T1* col;          /* col[j], j = 0..n2-1 */
  double *u, *l;    /* (n1, n2-1) */
  double *res, *resc, *xc;
  struct T2 *coarse, *fine;
} T2;

typedef struct T3 {
  int n1, n2, n3;
  T2** pl;          /* pl[k], k = 0..n3-1: plane matrices (finest 2D level of their chain) */
  double *u, *l;    /* (n1, n2, n3-1) */
  double *res, *resc, *xc;
  struct T3 *coarse, *fine;
} T3;

typedef struct {
  int nx, ny, nz;
  int ref_level, gauss_iter2, gauss_iter3, mult_iter2, mult_iter3;
  int zebra;
  double fac_anela;
  double fac1_l, fac1_r, fac2_l, fac2_r, fac3_l, fac3_r;
} PrjPar;

typedef struct {
  PrjPar par;
  T3* A;
  int n1, n2, n3;
  /* copies of the geometry/weights the projection needs after assembly */
  double *fu, *fv, *fw;       /* interior faces: (nx+1,ny,nz), (nx,ny+1,nz), (nx,ny,nz+1) */
  double *dtu, *dtv, *dtw, *duu, *duv, *duw;
  double *dut, *dtt, *vol;    /* interior (nx,ny,nz) */
  double* volp;               /* padded VolC (halo cells included) */
  double *dx, *dy, *dz;
  double *mxy, *mxz, *myx, *myz, *mzx, *mzy;
  double beta0, dtp;
  /* periodic side pairs (face unknowns) and the Dirichlet hierarchy */
  int per_x, per_y, per_z;
  double prefac2;      /* PreFac2 (MODULE/Control_Mod.f90:59, default 0.5) */
  T3* AD;              /* LaplDirichlet: SetFactorD factors */
  size_t nvec;         /* length of a PressureVelocity vector */
  long off[6];         /* offsets of u_w, u_e, v_s, v_n, w_b, w_t (-1: no face unknowns) */
} Proj;

static double* zalloc(size_t n) { return (double*)calloc(n ? n : 1, sizeof(double)); }
static int cdiv2(int n) { return (n + 1) / 2; }

/* ---------------------------------------------------------------------- */
/* Allocation: Allocate_1D/2D/3D, MULTI/TriDiagT_Mod.f90:92-111, 208-244, 645-688 */
static void t1_alloc(T1* a, int n) {
  a->n1 = n;
  a->d = zalloc(n);
  for (int i = 0; i < n; ++i) a->d[i] = 1.0e-40;
  a->u = zalloc(n > 1 ? n - 1 : 0);
  a->l = zalloc(n > 1 ? n - 1 : 0);
}

static T2* t2_alloc(int n2, int n1) {
  T2* a = (T2*)calloc(1, sizeof(T2));
  a->n1 = n1;
  a->n2 = n2;
  a->col = (T1*)calloc(n2, sizeof(T1));
  for (int j = 0; j < n2; ++j) t1_alloc(&a->col[j], n1);
  a->u = zalloc((size_t)n1 * (n2 > 1 ? n2 - 1 : 0));
  a->l = zalloc((size_t)n1 * (n2 > 1 ? n2 - 1 : 0));
  a->res = zalloc((size_t)n1 * n2);
  a->resc = zalloc((size_t)cdiv2(n1) * cdiv2(n2));
  a->xc = zalloc((size_t)cdiv2(n1) * cdiv2(n2));
  return a;
}

static T3* t3_alloc(int n3, int n2, int n1) {
  T3* a = (T3*)calloc(1, sizeof(T3));
  a->n1 = n1;
  a->n2 = n2;
  a->n3 = n3;
  a->pl = (T2**)calloc(n3, sizeof(T2*));
  for (int k = 0; k < n3; ++k) a->pl[k] = t2_alloc(n2, n1);
  size_t m = (size_t)n1 * n2;
  a->u = zalloc(m * (n3 > 1 ? n3 - 1 : 0));
  a->l = zalloc(m * (n3 > 1 ? n3 - 1 : 0));
  a->res = zalloc(m * n3);
  a->resc = zalloc((size_t)cdiv2(n1) * cdiv2(n2) * cdiv2(n3));
  a->xc = zalloc((size_t)cdiv2(n1) * cdiv2(n2) * cdiv2(n3));
  return a;
}

static void t1_free(T1* a) {
  free(a->d);
  free(a->u);
  free(a->l);
}

static void t2_free(T2* a) {
  while (a) {
    T2* c = a->coarse;
    for (int j = 0; j < a->n2; ++j) t1_free(&a->col[j]);
    free(a->col);
    free(a->u);
    free(a->l);
    free(a->res);
    free(a->resc);
    free(a->xc);
    free(a);
    a = c;
  }
}

static void t3_free(T3* a) {
  while (a) {
    T3* c = a->coarse;
    for (int k = 0; k < a->n3; ++k) t2_free(a->pl[k]);
    free(a->pl);
    free(a->u);
    free(a->l);
    free(a->res);
    free(a->resc);
    free(a->xc);
    free(a);
    a = c;
  }
}

/* ---------------------------------------------------------------------- */
/* Coarsened input fields of one level (reversed index space) */
typedef struct {
  int n1, n2, n3;
  double *F1, *F2, *F3;       /* F1(0:n1,1:n2,1:n3), F2(1:n1,0:n2,1:n3), F3(1:n1,1:n2,0:n3) */
  double *T1_, *T2_, *T3_;    /* DTU1..3 */
  double *U1, *U2, *U3;       /* DUU1..3 */
  double *d1, *d2, *d3;       /* d1G.. */
  double *m12, *m13, *m21, *m23, *m31, *m32;
  double *vol, *dut;          /* (n1,n2,n3) */
} Fields;

#define IDX1(f, i, j, k) ((size_t)(i) + ((size_t)(f)->n1 + 1) * ((size_t)((j) - 1) + (size_t)(f)->n2 * ((k) - 1)))
#define IDX2(f, i, j, k) ((size_t)((i) - 1) + (size_t)(f)->n1 * ((size_t)(j) + ((size_t)(f)->n2 + 1) * ((k) - 1)))
#define IDX3(f, i, j, k) ((size_t)((i) - 1) + (size_t)(f)->n1 * ((size_t)((j) - 1) + (size_t)(f)->n2 * (size_t)(k)))
#define IDXC(f, i, j, k) ((size_t)((i) - 1) + (size_t)(f)->n1 * ((size_t)((j) - 1) + (size_t)(f)->n2 * ((k) - 1)))

static void fields_alloc(Fields* f, int n1, int n2, int n3) {
  f->n1 = n1;
  f->n2 = n2;
  f->n3 = n3;
  size_t s1 = (size_t)(n1 + 1) * n2 * n3, s2 = (size_t)n1 * (n2 + 1) * n3, s3 = (size_t)n1 * n2 * (n3 + 1);
  f->F1 = zalloc(s1);
  f->T1_ = zalloc(s1);
  f->U1 = zalloc(s1);
  f->F2 = zalloc(s2);
  f->T2_ = zalloc(s2);
  f->U2 = zalloc(s2);
  f->F3 = zalloc(s3);
  f->T3_ = zalloc(s3);
  f->U3 = zalloc(s3);
  f->d1 = zalloc(n1);
  f->d2 = zalloc(n2);
  f->d3 = zalloc(n3);
  f->m12 = zalloc(n2);
  f->m13 = zalloc(n3);
  f->m21 = zalloc(n1);
  f->m23 = zalloc(n3);
  f->m31 = zalloc(n1);
  f->m32 = zalloc(n2);
  f->vol = zalloc((size_t)n1 * n2 * n3);
  f->dut = zalloc((size_t)n1 * n2 * n3);
}

static void fields_free(Fields* f) {
  double* p[] = {f->F1, f->T1_, f->U1, f->F2, f->T2_, f->U2, f->F3, f->T3_, f->U3, f->d1, f->d2,
                 f->d3, f->m12, f->m13, f->m21, f->m23, f->m31, f->m32, f->vol, f->dut};
  for (size_t i = 0; i < sizeof(p) / sizeof(p[0]); ++i) free(p[i]);
}

/* FaceCoarse + CFaceCoarse (JacAccGrav_Mod.f90:804-903), VolCoarse + CVolCoarse
 * (:724-745, :784-802), IncrCoarse + CIncrCoarse (:747-782), applied to the
 * fine fields g with shifts (s1,s2,s3) into the coarse fields c. */
static void coarsen(const Fields* g, Fields* c, int s1, int s2, int s3) {
  const int n = g->n1, m = g->n2, l = g->n3;
  const int nC = c->n1, mC = c->n2, lC = c->n3;
  /* FaceCoarse */
  for (int iC = 0; iC <= nC; ++iC) {
    int i = (s1 + 1) * iC < n ? (s1 + 1) * iC : n;
    for (int j = 1; j <= m; ++j) {
      int jC = (j + s2) / (s2 + 1);
      for (int k = 1; k <= l; ++k) {
        int kC = (k + s3) / (s3 + 1);
        c->F1[IDX1(c, iC, jC, kC)] += g->F1[IDX1(g, i, j, k)];
      }
    }
  }
  for (int i = 1; i <= n; ++i) {
    int iC = (i + s1) / (s1 + 1);
    for (int jC = 0; jC <= mC; ++jC) {
      int j = (s2 + 1) * jC < m ? (s2 + 1) * jC : m;
      for (int k = 1; k <= l; ++k) {
        int kC = (k + s3) / (s3 + 1);
        c->F2[IDX2(c, iC, jC, kC)] += g->F2[IDX2(g, i, j, k)];
      }
    }
  }
  for (int i = 1; i <= n; ++i) {
    int iC = (i + s1) / (s1 + 1);
    for (int j = 1; j <= m; ++j) {
      int jC = (j + s2) / (s2 + 1);
      for (int kC = 0; kC <= lC; ++kC) {
        int k = (s3 + 1) * kC < l ? (s3 + 1) * kC : l;
        c->F3[IDX3(c, iC, jC, kC)] += g->F3[IDX3(g, i, j, k)];
      }
    }
  }
  /* CFaceCoarse for DTU and DUU (same loop nests, then / (FC + Eps)) */
  const double* gs[2][3] = {{g->T1_, g->T2_, g->T3_}, {g->U1, g->U2, g->U3}};
  double* cs[2][3] = {{c->T1_, c->T2_, c->T3_}, {c->U1, c->U2, c->U3}};
  for (int w = 0; w < 2; ++w) {
    for (int iC = 0; iC <= nC; ++iC) {
      int i = (s1 + 1) * iC < n ? (s1 + 1) * iC : n;
      for (int j = 1; j <= m; ++j) {
        int jC = (j + s2) / (s2 + 1);
        for (int k = 1; k <= l; ++k) {
          int kC = (k + s3) / (s3 + 1);
          cs[w][0][IDX1(c, iC, jC, kC)] += gs[w][0][IDX1(g, i, j, k)] * g->F1[IDX1(g, i, j, k)];
        }
      }
    }
    for (size_t q = 0; q < (size_t)(nC + 1) * mC * lC; ++q) cs[w][0][q] = cs[w][0][q] / (c->F1[q] + EPS);
    for (int i = 1; i <= n; ++i) {
      int iC = (i + s1) / (s1 + 1);
      for (int jC = 0; jC <= mC; ++jC) {
        int j = (s2 + 1) * jC < m ? (s2 + 1) * jC : m;
        for (int k = 1; k <= l; ++k) {
          int kC = (k + s3) / (s3 + 1);
          cs[w][1][IDX2(c, iC, jC, kC)] += gs[w][1][IDX2(g, i, j, k)] * g->F2[IDX2(g, i, j, k)];
        }
      }
    }
    for (size_t q = 0; q < (size_t)nC * (mC + 1) * lC; ++q) cs[w][1][q] = cs[w][1][q] / (c->F2[q] + EPS);
    for (int i = 1; i <= n; ++i) {
      int iC = (i + s1) / (s1 + 1);
      for (int j = 1; j <= m; ++j) {
        int jC = (j + s2) / (s2 + 1);
        for (int kC = 0; kC <= lC; ++kC) {
          int k = (s3 + 1) * kC < l ? (s3 + 1) * kC : l;
          cs[w][2][IDX3(c, iC, jC, kC)] += gs[w][2][IDX3(g, i, j, k)] * g->F3[IDX3(g, i, j, k)];
        }
      }
    }
    for (size_t q = 0; q < (size_t)nC * mC * (lC + 1); ++q) cs[w][2][q] = cs[w][2][q] / (c->F3[q] + EPS);
  }
  /* IncrCoarse */
  for (int i = 1; i <= n; ++i) c->d1[(i + s1) / (s1 + 1) - 1] += g->d1[i - 1];
  for (int j = 1; j <= m; ++j) c->d2[(j + s2) / (s2 + 1) - 1] += g->d2[j - 1];
  for (int k = 1; k <= l; ++k) c->d3[(k + s3) / (s3 + 1) - 1] += g->d3[k - 1];
  /* CIncrCoarse (CC = sum d*C, then CC/dC) */
#define CINCR(nn, C, d, CC, dC, sh)                                                                  \
  do {                                                                                               \
    for (int i_ = 1; i_ <= (nn); ++i_) (CC)[(i_ + (sh)) / ((sh) + 1) - 1] += (d)[i_ - 1] * (C)[i_ - 1]; \
    for (int i_ = 0; i_ < ((nn) + (sh)) / ((sh) + 1); ++i_) (CC)[i_] = (CC)[i_] / (dC)[i_];          \
  } while (0)
  CINCR(m, g->m12, g->d2, c->m12, c->d2, s2);
  CINCR(l, g->m13, g->d3, c->m13, c->d3, s3);
  CINCR(n, g->m21, g->d1, c->m21, c->d1, s1);
  CINCR(l, g->m23, g->d3, c->m23, c->d3, s3);
  CINCR(n, g->m31, g->d1, c->m31, c->d1, s1);
  CINCR(m, g->m32, g->d2, c->m32, c->d2, s2);
#undef CINCR
  /* VolCoarse and CVolCoarse */
  for (int i = 1; i <= n; ++i) {
    int iC = (i + s1) / (s1 + 1);
    for (int j = 1; j <= m; ++j) {
      int jC = (j + s2) / (s2 + 1);
      for (int k = 1; k <= l; ++k) {
        int kC = (k + s3) / (s3 + 1);
        c->vol[IDXC(c, iC, jC, kC)] += g->vol[IDXC(g, i, j, k)];
      }
    }
  }
  for (int i = 1; i <= n; ++i) {
    int iC = (i + s1) / (s1 + 1);
    for (int j = 1; j <= m; ++j) {
      int jC = (j + s2) / (s2 + 1);
      for (int k = 1; k <= l; ++k) {
        int kC = (k + s3) / (s3 + 1);
        c->dut[IDXC(c, iC, jC, kC)] += g->dut[IDXC(g, i, j, k)] * g->vol[IDXC(g, i, j, k)];
      }
    }
  }
  for (size_t q = 0; q < (size_t)nC * mC * lC; ++q) c->dut[q] = c->dut[q] / (c->vol[q] + EPS);
}

/* ComputeFull_1D (TriDiagT_Mod.f90:62-90) for column j of plane k of the
 * coarse fields f: F = F1(:,j,k), dd = d1, Metr1 = m12(j), Metr2 = m13(k). */
static void compute_1d(const PrjPar* p, double bd2, T1* A, const Fields* f, int j, int k) {
  const int n1 = A->n1;
  const double M1 = f->m12[j - 1], M2 = f->m13[k - 1];
  const double* dd = f->d1;
#define F(i) f->F1[IDX1(f, (i) - 1, j, k)]
#define DT(i) f->T1_[IDX1(f, (i) - 1, j, k)]
#define DU(i) f->U1[IDX1(f, (i) - 1, j, k)]
#define DUT(i) f->dut[IDXC(f, (i), j, k)]
  A->d[0] = A->d[0] + bd2 * p->fac1_l * F(1) * DT(1) * DU(1) * DUT(1) / (dd[0] * M1 * M2);
  for (int i = 1; i <= n1 - 1; ++i) {
    const double den = (dd[i - 1] + dd[i]) * M1 * M2;
    A->u[i - 1] = -(bd2 * 2.0 * F(i + 1) * DT(i + 1) * DU(i + 1) * DUT(i + 1) / den);
    A->l[i - 1] = -(bd2 * 2.0 * F(i + 1) * DT(i + 1) * DU(i + 1) * DUT(i) / den);
    A->d[i - 1] = A->d[i - 1] + bd2 * 2.0 * F(i + 1) * DT(i + 1) * DU(i + 1) * DUT(i) / den;
    A->d[i] = A->d[i] + bd2 * 2.0 * F(i + 1) * DT(i + 1) * DU(i + 1) * DUT(i + 1) / den;
  }
  A->d[n1 - 1] = A->d[n1 - 1] + bd2 * p->fac1_r * F(n1 + 1) * DT(n1 + 1) * DU(n1 + 1) * DUT(n1) / (dd[n1 - 1] * M1 * M2);
  for (int i = 1; i <= n1; ++i) A->d[i - 1] = A->d[i - 1] + p->fac_anela * f->vol[IDXC(f, i, j, k)];
#undef F
#undef DT
#undef DU
#undef DUT
}

/* ComputeFull_2D (TriDiagT_Mod.f90:330-403, branch with u/l associated) for
 * plane k of the coarse fields f. */
static void compute_2d(const PrjPar* p, double bd2, T2* A, const Fields* f, int k) {
  const int n1 = A->n1, n2 = A->n2;
  const double M23 = f->m23[k - 1];
  const double* dd2 = f->d2;
#define F2(i, j) f->F2[IDX2(f, i, (j) - 1, k)]
#define DT2(i, j) f->T2_[IDX2(f, i, (j) - 1, k)]
#define DU2(i, j) f->U2[IDX2(f, i, (j) - 1, k)]
#define DUT(i, j) f->dut[IDXC(f, i, j, k)]
  compute_1d(p, bd2, &A->col[0], f, 1, k);
  for (int i = 1; i <= n1; ++i)
    A->col[0].d[i - 1] = A->col[0].d[i - 1] +
                         bd2 * p->fac2_l * F2(i, 1) * DT2(i, 1) * DU2(i, 1) * DUT(i, 1) / (dd2[0] * f->m21[i - 1] * M23);
  for (int j = 1; j <= n2 - 1; ++j) {
    for (int i = 1; i <= n1; ++i) {
      const double den = (dd2[j - 1] + dd2[j]) * f->m21[i - 1] * M23;
      A->u[(i - 1) + (size_t)n1 * (j - 1)] = -(bd2 * 2.0 * F2(i, j + 1) * DT2(i, j + 1) * DU2(i, j + 1) * DUT(i, j + 1) / den);
      A->l[(i - 1) + (size_t)n1 * (j - 1)] = -(bd2 * 2.0 * F2(i, j + 1) * DT2(i, j + 1) * DU2(i, j + 1) * DUT(i, j) / den);
      A->col[j - 1].d[i - 1] = A->col[j - 1].d[i - 1] + bd2 * 2.0 * F2(i, j + 1) * DT2(i, j + 1) * DU2(i, j + 1) * DUT(i, j) / den;
    }
    compute_1d(p, bd2, &A->col[j], f, j + 1, k);
    for (int i = 1; i <= n1; ++i) {
      const double den = (dd2[j - 1] + dd2[j]) * f->m21[i - 1] * M23;
      A->col[j].d[i - 1] = A->col[j].d[i - 1] + bd2 * 2.0 * F2(i, j + 1) * DT2(i, j + 1) * DU2(i, j + 1) * DUT(i, j + 1) / den;
    }
  }
  for (int i = 1; i <= n1; ++i)
    A->col[n2 - 1].d[i - 1] = A->col[n2 - 1].d[i - 1] + bd2 * p->fac2_r * F2(i, n2 + 1) * DT2(i, n2 + 1) * DU2(i, n2 + 1) *
                                                          DUT(i, n2) / (dd2[n2 - 1] * f->m21[i - 1] * M23);
#undef F2
#undef DT2
#undef DU2
#undef DUT
}

/* ComputeFull_3D (TriDiagT_Mod.f90:790-883).  full=1: the branch with the
 * 3D couplings u/l (no DUU3 in the interior terms and in the last boundary
 * term); full=0: the branch for the coarse plane levels (DUU3 in every term,
 * no u/l).  pl[k] are the plane matrices to fill. */
static void compute_3d(const PrjPar* p, double bd2, T2** pl, double* u3, double* l3, int n3, const Fields* f, int full) {
  const int n1 = f->n1, n2 = f->n2;
  const double* dd3 = f->d3;
#define F3(i, j, k) f->F3[IDX3(f, i, j, (k) - 1)]
#define DT3(i, j, k) f->T3_[IDX3(f, i, j, (k) - 1)]
#define DU3(i, j, k) f->U3[IDX3(f, i, j, (k) - 1)]
#define DUT(i, j, k) f->dut[IDXC(f, i, j, k)]
#define D(k, j, i) pl[(k) - 1]->col[(j) - 1].d[(i) - 1]
  compute_2d(p, bd2, pl[0], f, 1);
  for (int j = 1; j <= n2; ++j)
    for (int i = 1; i <= n1; ++i)
      D(1, j, i) = D(1, j, i) + bd2 * p->fac3_l * F3(i, j, 1) * DT3(i, j, 1) * DU3(i, j, 1) * DUT(i, j, 1) /
                                    (dd3[0] * f->m31[i - 1] * f->m32[j - 1]);
  for (int k = 1; k <= n3 - 1; ++k) {
    for (int j = 1; j <= n2; ++j)
      for (int i = 1; i <= n1; ++i) {
        const double den = (dd3[k - 1] + dd3[k]) * f->m31[i - 1] * f->m32[j - 1];
        if (full) {
          u3[(i - 1) + (size_t)n1 * ((j - 1) + (size_t)n2 * (k - 1))] =
              -(bd2 * 2.0 * F3(i, j, k + 1) * DT3(i, j, k + 1) * DUT(i, j, k + 1) / den);
          D(k, j, i) = D(k, j, i) + bd2 * 2.0 * F3(i, j, k + 1) * DT3(i, j, k + 1) * DUT(i, j, k) / den;
        } else {
          D(k, j, i) = D(k, j, i) + bd2 * 2.0 * F3(i, j, k + 1) * DT3(i, j, k + 1) * DU3(i, j, k + 1) * DUT(i, j, k) / den;
        }
      }
    compute_2d(p, bd2, pl[k], f, k + 1);
    for (int j = 1; j <= n2; ++j)
      for (int i = 1; i <= n1; ++i) {
        const double den = (dd3[k - 1] + dd3[k]) * f->m31[i - 1] * f->m32[j - 1];
        if (full) {
          l3[(i - 1) + (size_t)n1 * ((j - 1) + (size_t)n2 * (k - 1))] =
              -(bd2 * 2.0 * F3(i, j, k + 1) * DT3(i, j, k + 1) * DUT(i, j, k) / den);
          D(k + 1, j, i) = D(k + 1, j, i) + bd2 * 2.0 * F3(i, j, k + 1) * DT3(i, j, k + 1) * DUT(i, j, k + 1) / den;
        } else {
          D(k + 1, j, i) =
              D(k + 1, j, i) + bd2 * 2.0 * F3(i, j, k + 1) * DT3(i, j, k + 1) * DU3(i, j, k + 1) * DUT(i, j, k + 1) / den;
        }
      }
  }
  for (int j = 1; j <= n2; ++j)
    for (int i = 1; i <= n1; ++i) {
      if (full)
        D(n3, j, i) = D(n3, j, i) + bd2 * p->fac3_r * F3(i, j, n3 + 1) * DT3(i, j, n3 + 1) * DUT(i, j, n3) /
                                        (dd3[n3 - 1] * f->m31[i - 1] * f->m32[j - 1]);
      else
        D(n3, j, i) = D(n3, j, i) + bd2 * p->fac3_r * F3(i, j, n3 + 1) * DT3(i, j, n3 + 1) * DU3(i, j, n3 + 1) *
                                        DUT(i, j, n3) / (dd3[n3 - 1] * f->m31[i - 1] * f->m32[j - 1]);
    }
#undef F3
#undef DT3
#undef DU3
#undef DUT
#undef D
}

/* ---------------------------------------------------------------------- */
/* Solvers */

/* Solve_1D (TriDiagT_Mod.f90:135-155), in place on b */
static void solve_1d(const T1* A, double* b) {
  const int n = A->n1;
  double* w = (double*)malloc(sizeof(double) * (n > 1 ? n : 1));
  double t = A->d[0];
  b[0] = b[0] / t;
  for (int i = 2; i <= n; ++i) {
    w[i - 2] = A->u[i - 2] / t;
    t = A->d[i - 1] - A->l[i - 2] * w[i - 2];
    b[i - 1] = (b[i - 1] - A->l[i - 2] * b[i - 2]) / t;
  }
  for (int i = n - 1; i >= 1; --i) b[i - 1] = b[i - 1] - w[i - 1] * b[i];
  free(w);
}

/* MatVecT_1D (TriDiagT_Mod.f90:113-133) */
static void matvec_1d(double* y, const T1* A, const double* x) {
  const int n = A->n1;
  if (n > 1) {
    y[0] = A->d[0] * x[0] + A->u[0] * x[1];
    for (int i = 2; i <= n - 1; ++i) y[i - 1] = A->l[i - 2] * x[i - 2] + A->d[i - 1] * x[i - 1] + A->u[i - 1] * x[i];
    y[n - 1] = A->l[n - 2] * x[n - 2] + A->d[n - 1] * x[n - 1];
  } else {
    y[0] = A->d[0] * x[0];
  }
}

/* MatVecT_2D (TriDiagT_Mod.f90:405-431); x, y are (n1, n2) */
static void matvec_2d(double* y, const T2* A, const double* x) {
  const int n1 = A->n1, n2 = A->n2;
  matvec_1d(y, &A->col[0], x);
  if (n2 > 1) {
    for (int i = 0; i < n1; ++i) y[i] = y[i] + A->u[i] * x[i + n1];
    for (int j = 2; j <= n2 - 1; ++j) {
      matvec_1d(y + (size_t)n1 * (j - 1), &A->col[j - 1], x + (size_t)n1 * (j - 1));
      for (int i = 0; i < n1; ++i)
        y[i + (size_t)n1 * (j - 1)] = y[i + (size_t)n1 * (j - 1)] + A->l[i + (size_t)n1 * (j - 2)] * x[i + (size_t)n1 * (j - 2)] +
                                      A->u[i + (size_t)n1 * (j - 1)] * x[i + (size_t)n1 * j];
    }
    matvec_1d(y + (size_t)n1 * (n2 - 1), &A->col[n2 - 1], x + (size_t)n1 * (n2 - 1));
    for (int i = 0; i < n1; ++i)
      y[i + (size_t)n1 * (n2 - 1)] = y[i + (size_t)n1 * (n2 - 1)] + A->l[i + (size_t)n1 * (n2 - 2)] * x[i + (size_t)n1 * (n2 - 2)];
  }
}

/* MatVecT_3D (TriDiagT_Mod.f90:885-917); x, y are (n1, n2, n3) */
static void matvec_3d(double* y, const T3* A, const double* x) {
  const int n3 = A->n3;
  const size_t m = (size_t)A->n1 * A->n2;
  matvec_2d(y, A->pl[0], x);
  if (n3 > 1) {
    for (size_t q = 0; q < m; ++q) y[q] = y[q] + A->u[q] * x[q + m];
    for (int k = 2; k <= n3 - 1; ++k) {
      matvec_2d(y + m * (k - 1), A->pl[k - 1], x + m * (k - 1));
      for (size_t q = 0; q < m; ++q)
        y[q + m * (k - 1)] = y[q + m * (k - 1)] + A->l[q + m * (k - 2)] * x[q + m * (k - 2)] + A->u[q + m * (k - 1)] * x[q + m * k];
    }
    matvec_2d(y + m * (n3 - 1), A->pl[n3 - 1], x + m * (n3 - 1));
    for (size_t q = 0; q < m; ++q) y[q + m * (n3 - 1)] = y[q + m * (n3 - 1)] + A->l[q + m * (n3 - 2)] * x[q + m * (n3 - 2)];
  }
}

#define X(i, j) x[(i) + (size_t)n1 * ((j) - 1)]
#define B(i, j) b[(i) + (size_t)n1 * ((j) - 1)]
#define U(i, j) A->u[(i) + (size_t)n1 * ((j) - 1)]
#define L(i, j) A->l[(i) + (size_t)n1 * ((j) - 1)]

/* GaussSeidel_2D, reference order (TriDiagT_Mod.f90:433-471) */
static void gs_2d_ref(const T2* A, const double* b, double* x, int gi) {
  const int n1 = A->n1, n2 = A->n2;
  double* t = zalloc(n1);
  if (n2 > 1) {
    for (int it = 0; it < gi; ++it) {
      for (int i = 0; i < n1; ++i) t[i] = B(i, 1);
      for (int j = 1; j <= n2 - 1; ++j) {
        for (int i = 0; i < n1; ++i) X(i, j) = t[i] - U(i, j) * X(i, j + 1);
        solve_1d(&A->col[j - 1], &X(0, j));
        for (int i = 0; i < n1; ++i) t[i] = B(i, j + 1) - L(i, j) * X(i, j);
      }
      for (int i = 0; i < n1; ++i) X(i, n2) = t[i];
      solve_1d(&A->col[n2 - 1], &X(0, n2));
      for (int i = 0; i < n1; ++i) t[i] = B(i, n2 - 1) - U(i, n2 - 1) * X(i, n2);
      for (int j = n2 - 1; j >= 2; --j) {
        for (int i = 0; i < n1; ++i) X(i, j) = t[i] - L(i, j - 1) * X(i, j - 1);
        solve_1d(&A->col[j - 1], &X(0, j));
        for (int i = 0; i < n1; ++i) t[i] = B(i, j - 1) - U(i, j - 1) * X(i, j);
      }
    }
    for (int i = 0; i < n1; ++i) X(i, 1) = t[i];
    solve_1d(&A->col[0], &X(0, 1));
  } else {
    for (int i = 0; i < n1; ++i) X(i, 1) = B(i, 1);
    solve_1d(&A->col[0], &X(0, 1));
  }
  free(t);
}

/* One zebra half-sweep over the x-lines j of parity c (j-1 = c mod 2):
 * forward form rhs = (b - l x_{j-1}) - u x_{j+1}, backward form
 * rhs = (b - u x_{j+1}) - l x_{j-1} (the reference's two operation orders),
 * each followed by Solve_1D. */
static void gs_2d_half(const T2* A, const double* b, double* x, int c, int fwd) {
  const int n1 = A->n1, n2 = A->n2;
  for (int j = 1 + c; j <= n2; j += 2) {
    for (int i = 0; i < n1; ++i) {
      double t = B(i, j);
      if (fwd) {
        if (j > 1) t = t - L(i, j - 1) * X(i, j - 1);
        if (j < n2) t = t - U(i, j) * X(i, j + 1);
      } else {
        if (j < n2) t = t - U(i, j) * X(i, j + 1);
        if (j > 1) t = t - L(i, j - 1) * X(i, j - 1);
      }
      X(i, j) = t;
    }
    solve_1d(&A->col[j - 1], &X(0, j));
  }
}

/* GaussSeidel_2D in zebra order: per iteration the half-sweeps
 * (parity 0 fwd, parity 1 fwd, parity 1 bwd, parity 0 bwd). */
static void gs_2d_zebra(const T2* A, const double* b, double* x, int gi) {
  const int n1 = A->n1, n2 = A->n2;
  if (n2 > 1) {
    for (int it = 0; it < gi; ++it) {
      gs_2d_half(A, b, x, 0, 1);
      gs_2d_half(A, b, x, 1, 1);
      gs_2d_half(A, b, x, 1, 0);
      gs_2d_half(A, b, x, 0, 0);
    }
  } else {
    for (int i = 0; i < n1; ++i) X(i, 1) = B(i, 1);
    solve_1d(&A->col[0], &X(0, 1));
  }
}
#undef X
#undef B
#undef U
#undef L

/* RestrictT_2D / ProlongateT_2D (TriDiagT_Mod.f90:553-589) */
static void restrict_2d(const double* res, int n1, int n2, double* rc) {
  const int c1 = cdiv2(n1), c2 = cdiv2(n2);
  memset(rc, 0, sizeof(double) * (size_t)c1 * c2);
  for (int i1 = 1; i1 <= n1; ++i1) {
    int i1C = (i1 + 1) / 2;
    for (int i2 = 1; i2 <= n2; ++i2) {
      int i2C = (i2 + 1) / 2;
      rc[(i1C - 1) + (size_t)c1 * (i2C - 1)] = rc[(i1C - 1) + (size_t)c1 * (i2C - 1)] + res[(i1 - 1) + (size_t)n1 * (i2 - 1)];
    }
  }
}

static void prolong_2d(const double* xc, int n1, int n2, double* x) {
  const int c1 = cdiv2(n1);
  for (int i1 = 1; i1 <= n1; ++i1)
    for (int i2 = 1; i2 <= n2; ++i2) x[(i1 - 1) + (size_t)n1 * (i2 - 1)] = xc[((i1 + 1) / 2 - 1) + (size_t)c1 * ((i2 + 1) / 2 - 1)];
}

/* Multigrid_2D (TriDiagT_Mod.f90:490-551) */
static void multigrid_2d(const PrjPar* p, T2* A, const double* b, double* x) {
  T2* a = A;
  const double* bl = b;
  double* xl = x;
  int gi = 1;
  for (;;) {
    if (p->zebra)
      gs_2d_zebra(a, bl, xl, gi);
    else
      gs_2d_ref(a, bl, xl, gi);
    gi += p->gauss_iter2;
    if (a->coarse) {
      const size_t m = (size_t)a->n1 * a->n2;
      matvec_2d(a->res, a, xl);
      for (size_t q = 0; q < m; ++q) a->res[q] = bl[q] - a->res[q];
      restrict_2d(a->res, a->n1, a->n2, a->resc);
      bl = a->resc;
      xl = a->xc;
      memset(xl, 0, sizeof(double) * (size_t)cdiv2(a->n1) * cdiv2(a->n2));
      a = a->coarse;
    } else {
      gi -= p->gauss_iter2;
      break;
    }
  }
  for (;;) {
    if (p->zebra)
      gs_2d_zebra(a, bl, xl, gi);
    else
      gs_2d_ref(a, bl, xl, gi);
    gi -= p->gauss_iter2;
    if (a->fine) {
      a = a->fine;
      prolong_2d(xl, a->n1, a->n2, a->res);
      if (a->fine) {
        xl = a->fine->xc;
        bl = a->fine->resc;
      } else {
        xl = x;
        bl = b;
      }
      const size_t m = (size_t)a->n1 * a->n2;
      for (size_t q = 0; q < m; ++q) xl[q] = xl[q] + a->res[q];
    } else {
      break;
    }
  }
}

/* Solve_2D (TriDiagT_Mod.f90:475-488) */
static void solve_2d(const PrjPar* p, T2* A, const double* b, double* x) {
  for (int it = 0; it < p->mult_iter2; ++it) multigrid_2d(p, A, b, x);
}

#define XP(k) (x + m * ((k) - 1))
#define BP(k) (b + m * ((k) - 1))
#define UP(k) (A->u + m * ((k) - 1))
#define LP(k) (A->l + m * ((k) - 1))

/* GaussSeidel_3D, reference order (TriDiagT_Mod.f90:951-1007) */
static void gs_3d_ref(const PrjPar* p, T3* A, const double* b, double* x, int gi) {
  const int n3 = A->n3;
  const size_t m = (size_t)A->n1 * A->n2;
  double* t = zalloc(m);
  if (n3 > 1) {
    for (int it = 0; it < gi; ++it) {
      for (size_t q = 0; q < m; ++q) t[q] = BP(1)[q];
      for (int k = 1; k <= n3 - 1; ++k) {
        for (size_t q = 0; q < m; ++q) t[q] = t[q] - UP(k)[q] * XP(k + 1)[q];
        solve_2d(p, A->pl[k - 1], t, XP(k));
        for (size_t q = 0; q < m; ++q) t[q] = BP(k + 1)[q] - LP(k)[q] * XP(k)[q];
      }
      solve_2d(p, A->pl[n3 - 1], t, XP(n3));
      for (size_t q = 0; q < m; ++q) t[q] = BP(n3 - 1)[q] - UP(n3 - 1)[q] * XP(n3)[q];
      for (int k = n3 - 1; k >= 2; --k) {
        for (size_t q = 0; q < m; ++q) t[q] = t[q] - LP(k - 1)[q] * XP(k - 1)[q];
        solve_2d(p, A->pl[k - 1], t, XP(k));
        for (size_t q = 0; q < m; ++q) t[q] = BP(k - 1)[q] - UP(k - 1)[q] * XP(k)[q];
      }
    }
    solve_2d(p, A->pl[0], t, XP(1));
    for (size_t q = 0; q < m; ++q) t[q] = BP(n3)[q] - LP(n3 - 1)[q] * XP(n3 - 1)[q];
    solve_2d(p, A->pl[n3 - 1], t, XP(n3));
  } else {
    solve_2d(p, A->pl[0], BP(1), XP(1));
  }
  free(t);
}

/* GaussSeidel_3D in zebra order over the planes (see gs_2d_zebra); the plane
 * right-hand sides use the reference's forward/backward operation order. */
static void gs_3d_zebra(const PrjPar* p, T3* A, const double* b, double* x, int gi) {
  const int n3 = A->n3;
  const size_t m = (size_t)A->n1 * A->n2;
  double* t = zalloc(m);
  if (n3 > 1) {
    static const int order[4][2] = {{0, 1}, {1, 1}, {1, 0}, {0, 0}};
    for (int it = 0; it < gi; ++it) {
      for (int hs = 0; hs < 4; ++hs) {
        const int c = order[hs][0], fwd = order[hs][1];
        for (int k = 1 + c; k <= n3; k += 2) {
          for (size_t q = 0; q < m; ++q) {
            double v = BP(k)[q];
            if (fwd) {
              if (k > 1) v = v - LP(k - 1)[q] * XP(k - 1)[q];
              if (k < n3) v = v - UP(k)[q] * XP(k + 1)[q];
            } else {
              if (k < n3) v = v - UP(k)[q] * XP(k + 1)[q];
              if (k > 1) v = v - LP(k - 1)[q] * XP(k - 1)[q];
            }
            t[q] = v;
          }
          solve_2d(p, A->pl[k - 1], t, XP(k));
        }
      }
    }
  } else {
    solve_2d(p, A->pl[0], BP(1), XP(1));
  }
  free(t);
}
#undef XP
#undef BP
#undef UP
#undef LP

static void restrict_3d(const double* res, int n1, int n2, int n3, double* rc) {
  const int c1 = cdiv2(n1), c2 = cdiv2(n2), c3 = cdiv2(n3);
  memset(rc, 0, sizeof(double) * (size_t)c1 * c2 * c3);
  for (int i1 = 1; i1 <= n1; ++i1) {
    int a = (i1 + 1) / 2;
    for (int i2 = 1; i2 <= n2; ++i2) {
      int b = (i2 + 1) / 2;
      for (int i3 = 1; i3 <= n3; ++i3) {
        int c = (i3 + 1) / 2;
        size_t qc = (a - 1) + (size_t)c1 * ((b - 1) + (size_t)c2 * (c - 1));
        rc[qc] = rc[qc] + res[(i1 - 1) + (size_t)n1 * ((i2 - 1) + (size_t)n2 * (i3 - 1))];
      }
    }
  }
}

static void prolong_3d(const double* xc, int n1, int n2, int n3, double* x) {
  const int c1 = cdiv2(n1), c2 = cdiv2(n2);
  for (int i1 = 1; i1 <= n1; ++i1)
    for (int i2 = 1; i2 <= n2; ++i2)
      for (int i3 = 1; i3 <= n3; ++i3)
        x[(i1 - 1) + (size_t)n1 * ((i2 - 1) + (size_t)n2 * (i3 - 1))] =
            xc[((i1 + 1) / 2 - 1) + (size_t)c1 * (((i2 + 1) / 2 - 1) + (size_t)c2 * ((i3 + 1) / 2 - 1))];
}

/* Multigrid_3D (TriDiagT_Mod.f90:1009-1071) */
static void multigrid_3d(const PrjPar* p, T3* A, const double* b, double* x) {
  T3* a = A;
  const double* bl = b;
  double* xl = x;
  int gi = 1;
  for (;;) {
    if (p->zebra)
      gs_3d_zebra(p, a, bl, xl, gi);
    else
      gs_3d_ref(p, a, bl, xl, gi);
    gi += p->gauss_iter3;
    if (a->coarse) {
      const size_t m = (size_t)a->n1 * a->n2 * a->n3;
      matvec_3d(a->res, a, xl);
      for (size_t q = 0; q < m; ++q) a->res[q] = bl[q] - a->res[q];
      restrict_3d(a->res, a->n1, a->n2, a->n3, a->resc);
      bl = a->resc;
      xl = a->xc;
      memset(xl, 0, sizeof(double) * (size_t)cdiv2(a->n1) * cdiv2(a->n2) * cdiv2(a->n3));
      a = a->coarse;
    } else {
      gi -= p->gauss_iter3;
      break;
    }
  }
  for (;;) {
    if (p->zebra)
      gs_3d_zebra(p, a, bl, xl, gi);
    else
      gs_3d_ref(p, a, bl, xl, gi);
    gi -= p->gauss_iter3;
    if (a->fine) {
      a = a->fine;
      prolong_3d(xl, a->n1, a->n2, a->n3, a->res);
      if (a->fine) {
        xl = a->fine->xc;
        bl = a->fine->resc;
      } else {
        xl = x;
        bl = b;
      }
      const size_t m = (size_t)a->n1 * a->n2 * a->n3;
      for (size_t q = 0; q < m; ++q) xl[q] = xl[q] + a->res[q];
    } else {
      break;
    }
  }
}

/* ---------------------------------------------------------------------- */
/* Reverse / ReverseBack for cell fields: natural (x,y,z) <-> (z,x,y) */
static void reverse(const Proj* h, const double* nat, double* rev) {
  const int nx = h->par.nx, ny = h->par.ny, nz = h->par.nz;
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) rev[z + (size_t)nz * (x + (size_t)nx * y)] = nat[x + (size_t)nx * (y + (size_t)ny * z)];
}

static void reverse_back(const Proj* h, const double* rev, double* nat) {
  const int nx = h->par.nx, ny = h->par.ny, nz = h->par.nz;
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) nat[x + (size_t)nx * (y + (size_t)ny * z)] = rev[z + (size_t)nz * (x + (size_t)nx * y)];
}

/* ---------------------------------------------------------------------- */
/* Public oracle API */

/* ipar = {nx, ny, nz, RefLevel, GaussIter2, GaussIter3, MultIter2, MultIter3,
 * zebra}; dpar = {FacAnela}.  Geometry/weight arrays (natural Fortran
 * layouts, 0-based):
 *   fu  FU native (ix0-1:ix1+1, iy0+1:iy1, iz0+1:iz1)   (nx+3)*ny*nz
 *   fv  FV native (ix0+1:ix1, iy0-1:iy1+1, iz0+1:iz1)   nx*(ny+3)*nz
 *   fw  FW native (ix0+1:ix1, iy0+1:iy1, iz0-1:iz1+1)   nx*ny*(nz+3)
 *   volc padded (nx+2)*(ny+2)*(nz+2)
 *   dtu,duu uF extents (nx+1)*ny*nz; dtv,duv nx*(ny+1)*nz; dtw,duw nx*ny*(nz+1)
 *   dut, dtt interior nx*ny*nz
 *   dx[nx], dy[ny], dz[nz]; metr = 6 arrays back to back
 *     MetrXY[ny], MetrXZ[nz], MetrYX[nx], MetrYZ[nz], MetrZX[nx], MetrZY[ny]
 */
void* ora_proj_create(const int* ipar, const double* dpar, const double* fu, const double* fv, const double* fw,
                      const double* volc, const double* dtu, const double* dtv, const double* dtw, const double* duu,
                      const double* duv, const double* duw, const double* dut, const double* dtt, const double* dx,
                      const double* dy, const double* dz, const double* metr) {
  Proj* h = (Proj*)calloc(1, sizeof(Proj));
  PrjPar* p = &h->par;
  p->nx = ipar[0];
  p->ny = ipar[1];
  p->nz = ipar[2];
  p->ref_level = ipar[3];
  p->gauss_iter2 = ipar[4];
  p->gauss_iter3 = ipar[5];
  p->mult_iter2 = ipar[6];
  p->mult_iter3 = ipar[7];
  p->zebra = ipar[8];
  p->fac_anela = dpar[0];
  /* SetFactorN: all sides Neumann (Fac = 0) */
  p->fac1_l = p->fac1_r = p->fac2_l = p->fac2_r = p->fac3_l = p->fac3_r = 0.0;
  h->per_x = ipar[9];
  h->per_y = ipar[10];
  h->per_z = ipar[11];
  h->prefac2 = dpar[1];
  const int nx = p->nx, ny = p->ny, nz = p->nz;
  const size_t nc = (size_t)nx * ny * nz;
  {
    const int per[3] = {h->per_x, h->per_y, h->per_z};
    const size_t fsz[3] = {(size_t)ny * nz, (size_t)nx * nz, (size_t)nx * ny};
    size_t o = nc;
    for (int side = 0; side < 6; ++side) {
      if (per[side / 2]) {
        h->off[side] = (long)o;
        o += fsz[side / 2];
      } else {
        h->off[side] = -1;
      }
    }
    h->nvec = o;
  }
  h->fu = zalloc((size_t)(nx + 1) * ny * nz);
  h->fv = zalloc((size_t)nx * (ny + 1) * nz);
  h->fw = zalloc((size_t)nx * ny * (nz + 1));
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j)
      for (int i = 0; i <= nx; ++i)
        h->fu[i + (size_t)(nx + 1) * ((j - 1) + (size_t)ny * (k - 1))] = fu[(i + 1) + (size_t)(nx + 3) * ((j - 1) + (size_t)ny * (k - 1))];
  for (int k = 1; k <= nz; ++k)
    for (int j = 0; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i)
        h->fv[(i - 1) + (size_t)nx * (j + (size_t)(ny + 1) * (k - 1))] = fv[(i - 1) + (size_t)nx * ((j + 1) + (size_t)(ny + 3) * (k - 1))];
  for (int k = 0; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i)
        h->fw[(i - 1) + (size_t)nx * ((j - 1) + (size_t)ny * k)] = fw[(i - 1) + (size_t)nx * ((j - 1) + (size_t)ny * (k + 1))];
#define DUP(dst, src, n)                    \
  do {                                      \
    dst = zalloc(n);                        \
    memcpy(dst, src, sizeof(double) * (n)); \
  } while (0)
  DUP(h->dtu, dtu, (size_t)(nx + 1) * ny * nz);
  DUP(h->duu, duu, (size_t)(nx + 1) * ny * nz);
  DUP(h->dtv, dtv, (size_t)nx * (ny + 1) * nz);
  DUP(h->duv, duv, (size_t)nx * (ny + 1) * nz);
  DUP(h->dtw, dtw, (size_t)nx * ny * (nz + 1));
  DUP(h->duw, duw, (size_t)nx * ny * (nz + 1));
  DUP(h->dut, dut, nc);
  DUP(h->dtt, dtt, nc);
  DUP(h->dx, dx, (size_t)nx);
  DUP(h->dy, dy, (size_t)ny);
  DUP(h->dz, dz, (size_t)nz);
  DUP(h->mxy, metr, (size_t)ny);
  DUP(h->mxz, metr + ny, (size_t)nz);
  DUP(h->myx, metr + ny + nz, (size_t)nx);
  DUP(h->myz, metr + ny + nz + nx, (size_t)nz);
  DUP(h->mzx, metr + ny + 2 * nz + nx, (size_t)nx);
  DUP(h->mzy, metr + ny + 2 * nz + 2 * nx, (size_t)ny);
  DUP(h->volp, volc, (size_t)(nx + 2) * (ny + 2) * (nz + 2));
#undef DUP
  h->vol = zalloc(nc);
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i)
        h->vol[(i - 1) + (size_t)nx * ((j - 1) + (size_t)ny * (k - 1))] = volc[i + (size_t)(nx + 2) * (j + (size_t)(ny + 2) * k)];
  h->n1 = nz;
  h->n2 = nx;
  h->n3 = ny;
  return h;
}

void ora_proj_destroy(void* hv) {
  Proj* h = (Proj*)hv;
  if (!h) return;
  t3_free(h->A);
  t3_free(h->AD);
  double* p[] = {h->fu, h->fv, h->fw, h->dtu, h->dtv, h->dtw, h->duu, h->duv, h->duw, h->dut, h->dtt, h->vol, h->volp,
                 h->dx, h->dy, h->dz, h->mxy, h->mxz, h->myx, h->myz, h->mzx, h->mzy};
  for (size_t i = 0; i < sizeof(p) / sizeof(p[0]); ++i) free(p[i]);
  free(h);
}

void ora_proj_set_zebra(void* hv, int zebra) { ((Proj*)hv)->par.zebra = zebra; }

/* Length of a PressureVelocity vector: nx*ny*nz plus the face unknowns. */
long ora_proj_nvec(void* hv) { return (long)((Proj*)hv)->nvec; }

/* The semi-coarsening hierarchy of LaplTFullCompute (all 3D levels, the
 * plane levels of each) from the reversed fine fields g, with the boundary
 * factors of p. */
static T3* build_hierarchy(const PrjPar* p, const Fields* g, double bd2, int n1, int n2, int n3) {
  const int R = p->ref_level;
  T3 *top = NULL, *cur3 = NULL;
  for (int L3 = 0; L3 < R; ++L3) {
    const int s = (1 << L3) - 1;
    const int n1C = (n1 + s) / (s + 1), n2C = (n2 + s) / (s + 1), n3C = (n3 + s) / (s + 1);
    Fields c;
    fields_alloc(&c, n1C, n2C, n3C);
    coarsen(g, &c, s, s, s);
    T3* a = t3_alloc(n3C, n2C, n1C);
    compute_3d(p, bd2, a->pl, a->u, a->l, n3C, &c, 1);
    fields_free(&c);
    if (!cur3) {
      top = a;
    } else {
      cur3->coarse = a;
      a->fine = cur3;
    }
    cur3 = a;
    /* the coarse plane levels of this 3D level */
    T2** cur2 = (T2**)calloc(n3C, sizeof(T2*));
    for (int k = 0; k < n3C; ++k) cur2[k] = a->pl[k];
    for (int L2 = L3 + 1; L2 < R; ++L2) {
      const int s2 = (1 << L2) - 1;
      const int m1 = (n1 + s2) / (s2 + 1), m2 = (n2 + s2) / (s2 + 1);
      Fields c2;
      fields_alloc(&c2, m1, m2, n3C);
      coarsen(g, &c2, s2, s2, s);
      T2** neu = (T2**)calloc(n3C, sizeof(T2*));
      for (int k = 0; k < n3C; ++k) {
        neu[k] = t2_alloc(m2, m1);
        cur2[k]->coarse = neu[k];
        neu[k]->fine = cur2[k];
      }
      compute_3d(p, bd2, neu, NULL, NULL, n3C, &c2, 0);
      fields_free(&c2);
      for (int k = 0; k < n3C; ++k) cur2[k] = neu[k];
      free(neu);
    }
    free(cur2);
  }
  return top;
}

/* LaplTFullCompute (JacAccGrav_Mod.f90:1056-1310) with SetFactorN */
void ora_lapl_compute(void* hv, double beta0, double dtp) {
  Proj* h = (Proj*)hv;
  const PrjPar* p = &h->par;
  const int nx = p->nx, ny = p->ny, nz = p->nz;
  const int n1 = nz, n2 = nx, n3 = ny;
  h->beta0 = beta0;
  h->dtp = dtp;
  const double bd = beta0 * dtp, bd2 = bd * bd;
  t3_free(h->A);
  h->A = NULL;
  /* ReverseWeight / ReverseIncr / ReverseMetr / Reverse of the fine fields */
  Fields g;
  fields_alloc(&g, n1, n2, n3);
  for (int z = 0; z <= nz; ++z)
    for (int y = 1; y <= ny; ++y)
      for (int x = 1; x <= nx; ++x) {
        size_t src = (x - 1) + (size_t)nx * ((y - 1) + (size_t)ny * z), dst = IDX1(&g, z, x, y);
        g.F1[dst] = h->fw[src];
        g.T1_[dst] = h->dtw[src];
        g.U1[dst] = h->duw[src];
      }
  for (int z = 1; z <= nz; ++z)
    for (int y = 1; y <= ny; ++y)
      for (int x = 0; x <= nx; ++x) {
        size_t src = x + (size_t)(nx + 1) * ((y - 1) + (size_t)ny * (z - 1)), dst = IDX2(&g, z, x, y);
        g.F2[dst] = h->fu[src];
        g.T2_[dst] = h->dtu[src];
        g.U2[dst] = h->duu[src];
      }
  for (int z = 1; z <= nz; ++z)
    for (int y = 0; y <= ny; ++y)
      for (int x = 1; x <= nx; ++x) {
        size_t src = (x - 1) + (size_t)nx * (y + (size_t)(ny + 1) * (z - 1)), dst = IDX3(&g, z, x, y);
        g.F3[dst] = h->fv[src];
        g.T3_[dst] = h->dtv[src];
        g.U3[dst] = h->duv[src];
      }
  memcpy(g.d1, h->dz, sizeof(double) * nz);
  memcpy(g.d2, h->dx, sizeof(double) * nx);
  memcpy(g.d3, h->dy, sizeof(double) * ny);
  /* ReverseMetr with (xOrder,yOrder,zOrder) = (2,3,1) (Reverse_Mod.f90:441-541) */
  memcpy(g.m12, h->mzx, sizeof(double) * nx);
  memcpy(g.m13, h->mzy, sizeof(double) * ny);
  memcpy(g.m21, h->mxz, sizeof(double) * nz);
  memcpy(g.m23, h->mxy, sizeof(double) * ny);
  memcpy(g.m31, h->myz, sizeof(double) * nz);
  memcpy(g.m32, h->myx, sizeof(double) * nx);
  reverse(h, h->dut, g.dut);
  reverse(h, h->vol, g.vol);

  /* LaplNeumann with SetFactorN (p's factors are 0) */
  h->A = build_hierarchy(p, &g, bd2, n1, n2, n3);
  /* LaplDirichlet with SetFactorD: 2 on the periodic sides, 0 on the closed
   * ones (their velocity rule is not 'OutFlow'); order (z,x,y) -> factors
   * 1 = bottom/top, 2 = west/east, 3 = south/north */
  t3_free(h->AD);
  h->AD = NULL;
  if (h->per_x || h->per_y || h->per_z) {
    PrjPar pd = *p;
    pd.fac1_l = pd.fac1_r = h->per_z ? 2.0 : 0.0;
    pd.fac2_l = pd.fac2_r = h->per_x ? 2.0 : 0.0;
    pd.fac3_l = pd.fac3_r = h->per_y ? 2.0 : 0.0;
    h->AD = build_hierarchy(&pd, &g, bd2, n1, n2, n3);
  }
  fields_free(&g);
}

/* Export one assembled array in natural reversed order (i1 fastest, then i2,
 * then plane): which 0 d, 1 u (z), 2 l (z), 3 u (x), 4 l (x), 5 u (y), 6 l (y);
 * entries past the end of a coupling (last row / line) are 0.  L3 = 3D level,
 * L2 >= L3 = plane level.  Returns the number of values (-1: no such level). */
static long lapl_get(T3* a, int L3, int L2, int which, double* out);
long ora_lapl_get(void* hv, int L3, int L2, int which, double* out) {
  return lapl_get(((Proj*)hv)->A, L3, L2, which, out);
}
/* the same for LaplDirichlet (periodic blocks; -1 without one) */
long ora_lapl_get_dirichlet(void* hv, int L3, int L2, int which, double* out) {
  return lapl_get(((Proj*)hv)->AD, L3, L2, which, out);
}
static long lapl_get(T3* a, int L3, int L2, int which, double* out) {
  for (int q = 0; q < L3 && a; ++q) a = a->coarse;
  if (!a) return -1;
  const int n3 = a->n3;
  long cnt = 0;
  if (which >= 5) {
    if (L2 != L3) return -1;
    const size_t m = (size_t)a->n1 * a->n2;
    for (int k = 0; k < n3; ++k)
      for (size_t q = 0; q < m; ++q) {
        double v = 0.0;
        if (k < n3 - 1) v = which == 5 ? a->u[q + m * k] : a->l[q + m * k];
        if (out) out[cnt] = v;
        ++cnt;
      }
    return cnt;
  }
  for (int k = 0; k < n3; ++k) {
    T2* pl = a->pl[k];
    for (int q = L3; q < L2 && pl; ++q) pl = pl->coarse;
    if (!pl) return -1;
    const int n1 = pl->n1, n2 = pl->n2;
    if (which <= 2) {
      for (int j = 0; j < n2; ++j) {
        const T1* c = &pl->col[j];
        for (int i = 0; i < n1; ++i) {
          double v = 0.0;
          if (which == 0)
            v = c->d[i];
          else if (i < n1 - 1)
            v = which == 1 ? c->u[i] : c->l[i];
          if (out) out[cnt] = v;
          ++cnt;
        }
      }
    } else {
      for (int j = 0; j < n2; ++j)
        for (int i = 0; i < n1; ++i) {
          double v = 0.0;
          if (j < n2 - 1) v = which == 3 ? pl->u[i + (size_t)n1 * j] : pl->l[i + (size_t)n1 * j];
          if (out) out[cnt] = v;
          ++cnt;
        }
    }
  }
  return cnt;
}

/* MatVecP_Tri (JacAccGrav_Mod.f90:531-545): y = A x through Reverse /
 * MatVecT_3D / ReverseBack; x, y natural interior (nx,ny,nz). */
void ora_lapl_matvec(void* hv, const double* x, double* y) {
  Proj* h = (Proj*)hv;
  const size_t n = (size_t)h->par.nx * h->par.ny * h->par.nz;
  double* xr = zalloc(n);
  double* yr = zalloc(n);
  reverse(h, x, xr);
  matvec_3d(yr, h->A, xr);
  reverse_back(h, yr, y);
  free(xr);
  free(yr);
}

/* VCycleCG, MatrixT branch (JacAccGrav_Mod.f90:4466-4517) on LaplNeumann:
 * x = Solve_3D(A, b) from a zero start. */
static void vcycle_on(Proj* h, T3* A, const double* b, double* x);
void ora_lapl_vcycle(void* hv, const double* b, double* x) {
  Proj* h = (Proj*)hv;
  vcycle_on(h, h->A, b, x);
}

/* the same on LaplDirichlet (periodic blocks only; returns -1 otherwise) */
int ora_lapl_vcycle_dirichlet(void* hv, const double* b, double* x) {
  Proj* h = (Proj*)hv;
  if (!h->AD) return -1;
  vcycle_on(h, h->AD, b, x);
  return 0;
}

/* Solve_3D from a zero start on hierarchy A (VCycleCG, MatrixT branch,
 * JacAccGrav_Mod.f90:4466-4517): x = Solve(A, b), natural interior order. */
static void vcycle_on(Proj* h, T3* A, const double* b, double* x) {
  const size_t n = (size_t)h->par.nx * h->par.ny * h->par.nz;
  double* r = zalloc(n);
  double* xc = zalloc(n);
  reverse(h, b, r);
  for (int it = 0; it < h->par.mult_iter3; ++it) multigrid_3d(&h->par, A, r, xc);
  reverse_back(h, xc, x);
  free(r);
  free(xc);
}

/* Index helpers of the interior cells and faces (1-based logical indices). */
#define PV_C(i, j, k) ((size_t)((i) - 1) + (size_t)nx * ((size_t)((j) - 1) + (size_t)ny * ((k) - 1)))
#define PV_U(i, j, k) ((size_t)(i) + (size_t)(nx + 1) * ((size_t)((j) - 1) + (size_t)ny * ((k) - 1)))
#define PV_V(i, j, k) ((size_t)((i) - 1) + (size_t)nx * ((size_t)(j) + (size_t)(ny + 1) * ((k) - 1)))
#define PV_W(i, j, k) ((size_t)((i) - 1) + (size_t)nx * ((size_t)((j) - 1) + (size_t)ny * (k)))
#define FX(j, k) ((size_t)((j) - 1) + (size_t)ny * ((k) - 1)) /* u_w, u_e (iy, iz) */
#define FY(i, k) ((size_t)((i) - 1) + (size_t)nx * ((k) - 1)) /* v_s, v_n (ix, iz) */
#define FZ(i, j) ((size_t)((i) - 1) + (size_t)nx * ((j) - 1)) /* w_b, w_t (ix, iy) */

/* The pressure term of the boundary face unknowns of one side, as the
 * reference's array statements:
 *   p(ix0+1) += beta0*dtP*FU(ix0)*DTU(ix0)*DTT(ix0+1)*u_w, p(ix1) -= ... u_e, ...
 * (MatVecFull MATRIX/MatVec_Mod.f90:224-255 and b1pBTx2Full
 * MATRIX/PreCond_Mod.f90:642-665); v holds the face unknowns. */
static void face_to_p_side(const Proj* h, int side, double* p, const double* v) {
  const int nx = h->par.nx, ny = h->par.ny, nz = h->par.nz;
  const double bd = h->beta0 * h->dtp;
  const long o = h->off[side];
  if (o < 0) return;
  switch (side) {
    case 0:
      for (int k = 1; k <= nz; ++k)
        for (int j = 1; j <= ny; ++j) {
          const size_t q = PV_U(0, j, k);
          p[PV_C(1, j, k)] = p[PV_C(1, j, k)] + bd * h->fu[q] * h->dtu[q] * h->dtt[PV_C(1, j, k)] * v[o + FX(j, k)];
        }
      break;
    case 1:
      for (int k = 1; k <= nz; ++k)
        for (int j = 1; j <= ny; ++j) {
          const size_t q = PV_U(nx, j, k);
          p[PV_C(nx, j, k)] = p[PV_C(nx, j, k)] - bd * h->fu[q] * h->dtu[q] * h->dtt[PV_C(nx, j, k)] * v[o + FX(j, k)];
        }
      break;
    case 2:
      for (int k = 1; k <= nz; ++k)
        for (int i = 1; i <= nx; ++i) {
          const size_t q = PV_V(i, 0, k);
          p[PV_C(i, 1, k)] = p[PV_C(i, 1, k)] + bd * h->fv[q] * h->dtv[q] * h->dtt[PV_C(i, 1, k)] * v[o + FY(i, k)];
        }
      break;
    case 3:
      for (int k = 1; k <= nz; ++k)
        for (int i = 1; i <= nx; ++i) {
          const size_t q = PV_V(i, ny, k);
          p[PV_C(i, ny, k)] = p[PV_C(i, ny, k)] - bd * h->fv[q] * h->dtv[q] * h->dtt[PV_C(i, ny, k)] * v[o + FY(i, k)];
        }
      break;
    case 4:
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          const size_t q = PV_W(i, j, 0);
          p[PV_C(i, j, 1)] = p[PV_C(i, j, 1)] + bd * h->fw[q] * h->dtw[q] * h->dtt[PV_C(i, j, 1)] * v[o + FZ(i, j)];
        }
      break;
    default:
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          const size_t q = PV_W(i, j, nz);
          p[PV_C(i, j, nz)] = p[PV_C(i, j, nz)] - bd * h->fw[q] * h->dtw[q] * h->dtt[PV_C(i, j, nz)] * v[o + FZ(i, j)];
        }
      break;
  }
}

/* all sides in the order W, E, S, N, B, T */
static void face_to_p(const Proj* h, double* p, const double* v) {
  for (int side = 0; side < 6; ++side) face_to_p_side(h, side, p, v);
}

/* The coupling of a boundary face unknown to the pressure of its cell,
 * beta0*dtP*F*DUT*DUU*p (MatVecFull, b2pBx1Full, SchurPreFull). */
static double face_cp(const Proj* h, int side, int a, int b, const double* p) {
  const int nx = h->par.nx, ny = h->par.ny, nz = h->par.nz;
  const double bd = h->beta0 * h->dtp;
  size_t q, c;
  switch (side) {
    case 0: q = PV_U(0, a, b); c = PV_C(1, a, b); return bd * h->fu[q] * h->dut[c] * h->duu[q] * p[c];
    case 1: q = PV_U(nx, a, b); c = PV_C(nx, a, b); return bd * h->fu[q] * h->dut[c] * h->duu[q] * p[c];
    case 2: q = PV_V(a, 0, b); c = PV_C(a, 1, b); return bd * h->fv[q] * h->dut[c] * h->duv[q] * p[c];
    case 3: q = PV_V(a, ny, b); c = PV_C(a, ny, b); return bd * h->fv[q] * h->dut[c] * h->duv[q] * p[c];
    case 4: q = PV_W(a, b, 0); c = PV_C(a, b, 1); return bd * h->fw[q] * h->dut[c] * h->duw[q] * p[c];
    default: q = PV_W(a, b, nz); c = PV_C(a, b, nz); return bd * h->fw[q] * h->dut[c] * h->duw[q] * p[c];
  }
  (void)nz;
}

/* Half-cell factors of a boundary face unknown, in the two operation orders
 * of the reference: MatVecFull's face equation multiplies
 * Half*Metr1*Metr2*d (then *F*u), SchurPreFull divides by
 * 0.5d0*d*Metr1*Metr2 (then *F + Eps); the w faces have no metric factors. */
static double half_mv(const Proj* h, int side, int a, int b) {
  const int nx = h->par.nx, ny = h->par.ny, nz = h->par.nz;
  switch (side) {
    case 0: return 0.5 * h->mxy[a - 1] * h->mxz[b - 1] * h->dx[0];
    case 1: return 0.5 * h->mxy[a - 1] * h->mxz[b - 1] * h->dx[nx - 1];
    case 2: return 0.5 * h->myx[a - 1] * h->myz[b - 1] * h->dy[0];
    case 3: return 0.5 * h->myx[a - 1] * h->myz[b - 1] * h->dy[ny - 1];
    case 4: return 0.5 * h->dz[0];
    default: return 0.5 * h->dz[nz - 1];
  }
}
static double half_sp(const Proj* h, int side, int a, int b) {
  const int nx = h->par.nx, ny = h->par.ny, nz = h->par.nz;
  switch (side) {
    case 0: return 0.5 * h->dx[0] * h->mxy[a - 1] * h->mxz[b - 1];
    case 1: return 0.5 * h->dx[nx - 1] * h->mxy[a - 1] * h->mxz[b - 1];
    case 2: return 0.5 * h->dy[0] * h->myx[a - 1] * h->myz[b - 1];
    case 3: return 0.5 * h->dy[ny - 1] * h->myx[a - 1] * h->myz[b - 1];
    case 4: return 0.5 * h->dz[0];
    default: return 0.5 * h->dz[nz - 1];
  }
}

/* area of the face of a boundary unknown */
static double face_area(const Proj* h, int side, int a, int b) {
  const int nx = h->par.nx, ny = h->par.ny, nz = h->par.nz;
  switch (side) {
    case 0: return h->fu[PV_U(0, a, b)];
    case 1: return h->fu[PV_U(nx, a, b)];
    case 2: return h->fv[PV_V(a, 0, b)];
    case 3: return h->fv[PV_V(a, ny, b)];
    case 4: return h->fw[PV_W(a, b, 0)];
    default: return h->fw[PV_W(a, b, nz)];
  }
  (void)nz;
}

/* extents (a,b) of the face array of a side: (ny,nz), (nx,nz), (nx,ny) */
static void face_ext(const Proj* h, int side, int* na, int* nb) {
  const int nx = h->par.nx, ny = h->par.ny, nz = h->par.nz;
  *na = side < 2 ? ny : nx;
  *nb = side < 4 ? nz : ny;
}
static size_t face_idx(const Proj* h, int side, int a, int b) {
  const int na = side < 2 ? h->par.ny : h->par.nx;
  return (size_t)(a - 1) + (size_t)na * (b - 1);
}

/* MatVecFull, MultiTriT branch (MatVec_Mod.f90:184-258): b = Zero;
 * b%p = -(A x%p); then per periodic side (W, E, S, N, B, T) the pressure term
 * of the face unknown and the face equation
 *   b%u_w = Half*MetrXY*MetrXZ*dx(ix0+1)*FU(ix0)*x%u_w + beta0*dtP*FU*DUT*DUU*x%p(ix0+1)
 *   b%u_e = Half*MetrXY*MetrXZ*dx(ix1)*FU(ix1)*x%u_e - beta0*dtP*FU*DUT*DUU*x%p(ix1)
 * (w faces without the metric factors). */
static void matvec1(Proj* h, const double* x, double* b) {
  const size_t n = (size_t)h->par.nx * h->par.ny * h->par.nz;
  for (size_t q = n; q < h->nvec; ++q) b[q] = 0.0;
  ora_lapl_matvec(h, x, b);
  for (size_t q = 0; q < n; ++q) b[q] = -b[q];
  for (int side = 0; side < 6; ++side) {
    if (h->off[side] < 0) continue;
    face_to_p_side(h, side, b, x); /* the array statement before the face loop */
    int na, nb;
    face_ext(h, side, &na, &nb);
    for (int bb = 1; bb <= nb; ++bb)
      for (int a = 1; a <= na; ++a) {
        const size_t f = h->off[side] + face_idx(h, side, a, bb);
        const double m = half_mv(h, side, a, bb) * face_area(h, side, a, bb) * x[f];
        const double cp = face_cp(h, side, a, bb, x);
        b[f] = (side & 1) ? m - cp : m + cp;
      }
  }
}

/* Exchange (MODULE/VecPrVel_Mod.f90:855-974) of a block that is its own
 * neighbour: RandCopy's 'iw' branch (ibLoc<=ibnLoc) with CopyFluxVel
 * EqualEqual, u_w = u_w + u_e; u_e = u_w (likewise v_s/v_n, w_b/w_t). */
static void exchange_pv(const Proj* h, double* v) {
  for (int pair = 0; pair < 3; ++pair) {
    const long lo = h->off[2 * pair], hi = h->off[2 * pair + 1];
    if (lo < 0) continue;
    int na, nb;
    face_ext(h, 2 * pair, &na, &nb);
    const size_t m = (size_t)na * nb;
    for (size_t q = 0; q < m; ++q) {
      v[lo + q] = v[lo + q] + v[hi + q];
      v[hi + q] = v[lo + q];
    }
  }
}

/* DOT2 (MODULE/VecPrVel_Mod.f90:112-172): the pressure, then per neighbour
 * the face unknowns of the east/north/top side only (Refine>=RefineNachbar),
 * so a shared face is counted once; neighbour order W, E, S, N, B, T. */
static double dot2(const Proj* h, const double* x, const double* y) {
  const size_t n = (size_t)h->par.nx * h->par.ny * h->par.nz;
  double s = 0.0;
  for (size_t q = 0; q < n; ++q) s = s + x[q] * y[q];
  for (int side = 1; side < 6; side += 2) {
    if (h->off[side] < 0) continue;
    int na, nb;
    face_ext(h, side, &na, &nb);
    const size_t m = (size_t)na * nb;
    double t = 0.0;
    for (size_t q = 0; q < m; ++q) t = t + x[h->off[side] + q] * y[h->off[side] + q];
    s = s + t;
  }
  return s;
}

/* PSolve1 (PreCond_Mod.f90:1555-1571): b=x; PressurePre(b,x); b2pBx1Full;
 * Exchange; SchurPreFull; Exchange; b1pBTx2Full; PressurePre(b,b).
 * SchurPreFull saves b%p and restores it at the end, and b1pBTx2Full then
 * overwrites it with -x%p, so the saved value never matters; without face
 * unknowns only the last two steps change b. */
static void psolve1(Proj* h, double* b, const double* x) {
  const size_t n = (size_t)h->par.nx * h->par.ny * h->par.nz;
  const double eps = EPS;
  memcpy(b, x, sizeof(double) * h->nvec);
  if (h->nvec > n) {
    vcycle_on(h, h->A, x, b); /* PressurePre(b,x) */
    /* b2pBx1Full (PreCond_Mod.f90:694-728): b%u_w = x%u_w + beta0*dtP*FU*DUT*DUU*b%p(ix0+1), ... */
    for (int side = 0; side < 6; ++side) {
      if (h->off[side] < 0) continue;
      int na, nb;
      face_ext(h, side, &na, &nb);
      for (int bb = 1; bb <= nb; ++bb)
        for (int a = 1; a <= na; ++a) {
          const size_t f = h->off[side] + face_idx(h, side, a, bb);
          const double cp = face_cp(h, side, a, bb, b);
          b[f] = (side & 1) ? x[f] - cp : x[f] + cp;
        }
    }
    exchange_pv(h, b);
    /* SchurPreFull (PreCond_Mod.f90:138-216, 303-326, 327-404): the face
     * unknowns scaled by the half-cell mass into a pressure right-hand side,
     * one Solve_3D on LaplDirichlet, then the faces from that pressure */
    double* r = zalloc(n);
    double* rp = zalloc(n);
    {
      const int nx = h->par.nx, ny = h->par.ny, nz = h->par.nz;
      const double bd = h->beta0 * h->dtp;
      for (int side = 0; side < 6; ++side) {
        if (h->off[side] < 0) continue;
        int na, nb;
        face_ext(h, side, &na, &nb);
        for (int bb = 1; bb <= nb; ++bb)
          for (int a = 1; a <= na; ++a) {
            const size_t f = h->off[side] + face_idx(h, side, a, bb);
            const double F = face_area(h, side, a, bb);
            size_t q, c;
            double dt;
            switch (side) {
              case 0: q = PV_U(0, a, bb); c = PV_C(1, a, bb); dt = h->dtu[q]; break;
              case 1: q = PV_U(nx, a, bb); c = PV_C(nx, a, bb); dt = h->dtu[q]; break;
              case 2: q = PV_V(a, 0, bb); c = PV_C(a, 1, bb); dt = h->dtv[q]; break;
              case 3: q = PV_V(a, ny, bb); c = PV_C(a, ny, bb); dt = h->dtv[q]; break;
              case 4: q = PV_W(a, bb, 0); c = PV_C(a, bb, 1); dt = h->dtw[q]; break;
              default: q = PV_W(a, bb, nz); c = PV_C(a, bb, nz); dt = h->dtw[q]; break;
            }
            const double t = bd * F * dt * h->dtt[c] * b[f] / (half_sp(h, side, a, bb) * F + eps);
            r[c] = (side & 1) ? r[c] - t : r[c] + t;
          }
      }
    }
    vcycle_on(h, h->AD, r, rp);
    for (int side = 0; side < 6; ++side) {
      if (h->off[side] < 0) continue;
      int na, nb;
      face_ext(h, side, &na, &nb);
      for (int bb = 1; bb <= nb; ++bb)
        for (int a = 1; a <= na; ++a) {
          const size_t f = h->off[side] + face_idx(h, side, a, bb);
          const double cp = face_cp(h, side, a, bb, rp);
          const double den = half_sp(h, side, a, bb) * face_area(h, side, a, bb) + eps;
          b[f] = (side & 1) ? h->prefac2 * (b[f] + cp) / den : h->prefac2 * (b[f] - cp) / den;
        }
    }
    free(r);
    free(rp);
    exchange_pv(h, b);
  }
  /* b1pBTx2Full (PreCond_Mod.f90:624-665) and PressurePre(b,b) */
  double* tmp = zalloc(n);
  for (size_t q = 0; q < n; ++q) tmp[q] = -x[q];
  face_to_p(h, tmp, b);
  vcycle_on(h, h->A, tmp, b);
  free(tmp);
}

/* FGMRES (SOLU/Iter_Mod.f90:121-199) with StepGMRES = step on
 * PressureVelocity vectors (ora_proj_nvec).  x in/out, b in.  Returns the
 * number of inner steps taken in total; *rho_out = last residual estimate,
 * *rho0_out = initial residual norm. */
int ora_fgmres(void* hv, double* x, const double* b, int maxiter, double tol, int step, double* rho_out,
               double* rho0_out) {
  Proj* h = (Proj*)hv;
  const size_t n = h->nvec;
  double** v = (double**)calloc(step + 1, sizeof(double*));
  double** z = (double**)calloc(step, sizeof(double*));
  for (int i = 0; i <= step; ++i) v[i] = zalloc(n);
  for (int i = 0; i < step; ++i) z[i] = zalloc(n);
  double* H = zalloc((size_t)(step + 1) * step);
  double* c = zalloc(step);
  double* s = zalloc(step);
  double* bh = zalloc(step + 1);
  double* y = zalloc(step);
#define HH(i, j) H[((i) - 1) + (size_t)(step + 1) * ((j) - 1)]
  double rho = 0.0, rho0 = 0.0;
  int steps = 0;
  for (int iter = 1; iter <= maxiter; ++iter) {
    matvec1(h, x, v[0]);
    for (size_t q = 0; q < n; ++q) v[0][q] = b[q] + (-1.0) * v[0][q]; /* DXPBY(b,-One,v) */
    exchange_pv(h, v[0]);
    double beta = sqrt(dot2(h, v[0], v[0]));
    if (iter == 1) rho0 = beta;
    if (beta <= 0.0) break;
    const double sc = 1.0 / beta;
    for (size_t q = 0; q < n; ++q) v[0][q] = sc * v[0][q];
    bh[0] = beta * 1.0;
    int nr = step;
    for (int i = 1; i <= step; ++i) {
      psolve1(h, z[i - 1], v[i - 1]);
      matvec1(h, z[i - 1], v[i]);
      exchange_pv(h, v[i]);
      ++steps;
      for (int k = 1; k <= i; ++k) {
        HH(k, i) = dot2(h, v[k - 1], v[i]);
        for (size_t q = 0; q < n; ++q) v[i][q] = (-HH(k, i)) * v[k - 1][q] + v[i][q];
      }
      HH(i + 1, i) = sqrt(dot2(h, v[i], v[i]));
      const double sh = 1.0 / HH(i + 1, i);
      for (size_t q = 0; q < n; ++q) v[i][q] = sh * v[i][q];
      for (int k = 2; k <= i; ++k) {
        double temp = c[k - 2] * HH(k - 1, i) + s[k - 2] * HH(k, i);
        HH(k, i) = -s[k - 2] * HH(k - 1, i) + c[k - 2] * HH(k, i);
        HH(k - 1, i) = temp;
      }
      double delta = sqrt(HH(i, i) * HH(i, i) + HH(i + 1, i) * HH(i + 1, i));
      c[i - 1] = HH(i, i) / delta;
      s[i - 1] = HH(i + 1, i) / delta;
      HH(i, i) = c[i - 1] * HH(i, i) + s[i - 1] * HH(i + 1, i);
      bh[i] = -s[i - 1] * bh[i - 1];
      bh[i - 1] = c[i - 1] * bh[i - 1];
      rho = fabs(bh[i]);
      if (rho <= tol * rho0) {
        nr = i;
        break;
      }
      nr = step;
    }
    y[nr - 1] = bh[nr - 1] / HH(nr, nr);
    for (int k = nr - 1; k >= 1; --k) {
      y[k - 1] = bh[k - 1];
      for (int i = k + 1; i <= nr; ++i) y[k - 1] = y[k - 1] - HH(k, i) * y[i - 1];
      y[k - 1] = y[k - 1] / HH(k, k);
    }
    for (int i = 1; i <= nr; ++i)
      for (size_t q = 0; q < n; ++q) x[q] = y[i - 1] * z[i - 1][q] + x[q];
    if (rho <= tol * rho0) break;
  }
#undef HH
  for (int i = 0; i <= step; ++i) free(v[i]);
  for (int i = 0; i < step; ++i) free(z[i]);
  free(v);
  free(z);
  free(H);
  free(c);
  free(s);
  free(bh);
  free(y);
  if (rho_out) *rho_out = rho;
  if (rho0_out) *rho0_out = rho0;
  return steps;
}

/* PSolve1, MatVec1, Exchange and DOT2 on PressureVelocity vectors, exposed for the tests */
void ora_psolve1(void* hv, const double* x, double* b) { psolve1((Proj*)hv, b, x); }
void ora_matvec1(void* hv, const double* x, double* b) { matvec1((Proj*)hv, x, b); }
void ora_proj_exchange(void* hv, double* v) { exchange_pv((Proj*)hv, v); }
double ora_proj_dot2(void* hv, const double* x, const double* y) { return dot2((Proj*)hv, x, y); }

#define UI(i, j, k) ((size_t)(i) + (size_t)(nx + 1) * ((size_t)((j) - 1) + (size_t)ny * ((k) - 1)))
#define VI(i, j, k) ((size_t)((i) - 1) + (size_t)nx * ((size_t)(j) + (size_t)(ny + 1) * ((k) - 1)))
#define WI(i, j, k) ((size_t)((i) - 1) + (size_t)nx * ((size_t)((j) - 1) + (size_t)ny * (k)))
#define CI(i, j, k) ((size_t)((i) - 1) + (size_t)nx * ((size_t)((j) - 1) + (size_t)ny * ((k) - 1)))
#define PI(i, j, k) ((size_t)(i) + (size_t)(nx + 2) * ((size_t)(j) + (size_t)(ny + 2) * (k)))

/* Rhs (Rhs_Mod.f90:110-187) with DivergenceS (:41-78): b = beta0*dtP*div,
 * minus VolB*incr_th in the FacAnela>=1 branch.  u,v,w uF/vF/wF extents;
 * incr_th the padded theta increment (or NULL: no theta term); b a
 * PressureVelocity vector (ora_proj_nvec entries, face unknowns 0). */
void ora_proj_rhs(void* hv, const double* u, const double* v, const double* w, const double* incr_th, double* b) {
  Proj* h = (Proj*)hv;
  const int nx = h->par.nx, ny = h->par.ny, nz = h->par.nz;
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        double div = (-(h->fu[UI(i - 1, j, k)] * h->dtu[UI(i - 1, j, k)] * u[UI(i - 1, j, k)]) +
                      h->fu[UI(i, j, k)] * h->dtu[UI(i, j, k)] * u[UI(i, j, k)] -
                      h->fv[VI(i, j - 1, k)] * h->dtv[VI(i, j - 1, k)] * v[VI(i, j - 1, k)] +
                      h->fv[VI(i, j, k)] * h->dtv[VI(i, j, k)] * v[VI(i, j, k)] -
                      h->fw[WI(i, j, k - 1)] * h->dtw[WI(i, j, k - 1)] * w[WI(i, j, k - 1)] +
                      h->fw[WI(i, j, k)] * h->dtw[WI(i, j, k)] * w[WI(i, j, k)]) *
                     h->dtt[CI(i, j, k)];
        double val = h->beta0 * h->dtp * div;
        if (incr_th && h->par.fac_anela >= 1.0) val = val - h->vol[CI(i, j, k)] * incr_th[PI(i, j, k)];
        b[CI(i, j, k)] = val;
      }
  /* the face unknowns of b stay Zero (ProjectVelFace: b=Zero; Rhs sets p only) */
  for (size_t q = (size_t)nx * ny * nz; q < h->nvec; ++q) b[q] = 0.0;
}

/* UpdateVelocity (Rhs_Mod.f90:589-952) for GradFull + MultiTriT.  x is the
 * solved PressureVelocity vector; its pressure is overwritten with x*DUT
 * like the reference.  The boundary faces get Temp = x%u_w - b%u_w/(...)
 * (Rhs_Mod.f90:636-660) with b's face parts 0 (Rhs sets the pressure only):
 * the face unknown of a periodic side, 0 on a closed side.  u,v,w updated in
 * place; incr_th / incr_rho (padded, may be NULL) updated; ncs scalars
 * (increment + state arrays, padded) get the DivScalar update with rho
 * (padded). */
void ora_proj_update(void* hv, double* x, double* u, double* v, double* w, double* incr_th, double* incr_rho, int ncs,
                     double* const* incr_c, const double* const* c, const double* rho_pad) {
  Proj* h = (Proj*)hv;
  const int nx = h->par.nx, ny = h->par.ny, nz = h->par.nz;
  const double beta0 = h->beta0, dtp = h->dtp;
  const size_t n = (size_t)nx * ny * nz;
  for (size_t q = 0; q < n; ++q) x[q] = x[q] * h->dut[q];
  /* boundary faces: Temp = x%u_w - b%u_w/(...) with zero face parts of b */
  const long* o = h->off;
#define FACEX(side, idx) (o[side] >= 0 ? x[o[side] + (idx)] : 0.0)
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j) {
      const size_t f = (size_t)(j - 1) + (size_t)ny * (k - 1);
      double t0 = FACEX(0, f) - 0.0 / (0.5 * h->dx[0] * h->mxy[j - 1] * h->mxz[k - 1]);
      u[UI(0, j, k)] = u[UI(0, j, k)] + t0;
      double t1 = FACEX(1, f) - 0.0 / (0.5 * h->dx[nx - 1] * h->mxy[j - 1] * h->mxz[k - 1]);
      u[UI(nx, j, k)] = u[UI(nx, j, k)] + t1;
    }
  for (int i = 1; i <= nx; ++i)
    for (int k = 1; k <= nz; ++k) {
      const size_t f = (size_t)(i - 1) + (size_t)nx * (k - 1);
      double t0 = FACEX(2, f) - 0.0 / (0.5 * h->dy[0] * h->myx[i - 1] * h->myz[k - 1]);
      v[VI(i, 0, k)] = v[VI(i, 0, k)] + t0;
      double t1 = FACEX(3, f) - 0.0 / (0.5 * h->dy[ny - 1] * h->myx[i - 1] * h->myz[k - 1]);
      v[VI(i, ny, k)] = v[VI(i, ny, k)] + t1;
    }
  for (int i = 1; i <= nx; ++i)
    for (int j = 1; j <= ny; ++j) {
      const size_t f = (size_t)(i - 1) + (size_t)nx * (j - 1);
      double t0 = FACEX(4, f) - 0.0 / (0.5 * h->dz[0] * h->mzx[i - 1] * h->mzy[j - 1]);
      w[WI(i, j, 0)] = w[WI(i, j, 0)] + t0;
      double t1 = FACEX(5, f) - 0.0 / (0.5 * h->dz[nz - 1] * h->mzx[i - 1] * h->mzy[j - 1]);
      const double fwt = h->fw[WI(i, j, nz)];
      w[WI(i, j, nz)] = w[WI(i, j, nz)] + fwt / (fwt + EPS) * t1;
    }
#undef FACEX
  /* interior faces: u = utilde - grad p */
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx - 1; ++i) {
        double t = 2.0 * beta0 * dtp * h->duu[UI(i, j, k)] * (x[CI(i + 1, j, k)] - x[CI(i, j, k)]) /
                   ((h->dx[i] + h->dx[i - 1]) * h->mxy[j - 1] * h->mxz[k - 1]);
        u[UI(i, j, k)] = u[UI(i, j, k)] - t;
      }
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny - 1; ++j)
      for (int i = 1; i <= nx; ++i) {
        double t = 2.0 * beta0 * dtp * h->duv[VI(i, j, k)] * (x[CI(i, j + 1, k)] - x[CI(i, j, k)]) /
                   ((h->dy[j] + h->dy[j - 1]) * h->myx[i - 1] * h->myz[k - 1]);
        v[VI(i, j, k)] = v[VI(i, j, k)] - t;
      }
  for (int k = 1; k <= nz - 1; ++k)
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        double t = 2.0 * beta0 * dtp * h->duw[WI(i, j, k)] * (x[CI(i, j, k + 1)] - x[CI(i, j, k)]) / (h->dz[k] + h->dz[k - 1]);
        const double fw = h->fw[WI(i, j, k)];
        w[WI(i, j, k)] = w[WI(i, j, k)] - fw / (fw + EPS) * t;
      }
  /* ThPos and RhoPos increments */
  if (incr_th)
    for (int k = 1; k <= nz; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          double s = h->fu[UI(i, j, k)] * h->dtu[UI(i, j, k)] * u[UI(i, j, k)] -
                     h->fu[UI(i - 1, j, k)] * h->dtu[UI(i - 1, j, k)] * u[UI(i - 1, j, k)] +
                     h->fv[VI(i, j, k)] * h->dtv[VI(i, j, k)] * v[VI(i, j, k)] -
                     h->fv[VI(i, j - 1, k)] * h->dtv[VI(i, j - 1, k)] * v[VI(i, j - 1, k)] +
                     h->fw[WI(i, j, k)] * h->dtw[WI(i, j, k)] * w[WI(i, j, k)] -
                     h->fw[WI(i, j, k - 1)] * h->dtw[WI(i, j, k - 1)] * w[WI(i, j, k - 1)];
          incr_th[PI(i, j, k)] = incr_th[PI(i, j, k)] - dtp * beta0 * h->dtt[CI(i, j, k)] * s / (h->vol[CI(i, j, k)] + EPS);
        }
  if (incr_rho)
    for (int k = 1; k <= nz; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          double s = h->fu[UI(i, j, k)] * u[UI(i, j, k)] - h->fu[UI(i - 1, j, k)] * u[UI(i - 1, j, k)] +
                     h->fv[VI(i, j, k)] * v[VI(i, j, k)] - h->fv[VI(i, j - 1, k)] * v[VI(i, j - 1, k)] +
                     h->fw[WI(i, j, k)] * w[WI(i, j, k)] - h->fw[WI(i, j, k - 1)] * w[WI(i, j, k - 1)];
          incr_rho[PI(i, j, k)] = incr_rho[PI(i, j, k)] - dtp * beta0 * s / (h->vol[CI(i, j, k)] + EPS);
        }
  /* DivScalar (Rhs_Mod.f90:915-950) on padded scalar fields */
#define VP(i, j, k) h->volp[PI(i, j, k)]
  for (int ic = 0; ic < ncs; ++ic) {
    double* cd = incr_c[ic];
    const double* cc = c[ic];
    for (int k = 1; k <= nz; ++k)
      for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
          const double vC = VP(i, j, k);
          const double vW = VP(i - 1, j, k), vE = VP(i + 1, j, k);
          const double vS = VP(i, j - 1, k), vN = VP(i, j + 1, k);
          const double vB = VP(i, j, k - 1), vT = VP(i, j, k + 1);
          const double qC = vC * cc[PI(i, j, k)] / (rho_pad[PI(i, j, k)] + EPS);
          double s = h->fu[UI(i, j, k)] * u[UI(i, j, k)] * (qC + vE * cc[PI(i + 1, j, k)] / (rho_pad[PI(i + 1, j, k)] + EPS)) /
                         (vC + vE + EPS) -
                     h->fu[UI(i - 1, j, k)] * u[UI(i - 1, j, k)] *
                         (qC + vW * cc[PI(i - 1, j, k)] / (rho_pad[PI(i - 1, j, k)] + EPS)) / (vC + vW + EPS) +
                     h->fv[VI(i, j, k)] * v[VI(i, j, k)] * (qC + vN * cc[PI(i, j + 1, k)] / (rho_pad[PI(i, j + 1, k)] + EPS)) /
                         (vC + vN + EPS) -
                     h->fv[VI(i, j - 1, k)] * v[VI(i, j - 1, k)] *
                         (qC + vS * cc[PI(i, j - 1, k)] / (rho_pad[PI(i, j - 1, k)] + EPS)) / (vC + vS + EPS) +
                     h->fw[WI(i, j, k)] * w[WI(i, j, k)] * (qC + vT * cc[PI(i, j, k + 1)] / (rho_pad[PI(i, j, k + 1)] + EPS)) /
                         (vC + vT + EPS) -
                     h->fw[WI(i, j, k - 1)] * w[WI(i, j, k - 1)] *
                         (qC + vB * cc[PI(i, j, k - 1)] / (rho_pad[PI(i, j, k - 1)] + EPS)) / (vC + vB + EPS);
          cd[PI(i, j, k)] = cd[PI(i, j, k)] - dtp * beta0 * s / (vC + EPS);
        }
  }
#undef VP
}
#undef UI
#undef VI
#undef WI
#undef CI
#undef PI

/* WeightDiagCompute, ThetaKind='Density' branch (MULTI/JacAccGrav_Mod.f90:
 * 4259-4282) with CellToFaceRhoWeight (:3254-3702) for closed (outer walls,
 * no inflow) and periodic sides: DUT per cell, DTU/DTV/DTW the volume-weighted
 * face values of theta = (rho theta)/(rho+Eps) (one-sided on the walls, with
 * the halo image on a periodic side),
 * DUU/DUV/DUW = F/(F+Eps), DTT = 1.  Inputs are padded fields: rth = rho
 * theta, rho, rv (RhoV, may be NULL), rl (RhoL + RhoR summed by the caller:
 * rc and rr, each may be NULL), t = absolute temperature.  Outputs with the
 * library's weight layouts. */
#define CP_D 1004.0
#define CV_D 717.0
#define R_D (CP_D - CV_D)
#define CP_V 1885.0
#define R_V 461.0
#define CP_L 4186.0
void ora_weights_density(void* hv, const double* rth, const double* rho, const double* rv, const double* rc,
                         const double* rr, const double* t, double* dtu, double* dtv, double* dtw, double* duu,
                         double* duv, double* duw, double* dut, double* dtt) {
  Proj* h = (Proj*)hv;
  const int nx = h->par.nx, ny = h->par.ny, nz = h->par.nz;
  const double* V = h->volp;
#define PI(i, j, k) ((size_t)(i) + (size_t)(nx + 2) * ((size_t)(j) + (size_t)(ny + 2) * (k)))
#define UI(i, j, k) ((size_t)(i) + (size_t)(nx + 1) * ((size_t)((j) - 1) + (size_t)ny * ((k) - 1)))
#define VI(i, j, k) ((size_t)((i) - 1) + (size_t)nx * ((size_t)(j) + (size_t)(ny + 1) * ((k) - 1)))
#define WI(i, j, k) ((size_t)((i) - 1) + (size_t)nx * ((size_t)((j) - 1) + (size_t)ny * (k)))
#define CI(i, j, k) ((size_t)((i) - 1) + (size_t)nx * ((size_t)((j) - 1) + (size_t)ny * ((k) - 1)))
#define TH(P) (rth[P] / (rho[P] + EPS))
#define FACE(P, Q) ((V[P] * rth[P] / (rho[P] + EPS) + V[Q] * rth[Q] / (rho[Q] + EPS)) / (V[P] + V[Q] + EPS))
/* a periodic x or y side ('iw'/'ie'/'is'/'in' branches, equal refinement,
 * :3313-3321, 3360-3368, 3407-3415, 3454-3462): theta first, then times the
 * volume, with the halo cell holding the periodic image */
#define PFACE(P, Q) ((TH(P) * V[P] + TH(Q) * V[Q]) / (V[P] + V[Q] + EPS))
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        const size_t P = PI(i, j, k);
        const double rvl = rv ? rv[P] : 0.0;
        const double rll = (rc ? rc[P] : 0.0) + (rr ? rr[P] : 0.0);
        const double rd = rho[P] - rvl - rll + EPS;
        const double rm = R_D + R_V * rvl / rd;
        const double cpml = CP_D + CP_V * rvl / rd + CP_L * rll / rd;
        const double kap = rm / cpml;
        dut[CI(i, j, k)] = t[P] / (rth[P] + EPS) * (rd * R_D + rvl * R_V) / (1.0 - kap);
        dtt[CI(i, j, k)] = 1.0;
      }
  for (int k = 1; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j)
      for (int i = 0; i <= nx; ++i) {
        double v;
        if (i == 0)
          v = h->per_x ? PFACE(PI(1, j, k), PI(0, j, k)) : TH(PI(1, j, k));
        else if (i == nx)
          v = h->per_x ? PFACE(PI(nx + 1, j, k), PI(nx, j, k)) : TH(PI(nx, j, k));
        else
          v = FACE(PI(i, j, k), PI(i + 1, j, k));
        dtu[UI(i, j, k)] = v;
        const double f = h->fu[UI(i, j, k)];
        duu[UI(i, j, k)] = f / (f + EPS);
      }
  for (int k = 1; k <= nz; ++k)
    for (int j = 0; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        double v;
        if (j == 0)
          v = h->per_y ? PFACE(PI(i, 1, k), PI(i, 0, k)) : TH(PI(i, 1, k));
        else if (j == ny)
          v = h->per_y ? PFACE(PI(i, ny + 1, k), PI(i, ny, k)) : TH(PI(i, ny, k));
        else
          v = FACE(PI(i, j, k), PI(i, j + 1, k));
        dtv[VI(i, j, k)] = v;
        const double f = h->fv[VI(i, j, k)];
        duv[VI(i, j, k)] = f / (f + EPS);
      }
  for (int k = 0; k <= nz; ++k)
    for (int j = 1; j <= ny; ++j)
      for (int i = 1; i <= nx; ++i) {
        double v;
        if (k == 0)  /* 'ib'/'it' (:3501-3509, 3548-3556): the interior rounding */
          v = h->per_z ? FACE(PI(i, j, 1), PI(i, j, 0)) : TH(PI(i, j, 1));
        else if (k == nz)
          v = h->per_z ? FACE(PI(i, j, nz + 1), PI(i, j, nz)) : TH(PI(i, j, nz));
        else
          v = FACE(PI(i, j, k), PI(i, j, k + 1));
        dtw[WI(i, j, k)] = v;
        const double f = h->fw[WI(i, j, k)];
        duw[WI(i, j, k)] = f / (f + EPS);
      }
#undef PI
#undef UI
#undef VI
#undef WI
#undef CI
#undef TH
#undef FACE
#undef PFACE
}

/* Replace the oracle's weights (after ora_weights_density) */
void ora_proj_set_weights(void* hv, const double* dtu, const double* dtv, const double* dtw, const double* duu,
                          const double* duv, const double* duw, const double* dut, const double* dtt) {
  Proj* h = (Proj*)hv;
  const int nx = h->par.nx, ny = h->par.ny, nz = h->par.nz;
  const size_t nu = (size_t)(nx + 1) * ny * nz, nv = (size_t)nx * (ny + 1) * nz, nw = (size_t)nx * ny * (nz + 1);
  const size_t nc = (size_t)nx * ny * nz;
  memcpy(h->dtu, dtu, nu * sizeof(double));
  memcpy(h->duu, duu, nu * sizeof(double));
  memcpy(h->dtv, dtv, nv * sizeof(double));
  memcpy(h->duv, duv, nv * sizeof(double));
  memcpy(h->dtw, dtw, nw * sizeof(double));
  memcpy(h->duw, duw, nw * sizeof(double));
  memcpy(h->dut, dut, nc * sizeof(double));
  memcpy(h->dtt, dtt, nc * sizeof(double));
}
