// Pressure projection (sound solve) of one block on the device:
//   * assembly of the tridiagonal pressure-Laplacian hierarchy
//     (MULTI/JacAccGrav_Mod.f90:1056-1310 LaplTFullCompute with the
//     coarsening helpers :709-903 and MULTI/TriDiagT_Mod.f90 ComputeFull_1D/2D/3D),
//   * its operator MatVecT_3D (TriDiagT_Mod.f90:885-917, MatVecP_Tri),
//   * the semi-coarsening multigrid V-cycle Solve_3D (TriDiagT_Mod.f90:1009-1085)
//     with plane -> x-line -> z-column (Thomas) relaxation,
//   * FGMRES(StepGMRES) with MatVec1/PSolve1 (SOLU/Iter_Mod.f90:121-199,
//     MATRIX/MatVec_Mod.f90:184-258, MATRIX/PreCond_Mod.f90:1555-1571),
//   * Rhs/DivergenceS and UpdateVelocity (MATRIX/Rhs_Mod.f90:41-78, 110-187, 589-952).
//
// Scope: a block whose sides are closed outer boundaries (no boundary
// pressure unknowns) or periodic, i.e. the block is its own neighbour across
// the side pair (nType 'iw'/'ie' ...).  A periodic side carries the boundary
// face unknowns u_w ... w_t of PressureVelocity (MODULE/VecPrVel_Mod.f90:10-18):
// MatVecFull adds their face equations (MATRIX/MatVec_Mod.f90:224-255), every
// MatVec1 and residual is followed by Exchange (RandCopy with CopyFluxVel
// EqualEqual: u_w = u_w + u_e; u_e = u_w, MODULE/VecPrVel_Mod.f90:809-852,
// MODULE/Exchange_Mod.f90:769-800), DOT2 counts a shared face once
// (MODULE/VecPrVel_Mod.f90:112-172), and PSolve1 runs in full: PressurePre,
// b2pBx1Full, Exchange, SchurPreFull (one Solve_3D on the Dirichlet hierarchy
// LaplDirichlet of SetFactorD, Fac=2 on the periodic sides,
// MULTI/Reverse_Mod.f90:95-213, MATRIX/PreCond_Mod.f90:20-597), Exchange,
// b1pBTx2Full, PressurePre (MATRIX/PreCond_Mod.f90:599-844, 1555-1571).  A
// closed block has no face unknowns: the Schur step leaves the pressure
// unchanged and PSolve1 reduces to PressurePre(-x) (the first PressurePre
// only feeds the face unknowns, so it is not run).
//
// PressureVelocity vectors on the device: the pressure in the level-0 layout
// (below), then the face unknowns of the periodic sides in the order
// u_e, v_n, w_t, u_w, v_s, w_b (u: y fastest then z; v: x then z; w: x then y)
// -- the sides DOT2 counts first, so every dot product runs over one
// contiguous prefix of the vector.
//
// Data layout.  The hierarchy lives in the reference's reversed index space
// (n1,n2,n3) = (z,x,y) (MULTI/Reverse_Mod.f90 with xOrder=2,yOrder=3,zOrder=1).
// A level with c1 rows (z), c2 lines (x) and m3 planes (y) stores entry
// (i,j,k) at k*ps + i*w + (j&1)*h + (j>>1), h = ceil(c2/2), w = 2h, ps = c1*w:
// within a plane row the even lines come first, then the odd ones, so the
// threads that relax the lines of one parity read consecutive addresses.
//
// Smoother ordering.  The reference relaxes planes and lines in lexicographic
// order, a chain with no parallelism.  Here planes (then lines inside a plane)
// of one parity are relaxed concurrently -- the zebra ordering of the same
// smoother: every plane right-hand side, line right-hand side and Thomas solve
// uses the reference's arithmetic and operation order; only the order of the
// relaxations differs.  One CTA owns one plane and runs that plane's whole 2D
// multigrid with block barriers, so a half-sweep over all planes of one
// parity is a single launch.  FP64 without FMA contraction (-fmad=false);
// divisions by the Thomas pivots use the correctly rounded div_rn with
// precomputed reciprocals, so every value equals the oracle's zebra run bit
// for bit.
#include <cmath>
#include <cstring>
#include <vector>

#include "context.h"
#include "kernels.cuh"

namespace asam {

namespace prj {

constexpr int kMaxLev = 8;
constexpr int kPlaneBlock = 256;
constexpr int kRedGrid = 1024;
constexpr int kRedBlock = 256;
constexpr size_t kRingBytes = (size_t)4 * 8 * kPlaneBlock * sizeof(double);  // ring rows * fields * block, 64 KB
constexpr double kTiny = 1.0e-40;  // initial diagonal of Allocate_1D (TriDiagT_Mod.f90:99)

// One plane level of a 3D level (all its planes); T = double for the
// reference arithmetic, float for the single-precision copy of the multigrid
// that preconditions FGMRES in the refined mode.
template <typename T>
struct Lev2T {
  int c1, c2, h, w, m3;
  size_t ps;
  T *d, *uz, *lz, *fw, *ft, *frt, *ux, *lx, *res;
  T *x, *b;  // own vectors of the coarse plane levels (nullptr on the 3D level's own planes)
  // periodic-Laplacian hierarchy only (nullptr otherwise): the couplings
  // across the periodic x side, between line 0 and line c2-1 of row i of
  // plane k at [k*c1 + i]: wxl in the row of line 0, wxh in the row of line c2-1
  T *wxl, *wxh;
};
using Lev2 = Lev2T<double>;

template <typename T>
struct Lev3T {
  int m1, m2, m3, nl;
  Lev2T<T> pl[kMaxLev];
  T *u3, *l3, *x, *b, *res, *t;
  // periodic-Laplacian hierarchy only: couplings across the periodic y side
  // between plane 0 and plane m3-1 (one plane layout): wyl in the rows of
  // plane 0, wyh in the rows of plane m3-1
  T *wyl, *wyh;
};
using Lev3 = Lev3T<double>;

// Input fields of one level in the reversed index space with 1-based logical
// indices F1(0:n1,1:n2,1:n3), F2(1:n1,0:n2,1:n3), F3(1:n1,1:n2,0:n3) and cell
// arrays (1:n1,1:n2,1:n3).  In memory the x index (n2) runs fastest, then z
// (n1), then y (n3) -- the order of the Fortran inputs, so reading them and
// writing the level layout are both coalesced.  Every coarse sum follows the
// reference's loop order whatever the memory order.
struct Fields {
  int n1, n2, n3;
  double *F1, *T1, *U1, *F2, *T2, *U2, *F3, *T3, *U3, *vol, *dut;
  double *d1, *d2, *d3, *m12, *m13, *m21, *m23, *m31, *m32;
  __host__ __device__ size_t i1(int i, int j, int k) const {
    return (size_t)(j - 1) + (size_t)n2 * ((size_t)i + (size_t)(n1 + 1) * (size_t)(k - 1));
  }
  __host__ __device__ size_t i2(int i, int j, int k) const {
    return (size_t)j + (size_t)(n2 + 1) * ((size_t)(i - 1) + (size_t)n1 * (size_t)(k - 1));
  }
  __host__ __device__ size_t i3(int i, int j, int k) const {
    return (size_t)(j - 1) + (size_t)n2 * ((size_t)(i - 1) + (size_t)n1 * (size_t)k);
  }
  __host__ __device__ size_t ic(int i, int j, int k) const {
    return (size_t)(j - 1) + (size_t)n2 * ((size_t)(i - 1) + (size_t)n1 * (size_t)(k - 1));
  }
};

struct Facs {
  double f1l, f1r, f2l, f2r, f3l, f3r;
};

// Offsets of the six face arrays inside a PressureVelocity vector (-1: the
// side is closed and has none), sides numbered W, E, S, N, B, T.
struct PvFaces {
  long long off[6];
};


__host__ __device__ inline size_t slot(int w, int h, int i, int j) {
  return (size_t)i * w + (size_t)(j & 1) * h + (size_t)(j >> 1);
}

// line index j of a padded position pos in a plane row (-1: padding)
__device__ inline int line_of(int pos, int h, int c2) {
  const int j = pos < h ? 2 * pos : 2 * (pos - h) + 1;
  return j < c2 ? j : -1;
}

// Visits the slots s = 0 .. ps-1 of one plane (rows of w slots) with the
// block's threads in stride order, passing the row i and the position r in
// the row, which are tracked by increments: one integer division per call
// instead of one per slot (a division by a run-time value costs some twenty
// instructions on the GPU).
template <typename F>
__device__ __forceinline__ void for_plane(int w, size_t ps, F&& f) {
  const int bd = blockDim.x;
  int i = (int)threadIdx.x / w;
  int r = (int)threadIdx.x - i * w;
  const int di = bd / w, dr = bd - di * w;
  for (size_t s = threadIdx.x; s < ps; s += bd) {
    f(s, i, r);
    i += di;
    r += dr;
    if (r >= w) {
      r -= w;
      ++i;
    }
  }
}

// ---------------------------------------------------------------------------
// Assembly
// ---------------------------------------------------------------------------

// ReverseWeight / Reverse of the fine fields (Reverse_Mod.f90:330-360, 565-575)
__global__ void k_fine_fields(Dims d, const double* __restrict__ fu, const double* __restrict__ fv,
                              const double* __restrict__ fw, const double* __restrict__ volc,
                              const double* __restrict__ dtu, const double* __restrict__ dtv,
                              const double* __restrict__ dtw, const double* __restrict__ duu,
                              const double* __restrict__ duv, const double* __restrict__ duw,
                              const double* __restrict__ dut, Fields g) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const size_t n = (size_t)(nx + 1) * (nz + 1) * (ny + 1);
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const int x = (int)(e % (nx + 1));
    const size_t r = e / (nx + 1);
    const int z = (int)(r % (nz + 1));
    const int y = (int)(r / (nz + 1));
    if (x >= 1 && y >= 1) {  // F1 = FW(x,y,z), z = 0..nz
      const size_t q = g.i1(z, x, y);
      g.F1[q] = fw[d.FW(x, y, z)];
      g.T1[q] = dtw[d.WF(x, y, z)];
      g.U1[q] = duw[d.WF(x, y, z)];
    }
    if (y >= 1 && z >= 1) {  // F2 = FU(x,y,z), x = 0..nx
      const size_t q = g.i2(z, x, y);
      g.F2[q] = fu[d.FU(x, y, z)];
      g.T2[q] = dtu[d.UF(x, y, z)];
      g.U2[q] = duu[d.UF(x, y, z)];
    }
    if (x >= 1 && z >= 1) {  // F3 = FV(x,y,z), y = 0..ny
      const size_t q = g.i3(z, x, y);
      g.F3[q] = fv[d.FV(x, y, z)];
      g.T3[q] = dtv[d.VF(x, y, z)];
      g.U3[q] = duv[d.VF(x, y, z)];
    }
    if (x >= 1 && y >= 1 && z >= 1) {
      const size_t q = g.ic(z, x, y);
      g.vol[q] = volc[d.P(x, y, z)];
      g.dut[q] = dut[(size_t)(x - 1) + (size_t)nx * ((size_t)(y - 1) + (size_t)ny * (size_t)(z - 1))];
    }
  }
}

// ReverseIncr / ReverseMetr (Reverse_Mod.f90:362-541): d1=dz, d2=dx, d3=dy,
// Metr12=MetrZX, Metr13=MetrZY, Metr21=MetrXZ, Metr23=MetrXY, Metr31=MetrYZ, Metr32=MetrYX
__global__ void k_fine_1d(int nx, int ny, int nz, const double* dx, const double* dy, const double* dz,
                          const double* metr, Fields g) {
  const double* mxy = metr;
  const double* mxz = metr + ny;
  const double* myx = metr + ny + nz;
  const double* myz = metr + ny + nz + nx;
  const double* mzx = metr + ny + 2 * nz + nx;
  const double* mzy = metr + ny + 2 * nz + 2 * nx;
  for (int q = threadIdx.x; q < nz; q += blockDim.x) {
    g.d1[q] = dz[q];
    g.m21[q] = mxz[q];
    g.m31[q] = myz[q];
  }
  for (int q = threadIdx.x; q < nx; q += blockDim.x) {
    g.d2[q] = dx[q];
    g.m12[q] = mzx[q];
    g.m32[q] = myx[q];
  }
  for (int q = threadIdx.x; q < ny; q += blockDim.x) {
    g.d3[q] = dy[q];
    g.m13[q] = mzy[q];
    g.m23[q] = mxy[q];
  }
}

__device__ inline int blo(int c, int s) { return (c - 1) * (s + 1) + 1; }
__device__ inline int bhi(int c, int s, int n) { return min(c * (s + 1), n); }

// FaceCoarse + CFaceCoarse (JacAccGrav_Mod.f90:804-903): every coarse face sums
// its fine faces in the reference's loop order; then the face-weighted DTU
// and DUU averages.
__global__ void k_coarse_faces(Fields g, Fields c, int s1, int s2, int s3) {
  const int n = g.n1, m = g.n2, l = g.n3;
  const int nC = c.n1, mC = c.n2, lC = c.n3;
  const size_t n1f = (size_t)(nC + 1) * mC * lC, n2f = (size_t)nC * (mC + 1) * lC, n3f = (size_t)nC * mC * (lC + 1);
  const size_t tot = n1f + n2f + n3f;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot; e += (size_t)gridDim.x * blockDim.x) {
    double F = 0.0, TF = 0.0, UF = 0.0;
    if (e < n1f) {
      const int jC = (int)(e % mC) + 1;
      const size_t r = e / mC;
      const int iC = (int)(r % (nC + 1)), kC = (int)(r / (nC + 1)) + 1;
      const int i = min((s1 + 1) * iC, n);
      for (int j = blo(jC, s2); j <= bhi(jC, s2, m); ++j)
        for (int k = blo(kC, s3); k <= bhi(kC, s3, l); ++k) {
          const size_t q = g.i1(i, j, k);
          const double f = g.F1[q];
          F = F + f;
          TF = TF + g.T1[q] * f;
          UF = UF + g.U1[q] * f;
        }
      const size_t qc = c.i1(iC, jC, kC);
      c.F1[qc] = F;
      c.T1[qc] = TF / (F + asam::kEps);
      c.U1[qc] = UF / (F + asam::kEps);
    } else if (e < n1f + n2f) {
      const size_t ee = e - n1f;
      const int jC = (int)(ee % (mC + 1));
      const size_t r = ee / (mC + 1);
      const int iC = (int)(r % nC) + 1, kC = (int)(r / nC) + 1;
      const int j = min((s2 + 1) * jC, m);
      for (int i = blo(iC, s1); i <= bhi(iC, s1, n); ++i)
        for (int k = blo(kC, s3); k <= bhi(kC, s3, l); ++k) {
          const size_t q = g.i2(i, j, k);
          const double f = g.F2[q];
          F = F + f;
          TF = TF + g.T2[q] * f;
          UF = UF + g.U2[q] * f;
        }
      const size_t qc = c.i2(iC, jC, kC);
      c.F2[qc] = F;
      c.T2[qc] = TF / (F + asam::kEps);
      c.U2[qc] = UF / (F + asam::kEps);
    } else {
      const size_t ee = e - n1f - n2f;
      const int jC = (int)(ee % mC) + 1;
      const size_t r = ee / mC;
      const int iC = (int)(r % nC) + 1, kC = (int)(r / nC);
      const int k = min((s3 + 1) * kC, l);
      for (int i = blo(iC, s1); i <= bhi(iC, s1, n); ++i)
        for (int j = blo(jC, s2); j <= bhi(jC, s2, m); ++j) {
          const size_t q = g.i3(i, j, k);
          const double f = g.F3[q];
          F = F + f;
          TF = TF + g.T3[q] * f;
          UF = UF + g.U3[q] * f;
        }
      const size_t qc = c.i3(iC, jC, kC);
      c.F3[qc] = F;
      c.T3[qc] = TF / (F + asam::kEps);
      c.U3[qc] = UF / (F + asam::kEps);
    }
  }
}

// VolCoarse + CVolCoarse (JacAccGrav_Mod.f90:724-745, 784-802)
__global__ void k_coarse_cells(Fields g, Fields c, int s1, int s2, int s3) {
  const size_t tot = (size_t)c.n1 * c.n2 * c.n3;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot; e += (size_t)gridDim.x * blockDim.x) {
    const int jC = (int)(e % c.n2) + 1;
    const size_t r = e / c.n2;
    const int iC = (int)(r % c.n1) + 1, kC = (int)(r / c.n1) + 1;
    double V = 0.0, DV = 0.0;
    for (int i = blo(iC, s1); i <= bhi(iC, s1, g.n1); ++i)
      for (int j = blo(jC, s2); j <= bhi(jC, s2, g.n2); ++j)
        for (int k = blo(kC, s3); k <= bhi(kC, s3, g.n3); ++k) {
          const size_t q = g.ic(i, j, k);
          V = V + g.vol[q];
          DV = DV + g.dut[q] * g.vol[q];
        }
    const size_t qc = c.ic(iC, jC, kC);
    c.vol[qc] = V;
    c.dut[qc] = DV / (V + asam::kEps);
  }
}

// IncrCoarse + CIncrCoarse (JacAccGrav_Mod.f90:747-782), one block: every
// coarse entry sums its fine entries in increasing order (the reference's
// loop order), the increments first
__device__ inline void incr_entry(const double* d, int n, double* dc, int ic, int s) {
  double v = 0.0;
  for (int i = ic * (s + 1) + 1; i <= min((ic + 1) * (s + 1), n); ++i) v = v + d[i - 1];
  dc[ic] = v;
}
__device__ inline void cincr_entry(const double* C, const double* d, int n, double* CC, const double* dc, int ic, int s) {
  double v = 0.0;
  for (int i = ic * (s + 1) + 1; i <= min((ic + 1) * (s + 1), n); ++i) v = v + d[i - 1] * C[i - 1];
  CC[ic] = v / dc[ic];
}
__global__ void k_coarse_1d(Fields g, Fields c, int s1, int s2, int s3) {
  for (int q = threadIdx.x; q < c.n1 + c.n2 + c.n3; q += blockDim.x) {
    if (q < c.n1)
      incr_entry(g.d1, g.n1, c.d1, q, s1);
    else if (q < c.n1 + c.n2)
      incr_entry(g.d2, g.n2, c.d2, q - c.n1, s2);
    else
      incr_entry(g.d3, g.n3, c.d3, q - c.n1 - c.n2, s3);
  }
  __syncthreads();
  for (int q = threadIdx.x; q < 2 * (c.n1 + c.n2 + c.n3); q += blockDim.x) {
    int r = q;
    if (r < c.n2) { cincr_entry(g.m12, g.d2, g.n2, c.m12, c.d2, r, s2); continue; }
    r -= c.n2;
    if (r < c.n3) { cincr_entry(g.m13, g.d3, g.n3, c.m13, c.d3, r, s3); continue; }
    r -= c.n3;
    if (r < c.n1) { cincr_entry(g.m21, g.d1, g.n1, c.m21, c.d1, r, s1); continue; }
    r -= c.n1;
    if (r < c.n3) { cincr_entry(g.m23, g.d3, g.n3, c.m23, c.d3, r, s3); continue; }
    r -= c.n3;
    if (r < c.n1) { cincr_entry(g.m31, g.d1, g.n1, c.m31, c.d1, r, s1); continue; }
    r -= c.n1;
    cincr_entry(g.m32, g.d2, g.n2, c.m32, c.d2, r, s2);
  }
}

// ComputeFull_1D/2D/3D (TriDiagT_Mod.f90:62-90, 330-403, 790-883) for every
// cell of a level: the diagonal accumulates, in the reference's order, 1e-40,
// the two z terms, FacAnela*Vol, the two x terms and the two y terms; u/l are
// the negated coupling terms.  full = 1: the 3D level's own planes (y terms
// without DUU3 except the low boundary term, and the y couplings u3/l3);
// full = 0: a coarse plane level (DUU3 in every y term).
__global__ void k_assemble(Fields c, Lev2 P, double* __restrict__ u3, double* __restrict__ l3, int full, double bd2,
                           Facs fc, double fac_anela) {
  const int n1 = c.n1, n2 = c.n2, n3 = c.n3;
  const size_t tot = (size_t)n1 * n2 * n3;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot; e += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(e % n2) + 1;
    const size_t r = e / n2;
    const int i = (int)(r % n1) + 1, k = (int)(r / n1) + 1;
    const double M1 = c.m12[j - 1], M2 = c.m13[k - 1];
    const double M21 = c.m21[i - 1], M23 = c.m23[k - 1];
    const double M31 = c.m31[i - 1], M32 = c.m32[j - 1];
    auto DUT = [&](int ii, int jj, int kk) { return c.dut[c.ic(ii, jj, kk)]; };
    // face f (0-based) separates 1-based cells f and f+1
    auto zt = [&](int f, int cell) {
      const size_t q = c.i1(f, j, k);
      return bd2 * 2.0 * c.F1[q] * c.T1[q] * c.U1[q] * DUT(cell, j, k) / ((c.d1[f - 1] + c.d1[f]) * M1 * M2);
    };
    auto xt = [&](int f, int col) {
      const size_t q = c.i2(i, f, k);
      return bd2 * 2.0 * c.F2[q] * c.T2[q] * c.U2[q] * DUT(i, col, k) / ((c.d2[f - 1] + c.d2[f]) * M21 * M23);
    };
    auto yt = [&](int f, int pl, bool with_u) {
      const size_t q = c.i3(i, j, f);
      const double den = (c.d3[f - 1] + c.d3[f]) * M31 * M32;
      return with_u ? bd2 * 2.0 * c.F3[q] * c.T3[q] * c.U3[q] * DUT(i, j, pl) / den
                    : bd2 * 2.0 * c.F3[q] * c.T3[q] * DUT(i, j, pl) / den;
    };
    double dg = kTiny;
    {
      const size_t q0 = c.i1(0, j, k), qn = c.i1(n1, j, k);
      const double fl = bd2 * fc.f1l * c.F1[q0] * c.T1[q0] * c.U1[q0] * DUT(1, j, k) / (c.d1[0] * M1 * M2);
      const double fr = bd2 * fc.f1r * c.F1[qn] * c.T1[qn] * c.U1[qn] * DUT(n1, j, k) / (c.d1[n1 - 1] * M1 * M2);
      dg = dg + (i == 1 ? fl : zt(i - 1, i));
      dg = dg + (i == n1 ? fr : zt(i, i));
    }
    dg = dg + fac_anela * c.vol[c.ic(i, j, k)];
    {
      const size_t q0 = c.i2(i, 0, k), qn = c.i2(i, n2, k);
      const double fl = bd2 * fc.f2l * c.F2[q0] * c.T2[q0] * c.U2[q0] * DUT(i, 1, k) / (c.d2[0] * M21 * M23);
      const double fr = bd2 * fc.f2r * c.F2[qn] * c.T2[qn] * c.U2[qn] * DUT(i, n2, k) / (c.d2[n2 - 1] * M21 * M23);
      dg = dg + (j == 1 ? fl : xt(j - 1, j));
      dg = dg + (j == n2 ? fr : xt(j, j));
    }
    {
      const size_t q0 = c.i3(i, j, 0), qn = c.i3(i, j, n3);
      const double fl = bd2 * fc.f3l * c.F3[q0] * c.T3[q0] * c.U3[q0] * DUT(i, j, 1) / (c.d3[0] * M31 * M32);
      const double fr = full ? bd2 * fc.f3r * c.F3[qn] * c.T3[qn] * DUT(i, j, n3) / (c.d3[n3 - 1] * M31 * M32)
                             : bd2 * fc.f3r * c.F3[qn] * c.T3[qn] * c.U3[qn] * DUT(i, j, n3) / (c.d3[n3 - 1] * M31 * M32);
      dg = dg + (k == 1 ? fl : yt(k - 1, k, !full));
      dg = dg + (k == n3 ? fr : yt(k, k, !full));
    }
    const size_t s = (size_t)(k - 1) * P.ps + slot(P.w, P.h, i - 1, j - 1);
    P.d[s] = dg;
    P.uz[s] = i < n1 ? -zt(i, i + 1) : 0.0;
    P.lz[s] = i < n1 ? -zt(i, i) : 0.0;
    P.ux[s] = j < n2 ? -xt(j, j + 1) : 0.0;
    P.lx[s] = j < n2 ? -xt(j, j) : 0.0;
    if (full) {
      u3[s] = k < n3 ? -yt(k, k + 1, false) : 0.0;
      l3[s] = k < n3 ? -yt(k, k, false) : 0.0;
    }
  }
}

// The couplings across the periodic sides of one level of the periodic-
// Laplacian hierarchy (the refined mode's FGMRES preconditioner on blocks
// with periodic sides): the interior-face terms of ComputeFull_2D/3D
// (MULTI/TriDiagT_Mod.f90:330-403, 790-883) applied to the shared face between
// the last and the first line (x) or plane (y), coefficient
// -(beta0*dtP)^2*2*F*DT*DU*DUT(column)/((d(first)+d(last))*Metr); the y
// couplings of a 3D level carry no DU, like its interior ones.  Its
// diagonal terms come from k_assemble with boundary factor 1 on those sides.
__global__ void k_assemble_wrap(Fields c, Lev2 P, double* __restrict__ wyl, double* __restrict__ wyh, int full,
                                int per_x, int per_y, double bd2) {
  const int n1 = c.n1, n2 = c.n2, n3 = c.n3;
  const size_t nxw = per_x ? (size_t)n1 * n3 : 0, nyw = (per_y && full) ? (size_t)n1 * n2 : 0;
  auto DUT = [&](int ii, int jj, int kk) { return c.dut[c.ic(ii, jj, kk)]; };
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < nxw + nyw; e += (size_t)gridDim.x * blockDim.x) {
    if (e < nxw) {
      const int i = (int)(e % n1) + 1, k = (int)(e / n1) + 1;
      const size_t q = c.i2(i, 0, k);
      const double den = (c.d2[0] + c.d2[n2 - 1]) * c.m21[i - 1] * c.m23[k - 1];
      const double base = bd2 * 2.0 * c.F2[q] * c.T2[q] * c.U2[q];
      P.wxl[(size_t)(k - 1) * n1 + (i - 1)] = -(base * DUT(i, n2, k) / den);
      P.wxh[(size_t)(k - 1) * n1 + (i - 1)] = -(base * DUT(i, 1, k) / den);
    } else {
      const size_t r = e - nxw;
      const int i = (int)(r % n1) + 1, j = (int)(r / n1) + 1;
      const size_t q = c.i3(i, j, 0);
      const double den = (c.d3[0] + c.d3[n3 - 1]) * c.m31[i - 1] * c.m32[j - 1];
      const double base = bd2 * 2.0 * c.F3[q] * c.T3[q];
      const size_t s = slot(P.w, P.h, i - 1, j - 1);
      wyl[s] = -(base * DUT(i, j, n3) / den);
      wyh[s] = -(base * DUT(i, j, 1) / den);
    }
  }
}

// Thomas factors of every column (the t and w of Solve_1D, which depend on
// the matrix only): ft = t_i, frt = 1/t_i, fw = u_i/t_i
__global__ void k_factor(Lev2 P) {
  const size_t ncol = (size_t)P.m3 * P.c2;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < ncol; e += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(e % P.c2), k = (int)(e / P.c2);
    const size_t base = (size_t)k * P.ps + slot(P.w, P.h, 0, j);
    double t = P.d[base];
    P.ft[base] = t;
    P.frt[base] = 1.0 / t;
    for (int i = 1; i < P.c1; ++i) {
      const size_t q = base + (size_t)i * P.w, qm = q - P.w;
      const double wv = P.uz[qm] / t;
      P.fw[qm] = wv;
      t = P.d[q] - P.lz[qm] * wv;
      P.ft[q] = t;
      P.frt[q] = 1.0 / t;
    }
    P.fw[base + (size_t)(P.c1 - 1) * P.w] = 0.0;
  }
}

// ---------------------------------------------------------------------------
// Operator and multigrid
// ---------------------------------------------------------------------------

// MatVecT_2D at entry (i,j) of a plane (TriDiagT_Mod.f90:113-133, 405-431);
// x is the plane's vector, mo the plane's offset in the matrix arrays
template <typename T, bool kWrap = false>
__device__ inline T matvec2_at(const Lev2T<T>& P, size_t mo, const T* __restrict__ x, size_t s, int i, int j,
                               int k) {
  const int c1 = P.c1, c2 = P.c2, w = P.w;
  const T* d = P.d + mo;
  const T* uz = P.uz + mo;
  const T* lz = P.lz + mo;
  T y;
  if (c1 > 1) {
    if (i == 0)
      y = d[s] * x[s] + uz[s] * x[s + w];
    else if (i < c1 - 1)
      y = lz[s - w] * x[s - w] + d[s] * x[s] + uz[s] * x[s + w];
    else
      y = lz[s - w] * x[s - w] + d[s] * x[s];
  } else {
    y = d[s] * x[s];
  }
  if (c2 > 1) {
    const size_t row = (size_t)i * w;
    const T* ux = P.ux + mo;
    const T* lx = P.lx + mo;
    if (j == 0) {
      const size_t sr = row + slot(0, P.h, 0, j + 1);
      y = y + ux[s] * x[sr];
    } else if (j < c2 - 1) {
      const size_t sl = row + slot(0, P.h, 0, j - 1), sr = row + slot(0, P.h, 0, j + 1);
      y = y + lx[sl] * x[sl] + ux[s] * x[sr];
    } else {
      const size_t sl = row + slot(0, P.h, 0, j - 1);
      y = y + lx[sl] * x[sl];
    }
  }
  if (kWrap && P.wxl && (j == 0 || j == c2 - 1)) {  // periodic-Laplacian hierarchy: across the periodic x side
    const size_t row = (size_t)i * w, kc = (size_t)k * c1;
    if (j == 0) y = y + P.wxl[kc + i] * x[row + slot(0, P.h, 0, c2 - 1)];
    if (j == c2 - 1) y = y + P.wxh[kc + i] * x[row];
  }
  return y;
}

// One zebra half-sweep over the x-lines of parity c of one plane: the line
// right-hand side in the forward or backward operation order of
// GaussSeidel_2D, then Solve_1D with the precomputed factors.  The forward
// elimination streams the eight inputs of each row (b, the two neighbour
// lines, their couplings, the sub-diagonal of the previous row, the pivot
// and its reciprocal) through a per-thread ring of kRing rows in shared
// memory with cp.async, kAhead rows ahead of the recurrence; the copies read
// only the other parity's lines and the matrix, never this thread's column.
// The back substitution loads x and w four rows ahead in two register sets.
// Ring depth by value type: the same 64 KB per CTA hold 4 FP64 rows or 8 FP32
// rows, so the FP32 copy keeps twice as many rows in flight.
template <typename T>
struct RingCfg {
  static constexpr int ring = 4, ahead = 3;
};
template <>
struct RingCfg<float> {
  static constexpr int ring = 8, ahead = 7;
};
constexpr int kFields = 8;

__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// One half-sweep of the line solves with K lanes per line (FP32 copy only:
// the refined mode's preconditioner need not reproduce the reference's
// rounding).  On the coarsest plane levels a half-sweep has a handful of
// lines, and one thread per line left most of the block waiting at the
// barrier while a 128-row recurrence ran.  Both recurrences of the factored line system --
// forward y(i) = (t(i) - lz(i-1)*y(i-1))/ft(i) (the coupling of row i is
// stored at row i-1), backward x(i) = y(i) - fw(i)*x(i+1) -- are first-order
// affine recurrences, so each lane composes
// the affine map of its chunk of rows, a shuffle scan over the K lanes gives
// every chunk its entry value, and each lane re-runs its chunk with the
// sequential formulas (a chunked scan).  The line right-hand side t(i) is the
// one of the sequential sweep, neighbour lines and wrap couplings included.
template <typename T, bool kWrap>
__device__ void line_half_lanes(const Lev2T<T>& P, size_t mo, const T* __restrict__ b, T* __restrict__ x, int c,
                                int fwd, int K) {
  const int c1 = P.c1, c2 = P.c2, h = P.h, w = P.w;
  const T* __restrict__ lx = P.lx + mo;
  const T* __restrict__ ux = P.ux + mo;
  const T* __restrict__ lz = P.lz + mo;
  const T* __restrict__ ft = P.ft + mo;
  const T* __restrict__ frt = P.frt + mo;
  const T* __restrict__ fw = P.fw + mo;
  const int nl = (c2 - c + 1) / 2;
  const int q = threadIdx.x / K, p = threadIdx.x % K;
  const bool active = q < nl;
  const int j = 2 * q + c;
  const size_t col = (size_t)c * h + q;
  const bool hasL = j > 0, hasR = j < c2 - 1;
  const size_t colL = hasL ? (size_t)(1 - c) * h + ((j - 1) >> 1) : col;
  const size_t colR = hasR ? (size_t)(1 - c) * h + ((j + 1) >> 1) : col;
  const bool wrap = kWrap && P.wxl && c2 >= 2 && ((c2 - 1) & 1);
  const bool wL = wrap && j == 0, wR = wrap && j == c2 - 1;
  const bool useL = hasL || wL, useR = hasR || wR;
  const size_t wk = (mo / P.ps) * (size_t)c1;
  const size_t xL0 = wL ? slot(0, h, 0, c2 - 1) : colL, xR0 = wR ? slot(0, h, 0, 0) : colR;
  const int rows = (c1 + K - 1) / K;
  const int r0 = active ? min(c1, p * rows) : 0, r1 = active ? min(c1, r0 + rows) : 0;
  auto rhs = [&](int i) {
    const size_t o = (size_t)i * w;
    T t = b[col + o];
    const T xl = useL ? x[xL0 + o] : (T)0, cl = useL ? (wL ? P.wxl[wk + i] : lx[colL + o]) : (T)0;
    const T xr = useR ? x[xR0 + o] : (T)0, cr = useR ? (wR ? P.wxh[wk + i] : ux[col + o]) : (T)0;
    if (fwd) {
      if (useL) t = t - cl * xl;
      if (useR) t = t - cr * xr;
    } else {
      if (useR) t = t - cr * xr;
      if (useL) t = t - cl * xl;
    }
    return t;
  };
  // forward: the chunk's map y(r1-1) = A*y(r0-1) + B
  T A = (T)1, B = (T)0;
  for (int i = r0; i < r1; ++i) {
    const T ri = frt[col + (size_t)i * w];
    const T a = i > 0 ? -(lz[col + (size_t)(i - 1) * w] * ri) : (T)0;  // row i's coupling is stored at row i-1
    A = a * A;
    B = a * B + rhs(i) * ri;
  }
  for (int off = 1; off < K; off <<= 1) {  // inclusive scan over the lanes, chunk 0 first
    const T Ap = __shfl_up_sync(0xffffffffu, A, off, K), Bp = __shfl_up_sync(0xffffffffu, B, off, K);
    if (p >= off) B = A * Bp + B, A = A * Ap;
  }
  T prev = __shfl_up_sync(0xffffffffu, B, 1, K);  // y before the chunk (the whole line starts from 0)
  if (p == 0) prev = (T)0;
  for (int i = r0; i < r1; ++i) {
    T t = rhs(i);
    if (i > 0) t = t - lz[col + (size_t)(i - 1) * w] * prev;
    const T y = div_rn(t, ft[col + (size_t)i * w], frt[col + (size_t)i * w]);
    x[col + (size_t)i * w] = y;
    prev = y;
  }
  // backward: the chunk's map x(r0) = A*x(r1) + B (row c1-1 takes y alone)
  A = (T)1, B = (T)0;
  for (int i = r1 - 1; i >= r0; --i) {
    const T a = i < c1 - 1 ? -fw[col + (size_t)i * w] : (T)0;
    A = a * A;
    B = a * B + x[col + (size_t)i * w];
  }
  for (int off = 1; off < K; off <<= 1) {  // inclusive scan from the last chunk down
    const T An = __shfl_down_sync(0xffffffffu, A, off, K), Bn = __shfl_down_sync(0xffffffffu, B, off, K);
    if (p + off < K) B = A * Bn + B, A = A * An;
  }
  T next = __shfl_down_sync(0xffffffffu, B, 1, K);  // x after the chunk
  for (int i = r1 - 1; i >= r0; --i) {
    const T y = x[col + (size_t)i * w];
    const T v = i < c1 - 1 ? y - fw[col + (size_t)i * w] * next : y;
    x[col + (size_t)i * w] = v;
    next = v;
  }
}

template <typename T, bool kWrap = false>
__device__ __noinline__ void line_half(const Lev2T<T>& P, size_t mo, const T* __restrict__ b, T* __restrict__ x, int c,
                                       int fwd, T* __restrict__ ring) {
  if constexpr (sizeof(T) == 4) {  // few lines: K lanes per line (the whole block takes part in the shuffles)
    const int nl = (P.c2 - c + 1) / 2;
    int K = 1;
    while (K < 32 && nl * K * 2 <= (int)blockDim.x && K * 4 <= P.c1) K *= 2;
    if (K >= 8) {  // from 8 lanes up; with 2-4 lanes the prefetched sequential sweep below was faster
      line_half_lanes<T, kWrap>(P, mo, b, x, c, fwd, K);
      return;
    }
  }
  const int c1 = P.c1, c2 = P.c2, h = P.h, w = P.w;
  const T* __restrict__ lx = P.lx + mo;
  const T* __restrict__ ux = P.ux + mo;
  const T* __restrict__ lz = P.lz + mo;
  const T* __restrict__ ft = P.ft + mo;
  const T* __restrict__ frt = P.frt + mo;
  const T* __restrict__ fw = P.fw + mo;
  constexpr int kRing = RingCfg<T>::ring, kAhead = RingCfg<T>::ahead;
  const int nl = (c2 - c + 1) / 2;
  const int bd = blockDim.x, tid = threadIdx.x;
  for (int q = tid; q < nl; q += bd) {
    const int j = 2 * q + c;
    const size_t col = (size_t)c * h + q;
    const bool hasL = j > 0, hasR = j < c2 - 1;
    const size_t colL = hasL ? (size_t)(1 - c) * h + ((j - 1) >> 1) : col;
    const size_t colR = hasR ? (size_t)(1 - c) * h + ((j + 1) >> 1) : col;
    // periodic-Laplacian hierarchy: line 0's left neighbour is line c2-1 and
    // line c2-1's right neighbour is line 0, across the periodic side; used
    // only when the two have different parities (no line reads a line of its
    // own half-sweep).  The wrap neighbour and its coupling take the ring
    // slots of the missing neighbour, so they stream ahead like the others.
    const bool wrap = kWrap && P.wxl && c2 >= 2 && ((c2 - 1) & 1);
    const bool wL = wrap && j == 0, wR = wrap && j == c2 - 1;
    const bool useL = hasL || wL, useR = hasR || wR;
    const size_t wk = (mo / P.ps) * (size_t)c1;
    const size_t xL0 = wL ? slot(0, h, 0, c2 - 1) : colL, xR0 = wR ? slot(0, h, 0, 0) : colR;
    auto issue = [&](int i) {
      T* sl = ring + (size_t)(i % kRing) * kFields * bd + tid;
      const bool ok = i < c1;
      const size_t io = ok ? (size_t)i : 0, o = io * w;
      const size_t om = i > 0 && ok ? o - w : o;
      cp_async_elem(sl + 0 * bd, b + col + o, ok);
      cp_async_elem(sl + 1 * bd, x + xL0 + o, ok && useL);
      cp_async_elem(sl + 2 * bd, x + xR0 + o, ok && useR);
      cp_async_elem(sl + 3 * bd, wL ? P.wxl + wk + io : lx + colL + o, ok && useL);
      cp_async_elem(sl + 4 * bd, wR ? P.wxh + wk + io : ux + col + o, ok && useR);
      cp_async_elem(sl + 5 * bd, lz + col + om, ok && i > 0);
      cp_async_elem(sl + 6 * bd, ft + col + o, ok);
      cp_async_elem(sl + 7 * bd, frt + col + o, ok);
      cp_commit();
    };
    for (int r = 0; r < kAhead; ++r) issue(r);
    T prev = (T)0;
    for (int i = 0; i < c1; ++i) {
      issue(i + kAhead);
      cp_wait<kAhead>();
      const T* sl = ring + (size_t)(i % kRing) * kFields * bd + tid;
      T t = sl[0];
      if (fwd) {
        if (useL) t = t - sl[3 * bd] * sl[1 * bd];
        if (useR) t = t - sl[4 * bd] * sl[2 * bd];
      } else {
        if (useR) t = t - sl[4 * bd] * sl[2 * bd];
        if (useL) t = t - sl[3 * bd] * sl[1 * bd];
      }
      if (i > 0) t = t - sl[5 * bd] * prev;
      const T y = div_rn(t, sl[6 * bd], sl[7 * bd]);
      x[col + (size_t)i * w] = y;
      prev = y;
    }
    cp_wait<0>();
    // back substitution b(i) = b(i) - w(i)*b(i+1), rows c1-2 .. 0
    const int nb = c1 - 1;
    T xa[4], wa[4], xb[4], wb[4];
    auto load4 = [&](T* xs, T* ws, int r0) {
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const int i = c1 - 2 - (r0 + r);
        if (i >= 0) {
          xs[r] = x[col + (size_t)i * w];
          ws[r] = fw[col + (size_t)i * w];
        }
      }
    };
    auto solve4 = [&](const T* xs, const T* ws, int r0) {
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const int i = c1 - 2 - (r0 + r);
        if (i >= 0) {
          const T v = xs[r] - ws[r] * prev;
          x[col + (size_t)i * w] = v;
          prev = v;
        }
      }
    };
    if (nb > 0) load4(xa, wa, 0);
    for (int r0 = 0; r0 < nb; r0 += 8) {
      load4(xb, wb, r0 + 4);
      solve4(xa, wa, r0);
      load4(xa, wa, r0 + 8);
      solve4(xb, wb, r0 + 4);
    }
  }
}

template <typename T, bool kWrap = false>
__device__ void gs2d(const Lev2T<T>& P, size_t mo, const T* b, T* x, int gi, T* ring) {
  if (P.c2 > 1) {
    for (int it = 0; it < gi; ++it) {
      line_half<T, kWrap>(P, mo, b, x, 0, 1, ring);
      __syncthreads();
      line_half<T, kWrap>(P, mo, b, x, 1, 1, ring);
      __syncthreads();
      line_half<T, kWrap>(P, mo, b, x, 1, 0, ring);
      __syncthreads();
      line_half<T, kWrap>(P, mo, b, x, 0, 0, ring);
      __syncthreads();
    }
  } else {
    line_half<T, kWrap>(P, mo, b, x, 0, 1, ring);
    __syncthreads();
  }
}

// Multigrid_2D (TriDiagT_Mod.f90:490-551) on plane k of a 3D level, inside one CTA
template <typename T, bool kWrap = false>
__device__ void mg2d(const Lev3T<T>& A, int k, T* x0, const T* b0, int gi2, T* ring) {
  const int nl = A.nl;
  int gi = 1;
  int lv = 0;
  for (;;) {
    const Lev2T<T>& P = A.pl[lv];
    T* x = lv == 0 ? x0 : P.x + (size_t)k * P.ps;
    const T* b = lv == 0 ? b0 : P.b + (size_t)k * P.ps;
    const size_t mo = (size_t)k * P.ps;
    gs2d<T, kWrap>(P, mo, b, x, gi, ring);
    gi += gi2;
    if (lv + 1 < nl) {
      T* res = P.res + (size_t)k * P.ps;
      const size_t np = P.ps;
      for_plane(P.w, np, [&](size_t s, int i, int r) {
        const int j = line_of(r, P.h, P.c2);
        if (j >= 0) res[s] = b[s] - matvec2_at<T, kWrap>(P, mo, x, s, i, j, k);
      });
      __syncthreads();
      const Lev2T<T>& Q = A.pl[lv + 1];
      T* bq = Q.b + (size_t)k * Q.ps;
      T* xq = Q.x + (size_t)k * Q.ps;
      for_plane(Q.w, Q.ps, [&](size_t s, int a, int r) {
        const int bb = line_of(r, Q.h, Q.c2);
        if (bb < 0) return;
        T v = (T)0;
        for (int i1 = 2 * a; i1 <= 2 * a + 1 && i1 < P.c1; ++i1)
          for (int i2 = 2 * bb; i2 <= 2 * bb + 1 && i2 < P.c2; ++i2) v = v + res[slot(P.w, P.h, i1, i2)];
        bq[s] = v;
        xq[s] = (T)0;
      });
      __syncthreads();
      ++lv;
    } else {
      gi -= gi2;
      break;
    }
  }
  for (;;) {
    const Lev2T<T>& P = A.pl[lv];
    T* x = lv == 0 ? x0 : P.x + (size_t)k * P.ps;
    const T* b = lv == 0 ? b0 : P.b + (size_t)k * P.ps;
    gs2d<T, kWrap>(P, (size_t)k * P.ps, b, x, gi, ring);
    gi -= gi2;
    if (lv > 0) {
      const Lev2T<T>& F = A.pl[lv - 1];
      T* xf = lv - 1 == 0 ? x0 : F.x + (size_t)k * F.ps;
      for_plane(F.w, F.ps, [&](size_t s, int i, int r) {
        const int j = line_of(r, F.h, F.c2);
        if (j >= 0) xf[s] = xf[s] + x[slot(P.w, P.h, i >> 1, j >> 1)];
      });
      __syncthreads();
      --lv;
    } else {
      break;
    }
  }
}

// One zebra half-sweep of GaussSeidel_3D over the planes of parity `color` of
// 3D level L: each CTA forms its plane's right-hand side (forward or backward
// operation order of the reference) and runs Solve_2D on it.
template <typename T, bool kWrap = false>
__global__ void __launch_bounds__(kPlaneBlock, 2) k_plane_half(const Lev3T<T>* __restrict__ lvs, int L, int color, int fwd,
                                                             int mult_iter2, int gi2) {
  __shared__ Lev3T<T> A;
  extern __shared__ __align__(16) unsigned char ring_raw[];  // kRing * kFields * blockDim values of T
  T* ring = reinterpret_cast<T*>(ring_raw);
  if (threadIdx.x == 0) A = lvs[L];
  __syncthreads();
  const Lev2T<T>& P0 = A.pl[0];
  for (int q = blockIdx.x;; q += gridDim.x) {
    const int k = 2 * q + color;
    if (k >= A.m3) break;
    const size_t off = (size_t)k * P0.ps, ps = P0.ps;
    for_plane(P0.w, ps, [&](size_t s, int, int r) {
      if (line_of(r, P0.h, P0.c2) < 0) return;
      const size_t e = off + s;
      T v = A.b[e];
      if (fwd) {
        if (k > 0) v = v - A.l3[e - ps] * A.x[e - ps];
        if (k < A.m3 - 1) v = v - A.u3[e] * A.x[e + ps];
      } else {
        if (k < A.m3 - 1) v = v - A.u3[e] * A.x[e + ps];
        if (k > 0) v = v - A.l3[e - ps] * A.x[e - ps];
      }
      // periodic-Laplacian hierarchy: the plane across the periodic y side
      // (only when planes 0 and m3-1 have different parities)
      if (kWrap && A.wyl && A.m3 >= 2 && ((A.m3 - 1) & 1)) {
        if (k == 0) v = v - A.wyl[s] * A.x[(size_t)(A.m3 - 1) * ps + s];
        if (k == A.m3 - 1) v = v - A.wyh[s] * A.x[s];
      }
      A.t[e] = v;
    });
    __syncthreads();
    for (int it = 0; it < mult_iter2; ++it) mg2d<T, kWrap>(A, k, A.x + off, A.t + off, gi2, ring);
    __syncthreads();
  }
}

// MatVecT_3D at every entry of level L: mode 0 res = b - A x; mode 1 y = -(A x)
// (MatVecFull's sign); mode 2 y = A x.
template <typename T, bool kWrap = false>
__global__ void k_matvec3(const Lev3T<T>* __restrict__ lvs, int L, const T* __restrict__ x, const T* __restrict__ b,
                          T* __restrict__ y, int mode) {
  const Lev3T<T>& A = lvs[L];
  const Lev2T<T>& P = A.pl[0];
  const size_t tot = (size_t)A.m3 * P.ps, ps = P.ps;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot; e += (size_t)gridDim.x * blockDim.x) {
    const size_t s = e % ps;
    const int k = (int)(e / ps);
    const int i = (int)(s / P.w), j = line_of((int)(s % P.w), P.h, P.c2);
    if (j < 0) continue;
    T v = matvec2_at<T, kWrap>(P, (size_t)k * ps, x + (size_t)k * ps, s, i, j, k);
    if (A.m3 > 1) {
      if (k == 0)
        v = v + A.u3[e] * x[e + ps];
      else if (k < A.m3 - 1)
        v = v + A.l3[e - ps] * x[e - ps] + A.u3[e] * x[e + ps];
      else
        v = v + A.l3[e - ps] * x[e - ps];
    }
    if (kWrap && A.wyl) {  // periodic-Laplacian hierarchy: across the periodic y side
      if (k == 0) v = v + A.wyl[s] * x[(size_t)(A.m3 - 1) * ps + s];
      if (k == A.m3 - 1) v = v + A.wyh[s] * x[s];
    }
    y[e] = mode == 0 ? b[e] - v : (mode == 1 ? -v : v);
  }
}

// RestrictT_3D (level L residual -> level L+1 right-hand side), zero x of L+1
template <typename T>
__global__ void k_restrict3(const Lev3T<T>* __restrict__ lvs, int L) {
  const Lev3T<T>& A = lvs[L];
  const Lev3T<T>& C = lvs[L + 1];
  const Lev2T<T>& P = A.pl[0];
  const Lev2T<T>& Q = C.pl[0];
  const size_t tot = (size_t)C.m3 * Q.ps;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot; e += (size_t)gridDim.x * blockDim.x) {
    const size_t s = e % Q.ps;
    const int kc = (int)(e / Q.ps);
    const int a = (int)(s / Q.w), bb = line_of((int)(s % Q.w), Q.h, Q.c2);
    if (bb < 0) continue;
    T v = (T)0;
    for (int i1 = 2 * a; i1 <= 2 * a + 1 && i1 < P.c1; ++i1)
      for (int i2 = 2 * bb; i2 <= 2 * bb + 1 && i2 < P.c2; ++i2)
        for (int i3 = 2 * kc; i3 <= 2 * kc + 1 && i3 < A.m3; ++i3) v = v + A.res[(size_t)i3 * P.ps + slot(P.w, P.h, i1, i2)];
    C.b[e] = v;
    C.x[e] = (T)0;
  }
}

// ProlongateT_3D + x = x + Res (level L+1 -> level L)
template <typename T>
__global__ void k_prolong3(const Lev3T<T>* __restrict__ lvs, int L) {
  const Lev3T<T>& A = lvs[L];
  const Lev3T<T>& C = lvs[L + 1];
  const Lev2T<T>& P = A.pl[0];
  const Lev2T<T>& Q = C.pl[0];
  const size_t tot = (size_t)A.m3 * P.ps;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot; e += (size_t)gridDim.x * blockDim.x) {
    const size_t s = e % P.ps;
    const int k = (int)(e / P.ps);
    const int i = (int)(s / P.w), j = line_of((int)(s % P.w), P.h, P.c2);
    if (j < 0) continue;
    A.x[e] = A.x[e] + C.x[(size_t)(k >> 1) * Q.ps + slot(Q.w, Q.h, i >> 1, j >> 1)];
  }
}

// natural (x,y,z) interior <-> level-0 layout (z,x,y)
__global__ void k_to_layout(Lev2 P, int nx, int ny, int nz, const double* __restrict__ nat, double* __restrict__ lay,
                            double scale) {
  const size_t tot = (size_t)nx * ny * nz;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot; e += (size_t)gridDim.x * blockDim.x) {
    const int x = (int)(e % nx);
    const size_t r = e / nx;
    const int y = (int)(r % ny), z = (int)(r / ny);
    const double v = nat[e];
    lay[(size_t)y * P.ps + slot(P.w, P.h, z, x)] = scale == 1.0 ? v : scale * v;
  }
}
__global__ void k_from_layout(Lev2 P, int nx, int ny, int nz, const double* __restrict__ lay, double* __restrict__ nat) {
  const size_t tot = (size_t)nx * ny * nz;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot; e += (size_t)gridDim.x * blockDim.x) {
    const int x = (int)(e % nx);
    const size_t r = e / nx;
    const int y = (int)(r % ny), z = (int)(r / ny);
    nat[e] = lay[(size_t)y * P.ps + slot(P.w, P.h, z, x)];
  }
}

// ---------------------------------------------------------------------------
// FGMRES vector kernels (padding entries of the layout stay 0)
// ---------------------------------------------------------------------------
__global__ void k_pdot_partial(const double* __restrict__ a, const double* __restrict__ b, size_t n,
                               double* __restrict__ partial) {
  __shared__ double sh[kRedBlock];
  double s = 0.0;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x)
    s = s + a[e] * b[e];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] = sh[threadIdx.x] + sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}
// out = sum (mode 0) or sqrt(sum) (mode 1)
__global__ void k_pdot_final(const double* __restrict__ partial, int n, double* out, int mode) {
  __shared__ double sh[kRedBlock];
  double s = 0.0;
  for (int e = threadIdx.x; e < n; e += blockDim.x) s = s + partial[e];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] = sh[threadIdx.x] + sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = mode == 1 ? sqrt(sh[0]) : sh[0];
}
// y = (-*h)*x + y   (DAXPY with the Gram-Schmidt coefficient held on the device)
__global__ void k_axpy_negdev(double* __restrict__ y, const double* __restrict__ x, const double* h, size_t n) {
  const double a = -*h;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x)
    y[e] = a * x[e] + y[e];
}
// v = (1/*h)*v   (DSCALE(One/H(i+1,i)))
__global__ void k_scale_recipdev(double* __restrict__ v, const double* h, size_t n) {
  const double a = 1.0 / *h;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) v[e] = a * v[e];
}
// y = a*x + y (host scalar)
__global__ void k_axpy(double* __restrict__ y, const double* __restrict__ x, double a, size_t n) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x)
    y[e] = a * x[e] + y[e];
}
// y = x + a*y (DXPBY)
__global__ void k_xpby(const double* __restrict__ x, double a, double* __restrict__ y, size_t n) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x)
    y[e] = x[e] + a * y[e];
}
// v = a*v
__global__ void k_scale(double* __restrict__ v, double a, size_t n) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) v[e] = a * v[e];
}
// y = -x
__global__ void k_neg(double* __restrict__ y, const double* __restrict__ x, size_t n) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) y[e] = -x[e];
}

// ---------------------------------------------------------------------------
// Rhs / UpdateVelocity (MATRIX/Rhs_Mod.f90)
// ---------------------------------------------------------------------------
struct Wts {
  double *dtu, *dtv, *dtw, *duu, *duv, *duw, *dut, *dtt;
  double *dx, *dy, *dz, *metr;
};

// Rhs with DivergenceS: b = beta0*dtP*div (- VolB*incr_th), written in the level-0 layout
__global__ void k_rhs(Dims d, GeomT<double> g, Wts wt, const double* __restrict__ u, const double* __restrict__ v,
                      const double* __restrict__ w, const double* __restrict__ incr_th, double bdt, int anela,
                      Lev2 P, double* __restrict__ b) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const size_t tot = (size_t)nx * ny * nz;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot; e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e % nx) + 1;
    const size_t r = e / nx;
    const int j = (int)(r % ny) + 1, k = (int)(r / ny) + 1;
    const double div = (-(g.fu[d.FU(i - 1, j, k)] * wt.dtu[d.UF(i - 1, j, k)] * u[d.UF(i - 1, j, k)]) +
                        g.fu[d.FU(i, j, k)] * wt.dtu[d.UF(i, j, k)] * u[d.UF(i, j, k)] -
                        g.fv[d.FV(i, j - 1, k)] * wt.dtv[d.VF(i, j - 1, k)] * v[d.VF(i, j - 1, k)] +
                        g.fv[d.FV(i, j, k)] * wt.dtv[d.VF(i, j, k)] * v[d.VF(i, j, k)] -
                        g.fw[d.FW(i, j, k - 1)] * wt.dtw[d.WF(i, j, k - 1)] * w[d.WF(i, j, k - 1)] +
                        g.fw[d.FW(i, j, k)] * wt.dtw[d.WF(i, j, k)] * w[d.WF(i, j, k)]) *
                       wt.dtt[e];
    double val = bdt * div;
    if (incr_th && anela) val = val - g.volc[d.P(i, j, k)] * incr_th[d.P(i, j, k)];
    b[(size_t)(j - 1) * P.ps + slot(P.w, P.h, k - 1, i - 1)] = val;
  }
}

// UpdateVelocity, GradFull + MultiTriT: p = p*DUT, the boundary-face terms
// Temp = x%u_w - b%u_w/(...) (Rhs_Mod.f90:636-660; b's face parts are 0: the
// face unknown of a periodic side, 0 on a closed one) and u = utilde - grad p
// on interior faces.  pv is the solved PressureVelocity vector (its faces at fc).
__global__ void k_update_vel(Dims d, GeomT<double> g, Wts wt, double* __restrict__ p, const double* __restrict__ pv,
                             PvFaces fc, double* __restrict__ u, double* __restrict__ v, double* __restrict__ w,
                             double beta0, double dtp) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const double* mxy = wt.metr;
  const double* mxz = wt.metr + ny;
  const double* myx = wt.metr + ny + nz;
  const double* myz = wt.metr + ny + nz + nx;
  const double* mzx = wt.metr + ny + 2 * nz + nx;
  const double* mzy = wt.metr + ny + 2 * nz + 2 * nx;
  auto C = [&](int i, int j, int k) { return (size_t)(i - 1) + (size_t)nx * ((size_t)(j - 1) + (size_t)ny * (size_t)(k - 1)); };
  auto pd = [&](int i, int j, int k) { const size_t q = C(i, j, k); return p[q] * wt.dut[q]; };
  const size_t nu = (size_t)(nx + 1) * ny * nz, nv = (size_t)nx * (ny + 1) * nz, nw = (size_t)nx * ny * (nz + 1);
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < nu + nv + nw; e += (size_t)gridDim.x * blockDim.x) {
    if (e < nu) {
      const int i = (int)(e % (nx + 1));
      const size_t r = e / (nx + 1);
      const int j = (int)(r % ny) + 1, k = (int)(r / ny) + 1;
      if (i == 0 || i == nx) {
        const int side = i == 0 ? 0 : 1;
        const double xf = fc.off[side] >= 0 ? pv[fc.off[side] + (j - 1) + (size_t)ny * (k - 1)] : 0.0;
        const double t = xf - 0.0 / (0.5 * wt.dx[i == 0 ? 0 : nx - 1] * mxy[j - 1] * mxz[k - 1]);
        u[e] = u[e] + t;
      }
      if (i >= 1 && i <= nx - 1) {
        const double t = 2.0 * beta0 * dtp * wt.duu[e] * (pd(i + 1, j, k) - pd(i, j, k)) /
                         ((wt.dx[i] + wt.dx[i - 1]) * mxy[j - 1] * mxz[k - 1]);
        u[e] = u[e] - t;
      }
    } else if (e < nu + nv) {
      const size_t ee = e - nu;
      const int i = (int)(ee % nx) + 1;
      const size_t r = ee / nx;
      const int j = (int)(r % (ny + 1)), k = (int)(r / (ny + 1)) + 1;
      if (j == 0 || j == ny) {
        const int side = j == 0 ? 2 : 3;
        const double xf = fc.off[side] >= 0 ? pv[fc.off[side] + (i - 1) + (size_t)nx * (k - 1)] : 0.0;
        const double t = xf - 0.0 / (0.5 * wt.dy[j == 0 ? 0 : ny - 1] * myx[i - 1] * myz[k - 1]);
        v[ee] = v[ee] + t;
      }
      if (j >= 1 && j <= ny - 1) {
        const double t = 2.0 * beta0 * dtp * wt.duv[ee] * (pd(i, j + 1, k) - pd(i, j, k)) /
                         ((wt.dy[j] + wt.dy[j - 1]) * myx[i - 1] * myz[k - 1]);
        v[ee] = v[ee] - t;
      }
    } else {
      const size_t ee = e - nu - nv;
      const int i = (int)(ee % nx) + 1;
      const size_t r = ee / nx;
      const int j = (int)(r % ny) + 1, k = (int)(r / ny);
      const double fwv = g.fw[d.FW(i, j, k)];
      if (k == 0) {
        const double xf = fc.off[4] >= 0 ? pv[fc.off[4] + (i - 1) + (size_t)nx * (j - 1)] : 0.0;
        const double t = xf - 0.0 / (0.5 * wt.dz[0] * mzx[i - 1] * mzy[j - 1]);
        w[ee] = w[ee] + t;
      } else if (k == nz) {
        const double xf = fc.off[5] >= 0 ? pv[fc.off[5] + (i - 1) + (size_t)nx * (j - 1)] : 0.0;
        const double t = xf - 0.0 / (0.5 * wt.dz[nz - 1] * mzx[i - 1] * mzy[j - 1]);
        w[ee] = w[ee] + fwv / (fwv + asam::kEps) * t;
      }
      if (k >= 1 && k <= nz - 1) {
        const double t = 2.0 * beta0 * dtp * wt.duw[ee] * (pd(i, j, k + 1) - pd(i, j, k)) / (wt.dz[k] + wt.dz[k - 1]);
        w[ee] = w[ee] - fwv / (fwv + asam::kEps) * t;
      }
    }
  }
}

// p = p*DUT (the pressure the reference leaves in x after UpdateVelocity)
__global__ void k_scale_dut(double* __restrict__ p, const double* __restrict__ dut, size_t n) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) p[e] = p[e] * dut[e];
}

// ThPos / RhoPos increments and DivScalar of the other listed components
// (Rhs_Mod.f90:834-871, 915-950), all from the projected face velocities
__global__ void k_update_incr(Dims d, GeomT<double> g, Wts wt, const double* __restrict__ u, const double* __restrict__ v,
                              const double* __restrict__ w, double* __restrict__ incr, int th_pos, int rho_pos,
                              double beta0, double dtp) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const size_t npad = d.npad();
  const size_t tot = (size_t)nx * ny * nz;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot; e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e % nx) + 1;
    const size_t r = e / nx;
    const int j = (int)(r % ny) + 1, k = (int)(r / ny) + 1;
    const size_t P = d.P(i, j, k);
    const double vC = g.volc[P];
    const double fuR = g.fu[d.FU(i, j, k)], fuL = g.fu[d.FU(i - 1, j, k)];
    const double fvR = g.fv[d.FV(i, j, k)], fvL = g.fv[d.FV(i, j - 1, k)];
    const double fwR = g.fw[d.FW(i, j, k)], fwL = g.fw[d.FW(i, j, k - 1)];
    const double uR = u[d.UF(i, j, k)], uL = u[d.UF(i - 1, j, k)];
    const double vR = v[d.VF(i, j, k)], vL = v[d.VF(i, j - 1, k)];
    const double wR = w[d.WF(i, j, k)], wL = w[d.WF(i, j, k - 1)];
    if (th_pos >= 0) {
      const double s = fuR * wt.dtu[d.UF(i, j, k)] * uR - fuL * wt.dtu[d.UF(i - 1, j, k)] * uL +
                       fvR * wt.dtv[d.VF(i, j, k)] * vR - fvL * wt.dtv[d.VF(i, j - 1, k)] * vL +
                       fwR * wt.dtw[d.WF(i, j, k)] * wR - fwL * wt.dtw[d.WF(i, j, k - 1)] * wL;
      double* c = incr + (size_t)th_pos * npad;
      c[P] = c[P] - dtp * beta0 * wt.dtt[e] * s / (vC + asam::kEps);
    }
    if (rho_pos >= 0) {
      const double s = fuR * uR - fuL * uL + fvR * vR - fvL * vL + fwR * wR - fwL * wL;
      double* c = incr + (size_t)rho_pos * npad;
      c[P] = c[P] - dtp * beta0 * s / (vC + asam::kEps);
    }
  }
}

// DivScalar of UpdateVelocity for one scalar (MATRIX/Rhs_Mod.f90:589-952): the
// flux through a face is |F u| times the volume-weighted mean mixing ratio
// of its two cells, (m_L + m_R)/(V_L + V_R + Eps) with m = V c/(Rho + Eps).
// The reference evaluates each face once from either cell; the two
// evaluations are equal bit for bit (the sums are commutative, the product
// and the quotient are taken in the same order), so the face terms are
// computed once per face here: 5 divisions per cell instead of 14.
__global__ void k_div_m(size_t npad, const double* __restrict__ volc, const double* __restrict__ cc,
                        const double* __restrict__ rho, double* __restrict__ m) {
  for (size_t P = blockIdx.x * (size_t)blockDim.x + threadIdx.x; P < npad; P += (size_t)gridDim.x * blockDim.x)
    m[P] = volc[P] * cc[P] / (rho[P] + asam::kEps);
}

// face terms F = Fa * u * (m_L + m_R) / (V_L + V_R + Eps) of the u, v and w
// faces, in the face-velocity layouts
__global__ void k_div_faces(Dims d, GeomT<double> g, const double* __restrict__ u, const double* __restrict__ v,
                            const double* __restrict__ w, const double* __restrict__ m, double* __restrict__ fu,
                            double* __restrict__ fv, double* __restrict__ fw) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const size_t nu = d.n_uf(), nv = d.n_vf(), tot = nu + nv + d.n_wf();
  const size_t sy = (size_t)d.NX(), sz = (size_t)d.NX() * d.NY();
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot; e += (size_t)gridDim.x * blockDim.x) {
    if (e < nu) {  // i = 0..nx between cells i and i+1
      const int i = (int)(e % (nx + 1));
      const size_t r = e / (nx + 1);
      const int j = (int)(r % ny) + 1, k = (int)(r / ny) + 1;
      const size_t L = d.P(i, j, k), R = L + 1;
      fu[e] = g.fu[d.FU(i, j, k)] * u[e] * (m[L] + m[R]) / (g.volc[L] + g.volc[R] + asam::kEps);
    } else if (e < nu + nv) {  // j = 0..ny
      const size_t q = e - nu;
      const int i = (int)(q % nx) + 1;
      const size_t r = q / nx;
      const int j = (int)(r % (ny + 1)), k = (int)(r / (ny + 1)) + 1;
      const size_t L = d.P(i, j, k), R = L + sy;
      fv[q] = g.fv[d.FV(i, j, k)] * v[q] * (m[L] + m[R]) / (g.volc[L] + g.volc[R] + asam::kEps);
    } else {  // k = 0..nz
      const size_t q = e - nu - nv;
      const int i = (int)(q % nx) + 1;
      const size_t r = q / nx;
      const int j = (int)(r % ny) + 1, k = (int)(r / ny);
      const size_t L = d.P(i, j, k), R = L + sz;
      fw[q] = g.fw[d.FW(i, j, k)] * w[q] * (m[L] + m[R]) / (g.volc[L] + g.volc[R] + asam::kEps);
    }
  }
}

// the scalar's increment: incr -= dtP*beta0*(sum of the signed face terms)/(V + Eps)
__global__ void k_div_apply(Dims d, GeomT<double> g, const double* __restrict__ fu, const double* __restrict__ fv,
                            const double* __restrict__ fw, double* __restrict__ cd, double beta0, double dtp) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const size_t tot = (size_t)nx * ny * nz;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot; e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e % nx) + 1;
    const size_t r = e / nx;
    const int j = (int)(r % ny) + 1, k = (int)(r / ny) + 1;
    const size_t P = d.P(i, j, k);
    const double s = fu[d.UF(i, j, k)] - fu[d.UF(i - 1, j, k)] + fv[d.VF(i, j, k)] - fv[d.VF(i, j - 1, k)] +
                     fw[d.WF(i, j, k)] - fw[d.WF(i, j, k - 1)];
    cd[P] = cd[P] - dtp * beta0 * s / (g.volc[P] + asam::kEps);
  }
}

// ---------------------------------------------------------------------------
// Boundary face unknowns of periodic sides (PressureVelocity u_w ... w_t)
// ---------------------------------------------------------------------------
// Everything the face terms read: the cell of side `side` at face element
// (a, b) -- (iy, iz) on W/E, (ix, iz) on S/N, (ix, iy) on B/T -- its face
// index in the uF/vF/wF arrays, the face area, and the two half-cell
// factors of the reference (MatVecFull: Half*Metr1*Metr2*d; SchurPreFull:
// 0.5d0*d*Metr1*Metr2; the w faces have no metric factors).
struct FaceAt {
  int i, j, k;   // adjacent interior cell (1-based)
  size_t fq;     // index in the uF/vF/wF extents
  double F, DT, DU, hmv, hsp;
};
__device__ inline FaceAt face_at(const Dims& d, const GeomT<double>& g, const Wts& wt, int side, int a, int b) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const double* mxy = wt.metr;
  const double* mxz = wt.metr + ny;
  const double* myx = wt.metr + ny + nz;
  const double* myz = wt.metr + ny + nz + nx;
  FaceAt f;
  if (side < 2) {
    const int i = side == 0 ? 0 : nx;
    f.i = side == 0 ? 1 : nx, f.j = a, f.k = b;
    f.fq = d.UF(i, a, b);
    f.F = g.fu[d.FU(i, a, b)];
    f.DT = wt.dtu[f.fq];
    f.DU = wt.duu[f.fq];
    const double dd = wt.dx[side == 0 ? 0 : nx - 1];
    f.hmv = 0.5 * mxy[a - 1] * mxz[b - 1] * dd;
    f.hsp = 0.5 * dd * mxy[a - 1] * mxz[b - 1];
  } else if (side < 4) {
    const int j = side == 2 ? 0 : ny;
    f.i = a, f.j = side == 2 ? 1 : ny, f.k = b;
    f.fq = d.VF(a, j, b);
    f.F = g.fv[d.FV(a, j, b)];
    f.DT = wt.dtv[f.fq];
    f.DU = wt.duv[f.fq];
    const double dd = wt.dy[side == 2 ? 0 : ny - 1];
    f.hmv = 0.5 * myx[a - 1] * myz[b - 1] * dd;
    f.hsp = 0.5 * dd * myx[a - 1] * myz[b - 1];
  } else {
    const int k = side == 4 ? 0 : nz;
    f.i = a, f.j = b, f.k = side == 4 ? 1 : nz;
    f.fq = d.WF(a, b, k);
    f.F = g.fw[d.FW(a, b, k)];
    f.DT = wt.dtw[f.fq];
    f.DU = wt.duw[f.fq];
    f.hmv = 0.5 * wt.dz[side == 4 ? 0 : nz - 1];
    f.hsp = f.hmv;
  }
  return f;
}
__device__ inline size_t cell_nat(const Dims& d, int i, int j, int k) {
  return (size_t)(i - 1) + (size_t)d.nx * ((size_t)(j - 1) + (size_t)d.ny * (size_t)(k - 1));
}
__device__ inline size_t cell_lay(const Lev2& P, int i, int j, int k) {
  return (size_t)(j - 1) * P.ps + slot(P.w, P.h, k - 1, i - 1);
}

// The pressure terms of the face unknowns at the cells next to periodic
// sides, each cell once, its sides in the reference's statement order W, E,
// S, N, B, T:
//   schur = 0: p += (W/S/B) or -= (E/N/T) beta0*dtP*F*DT*DTT*u
//              (MatVecFull MATRIX/MatVec_Mod.f90:224-255, b1pBTx2Full
//              MATRIX/PreCond_Mod.f90:642-665);
//   schur = 1: the same divided by (0.5d0*d*Metr1*Metr2*F+Eps)
//              (SchurPreFull MATRIX/PreCond_Mod.f90:138-216, p starting at 0);
//   schur = 2: with the opposite signs, divided by the whole mass of the
//              shared face (both halves): the right-hand side of the
//              periodic-Laplacian preconditioner (face unknowns eliminated).
// v holds the face unknowns (at fc.off), p is a level-0 layout vector.
__global__ void k_pv_face_p(Dims d, GeomT<double> g, Wts wt, Lev2 P, PvFaces fc, double bd, int schur,
                            const double* __restrict__ v, double* __restrict__ p) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const bool px = fc.off[0] >= 0, py = fc.off[2] >= 0, pz = fc.off[4] >= 0;
  // cells of the x sides, then of the y sides not on an x side, then of the z sides on neither
  const int ni = nx > 1 ? 2 : 1, nj = ny > 1 ? 2 : 1, nk = nz > 1 ? 2 : 1;
  const int ri = px ? (nx > 2 ? nx - 2 : 0) : nx;  // i not on an x side
  const int rj = py ? (ny > 2 ? ny - 2 : 0) : ny;
  const size_t cx = px ? (size_t)ni * ny * nz : 0, cy = py ? (size_t)nj * ri * nz : 0;
  const size_t cz = pz ? (size_t)nk * ri * rj : 0;
  const size_t tot = cx + cy + cz;
  const double eps = asam::kEps;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot; e += (size_t)gridDim.x * blockDim.x) {
    int i, j, k;
    if (e < cx) {
      const int s = (int)(e % ni);
      const size_t r = e / ni;
      i = s == 0 ? 1 : nx, j = (int)(r % ny) + 1, k = (int)(r / ny) + 1;
    } else if (e < cx + cy) {
      const size_t q = e - cx;
      const int s = (int)(q % nj);
      const size_t r = q / nj;
      i = (int)(r % ri) + 1 + (px ? 1 : 0), j = s == 0 ? 1 : ny, k = (int)(r / ri) + 1;
    } else {
      const size_t q = e - cx - cy;
      const int s = (int)(q % nk);
      const size_t r = q / nk;
      i = (int)(r % ri) + 1 + (px ? 1 : 0), j = (int)(r / ri) + 1 + (py ? 1 : 0), k = s == 0 ? 1 : nz;
    }
    const size_t cl = cell_lay(P, i, j, k);
    const double dtt = wt.dtt[cell_nat(d, i, j, k)];
    double acc = p[cl];
    for (int side = 0; side < 6; ++side) {
      if (fc.off[side] < 0) continue;
      int a, b;
      if (side < 2) {
        if (i != (side == 0 ? 1 : nx)) continue;
        a = j, b = k;
      } else if (side < 4) {
        if (j != (side == 2 ? 1 : ny)) continue;
        a = i, b = k;
      } else {
        if (k != (side == 4 ? 1 : nz)) continue;
        a = i, b = j;
      }
      const FaceAt f = face_at(d, g, wt, side, a, b);
      const int na = side < 2 ? ny : nx;
      const double u = v[fc.off[side] + (a - 1) + (size_t)na * (b - 1)];
      double t = bd * f.F * f.DT * dtt * u;
      if (schur == 1) t = t / (f.hsp * f.F + eps);
      if (schur == 2) {  // the face unknown eliminated with the pair's whole mass
        const FaceAt o = face_at(d, g, wt, side ^ 1, a, b);
        t = t / (f.hmv * f.F + o.hmv * o.F + eps);
        acc = (side & 1) ? acc + t : acc - t;
      } else {
        acc = (side & 1) ? acc - t : acc + t;
      }
    }
    p[cl] = acc;
  }
}

// Face equations of one periodic side pair per thread (the W and E copies of
// one face, likewise S/N and B/T), then optionally the Exchange of the pair
// (u_w = u_w + u_e; u_e = u_w).  cp = beta0*dtP*F*DUT*DU*p(cell) with p the
// level-0 layout vector pv.
//   op 0 MatVecFull face equation (MATRIX/MatVec_Mod.f90:224-255):
//        out = Half*Metr1*Metr2*d*F*in (+W/S/B, -E/N/T) cp
//   op 1 b2pBx1Full (MATRIX/PreCond_Mod.f90:694-728): out = in (+/-) cp
//   op 2 SchurPreFull after its Solve_3D (MATRIX/PreCond_Mod.f90:303-404):
//        out = PreFac2*(in (-W/S/B, +E/N/T) cp)/(0.5d0*d*Metr1*Metr2*F+Eps)
//   op 3 the periodic-Laplacian preconditioner's face unknowns:
//        out = (in - cp_W + cp_E) / (whole mass of the shared face + Eps),
//        written to both copies (in holds equal copies after Exchange)
__global__ void k_pv_faces(Dims d, GeomT<double> g, Wts wt, Lev2 P, PvFaces fc, double bd, double prefac2, int op,
                           int exchange, const double* in, const double* __restrict__ pv, double* out) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const size_t nX = fc.off[0] >= 0 ? (size_t)ny * nz : 0, nY = fc.off[2] >= 0 ? (size_t)nx * nz : 0;
  const size_t nZ = fc.off[4] >= 0 ? (size_t)nx * ny : 0;
  const double eps = asam::kEps;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < nX + nY + nZ;
       e += (size_t)gridDim.x * blockDim.x) {
    int pair, a, b;
    size_t q;
    if (e < nX) {
      pair = 0, q = e, a = (int)(q % ny) + 1, b = (int)(q / ny) + 1;
    } else if (e < nX + nY) {
      pair = 1, q = e - nX, a = (int)(q % nx) + 1, b = (int)(q / nx) + 1;
    } else {
      pair = 2, q = e - nX - nY, a = (int)(q % nx) + 1, b = (int)(q / nx) + 1;
    }
    double val[2], mass = 0.0;
    for (int h = 0; h < 2; ++h) {
      const int side = 2 * pair + h;
      const FaceAt f = face_at(d, g, wt, side, a, b);
      const size_t fi = fc.off[side] + q;
      const double dut = wt.dut[cell_nat(d, f.i, f.j, f.k)];
      const double cp = bd * f.F * dut * f.DU * pv[cell_lay(P, f.i, f.j, f.k)];
      double r;
      if (op == 0) {
        const double m = f.hmv * f.F * in[fi];
        r = h ? m - cp : m + cp;
      } else if (op == 1) {
        r = h ? in[fi] - cp : in[fi] + cp;
      } else if (op == 2) {
        const double den = f.hsp * f.F + eps;
        r = h ? prefac2 * (in[fi] + cp) / den : prefac2 * (in[fi] - cp) / den;
      } else {  // op 3: the cp terms of both halves, combined below
        r = h ? cp : -cp;
        mass = mass + f.hmv * f.F;
      }
      val[h] = r;
    }
    if (op == 3) {  // u = (v - cp_W + cp_E) / (whole mass), both copies
      const size_t lo = fc.off[2 * pair] + q, hi = fc.off[2 * pair + 1] + q;
      const double u = (in[lo] + val[0] + val[1]) / (mass + eps);
      out[lo] = u;
      out[hi] = u;
      continue;
    }
    const size_t lo = fc.off[2 * pair] + q, hi = fc.off[2 * pair + 1] + q;
    if (exchange) {
      const double s = val[0] + val[1];
      out[lo] = s;
      out[hi] = s;
    } else {
      out[lo] = val[0];
      out[hi] = val[1];
    }
  }
}

// Exchange alone (after a DXPBY): u_w = u_w + u_e; u_e = u_w per pair
__global__ void k_pv_exchange(PvFaces fc, size_t nX, size_t nY, size_t nZ, double* __restrict__ v) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < nX + nY + nZ;
       e += (size_t)gridDim.x * blockDim.x) {
    const int pair = e < nX ? 0 : (e < nX + nY ? 1 : 2);
    const size_t q = pair == 0 ? e : (pair == 1 ? e - nX : e - nX - nY);
    const size_t lo = fc.off[2 * pair] + q, hi = fc.off[2 * pair + 1] + q;
    const double s = v[lo] + v[hi];
    v[lo] = s;
    v[hi] = s;
  }
}

// WeightDiagCompute, ThetaKind='Density' (MULTI/JacAccGrav_Mod.f90:4259-4282)
// with CellToFaceRhoWeight (:3254-3702): DUT and DTT per cell, the face
// potential temperature DTU/DTV/DTW (volume-weighted between the two cells,
// with the halo image on a periodic side, one-sided on the walls),
// DUU/DUV/DUW = F/(F+Eps).
// Constants of MODULE/Parameter_Mod.f90:21-29.
constexpr double kCpd = 1004.0, kCvd = 717.0, kRd = kCpd - kCvd, kCpv = 1885.0, kRv = 461.0, kCpl = 4186.0;

__global__ void k_weights_density(Dims d, GeomT<double> g, Wts wt, const double* __restrict__ rth,
                                  const double* __restrict__ rho, const double* __restrict__ rv,
                                  const double* __restrict__ rc, const double* __restrict__ rr,
                                  const double* __restrict__ tabs) {
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const size_t nc = (size_t)nx * ny * nz, nu = (size_t)(nx + 1) * ny * nz, nv = (size_t)nx * (ny + 1) * nz,
               nw = (size_t)nx * ny * (nz + 1);
  const size_t tot = nc + nu + nv + nw;
  auto th = [&](size_t P) { return rth[P] / (rho[P] + asam::kEps); };
  auto face = [&](size_t P, size_t Q) {
    const double* V = g.volc;
    return (V[P] * rth[P] / (rho[P] + asam::kEps) + V[Q] * rth[Q] / (rho[Q] + asam::kEps)) / (V[P] + V[Q] + asam::kEps);
  };
  // a periodic x or y side ('iw'/'ie'/'is'/'in' with equal refinement,
  // MULTI/JacAccGrav_Mod.f90:3313-3321, 3360-3368, 3407-3415, 3454-3462): theta
  // first, then times the volume; the halo cell holds the periodic image
  auto pface = [&](size_t P, size_t Q) {
    const double* V = g.volc;
    return (th(P) * V[P] + th(Q) * V[Q]) / (V[P] + V[Q] + asam::kEps);
  };
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < tot; e += (size_t)gridDim.x * blockDim.x) {
    if (e < nc) {
      const int i = (int)(e % nx) + 1;
      const size_t r = e / nx;
      const int j = (int)(r % ny) + 1, k = (int)(r / ny) + 1;
      const size_t P = d.P(i, j, k);
      const double rvl = rv ? rv[P] : 0.0;
      const double rll = (rc ? rc[P] : 0.0) + (rr ? rr[P] : 0.0);
      const double rd = rho[P] - rvl - rll + asam::kEps;
      const double rm = kRd + kRv * rvl / rd;
      const double cpml = kCpd + kCpv * rvl / rd + kCpl * rll / rd;
      const double kap = rm / cpml;
      wt.dut[e] = tabs[P] / (rth[P] + asam::kEps) * (rd * kRd + rvl * kRv) / (1.0 - kap);
      wt.dtt[e] = 1.0;
    } else if (e < nc + nu) {
      const size_t q = e - nc;
      const int i = (int)(q % (nx + 1));
      const size_t r = q / (nx + 1);
      const int j = (int)(r % ny) + 1, k = (int)(r / ny) + 1;
      if (d.per_x && (i == 0 || i == nx))
        wt.dtu[q] = i == 0 ? pface(d.P(1, j, k), d.P(0, j, k)) : pface(d.P(nx + 1, j, k), d.P(nx, j, k));
      else
        wt.dtu[q] = i == 0 ? th(d.P(1, j, k)) : (i == nx ? th(d.P(nx, j, k)) : face(d.P(i, j, k), d.P(i + 1, j, k)));
      const double f = g.fu[d.FU(i, j, k)];
      wt.duu[q] = f / (f + asam::kEps);
    } else if (e < nc + nu + nv) {
      const size_t q = e - nc - nu;
      const int i = (int)(q % nx) + 1;
      const size_t r = q / nx;
      const int j = (int)(r % (ny + 1)), k = (int)(r / (ny + 1)) + 1;
      if (d.per_y && (j == 0 || j == ny))
        wt.dtv[q] = j == 0 ? pface(d.P(i, 1, k), d.P(i, 0, k)) : pface(d.P(i, ny + 1, k), d.P(i, ny, k));
      else
        wt.dtv[q] = j == 0 ? th(d.P(i, 1, k)) : (j == ny ? th(d.P(i, ny, k)) : face(d.P(i, j, k), d.P(i, j + 1, k)));
      const double f = g.fv[d.FV(i, j, k)];
      wt.duv[q] = f / (f + asam::kEps);
    } else {
      const size_t q = e - nc - nu - nv;
      const int i = (int)(q % nx) + 1;
      const size_t r = q / nx;
      const int j = (int)(r % ny) + 1, k = (int)(r / ny);
      if (d.per_z && (k == 0 || k == nz))  // 'ib'/'it': the interior rounding
        wt.dtw[q] = k == 0 ? face(d.P(i, j, 1), d.P(i, j, 0)) : face(d.P(i, j, nz + 1), d.P(i, j, nz));
      else
        wt.dtw[q] = k == 0 ? th(d.P(i, j, 1)) : (k == nz ? th(d.P(i, j, nz)) : face(d.P(i, j, k), d.P(i, j, k + 1)));
      const double f = g.fw[d.FW(i, j, k)];
      wt.duw[q] = f / (f + asam::kEps);
    }
  }
}

}  // namespace prj

using namespace prj;

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
struct ProjState {
  asam_proj_config cfg{};
  cudaStream_t st = nullptr;  // the context's stream at the current call
  int R = 0;
  Wts wt{};
  bool weights = false, assembled = false;
  double beta0 = 0.0, dtp = 0.0;
  std::vector<Lev3> lv;
  Lev3* d_lv = nullptr;
  Fields g{}, c{};
  std::vector<void*> allocs;
  // FGMRES storage (level-0 layout)
  std::vector<double*> v, z;
  double *H = nullptr, *partial = nullptr, *scal_h = nullptr;
  double *tmp = nullptr, *xn = nullptr, *bn = nullptr, *xl = nullptr, *bl = nullptr;
  double *stage_u = nullptr, *stage_v = nullptr, *stage_w = nullptr, *tabs = nullptr;
  double *div_m = nullptr, *div_fu = nullptr, *div_fv = nullptr, *div_fw = nullptr;  // DivScalar scratch
  long long vcycles = 0;
  // single-precision copy of the multigrid hierarchy: FGMRES is flexible (it
  // keeps the preconditioned vectors), so a V-cycle in FP32 preconditions the
  // FP64 iteration without touching its residual test
  std::vector<prj::Lev3T<float>> lv32;
  prj::Lev3T<float>* d_lv32 = nullptr;
  int mg_prec = -1;  // -1: follow the context's precision, 0: FP64, 1: FP32
  bool lv32_ready = false;
  // periodic sides: boundary face unknowns and the Dirichlet hierarchy
  // (LaplDirichlet: its own matrices, the vectors shared with lv)
  PvFaces fc{{-1, -1, -1, -1, -1, -1}};
  size_t nface = 0;  // face unknowns in a PressureVelocity vector
  std::vector<Lev3> lvD;
  Lev3* d_lvD = nullptr;
  std::vector<prj::Lev3T<float>> lvD32;
  prj::Lev3T<float>* d_lvD32 = nullptr;
  double* tmp2 = nullptr;  // level-0 scratch of PSolve1
  // the periodic-Laplacian preconditioner (face unknowns eliminated, one
  // V-cycle on the Laplacian with the couplings across the periodic sides):
  // -1 follow the precision (refined contexts), 0 PSolve1, 1 periodic
  int pre_kind = -1;
  // smoothing schedule of the periodic preconditioner's V-cycle (GaussIter2,
  // GaussIter3 of its hierarchy): one sweep per level by default -- the
  // reference's growth of the sweeps with the level buys no FGMRES step
  // there (9/9/8 steps per stage either way at 512x512x128) and costs a fifth
  // of the refined step
  int pre_gi2 = 0, pre_gi3 = 0;
  std::vector<Lev3> lvP;
  Lev3* d_lvP = nullptr;
  std::vector<prj::Lev3T<float>> lvP32;
  prj::Lev3T<float>* d_lvP32 = nullptr;
  bool lvP_ready = false, lvP32_ready = false, lvD_ready = false;
};

namespace prj {

int grid_of(size_t n) {
  size_t g = (n + 255) / 256;
  if (g > 152 * 16) g = 152 * 16;
  return (int)(g ? g : 1);
}

// allocate and zero on the context's stream, so the zeroing is ordered before
// every later upload and kernel on that stream
template <typename T>
int palloc(ProjState* s, T** p, size_t n) {
  void* q = nullptr;
  CK(cudaMalloc(&q, (n ? n : 1) * sizeof(T)));
  CK(cudaMemsetAsync(q, 0, (n ? n : 1) * sizeof(T), s->st));
  s->allocs.push_back(q);
  *p = (T*)q;
  return kOk;
}

int alloc_fields(ProjState* s, Fields& f, int n1, int n2, int n3) {
  f.n1 = n1;
  f.n2 = n2;
  f.n3 = n3;
  const size_t s1 = (size_t)(n1 + 1) * n2 * n3, s2 = (size_t)n1 * (n2 + 1) * n3, s3 = (size_t)n1 * n2 * (n3 + 1);
  const size_t sc = (size_t)n1 * n2 * n3;
  struct {
    double** p;
    size_t n;
  } a[] = {{&f.F1, s1}, {&f.T1, s1}, {&f.U1, s1}, {&f.F2, s2}, {&f.T2, s2}, {&f.U2, s2}, {&f.F3, s3},
           {&f.T3, s3}, {&f.U3, s3}, {&f.vol, sc}, {&f.dut, sc}, {&f.d1, (size_t)n1}, {&f.d2, (size_t)n2},
           {&f.d3, (size_t)n3}, {&f.m12, (size_t)n2}, {&f.m13, (size_t)n3}, {&f.m21, (size_t)n1}, {&f.m23, (size_t)n3},
           {&f.m31, (size_t)n1}, {&f.m32, (size_t)n2}};
  for (auto& q : a)
    if (int rc = palloc(s, q.p, q.n)) return rc;
  return kOk;
}

int alloc_lev2(ProjState* s, Lev2& P, int c1, int c2, int m3, bool own_vectors) {
  P.c1 = c1;
  P.c2 = c2;
  P.h = (c2 + 1) / 2;
  P.w = 2 * P.h;
  P.m3 = m3;
  P.ps = (size_t)c1 * P.w;
  const size_t n = P.ps * m3;
  double** arr[] = {&P.d, &P.uz, &P.lz, &P.fw, &P.ft, &P.frt, &P.ux, &P.lx, &P.res};
  for (double** q : arr)
    if (int rc = palloc(s, q, n)) return rc;
  P.x = P.b = nullptr;
  if (own_vectors) {
    if (int rc = palloc(s, &P.x, n)) return rc;
    if (int rc = palloc(s, &P.b, n)) return rc;
  }
  return kOk;
}

size_t len0(const ProjState* s) { return (size_t)s->lv[0].m3 * s->lv[0].pl[0].ps; }
// length of a PressureVelocity vector, and of its prefix that DOT2 counts
size_t lenv(const ProjState* s) { return len0(s) + s->nface; }
size_t lendot(const ProjState* s) { return len0(s) + s->nface / 2; }

}  // namespace prj

void proj_free(asam_ctx* h) {
  ProjState* s = h->proj;
  if (!s) return;
  for (void* p : s->allocs) cudaFree(p);
  if (s->scal_h) cudaFreeHost(s->scal_h);
  delete s;
  h->proj = nullptr;
}

bool proj_grid(asam_ctx* h, ProjGrid* out) {
  ProjState* s = h->proj;
  if (!s) return false;
  const Dims& d = h->d;
  out->dx = s->wt.dx;
  out->dy = s->wt.dy;
  out->dz = s->wt.dz;
  out->mxy = s->wt.metr;                    // MetrXY[ny]
  out->myx = s->wt.metr + d.ny + d.nz;      // MetrYX[nx]
  return true;
}

namespace prj {

int proj_build(asam_ctx* h) {
  ProjState* s = h->proj;
  const Dims& d = h->d;
  const int n1 = d.nz, n2 = d.nx, n3 = d.ny;
  const int R = s->R;
  s->lv.assign(R, Lev3{});
  for (int L = 0; L < R; ++L) {
    const int sh = (1 << L) - 1;
    Lev3& A = s->lv[L];
    A.m1 = (n1 + sh) / (sh + 1);
    A.m2 = (n2 + sh) / (sh + 1);
    A.m3 = (n3 + sh) / (sh + 1);
    A.nl = R - L;
    for (int L2 = L; L2 < R; ++L2) {
      const int s2 = (1 << L2) - 1;
      if (int rc = alloc_lev2(s, A.pl[L2 - L], (n1 + s2) / (s2 + 1), (n2 + s2) / (s2 + 1), A.m3, L2 > L)) return rc;
    }
    const size_t n = A.pl[0].ps * A.m3;
    double** arr[] = {&A.u3, &A.l3, &A.x, &A.b, &A.res, &A.t};
    for (double** q : arr)
      if (int rc = palloc(s, q, n)) return rc;
  }
  {
    // face unknowns of the periodic sides: u_e, v_n, w_t, then u_w, v_s, w_b
    const int per[3] = {d.per_x, d.per_y, d.per_z};
    const size_t fsz[3] = {(size_t)d.ny * d.nz, (size_t)d.nx * d.nz, (size_t)d.nx * d.ny};
    size_t o = (size_t)s->lv[0].m3 * s->lv[0].pl[0].ps, half = 0;
    for (int a = 0; a < 3; ++a) half += per[a] ? fsz[a] : 0;
    for (int a = 0; a < 3; ++a) {
      s->fc.off[2 * a] = s->fc.off[2 * a + 1] = -1;
      if (!per[a]) continue;
      s->fc.off[2 * a + 1] = (long long)o;           // E / N / T
      s->fc.off[2 * a] = (long long)(o + half);      // W / S / B
      o += fsz[a];
    }
    s->nface = 2 * half;
  }
  if (s->nface > 0) {
    s->lvD = s->lv;
    for (int L = 0; L < R; ++L) {
      Lev3& A = s->lvD[L];
      for (int q = 0; q < A.nl; ++q) {
        Lev2& P = A.pl[q];
        const size_t n = P.ps * P.m3;
        double** arr[] = {&P.d, &P.uz, &P.lz, &P.fw, &P.ft, &P.frt, &P.ux, &P.lx};
        for (double** r : arr)
          if (int rc = palloc(s, r, n)) return rc;
      }
      const size_t n = A.pl[0].ps * A.m3;
      if (int rc = palloc(s, &A.u3, n)) return rc;
      if (int rc = palloc(s, &A.l3, n)) return rc;
    }
    if (int rc = palloc(s, &s->d_lvD, (size_t)R)) return rc;
    CK(cudaMemcpyAsync(s->d_lvD, s->lvD.data(), sizeof(Lev3) * R, cudaMemcpyHostToDevice, s->st));
  }
  CK(cudaFuncSetAttribute(k_plane_half<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRingBytes));
  CK(cudaFuncSetAttribute(k_plane_half<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRingBytes));
  CK(cudaFuncSetAttribute(k_plane_half<double, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRingBytes));
  CK(cudaFuncSetAttribute(k_plane_half<float, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRingBytes));
  if (int rc = palloc(s, &s->d_lv, (size_t)R)) return rc;
  CK(cudaMemcpyAsync(s->d_lv, s->lv.data(), sizeof(Lev3) * R, cudaMemcpyHostToDevice, s->st));
  CK(cudaStreamSynchronize(s->st));
  if (int rc = alloc_fields(s, s->g, n1, n2, n3)) return rc;
  if (int rc = alloc_fields(s, s->c, n1, n2, n3)) return rc;
  // FGMRES storage: PressureVelocity vectors (pressure + face unknowns)
  const int step = s->cfg.step_gmres;
  const size_t n = lenv(s);
  s->v.assign(step + 1, nullptr);
  s->z.assign(step, nullptr);
  for (auto& p : s->v)
    if (int rc = palloc(s, &p, n)) return rc;
  for (auto& p : s->z)
    if (int rc = palloc(s, &p, n)) return rc;
  if (int rc = palloc(s, &s->H, (size_t)(step + 1) * (step + 1))) return rc;
  if (int rc = palloc(s, &s->partial, (size_t)kRedGrid)) return rc;
  if (int rc = palloc(s, &s->tmp, n)) return rc;
  if (int rc = palloc(s, &s->tmp2, len0(s))) return rc;
  if (int rc = palloc(s, &s->xl, n)) return rc;
  if (int rc = palloc(s, &s->bl, n)) return rc;
  const size_t nc = (size_t)d.nx * d.ny * d.nz;
  if (int rc = palloc(s, &s->xn, nc + s->nface)) return rc;
  if (int rc = palloc(s, &s->bn, nc + s->nface)) return rc;
  CK(cudaMallocHost((void**)&s->scal_h, sizeof(double) * (step + 2)));
  return kOk;
}

// Solve_3D from a zero start on level 0 (VCycleCG's MatrixT branch): lv[0].b
// holds the right-hand side, the result is left in lv[0].x
template <typename T, bool kWrap = false>
void vcycle_run(asam_ctx* h, std::vector<Lev3T<T>>& lv, Lev3T<T>* d_lv, int gi2, int gi3) {
  ProjState* s = h->proj;
  const cudaStream_t st = h->L.stream;
  const int R = s->R;
  const int mi2 = s->cfg.mult_iter2;
  const size_t ring = (size_t)RingCfg<T>::ring * kFields * kPlaneBlock * sizeof(T);
  long long nl = 0;
  cudaMemsetAsync(lv[0].x, 0, sizeof(T) * len0(s), st);
  auto gs3 = [&](int L, int gi) {
    const Lev3T<T>& A = lv[L];
    auto half = [&](int c, int fwd) {
      const int np = (A.m3 - c + 1) / 2;
      if (np <= 0) return;
      k_plane_half<T, kWrap><<<np, kPlaneBlock, ring, st>>>(d_lv, L, c, fwd, mi2, gi2);
      ++nl;
    };
    if (A.m3 > 1) {
      for (int it = 0; it < gi; ++it) {
        half(0, 1);
        half(1, 1);
        half(1, 0);
        half(0, 0);
      }
    } else {
      half(0, 1);
    }
  };
  for (int it = 0; it < s->cfg.mult_iter3; ++it) {
    int gi = 1, L = 0;
    for (;;) {
      gs3(L, gi);
      gi += gi3;
      if (L + 1 < R) {
        const Lev3T<T>& A = lv[L];
        const size_t n = A.pl[0].ps * A.m3;
        k_matvec3<T, kWrap><<<grid_of(n), 256, 0, st>>>(d_lv, L, A.x, A.b, A.res, 0);
        const size_t nc = lv[L + 1].pl[0].ps * lv[L + 1].m3;
        k_restrict3<T><<<grid_of(nc), 256, 0, st>>>(d_lv, L);
        nl += 2;
        ++L;
      } else {
        gi -= gi3;
        break;
      }
    }
    for (;;) {
      gs3(L, gi);
      gi -= gi3;
      if (L > 0) {
        --L;
        const size_t n = lv[L].pl[0].ps * lv[L].m3;
        k_prolong3<T><<<grid_of(n), 256, 0, st>>>(d_lv, L);
        ++nl;
      } else {
        break;
      }
    }
  }
  count_launches(nl);
  ++s->vcycles;
}

bool use_mg32(const asam_ctx* h) {
  const ProjState* s = h->proj;
  return s->mg_prec == 1 || (s->mg_prec < 0 && h->cfg.precision == ASAM_PREC_FP32_REFINED);
}

// FGMRES preconditioned by the periodic-Laplacian multigrid instead of the
// reference's PSolve1: blocks with face unknowns of periodic x/y sides only
bool use_per(const asam_ctx* h) {
  const ProjState* s = h->proj;
  if (!s->nface || h->d.per_z) return false;
  return s->pre_kind == 1 || (s->pre_kind < 0 && h->cfg.precision == ASAM_PREC_FP32_REFINED);
}

// the periodic-Laplacian hierarchy: its own matrices and couplings across the
// periodic sides, the vectors of lv (FP64) / lv32 (FP32)
int alloc_levP(ProjState* s, const Dims& d) {
  if (s->d_lvP) return kOk;
  const int R = s->R;
  s->lvP = s->lv;
  for (int L = 0; L < R; ++L) {
    Lev3& A = s->lvP[L];
    for (int q = 0; q < A.nl; ++q) {
      Lev2& P = A.pl[q];
      const size_t n = P.ps * P.m3;
      double** arr[] = {&P.d, &P.uz, &P.lz, &P.fw, &P.ft, &P.frt, &P.ux, &P.lx};
      for (double** r : arr)
        if (int rc = palloc(s, r, n)) return rc;
      if (d.per_x) {
        if (int rc = palloc(s, &P.wxl, (size_t)P.c1 * P.m3)) return rc;
        if (int rc = palloc(s, &P.wxh, (size_t)P.c1 * P.m3)) return rc;
      }
    }
    const size_t n = A.pl[0].ps * A.m3;
    if (int rc = palloc(s, &A.u3, n)) return rc;
    if (int rc = palloc(s, &A.l3, n)) return rc;
    if (d.per_y) {
      if (int rc = palloc(s, &A.wyl, A.pl[0].ps)) return rc;
      if (int rc = palloc(s, &A.wyh, A.pl[0].ps)) return rc;
    }
  }
  if (int rc = palloc(s, &s->d_lvP, (size_t)R)) return rc;
  CK(cudaMemcpyAsync(s->d_lvP, s->lvP.data(), sizeof(Lev3) * R, cudaMemcpyHostToDevice, s->st));
  CK(cudaStreamSynchronize(s->st));
  return kOk;
}

__global__ void k_cvt_to_f32(const double* __restrict__ a, float* __restrict__ b, size_t n, double sign) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x)
    b[e] = (float)(sign * a[e]);
}
// Thomas pivots and their reciprocals in FP32.  A cell without volume has
// the pivot 1e-40 (Allocate_1D's initial diagonal), below FP32's normal range
// and with a reciprocal beyond it; its couplings and right-hand side are 0,
// so the FP32 copy solves that row with the pivot 1 instead, which leaves it 0.
__global__ void k_cvt_pivot(const double* __restrict__ ft, const double* __restrict__ frt, float* __restrict__ ft32,
                            float* __restrict__ frt32, size_t n) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
    const double p = ft[e];
    const bool ok = fabs(p) >= 1.0e-30 && fabs(frt[e]) <= 1.0e30;
    ft32[e] = ok ? (float)p : 1.0f;
    frt32[e] = ok ? (float)frt[e] : 1.0f;
  }
}
__global__ void k_cvt_to_f64(const float* __restrict__ a, double* __restrict__ b, size_t n) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x)
    b[e] = (double)a[e];
}

// the FP32 hierarchy with the shapes of the FP64 one (allocated once)
int alloc_lev32(ProjState* s) {
  if (s->d_lv32) return kOk;
  const int R = s->R;
  s->lv32.assign(R, Lev3T<float>{});
  for (int L = 0; L < R; ++L) {
    const Lev3& A = s->lv[L];
    Lev3T<float>& B = s->lv32[L];
    B.m1 = A.m1;
    B.m2 = A.m2;
    B.m3 = A.m3;
    B.nl = A.nl;
    for (int q = 0; q < A.nl; ++q) {
      const Lev2& P = A.pl[q];
      Lev2T<float>& Q = B.pl[q];
      Q.c1 = P.c1;
      Q.c2 = P.c2;
      Q.h = P.h;
      Q.w = P.w;
      Q.m3 = P.m3;
      Q.ps = P.ps;
      const size_t n = P.ps * P.m3;
      float** arr[] = {&Q.d, &Q.uz, &Q.lz, &Q.fw, &Q.ft, &Q.frt, &Q.ux, &Q.lx, &Q.res};
      for (float** r : arr)
        if (int rc = palloc(s, r, n)) return rc;
      Q.x = Q.b = nullptr;
      if (P.x) {
        if (int rc = palloc(s, &Q.x, n)) return rc;
        if (int rc = palloc(s, &Q.b, n)) return rc;
      }
    }
    const size_t n = A.pl[0].ps * A.m3;
    float** arr[] = {&B.u3, &B.l3, &B.x, &B.b, &B.res, &B.t};
    for (float** r : arr)
      if (int rc = palloc(s, r, n)) return rc;
  }
  if (int rc = palloc(s, &s->d_lv32, (size_t)R)) return rc;
  CK(cudaMemcpyAsync(s->d_lv32, s->lv32.data(), sizeof(Lev3T<float>) * R, cudaMemcpyHostToDevice, s->st));
  if (s->nface > 0) {  // the Dirichlet copy: own matrices, the vectors of lv32
    s->lvD32 = s->lv32;
    for (int L = 0; L < R; ++L) {
      Lev3T<float>& B = s->lvD32[L];
      for (int q = 0; q < B.nl; ++q) {
        Lev2T<float>& Q = B.pl[q];
        const size_t n = Q.ps * Q.m3;
        float** arr[] = {&Q.d, &Q.uz, &Q.lz, &Q.fw, &Q.ft, &Q.frt, &Q.ux, &Q.lx};
        for (float** r : arr)
          if (int rc = palloc(s, r, n)) return rc;
      }
      const size_t n = B.pl[0].ps * B.m3;
      if (int rc = palloc(s, &B.u3, n)) return rc;
      if (int rc = palloc(s, &B.l3, n)) return rc;
    }
    if (int rc = palloc(s, &s->d_lvD32, (size_t)R)) return rc;
    CK(cudaMemcpyAsync(s->d_lvD32, s->lvD32.data(), sizeof(Lev3T<float>) * R, cudaMemcpyHostToDevice, s->st));
  }
  return kOk;
}

// round the assembled FP64 hierarchy (matrix and Thomas factors) to FP32
long long convert_one(cudaStream_t st, int R, const std::vector<Lev3>& lv, const std::vector<Lev3T<float>>& lv32) {
  long long nl = 0;
  for (int L = 0; L < R; ++L) {
    const Lev3& A = lv[L];
    const Lev3T<float>& B = lv32[L];
    for (int q = 0; q < A.nl; ++q) {
      const Lev2& P = A.pl[q];
      const Lev2T<float>& Q = B.pl[q];
      const size_t n = P.ps * P.m3;
      const double* src[] = {P.d, P.uz, P.lz, P.fw, P.ux, P.lx};
      float* dst[] = {Q.d, Q.uz, Q.lz, Q.fw, Q.ux, Q.lx};
      for (int a = 0; a < 6; ++a, ++nl) k_cvt_to_f32<<<grid_of(n), 256, 0, st>>>(src[a], dst[a], n, 1.0);
      k_cvt_pivot<<<grid_of(n), 256, 0, st>>>(P.ft, P.frt, Q.ft, Q.frt, n);
      ++nl;
    }
    const size_t n = A.pl[0].ps * A.m3;
    k_cvt_to_f32<<<grid_of(n), 256, 0, st>>>(A.u3, B.u3, n, 1.0);
    k_cvt_to_f32<<<grid_of(n), 256, 0, st>>>(A.l3, B.l3, n, 1.0);
    nl += 2;
  }
  return nl;
}

int convert_lev32(asam_ctx* h) {
  ProjState* s = h->proj;
  if (int rc = alloc_lev32(s)) return rc;
  const cudaStream_t st = h->L.stream;
  long long nl = convert_one(st, s->R, s->lv, s->lv32);
  if (s->nface > 0) nl += convert_one(st, s->R, s->lvD, s->lvD32);
  count_launches(nl);
  s->lv32_ready = true;
  return kOk;
}

// the FP32 copy of the periodic-Laplacian hierarchy (matrices, factors and
// couplings across the periodic sides; the vectors of lv32)
int convert_levP32(asam_ctx* h) {
  ProjState* s = h->proj;
  if (int rc = alloc_lev32(s)) return rc;
  const cudaStream_t st = h->L.stream;
  const int R = s->R;
  if (!s->d_lvP32) {
    s->lvP32 = s->lv32;
    for (int L = 0; L < R; ++L) {
      Lev3T<float>& B = s->lvP32[L];
      const Lev3& A = s->lvP[L];
      for (int q = 0; q < B.nl; ++q) {
        Lev2T<float>& Q = B.pl[q];
        const size_t n = Q.ps * Q.m3;
        float** arr[] = {&Q.d, &Q.uz, &Q.lz, &Q.fw, &Q.ft, &Q.frt, &Q.ux, &Q.lx};
        for (float** r : arr)
          if (int rc = palloc(s, r, n)) return rc;
        if (A.pl[q].wxl) {
          if (int rc = palloc(s, &Q.wxl, (size_t)Q.c1 * Q.m3)) return rc;
          if (int rc = palloc(s, &Q.wxh, (size_t)Q.c1 * Q.m3)) return rc;
        }
      }
      const size_t n = B.pl[0].ps * B.m3;
      if (int rc = palloc(s, &B.u3, n)) return rc;
      if (int rc = palloc(s, &B.l3, n)) return rc;
      if (A.wyl) {
        if (int rc = palloc(s, &B.wyl, B.pl[0].ps)) return rc;
        if (int rc = palloc(s, &B.wyh, B.pl[0].ps)) return rc;
      }
    }
    if (int rc = palloc(s, &s->d_lvP32, (size_t)R)) return rc;
    CK(cudaMemcpyAsync(s->d_lvP32, s->lvP32.data(), sizeof(Lev3T<float>) * R, cudaMemcpyHostToDevice, st));
  }
  long long nl = convert_one(st, R, s->lvP, s->lvP32);
  for (int L = 0; L < R; ++L) {
    const Lev3& A = s->lvP[L];
    const Lev3T<float>& B = s->lvP32[L];
    for (int q = 0; q < A.nl; ++q)
      if (A.pl[q].wxl) {
        const size_t n = (size_t)A.pl[q].c1 * A.pl[q].m3;
        k_cvt_to_f32<<<grid_of(n), 256, 0, st>>>(A.pl[q].wxl, B.pl[q].wxl, n, 1.0);
        k_cvt_to_f32<<<grid_of(n), 256, 0, st>>>(A.pl[q].wxh, B.pl[q].wxh, n, 1.0);
        nl += 2;
      }
    if (A.wyl) {
      k_cvt_to_f32<<<grid_of(A.pl[0].ps), 256, 0, st>>>(A.wyl, B.wyl, A.pl[0].ps, 1.0);
      k_cvt_to_f32<<<grid_of(A.pl[0].ps), 256, 0, st>>>(A.wyh, B.wyh, A.pl[0].ps, 1.0);
      nl += 2;
    }
  }
  count_launches(nl);
  s->lvP32_ready = true;
  return kOk;
}

// Solve_3D in the selected precision on LaplNeumann (or LaplDirichlet): b
// (level-0 layout, FP64) scaled by sign -> x (FP64)
// which hierarchy a V-cycle runs on
enum { kHierNeumann = 0, kHierDirichlet = 1, kHierPeriodic = 2 };
void vcycle_any(asam_ctx* h, const double* b, double sign, double* x, int which = kHierNeumann) {
  ProjState* s = h->proj;
  const size_t n = len0(s);
  const cudaStream_t st = h->L.stream;
  if (use_mg32(h) && s->lv32_ready && (which != kHierPeriodic || s->lvP32_ready)) {
    k_cvt_to_f32<<<grid_of(n), 256, 0, st>>>(b, s->lv32[0].b, n, sign);
    if (which == kHierDirichlet)
      vcycle_run<float>(h, s->lvD32, s->d_lvD32, s->cfg.gauss_iter2, s->cfg.gauss_iter3);
    else if (which == kHierPeriodic)
      vcycle_run<float, true>(h, s->lvP32, s->d_lvP32, s->pre_gi2, s->pre_gi3);
    else
      vcycle_run<float>(h, s->lv32, s->d_lv32, s->cfg.gauss_iter2, s->cfg.gauss_iter3);
    k_cvt_to_f64<<<grid_of(n), 256, 0, st>>>(s->lv32[0].x, x, n);
    count_launches(2);
    return;
  }
  if (sign == 1.0) {
    if (b != s->lv[0].b) cudaMemcpyAsync(s->lv[0].b, b, n * sizeof(double), cudaMemcpyDeviceToDevice, st);
  } else {
    k_neg<<<grid_of(n), 256, 0, st>>>(s->lv[0].b, b, n);
    count_launches(1);
  }
  if (which == kHierDirichlet)
    vcycle_run<double>(h, s->lvD, s->d_lvD, s->cfg.gauss_iter2, s->cfg.gauss_iter3);
  else if (which == kHierPeriodic)
    vcycle_run<double, true>(h, s->lvP, s->d_lvP, s->pre_gi2, s->pre_gi3);
  else
    vcycle_run<double>(h, s->lv, s->d_lv, s->cfg.gauss_iter2, s->cfg.gauss_iter3);
  if (x != s->lv[0].x) cudaMemcpyAsync(x, s->lv[0].x, n * sizeof(double), cudaMemcpyDeviceToDevice, st);
}

// DOT2 of two PressureVelocity vectors: the pressure and the counted face
// copies (E/N/T), one contiguous prefix
int dot_dev(asam_ctx* h, const double* a, const double* b, double* out, int mode) {
  ProjState* s = h->proj;
  const size_t n = lendot(s);
  k_pdot_partial<<<kRedGrid, kRedBlock, 0, h->L.stream>>>(a, b, n, s->partial);
  k_pdot_final<<<1, kRedBlock, 0, h->L.stream>>>(s->partial, kRedGrid, out, mode);
  count_launches(2);
  return kOk;
}

// PreFac2 (MODULE/Control_Mod.f90:59): the configured value, 0.5 when unset
double prefac2_of(const ProjState* s) { return s->cfg.prefac2 > 0.0 ? s->cfg.prefac2 : 0.5; }

size_t faces_per_pair(const ProjState* s, const Dims& d, int pair) {
  const size_t sz[3] = {(size_t)d.ny * d.nz, (size_t)d.nx * d.nz, (size_t)d.nx * d.ny};
  return s->fc.off[2 * pair] >= 0 ? sz[pair] : 0;
}

// Exchange of the face unknowns of v
void exchange_dev(asam_ctx* h, double* v) {
  ProjState* s = h->proj;
  if (!s->nface) return;
  const Dims& d = h->d;
  const size_t nX = faces_per_pair(s, d, 0), nY = faces_per_pair(s, d, 1), nZ = faces_per_pair(s, d, 2);
  k_pv_exchange<<<grid_of(nX + nY + nZ), 256, 0, h->L.stream>>>(s->fc, nX, nY, nZ, v);
  count_launches(1);
}

// y = MatVec1(x) = MatVecFull: -(A x) on the pressure, plus the face terms
// and face equations of the periodic sides (then Exchange when asked)
void matvec1_dev(asam_ctx* h, const double* x, double* y, bool exchange) {
  ProjState* s = h->proj;
  const size_t n = len0(s);
  const cudaStream_t st = h->L.stream;
  k_matvec3<double><<<grid_of(n), 256, 0, st>>>(s->d_lv, 0, x, nullptr, y, 1);
  count_launches(1);
  if (!s->nface) return;
  const Dims& d = h->d;
  const double bd = s->beta0 * s->dtp;
  const Lev2& P0 = s->lv[0].pl[0];
  k_pv_face_p<<<grid_of(s->nface), 256, 0, st>>>(d, h->geom(), s->wt, P0, s->fc, bd, 0, x, y);
  k_pv_faces<<<grid_of(s->nface / 2), 256, 0, st>>>(d, h->geom(), s->wt, P0, s->fc, bd, prefac2_of(s), 0,
                                                     exchange ? 1 : 0, x, x, y);
  count_launches(2);
}

// z = PSolve1(v) (PreCond_Mod.f90:1555-1571).  Closed block: PressurePre(-v).
// With face unknowns: PressurePre; b2pBx1Full + Exchange; SchurPreFull (the
// face terms as a pressure right-hand side, Solve_3D on LaplDirichlet, the
// faces from that pressure) + Exchange; b1pBTx2Full; PressurePre.
void psolve_per_dev(asam_ctx* h, const double* v, double* z);
void psolve1_dev(asam_ctx* h, const double* v, double* z) {
  ProjState* s = h->proj;
  if (!s->nface) {
    vcycle_any(h, v, -1.0, z);
    return;
  }
  if (use_per(h) && s->lvP_ready) {
    psolve_per_dev(h, v, z);
    return;
  }
  const Dims& d = h->d;
  const cudaStream_t st = h->L.stream;
  const size_t n = len0(s);
  const double bd = s->beta0 * s->dtp;
  const Lev2& P0 = s->lv[0].pl[0];
  const double pf = prefac2_of(s);
  vcycle_any(h, v, 1.0, s->tmp);  // PressurePre(z, v): the pressure of z in tmp
  k_pv_faces<<<grid_of(s->nface / 2), 256, 0, st>>>(d, h->geom(), s->wt, P0, s->fc, bd, pf, 1, 1, v, s->tmp, z);
  cudaMemsetAsync(s->tmp2, 0, n * sizeof(double), st);  // SchurPreBlock: BVec%p = 0
  k_pv_face_p<<<grid_of(s->nface), 256, 0, st>>>(d, h->geom(), s->wt, P0, s->fc, bd, 1, z, s->tmp2);
  vcycle_any(h, s->tmp2, 1.0, s->tmp, kHierDirichlet);
  k_pv_faces<<<grid_of(s->nface / 2), 256, 0, st>>>(d, h->geom(), s->wt, P0, s->fc, bd, pf, 2, 1, z, s->tmp, z);
  k_neg<<<grid_of(n), 256, 0, st>>>(s->tmp2, v, n);  // b1pBTx2Full: -x%p + the face terms
  k_pv_face_p<<<grid_of(s->nface), 256, 0, st>>>(d, h->geom(), s->wt, P0, s->fc, bd, 0, z, s->tmp2);
  count_launches(5);
  vcycle_any(h, s->tmp2, 1.0, z);  // PressurePre(z, z)
}

// The refined mode's preconditioner on a block with periodic x/y sides (no
// reference counterpart; FGMRES is flexible, so any preconditioner leaves its
// FP64 Arnoldi relation and residual test unchanged): the face unknowns of
// the PressureVelocity system are eliminated exactly -- the Schur complement
// on the pressure is the Laplacian with the shared face treated as an
// interior face -- and that periodic Laplacian is solved by one V-cycle of
// the same multigrid whose plane and line relaxations also couple across the
// periodic sides.  One V-cycle per FGMRES step instead of PSolve1's three.
//   rhs' = v_p - b_W v_u/M at the first cell + b_E v_u/M at the last
//   p    = L_per^-1 (-rhs')
//   u    = (v_u - cp_W(p) + cp_E(p))/M on both copies of the face
// (b = beta0*dtP*F*DT*DTT, cp = beta0*dtP*F*DUT*DU*p, M the face's whole mass).
void psolve_per_dev(asam_ctx* h, const double* v, double* z) {
  ProjState* s = h->proj;
  const Dims& d = h->d;
  const cudaStream_t st = h->L.stream;
  const size_t n = len0(s);
  const double bd = s->beta0 * s->dtp;
  const Lev2& P0 = s->lv[0].pl[0];
  cudaMemcpyAsync(s->tmp2, v, n * sizeof(double), cudaMemcpyDeviceToDevice, st);
  k_pv_face_p<<<grid_of(s->nface), 256, 0, st>>>(d, h->geom(), s->wt, P0, s->fc, bd, 2, v, s->tmp2);
  count_launches(1);
  vcycle_any(h, s->tmp2, -1.0, z, kHierPeriodic);
  k_pv_faces<<<grid_of(s->nface / 2), 256, 0, st>>>(d, h->geom(), s->wt, P0, s->fc, bd, 0.0, 3, 1, v, z, z);
  count_launches(1);
}

// FGMRES (SOLU/Iter_Mod.f90:121-199) on PressureVelocity vectors x (in/out), b
int fgmres_dev(asam_ctx* h, double* x, const double* b, int maxiter, double tol, int* steps_out, double* rho_out,
               double* rho0_out) {
  ProjState* s = h->proj;
  const cudaStream_t st = h->L.stream;
  const int step = s->cfg.step_gmres;
  const size_t n = lenv(s);
  const int g = grid_of(n);
  std::vector<double> Hh((size_t)(step + 1) * step, 0.0), c(step), sn(step), bh(step + 1), y(step);
  auto HH = [&](int i, int j) -> double& { return Hh[(size_t)(i - 1) + (size_t)(step + 1) * (j - 1)]; };
  double rho = 0.0, rho0 = 0.0;
  int steps = 0;
  double* hd = s->H;  // device slots: column i of H at hd + (step+1)*(i-1)
  for (int iter = 1; iter <= maxiter; ++iter) {
    matvec1_dev(h, x, s->v[0], false);
    k_xpby<<<g, 256, 0, st>>>(b, -1.0, s->v[0], n);
    count_launches(1);
    exchange_dev(h, s->v[0]);
    dot_dev(h, s->v[0], s->v[0], hd, 1);
    CK(cudaMemcpyAsync(s->scal_h, hd, sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    const double beta = s->scal_h[0];
    if (std::isnan(beta)) return kNanDetected;
    if (iter == 1) rho0 = beta;
    if (beta <= 0.0) break;
    k_scale<<<g, 256, 0, st>>>(s->v[0], 1.0 / beta, n);
    count_launches(1);
    bh[0] = beta * 1.0;
    int nr = step;
    for (int i = 1; i <= step; ++i) {
      psolve1_dev(h, s->v[i - 1], s->z[i - 1]);
      matvec1_dev(h, s->z[i - 1], s->v[i], true);
      ++steps;
      double* col = hd + (size_t)(step + 1) * (i - 1);
      for (int k = 1; k <= i; ++k) {
        dot_dev(h, s->v[k - 1], s->v[i], col + (k - 1), 0);
        k_axpy_negdev<<<g, 256, 0, st>>>(s->v[i], s->v[k - 1], col + (k - 1), n);
        count_launches(1);
      }
      dot_dev(h, s->v[i], s->v[i], col + i, 1);
      k_scale_recipdev<<<g, 256, 0, st>>>(s->v[i], col + i, n);
      count_launches(1);
      CK(cudaMemcpyAsync(s->scal_h, col, sizeof(double) * (i + 1), cudaMemcpyDeviceToHost, st));
      CK(cudaStreamSynchronize(st));
      for (int k = 1; k <= i + 1; ++k) HH(k, i) = s->scal_h[k - 1];
      for (int k = 2; k <= i; ++k) {
        const double temp = c[k - 2] * HH(k - 1, i) + sn[k - 2] * HH(k, i);
        HH(k, i) = -sn[k - 2] * HH(k - 1, i) + c[k - 2] * HH(k, i);
        HH(k - 1, i) = temp;
      }
      const double delta = std::sqrt(HH(i, i) * HH(i, i) + HH(i + 1, i) * HH(i + 1, i));
      c[i - 1] = HH(i, i) / delta;
      sn[i - 1] = HH(i + 1, i) / delta;
      HH(i, i) = c[i - 1] * HH(i, i) + sn[i - 1] * HH(i + 1, i);
      bh[i] = -sn[i - 1] * bh[i - 1];
      bh[i - 1] = c[i - 1] * bh[i - 1];
      rho = std::fabs(bh[i]);
      if (std::isnan(rho)) return kNanDetected;
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
    for (int i = 1; i <= nr; ++i) k_axpy<<<g, 256, 0, st>>>(x, s->z[i - 1], y[i - 1], n);
    count_launches(nr);
    if (rho <= tol * rho0) break;
  }
  if (steps_out) *steps_out = steps;
  if (rho_out) *rho_out = rho;
  if (rho0_out) *rho0_out = rho0;
  return check_launch();
}

int need_assembled(asam_ctx* h) {
  if (!h || !h->proj) {
    set_last_error("projection not set up (asam_proj_setup)", __FILE__, __LINE__);
    return kBadArg;
  }
  if (!h->proj->assembled) {
    set_last_error("pressure Laplacian not assembled (asam_lapl_compute)", __FILE__, __LINE__);
    return kBadArg;
  }
  return kOk;
}

// copy n doubles from host or device pointer p into device buffer dst
int copy_in(asam_ctx* h, double* dst, const double* p, size_t n) {
  CK(cudaMemcpyAsync(dst, p, n * sizeof(double), cudaMemcpyDefault, h->L.stream));
  return kOk;
}

// Offset of each side's face unknowns in a PressureVelocity vector of the
// C-ABI: the pressure (nx*ny*nz, x fastest) then the present sides in the
// reference's order u_w, u_e, v_s, v_n, w_b, w_t.
void api_offsets(const asam_ctx* h, size_t off[6]) {
  const ProjState* s = h->proj;
  const Dims& d = h->d;
  size_t o = (size_t)d.nx * d.ny * d.nz;
  for (int side = 0; side < 6; ++side) {
    off[side] = o;
    if (s->fc.off[side] >= 0) o += faces_per_pair(s, d, side / 2);
  }
}

// C-ABI PressureVelocity vector (host or device) -> internal vector dst
int pv_in(asam_ctx* h, const double* api, double* dst) {
  ProjState* s = h->proj;
  const Dims& d = h->d;
  const size_t nc = (size_t)d.nx * d.ny * d.nz;
  const cudaStream_t st = h->L.stream;
  if (int rc = copy_in(h, s->bn, api, nc + s->nface)) return rc;
  k_to_layout<<<grid_of(nc), 256, 0, st>>>(s->lv[0].pl[0], d.nx, d.ny, d.nz, s->bn, dst, 1.0);
  count_launches(1);
  size_t off[6];
  api_offsets(h, off);
  for (int side = 0; side < 6; ++side)
    if (s->fc.off[side] >= 0)
      CK(cudaMemcpyAsync(dst + s->fc.off[side], s->bn + off[side], faces_per_pair(s, d, side / 2) * sizeof(double),
                         cudaMemcpyDeviceToDevice, st));
  return kOk;
}

// internal vector src -> C-ABI PressureVelocity vector (host or device)
int pv_out(asam_ctx* h, const double* src, double* api) {
  ProjState* s = h->proj;
  const Dims& d = h->d;
  const size_t nc = (size_t)d.nx * d.ny * d.nz;
  const cudaStream_t st = h->L.stream;
  k_from_layout<<<grid_of(nc), 256, 0, st>>>(s->lv[0].pl[0], d.nx, d.ny, d.nz, src, s->xn);
  count_launches(1);
  size_t off[6];
  api_offsets(h, off);
  for (int side = 0; side < 6; ++side)
    if (s->fc.off[side] >= 0)
      CK(cudaMemcpyAsync(s->xn + off[side], src + s->fc.off[side], faces_per_pair(s, d, side / 2) * sizeof(double),
                         cudaMemcpyDeviceToDevice, st));
  CK(cudaMemcpyAsync(api, s->xn, (nc + s->nface) * sizeof(double), cudaMemcpyDefault, st));
  return kOk;
}

}  // namespace prj
}  // namespace asam

using namespace asam;
using namespace asam::prj;

extern "C" {

int asam_proj_setup(asam_ctx* h, const asam_proj_config* cfg, const double* dx, const double* dy, const double* dz,
                    const double* metr) {
  if (!h || !cfg || !dx || !dy || !dz) return kBadArg;
  if (cfg->ref_level < 1 || cfg->ref_level > kMaxLev || cfg->gauss_iter2 < 0 || cfg->gauss_iter3 < 0 ||
      cfg->mult_iter2 < 1 || cfg->mult_iter3 < 1 || cfg->step_gmres < 1 || cfg->step_gmres > 64 ||
      cfg->max_restart < 1 || cfg->prefac2 < 0.0) {
    set_last_error("asam_proj_setup: configuration out of range", __FILE__, __LINE__);
    return kBadArg;
  }
  proj_free(h);
  ProjState* s = new ProjState();
  h->proj = s;
  s->st = h->L.stream;
  s->cfg = *cfg;
  s->R = cfg->ref_level;
  const Dims& d = h->d;
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  int rc = kOk;
  Wts& w = s->wt;
  const size_t nc = (size_t)nx * ny * nz;
  struct {
    double** p;
    size_t n;
  } a[] = {{&w.dtu, d.n_uf()}, {&w.dtv, d.n_vf()}, {&w.dtw, d.n_wf()}, {&w.duu, d.n_uf()},
           {&w.duv, d.n_vf()}, {&w.duw, d.n_wf()}, {&w.dut, nc},       {&w.dtt, nc},
           {&w.dx, (size_t)nx}, {&w.dy, (size_t)ny}, {&w.dz, (size_t)nz}, {&w.metr, (size_t)2 * (nx + ny + nz)}};
  for (auto& q : a)
    if ((rc = palloc(s, q.p, q.n))) return rc;
  if ((rc = copy_in(h, w.dx, dx, nx)) || (rc = copy_in(h, w.dy, dy, ny)) || (rc = copy_in(h, w.dz, dz, nz))) return rc;
  if (metr) {
    if ((rc = copy_in(h, w.metr, metr, (size_t)2 * (nx + ny + nz)))) return rc;
  } else {
    std::vector<double> ones((size_t)2 * (nx + ny + nz), 1.0);
    CK(cudaMemcpyAsync(w.metr, ones.data(), ones.size() * sizeof(double), cudaMemcpyHostToDevice, h->L.stream));
    CK(cudaStreamSynchronize(h->L.stream));
  }
  if ((rc = proj_build(h))) return rc;
  CK(cudaStreamSynchronize(h->L.stream));
  return kOk;
}

int asam_proj_weights(asam_ctx* h, const double* dtu, const double* dtv, const double* dtw, const double* duu,
                      const double* duv, const double* duw, const double* dut, const double* dtt) {
  if (!h || !h->proj || !dtu || !dtv || !dtw || !duu || !duv || !duw || !dut || !dtt) return kBadArg;
  ProjState* s = h->proj;
  const Dims& d = h->d;
  const size_t nc = (size_t)d.nx * d.ny * d.nz;
  int rc;
  if ((rc = copy_in(h, s->wt.dtu, dtu, d.n_uf())) || (rc = copy_in(h, s->wt.dtv, dtv, d.n_vf())) ||
      (rc = copy_in(h, s->wt.dtw, dtw, d.n_wf())) || (rc = copy_in(h, s->wt.duu, duu, d.n_uf())) ||
      (rc = copy_in(h, s->wt.duv, duv, d.n_vf())) || (rc = copy_in(h, s->wt.duw, duw, d.n_wf())) ||
      (rc = copy_in(h, s->wt.dut, dut, nc)) || (rc = copy_in(h, s->wt.dtt, dtt, nc)))
    return rc;
  CK(cudaStreamSynchronize(h->L.stream));
  s->weights = true;
  s->assembled = false;
  return kOk;
}

int asam_proj_weights_density(asam_ctx* h, const double* state, int th_pos, int rho_pos, int rv_pos, int rc_pos,
                              int rr_pos, const double* tabs) {
  if (!h || !h->proj || !state || !tabs) return kBadArg;
  const int nc = h->cfg.ncomp;
  auto bad = [&](int p, bool opt) { return opt ? (p < -1 || p >= nc) : (p < 0 || p >= nc); };
  if (bad(th_pos, false) || bad(rho_pos, false) || bad(rv_pos, true) || bad(rc_pos, true) || bad(rr_pos, true))
    return kBadArg;
  ProjState* s = h->proj;
  const Dims& d = h->d;
  const cudaStream_t st = h->L.stream;
  s->st = st;
  const size_t len = (size_t)nc * h->npad;
  const double* ds;
  int rc;
  if ((rc = stage_in(h, state, len, h->stage_a, &ds))) return rc;
  if (!s->tabs) {
    if ((rc = palloc(s, &s->tabs, h->npad))) return rc;
  }
  if ((rc = copy_in(h, s->tabs, tabs, h->npad))) return rc;
  auto comp = [&](int p) { return p >= 0 ? ds + (size_t)p * h->npad : nullptr; };
  const size_t tot = (size_t)d.nx * d.ny * d.nz + d.n_uf() + d.n_vf() + d.n_wf();
  k_weights_density<<<grid_of(tot), 256, 0, st>>>(d, h->geom(), s->wt, comp(th_pos), comp(rho_pos), comp(rv_pos),
                                                   comp(rc_pos), comp(rr_pos), s->tabs);
  count_launches(1);
  CK(cudaStreamSynchronize(st));
  if ((rc = check_launch())) return rc;
  s->weights = true;
  s->assembled = false;
  return kOk;
}

long asam_proj_get_weights(asam_ctx* h, int which, double* out) {
  if (!h || !h->proj || which < 0 || which > 7) return -1;
  ProjState* s = h->proj;
  const Dims& d = h->d;
  const size_t nc = (size_t)d.nx * d.ny * d.nz;
  const double* src[] = {s->wt.dtu, s->wt.dtv, s->wt.dtw, s->wt.duu, s->wt.duv, s->wt.duw, s->wt.dut, s->wt.dtt};
  const size_t n[] = {d.n_uf(), d.n_vf(), d.n_wf(), d.n_uf(), d.n_vf(), d.n_wf(), nc, nc};
  if (!out) return (long)n[which];
  if (cudaStreamSynchronize(h->L.stream) != cudaSuccess) return -1;
  if (cudaMemcpy(out, src[which], n[which] * sizeof(double), cudaMemcpyDefault) != cudaSuccess) return -1;
  return (long)n[which];
}

int asam_lapl_compute(asam_ctx* h, double beta0, double dtp) {
  if (!h || !h->proj || !h->proj->weights) {
    set_last_error("asam_lapl_compute: call asam_proj_setup and asam_proj_weights first", __FILE__, __LINE__);
    return kBadArg;
  }
  ProjState* s = h->proj;
  const Dims& d = h->d;
  const cudaStream_t st = h->L.stream;
  s->st = st;
  s->beta0 = beta0;
  s->dtp = dtp;
  const double bd = beta0 * dtp, bd2 = bd * bd;
  const Facs fc{0.0, 0.0, 0.0, 0.0, 0.0, 0.0};  // SetFactorN
  // SetFactorD (MULTI/Reverse_Mod.f90:95-213): 2 on a periodic side, 0 on a
  // closed wall (velocity rule other than 'OutFlow'); axes (1,2,3) = (z,x,y)
  const double fz = d.per_z ? 2.0 : 0.0, fx = d.per_x ? 2.0 : 0.0, fy = d.per_y ? 2.0 : 0.0;
  const Facs fcD{fz, fz, fx, fx, fy, fy};
  // the periodic Laplacian: the diagonal term of the shared face is the
  // interior-face term 2*F*../(d(first)+d(last)), i.e. the boundary term with
  // factor 2*d(first)/(d(first)+d(last)) -- 1 on the uniform horizontal grids
  // of the configurations (taken as 1: the hierarchy only preconditions)
  const bool per = use_per(h);
  const Facs fcP{0.0, 0.0, d.per_x ? 1.0 : 0.0, d.per_x ? 1.0 : 0.0, d.per_y ? 1.0 : 0.0, d.per_y ? 1.0 : 0.0};
  if (per) {
    if (int rc = alloc_levP(s, d)) return rc;
  }
  const double fa = s->cfg.fac_anela;
  k_fine_fields<<<grid_of((size_t)(d.nx + 1) * (d.nz + 1) * (d.ny + 1)), 256, 0, st>>>(
      d, h->fu, h->fv, h->fw, h->volc, s->wt.dtu, s->wt.dtv, s->wt.dtw, s->wt.duu, s->wt.duv, s->wt.duw, s->wt.dut, s->g);
  k_fine_1d<<<1, 256, 0, st>>>(d.nx, d.ny, d.nz, s->wt.dx, s->wt.dy, s->wt.dz, s->wt.metr, s->g);
  long long nl = 2;
  const int n1 = d.nz, n2 = d.nx, n3 = d.ny;
  for (int L = 0; L < s->R; ++L) {
    Lev3& A = s->lv[L];
    const int sh3 = (1 << L) - 1;
    for (int L2 = L; L2 < s->R; ++L2) {
      const int sh = (1 << L2) - 1;
      Fields c = s->c;
      c.n1 = (n1 + sh) / (sh + 1);
      c.n2 = (n2 + sh) / (sh + 1);
      c.n3 = (n3 + sh3) / (sh3 + 1);
      const size_t nf = (size_t)(c.n1 + 1) * c.n2 * c.n3 + (size_t)c.n1 * (c.n2 + 1) * c.n3 + (size_t)c.n1 * c.n2 * (c.n3 + 1);
      const size_t ncell = (size_t)c.n1 * c.n2 * c.n3;
      k_coarse_faces<<<grid_of(nf), 256, 0, st>>>(s->g, c, sh, sh, sh3);
      k_coarse_cells<<<grid_of(ncell), 256, 0, st>>>(s->g, c, sh, sh, sh3);
      k_coarse_1d<<<1, 256, 0, st>>>(s->g, c, sh, sh, sh3);
      Lev2& P = A.pl[L2 - L];
      const bool full = L2 == L;
      k_assemble<<<grid_of(ncell), 256, 0, st>>>(c, P, full ? A.u3 : nullptr, full ? A.l3 : nullptr, full ? 1 : 0, bd2, fc, fa);
      k_factor<<<grid_of((size_t)P.m3 * P.c2), 256, 0, st>>>(P);
      nl += 5;
      if (s->nface > 0 && !per) {  // LaplDirichlet from the same coarse fields
        Lev3& B = s->lvD[L];
        Lev2& Q = B.pl[L2 - L];
        k_assemble<<<grid_of(ncell), 256, 0, st>>>(c, Q, full ? B.u3 : nullptr, full ? B.l3 : nullptr, full ? 1 : 0, bd2,
                                                   fcD, fa);
        k_factor<<<grid_of((size_t)Q.m3 * Q.c2), 256, 0, st>>>(Q);
        nl += 2;
      }
      if (per) {  // the periodic Laplacian of the refined mode's preconditioner
        Lev3& B = s->lvP[L];
        Lev2& Q = B.pl[L2 - L];
        k_assemble<<<grid_of(ncell), 256, 0, st>>>(c, Q, full ? B.u3 : nullptr, full ? B.l3 : nullptr, full ? 1 : 0, bd2,
                                                   fcP, fa);
        const size_t nw = (size_t)c.n1 * (c.n3 + (full ? c.n2 : 0));
        k_assemble_wrap<<<grid_of(nw), 256, 0, st>>>(c, Q, full ? B.wyl : nullptr, full ? B.wyh : nullptr, full ? 1 : 0,
                                                     d.per_x, d.per_y, bd2);
        k_factor<<<grid_of((size_t)Q.m3 * Q.c2), 256, 0, st>>>(Q);
        nl += 3;
      }
    }
  }
  count_launches(nl);
  s->lv32_ready = false;
  s->lvP32_ready = false;
  s->lvP_ready = per;
  s->lvD_ready = s->nface > 0 && !per;
  if (use_mg32(h)) {
    if (int rc = convert_lev32(h)) return rc;
    if (per) {
      if (int rc = convert_levP32(h)) return rc;
    }
  }
  CK(cudaStreamSynchronize(st));
  int rc = check_launch();
  if (!rc) s->assembled = true;
  return rc;
}

int asam_proj_set_pre_schedule(asam_ctx* h, int gauss_iter2, int gauss_iter3) {
  if (!h || !h->proj || gauss_iter2 < 0 || gauss_iter3 < 0) return kBadArg;
  h->proj->pre_gi2 = gauss_iter2;
  h->proj->pre_gi3 = gauss_iter3;
  return kOk;
}

int asam_proj_set_preconditioner(asam_ctx* h, int kind) {
  if (!h || !h->proj || kind < -1 || kind > 1) return kBadArg;
  ProjState* s = h->proj;
  if (s->pre_kind != kind) {
    s->pre_kind = kind;
    s->assembled = false;  // the next asam_lapl_compute assembles what it needs
  }
  return kOk;
}

int asam_proj_set_precision(asam_ctx* h, int prec) {
  if (!h || !h->proj || prec < -1 || prec > 1) return kBadArg;
  ProjState* s = h->proj;
  s->mg_prec = prec;
  if (s->assembled && use_mg32(h) && !s->lv32_ready) {
    s->st = h->L.stream;
    if (int rc = convert_lev32(h)) return rc;
    if (s->lvP_ready) {
      if (int rc = convert_levP32(h)) return rc;
    }
    CK(cudaStreamSynchronize(h->L.stream));
    return check_launch();
  }
  return kOk;
}

long asam_lapl_get(asam_ctx* h, int level3, int level2, int which, double* out) {
  if (need_assembled(h)) return -1;
  ProjState* s = h->proj;
  if (level3 < 0 || level3 >= s->R || level2 < level3 || level2 >= s->R || which < 0 || which > 6) return -1;
  if (which >= 5 && level2 != level3) return -1;
  const Lev3& A = s->lv[level3];
  const Lev2& P = A.pl[level2 - level3];
  const double* src[] = {P.d, P.uz, P.lz, P.ux, P.lx, A.u3, A.l3};
  const size_t n = P.ps * P.m3;
  const long cnt = (long)P.c1 * P.c2 * P.m3;
  if (!out) return cnt;
  std::vector<double> buf(n);
  if (cudaStreamSynchronize(h->L.stream) != cudaSuccess) return -1;
  if (cudaMemcpy(buf.data(), src[which], n * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
  long q = 0;
  for (int k = 0; k < P.m3; ++k)
    for (int j = 0; j < P.c2; ++j)
      for (int i = 0; i < P.c1; ++i) out[q++] = buf[(size_t)k * P.ps + slot(P.w, P.h, i, j)];
  return cnt;
}

int asam_lapl_matvec(asam_ctx* h, const double* x, double* y) {
  if (int rc = need_assembled(h)) return rc;
  if (!x || !y) return kBadArg;
  ProjState* s = h->proj;
  const Dims& d = h->d;
  const size_t nc = (size_t)d.nx * d.ny * d.nz, n = len0(s);
  const cudaStream_t st = h->L.stream;
  const Lev2& P0 = s->lv[0].pl[0];
  int rc;
  if ((rc = copy_in(h, s->xn, x, nc))) return rc;
  k_to_layout<<<grid_of(nc), 256, 0, st>>>(P0, d.nx, d.ny, d.nz, s->xn, s->tmp, 1.0);
  k_matvec3<double><<<grid_of(n), 256, 0, st>>>(s->d_lv, 0, s->tmp, nullptr, s->v[0], 2);
  k_from_layout<<<grid_of(nc), 256, 0, st>>>(P0, d.nx, d.ny, d.nz, s->v[0], s->bn);
  count_launches(3);
  CK(cudaMemcpyAsync(y, s->bn, nc * sizeof(double), cudaMemcpyDefault, st));
  CK(cudaStreamSynchronize(st));
  return check_launch();
}

int asam_lapl_vcycle(asam_ctx* h, const double* b, double* x) {
  if (int rc = need_assembled(h)) return rc;
  if (!x || !b) return kBadArg;
  ProjState* s = h->proj;
  const Dims& d = h->d;
  const size_t nc = (size_t)d.nx * d.ny * d.nz;
  const cudaStream_t st = h->L.stream;
  const Lev2& P0 = s->lv[0].pl[0];
  int rc;
  if ((rc = copy_in(h, s->bn, b, nc))) return rc;
  k_to_layout<<<grid_of(nc), 256, 0, st>>>(P0, d.nx, d.ny, d.nz, s->bn, s->lv[0].b, 1.0);
  count_launches(1);
  vcycle_any(h, s->lv[0].b, 1.0, s->lv[0].x);
  k_from_layout<<<grid_of(nc), 256, 0, st>>>(P0, d.nx, d.ny, d.nz, s->lv[0].x, s->xn);
  count_launches(1);
  CK(cudaMemcpyAsync(x, s->xn, nc * sizeof(double), cudaMemcpyDefault, st));
  CK(cudaStreamSynchronize(st));
  return check_launch();
}

int asam_solve_sound(asam_ctx* h, double* x, const double* b, int* maxiter, double* tol) {
  if (int rc = need_assembled(h)) return rc;
  if (!x || !b || !maxiter || !tol || *maxiter < 1) return kBadArg;
  ProjState* s = h->proj;
  const cudaStream_t st = h->L.stream;
  int rc;
  if ((rc = pv_in(h, b, s->bl)) || (rc = pv_in(h, x, s->xl))) return rc;
  int steps = 0;
  double rho = 0.0, rho0 = 0.0;
  rc = fgmres_dev(h, s->xl, s->bl, *maxiter, *tol, &steps, &rho, &rho0);
  if (rc && rc != kNotConverged) return rc;
  if ((rc = pv_out(h, s->xl, x))) return rc;
  CK(cudaStreamSynchronize(st));
  if ((rc = check_launch())) return rc;
  const double lim = *tol * rho0;
  *maxiter = steps;
  *tol = rho0 > 0.0 ? rho / rho0 : 0.0;
  return rho0 > 0.0 && rho > lim ? kNotConverged : kOk;
}

long asam_proj_face_count(asam_ctx* h) { return h && h->proj ? (long)h->proj->nface : -1; }

int asam_proj_matvec1(asam_ctx* h, const double* x, double* b) {
  if (int rc = need_assembled(h)) return rc;
  if (!x || !b) return kBadArg;
  ProjState* s = h->proj;
  int rc;
  if ((rc = pv_in(h, x, s->xl))) return rc;
  matvec1_dev(h, s->xl, s->tmp, false);
  if ((rc = pv_out(h, s->tmp, b))) return rc;
  CK(cudaStreamSynchronize(h->L.stream));
  return check_launch();
}

int asam_proj_psolve1(asam_ctx* h, const double* x, double* b) {
  if (int rc = need_assembled(h)) return rc;
  if (!x || !b) return kBadArg;
  ProjState* s = h->proj;
  int rc;
  if ((rc = pv_in(h, x, s->xl))) return rc;
  psolve1_dev(h, s->xl, s->bl);
  if ((rc = pv_out(h, s->bl, b))) return rc;
  CK(cudaStreamSynchronize(h->L.stream));
  return check_launch();
}

long asam_lapl_get_dirichlet(asam_ctx* h, int level3, int level2, int which, double* out) {
  if (need_assembled(h)) return -1;
  ProjState* s = h->proj;
  if (!s->nface || !s->lvD_ready) return -1;
  std::swap(s->lv, s->lvD);
  const long r = asam_lapl_get(h, level3, level2, which, out);
  std::swap(s->lv, s->lvD);
  return r;
}

int asam_lapl_vcycle_dirichlet(asam_ctx* h, const double* b, double* x) {
  if (int rc = need_assembled(h)) return rc;
  if (!x || !b) return kBadArg;
  ProjState* s = h->proj;
  if (!s->nface || !s->lvD_ready) return kBadArg;
  const Dims& d = h->d;
  const size_t nc = (size_t)d.nx * d.ny * d.nz;
  const cudaStream_t st = h->L.stream;
  const Lev2& P0 = s->lv[0].pl[0];
  int rc;
  if ((rc = copy_in(h, s->bn, b, nc))) return rc;
  k_to_layout<<<grid_of(nc), 256, 0, st>>>(P0, d.nx, d.ny, d.nz, s->bn, s->tmp2, 1.0);
  count_launches(1);
  vcycle_any(h, s->tmp2, 1.0, s->tmp, kHierDirichlet);
  k_from_layout<<<grid_of(nc), 256, 0, st>>>(P0, d.nx, d.ny, d.nz, s->tmp, s->xn);
  count_launches(1);
  CK(cudaMemcpyAsync(x, s->xn, nc * sizeof(double), cudaMemcpyDefault, st));
  CK(cudaStreamSynchronize(st));
  return check_launch();
}

int asam_project_vel_face(asam_ctx* h, double* uf, double* vf, double* wf, double* incr, const double* state,
                          int th_pos, int rho_pos, const int* scalars, int nscalar, double* pressure, int* steps,
                          double* resid) {
  if (int rc = need_assembled(h)) return rc;
  const int ncomp = h->cfg.ncomp;
  if (!uf || !vf || !wf || !incr || th_pos >= ncomp || rho_pos >= ncomp || nscalar < 0 ||
      (nscalar > 0 && (!scalars || !state || rho_pos < 0)))
    return kBadArg;
  for (int q = 0; q < nscalar; ++q)
    if (scalars[q] < 0 || scalars[q] >= ncomp) return kBadArg;
  ProjState* s = h->proj;
  const Dims& d = h->d;
  const size_t nc = (size_t)d.nx * d.ny * d.nz, len = (size_t)ncomp * h->npad;
  const cudaStream_t st = h->L.stream;
  s->st = st;
  const Lev2& P0 = s->lv[0].pl[0];
  int rc;
  if (!s->stage_u) {
    if ((rc = palloc(s, &s->stage_u, d.n_uf())) || (rc = palloc(s, &s->stage_v, d.n_vf())) ||
        (rc = palloc(s, &s->stage_w, d.n_wf())))
      return rc;
  }
  double *du, *dv, *dw, *di;
  const double* ds = nullptr;
  du = is_device_ptr(uf) ? uf : s->stage_u;
  dv = is_device_ptr(vf) ? vf : s->stage_v;
  dw = is_device_ptr(wf) ? wf : s->stage_w;
  if (du != uf) CK(cudaMemcpyAsync(du, uf, d.n_uf() * sizeof(double), cudaMemcpyHostToDevice, st));
  if (dv != vf) CK(cudaMemcpyAsync(dv, vf, d.n_vf() * sizeof(double), cudaMemcpyHostToDevice, st));
  if (dw != wf) CK(cudaMemcpyAsync(dw, wf, d.n_wf() * sizeof(double), cudaMemcpyHostToDevice, st));
  if ((rc = stage_out_begin(h, incr, len, h->stage_a, &di, true))) return rc;
  if (state) {
    if ((rc = stage_in(h, state, len, h->stage_b, &ds))) return rc;
  }
  // Rhs
  k_rhs<<<grid_of(nc), 256, 0, st>>>(d, h->geom(), s->wt, du, dv, dw, th_pos >= 0 ? di + (size_t)th_pos * h->npad : nullptr,
                                      s->beta0 * s->dtp, s->cfg.fac_anela >= 1.0 ? 1 : 0, P0, s->bl);
  if (s->nface) CK(cudaMemsetAsync(s->bl + len0(s), 0, sizeof(double) * s->nface, st));  // b=Zero: faces stay 0
  CK(cudaMemsetAsync(s->xl, 0, sizeof(double) * lenv(s), st));
  count_launches(1);
  int nsteps = 0;
  double rho = 0.0, rho0 = 0.0;
  rc = fgmres_dev(h, s->xl, s->bl, s->cfg.max_restart, s->cfg.tol, &nsteps, &rho, &rho0);
  if (rc) return rc;
  // UpdateVelocity
  k_from_layout<<<grid_of(nc), 256, 0, st>>>(P0, d.nx, d.ny, d.nz, s->xl, s->xn);
  k_update_vel<<<grid_of(d.n_uf() + d.n_vf() + d.n_wf()), 256, 0, st>>>(d, h->geom(), s->wt, s->xn, s->xl, s->fc, du, dv,
                                                                         dw, s->beta0, s->dtp);
  k_update_incr<<<grid_of(nc), 256, 0, st>>>(d, h->geom(), s->wt, du, dv, dw, di, th_pos, rho_pos, s->beta0,
                                             s->dtp);
  k_scale_dut<<<grid_of(nc), 256, 0, st>>>(s->xn, s->wt.dut, nc);
  count_launches(4);
  if (nscalar > 0) {  // DivScalar, one scalar at a time through the face terms
    if (!s->div_m) {
      if ((rc = palloc(s, &s->div_m, d.npad())) || (rc = palloc(s, &s->div_fu, d.n_uf())) ||
          (rc = palloc(s, &s->div_fv, d.n_vf())) || (rc = palloc(s, &s->div_fw, d.n_wf())))
        return rc;
    }
    const size_t npad = h->npad;
    const double* rho = ds + (size_t)rho_pos * npad;
    for (int q = 0; q < nscalar; ++q) {
      k_div_m<<<grid_of(npad), 256, 0, st>>>(npad, h->geom().volc, ds + (size_t)scalars[q] * npad, rho, s->div_m);
      k_div_faces<<<grid_of(d.n_uf() + d.n_vf() + d.n_wf()), 256, 0, st>>>(d, h->geom(), du, dv, dw, s->div_m,
                                                                          s->div_fu, s->div_fv, s->div_fw);
      k_div_apply<<<grid_of(nc), 256, 0, st>>>(d, h->geom(), s->div_fu, s->div_fv, s->div_fw,
                                               di + (size_t)scalars[q] * npad, s->beta0, s->dtp);
      count_launches(3);
    }
  }
  if (du != uf) CK(cudaMemcpyAsync(uf, du, d.n_uf() * sizeof(double), cudaMemcpyDeviceToHost, st));
  if (dv != vf) CK(cudaMemcpyAsync(vf, dv, d.n_vf() * sizeof(double), cudaMemcpyDeviceToHost, st));
  if (dw != wf) CK(cudaMemcpyAsync(wf, dw, d.n_wf() * sizeof(double), cudaMemcpyDeviceToHost, st));
  if (pressure) CK(cudaMemcpyAsync(pressure, s->xn, nc * sizeof(double), cudaMemcpyDefault, st));
  if ((rc = stage_out_end(h, incr, len, di))) return rc;
  CK(cudaStreamSynchronize(st));
  if ((rc = check_launch())) return rc;
  if (steps) *steps = nsteps;
  if (resid) *resid = rho0 > 0.0 ? rho / rho0 : 0.0;
  return rho0 > 0.0 && rho > s->cfg.tol * rho0 ? kNotConverged : kOk;
}

long long asam_proj_vcycles(asam_ctx* h) { return h && h->proj ? h->proj->vcycles : 0; }

}  // extern "C"
