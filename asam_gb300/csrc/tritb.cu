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

__global__ void k_tri_tb_solve(int ncol, int n1, const double* __restrict__ d, const double* __restrict__ u,
                               const double* __restrict__ l, double* __restrict__ b, double* __restrict__ w) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= ncol) return;
  const double* dc = d + (size_t)col * n1 * 4;
  const double* uc = u + (size_t)col * (n1 - 1) * 4;
  const double* lc = l + (size_t)col * (n1 - 1) * 4;
  double* bc = b + (size_t)col * n1 * 2;
  const size_t ws = (size_t)ncol;
  M2 t = ld_m(dc);
  V2 bp = div_2(ld_v(bc), t);
  st_v(bc, bp);
  for (int i = 1; i < n1; ++i) {
    const M2 li = ld_m(lc + (size_t)(i - 1) * 4);
    const M2 wi = div_22(ld_m(uc + (size_t)(i - 1) * 4), t);
    double* wp = w + (size_t)(i - 1) * 4 * ws + col;
    wp[0] = wi.a11;
    wp[ws] = wi.a21;
    wp[2 * ws] = wi.a12;
    wp[3 * ws] = wi.a22;
    t = sub_m(ld_m(dc + (size_t)i * 4), mult_22(li, wi));
    bp = div_2(sub_v(ld_v(bc + (size_t)i * 2), mult_2(li, bp)), t);
    st_v(bc + (size_t)i * 2, bp);
  }
  for (int i = n1 - 2; i >= 0; --i) {
    const double* wp = w + (size_t)i * 4 * ws + col;
    const M2 wi{wp[0], wp[ws], wp[2 * ws], wp[3 * ws]};
    bp = sub_v(ld_v(bc + (size_t)i * 2), mult_2(wi, bp));
    st_v(bc + (size_t)i * 2, bp);
  }
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

}  // namespace

extern "C" {

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
