// FP64 kernels, compiled with -fmad=false: every product and sum is rounded
// separately, as in the reference Fortran built without FMA contraction.
#include "launchers_impl.cuh"

ASAM_DEFINE_LAUNCHERS(double, double)

namespace {
__global__ void k_cvt_d2f(size_t len, const double* __restrict__ x, float* __restrict__ y) {
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < len; q += (size_t)gridDim.x * blockDim.x)
    y[q] = (float)x[q];
}
__global__ void k_cvt_f2d(size_t len, const float* __restrict__ x, double* __restrict__ y) {
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < len; q += (size_t)gridDim.x * blockDim.x)
    y[q] = (double)x[q];
}
// y += s * x widened to FP64 (the refinement's correction, one pass)
__global__ void k_add_f2d(size_t len, const float* __restrict__ x, double s, double* __restrict__ y) {
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < len; q += (size_t)gridDim.x * blockDim.x)
    y[q] = y[q] + s * (double)x[q];
}
// y = (float)(s * x): the residual handed to the FP32 inner solver, scaled to
// unit norm so that neither tiny nor huge residuals leave the FP32 range
__global__ void k_cvt_d2f_scaled(size_t len, const double* __restrict__ x, double s, float* __restrict__ y) {
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < len; q += (size_t)gridDim.x * blockDim.x)
    y[q] = (float)(s * x[q]);
}
// slot 7 of the DIA storage: 1/diagonal (IEEE division)
__global__ void k_recip_diag(size_t n, double* __restrict__ val) {
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
    val[7 * n + q] = 1.0 / val[3 * n + q];
}
}  // namespace

namespace asam {
void launch_beta(const Launch& L, KrylovScalars* sc) {
  k_beta<<<1, 1, 0, L.stream>>>(sc);
  count_launches(1);
}
void launch_mass(const Launch& L, const Dims& d, const double* c, const double* volc, double* partial, double* out) {
  k_mass_partial<<<RED_GRID, RED_BLOCK, 0, L.stream>>>(d, c, volc, partial);
  k_dot_final<<<1, RED_BLOCK, 0, L.stream>>>(partial, RED_GRID, nullptr, -1, out);
  count_launches(2);
}
void launch_recip_diag(const Launch& L, size_t npad, double* val) {
  k_recip_diag<<<gs_grid(L, npad), kBlock, 0, L.stream>>>(npad, val);
  count_launches(1);
}
void launch_convert_f64_to_f32(const Launch& L, size_t len, const double* x, float* y) {
  k_cvt_d2f<<<gs_grid(L, len), kBlock, 0, L.stream>>>(len, x, y);
  count_launches(1);
}
void launch_add_f32_to_f64(const Launch& L, size_t len, const float* x, double s, double* y) {
  k_add_f2d<<<gs_grid(L, len), kBlock, 0, L.stream>>>(len, x, s, y);
  count_launches(1);
}
void launch_convert_f64_to_f32_scaled(const Launch& L, size_t len, const double* x, double s, float* y) {
  k_cvt_d2f_scaled<<<gs_grid(L, len), kBlock, 0, L.stream>>>(len, x, s, y);
  count_launches(1);
}
void launch_resid_dot(const Launch& L, const Dims& d, int ncomp, const double* val, const double* x, const double* b,
                      double* r, double* partial, KrylovScalars* sc, int op, double* out) {
  k_resid_dot<double><<<RED_GRID, RED_BLOCK, 0, L.stream>>>(d, ncomp, val, x, b, r, partial);
  k_dot_final<<<1, RED_BLOCK, 0, L.stream>>>(partial, RED_GRID, sc, op, out);
  count_launches(2);
}
void launch_convert_f32_to_f64(const Launch& L, size_t len, const float* x, double* y) {
  k_cvt_f2d<<<gs_grid(L, len), kBlock, 0, L.stream>>>(len, x, y);
  count_launches(1);
}
}  // namespace asam
