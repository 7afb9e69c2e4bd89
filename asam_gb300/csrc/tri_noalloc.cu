// Batched vertical-column Thomas solve that allocates nothing.
//
// asam_tri_solve (capi.cu) allocates device buffers for its inputs and for
// the elimination factors w of Solve_1D on every call.  Some callers cannot
// let a library allocate device memory: a host model that hands out all
// device memory from its own pool at start-up, and a caller that overlaps this
// solve with work on other streams (cudaMalloc and cudaFree synchronise the
// device, which would serialise that work).  For them this entry point takes
// device pointers for every input and output and keeps w in a fixed-size
// array that lives in the library's device image.
//
// Compiled with -fmad=false like k64.cu, so the solution is bit-identical to
// asam_tri_solve's.
#include "kernels.cuh"

namespace asam {
void set_last_error(const char* msg, const char* file, int line);
void count_launches(long long n);
}  // namespace asam

namespace {

// Elimination factors of the column solve.  Every GPU that loads the library
// holds this array (32 MiB) until the process exits.  All calls share it: it
// keeps the previous call's contents, which is harmless because the Thomas
// forward sweep writes each w before the backward sweep reads it (nothing has
// to start at zero).  Calls that overlap on the GPU (two streams at once) race
// on it.
constexpr long long kTriNoAllocMax = 1LL << 22;  // ncol*n1 doubles
static __device__ __align__(256) double g_tri_scratch[kTriNoAllocMax];

// Device address of the scratch array on the current device (the host-side
// symbol is only a stand-in and must not be passed to a kernel).  Looked up
// on every call: the lookup is cheap, and a cached address would go stale
// when the device's primary context is reset or recreated.
int scratch_on_current_device(double** out) {
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_tri_scratch);
  if (e != cudaSuccess) {
    asam::set_last_error(cudaGetErrorString(e), __FILE__, __LINE__);
    return asam::kCudaError;
  }
  *out = static_cast<double*>(p);
  return asam::kOk;
}

// A pointer the kernel on the current device may use: device memory of this
// device, or managed memory.
bool on_device(const void* p, int dev) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return (a.type == cudaMemoryTypeDevice && a.device == dev) || a.type == cudaMemoryTypeManaged;
}

}  // namespace

extern "C" int asam_tri_solve_noalloc(int ncol, int n1, const double* d, const double* u, const double* l, double* b,
                                      void* stream) {
  if (ncol < 1 || n1 < 1 || !d || !b || (n1 > 1 && (!u || !l))) {
    asam::set_last_error("asam_tri_solve_noalloc: bad sizes or null pointer", __FILE__, __LINE__);
    return asam::kBadArg;
  }
  if ((long long)ncol * n1 > kTriNoAllocMax) {
    asam::set_last_error(
        "asam_tri_solve_noalloc: ncol*n1 exceeds the fixed scratch of 4194304 values; use asam_tri_solve",
        __FILE__, __LINE__);
    return asam::kBadArg;
  }
  int dev = 0;
  cudaError_t de = cudaGetDevice(&dev);
  if (de != cudaSuccess) {
    asam::set_last_error(cudaGetErrorString(de), __FILE__, __LINE__);
    return asam::kCudaError;
  }
  if (!on_device(d, dev) || !on_device(b, dev) || (n1 > 1 && (!on_device(u, dev) || !on_device(l, dev)))) {
    asam::set_last_error("asam_tri_solve_noalloc: d, u, l and b must be device pointers of the current device",
                         __FILE__, __LINE__);
    return asam::kBadArg;
  }
  double* w = nullptr;
  int rc = scratch_on_current_device(&w);
  if (rc) return rc;
  k_tri_solve_w<double><<<(ncol + 32 * kTriWarps - 1) / (32 * kTriWarps), 32 * kTriWarps, 0, (cudaStream_t)stream>>>(
      ncol, n1, d, u, l, b, w);
  asam::count_launches(1);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    asam::set_last_error(cudaGetErrorString(e), __FILE__, __LINE__);
    return asam::kCudaError;
  }
  return asam::kOk;
}
