// Shared definitions of the GB300 transport-stage library.
//
// Memory layout in HBM is the Fortran layout of ASAM, so a Fortran caller can
// hand its arrays over without reshuffling:
//   cell fields   c(ix0:ix1+1, iy0:iy1+1, iz0:iz1+1)  (MODULE/Vector4Cell_Mod.f90:913-926)
//                 padded (i,j,k) -> i + NX*(j + NY*k), NX=nx+2, NY=ny+2
//   face areas    FU(ix0-1:ix1+1, iy0+1:iy1, iz0+1:iz1) etc. (MODULE/Domain_Mod.f90:447-449)
//   volumes       VolC(ix0:ix1+1, iy0:iy1+1, iz0:iz1+1)     (MODULE/Domain_Mod.f90:460)
//   face velocity uF(ix0:ix1, iy0+1:iy1, iz0+1:iz1) etc.   (MODULE/VelocityFace_Mod.f90:211-213)
//   DIA matrix    Val(m,7) column-major, offsets -NXY,-NX,-1,0,1,NX,NXY
//                 (MODULE/Vector4Cell_Mod.f90:1020-1036)
// Several components are stored back to back: comp ic at c + ic*npad.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace asam {

constexpr double kEps = 1.0e-30;  // Eps of CG/Kind_Mod_gf.f90
constexpr int kMaxComp = 16;

struct Dims {
  int nx, ny, nz;        // interior cells
  int per_x, per_y, per_z;  // 1 = periodic side pair (block is its own neighbour), 0 = closed wall
  __host__ __device__ int NX() const { return nx + 2; }
  __host__ __device__ int NY() const { return ny + 2; }
  __host__ __device__ int NZ() const { return nz + 2; }
  __host__ __device__ size_t npad() const { return (size_t)(nx + 2) * (ny + 2) * (nz + 2); }
  __host__ __device__ size_t P(int i, int j, int k) const {
    return (size_t)i + (size_t)(nx + 2) * ((size_t)j + (size_t)(ny + 2) * (size_t)k);
  }
  // native Fortran extents of the face arrays
  __host__ __device__ size_t FU(int i, int j, int k) const {
    return (size_t)(i + 1) + (size_t)(nx + 3) * ((size_t)(j - 1) + (size_t)ny * (size_t)(k - 1));
  }
  __host__ __device__ size_t FV(int i, int j, int k) const {
    return (size_t)(i - 1) + (size_t)nx * ((size_t)(j + 1) + (size_t)(ny + 3) * (size_t)(k - 1));
  }
  __host__ __device__ size_t FW(int i, int j, int k) const {
    return (size_t)(i - 1) + (size_t)nx * ((size_t)(j - 1) + (size_t)ny * (size_t)(k + 1));
  }
  __host__ __device__ size_t UF(int i, int j, int k) const {
    return (size_t)i + (size_t)(nx + 1) * ((size_t)(j - 1) + (size_t)ny * (size_t)(k - 1));
  }
  __host__ __device__ size_t VF(int i, int j, int k) const {
    return (size_t)(i - 1) + (size_t)nx * ((size_t)j + (size_t)(ny + 1) * (size_t)(k - 1));
  }
  __host__ __device__ size_t WF(int i, int j, int k) const {
    return (size_t)(i - 1) + (size_t)nx * ((size_t)(j - 1) + (size_t)ny * (size_t)k);
  }
  // (i, j, k) of padded cell P; 32-bit division whenever the box allows it
  __host__ __device__ void ijk(size_t P, int& i, int& j, int& k) const {
    const unsigned NXu = (unsigned)(nx + 2), NYu = (unsigned)(ny + 2);
    if (P < (size_t)0xffffffffu) {
      const unsigned p = (unsigned)P, r = p / NXu;
      i = (int)(p - r * NXu);
      k = (int)(r / NYu);
      j = (int)(r - (unsigned)k * NYu);
    } else {
      const size_t r = P / NXu;
      i = (int)(P - r * NXu);
      k = (int)(r / NYu);
      j = (int)(r - (size_t)k * NYu);
    }
  }
  __host__ __device__ size_t n_fu() const { return (size_t)(nx + 3) * ny * nz; }
  __host__ __device__ size_t n_fv() const { return (size_t)nx * (ny + 3) * nz; }
  __host__ __device__ size_t n_fw() const { return (size_t)nx * ny * (nz + 3); }
  __host__ __device__ size_t n_uf() const { return (size_t)(nx + 1) * ny * nz; }
  __host__ __device__ size_t n_vf() const { return (size_t)nx * (ny + 1) * nz; }
  __host__ __device__ size_t n_wf() const { return (size_t)nx * ny * (nz + 1); }
};

// Geometry and prescribed face velocities resident on the device.
template <typename T>
struct GeomT {
  const T* volc;
  const T* fu;
  const T* fv;
  const T* fw;
  const T* uf;
  const T* vf;
  const T* wf;
};

// Momentum sources of the dynamical stage of a closed block, added by FcnMet
// to the six LR momentum components (ADVECT/Function_Mod.f90:1267-1297,
// 1389-1393): the pressure gradient before AdvectionScale and the buoyancy
// after it.
template <typename T>
struct MomSrc {
  const T* p;    // PreCell, padded
  const T* rho;  // density component of the state, padded
  const T *dx, *dy, *dz;  // widths of the interior cells
  const T *mxy, *myx;     // MetrXY(iy), MetrYX(ix)
  int pos[6];             // uL, uR, vL, vR, wL, wR components (-1: none)
  int pgrad, buoy;        // PGradient, Buoyancy
  T grav;                 // Grav
};

// Diffusion of the flux right-hand side (DiffusionCompute,
// ADVECT/Diffusion_Mod.f90:11-275): per face the coefficient
// K = DRhoF*F*F/(VL+VR+Eps) (DRhoF the arithmetic face mean DF of the cell
// coefficients, ADVECT/Operator_Mod.f90:49-53, or on an outer wall the interior
// cell's), computed once per coefficient field; a face between two cells of
// the block carries the flux 2K*(phiR-phiL), a face of a periodic side K*(...)
// from each side.  phi = c/(Rho+Eps) of every component.
template <typename T>
struct DiffSrc {
  const T *kx, *ky, *kz;  // uF, vF, wF extents
  const T* phi;
};

// State read by the inflow through the faces of the outer walls
// (AdvectionComputeP, ADVECT/Advection_Mod.f90:975-1044): the ncomp padded
// fields and the density; c == nullptr leaves the inflow and the zeroing of
// the wall halos out (the linearised operators of the adjoint).
template <typename T>
struct WallIn {
  const T* c = nullptr;
  const T* rho = nullptr;
};

// Halo rule of each component on each side that is not periodic (the outer
// walls 'ow'...'ot' of a block): BoundaryCompute
// (ADVECT/BoundaryCondition_Mod.f90:70-346) for the scalars and
// BoundaryVelocityCellCompute (:424-970) for the momentum components.  Sides
// in the order W, E, S, N, B, T; only the face halo cells (tangential interior
// ranges) are set, like the reference's loops.
// The open-boundary kinds of BoundaryCompute take their data from the
// pointers below (device memory, set with the kinds):
//   MeanValue      halo = 2*MeanProfile(ic,iz) - interior (:102-107, 194-199,
//                  282-287: the bottom and top take the first and last level)
//   Function       halo = 2*F - interior, F the caller's value of the start
//                  function (times RhoFun for the non-number components) at
//                  the halo cell (:108-120)
//   InFlowOutFlow  W/E/S/N: on inflow (the face velocity into the block, zero
//                  included) halo = Rho(halo)*VecAmb(halo), else the interior
//                  value (:86-95); no branch on the bottom and top
//   Extrapolation  B/T: halo = 2*c(iz0+1) - c(iz0+2) (:276-281); no branch on
//                  the lateral sides
// A side without the kind's branch leaves its halo as it is, like the
// reference's IF chains.
enum BcKind : signed char {
  kBcNone = 0,       // halo left as it is
  kBcZeroGrad = 1,   // halo = adjacent interior cell
  kBcZeroValue = 2,  // halo = -adjacent interior cell
  kBcMeanValue = 3,
  kBcFunction = 4,
  kBcInflowOutflow = 5,
  kBcExtrapolation = 6,
};
struct BcKinds {
  signed char k[kMaxComp][6];
  const double* mean = nullptr;  // MeanProfile: ncomp x nz, level iz at [ic*nz + iz-1]
  const double* fval = nullptr;  // Function values: ncomp padded fields (halo cells read)
  const double* amb = nullptr;   // VecAmb: ncomp padded fields (halo cells read)
  const double* uf = nullptr;    // face velocities whose sign InFlowOutFlow tests
  const double* vf = nullptr;
  int rho = 0;                   // density component (RhoPos)
};

// Krylov scalars that stay on the device between kernels.
struct KrylovScalars {
  double rho, rho_old, alpha, beta, omega;
  double rnorm, rnorm0, tol;
  double dot_a, dot_b;
  int done;       // 0 running; 1 converged at half step; 2 converged; 3 breakdown
  int iter;
  int gs_err;     // set by the persistent Gauss-Seidel schedule when a wait gave up
  // device-driven iteration (CUDA-graph WHILE loop): limit and the reference's
  // MaxIter/Tol outputs, written by the loop's condition kernel
  int maxiter;
  int out_iters;
  double out_tol;
  // device-driven refined solve (outer FP64 refinement around the FP32
  // BiCGStab): passes of the inner loop's two halves, summed over the outer
  // passes (iter counts the outer passes), to count the kernels that ran
  int passes1, passes2;
};

// Schedule of the persistent Gauss-Seidel wavefront (k_gs_persist): tickets
// (I, J, K, sweep) in pipelined-level order, per-tile completion counters
// (base + last completed sweep + 1, compared in wrap-around arithmetic), the
// epoch base in device memory (advanced by the sweep count after every call
// by a kernel of the same stream, so a captured call replays correctly and
// the counters never need clearing), the ticket counter (zeroed before each
// call) and the error flag.
constexpr int kGsSpinLimit = 1 << 21;  // default polls of one dependency wait
struct GsTileSched {
  const int4* order;
  int nticket;
  int* flags;
  int* counter;
  int* err;
  unsigned* base;
  int group;  // components per CTA
  int spin;   // polls of one dependency wait before the CTA gives up
};

// What a reduction's final kernel does with the sum (Krylov recurrences of
// BiCGStabMet_Vec4CellSp, MODULE/SpMatrix4CellPar_Mod.f90:283-338).
enum ScalarOp {
  OP_STORE_A = 0,     // dot_a = sum
  OP_STORE_B = 1,     // dot_b = sum
  OP_RNORM0 = 2,      // rnorm0 = sqrt(sum)
  OP_RHO = 3,         // rho_old = rho; rho = sum; breakdown flag if rho == 0
  OP_ALPHA = 4,       // alpha = rho / sum
  OP_RNORM_HALF = 5,  // rnorm = sqrt(sum); converged-at-half-step flag
  OP_OMEGA = 6,       // omega = dot_a / sum   (dot_a = (t,r), sum = (t,t))
  OP_RNORM_FULL = 7,  // rnorm = sqrt(sum); converged flag
};
// Which device scalar scales an update.
enum ScalarSel { SEL_ALPHA = 0, SEL_OMEGA = 1, SEL_BETA = 2 };

// Error codes of the C-ABI (mirrored in include/asam_gb300.h).
enum Status {
  kOk = 0,
  kNotConverged = 1,
  kBreakdown = 2,
  kNanDetected = 3,
  kBadArg = 4,
  kCudaError = 5,
  kNoDevice = 6,
  kIoError = 7,
};

}  // namespace asam

#define ASAM_CUDA_OK(expr)                                   \
  do {                                                       \
    cudaError_t _e = (expr);                                 \
    if (_e != cudaSuccess) {                                 \
      asam::set_last_error(cudaGetErrorString(_e), __FILE__, __LINE__); \
      return asam::kCudaError;                               \
    }                                                        \
  } while (0)

namespace asam {
void set_last_error(const char* msg, const char* file, int line);
inline int grid_for(size_t n, int block) { return (int)((n + block - 1) / block); }
}  // namespace asam
