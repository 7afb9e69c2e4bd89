// FP32 kernels: the inner Krylov solver and preconditioner of the refined
// mode (FMA contraction allowed; dot products still accumulate in FP64).
#include "launchers_impl.cuh"

ASAM_DEFINE_LAUNCHERS(float, float)
