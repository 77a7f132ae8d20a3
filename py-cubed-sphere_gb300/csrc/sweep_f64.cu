// float64 instantiations of the line-marching step kernel (FMA contraction allowed; parity
// with the reference is checked at 1e-12 relative by the GPU tests).
#include "sweep.cuh"

namespace csadv {
template int sweep_launch<double>(int, int, const SweepSolve *, const int2 *, int, int, size_t, cudaStream_t, int);
}
