// float32 instantiations of the line-marching step kernel (FMA contraction allowed).
#include "sweep.cuh"

namespace csadv {
template int sweep_launch<float>(int, int, const SweepSolve *, const int2 *, int, int, size_t, cudaStream_t);
}
