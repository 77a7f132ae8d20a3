// FP32 step kernels for launches whose tracers are grouped as SWEEP_TG_ONE (one tracer per solve).
#include "sweep2.cuh"

namespace csadv {
namespace pairk {
template int launch_group<SWEEP_TG_ONE>(int, int, const SweepSolve *, const int2 *, int, int, size_t, cudaStream_t);
}  // namespace pairk
}  // namespace csadv
