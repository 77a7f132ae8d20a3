// FP32 step kernels for launches whose tracers are grouped as SWEEP_TG_PAIRS (every solve of the launch has an even number of tracers).
#include "sweep2.cuh"

namespace csadv {
namespace pairk {
template int launch_group<SWEEP_TG_PAIRS>(int, int, const SweepSolve *, const int2 *, int, int, size_t, cudaStream_t);
}  // namespace pairk
}  // namespace csadv
