// float64 instantiations of the fused step kernel (FMA contraction allowed; parity with the
// reference is checked at 1e-12 relative in tests/test_gpu_fused.py).
#include "fused.cuh"

namespace csadv {
template int fused_launch<double>(const FusedArgs &, int, int, cudaStream_t);
}
