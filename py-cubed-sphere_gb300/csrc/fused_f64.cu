// float64 instantiations of the fused step kernel.
#include "fused.cuh"

namespace csadv {
template int fused_launch<double>(const FusedArgs &, int, int, cudaStream_t);
}
