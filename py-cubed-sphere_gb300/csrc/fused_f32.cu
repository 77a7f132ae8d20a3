// float32 instantiations of the fused step kernel (FMA contraction allowed).
#include "fused.cuh"

namespace csadv {
template int fused_launch<float>(const FusedArgs &, int, int, cudaStream_t);
}
