// FP32 step kernel: the paired-tracer line-marching kernel (every operation rounded explicitly).
#include "sweep2.cuh"
