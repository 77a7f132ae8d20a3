// FP32 step kernel: the paired-tracer line-marching kernel (every operation rounded explicitly).
// This unit holds the kernels for any tracer count and the launch dispatch; the pair-only and
// one-tracer kernels are compiled in sweep_f32_pairs.cu and sweep_f32_one.cu.
#include "sweep2.cuh"

namespace csadv {
namespace pairk {
extern template int launch_group<SWEEP_TG_PAIRS>(int, int, const SweepSolve *, const int2 *, int, int, size_t,
                                                 cudaStream_t);
extern template int launch_group<SWEEP_TG_ONE>(int, int, const SweepSolve *, const int2 *, int, int, size_t,
                                               cudaStream_t);
}  // namespace pairk

template <>
int sweep_launch<float>(int recon, int spl, const SweepSolve *dsolves, const int2 *work, int nwork, int grid,
                        size_t smem, cudaStream_t st, int tgroup) {
    if (st == (cudaStream_t)-1) {  // prepare every grouping
        int rc = pairk::launch_group<SWEEP_TG_ANY>(recon, spl, dsolves, work, nwork, grid, smem, st);
        if (!rc) rc = pairk::launch_group<SWEEP_TG_PAIRS>(recon, spl, dsolves, work, nwork, grid, smem, st);
        if (!rc) rc = pairk::launch_group<SWEEP_TG_ONE>(recon, spl, dsolves, work, nwork, grid, smem, st);
        return rc;
    }
    switch (tgroup) {
        case SWEEP_TG_PAIRS: return pairk::launch_group<SWEEP_TG_PAIRS>(recon, spl, dsolves, work, nwork, grid, smem, st);
        case SWEEP_TG_ONE: return pairk::launch_group<SWEEP_TG_ONE>(recon, spl, dsolves, work, nwork, grid, smem, st);
        default: return pairk::launch_group<SWEEP_TG_ANY>(recon, spl, dsolves, work, nwork, grid, smem, st);
    }
}

}  // namespace csadv
