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

// Forms the deferred MF-PR corrections of a field: the descriptor is that of the launch that
// reads it (Qin, part_in, pend_in, corr_in); the corrections go to corr_in and the field is marked
// as having none pending.  One block; the order of the sums is psum_all's, as in the step kernel.
__global__ void __launch_bounds__(SWEEP_THREADS) k_sweep2_finalize(const SweepSolve *__restrict__ Sp) {
    __shared__ double red[SWEEP_THREADS];
    const SweepSolve &S = *Sp;
    const int2 pend = *S.pend_in;
    if (!pend.x) return;
    psum_all(S, S.part_in, pend.y, const_cast<double *>(S.corr_in), red);
    __syncthreads();
    if (threadIdx.x == 0) *const_cast<int2 *>(S.pend_in) = make_int2(0, 0);
}

}  // namespace pairk

int sweep_finalize_launch(const SweepSolve *dsolve, cudaStream_t st) {
    pairk::k_sweep2_finalize<<<1, SWEEP_THREADS, 0, st>>>(dsolve);
    CSADV_CUDA(cudaGetLastError());
    return CSADV_OK;
}

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
