// Allocation-free entry point: the divergence-projection mass fixer (MF-PR) on arrays
// the caller owns, with its reduction scratch in a fixed file-scope device array.
//
// Why: a caller that cannot call cudaMalloc -- a long-running service that has committed
// its whole device-memory budget to resident solves up front, or a host program whose
// device memory all comes from another runtime's pool that it must not grow -- can still
// apply the mass fixer to a divergence it computed itself.  The plan-based entry points
// allocate their scratch (block partial sums) when a plan is created; this one needs no
// plan and allocates nothing.
//
// The scratch lives in g_noalloc_scratch below (98 KB per device, held by every GPU that
// loads the library until the process exits).  Host code must not pass the symbol itself
// to a kernel (on the host it is only a stand-in for the device address); its device
// address is looked up once per device with cudaGetSymbolAddress, with that device
// current, by the first call made on the device.  That first call should therefore come
// before any stream capture.  The remembered address belongs to the device's primary
// context: after cudaDeviceReset it is stale, and the entry point must not be called again
// in that process.  Every call uses the same scratch: calls whose work overlaps
// on the GPU (different streams without ordering) race and give wrong results.  Each call
// writes every scratch slot it reads before reading it, so nothing carries over from the
// previous call.
#include <mutex>

#include "../../include/csadv.h"
#include "common.cuh"
#include "internal.h"

namespace csadv {

constexpr int NA_THREADS = 256;                 // threads per block
constexpr int NA_CHUNK = 4096;                  // interior cells reduced by one block
constexpr int NA_MAX_N = 2048;                  // largest cube size accepted
constexpr int NA_MAX_PARTIALS = (NFACE * NA_MAX_N * NA_MAX_N + NA_CHUNK - 1) / NA_CHUNK;  // 6144

// [0, MAXP): partial sums of div*g;  [MAXP, 2 MAXP): partial sums of g*g;  then m0, a2
static __device__ __align__(256) double g_noalloc_scratch[2 * NA_MAX_PARTIALS + 2];

namespace {

std::mutex g_na_mu;
double *g_na_ptr[64] = {};

// device address of the scratch array on the current device (set up once per device)
int noalloc_scratch(double **out) {
    int dev = 0;
    CSADV_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return CSADV_ERR_ARG;
    std::lock_guard<std::mutex> lock(g_na_mu);
    if (!g_na_ptr[dev]) {
        void *p = nullptr;
        CSADV_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_na_ptr[dev] = (double *)p;
    }
    *out = g_na_ptr[dev];
    return CSADV_OK;
}

// interior cell t (reference layout order: i, j, then panel fastest) -> array offset
__device__ __forceinline__ long long na_offset(int N, long long t) {
    const int n = N + 2 * NG;
    const int p = (int)(t % NFACE);
    const long long ij = t / NFACE;
    const int j = NG + (int)(ij % N), i = NG + (int)(ij / N);
    return ((long long)i * n + j) * NFACE + p;
}

__global__ void k_na_partials(const double *__restrict__ div, const double *__restrict__ g, int N,
                              double *scratch) {
    __shared__ double r0[NA_THREADS], r1[NA_THREADS];
    const long long total = (long long)NFACE * N * N;
    const long long begin = (long long)blockIdx.x * NA_CHUNK;
    double a = 0.0, b = 0.0;
    for (int k = threadIdx.x; k < NA_CHUNK; k += NA_THREADS) {
        const long long t = begin + k;
        if (t >= total) break;
        const long long o = na_offset(N, t);
        const double gv = g[o];
        a += div[o] * gv;
        b += gv * gv;
    }
    r0[threadIdx.x] = a;
    r1[threadIdx.x] = b;
    __syncthreads();
    for (int s = NA_THREADS / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            r0[threadIdx.x] += r0[threadIdx.x + s];
            r1[threadIdx.x] += r1[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        scratch[blockIdx.x] = r0[0];
        scratch[NA_MAX_PARTIALS + blockIdx.x] = r1[0];
    }
}

// fixed-order sums of the partials -> m0, a2 (one block)
__global__ void k_na_finalize(double *scratch, int nparts) {
    __shared__ double r0[NA_THREADS], r1[NA_THREADS];
    double a = 0.0, b = 0.0;
    for (int k = threadIdx.x; k < nparts; k += NA_THREADS) {
        a += scratch[k];
        b += scratch[NA_MAX_PARTIALS + k];
    }
    r0[threadIdx.x] = a;
    r1[threadIdx.x] = b;
    __syncthreads();
    for (int s = NA_THREADS / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            r0[threadIdx.x] += r0[threadIdx.x + s];
            r1[threadIdx.x] += r1[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        scratch[2 * NA_MAX_PARTIALS] = r0[0];
        scratch[2 * NA_MAX_PARTIALS + 1] = r1[0];
    }
}

// div_out = div_in - g m0 / a2 on the interior; other cells copied
__global__ void k_na_apply(const double *div, const double *__restrict__ g, double *out, int N,
                           const double *__restrict__ scratch) {
    const int n = N + 2 * NG;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)n * n * NFACE) return;
    const long long ij = t / NFACE;
    const int j = (int)(ij % n), i = (int)(ij / n);
    const bool in = i >= NG && i < NG + N && j >= NG && j < NG + N;
    const double m0 = scratch[2 * NA_MAX_PARTIALS], a2 = scratch[2 * NA_MAX_PARTIALS + 1];
    out[t] = in ? div[t] - g[t] * m0 / a2 : div[t];
}

}  // namespace
}  // namespace csadv

using namespace csadv;

extern "C" int csadv_mass_fixer_noalloc(const double *div_in, const double *metric, double *div_out, int N,
                                        void *stream) {
    if (!div_in || !metric || !div_out || N < 8) return CSADV_ERR_ARG;
    if (N > NA_MAX_N) return CSADV_ERR_TOO_LARGE;
    double *scratch = nullptr;
    int rc = noalloc_scratch(&scratch);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const long long cells = (long long)NFACE * N * N;
    const int nparts = (int)((cells + NA_CHUNK - 1) / NA_CHUNK);
    k_na_partials<<<nparts, NA_THREADS, 0, st>>>(div_in, metric, N, scratch);
    k_na_finalize<<<1, NA_THREADS, 0, st>>>(scratch, nparts);
    const long long n = N + 2 * NG;
    k_na_apply<<<ceil_div(n * n * NFACE, NA_THREADS), NA_THREADS, 0, st>>>(div_in, metric, div_out, N, scratch);
    CSADV_CUDA(cudaGetLastError());
    return CSADV_OK;
}
