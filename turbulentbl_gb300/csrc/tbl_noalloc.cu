// tbl_noalloc.cu -- the divergence diagnostic for callers that cannot
// allocate device memory.
//
// Some callers of this library cannot call cudaMalloc: a host code that owns
// all device memory through its own pool allocator (and must account for
// every byte), or one that calls us from inside its own time loop where an
// allocation could synchronise the device or fail once its pool has carved up
// the GPU.  tbl_div_diag_noalloc gives such callers the divergence printout of
// the reference time loop for velocity fields they already hold on the
// device.  Its only scratch is a fixed array that is part of the library
// image: every GPU that loads the library holds those TBL_NOALLOC_BLOCKS
// doubles (32 KB) until the process exits.  The call allocates nothing and
// calls no allocating library routine.
//
// Set-up: every call looks up the device address of the scratch array and of
// its arrival counter with cudaGetSymbolAddress, on the device that is current
// at call time, and checks the return code.  The lookup allocates nothing; on
// the first call on a device it also loads the library's kernels there, so
// make that first call before any stream capture.  The counter is zero when
// the library is loaded and every completed call returns it to zero, so no
// call needs to clear it.  All calls share the scratch array and it keeps the
// last call's partial sums; calls that overlap on the GPU (different streams,
// or different host threads) race on the scratch and give wrong results.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/tbl_gpu.h"

namespace {

constexpr int NA_THREADS = 256;
constexpr int NA_BLOCKS = TBL_NOALLOC_BLOCKS;

static __device__ __align__(256) double g_na_partial[NA_BLOCKS];
static __device__ __align__(256) unsigned int g_na_count;

__device__ __forceinline__ double na_warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ double na_block_sum(double v, double* smem) {
    v = na_warp_sum(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) smem[wid] = v;
    __syncthreads();
    double r = 0.0;
    if (wid == 0) r = na_warp_sum(lane < (int)(blockDim.x >> 5) ? smem[lane] : 0.0);
    return r;
}

// The 4th-order divergence sum of dnstbl2/dnstbl.f90:1526-1577 over the
// interior, fields in the reference layout (i fastest, no padding), divided by
// (nx-2)(ny-2)(nz-2) in absolute value; originalTBL prints the square root of
// that (originalTBL/fnldnstbl.f90:1586), selected by take_sqrt.  Partial sums
// go to the scratch array; the last block to arrive sums them in block order.
__global__ void __launch_bounds__(NA_THREADS) k_div_diag_static(int nx, int ny, int nz, double invdx, double invdy,
                                                               double invdxi, const double* __restrict__ U1,
                                                               const double* __restrict__ U2,
                                                               const double* __restrict__ U3,
                                                               const double* __restrict__ jacinv, double* partial,
                                                               unsigned int* count, int take_sqrt, double* out) {
    __shared__ double s_red[NA_THREADS / 32];
    __shared__ bool s_last;
    const int ni = nx - 2, J = ny - 2, nk = nz - 2;
    const long long n = (long long)ni * J * nk;
    const long long sy = nx, sz = (long long)nx * ny;
    const double c12 = 1.0 / 12.0;
    double acc = 0.0;
    for (long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x; t0 < n;
         t0 += (long long)gridDim.x * blockDim.x) {
        const int i = 1 + (int)(t0 % ni);
        const long long r = t0 / ni;
        const int j = 1 + (int)(r % J);
        const int k = 1 + (int)(r / J);
        const long long p = i + sy * j + sz * k;
        const int jm1 = j == 1 ? ny - 2 : j - 1, jp1 = j == ny - 2 ? 1 : j + 1;
        const int jm2 = j == 2 ? ny - 2 : jm1 - 1, jp2 = j == ny - 3 ? 1 : jp1 + 1;
        double d1, d2, d3;
        if (i == 1 || i == nx - 2) d1 = (U1[p + 1] - U1[p - 1]) * (0.5 * invdx);
        else d1 = ((U1[p - 2] - 8.0 * U1[p - 1] + 8.0 * U1[p + 1] - U1[p + 2]) * (c12 * invdx));
        const long long pj = i + sz * k;
        if (j == 1 || j == ny - 2) d2 = (U2[pj + sy * jp1] - U2[pj + sy * jm1]) * (0.5 * invdy);
        else
            d2 = ((U2[pj + sy * jm2] - 8.0 * U2[pj + sy * jm1] + 8.0 * U2[pj + sy * jp1] - U2[pj + sy * jp2]) *
                  (c12 * invdy));
        if (k <= 1 || k >= nz - 2) d3 = ((U3[p + sz] - U3[p - sz]) * (0.5 * invdxi));
        else d3 = ((U3[p - 2 * sz] - 8.0 * U3[p - sz] + 8.0 * U3[p + sz] - U3[p + 2 * sz]) * (c12 * invdxi));
        acc += (d1 + d2 + (d3 * jacinv[k]));
    }
    const double bt = na_block_sum(acc, s_red);
    if (threadIdx.x == 0) {
        partial[blockIdx.x] = bt;
        __threadfence();
        s_last = atomicAdd(count, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    double tot = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) tot += __ldcg(&partial[b]);
    tot = na_block_sum(tot, s_red);
    if (threadIdx.x == 0) {
        const double d = fabs(tot) / ((double)(ny - 2) * (nx - 2) * (nz - 2));
        *out = take_sqrt ? sqrt(d) : d;
        *count = 0u;  // ready for the next call
    }
}

// Device addresses of the scratch array and its counter on the current device.
int scratch_addresses(double** partial, unsigned int** count) {
    void* p = nullptr;
    void* c = nullptr;
    if (cudaGetSymbolAddress(&p, g_na_partial) != cudaSuccess) return TBL_ERR_CUDA;
    if (cudaGetSymbolAddress(&c, g_na_count) != cudaSuccess) return TBL_ERR_CUDA;
    *partial = static_cast<double*>(p);
    *count = static_cast<unsigned int*>(c);
    return TBL_OK;
}

}  // namespace

extern "C" int tbl_div_diag_noalloc(const tbl_config* cfg, const double* jacinv, const double* u, const double* v,
                                    const double* w, double* out) {
    if (!cfg || !jacinv || !u || !v || !w || !out) return TBL_ERR_BAD_ARG;
    if (cfg->nx < 5 || cfg->ny < 5 || cfg->nz < 5 || !(cfg->dx > 0) || !(cfg->dy > 0) || !(cfg->dxi > 0))
        return TBL_ERR_BAD_ARG;
    const long long n = (long long)(cfg->nx - 2) * (cfg->ny - 2) * (cfg->nz - 2);
    if (n > TBL_NOALLOC_MAX_POINTS) return TBL_ERR_TOO_LARGE;  // beyond what the fixed scratch is sized for
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return TBL_ERR_NO_DEVICE;
    double* partial = nullptr;
    unsigned int* count = nullptr;
    int s = scratch_addresses(&partial, &count);
    if (s != TBL_OK) return s;
    long long blocks = (n + (long long)NA_THREADS * 16 - 1) / ((long long)NA_THREADS * 16);
    if (blocks > NA_BLOCKS) blocks = NA_BLOCKS;
    if (blocks < 1) blocks = 1;
    k_div_diag_static<<<(unsigned)blocks, NA_THREADS>>>(cfg->nx, cfg->ny, cfg->nz, 1.0 / cfg->dx, 1.0 / cfg->dy,
                                                        1.0 / cfg->dxi, u, v, w, jacinv, partial, count,
                                                        cfg->variant == TBL_VARIANT_ORIGINAL ? 1 : 0, out);
    if (cudaGetLastError() != cudaSuccess) return TBL_ERR_CUDA;
    return TBL_OK;
}
