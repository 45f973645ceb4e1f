// tbl_reduce.cuh -- deterministic grid reductions (warp shuffle -> block ->
// last-arriving block sums the per-block partials in a fixed order).
// Replaces the reference's mpi_allreduce / mpi_reduce of one double
// (dnstbl2/dnstbl.f90:824, :1048, :1145, :1155, :1576, :1733).
#pragma once
#include "tbl_internal.cuh"

namespace tbl {

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <typename T>
__device__ __forceinline__ T warp_max(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Sum over the block; valid in thread 0.  smem must hold blockDim.x/32 values.
template <typename T>
__device__ __forceinline__ T block_sum(T v, T* smem) {
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nw = (blockDim.x + 31) >> 5;
    __syncthreads();
    if (lane == 0) smem[wid] = v;
    __syncthreads();
    T r = T(0);
    if (wid == 0) {
        r = lane < nw ? smem[lane] : T(0);
        r = warp_sum(r);
    }
    return r;
}

// Publishes this block's partial of reduction `slot`; the last block to arrive
// sums all partials (in block order) and writes the total to *out (if op==0),
// sqrt(total) (op==1).  Returns true in the finishing block.
__device__ __forceinline__ bool grid_finish(double block_total, RedWork rw, int slot, int nblocks,
                                            int block_id, double* out, int op) {
    __shared__ bool s_last;
    __shared__ double s_red[32];
    if (threadIdx.x == 0) {
        rw.partial[(size_t)slot * rw.max_blocks + block_id] = block_total;
        __threadfence();
        unsigned int t = atomicAdd(&rw.count[slot], 1u);
        s_last = (t == (unsigned)nblocks - 1);
    }
    __syncthreads();
    if (!s_last) return false;
    __threadfence();
    double acc = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x)
        acc += __ldcg(&rw.partial[(size_t)slot * rw.max_blocks + b]);
    acc = block_sum(acc, s_red);
    if (threadIdx.x == 0) {
        *out = op == 1 ? sqrt(acc) : acc;
        rw.count[slot] = 0u;
    }
    return true;
}

}  // namespace tbl
