// Moment-image compaction (MomentImageHost::compact, src/moment_image.cpp:69-94; MomentImageDevice::compact,
// src/moment_image_device.cu:83-110): exclusive scan of the per-pixel moment counts into the u32 index
// (W*H + 1 entries, the last one the total), then a copy of each pixel's first n moments to index[p].
//
// The scan is the classic reduce / scan-of-sums / scan-and-add sequence over 2048-element tiles (recursing on
// the tile sums), so no kernel waits on another block.

#include "internal.h"

namespace mraygb
{

namespace
{

constexpr int kThreads = 256;
constexpr int kItems = 8;
constexpr int kTile = kThreads * kItems;

__device__ __forceinline__ uint32_t warp_inclusive_scan(uint32_t v, int lane)
{
#pragma unroll
    for (int d = 1; d < 32; d <<= 1)
    {
        uint32_t u = __shfl_up_sync(0xffffffffu, v, d);
        if (lane >= d)
            v += u;
    }
    return v;
}

// block-wide exclusive scan of one value per thread; returns the exclusive prefix, total in *total
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t *total)
{
    __shared__ uint32_t warp_sums[kThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t inc = warp_inclusive_scan(v, lane);
    if (lane == 31)
        warp_sums[warp] = inc;
    __syncthreads();
    if (warp == 0)
    {
        uint32_t s = lane < kThreads / 32 ? warp_sums[lane] : 0u;
        s = warp_inclusive_scan(s, lane);
        if (lane < kThreads / 32)
            warp_sums[lane] = s;
    }
    __syncthreads();
    const uint32_t warp_prefix = warp == 0 ? 0u : warp_sums[warp - 1];
    *total = warp_sums[kThreads / 32 - 1];
    return warp_prefix + inc - v;
}

__global__ void __launch_bounds__(kThreads) tile_reduce_kernel(const uint32_t *__restrict__ in, size_t n,
                                                               uint32_t *__restrict__ sums)
{
    const size_t base = (size_t)blockIdx.x * kTile;
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kItems; ++k)
    {
        const size_t i = base + (size_t)k * kThreads + threadIdx.x;
        if (i < n)
            s += in[i];
    }
    uint32_t total;
    block_exclusive_scan(s, &total);
    if (threadIdx.x == 0)
        sums[blockIdx.x] = total;
}

// exclusive scan of one tile plus its offset; the block holding the last element also writes out[n]
__global__ void __launch_bounds__(kThreads) tile_scan_kernel(const uint32_t *__restrict__ in, size_t n,
                                                             const uint32_t *__restrict__ offsets,
                                                             uint32_t *__restrict__ out)
{
    __shared__ uint32_t tile[kTile];
    const size_t base = (size_t)blockIdx.x * kTile;
#pragma unroll
    for (int k = 0; k < kItems; ++k)
    {
        const int li = k * kThreads + threadIdx.x;
        const size_t i = base + li;
        tile[li] = i < n ? in[i] : 0u;
    }
    __syncthreads();
    uint32_t v[kItems];
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kItems; ++k)
    {
        v[k] = tile[threadIdx.x * kItems + k];
        s += v[k];
    }
    uint32_t total;
    uint32_t prefix = block_exclusive_scan(s, &total);
    const uint32_t off = offsets ? offsets[blockIdx.x] : 0u;
    prefix += off;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kItems; ++k)
    {
        tile[threadIdx.x * kItems + k] = prefix;
        prefix += v[k];
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kItems; ++k)
    {
        const int li = k * kThreads + threadIdx.x;
        const size_t i = base + li;
        if (i < n)
            out[i] = tile[li];
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0)
        out[n] = off + total;
}

__global__ void compact_copy_kernel(size_t total, int m, const uint32_t *__restrict__ counts,
                                    const uint32_t *__restrict__ index, const float *__restrict__ moments,
                                    float *__restrict__ compact)
{
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x)
    {
        const size_t p = e / (size_t)m;
        const uint32_t j = (uint32_t)(e - p * (size_t)m);
        if (j < counts[p])
            compact[(size_t)index[p] + j] = moments[e];
    }
}

} // namespace

size_t scan_scratch_words(size_t n)
{
    const size_t nb = (n + kTile - 1) / kTile;
    if (nb <= 1)
        return 0;
    return nb + (nb + 1) + scan_scratch_words(nb);
}

cudaError_t launch_exclusive_scan(const uint32_t *counts, uint32_t *out, size_t n, uint32_t *scratch,
                                  cudaStream_t stream, int *launches)
{
    if (n == 0)
        return cudaMemsetAsync(out, 0, sizeof(uint32_t), stream);
    const size_t nb = (n + kTile - 1) / kTile;
    if (nb == 1)
    {
        tile_scan_kernel<<<1, kThreads, 0, stream>>>(counts, n, nullptr, out);
        if (launches)
            *launches += 1;
        return cudaGetLastError();
    }
    uint32_t *sums = scratch;
    uint32_t *offs = scratch + nb;
    tile_reduce_kernel<<<(unsigned)nb, kThreads, 0, stream>>>(counts, n, sums);
    if (launches)
        *launches += 1;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return e;
    e = launch_exclusive_scan(sums, offs, nb, scratch + nb + (nb + 1), stream, launches);
    if (e != cudaSuccess)
        return e;
    tile_scan_kernel<<<(unsigned)nb, kThreads, 0, stream>>>(counts, n, offs, out);
    if (launches)
        *launches += 1;
    return cudaGetLastError();
}

cudaError_t launch_compact_copy(int num_pixels, int m, const uint32_t *counts, const uint32_t *index,
                                const float *moments, float *compact, cudaStream_t stream)
{
    const size_t total = (size_t)num_pixels * (size_t)m;
    if (total == 0)
        return cudaSuccess;
    const int block = 256;
    size_t blocks = (total + block - 1) / block;
    if (blocks > 152 * 64)
        blocks = 152 * 64;
    compact_copy_kernel<<<(unsigned)blocks, block, 0, stream>>>(total, m, counts, index, moments, compact);
    return cudaGetLastError();
}

} // namespace mraygb
