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

template <typename T> __device__ __forceinline__ T warp_inclusive_scan(T v, int lane)
{
#pragma unroll
    for (int d = 1; d < 32; d <<= 1)
    {
        T u = __shfl_up_sync(0xffffffffu, v, d);
        if (lane >= d)
            v += u;
    }
    return v;
}

// block-wide exclusive scan of one value per thread; returns the exclusive prefix, total in *total
template <typename T> __device__ __forceinline__ T block_exclusive_scan(T v, T *total)
{
    __shared__ T warp_sums[kThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const T inc = warp_inclusive_scan<T>(v, lane);
    if (lane == 31)
        warp_sums[warp] = inc;
    __syncthreads();
    if (warp == 0)
    {
        T s = lane < kThreads / 32 ? warp_sums[lane] : T(0);
        s = warp_inclusive_scan<T>(s, lane);
        if (lane < kThreads / 32)
            warp_sums[lane] = s;
    }
    __syncthreads();
    const T warp_prefix = warp == 0 ? T(0) : warp_sums[warp - 1];
    *total = warp_sums[kThreads / 32 - 1];
    return warp_prefix + inc - v;
}

template <typename T>
__global__ void __launch_bounds__(kThreads) tile_reduce_kernel(const T *__restrict__ in, size_t n,
                                                               T *__restrict__ sums)
{
    const size_t base = (size_t)blockIdx.x * kTile;
    T s = 0;
#pragma unroll
    for (int k = 0; k < kItems; ++k)
    {
        const size_t i = base + (size_t)k * kThreads + threadIdx.x;
        if (i < n)
            s += in[i];
    }
    T total;
    block_exclusive_scan<T>(s, &total);
    if (threadIdx.x == 0)
        sums[blockIdx.x] = total;
}

// exclusive scan of one tile plus its offset; the block holding the last element also writes out[n]
template <typename T>
__global__ void __launch_bounds__(kThreads) tile_scan_kernel(const T *__restrict__ in, size_t n,
                                                             const T *__restrict__ offsets, T *__restrict__ out)
{
    __shared__ T tile[kTile];
    const size_t base = (size_t)blockIdx.x * kTile;
#pragma unroll
    for (int k = 0; k < kItems; ++k)
    {
        const int li = k * kThreads + threadIdx.x;
        const size_t i = base + li;
        tile[li] = i < n ? in[i] : T(0);
    }
    __syncthreads();
    T v[kItems];
    T s = 0;
#pragma unroll
    for (int k = 0; k < kItems; ++k)
    {
        v[k] = tile[threadIdx.x * kItems + k];
        s += v[k];
    }
    T total;
    T prefix = block_exclusive_scan<T>(s, &total);
    const T off = offsets ? offsets[blockIdx.x] : T(0);
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

// m a multiple of 4, W*H*m < 2^32 (the u32 moment index) and both buffers 16-byte aligned: four consecutive moments
// of one pixel per thread, one 16-byte load, a 32-bit division for the pixel, a 16-byte store where the
// destination element is aligned
__global__ void compact_copy4_kernel(uint32_t total4, uint32_t m, const uint32_t *__restrict__ counts,
                                     const uint32_t *__restrict__ index, const float4 *__restrict__ moments,
                                     float *__restrict__ compact)
{
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < total4; q += gridDim.x * blockDim.x)
    {
        const uint32_t e = q * 4u;
        const uint32_t p = e / m;
        const uint32_t j = e - p * m;
        const uint32_t n = counts[p];
        if (j >= n)
            continue;
        const float4 v = moments[q];
        const size_t d = (size_t)index[p] + j;
        if (j + 4u <= n && (d & 3u) == 0)
            *reinterpret_cast<float4 *>(compact + d) = v;
        else
        {
            compact[d] = v.x;
            if (j + 1u < n)
                compact[d + 1] = v.y;
            if (j + 2u < n)
                compact[d + 2] = v.z;
            if (j + 3u < n)
                compact[d + 3] = v.w;
        }
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

template <typename T>
cudaError_t exclusive_scan_t(const T *counts, T *out, size_t n, T *scratch, cudaStream_t stream, int *launches)
{
    if (n == 0)
        return cudaMemsetAsync(out, 0, sizeof(T), stream);
    const size_t nb = (n + kTile - 1) / kTile;
    if (nb == 1)
    {
        tile_scan_kernel<T><<<1, kThreads, 0, stream>>>(counts, n, nullptr, out);
        if (launches)
            *launches += 1;
        return cudaGetLastError();
    }
    T *sums = scratch;
    T *offs = scratch + nb;
    tile_reduce_kernel<T><<<(unsigned)nb, kThreads, 0, stream>>>(counts, n, sums);
    if (launches)
        *launches += 1;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return e;
    e = exclusive_scan_t<T>(sums, offs, nb, scratch + nb + (nb + 1), stream, launches);
    if (e != cudaSuccess)
        return e;
    tile_scan_kernel<T><<<(unsigned)nb, kThreads, 0, stream>>>(counts, n, offs, out);
    if (launches)
        *launches += 1;
    return cudaGetLastError();
}

cudaError_t launch_exclusive_scan(const uint32_t *counts, uint32_t *out, size_t n, uint32_t *scratch,
                                  cudaStream_t stream, int *launches)
{
    return exclusive_scan_t<uint32_t>(counts, out, n, scratch, stream, launches);
}

cudaError_t launch_exclusive_scan_u64(const unsigned long long *in, unsigned long long *out, size_t n,
                                      unsigned long long *scratch, cudaStream_t stream, int *launches)
{
    return exclusive_scan_t<unsigned long long>(in, out, n, scratch, stream, launches);
}

cudaError_t launch_compact_copy(int num_pixels, int m, const uint32_t *counts, const uint32_t *index,
                                const float *moments, float *compact, cudaStream_t stream)
{
    const size_t total = (size_t)num_pixels * (size_t)m;
    if (total == 0)
        return cudaSuccess;
    const int block = 256;
    if (m % 4 == 0 && total < (1ull << 32) && ((reinterpret_cast<uintptr_t>(moments) | reinterpret_cast<uintptr_t>(compact)) & 15u) == 0)
    {
        const size_t total4 = total / 4;
        size_t blocks = (total4 + block - 1) / block;
        if (blocks > 152 * 64)
            blocks = 152 * 64;
        compact_copy4_kernel<<<(unsigned)blocks, block, 0, stream>>>(
            (uint32_t)total4, (uint32_t)m, counts, index, reinterpret_cast<const float4 *>(moments), compact);
        return cudaGetLastError();
    }
    size_t blocks = (total + block - 1) / block;
    if (blocks > 152 * 64)
        blocks = 152 * 64;
    compact_copy_kernel<<<(unsigned)blocks, block, 0, stream>>>(total, m, counts, index, moments, compact);
    return cudaGetLastError();
}

} // namespace mraygb
