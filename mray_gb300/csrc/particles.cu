// SPH particles: the reference's uniform grid built on the device.
//
// Reference: Particles::create_grid (src/volume.cpp:55-81), createGridFromDomain (src/particle_grid.cuh:392-403,
// src/particle_grid.cpp:37-56), UniformGrid (src/particle_grid.cuh:284-306), getIndexFromCell (:64-83).  The grid
// has cell size h (the smoothing length), its origin at the particles' minimum and a 4x4x4-tiled cell order.  The
// reference sorts the particles by cell on the host (std::sort, cut/sort_util.h:38-41, whose order inside a
// cell is unspecified) and marks each cell's first particle, EMPTY_CELL elsewhere, counting a cell's particles by
// scanning forward to the next occupied cell.  Here:
//   1. min / max of the positions (per-block partials, one finishing block)
//   2. cell of every particle and per-cell counts (atomics on counts only: the counts are order-free)
//   3. exclusive scan of the counts -> the CSR array cell_start
//   4. a stable LSD radix sort of the cell keys (8-bit digits, as many passes as the cell count needs) with the
//      particle index as payload, so the order inside a cell is the input order on every run
//   5. a gather into float4 (x, y, z, value) records: one 16-byte load per particle in the sampler.
//
// Radix pass: each 256-thread block owns a tile of 4096 keys, each warp a contiguous run of 512.  Phase 1 counts
// the digits per warp; the per-(digit, block) totals are written digit-major and scanned, which gives every block
// the global start of each digit.  Phase 2 walks each warp's run again in order and ranks each key among the
// equal digits of its warp with __match_any_sync, so equal digits keep their input order (stable).

#include "device_common.cuh"
#include "internal.h"

namespace mraygb
{

namespace
{

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kRun = 512; // keys per warp and pass
constexpr int kTile = kWarps * kRun;
constexpr int kRadix = 256;

__global__ void minmax_partial_kernel(const float *__restrict__ x, const float *__restrict__ y,
                                      const float *__restrict__ z, uint64_t n, float *__restrict__ partial)
{
    __shared__ float s[6][kThreads];
    float mn[3] = {x[0], y[0], z[0]}, mx[3] = {x[0], y[0], z[0]};
    for (uint64_t i = (uint64_t)blockIdx.x * kThreads + threadIdx.x; i < n; i += (uint64_t)gridDim.x * kThreads)
    {
        const float q[3] = {x[i], y[i], z[i]};
#pragma unroll
        for (int k = 0; k < 3; ++k)
        {
            mn[k] = q[k] < mn[k] ? q[k] : mn[k];
            mx[k] = mx[k] < q[k] ? q[k] : mx[k];
        }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k)
    {
        s[k][threadIdx.x] = mn[k];
        s[3 + k][threadIdx.x] = mx[k];
    }
    __syncthreads();
    for (int w = kThreads / 2; w > 0; w >>= 1)
    {
        if (threadIdx.x < w)
        {
#pragma unroll
            for (int k = 0; k < 3; ++k)
            {
                const float a = s[k][threadIdx.x + w], b = s[3 + k][threadIdx.x + w];
                s[k][threadIdx.x] = a < s[k][threadIdx.x] ? a : s[k][threadIdx.x];
                s[3 + k][threadIdx.x] = s[3 + k][threadIdx.x] < b ? b : s[3 + k][threadIdx.x];
            }
        }
        __syncthreads();
    }
    if (threadIdx.x < 6)
        partial[blockIdx.x * 6 + threadIdx.x] = s[threadIdx.x][0];
}

__global__ void minmax_final_kernel(const float *__restrict__ partial, int blocks, float *__restrict__ out)
{
    if (threadIdx.x >= 6)
        return;
    const int k = threadIdx.x;
    float v = partial[k];
    for (int b = 1; b < blocks; ++b)
    {
        const float a = partial[b * 6 + k];
        v = (k < 3) ? (a < v ? a : v) : (v < a ? a : v);
    }
    out[k] = v;
}

__global__ void cell_count_kernel(const float *__restrict__ x, const float *__restrict__ y,
                                  const float *__restrict__ z, uint64_t n, ParticleGridParams g,
                                  uint32_t *__restrict__ cell_of, uint32_t *__restrict__ counts)
{
    for (uint64_t i = (uint64_t)blockIdx.x * kThreads + threadIdx.x; i < n; i += (uint64_t)gridDim.x * kThreads)
    {
        const uint32_t c = particle_cell(g, x[i], y[i], z[i]);
        cell_of[i] = c;
        atomicAdd(counts + c, 1u);
    }
}

// phase 1 of a radix pass: digit counts of each block, written digit-major (hist[d * blocks + b])
__global__ void __launch_bounds__(kThreads) radix_count_kernel(const uint32_t *__restrict__ keys, uint32_t n,
                                                               int shift, uint32_t *__restrict__ hist)
{
    __shared__ uint32_t cnt[kRadix];
    for (int d = threadIdx.x; d < kRadix; d += kThreads)
        cnt[d] = 0;
    __syncthreads();
    const uint32_t base = blockIdx.x * kTile;
    for (int k = threadIdx.x; k < kTile; k += kThreads)
    {
        const uint32_t i = base + k;
        if (i < n)
            atomicAdd(&cnt[(keys[i] >> shift) & (kRadix - 1)], 1u);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < kRadix; d += kThreads)
        hist[(size_t)d * gridDim.x + blockIdx.x] = cnt[d];
}

// phase 2: stable scatter.  offsets = the exclusive scan of hist.
__global__ void __launch_bounds__(kThreads)
    radix_scatter_kernel(const uint32_t *__restrict__ keys, const uint32_t *__restrict__ vals, uint32_t n, int shift,
                         const uint32_t *__restrict__ offsets, uint32_t *__restrict__ keys_out,
                         uint32_t *__restrict__ vals_out)
{
    __shared__ uint32_t wcnt[kWarps][kRadix]; // per-warp digit counts, then per-warp running positions
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int d = lane; d < kRadix; d += 32)
        wcnt[warp][d] = 0;
    __syncwarp();
    const uint32_t run = blockIdx.x * kTile + warp * kRun;
    // counts of this warp's run
    for (int r = 0; r < kRun; r += 32)
    {
        const uint32_t i = run + r + lane;
        const bool ok = i < n;
        const uint32_t d = ok ? (keys[i] >> shift) & (kRadix - 1) : kRadix; // kRadix: no key
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        if (ok && lane == __ffs(peers) - 1)
            wcnt[warp][d] += __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    // start of each digit for each warp: the block's global start plus the counts of the warps before it
    for (int d = threadIdx.x; d < kRadix; d += kThreads)
    {
        uint32_t pos = offsets[(size_t)d * gridDim.x + blockIdx.x];
        for (int w = 0; w < kWarps; ++w)
        {
            const uint32_t c = wcnt[w][d];
            wcnt[w][d] = pos;
            pos += c;
        }
    }
    __syncthreads();
    const unsigned lt = (1u << lane) - 1u;
    for (int r = 0; r < kRun; r += 32)
    {
        const uint32_t i = run + r + lane;
        const bool ok = i < n;
        const uint32_t key = ok ? keys[i] : 0u;
        const uint32_t d = ok ? (key >> shift) & (kRadix - 1) : kRadix;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        if (ok)
        {
            const uint32_t dst = wcnt[warp][d] + __popc(peers & lt);
            keys_out[dst] = key;
            vals_out[dst] = vals ? vals[i] : i;
        }
        __syncwarp();
        if (ok && lane == __ffs(peers) - 1)
            wcnt[warp][d] += __popc(peers);
        __syncwarp();
    }
}

__global__ void gather_kernel(uint64_t n, const uint32_t *__restrict__ order, const float *__restrict__ x,
                              const float *__restrict__ y, const float *__restrict__ z, const float *__restrict__ v,
                              float4 *__restrict__ pts)
{
    for (uint64_t i = (uint64_t)blockIdx.x * kThreads + threadIdx.x; i < n; i += (uint64_t)gridDim.x * kThreads)
    {
        const uint32_t j = order[i];
        pts[i] = make_float4(x[j], y[j], z[j], v[j]);
    }
}

// per-particle smoothing lengths: the largest (its bits: h > 0, so the float order is the integer order) and a
// count of those that are not finite and > 0
__global__ void h_range_kernel(uint64_t n, const float *__restrict__ h, unsigned int *__restrict__ out2)
{
    unsigned int mx = 0, bad = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * kThreads + threadIdx.x; i < n; i += (uint64_t)gridDim.x * kThreads)
    {
        const float v = h[i];
        if (v > 0.f && v <= 3.402823466e38f)
            mx = max(mx, __float_as_uint(v));
        else
            ++bad;
    }
    mx = __reduce_max_sync(0xffffffffu, mx);
    bad = __reduce_add_sync(0xffffffffu, bad);
    if ((threadIdx.x & 31) == 0)
    {
        atomicMax(out2, mx);
        if (bad)
            atomicAdd(out2 + 1, bad);
    }
}

// (1 / h, 1 / h^3) of every record, in the records' (sorted) order
__global__ void gather_h_kernel(uint64_t n, const uint32_t *__restrict__ order, const float *__restrict__ h,
                                float2 *__restrict__ inv_h)
{
    for (uint64_t i = (uint64_t)blockIdx.x * kThreads + threadIdx.x; i < n; i += (uint64_t)gridDim.x * kThreads)
    {
        const float v = h[order[i]];
        inv_h[i] = make_float2(__fdiv_rn(1.f, v), __fdiv_rn(1.f, __fmul_rn(__fmul_rn(v, v), v)));
    }
}

unsigned grid_blocks(uint64_t n)
{
    const uint64_t b = (n + kThreads - 1) / kThreads;
    return (unsigned)(b < 152 * 32 ? (b > 0 ? b : 1) : 152 * 32);
}

uint32_t radix_blocks(uint32_t n) { return (n + kTile - 1) / kTile; }

// getNextMultiple (src/particle_grid.cuh:40-43)
uint32_t next_multiple(uint32_t x, int multiple) { return ((x - 1) / (uint32_t)multiple + 1) * (uint32_t)multiple; }

} // namespace

ParticleGridParams particle_grid_params(const float mn[3], const float mx[3], float h)
{
    ParticleGridParams g;
    uint32_t s[3];
    for (int k = 0; k < 3; ++k)
    {
        s[k] = (uint32_t)((mx[k] - mn[k]) / h + 1.0f); // static_cast<uint32_t>(cells + 1)
        g.gmin[k] = mn[k];
    }
    g.sx = (int)next_multiple(s[0], 4);
    g.sy = (int)next_multiple(s[1], 4);
    g.sz = s[2] > 1 ? (int)next_multiple(s[2], 4) : (int)s[2];
    g.tz = g.sz == 1 ? 1 : 4;
    g.inv_cell = (float)(1.0 / (double)h);
    g.r2 = h * h;
    g.inv_h = 1.f / h;
    g.total = (uint32_t)((uint64_t)g.sx * (uint64_t)g.sy * (uint64_t)g.sz);
    return g;
}

size_t particle_minmax_scratch_floats(uint64_t n) { return (size_t)grid_blocks(n) * 6 + 6; }

size_t particle_radix_hist_words(uint32_t n) { return (size_t)radix_blocks(n) * kRadix; }

cudaError_t launch_particle_minmax(const float *x, const float *y, const float *z, uint64_t n, float *scratch,
                                   float *out6, cudaStream_t stream)
{
    const unsigned blocks = grid_blocks(n);
    minmax_partial_kernel<<<blocks, kThreads, 0, stream>>>(x, y, z, n, scratch);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return e;
    minmax_final_kernel<<<1, 32, 0, stream>>>(scratch, (int)blocks, out6);
    return cudaGetLastError();
}

cudaError_t launch_particle_cells(const float *x, const float *y, const float *z, uint64_t n,
                                  const ParticleGridParams &g, uint32_t *cell_of, uint32_t *counts,
                                  cudaStream_t stream)
{
    cell_count_kernel<<<grid_blocks(n), kThreads, 0, stream>>>(x, y, z, n, g, cell_of, counts);
    return cudaGetLastError();
}

cudaError_t launch_particle_sort(uint32_t n, uint32_t total, uint32_t *keys, uint32_t *keys_alt, uint32_t *vals,
                                 uint32_t *vals_alt, uint32_t *hist, uint32_t *hist_scan, uint32_t *scan_scratch,
                                 uint32_t **sorted_vals, cudaStream_t stream, int *launches)
{
    int bits = 1;
    while (bits < 32 && ((uint64_t)1 << bits) < (uint64_t)total)
        ++bits;
    const int passes = (bits + 7) / 8;
    const uint32_t blocks = radix_blocks(n);
    const size_t hw = (size_t)blocks * kRadix;
    uint32_t *kin = keys, *kout = keys_alt, *vin = nullptr, *vout = vals;
    for (int p = 0; p < passes; ++p)
    {
        radix_count_kernel<<<blocks, kThreads, 0, stream>>>(kin, n, 8 * p, hist);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess)
            return e;
        int sl = 0;
        e = launch_exclusive_scan(hist, hist_scan, hw, scan_scratch, stream, &sl);
        if (e != cudaSuccess)
            return e;
        radix_scatter_kernel<<<blocks, kThreads, 0, stream>>>(kin, vin, n, 8 * p, hist_scan, kout, vout);
        e = cudaGetLastError();
        if (e != cudaSuccess)
            return e;
        *launches += 2 + sl;
        // the output of this pass is the input of the next
        uint32_t *t = kin;
        kin = kout;
        kout = t;
        vin = vout;
        vout = (vout == vals) ? vals_alt : vals;
    }
    *sorted_vals = vin;
    return cudaSuccess;
}

cudaError_t launch_particle_h_range(uint64_t n, const float *h, unsigned int *out2, cudaStream_t stream)
{
    cudaError_t e = cudaMemsetAsync(out2, 0, 2 * sizeof(unsigned int), stream);
    if (e != cudaSuccess)
        return e;
    h_range_kernel<<<grid_blocks(n), kThreads, 0, stream>>>(n, h, out2);
    return cudaGetLastError();
}

cudaError_t launch_particle_gather_h(uint64_t n, const uint32_t *order, const float *h, float2 *inv_h,
                                     cudaStream_t stream)
{
    gather_h_kernel<<<grid_blocks(n), kThreads, 0, stream>>>(n, order, h, inv_h);
    return cudaGetLastError();
}

cudaError_t launch_particle_gather(uint64_t n, const uint32_t *order, const float *x, const float *y, const float *z,
                                   const float *v, float4 *pts, cudaStream_t stream)
{
    gather_kernel<<<grid_blocks(n), kThreads, 0, stream>>>(n, order, x, y, z, v, pts);
    return cudaGetLastError();
}

} // namespace mraygb
