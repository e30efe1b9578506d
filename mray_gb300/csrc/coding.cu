// Coding parameters, warp, quantization and bit packing of a prediction-coded moment image.  Integer / byte
// work: built without FMA contraction; every float operation is the reference's, so the codes and packed bytes
// are bit-identical to the reference's for the same prediction-coded floats.
//
//   find_coding_transform_parameters   src/coding_transform.h:37-68
//   CodingParamType::quantize          src/coding_params.h:56-66
//   transform_quantization_real_warp   src/moment_prediction_coding.h:72-76 (prediction_coding_warp :47-56)
//   quantize / dequantize              src/moment_quantization.cpp:37-66
//   quantize_prediction_coding         src/moment_quantization.cpp:239-276 with pack_bits :92-114
//   dequantize_prediction_coding       src/moment_quantization.cpp:278-332 with unpack_bits :135-160
//   quantize / dequantize (plain)      src/moment_quantization.cpp:340-407, fixed bits, [-1/pi, 1/pi]
//   entropy coder symbols              src/moment_image_coding.cpp:110-143
//
// Layout: one warp per pixel (lanes take the moment indices l = lane, lane + 32, ...), so reads of the compact
// moment buffer are coalesced.  Codes are OR-ed into a zeroed u32 word stream at their bit offsets (pixel
// offsets from an exclusive u64 scan of the per-pixel bit counts); a code touches at most two words.

#include "device_common.cuh"
#include "internal.h"

namespace mraygb
{

namespace
{

constexpr int kWarpsPerBlock = 8;
constexpr int kMaxSlots = 8; // (255 + 31) / 32

__device__ __forceinline__ float clampf(float v, float lo, float hi) { return rmin(rmax(v, lo), hi); }

// per-block partial min / max of clamp(data[idx + l], -1, 1) over the pixels with at least l moments; a pixel
// with exactly l moments contributes the value after its last one, as the reference's `num_moments < l` skip
// does (coding_transform.h:48-49), unless that is past the end of the buffer
__global__ void __launch_bounds__(kWarpsPerBlock * 32)
    coding_minmax_kernel(int num_pixels, int m, const uint32_t *__restrict__ index, const float *__restrict__ data,
                         uint64_t total, float2 *__restrict__ partial)
{
    __shared__ float s_min[kWarpsPerBlock][256];
    __shared__ float s_max[kWarpsPerBlock][256];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float vmin[kMaxSlots], vmax[kMaxSlots];
#pragma unroll
    for (int k = 0; k < kMaxSlots; ++k)
    {
        vmin[k] = 0.f;
        vmax[k] = 0.f;
    }
    const int gw = blockIdx.x * kWarpsPerBlock + warp;
    const int nw = gridDim.x * kWarpsPerBlock;
    for (int p = gw; p < num_pixels; p += nw)
    {
        const size_t idx = index[p];
        const int n = (int)(index[p + 1] - index[p]);
        const int lmax = n < m - 1 ? n : m - 1;
#pragma unroll
        for (int k = 0; k < kMaxSlots; ++k)
        {
            const int l = 1 + lane + 32 * k;
            if (l <= lmax && (uint64_t)(idx + l) < total)
            {
                const float v = clampf(data[idx + l], -1.f, 1.f);
                vmin[k] = (v < vmin[k]) ? v : vmin[k]; // std::min(params, value)
                vmax[k] = (vmax[k] < v) ? v : vmax[k]; // std::max(params, value)
            }
        }
    }
#pragma unroll
    for (int k = 0; k < kMaxSlots; ++k)
    {
        const int slot = lane + 32 * k; // l - 1
        if (slot < 256)
        {
            s_min[warp][slot] = vmin[k];
            s_max[warp][slot] = vmax[k];
        }
    }
    __syncthreads();
    for (int slot = threadIdx.x; slot < m - 1; slot += blockDim.x)
    {
        float a = 0.f, b = 0.f;
        for (int w = 0; w < kWarpsPerBlock; ++w)
        {
            const float x = s_min[w][slot], y = s_max[w][slot];
            a = (x < a) ? x : a;
            b = (b < y) ? y : b;
        }
        partial[(size_t)blockIdx.x * (m - 1) + slot] = make_float2(a, b);
    }
}

// reduce the partials, form (|min|, |max - min| / 2), quantize to u16 by ceil and dequantize for the warp
__global__ void coding_params_kernel(int blocks, int m, const float2 *__restrict__ partial,
                                     uint16_t *__restrict__ params_u16, float *__restrict__ params_f)
{
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= m - 1)
        return;
    float a = 0.f, b = 0.f;
    for (int i = 0; i < blocks; ++i)
    {
        const float2 v = partial[(size_t)i * (m - 1) + slot];
        a = (v.x < a) ? v.x : a;
        b = (b < v.y) ? v.y : b;
    }
    const float d = b - a;
    const float p2 = ((d < 0.f) ? -d : d) * 0.5f;
    const float p1 = (a < 0.f) ? -a : a;
    const uint16_t q1 = (uint16_t)ceilf(clampf(p1, 0.f, 1.f) * 65535.f);
    const uint16_t q2 = (uint16_t)ceilf(clampf(p2, 0.f, 1.f) * 65535.f);
    params_u16[2 * slot] = q1;
    params_u16[2 * slot + 1] = q2;
    params_f[2 * slot] = q1 / 65535.f;
    params_f[2 * slot + 1] = q2 / 65535.f;
}

__global__ void __launch_bounds__(kWarpsPerBlock * 32)
    coding_warp_kernel(int num_pixels, const uint32_t *__restrict__ index, float *__restrict__ data, int warp_type,
                       const float *__restrict__ params)
{
    const int lane = threadIdx.x & 31;
    const int gw = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    const int nw = gridDim.x * kWarpsPerBlock;
    for (int p = gw; p < num_pixels; p += nw)
    {
        const size_t idx = index[p];
        const int n = (int)(index[p + 1] - index[p]);
        for (int l = 1 + lane; l < n; l += 32)
        {
            const float x = data[idx + l];
            float w;
            if (warp_type == MRAYGB_CODING_WARP_DEFAULT_TRANSFORMED)
                w = (x + params[(l - 1) * 2]) / (params[(l - 1) * 2 + 1] * 2.f);
            else
                w = x * 0.5f + 0.5f;
            data[idx + l] = clampf(w, 0.f, 1.f);
        }
    }
}

// quantize(value, bits, lo, hi) / dequantize (src/moment_quantization.cpp:37-66); prediction codes use [0, 1],
// the plain quantizer [0, 1] for the zeroth moment and [-1/pi, 1/pi] for the others
__device__ __forceinline__ uint32_t quantize_code(float value, int bits, float lo = 0.f, float hi = 1.f)
{
    value = clampf(value, lo, hi);
    if (bits == 32)
        return __float_as_uint(value);
    const float norm = (value - lo) / (hi - lo);
    const uint32_t q = (uint32_t)(norm * (float)((1 << bits) - 1));
    return q & (uint32_t)((1u << bits) - 1u);
}

__device__ __forceinline__ float dequantize_code(uint32_t q, int bits, float lo = 0.f, float hi = 1.f)
{
    if (bits == 32)
        return clampf(__uint_as_float(q), lo, hi);
    const float norm = (float)q / (float)((1 << bits) - 1);
    return norm * (hi - lo) + lo;
}

__global__ void pixel_bits_kernel(int num_pixels, const uint32_t *__restrict__ index,
                                  const uint32_t *__restrict__ prefix_bits, unsigned long long *__restrict__ bits)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= num_pixels)
        return;
    bits[p] = prefix_bits[index[p + 1] - index[p]];
}

__global__ void __launch_bounds__(kWarpsPerBlock * 32)
    pack_kernel(int num_pixels, const uint32_t *__restrict__ index, const float *__restrict__ data,
                const uint8_t *__restrict__ table, const uint32_t *__restrict__ prefix_bits,
                const unsigned long long *__restrict__ bit_offset, float lo1, float hi1, uint32_t *__restrict__ words)
{
    const int lane = threadIdx.x & 31;
    const int gw = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    const int nw = gridDim.x * kWarpsPerBlock;
    for (int p = gw; p < num_pixels; p += nw)
    {
        const size_t idx = index[p];
        const int n = (int)(index[p + 1] - index[p]);
        const unsigned long long base = bit_offset[p];
        for (int l = lane; l < n; l += 32)
        {
            const int b = table[l];
            const uint32_t code = l ? quantize_code(data[idx + l], b, lo1, hi1) : quantize_code(data[idx], b);
            const unsigned long long pos = base + prefix_bits[l];
            const size_t w = (size_t)(pos >> 5);
            const int sh = (int)(pos & 31);
            atomicOr(words + w, code << sh);
            if (sh + b > 32)
                atomicOr(words + w + 1, code >> (32 - sh));
        }
    }
}

__global__ void __launch_bounds__(kWarpsPerBlock * 32)
    unpack_kernel(int num_pixels, const uint32_t *__restrict__ index, const uint8_t *__restrict__ table,
                  const uint32_t *__restrict__ prefix_bits, const unsigned long long *__restrict__ bit_offset,
                  const uint8_t *__restrict__ bytes, unsigned long long num_bytes, float lo1, float hi1,
                  float *__restrict__ data)
{
    const int lane = threadIdx.x & 31;
    const int gw = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    const int nw = gridDim.x * kWarpsPerBlock;
    const unsigned long long avail = num_bytes * 8ull;
    for (int p = gw; p < num_pixels; p += nw)
    {
        const size_t idx = index[p];
        const int n = (int)(index[p + 1] - index[p]);
        const unsigned long long base = bit_offset[p];
        for (int l = lane; l < n; l += 32)
        {
            const int b = table[l];
            const unsigned long long pos = base + prefix_bits[l];
            uint32_t q = 0;
            if (pos + (unsigned long long)b <= avail)
            {
                // gather up to five bytes around the code
                unsigned long long acc = 0;
                const unsigned long long first = pos >> 3;
                const int nbytes = (int)(((pos & 7) + b + 7) >> 3);
                for (int i = 0; i < nbytes; ++i)
                    acc |= (unsigned long long)bytes[first + i] << (8 * i);
                acc >>= (pos & 7);
                q = (uint32_t)(b == 32 ? acc : (acc & ((1ull << b) - 1ull)));
            }
            data[idx + l] = l ? dequantize_code(q, b, lo1, hi1) : dequantize_code(q, b);
        }
    }
}

// one u16 symbol per moment for the entropy coder, in the layout of the moment data: quantize(value, table[l], ...)
// with the ranges above (the zeroth moment's code is cast to u16 as the reference stores it)
__global__ void __launch_bounds__(kWarpsPerBlock * 32)
    symbols_kernel(int num_pixels, const uint32_t *__restrict__ index, const float *__restrict__ data,
                   const uint8_t *__restrict__ table, float lo1, float hi1, uint16_t *__restrict__ symbols)
{
    const int lane = threadIdx.x & 31;
    const int gw = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    const int nw = gridDim.x * kWarpsPerBlock;
    for (int p = gw; p < num_pixels; p += nw)
    {
        const size_t idx = index[p];
        const int n = (int)(index[p + 1] - index[p]);
        for (int l = lane; l < n; l += 32)
            symbols[idx + l] = (uint16_t)(l ? quantize_code(data[idx + l], table[l], lo1, hi1)
                                            : quantize_code(data[idx], table[0]));
    }
}

__global__ void __launch_bounds__(kWarpsPerBlock * 32)
    desymbols_kernel(int num_pixels, const uint32_t *__restrict__ index, const uint16_t *__restrict__ symbols,
                     const uint8_t *__restrict__ table, float lo1, float hi1, float *__restrict__ data)
{
    const int lane = threadIdx.x & 31;
    const int gw = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    const int nw = gridDim.x * kWarpsPerBlock;
    for (int p = gw; p < num_pixels; p += nw)
    {
        const size_t idx = index[p];
        const int n = (int)(index[p + 1] - index[p]);
        for (int l = lane; l < n; l += 32)
            data[idx + l] = l ? dequantize_code(symbols[idx + l], table[l], lo1, hi1)
                              : dequantize_code(symbols[idx], table[0]);
    }
}

// the byte-aligned quantizer of images without compaction (quantize(moments, m, bits), moment_quantization.cpp:
// 464-485 with append :409-433): value i of the W*H*m array as (bits + 7) / 8 little-endian bytes
__global__ void static_quantize_kernel(size_t count, int m, const float *__restrict__ data, int bits, int nbytes,
                                       float lo1, float hi1, uint8_t *__restrict__ out)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x)
    {
        const uint32_t q = (i % (size_t)m) ? quantize_code(data[i], bits, lo1, hi1) : quantize_code(data[i], bits);
        for (int k = 0; k < nbytes; ++k)
            out[i * (size_t)nbytes + k] = (uint8_t)(q >> (8 * k));
    }
}

int grid_for(int num_pixels)
{
    int blocks = (num_pixels + kWarpsPerBlock - 1) / kWarpsPerBlock;
    return blocks < 152 * 16 ? (blocks > 0 ? blocks : 1) : 152 * 16;
}

} // namespace

int coding_minmax_blocks(int num_pixels) { return grid_for(num_pixels); }

cudaError_t launch_coding_params(int num_pixels, int m, const uint32_t *index, const float *data, uint64_t total,
                                 float2 *partial, uint16_t *params_u16, float *params_f, cudaStream_t stream)
{
    const int blocks = grid_for(num_pixels);
    coding_minmax_kernel<<<blocks, kWarpsPerBlock * 32, 0, stream>>>(num_pixels, m, index, data, total, partial);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return e;
    coding_params_kernel<<<(m - 1 + 127) / 128, 128, 0, stream>>>(blocks, m, partial, params_u16, params_f);
    return cudaGetLastError();
}

cudaError_t launch_coding_warp(int num_pixels, const uint32_t *index, float *data, int warp_type,
                               const float *params, cudaStream_t stream)
{
    coding_warp_kernel<<<grid_for(num_pixels), kWarpsPerBlock * 32, 0, stream>>>(num_pixels, index, data, warp_type,
                                                                                   params);
    return cudaGetLastError();
}

cudaError_t launch_pixel_bits(int num_pixels, const uint32_t *index, const uint32_t *prefix_bits,
                              unsigned long long *bits, cudaStream_t stream)
{
    pixel_bits_kernel<<<(num_pixels + 255) / 256, 256, 0, stream>>>(num_pixels, index, prefix_bits, bits);
    return cudaGetLastError();
}

cudaError_t launch_pack(int num_pixels, const uint32_t *index, const float *data, const uint8_t *table,
                        const uint32_t *prefix_bits, const unsigned long long *bit_offset, uint32_t *words,
                        cudaStream_t stream, float lo1, float hi1)
{
    pack_kernel<<<grid_for(num_pixels), kWarpsPerBlock * 32, 0, stream>>>(num_pixels, index, data, table, prefix_bits,
                                                                            bit_offset, lo1, hi1, words);
    return cudaGetLastError();
}

cudaError_t launch_unpack(int num_pixels, const uint32_t *index, const uint8_t *table, const uint32_t *prefix_bits,
                          const unsigned long long *bit_offset, const uint8_t *bytes, unsigned long long num_bytes,
                          float *data, cudaStream_t stream, float lo1, float hi1)
{
    unpack_kernel<<<grid_for(num_pixels), kWarpsPerBlock * 32, 0, stream>>>(num_pixels, index, table, prefix_bits,
                                                                              bit_offset, bytes, num_bytes, lo1, hi1,
                                                                              data);
    return cudaGetLastError();
}

cudaError_t launch_symbols(int num_pixels, const uint32_t *index, const float *data, const uint8_t *table, float lo1,
                           float hi1, uint16_t *symbols, cudaStream_t stream)
{
    symbols_kernel<<<grid_for(num_pixels), kWarpsPerBlock * 32, 0, stream>>>(num_pixels, index, data, table, lo1, hi1,
                                                                               symbols);
    return cudaGetLastError();
}

cudaError_t launch_desymbols(int num_pixels, const uint32_t *index, const uint16_t *symbols, const uint8_t *table,
                             float lo1, float hi1, float *data, cudaStream_t stream)
{
    desymbols_kernel<<<grid_for(num_pixels), kWarpsPerBlock * 32, 0, stream>>>(num_pixels, index, symbols, table, lo1,
                                                                                 hi1, data);
    return cudaGetLastError();
}

cudaError_t launch_static_quantize(size_t count, int m, const float *data, int bits, float lo1, float hi1,
                                   uint8_t *out, cudaStream_t stream)
{
    const size_t want = (count + 255) / 256;
    const int blocks = (int)(want < 152 * 16 ? (want ? want : 1) : 152 * 16);
    static_quantize_kernel<<<blocks, 256, 0, stream>>>(count, m, data, bits, (bits + 7) / 8, lo1, hi1, out);
    return cudaGetLastError();
}

} // namespace mraygb
