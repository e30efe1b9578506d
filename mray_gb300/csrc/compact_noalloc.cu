// Moment-image compaction that allocates nothing (mraygb_stage_compact_noalloc, include/mraygb.h).
//
// Some callers cannot allocate device memory when they compact a frame: renderers and services that reserve
// all device memory up front in their own pool or arena and forbid cudaMalloc / cudaFree afterwards (an
// allocation there can stall every stream on the device, fail under the pool's budget, or fragment memory
// that the pool manages).  mraygb_stage_compact needs a context, and a context allocates its work buffers on
// demand.  This entry point needs no context: the scan's block sums live in the file-scope device array below,
// which every GPU that loads the library holds until the process exits.
//
// The array is reached from the host through cudaGetSymbolAddress, once per device, with that device current
// (the host-side name of a __device__ array is only a stand-in, not a device address).  The first call on a
// device does that set-up and the address is kept for the process: it belongs to the device's primary context,
// so it is not valid after cudaDeviceReset or under another driver context on the same device.  Each call reads
// the compact size back and waits for its stream, so no call can be captured into a CUDA graph.  All calls share the one array and the scan overwrites every word it reads, so no
// clearing is needed; two calls that overlap on the GPU (different streams, or different host threads on the
// same device) race on the array and must be ordered by the caller.

#include "../../include/mraygb.h"

#include <mutex>

#include "internal.h"

namespace
{

// largest image: 2^24 pixels (4096 x 4096); the scan of that many counts needs scan_scratch_words(2^24) = 16394
// words of block sums
constexpr size_t kNoAllocMaxPixels = size_t(1) << 24;
constexpr size_t kNoAllocScratchWords = 16448;

static __device__ __align__(256) uint32_t g_noalloc_scan_scratch[kNoAllocScratchWords];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
uint32_t *g_scratch_ptr[kMaxDevices] = {};

// device address of the scratch array on the current device (set up on first use)
int scratch_for_current_device(uint32_t **out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return MRAYGB_CUDA_ERROR;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[dev])
    {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scan_scratch) != cudaSuccess || !p)
        {
            cudaGetLastError();
            return MRAYGB_CUDA_ERROR;
        }
        g_scratch_ptr[dev] = static_cast<uint32_t *>(p);
    }
    *out = g_scratch_ptr[dev];
    return MRAYGB_OK;
}

} // namespace

extern "C" int mraygb_stage_compact_noalloc(void *stream, int width, int height, int num_moments,
                                            const uint32_t *d_counts, const float *d_moments, uint32_t *d_index,
                                            float *d_compact, uint64_t capacity, uint64_t *h_total)
{
    if (width <= 0 || height <= 0 || num_moments < 1 || num_moments > MRAYGB_MAX_MOMENTS || !d_counts ||
        !d_moments || !d_index || !d_compact || !h_total)
        return MRAYGB_INVALID_ARGUMENT;
    const size_t P = (size_t)width * (size_t)height;
    if (P > kNoAllocMaxPixels || mraygb::scan_scratch_words(P) > kNoAllocScratchWords)
        return MRAYGB_INVALID_ARGUMENT;
    if ((uint64_t)P * (uint64_t)num_moments >= (1ull << 32))
        return MRAYGB_INVALID_ARGUMENT;
    uint32_t *scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc != MRAYGB_OK)
        return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (mraygb::launch_exclusive_scan(d_counts, d_index, P, scratch, s, nullptr) != cudaSuccess)
        return MRAYGB_CUDA_ERROR;
    uint32_t total = 0;
    if (cudaMemcpyAsync(&total, d_index + P, sizeof(uint32_t), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return MRAYGB_CUDA_ERROR;
    if ((uint64_t)total > capacity)
        return MRAYGB_INVALID_ARGUMENT;
    if (mraygb::launch_compact_copy((int)P, num_moments, d_counts, d_index, d_moments, d_compact, s) != cudaSuccess)
        return MRAYGB_CUDA_ERROR;
    *h_total = total;
    return MRAYGB_OK;
}
