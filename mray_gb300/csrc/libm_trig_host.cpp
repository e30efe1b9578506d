// Upload of the sinf / cosf exception table (libm_trig_core.h).  The table is generated at build time from the
// host C library (libm_trig_gen.cpp) and linked into this library as a read-only blob; each device gets one copy
// (about 7 MB) on the first context created there, kept until the process exits (contexts on the same device
// share it, so no context frees it).

#include <cstring>
#include <mutex>

#include "internal.h"
#include "libm_trig_core.h"

extern "C" {
extern const unsigned char mraygb_libm_trig_table_begin[] __attribute__((visibility("hidden")));
extern const unsigned char mraygb_libm_trig_table_end[] __attribute__((visibility("hidden")));
}

namespace mraygb
{

namespace
{

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
LibmTrigTable g_tables[kMaxDevices] = {};

} // namespace

cudaError_t libm_trig_device_table(LibmTrigTable *out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return e;
    if (dev < 0 || dev >= kMaxDevices)
        return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_tables[dev].offsets)
    {
        const size_t size = (size_t)(mraygb_libm_trig_table_end - mraygb_libm_trig_table_begin);
        libm_trig::Header h;
        if (size < sizeof h)
            return cudaErrorInvalidValue;
        std::memcpy(&h, mraygb_libm_trig_table_begin, sizeof h);
        const size_t off_bytes = ((size_t)h.n_buckets + 1) * sizeof(uint32_t);
        const size_t ent_bytes = (size_t)h.n_entries * sizeof(uint16_t);
        if (h.magic != libm_trig::kMagic || h.version != libm_trig::kVersion || h.shift != libm_trig::kShift ||
            h.n_buckets != libm_trig::kBuckets || h.max_abs_bits != libm_trig::kMaxAbsBits ||
            size != sizeof h + off_bytes + ent_bytes)
            return cudaErrorInvalidValue;
        void *d = nullptr;
        // the offsets, then the entries
        if ((e = cudaMalloc(&d, off_bytes + ent_bytes)) != cudaSuccess)
            return e;
        if ((e = cudaMemcpy(d, mraygb_libm_trig_table_begin + sizeof h, off_bytes + ent_bytes,
                            cudaMemcpyHostToDevice)) != cudaSuccess)
        {
            cudaFree(d);
            return e;
        }
        g_tables[dev].offsets = static_cast<const uint32_t *>(d);
        g_tables[dev].entries = reinterpret_cast<const uint16_t *>(static_cast<const char *>(d) + off_bytes);
    }
    *out = g_tables[dev];
    return cudaSuccess;
}

} // namespace mraygb
