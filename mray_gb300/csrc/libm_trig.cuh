// Device sinf / cosf with the host C library's results (libm_trig_core.h): the core's double evaluation, then the
// correction of the exception table, which the library uploads once per device (libm_trig_host.cpp).
// Internal linkage: every translation unit that includes this header holds its own constant copy of the table's
// address and sets it in its init function.
#pragma once

#include <cuda_runtime.h>

#include "internal.h"
#include "libm_trig_core.h"

namespace mraygb
{
namespace
{

__constant__ LibmTrigTable c_libm_trig;

inline cudaError_t set_libm_trig_constants(const LibmTrigTable &t)
{
    return cudaMemcpyToSymbol(c_libm_trig, &t, sizeof t);
}

__device__ __forceinline__ void libm_sincosf(float x, float *s, float *c)
{
    const uint32_t bits = __float_as_uint(x);
    if (!libm_trig::in_domain(bits))
    {
        double sd, cd;
        sincos((double)x, &sd, &cd);
        *s = (float)sd;
        *c = (float)cd;
        return;
    }
    float cs, cc;
    libm_trig::core_sincosf(x, cs, cc);
    uint32_t sb = __float_as_uint(cs), cb = __float_as_uint(cc);
    const LibmTrigTable t = c_libm_trig;
    // mraygb_create fails when the table cannot be set, so the address is never null once a context exists
    if (t.offsets)
        libm_trig::apply_entry(libm_trig::find_entry(t.offsets, t.entries, bits), sb, cb);
    *s = __uint_as_float(sb);
    *c = __uint_as_float(cb);
}

} // namespace
} // namespace mraygb
