// The FP64 form of the Lagrange-multiplier preparation (MRAYGB_PRECISION_COMPENSATED_FP64_MESE): the kernels of
// mese_kernels.cuh instantiated for double, in a translation unit compiled with FMA contraction.
#include "mese_kernels.cuh"

namespace mraygb
{

cudaError_t mese_f64_init_constants(const LibmTrigTable &trig)
{
    cudaError_t e = set_libm_trig_constants(trig);
    return e != cudaSuccess ? e : init_tables();
}

cudaError_t launch_prepare_f64(int num_pixels, int m, const uint32_t *index, const float *data, int prediction_code,
                               int coding_warp, const uint16_t *coding_params, float bias, float *pmoments,
                               cudaStream_t stream)
{
    return launch_prepare_m<double>(num_pixels, m, index, data, prediction_code, coding_warp, coding_params, bias,
                                    pmoments, stream);
}

} // namespace mraygb
