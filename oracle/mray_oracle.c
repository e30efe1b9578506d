/*
 * ORACLE — test infrastructure only.  CPU restatement of the reference (TobiasRp/mray) moment-image hot path,
 * used by tests/ to check the product and by bench.py as the timed CPU baseline.  Never linked into the product.
 *
 * Build: see oracle/Makefile (gcc -O2 -ffp-contract=off -fopenmp; contraction must stay off so that the f32
 * body reproduces the reference's separately rounded float operations on both x86-64 and aarch64).
 */
#define _GNU_SOURCE
#include "mray_oracle.h"

#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

#define ORACLE_MAX_MOMENTS 256

/* How the reference's CPU build evaluates the unqualified cos/sin of euler_exp (complex_algebra.h:155-158)
 * and exp(-tau) (raymarch_reconstruct.h:188): name lookup finds the C library's double functions, so the
 * float argument is widened and the double result rounded back to float.  Checked against the reference
 * build (tests/golden/make_golden.py writes the "euler_exp" fixture that pins it). */
void oracle_euler_exp_f32(float x, float out[2])
{
    out[0] = (float)cos((double)x);
    out[1] = (float)sin((double)x);
}
#define ORACLE_EXP_F32(v) ((float)exp((double)(v)))

/* cosf / sinf of transform_dequantization_real (moment_prediction_coding.h:103-104): the C library's (the
 * reference's CPU build) by default; the correctly rounded values (the double functions rounded to float) when
 * set, for checking a device implementation that rounds correctly operation by operation. */
static int oracle_rounded_trig = 0;
void oracle_set_rounded_trig(int on) { oracle_rounded_trig = on != 0; }

/* UniformGridDevice::getIndexFromCell (particle_grid.cuh:64-83): 4x4x4 tiles (4x4x1 for a flat grid) */
uint32_t oracle_particles_cell_index(const oracle_particles *p, int cx, int cy, int cz)
{
    const int tx = 4, ty = 4, tz = p->tz;
    int width_tiles = (p->sx + tx - 1) / tx;
    int height_tiles = (p->sy + ty - 1) / ty;
    int tile_x = cx / tx, tile_y = cy / ty, tile_z = cz / tz;
    int in_x = cx % tx, in_y = cy % ty, in_z = cz % tz;
    return (uint32_t)((tile_z * height_tiles * width_tiles + tile_y * width_tiles + tile_x) * (tx * ty * tz) +
                      in_z * tx * ty + in_y * tx + in_x);
}

/* f32: the reference's arithmetic */
#define R float
#define SFX f32
#define ORACLE_F32 1
#include "oracle_body.inc"
#undef R
#undef SFX
#undef ORACLE_F32

/* f64: the same method in double */
#define R double
#define SFX f64
#define ORACLE_F32 0
#include "oracle_body.inc"
#undef R
#undef SFX
#undef ORACLE_F32

/* -------------------------------------------------------------------------------------------------------------
 * SPH particle grid (Particles::create_grid, volume.cpp:55-81; createGridFromDomain, particle_grid.cuh:392-403,
 * particle_grid.cpp:37-56; UniformGrid, particle_grid.cuh:284-306)
 * ----------------------------------------------------------------------------------------------------------- */

static uint32_t next_multiple(uint32_t x, int multiple) { return ((x - 1) / (uint32_t)multiple + 1) * (uint32_t)multiple; }

typedef struct
{
    uint32_t cell;
    uint64_t index;
} cell_key;

static int cmp_cell_key(const void *a, const void *b)
{
    const cell_key *x = (const cell_key *)a, *y = (const cell_key *)b;
    if (x->cell != y->cell)
        return x->cell < y->cell ? -1 : 1;
    return x->index < y->index ? -1 : (x->index > y->index ? 1 : 0);
}

static oracle_particles *particles_build(const float *x, const float *y, const float *z, const float *v,
                                         const float *hs, uint64_t n, float h, const float dmin[3],
                                         const float dmax[3]);

oracle_particles *oracle_particles_create(const float *x, const float *y, const float *z, const float *v, uint64_t n,
                                          float h, const float dmin[3], const float dmax[3])
{
    return particles_build(x, y, z, v, NULL, n, h, dmin, dmax);
}

oracle_particles *oracle_particles_create_h(const float *x, const float *y, const float *z, const float *v,
                                            const float *hs, uint64_t n, const float dmin[3], const float dmax[3])
{
    if (n == 0 || !hs)
        return NULL;
    float h = hs[0];
    for (uint64_t i = 1; i < n; ++i)
        h = hs[i] > h ? hs[i] : h;
    return particles_build(x, y, z, v, hs, n, h, dmin, dmax);
}

static oracle_particles *particles_build(const float *x, const float *y, const float *z, const float *v,
                                         const float *hs, uint64_t n, float h, const float dmin[3],
                                         const float dmax[3])
{
    if (n == 0)
        return NULL;
    oracle_particles *P = (oracle_particles *)calloc(1, sizeof(oracle_particles));
    float mn[3] = {x[0], y[0], z[0]}, mx[3] = {x[0], y[0], z[0]};
    for (uint64_t i = 1; i < n; ++i)
    {
        const float q[3] = {x[i], y[i], z[i]};
        for (int k = 0; k < 3; ++k)
        {
            mn[k] = q[k] < mn[k] ? q[k] : mn[k]; /* std::min(min, x) */
            mx[k] = mx[k] < q[k] ? q[k] : mx[k]; /* std::max(max, x) */
        }
    }
    uint32_t g[3];
    for (int k = 0; k < 3; ++k)
        g[k] = (uint32_t)((mx[k] - mn[k]) / h + 1.0f);
    P->sx = (int)next_multiple(g[0], 4);
    P->sy = (int)next_multiple(g[1], 4);
    P->sz = g[2] > 1 ? (int)next_multiple(g[2], 4) : (int)g[2];
    P->tz = P->sz == 1 ? 1 : 4;
    for (int k = 0; k < 3; ++k)
    {
        P->gmin[k] = mn[k];
        P->dmin[k] = dmin[k];
        P->dmax[k] = dmax[k];
    }
    P->inv_cell = (float)(1.0 / (double)h);
    P->r2 = h * h;
    P->h = h;
    P->inv_h = 1.f / h;
    P->total = (uint32_t)P->sx * (uint32_t)P->sy * (uint32_t)P->sz;
    P->n = n;
    cell_key *keys = (cell_key *)malloc(sizeof(cell_key) * n);
    for (uint64_t i = 0; i < n; ++i)
    {
        int c[3];
        const float q[3] = {x[i], y[i], z[i]};
        const int sz[3] = {P->sx, P->sy, P->sz};
        for (int k = 0; k < 3; ++k)
        {
            c[k] = (int)((q[k] - P->gmin[k]) * P->inv_cell);
            /* the reference indexes out of its grid here when rounding lands on the padded edge; clamp */
            c[k] = c[k] < 0 ? 0 : (c[k] > sz[k] - 1 ? sz[k] - 1 : c[k]);
        }
        keys[i].cell = oracle_particles_cell_index(P, c[0], c[1], c[2]);
        keys[i].index = i;
    }
    qsort(keys, n, sizeof(cell_key), cmp_cell_key);
    P->x = (float *)malloc(sizeof(float) * n);
    P->y = (float *)malloc(sizeof(float) * n);
    P->z = (float *)malloc(sizeof(float) * n);
    P->v = (float *)malloc(sizeof(float) * n);
    P->hh = hs ? (float *)malloc(sizeof(float) * n) : NULL;
    P->cell_start = (uint32_t *)calloc((size_t)P->total + 1, sizeof(uint32_t));
    for (uint64_t i = 0; i < n; ++i)
    {
        const uint64_t j = keys[i].index;
        P->x[i] = x[j];
        P->y[i] = y[j];
        P->z[i] = z[j];
        P->v[i] = v[j];
        if (hs)
            P->hh[i] = hs[j];
        P->cell_start[keys[i].cell + 1] += 1;
    }
    for (uint32_t c = 0; c < P->total; ++c)
        P->cell_start[c + 1] += P->cell_start[c];
    free(keys);
    return P;
}

void oracle_particles_destroy(oracle_particles *P)
{
    if (!P)
        return;
    free(P->x);
    free(P->y);
    free(P->z);
    free(P->v);
    free(P->hh);
    free(P->cell_start);
    free(P);
}

/* -------------------------------------------------------------------------------------------------------------
 * Float-only container steps and integer / byte work
 * ----------------------------------------------------------------------------------------------------------- */

/* MomentImageHost::compact (moment_image.cpp:69-94) */
uint64_t oracle_compact(int width, int height, int m, const uint32_t *counts, const float *moments, uint32_t *index,
                        float *compact)
{
    uint32_t idx_sum = 0;
    for (int y = 0; y < height; ++y)
    {
        for (int x = 0; x < width; ++x)
        {
            size_t pix = (size_t)y * (size_t)width + (size_t)x;
            uint32_t num = counts[pix];
            index[pix] = idx_sum;
            const float *src = moments + pix * (size_t)m;
            if (compact)
                for (uint32_t l = 0; l < num; ++l)
                    compact[(size_t)idx_sum + l] = src[l];
            idx_sum += num;
        }
    }
    index[(size_t)height * (size_t)width] = idx_sum;
    return idx_sum;
}

static inline float clampf_ref(float v, float lo, float hi) { return rmin_f32(rmax_f32(v, lo), hi); }

/* find_coding_transform_parameters (coding_transform.h:37-68).  The reference skips a pixel only when its
 * moment count is < l, so a pixel with exactly l moments contributes data[idx + l], the next value in the
 * compact buffer.  Where that index is past the end of the buffer the reference reads out of bounds; here
 * the value is skipped. */
void oracle_find_coding_transform_parameters(int width, int height, int m, const uint32_t *index, const float *data,
                                             uint64_t data_size, float *params)
{
    for (int i = 0; i < 2 * (m - 1); ++i)
        params[i] = 0.0f;
    for (int l = 1; l < m; ++l)
    {
        float pmin = 0.0f, pmax = 0.0f;
        for (int y = 0; y < height; ++y)
        {
            for (int x = 0; x < width; ++x)
            {
                size_t idx;
                int n;
                pixel_span_f32(index, width, m, x, y, &idx, &n);
                if (n < l)
                    continue;
                if ((uint64_t)(idx + (size_t)l) >= data_size)
                    continue;
                float v = clampf_ref(data[idx + (size_t)l], -1.0f, 1.0f);
                pmin = (v < pmin) ? v : pmin; /* std::min(params, value) */
                pmax = (pmax < v) ? v : pmax; /* std::max(params, value) */
            }
        }
        params[(l - 1) * 2] = pmin;
        params[(l - 1) * 2 + 1] = pmax;
    }
    for (int p = 0; p < m - 1; ++p)
    {
        params[p * 2 + 1] = rabs_f32(params[p * 2 + 1] - params[p * 2]) * 0.5f;
        params[p * 2] = rabs_f32(params[p * 2]);
    }
}

/* CodingParamType::quantize (coding_params.h:56-66) */
void oracle_quantize_coding_params(int num_params, const float *params, uint16_t *q)
{
    for (int i = 0; i < num_params; ++i)
        q[i] = (uint16_t)ceilf(clampf_ref(params[i], 0.0f, 1.0f) * 65535.f);
}

/* MomentImageHost::prediction_encode (moment_image.cpp:96-152) */
void oracle_prediction_encode(int width, int height, int m, const uint32_t *index, float *data, uint64_t data_size,
                              int coding_warp, float bias, uint16_t *coding_params, const oracle_options *opt)
{
    int nthreads = (opt && opt->nthreads > 0) ? opt->nthreads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
    for (int y = 0; y < height; ++y)
    {
        cx_f32 e[ORACLE_MAX_MOMENTS], code[ORACLE_MAX_MOMENTS], poly[ORACLE_MAX_MOMENTS], tmp[ORACLE_MAX_MOMENTS];
        for (int x = 0; x < width; ++x)
        {
            size_t idx;
            int n;
            pixel_span_f32(index, width, m, x, y, &idx, &n);
            if (n <= 0)
                continue;
            float *d = data + idx;
            d[0] = (1 - bias) * d[0] + bias * 0.5f;
            for (int i = 1; i < n; ++i)
                d[i] = (1 - bias) * d[i] + bias * 0.0f;
            trig_to_exp_f32(n, e, d);
            encode_f32(n, e, code, poly, tmp);
            tq_real_f32(n, code, d[0], d);
        }
    }

    float params[2 * ORACLE_MAX_MOMENTS];
    if (coding_warp == MRAYGB_CODING_WARP_DEFAULT_TRANSFORMED)
    {
        float raw[2 * ORACLE_MAX_MOMENTS];
        uint16_t q[2 * ORACLE_MAX_MOMENTS];
        oracle_find_coding_transform_parameters(width, height, m, index, data, data_size, raw);
        oracle_quantize_coding_params(2 * (m - 1), raw, q);
        for (int i = 0; i < 2 * (m - 1); ++i)
        {
            if (coding_params)
                coding_params[i] = q[i];
            params[i] = q[i] / 65535.f;
        }
    }

#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
    for (int y = 0; y < height; ++y)
    {
        for (int x = 0; x < width; ++x)
        {
            size_t idx;
            int n;
            pixel_span_f32(index, width, m, x, y, &idx, &n);
            if (n <= 0)
                continue;
            for (int l = 1; l < n; ++l)
                data[idx + l] = pc_warp_f32(l, data[idx + l], coding_warp, params);
        }
    }
}

/* quantize (moment_quantization.cpp:37-53) */
uint32_t oracle_quantize(float value, int num_bits, float vmin, float vmax)
{
    if (num_bits == 32)
    {
        value = clampf_ref(value, vmin, vmax);
        uint32_t u;
        memcpy(&u, &value, sizeof(float));
        return u;
    }
    value = clampf_ref(value, vmin, vmax);
    float norm = (value - vmin) / (vmax - vmin);
    uint32_t bits = (uint32_t)(norm * (float)((1 << num_bits) - 1));
    uint32_t mask = 0xFFFFFFFFu & (uint32_t)((1 << num_bits) - 1);
    return bits & mask;
}

/* dequantize (moment_quantization.cpp:55-66) */
float oracle_dequantize(uint32_t q, int num_bits, float vmin, float vmax)
{
    if (num_bits == 32)
    {
        float f;
        memcpy(&f, &q, sizeof(float));
        return clampf_ref(f, vmin, vmax);
    }
    float norm = (float)q / (float)((1 << num_bits) - 1);
    return norm * (vmax - vmin) + vmin;
}

/* sample_moment_image (moment_image_sample.h:33-62): the sample is a full image whose index holds the moment
 * counts; compact() (moment_image.cpp:69-94) then turns the counts into offsets and packs the data. */
uint64_t oracle_sample_moment_image(int width, int height, const uint32_t *index, const float *data, int s,
                                    uint32_t *s_index, float *s_data)
{
    const int factor_x = width / s, factor_y = height / s;
    uint32_t sum = 0;
    for (int y = 0; y < s; ++y)
    {
        for (int x = 0; x < s; ++x)
        {
            size_t src = (size_t)(y * factor_y) * (size_t)width + (size_t)(x * factor_x);
            uint32_t n = index[src + 1] - index[src];
            s_index[y * s + x] = sum;
            if (s_data)
                for (uint32_t l = 0; l < n; ++l)
                    s_data[(size_t)sum + l] = data[(size_t)index[src] + l];
            sum += n;
        }
    }
    s_index[(size_t)s * (size_t)s] = sum;
    return sum;
}

void oracle_default_quantization_table(int m, int num_bits, uint8_t *table)
{
    for (int l = 0; l < m; ++l)
        table[l] = (uint8_t)(l == 0 ? 16 : num_bits);
}

/* quantize_prediction_coding (moment_quantization.cpp:239-276) with pack_bits (:92-114): LSB-first bit stream
 * in pixel row-major order, l ascending; a trailing partial byte is not emitted. */
uint64_t oracle_quantize_prediction_coding(int width, int height, int m, const uint32_t *index, const float *data,
                                           const uint8_t *table, uint8_t *out)
{
    uint64_t nbytes = 0;
    uint8_t buffer = 0;
    int current_bit = 0;
    for (int y = 0; y < height; ++y)
    {
        for (int x = 0; x < width; ++x)
        {
            size_t idx;
            int n;
            pixel_span_f32(index, width, m, x, y, &idx, &n);
            if (n == 0)
                continue;
            for (int l = 0; l < n; ++l)
            {
                int nb = table[l];
                uint32_t w = oracle_quantize(data[idx + l], nb, 0.0f, 1.0f);
                for (int b = 0; b < nb; ++b)
                {
                    if (w & (1u << b))
                        buffer |= (uint8_t)(1u << current_bit);
                    ++current_bit;
                    if (current_bit == 8)
                    {
                        if (out)
                            out[nbytes] = buffer;
                        ++nbytes;
                        buffer = 0;
                        current_bit = 0;
                    }
                }
            }
        }
    }
    return nbytes;
}

/* dequantize_prediction_coding (moment_quantization.cpp:278-332) with unpack_bits (:135-160).  Words that the
 * byte stream does not contain (the packer drops a trailing partial byte) read as 0. */
void oracle_dequantize_prediction_coding(int width, int height, int m, const uint32_t *index, const uint8_t *table,
                                         const uint8_t *bytes, uint64_t num_bytes, float *data)
{
    uint64_t bitpos = 0;
    const uint64_t total_bits = num_bytes * 8;
    for (int y = 0; y < height; ++y)
    {
        for (int x = 0; x < width; ++x)
        {
            size_t idx;
            int n;
            pixel_span_f32(index, width, m, x, y, &idx, &n);
            if (n == 0)
                continue;
            for (int l = 0; l < n; ++l)
            {
                int nb = table[l];
                uint32_t w = 0;
                if (bitpos + (uint64_t)nb <= total_bits)
                {
                    for (int b = 0; b < nb; ++b)
                    {
                        uint64_t bp = bitpos + (uint64_t)b;
                        if (bytes[bp >> 3] & (1u << (bp & 7)))
                            w |= (1u << b);
                    }
                }
                bitpos += (uint64_t)nb;
                data[idx + l] = oracle_dequantize(w, nb, 0.0f, 1.0f);
            }
        }
    }
}

/* preintegrate (transfer_function.cpp:46-97): the stored entry for column x is the premultiplied tf1d[x]; the
 * numerically integrated value computed beside it is discarded by the reference and so is not reproduced. */
void oracle_preintegrate(const float *tf1d, float step_size, float *table)
{
    for (int x = 0; x < 256; ++x)
    {
        float w = tf1d[4 * x + 3] * step_size;
        table[4 * x + 0] = tf1d[4 * x + 0] * w;
        table[4 * x + 1] = tf1d[4 * x + 1] * w;
        table[4 * x + 2] = tf1d[4 * x + 2] * w;
        table[4 * x + 3] = w;
    }
}

/* cosf / sinf of trigonometricToExponentialMoments (mese/MESE_dynamic.h:38-40): the C library's */
void oracle_libm_sincosf(uint64_t n, const float *x, float *s, float *c)
{
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; ++i)
    {
        c[i] = cosf(x[i]);
        s[i] = sinf(x[i]);
    }
}

/* ColorImageHost::set_color / rgba8_t (color_image.h:41-47, 60-65) */
void oracle_rgba_to_u8(uint64_t num_pixels, const float *rgba, uint8_t *out)
{
    for (uint64_t i = 0; i < 4 * num_pixels; ++i)
        out[i] = (uint8_t)(clampf_ref(rgba[i], 0.0f, 1.0f) * 255.f);
}
