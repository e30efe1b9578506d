// The moment-image file format (write_moment_image / load_moment_image, src/moment_image_io.cpp:32-529) and its
// entropy-coded payload (src/moment_image_coding.cpp:34-234): host-side serialisation.  The quantization of the
// payload runs on the GPU (coding.cu); this file holds the byte layout, LZ4 sections and the arithmetic-coded
// streams.
//
// Layout (little-endian):
//   header   u16 width, u16 height, u8 moments, u8 coding warp, u8 flags, u8 bits, f32 domain min[3], max[3]
//            flags: 1 compressed, 2 compact, 4 prediction coded, 16 bounds, 32 error bounds, 128 coding params;
//            bits: quantization bits (low six), 64 entropy coded, 128 quantization table follows
//   [table]  the prediction-coding table, one byte per moment index (a section)
//   compact: the per-pixel moment counts as u8 (a section), [bounds u16 pairs], [error bounds u16], [coding
//            params u16 pairs], the payload (a section): floats, packed codes or the entropy-coded streams
//   static:  [bounds], [error bounds], [coding params], then the payload without a size prefix
// A section is stored as is, or when compressed as u32 size + LZ4 block (u32 size + the bytes where LZ4 does not
// shrink them).
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace mraygb
{

struct FileHeader
{
    uint16_t width = 0, height = 0;
    uint8_t moments = 0, coding_warp = 0, flags = 0, bits = 0;
    float dmin[3] = {0, 0, 0}, dmax[3] = {0, 0, 0};

    bool compressed() const { return flags & 1; }
    bool compact() const { return flags & 2; }
    bool prediction_coded() const { return flags & 4; }
    bool has_bounds() const { return flags & 16; }
    bool has_error_bounds() const { return flags & 32; }
    bool has_coding_params() const { return flags & 128; }
    int quantization_bits() const { return bits & 0x3f; }
    bool entropy_coded() const { return bits & 64; }
    bool has_table() const { return bits & 128; }
};

constexpr size_t kFileHeaderBytes = 32;

void put_header(std::vector<uint8_t> &out, const FileHeader &h);
// false when fewer than kFileHeaderBytes remain
bool get_header(const uint8_t *p, size_t n, FileHeader &h);

// write_bytes (moment_image_io.cpp:315-336)
void put_section(std::vector<uint8_t> &out, const uint8_t *data, size_t n, bool compress);

// reads one section of byte_size bytes at *pos (read_bytes, moment_image_io.cpp:32-60); false on a truncated file
bool get_section(const uint8_t *file, size_t file_size, size_t *pos, size_t byte_size, bool compressed, uint8_t *out);

// the payload section of a compact image (read_moment_bytes, moment_image_io.cpp:62-105): bound = 4 * moments; to
// the end of the file when not compressed
bool get_payload(const uint8_t *file, size_t file_size, size_t *pos, size_t bound, bool compressed,
                 std::vector<uint8_t> &bytes);

// entropy_encode / entropy_decode (moment_image_coding.cpp:206-234): symbols are the u16 codes in the layout of the
// moment data (index: W*H+1 offsets), the zeroth moments stored as u16, index l >= 1 coded in its own stream with an
// adaptive model of 2^table[l] symbols; the streams run on up to `threads` host threads
std::vector<uint8_t> entropy_encode(int width, int height, int m, const uint32_t *index, const uint16_t *symbols,
                                    const uint8_t *table, int threads);
// returns false on a malformed container
bool entropy_decode(const uint8_t *bytes, size_t n, int width, int height, int m, const uint32_t *index,
                    const uint8_t *table, uint16_t *symbols, int threads);

} // namespace mraygb
