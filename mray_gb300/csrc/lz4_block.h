// LZ4 block format (the compressed layout that LZ4_compress_default / LZ4_decompress_safe read and write, as the
// reference's moment-image files use it, src/moment_image_io.cpp:32-105 and 315-336).  Host code.
//
// A block is a series of sequences: a token (high nibble: literal count, low nibble: match length - 4, 15 meaning
// "more in following bytes of 255 ... until one below 255"), the literals, a 16-bit little-endian back offset
// (1..65535) and the match length extension.  The last sequence carries literals only; a block's last five bytes
// are literals and its last match starts at least twelve bytes before its end.
#pragma once

#include <cstddef>
#include <cstdint>

namespace mraygb
{

// worst-case compressed size of n input bytes (all literals)
size_t lz4_bound(size_t n);

// compresses src[0, n) into dst (capacity cap); returns the block size, or 0 when it does not fit in cap (callers
// then store the bytes uncompressed, as the reference does).  n < 2^31.
size_t lz4_compress(const uint8_t *src, size_t n, uint8_t *dst, size_t cap);

// decompresses a block of n bytes into dst (capacity cap); returns the decoded size, or -1 for a malformed block or
// one that does not fit in cap (never reads or writes outside the two buffers).
long long lz4_decompress(const uint8_t *src, size_t n, uint8_t *dst, size_t cap);

} // namespace mraygb
