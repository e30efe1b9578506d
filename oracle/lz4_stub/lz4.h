/*
 * ORACLE — test infrastructure only.
 *
 * The two LZ4 calls the reference's moment-image files make (src/moment_image_io.cpp:30, 51, 83, 230, 240, 320,
 * 435, 449), declared so that the reference's file-format sources compile here without liblz4, and implemented by
 * oracle/lz4_ref.c: a decoder of the LZ4 block format and a simple encoder of valid blocks.
 */
#ifndef MRAY_ORACLE_LZ4_STUB_H
#define MRAY_ORACLE_LZ4_STUB_H

#ifdef __cplusplus
extern "C" {
#endif

/* returns the block size, 0 when it does not fit in dst_capacity */
int LZ4_compress_default(const char *src, char *dst, int src_size, int dst_capacity);
/* returns the decoded size, a negative value for a malformed block or one that does not fit */
int LZ4_decompress_safe(const char *src, char *dst, int compressed_size, int dst_capacity);

#ifdef __cplusplus
}
#endif

#endif
