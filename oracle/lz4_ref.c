/*
 * ORACLE — test infrastructure only.
 *
 * LZ4 block format, written independently of the product's codec so that each checks the other: a decoder that
 * follows the format description (token with literal and match-length nibbles, 255-continued lengths, literals,
 * 16-bit little-endian offset; the last sequence holds literals only) and an encoder that finds matches by a
 * 5-byte hash with one candidate per bucket, no backward extension, and keeps the format's end rules (the last
 * 5 bytes are literals, no match starts in the last 12).
 */
#include <stdint.h>
#include <string.h>

#include "lz4_stub/lz4.h"

static int put_len(unsigned char **op, unsigned char *oend, int v)
{
    while (v >= 255)
    {
        if (*op >= oend)
            return 0;
        *(*op)++ = 255;
        v -= 255;
    }
    if (*op >= oend)
        return 0;
    *(*op)++ = (unsigned char)v;
    return 1;
}

static int put_seq(unsigned char **op, unsigned char *oend, const unsigned char *lit, int nlit, int off, int mlen)
{
    if (*op >= oend)
        return 0;
    int ml = mlen ? mlen - 4 : 0;
    *(*op)++ = (unsigned char)(((nlit >= 15 ? 15 : nlit) << 4) | (mlen ? (ml >= 15 ? 15 : ml) : 0));
    if (nlit >= 15 && !put_len(op, oend, nlit - 15))
        return 0;
    if (oend - *op < nlit)
        return 0;
    memcpy(*op, lit, (size_t)nlit);
    *op += nlit;
    if (!mlen)
        return 1;
    if (oend - *op < 2)
        return 0;
    *(*op)++ = (unsigned char)(off & 255);
    *(*op)++ = (unsigned char)(off >> 8);
    if (ml >= 15 && !put_len(op, oend, ml - 15))
        return 0;
    return 1;
}

#define HBITS 14
static unsigned hash5(const unsigned char *p)
{
    uint64_t v = (uint64_t)p[0] | ((uint64_t)p[1] << 8) | ((uint64_t)p[2] << 16) | ((uint64_t)p[3] << 24) |
                 ((uint64_t)p[4] << 32);
    return (unsigned)((v * 889523592379ull) >> (40 - HBITS)) & ((1u << HBITS) - 1);
}

int LZ4_compress_default(const char *source, char *dest, int n, int cap)
{
    const unsigned char *src = (const unsigned char *)source;
    unsigned char *op = (unsigned char *)dest, *oend = op + cap;
    static int table[1 << HBITS];
    int anchor = 0;
    if (n < 0)
        return 0;
    for (int k = 0; k < (1 << HBITS); ++k)
        table[k] = -1;
    if (n >= 13)
    {
        const int start_end = n - 12, end = n - 5;
        int i = 0;
        while (i < start_end)
        {
            const unsigned h = hash5(src + i);
            const int c = table[h];
            table[h] = i;
            if (c >= 0 && i - c <= 65535 && memcmp(src + c, src + i, 4) == 0)
            {
                int e = i + 4;
                while (e < end && src[e] == src[c + (e - i)])
                    ++e;
                if (!put_seq(&op, oend, src + anchor, i - anchor, i - c, e - i))
                    return 0;
                anchor = i = e;
            }
            else
                ++i;
        }
    }
    if (!put_seq(&op, oend, src + anchor, n - anchor, 0, 0))
        return 0;
    return (int)(op - (unsigned char *)dest);
}

int LZ4_decompress_safe(const char *source, char *dest, int n, int cap)
{
    const unsigned char *ip = (const unsigned char *)source, *iend = ip + n;
    unsigned char *out = (unsigned char *)dest;
    long op = 0;
    if (n <= 0)
        return -1;
    for (;;)
    {
        if (ip >= iend)
            return -1;
        unsigned token = *ip++;
        long nlit = token >> 4;
        if (nlit == 15)
        {
            unsigned b;
            do
            {
                if (ip >= iend)
                    return -1;
                b = *ip++;
                nlit += b;
            } while (b == 255);
        }
        if (iend - ip < nlit || cap - op < nlit)
            return -1;
        memcpy(out + op, ip, (size_t)nlit);
        ip += nlit;
        op += nlit;
        if (ip == iend)
            return (int)op;
        if (iend - ip < 2)
            return -1;
        long off = ip[0] | (ip[1] << 8);
        ip += 2;
        if (off == 0 || off > op)
            return -1;
        long ml = token & 15;
        if (ml == 15)
        {
            unsigned b;
            do
            {
                if (ip >= iend)
                    return -1;
                b = *ip++;
                ml += b;
            } while (b == 255);
        }
        ml += 4;
        if (cap - op < ml)
            return -1;
        for (long k = 0; k < ml; ++k)
            out[op + k] = out[op - off + k];
        op += ml;
    }
}
