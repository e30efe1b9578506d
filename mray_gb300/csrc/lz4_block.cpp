// LZ4 block compression and decompression (format in lz4_block.h).  The compressor is a greedy single-pass match
// finder: a 2^16-entry table maps a hash of the four bytes at a position to the last position with that hash; a
// candidate within the 64 KiB window whose four bytes agree starts a match, extended forward as far as the block's
// end rules allow and backward over the pending literals.  Runs of misses widen the scan step, so incompressible
// input costs little.  Any valid block decodes to the same bytes, so the output need not equal another LZ4
// encoder's.

#include "lz4_block.h"

#include <cstring>
#include <vector>

namespace mraygb
{

namespace
{

constexpr size_t kMinMatch = 4;
constexpr size_t kLastLiterals = 5; // the block's last five bytes are literals
constexpr size_t kMatchStartLimit = 12; // no match starts in the block's last twelve bytes
constexpr size_t kMaxOffset = 65535;
constexpr int kHashLog = 16;

inline uint32_t read32(const uint8_t *p)
{
    uint32_t v;
    std::memcpy(&v, p, 4);
    return v;
}

inline uint32_t hash4(uint32_t v) { return (v * 2654435761u) >> (32 - kHashLog); }

struct Writer
{
    uint8_t *p, *end;
    bool ok = true;

    bool room(size_t n)
    {
        if ((size_t)(end - p) < n)
            ok = false;
        return ok;
    }
    void length_extension(size_t v) // v >= 15 already taken by the nibble
    {
        v -= 15;
        while (v >= 255 && room(1))
        {
            *p++ = 255;
            v -= 255;
        }
        if (room(1))
            *p++ = (uint8_t)v;
    }
    void sequence(const uint8_t *lit, size_t nlit, size_t offset, size_t mlen) // mlen = 0: literals only
    {
        if (!room(1))
            return;
        const size_t ml = mlen ? mlen - kMinMatch : 0;
        *p++ = (uint8_t)(((nlit < 15 ? nlit : 15) << 4) | (mlen ? (ml < 15 ? ml : 15) : 0));
        if (nlit >= 15)
            length_extension(nlit);
        if (!room(nlit))
            return;
        std::memcpy(p, lit, nlit);
        p += nlit;
        if (!mlen)
            return;
        if (!room(2))
            return;
        *p++ = (uint8_t)(offset & 0xff);
        *p++ = (uint8_t)(offset >> 8);
        if (ml >= 15)
            length_extension(ml);
    }
};

} // namespace

size_t lz4_bound(size_t n) { return n + n / 255 + 16; }

size_t lz4_compress(const uint8_t *src, size_t n, uint8_t *dst, size_t cap)
{
    Writer w{dst, dst + cap};
    size_t anchor = 0;
    if (n >= kMatchStartLimit + 1)
    {
        std::vector<uint32_t> table((size_t)1 << kHashLog, 0xffffffffu);
        const size_t match_start_end = n - kMatchStartLimit; // matches start before this
        const size_t match_end = n - kLastLiterals;          // and end at or before this
        size_t i = 0;
        unsigned misses = 0;
        while (i < match_start_end && w.ok)
        {
            const uint32_t v = read32(src + i);
            const uint32_t h = hash4(v);
            const uint32_t c = table[h];
            table[h] = (uint32_t)i;
            if (c != 0xffffffffu && i - c <= kMaxOffset && read32(src + c) == v)
            {
                size_t s = i, cand = c;
                size_t e = i + kMinMatch, ce = c + kMinMatch;
                while (e < match_end && src[e] == src[ce])
                {
                    ++e;
                    ++ce;
                }
                while (s > anchor && cand > 0 && src[s - 1] == src[cand - 1])
                {
                    --s;
                    --cand;
                }
                w.sequence(src + anchor, s - anchor, i - c, e - s);
                // index two positions inside the match so that repeats are found soon
                if (e - 2 > i && e - 2 < match_start_end)
                    table[hash4(read32(src + e - 2))] = (uint32_t)(e - 2);
                anchor = i = e;
                misses = 0;
            }
            else
            {
                ++misses;
                i += 1 + (misses >> 6);
            }
        }
    }
    w.sequence(src + anchor, n - anchor, 0, 0);
    return w.ok ? (size_t)(w.p - dst) : 0;
}

long long lz4_decompress(const uint8_t *src, size_t n, uint8_t *dst, size_t cap)
{
    const uint8_t *ip = src, *const iend = src + n;
    size_t op = 0;
    if (n == 0)
        return -1;
    for (;;)
    {
        if (ip >= iend)
            return -1;
        const unsigned token = *ip++;
        size_t nlit = token >> 4;
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
        if ((size_t)(iend - ip) < nlit || cap - op < nlit)
            return -1;
        std::memcpy(dst + op, ip, nlit);
        ip += nlit;
        op += nlit;
        if (ip == iend)
            return (long long)op; // the last sequence: literals only
        if (iend - ip < 2)
            return -1;
        const size_t offset = (size_t)ip[0] | ((size_t)ip[1] << 8);
        ip += 2;
        if (offset == 0 || offset > op)
            return -1;
        size_t mlen = (token & 15u);
        if (mlen == 15)
        {
            unsigned b;
            do
            {
                if (ip >= iend)
                    return -1;
                b = *ip++;
                mlen += b;
            } while (b == 255);
        }
        mlen += kMinMatch;
        if (cap - op < mlen)
            return -1;
        // byte by byte: the match may overlap its own output (offset < length repeats a pattern)
        const uint8_t *m = dst + op - offset;
        for (size_t k = 0; k < mlen; ++k)
            dst[op + k] = m[k];
        op += mlen;
    }
}

} // namespace mraygb
