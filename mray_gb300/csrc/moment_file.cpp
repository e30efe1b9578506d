// Host-side serialisation of moment-image files (layout in moment_file.h).

#include "moment_file.h"

#include <algorithm>
#include <atomic>
#include <cstring>
#include <thread>

#include "arith_coder.h"
#include "lz4_block.h"

namespace mraygb
{

namespace
{

template <class T> void put(std::vector<uint8_t> &out, const T &v)
{
    const size_t o = out.size();
    out.resize(o + sizeof(T));
    std::memcpy(out.data() + o, &v, sizeof(T));
}

template <class T> bool get(const uint8_t *p, size_t n, size_t *pos, T &v)
{
    if (n - *pos < sizeof(T) || *pos > n)
        return false;
    std::memcpy(&v, p + *pos, sizeof(T));
    *pos += sizeof(T);
    return true;
}

// runs job(l) for l in [first, last) on up to `threads` host threads
template <class F> void parallel_for(int first, int last, int threads, F job)
{
    const int count = last - first;
    if (count <= 0)
        return;
    const int t = std::max(1, std::min(threads, count));
    if (t == 1)
    {
        for (int l = first; l < last; ++l)
            job(l);
        return;
    }
    std::atomic<int> next(first);
    std::vector<std::thread> pool;
    for (int i = 0; i < t; ++i)
        pool.emplace_back([&] {
            for (int l = next++; l < last; l = next++)
                job(l);
        });
    for (auto &th : pool)
        th.join();
}

} // namespace

void put_header(std::vector<uint8_t> &out, const FileHeader &h)
{
    put(out, h.width);
    put(out, h.height);
    put(out, h.moments);
    put(out, h.coding_warp);
    put(out, h.flags);
    put(out, h.bits);
    for (int i = 0; i < 3; ++i)
        put(out, h.dmin[i]);
    for (int i = 0; i < 3; ++i)
        put(out, h.dmax[i]);
}

bool get_header(const uint8_t *p, size_t n, FileHeader &h)
{
    size_t pos = 0;
    bool ok = get(p, n, &pos, h.width) && get(p, n, &pos, h.height) && get(p, n, &pos, h.moments) &&
              get(p, n, &pos, h.coding_warp) && get(p, n, &pos, h.flags) && get(p, n, &pos, h.bits);
    for (int i = 0; i < 3 && ok; ++i)
        ok = get(p, n, &pos, h.dmin[i]);
    for (int i = 0; i < 3 && ok; ++i)
        ok = get(p, n, &pos, h.dmax[i]);
    return ok;
}

void put_section(std::vector<uint8_t> &out, const uint8_t *data, size_t n, bool compress)
{
    if (!compress)
    {
        out.insert(out.end(), data, data + n);
        return;
    }
    // the block must come out shorter than the input, else the bytes are stored as they are
    std::vector<uint8_t> block(n);
    const size_t r = n ? lz4_compress(data, n, block.data(), n) : 0;
    const bool packed = r > 0 && r < n;
    put(out, (uint32_t)(packed ? r : n));
    if (packed)
        out.insert(out.end(), block.begin(), block.begin() + (long)r);
    else
        out.insert(out.end(), data, data + n);
}

bool get_section(const uint8_t *file, size_t file_size, size_t *pos, size_t byte_size, bool compressed, uint8_t *out)
{
    if (!compressed)
    {
        if (file_size - *pos < byte_size || *pos > file_size)
            return false;
        std::memcpy(out, file + *pos, byte_size);
        *pos += byte_size;
        return true;
    }
    uint32_t stored = 0;
    if (!get(file, file_size, pos, stored) || file_size - *pos < stored || stored > byte_size)
        return false;
    if (stored == byte_size)
        std::memcpy(out, file + *pos, byte_size);
    else if (lz4_decompress(file + *pos, stored, out, byte_size) < 0)
        std::memcpy(out, file + *pos, stored); // not a block: the bytes themselves (as the reference reads them)
    *pos += stored;
    return true;
}

bool get_payload(const uint8_t *file, size_t file_size, size_t *pos, size_t bound, bool compressed,
                 std::vector<uint8_t> &bytes)
{
    if (!compressed)
    {
        if (*pos > file_size)
            return false;
        bytes.assign(file + *pos, file + file_size);
        *pos = file_size;
        return true;
    }
    uint32_t stored = 0;
    if (!get(file, file_size, pos, stored))
        return false;
    if (stored == bound || stored == 0)
    {
        if (file_size - *pos < bound)
            return false;
        bytes.assign(file + *pos, file + *pos + bound);
        *pos += bound;
        return true;
    }
    if (file_size - *pos < stored)
        return false;
    bytes.resize(bound);
    const long long r = lz4_decompress(file + *pos, stored, bytes.data(), bound);
    if (r < 0)
        bytes.assign(file + *pos, file + *pos + stored);
    else
        bytes.resize((size_t)r);
    *pos += stored;
    return true;
}

std::vector<uint8_t> entropy_encode(int width, int height, int m, const uint32_t *index, const uint16_t *symbols,
                                    const uint8_t *table, int threads)
{
    const size_t P = (size_t)width * (size_t)height;
    std::vector<uint16_t> zeroth;
    zeroth.reserve(P);
    for (size_t p = 0; p < P; ++p)
        if (index[p + 1] > index[p])
            zeroth.push_back(symbols[index[p]]);
    std::vector<std::vector<uint8_t>> streams((size_t)(m > 1 ? m - 1 : 0));
    parallel_for(1, m, threads, [&](int l) {
        AdaptiveModel model(1u << table[l]);
        ArithEncoder enc(P);
        for (size_t p = 0; p < P; ++p)
            if (index[p + 1] - index[p] > (uint32_t)l)
                enc.put(symbols[index[p] + l], model);
        streams[l - 1] = std::move(enc.finish());
    });
    std::vector<uint8_t> out;
    put(out, (uint32_t)zeroth.size());
    const size_t o = out.size();
    out.resize(o + zeroth.size() * sizeof(uint16_t));
    if (!zeroth.empty())
        std::memcpy(out.data() + o, zeroth.data(), zeroth.size() * sizeof(uint16_t));
    for (const auto &s : streams)
    {
        put(out, (uint32_t)s.size());
        out.insert(out.end(), s.begin(), s.end());
    }
    return out;
}

bool entropy_decode(const uint8_t *bytes, size_t n, int width, int height, int m, const uint32_t *index,
                    const uint8_t *table, uint16_t *symbols, int threads)
{
    const size_t P = (size_t)width * (size_t)height;
    size_t pos = 0;
    uint32_t nz = 0;
    if (!get(bytes, n, &pos, nz) || (n - pos) / sizeof(uint16_t) < nz)
        return false;
    const size_t zeroth_at = pos;
    pos += (size_t)nz * sizeof(uint16_t);
    std::vector<size_t> at((size_t)(m > 1 ? m - 1 : 0)), len(at.size());
    for (size_t i = 0; i < at.size(); ++i)
    {
        uint32_t s = 0;
        if (!get(bytes, n, &pos, s) || n - pos < s)
            return false;
        at[i] = pos;
        len[i] = s;
        pos += s;
    }
    size_t k = 0;
    for (size_t p = 0; p < P; ++p)
        if (index[p + 1] > index[p])
        {
            if (k == nz)
                return false;
            uint16_t v;
            std::memcpy(&v, bytes + zeroth_at + k * sizeof(uint16_t), sizeof(v));
            symbols[index[p]] = v;
            ++k;
        }
    parallel_for(1, m, threads, [&](int l) {
        AdaptiveModel model(1u << table[l]);
        ArithDecoder dec(bytes + at[l - 1], len[l - 1]);
        for (size_t p = 0; p < P; ++p)
            if (index[p + 1] - index[p] > (uint32_t)l)
                symbols[index[p] + l] = (uint16_t)dec.get(model);
    });
    return true;
}

} // namespace mraygb
