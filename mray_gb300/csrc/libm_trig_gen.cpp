// Build-time generator of the exception table of libm_trig_core.h: runs the host C library's sinf / cosf over
// every float of [-pi, pi] and records where they differ from the core's double-evaluated result.  It runs on the
// machine that builds the library, so the table describes the C library the reference's CPU code calls there.
//
//   libm_trig_gen OUT.bin            write the table (fails if a difference is not exactly one ulp)
//   libm_trig_gen --verify IN.bin    check core + table against the C library for every float of [-pi, pi]
//
// Compiled with -ffp-contract=off, so the core's double arithmetic rounds exactly as the device form does.

#include "libm_trig_core.h"

#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <thread>
#include <vector>

using namespace mraygb::libm_trig;

namespace
{

// The C library's functions, called separately as the reference's expression does (gcc may merge the pair into
// sincosf, which glibc evaluates identically).
float (*volatile g_sinf)(float) = sinf;
float (*volatile g_cosf)(float) = cosf;

uint32_t f2u(float f)
{
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
}
float u2f(uint32_t u)
{
    float f;
    memcpy(&f, &u, 4);
    return f;
}

// Entry for x (bits), 0 if the core already agrees; -1 if a difference is not one ulp of the same sign.
int entry_for(uint32_t bits)
{
    const float x = u2f(bits);
    float cs, cc;
    core_sincosf(x, cs, cc);
    const uint32_t ls = f2u(g_sinf(x)), lc = f2u(g_cosf(x));
    const uint32_t ms = f2u(cs), mc = f2u(cc);
    uint32_t e = 0;
    if (ls != ms)
    {
        if (ls == ms + 1u)
            e |= kSinDiffers | kSinUp;
        else if (ls == ms - 1u)
            e |= kSinDiffers;
        else
            return -1;
    }
    if (lc != mc)
    {
        if (lc == mc + 1u)
            e |= kCosDiffers | kCosUp;
        else if (lc == mc - 1u)
            e |= kCosDiffers;
        else
            return -1;
    }
    if (e)
        e |= bits & kLowMask;
    return (int)e;
}

unsigned num_threads()
{
    const unsigned n = std::thread::hardware_concurrency();
    return n ? std::min(n, 64u) : 4u;
}

// Buckets [b0, b1) of every worker: per bucket its entries in ascending low bits.
struct Span
{
    std::vector<uint32_t> counts; // entries per bucket
    std::vector<uint16_t> entries;
    bool ok = true;
    uint32_t bad_bits = 0;
};

void scan_buckets(uint32_t b0, uint32_t b1, Span &out)
{
    out.counts.assign(b1 - b0, 0);
    for (uint32_t b = b0; b < b1; ++b)
    {
        const uint32_t sign = (b & 1u) << 31;
        const uint32_t abs0 = (b >> 1) << kShift;
        for (uint32_t low = 0; low <= kLowMask; ++low)
        {
            const uint32_t a = abs0 | low;
            if (a > kMaxAbsBits)
                break;
            const int e = entry_for(sign | a);
            if (e < 0)
            {
                out.ok = false;
                out.bad_bits = sign | a;
                return;
            }
            if (e)
            {
                out.entries.push_back((uint16_t)e);
                ++out.counts[b - b0];
            }
        }
    }
}

int generate(const char *path)
{
    const unsigned nt = num_threads();
    std::vector<Span> spans(nt);
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nt; ++t)
    {
        const uint32_t b0 = (uint32_t)((uint64_t)kBuckets * t / nt);
        const uint32_t b1 = (uint32_t)((uint64_t)kBuckets * (t + 1) / nt);
        th.emplace_back(scan_buckets, b0, b1, std::ref(spans[t]));
    }
    for (auto &x : th)
        x.join();
    std::vector<uint32_t> offsets;
    offsets.reserve(kBuckets + 1);
    std::vector<uint16_t> entries;
    uint32_t run = 0;
    for (const Span &s : spans)
    {
        if (!s.ok)
        {
            fprintf(stderr, "libm_trig_gen: the C library differs from the core by more than one ulp at 0x%08x\n",
                    s.bad_bits);
            return 1;
        }
        for (uint32_t c : s.counts)
        {
            offsets.push_back(run);
            run += c;
        }
        entries.insert(entries.end(), s.entries.begin(), s.entries.end());
    }
    offsets.push_back(run);
    Header h = {kMagic, kVersion, kShift, kBuckets, (uint32_t)entries.size(), kMaxAbsBits, 0, 0};
    FILE *f = fopen(path, "wb");
    if (!f)
    {
        perror(path);
        return 1;
    }
    bool ok = fwrite(&h, sizeof h, 1, f) == 1 &&
              fwrite(offsets.data(), sizeof(uint32_t), offsets.size(), f) == offsets.size() &&
              fwrite(entries.data(), sizeof(uint16_t), entries.size(), f) == entries.size();
    ok = (fclose(f) == 0) && ok;
    if (!ok)
    {
        fprintf(stderr, "libm_trig_gen: writing %s failed\n", path);
        return 1;
    }
    printf("libm_trig_gen: %u entries in %u buckets\n", h.n_entries, h.n_buckets);
    return 0;
}

int verify(const char *path)
{
    FILE *f = fopen(path, "rb");
    if (!f)
    {
        perror(path);
        return 1;
    }
    Header h;
    if (fread(&h, sizeof h, 1, f) != 1 || h.magic != kMagic || h.version != kVersion || h.shift != kShift ||
        h.n_buckets != kBuckets || h.max_abs_bits != kMaxAbsBits)
    {
        fprintf(stderr, "libm_trig_gen: %s is not a table of this version\n", path);
        fclose(f);
        return 1;
    }
    std::vector<uint32_t> offsets(h.n_buckets + 1);
    std::vector<uint16_t> entries(h.n_entries + 1);
    const bool ok = fread(offsets.data(), sizeof(uint32_t), offsets.size(), f) == offsets.size() &&
                    fread(entries.data(), sizeof(uint16_t), h.n_entries, f) == h.n_entries;
    fclose(f);
    if (!ok || offsets.back() != h.n_entries)
    {
        fprintf(stderr, "libm_trig_gen: %s is truncated\n", path);
        return 1;
    }
    const unsigned nt = num_threads();
    std::vector<uint64_t> bad(nt, 0), first(nt, 0);
    std::vector<std::thread> th;
    const uint64_t n_abs = (uint64_t)kMaxAbsBits + 1;
    for (unsigned t = 0; t < nt; ++t)
        th.emplace_back([&, t] {
            for (uint64_t a = n_abs * t / nt; a < n_abs * (t + 1) / nt; ++a)
                for (uint32_t sign = 0; sign < 2; ++sign)
                {
                    const uint32_t bits = (uint32_t)a | (sign << 31);
                    const float x = u2f(bits);
                    float cs, cc;
                    core_sincosf(x, cs, cc);
                    uint32_t sb = f2u(cs), cb = f2u(cc);
                    apply_entry(find_entry(offsets.data(), entries.data(), bits), sb, cb);
                    if (sb != f2u(g_sinf(x)) || cb != f2u(g_cosf(x)))
                    {
                        if (!bad[t])
                            first[t] = bits;
                        ++bad[t];
                    }
                }
        });
    for (auto &x : th)
        x.join();
    uint64_t total = 0;
    for (unsigned t = 0; t < nt; ++t)
    {
        if (bad[t] && !total)
            fprintf(stderr, "libm_trig_gen: first mismatch at 0x%08llx\n", (unsigned long long)first[t]);
        total += bad[t];
    }
    printf("libm_trig_gen: %llu floats checked, %llu mismatches\n", (unsigned long long)(2 * n_abs),
           (unsigned long long)total);
    return total ? 1 : 0;
}

} // namespace

int main(int argc, char **argv)
{
    if (argc == 2)
        return generate(argv[1]);
    if (argc == 3 && strcmp(argv[1], "--verify") == 0)
        return verify(argv[2]);
    fprintf(stderr, "usage: libm_trig_gen OUT.bin | libm_trig_gen --verify IN.bin\n");
    return 2;
}
