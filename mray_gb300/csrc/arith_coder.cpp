// The floating-point adaptive arithmetic coder (see arith_coder.h).  Built with -ffp-contract=off: a fused
// multiply-add in `base + length * cdf` would change the stream.

// Attribution.  The coding steps restate the FastAC arithmetic coder, whose notice reads:
//
//   Fast arithmetic coding implementation -> double-precision floating-point arithmetic, Version 1.00, April 25,
//   2004.  WARNING: The only purpose of this program is to demonstrate the basic principles of arithmetic coding.
//   It is provided as is, without any express or implied warranty, without even the warranty of fitness for any
//   particular purpose, or that the implementations are correct.  Permission to copy and redistribute this code is
//   hereby granted, provided that this warning and copyright notices are not removed or altered.
//   Copyright (c) 2004 by Amir Said (said@ieee.org) & William A. Pearlman (pearlw@ecse.rpi.edu)
//
//   The method is described in: Lossless Compression Handbook, ed. K. Sayood, Chapter 5: Arithmetic Coding
//   (A. Said), pp. 101-152, Academic Press, 2003; and A. Said, Introduction to Arithmetic Coding - Theory and
//   Practice, HP Labs report HPL-2004-76.

#include "arith_coder.h"

namespace mraygb
{

namespace
{

constexpr double kOut = 65536.0;               // sixteen bits leave the interval per renormalisation step
constexpr double kMinLength = 1.0 / 65536.0;   // renormalise once the interval is this short
constexpr double kLsb = 1.0 / 16777216.0 / 16777216.0; // 2^-48, the weight of the last code bit
constexpr double kLeakage = 2.0 * kLsb;        // taken off every interval, so rounding never widens it
constexpr unsigned kMaxTotal = 1u << 17;       // counts are halved once their sum passes this

} // namespace

AdaptiveModel::AdaptiveModel(unsigned symbols) : n_(symbols), count_(symbols, 1u), cdf_(symbols, 0.0)
{
    // uniform start: the rebuild adds the first period (n) to the total of the n unit counts
    period_ = n_;
    rebuild();
    until_ = period_ = (n_ + 6) >> 1;
}

void AdaptiveModel::rebuild()
{
    total_ += period_;
    if (total_ > kMaxTotal)
    {
        total_ = 0;
        for (unsigned k = 0; k < n_; ++k)
        {
            count_[k] = (count_[k] + 1) >> 1;
            total_ += count_[k];
        }
    }
    const double scale = 1.0 / double(total_);
    unsigned below = 0;
    for (unsigned k = 0; k < n_; ++k)
    {
        cdf_[k] = scale * below;
        below += count_[k];
    }
    period_ = (5 * period_) >> 2;
    const unsigned longest = (n_ + 6) << 3;
    if (period_ > longest)
        period_ = longest;
    until_ = period_;
    if (buckets_)
        index_buckets();
}

void AdaptiveModel::index_buckets()
{
    const unsigned nb = 1u << kBucketBits;
    bucket_.resize(nb + 1);
    unsigned s = 0;
    for (unsigned b = 0; b <= nb; ++b)
    {
        const double x = double(b) / double(nb);
        while (s + 1 < n_ && cdf_[s + 1] <= x)
            ++s;
        bucket_[b] = s;
    }
}

void ArithEncoder::carry()
{
    base_ -= 1.0;
    // add one to the bytes already out: trailing 0xff become 0, the first other byte grows by one
    size_t i = out_.size();
    while (i > 0 && out_[i - 1] == 0xffu)
        out_[--i] = 0;
    if (i > 0)
        ++out_[i - 1];
}

void ArithEncoder::renormalize()
{
    do
    {
        base_ *= kOut;
        const unsigned a = unsigned(base_);
        out_.push_back((uint8_t)(a >> 8));
        out_.push_back((uint8_t)(a & 0xffu));
        base_ -= double(a);
        length_ *= kOut;
    } while (length_ <= kMinLength);
}

void ArithEncoder::put(unsigned s, AdaptiveModel &m)
{
    const double top = (s == m.n_ - 1) ? base_ + length_ : base_ + length_ * m.cdf_[s + 1];
    base_ += length_ * m.cdf_[s];
    length_ = top - base_;
    if (base_ >= 1.0)
        carry();
    length_ -= kLeakage;
    if (length_ <= kMinLength)
        renormalize();
    m.seen(s);
}

std::vector<uint8_t> &ArithEncoder::finish()
{
    // as few final bytes as identify a point of the interval
    const unsigned lo = unsigned(kOut * base_);
    const unsigned hi = unsigned(kOut * (base_ + length_));
    unsigned last;
    if (hi - lo < 2)
    {
        base_ += 0.5 * kMinLength;
        last = 3;
    }
    else if ((hi >> 8) - (lo >> 8) < 2)
    {
        base_ += kMinLength;
        last = 2;
    }
    else
    {
        base_ += 256.0 * kMinLength;
        last = 1;
    }
    if (base_ >= 1.0)
        carry();
    do
    {
        base_ *= 256.0;
        const unsigned a = unsigned(base_);
        out_.push_back((uint8_t)a);
        base_ -= double(a);
    } while (--last);
    return out_;
}

ArithDecoder::ArithDecoder(const uint8_t *bytes, size_t n) : bytes_(bytes), n_(n)
{
    for (size_t k = 0; k < 6; ++k)
        value_ = 256.0 * value_ + kLsb * byte(k);
}

void ArithDecoder::renormalize()
{
    do
    {
        base_ *= kOut;
        const unsigned a = unsigned(base_);
        base_ -= double(a);
        value_ = (kOut * value_ - double(a)) + kLsb * (256.0 * double(byte(pos_)) + double(byte(pos_ + 1)));
        pos_ += 2;
        length_ *= kOut;
    } while (length_ <= kMinLength);
}

unsigned ArithDecoder::get(AdaptiveModel &m)
{
    // the symbol s with z(s) <= value + lsb < z(s + 1), z(k) = base + length * cdf[k] (z(n) = base + length): the
    // coder's bisection finds the same s, since z strictly grows with k, and ends with base = z(s) and
    // length = z(s + 1) - z(s) as computed here.  The model's bucket table gives the starting guess.
    if (!m.buckets_)
    {
        m.buckets_ = true;
        m.index_buckets();
    }
    const double target = value_ + kLsb;
    const unsigned nb = 1u << AdaptiveModel::kBucketBits;
    double r = (target - base_) / length_;
    r = r < 0.0 ? 0.0 : (r > 1.0 ? 1.0 : r);
    unsigned s = m.bucket_[(unsigned)(r * nb)];
    auto z = [&](unsigned k) { return k >= m.n_ ? base_ + length_ : base_ + length_ * m.cdf_[k]; };
    while (s > 0 && z(s) > target)
        --s;
    while (s + 1 < m.n_ && z(s + 1) <= target)
        ++s;
    const double lo = s == 0 ? base_ : z(s);
    const double hi = z(s + 1);
    base_ = lo;
    length_ = hi - lo;
    if (base_ >= 1.0)
    {
        base_ -= 1.0;
        value_ -= 1.0;
    }
    length_ -= kLeakage;
    if (length_ <= kMinLength)
        renormalize();
    m.seen(s);
    return s;
}

} // namespace mraygb
