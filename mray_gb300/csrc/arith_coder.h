// Adaptive arithmetic coding of quantized moments (entropy_encode / entropy_decode, src/moment_image_coding.cpp:
// 98-234): one independent stream per moment index, each with its own adaptive frequency model.  The reference
// vendors the floating-point form of Amir Said's FastAC coder (A. Said, "Introduction to Arithmetic Coding - Theory
// and Practice", HP Labs HPL-2004-76, and the FastAC package, 2004): the coding interval [base, base + length) is
// held in doubles, renormalised sixteen bits at a time; the model keeps symbol counts and a cumulative distribution
// rebuilt at a growing period.  The stream bytes are a function of every rounding in those steps, so this is the
// same sequence of double operations (host code, built without FMA contraction), written here from the published
// method.
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
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

namespace mraygb
{

// adaptive model of an alphabet of 2 .. 2^14 symbols: counts start at 1, the cumulative distribution is rebuilt
// after `period` coded symbols; the period grows by 5/4 up to 8 (symbols + 6); counts are halved once their sum
// passes 2^17
class AdaptiveModel
{
  public:
    explicit AdaptiveModel(unsigned symbols);
    unsigned symbols() const { return n_; }

  private:
    friend class ArithEncoder;
    friend class ArithDecoder;
    void rebuild();
    void seen(unsigned s)
    {
        ++count_[s];
        if (--until_ == 0)
            rebuild();
    }
    // decoder only: bucket[b] = the symbol whose cumulative interval holds b / 2^kBucketBits (a starting point for
    // the search; the decision itself uses the coder's own comparisons)
    void index_buckets();
    static constexpr int kBucketBits = 12;
    unsigned n_, total_ = 0, period_ = 0, until_ = 0;
    bool buckets_ = false;
    std::vector<unsigned> count_;
    std::vector<double> cdf_;
    std::vector<unsigned> bucket_;
};

class ArithEncoder
{
  public:
    explicit ArithEncoder(size_t expected_bytes = 0) { out_.reserve(expected_bytes); }
    void put(unsigned symbol, AdaptiveModel &model);
    // flushes the final bytes; the encoder is done afterwards
    std::vector<uint8_t> &finish();

  private:
    void carry();
    void renormalize();
    double base_ = 0.0, length_ = 1.0;
    std::vector<uint8_t> out_;
};

class ArithDecoder
{
  public:
    // reads past the end as zero bytes (the stream's last bytes fix every symbol it holds)
    ArithDecoder(const uint8_t *bytes, size_t n);
    unsigned get(AdaptiveModel &model);

  private:
    unsigned byte(size_t i) const { return i < n_ ? bytes_[i] : 0u; }
    void renormalize();
    const uint8_t *bytes_;
    size_t n_, pos_ = 6;
    double base_ = 0.0, length_ = 1.0, value_ = 0.0;
};

} // namespace mraygb
