// Exact FP32 high/low split of an FP64 value with integer arithmetic:
//   hi = fl32(v) (round to nearest, ties to even), lo = fl32(v - hi)
// bit for bit, for v whose float results are normal numbers; every other v
// (zero, subnormal, huge, infinite, NaN) takes the FP64 expression.  GB300's
// FP64 rate is a small fraction of its integer and FP32 rates, and the
// FP64 form costs three conversions and a subtraction per value.
//
// v = M * 2^(E - 52) with M = 2^52 + mantissa (53 bits).  hi = R * 2^(E - 23)
// with R = M / 2^29 rounded to nearest even (2^23 <= R <= 2^24; R = 2^24
// carries into the exponent).  v - hi = D * 2^(E - 52) exactly, with
// D = M - R * 2^29 and |D| <= 2^28, so lo = fl32(D) * 2^(E - 52): the
// int -> float conversion rounds like fl32, and the power-of-two scale is
// exact while the result stays normal (E >= -74).  A zero difference gives
// +0.0, as v - hi does in FP64.
#pragma once

#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define PYCI_HD __host__ __device__
#else
#define PYCI_HD
#endif

namespace pyci_gpu {

PYCI_HD inline uint64_t split_bits_of(double v) {
    uint64_t u;
    std::memcpy(&u, &v, sizeof(u));
    return u;
}

PYCI_HD inline float split_float_of(uint32_t b) {
    float f;
    std::memcpy(&f, &b, sizeof(f));
    return f;
}

PYCI_HD inline void split_hi_lo(double v, float &hi, float &lo) {
    const uint64_t u = split_bits_of(v);
    const int e = static_cast<int>((u >> 52) & 0x7FF);
    const int E = e - 1023;
    if (e == 0 || e == 0x7FF || E < -74 || E > 126) {
        hi = static_cast<float>(v);
        lo = static_cast<float>(v - static_cast<double>(hi));
        return;
    }
    const uint32_t sign = static_cast<uint32_t>(u >> 63) << 31;
    const uint64_t M = (u & ((1ULL << 52) - 1)) | (1ULL << 52);
    uint64_t R = M >> 29;
    const uint64_t rem = M & ((1ULL << 29) - 1), half = 1ULL << 28;
    if (rem > half || (rem == half && (R & 1)))
        ++R;
    // hi: exponent E (or E + 1 on a carry to 2^24), 23-bit fraction.
    const uint32_t hbits = (R == (1ULL << 24)) ? sign | (static_cast<uint32_t>(E + 1 + 127) << 23)
                                               : sign | (static_cast<uint32_t>(E + 127) << 23) |
                                                     static_cast<uint32_t>(R - (1ULL << 23));
    hi = split_float_of(hbits);
    const int64_t D = static_cast<int64_t>(M) - static_cast<int64_t>(R << 29);
    if (D == 0) {
        lo = 0.0f;
        return;
    }
    const float scale = split_float_of(static_cast<uint32_t>(E - 52 + 127) << 23); // 2^(E - 52), normal
    const float mag = static_cast<float>(static_cast<int32_t>(D)) * scale;
    lo = sign ? -mag : mag;
}

} // namespace pyci_gpu
