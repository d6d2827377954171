/* Minimal IEEE 754 binary16 type for compiling the reference's CPU code.
 * Conversion to float follows the binary16 format definition (1 sign bit,
 * 5 exponent bits with bias 15, 10 fraction bits; exponent 0 = subnormal,
 * exponent 31 = inf/NaN). */
#pragma once
#include <cmath>
#include <cstdint>
struct half {
    uint16_t bits;
    operator float() const {
        const uint32_t s = (bits >> 15) & 1u, e = (bits >> 10) & 0x1fu, m = bits & 0x3ffu;
        float f;
        if (e == 0) f = std::ldexp((float)m, -24);
        else if (e == 31) f = m ? NAN : INFINITY;
        else f = std::ldexp((float)(m | 0x400u), (int)e - 25);
        return s ? -f : f;
    }
};
