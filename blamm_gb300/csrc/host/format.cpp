// format.cpp -- see format.h.
//
// The occurrence file holds one line per hit; printf's %g is most of the cost of
// writing it.  Scores of magnitude 1e-4 .. 1e6 -- every score of a PWM scan in
// practice -- are printed here from exact integer arithmetic: a float is
// m * 2^-s with a 24-bit m, so m * 10^k (k <= 9) fits 64 bits and the decimal
// rounding to 6 significant digits is exact.  Other values go to snprintf.
#include "format.h"

#include <cmath>
#include <cstdio>
#include <cstring>

namespace blamm {

int formatUnsigned(uint64_t v, char *out)
{
    char tmp[24];
    int n = 0;
    do {
        tmp[n++] = (char)('0' + v % 10);
        v /= 10;
    } while (v);
    for (int i = 0; i < n; ++i) out[i] = tmp[n - 1 - i];
    return n;
}

int formatScore(float value, char *out)
{
    const float ax = std::fabs(value);
    if (!(ax >= 1e-4f && ax < 1e6f)) return std::snprintf(out, 16, "%g", (double)value);
    // |value| = m * 2^-s
    int e2;
    const double fr = std::frexp((double)ax, &e2);  // ax = fr * 2^e2, fr in [0.5, 1)
    const uint64_t m = (uint64_t)std::ldexp(fr, 24);  // exact: 24 significant bits
    const int s = 24 - e2;                             // 4 <= s <= 38 in this range
    static const uint64_t p10[10] = {1ull,      10ull,      100ull,      1000ull,      10000ull,
                                     100000ull, 1000000ull, 10000000ull, 100000000ull, 1000000000ull};
    // decimal exponent X = floor(log10 |value|), from an estimate corrected exactly
    int X = (int)std::floor((e2 - 1) * 0.30102999566398120);
    uint64_t v = 0;
    for (int guard = 0; guard < 4; ++guard) {
        const int k = 5 - X;
        if (k < 0 || k > 9) return std::snprintf(out, 16, "%g", (double)value);
        v = m * p10[k];
        if (v < (100000ull << s)) {
            --X;
        } else if (v >= (1000000ull << s)) {
            ++X;
        } else {
            break;
        }
    }
    if (v < (100000ull << s) || v >= (1000000ull << s)) return std::snprintf(out, 16, "%g", (double)value);
    // round to 6 digits, half to even
    uint64_t n = v >> s;
    const uint64_t rem = v & ((1ull << s) - 1), half = 1ull << (s - 1);
    if (rem > half || (rem == half && (n & 1))) ++n;
    if (n == 1000000) {
        n = 100000;
        ++X;
    }
    if (X < -4 || X > 5) return std::snprintf(out, 16, "%g", (double)value);
    char digits[8];
    formatUnsigned(n, digits);  // 6 digits
    int nd = 6;
    while (nd > 1 && digits[nd - 1] == '0') --nd;  // significant digits left
    int o = 0;
    if (value < 0) out[o++] = '-';
    if (X >= 0) {
        for (int i = 0; i <= X; ++i) out[o++] = digits[i];  // integer part (X + 1 <= 6 digits)
        if (nd > X + 1) {
            out[o++] = '.';
            for (int i = X + 1; i < nd; ++i) out[o++] = digits[i];
        }
    } else {
        out[o++] = '0';
        out[o++] = '.';
        for (int i = 0; i < -X - 1; ++i) out[o++] = '0';
        for (int i = 0; i < nd; ++i) out[o++] = digits[i];
    }
    out[o] = '\0';
    return o;
}

}  // namespace blamm
